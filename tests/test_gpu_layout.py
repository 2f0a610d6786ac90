"""The coupler's layout transforms on the device (through the C-ABI) against
the oracle (code/x86/TradDA/DA/EnDNN/src/data_trans.F90:1-70): pure copies,
so the bar is bit-exact, including the parts of the destination outside the
placed block, which stay as they were."""
import numpy as np
import pytest

from conftest import pkg
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def letkf():
    pkg("build").build()
    m = pkg("letkf")
    m.load_library()
    return m


@pytest.mark.parametrize("n,nx,ny,ens,n_max,ens_max,ns,es",
                         [(3, 5, 7, 4, 9, 6, 4, 2), (97, 18, 36, 64, 97, 64, 1, 1), (1, 9, 4, 33, 2, 40, 2, 8)])
def test_state_transforms_match_oracle(letkf, n, nx, ny, ens, n_max, ens_max, ns, es):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(n + ens)
    xb = rng.standard_normal((n, nx, ny, ens))
    fill = rng.standard_normal((ny, nx, n_max, ens_max))
    ref2 = O.struct_atm2endnn(xb, ens_max, n_max, ens_start=es, n_start=ns, xb2=fill.copy())
    xb_d = torch.from_numpy(xb).to(dev)
    xb2_d = torch.from_numpy(fill).to(dev)
    letkf.struct_atm2endnn(xb_d, xb2_d, ens_start=es, n_start=ns)
    torch.cuda.synchronize()
    assert np.array_equal(xb2_d.cpu().numpy(), ref2)
    back_d = torch.empty_like(xb_d)
    letkf.struct_endnn2atm(xb2_d, back_d, ens_start=es, n_start=ns)
    torch.cuda.synchronize()
    assert np.array_equal(back_d.cpu().numpy(), O.struct_endnn2atm(ref2, ens, n, ens_start=es, n_start=ns))
    assert np.array_equal(back_d.cpu().numpy(), xb)


def test_mean_transforms_match_oracle(letkf):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(9)
    n, nx, ny, n_max, ns = 32, 18, 36, 97, 34
    axb = rng.standard_normal((n, nx, ny))
    fill = rng.standard_normal((ny, nx, n_max))
    ref2 = O.struct_atm2endnn_a(axb, n_max, n_start=ns, axb2=fill.copy())
    a_d = torch.from_numpy(axb).to(dev)
    a2_d = torch.from_numpy(fill).to(dev)
    letkf.struct_atm2endnn_a(a_d, a2_d, n_start=ns)
    torch.cuda.synchronize()
    assert np.array_equal(a2_d.cpu().numpy(), ref2)
    back = torch.empty_like(a_d)
    letkf.struct_endnn2atm_a(a2_d, back, n_start=ns)
    torch.cuda.synchronize()
    assert np.array_equal(back.cpu().numpy(), axb)


def test_bad_block_is_rejected(letkf):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    xb = torch.zeros((3, 4, 5, 8), dtype=torch.float64, device=dev)
    xb2 = torch.zeros((5, 4, 4, 8), dtype=torch.float64, device=dev)
    with pytest.raises(letkf.LetkfError):
        letkf.struct_atm2endnn(xb, xb2, n_start=3)      # rows 3..5 of 4
