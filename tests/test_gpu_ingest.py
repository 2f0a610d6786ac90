"""Observations built on the device from the obs store's raw buffers
(read_obs and read_obs_regular, code/x86/TradDA/DA/LETKF/src/read_obs_mod.F90:339-651),
through the C-ABI, against the oracle: bit-exact arrays, and an analysis on
the device-built observations equal to one on the same observations passed
as arrays."""
import numpy as np
import pytest

from conftest import pkg
from oracle import oracle as O
from test_oracle_ingest import _records

pytestmark = pytest.mark.gpu
f32 = np.float32


@pytest.fixture(scope="module")
def letkf():
    pkg("build").build()
    m = pkg("letkf")
    m.load_library()
    return m


def _same(a, b):
    for key in ("lat", "lon", "ph", "lev", "var", "yo", "rinv"):
        assert np.array_equal(a[key], b[key]), key


@pytest.mark.parametrize("nvar,nz,with_randn", [(2, 1, True), (3, 4, True), (1, 1, False)])
def test_records_on_device(letkf, nvar, nz, with_randn):
    w = pkg("synthetic").small_case(nlat=12, nlon=24, nz=4, k=8, nobs=10, seed=70)
    rng = np.random.default_rng(nvar * 10 + nz)
    lon, lat, lev, val, randn = _records(rng, 40 * nz, nvar, nz)
    randn = randn if with_randn else None
    var_of = np.array([1, 2, 3][:nvar], dtype=np.int32)
    ctx = letkf.LetkfGPU.from_workload(w)
    view = ctx.obs_from_records(lon, lat, lev, val, var_of, nz=nz, randn=randn)
    _same(view.to_host(), O.obs_from_records(lon, lat, lev, val, var_of, nz=nz, randn=randn))


def test_broken_profile_is_rejected(letkf):
    w = pkg("synthetic").small_case(nlat=12, nlon=24, nz=4, k=8, nobs=10, seed=71)
    rng = np.random.default_rng(2)
    lon, lat, lev, val, _ = _records(rng, 12, 2, 3)
    lev[5] = 1.0
    ctx = letkf.LetkfGPU.from_workload(w)
    with pytest.raises(letkf.LetkfError):
        ctx.obs_from_records(lon, lat, lev, val, [1, 2], nz=3)


def _regular(rng, nlat_o, nlon_o, nz, nvar):
    lats = rng.uniform(-60, 55, nlat_o).astype(f32)
    latn = (lats + f32(2.0)).astype(f32)
    lonw = rng.uniform(0, 350, nlon_o).astype(f32)
    lone = (lonw + f32(3.0)).astype(f32)
    r = rng.uniform(0.8, 1.5, (nz, nvar)).astype(f32)
    corners = [(rng.standard_normal((nlon_o, nlat_o, nz, nvar + 1)) * 2 + 10).astype(f32) for _ in range(4)]
    for c in corners:
        c[..., 0] = rng.uniform(5e4, 9e4, c.shape[:-1])
    randn = rng.standard_normal((nlat_o * nlon_o, nz, nvar)).astype(f32)
    return latn, lats, lonw, lone, r, corners, randn


def test_regular_grid_on_device_and_analysis(letkf):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    w = pkg("synthetic").small_case(nlat=12, nlon=24, nz=4, k=8, nobs=10, seed=72)
    rng = np.random.default_rng(6)
    latn, lats, lonw, lone, r, corners, randn = _regular(rng, 5, 7, 3, 2)
    var_of = np.array([1, 3], dtype=np.int32)
    ctx = letkf.LetkfGPU.from_workload(w)
    view = ctx.obs_regular(latn, lats, lonw, lone, r, *corners, var_of=var_of, randn=randn)
    ref = O.obs_regular(latn, lats, lonw, lone, r, *corners, var_of=var_of, randn=randn)
    _same(view.to_host(), ref)
    # the analysis on the device-built observations equals the one on the same arrays
    xb = torch.from_numpy(w.xb).to(dev)
    axb = torch.from_numpy(w.axb).to(dev)
    xa, axa = torch.empty_like(xb), torch.empty_like(axb)
    ctx.run_device(xb, axb, view, xa, axa)
    torch.cuda.synchronize()
    xa_h, axa_h = letkf.LetkfGPU.from_workload(w).run(w.xb, w.axb, ref)
    assert np.array_equal(xa.cpu().numpy(), xa_h) and np.array_equal(axa.cpu().numpy(), axa_h)
