"""The batching form: several analysis instances (different grids, ensemble
sizes and forms) in one CUDA graph, and the schedule autotuner.

Bar: a graph replay reproduces the separate runs of the same contexts bitwise
(the same kernels on the same inputs), twice in a row; the autotuned mixed
form stays within the mixed tolerance of the oracle.
"""
import numpy as np
import pytest

from conftest import mean_spread_errors, pkg
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def letkf():
    pkg("build").build()
    m = pkg("letkf")
    m.load_library()
    return m


def _device_case(letkf, torch, w):
    dev = torch.device("cuda", 0)
    xb = torch.from_numpy(w.xb).to(dev)
    axb = torch.from_numpy(w.axb).to(dev)
    obs = letkf.ObsArrays({k: torch.from_numpy(np.ascontiguousarray(w.obs[k])).to(dev)
                           for k in ("lat", "lon", "ph", "lev", "var", "yo", "rinv")}, device=True)
    return xb, axb, obs, torch.empty_like(xb), torch.empty_like(axb)


def test_graph_of_instances_matches_separate_runs(letkf):
    torch = pytest.importorskip("torch")
    synthetic = pkg("synthetic")
    cases = [
        (synthetic.small_case(nlat=12, nlon=24, nz=4, k=32, nobs=900, loc_dist_km=900.0, seed=51),
         letkf.LETKF_PREC_MIXED),
        (synthetic.small_case(nlat=18, nlon=36, nz=3, k=48, nobs=1500, loc_dist_km=700.0, seed=52),
         letkf.LETKF_PREC_MIXED),
        (synthetic.small_case(nlat=12, nlon=24, nz=2, k=16, nobs=600, loc_dist_km=900.0, seed=53),
         letkf.LETKF_PREC_FP64),
    ]
    ctxs, bufs, ref = [], [], []
    for w, prec in cases:
        ctx = letkf.LetkfGPU.from_workload(w, precision=prec)
        b = _device_case(letkf, torch, w)
        ctx.run_device(*b)
        torch.cuda.synchronize()
        ref.append((b[3].cpu().numpy().copy(), b[4].cpu().numpy().copy()))
        ctxs.append(ctx)
        bufs.append(b)
    batch = letkf.Batch(ctxs, [b[0] for b in bufs], [b[1] for b in bufs], [b[2] for b in bufs],
                        [b[3] for b in bufs], [b[4] for b in bufs])
    assert batch.launches >= 6 * len(cases)
    for rep in range(2):
        for b in bufs:
            b[3].zero_()
            b[4].zero_()
        torch.cuda.synchronize()
        batch.launch()
        batch.sync()
        for (xa, axa), b in zip(ref, bufs):
            assert np.array_equal(b[3].cpu().numpy(), xa)
            assert np.array_equal(b[4].cpu().numpy(), axa)
    for ctx in ctxs:
        assert ctx.stats()["sum_p"] > 0
    batch.close()


def test_autotuned_mixed_form(letkf):
    torch = pytest.importorskip("torch")
    synthetic = pkg("synthetic")
    w = synthetic.config(0)
    ctx = letkf.LetkfGPU.from_workload(w, precision=letkf.LETKF_PREC_MIXED)
    b = _device_case(letkf, torch, w)
    chunk = ctx.autotune_device(*b)
    assert chunk in (8, 16, 32, 64)
    ctx.run_device(*b)
    torch.cuda.synchronize()
    assert ctx.stats()["sched_chunk"] == chunk
    xa_o, axa_o = O.Oracle(w).run()
    errs = mean_spread_errors(b[3].cpu().numpy(), b[4].cpu().numpy(), xa_o, axa_o, w)
    assert max(max(v.values()) for v in errs.values()) <= 1e-4, errs


def test_decomposed_contexts_are_not_captured(letkf):
    torch = pytest.importorskip("torch")
    synthetic = pkg("synthetic")
    w = synthetic.small_case(nlat=12, nlon=24, nz=2, k=8, nobs=300, seed=54)
    ctx = letkf.LetkfGPU.from_workload(w, decomp=(2, 2))
    b = _device_case(letkf, torch, w)
    with pytest.raises(letkf.LetkfError) as ei:
        letkf.Batch([ctx], [b[0]], [b[1]], [b[2]], [b[3]], [b[4]])
    assert ei.value.code == letkf.LETKF_ERR_UNSUPPORTED
