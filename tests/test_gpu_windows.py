"""Cube windows and cube ranges (through the C-ABI).

A list limit smaller than the lists of all cubes makes a run search and
analyse the cubes in consecutive windows; a cube range analyses one block of
cubes, as one DA rank analyses its own sub-domain.  Bar: both reproduce the
whole run bitwise on the cubes they analyse (each cube's analysis depends
only on its own list and its own columns; windows of the mixed form end on
work-queue chunk boundaries, so each cube keeps the eigenvector warm start of
its chunk), leave the other columns alone, and a windowed or range run
reports that it kept no complete lists.  A range that starts or ends inside a
chunk starts that chunk's first cube cold: the mixed form then agrees within
its own bar (1e-4 of the field's magnitude; the two runs differ by their
FP32 eigensolves from different starting points).
"""
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


def _case(k, seed, nobs=1500, nlat=18, nlon=36, nz=3, loc=800.0):
    return pkg("synthetic").small_case(nlat=nlat, nlon=nlon, nz=nz, k=k, nobs=nobs, loc_dist_km=loc,
                                       seed=seed)


def _whole(letkf, w, **kw):
    ctx = letkf.LetkfGPU.from_workload(w, **kw)
    xa, axa = ctx.run(w.xb, w.axb, w.obs)
    return ctx, xa, axa, ctx.stats()


@pytest.mark.parametrize("k,prec,decomp", [(8, "FP64", (0, 0)), (32, "MIXED", (0, 0)),
                                           (64, "MIXED", (0, 0)), (96, "MIXED", (0, 0)),
                                           (16, "FP64", (2, 3))])
def test_windows_match_the_whole_run(letkf, k, prec, decomp):
    w = _case(k, seed=60 + k)
    precision = getattr(letkf, f"LETKF_PREC_{prec}")
    _, xa0, axa0, st0 = _whole(letkf, w, precision=precision, decomp=decomp)
    assert st0["n_windows"] == 1
    ctx = letkf.LetkfGPU.from_workload(w, precision=precision, decomp=decomp)
    ctx.set_list_limit(max(st0["sum_p"] // 7, st0["max_p"]))
    xa, axa = ctx.run(w.xb, w.axb, w.obs)
    st = ctx.stats()
    assert st["n_windows"] >= 7
    assert st["sum_p"] == st0["sum_p"] and st["max_p"] == st0["max_p"]
    assert st["n_truncated"] == st0["n_truncated"]
    assert np.array_equal(xa, xa0) and np.array_equal(axa, axa0)
    with pytest.raises(letkf.LetkfError):
        ctx.local_obs()
    # a limit below the longest list still runs: the pool grows to the
    # heaviest window unit (a cube, or a mixed-form chunk)
    ctx.set_list_limit(1)
    xa1, axa1 = ctx.run(w.xb, w.axb, w.obs)
    assert ctx.stats()["n_windows"] >= 7
    assert np.array_equal(xa1, xa0) and np.array_equal(axa1, axa0)
    # back to the automatic pool: one window, lists kept
    ctx.set_list_limit(0)
    ctx.run(w.xb, w.axb, w.obs)
    assert ctx.stats()["n_windows"] == 1
    off, idx, _ = ctx.local_obs()
    assert off[-1] == st0["sum_p"]


def test_windows_match_the_oracle(letkf):
    w = _case(8, seed=71, nobs=900)
    ctx = letkf.LetkfGPU.from_workload(w)
    ctx.set_list_limit(200)
    xa, axa = ctx.run(w.xb, w.axb, w.obs)
    assert ctx.stats()["n_windows"] > 1
    xa_o, axa_o = O.Oracle(w).run()
    assert np.max(np.abs(axa - axa_o)) <= 1e-10 * max(1.0, np.max(np.abs(axa_o)))
    assert np.max(np.abs(xa - xa_o)) <= 1e-10 * max(1.0, np.max(np.abs(xa_o)))


def _same(prec, a, b):
    if prec == "FP64":
        assert np.array_equal(a, b)
    else:
        assert np.max(np.abs(a - b)) <= 1e-4 * np.max(np.abs(b))


@pytest.mark.parametrize("k,prec", [(16, "FP64"), (64, "MIXED")])
def test_cube_range_is_a_sub_domain(letkf, k, prec):
    w = _case(k, seed=80 + k)
    precision = getattr(letkf, f"LETKF_PREC_{prec}")
    _, xa0, axa0, st0 = _whole(letkf, w, precision=precision)
    ctx = letkf.LetkfGPU.from_workload(w, precision=precision)
    first, count = 5 * w.nlat + 3, 4 * w.nlat + 7
    ctx.set_cube_range(first, count)
    xa = np.full_like(xa0, np.nan)
    axa = np.full_like(axa0, np.nan)
    ctx.run(w.xb, w.axb, w.obs, xa, axa)
    assert ctx.stats()["ncubes"] == count
    sl = slice(first, first + count)
    _same(prec, xa[sl], xa0[sl])
    _same(prec, axa[sl], axa0[sl])
    assert np.isnan(xa[:first]).all() and np.isnan(xa[first + count:]).all()
    assert np.isnan(axa[:first]).all() and np.isnan(axa[first + count:]).all()
    with pytest.raises(letkf.LetkfError):
        ctx.local_obs()
    # a range and windows together (windows never cut a chunk)
    ctx.set_list_limit(max(st0["max_p"], 1))
    xa2 = np.full_like(xa0, np.nan)
    axa2 = np.full_like(axa0, np.nan)
    ctx.run(w.xb, w.axb, w.obs, xa2, axa2)
    assert ctx.stats()["n_windows"] > 1
    assert np.array_equal(xa2[sl], xa[sl]) and np.array_equal(axa2[sl], axa[sl])
    assert np.isnan(xa2[first + count:]).all()
    # the whole grid again
    ctx.set_cube_range(0, -1)
    ctx.set_list_limit(0)
    xa3, axa3 = ctx.run(w.xb, w.axb, w.obs)
    assert np.array_equal(xa3, xa0) and np.array_equal(axa3, axa0)


def test_cube_range_with_cubes_of_several_columns(letkf):
    w = _case(8, seed=91, nlat=12, nlon=24)
    _, xa0, axa0, _ = _whole(letkf, w, cube_n=2)
    ctx = letkf.LetkfGPU.from_workload(w, cube_n=2)
    nbj = 6
    with pytest.raises(letkf.LetkfError):
        ctx.set_cube_range(3, nbj)
    with pytest.raises(letkf.LetkfError):
        ctx.set_cube_range(nbj, nbj + 1)
    with pytest.raises(letkf.LetkfError):
        ctx.set_cube_range(0, 10 ** 6)
    ctx.set_cube_range(2 * nbj, 3 * nbj)
    xa = np.full_like(xa0, np.nan)
    axa = np.full_like(axa0, np.nan)
    ctx.run(w.xb, w.axb, w.obs, xa, axa)
    cols = slice(2 * 2 * w.nlat, 5 * 2 * w.nlat)   # lon strips 2..4 of two columns each
    assert np.array_equal(xa[cols], xa0[cols]) and np.array_equal(axa[cols], axa0[cols])
    assert np.isnan(xa[:cols.start]).all() and np.isnan(xa[cols.stop:]).all()


def test_host_run_in_blocks_matches_the_device_run(letkf):
    """A run with host buffers analyses the k = 64 mixed core in blocks of
    cubes (up to three) and copies each block out while the next runs; the
    blocks end on multiples of the work-queue chunk and of the eigensolve run,
    so the analysis is bitwise the one of a run on device buffers (one block)."""
    torch = pytest.importorskip("torch")
    w = pkg("synthetic").small_case(nlat=90, nlon=180, nz=3, k=64, nobs=8000, loc_dist_km=600.0, seed=71)
    ctx = letkf.LetkfGPU.from_workload(w, precision=letkf.LETKF_PREC_MIXED)
    assert ctx.ncubes > 2 * 4096                     # at least two blocks of a host run
    xa_h, axa_h = ctx.run(w.xb, w.axb, w.obs)
    dev = torch.device("cuda", 0)
    xb, axb = torch.from_numpy(w.xb).to(dev), torch.from_numpy(w.axb).to(dev)
    obs = letkf.ObsArrays({k: torch.from_numpy(np.ascontiguousarray(w.obs[k])).to(dev)
                           for k in ("lat", "lon", "ph", "lev", "var", "yo", "rinv")}, device=True)
    xa, axa = torch.empty_like(xb), torch.empty_like(axb)
    ctx.run_device(xb, axb, obs, xa, axa)
    torch.cuda.synchronize()
    assert np.array_equal(xa.cpu().numpy(), xa_h)
    assert np.array_equal(axa.cpu().numpy(), axa_h)
    # and again with host buffers (the copy streams are reused)
    xa2, axa2 = ctx.run(w.xb, w.axb, w.obs)
    assert np.array_equal(xa2, xa_h) and np.array_equal(axa2, axa_h)
    ctx.close()


@pytest.mark.parametrize("k,prec,decomp,windows", [(64, "MIXED", (0, 0), False), (64, "MIXED", (0, 0), True),
                                                   (32, "MIXED", (2, 3), True), (96, "MIXED", (0, 0), False),
                                                   (16, "FP64", (0, 0), True)])
def test_host_run_equals_device_run(letkf, k, prec, decomp, windows):
    """With host buffers the search runs while the state copies in (H's
    member pass after it; the mixed form completes its list entries' second
    factor then), and the analysis is copied out in blocks: bitwise the run on
    device buffers, also in cube windows and with the decomposed sets."""
    torch = pytest.importorskip("torch")
    w = _case(k, seed=90 + k)
    precision = getattr(letkf, f"LETKF_PREC_{prec}")
    ctx = letkf.LetkfGPU.from_workload(w, precision=precision, decomp=decomp)
    if windows:
        xa0, axa0 = ctx.run(w.xb, w.axb, w.obs)
        st0 = ctx.stats()
        ctx.set_list_limit(max(st0["sum_p"] // 5, st0["max_p"]))
    xa_h, axa_h = ctx.run(w.xb, w.axb, w.obs)
    if windows:
        assert ctx.stats()["n_windows"] >= 3
    dev = torch.device("cuda", 0)
    xb, axb = torch.from_numpy(w.xb).to(dev), torch.from_numpy(w.axb).to(dev)
    obs = letkf.ObsArrays({key: torch.from_numpy(np.ascontiguousarray(w.obs[key])).to(dev)
                           for key in ("lat", "lon", "ph", "lev", "var", "yo", "rinv")}, device=True)
    xa, axa = torch.empty_like(xb), torch.empty_like(axb)
    ctx.run_device(xb, axb, obs, xa, axa)
    torch.cuda.synchronize()
    assert np.array_equal(xa.cpu().numpy(), xa_h)
    assert np.array_equal(axa.cpu().numpy(), axa_h)
    if windows:
        assert np.array_equal(xa_h, xa0) and np.array_equal(axa_h, axa0)
    ctx.close()
