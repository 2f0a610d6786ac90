"""GPU parity of the FP64 LETKF against the CPU oracle (through the C-ABI).

Bar: local observation index sets bit-exact; H, analysis mean and
perturbations and the transform matrices within 1e-10 relative (per state
variable: max |gpu - oracle| / max |oracle|), the tolerance of the plain FP64
form.
"""
import ctypes as C
import math

import numpy as np
import pytest

from conftest import GOLDEN_CASES, field_rel_err, golden_case, pkg
from oracle import oracle as O

pytestmark = pytest.mark.gpu
TOL = 1e-10


@pytest.fixture(scope="module")
def letkf():
    pkg("build").build()
    m = pkg("letkf")
    m.load_library()
    return m


@pytest.fixture(scope="module")
def synthetic():
    return pkg("synthetic")


def assert_fields(a, b, w, tol=TOL):
    errs = field_rel_err(a, b, w)
    assert max(errs.values()) <= tol, errs


def compare_lists(ctx, orc):
    off_g, idx_g, rloc_g = ctx.local_obs()
    off_o, idx_o, rloc_o = orc.local_obs()
    assert np.array_equal(off_g, off_o)
    assert np.array_equal(idx_g, idx_o)
    if rloc_o.size:
        # CUDA's and glibc's cos/acos differ by ulps; acos amplifies them near
        # zero distance (the weights themselves are <= 1)
        assert np.max(np.abs(rloc_g - rloc_o)) <= 1e-12
    return off_o


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_golden_cases(letkf, name):
    w, exp = golden_case(name)
    ctx = letkf.LetkfGPU.from_workload(w)
    ctx.keep_trans(True)
    orc = O.Oracle(w)
    yb, dep = ctx.obs_operator(w.xb, w.axb, w.obs)
    yb_o, dep_o = orc.obs_operator()
    assert np.max(np.abs(yb - yb_o)) <= TOL * np.abs(yb_o).max()
    assert np.max(np.abs(dep - dep_o)) <= TOL * np.abs(dep_o).max()
    xa, axa = ctx.run(w.xb, w.axb, w.obs)
    compare_lists(ctx, orc)
    assert np.array_equal(ctx.local_obs()[1], exp["idx"])
    xa_o, axa_o = orc.run()
    assert_fields(axa, axa_o, w)
    assert_fields(xa, xa_o, w)
    tr, _ = ctx.last_trans(np.arange(ctx.ncubes))
    assert np.max(np.abs(tr - exp["trans"])) <= TOL * np.abs(exp["trans"]).max()
    st = ctx.stats()
    assert st["n_borderline"] == 0 and st["n_not_converged"] == 0


def test_config0_full(letkf, synthetic):
    w = synthetic.config(0)
    orc = O.Oracle(w)
    ctx = letkf.LetkfGPU.from_workload(w)
    xa, axa = ctx.run(w.xb, w.axb, w.obs)
    compare_lists(ctx, orc)
    xa_o, axa_o = orc.run()
    assert_fields(axa, axa_o, w)
    assert_fields(xa, xa_o, w)
    st = ctx.stats()
    assert st["n_borderline"] == 0 and st["n_not_converged"] == 0


def test_config1_sampled_columns_and_invariants(letkf, synthetic):
    w = synthetic.config(1)
    ctx = letkf.LetkfGPU.from_workload(w)
    xa, axa = ctx.run(w.xb, w.axb, w.obs)
    st = ctx.stats()
    assert st["n_borderline"] == 0 and st["n_not_converged"] == 0
    assert 0 < st["max_p"] <= 10000
    # size-independent properties over every column
    assert np.isfinite(xa).all() and np.isfinite(axa).all()
    scale = np.abs(w.xb).max(axis=2, keepdims=True)
    assert np.max(np.abs(xa.mean(axis=2, keepdims=True)) / np.maximum(scale, 1e-300)) <= 1e-12
    # sampled columns against the oracle
    rng = np.random.default_rng(1)
    cubes = np.sort(rng.choice(ctx.ncubes, 300, replace=False))
    orc = O.Oracle(w)
    off_g, idx_g, _ = ctx.local_obs()
    for c in cubes[:60]:
        j, i = c % w.nlat, c // w.nlat
        n = O.lib().orc_local_obs_point(C.byref(orc.cfg), C.byref(orc.obs), C.c_double(float(w.glat[j])),
                                        C.c_double(float(w.glon[i])), None, None)
        ib = np.empty(max(n, 1), np.int32)
        O.lib().orc_local_obs_point(C.byref(orc.cfg), C.byref(orc.obs), C.c_double(float(w.glat[j])),
                                    C.c_double(float(w.glon[i])),
                                    ib.ctypes.data_as(C.POINTER(C.c_int32)), None)
        assert np.array_equal(idx_g[off_g[c]:off_g[c + 1]], ib[:n]), c
    xa_o, axa_o = orc.run_cubes(cubes)
    assert_fields(axa[cubes], axa_o[cubes], w)
    assert_fields(xa[cubes], xa_o[cubes], w)


@pytest.mark.parametrize("k", [8, 16, 32, 48, 64, 96, 128])
def test_ensemble_sizes(letkf, synthetic, k):
    w = synthetic.small_case(nlat=10, nlon=20, nz=3, k=k, nobs=400, loc_dist_km=1000.0, seed=k)
    ctx = letkf.LetkfGPU.from_workload(w)
    xa, axa = ctx.run(w.xb, w.axb, w.obs)
    orc = O.Oracle(w)
    compare_lists(ctx, orc)
    xa_o, axa_o = orc.run()
    assert_fields(axa, axa_o, w)
    assert_fields(xa, xa_o, w)


def test_log_pressure_observation_operator(letkf, synthetic):
    w = synthetic.small_case(nlat=12, nlon=24, nz=8, k=16, nobs=500, loc_dist_km=900.0, seed=21,
                             h_mode=0)
    # pressures above the model top and below the surface exercise the clamps
    w.obs["ph"][:20] = 50.0
    w.obs["ph"][20:40] = 2.0e5
    ctx = letkf.LetkfGPU.from_workload(w)
    yb, dep = ctx.obs_operator(w.xb, w.axb, w.obs)
    orc = O.Oracle(w)
    yb_o, dep_o = orc.obs_operator()
    assert np.max(np.abs(yb - yb_o)) <= TOL * np.abs(yb_o).max()
    assert np.max(np.abs(dep - dep_o)) <= TOL * np.abs(dep_o).max()
    xa, axa = ctx.run(w.xb, w.axb, w.obs)
    xa_o, axa_o = orc.run()
    assert_fields(xa, xa_o, w)


def test_no_observations_is_pure_inflation(letkf, synthetic):
    w = synthetic.small_case(nlat=8, nlon=16, nz=2, k=8, nobs=10, seed=2)
    w.obs = {key: v[:0] for key, v in w.obs.items()}
    ctx = letkf.LetkfGPU.from_workload(w)
    xa, axa = ctx.run(w.xb, w.axb, w.obs)
    assert np.max(np.abs(axa - w.axb)) <= 1e-12 * np.abs(w.axb).max()
    assert np.max(np.abs(xa - math.sqrt(w.inflation) * w.xb)) <= 1e-12 * np.abs(w.xb).max()


def test_special_positions_and_collisions(letkf, synthetic):
    w = synthetic.small_case(nlat=12, nlon=24, nz=2, k=8, nobs=300, loc_dist_km=800.0, seed=9)
    lat = [float(w.glat[0]), 90.0, -90.0, 0.0, 37.5, 37.5, float(w.glat[5]), -float(w.glat[3]), 89.99]
    lon = [float(w.glon[0]), 10.0, 200.0, 360.0, 0.0, 0.0, float(w.glon[7]), float(w.glon[4]) + 180.0, 359.99]
    m = len(lat)
    for key, val in (("lat", lat), ("lon", lon)):
        w.obs[key] = np.concatenate([w.obs[key], val])
    for key, fill in (("ph", 5e4), ("lev", 1), ("var", 1), ("yo", 3.0), ("rinv", 0.25)):
        w.obs[key] = np.concatenate([w.obs[key], np.full(m, fill, dtype=w.obs[key].dtype)])
    ctx = letkf.LetkfGPU.from_workload(w)
    xa, axa = ctx.run(w.xb, w.axb, w.obs)
    orc = O.Oracle(w)
    compare_lists(ctx, orc)
    xa_o, axa_o = orc.run()
    assert_fields(xa, xa_o, w)
    assert_fields(axa, axa_o, w)


def test_boxcar_polar_discard_and_cubes(letkf, synthetic):
    w = synthetic.small_case(nlat=11, nlon=22, nz=2, k=16, nobs=500, loc_dist_km=700.0, seed=4)
    w.gc_filter = 0
    w.obs_polar = 70.0
    for cube_n in (1, 2, 3):
        ctx = letkf.LetkfGPU.from_workload(w, cube_n=cube_n)
        xa, axa = ctx.run(w.xb, w.axb, w.obs)
        orc = O.Oracle(w, cube_n=cube_n)
        compare_lists(ctx, orc)
        xa_o, axa_o = orc.run()
        assert_fields(xa, xa_o, w)
        assert_fields(axa, axa_o, w)


def test_truncation_with_dense_clusters(letkf, synthetic):
    w = synthetic.generate("dense", 4.0, 2, 16, 6000, 900.0, 1.1, 77,
                           boxes=((10.0, 30.0, 0.0, 20.0),), box_factor=40.0, lmax_noise=6)
    w.max_obs = 300
    ctx = letkf.LetkfGPU.from_workload(w)
    xa, axa = ctx.run(w.xb, w.axb, w.obs)
    orc = O.Oracle(w)
    compare_lists(ctx, orc)
    assert ctx.stats()["n_truncated"] > 0
    xa_o, axa_o = orc.run()
    assert_fields(xa, xa_o, w)


def test_overflow_selection_beyond_shared_memory(letkf, synthetic):
    # more kept obs than the search holds in shared memory (16384 for max_obs
    # 10000) takes the threshold-search path
    w = synthetic.generate("overflow", 6.0, 1, 8, 30000, 1500.0, 1.1, 5,
                           boxes=((0.0, 20.0, -10.0, 10.0),), box_factor=200.0, lmax_noise=5)
    ctx = letkf.LetkfGPU.from_workload(w)
    xa, axa = ctx.run(w.xb, w.axb, w.obs)
    st = ctx.stats()
    assert st["n_truncated"] > 0
    orc = O.Oracle(w)
    compare_lists(ctx, orc)
    xa_o, axa_o = orc.run()
    assert_fields(xa, xa_o, w)


@pytest.mark.parametrize("loc_km", [300.0, 1500.0])
def test_search_without_the_bitmap(letkf, synthetic, loc_km):
    # more than 786,432 obs: the search keeps its candidates in a sorted key
    # buffer instead of an index bitmap; at 1500 km more obs are kept than that
    # buffer holds (threshold-search path)
    w = synthetic.generate("manyobs", 7.5, 1, 4, 800_000, loc_km, 1.1, 9, lmax_noise=4)
    ctx = letkf.LetkfGPU.from_workload(w)
    xa, axa = ctx.run(w.xb, w.axb, w.obs)
    orc = O.Oracle(w)
    compare_lists(ctx, orc)
    if loc_km > 1000.0:
        assert ctx.stats()["n_truncated"] > 0
    else:
        xa_o, axa_o = orc.run()
        assert_fields(xa, xa_o, w)



def test_search_threshold_inside_a_histogram_bin(letkf, synthetic):
    # more than 786,432 obs, indexed by distance from one column (after 100
    # far ones): that column's kept indices fill whole bins of the search's
    # index histogram, so the bin holding its max_obs-th kept index runs past
    # the key buffer (2048 keys for max_obs 2000) and the threshold search
    # inside that bin is taken; other columns take the plain histogram path
    w = synthetic.generate("binfill", 7.5, 1, 4, 800_000, 1500.0, 1.1, 10, lmax_noise=4)
    lat0, lon0 = np.deg2rad(float(w.glat[10])), np.deg2rad(float(w.glon[20]))
    la, lo = np.deg2rad(w.obs["lat"]), np.deg2rad(w.obs["lon"])
    cosd = np.sin(la) * np.sin(lat0) + np.cos(la) * np.cos(lat0) * np.cos(lo - lon0)
    by_dist = np.argsort(-cosd, kind="stable")
    order = np.concatenate([by_dist[-100:], by_dist[:-100]])
    for key in w.obs:
        w.obs[key] = np.ascontiguousarray(w.obs[key][order])
    w.max_obs = 2000
    ctx = letkf.LetkfGPU.from_workload(w)
    ctx.run(w.xb, w.axb, w.obs)
    assert ctx.stats()["n_truncated"] > 0
    compare_lists(ctx, O.Oracle(w))

def test_bad_observation_is_rejected(letkf, synthetic):
    w = synthetic.small_case(nlat=8, nlon=16, nz=2, k=8, nobs=50, seed=3)
    w.obs["lat"] = w.obs["lat"].copy()
    w.obs["lat"][7] = 95.0
    ctx = letkf.LetkfGPU.from_workload(w)
    with pytest.raises(letkf.LetkfError) as ei:
        ctx.run(w.xb, w.axb, w.obs)
    assert ei.value.code == letkf.LETKF_ERR_INVALID
    w.obs["lat"][7] = 10.0
    w.obs["lev"] = w.obs["lev"].copy()
    w.obs["lev"][w.obs["var"] > 0][:1] = 0
    bad = np.nonzero(w.obs["var"] > 0)[0][0]
    w.obs["lev"][bad] = 99
    with pytest.raises(letkf.LetkfError):
        ctx.run(w.xb, w.axb, w.obs)


def test_runs_are_bitwise_deterministic(letkf, synthetic):
    w = synthetic.small_case(nlat=16, nlon=32, nz=3, k=32, nobs=2000, loc_dist_km=900.0, seed=8)
    ctx = letkf.LetkfGPU.from_workload(w)
    a1, m1 = ctx.run(w.xb, w.axb, w.obs)
    a2, m2 = ctx.run(w.xb, w.axb, w.obs)
    assert np.array_equal(a1, a2) and np.array_equal(m1, m2)


def test_core_batch_matches_letkf_core(letkf, synthetic):
    rng = np.random.default_rng(3)
    k = 32
    sizes = [0, 1, 7, 64, 300, 1200]
    offs = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    p = offs[-1]
    hx = rng.standard_normal((p, k))
    hx -= hx.mean(axis=1, keepdims=True)
    rdi = (1.0 / rng.uniform(0.5, 2.0, p) ** 2).astype(np.float32)
    dep = rng.standard_normal(p)
    rloc = rng.uniform(0.0, 1.0, p)
    w = synthetic.small_case(nlat=8, nlon=16, nz=1, k=k, nobs=10)
    ctx = letkf.LetkfGPU.from_workload(w)
    tr, wb = ctx.core_batch(offs, hx, rdi, dep, rloc)
    for b in range(len(sizes)):
        s = slice(offs[b], offs[b + 1])
        t_o, w_o = O.letkf_core(hx[s], rdi[s], dep[s], rloc[s], w.inflation)
        assert np.max(np.abs(tr[b] - t_o)) <= TOL * np.abs(t_o).max()
        assert np.max(np.abs(wb[b] - w_o)) <= TOL * max(np.abs(w_o).max(), 1e-12)


def test_fortran_shim_with_halo(letkf, synthetic):
    w = synthetic.small_case(nlat=8, nlon=16, nz=2, k=8, nobs=200, loc_dist_km=900.0, seed=6)
    L = letkf.load_library()
    i = lambda v: C.byref(C.c_int(v))
    d = lambda v: C.byref(C.c_double(v))
    ierr = C.c_int(1)
    L.letkf_init_gpu_(i(w.nlat), i(w.nlon), i(w.nz), i(1), i(3), i(w.k),
                      w.glat.ctypes.data_as(C.c_void_p), w.glon.ctypes.data_as(C.c_void_p),
                      w.hyai.ctypes.data_as(C.c_void_p), w.hybi.ctypes.data_as(C.c_void_p),
                      d(w.p0), d(w.ptop), i(1), d(w.loc_dist_km), d(-999.0), d(w.inflation),
                      d(91.0), i(1), i(1), i(1), i(1), i(0), i(1), i(0), C.byref(ierr))
    assert ierr.value == 0
    o = {key: np.ascontiguousarray(v) for key, v in w.obs.items()}
    var1 = (o["var"] + 1).astype(np.int32)
    lev = o["lev"].astype(np.int32)
    L.letkf_set_obs_gpu_(C.byref(C.c_int64(o["lat"].size)), o["lat"].ctypes.data_as(C.c_void_p),
                         o["lon"].ctypes.data_as(C.c_void_p), o["ph"].ctypes.data_as(C.c_void_p),
                         lev.ctypes.data_as(C.c_void_p), var1.ctypes.data_as(C.c_void_p),
                         o["yo"].ctypes.data_as(C.c_void_p), o["rinv"].ctypes.data_as(C.c_void_p),
                         C.byref(ierr))
    assert ierr.value == 0
    h = 1
    n, k = w.n, w.k
    xb_h = np.full((w.nlon + 2 * h, w.nlat + 2 * h, n, k), np.nan)
    axb_h = np.full((w.nlon + 2 * h, w.nlat + 2 * h, n), np.nan)
    xb_h[h:-h, h:-h] = w.xb.reshape(w.nlon, w.nlat, n, k)
    axb_h[h:-h, h:-h] = w.axb.reshape(w.nlon, w.nlat, n)
    xa_h = np.zeros_like(xb_h)
    axa_h = np.zeros_like(axb_h)
    L.letkf_run_gpu_(i(0), i(h), xb_h.ctypes.data_as(C.c_void_p), axb_h.ctypes.data_as(C.c_void_p),
                     xa_h.ctypes.data_as(C.c_void_p), axa_h.ctypes.data_as(C.c_void_p), C.byref(ierr))
    assert ierr.value == 0
    L.letkf_final_gpu_(C.byref(ierr))
    xa_o, axa_o = O.Oracle(w).run()
    assert_fields(xa_h[h:-h, h:-h].reshape(-1, n, k), xa_o, w)
    assert_fields(axa_h[h:-h, h:-h].reshape(-1, n), axa_o, w)
    assert np.all(xa_h[0] == 0)            # halo untouched
