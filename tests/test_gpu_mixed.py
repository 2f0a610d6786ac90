"""Mixed-precision form against the FP64 oracle and the FP64 GPU form.

The form (LETKF_PREC_MIXED): FP16 hi/lo tensor-core products for the
off-diagonal of A (summed in groups of chunks, the groups added in FP32
round to nearest), g and the diagonal of A on the FP32 pipe, BF16 hi/lo
products for the update, an FP32 Jacobi eigensolve and FP32 T, w-bar solved
in FP32 with one FP64-residual refinement step, and the mean increment in
FP64.

Bar: relative error of the analysis mean and of the analysis spread of every
state variable (ps, u, v, T) within 1e-4 of the FP64 result; local observation
sets identical (the search is shared with the FP64 form).
"""
import numpy as np
import pytest

from conftest import increment_errors, mean_spread_errors, pkg
from oracle import oracle as O

pytestmark = pytest.mark.gpu
TOL_MIXED = 1e-4


@pytest.fixture(scope="module")
def letkf():
    pkg("build").build()
    m = pkg("letkf")
    m.load_library()
    return m


@pytest.fixture(scope="module")
def synthetic():
    return pkg("synthetic")


def assert_mixed(xa, axa, xa_ref, axa_ref, w):
    errs = mean_spread_errors(xa, axa, xa_ref, axa_ref, w)
    worst = max(max(v.values()) for v in errs.values())
    assert worst <= TOL_MIXED, errs
    return errs


@pytest.mark.parametrize("k", [32, 48, 64, 96, 128])
def test_mixed_small_cases_vs_oracle(letkf, synthetic, k):
    w = synthetic.small_case(nlat=12, nlon=24, nz=4, k=k, nobs=900, loc_dist_km=900.0, seed=100 + k)
    ctx = letkf.LetkfGPU.from_workload(w, precision=letkf.LETKF_PREC_MIXED)
    xa, axa = ctx.run(w.xb, w.axb, w.obs)
    orc = O.Oracle(w)
    off_g, idx_g, _ = ctx.local_obs()
    off_o, idx_o, _ = orc.local_obs()
    assert np.array_equal(off_g, off_o) and np.array_equal(idx_g, idx_o)
    xa_o, axa_o = orc.run()
    assert_mixed(xa, axa, xa_o, axa_o, w)
    assert np.isfinite(xa).all()


def test_mixed_no_observations(letkf, synthetic):
    w = synthetic.small_case(nlat=8, nlon=16, nz=2, k=32, nobs=10, seed=2)
    w.obs = {key: v[:0] for key, v in w.obs.items()}
    ctx = letkf.LetkfGPU.from_workload(w, precision=letkf.LETKF_PREC_MIXED)
    xa, axa = ctx.run(w.xb, w.axb, w.obs)
    assert np.max(np.abs(axa - w.axb)) <= 1e-6 * np.abs(w.axb).max()
    assert np.max(np.abs(xa - np.sqrt(w.inflation) * w.xb)) <= 1e-4 * np.abs(w.xb).max()


@pytest.mark.parametrize("k", [64, 96, 128])
def test_mixed_transforms_close_to_fp64(letkf, synthetic, k):
    w = synthetic.small_case(nlat=10, nlon=20, nz=3, k=k, nobs=1500, loc_dist_km=1000.0, seed=31)
    fp = letkf.LetkfGPU.from_workload(w)
    mx = letkf.LetkfGPU.from_workload(w, precision=letkf.LETKF_PREC_MIXED)
    fp.keep_trans(True)
    mx.keep_trans(True)
    fp.run(w.xb, w.axb, w.obs)
    mx.run(w.xb, w.axb, w.obs)
    cubes = np.arange(fp.ncubes)
    t64, w64 = fp.last_trans(cubes)
    t16, w16 = mx.last_trans(cubes)
    assert np.max(np.abs(t16 - t64)) <= 1e-4 * np.abs(t64).max()
    assert np.max(np.abs(w16 - w64)) <= 1e-3 * np.abs(w64).max()


def test_mixed_wide_ensemble_vs_fp64(letkf, synthetic):
    # k = 96 (two accumulators, two member tiles) on a 2-degree grid with
    # clustered obs, warm starts along every chunk
    w = synthetic.generate("k96", 2.0, 8, 96, 60_000, 500.0, 1.08, 96,
                           boxes=((0.0, 60.0, -10.0, 30.0),), box_factor=4.0)
    fp = letkf.LetkfGPU.from_workload(w)
    mx = letkf.LetkfGPU.from_workload(w, precision=letkf.LETKF_PREC_MIXED)
    xa64, axa64 = fp.run(w.xb, w.axb, w.obs)
    xa16, axa16 = mx.run(w.xb, w.axb, w.obs)
    assert_mixed(xa16, axa16, xa64, axa64, w)
    st = mx.stats()
    assert st["n_not_converged"] == 0 and st["max_p"] > 1000


def _wbar_error_by_p(letkf, w):
    out = {}
    for nm, prec in (("fp64", letkf.LETKF_PREC_FP64), ("mixed", letkf.LETKF_PREC_MIXED)):
        c = letkf.LetkfGPU.from_workload(w, precision=prec)
        c.keep_trans(True)
        c.run(w.xb, w.axb, w.obs)
        out[nm] = c.last_trans(np.arange(c.ncubes))[1]
        off = c.local_obs()[0]
        c.close()
    w64, w16 = out["fp64"], out["mixed"]
    rel = np.abs(w16 - w64).max(1) / np.maximum(np.abs(w64).max(1), 1e-300)
    return rel, np.diff(off)


@pytest.mark.parametrize("k", [64, 128])
def test_mixed_wbar_error_does_not_grow_with_p(letkf, synthetic, k):
    # w-bar = A'^-1 g inherits the relative error of A and g, times the
    # conditioning.  Summed by the tensor cores alone over thousands of
    # observations, A and g drift (k = 64: w-bar errors of 1.3e-5 median at
    # p >= 1000 against 1e-6 at p < 300); with g and diag(A) on the FP32 pipe
    # and the tensor-core sums added to the running ones every 16 chunks,
    # k = 64 stays near the small-p level.  At k = 128, A' is worse
    # conditioned as p grows, so the error still grows with p (measured:
    # median 9.4e-6 at p in [1000, 2000), 3.0e-5 at p >= 2000).
    if k == 64:
        w = synthetic.config(1, res_deg=2.0, nobs=50_000)
        bounds = {(1000, 10**9): (5e-6, 1.2e-5)}
    else:
        w = synthetic.generate("k128p", 3.0, 4, 128, 120_000, 400.0, 1.05, 128,
                               boxes=((0.0, 60.0, -10.0, 30.0),), box_factor=4.0)
        bounds = {(1000, 2000): (1.5e-5, 4e-5), (2000, 10**9): (5e-5, 2.5e-4)}
    rel, p = _wbar_error_by_p(letkf, w)
    for (lo, hi), (med, mx) in bounds.items():
        sel = (p >= lo) & (p < hi)
        assert sel.sum() >= 100, (lo, hi, sel.sum())
        print(f"k={k}: w-bar rel error, p in [{lo}, {hi}): median {np.median(rel[sel]):.2e} "
              f"max {rel[sel].max():.2e}; p < 300: median {np.median(rel[p < 300]):.2e}")
        assert np.median(rel[sel]) <= med
        assert rel[sel].max() <= mx


def test_mixed_config0_vs_oracle(letkf, synthetic):
    w = synthetic.config(0)
    ctx = letkf.LetkfGPU.from_workload(w, precision=letkf.LETKF_PREC_MIXED)
    xa, axa = ctx.run(w.xb, w.axb, w.obs)
    xa_o, axa_o = O.Oracle(w).run()
    assert_mixed(xa, axa, xa_o, axa_o, w)


def test_mixed_config1_vs_fp64(letkf, synthetic):
    w = synthetic.config(1)
    fp = letkf.LetkfGPU.from_workload(w)
    mx = letkf.LetkfGPU.from_workload(w, precision=letkf.LETKF_PREC_MIXED)
    xa64, axa64 = fp.run(w.xb, w.axb, w.obs)
    xa16, axa16 = mx.run(w.xb, w.axb, w.obs)
    errs = assert_mixed(xa16, axa16, xa64, axa64, w)
    st = mx.stats()
    assert st["n_borderline"] == 0
    # A' stays well conditioned at this size (lambda_max / lambda_min < 1e4)
    assert st["n_ill_conditioned"] == 0 and st["n_not_converged"] == 0
    # on the scale of the increment too (9e-6 measured; 6.4e-5 when A's sums
    # were left to the tensor cores' accumulation)
    inc = increment_errors(xa16, axa16, xa64, axa64, w.xb, w.axb, w)
    assert max(max(v.values()) for v in inc.values()) <= 3e-5, inc
    print("config1 mixed vs fp64:", errs, "increment scale:", inc)


@pytest.mark.parametrize("k", [32, 64, 128])
def test_mixed_wait_timeout_leaves_context_usable(letkf, synthetic, k):
    # Every bounded wait of the mixed cores on their own tensor-core products
    # gives up at once (0 polls): the run reports LETKF_ERR_TIMEOUT, each CTA
    # lets its committed products finish before it frees its tensor memory,
    # and the next run on the same context with the default limit is bitwise
    # the run of a fresh context.  Covers the single-launch core (k = 32), the
    # staged k = 64 core and the wide core (k = 128).
    w = synthetic.small_case(nlat=10, nlon=20, nz=3, k=k, nobs=1200, loc_dist_km=900.0, seed=70 + k)
    ref = letkf.LetkfGPU.from_workload(w, precision=letkf.LETKF_PREC_MIXED)
    xa_ref, axa_ref = ref.run(w.xb, w.axb, w.obs)
    ref.close()
    ctx = letkf.LetkfGPU.from_workload(w, precision=letkf.LETKF_PREC_MIXED)
    ctx.set_wait_limit(0)
    with pytest.raises(letkf.LetkfError) as ei:
        ctx.run(w.xb, w.axb, w.obs)
    assert ei.value.code == letkf.LETKF_ERR_TIMEOUT
    ctx.set_wait_limit(-1)
    xa, axa = ctx.run(w.xb, w.axb, w.obs)
    assert np.array_equal(xa, xa_ref) and np.array_equal(axa, axa_ref)
    ctx.close()


def test_f64eig_small_case_vs_oracle(letkf, synthetic):
    # LETKF_PREC_MIXED_F64EIG: the FP32 Jacobi eigenpairs refined to FP64 (one
    # Ogita-Aishima step), FP64 T and wbar, on a small k = 64 case
    w = synthetic.small_case(nlat=12, nlon=24, nz=4, k=64, nobs=900, loc_dist_km=900.0, seed=164)
    ctx = letkf.LetkfGPU.from_workload(w, precision=letkf.LETKF_PREC_MIXED_F64EIG)
    xa, axa = ctx.run(w.xb, w.axb, w.obs)
    orc = O.Oracle(w)
    off_g, idx_g, _ = ctx.local_obs()
    off_o, idx_o, _ = orc.local_obs()
    assert np.array_equal(off_g, off_o) and np.array_equal(idx_g, idx_o)
    xa_o, axa_o = orc.run()
    assert_mixed(xa, axa, xa_o, axa_o, w)
    st = ctx.stats()
    assert st["precision"] == letkf.LETKF_PREC_MIXED_F64EIG and st["ms_stage"][3] > 0.0


def test_f64eig_transforms_vs_fp64(letkf, synthetic):
    # T and wbar of the F64EIG form against the FP64 form: the remaining
    # difference is the BF16 hi/lo representation of A and g, so both forms
    # meet the same bound, and the F64EIG form's T is no farther from FP64 than
    # the FP32-eigensolve form's by more than FP32 rounding of T
    w = synthetic.small_case(nlat=10, nlon=20, nz=3, k=64, nobs=1500, loc_dist_km=1000.0, seed=31)
    out = {}
    for nm, prec in (("fp64", letkf.LETKF_PREC_FP64), ("mixed", letkf.LETKF_PREC_MIXED),
                     ("f64eig", letkf.LETKF_PREC_MIXED_F64EIG)):
        c = letkf.LetkfGPU.from_workload(w, precision=prec)
        c.keep_trans(True)
        c.run(w.xb, w.axb, w.obs)
        out[nm] = c.last_trans(np.arange(c.ncubes))
        c.close()
    t64, w64 = out["fp64"]
    for nm in ("mixed", "f64eig"):
        t, wv = out[nm]
        assert np.max(np.abs(t - t64)) <= 1e-4 * np.abs(t64).max(), nm
        assert np.max(np.abs(wv - w64)) <= 1e-3 * np.abs(w64).max(), nm
    d_mixed = np.max(np.abs(out["mixed"][0] - t64))
    d_f64 = np.max(np.abs(out["f64eig"][0] - t64))
    assert d_f64 <= 1.1 * d_mixed + 1e-6 * np.abs(t64).max(), (d_f64, d_mixed)


def test_f64eig_config1_vs_fp64(letkf, synthetic):
    w = synthetic.config(1)
    fp = letkf.LetkfGPU.from_workload(w)
    mx = letkf.LetkfGPU.from_workload(w, precision=letkf.LETKF_PREC_MIXED_F64EIG)
    xa64, axa64 = fp.run(w.xb, w.axb, w.obs)
    xa16, axa16 = mx.run(w.xb, w.axb, w.obs)
    errs = assert_mixed(xa16, axa16, xa64, axa64, w)
    assert mx.stats()["n_not_converged"] == 0
    print("config1 mixed (FP64 eigenpairs) vs fp64:", errs)


def test_f64eig_needs_ensemble_64(letkf, synthetic):
    w = synthetic.small_case(nlat=8, nlon=16, nz=2, k=32, nobs=50, seed=3)
    with pytest.raises(letkf.LetkfError) as ei:
        letkf.LetkfGPU.from_workload(w, precision=letkf.LETKF_PREC_MIXED_F64EIG)
    assert ei.value.code == letkf.LETKF_ERR_UNSUPPORTED
