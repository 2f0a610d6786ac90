"""The CPU oracle against known answers, LAPACK and the golden fixtures.

The reference ships no LETKF tests or golden vectors and cannot be built here,
so the oracle is pinned by (i) closed-form known answers, (ii) an
independent numpy/LAPACK restatement (tests/golden/make_golden.py, whose
outputs are the committed fixtures) and (iii) brute-force scans.
"""
import math

import numpy as np
import pytest
import scipy.linalg as sl

from conftest import GOLDEN_CASES, field_rel_err, golden_case, pkg
from oracle import oracle as O



def _golden_module():
    import importlib.util
    import os
    here = os.path.dirname(os.path.abspath(__file__))
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(here, "golden", "make_golden.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


MG = _golden_module()


# ---- KAT-4: Gaspari-Cohn with the reference's float-rounded literals ------------
def test_schr2_known_values():
    assert O.schr2(0.0) == 1.0
    assert O.schr2(1.0) == 0.20833301544189453
    assert O.schr2(2.0) == 1.2616316471536493e-06
    assert O.schr2(2.0 + 1e-15) == 0.0
    assert O.schr2(0.5) == 0.6848957538604736
    assert O.schr2(-1.0) == 1.0
    assert O.schr2(float("nan")) == 1.0          # all comparisons false
    assert O.schr(2.0) == 1.0 and O.schr(2.0000001) == 0.0


def test_schr2_matches_numpy_restatement():
    ri = np.concatenate([np.linspace(0, 2.2, 2001), [1.0, 2.0, np.nextafter(2.0, 3.0)]])
    ref = MG.schr2(ri)
    got = np.array([O.schr2(float(r)) for r in ri])
    assert np.array_equal(ref, got)


def test_gc_positive_iff_within_twice_c():
    ri = np.linspace(0.0, 2.0, 20001)
    assert all(O.schr2(float(r)) > 0 for r in ri)
    assert O.schr2(float(np.nextafter(2.0, 3.0))) == 0.0


# ---- distance ---------------------------------------------------------------------
def test_latlon_dist_constants_and_values():
    # the reference's pi is float(pi) and a is float(6371.393)
    a = float(np.float32(6371.393))
    pif = float(np.float32(math.pi))
    d = O.latlon_dist(0.0, 0.0, 0.0, 90.0)
    assert abs(d - a * math.acos(math.cos(90.0 / 180.0 * pif))) < 1e-9
    assert O.latlon_dist(10.0, 20.0, 10.0, 20.0) < 1e-3   # acos rounding near 1
    for (x1, y1, x2, y2) in [(0, 0, 1, 0), (45, 10, 46, 12), (-60, 350, -61, 2), (89.5, 0.5, 89.5, 180.5)]:
        exp = MG.latlon_dist(x1, y1, x2, y2)
        assert abs(O.latlon_dist(x1, y1, x2, y2) - exp) <= 1e-9 * max(1.0, exp)


# ---- eigensolver and core vs LAPACK -------------------------------------------------
@pytest.mark.parametrize("k", [2, 4, 8, 16, 32, 64])
def test_jacobi_vs_lapack(k):
    rng = np.random.default_rng(k)
    y = rng.standard_normal((k, 3 * k))
    a = y @ y.T + 2.0 * np.eye(k)
    lam, v, sweeps = O.jacobi_eig(a)
    assert sweeps > 0
    ref = np.linalg.eigvalsh(a)
    assert np.max(np.abs(lam - ref)) <= 1e-12 * ref.max()
    assert np.max(np.abs(v.T @ v - np.eye(k))) < 1e-13
    assert np.max(np.abs(v @ np.diag(lam) @ v.T - a)) <= 1e-12 * np.abs(a).max()


@pytest.mark.parametrize("k,p", [(4, 0), (4, 1), (8, 5), (16, 3), (16, 200), (32, 64), (64, 300)])
def test_letkf_core_vs_lapack(k, p):
    rng = np.random.default_rng(100 * k + p)
    hx = rng.standard_normal((p, k))
    hx -= hx.mean(axis=1, keepdims=True)
    rdi = (1.0 / rng.uniform(0.5, 2.0, p) ** 2).astype(np.float32)
    dep = rng.standard_normal(p)
    rloc = rng.uniform(0.0, 1.0, p)
    trans, w = O.letkf_core(hx, rdi, dep, rloc, 1.08)
    t_ref, w_ref = MG.letkf_core(hx, rdi, dep, rloc, 1.08)
    assert np.max(np.abs(trans - t_ref)) <= 1e-12 * np.abs(t_ref).max()
    assert np.max(np.abs(w - w_ref)) <= 1e-12 * max(np.abs(w_ref).max(), 1e-300)


# ---- KAT-1: no local observations -------------------------------------------------
def test_kat1_no_obs_is_pure_inflation():
    k, rho = 16, 1.1
    trans, w = O.letkf_core(np.zeros((0, k)), np.zeros(0, np.float32), np.zeros(0), np.zeros(0), rho)
    assert np.allclose(trans, math.sqrt(rho) * np.eye(k), rtol=0, atol=1e-15)
    assert np.all(w == 0.0)


# ---- KAT-2: two members, one observation: closed-form scalar update --------------
def test_kat2_two_members_one_obs():
    a, r, rl, d, rho = 0.7, np.float32(0.8), 0.6, 1.3, 1.05
    hx = np.array([[a, -a]])
    trans, w = O.letkf_core(hx, np.array([r]), np.array([d]), np.array([rl]), rho)
    s2 = float(r) * rl
    c = 1.0 / rho                       # (k-1)/rho with k = 2
    lam2 = c + 2.0 * s2 * a * a
    alpha, beta = math.sqrt(1.0 / c), math.sqrt(1.0 / lam2)
    t_exp = 0.5 * np.array([[alpha + beta, alpha - beta], [alpha - beta, alpha + beta]])
    w_exp = (s2 * d / lam2) * np.array([a, -a])
    assert np.allclose(w, w_exp, rtol=1e-14, atol=1e-15)
    assert np.allclose(trans, t_exp + w_exp[:, None], rtol=1e-14, atol=1e-15)


# ---- KAT-3: textbook ETKF (Hunt et al. 2007, eqs. 20-23) on an analysis -----------
def test_kat3_single_obs_at_grid_point_matches_textbook_etkf():
    synthetic = pkg("synthetic")
    w = synthetic.small_case(nlat=6, nlon=12, nz=2, k=6, nobs=1, loc_dist_km=3000.0, seed=3)
    # one T obs exactly at a grid point: H is the grid value
    j, i, lev = 2, 5, 2
    c = j + w.nlat * i
    row = w.nvar2d + 2 * w.nz + (lev - 1)
    w.obs = dict(lat=np.array([float(w.glat[j])]), lon=np.array([float(w.glon[i])]),
                 ph=np.array([50000.0]), lev=np.array([lev], np.int32), var=np.array([3], np.int32),
                 yo=np.array([w.axb[c, row] + 1.5]), rinv=np.array([1.0]))
    orc = O.Oracle(w)
    xa, axa = orc.run()
    yb = w.xb[c, row, :]                          # obs-space perturbations
    dep = w.obs["yo"][0] - (w.axb[c, row] + yb.sum() / w.k) + 0.0
    k, rho = w.k, w.inflation
    # at the obs column rho_loc = 1 (zero distance)
    Y = yb[None, :]                               # 1 x k
    pa = np.linalg.inv((k - 1) / rho * np.eye(k) + Y.T @ Y)
    W = np.real(sl.sqrtm((k - 1) * pa))
    wbar = pa @ Y.T[:, 0] * dep
    x_exp = w.axb[c][:, None] + w.xb[c] @ (W + wbar[:, None])
    m = x_exp.mean(axis=1)
    assert np.max(np.abs(axa[c] - m)) <= 1e-10 * np.abs(m).max()
    assert np.max(np.abs(xa[c] - (x_exp - m[:, None]))) <= 1e-10 * np.abs(w.xb[c]).max()


# ---- KAT-5: toy sine-wave experiment (unit/main.f90 + toy_model.f90) ---------------
def test_kat5_toy_model_error_decreases():
    synthetic = pkg("synthetic")
    nlat, nlon, k = 18, 36, 16
    glat, glon = synthetic.make_grid(10.0)
    lat, lon = synthetic.grid_points(glat, glon)
    truth = 100 + 100 * np.sin(2 * np.pi * (lat / 360.0 + lon / 2.0 / 180.0))
    phase = 0.3
    members = np.stack([100 + 100 * np.sin(2 * np.pi * (lat / 360.0 + lon / 2.0 / 180.0 + phase * e / k))
                        for e in range(1, k + 1)], axis=1)
    w = synthetic.small_case(nlat=nlat, nlon=nlon, nz=1, k=k, nobs=1, loc_dist_km=1500.0)
    w.nvar3d = 0
    w.nvar2d = 1
    axb = members.mean(axis=1)
    xb = members - axb[:, None]
    rng = np.random.default_rng(0)
    sel = rng.choice(lat.size, 150, replace=False)
    obs = dict(lat=lat[sel], lon=lon[sel], ph=np.full(150, 1e5), lev=np.ones(150, np.int32),
               var=np.zeros(150, np.int32), yo=truth[sel], rinv=np.full(150, 1.0))
    errs = []
    for it in range(4):
        w.xb = xb[:, None, :].copy()
        w.axb = axb[:, None].copy()
        w.obs = obs
        errs.append(np.abs(axb - truth).max())
        xa, axa = O.Oracle(w).run()
        xb, axb = xa[:, 0, :], axa[:, 0]
    errs.append(np.abs(axb - truth).max())
    assert errs[-1] < 0.5 * errs[0]
    assert all(b <= a * 1.001 for a, b in zip(errs, errs[1:]))


# ---- local observation search: prefiltered scan == brute force --------------------
def _brute_force_point(w, clat, clon):
    keep, gcs = [], []
    for o in range(w.obs["lat"].size):
        if not abs(w.obs["lat"][o]) <= w.obs_polar:
            continue
        d = O.latlon_dist(float(w.obs["lat"][o]), float(w.obs["lon"][o]), clat, clon)
        gc = O.schr2(d * 1.0 / w.loc_dist_km)
        if gc > 0:
            keep.append(o)
            gcs.append(gc)
            if len(keep) >= w.max_obs:
                break
    return np.array(keep, dtype=np.int32), np.array(gcs)


def test_local_search_equals_brute_force_scan():
    synthetic = pkg("synthetic")
    w = synthetic.small_case(nlat=12, nlon=24, nz=2, k=4, nobs=600, loc_dist_km=700.0, seed=5)
    # obs on grid points, at the poles, on the date line, at lon 360, duplicated,
    # and exactly antipodal to a cube centre
    extra_lat = [float(w.glat[0]), 90.0, -90.0, 0.0, 37.5, 37.5, -float(w.glat[3])]
    extra_lon = [float(w.glon[0]), 10.0, 200.0, 360.0, 0.0, 0.0, float(w.glon[4]) + 180.0]
    for key, val in (("lat", extra_lat), ("lon", extra_lon)):
        w.obs[key] = np.concatenate([w.obs[key], val])
    n_extra = len(extra_lat)
    for key, fill in (("ph", 5e4), ("lev", 1), ("var", 0), ("yo", 1e5), ("rinv", 1e-4)):
        w.obs[key] = np.concatenate([w.obs[key], np.full(n_extra, fill, dtype=w.obs[key].dtype)])
    w.max_obs = 25
    orc = O.Oracle(w)
    off, idx, rloc = orc.local_obs()
    for cube in range(0, orc.ncubes, 7):
        j, i = cube % w.nlat, cube // w.nlat
        e_idx, e_gc = _brute_force_point(w, float(w.glat[j]), float(w.glon[i]))
        assert np.array_equal(idx[off[cube]:off[cube + 1]], e_idx), cube
        assert np.array_equal(rloc[off[cube]:off[cube + 1]], e_gc), cube


def test_local_obs_cubes_equals_whole_grid_lists():
    # the selected-cubes search (used to check samples of large grids) packs
    # the same lists as the whole-grid search, in the order asked for
    synthetic = pkg("synthetic")
    w = synthetic.small_case(nlat=12, nlon=24, nz=2, k=4, nobs=900, loc_dist_km=800.0, seed=9)
    w.max_obs = 40
    orc = O.Oracle(w)
    off, idx, rloc = orc.local_obs()
    cubes = np.array([5, 0, 287, 5, 131, 17], dtype=np.int64)
    off_s, idx_s, rloc_s = orc.local_obs_cubes(cubes)
    for n, c in enumerate(cubes):
        assert np.array_equal(idx_s[off_s[n]:off_s[n + 1]], idx[off[c]:off[c + 1]])
        assert np.array_equal(rloc_s[off_s[n]:off_s[n + 1]], rloc[off[c]:off[c + 1]])


def test_instance_without_members_keeps_the_draws():
    # members=False draws the same random numbers: same grid, mean and
    # observations as the full instance (configuration 4's recipe on a
    # 2-degree grid with its observation density)
    synthetic = pkg("synthetic")
    full = synthetic.config(4, res_deg=2.0)
    bare = synthetic.config(4, res_deg=2.0, members=False)
    assert bare.xb is None and full.xb is not None
    assert np.array_equal(full.axb, bare.axb)
    for key in full.obs:
        assert np.array_equal(full.obs[key], bare.obs[key]), key


# ---- oracle vs the golden fixtures ---------------------------------------------------
@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_oracle_matches_golden(name):
    w, exp = golden_case(name)
    orc = O.Oracle(w)
    yb, dep = orc.obs_operator()
    assert np.max(np.abs(yb - exp["yb"])) <= 1e-10 * np.abs(exp["yb"]).max()
    assert np.max(np.abs(dep - exp["dep"])) <= 1e-10 * np.abs(exp["dep"]).max()
    off, idx, rloc = orc.local_obs()
    assert np.array_equal(off, exp["off"])
    assert np.array_equal(idx, exp["idx"])
    assert np.max(np.abs(rloc - exp["rloc"])) <= 1e-13    # libm ulps in cos/acos
    xa, axa = orc.run()
    errs = field_rel_err(axa, exp["axa"], w)
    assert max(errs.values()) <= 1e-10, errs
    errs = field_rel_err(xa, exp["xa"], w)
    assert max(errs.values()) <= 1e-10, errs


def test_golden_truncation_case_hits_max_obs():
    w, exp = golden_case("small_k16_trunc")
    counts = np.diff(exp["off"])
    assert counts.max() == w.max_obs and (counts == w.max_obs).sum() > 10
