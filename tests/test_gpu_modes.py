"""The alternate LETKF modes on the GPU against the oracle (through the C-ABI).

Overlapped cubes (letkf_compute and xb_add2_xa, letkf_compute.F90:128-228,
304-354): cubes of cube_n x cube_n columns start every cube_n - overlap grid
points and every column's analysis is the average over the cubes that cover
it.  Vertical localization (letkf_compute_nooverlap_vertical,
letkf_compute.F90:358-526, with gen_yb_dis_vertical and
vertical_localization, letkf_yb.F90:137-243): each block of cube_nz levels
solves its own problem with the weights multiplied by a Gaspari-Cohn (or
box-car) factor of the ln-p distance.  Both run in the FP64 form; the bar is
the FP64 one, 1e-10 relative per state variable.
"""
import numpy as np
import pytest

from conftest import field_rel_err, pkg
from oracle import oracle as O

pytestmark = pytest.mark.gpu

TOL = 1e-10


@pytest.fixture(scope="module")
def letkf():
    pkg("build").build()
    m = pkg("letkf")
    m.load_library()
    return m


def _case(k=8, nz=3, nobs=700, seed=5, loc=900.0, h_mode=1):
    return pkg("synthetic").small_case(nlat=12, nlon=24, nz=nz, k=k, nobs=nobs, loc_dist_km=loc,
                                       seed=seed, h_mode=h_mode)


def _check(xa, axa, xa_o, axa_o, w):
    assert max(field_rel_err(axa, axa_o, w).values()) <= TOL
    assert max(field_rel_err(xa, xa_o, w).values()) <= TOL


@pytest.mark.parametrize("cube_n,overlap,k", [(2, 1, 8), (3, 1, 8), (3, 2, 16), (4, 2, 4), (5, 3, 32)])
def test_overlapped_cubes_match_oracle(letkf, cube_n, overlap, k):
    w = _case(k=k, seed=20 + cube_n + overlap)
    ctx = letkf.LetkfGPU.from_workload(w, cube_n=cube_n, overlap=overlap)
    xa, axa = ctx.run(w.xb, w.axb, w.obs)
    xa_o, axa_o = O.Oracle(w, cube_n=cube_n, overlap=overlap).run()
    _check(xa, axa, xa_o, axa_o, w)
    step = cube_n - overlap
    assert ctx.stats()["ncubes"] == (-(-w.nlat // step)) * (-(-w.nlon // step))
    # the same in cube windows
    ctx.set_list_limit(max(ctx.stats()["sum_p"] // 5, ctx.stats()["max_p"]))
    xa2, axa2 = ctx.run(w.xb, w.axb, w.obs)
    assert ctx.stats()["n_windows"] > 1
    assert np.array_equal(xa2, xa) and np.array_equal(axa2, axa)


@pytest.mark.parametrize("vert_dist,cube_nz,gcv,h_mode,cube_n",
                         [(1.0, 1, 1, 1, 1), (0.3, 1, 1, 1, 1), (0.6, 2, 1, 0, 1), (0.8, 3, 0, 1, 1),
                          (0.5, 4, 1, 1, 2), (2.0, 2, 1, 0, 3)])
def test_vertical_localization_matches_oracle(letkf, vert_dist, cube_nz, gcv, h_mode, cube_n):
    w = _case(k=16, nz=4, seed=30 + cube_nz, h_mode=h_mode)
    ctx = letkf.LetkfGPU.from_workload(w, vert_dist=vert_dist, cube_nz=cube_nz, gc_filter_vertical=gcv,
                                       cube_n=cube_n)
    xa, axa = ctx.run(w.xb, w.axb, w.obs)
    orc = O.Oracle(w, vert_dist=vert_dist, cube_nz=cube_nz, gc_filter_vertical=gcv, cube_n=cube_n)
    xa_o, axa_o = orc.run()
    _check(xa, axa, xa_o, axa_o, w)
    # the horizontal lists are the no-overlap ones
    off_g, idx_g, _ = ctx.local_obs()
    off_o, idx_o, _ = orc.local_obs()
    assert np.array_equal(off_g, off_o) and np.array_equal(idx_g, idx_o)


def test_vertical_localization_differs_from_horizontal(letkf):
    w = _case(k=8, nz=4, seed=41)
    xa_h, axa_h = letkf.LetkfGPU.from_workload(w).run(w.xb, w.axb, w.obs)
    xa_v, axa_v = letkf.LetkfGPU.from_workload(w, vert_dist=0.3).run(w.xb, w.axb, w.obs)
    assert np.abs(axa_v - axa_h).max() > 1e-6 * np.abs(axa_h).max()


def test_alternate_modes_need_the_fp64_form(letkf):
    w = _case(k=32, seed=43)
    for kw in ({"overlap": 1, "cube_n": 2}, {"vert_dist": 0.5}):
        with pytest.raises(letkf.LetkfError) as ei:
            letkf.LetkfGPU.from_workload(w, precision=letkf.LETKF_PREC_MIXED, **kw)
        assert ei.value.code == letkf.LETKF_ERR_UNSUPPORTED
    ctx = letkf.LetkfGPU.from_workload(w, vert_dist=0.5)
    with pytest.raises(letkf.LetkfError):
        ctx.keep_trans(True)
    ctx = letkf.LetkfGPU.from_workload(w, cube_n=2, overlap=1)
    ctx.set_cube_range(0, w.nlat)
    with pytest.raises(letkf.LetkfError):
        ctx.run(w.xb, w.axb, w.obs)
