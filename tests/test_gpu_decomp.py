"""GPU decomposed observation sets against the oracle (through the C-ABI).

A context created with decomp_lat_blocks x decomp_lon_blocks reproduces the
local lists of a DA group of that many MPI ranks (each block's box of obs,
the block neighbour sets, the block-ordered scan, the duplicates of obs on
shared box edges and of the one-rank self wrap).  Bar: local index lists
bit-exact against the oracle's decomposed mode, analyses within 1e-10 (FP64
form) and within the mixed form's 1e-4.
"""
import numpy as np
import pytest

from conftest import field_rel_err, mean_spread_errors, pkg
from oracle import oracle as O
from test_oracle_decomp import _edge_case

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def letkf():
    pkg("build").build()
    m = pkg("letkf")
    m.load_library()
    return m


def _lists_equal(ctx, orc):
    off_g, idx_g, rloc_g = ctx.local_obs()
    off_o, idx_o, rloc_o = orc.local_obs()
    assert np.array_equal(off_g, off_o)
    assert np.array_equal(idx_g, idx_o)
    if rloc_o.size:
        assert np.max(np.abs(rloc_g - rloc_o)) <= 1e-12
    return off_o, idx_o


@pytest.mark.parametrize("dec,max_obs", [((1, 1), 10000), ((1, 1), 60), ((2, 3), 10000),
                                         ((3, 4), 10000), ((4, 8), 10000), ((3, 4), 40)])
def test_decomposed_lists_and_analysis(letkf, dec, max_obs):
    w = _edge_case(max_obs=max_obs)
    ctx = letkf.LetkfGPU.from_workload(w, decomp=dec)
    xa, axa = ctx.run(w.xb, w.axb, w.obs)
    orc = O.Oracle(w, decomp=dec)
    off, idx = _lists_equal(ctx, orc)
    xa_o, axa_o = orc.run()
    assert max(field_rel_err(axa, axa_o, w).values()) <= 1e-10
    assert max(field_rel_err(xa, xa_o, w).values()) <= 1e-10
    if dec == (1, 1) and max_obs == 10000:
        # one rank scans its own box twice
        counts = np.diff(off)
        assert (counts % 2 == 0).all() and counts.max() > 0


def test_decomposed_differs_from_global(letkf):
    w = _edge_case(loc=900.0)
    g = letkf.LetkfGPU.from_workload(w)
    d = letkf.LetkfGPU.from_workload(w, decomp=letkf.decomp_dims(32))
    g.run(w.xb, w.axb, w.obs)
    d.run(w.xb, w.axb, w.obs)
    off_g, idx_g, _ = g.local_obs()
    off_d, idx_d, _ = d.local_obs()
    assert not np.array_equal(off_g, off_d)
    for cube in range(0, w.nlat * w.nlon, 5):
        assert set(idx_d[off_d[cube]:off_d[cube + 1]]) <= set(idx_g[off_g[cube]:off_g[cube + 1]])


def test_decomposed_config0_lists(letkf):
    synthetic = pkg("synthetic")
    w = synthetic.config(0)
    dec = letkf.decomp_dims(12)
    ctx = letkf.LetkfGPU.from_workload(w, decomp=dec)
    ctx.run(w.xb, w.axb, w.obs)
    _lists_equal(ctx, O.Oracle(w, decomp=dec))


def test_decomposed_mixed_form(letkf):
    synthetic = pkg("synthetic")
    w = synthetic.small_case(nlat=12, nlon=24, nz=4, k=32, nobs=900, loc_dist_km=900.0, seed=41)
    dec = (2, 4)
    ctx = letkf.LetkfGPU.from_workload(w, decomp=dec, precision=letkf.LETKF_PREC_MIXED)
    xa, axa = ctx.run(w.xb, w.axb, w.obs)
    orc = O.Oracle(w, decomp=dec)
    off_g, idx_g, _ = ctx.local_obs()
    off_o, idx_o, _ = orc.local_obs()
    assert np.array_equal(off_g, off_o) and np.array_equal(idx_g, idx_o)
    xa_o, axa_o = orc.run()
    errs = mean_spread_errors(xa, axa, xa_o, axa_o, w)
    assert max(max(v.values()) for v in errs.values()) <= 1e-4, errs


def test_decomposition_needs_single_column_cubes(letkf):
    w = _edge_case()
    with pytest.raises(letkf.LetkfError):
        letkf.LetkfGPU.from_workload(w, decomp=(2, 2), cube_n=2)
    with pytest.raises(letkf.LetkfError):
        letkf.LetkfGPU.from_workload(w, decomp=(0, 3))
