"""letkf_gpu_run_members (through the C-ABI) against the oracle: the caller's
conversion around letkf_run (run_da_parallel,
code/x86/TradDA/DA/EnDNN/src/module_da_parallel.F90:184-258) on the device.
Full members in; the oracle splits them, runs the analysis and blends.  Bar:
the FP64 one (1e-10 relative per state variable) for the analysis members and
both spreads."""
import dataclasses

import numpy as np
import pytest

from conftest import field_rel_err, pkg
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def letkf():
    pkg("build").build()
    m = pkg("letkf")
    m.load_library()
    return m


def _reference(w, xin, g1, g2, polar, **kw):
    orc0 = O.Oracle(w, **kw)
    xb, axb = O.members_split(orc0, xin)
    w2 = dataclasses.replace(w, xb=xb, axb=axb)
    orc = O.Oracle(w2, **kw)
    xa, axa = orc.run()
    return O.members_blend(orc, g1, g2, polar, xb, axb, xa, axa)


@pytest.mark.parametrize("g1,g2,polar,k", [(0.0, 1.0, 90.0, 8), (0.3, 0.7, 60.0, 16), (0.5, 0.5, 30.0, 4)])
def test_members_match_oracle(letkf, g1, g2, polar, k):
    w = pkg("synthetic").small_case(nlat=12, nlon=24, nz=3, k=k, nobs=600, seed=50 + k)
    xin = w.xb + w.axb[..., None]
    ctx = letkf.LetkfGPU.from_workload(w)
    xout, sb, sa = ctx.run_members(xin, w.obs, gamma1=g1, gamma2=g2, polar_lat_deg=polar)
    xo_r, sb_r, sa_r = _reference(w, xin, g1, g2, polar)
    assert max(field_rel_err(xout, xo_r, w).values()) <= 1e-10
    assert max(field_rel_err(sb, sb_r, w).values()) <= 1e-12
    assert max(field_rel_err(sa, sa_r, w).values()) <= 1e-10
    # the analysis members' mean is the analysis mean of the plain entry point
    # where the blend is the analysis alone
    if g1 == 0.0 and g2 == 1.0:
        xa, axa = letkf.LetkfGPU.from_workload(w).run(w.xb - 0.0, w.axb, w.obs)
        assert max(field_rel_err(xout.mean(axis=-1), axa, w).values()) <= 1e-10


def test_members_in_the_mixed_form(letkf):
    w = pkg("synthetic").small_case(nlat=12, nlon=24, nz=3, k=32, nobs=900, seed=61)
    xin = w.xb + w.axb[..., None]
    ctx = letkf.LetkfGPU.from_workload(w, precision=letkf.LETKF_PREC_MIXED)
    xout, sb, sa = ctx.run_members(xin, w.obs, gamma1=0.2, gamma2=0.8, polar_lat_deg=70.0)
    xo_r, sb_r, sa_r = _reference(w, xin, 0.2, 0.8, 70.0)
    assert max(field_rel_err(xout.mean(axis=-1), xo_r.mean(axis=-1), w).values()) <= 1e-4
    assert max(field_rel_err(sa, sa_r, w).values()) <= 1e-4


def test_members_reject_nan_background(letkf):
    w = pkg("synthetic").small_case(nlat=8, nlon=16, nz=2, k=8, nobs=50, seed=62)
    xin = w.xb + w.axb[..., None]
    xin[5, 2, 3] = np.nan
    ctx = letkf.LetkfGPU.from_workload(w)
    with pytest.raises(letkf.LetkfError) as ei:
        ctx.run_members(xin, w.obs)
    assert ei.value.code == letkf.LETKF_ERR_INVALID
    # the context stays usable
    xin[5, 2, 3] = 0.0
    ctx.run_members(xin, w.obs)
