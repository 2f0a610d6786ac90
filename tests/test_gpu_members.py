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


@pytest.mark.parametrize("k", [64, 128])
def test_members_mixed_staged_and_wide(letkf, k):
    # k = 64: the split and the blend fused into H and the staged core's
    # update; k = 128: the wide core, which keeps them as separate passes
    w = pkg("synthetic").small_case(nlat=12, nlon=24, nz=3, k=k, nobs=1200, seed=63 + k)
    xin = w.xb + w.axb[..., None]
    ctx = letkf.LetkfGPU.from_workload(w, precision=letkf.LETKF_PREC_MIXED)
    xout, sb, sa = ctx.run_members(xin, w.obs, gamma1=0.3, gamma2=0.7, polar_lat_deg=70.0)
    xo_r, sb_r, sa_r = _reference(w, xin, 0.3, 0.7, 70.0)
    assert max(field_rel_err(xout.mean(axis=-1), xo_r.mean(axis=-1), w).values()) <= 1e-4
    assert max(field_rel_err(sb, sb_r, w).values()) <= 1e-6
    assert max(field_rel_err(sa, sa_r, w).values()) <= 1e-4
    # columns poleward of 70 deg keep the background members (exactly in the
    # fused form; as mean + perturbation in the separate passes)
    polar_cols = np.flatnonzero(np.abs(np.tile(w.glat, w.nlon)) > 70.0)
    assert polar_cols.size > 0
    if k == 64:
        assert np.array_equal(xout[polar_cols], xin[polar_cols])
    else:
        assert np.max(np.abs(xout[polar_cols] - xin[polar_cols])) <= 1e-12 * np.abs(xin).max()


def test_members_fused_cost_near_plain_run(letkf):
    # The fused members run makes no state pass of its own: on device memory
    # at configuration 1 it takes the time of letkf_gpu_run plus the FP64
    # arithmetic of the split and the blend (three FP64 operations per member
    # and row, 1.2 G on GB300's narrow FP64 pipe); the separate passes would
    # move 16 GB of state and do twice that FP64 work
    import ctypes as C

    import torch
    w = pkg("synthetic").config(1)
    dev = torch.device("cuda", 0)
    ctx = letkf.LetkfGPU.from_workload(w, precision=letkf.LETKF_PREC_MIXED)
    keys = ("lat", "lon", "ph", "lev", "var", "yo", "rinv")
    obs = letkf.ObsArrays({k: torch.from_numpy(np.ascontiguousarray(w.obs[k])).to(dev) for k in keys}, device=True)
    xb = torch.from_numpy(w.xb).to(dev)
    axb = torch.from_numpy(w.axb).to(dev)
    xin = xb + axb[..., None]
    xa, axa = torch.empty_like(xb), torch.empty_like(axb)
    xo, sb, sa = torch.empty_like(xb), torch.empty_like(axb), torch.empty_like(axb)
    bl = letkf.Blend(gamma1=0.2, gamma2=0.8, polar_lat_deg=80.0)

    def members():
        rc = ctx.L.letkf_gpu_run_members(ctx.h, xin.data_ptr(), C.byref(obs.c), C.byref(bl), xo.data_ptr(),
                                         sb.data_ptr(), sa.data_ptr(), letkf.LETKF_DEVICE_PTRS)
        ctx._check(rc, "run_members")
        return ctx.stats()["ms_total"]

    def plain():
        ctx.run_device(xb, axb, obs, xa, axa)
        torch.cuda.synchronize()
        return ctx.stats()["ms_total"]

    for f in (members, plain):
        f()
    t_m = sorted(members() for _ in range(3))[1]
    t_p = sorted(plain() for _ in range(3))[1]
    print(f"members run {t_m:.2f} ms, plain run {t_p:.2f} ms")
    assert t_m <= 1.15 * t_p, (t_m, t_p)
    # and it is the same analysis: the blend of the plain run's output
    g1, g2 = 0.2, 0.8
    ref = g1 * (axb[..., None] + xb) + g2 * (axa[..., None] + xa)
    lat = torch.from_numpy(np.tile(w.glat.astype(np.float64), w.nlon)).to(dev)
    blend_cols = lat.abs() <= 80.0
    err = (xo[blend_cols] - ref[blend_cols]).abs().max() / ref[blend_cols].abs().max()
    assert float(err) <= 1e-6, float(err)
