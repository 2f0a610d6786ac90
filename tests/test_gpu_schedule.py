"""The mixed form's analysis does not depend on its schedule.

The work-queue chunk (letkf_gpu_set_schedule, letkf_gpu_autotune) decides
which CTA takes which cubes and in what order; the eigensolves warm-start
only inside aligned runs of cubes (8 for the staged k = 64 core, 16 for the
one-launch cores), so every chunk size must give the same analysis bit for
bit: at the 1-degree configuration (64,800 columns, k = 64) and on small
grids for the one-launch cores (k = 32, 48, 96, 128).
"""
import numpy as np
import pytest

from conftest import pkg

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def letkf():
    pkg("build").build()
    m = pkg("letkf")
    m.load_library()
    return m


@pytest.fixture(scope="module")
def synthetic():
    return pkg("synthetic")


def _device_state(w):
    import torch
    dev = torch.device("cuda:0")
    xb = torch.from_numpy(w.xb).to(dev)
    axb = torch.from_numpy(w.axb).to(dev)
    return xb, axb, torch.empty_like(xb), torch.empty_like(axb)


def _runs(letkf, ctx, w, chunks):
    import torch
    xb, axb, xa, axa = _device_state(w)
    obs = letkf.ObsArrays(w.obs)
    torch.cuda.synchronize()
    out = {}
    for c in chunks:
        ctx.set_schedule(c)
        ctx.run_device(xb, axb, obs, xa, axa)
        ctx._check(ctx.L.letkf_gpu_synchronize(ctx.h), "synchronize")
        out[c] = (xa.cpu().numpy(), axa.cpu().numpy())
    return out


def test_config1_analysis_independent_of_chunk(letkf, synthetic):
    w = synthetic.config(1)
    ctx = letkf.LetkfGPU.from_workload(w, precision=letkf.LETKF_PREC_MIXED)
    out = _runs(letkf, ctx, w, (8, 16, 32, 64))
    xa0, axa0 = out[8]
    assert np.isfinite(xa0).all()
    for c in (16, 32, 64):
        assert np.array_equal(out[c][0], xa0), c
        assert np.array_equal(out[c][1], axa0), c
    # the autotuner's pick changes nothing either
    import torch
    xb, axb, xa, axa = _device_state(w)
    torch.cuda.synchronize()
    pick = ctx.autotune_device(xb, axb, letkf.ObsArrays(w.obs), xa, axa)
    assert pick in (8, 16, 32, 64)
    assert np.array_equal(xa.cpu().numpy(), xa0)
    ctx.close()


@pytest.mark.parametrize("k", [32, 48, 96, 128])
def test_one_launch_cores_independent_of_chunk(letkf, synthetic, k):
    w = synthetic.small_case(nlat=30, nlon=60, nz=2, k=k, nobs=3000, loc_dist_km=900.0, seed=90 + k)
    ctx = letkf.LetkfGPU.from_workload(w, precision=letkf.LETKF_PREC_MIXED)
    out = _runs(letkf, ctx, w, (8, 16, 32, 64, 128))
    xa0, axa0 = out[16]
    assert np.isfinite(xa0).all()
    for c in (8, 32, 64, 128):
        assert np.array_equal(out[c][0], xa0), c
        assert np.array_equal(out[c][1], axa0), c
    # a cube range starting on a warm-start run boundary: its columns as in
    # the whole run
    ctx.set_schedule(0)
    first, count = 16 * 37, 16 * 21 + 5
    ctx.set_cube_range(first, count)
    r = _runs(letkf, ctx, w, (0,))[0]
    assert np.array_equal(r[0][first:first + count], xa0[first:first + count])
    assert np.array_equal(r[1][first:first + count], axa0[first:first + count])


def test_set_schedule_rejects_bad_chunks(letkf, synthetic):
    w = synthetic.small_case(nlat=8, nlon=16, nz=2, k=32, nobs=100, seed=95)
    ctx = letkf.LetkfGPU.from_workload(w, precision=letkf.LETKF_PREC_MIXED)
    for bad in (-1, 4, 12, 2048):
        with pytest.raises(letkf.LetkfError):
            ctx.set_schedule(bad)
    ctx.set_schedule(0)
    ctx.set_schedule(1024)
