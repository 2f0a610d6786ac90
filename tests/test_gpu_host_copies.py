"""Host-buffer paths of letkf_gpu_run against the device-buffer path.

With host buffers the state goes in on the copy streams and the staged core's
finished blocks of columns go out while later blocks run; pageable buffers take
the same route through the context's copy thread, and letkf_gpu_run_halo (the
Fortran shim's call) reads and writes the interior of arrays in letkf_run's
halo layout with strided copies.  Every one of them must give the device run's
analysis bit for bit and write nothing outside the analysed columns.
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


def device_run(letkf, ctx, w):
    import torch
    dev = torch.device("cuda:0")
    xb = torch.from_numpy(w.xb).to(dev)
    axb = torch.from_numpy(w.axb).to(dev)
    xa = torch.empty_like(xb)
    axa = torch.empty_like(axb)
    obs = letkf.ObsArrays(w.obs)
    torch.cuda.synchronize()
    ctx.run_device(xb, axb, obs, xa, axa)
    ctx._check(ctx.L.letkf_gpu_synchronize(ctx.h), "synchronize")
    return xa.cpu().numpy(), axa.cpu().numpy()


def pinned_like(a):
    import torch
    t = torch.empty(a.shape, dtype=torch.float64, pin_memory=True)
    v = t.numpy()
    v[...] = a
    return t, v


def with_halo(a, w, h, fill):
    out = np.full((w.nlon + 2 * h, w.nlat + 2 * h) + a.shape[1:], fill)
    out[h:h + w.nlon, h:h + w.nlat] = a.reshape((w.nlon, w.nlat) + a.shape[1:])
    return out


def interior(a, w, h):
    return a[h:h + w.nlon, h:h + w.nlat].reshape((w.nlon * w.nlat,) + a.shape[2:])


def halo_untouched(a, w, h, fill):
    m = np.ones(a.shape[:2], bool)
    m[h:h + w.nlon, h:h + w.nlat] = False
    return np.all(a[m] == fill)


# 91 x 182 columns: the staged core's three copy-out blocks end at cubes 12288
# and 16384, both in the middle of a longitude line (91 columns each).
# host_read: H reads its rows from the host arrays while the state is copied
# in (each block's update waits for its own columns), or waits for the copy.
@pytest.mark.parametrize("precision,h_mode,host_read", [("mixed", 1, True), ("mixed", 1, False),
                                                        ("fp64", 1, True), ("fp64", 0, True),
                                                        ("fp64", 0, False)])
def test_host_paths_equal_device_run(letkf, synthetic, precision, h_mode, host_read):
    nlat = 91 if precision == "mixed" else 15
    k = 64 if precision == "mixed" else 16
    w = synthetic.small_case(nlat=nlat, nlon=2 * nlat, nz=2, k=k, nobs=2500, loc_dist_km=900.0, seed=71,
                             h_mode=h_mode)
    prec = letkf.LETKF_PREC_MIXED if precision == "mixed" else letkf.LETKF_PREC_FP64
    ctx = letkf.LetkfGPU.from_workload(w, precision=prec)
    ctx.set_host_read(host_read)
    xa_d, axa_d = device_run(letkf, ctx, w)
    # pageable numpy buffers (the copy thread)
    xa_p, axa_p = ctx.run(np.array(w.xb), np.array(w.axb), w.obs)
    assert np.array_equal(xa_p, xa_d) and np.array_equal(axa_p, axa_d)
    # page-locked buffers (copies issued by the calling thread)
    _, xb_pin = pinned_like(w.xb)
    _, axb_pin = pinned_like(w.axb)
    txa, xa_pin = pinned_like(np.zeros_like(w.xb))
    taxa, axa_pin = pinned_like(np.zeros_like(w.axb))
    ctx.run(xb_pin, axb_pin, w.obs, xa_pin, axa_pin)
    assert np.array_equal(xa_pin, xa_d) and np.array_equal(axa_pin, axa_d)
    # letkf_run's layout with a halo: the halo of xb is never read (NaN
    # there would spread), the halo of xa is never written
    for h in (1, 3):
        xb_h, axb_h = with_halo(w.xb, w, h, np.nan), with_halo(w.axb, w, h, np.nan)
        xa_h = np.full_like(xb_h, -7.0)
        axa_h = np.full_like(axb_h, -7.0)
        ctx.run_halo(h, xb_h, axb_h, w.obs, xa_h, axa_h)
        assert np.array_equal(interior(xa_h, w, h), xa_d)
        assert np.array_equal(interior(axa_h, w, h), axa_d)
        assert halo_untouched(xa_h, w, h, -7.0) and halo_untouched(axa_h, w, h, -7.0)
    # the halo layout from page-locked buffers
    h = 2
    _, xb_hp = pinned_like(with_halo(w.xb, w, h, np.nan))
    _, axb_hp = pinned_like(with_halo(w.axb, w, h, np.nan))
    _, xa_hp = pinned_like(with_halo(np.zeros_like(w.xb), w, h, -7.0))
    _, axa_hp = pinned_like(with_halo(np.zeros_like(w.axb), w, h, -7.0))
    ctx.run_halo(h, xb_hp, axb_hp, w.obs, xa_hp, axa_hp)
    assert np.array_equal(interior(xa_hp, w, h), xa_d)
    assert np.array_equal(interior(axa_hp, w, h), axa_d)
    assert halo_untouched(xa_hp, w, h, -7.0)
    del txa, taxa


def test_halo_cube_range_writes_only_its_columns(letkf, synthetic):
    # cube_n = 2 (no copy-out blocks: one copy of whole longitude strips at
    # the end) and a cube range of some strips
    w = synthetic.small_case(nlat=15, nlon=30, nz=2, k=16, nobs=900, loc_dist_km=900.0, seed=72)
    ctx = letkf.LetkfGPU.from_workload(w, cube_n=2)
    xa_all, axa_all = ctx.run(w.xb, w.axb, w.obs)
    nbj = -(-w.nlat // 2)
    first, count = 3 * nbj, 4 * nbj
    ctx.set_cube_range(first, count)
    h = 2
    xb_h, axb_h = with_halo(w.xb, w, h, np.nan), with_halo(w.axb, w, h, np.nan)
    xa_h = np.full_like(xb_h, -7.0)
    axa_h = np.full_like(axb_h, -7.0)
    ctx.run_halo(h, xb_h, axb_h, w.obs, xa_h, axa_h)
    # the range's columns: longitude lines 6 .. 13
    c0, c1 = 3 * 2 * w.nlat, 7 * 2 * w.nlat
    xi, ai = interior(xa_h, w, h), interior(axa_h, w, h)
    assert np.array_equal(xi[c0:c1], xa_all[c0:c1]) and np.array_equal(ai[c0:c1], axa_all[c0:c1])
    assert np.all(xi[:c0] == -7.0) and np.all(xi[c1:] == -7.0)
    assert halo_untouched(xa_h, w, h, -7.0)


def test_run_halo_rejects_bad_arguments(letkf, synthetic):
    import ctypes as C
    w = synthetic.small_case(nlat=8, nlon=16, nz=2, k=8, nobs=100, seed=73)
    ctx = letkf.LetkfGPU.from_workload(w)
    xb_h, axb_h = with_halo(w.xb, w, 1, 0.0), with_halo(w.axb, w, 1, 0.0)
    xa_h, axa_h = np.zeros_like(xb_h), np.zeros_like(axb_h)
    with pytest.raises(ValueError):
        ctx.run_halo(2, xb_h, axb_h, w.obs, xa_h, axa_h)
    obs = letkf.ObsArrays(w.obs)
    p = lambda a: a.ctypes.data_as(C.c_void_p)
    rc = ctx.L.letkf_gpu_run_halo(ctx.h, -1, p(xb_h), p(axb_h), C.byref(obs.c), p(xa_h), p(axa_h))
    assert rc == letkf.LETKF_ERR_INVALID
    rc = ctx.L.letkf_gpu_run_halo(ctx.h, 1, None, p(axb_h), C.byref(obs.c), p(xa_h), p(axa_h))
    assert rc == letkf.LETKF_ERR_INVALID
    assert np.all(xa_h == 0.0)
    ctx.run_halo(1, xb_h, axb_h, w.obs, xa_h, axa_h)
    assert np.isfinite(interior(xa_h, w, 1)).all()
