"""The C-ABI library loads and exports every entry point include/letkf_gpu.h
declares; argument checks run without a GPU (no compute calls)."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import REPO, pkg

HEADER = os.path.join(REPO, "include", "letkf_gpu.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(letkf_\w+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    build = pkg("build")
    build.build()
    letkf = pkg("letkf")
    return letkf.load_library()


def test_header_declares_the_boundary():
    names = declared_functions()
    for must in ("letkf_gpu_create", "letkf_gpu_run", "letkf_gpu_destroy", "letkf_run_gpu_",
                 "letkf_init_gpu_", "letkf_gpu_core_batch", "letkf_gpu_local_obs"):
        assert must in names


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    letkf = pkg("letkf")
    assert sorted(letkf.EXPORTED) == sorted(declared_functions())


def _grid_params(letkf, nlat=4, nlon=8, ens=8, loc=500.0, lat=None):
    glat = np.asarray(lat if lat is not None else [-67.5, -22.5, 22.5, 67.5], np.float32)
    glon = (22.5 + 45.0 * np.arange(nlon)).astype(np.float32)
    g = letkf.Grid(nlat=nlat, nlon=nlon, nz=2, nvar2d=1, nvar3d=1, ens=ens,
                   lat=glat.ctypes.data_as(C.POINTER(C.c_float)),
                   lon=glon.ctypes.data_as(C.POINTER(C.c_float)), hyai=None, hybi=None,
                   p0=1e5, ptop=219.4, ps_row=0)
    p = letkf.Params(loc_dist_km=loc, vert_dist=-999.0, inflation=1.1, obs_polar_deg=91.0,
                     gc_filter=1, gc_filter_vertical=1, max_obs=10000, cube_n=1, cube_nz=1,
                     overlap=0, h_mode=1, precision=0)
    return g, p, (glat, glon)


def test_create_rejects_bad_arguments_before_touching_cuda(lib):
    letkf = pkg("letkf")
    h = C.c_void_p()
    g, p, keep = _grid_params(letkf, loc=-1.0)
    assert lib.letkf_gpu_create(C.byref(h), C.byref(g), C.byref(p), 0) == letkf.LETKF_ERR_INVALID
    g, p, keep = _grid_params(letkf, lat=[10.0, 5.0, 20.0, 30.0])          # not ascending
    assert lib.letkf_gpu_create(C.byref(h), C.byref(g), C.byref(p), 0) == letkf.LETKF_ERR_INVALID
    g, p, keep = _grid_params(letkf, ens=7)                                 # unsupported k
    assert lib.letkf_gpu_create(C.byref(h), C.byref(g), C.byref(p), 0) == letkf.LETKF_ERR_UNSUPPORTED
    assert lib.letkf_gpu_create(None, C.byref(g), C.byref(p), 0) == letkf.LETKF_ERR_INVALID
    assert lib.letkf_gpu_destroy(None) == letkf.LETKF_OK


def test_no_cpu_fallback_without_a_device(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    letkf = pkg("letkf")
    h = C.c_void_p()
    g, p, keep = _grid_params(letkf)
    assert lib.letkf_gpu_create(C.byref(h), C.byref(g), C.byref(p), 0) == letkf.LETKF_ERR_CUDA
    with pytest.raises(letkf.LetkfError):
        letkf.LetkfGPU(keep[0], keep[1], 2, 8, nvar3d=1, loc_dist_km=500.0, inflation=1.1)


def test_missing_library_fails_loudly(tmp_path):
    letkf = pkg("letkf")
    saved = letkf._lib
    try:
        letkf._lib = None
        with pytest.raises(ImportError):
            letkf.load_library(str(tmp_path / "nope.so"))
    finally:
        letkf._lib = saved


def test_decomp_dims_matches_oracle_without_gpu():
    letkf = pkg("letkf")
    letkf.load_library()
    from oracle import oracle as O
    for p in range(1, 200):
        assert letkf.decomp_dims(p) == O.decomp_dims(p), p
    with pytest.raises(letkf.LetkfError):
        letkf.decomp_dims(0)
