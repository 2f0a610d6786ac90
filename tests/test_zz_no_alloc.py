"""letkf_gpu_core_batch_noalloc against letkf_gpu_core_batch.

The no-allocation entry point is for callers that may not call cudaMalloc or
cudaFree: a model whose memory pool owns all of the GPU's memory, or code that
must not add the device-wide synchronization those calls bring.  They pass
every input and output as device memory they own; the library's scratch is a
fixed array inside the library.  This file is collected last, so a -x run that
stops here has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import pkg

pytestmark = pytest.mark.gpu
TOL = 1e-10


def _problems(seed, k, sizes):
    rng = np.random.default_rng(seed)
    offs = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    p = int(offs[-1])
    hx = rng.standard_normal((p, k))
    hx -= hx.mean(axis=1, keepdims=True)
    rdi = (1.0 / rng.uniform(0.5, 2.0, p) ** 2).astype(np.float32)
    dep = rng.standard_normal(p)
    rloc = rng.uniform(0.0, 1.0, p)
    return offs, hx, rdi, dep, rloc


@pytest.fixture(scope="module")
def lib():
    pkg("build").build()
    letkf = pkg("letkf")
    return letkf, letkf.load_library()


def _call(L, k, infl, nb, dev, tr, wb):
    return L.letkf_gpu_core_batch_noalloc(
        k, C.c_double(infl), C.c_int64(nb), C.c_void_p(dev["offs"].data_ptr()),
        C.c_void_p(dev["hx"].data_ptr()), C.c_void_p(dev["rdi"].data_ptr()),
        C.c_void_p(dev["dep"].data_ptr()), C.c_void_p(dev["rloc"].data_ptr()),
        C.c_void_p(tr.data_ptr()), C.c_void_p(wb.data_ptr()), None)


def test_noalloc_matches_core_batch_on_two_calls(lib):
    import torch
    letkf, L = lib
    k, infl = 32, 1.08
    synthetic = pkg("synthetic")
    w = synthetic.small_case(nlat=8, nlon=16, nz=1, k=k, nobs=10)
    ctx = letkf.LetkfGPU.from_workload(w, inflation=infl)
    for call, (seed, sizes) in enumerate(((1, [0, 3, 40, 700, 65]), (2, [9, 0, 0, 1200, 31, 5, 300]))):
        offs, hx, rdi, dep, rloc = _problems(seed, k, sizes)
        t_ref, w_ref = ctx.core_batch(offs, hx, rdi, dep, rloc)
        nb = len(sizes)
        dev = {name: torch.from_numpy(np.ascontiguousarray(a)).cuda()
               for name, a in (("offs", offs), ("hx", hx), ("rdi", rdi), ("dep", dep),
                               ("rloc", rloc))}
        tr = torch.full((nb, k, k), float("nan"), dtype=torch.float64, device="cuda")
        wb = torch.full((nb, k), float("nan"), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        rc = _call(L, k, infl, nb, dev, tr, wb)
        torch.cuda.synchronize()
        free_after = torch.cuda.mem_get_info()[0]
        assert rc == letkf.LETKF_OK
        got_t = np.transpose(tr.cpu().numpy(), (0, 2, 1))   # column-major per problem
        got_w = wb.cpu().numpy()
        assert np.max(np.abs(got_t - t_ref)) <= TOL * np.abs(t_ref).max()
        assert np.max(np.abs(got_w - w_ref)) <= TOL * np.abs(w_ref).max()
        if call == 1:
            assert free_after == free_before       # nothing allocated on the device


def test_noalloc_rejects_sizes_beyond_its_scratch(lib):
    letkf, L = lib
    nmax = 65536
    rc = L.letkf_gpu_core_batch_noalloc(32, C.c_double(1.1), C.c_int64(nmax + 1), None, None,
                                        None, None, None, None, None, None)
    assert rc == letkf.LETKF_ERR_INVALID


def test_noalloc_rejects_offsets_that_go_backwards(lib):
    # offsets start at 0 and step back once (problem 1 would have -25 rows):
    # the call returns LETKF_ERR_INVALID and no row is read (every row index
    # the offsets name lies inside the 100-row arrays anyway); a following
    # call with good offsets is unaffected by the flag the bad one left.
    import torch
    letkf, L = lib
    k, infl = 16, 1.1
    offs, hx, rdi, dep, rloc = _problems(5, k, [40, 35, 25])
    bad = np.array([0, 40, 15, 100], dtype=np.int64)
    dev = {name: torch.from_numpy(np.ascontiguousarray(a)).cuda()
           for name, a in (("offs", bad), ("hx", hx), ("rdi", rdi), ("dep", dep), ("rloc", rloc))}
    tr = torch.zeros((3, k, k), dtype=torch.float64, device="cuda")
    wb = torch.zeros((3, k), dtype=torch.float64, device="cuda")
    assert _call(L, k, infl, 3, dev, tr, wb) == letkf.LETKF_ERR_INVALID
    dev["offs"] = torch.from_numpy(offs).cuda()
    assert _call(L, k, infl, 3, dev, tr, wb) == letkf.LETKF_OK
    assert np.isfinite(tr.cpu().numpy()).all()
