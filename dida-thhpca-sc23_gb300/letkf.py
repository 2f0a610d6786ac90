"""Python binding of the GB300 LETKF C-ABI (include/letkf_gpu.h).

Mirrors the reference's module interface (code/x86/TradDA/DA/LETKF/src/):
``letkf_init`` (letkf_init.F90:2-98), ``letkf_run`` (letkf.F90:157-257) and
``letkf_final`` (letkf_final.F90:1-13), with the observations passed as arrays
instead of being read from Redis.  Every call goes to the CUDA library
``_build/libletkf_gpu.so``; there is no CPU fallback, and loading fails with
an error when the library or a CUDA device is missing.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libletkf_gpu.so")

LETKF_OK = 0
LETKF_ERR_INVALID = -1
LETKF_ERR_CUDA = -2
LETKF_ERR_ALLOC = -3
LETKF_ERR_TIMEOUT = -4
LETKF_ERR_NOT_CONVERGED = -5
LETKF_ERR_UNSUPPORTED = -6
LETKF_ERR_STATE = -7
LETKF_HOST_PTRS = 0
LETKF_DEVICE_PTRS = 1
LETKF_PREC_FP64 = 0
LETKF_PREC_MIXED = 1
LETKF_PREC_MIXED_F64EIG = 2

ERROR_NAMES = {
    LETKF_ERR_INVALID: "LETKF_ERR_INVALID", LETKF_ERR_CUDA: "LETKF_ERR_CUDA",
    LETKF_ERR_ALLOC: "LETKF_ERR_ALLOC", LETKF_ERR_TIMEOUT: "LETKF_ERR_TIMEOUT",
    LETKF_ERR_NOT_CONVERGED: "LETKF_ERR_NOT_CONVERGED",
    LETKF_ERR_UNSUPPORTED: "LETKF_ERR_UNSUPPORTED", LETKF_ERR_STATE: "LETKF_ERR_STATE",
}

EXPORTED = [
    "letkf_gpu_create", "letkf_gpu_set_stream", "letkf_gpu_set_keep_trans", "letkf_gpu_run",
    "letkf_gpu_run_halo", "letkf_gpu_set_schedule", "letkf_gpu_set_host_read",
    "letkf_gpu_synchronize", "letkf_gpu_obs_operator", "letkf_gpu_local_obs",
    "letkf_gpu_last_trans", "letkf_gpu_core_batch", "letkf_gpu_get_stats",
    "letkf_gpu_last_error", "letkf_gpu_destroy", "letkf_gpu_launch_count",
    "letkf_gpu_core_batch_noalloc", "letkf_decomp_dims", "letkf_gpu_autotune",
    "letkf_batch_create", "letkf_batch_launch", "letkf_batch_sync", "letkf_batch_launches",
    "letkf_batch_destroy", "letkf_gpu_set_list_limit", "letkf_gpu_set_cube_range", "letkf_gpu_run_members",
    "letkf_struct_atm2endnn", "letkf_struct_endnn2atm", "letkf_struct_atm2endnn_a", "letkf_struct_endnn2atm_a",
    "letkf_gpu_obs_from_records", "letkf_gpu_obs_regular", "letkf_gpu_set_wait_limit",
    "letkf_gpu_local_obs_cubes", "letkf_init_gpu_", "letkf_set_obs_gpu_", "letkf_run_gpu_", "letkf_final_gpu_",
]


class LetkfError(RuntimeError):
    def __init__(self, code, msg=""):
        super().__init__(f"{ERROR_NAMES.get(code, code)}: {msg}")
        self.code = code


class Grid(C.Structure):
    _fields_ = [
        ("nlat", C.c_int), ("nlon", C.c_int), ("nz", C.c_int), ("nvar2d", C.c_int),
        ("nvar3d", C.c_int), ("ens", C.c_int),
        ("lat", C.POINTER(C.c_float)), ("lon", C.POINTER(C.c_float)),
        ("hyai", C.POINTER(C.c_double)), ("hybi", C.POINTER(C.c_double)),
        ("p0", C.c_double), ("ptop", C.c_double), ("ps_row", C.c_int),
    ]


class Params(C.Structure):
    _fields_ = [
        ("loc_dist_km", C.c_double), ("vert_dist", C.c_double), ("inflation", C.c_double),
        ("obs_polar_deg", C.c_double), ("gc_filter", C.c_int), ("gc_filter_vertical", C.c_int),
        ("max_obs", C.c_int), ("cube_n", C.c_int), ("cube_nz", C.c_int), ("overlap", C.c_int),
        ("h_mode", C.c_int), ("precision", C.c_int),
        ("decomp_lat_blocks", C.c_int), ("decomp_lon_blocks", C.c_int),
    ]


class Blend(C.Structure):
    _fields_ = [("gamma1", C.c_double), ("gamma2", C.c_double), ("polar_lat_deg", C.c_double)]


class Obs(C.Structure):
    _fields_ = [
        ("nobs", C.c_int64), ("lat", C.c_void_p), ("lon", C.c_void_p), ("ph", C.c_void_p),
        ("lev", C.c_void_p), ("var", C.c_void_p), ("yo", C.c_void_p), ("rinv", C.c_void_p),
    ]


class Stats(C.Structure):
    _fields_ = [
        ("ncubes", C.c_int64), ("sum_p", C.c_int64), ("max_p", C.c_int64),
        ("n_truncated", C.c_int64), ("n_borderline", C.c_int64),
        ("n_not_converged", C.c_int64), ("max_sweeps", C.c_int32), ("precision", C.c_int32),
        ("ms_h2d", C.c_double), ("ms_obs", C.c_double), ("ms_search", C.c_double),
        ("ms_core", C.c_double), ("ms_d2h", C.c_double), ("ms_total", C.c_double),
        ("sum_sweeps", C.c_int64), ("n_ill_conditioned", C.c_int64),
        ("sched_chunk", C.c_int32), ("n_windows", C.c_int32),
        ("ms_stage", C.c_double * 4),
    ]

    def as_dict(self):
        d = {f: getattr(self, f) for f, _ in self._fields_}
        d["ms_stage"] = list(self.ms_stage)
        return d


_lib = None


def load_library(path: str = LIB_PATH):
    """Load the CUDA library; raises if it is missing (no fallback path)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError(f"GB300 LETKF library not built: {path} (run build())")
    L = C.CDLL(path)
    vp, i64, i32 = C.c_void_p, C.c_int64, C.c_int
    L.letkf_gpu_create.argtypes = [C.POINTER(vp), C.POINTER(Grid), C.POINTER(Params), i32]
    L.letkf_gpu_set_stream.argtypes = [vp, vp]
    L.letkf_gpu_set_keep_trans.argtypes = [vp, i32]
    L.letkf_gpu_set_wait_limit.argtypes = [vp, i64]
    L.letkf_gpu_run.argtypes = [vp, vp, vp, C.POINTER(Obs), vp, vp, i32]
    L.letkf_gpu_run_halo.argtypes = [vp, i32, vp, vp, C.POINTER(Obs), vp, vp]
    L.letkf_gpu_set_schedule.argtypes = [vp, i32]
    L.letkf_gpu_set_host_read.argtypes = [vp, i32]
    L.letkf_gpu_synchronize.argtypes = [vp]
    L.letkf_gpu_obs_operator.argtypes = [vp, vp, vp, C.POINTER(Obs), vp, vp]
    L.letkf_gpu_local_obs.argtypes = [vp, vp, vp, vp]
    L.letkf_gpu_local_obs_cubes.argtypes = [vp, vp, i64, vp, vp, vp]
    L.letkf_gpu_last_trans.argtypes = [vp, vp, i64, vp, vp]
    L.letkf_gpu_core_batch.argtypes = [vp, i64, vp, vp, vp, vp, vp, vp, vp]
    L.letkf_gpu_get_stats.argtypes = [vp, C.POINTER(Stats)]
    L.letkf_gpu_last_error.argtypes = [vp]
    L.letkf_gpu_last_error.restype = C.c_char_p
    L.letkf_gpu_destroy.argtypes = [vp]
    L.letkf_gpu_launch_count.restype = i64
    L.letkf_gpu_core_batch_noalloc.argtypes = [i32, C.c_double, i64, vp, vp, vp, vp, vp, vp, vp, vp]
    L.letkf_decomp_dims.argtypes = [i32, C.POINTER(C.c_int), C.POINTER(C.c_int)]
    L.letkf_gpu_autotune.argtypes = [vp, vp, vp, C.POINTER(Obs), vp, vp, i32]
    L.letkf_batch_create.argtypes = [C.POINTER(vp), i32, C.POINTER(vp), C.POINTER(vp), C.POINTER(vp),
                                     C.POINTER(Obs), C.POINTER(vp), C.POINTER(vp)]
    L.letkf_batch_launch.argtypes = [vp, vp]
    L.letkf_batch_sync.argtypes = [vp, vp]
    L.letkf_batch_launches.argtypes = [vp]
    L.letkf_batch_launches.restype = i64
    L.letkf_batch_destroy.argtypes = [vp]
    L.letkf_gpu_set_list_limit.argtypes = [vp, i64]
    L.letkf_gpu_set_cube_range.argtypes = [vp, i64, i64]
    L.letkf_gpu_run_members.argtypes = [vp, vp, C.POINTER(Obs), C.POINTER(Blend), vp, vp, vp, i32]
    L.letkf_gpu_obs_from_records.argtypes = [vp, i64, i32, i32, vp, vp, vp, vp, vp, vp, C.POINTER(Obs), i32]
    L.letkf_gpu_obs_regular.argtypes = [vp, i32, i32, i32, i32] + [vp] * 11 + [C.POINTER(Obs), i32]
    L.letkf_struct_atm2endnn.argtypes = [i32] * 8 + [vp, vp, vp]
    L.letkf_struct_endnn2atm.argtypes = [i32] * 8 + [vp, vp, vp]
    L.letkf_struct_atm2endnn_a.argtypes = [i32] * 5 + [vp, vp, vp]
    L.letkf_struct_endnn2atm_a.argtypes = [i32] * 5 + [vp, vp, vp]
    _lib = L
    return L


def _ptr(a):
    return None if a is None else a.ctypes.data


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class ObsArrays:
    """Observation arrays kept alive for one call (host numpy or device torch)."""

    def __init__(self, obs: dict, device: bool = False):
        self.device = device
        if device:
            import torch
            t = {k: v.contiguous() for k, v in obs.items()}
            self._keep = t
            p = lambda k: (t[k].data_ptr() if k in t and t[k] is not None else None)
            n = int(t["lat"].numel())
        else:
            t = {
                "lat": _f64(obs["lat"]), "lon": _f64(obs["lon"]),
                "ph": _f64(obs["ph"]) if obs.get("ph") is not None else None,
                "lev": (np.ascontiguousarray(obs["lev"], dtype=np.int32)
                        if obs.get("lev") is not None else None),
                "var": np.ascontiguousarray(obs["var"], dtype=np.int32),
                "yo": _f64(obs["yo"]), "rinv": _f64(obs["rinv"]),
            }
            self._keep = t
            p = lambda k: _ptr(t[k])
            n = int(t["lat"].size)
        self.c = Obs(nobs=n, lat=p("lat"), lon=p("lon"), ph=p("ph"), lev=p("lev"),
                     var=p("var"), yo=p("yo"), rinv=p("rinv"))

    @classmethod
    def empty_view(cls):
        """A view whose pointers the library fills (device memory it owns)."""
        v = cls.__new__(cls)
        v.device = True
        v._keep = None
        v.c = Obs()
        return v

    def to_host(self) -> dict:
        """Copies of a device view's arrays (through the CUDA runtime)."""
        cudart = _cudart()
        n = int(self.c.nobs)
        out = {}
        for key, dt in (("lat", np.float64), ("lon", np.float64), ("ph", np.float64), ("lev", np.int32),
                        ("var", np.int32), ("yo", np.float64), ("rinv", np.float64)):
            a = np.empty(n, dtype=dt)
            ptr = getattr(self.c, key)
            if n and ptr:
                rc = cudart.cudaMemcpy(C.c_void_p(a.ctypes.data), C.c_void_p(ptr), C.c_size_t(a.nbytes), 2)
                if rc != 0:
                    raise LetkfError(LETKF_ERR_CUDA, f"cudaMemcpy {rc}")
            out[key] = a
        return out


_CUDART = None


def _cudart():
    global _CUDART
    if _CUDART is None:
        home = os.environ.get("CUDA_HOME", "/usr/local/cuda")
        _CUDART = C.CDLL(os.path.join(home, "lib64", "libcudart.so"))
        _CUDART.cudaMemcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
    return _CUDART


class Batch:
    """One CUDA graph over the analyses of several contexts (letkf_batch_*):
    device tensors in and out, replayed on the same tensors."""

    def __init__(self, ctxs, xb, axb, obs, xa, axa):
        L = load_library()
        n = len(ctxs)
        vpa = lambda vals: (C.c_void_p * n)(*vals)
        self._obs = (Obs * n)(*[o.c for o in obs])
        self._keep = (ctxs, xb, axb, obs, xa, axa)
        h = C.c_void_p()
        rc = L.letkf_batch_create(C.byref(h), n, vpa([c.h.value for c in ctxs]),
                                  vpa([t.data_ptr() for t in xb]), vpa([t.data_ptr() for t in axb]),
                                  self._obs, vpa([t.data_ptr() for t in xa]), vpa([t.data_ptr() for t in axa]))
        if rc != LETKF_OK:
            raise LetkfError(rc, "letkf_batch_create")
        self.h, self.L = h, L
        self.launches = int(L.letkf_batch_launches(h))

    def launch(self, stream_handle=None):
        rc = self.L.letkf_batch_launch(self.h, stream_handle)
        if rc != LETKF_OK:
            raise LetkfError(rc, "letkf_batch_launch")

    def sync(self, stream_handle=None):
        rc = self.L.letkf_batch_sync(self.h, stream_handle)
        if rc != LETKF_OK:
            raise LetkfError(rc, "letkf_batch_sync")

    def close(self):
        if getattr(self, "h", None):
            self.L.letkf_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def decomp_dims(nranks: int):
    """(lat_blocks, lon_blocks) of a DA group of nranks ranks (letkf_decomp_dims)."""
    L = load_library()
    a, b = C.c_int(), C.c_int()
    rc = L.letkf_decomp_dims(nranks, C.byref(a), C.byref(b))
    if rc != LETKF_OK:
        raise LetkfError(rc, "letkf_decomp_dims")
    return a.value, b.value


class LetkfGPU:
    """One analysis context (grid + namelist parameters) on one GPU."""

    def __init__(self, glat, glon, nz, ens, *, nvar2d=1, nvar3d=3, hyai=None, hybi=None,
                 p0=1.0e5, ptop=219.4, ps_row=0, loc_dist_km, inflation, vert_dist=-999.0,
                 obs_polar_deg=91.0, gc_filter=1, gc_filter_vertical=1, max_obs=10000,
                 cube_n=1, cube_nz=1, overlap=0, h_mode=1, precision=LETKF_PREC_FP64,
                 decomp=(0, 0), device=0):
        L = load_library()
        self._glat = np.ascontiguousarray(glat, dtype=np.float32)
        self._glon = np.ascontiguousarray(glon, dtype=np.float32)
        self._hyai = None if hyai is None else _f64(hyai)
        self._hybi = None if hybi is None else _f64(hybi)
        g = Grid(nlat=self._glat.size, nlon=self._glon.size, nz=nz, nvar2d=nvar2d, nvar3d=nvar3d,
                 ens=ens, lat=self._glat.ctypes.data_as(C.POINTER(C.c_float)),
                 lon=self._glon.ctypes.data_as(C.POINTER(C.c_float)),
                 hyai=(None if self._hyai is None else self._hyai.ctypes.data_as(C.POINTER(C.c_double))),
                 hybi=(None if self._hybi is None else self._hybi.ctypes.data_as(C.POINTER(C.c_double))),
                 p0=p0, ptop=ptop, ps_row=ps_row)
        prm = Params(loc_dist_km=loc_dist_km, vert_dist=vert_dist, inflation=inflation,
                     obs_polar_deg=obs_polar_deg, gc_filter=gc_filter,
                     gc_filter_vertical=gc_filter_vertical, max_obs=max_obs, cube_n=cube_n,
                     cube_nz=cube_nz, overlap=overlap, h_mode=h_mode, precision=precision,
                     decomp_lat_blocks=decomp[0], decomp_lon_blocks=decomp[1])
        h = C.c_void_p()
        rc = L.letkf_gpu_create(C.byref(h), C.byref(g), C.byref(prm), device)
        if rc != LETKF_OK:
            raise LetkfError(rc, "letkf_gpu_create")
        self.h = h
        self.L = L
        self.nlat, self.nlon, self.nz, self.k = self._glat.size, self._glon.size, nz, ens
        self.n = nvar2d + nvar3d * nz
        self.cube_n = cube_n
        step = cube_n - overlap                  # cubes start every cube_n - overlap points
        self.ncubes = (-(-self.nlat // step)) * (-(-self.nlon // step))

    @classmethod
    def from_workload(cls, w, **kw):
        args = dict(nvar2d=w.nvar2d, nvar3d=w.nvar3d, hyai=w.hyai, hybi=w.hybi, p0=w.p0,
                    ptop=w.ptop, ps_row=w.ps_row, loc_dist_km=w.loc_dist_km,
                    inflation=w.inflation, obs_polar_deg=w.obs_polar, gc_filter=w.gc_filter,
                    max_obs=w.max_obs, h_mode=w.h_mode)
        args.update(kw)
        return cls(w.glat, w.glon, w.nz, w.k, **args)

    def _check(self, rc, what):
        if rc != LETKF_OK:
            msg = self.L.letkf_gpu_last_error(self.h)
            raise LetkfError(rc, f"{what}: {msg.decode() if msg else ''}")

    def close(self):
        if getattr(self, "h", None):
            self.L.letkf_gpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream_handle: int | None):
        self._check(self.L.letkf_gpu_set_stream(self.h, stream_handle), "set_stream")

    def keep_trans(self, keep: bool = True):
        self._check(self.L.letkf_gpu_set_keep_trans(self.h, int(keep)), "set_keep_trans")

    def set_list_limit(self, max_entries: int = 0):
        """Most local-list entries held at once (0: from free memory); runs
        whose lists exceed it go through consecutive cube windows."""
        self._check(self.L.letkf_gpu_set_list_limit(self.h, int(max_entries)), "set_list_limit")

    def set_wait_limit(self, polls: int = -1):
        """Most polls of each bounded tensor-core wait (< 0: the default; 0:
        every wait gives up at once, which exercises the timeout path)."""
        self._check(self.L.letkf_gpu_set_wait_limit(self.h, int(polls)), "set_wait_limit")

    def set_host_read(self, on: bool = True):
        """Let H read its state rows from the host arrays while the state is
        copied in (same results; off: H waits for the whole state)."""
        self._check(self.L.letkf_gpu_set_host_read(self.h, int(on)), "set_host_read")

    def set_schedule(self, chunk: int = 0):
        """Work-queue chunk of the mixed form (0: the default); speed only."""
        self._check(self.L.letkf_gpu_set_schedule(self.h, int(chunk)), "set_schedule")

    def set_cube_range(self, first: int = 0, count: int = -1):
        """Analyse only cubes first .. first+count-1 (count < 0: all)."""
        self._check(self.L.letkf_gpu_set_cube_range(self.h, int(first), int(count)), "set_cube_range")

    def run(self, xb, axb, obs, xa=None, axa=None, allow_not_converged=False):
        """Host arrays in, host arrays out (letkf_run)."""
        xb = _f64(xb)
        axb = _f64(axb)
        xa = np.empty_like(xb) if xa is None else xa
        axa = np.empty_like(axb) if axa is None else axa
        o = obs if isinstance(obs, ObsArrays) else ObsArrays(obs)
        rc = self.L.letkf_gpu_run(self.h, _ptr(xb), _ptr(axb), C.byref(o.c), _ptr(xa), _ptr(axa),
                                  LETKF_HOST_PTRS)
        if not (allow_not_converged and rc == LETKF_ERR_NOT_CONVERGED):
            self._check(rc, "letkf_gpu_run")
        return xa, axa

    def run_halo(self, halo, xb, axb, obs, xa, axa, allow_not_converged=False):
        """letkf_run on arrays in its own layout with a halo: xb of shape
        (nlon + 2 halo, nlat + 2 halo, n, k) in C order (the Fortran
        xb(ens, n, 1-halo:nlat+halo, 1-halo:nlon+halo)), axb of shape
        (nlon + 2 halo, nlat + 2 halo, n); xa, axa alike, written in place
        (their halo is left as it was)."""
        for a in (xb, axb, xa, axa):
            if not (isinstance(a, np.ndarray) and a.dtype == np.float64 and a.flags.c_contiguous):
                raise TypeError("run_halo takes C-contiguous float64 arrays")
        lay = (self.nlon + 2 * halo, self.nlat + 2 * halo, self.n)
        if xb.shape != lay + (self.k,) or xa.shape != xb.shape or axb.shape != lay or axa.shape != lay:
            raise ValueError(f"run_halo wants xb, xa of shape {lay + (self.k,)} and axb, axa of shape {lay}")
        o = obs if isinstance(obs, ObsArrays) else ObsArrays(obs)
        rc = self.L.letkf_gpu_run_halo(self.h, int(halo), _ptr(xb), _ptr(axb), C.byref(o.c), _ptr(xa), _ptr(axa))
        if not (allow_not_converged and rc == LETKF_ERR_NOT_CONVERGED):
            self._check(rc, "letkf_gpu_run_halo")
        return xa, axa

    def run_members(self, xb_in, obs, gamma1=0.0, gamma2=1.0, polar_lat_deg=90.0):
        """run_da_parallel on the GPU: full members in (host arrays), analysis
        members and the background and analysis spreads out."""
        xin = _f64(xb_in)
        xout = np.empty_like(xin)
        sb = np.empty(xin.shape[:-1])
        sa = np.empty(xin.shape[:-1])
        o = obs if isinstance(obs, ObsArrays) else ObsArrays(obs)
        bl = Blend(gamma1=gamma1, gamma2=gamma2, polar_lat_deg=polar_lat_deg)
        self._check(self.L.letkf_gpu_run_members(self.h, _ptr(xin), C.byref(o.c), C.byref(bl), _ptr(xout),
                                                  _ptr(sb), _ptr(sa), LETKF_HOST_PTRS), "run_members")
        return xout, sb, sa

    def obs_from_records(self, lon, lat, lev, val, var_of, nz=1, randn=None):
        """Build observations on the device from obs-store records (host
        float32 arrays); returns an ObsArrays view of device memory."""
        f = lambda a: None if a is None else np.ascontiguousarray(a, dtype=np.float32)
        lon, lat, lev, val, randn = f(lon), f(lat), f(lev), f(val), f(randn)
        vo = np.ascontiguousarray(var_of, dtype=np.int32)
        nrec, nvar = lon.size, vo.size
        view = ObsArrays.empty_view()
        self._check(self.L.letkf_gpu_obs_from_records(self.h, nrec, nvar, nz, _ptr(lon), _ptr(lat), _ptr(lev),
                                                      _ptr(val), None if randn is None else _ptr(randn),
                                                      _ptr(vo), C.byref(view.c), LETKF_HOST_PTRS),
                    "obs_from_records")
        return view

    def obs_regular(self, latn, lats, lonw, lone, r, nw, sw, ne, se, var_of, randn=None):
        """Build a regular obs grid on the device (host float32 arrays in
        C order: r [nz][nvar], corners [nlon_o][nlat_o][nz][nvar+1], randn
        [nobs][nz][nvar]); returns an ObsArrays view of device memory."""
        f = lambda a: None if a is None else np.ascontiguousarray(a, dtype=np.float32)
        arrs = [f(a) for a in (latn, lats, lonw, lone, r, nw, sw, ne, se)]
        randn = f(randn)
        vo = np.ascontiguousarray(var_of, dtype=np.int32)
        nlon_o, nlat_o, nz, _ = arrs[5].shape
        view = ObsArrays.empty_view()
        self._check(self.L.letkf_gpu_obs_regular(self.h, nlat_o, nlon_o, nz, vo.size, *[_ptr(a) for a in arrs],
                                                 None if randn is None else _ptr(randn), _ptr(vo),
                                                 C.byref(view.c), LETKF_HOST_PTRS), "obs_regular")
        return view

    def run_device(self, xb, axb, obs: ObsArrays, xa, axa):
        """Device tensors (torch, this GPU) in and out."""
        rc = self.L.letkf_gpu_run(self.h, xb.data_ptr(), axb.data_ptr(), C.byref(obs.c),
                                  xa.data_ptr(), axa.data_ptr(), LETKF_DEVICE_PTRS)
        self._check(rc, "letkf_gpu_run")

    def autotune_device(self, xb, axb, obs: ObsArrays, xa, axa):
        """letkf_gpu_autotune on device tensors; returns the chosen chunk size."""
        rc = self.L.letkf_gpu_autotune(self.h, xb.data_ptr(), axb.data_ptr(), C.byref(obs.c),
                                       xa.data_ptr(), axa.data_ptr(), LETKF_DEVICE_PTRS)
        self._check(rc, "letkf_gpu_autotune")
        return self.stats()["sched_chunk"]

    def obs_operator(self, xb, axb, obs):
        xb = _f64(xb)
        axb = _f64(axb)
        o = obs if isinstance(obs, ObsArrays) else ObsArrays(obs)
        yb = np.empty((o.c.nobs, self.k))
        dep = np.empty(o.c.nobs)
        self._check(self.L.letkf_gpu_obs_operator(self.h, _ptr(xb), _ptr(axb), C.byref(o.c),
                                                  _ptr(yb), _ptr(dep)), "obs_operator")
        return yb, dep

    def local_obs(self):
        off = np.zeros(self.ncubes + 1, dtype=np.int64)
        self._check(self.L.letkf_gpu_local_obs(self.h, _ptr(off), None, None), "local_obs")
        idx = np.empty(max(int(off[-1]), 1), dtype=np.int32)
        rloc = np.empty(max(int(off[-1]), 1))
        self._check(self.L.letkf_gpu_local_obs(self.h, _ptr(off), _ptr(idx), _ptr(rloc)), "local_obs")
        return off, idx[:off[-1]], rloc[:off[-1]]

    def local_obs_cubes(self, cubes):
        """(offsets, idx, rloc) of the listed cubes only, packed in their order."""
        cubes = np.ascontiguousarray(cubes, dtype=np.int64)
        off = np.zeros(cubes.size + 1, dtype=np.int64)
        self._check(self.L.letkf_gpu_local_obs_cubes(self.h, _ptr(cubes), cubes.size, _ptr(off), None, None),
                    "local_obs_cubes")
        idx = np.empty(max(int(off[-1]), 1), dtype=np.int32)
        rloc = np.empty(max(int(off[-1]), 1))
        self._check(self.L.letkf_gpu_local_obs_cubes(self.h, _ptr(cubes), cubes.size, _ptr(off), _ptr(idx),
                                                     _ptr(rloc)), "local_obs_cubes")
        return off, idx[:off[-1]], rloc[:off[-1]]

    def last_trans(self, cubes):
        cubes = np.ascontiguousarray(cubes, dtype=np.int64)
        tr = np.empty((cubes.size, self.k, self.k))
        w = np.empty((cubes.size, self.k))
        self._check(self.L.letkf_gpu_last_trans(self.h, _ptr(cubes), cubes.size, _ptr(tr), _ptr(w)),
                    "last_trans")
        # stored column-major: tr[b].T[i, j] = trans(i+1, j+1)
        return np.ascontiguousarray(np.transpose(tr, (0, 2, 1))), w

    def core_batch(self, offsets, hxens, rdiaginv, dep, rloc):
        offsets = np.ascontiguousarray(offsets, dtype=np.int64)
        nb = offsets.size - 1
        hx = _f64(hxens)
        rd = np.ascontiguousarray(rdiaginv, dtype=np.float32)
        dp = _f64(dep)
        rl = _f64(rloc)
        tr = np.empty((nb, self.k, self.k))
        w = np.empty((nb, self.k))
        self._check(self.L.letkf_gpu_core_batch(self.h, nb, _ptr(offsets), _ptr(hx), _ptr(rd),
                                                _ptr(dp), _ptr(rl), _ptr(tr), _ptr(w)), "core_batch")
        return np.ascontiguousarray(np.transpose(tr, (0, 2, 1))), w

    def stats(self) -> dict:
        s = Stats()
        self._check(self.L.letkf_gpu_get_stats(self.h, C.byref(s)), "get_stats")
        return s.as_dict()


def struct_atm2endnn(xb, xb2, ens_start=1, n_start=1, stream=None):
    """struct_atm2endnn on device tensors: xb is the Fortran array
    xb(ens, ny, nx, n), i.e. a C-order tensor [n][nx][ny][ens]; xb2 is
    xb2(ens_max, n_max, nx, ny), a C-order tensor [ny][nx][n_max][ens_max]."""
    n, nx, ny, ens = xb.shape
    ny2, nx2, n_max, ens_max = xb2.shape
    assert (nx2, ny2) == (nx, ny)
    rc = load_library().letkf_struct_atm2endnn(ens, n, nx, ny, ens_max, n_max, ens_start, n_start,
                                               xb.data_ptr(), xb2.data_ptr(), stream)
    if rc != LETKF_OK:
        raise LetkfError(rc, "letkf_struct_atm2endnn")


def struct_endnn2atm(xb, xb2, ens_start=1, n_start=1, stream=None):
    """struct_endnn2atm on device tensors: xb [ny][nx][n_max][ens_max] ->
    xb2 [n][nx][ny][ens] (xb2 is the Fortran xb2(ens, ny, nx, n))."""
    ny, nx, n_max, ens_max = xb.shape
    n, nx2, ny2, ens = xb2.shape
    assert (nx2, ny2) == (nx, ny)
    rc = load_library().letkf_struct_endnn2atm(ens, n, nx, ny, ens_max, n_max, ens_start, n_start,
                                               xb.data_ptr(), xb2.data_ptr(), stream)
    if rc != LETKF_OK:
        raise LetkfError(rc, "letkf_struct_endnn2atm")


def struct_atm2endnn_a(axb, axb2, n_start=1, stream=None):
    """struct_atm2endnn_a: axb [n][nx][ny] -> axb2 [ny][nx][n_max]."""
    n, nx, ny = axb.shape
    n_max = axb2.shape[2]
    rc = load_library().letkf_struct_atm2endnn_a(n, nx, ny, n_max, n_start, axb.data_ptr(), axb2.data_ptr(),
                                                 stream)
    if rc != LETKF_OK:
        raise LetkfError(rc, "letkf_struct_atm2endnn_a")


def struct_endnn2atm_a(axb, axb2, n_start=1, stream=None):
    """struct_endnn2atm_a: axb [ny][nx][n_max] -> axb2 [n][nx][ny]."""
    ny, nx, n_max = axb.shape
    n = axb2.shape[0]
    rc = load_library().letkf_struct_endnn2atm_a(n, nx, ny, n_max, n_start, axb.data_ptr(), axb2.data_ptr(),
                                                 stream)
    if rc != LETKF_OK:
        raise LetkfError(rc, "letkf_struct_endnn2atm_a")


def launch_count() -> int:
    return int(load_library().letkf_gpu_launch_count())


# ---- module interface of the reference (letkf_init / letkf_run / letkf_final)

_module_ctx: LetkfGPU | None = None
_module_obs = None


def letkf_init(glat, glon, nz, ens, **kw):
    """letkf_init: build the analysis context (grid, namelist knobs)."""
    global _module_ctx
    letkf_final()
    _module_ctx = LetkfGPU(glat, glon, nz, ens, **kw)
    return _module_ctx


def letkf_set_obs(obs: dict):
    """Stage the observations of the next letkf_run (replaces the Redis read)."""
    global _module_obs
    _module_obs = ObsArrays(obs)


def letkf_run(ntimes, xb, axb):
    """letkf_run(ntimes, xb, axb) -> (xa, axa); ntimes selects the obs time in
    the reference and is accepted for interface parity."""
    del ntimes
    if _module_ctx is None or _module_obs is None:
        raise LetkfError(LETKF_ERR_STATE, "letkf_init and letkf_set_obs come first")
    return _module_ctx.run(xb, axb, _module_obs)


def letkf_final():
    global _module_ctx, _module_obs
    if _module_ctx is not None:
        _module_ctx.close()
    _module_ctx = None
    _module_obs = None
