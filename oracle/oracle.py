"""ctypes binding of the CPU oracle (letkf_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, always as the checker, never as the product.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libletkf_oracle.so")
_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (gcc) if needed."""
    src = os.path.join(_HERE, "letkf_oracle.c")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return LIB_PATH


class OrcConfig(C.Structure):
    _fields_ = [
        ("nlat", C.c_int), ("nlon", C.c_int), ("nz", C.c_int), ("nvar2d", C.c_int),
        ("nvar3d", C.c_int), ("k", C.c_int),
        ("glat", C.POINTER(C.c_float)), ("glon", C.POINTER(C.c_float)),
        ("hyai", C.POINTER(C.c_double)), ("hybi", C.POINTER(C.c_double)),
        ("p0", C.c_double), ("ptop", C.c_double), ("ps_row", C.c_int),
        ("local_dist", C.c_double), ("vert_dist", C.c_double), ("inflation", C.c_double),
        ("obs_polar", C.c_double), ("gc_filter", C.c_int), ("gc_filter_vertical", C.c_int),
        ("max_obs", C.c_int), ("cube_n", C.c_int), ("cube_nz", C.c_int), ("overlap", C.c_int),
        ("h_mode", C.c_int), ("dec_lat_blocks", C.c_int), ("dec_lon_blocks", C.c_int),
    ]


class OrcObs(C.Structure):
    _fields_ = [
        ("nobs", C.c_int64),
        ("lat", C.POINTER(C.c_double)), ("lon", C.POINTER(C.c_double)),
        ("ph", C.POINTER(C.c_double)), ("lev", C.POINTER(C.c_int)),
        ("var", C.POINTER(C.c_int)), ("yo", C.POINTER(C.c_double)),
        ("rinv", C.POINTER(C.c_double)),
    ]


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        d, i64, i32 = C.c_double, C.c_int64, C.c_int
        L.orc_schr2.restype = d
        L.orc_schr2.argtypes = [d]
        L.orc_schr.restype = d
        L.orc_schr.argtypes = [d]
        L.orc_latlon_dist.restype = d
        L.orc_latlon_dist.argtypes = [d, d, d, d]
        L.orc_num_cubes.restype = i64
        L.orc_local_obs.restype = i64
        L.orc_local_obs_point.restype = i32
        L.orc_num_threads.restype = i32
        L.orc_jacobi_eig.restype = i32
        _lib = L
    return _lib


def _p(a, ctype):
    return a.ctypes.data_as(C.POINTER(ctype))


class Oracle:
    """Oracle bound to one workload (see synthetic.Workload) and its parameters."""

    def __init__(self, w, *, vert_dist=-999.0, cube_n=1, cube_nz=1, overlap=0,
                 gc_filter_vertical=1, decomp=(0, 0)):
        self.w = w
        self._keep = []
        k = lambda a, dt: self._hold(np.ascontiguousarray(a, dtype=dt))
        self.glat = k(w.glat, np.float32)
        self.glon = k(w.glon, np.float32)
        self.hyai = k(w.hyai, np.float64)
        self.hybi = k(w.hybi, np.float64)
        self.cfg = OrcConfig(
            nlat=w.nlat, nlon=w.nlon, nz=w.nz, nvar2d=w.nvar2d, nvar3d=w.nvar3d, k=w.k,
            glat=_p(self.glat, C.c_float), glon=_p(self.glon, C.c_float),
            hyai=_p(self.hyai, C.c_double), hybi=_p(self.hybi, C.c_double),
            p0=w.p0, ptop=w.ptop, ps_row=w.ps_row, local_dist=w.loc_dist_km,
            vert_dist=vert_dist, inflation=w.inflation, obs_polar=w.obs_polar,
            gc_filter=w.gc_filter, gc_filter_vertical=gc_filter_vertical,
            max_obs=w.max_obs, cube_n=cube_n, cube_nz=cube_nz, overlap=overlap,
            h_mode=w.h_mode, dec_lat_blocks=decomp[0], dec_lon_blocks=decomp[1])
        o = w.obs
        self.olat = k(o["lat"], np.float64)
        self.olon = k(o["lon"], np.float64)
        self.oph = k(o["ph"], np.float64)
        self.olev = k(o["lev"], np.int32)
        self.ovar = k(o["var"], np.int32)
        self.oyo = k(o["yo"], np.float64)
        self.orinv = k(o["rinv"], np.float64)
        self.obs = OrcObs(nobs=self.olat.size, lat=_p(self.olat, C.c_double),
                          lon=_p(self.olon, C.c_double), ph=_p(self.oph, C.c_double),
                          lev=_p(self.olev, C.c_int), var=_p(self.ovar, C.c_int),
                          yo=_p(self.oyo, C.c_double), rinv=_p(self.orinv, C.c_double))
        self.xb = k(w.xb, np.float64)
        self.axb = k(w.axb, np.float64)

    def _hold(self, a):
        self._keep.append(a)
        return a

    @property
    def ncubes(self):
        return int(lib().orc_num_cubes(C.byref(self.cfg)))

    def obs_operator(self):
        nobs, kk = self.olat.size, self.w.k
        yb = np.empty((nobs, kk))
        dep = np.empty(nobs)
        rc = lib().orc_obs_operator(C.byref(self.cfg), _p(self.xb, C.c_double),
                                    _p(self.axb, C.c_double), C.byref(self.obs),
                                    _p(yb, C.c_double), _p(dep, C.c_double))
        if rc != 0:
            raise RuntimeError(f"oracle obs operator failed ({rc})")
        return yb, dep

    def local_obs(self):
        nc = self.ncubes
        off = np.zeros(nc + 1, dtype=np.int64)
        total = lib().orc_local_obs(C.byref(self.cfg), C.byref(self.obs), _p(off, C.c_int64),
                                    None, None, C.c_int64(0))
        idx = np.empty(max(total, 1), dtype=np.int32)
        rloc = np.empty(max(total, 1))
        total2 = lib().orc_local_obs(C.byref(self.cfg), C.byref(self.obs), _p(off, C.c_int64),
                                     _p(idx, C.c_int32), _p(rloc, C.c_double), C.c_int64(idx.size))
        assert total2 == total
        return off, idx[:total], rloc[:total]

    def local_obs_cubes(self, cubes):
        """(offsets, idx, rloc) of the listed cubes only, packed in their order."""
        cubes = np.ascontiguousarray(cubes, dtype=np.int64)
        L = lib()
        L.orc_local_obs_cubes.restype = C.c_int64
        off = np.zeros(cubes.size + 1, dtype=np.int64)
        total = L.orc_local_obs_cubes(C.byref(self.cfg), C.byref(self.obs), C.c_int64(cubes.size),
                                      _p(cubes, C.c_int64), _p(off, C.c_int64), None, None, C.c_int64(0))
        idx = np.empty(max(total, 1), dtype=np.int32)
        rloc = np.empty(max(total, 1))
        total2 = L.orc_local_obs_cubes(C.byref(self.cfg), C.byref(self.obs), C.c_int64(cubes.size),
                                       _p(cubes, C.c_int64), _p(off, C.c_int64), _p(idx, C.c_int32),
                                       _p(rloc, C.c_double), C.c_int64(idx.size))
        assert total2 == total
        return off, idx[:total], rloc[:total]

    def run(self):
        xa = np.empty_like(self.xb)
        axa = np.empty_like(self.axb)
        rc = lib().orc_letkf_run(C.byref(self.cfg), C.byref(self.obs), _p(self.xb, C.c_double),
                                 _p(self.axb, C.c_double), _p(xa, C.c_double), _p(axa, C.c_double))
        if rc != 0:
            raise RuntimeError(f"oracle letkf_run failed ({rc})")
        return xa, axa

    def run_cubes(self, cubes, yb=None, dep=None, xa=None, axa=None):
        """Plain column loop on a subset of cubes; other columns are left as
        they are in xa/axa (NaN if not given)."""
        if yb is None:
            yb, dep = self.obs_operator()
        cubes = np.ascontiguousarray(cubes, dtype=np.int64)
        if xa is None:
            xa = np.full_like(self.xb, np.nan)
            axa = np.full_like(self.axb, np.nan)
        rc = lib().orc_letkf_cubes(C.byref(self.cfg), C.byref(self.obs), _p(yb, C.c_double),
                                   _p(dep, C.c_double), _p(self.xb, C.c_double),
                                   _p(self.axb, C.c_double), _p(xa, C.c_double),
                                   _p(axa, C.c_double), _p(cubes, C.c_int64),
                                   C.c_int64(cubes.size))
        if rc != 0:
            raise RuntimeError(f"oracle column loop failed ({rc})")
        return xa, axa


def members_split(orc: "Oracle", xin):
    """dnn2letkf (module_da_parallel.F90:184-204): full members -> (xb, axb)."""
    x = np.ascontiguousarray(xin, dtype=np.float64)
    xb = np.empty_like(x)
    axb = np.empty(x.shape[:-1])
    rc = lib().orc_members_split(C.byref(orc.cfg), _p(x, C.c_double), _p(xb, C.c_double),
                                 _p(axb, C.c_double))
    if rc != 0:
        raise RuntimeError("NaN in the background members")
    return xb, axb


def members_blend(orc: "Oracle", gamma1, gamma2, polar_lat, xb, axb, xa, axa):
    """letkf2dnn (module_da_parallel.F90:214-258): -> (xa_out, spread_b, spread_a)."""
    arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (xb, axb, xa, axa)]
    xout = np.empty_like(arrs[0])
    sb = np.empty_like(arrs[1])
    sa = np.empty_like(arrs[1])
    lib().orc_members_blend(C.byref(orc.cfg), C.c_double(gamma1), C.c_double(gamma2),
                            C.c_double(polar_lat), *[_p(a, C.c_double) for a in arrs],
                            _p(xout, C.c_double), _p(sb, C.c_double), _p(sa, C.c_double))
    return xout, sb, sa


def _obs_out(m):
    return {"lat": np.empty(m), "lon": np.empty(m), "ph": np.empty(m), "lev": np.empty(m, np.int32),
            "var": np.empty(m, np.int32), "yo": np.empty(m), "rinv": np.empty(m)}


def _obs_ptrs(o):
    return [_p(o["lat"], C.c_double), _p(o["lon"], C.c_double), _p(o["ph"], C.c_double),
            _p(o["lev"], C.c_int32), _p(o["var"], C.c_int32), _p(o["yo"], C.c_double),
            _p(o["rinv"], C.c_double)]


def obs_from_records(lon, lat, lev, val, var_of, nz=1, randn=None):
    """read_obs (read_obs_mod.F90:388-441) flattened: -> obs dict."""
    f = lambda a: np.ascontiguousarray(a, dtype=np.float32)
    lon, lat, lev, val = f(lon), f(lat), f(lev), f(val)
    rn = None if randn is None else f(randn)
    vo = np.ascontiguousarray(var_of, dtype=np.int32)
    out = _obs_out(lon.size * vo.size)
    L = lib()
    L.orc_obs_from_records.restype = C.c_int64
    m = L.orc_obs_from_records(C.c_int64(lon.size), vo.size, nz, _p(lon, C.c_float), _p(lat, C.c_float),
                               _p(lev, C.c_float), _p(val, C.c_float),
                               None if rn is None else _p(rn, C.c_float), _p(vo, C.c_int32), *_obs_ptrs(out))
    if m < 0:
        raise ValueError("profile records must hold levels 1..nz in order")
    return out


def obs_regular(latn, lats, lonw, lone, r, nw, sw, ne, se, var_of, randn=None):
    """read_obs_regular (read_obs_mod.F90:506-627) flattened: -> obs dict.
    C-order arrays: r [nz][nvar], corners [nlon_o][nlat_o][nz][nvar+1],
    randn [nobs][nz][nvar]."""
    f = lambda a: np.ascontiguousarray(a, dtype=np.float32)
    arrs = [f(a) for a in (latn, lats, lonw, lone, r, nw, sw, ne, se)]
    rn = None if randn is None else f(randn)
    vo = np.ascontiguousarray(var_of, dtype=np.int32)
    nlon_o, nlat_o, nz, _ = arrs[5].shape
    out = _obs_out(nlat_o * nlon_o * nz * vo.size)
    L = lib()
    L.orc_obs_regular.restype = C.c_int64
    L.orc_obs_regular(nlat_o, nlon_o, nz, vo.size, *[_p(a, C.c_float) for a in arrs],
                      None if rn is None else _p(rn, C.c_float), _p(vo, C.c_int32), *_obs_ptrs(out))
    return out


def struct_atm2endnn(xb, ens_max, n_max, ens_start=1, n_start=1, xb2=None):
    """struct_atm2endnn (data_trans.F90:2-18): xb C-order [n][nx][ny][ens]
    (Fortran xb(ens, ny, nx, n)) into xb2 C-order [ny][nx][n_max][ens_max]."""
    n, nx, ny, ens = xb.shape
    src = np.ascontiguousarray(xb, dtype=np.float64)
    out = np.zeros((ny, nx, n_max, ens_max)) if xb2 is None else xb2
    lib().orc_struct_atm2endnn(ens, n, nx, ny, ens_max, n_max, ens_start, n_start, _p(src, C.c_double),
                               _p(out, C.c_double))
    return out


def struct_endnn2atm(xb2, ens, n, ens_start=1, n_start=1):
    """struct_endnn2atm (data_trans.F90:21-38): xb2 [ny][nx][n_max][ens_max] ->
    xb [n][nx][ny][ens]."""
    ny, nx, n_max, ens_max = xb2.shape
    src = np.ascontiguousarray(xb2, dtype=np.float64)
    out = np.empty((n, nx, ny, ens))
    lib().orc_struct_endnn2atm(ens, n, nx, ny, ens_max, n_max, ens_start, n_start, _p(src, C.c_double),
                               _p(out, C.c_double))
    return out


def struct_atm2endnn_a(axb, n_max, n_start=1, axb2=None):
    n, nx, ny = axb.shape
    src = np.ascontiguousarray(axb, dtype=np.float64)
    out = np.zeros((ny, nx, n_max)) if axb2 is None else axb2
    lib().orc_struct_atm2endnn_a(n, nx, ny, n_max, n_start, _p(src, C.c_double), _p(out, C.c_double))
    return out


def struct_endnn2atm_a(axb2, n, n_start=1):
    ny, nx, n_max = axb2.shape
    src = np.ascontiguousarray(axb2, dtype=np.float64)
    out = np.empty((n, nx, ny))
    lib().orc_struct_endnn2atm_a(n, nx, ny, n_max, n_start, _p(src, C.c_double), _p(out, C.c_double))
    return out


def schr2(ri: float) -> float:
    return lib().orc_schr2(ri)


def schr(ri: float) -> float:
    return lib().orc_schr(ri)


def latlon_dist(x1, y1, x2, y2) -> float:
    return lib().orc_latlon_dist(x1, y1, x2, y2)


def jacobi_eig(a: np.ndarray, max_sweeps: int = 100):
    k = a.shape[0]
    m = np.asfortranarray(a, dtype=np.float64).copy(order="F")
    lam = np.empty(k)
    v = np.empty((k, k), order="F")
    sw = lib().orc_jacobi_eig(k, _p(m, C.c_double), _p(lam, C.c_double), _p(v, C.c_double),
                              max_sweeps)
    return lam, v, sw


def letkf_core(hxens, rdiaginv, dep, rloc, inflation):
    """hxens [p][k]; returns trans (k x k, trans[i, j] = trans(i+1, j+1)) and w."""
    hx = np.ascontiguousarray(hxens, dtype=np.float64)
    p, k = hx.shape if hx.size else (0, hx.shape[-1])
    rd = np.ascontiguousarray(rdiaginv, dtype=np.float32)
    dp = np.ascontiguousarray(dep, dtype=np.float64)
    rl = np.ascontiguousarray(rloc, dtype=np.float64)
    trans = np.empty((k, k), order="F")
    w = np.empty(k)
    rc = lib().orc_letkf_core(k, p, _p(hx, C.c_double), _p(rd, C.c_float), _p(dp, C.c_double),
                              _p(rl, C.c_double), C.c_double(inflation), _p(trans, C.c_double),
                              _p(w, C.c_double))
    if rc != 0:
        raise RuntimeError("oracle letkf_core: eigensolver did not converge")
    return np.asarray(trans), w


def decomp_dims(nranks: int):
    """(lat_blocks, lon_blocks) of an nranks-way DA decomposition."""
    a, b = C.c_int(), C.c_int()
    if lib().orc_decomp_dims(nranks, C.byref(a), C.byref(b)) != 0:
        raise ValueError("nranks must be >= 1")
    return a.value, b.value


def block_slots(orc: "Oracle", bx: int, by: int):
    """Neighbour blocks (ids bx' * lon_blocks + by') that block (bx, by) scans."""
    cap = 4 * max(1, orc.cfg.dec_lat_blocks * orc.cfg.dec_lon_blocks) + 4
    buf = np.empty(cap, dtype=np.int32)
    n = lib().orc_block_slots(C.byref(orc.cfg), bx, by, _p(buf, C.c_int32), cap)
    return buf[:n].copy()


def num_threads() -> int:
    return int(lib().orc_num_threads())
