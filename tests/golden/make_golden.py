"""Generate the committed golden fixtures of the LETKF path.

The reference cannot be built here (its LETKF is Fortran against MKL and MPI,
and no Fortran compiler is installed), and it ships no golden vectors or
known-answer tests for this path.  These fixtures therefore come from a
second, independent restatement of the reference algorithm written with
numpy and LAPACK (numpy.linalg.eigh, i.e. dsyevd, the routine the reference
calls at code/x86/TradDA/DA/LETKF/src/letkf_core.F90:98).  It shares no code
with the C oracle: the oracle is checked against these files.

Run:  python tests/golden/make_golden.py     (writes tests/golden/*.npz)
"""
from __future__ import annotations

import importlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
synthetic = importlib.import_module("dida-thhpca-sc23_gb300.synthetic")

PI_F32 = float(np.float32(np.arctan(np.float32(1.0))) * np.float32(4.0))
EARTH_A = float(np.float32(6371.393))
GC_C1 = float(np.float32(1.666667))
GC_C2 = float(np.float32(0.6666667))


def schr2(ri):
    """letkf_yb.F90:245-269 with the float-rounded literals (vectorized)."""
    ri = np.asarray(ri, dtype=np.float64)
    out = np.ones_like(ri)
    m2 = ri > 2.0
    m1 = (~m2) & (ri > 1.0)
    m0 = (~m2) & (~m1) & (ri > 0.0)
    r = ri[m1]
    rj = r / 12.0 - 0.5
    rj = rj * r + 0.625
    rj = rj * r + GC_C1
    out[m1] = (rj * r - 5.0) * r + 4.0 - GC_C2 / r
    r = ri[m0]
    rk = r * r
    rj = (-0.25 * r + 0.5) * r + 0.625
    out[m0] = (rj * r - GC_C1) * rk + 1.0
    out[m2] = 0.0
    return out


def latlon_dist(x1, y1, x2, y2):
    """pro_info.F90:149-161."""
    r = lambda d: np.asarray(d, dtype=np.float64) / 180.0 * PI_F32
    v = np.cos(r(x1)) * np.cos(r(x2)) * np.cos(r(y1) - r(y2)) + np.sin(r(x1)) * np.sin(r(x2))
    return EARTH_A * np.arccos(np.minimum(v, 1.0))


def obs_operator(w):
    """H (level select) on all members, then mean removal (letkf_obs.F90:156-178)."""
    o = w.obs
    n = w.n
    rows = np.where(o["var"] < w.nvar2d, o["var"],
                    w.nvar2d + (o["var"] - w.nvar2d) * w.nz + (o["lev"] - 1))
    full = w.xb + w.axb[:, :, None]           # [ncol][n][k]
    yb = np.empty((o["lat"].size, w.k))
    for e in range(w.k):
        yb[:, e] = synthetic.horizontal_interp(w.glat, w.glon, full[:, :, e], o["lat"], o["lon"], rows)
    mean = yb.sum(axis=1) / w.k
    del n
    return yb - mean[:, None], o["yo"] - mean


def local_obs(w, clat, clon):
    o = w.obs
    dist = latlon_dist(o["lat"], o["lon"], clat, clon)
    gc = schr2(dist * 1.0 / w.loc_dist_km)
    keep = (np.abs(o["lat"]) <= w.obs_polar) & (gc > 0)
    idx = np.nonzero(keep)[0][: w.max_obs]
    return idx.astype(np.int32), gc[idx]


def letkf_core(hx, rdi, dep, rloc, infl):
    """letkf_core.F90:14-233 step by step, with numpy/LAPACK."""
    p, k = hx.shape
    rr = np.sqrt(rdi.astype(np.float64) * rloc)
    h = (hx * rr[:, None]).T                     # k x p
    work1 = h @ h.T
    lam, vec = np.linalg.eigh(work1)
    lam = lam + (k - 1) / infl
    pa = (vec / lam) @ vec.T
    h2 = h * rr[None, :]
    work2 = pa @ h2
    wbar = work2 @ dep
    trans = (vec * np.sqrt((k - 1) / lam)) @ vec.T + wbar[:, None]
    return trans, wbar


def analysis(w):
    yb, dep = obs_operator(w)
    rdi = w.obs["rinv"].astype(np.float32)
    xa = np.empty_like(w.xb)
    axa = np.empty_like(w.axb)
    counts, idx_all, rloc_all, trans_all = [], [], [], []
    for i in range(w.nlon):
        for j in range(w.nlat):
            c = j + w.nlat * i
            idx, rl = local_obs(w, float(w.glat[j]), float(w.glon[i]))
            trans, _ = letkf_core(yb[idx], rdi[idx], dep[idx], rl, w.inflation)
            v = np.einsum("ie,ri->re", trans, w.xb[c]) + w.axb[c][:, None]
            m = v.sum(axis=1) / w.k
            xa[c] = v - m[:, None]
            axa[c] = m
            counts.append(idx.size)
            idx_all.append(idx)
            rloc_all.append(rl)
            trans_all.append(trans)
    off = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
    return dict(yb=yb, dep=dep, xa=xa, axa=axa, off=off, idx=np.concatenate(idx_all),
                rloc=np.concatenate(rloc_all), trans=np.stack(trans_all))


CASES = {
    # name: (nlat, nlon, nz, k, nobs, loc_dist_km, inflation, seed, max_obs, obs_polar)
    "small_k8": (12, 24, 4, 8, 300, 900.0, 1.1, 7, 10000, 91.0),
    "small_k16_trunc": (10, 20, 3, 16, 800, 1200.0, 1.05, 11, 40, 91.0),
    "small_k4_polar": (8, 16, 2, 4, 200, 1500.0, 1.2, 13, 10000, 60.0),
}


def case_workload(name):
    nlat, nlon, nz, k, nobs, loc, infl, seed, max_obs, polar = CASES[name]
    w = synthetic.small_case(nlat=nlat, nlon=nlon, nz=nz, k=k, nobs=nobs, loc_dist_km=loc,
                             inflation=infl, seed=seed)
    w.max_obs = max_obs
    w.obs_polar = polar
    return w


def main():
    for name in CASES:
        w = case_workload(name)
        res = analysis(w)
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(
            path, glat=w.glat, glon=w.glon, xb=w.xb, axb=w.axb,
            obs_lat=w.obs["lat"], obs_lon=w.obs["lon"], obs_ph=w.obs["ph"], obs_lev=w.obs["lev"],
            obs_var=w.obs["var"], obs_yo=w.obs["yo"], obs_rinv=w.obs["rinv"],
            meta=np.array([w.nz, w.k, w.loc_dist_km, w.inflation, w.max_obs, w.obs_polar]),
            **{f"exp_{k}": v for k, v in res.items()})
        print(path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
