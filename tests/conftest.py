"""Shared test set-up: package import helpers and the `gpu` marker."""
from __future__ import annotations

import importlib
import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(REPO, "tests", "golden")
if REPO not in sys.path:
    sys.path.insert(0, REPO)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300)")


def pkg(name: str):
    """Import a module of the dida-thhpca-sc23_gb300 package."""
    return importlib.import_module(f"dida-thhpca-sc23_gb300.{name}")


def golden_case(name: str):
    """(workload, expected dict) of a committed golden fixture."""
    synthetic = pkg("synthetic")
    z = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    nz, k, loc, infl, max_obs, polar = z["meta"]
    hyai, hybi = synthetic.hybrid_coefficients(int(nz))
    obs = dict(lat=z["obs_lat"], lon=z["obs_lon"], ph=z["obs_ph"], lev=z["obs_lev"],
               var=z["obs_var"], yo=z["obs_yo"], rinv=z["obs_rinv"])
    w = synthetic.Workload(name=name, glat=z["glat"], glon=z["glon"], nz=int(nz), k=int(k),
                           hyai=hyai, hybi=hybi, xb=z["xb"], axb=z["axb"], truth=z["axb"],
                           obs=obs, loc_dist_km=float(loc), inflation=float(infl),
                           max_obs=int(max_obs), obs_polar=float(polar))
    exp = {key[4:]: z[key] for key in z.files if key.startswith("exp_")}
    return w, exp


GOLDEN_CASES = ["small_k8", "small_k16_trunc", "small_k4_polar"]


def field_rel_err(a, b, w):
    """Largest relative error per state variable of [ncol][n](...) arrays:
    max|a-b| over a variable's rows divided by max|b| over the same rows."""
    rows = {"ps": slice(0, w.nvar2d)}
    names = ["u", "v", "T"][: w.nvar3d]
    for i, nm in enumerate(names):
        s = w.nvar2d + i * w.nz
        rows[nm] = slice(s, s + w.nz)
    out = {}
    for nm, sl in rows.items():
        d = np.abs(a[:, sl] - b[:, sl]).max()
        s = np.abs(b[:, sl]).max()
        out[nm] = float(d / s) if s > 0 else float(d)
    return out


def spread(xa):
    """Ensemble spread per column and row: sqrt(mean over members of xa^2)."""
    return np.sqrt(np.mean(xa * xa, axis=-1))


def var_rows(w):
    """Row slice of each state variable: ps, then u, v, T on w.nz levels."""
    rows = {"ps": slice(0, w.nvar2d)}
    for i, nm in enumerate(["u", "v", "T"][: w.nvar3d]):
        rows[nm] = slice(w.nvar2d + i * w.nz, w.nvar2d + (i + 1) * w.nz)
    return rows


def increment_errors(xa, axa, xa_ref, axa_ref, xb, axb, w):
    """Per-variable errors of the analysis mean and spread on the scale of
    what the analysis adds: max|a - ref| over a variable's rows divided by
    max|ref - background| there (the mean's change axa - axb, the spread's
    change spread_a - spread_b)."""
    out = {}
    for kind, a, r, bg in (("mean", axa, axa_ref, axb),
                           ("spread", spread(xa), spread(xa_ref), spread(xb))):
        out[kind] = {}
        for nm, sl in var_rows(w).items():
            d = np.abs(a[:, sl] - r[:, sl]).max()
            inc = np.abs(r[:, sl] - bg[:, sl]).max()
            out[kind][nm] = float(d / inc) if inc > 0 else float(d)
    return out


def mean_spread_errors(xa, axa, xa_ref, axa_ref, w):
    """Per-variable relative errors of the analysis mean and spread (max abs
    difference over the variable's rows and columns / max abs reference)."""
    return {"mean": field_rel_err(axa, axa_ref, w),
            "spread": field_rel_err(spread(xa), spread(xa_ref), w)}
