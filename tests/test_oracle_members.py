"""The oracle's restatement of the caller's conversion around letkf_run
(run_da_parallel, code/x86/TradDA/DA/EnDNN/src/module_da_parallel.F90:184-258)
against numpy."""
import numpy as np
import pytest

from conftest import pkg
from oracle import oracle as O


def _orc():
    w = pkg("synthetic").small_case(nlat=8, nlon=16, nz=2, k=8, nobs=40, seed=3)
    return w, O.Oracle(w)


def test_split_is_mean_and_perturbations():
    w, orc = _orc()
    xin = w.xb + w.axb[..., None] + 0.25
    xb, axb = O.members_split(orc, xin)
    assert np.allclose(axb, xin.mean(axis=-1), rtol=0, atol=1e-12 * np.abs(xin).max())
    assert np.allclose(xb, xin - axb[..., None], rtol=0, atol=1e-12 * np.abs(xin).max())
    bad = xin.copy()
    bad[3, 1, 5] = np.nan
    with pytest.raises(RuntimeError):
        O.members_split(orc, bad)


def test_blend_and_spreads():
    w, orc = _orc()
    rng = np.random.default_rng(4)
    xb = rng.standard_normal(w.xb.shape)
    xa = rng.standard_normal(w.xb.shape)
    axb = rng.standard_normal(w.axb.shape)
    axa = rng.standard_normal(w.axb.shape)
    g1, g2, polar = 0.3, 0.7, 50.0
    xout, sb, sa = O.members_blend(orc, g1, g2, polar, xb, axb, xa, axa)
    lat = np.tile(w.glat.astype(np.float64), w.nlon)
    inside = np.abs(lat) <= polar
    ref = np.where(inside[:, None, None], g1 * (axb[..., None] + xb) + g2 * (axa[..., None] + xa),
                   xb + axb[..., None])
    assert np.allclose(xout, ref, rtol=1e-15, atol=1e-14)
    assert np.allclose(sb, np.sqrt(np.mean(xb * xb, axis=-1)), rtol=1e-14)
    sa_ref = np.where(inside[:, None], np.sqrt(np.mean((ref - axa[..., None]) ** 2, axis=-1)),
                      np.sqrt(np.mean(xb * xb, axis=-1)))
    assert np.allclose(sa, sa_ref, rtol=1e-14)
    assert (~inside).any() and inside.any()
