"""The oracle's restatement of the observation builders (read_obs and
read_obs_regular, code/x86/TradDA/DA/LETKF/src/read_obs_mod.F90:339-651)
against numpy in single precision, as the reference's real(4) buffers."""
import numpy as np
import pytest

from oracle import oracle as O

f32 = np.float32


def _records(rng, nrec, nvar, nz):
    lon = rng.uniform(0, 360, nrec).astype(f32)
    lat = rng.uniform(-80, 80, nrec).astype(f32)
    lev = np.tile(np.arange(1, nz + 1, dtype=f32), nrec // nz)
    val = rng.standard_normal((nrec, 2 * nvar + 1)).astype(f32)
    val[:, 1:2 * nvar:2] = rng.uniform(0.5, 2.0, (nrec, nvar)).astype(f32)
    val[:, -1] = rng.uniform(2e4, 1e5, nrec).astype(f32)
    randn = rng.standard_normal((nvar, nrec)).astype(f32)
    return lon, lat, lev, val, randn


@pytest.mark.parametrize("nvar,nz", [(2, 1), (3, 4)])
def test_records(nvar, nz):
    rng = np.random.default_rng(nz)
    nrec = 12 * nz
    lon, lat, lev, val, randn = _records(rng, nrec, nvar, nz)
    var_of = np.arange(nvar, dtype=np.int32)[::-1].copy()
    o = O.obs_from_records(lon, lat, lev, val, var_of, nz=nz, randn=randn)
    e = 0
    for prof in range(nrec // nz):
        for lv in range(nz):
            r = prof * nz + lv
            for n in range(nvar):
                v, sg = val[r, 2 * n], val[r, 2 * n + 1]
                assert o["yo"][e] == float(f32(v + f32(randn[n, r] * sg)))
                assert o["rinv"][e] == float(f32(f32(1.0) / f32(sg * sg)))
                assert o["ph"][e] == float(val[r, -1])
                assert o["lat"][e] == float(lat[prof * nz]) and o["lon"][e] == float(lon[prof * nz])
                assert o["lev"][e] == lv + 1 and o["var"][e] == var_of[n]
                e += 1
    assert e == o["yo"].size


def test_records_reject_broken_profiles():
    rng = np.random.default_rng(3)
    lon, lat, lev, val, randn = _records(rng, 12, 2, 3)
    lev[4] = 3.0
    with pytest.raises(ValueError):
        O.obs_from_records(lon, lat, lev, val, [0, 1], nz=3)


def test_regular_grid():
    rng = np.random.default_rng(5)
    nlat_o, nlon_o, nz, nvar = 3, 4, 2, 2
    lats = rng.uniform(-60, 60, nlat_o).astype(f32)
    latn = (lats + f32(1.5)).astype(f32)
    lonw = rng.uniform(0, 350, nlon_o).astype(f32)
    lone = (lonw + f32(2.5)).astype(f32)
    r = rng.uniform(0.5, 2, (nz, nvar)).astype(f32)
    corners = [rng.standard_normal((nlon_o, nlat_o, nz, nvar + 1)).astype(f32) for _ in range(4)]
    randn = rng.standard_normal((nlat_o * nlon_o, nz, nvar)).astype(f32)
    o = O.obs_regular(latn, lats, lonw, lone, r, *corners, var_of=[1, 2], randn=randn)
    nw, sw, ne, se = corners
    avg = (((nw + sw) + ne) + se) / f32(4.0)
    e = 0
    for i in range(nlon_o):
        for j in range(nlat_o):
            ob = j + nlat_o * i
            for k in range(nz):
                for n in range(nvar):
                    rinv = float(f32(1.0) / f32(r[k, n] * r[k, n]))
                    assert o["rinv"][e] == rinv
                    assert o["yo"][e] == float(avg[i, j, k, n + 1]) + float(randn[ob, k, n]) / np.sqrt(rinv)
                    assert o["ph"][e] == float(avg[i, j, k, 0])
                    assert o["lat"][e] == float((latn[j] + lats[j]) / f32(2.0))
                    assert o["lon"][e] == float((lonw[i] + lone[i]) / f32(2.0))
                    assert o["lev"][e] == k + 1 and o["var"][e] == n + 1
                    e += 1
