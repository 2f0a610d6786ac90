"""The oracle's decomposed observation-set mode against a Python restatement.

In the decomposed mode the analysis emulates a DA group of P ranks: the globe
is cut into lat x lon blocks (MPI_Dims_create, pro_info_get_indx), each block
holds the observations inside its box, and a column scans the blocks of its
neighbour set (comm_info_init, nearest_dist) in the reference's order.  The
restatement below is written independently of letkf_oracle.c, from the same
reference routines (code/x86/TradDA/DA/LETKF/src/letkf_init.F90:100-341,
DA/utils/pro_info.F90:96-175, EnDNN/src/module_da_parallel.F90:73-103,
LETKF/src/read_obs_mod.F90:73-165, LIB/REDIS/src/redis_wrapper.c:4089-4160,
LETKF/src/letkf_yb.F90:71-133).
"""
import math

import numpy as np
import pytest

from conftest import pkg
from oracle import oracle as O

f32 = np.float32


def _block_range(n, nb, b):
    sec, res = divmod(n, nb)
    if b - 1 < res:
        s = (b - 1) * (sec + 1) + 1
        return s, s + sec
    s = (b - 1) * sec + res + 1
    return s, s + sec - 1


def _glat(w, i):
    return f32(w.glat[i - 1]) if i <= w.nlat else f32(90.0)


def _glon(w, j):
    return f32(w.glon[j - 1]) if j <= w.nlon else f32(360.0)


def _dist_r8(x1, y1, x2, y2):
    pi = float(f32(math.atan(1.0)) * f32(4.0))
    a = float(f32(6371.393))
    r = lambda v: v / 180.0 * pi
    v = math.cos(r(x1)) * math.cos(r(x2)) * math.cos(r(y1) - r(y2)) + math.sin(r(x1)) * math.sin(r(x2))
    return a * math.acos(min(v, 1.0))


def _dist_r4(x1, y1, x2, y2):
    pi = f32(math.atan(1.0)) * f32(4.0)
    r = lambda v: f32(v) / f32(180.0) * pi
    c = lambda v: f32(math.cos(float(v)))
    s = lambda v: f32(math.sin(float(v)))
    v = c(r(x1)) * c(r(x2)) * c(r(y1) - r(y2)) + s(r(x1)) * s(r(x2))
    v = min(v, f32(1.0))
    return float(f32(6371.393) * f32(math.acos(float(v))))


def _nearest(w, NX, NY, bx1, by1, bx2, by2):
    xs1, xe1 = _block_range(w.nlat, NX, bx1)
    ys1, ye1 = _block_range(w.nlon, NY, by1)
    xs2, xe2 = _block_range(w.nlat, NX, bx2)
    ys2, ye2 = _block_range(w.nlon, NY, by2)
    if bx1 > bx2:
        tx1, tx2 = xs1, xe2 + 1
    elif bx1 < bx2:
        tx1, tx2 = xe1 + 1, xs2
    elif bx1 > NX // 2:
        tx1, tx2 = xe1 + 1, xe2 + 1
    else:
        tx1, tx2 = xs1, xs2
    lat1, lat2 = _glat(w, tx1), _glat(w, tx2)
    if abs(float(lat1)) > w.obs_polar:
        lat1 = f32(math.copysign(w.obs_polar, lat1))
    if abs(float(lat2)) > w.obs_polar:
        lat2 = f32(math.copysign(w.obs_polar, lat2))
    if by1 == by2:
        return _dist_r4(lat1, _glon(w, ys1), lat2, _glon(w, ys2))
    d1 = _dist_r4(lat1, _glon(w, ys1), lat2, _glon(w, ye2 % w.nlon + 1))
    d2 = _dist_r4(lat1, _glon(w, ye1 % w.nlon + 1), lat2, _glon(w, ys2))
    return min(d1, d2)


def _slots(w, NX, NY, bx, by):
    """Neighbour blocks of 1-based block (bx, by), 0-based ids, scan order."""
    c = w.loc_dist_km
    s_lat, e_lat = _block_range(w.nlat, NX, bx)
    s_lon, _ = _block_range(w.nlon, NY, by)
    y1 = float(_glon(w, s_lon))
    north = 0
    for t in range(bx - 1, 0, -1):
        _, te = _block_range(w.nlat, NX, t)
        if _dist_r8(float(_glat(w, s_lat)), y1, float(_glat(w, te + 1)), y1) > c:
            break
        north += 1
    south = 0
    for t in range(bx + 1, NX + 1):
        ts, _ = _block_range(w.nlat, NX, t)
        if _dist_r8(float(_glat(w, e_lat + 1)), y1, float(_glat(w, ts)), y1) > c:
            break
        south += 1
    out = []
    for i in range(-north, south + 1):
        tbx = bx + i
        west = east = 0
        tby = by
        while west <= (NY - 1) // 2:
            tby = (tby + NY - 2) % NY + 1
            if _nearest(w, NX, NY, bx, by, tbx, tby) > c:
                break
            west += 1
        tby = by
        while east <= (NY - 1) // 2:
            tby = tby % NY + 1
            if _nearest(w, NX, NY, bx, by, tbx, tby) > c:
                break
            east += 1
        if west + east > NY - 1:
            east -= 1
        out += [(tbx - 1) * NY + (by - 1 + j) % NY for j in range(-west, east + 1)]
    return out


def _bound(v):
    return float(f"{float(v):.5f}")


def _block_obs(w, NX, NY):
    lat, lon = w.obs["lat"], w.obs["lon"]
    blocks = []
    for bx in range(1, NX + 1):
        s, e = _block_range(w.nlat, NX, bx)
        inlat = (lat >= _bound(_glat(w, s))) & (lat <= _bound(_glat(w, e + 1)))
        for by in range(1, NY + 1):
            s2, e2 = _block_range(w.nlon, NY, by)
            inlon = (lon >= _bound(_glon(w, s2))) & (lon <= _bound(_glon(w, e2 + 1)))
            blocks.append(np.nonzero(inlat & inlon)[0])
    return blocks


def _decomposed_lists(w, NX, NY):
    blocks = _block_obs(w, NX, NY)
    slots = {}
    lists = []
    for cube in range(w.nlat * w.nlon):
        j, i = cube % w.nlat, cube // w.nlat
        bx = next(b for b in range(1, NX + 1) if _block_range(w.nlat, NX, b)[0] <= j + 1 <= _block_range(w.nlat, NX, b)[1])
        by = next(b for b in range(1, NY + 1) if _block_range(w.nlon, NY, b)[0] <= i + 1 <= _block_range(w.nlon, NY, b)[1])
        if (bx, by) not in slots:
            slots[(bx, by)] = _slots(w, NX, NY, bx, by)
        clat, clon = float(w.glat[j]), float(w.glon[i])
        out = []
        for b in slots[(bx, by)]:
            for o in blocks[b]:
                if not abs(w.obs["lat"][o]) <= w.obs_polar:
                    continue
                d = O.latlon_dist(float(w.obs["lat"][o]), float(w.obs["lon"][o]), clat, clon)
                if O.schr2(d / w.loc_dist_km) > 0:
                    out.append(o)
                    if len(out) >= w.max_obs:
                        break
            if len(out) >= w.max_obs:
                break
        lists.append(np.array(out, dtype=np.int32))
    return lists


def _edge_case(seed=11, nobs=500, max_obs=10000, loc=800.0):
    synthetic = pkg("synthetic")
    w = synthetic.small_case(nlat=12, nlon=24, nz=2, k=4, nobs=nobs, loc_dist_km=loc, seed=seed)
    # obs exactly on block edges (grid centres), south of the first row of
    # centres, west of the first column, at the poles and at lon 360
    extra_lat = [float(w.glat[0]), float(w.glat[6]), float(w.glat[4]), -89.9, 10.0, 90.0, -90.0, 0.0]
    extra_lon = [float(w.glon[0]), float(w.glon[12]), float(w.glon[8]), 30.0, 0.2, 15.0, 100.0, 360.0]
    n_extra = len(extra_lat)
    w.obs["lat"] = np.concatenate([w.obs["lat"], extra_lat])
    w.obs["lon"] = np.concatenate([w.obs["lon"], extra_lon])
    for key, fill in (("ph", 5e4), ("lev", 1), ("var", 0), ("yo", 1e5), ("rinv", 1e-4)):
        w.obs[key] = np.concatenate([w.obs[key], np.full(n_extra, fill, dtype=w.obs[key].dtype)])
    w.max_obs = max_obs
    return w


@pytest.mark.parametrize("nranks,expect", [(1, (1, 1)), (2, (1, 2)), (4, (2, 2)), (6, (2, 3)),
                                           (12, (3, 4)), (18, (3, 6)), (64, (8, 8)), (128, (8, 16))])
def test_decomp_dims_is_the_balanced_factor_pair(nranks, expect):
    assert O.decomp_dims(nranks) == expect


def test_single_rank_scans_its_box_twice():
    # one DA rank: the neighbour list holds the rank itself twice
    # (letkf_init.F90:146-163), and the box starts at the first centres
    w = _edge_case(max_obs=60)
    glob = O.Oracle(w)
    dec = O.Oracle(w, decomp=(1, 1))
    assert list(O.block_slots(dec, 0, 0)) == [0, 0]
    off_d, idx_d, _ = dec.local_obs()
    inbox = (w.obs["lat"] >= float(w.glat[0])) & (w.obs["lon"] >= float(w.glon[0]))
    keep = np.nonzero(inbox)[0]
    w2 = _edge_case(max_obs=10000)
    for key in w2.obs:
        w2.obs[key] = w2.obs[key][keep]
    off_g, idx_g, _ = O.Oracle(w2).local_obs()
    for cube in range(glob.ncubes):
        one = keep[idx_g[off_g[cube]:off_g[cube + 1]]]
        expect = np.concatenate([one, one])[:w.max_obs]
        assert np.array_equal(idx_d[off_d[cube]:off_d[cube + 1]], expect), cube


@pytest.mark.parametrize("dec,max_obs", [((2, 3), 10000), ((3, 4), 10000), ((4, 8), 10000),
                                         ((3, 4), 40)])
def test_decomposed_lists_match_restatement(dec, max_obs):
    w = _edge_case(max_obs=max_obs)
    orc = O.Oracle(w, decomp=dec)
    NX, NY = dec
    for bx in range(NX):
        for by in range(NY):
            assert list(O.block_slots(orc, bx, by)) == _slots(w, NX, NY, bx + 1, by + 1)
    off, idx, rloc = orc.local_obs()
    lists = _decomposed_lists(w, NX, NY)
    for cube, ref in enumerate(lists):
        assert np.array_equal(idx[off[cube]:off[cube + 1]], ref), cube
    # edge obs appear twice where both of their blocks are scanned
    assert any(len(np.unique(l)) < len(l) for l in lists) or max_obs < 100


def test_decomposed_mode_drops_far_blocks():
    # obs between c and 2c in blocks that are not neighbours are not scanned,
    # so the decomposed lists are sub-multisets of the global lists
    w = _edge_case(loc=900.0)
    off_g, idx_g, _ = O.Oracle(w).local_obs()
    off_d, idx_d, _ = O.Oracle(w, decomp=(4, 8)).local_obs()
    fewer = 0
    for cube in range(w.nlat * w.nlon):
        g = set(idx_g[off_g[cube]:off_g[cube + 1]].tolist())
        d = set(idx_d[off_d[cube]:off_d[cube + 1]].tolist())
        assert d <= g, cube
        fewer += len(d) < len(g)
    assert fewer > 0


def test_decomposed_analysis_runs_on_its_lists():
    w = _edge_case(nobs=200)
    orc = O.Oracle(w, decomp=(2, 3))
    xa, axa = orc.run()
    assert np.isfinite(xa).all() and np.isfinite(axa).all()
    with pytest.raises(RuntimeError):
        O.Oracle(w, decomp=(2, 3), cube_n=2).run()
