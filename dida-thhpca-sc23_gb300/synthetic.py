"""Seeded synthetic LETKF workloads (grids, background ensembles, observations).

The reference measures its LETKF only inside full coupled runs with Redis
observations; no public dataset exists for this path.  These generators build
the benchmark workloads from a written recipe instead:

* grid: cell centres at multiples of half the spacing, exact in float32
  (1 deg: lat -89.5..89.5, lon 0.5..359.5); 32 hybrid levels; state rows
  ps, then u, v, T on every level (the reference's 'ps,u,v,pt' order:
  code/x86/TradDA/DA/LETKF/src/letkf_init.F90:63-73).
* truth: T = 250 K + 30 cos(lat) + 20 random spherical harmonics of degree <= 8
  (2 K); u, v: degree <= 8 harmonic sums (10 m/s); ps = 1000 hPa +- 10 hPa.
* background: mean = truth + one draw of Gaussian-correlated noise (2000 km
  length scale; std 1 K, 2 m/s, 1 hPa); perturbations = k further draws with
  their sample mean removed, so the truth is statistically one more member.
* observations: variable uniform over ps/u/v/T, lat and lon uniform, level
  uniform in 1..nz (ps at the surface); value = H(truth) + N(0, sigma^2) with
  sigma = 1 K / 1.5 m/s / 1 hPa; R^-1 = 1/sigma^2 rounded through float32 as
  the reference's reader does (code/x86/TradDA/DA/LETKF/src/read_obs_mod.F90:438).

Random numbers come from numpy's PCG64 with seed 1000*config + instance.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

EARTH_A_KM = 6371.39306640625

# wrf_l32 hybrid coefficients: the reference writes them as default-real
# (float32) literals (code/x86/TradDA/DA/utils/vert_coord_mod.F90:330-402),
# so the values it computes with are these literals rounded to float32.
_WRF_L32_HYAI = [
    0.0000000000000000, 0.0027008056640625, 0.0076868347823620, 0.0158526937798342,
    0.0276367470939261, 0.0414515552099706, 0.0562277844155789, 0.0724737972365225,
    0.0893795253309864, 0.1063548465048298, 0.1254725257849640, 0.1479642011314251,
    0.1744233770857367, 0.2054476619883455, 0.2362396334209435, 0.2617261684535087,
    0.2783057827853432, 0.2816243248017372, 0.2683280168286641, 0.2429473354807992,
    0.2108099294331058, 0.1759998110016148, 0.1415334037742616, 0.1095123294032484,
    0.0812761592574764, 0.0575423961814687, 0.0385285881906738, 0.0240694984015316,
    0.0137226170696702, 0.0068720184783044, 0.0027973066609278, 0.0007580797514921,
    0.0000000000000000,
]
_WRF_L32_HYBI = [
    0.0000000000000000, 0.0000000000000000, 0.0000000000000000, 0.0000000000000000,
    0.0000000000000000, 0.0000000000000000, 0.0000000000000000, 0.0000000000000000,
    0.0000000000000000, 0.0000000000000000, 0.0000000000000000, 0.0000000000000000,
    0.0000000000000000, 0.0001056069805219, 0.0059397906834944, 0.0235374270991938,
    0.0576439176162314, 0.1139578493851603, 0.1932313936022966, 0.2808764820852269,
    0.3715629284436812, 0.4612091687348547, 0.5467954414732804, 0.6262219272258057,
    0.6981497395977654, 0.7618575996945027, 0.8171268253424389, 0.8641240158900223,
    0.9032994538662682, 0.9352560448161740, 0.9607227915792738, 0.9804356127137464,
    1.0000000000000000,
]
WRF_L32_HYAI = np.asarray(_WRF_L32_HYAI, dtype=np.float32).astype(np.float64)
WRF_L32_HYBI = np.asarray(_WRF_L32_HYBI, dtype=np.float32).astype(np.float64)
P0_PA = 1.0e5
# GMCORE's default model-top pressure (code/x86/TradDA/ATM/utils/namelist_mod.F90:78)
PTOP_PA = 219.4

VAR_PS, VAR_U, VAR_V, VAR_T = 0, 1, 2, 3
OBS_SIGMA = {VAR_PS: 100.0, VAR_U: 1.5, VAR_V: 1.5, VAR_T: 1.0}      # Pa, m/s, m/s, K
NOISE_STD = {VAR_PS: 100.0, VAR_U: 2.0, VAR_V: 2.0, VAR_T: 1.0}


def hybrid_coefficients(nz: int):
    """Interface coefficients (hyai, hybi) for nz levels (wrf_l32 for nz=32,
    else a smooth hybrid profile with the same end points)."""
    if nz == 32:
        return WRF_L32_HYAI.copy(), WRF_L32_HYBI.copy()
    s = np.linspace(0.0, 1.0, nz + 1)
    hybi = np.clip((s - 0.2) / 0.8, 0.0, 1.0) ** 1.5
    hyai = s - hybi
    return (hyai.astype(np.float32).astype(np.float64),
            hybi.astype(np.float32).astype(np.float64))


def make_grid(res_deg: float):
    """Cell-centre latitudes/longitudes (float32) of a global res_deg grid."""
    nlat = int(round(180.0 / res_deg))
    nlon = int(round(360.0 / res_deg))
    glat = (-90.0 + res_deg * (np.arange(nlat) + 0.5)).astype(np.float32)
    glon = (res_deg * (np.arange(nlon) + 0.5)).astype(np.float32)
    return glat, glon


def _legendre_normalized(lmax: int, x: np.ndarray) -> np.ndarray:
    """Fully normalized associated Legendre functions P[l, m, :] (4 pi norm / 4 pi)."""
    p = np.zeros((lmax + 1, lmax + 1, x.size))
    s = np.sqrt(np.maximum(0.0, 1.0 - x * x))
    p[0, 0] = math.sqrt(1.0 / (4.0 * math.pi))
    for m in range(1, lmax + 1):
        p[m, m] = math.sqrt((2 * m + 1) / (2.0 * m)) * s * p[m - 1, m - 1]
    for m in range(0, lmax):
        p[m + 1, m] = math.sqrt(2 * m + 3) * x * p[m, m]
    for m in range(0, lmax + 1):
        for l in range(m + 2, lmax + 1):
            a = math.sqrt((4.0 * l * l - 1.0) / (l * l - m * m))
            b = math.sqrt(((l - 1.0) ** 2 - m * m) / (4.0 * (l - 1.0) ** 2 - 1.0))
            p[l, m] = a * (x * p[l - 1, m] - b * p[l - 2, m])
    return p


def sh_basis(lmax: int, lat_deg: np.ndarray, lon_deg: np.ndarray):
    """Real orthonormal spherical harmonics at points (lat, lon).
    Returns (basis [npts, nharm], degree [nharm])."""
    x = np.sin(np.deg2rad(np.asarray(lat_deg, dtype=np.float64)))
    lam = np.deg2rad(np.asarray(lon_deg, dtype=np.float64))
    p = _legendre_normalized(lmax, x)
    cols, degs = [], []
    for l in range(lmax + 1):
        cols.append(p[l, 0])
        degs.append(l)
        for m in range(1, l + 1):
            cols.append(math.sqrt(2.0) * p[l, m] * np.cos(m * lam))
            degs.append(l)
            cols.append(math.sqrt(2.0) * p[l, m] * np.sin(m * lam))
            degs.append(l)
    return np.stack(cols, axis=1), np.asarray(degs)


def grid_points(glat, glon):
    """(lat, lon) of every column, column index = ilat + nlat*ilon."""
    lat = np.tile(glat.astype(np.float64), glon.size)
    lon = np.repeat(glon.astype(np.float64), glat.size)
    return lat, lon


def _noise_spectrum(lmax: int, degs: np.ndarray, length_km: float) -> np.ndarray:
    """Per-harmonic std giving unit pointwise variance and a Gaussian
    correlation of the given length scale."""
    l = np.arange(lmax + 1, dtype=np.float64)
    var_l = np.exp(-0.5 * l * (l + 1) * (length_km / EARTH_A_KM) ** 2)
    total = np.sum(var_l * (2 * l + 1) / (4 * math.pi))
    return np.sqrt(var_l[degs] / total)


@dataclass
class Workload:
    """One analysis instance: grid, parameters, background and observations."""
    name: str
    glat: np.ndarray
    glon: np.ndarray
    nz: int
    k: int
    hyai: np.ndarray
    hybi: np.ndarray
    xb: np.ndarray          # [ncol][n][k] perturbations
    axb: np.ndarray         # [ncol][n] mean
    truth: np.ndarray       # [ncol][n]
    obs: dict               # lat, lon, ph, lev, var, yo, rinv
    loc_dist_km: float      # Gaspari-Cohn half-width c; obs kept out to 2c
    inflation: float
    nvar2d: int = 1
    nvar3d: int = 3
    p0: float = P0_PA
    ptop: float = PTOP_PA
    ps_row: int = 0
    obs_polar: float = 91.0
    gc_filter: int = 1
    max_obs: int = 10000
    h_mode: int = 1
    extra: dict = field(default_factory=dict)

    @property
    def nlat(self):
        return self.glat.size

    @property
    def nlon(self):
        return self.glon.size

    @property
    def ncol(self):
        return self.glat.size * self.glon.size

    @property
    def n(self):
        return self.nvar2d + self.nvar3d * self.nz


def _truth_fields(rng, glat, glon, nz, lmax_truth=8):
    lat, lon = grid_points(glat, glon)
    basis, degs = sh_basis(lmax_truth, lat, lon)
    nh = basis.shape[1]
    nonconst = np.nonzero(degs >= 1)[0]

    def harmonic_sum(amplitude, nterms=20):
        pick = rng.choice(nonconst, size=nterms, replace=False)
        coef = rng.standard_normal(nterms)
        f = basis[:, pick] @ coef
        return amplitude * f / max(np.sqrt(np.mean(f * f)), 1e-30)

    ncol = lat.size
    n = 1 + 3 * nz
    truth = np.empty((ncol, n))
    truth[:, 0] = 100000.0 + harmonic_sum(1000.0)
    coslat = np.cos(np.deg2rad(lat))
    for z in range(nz):
        truth[:, 1 + z] = harmonic_sum(10.0)
        truth[:, 1 + nz + z] = harmonic_sum(10.0)
        truth[:, 1 + 2 * nz + z] = 250.0 + 30.0 * coslat + harmonic_sum(2.0)
    del nh
    return truth


def _row_std(nz):
    return np.concatenate([[NOISE_STD[VAR_PS]], np.full(nz, NOISE_STD[VAR_U]),
                           np.full(nz, NOISE_STD[VAR_V]), np.full(nz, NOISE_STD[VAR_T])])


def _correlated_noise(rng, basis_t, spec, nfields):
    """nfields independent correlated fields [ncol, nfields] of unit std."""
    coef = rng.standard_normal((basis_t.shape[0], nfields)) * spec[:, None]
    return basis_t.T @ coef


def horizontal_interp(glat, glon, field_cols, lat, lon, rows):
    """Bilinear value of a single state (no members) at points, using the
    reference's grid search and weights (letkf_obs.F90:187-243) with rows
    clamped at the poles and columns periodic.  field_cols is [ncol][n]."""
    nlat, nlon = glat.size, glon.size
    glat_ext = np.concatenate([glat, np.float32([90.0])])
    glon_ext = np.concatenate([glon, np.float32([360.0])])
    tx = np.searchsorted(glat_ext.astype(np.float64), lat, side="left") + 1
    ty = np.searchsorted(glon_ext.astype(np.float64), lon, side="left") + 1
    dlat = (glat_ext[np.maximum(tx - 1, 1)] - glat_ext[np.maximum(tx - 2, 0)]).astype(np.float64)
    dlon = (glon_ext[np.maximum(ty - 1, 1)] - glon_ext[np.maximum(ty - 2, 0)]).astype(np.float64)
    ax = np.where(tx > 1, (dlat - lat + glat_ext[np.maximum(tx - 2, 0)].astype(np.float64)) / dlat, 0.0)
    ay = np.where(ty > 1, (dlon - lon + glon_ext[np.maximum(ty - 2, 0)].astype(np.float64)) / dlon, 0.0)
    la0 = np.clip(tx - 2, 0, nlat - 1)
    la1 = np.clip(tx - 1, 0, nlat - 1)
    lo0 = (ty - 2) % nlon
    lo1 = (ty - 1) % nlon
    f = field_cols
    v11 = f[la0 + nlat * lo0, rows]
    v21 = f[la1 + nlat * lo0, rows]
    v12 = f[la0 + nlat * lo1, rows]
    v22 = f[la1 + nlat * lo1, rows]
    r1 = v11 * ax + v21 * (1 - ax)
    r2 = v12 * ax + v22 * (1 - ax)
    return r1 * ay + r2 * (1 - ay)


def _make_obs(rng, glat, glon, nz, hyai, hybi, truth, nobs, boxes=(), box_factor=1.0):
    """Observations: uniform over the globe plus extra density in boxes.
    boxes: (lon0, lon1, lat0, lat1) in degrees; the density inside each box is
    box_factor times the density outside."""
    lat = rng.uniform(-90.0, 90.0, nobs)
    lon = rng.uniform(0.0, 360.0, nobs)
    if boxes and box_factor > 1.0:
        # a box of area fraction f gets density ratio R when it receives an
        # extra (R-1) f / (1 + sum (R-1) f) share of all obs
        fracs = [((b[1] - b[0]) / 360.0) * ((b[3] - b[2]) / 180.0) for b in boxes]
        extra = [(box_factor - 1.0) * f for f in fracs]
        denom = 1.0 + sum(extra)
        start = 0
        order = rng.permutation(nobs)
        for b, e in zip(boxes, extra):
            m = int(round(nobs * e / denom))
            sel = order[start:start + m]
            start += m
            lon[sel] = rng.uniform(b[0], b[1], m)
            lat[sel] = rng.uniform(b[2], b[3], m)
    lat = lat.astype(np.float32).astype(np.float64)
    lon = np.mod(lon, 360.0).astype(np.float32).astype(np.float64)
    var = rng.integers(0, 4, nobs).astype(np.int32)
    lev = rng.integers(1, nz + 1, nobs).astype(np.int32)
    lev[var == VAR_PS] = nz
    rows = np.where(var == VAR_PS, 0, 1 + (var - 1) * nz + (lev - 1))
    clean = horizontal_interp(glat, glon, truth, lat, lon, rows)
    ps_obs = horizontal_interp(glat, glon, truth, lat, lon, np.zeros(nobs, dtype=np.int64))
    ph_if = lambda i: hyai[i] * (P0_PA - PTOP_PA) + hybi[i] * (ps_obs - PTOP_PA) + PTOP_PA
    ph = 0.5 * (ph_if(lev - 1) + ph_if(lev))
    ph = np.where(var == VAR_PS, ps_obs, ph)
    sigma = np.array([OBS_SIGMA[v] for v in range(4)], dtype=np.float32)[var]
    yo = clean + sigma.astype(np.float64) * rng.standard_normal(nobs)
    rinv = (np.float32(1.0) / (sigma * sigma)).astype(np.float64)
    return dict(lat=lat, lon=lon, ph=ph, lev=lev, var=var, yo=yo, rinv=rinv)


def _members_on_device(basis, coef2d, device, chunk_cols=1 << 16):
    """xb = basis @ coef as a float64 torch tensor [ncol][n*k] on `device`,
    built a block of columns at a time (the host never holds the ensemble)."""
    import torch
    ncol = basis.shape[0]
    coef_d = torch.from_numpy(np.ascontiguousarray(coef2d)).to(device)
    xb = torch.empty((ncol, coef2d.shape[1]), dtype=torch.float64, device=device)
    for c0 in range(0, ncol, chunk_cols):
        c1 = min(ncol, c0 + chunk_cols)
        b = torch.from_numpy(np.ascontiguousarray(basis[c0:c1])).to(device)
        torch.matmul(b, coef_d, out=xb[c0:c1])
    return xb


def generate(name, res_deg, nz, k, nobs, loc_dist_km, inflation, seed,
             boxes=(), box_factor=1.0, lmax_noise=12, noise_len_km=2000.0, device=None, members=True):
    """Build one analysis instance (see the module docstring for the recipe).
    With a torch `device` the members xb are built there (a torch float64
    tensor [ncol][n][k]) from the same random draws, for ensembles larger than
    host memory; everything else stays on the host.  members=False draws the
    same random numbers but leaves xb None (the grid, mean and observations
    are those of the full instance: for checks of the observation lists)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    glat, glon = make_grid(res_deg)
    hyai, hybi = hybrid_coefficients(nz)
    truth = _truth_fields(rng, glat, glon, nz)
    lat, lon = grid_points(glat, glon)
    basis, degs = sh_basis(lmax_noise, lat, lon)
    basis_t = np.ascontiguousarray(basis.T)
    spec = _noise_spectrum(lmax_noise, degs, noise_len_km)
    n = 1 + 3 * nz
    std = _row_std(nz)
    ncol = lat.size
    # mean error: one correlated draw per state row
    axb = truth + _correlated_noise(rng, basis_t, spec, n) * std[None, :]
    # members: coefficient matrix [nharm][n*k] so that basis @ coef is [ncol][n][k]
    coef = rng.standard_normal((basis_t.shape[0], n, k))
    coef -= coef.mean(axis=2, keepdims=True)      # sample mean removed (linear)
    coef *= spec[:, None, None] * std[None, :, None]
    if not members:
        xb = None
    elif device is None:
        xb = (basis_t.T @ coef.reshape(basis_t.shape[0], n * k)).reshape(ncol, n, k)
    else:
        xb = _members_on_device(basis, coef.reshape(basis_t.shape[0], n * k), device).view(ncol, n, k)
    del basis, basis_t
    obs = _make_obs(rng, glat, glon, nz, hyai, hybi, truth, nobs, boxes, box_factor)
    return Workload(name=name, glat=glat, glon=glon, nz=nz, k=k, hyai=hyai, hybi=hybi,
                    xb=xb, axb=axb, truth=truth, obs=obs, loc_dist_km=loc_dist_km,
                    inflation=inflation)


# Benchmark configurations.  The localization radius of each configuration is
# the cut-off 2c of the Gaspari-Cohn function, so c = radius / 2.
CLUSTER_BOX_1 = ((0.0, 60.0, -10.0, 30.0),)
CLUSTERS_4 = ((100.0, 140.0, 20.0, 50.0), (260.0, 300.0, 25.0, 50.0), (0.0, 30.0, 35.0, 60.0))
INSTANCES_3 = [  # (res_deg, k, nobs, radius_km, inflation)
    (2.0, 32, 20_000, 1000.0, 1.10), (2.0, 48, 40_000, 1000.0, 1.10),
    (1.5, 48, 60_000, 1000.0, 1.10), (1.5, 64, 100_000, 1000.0, 1.10),
    (1.0, 64, 200_000, 800.0, 1.08), (1.0, 96, 150_000, 800.0, 1.08),
    (0.75, 32, 300_000, 800.0, 1.08), (0.75, 96, 400_000, 800.0, 1.08),
]


def config(cfg: int, instance: int = 0, nobs: int | None = None, res_deg: float | None = None,
           device=None, members: bool = True):
    """Workload of a benchmark configuration (0, 1, 2, the instances of 3, and
    4).  nobs overrides the observation count and res_deg the grid spacing
    (smaller cases with the same observation density when both are scaled,
    e.g. for profiling).  device: build the members on this torch device
    (configuration 4's ensemble, 103 GB in float64, is built only there).
    members=False: the same instance without its members (see generate)."""
    if cfg == 4:
        res = res_deg or 0.25
        no = nobs if nobs is not None else int(round(4_000_000 * (0.25 / res) ** 2))
        return generate("cfg4", res, 32, 128, no, 250.0, 1.05, 4000, boxes=CLUSTERS_4,
                        box_factor=10.0, device=device, members=members)
    seed = 1000 * cfg + instance
    if cfg == 0:
        return generate("cfg0", res_deg or 2.0, 32, 32, nobs or 20_000, 500.0, 1.1, seed)
    if cfg in (1, 2):
        # configuration 2 runs on configuration 1's inputs
        return generate("cfg1", res_deg or 1.0, 32, 64, nobs or 200_000, 400.0, 1.08,
                        1000 + instance, boxes=CLUSTER_BOX_1, box_factor=4.0)
    if cfg == 3:
        res, k, no, radius, infl = INSTANCES_3[instance]
        return generate(f"cfg3.{instance}", res, 32, k, nobs or no, radius / 2, infl, seed)
    raise ValueError(f"configuration {cfg} has no host generator")


def small_case(nlat=12, nlon=24, nz=4, k=8, nobs=300, loc_dist_km=900.0, inflation=1.1,
               seed=7, h_mode=1):
    """A small instance for unit tests (a coarse global grid)."""
    res = 180.0 / nlat
    assert abs(360.0 / nlon - res) < 1e-9
    w = generate(f"small{nlat}x{nlon}", res, nz, k, nobs, loc_dist_km, inflation, seed,
                 lmax_noise=6, noise_len_km=3000.0)
    w.h_mode = h_mode
    return w
