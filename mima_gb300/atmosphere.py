"""Seeded synthetic atmospheres in the form MiMA's ``run_rrtmg`` hands to RRTMG.

The reference drives RRTMG from ``run_rrtmg`` (``src/atmos_param/rrtm_radiation/
rrtm_radiation.f90:464-834``), which reshapes the GCM state to (column, layer)
with layer 1 at the surface (``:649-664``), converts pressure to hPa, fixes the
top interface (``:655-656``) and clamps ``h2o >= 2e-7``, ``100 <= T <= 370``
(``:673-677``).  It passes *specific humidity* in the ``h2ovmr`` argument and the
O3 *mass* mixing ratio in ``o3vmr`` (``rrtmg_lw_rad.nomcica.f90:775-778``).
This generator produces exactly that form.

Memory layout: every 2-D field is a C-contiguous ``(nlev, ncol)`` array, i.e. the
Fortran ``(ncol, nlev)`` column-major layout with the column index fastest, which
is what the C-ABI takes.  Columns are ordered longitude-fastest.

Profile recipe (the published benchmark configurations name no dataset; these
seeded profiles stand in for MiMA's state):

* Gaussian grid: T42 128x64, T85 256x128, T170 512x256 (Gauss-Legendre latitudes).
* Interfaces log-spaced in p from ps = 1000 hPa to the top (0.1 hPa for 40
  layers, 0.01 hPa for 60); layer pressure = geometric mean of its interfaces.
* Ts = 240 + 60 cos^2(lat) + N(0, sigma).
* Constant lapse rate 6.5 K/km in hydrostatic form T = Ts (p/ps)^(R Gamma / g)
  (R = 287.04, g = 9.80) down to a 200 K tropopause, isothermal above;
  interface temperatures are linear in ln p between layers, Ts at the surface.
* q = RH qsat(T, p) (Bolton 1980 saturation vapour pressure) below the
  tropopause, RH = 0.7 or U(0.2, 0.95) per column; 3e-6 kg/kg at and above the
  tropopause and as a lower bound everywhere.
* O3 vmr = 8e-6 exp(-0.5 log10(p / 10 hPa)^2), passed as mass mixing ratio.
* CO2 300 ppmv, every other gas zero; emissivity 1; all SW albedos 0.27.
* cos(zenith): annual mean of the daily-mean value of ``astro.f90``
  ((aa h + bb sin h)/pi), 365 declinations, obliquity 23.439 deg.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

AMDO = 0.603428  # dry air / ozone molecular weight ratio (rrtmg_lw_rad.nomcica.f90)
R_DRY = 287.04
GRAV = 9.80
LAPSE = 6.5e-3
T_TROP = 200.0


@dataclass
class Atmosphere:
    """Inputs of ``rrtmg_lw`` / ``rrtmg_sw`` for ``ncol`` columns (see module doc)."""
    ncol: int
    nlay: int
    play: np.ndarray      # (nlay, ncol) hPa
    plev: np.ndarray      # (nlay+1, ncol) hPa
    tlay: np.ndarray      # (nlay, ncol) K
    tlev: np.ndarray      # (nlay+1, ncol) K
    tsfc: np.ndarray      # (ncol,) K
    h2o: np.ndarray       # (nlay, ncol) specific humidity kg/kg
    o3: np.ndarray        # (nlay, ncol) O3 mass mixing ratio
    co2: np.ndarray       # (nlay, ncol) vmr
    ch4: np.ndarray
    n2o: np.ndarray
    o2: np.ndarray
    cfc11: np.ndarray
    cfc12: np.ndarray
    cfc22: np.ndarray
    ccl4: np.ndarray
    emis: np.ndarray      # (16, ncol)
    asdir: np.ndarray     # (ncol,)
    asdif: np.ndarray
    aldir: np.ndarray
    aldif: np.ndarray
    coszen: np.ndarray    # (ncol,)
    scon: float = 1360.0
    adjes: float = 1.0
    dyofyr: int = 0
    meta: dict = field(default_factory=dict)

    def subset(self, idx) -> "Atmosphere":
        idx = np.asarray(idx)
        kw = {}
        for k, v in self.__dict__.items():
            if isinstance(v, np.ndarray):
                kw[k] = np.ascontiguousarray(v[..., idx])
            else:
                kw[k] = v
        kw["ncol"] = int(idx.size)
        kw["meta"] = dict(self.meta, subset=True)
        return Atmosphere(**kw)


GRIDS = {"T42": (128, 64), "T85": (256, 128), "T170": (512, 256)}


def gaussian_latitudes(nlat: int) -> np.ndarray:
    x, _ = np.polynomial.legendre.leggauss(nlat)
    return np.arcsin(x)[::-1]  # north to south, radians


def annual_mean_coszen(lat: np.ndarray, obliquity_deg: float = 23.439) -> np.ndarray:
    """Annual mean of the daily-mean cos(zenith) of astro.f90's daily formula
    (evaluated once per distinct latitude: the grids repeat each latitude for
    every longitude)."""
    lat = np.asarray(lat, dtype=np.float64)
    uniq, inv = np.unique(lat, return_inverse=True)
    if uniq.size < lat.size:
        return annual_mean_coszen(uniq, obliquity_deg)[inv.reshape(lat.shape)]
    eps = np.deg2rad(obliquity_deg)
    days = np.arange(365)
    dec = np.arcsin(np.sin(eps) * np.sin(2.0 * np.pi * days / 365.0))
    phi = lat[:, None]
    d = dec[None, :]
    aa = np.sin(phi) * np.sin(d)
    bb = np.cos(phi) * np.cos(d)
    with np.errstate(divide="ignore", invalid="ignore"):
        x = -np.tan(phi) * np.tan(d)
    h = np.arccos(np.clip(x, -1.0, 1.0))
    cosz = (aa * h + bb * np.sin(h)) / np.pi
    return np.clip(cosz, 0.0, None).mean(axis=1)


def qsat(T: np.ndarray, p_hpa: np.ndarray) -> np.ndarray:
    es = 6.112 * np.exp(17.67 * (T - 273.15) / (T - 29.65))
    es = np.minimum(es, 0.5 * p_hpa)
    return 0.622 * es / (p_hpa - 0.378 * es)


def make_columns(lat: np.ndarray, nlay: int, p_top: float, rng: np.random.Generator,
                 ts_sigma: float, rh=0.7, ps: float = 1000.0) -> Atmosphere:
    """Build columns at latitudes ``lat`` (radians, one per column)."""
    ncol = lat.size
    # Interfaces, surface first (RRTM order); layer = geometric mean.
    plev1 = np.exp(np.linspace(np.log(ps), np.log(p_top), nlay + 1))
    play1 = np.sqrt(plev1[:-1] * plev1[1:])
    plev = np.repeat(plev1[:, None], ncol, axis=1)
    play = np.repeat(play1[:, None], ncol, axis=1)

    ts = 240.0 + 60.0 * np.cos(lat) ** 2 + ts_sigma * rng.standard_normal(ncol)
    kappa = R_DRY * LAPSE / GRAV
    tl = ts[None, :] * (play / ps) ** kappa
    strat = tl <= T_TROP
    tlay = np.maximum(tl, T_TROP)
    lp_lay = np.log(play)
    lp_lev = np.log(plev)
    tlev = np.empty((nlay + 1, ncol))
    tlev[0] = ts
    w = (lp_lev[1:-1] - lp_lay[:-1]) / (lp_lay[1:] - lp_lay[:-1])
    tlev[1:-1] = tlay[:-1] + w * (tlay[1:] - tlay[:-1])
    tlev[-1] = tlay[-1]

    if np.isscalar(rh):
        rhc = np.full(ncol, float(rh))
    else:
        rhc = np.asarray(rh, dtype=np.float64)
    q = rhc[None, :] * qsat(tlay, play)
    q = np.where(strat, 3.0e-6, q)
    q = np.maximum(q, 3.0e-6)

    o3vmr = 8.0e-6 * np.exp(-0.5 * np.log10(play / 10.0) ** 2)
    z = np.zeros((nlay, ncol))
    return Atmosphere(
        ncol=ncol, nlay=nlay, play=play, plev=plev, tlay=tlay, tlev=tlev, tsfc=ts,
        h2o=q, o3=o3vmr / AMDO, co2=np.full((nlay, ncol), 300.0e-6), ch4=z.copy(),
        n2o=z.copy(), o2=z.copy(), cfc11=z.copy(), cfc12=z.copy(), cfc22=z.copy(),
        ccl4=z.copy(), emis=np.ones((16, ncol)), asdir=np.full(ncol, 0.27),
        asdif=np.full(ncol, 0.27), aldir=np.full(ncol, 0.27), aldif=np.full(ncol, 0.27),
        coszen=annual_mean_coszen(lat), scon=1360.0, adjes=1.0, dyofyr=0)


def grid_atmosphere(grid: str, nlay: int, seed: int, ts_sigma: float = 2.0,
                    rh_random: bool = False) -> Atmosphere:
    """Full Gaussian grid (longitude fastest)."""
    nlon, nlat = GRIDS[grid]
    p_top = 0.1 if nlay <= 40 else 0.01
    rng = np.random.default_rng(seed)
    lat = np.repeat(gaussian_latitudes(nlat), nlon)
    rh = rng.uniform(0.2, 0.95, size=lat.size) if rh_random else 0.7
    atm = make_columns(lat, nlay, p_top, rng, ts_sigma, rh=rh)
    atm.meta.update(grid=grid, nlon=nlon, nlat=nlat, seed=seed, ts_sigma=ts_sigma,
                    rh_random=rh_random, p_top=p_top)
    return atm


# The five workload configurations (seed = 12345 + index).
CONFIGS = {
    0: dict(name="T42x40 FP64", grid="T42", nlay=40, ts_sigma=2.0, rh_random=False),
    1: dict(name="T85x40 FP64 via C-ABI + CUDA graph", grid="T85", nlay=40, ts_sigma=2.0, rh_random=False),
    2: dict(name="T170x60 FP32-split", grid="T170", nlay=60, ts_sigma=5.0, rh_random=True),
    3: dict(name="T42x40 adjoint (256 columns)", grid="T42", nlay=40, ts_sigma=2.0, rh_random=False),
    # 32 members x 32768 columns = 1,048,576 columns; each member has the T170
    # configuration's column (60 layers, top 0.01 hPa) on the 256 x 128 Gaussian
    # latitudes, with its own seed and Ts noise 3 K
    4: dict(name="1048576x60 stress (32 members of 32768 T170-like columns)", grid="T85", nlay=60, ts_sigma=3.0,
            rh_random=False),
}


def config_atmosphere(index: int, member: int = 0) -> Atmosphere:
    c = CONFIGS[index]
    seed = 12345 + index + 1000 * member
    atm = grid_atmosphere(c["grid"], c["nlay"], seed, c["ts_sigma"], c["rh_random"])
    if index == 3:
        idx = np.random.default_rng(seed).choice(atm.ncol, size=256, replace=False)
        atm = atm.subset(np.sort(idx))
    atm.meta["config"] = index
    return atm


def small_atmosphere(ncol: int, nlay: int = 40, seed: int = 7, ts_sigma: float = 2.0,
                     rh_random: bool = True) -> Atmosphere:
    """Columns at random latitudes (tests)."""
    rng = np.random.default_rng(seed)
    lat = np.arcsin(rng.uniform(-1.0, 1.0, size=ncol))
    p_top = 0.1 if nlay <= 40 else 0.01
    rh = rng.uniform(0.2, 0.95, size=ncol) if rh_random else 0.7
    atm = make_columns(lat, nlay, p_top, rng, ts_sigma, rh=rh)
    atm.meta.update(seed=seed, small=True)
    return atm



def cloud_physics_fields(atm: Atmosphere, seed: int) -> dict:
    """Seeded overcast clouds for the cloud-physics paths, (nlay, ncol) arrays:
    about 35 % of the layers below 100 hPa overcast (cover 1, so that the
    non-McICA SW takes them too); ice water path up to ~120 g/m2 above
    600 hPa, liquid up to ~140 g/m2 below 300 hPa (both in between), one
    cloudy layer in twenty without water; ice effective sizes 14-125 um and
    liquid radii 3-55 um, inside every parameterisation's range."""
    rng = np.random.default_rng(seed)
    L, n = atm.nlay, atm.ncol
    cf = np.where((rng.uniform(size=(L, n)) < 0.35) & (atm.play > 100.0), 1.0, 0.0)
    ciwp = np.where(atm.play < 600.0, rng.uniform(0.0, 40.0, (L, n)) ** 1.3, 0.0)
    clwp = np.where(atm.play > 300.0, rng.uniform(0.0, 60.0, (L, n)) ** 1.2, 0.0)
    dry = rng.uniform(size=(L, n)) < 0.05
    ciwp[dry] = 0.0
    clwp[dry] = 0.0
    return dict(cldfr=cf, cicewp=ciwp, cliqwp=clwp, reice=rng.uniform(14.0, 125.0, (L, n)),
                reliq=rng.uniform(3.0, 55.0, (L, n)))


@dataclass
class GcmSlab:
    """One GCM slab as MiMA's ``run_rrtmg`` receives it
    (``rrtm_radiation.f90:464-510``; the heights feed ``interp_temp``,
    ``:420-460``).  Every array is C-ordered (level, latitude, longitude), i.e.
    Fortran (si, sj, sk) with the longitude fastest; level 0 is the model top.
    Pressures in Pa, heights in m, lat/lon in radians."""
    si: int
    sj: int
    sk: int
    lat: np.ndarray          # (sj, si)
    lon: np.ndarray          # (sj, si)
    p_full: np.ndarray       # (sk, sj, si)
    p_half: np.ndarray       # (sk+1, sj, si), top interface 0 Pa as in MiMA
    z_full: np.ndarray       # (sk, sj, si)
    z_half: np.ndarray       # (sk+1, sj, si), 0 at the top as in MiMA (unused there)
    t: np.ndarray            # (sk, sj, si) K
    q: np.ndarray            # (sk, sj, si) kg/kg
    o3: np.ndarray | None    # (sk, sj, si) O3 mass mixing ratio, or None (o3_val)
    t_surf_rad: np.ndarray   # (sj, si) K
    albedo: np.ndarray       # (sj, si)
    rrtm_precip: np.ndarray | None  # (sj, si) accumulated precipitation (do_precip_albedo)
    tdt: np.ndarray          # (sk, sj, si) K/s, the tendency before radiation


def gcm_slab(nlon: int, nlat: int, nlev: int, seed: int, p_top: float = 10.0, ts_sigma: float = 2.0,
             ozone: bool = True) -> GcmSlab:
    """A seeded slab on nlon x nlat Gaussian points: surface pressure
    1000 hPa + N(0, 10 hPa); half levels 0 Pa at the top, then log-spaced from
    ``p_top`` (Pa) x ps/1000 hPa to ps; full levels the geometric mean of
    their interfaces (half the first interface for the top level); the
    temperature, humidity (RH U(0.2, 0.95)) and ozone profiles of
    :func:`make_columns`; hydrostatic heights; albedo 0.27 +- 0.05; random
    precipitation sums and a random prior tendency."""
    rng = np.random.default_rng(seed)
    lat = np.repeat(gaussian_latitudes(nlat)[:, None], nlon, axis=1)
    lon = np.repeat((2.0 * np.pi * np.arange(nlon) / nlon)[None, :], nlat, axis=0)
    ps = 1.0e5 + 1.0e3 * rng.standard_normal((nlat, nlon))
    sig = np.exp(np.linspace(np.log(p_top / 1.0e5), 0.0, nlev))
    p_half = np.empty((nlev + 1, nlat, nlon))
    p_half[0] = 0.0
    p_half[1:] = sig[:, None, None] * ps[None]
    p_full = np.empty((nlev, nlat, nlon))
    p_full[0] = 0.5 * p_half[1]
    p_full[1:] = np.sqrt(p_half[1:-1] * p_half[2:])
    ts = 240.0 + 60.0 * np.cos(lat) ** 2 + ts_sigma * rng.standard_normal((nlat, nlon))
    tl = ts[None] * (p_full / ps[None]) ** (R_DRY * LAPSE / GRAV)
    strat = tl <= T_TROP
    t = np.maximum(tl, T_TROP)
    z_half = np.zeros((nlev + 1, nlat, nlon))
    z_full = np.empty((nlev, nlat, nlon))
    for k in range(nlev - 1, -1, -1):
        z_full[k] = z_half[k + 1] + R_DRY * t[k] / GRAV * np.log(p_half[k + 1] / p_full[k])
        if k > 0:
            z_half[k] = z_half[k + 1] + R_DRY * t[k] / GRAV * np.log(p_half[k + 1] / p_half[k])
    rh = rng.uniform(0.2, 0.95, size=(nlat, nlon))
    q = rh[None] * qsat(t, p_full / 100.0)
    q = np.maximum(np.where(strat, 3.0e-6, q), 3.0e-6)
    o3 = 8.0e-6 * np.exp(-0.5 * np.log10(p_full / 1000.0) ** 2) / AMDO if ozone else None
    return GcmSlab(si=nlon, sj=nlat, sk=nlev, lat=lat, lon=lon, p_full=p_full, p_half=p_half, z_full=z_full,
                   z_half=z_half, t=t, q=q, o3=o3, t_surf_rad=ts,
                   albedo=0.27 + 0.05 * rng.uniform(-1.0, 1.0, size=(nlat, nlon)),
                   rrtm_precip=rng.uniform(0.0, 2.0e-4, size=(nlat, nlon)),
                   tdt=1.0e-5 * rng.standard_normal((nlev, nlat, nlon)))
