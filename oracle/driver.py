"""CPU restatement of MiMA's radiation driver -- TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg use
this module, as the checker of ``rrtmg_run_dev`` / ``rrtmg_run_c``.  It
restates, in numpy IEEE double arithmetic with the reference's evaluation
order:

* ``interp_temp``   src/atmos_param/rrtm_radiation/rrtm_radiation.f90:420-460
* ``compute_zenith`` src/atmos_param/rrtm_radiation/astro.f90:59-248
* ``run_rrtmg``     src/atmos_param/rrtm_radiation/rrtm_radiation.f90:464-834
  (input side :596-677, output side :715-815), with the RRTMG calls made by
  the C++ oracle (oracle.py).

Arrays are C-ordered (level, latitude, longitude) = Fortran (si, sj, sk).
Zonal sums are accumulated in index order (``np.add.accumulate``), as the
Fortran SUM intrinsic does, not pairwise.

Parity: the reference's driver cannot run here (no Fortran compiler, and it
needs FMS); this restatement is checked against hand-worked cases in
tests/test_oracle_driver.py, so its parity with the reference is unpinned
beyond those.
"""
from __future__ import annotations

from types import SimpleNamespace

import numpy as np

PI = 3.14159265358979323846  # FMS constants_mod PI
DAYPERSEC = 1.0 / 86400      # rrtm_radiation.f90:104


def _seqsum(a, axis):
    """Sum in index order (the Fortran SUM intrinsic), not numpy's pairwise sum."""
    return np.add.accumulate(a, axis=axis).take(-1, axis=axis)


def interp_temp(z_full, z_half, t_surf_rad, t):
    """Half-level temperature (rrtm_radiation.f90:420-460): linear in height
    between full levels, linear extrapolation at the top, the surface
    temperature at the bottom."""
    sk = t.shape[0]
    th = np.empty((sk + 1,) + t.shape[1:])
    for k in range(1, sk):  # Fortran k = 2..kend
        dzk2 = 1.0 / (z_full[k - 1] - z_full[k])
        dzk = (z_half[k] - z_full[k]) * dzk2
        dzk1 = (z_full[k - 1] - z_half[k]) * dzk2
        th[k] = t[k] * dzk1 + t[k - 1] * dzk
    th[0] = 0.5 * (3.0 * t[0] - t[1])
    th[sk] = t_surf_rad
    return th


def model_time(prm, seconds, days):
    """Time_loc of run_rrtmg (rrtm_radiation.f90:550-558): perpetual solday,
    or the model time scaled by slowdown_rad."""
    if prm.solday > 0:
        return seconds, prm.solday
    if prm.slowdown_rad != 1.0:
        t = int((days * 86400 + seconds) * prm.slowdown_rad)
        return t % 86400, t // 86400
    return seconds, days


def declination(prm, seconds, days, days_per_year):
    """Scalars of compute_zenith (astro.f90:98-137): radsec, dt_pi, dyofyr and
    sin/cos/tan of the declination."""
    radpersec = 2 * PI / 86400.0
    radperday = 2 * PI / days_per_year
    radsec = seconds * radpersec
    dt_pi = prm.dt_rad_avg * radpersec
    dyofyr = (days - int(prm.equinox_day * days_per_year)) % days_per_year
    radday = dyofyr * radperday
    dec_sin = np.sin(prm.obliq * (PI / 180.0)) * np.sin(radday)
    dec = np.arcsin(dec_sin)
    return SimpleNamespace(radpersec=radpersec, radsec=radsec, dt_pi=dt_pi, dyofyr=dyofyr, dec_sin=dec_sin,
                           dec_cos=np.cos(dec), dec_tan=np.tan(dec))


def compute_zenith(prm, seconds, days, days_per_year, lat, lon):
    """cos(zenith) at every point (astro.f90:59-248), averaged over
    dt_rad_avg seconds (0: instantaneous, >= 86400: daily mean)."""
    d = declination(prm, seconds, days, days_per_year)
    twopi = 2 * PI
    tp = np.fmod(d.radsec + lon, twopi)
    tp = np.where(tp < 0.0, tp + twopi, tp) - PI
    tp = np.where(tp >= PI, tp - twopi, tp)
    tp = np.where(tp < -PI, tp + twopi, tp)
    lat_h = np.where(lat == 0.5 * PI, lat - 1.0e-5, lat)
    lat_h = np.where(lat_h == -0.5 * PI, lat + 1.0e-5, lat_h)
    cos_h = -np.tan(lat_h) * d.dec_tan
    with np.errstate(invalid="ignore"):
        h = np.where(cos_h <= -1.0, PI, np.where(cos_h >= 1.0, 0.0, np.arccos(np.clip(cos_h, -1.0, 1.0))))
    aa = np.sin(lat) * d.dec_sin
    bb = np.cos(lat) * d.dec_cos
    dt = prm.dt_rad_avg
    if 0 < dt < 86400:
        tt = tp + d.dt_pi
        st, stt, sh = np.sin(tp), np.sin(tt), np.sin(h)
        tth = (tt + h) - twopi
        cz = np.zeros_like(lat)
        with np.errstate(divide="ignore", invalid="ignore"):
            cz = np.where(((tt + h) != 0.0) & (tp < -h) & (np.abs(tt) <= h), aa + bb * (stt + sh) / (tt + h), cz)
            cz = np.where((tp < -h) & (h != 0.0) & (h < tt), aa + bb * (sh + sh) / (h + h), cz)
            cz = np.where((np.abs(tp) <= h) & (np.abs(tt) <= h), aa + bb * (stt - st) / (tt - tp), cz)
            cz = np.where(((h - tp) != 0.0) & (np.abs(tp) <= h) & (h < tt), aa + bb * (sh - st) / (h - tp), cz)
            cz = np.where(((twopi - h) < tt) & (tth != 0.0) & (tp <= h),
                          (cz * (h - tp) + (aa * tth + bb * (stt + sh))) / ((h - tp) + tth), cz)
            cz = np.where((h < tp) & ((twopi - h) >= tt), 0.0, cz)
            cz = np.where((h < tp) & ((twopi - h) < tt), aa + bb * (stt + sh) / tth, cz)
            fr = np.zeros_like(lat)
            fr = np.where((tp < -h) & (np.abs(tt) <= h), (tt + h) / dt, fr)
            fr = np.where((tp < -h) & (h < tt), (h + h) / dt, fr)
            fr = np.where((np.abs(tp) <= h) & (np.abs(tt) <= h), (tt - tp) / dt, fr)
            fr = np.where((np.abs(tp) <= h) & (h < tt), (h - tp) / dt, fr)
            fr = np.where(h < tp, 0.0, fr)
            fr = np.where((twopi - h) < tt, fr + tth / dt, fr)
        cz = cz * fr / d.radpersec
    elif dt >= 86400:
        cz = (aa * h + bb * np.sin(h)) / PI
    else:
        cz = np.where(np.abs(tp) <= h, aa + bb * np.cos(tp), 0.0)
    return np.where(cz > 0.0, cz, 0.0)


def _clamp(x, lo, hi):
    x = np.where(x < lo, lo, x)
    return np.where(x > hi, hi, x)


def run_prep(prm, slab, coszen, t_half, dyofyr):
    """RRTM columns from the GCM slab (rrtm_radiation.f90:596-677): returns an
    object with the attributes of an rrtmg_lw / rrtmg_sw call."""
    si, sj, sk, ls = slab.si, slab.sj, slab.sk, prm.lonstep
    nsub = si // ls
    ncol = nsub * sj
    # do_precip_albedo (:604-611)
    albedo = slab.albedo
    if prm.do_precip_albedo and prm.num_precip > 0:
        pr = np.where(np.abs(slab.lat) < prm.precip_lat * 3.14159265 / 180.0, 0.0, slab.rrtm_precip)
        zs = _seqsum(pr, axis=1)[:, None]
        albedo = albedo + (prm.precip_albedo - albedo) * zs / si / prm.num_precip
    # do_zm_tracers (:613-620), do_fixed_water (:631-641)
    q = slab.q
    if prm.do_zm_tracers:
        q = np.broadcast_to((_seqsum(q, axis=2) / si)[:, :, None], q.shape)
    if prm.do_fixed_water:
        sel = (np.abs(slab.lat)[None] <= prm.fixed_water_lat) & (slab.p_full <= prm.fixed_water_pres * 100.0)
        q = np.where(sel, prm.fixed_water, q)

    def cols(a):  # (levels, sj, si) -> (levels, ncol), every lonstep-th longitude, surface first
        return np.ascontiguousarray(a[::-1, :, ::ls].reshape(a.shape[0], ncol))

    def surf(a):
        return np.ascontiguousarray(a[:, ::ls].reshape(ncol))

    play = cols(slab.p_full) * 0.01
    plev = cols(slab.p_half) * 0.01
    if plev[sk].min() <= 0.0:  # :655-656
        plev[sk] = play[sk - 1] * 0.5
    tlay = _clamp(cols(slab.t), prm.temp_lower_limit, prm.temp_upper_limit)
    tlev = _clamp(cols(t_half), prm.temp_lower_limit, prm.temp_upper_limit)
    h2o = cols(q)
    h2o = np.where(h2o < prm.h2o_lower_limit, prm.h2o_lower_limit, h2o)
    o3 = cols(slab.o3) if slab.o3 is not None else np.full((sk, ncol), prm.o3_val)
    z = np.zeros((sk, ncol))
    sec = bool(prm.include_secondary_gases)
    gas = lambda v: np.full((sk, ncol), v) if sec else z
    alb = surf(albedo)
    return SimpleNamespace(
        ncol=ncol, nlay=sk, play=play, plev=plev, tlay=tlay, tlev=tlev, tsfc=surf(slab.t_surf_rad), h2o=h2o,
        o3=o3, co2=np.full((sk, ncol), prm.co2ppmv * 1.e-6), ch4=gas(prm.ch4_val), n2o=gas(prm.n2o_val),
        o2=gas(prm.o2_val), cfc11=gas(prm.cfc11_val), cfc12=gas(prm.cfc12_val), cfc22=gas(prm.cfc22_val),
        ccl4=gas(prm.ccl4_val), emis=np.ones((16, ncol)), asdir=alb, asdif=alb, aldir=alb, aldif=alb,
        coszen=surf(coszen), scon=prm.solr_cnst, adjes=prm.solrad, dyofyr=dyofyr if prm.use_dyofyr else 0)


def run_post(prm, slab, lw, sw, tdt):
    """GCM tendencies and surface fluxes from the RRTM results
    (rrtm_radiation.f90:715-815)."""
    si, sj, sk, ls = slab.si, slab.sj, slab.sk, prm.lonstep
    nsub = si // ls
    g = lambda a: a[::-1].reshape(a.shape[0], sj, nsub)  # (levels, ncol) -> GCM order, top first
    swijk = g(sw["swhr"]) * DAYPERSEC
    lwijk = g(lw["hr"]) * DAYPERSEC
    s2 = lambda a: a.reshape(sj, nsub)
    olrijk = s2(lw["uflx"][sk])
    isrijk = s2(sw["swdflx"][sk] - sw["swuflx"][sk])
    swflx = s2(sw["swdflx"][0] - sw["swuflx"][0])
    lwflx = s2(lw["dflx"][0])
    i = np.arange(si)
    i0 = i // ls
    i1 = np.where(i0 + 1 < nsub, i0 + 1, 0)
    di = (i % ls) * (1.0 / ls)
    omd = 1.0 - di
    lerp = lambda a: di * a[..., i1] + omd * a[..., i0]
    n = max(1, nsub)
    tot = swijk + lwijk
    if prm.do_zm_rad:
        tdt_rrtm = np.broadcast_to((_seqsum(tot, axis=2) / n)[:, :, None], (sk, sj, si)).copy()
        fsw = np.broadcast_to((_seqsum(swflx, axis=1) / n)[:, None], (sj, si)).copy()
        flw = np.broadcast_to((_seqsum(lwflx, axis=1) / n)[:, None], (sj, si)).copy()
    else:
        tdt_rrtm = di * tot[..., i1] + omd * tot[..., i0]
        fsw, flw = lerp(swflx), lerp(lwflx)
    return {"tdt": tdt + tdt_rrtm, "tdt_rad": tdt_rrtm, "tdt_sw": lerp(swijk), "tdt_lw": lerp(lwijk),
            "olr": lerp(olrijk), "isr": lerp(isrijk), "flux_sw": fsw, "flux_lw": flw}


def run_rrtmg(orc, prm, slab, seconds, days, days_per_year=365, coszen=None, lw_sw=None):
    """The whole driver step.  ``orc`` is the loaded C++ oracle module
    (oracle.py).  ``coszen`` replaces the zenith angle (e.g. to chain a device
    result through the remaining, bit-reproducible steps); ``lw_sw`` replaces
    the RRTMG call: a function of the prepared columns returning (lw, sw)."""
    sec, day = model_time(prm, seconds, days)
    th = interp_temp(slab.z_full, slab.z_half, slab.t_surf_rad, slab.t)
    cz = compute_zenith(prm, sec, day, days_per_year, slab.lat, slab.lon) if coszen is None else coszen
    dyofyr = declination(prm, sec, day, days_per_year).dyofyr
    atm = run_prep(prm, slab, cz, th, dyofyr)
    if lw_sw is None:
        lw, sw = orc.rrtmg_lw(atm), orc.rrtmg_sw(atm)
    else:
        lw, sw = lw_sw(atm)
    out = run_post(prm, slab, lw, sw, slab.tdt)
    out.update(coszen=cz, t_half=th, atm=atm)
    return out
