"""The CPU restatement of MiMA's radiation driver (oracle/driver.py) against
hand-worked answers and exact properties of interp_temp, compute_zenith and
the input / output sides of run_rrtmg.  No GPU."""
from types import SimpleNamespace

import numpy as np
import pytest

from mima_gb300 import atmosphere as A
from oracle import driver as D


def params(**kw):
    """The reference's namelist defaults (rrtm_radiation.f90:106-198, astro.f90:22-31)."""
    p = dict(lonstep=1, do_zm_tracers=0, do_zm_rad=0, do_fixed_water=0, include_secondary_gases=0,
             do_precip_albedo=0, num_precip=0, use_dyofyr=0, solday=0, dt_rad_avg=86400, h2o_lower_limit=2e-7,
             temp_lower_limit=100.0, temp_upper_limit=370.0, co2ppmv=300.0, o3_val=0.0, fixed_water=2e-6,
             fixed_water_pres=100e2, fixed_water_lat=90.0, ch4_val=0.0, n2o_val=0.0, o2_val=0.0, cfc11_val=0.0,
             cfc12_val=0.0, cfc22_val=0.0, ccl4_val=0.0, precip_albedo=0.35, precip_lat=0.0, slowdown_rad=1.0,
             obliq=23.439, solr_cnst=1368.22, solrad=1.0, equinox_day=0.25)
    p.update(kw)
    return SimpleNamespace(**p)


def test_params_match_library_defaults():
    from mima_gb300 import rrtmg as R
    lib_p = R.run_params()
    for k, v in vars(params()).items():
        assert getattr(lib_p, k) == v, k


def test_interp_temp_linear_profile():
    """T linear in height is reproduced at interior half levels; the top is
    0.5 (3 t1 - t2) and the bottom the surface temperature."""
    rng = np.random.default_rng(1)
    sk = 12
    zf = np.sort(rng.uniform(100, 30000, size=(sk, 3, 5)), axis=0)[::-1].copy()
    zh = np.empty((sk + 1, 3, 5))
    zh[1:-1] = zf[:-1] - rng.uniform(0.2, 0.8, size=(sk - 1, 3, 5)) * (zf[:-1] - zf[1:])
    zh[0] = 0.0
    zh[-1] = 0.0
    a, b = 288.0, -6.5e-3
    t = a + b * zf
    ts = rng.uniform(250, 300, size=(3, 5))
    th = D.interp_temp(zf, zh, ts, t)
    np.testing.assert_allclose(th[1:-1], a + b * zh[1:-1], rtol=1e-12)
    np.testing.assert_array_equal(th[0], 0.5 * (3 * t[0] - t[1]))
    np.testing.assert_array_equal(th[-1], ts)


def test_zenith_daily_mean_at_equinox():
    """Declination 0 (the equinox of equinox_day): daily mean cos(lat)/pi."""
    lat = np.linspace(-1.5, 1.5, 31)[:, None] * np.ones((1, 4))
    lon = np.zeros_like(lat) + np.arange(4)[None, :]
    p = params()
    days = int(0.25 * 365)  # dyofyr = 0 -> declination 0
    cz = D.compute_zenith(p, 0, days, 365, lat, lon)
    np.testing.assert_allclose(cz, np.cos(lat) / np.pi, rtol=1e-14, atol=1e-15)


def test_zenith_instantaneous_noon_and_night():
    p = params(dt_rad_avg=0)
    days = int(0.25 * 365)
    lat = np.zeros((1, 4))
    # local time = modulo(radsec + lon, 2 pi) - pi: lon = pi at seconds 0 is noon
    lon = np.array([[np.pi, 0.0, np.pi / 2, 3 * np.pi / 2]])
    cz = D.compute_zenith(p, 0, days, 365, lat, lon)
    np.testing.assert_allclose(cz[0], [1.0, 0.0, 0.0, 0.0], atol=1e-15)
    # cos(lat) cos(local time) at the equinox
    lon2 = np.array([[np.pi + 0.3, np.pi - 1.0, np.pi + 1.2, np.pi]])
    cz2 = D.compute_zenith(p, 0, days, 365, np.full((1, 4), 0.4), lon2)
    np.testing.assert_allclose(cz2[0], np.cos(0.4) * np.cos([0.3, -1.0, 1.2, 0.0]), rtol=1e-14)


@pytest.mark.parametrize("dt", [3600, 10800, 43200])
def test_zenith_time_average_is_mean_of_instantaneous(dt):
    """The eight-case interval mean of compute_zenith equals the quadrature of
    max(0, instantaneous cos zenith) over [t, t + dt] at the same declination,
    across sunrise, sunset, polar day and night and the day boundary."""
    rng = np.random.default_rng(dt)
    lat = rng.uniform(-1.55, 1.55, size=(40, 25))
    lon = rng.uniform(0, 2 * np.pi, size=(40, 25))
    for days, seconds in ((10, 0), (100, 40000), (200, 80000), (300, 12345)):
        p = params(dt_rad_avg=dt)
        cz = D.compute_zenith(p, seconds, days, 365, lat, lon)
        n = 4001
        acc = np.zeros_like(lat)
        w = np.ones(n)
        w[0] = w[-1] = 0.5
        for m in range(n):
            s = seconds + dt * m / (n - 1)
            pi_ = params(dt_rad_avg=0)
            # the same declination: instantaneous angle at second s of the same day
            acc += w[m] * D.compute_zenith(pi_, s, days, 365, lat, lon)
        ref = acc / (n - 1)
        np.testing.assert_allclose(cz, ref, atol=2e-6)


def fake_rrtm(atm):
    """Deterministic stand-in RRTMG results that depend on the columns."""
    L, n = atm.nlay, atm.ncol
    col = np.arange(n)[None, :]
    lev = np.arange(L + 1)[:, None]
    lw = {"hr": np.sin(0.1 * col + 0.3 * lev[:-1]) + atm.tlay / 300.0, "uflx": 200.0 + col + lev,
          "dflx": 300.0 - 0.5 * col + lev}
    sw = {"swhr": np.cos(0.2 * col + 0.1 * lev[:-1]) * atm.coszen[None, :], "swuflx": 50.0 + 0.1 * col + lev,
          "swdflx": 400.0 + 0.3 * col - lev}
    return lw, sw


def test_run_prep_layout_and_clamps():
    slab = A.gcm_slab(16, 4, 10, seed=3)
    slab.t[2, 1, 4] = 50.0      # below temp_lower_limit (on sampled longitudes)
    slab.t[3, 2, 6] = 400.0     # above temp_upper_limit
    slab.q[4, 3, 8] = 1e-9      # below h2o_lower_limit
    p = params(lonstep=2)
    th = D.interp_temp(slab.z_full, slab.z_half, slab.t_surf_rad, slab.t)
    cz = np.full((4, 16), 0.5)
    atm = D.run_prep(p, slab, cz, th, 0)
    nsub = 8
    # column c = isub + nsub*j is GCM point (2*isub, j); layer l is GCM level sk-1-l
    for c, (isub, j) in {0: (0, 0), 5: (5, 0), 9: (1, 1), 30: (6, 3)}.items():
        i = 2 * isub
        for lay in (0, 4, 9):
            k = 9 - lay
            assert atm.play[lay, c] == slab.p_full[k, j, i] * 0.01
            assert atm.tlay[lay, c] == min(max(slab.t[k, j, i], 100.0), 370.0)
            assert atm.h2o[lay, c] == max(slab.q[k, j, i], 2e-7)
        assert atm.tsfc[c] == slab.t_surf_rad[j, i]
    assert atm.tlay.min() == 100.0 and atm.tlay.max() == 370.0
    assert atm.h2o.min() == 2e-7
    # the top interface is 0 Pa in the slab: replaced by half the top layer pressure
    np.testing.assert_array_equal(atm.plev[10], atm.play[9] * 0.5)
    np.testing.assert_array_equal(atm.plev[0], (slab.p_half[10, :, ::2] * 0.01).reshape(-1))
    np.testing.assert_array_equal(atm.co2, np.full((10, 32), 300.0 * 1e-6))


def test_run_prep_options():
    slab = A.gcm_slab(8, 6, 8, seed=4)
    th = D.interp_temp(slab.z_full, slab.z_half, slab.t_surf_rad, slab.t)
    cz = np.zeros((6, 8))
    # zonal-mean tracers: every column of a latitude gets the same humidity
    atm = D.run_prep(params(do_zm_tracers=1), slab, cz, th, 0)
    h = atm.h2o.reshape(8, 6, 8)
    assert np.all(h == h[:, :, :1])
    np.testing.assert_allclose(h[:, :, 0], np.maximum(slab.q.mean(axis=2), 2e-7)[::-1], rtol=1e-14)
    # fixed water above 50 hPa, within 0.5 rad of the equator
    atm = D.run_prep(params(do_fixed_water=1, fixed_water=5e-6, fixed_water_pres=50.0, fixed_water_lat=0.5),
                     slab, cz, th, 0)
    sel = ((slab.p_full <= 5000.0) & (np.abs(slab.lat)[None] <= 0.5))[::-1].reshape(8, 48)
    assert sel.any() and (~sel).any()
    assert np.all(atm.h2o[sel] == 5e-6)
    # precipitation albedo: albedo + (0.35 - albedo) * zonal-mean precip / num_precip
    atm = D.run_prep(params(do_precip_albedo=1, num_precip=3, precip_lat=20.0), slab, cz, th, 0)
    pr = np.where(np.abs(slab.lat) < np.deg2rad(20.0), 0.0, slab.rrtm_precip)
    ref = slab.albedo + (0.35 - slab.albedo) * pr.mean(axis=1)[:, None] / 3
    np.testing.assert_allclose(atm.asdir.reshape(6, 8), ref, rtol=1e-14)
    # secondary gases and ozone constant
    slab.o3 = None
    atm = D.run_prep(params(include_secondary_gases=1, ch4_val=1.8e-6, ccl4_val=1e-10, o3_val=3e-7), slab, cz, th, 0)
    assert np.all(atm.ch4 == 1.8e-6) and np.all(atm.ccl4 == 1e-10) and np.all(atm.o3 == 3e-7)
    assert np.all(atm.n2o == 0.0)


@pytest.mark.parametrize("lonstep", [1, 2, 4])
def test_run_post_interpolation(lonstep):
    slab = A.gcm_slab(16, 3, 6, seed=5)
    p = params(lonstep=lonstep)
    out = D.run_rrtmg(None, p, slab, 0, 10, lw_sw=fake_rrtm)
    atm = out["atm"]
    lw, sw = fake_rrtm(atm)
    nsub = 16 // lonstep
    tot = ((sw["swhr"] + lw["hr"]) / 86400.0)[::-1].reshape(6, 3, nsub)
    # sampled longitudes carry their own column, the others interpolate toward the next (cyclically)
    for i in range(16):
        i0, r = divmod(i, lonstep)
        i1 = (i0 + 1) % nsub
        w = r / lonstep
        np.testing.assert_allclose(out["tdt_rad"][:, :, i], (1 - w) * tot[:, :, i0] + w * tot[:, :, i1],
                                   rtol=1e-13, atol=1e-20)
    np.testing.assert_array_equal(out["tdt"], slab.tdt + out["tdt_rad"])
    if lonstep == 1:
        np.testing.assert_array_equal(out["flux_lw"], lw["dflx"][0].reshape(3, 16))
        np.testing.assert_array_equal(out["olr"], lw["uflx"][6].reshape(3, 16))
        np.testing.assert_array_equal(out["flux_sw"], (sw["swdflx"][0] - sw["swuflx"][0]).reshape(3, 16))


def test_run_post_zonal_mean():
    slab = A.gcm_slab(12, 3, 5, seed=6)
    out = D.run_rrtmg(None, params(lonstep=3, do_zm_rad=1), slab, 0, 10, lw_sw=fake_rrtm)
    assert np.all(out["tdt_rad"] == out["tdt_rad"][:, :, :1])
    assert np.all(out["flux_sw"] == out["flux_sw"][:, :1])
    lw, sw = fake_rrtm(out["atm"])
    ref = ((sw["swhr"] + lw["hr"]) / 86400.0)[::-1].reshape(5, 3, 4).mean(axis=2)
    np.testing.assert_allclose(out["tdt_rad"][:, :, 0], ref, rtol=1e-14)


def test_model_time():
    assert D.model_time(params(solday=100), 500, 7) == (500, 100)
    assert D.model_time(params(slowdown_rad=0.5), 3600, 3) == ((3 * 86400 + 3600) // 2 % 86400, 1)
    assert D.model_time(params(), 5, 9) == (5, 9)
