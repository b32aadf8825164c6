"""Property tests over randomly drawn atmospheres and driver options
(hypothesis): invariants of the CPU oracle's clear-sky RRTMG and of the
driver restatement that hold for every valid input.  No GPU."""
import numpy as np
import pytest

hypothesis = pytest.importorskip("hypothesis")
from hypothesis import given, settings, strategies as st  # noqa: E402

from mima_gb300 import atmosphere as A  # noqa: E402
from oracle import driver as D  # noqa: E402

HEATFAC_CP = 1004.64


@st.composite
def atmospheres(draw):
    ncol = draw(st.integers(1, 4))
    nlay = draw(st.sampled_from([12, 40, 60]))
    seed = draw(st.integers(0, 2**31 - 1))
    atm = A.small_atmosphere(ncol, nlay, seed=seed, ts_sigma=draw(st.floats(0.0, 15.0)))
    rng = np.random.default_rng(seed)
    atm.co2 = np.full(atm.play.shape, draw(st.floats(100e-6, 2000e-6)))
    atm.o3 = atm.o3 * draw(st.floats(0.0, 3.0))
    atm.h2o = np.clip(atm.h2o * draw(st.floats(0.05, 1.5)), 1e-7, 0.05)
    atm.coszen = rng.uniform(0.0, 1.0, size=ncol) * draw(st.sampled_from([0.0, 1.0]) | st.just(1.0))
    alb = draw(st.floats(0.0, 0.9))
    for k in ("asdir", "asdif", "aldir", "aldif"):
        setattr(atm, k, np.full(ncol, alb))
    return atm


@settings(max_examples=25, deadline=None)
@given(atmospheres())
def test_oracle_invariants(orc, atm):
    lw, sw = orc.rrtmg_lw(atm), orc.rrtmg_sw(atm)
    L = atm.nlay
    for d in (lw, sw):
        for v in d.values():
            assert np.isfinite(v).all()
    # clear sky: total and clear-sky outputs are the same computation
    for a, b in (("uflx", "uflxc"), ("dflx", "dflxc"), ("hr", "hrc")):
        np.testing.assert_array_equal(lw[a], lw[b])
    for a, b in (("swuflx", "swuflxc"), ("swdflx", "swdflxc"), ("swhr", "swhrc")):
        np.testing.assert_array_equal(sw[a], sw[b])
    # fluxes are non-negative; no downward LW enters at the top
    for k in ("uflx", "dflx"):
        assert (lw[k] >= -1e-9).all(), k
    assert np.all(lw["dflx"][L] == 0.0)
    for k in ("swuflx", "swdflx"):
        assert (sw[k] >= -1e-9).all(), k
    # dark columns carry no SW at all
    dark = atm.coszen < 1e-10
    assert np.all(sw["swdflx"][:, dark] == 0.0) and np.all(sw["swhr"][:, dark] == 0.0)
    # energy budget: the heating rates are the net-flux divergence of their
    # layers, so summed with the layer masses they telescope to the net-flux
    # difference between the surface and the top of the rated layers
    dp = atm.plev[:-1] - atm.plev[1:]
    heatfac = 9.8066 * 86400.0 / (HEATFAC_CP * 100.0)
    net_lw = lw["uflx"] - lw["dflx"]
    lhs = (lw["hr"] * dp).sum(axis=0) / heatfac
    rhs = net_lw[0] - net_lw[L]
    assert np.allclose(lhs, rhs, rtol=1e-9, atol=1e-9 * np.abs(net_lw).max())
    net_sw = sw["swdflx"] - sw["swuflx"]
    lhs = (sw["swhr"][:L - 1] * dp[:L - 1]).sum(axis=0) / heatfac  # MiMA: top layer rate 0
    rhs = net_sw[0] - net_sw[L - 1]
    assert np.allclose(lhs, -rhs, rtol=1e-9, atol=1e-9 * max(1.0, np.abs(net_sw).max()))
    # the surface absorbs (1 - albedo) of what reaches it; the column absorbs what the top loses
    assert np.all(net_sw[0] >= -1e-9)
    assert np.all(net_sw[L] + 1e-9 >= net_sw[0])


@st.composite
def driver_cases(draw):
    nlat = draw(st.integers(1, 4))
    ls = draw(st.sampled_from([1, 2, 3, 4]))
    nlon = ls * draw(st.integers(1, 6))
    nlev = draw(st.sampled_from([5, 12]))
    prm = dict(lonstep=ls, do_zm_tracers=draw(st.integers(0, 1)), do_zm_rad=draw(st.integers(0, 1)),
               do_fixed_water=0, include_secondary_gases=0, do_precip_albedo=0, num_precip=0, use_dyofyr=0,
               solday=0, dt_rad_avg=draw(st.sampled_from([0, 3600, 86400])), h2o_lower_limit=2e-7,
               temp_lower_limit=100.0, temp_upper_limit=370.0, co2ppmv=300.0, o3_val=0.0, fixed_water=2e-6,
               fixed_water_pres=100e2, fixed_water_lat=90.0, ch4_val=0.0, n2o_val=0.0, o2_val=0.0, cfc11_val=0.0,
               cfc12_val=0.0, cfc22_val=0.0, ccl4_val=0.0, precip_albedo=0.35, precip_lat=0.0, slowdown_rad=1.0,
               obliq=23.439, solr_cnst=1368.22, solrad=1.0, equinox_day=0.25)
    from types import SimpleNamespace
    return (A.gcm_slab(nlon, nlat, nlev, seed=draw(st.integers(0, 2**31 - 1))), SimpleNamespace(**prm),
            draw(st.integers(0, 86399)), draw(st.integers(0, 3000)))


def fake_rrtm(atm):
    L, n = atm.nlay, atm.ncol
    col = np.arange(n)[None, :]
    lev = np.arange(L + 1)[:, None]
    lw = {"hr": np.sin(0.1 * col + 0.3 * lev[:-1]) + atm.tlay / 300.0, "uflx": 200.0 + col + lev,
          "dflx": 300.0 - 0.5 * col + lev}
    sw = {"swhr": np.cos(0.2 * col + 0.1 * lev[:-1]) * atm.coszen[None, :], "swuflx": 50.0 + 0.1 * col + lev,
          "swdflx": 400.0 + 0.3 * col - lev}
    return lw, sw


@settings(max_examples=30, deadline=None)
@given(driver_cases())
def test_driver_invariants(case):
    slab, prm, seconds, days = case
    out = D.run_rrtmg(None, prm, slab, seconds, days, lw_sw=fake_rrtm)
    # tdt gains exactly the radiative tendency
    np.testing.assert_array_equal(out["tdt"], slab.tdt + out["tdt_rad"])
    # the zenith angle is a cosine, zero or positive
    assert ((out["coszen"] >= 0.0) & (out["coszen"] <= 1.0 + 1e-12)).all()
    # RRTM columns are surface-first and monotone in pressure
    atm = out["atm"]
    assert (np.diff(atm.plev, axis=0) < 0).all() and (atm.plev > 0).all()
    # sampled longitudes carry their own column's tendency; a zonal mean is uniform
    if prm.do_zm_rad:
        assert np.all(out["tdt_rad"] == out["tdt_rad"][:, :, :1])
    else:
        lw, sw = fake_rrtm(atm)
        own = ((sw["swhr"] + lw["hr"]) / 86400.0)[::-1].reshape(slab.sk, slab.sj, slab.si // prm.lonstep)
        np.testing.assert_allclose(out["tdt_rad"][:, :, ::prm.lonstep], own, rtol=1e-13, atol=1e-20)
    # interpolation stays between the two neighbouring sampled columns
    lo = np.minimum(out["tdt_sw"][:, :, ::prm.lonstep], np.roll(out["tdt_sw"][:, :, ::prm.lonstep], -1, axis=2))
    hi = np.maximum(out["tdt_sw"][:, :, ::prm.lonstep], np.roll(out["tdt_sw"][:, :, ::prm.lonstep], -1, axis=2))
    for r in range(prm.lonstep):
        v = out["tdt_sw"][:, :, r::prm.lonstep]
        assert (v >= lo - 1e-18).all() and (v <= hi + 1e-18).all()
