"""FP32/FP64-split path against the FP64 oracle across its input regions and
on subsets of the benchmark configurations.

Bars (tests/split_bars.py): fluxes within 0.1 W/m2 at every level (OLR and the
surface fluxes among them), heating rates within 0.05 K/day; a column that
misses a bar in table mode must be reproduced within the bars by the oracle on
inputs within FP32 rounding of the given ones (the reference's table-mode
delta-Eddington is ill-conditioned at k mu0 = 1).  The max and RMS errors of
each configuration are asserted against the bars and printed.
"""
import numpy as np
import pytest

import split_bars as SB
from mima_gb300 import atmosphere as A

pytestmark = pytest.mark.gpu


def _split(gpu, atm, mode="table", idrv=0, lw_aer=None, aer=None):
    gpu.set_precision("split")
    gpu.set_transcendentals(mode)
    try:
        return gpu.lw(atm, idrv=idrv, tauaer=lw_aer), gpu.sw(atm, **(aer or {}))
    finally:
        gpu.set_transcendentals("table")
        gpu.set_precision("fp64")


def _oracle(orc, atm, mode="table", idrv=0, lw_aer=None, aer=None):
    orc.set_table_mode(mode == "table")
    try:
        return orc.rrtmg_lw(atm, idrv=idrv, tauaer=lw_aer), orc.rrtmg_sw(atm, **(aer or {}))
    finally:
        orc.set_table_mode(True)


def aerosol_profile(atm, rng, nbands, tau_col_max):
    """Aerosol optical depths (band, layer, column): a column total drawn per
    band and column in [0, tau_col_max), spread over the layers in proportion
    to their mass times (p / ps)^3.75 -- an aerosol scale height of about 2 km
    under an atmospheric one of 7.5 km, so the depth sits in the lower
    troposphere as real aerosol does."""
    dp = atm.plev[:-1] - atm.plev[1:]
    w = dp * (atm.play / atm.plev[0]) ** 3.75
    w = w / w.sum(axis=0)
    return rng.uniform(0.0, tau_col_max, size=(nbands, 1, atm.ncol)) * w[None]


def _assert_stats(st, label):
    print(label, {k: (f"{m:.3g}", f"{r:.3g}") for k, (m, r) in st.items()})
    assert st["lw_hr"][0] <= SB.HR_BAR and st["sw_hr"][0] <= SB.HR_BAR, (label, st)
    for k in ("olr", "lw_sfc_net", "sw_sfc_net"):
        assert st[k][0] <= SB.FLUX_BAR, (label, k, st)


@pytest.mark.parametrize("nlay", [40, 60])
@pytest.mark.parametrize("mode", ["table", "analytic"])
def test_split_input_matrix(gpu, orc, nlay, mode):
    """SW aerosols (iaer = 10: column depth up to 1 per band in the lower
    troposphere, single-scattering albedo 0.8-1, asymmetry 0-0.8), every
    secondary gas, albedos up to 0.9, CO2 100-2000 ppmv, suns from grazing
    (coszen 1e-4) to overhead, LW aerosols (column depth up to 0.3) and
    idrv = 1: split against the oracle, every column within the bars (table
    mode: or reproduced by the oracle within FP32 rounding of its inputs; in
    the layers thinner than 0.01 hPa of the 60-layer columns, the heating bar
    in its net-flux-divergence form)."""
    rng = np.random.default_rng(700 + nlay)
    n = 768
    atm = A.small_atmosphere(n, nlay, seed=710 + nlay, ts_sigma=5.0, rh_random=True)
    shp = atm.play.shape
    atm.co2 = rng.uniform(100e-6, 2000e-6, size=shp)
    atm.ch4, atm.n2o, atm.o2 = np.full(shp, 1.8e-6), np.full(shp, 3.2e-7), np.full(shp, 0.209)
    atm.cfc11, atm.cfc12 = np.full(shp, 2.5e-10), np.full(shp, 5.0e-10)
    atm.cfc22, atm.ccl4 = np.full(shp, 1.5e-10), np.full(shp, 1.0e-10)
    atm.emis = rng.uniform(0.8, 1.0, size=(16, n))
    for k in ("asdir", "asdif", "aldir", "aldif"):
        setattr(atm, k, rng.uniform(0.0, 0.9, n))
    atm.coszen = np.concatenate([10.0 ** rng.uniform(-4, -1, n // 4), rng.uniform(0.1, 1.0, n - n // 4)])
    lw_aer = aerosol_profile(atm, rng, 16, 0.3)
    aer = dict(iaer=10, tauaer=aerosol_profile(atm, rng, 14, 1.0),
               ssaaer=rng.uniform(0.8, 1.0, size=(14, nlay, n)), asmaer=rng.uniform(0.0, 0.8, size=(14, nlay, n)))
    rlw, rsw = _oracle(orc, atm, mode, 1, lw_aer, aer)
    lw, sw = _split(gpu, atm, mode, 1, lw_aer, aer)
    if mode == "table":
        ex = SB.check_lw(orc, atm, lw, rlw, idrv=1, tauaer=lw_aer) + SB.check_sw(orc, atm, sw, rsw, aer=aer)
        print("excused (column, input scale, inputs):", ex)
    else:
        for k in ("uflx", "dflx"):
            assert np.abs(lw[k] - rlw[k]).max() <= SB.FLUX_BAR, k
        for k in ("swuflx", "swdflx"):
            assert np.abs(sw[k] - rsw[k]).max() <= SB.FLUX_BAR, k
        bar = SB.hr_bar(atm)
        assert np.all(np.abs(lw["hr"] - rlw["hr"]) <= bar)
        assert np.all(np.abs(sw["swhr"] - rsw["swhr"]) <= bar)
        st = SB.error_stats(lw, rlw, sw, rsw)
        print(f"matrix L={nlay} analytic", st)
        for k in ("olr", "lw_sfc_net", "sw_sfc_net"):
            assert st[k][0] <= SB.FLUX_BAR, (k, st)
    assert np.abs(lw["duflx_dt"] - rlw["duflx_dt"]).max() <= 1e-3


def test_split_t170_subset(gpu, orc):
    """Configuration 2 of the benchmark set (T170 x 60 layers, top 0.01 hPa,
    Ts noise 5 K, RH U(0.2, 0.95) per column): a seeded 4096-column subset,
    max and RMS heating (K/day), OLR and surface net fluxes (W/m2) against the
    oracle within the bars."""
    atm = A.config_atmosphere(2)
    idx = np.sort(np.random.default_rng(2).choice(atm.ncol, 4096, replace=False))
    sub = atm.subset(idx)
    rlw, rsw = _oracle(orc, sub)
    lw, sw = _split(gpu, sub)
    SB.check_lw(orc, sub, lw, rlw)
    SB.check_sw(orc, sub, sw, rsw)
    _assert_stats(SB.error_stats(lw, rlw, sw, rsw), "T170x60 subset")


def test_split_stress_subset(gpu, orc):
    """The stress ensemble (32 members of 32768 T170-like columns x 60 layers,
    Ts noise 3 K per member): 1024 seeded columns from each of members 0, 9,
    20 and 31 (4096 in all), against the oracle within the bars."""
    for m in (0, 9, 20, 31):
        atm = A.config_atmosphere(4, member=m)
        sub = atm.subset(np.sort(np.random.default_rng(40 + m).choice(atm.ncol, 1024, replace=False)))
        rlw, rsw = _oracle(orc, sub)
        lw, sw = _split(gpu, sub)
        SB.check_lw(orc, sub, lw, rlw)
        SB.check_sw(orc, sub, sw, rsw)
        _assert_stats(SB.error_stats(lw, rlw, sw, rsw), f"stress member {m} subset")
