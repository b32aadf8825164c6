"""The oracle's FLOP-count build (oracle/opcount.hpp, oracle/opcount.py): it
computes what the normal build computes, bit for bit, and its counts of the
algorithmic work per column are linear in the layer count.  No GPU."""
import numpy as np
import pytest

from mima_gb300 import atmosphere as A
from oracle import opcount as P


@pytest.fixture(scope="module")
def counting(blob):
    return P.load(blob)


def test_counting_build_reproduces_the_oracle(orc, counting):
    atm = A.small_atmosphere(5, 40, seed=21)
    orc.set_table_mode(False)  # the count is taken in the analytic form
    try:
        rlw, rsw = orc.rrtmg_lw(atm), orc.rrtmg_sw(atm)
    finally:
        orc.set_table_mode(True)
    lw, sw, cl, cs = P.count(atm)
    for k in rlw:
        np.testing.assert_array_equal(lw[k], rlw[k], err_msg=k)
    for k in rsw:
        np.testing.assert_array_equal(sw[k], rsw[k], err_msg=k)
    assert P.flops(cl) > 0 and P.flops(cs) > 0


def test_flops_per_column_linear_in_layers(blob, counting):
    rows, flw, fsw = P.table(blob, layers=(20, 40, 60), ncol=4)
    for L, lw, sw, _, _ in rows:
        assert abs(lw - np.polyval(flw, L)) <= 0.02 * lw
        assert abs(sw - np.polyval(fsw, L)) <= 0.02 * sw
        # the structural estimates (LW 140 g x L x ~55, SW 112 g x L x ~150 FLOPs)
        assert 0.5 <= lw / (140 * L * 55) <= 2.0
        assert 0.5 <= sw / (112 * L * 150) <= 2.0
    # the committed per-column figures at 40 layers (0.285 / 0.812 MFLOP), within 3 %
    L40 = {r[0]: r for r in rows}[40]
    assert abs(L40[1] / 0.285e6 - 1) <= 0.03 and abs(L40[2] / 0.812e6 - 1) <= 0.03


def test_bench_constants_are_the_counted_table(blob, counting):
    import bench
    rows, flw, fsw = P.table(blob, layers=bench.ALG_FLOPS_LAYERS)
    assert tuple(round(r[1]) for r in rows) == bench.ALG_FLOPS_PER_COLUMN["lw_gpoint"]
    assert tuple(round(r[2]) for r in rows) == bench.ALG_FLOPS_PER_COLUMN["sw_gpoint"]
    np.testing.assert_allclose(bench.ALG_FLOPS_FIT["lw_gpoint"], flw, rtol=1e-6)
    np.testing.assert_allclose(bench.ALG_FLOPS_FIT["sw_gpoint"], fsw, rtol=1e-6)
    assert bench.algorithmic_flops("sw_gpoint", 40) == bench.ALG_FLOPS_PER_COLUMN["sw_gpoint"][1]
    assert bench.algorithmic_flops("lw_gpoint", 100) == pytest.approx(flw[0] * 100 + flw[1])


def test_phase_flops_add_up_to_the_path(blob, counting):
    """The per-phase counts (orc_*_phase_counts) add up to the whole path's:
    exactly for LW; for SW but for the clear-sky heating rates, which the
    whole call also computes (a few operations per layer)."""
    atm = A.small_atmosphere(6, 40, seed=11, rh_random=False)
    lw, sw = P.phase_flops(atm)
    _, _, cl, cs = P.count(atm)
    assert all(v > 0 for v in list(lw.values()) + list(sw.values()))
    assert sum(lw.values()) == pytest.approx(P.flops(cl), rel=1e-12)
    assert 0 <= P.flops(cs) - sum(sw.values()) <= 10 * atm.nlay
    # the g-point work dominates both paths
    assert (lw["taumol"] + lw["rtrnmr"]) / sum(lw.values()) > 0.9
    assert (sw["taumol_sw"] + sw["spcvrt_sw"]) / sum(sw.values()) > 0.9


def test_cloudy_counts(orc, counting):
    """Cloudy calls in the counting build: the same fluxes as the normal
    build, bit for bit; with no cover the LW cloudy call does the clear work
    and rtrnmr's overlap bookkeeping over every layer (under 5 % more), the SW
    one adds its total-sky pass (counted in a call with clouds); overcast
    layers with the cloud physics add work on both sides."""
    atm = A.small_atmosphere(6, 40, seed=23)
    cf = np.zeros((atm.nlay, atm.ncol))
    none = dict(cldfr=cf, cicewp=cf, cliqwp=cf, reice=cf + 30.0, reliq=cf + 10.0, inflag=2, iceflag=3, liqflag=1)
    cf1 = cf.copy()
    cf1[5:9] = 1.0
    over = dict(none, cldfr=cf1, cicewp=cf1 * 20.0, cliqwp=cf1 * 30.0)
    _, _, clr_lw, clr_sw = P.count(atm)
    n_lw, n_sw = P.count_clouds(atm, none, none)
    o_lw, o_sw = P.count_clouds(atm, over, over)
    assert P.flops(clr_lw) <= P.flops(n_lw) < 1.05 * P.flops(clr_lw)
    assert 1.2 * P.flops(clr_sw) < P.flops(n_sw) < 2.0 * P.flops(clr_sw)
    assert P.flops(o_lw) > P.flops(n_lw) and P.flops(o_sw) > P.flops(n_sw)
    orc.set_table_mode(False)
    try:
        rlw = orc.rrtmg_lw(atm, cloud=over, icld=2)
        rsw = orc.rrtmg_sw(atm, cloud=over)
    finally:
        orc.set_table_mode(True)
    lw, _ = P._counted(orc.rrtmg_lw, atm, cloud=over, icld=2)
    sw, _ = P._counted(orc.rrtmg_sw, atm, cloud=over)
    for k in rlw:
        np.testing.assert_array_equal(lw[k], rlw[k], err_msg=k)
    for k in rsw:
        np.testing.assert_array_equal(sw[k], rsw[k], err_msg=k)
