"""The oracle's cloud physics (cldprop / cldprop_sw with optical properties
formed from water paths and effective sizes) against the numpy statement of
the same parameterisations in ``cloud_optics.py``: with the cloud-band
optics computed there and handed in as given optics (inflag = 0), the
oracle's fluxes must not move."""
import numpy as np
import pytest

from mima_gb300 import atmosphere as A
from tests import cloud_optics as CO


def physics_fields(atm, rng, overcast=False):
    """Seeded clouds below 100 hPa: ice above 600 hPa, liquid below 300 hPa,
    some layers with both; effective sizes inside every parameterisation's
    range (ice 14-125 um, liquid 3-55 um, with a few at the table ends);
    some cloudy layers with no water at all.  ``overcast``: covers 0 or 1."""
    L, n = atm.nlay, atm.ncol
    u = rng.uniform(size=(L, n))
    cf = np.where(u < 0.35, rng.uniform(0.1, 1.0, (L, n)), 0.0)
    if overcast:
        cf = np.where(cf > 0.0, 1.0, 0.0)
    cf = np.where(atm.play > 100.0, cf, 0.0)
    ciwp = np.where(atm.play < 600.0, rng.uniform(0.0, 40.0, (L, n)) ** 1.3, 0.0)
    clwp = np.where(atm.play > 300.0, rng.uniform(0.0, 60.0, (L, n)) ** 1.2, 0.0)
    ciwp[rng.uniform(size=(L, n)) < 0.1] = 0.0
    dry = rng.uniform(size=(L, n)) < 0.05
    ciwp[dry] = 0.0
    clwp[dry] = 0.0
    reice = rng.uniform(14.0, 125.0, (L, n))
    reliq = rng.uniform(3.0, 55.0, (L, n))
    reice.flat[::17] = 130.0
    reliq.flat[::13] = 2.5
    reliq.flat[5::19] = 60.0
    return dict(cldfr=cf, cicewp=ciwp, cliqwp=clwp, reice=reice, reliq=reliq)


def _lw_given(blob, atm, phys, iceflag):
    L, n = atm.nlay, atm.ncol
    tau = CO.lw_taucloud(blob, phys["cicewp"].T, phys["cliqwp"].T, phys["reice"].T, phys["reliq"].T, iceflag)
    tau = tau.reshape(n, L, 16).transpose(1, 0, 2)
    return dict(cldfr=phys["cldfr"], taucld=tau, cicewp=phys["cicewp"], cliqwp=phys["cliqwp"])


@pytest.mark.parametrize("iceflag", [2, 3])
@pytest.mark.parametrize("icld", [1, 2])
def test_lw_physics_matches_given_optics(orc, blob, iceflag, icld):
    """inflag = 2 with iceflag 2 / 3 and liqflag 1 forms the 16 bands' depths
    from the tables; the same depths given directly (inflag = 0) give the
    same fluxes to rounding."""
    atm = A.small_atmosphere(24, 40, seed=11)
    phys = physics_fields(atm, np.random.default_rng(3))
    r = orc.rrtmg_lw(atm, idrv=1, icld=icld, cloud=dict(phys, inflag=2, iceflag=iceflag, liqflag=1))
    g = orc.rrtmg_lw(atm, idrv=1, icld=icld, cloud=_lw_given(blob, atm, phys, iceflag))
    for k in r:
        np.testing.assert_allclose(r[k], g[k], rtol=1e-11, atol=1e-9, err_msg=k)
    clear = orc.rrtmg_lw(atm, idrv=1)
    assert np.abs(r["uflx"][-1] - clear["uflx"][-1]).max() > 5.0


def test_lw_physics_five_band_ice(orc, blob):
    """iceflag = 1 keeps 5 ice bands; with liquid (liqflag 1) in every cloudy
    layer the column holds 16 cloud bands and each maps onto its ice band
    through icb."""
    atm = A.small_atmosphere(16, 40, seed=12)
    phys = physics_fields(atm, np.random.default_rng(4))
    cloudy = (phys["cldfr"] > 0.0)
    phys["cliqwp"] = np.where(cloudy, np.maximum(phys["cliqwp"], 0.5), 0.0)
    phys["cicewp"] = np.where(cloudy, phys["cicewp"], 0.0)
    r = orc.rrtmg_lw(atm, cloud=dict(phys, inflag=2, iceflag=1, liqflag=1))
    g = orc.rrtmg_lw(atm, cloud=_lw_given(blob, atm, phys, 1))
    for k in r:
        np.testing.assert_allclose(r[k], g[k], rtol=1e-11, atol=1e-9, err_msg=k)


def test_lw_physics_single_band(orc, blob):
    """inflag = 1 forms abscld1 x (ciwp + clwp) in all 16 bands: bit for bit
    the same as that depth given; iceflag 0 / liqflag 0 keep one cloud band,
    which an opaque cloud cannot tell from 16."""
    atm = A.small_atmosphere(16, 40, seed=13)
    L, n = atm.nlay, atm.ncol
    phys = physics_fields(atm, np.random.default_rng(5))
    T = CO._tab(blob)
    r = orc.rrtmg_lw(atm, idrv=1, cloud=dict(phys, inflag=1))
    tau = np.repeat((T["lwcld.abscld1"][0] * (phys["cicewp"] + phys["cliqwp"]))[:, :, None], 16, axis=2)
    g = orc.rrtmg_lw(atm, idrv=1, cloud=dict(phys, taucld=tau))
    for k in r:
        assert np.array_equal(r[k], g[k]), k
    k = 14
    cf, z = np.zeros((L, n)), np.zeros((L, n))
    cf[k] = 1.0
    thick = dict(cldfr=cf, cicewp=z + np.where(np.arange(L) == k, 1e6, 0.0)[:, None], cliqwp=z,
                 reice=z + 50.0, reliq=z + 10.0)
    one = orc.rrtmg_lw(atm, cloud=dict(thick, inflag=2, iceflag=0, liqflag=0))
    many = orc.rrtmg_lw(atm, cloud=dict(thick, inflag=2, iceflag=2, liqflag=1))
    for name in ("uflx", "dflx"):
        np.testing.assert_allclose(one[name], many[name], rtol=1e-12, atol=1e-9)


@pytest.mark.parametrize("iceflag", [1, 2, 3])
def test_sw_physics_matches_given_optics(orc, blob, iceflag):
    """inflag = 2 forms the 14 bands' delta-scaled optics; given as optics
    with no forward fraction (inflag = 0, fsfcld = 0, where delta-M is the
    identity) they give the same fluxes to rounding."""
    atm = A.small_atmosphere(24, 40, seed=14)
    L, n = atm.nlay, atm.ncol
    phys = physics_fields(atm, np.random.default_rng(6), overcast=True)
    r = orc.rrtmg_sw(atm, cloud=dict(phys, inflag=2, iceflag=iceflag, liqflag=1))
    args = [phys[k].T for k in ("cicewp", "cliqwp", "reice", "reliq")]
    tau, ssa, asm = (a.reshape(n, L, 14).transpose(1, 0, 2) for a in CO.sw_cloud(blob, *args, iceflag))
    wet = (phys["cicewp"] + phys["cliqwp"] > 0.0)[:, :, None]
    given = dict(cldfr=phys["cldfr"], taucld=np.where(wet, tau, 0.0), ssacld=np.where(wet, ssa, 1.0),
                 asmcld=np.where(wet, asm, 0.0), fsfcld=np.zeros_like(tau))
    g = orc.rrtmg_sw(atm, cloud=given)
    for k in r:
        np.testing.assert_allclose(r[k], g[k], rtol=1e-11, atol=1e-9, err_msg=k)
    clear = orc.rrtmg_sw(atm)
    assert np.abs(r["swuflx"][-1] - clear["swuflx"][-1]).max() > 20.0


@pytest.mark.parametrize("case", [
    ("lw", dict(iceflag=0, liqflag=0), "reice", 9.0),
    ("lw", dict(iceflag=1, liqflag=1), "reice", 131.0),
    ("lw", dict(iceflag=2, liqflag=1), "reice", 4.0),
    ("lw", dict(iceflag=3, liqflag=1), "reice", 141.0),
    ("lw", dict(iceflag=2, liqflag=1), "reliq", 61.0),
    ("sw", dict(iceflag=1, liqflag=1), "reice", 12.0),
    ("sw", dict(iceflag=2, liqflag=1), "reice", 132.0),
    ("sw", dict(iceflag=3, liqflag=1), "reice", 141.0),
    ("sw", dict(iceflag=3, liqflag=1), "reliq", 2.0),
])
def test_physics_size_out_of_range_stops(orc, case):
    """A size outside its table in a layer whose optics are formed stops the
    reference's cldprop / cldprop_sw; the oracle reports it.  The same size
    in a layer without that water is not looked at."""
    from oracle import oracle as O
    side, flags, key, bad = case
    atm = A.small_atmosphere(8, 40, seed=15)
    phys = physics_fields(atm, np.random.default_rng(7), overcast=side == "sw")
    water = "cicewp" if key == "reice" else "cliqwp"
    col = int(np.argmax(atm.coszen))  # a sunlit column: the SW looks at no other
    lay = int(np.argmin(np.abs(atm.play[:, col] - 450.0)))
    phys["cldfr"][lay, col] = 1.0
    phys[water][lay, col] = 5.0
    phys[key][lay, col] = bad
    call = orc.rrtmg_lw if side == "lw" else orc.rrtmg_sw
    with pytest.raises(O.CloudRangeError):
        call(atm, cloud=dict(phys, inflag=2, **flags))
    phys[water][lay, col] = 0.0
    call(atm, cloud=dict(phys, inflag=2, **flags))


# secdiff of a column without water vapour (pwvcm = 0): a0 + a1 clipped to
# [1.50, 1.80], 1.66 in bands 1, 4 and 10-16 (rrtmg_lw_rtrnmr.f90:271-279)
_A0 = [1.66, 1.55, 1.58, 1.66, 1.54, 1.454, 1.89, 1.33, 1.668] + [1.66] * 7
_A1 = [0.00, 0.25, 0.22, 0.00, 0.13, 0.446, -0.10, 0.40, -0.006] + [0.00] * 7


def _secdiff_dry():
    s = []
    for b in range(1, 17):
        if b in (1, 4) or b >= 10:
            s.append(1.66)
        else:
            v = _A0[b - 1] + _A1[b - 1] * 1.0
            s.append(1.80 if v > 1.80 else 1.50 if v < 1.50 else v)
    return np.array(s)


def test_lw_physics_running_band_count(orc, blob):
    """cldprop's count of cloud bands runs across its layer loop, and rtrn
    takes band b's cloud depth from cloud band ipat(b, count) along that
    cloud band's diffusivity angle: two lower layers of ice and liquid
    (iceflag 1, liqflag 1: 16 cloud bands) under an ice-only layer (5 cloud
    bands) leave the whole column with 5, so every layer's depth in band b is
    secdiff(ib) x taucloud(ib), ib = ipat(b, 5), with the ice coefficient band
    icb(ib, 1) in the mixed layers and ib in the ice-only one.  Stated here
    from the tables in a dry column (known secdiff) and handed to the given-
    depth path, the fluxes agree."""
    atm = A.small_atmosphere(6, 40, seed=21)
    atm.h2o = np.zeros_like(atm.h2o)
    L, n = atm.nlay, atm.ncol
    k1, k2 = (int(np.argmin(np.abs(atm.play[:, 0] - p))) for p in (800.0, 600.0))
    k3 = int(np.argmin(np.abs(atm.play[:, 0] - 300.0)))
    assert k1 < k2 < k3
    z = np.zeros((L, n))
    cf, ciwp, clwp, rei, rel = z.copy(), z.copy(), z.copy(), z + 40.0, z + 10.0
    col = lambda *v: np.array(v)[:, None]
    cf[[k1, k2, k3]] = col(0.7, 0.6, 0.5)
    ciwp[[k1, k2, k3]] = col(8.0, 15.0, 30.0)
    clwp[[k1, k2]] = col(60.0, 25.0)
    rei[[k1, k2, k3]] = col(25.0, 50.0, 90.0)
    rel[[k1, k2]] = col(7.0, 14.0)
    phys = dict(cldfr=cf, cicewp=ciwp, cliqwp=clwp, reice=rei, reliq=rel)
    r = orc.rrtmg_lw(atm, idrv=1, cloud=dict(phys, inflag=2, iceflag=1, liqflag=1))

    T = CO._tab(blob)
    ice1 = T["lwcld.absice1"]  # (2, 5)
    sec = _secdiff_dry()
    ipat5 = CO.ICB5  # ipat(b, 5-band count) = icb(b, 1)
    tau = np.zeros((L, n, 16))
    for k in (k1, k2, k3):
        liq = CO.lw_taucloud(blob, np.zeros(n), clwp[k], rei[k], rel[k], 2) / np.maximum(clwp[k], 1e-300)[:, None]
        for b in range(1, 17):
            ib = ipat5[b - 1]
            kice = ipat5[ib - 1] if clwp[k, 0] != 0.0 else ib   # icb(ib, iceind)
            absice = ice1[0, kice - 1] + ice1[1, kice - 1] / rei[k]
            tc = ciwp[k] * absice + (clwp[k] * liq[:, ib - 1] if clwp[k, 0] != 0.0 else 0.0)
            tau[k, :, b - 1] = sec[ib - 1] * tc / sec[b - 1]
    g = orc.rrtmg_lw(atm, idrv=1, cloud=dict(cldfr=cf, taucld=tau, cicewp=ciwp, cliqwp=clwp))
    for key in r:
        np.testing.assert_allclose(r[key], g[key], rtol=1e-11, atol=1e-9, err_msg=key)
    # the count matters: with liquid in the top layer too (16 bands) the fluxes move
    clwp16 = clwp.copy()
    clwp16[k3] = 1.0
    r16 = orc.rrtmg_lw(atm, cloud=dict(phys, cliqwp=clwp16, inflag=2, iceflag=1, liqflag=1))
    assert np.abs(r16["uflx"][-1] - r["uflx"][-1]).max() > 0.1


def test_lw_physics_single_cloud_band(orc, blob):
    """iceflag 0 with liqflag 0 keeps one cloud band (absice0, absliq0): every
    band takes cloud band 1's depth along secdiff(1) = 1.66, stated here in a
    dry column and handed in as given depths."""
    atm = A.small_atmosphere(6, 40, seed=22)
    atm.h2o = np.zeros_like(atm.h2o)
    L, n = atm.nlay, atm.ncol
    rng = np.random.default_rng(23)
    cf = np.where((rng.uniform(size=(L, n)) < 0.3) & (atm.play > 150.0), rng.uniform(0.2, 1.0, (L, n)), 0.0)
    ciwp = np.where(atm.play < 600.0, rng.uniform(0.0, 30.0, (L, n)), 0.0)
    clwp = np.where(atm.play > 400.0, rng.uniform(0.0, 50.0, (L, n)), 0.0)
    rei = rng.uniform(10.0, 120.0, (L, n))
    phys = dict(cldfr=cf, cicewp=ciwp, cliqwp=clwp, reice=rei, reliq=rei * 0 + 10.0)
    r = orc.rrtmg_lw(atm, cloud=dict(phys, inflag=2, iceflag=0, liqflag=0), icld=2)
    T = CO._tab(blob)
    ice0, liq0 = T["lwcld.absice0"], T["lwcld.absliq0"][0]
    tc = np.where(ciwp != 0.0, ciwp * (ice0[0] + ice0[1] / rei), 0.0) + clwp * liq0
    sec = _secdiff_dry()
    tau = (1.66 * tc)[:, :, None] / sec[None, None, :]
    g = orc.rrtmg_lw(atm, cloud=dict(cldfr=cf, taucld=tau, cicewp=ciwp, cliqwp=clwp), icld=2)
    for key in r:
        np.testing.assert_allclose(r[key], g[key], rtol=1e-11, atol=1e-9, err_msg=key)
