"""The CPU oracle against physical known answers and internal consistency.

The reference ships no golden vectors for this path (no tests; the LW
known-answer files in doc_rrtm need LW coefficient data that is not in the
distribution), so these checks pin what physics pins independently of the
k-distribution: blackbody emission of isothermal columns (Planck tables, flux
factors, band widths), the incident solar flux (Kurucz source, scon scaling),
flux/heating-rate bookkeeping, and the sign of gas sensitivities.
"""
import numpy as np
import pytest

from mima_gb300 import atmosphere as A

SIGMA = 5.670374419e-8
HEATFAC = 9.8066 * 86400.0 / (1004.64 * 1.0e2)


def test_isothermal_column_emits_blackbody(orc):
    for T in (220.0, 288.0, 310.0):
        atm = A.small_atmosphere(16, 40, seed=1)
        atm.tlay[:] = T
        atm.tlev[:] = T
        atm.tsfc[:] = T
        lw = orc.rrtmg_lw(atm)
        bb = SIGMA * T ** 4
        assert np.allclose(lw["uflx"], bb, rtol=0.01), (T, lw["uflx"].min(), lw["uflx"].max(), bb)
        assert np.all(lw["dflx"][0] <= bb * 1.01)
        # an isothermal column cools to space; it can not heat anywhere
        assert lw["hr"].max() < 0.05


def test_toa_insolation(orc):
    atm = A.small_atmosphere(32, 40, seed=2)
    sw = orc.rrtmg_sw(atm)
    toa = sw["swdflx"][-1]
    assert np.allclose(toa, atm.scon * atm.coszen, rtol=2e-3)
    atm.scon = 1368.22 * 1.1
    sw2 = orc.rrtmg_sw(atm)
    assert np.allclose(sw2["swdflx"], sw["swdflx"] * (1368.22 * 1.1 / 1360.0), rtol=1e-12)


def scattering_only(ncol=8, nlay=40, seed=5, albedo=1.0):
    """Columns without absorbers (no H2O, O3, CO2, CH4, N2O, O2): in the SW
    only Rayleigh scattering remains."""
    atm = A.small_atmosphere(ncol, nlay, seed=seed)
    for k in ("h2o", "o3", "co2", "ch4", "n2o", "o2"):
        setattr(atm, k, np.zeros_like(atm.play))
    atm.coszen = np.linspace(0.1, 1.0, ncol)
    for k in ("asdir", "asdif", "aldir", "aldif"):
        setattr(atm, k, np.full(ncol, albedo))
    return atm


@pytest.mark.parametrize("albedo", [1.0, 0.3, 0.0])
def test_sw_conserves_energy_without_absorbers(orc, albedo):
    """Pure scattering absorbs nothing: the net SW flux is the same at every
    level (no heating), and with a white surface it is zero -- everything
    that comes in goes back out at the top.  The reference caps the single
    scattering albedo at oneminus = 1 - 1e-6 (rrtmg_sw_rad.nomcica.f90:447), so
    a layer keeps up to 1e-6 of what it extinguishes: 1e-3 W/m2 of 1300 in all
    here.  Checks reftra's conservative branch and the adding method without
    any k-table."""
    atm = scattering_only(albedo=albedo)
    for tables_mode in (True, False):
        orc.set_table_mode(tables_mode)
        try:
            sw = orc.rrtmg_sw(atm)
        finally:
            orc.set_table_mode(True)
        L = atm.nlay
        net = sw["swdflx"] - sw["swuflx"]
        assert np.abs(net - net[L]).max() <= 1e-3
        assert np.abs(sw["swhr"]).max() <= 1e-5
        if albedo == 1.0:
            assert np.abs(net[L]).max() <= 1e-3
        else:  # the surface absorbs (1 - albedo) of what reaches it, and something does
            assert (net[0] > 0.0).all()


def test_heating_rates_follow_from_fluxes(orc):
    atm = A.small_atmosphere(32, 60, seed=3)
    lw = orc.rrtmg_lw(atm)
    sw = orc.rrtmg_sw(atm)
    dp = atm.plev[:-1] - atm.plev[1:]
    fnet = lw["uflx"] - lw["dflx"]
    hr = HEATFAC * (fnet[:-1] - fnet[1:]) / dp
    assert np.allclose(lw["hr"], hr, rtol=1e-12, atol=1e-12)
    snet = sw["swdflx"] - sw["swuflx"]
    shr = (snet[1:] - snet[:-1]) * HEATFAC / dp
    shr[-1] = 0.0  # MiMA zeroes the top SW layer
    assert np.allclose(sw["swhr"], shr, rtol=1e-12, atol=1e-12)
    # clear-sky outputs equal total-sky outputs in clear sky
    assert np.array_equal(lw["uflx"], lw["uflxc"]) and np.array_equal(sw["swuflx"], sw["swuflxc"])
    # absorbed SW is positive and bounded by the incident flux
    absorbed = snet[-1] - snet[0]
    assert np.all(absorbed > 0) and np.all(absorbed < sw["swdflx"][-1])


def test_gas_sensitivities(orc):
    atm = A.small_atmosphere(32, 40, seed=4)
    base_lw, base_sw = orc.rrtmg_lw(atm), orc.rrtmg_sw(atm)
    atm.co2 = atm.co2 * 2.0
    lw2 = orc.rrtmg_lw(atm)
    assert np.all(lw2["dflx"][0] > base_lw["dflx"][0])   # more back-radiation
    assert np.mean(lw2["uflx"][-1]) < np.mean(base_lw["uflx"][-1])  # lower OLR on average
    atm.co2 = atm.co2 / 2.0
    atm.h2o = atm.h2o * 1.5
    sw2 = orc.rrtmg_sw(atm)
    assert np.all(sw2["swdflx"][0] < base_sw["swdflx"][0])  # more SW absorption by water vapour


def test_dark_column_is_skipped(orc):
    atm = A.small_atmosphere(4, 40, seed=5)
    atm.coszen[1] = 0.0
    sw = orc.rrtmg_sw(atm)
    for k in ("swuflx", "swdflx", "swhr"):
        assert np.all(sw[k][:, 1] == 0.0)
    assert np.all(sw["swdflx"][-1, [0, 2, 3]] > 0)


def test_table_and_analytic_modes_agree_closely(orc):
    """The lookup tables sample exp / the tau transition function at 1e-4 in
    tau/(tau + 1/0.278); analytic evaluation differs by well under 0.5%."""
    atm = A.small_atmosphere(16, 40, seed=6)
    t_lw, t_sw = orc.rrtmg_lw(atm), orc.rrtmg_sw(atm)
    orc.set_table_mode(False)
    try:
        a_lw, a_sw = orc.rrtmg_lw(atm), orc.rrtmg_sw(atm)
    finally:
        orc.set_table_mode(True)
    assert np.allclose(a_lw["uflx"], t_lw["uflx"], rtol=5e-3)
    assert np.allclose(a_sw["swdflx"], t_sw["swdflx"], rtol=5e-3, atol=1e-3)


def test_idrv_matches_finite_difference_of_surface_temperature(orc):
    """dF_up/dTs (idrv = 1) against a central difference in Ts in analytic mode."""
    atm = A.small_atmosphere(8, 40, seed=8)
    orc.set_table_mode(False)
    try:
        d = orc.rrtmg_lw(atm, idrv=1)["duflx_dt"]
        h = 0.01
        atm.tsfc = atm.tsfc + h
        up = orc.rrtmg_lw(atm)["uflx"]
        atm.tsfc = atm.tsfc - 2 * h
        dn = orc.rrtmg_lw(atm)["uflx"]
    finally:
        orc.set_table_mode(True)
    fd = (up - dn) / (2 * h)
    # idrv uses the separately tabulated Planck derivative totplnkderiv
    # (rrtmg_lw_setcoef.f90:1287-1990), not the slope of the interpolated
    # totplnk, so the two agree to the tables' mutual consistency (~0.3%).
    assert np.allclose(d, fd, rtol=1e-2, atol=1e-4)


def test_oracle_reproduces_golden_fixtures(orc):
    """Regression fixtures of the oracle (tests/golden/make_golden.py)."""
    import importlib.util
    from pathlib import Path
    from mima_gb300 import tables
    g = Path(__file__).with_name("golden")
    ref = np.load(g / "oracle_regression.npz")
    blob = Path(tables.ensure_blob()).read_bytes()
    assert int(ref["blob_checksum"][0]) == tables.blob_checksum(blob), "table blob differs from the fixtures'"
    spec = importlib.util.spec_from_file_location("make_golden", g / "make_golden.py")
    mk = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mk)
    now = mk.compute()
    for k in ref.files:
        if k == "blob_checksum":
            continue
        np.testing.assert_allclose(now[k], ref[k], rtol=1e-11, atol=1e-12, err_msg=k)


def test_phase_times_cover_the_call(orc):
    """Where the time goes (orc_*_phase_times): every phase takes time, and the
    phases together account for a plain single-threaded call of the same
    columns (loose bounds: timings on a shared host)."""
    import time
    atm = A.small_atmosphere(64, 40, seed=8)
    lw, sw = orc.phase_times(atm)
    assert set(lw) == set(orc.LW_PHASES) and set(sw) == set(orc.SW_PHASES)
    assert all(v > 0 for v in list(lw.values()) + list(sw.values()))
    t0 = time.perf_counter()
    orc.rrtmg_lw(atm, nthreads=1)
    t1 = time.perf_counter()
    orc.rrtmg_sw(atm, nthreads=1)
    t2 = time.perf_counter()
    lit = int((atm.coszen >= 1e-10).sum())
    assert 0.2 <= sum(lw.values()) * atm.ncol / (t1 - t0) <= 5.0
    assert 0.2 <= sum(sw.values()) * lit / (t2 - t1) <= 5.0


def edge_columns():
    """Columns at the edges of the layer structure: the fewest layers (2, 3);
    a column wholly below the troposphere boundary ln p = 4.56 (200-1000 hPa:
    laytrop = nlay, so the lower-atmosphere loops reach the last layer and the
    upper ones are empty); one wholly above it (0.1-90 hPa: laytrop = 0)."""
    def remap(atm, top, bot, log=False):
        pt, pb = atm.plev[-1, 0], atm.plev[0, 0]
        if log:
            k = (np.log(bot) - np.log(top)) / (np.log(pb) - np.log(pt))
            f = lambda p: np.exp(np.log(top) + (np.log(p) - np.log(pt)) * k)
        else:
            f = lambda p: top + (p - pt) * (bot - top) / (pb - pt)
        atm.plev, atm.play = f(atm.plev), f(atm.play)
        return atm
    return {"nlay2": A.small_atmosphere(33, 2, seed=71), "nlay3": A.small_atmosphere(33, 3, seed=72),
            "below_tropopause": remap(A.small_atmosphere(33, 20, seed=73), 200.0, 1000.0),
            "above_tropopause": remap(A.small_atmosphere(33, 20, seed=74), 0.1, 90.0, log=True)}


def test_edge_columns(orc):
    cols = edge_columns()
    lt = {k: (np.log(a.play) > 4.56).sum(axis=0) for k, a in cols.items()}
    assert (lt["below_tropopause"] == 20).all() and (lt["above_tropopause"] == 0).all()
    for k, atm in cols.items():
        lw, sw = orc.rrtmg_lw(atm), orc.rrtmg_sw(atm)
        for d in (lw, sw):
            for name, v in d.items():
                assert np.isfinite(v).all(), (k, name)
        assert (lw["uflx"] > 0).all() and (sw["swdflx"][-1] > 0).all(), k


def test_gas_optics_stage(orc, blob):
    """The gas-optics stage on its own (orc_lw_optics / orc_sw_optics): in
    every layer the Planck fractions of a band sum to 1 over its g-points (the
    eta-interpolation weights sum to 1), except in LW bands 12 and 15 above
    the troposphere boundary, which have no upper-atmosphere absorber (optical
    depth and fractions 0, rrtmg_lw_taumol.f90 taugb12 / taugb15); the SW
    solar source of every column sums to the Kurucz total, 1368.22 W/m2; the
    Rayleigh optical depths are positive."""
    from mima_gb300 import tables
    atm = A.small_atmosphere(16, 40, seed=3, ts_sigma=8.0)
    taug, fracs, laytrop = orc.lw_optics(atm)
    ngc = tables.read_blob(blob)["lw.ngc"][0].ravel()
    edges = np.concatenate([[0], np.cumsum(ngc)])
    upper = np.arange(atm.nlay)[:, None] >= laytrop[None, :]
    for b in range(16):
        s = fracs[edges[b]:edges[b + 1]].sum(axis=0)
        if b + 1 in (12, 15):
            np.testing.assert_allclose(s[~upper], 1.0, atol=1e-12)
            assert (s[upper] == 0.0).all() and (taug[edges[b]:edges[b + 1]][:, upper] == 0.0).all()
        else:
            np.testing.assert_allclose(s, 1.0, atol=1e-12, err_msg=f"band {b + 1}")
    gtaug, taur, sfz = orc.sw_optics(atm)
    np.testing.assert_allclose(sfz.sum(axis=0), 1368.22, rtol=1e-5)
    assert (taur > 0).all() and (gtaug >= 0).all()


def test_lw_clouds_random_overlap(orc):
    """The oracle's LW clouds (icld = 1, rtrn with cldprop inflag = 0):
    * icld = 1 with no cloud reproduces clear sky bit for bit;
    * the clear-sky outputs of a cloudy call are the clear-sky call's;
    * an opaque overcast layer (cover 1, depth 1e3 in every band) emits as a
      blackbody at its own temperature, so the OLR of an isothermal column above
      it is sigma T^4 of that temperature;
    * random overlap is linear in the cover of a single cloudy layer: the
      fluxes at half cover are the mean of clear and overcast;
    * cldprop keeps no optical depth for a layer with cover but neither depth
      nor water path, and rtrn treats a cover below 1e-6 as clear."""
    atm = A.small_atmosphere(24, 40, seed=5)
    L, n = atm.nlay, atm.ncol
    clear = orc.rrtmg_lw(atm, idrv=1)
    none = orc.rrtmg_lw(atm, idrv=1, cloud=dict(cldfr=np.zeros((L, n)), taucld=np.zeros((L, n, 16))))
    for k in clear:
        assert np.array_equal(none[k], clear[k]), k
    k = 12
    cf = np.zeros((L, n))
    cf[k] = 1.0
    tau = np.zeros((L, n, 16))
    tau[k] = 1.0e3
    over = orc.rrtmg_lw(atm, idrv=1, cloud=dict(cldfr=cf, taucld=tau))
    for name in ("uflx", "dflx", "hr", "duflx_dt"):
        c = "hrc" if name == "hr" else name[:-3] + "c_dt" if name == "duflx_dt" else name + "c"
        assert np.allclose(over[c], clear[name], rtol=1e-12, atol=1e-12), name
    half = orc.rrtmg_lw(atm, cloud=dict(cldfr=cf * 0.5, taucld=tau))
    assert np.allclose(half["uflx"], 0.5 * (clear["uflx"] + over["uflx"]), rtol=2e-3)
    # isothermal stratosphere above an opaque cloud: OLR = sigma T^4
    iso = A.small_atmosphere(8, 40, seed=6)
    T = 230.0
    iso.tlay[k:] = T
    iso.tlev[k:] = T
    cfi, taui = np.zeros((L, iso.ncol)), np.zeros((L, iso.ncol, 16))
    cfi[k], taui[k] = 1.0, 1.0e3
    lw = orc.rrtmg_lw(iso, cloud=dict(cldfr=cfi, taucld=taui))
    assert np.allclose(lw["uflx"][-1], SIGMA * T ** 4, rtol=0.02), (lw["uflx"][-1], SIGMA * T ** 4)
    # no depth and no water path: no cloud optical depth; cover < 1e-6: clear layer
    zero = orc.rrtmg_lw(atm, cloud=dict(cldfr=cf, taucld=np.zeros_like(tau)))
    assert np.allclose(zero["uflx"], clear["uflx"], rtol=1e-12, atol=1e-9)
    tiny = orc.rrtmg_lw(atm, cloud=dict(cldfr=cf * 5e-7, taucld=tau))
    assert np.array_equal(tiny["uflx"], clear["uflx"])


def sw_cloud_fields(atm, rng, partial_night=True):
    """Seeded SW clouds below 100 hPa: every layer clear or overcast (cover 0 or
    1; a few at 5e-7 and 1 - 5e-7, inside the reference's 1e-6 margins),
    per-band optical depths up to 75, single-scattering albedo 0.8-1,
    asymmetry 0.7-0.9 with the delta-M forward fraction g^2; some overcast
    layers without depth or water path.  With ``partial_night``, unlit columns
    carry partly cloudy layers (the reference checks sunlit columns only)."""
    L, n = atm.nlay, atm.ncol
    u = rng.uniform(size=(L, n))
    cf = np.where(u < 0.3, 1.0, 0.0)
    cf[u > 0.98] = 5e-7
    cf[(u > 0.96) & (u <= 0.98)] = 1.0 - 5e-7
    cf = np.where(atm.play > 100.0, cf, 0.0)
    if partial_night:
        night = np.asarray(atm.coszen) < 1e-10
        cf[:, night] = rng.uniform(0.2, 0.8, (L, int(night.sum())))
    tau = (rng.uniform(0.0, 1.0, (L, n, 1)) ** 3 * 50.0) * rng.uniform(0.5, 1.5, (L, n, 14))
    tau[rng.uniform(size=(L, n)) < 0.03] = 0.0
    ssa = rng.uniform(0.8, 1.0, (L, n, 14))
    ssa[rng.uniform(size=(L, n, 14)) < 0.05] = 1.0
    asm = rng.uniform(0.7, 0.9, (L, n, 14))
    return dict(cldfr=cf, taucld=tau, ssacld=ssa, asmcld=asm, fsfcld=asm * asm)


def test_sw_clouds_overcast(orc):
    """The oracle's SW clouds (icld = 1, cldprop_sw inflag = 0, spcvrt's
    clear/total passes):
    * icld = 1 with no cloud reproduces clear sky bit for bit, and the
      clear-sky outputs of a cloudy call are the clear-sky call's;
    * a thick overcast layer raises the reflected flux at the top and cuts
      the surface downward flux;
    * a scattering-only cloud (albedo 1) over a transparent column with black
      ground sends all the sunlight either back up or down to the ground;
    * an overcast layer without depth or water path keeps no cloud optics;
    * a partly cloudy sunlit layer is refused as the reference stops, a partly
      cloudy unlit one is not looked at."""
    from oracle import oracle as O
    atm = A.small_atmosphere(24, 40, seed=5)
    L, n = atm.nlay, atm.ncol
    z14 = np.zeros((L, n, 14))
    clear = orc.rrtmg_sw(atm)
    none = orc.rrtmg_sw(atm, cloud=dict(cldfr=np.zeros((L, n)), taucld=z14, ssacld=z14 + 1, asmcld=z14,
                                        fsfcld=z14))
    for k in clear:
        assert np.array_equal(none[k], clear[k]), k
    k = 10
    cf = np.zeros((L, n))
    cf[k] = 1.0
    tau, ssa, asm = z14.copy(), z14 + 0.999, z14 + 0.85
    tau[k] = 40.0
    cl = dict(cldfr=cf, taucld=tau, ssacld=ssa, asmcld=asm, fsfcld=asm * asm)
    over = orc.rrtmg_sw(atm, cloud=cl)
    for name in ("swuflx", "swdflx", "swhr"):
        assert np.array_equal(over[name + "c" if name != "swhr" else "swhrc"], clear[name]), name
    assert np.all(over["swuflx"][-1] > 2.0 * clear["swuflx"][-1])
    assert np.all(over["swdflx"][0] < 0.6 * clear["swdflx"][0])
    # cover without depth or water path: no cloud optics (rounding only)
    noop = orc.rrtmg_sw(atm, cloud=dict(cl, taucld=z14))
    assert np.allclose(noop["swuflx"], clear["swuflx"], rtol=1e-12, atol=1e-9)
    # scattering-only cloud, no absorbers, black ground: up at the top + down at the ground = incident
    dry = A.small_atmosphere(6, 40, seed=3)
    for g in ("h2o", "o3", "co2", "ch4", "n2o", "o2"):
        setattr(dry, g, np.zeros_like(getattr(dry, g)))
    for a in ("asdir", "asdif", "aldir", "aldif"):
        setattr(dry, a, np.zeros_like(getattr(dry, a)))
    cfd = np.zeros((L, dry.ncol))
    cfd[k] = 1.0
    taud = np.zeros((L, dry.ncol, 14))
    taud[k] = 25.0
    sca = dict(cldfr=cfd, taucld=taud, ssacld=taud * 0 + 1.0, asmcld=taud * 0 + 0.85, fsfcld=taud * 0 + 0.85 ** 2)
    s = orc.rrtmg_sw(dry, cloud=sca)
    assert np.allclose(s["swuflx"][-1] + s["swdflx"][0], s["swdflx"][-1], rtol=1e-6)
    assert np.all(s["swuflx"][-1] > 0.3 * s["swdflx"][-1])
    # partial cover: refused in a sunlit column, ignored in an unlit one
    part = dict(cl, cldfr=cf * 0.5)
    with pytest.raises(O.PartialCloud):
        orc.rrtmg_sw(atm, cloud=part)
    night = A.small_atmosphere(24, 40, seed=5)
    night.coszen = np.zeros_like(night.coszen)
    dark = orc.rrtmg_sw(night, cloud=part)
    assert not any(np.any(v) for v in dark.values())


def test_lw_clouds_maximum_random_overlap(orc):
    """The oracle's maximum/random overlap (icld = 2, 3: rtrnmr's cloudy
    branches):
    * with no cloud it reproduces clear sky bit for bit, for icld = 2 and 3;
    * isolated cloudy layers overlap the same way under every assumption, so
      it agrees with random overlap up to the transmittance tables' steps;
    * two adjacent opaque layers of equal cover c overlap maximally: the
      fluxes are (1 - c) x clear sky + c x overcast, where random overlap
      leaves less of the column clear;
    * fully overcast layers are the same under both overlaps."""
    atm = A.small_atmosphere(24, 40, seed=5)
    L, n = atm.nlay, atm.ncol
    clear = orc.rrtmg_lw(atm, idrv=1)
    z = dict(cldfr=np.zeros((L, n)), taucld=np.zeros((L, n, 16)))
    for icld in (2, 3):
        r = orc.rrtmg_lw(atm, idrv=1, cloud=z, icld=icld)
        for k in clear:
            assert np.array_equal(r[k], clear[k]), (icld, k)
    cf, tau = np.zeros((L, n)), np.zeros((L, n, 16))
    cf[8], cf[15], cf[22] = 0.4, 0.7, 0.3
    tau[8], tau[15], tau[22] = 2.0, 5.0, 1.0
    iso = dict(cldfr=cf, taucld=tau)
    a, b = orc.rrtmg_lw(atm, idrv=1, cloud=iso, icld=1), orc.rrtmg_lw(atm, idrv=1, cloud=iso, icld=2)
    for k in ("uflx", "dflx"):
        assert np.abs(a[k] - b[k]).max() < 2e-3, k
    assert np.array_equal(a["duflx_dt"], b["duflx_dt"])
    c2, t2 = np.zeros((L, n)), np.zeros((L, n, 16))
    c2[12:14], t2[12:14] = 0.5, 1e3
    half_mr = orc.rrtmg_lw(atm, cloud=dict(cldfr=c2, taucld=t2), icld=2)
    half_r = orc.rrtmg_lw(atm, cloud=dict(cldfr=c2, taucld=t2), icld=1)
    over = orc.rrtmg_lw(atm, cloud=dict(cldfr=2 * c2, taucld=t2), icld=2)
    for k in ("uflx", "dflx"):
        assert np.allclose(half_mr[k], 0.5 * (clear[k] + over[k]), rtol=1e-12, atol=1e-9), k
    assert np.all(half_mr["uflx"][-1] > half_r["uflx"][-1] + 5.0)
    over_r = orc.rrtmg_lw(atm, cloud=dict(cldfr=2 * c2, taucld=t2), icld=1)
    assert np.allclose(over["uflx"], over_r["uflx"], rtol=1e-12, atol=1e-9)
