"""The oracle's McICA stochastic cloud generator (mcica_subcol_gen_lw.f90 /
mcica_subcol_gen_sw.f90 with mcica_random_numbers.f90), CPU:
* its Mersenne Twister against numpy's MT19937 with the same scalar seeding;
* the sub-column masks: the cloudy share of every layer is its cover, binary
  covers give binary masks, maximum overlap nests the masks by cover,
  maximum/random overlap keeps adjacent layers of equal cover identical,
  random overlap draws layers independently;
* the band optics of a cloudy sub-column are those of its g-point's band,
  clear sub-columns carry the clear values;
* the reference's stops: kissvec's seeding needs the layers from the surface
  up, icld must be in 0..3;
* McICA LW (cldprmc, rtrnmc of rrtmg_lw_cldprmc.f90 / rrtmg_lw_rtrnmc.f90):
  binary covers reproduce rtrn's random overlap bit for bit, with given
  depths and with cldprmc's ice / liquid parameterisations; partial covers
  move the fluxes with the overlap;
* McICA SW (cldprmc_sw, spcvmc_sw of rrtmg_sw_cldprmc.f90 /
  rrtmg_sw_spcvmc.f90): the same pins against spcvrt on clear / overcast
  layers, and the McICA driver's dark columns (computed at cos(zenith) =
  1e-10, not skipped)."""
import numpy as np
import pytest

from mima_gb300 import atmosphere as A


@pytest.mark.parametrize("seed", [1, 5489, 123456789])
def test_mersenne_twister_matches_numpy(orc, seed):
    bg = np.random.MT19937()
    bg._legacy_seeding(seed)
    assert np.array_equal(orc.mt_ints(seed, 2000), bg.random_raw(2000).astype(np.uint32))


def _clouds(atm, rng, binary=False):
    L, n = atm.nlay, atm.ncol
    cf = rng.uniform(0.05, 1.0, (L, n)) * (rng.uniform(size=(L, n)) < 0.5)
    if binary:
        cf = np.where(cf > 0.0, 1.0, 0.0)
    cf = np.where(atm.play > 150.0, cf, 0.0)
    tau = rng.uniform(0.5, 20.0, (L, n, 16))
    return dict(cldfr=cf, cicewp=cf * 11.0, cliqwp=cf * 23.0, taucld=tau)


@pytest.mark.parametrize("irng", [0, 1])
@pytest.mark.parametrize("icld", [1, 2, 3])
def test_subcolumn_cover_is_the_layer_cover(orc, irng, icld):
    atm = A.small_atmosphere(64, 40, seed=31)
    cl = _clouds(atm, np.random.default_rng(32))
    s = orc.mcica_subcol("lw", atm, cl, icld=icld, irng=irng, permuteseed=7)
    share = s["cldfr"].mean(axis=2)           # (nlay, ncol): 140 draws each
    err = np.abs(share - cl["cldfr"])
    # the share of 140 g-points per (layer, column), pooled over the columns
    assert np.abs(share.mean(axis=1) - cl["cldfr"].mean(axis=1)).max() < 0.06
    assert err.mean() < 0.05
    assert set(np.unique(s["cldfr"])) <= {0.0, 1.0}
    cloudy = s["cldfr"] == 1.0
    assert np.array_equal(s["cicewp"], np.where(cloudy, cl["cicewp"][:, :, None], 0.0))
    assert np.array_equal(s["cliqwp"], np.where(cloudy, cl["cliqwp"][:, :, None], 0.0))


def test_binary_covers_give_binary_masks(orc):
    atm = A.small_atmosphere(16, 40, seed=33)
    cl = _clouds(atm, np.random.default_rng(34), binary=True)
    for icld in (1, 2, 3):
        s = orc.mcica_subcol("lw", atm, cl, icld=icld, irng=0)
        assert np.array_equal(s["cldfr"], np.repeat(cl["cldfr"][:, :, None], 140, axis=2)), icld


def test_overlap_structure(orc):
    atm = A.small_atmosphere(32, 40, seed=35)
    L, n = atm.nlay, atm.ncol
    rng = np.random.default_rng(36)
    cf = np.zeros((L, n))
    cf[5:9] = rng.uniform(0.2, 0.8, (4, n))
    cf[12:14] = 0.5
    cl = dict(cldfr=cf, cicewp=cf, cliqwp=cf, taucld=np.ones((L, n, 16)))
    # maximum overlap: a sub-column cloudy in a layer is cloudy in every layer of larger cover
    s3 = orc.mcica_subcol("lw", atm, cl, icld=3, irng=1)["cldfr"] == 1.0
    for a in range(L):
        for b in range(L):
            wider = cf[b] >= cf[a]
            assert np.all(~s3[a] | ~wider[:, None] | s3[b])
    # maximum/random: adjacent layers of equal cover share their masks
    s2 = orc.mcica_subcol("lw", atm, cl, icld=2, irng=1)["cldfr"] == 1.0
    assert np.array_equal(s2[12], s2[13])
    # random overlap: adjacent layers independent (joint share ~ product)
    s1 = orc.mcica_subcol("lw", atm, cl, icld=1, irng=1)["cldfr"] == 1.0
    joint = (s1[12] & s1[13]).mean()
    assert abs(joint - 0.25) < 0.04
    assert abs((s2[12] & s2[13]).mean() - 0.5) < 0.05


def test_band_optics_follow_the_g_point(orc, blob):
    from mima_gb300 import tables
    atm = A.small_atmosphere(8, 40, seed=37)
    L, n = atm.nlay, atm.ncol
    rng = np.random.default_rng(38)
    cf = np.where(atm.play > 150.0, 0.7, 0.0)
    sw = dict(cldfr=cf, cicewp=cf, cliqwp=cf, taucld=rng.uniform(1, 5, (L, n, 14)),
              ssacld=rng.uniform(0.9, 1.0, (L, n, 14)), asmcld=rng.uniform(0.7, 0.9, (L, n, 14)),
              fsfcld=rng.uniform(0.5, 0.8, (L, n, 14)))
    s = orc.mcica_subcol("sw", atm, sw, icld=2, irng=0)
    ngb = np.asarray(tables.read_blob(blob)["sw.ngb"][0]) - 16
    cloudy = s["cldfr"] == 1.0
    assert cloudy.any() and (~cloudy).any()
    for k, clear in (("taucld", 0.0), ("ssacld", 1.0), ("asmcld", 0.0), ("fsfcld", 0.0)):
        want = np.where(cloudy, sw[k][:, :, ngb], clear)
        assert np.array_equal(s[k], want), k


def test_generator_stops(orc):
    atm = A.small_atmosphere(4, 40, seed=39)
    cl = _clouds(atm, np.random.default_rng(40))
    top_down = atm.subset(np.arange(4))
    top_down.play = top_down.play[::-1].copy()
    with pytest.raises(RuntimeError):
        orc.mcica_subcol("lw", top_down, {k: v[::-1].copy() for k, v in cl.items()}, icld=2, irng=0)
    orc.mcica_subcol("lw", top_down, {k: v[::-1].copy() for k, v in cl.items()}, icld=2, irng=1)
    with pytest.raises(RuntimeError):
        orc.mcica_subcol("lw", atm, cl, icld=4)


def test_lw_mcica_binary_covers_equal_random_overlap(orc):
    """rtrnmc on binary sub-columns (every g-point of a layer cloudy or clear)
    is rtrn's random overlap of covers 0 / 1, bit for bit: same depths along
    secdiff(ngb), same cloudy branch."""
    atm = A.small_atmosphere(24, 40, seed=41)
    cl = _clouds(atm, np.random.default_rng(42), binary=True)
    sub = orc.mcica_subcol("lw", atm, cl, icld=2, irng=0)
    mc = orc.rrtmg_lw_mcica(atm, sub, idrv=1)
    ref = orc.rrtmg_lw(atm, idrv=1, cloud=dict(cldfr=cl["cldfr"], taucld=cl["taucld"]), icld=1)
    for k in ref:
        assert np.array_equal(mc[k], ref[k]), k


@pytest.mark.parametrize("iceflag", [0, 1, 2, 3])
def test_lw_mcica_physics_binary_covers(orc, iceflag):
    """cldprmc's per-g-point parameterisations on binary sub-columns equal
    cldprop's per band when the column keeps 16 cloud bands (liquid, liqflag 1,
    in every cloudy layer), bit for bit, gray ice (iceflag 0) included."""
    atm = A.small_atmosphere(16, 40, seed=43)
    rng = np.random.default_rng(44)
    cl = _clouds(atm, rng, binary=True)
    cl["cliqwp"] = np.where(cl["cldfr"] > 0, rng.uniform(1.0, 40.0, cl["cldfr"].shape), 0.0)
    cl["cicewp"] = np.where((cl["cldfr"] > 0) & (atm.play < 700), rng.uniform(0.5, 30.0, cl["cldfr"].shape), 0.0)
    rei, rel = rng.uniform(20.0, 120.0, cl["cldfr"].shape), rng.uniform(4.0, 40.0, cl["cldfr"].shape)
    sub = orc.mcica_subcol("lw", atm, dict(cl, taucld=np.zeros_like(cl["taucld"])), icld=1, irng=1)
    mc = orc.rrtmg_lw_mcica(atm, sub, inflag=2, iceflag=iceflag, liqflag=1, reice=rei, reliq=rel)
    ref = orc.rrtmg_lw(atm, icld=1, cloud=dict(cldfr=cl["cldfr"], cicewp=cl["cicewp"], cliqwp=cl["cliqwp"],
                                               reice=rei, reliq=rel, inflag=2, iceflag=iceflag, liqflag=1))
    for k in ref:
        assert np.array_equal(mc[k], ref[k]), k


def test_lw_mcica_partial_covers(orc):
    """Twelve adjacent layers at cover 0.5 with opaque cloud: random overlap
    leaves almost no g-point clear (0.5^12), so its fluxes are the overcast
    column's; maximum and maximum/random overlap make one block, clear in
    half the g-points, so their OLR is the mean of clear sky and overcast
    (within the scatter of 140 draws)."""
    atm = A.small_atmosphere(64, 40, seed=45)
    L, n = atm.nlay, atm.ncol
    cf = np.zeros((L, n))
    cf[8:20] = 0.5
    cl = dict(cldfr=cf, cicewp=cf * 0, cliqwp=cf * 0, taucld=np.full((L, n, 16), 5.0))
    clear = orc.rrtmg_lw(atm)["uflx"][-1]
    over = orc.rrtmg_lw(atm, cloud=dict(cldfr=np.where(cf > 0, 1.0, 0.0), taucld=cl["taucld"]), icld=1)["uflx"][-1]
    olr = {icld: orc.rrtmg_lw_mcica(atm, orc.mcica_subcol("lw", atm, cl, icld=icld, irng=1))["uflx"][-1]
           for icld in (1, 2, 3)}
    assert np.abs(olr[1] - over).max() < 0.5
    for icld in (2, 3):
        assert np.all(olr[icld] > over + 10.0) and np.all(olr[icld] < clear - 10.0)
        assert abs((olr[icld] - 0.5 * (clear + over)).mean()) < 5.0
    with pytest.raises(orc.CloudRangeError):
        s = orc.mcica_subcol("lw", atm, dict(cl, cicewp=cf * 3.0), icld=1, irng=1)
        orc.rrtmg_lw_mcica(atm, s, inflag=1)


def _sw_clouds(atm, rng, binary=True):
    L, n = atm.nlay, atm.ncol
    cf = (rng.uniform(size=(L, n)) < 0.3) * 1.0
    if not binary:
        cf = cf * rng.uniform(0.1, 1.0, (L, n))
    cf = np.where(atm.play > 150.0, cf, 0.0)
    return dict(cldfr=cf, cicewp=cf * 0.0, cliqwp=cf * 0.0, taucld=rng.uniform(0.5, 20.0, (L, n, 14)),
                ssacld=rng.uniform(0.9, 0.999999, (L, n, 14)), asmcld=rng.uniform(0.7, 0.9, (L, n, 14)),
                fsfcld=rng.uniform(0.5, 0.8, (L, n, 14)))


def _sunlit_and_dark(atm, mc, ref):
    """McICA computes dark columns too (cos(zenith) clamped to 1e-10): their
    fluxes are of order 1e-7 W/m2 where the non-McICA driver writes zeros."""
    lit = atm.coszen >= 1e-10
    for k in ref:
        assert np.array_equal(mc[k][:, lit], ref[k][:, lit]), k
        assert np.all(np.abs(mc[k][:, ~lit]) < 1e-5) and np.all(ref[k][:, ~lit] == 0.0), k


@pytest.mark.parametrize("iaer", [0, 10])
def test_sw_mcica_binary_covers_equal_overcast_layers(orc, iaer):
    """spcvmc on binary sub-columns is spcvrt on clear / overcast layers, bit
    for bit in the sunlit columns, without and with aerosols (iaer = 10):
    cldprmc_sw delta-scales each g-point's copy of its band's optics as
    cldprop_sw scales the band's."""
    atm = A.small_atmosphere(24, 40, seed=51)
    atm.coszen[3] = 0.0
    rng = np.random.default_rng(52)
    cl = _sw_clouds(atm, rng)
    L, n = atm.nlay, atm.ncol
    prof = (atm.play / atm.play[0]) ** 3.75
    aer = {} if iaer == 0 else dict(tauaer=rng.uniform(0.0, 0.05, (14, L, n)) * prof,
                                    ssaaer=rng.uniform(0.8, 1.0, (14, L, n)),
                                    asmaer=rng.uniform(0.5, 0.8, (14, L, n)))
    sub = orc.mcica_subcol("sw", atm, cl, icld=2, irng=0)
    mc = orc.rrtmg_sw_mcica(atm, sub, iaer=iaer, **aer)
    ref = orc.rrtmg_sw(atm, iaer=iaer, cloud=cl, **aer)
    if iaer:
        assert np.abs(mc["swuflxc"] - orc.rrtmg_sw(atm, cloud=cl)["swuflxc"]).max() > 0.1
    _sunlit_and_dark(atm, mc, ref)


@pytest.mark.parametrize("iceflag", [1, 2, 3])
def test_sw_mcica_physics_binary_covers(orc, iceflag):
    """cldprmc_sw's parameterisations, one g-point on its band, equal
    cldprop_sw's on all 14 bands for binary sub-columns, bit for bit."""
    atm = A.small_atmosphere(16, 40, seed=53)
    rng = np.random.default_rng(54)
    cl = _sw_clouds(atm, rng)
    cf = cl["cldfr"]
    cl["cliqwp"] = np.where(cf > 0, rng.uniform(1.0, 40.0, cf.shape), 0.0)
    cl["cicewp"] = np.where((cf > 0) & (atm.play < 700), rng.uniform(0.5, 30.0, cf.shape), 0.0)
    rei, rel = rng.uniform(20.0, 120.0, cf.shape), rng.uniform(4.0, 40.0, cf.shape)
    sub = orc.mcica_subcol("sw", atm, cl, icld=1, irng=1)
    mc = orc.rrtmg_sw_mcica(atm, sub, inflag=2, iceflag=iceflag, liqflag=1, reice=rei, reliq=rel)
    ref = orc.rrtmg_sw(atm, cloud=dict(cldfr=cf, cicewp=cl["cicewp"], cliqwp=cl["cliqwp"], reice=rei, reliq=rel,
                                       inflag=2, iceflag=iceflag, liqflag=1))
    _sunlit_and_dark(atm, mc, ref)


def test_sw_mcica_partial_covers(orc):
    """Twelve adjacent layers at cover 0.5: maximum and maximum/random
    overlap make one block, clear in half the g-points, so the upward flux at
    the top lies halfway between clear sky and overcast (within the scatter of
    112 draws); random overlap leaves about six of the twelve layers cloudy in
    every g-point, which reflects most but not all of what the overcast
    column does; inflag = 1 stops, as cldprmc_sw does."""
    atm = A.small_atmosphere(64, 40, seed=55)
    L, n = atm.nlay, atm.ncol
    cf = np.zeros((L, n))
    cf[8:20] = 0.5
    cl = dict(cldfr=cf, cicewp=cf * 0, cliqwp=cf * 0, taucld=np.full((L, n, 14), 5.0),
              ssacld=np.full((L, n, 14), 0.999), asmcld=np.full((L, n, 14), 0.85),
              fsfcld=np.full((L, n, 14), 0.7225))
    lit = atm.coszen >= 1e-10
    clear = orc.rrtmg_sw(atm)["swuflx"][-1]
    over = orc.rrtmg_sw(atm, cloud=dict(cl, cldfr=np.where(cf > 0, 1.0, 0.0)))["swuflx"][-1]
    up = {icld: orc.rrtmg_sw_mcica(atm, orc.mcica_subcol("sw", atm, cl, icld=icld, irng=1))["swuflx"][-1]
          for icld in (1, 2, 3)}
    span = (over - clear)[lit]
    assert span.min() > 20.0
    frac = (up[1] - clear)[lit] / span
    assert np.all(frac > 0.8) and np.all(frac < 1.0)
    for icld in (2, 3):
        frac = (up[icld] - clear)[lit] / span
        assert np.all(frac > 0.15) and np.all(frac < 0.85)
        assert abs(frac.mean() - 0.5) < 0.08
    with pytest.raises(orc.CloudRangeError):
        s = orc.mcica_subcol("sw", atm, dict(cl, cicewp=cf * 3.0), icld=1, irng=1)
        orc.rrtmg_sw_mcica(atm, s, inflag=1)


def _kiss_masks_numpy(play, cldfr, nsub, icld, permuteseed):
    """A second restatement of generate_stochastic_clouds with kissvec
    (mcica_subcol_gen_lw.f90), vectorised over the columns in numpy uint32
    arithmetic: the masks (nlay, ncol, nsub)."""
    L, n = cldfr.shape
    p = play[:4] * 1.0e2
    s = np.trunc((p - np.trunc(p)) * 1.0e9).astype(np.int64).astype(np.uint32)
    st = [s[0].copy(), s[1].copy(), s[2].copy(), s[3].copy()]
    u = np.uint32

    def m(k, sh):
        return k ^ ((k << u(sh)) if sh > 0 else (k >> u(-sh)))

    def draw():
        with np.errstate(over="ignore"):
            st[0] = u(69069) * st[0] + u(1327217885)
            st[1] = m(m(m(st[1], 13), -17), 5)
            st[2] = u(18000) * (st[2] & u(65535)) + (st[2] >> u(16))
            st[3] = u(30903) * (st[3] & u(65535)) + (st[3] >> u(16))
            k = (st[0] + st[1] + (st[2] << u(16)) + st[3]).view(np.int32)
        return k.astype(np.float64) * 2.328306e-10 + 0.5

    for _ in range(permuteseed):
        draw()
    cdf = np.zeros((nsub, n, L))
    for g in range(nsub):
        if icld == 3:
            cdf[g] = draw()[:, None]
        else:
            for lay in range(L):
                cdf[g, :, lay] = draw()
    return _masks(cdf, cldfr, icld)


def _mt_masks_numpy(cldfr, nsub, icld, permuteseed):
    """The same with the Mersenne Twister (numpy's MT19937 under the scalar
    seeding), drawn sub-column by sub-column, column by column, layer by
    layer (one draw per column and sub-column under maximum overlap)."""
    L, n = cldfr.shape
    bg = np.random.MT19937()
    bg._legacy_seeding(permuteseed)
    per = 1 if icld == 3 else L
    r = bg.random_raw(nsub * n * per).astype(np.float64) / 4294967295.0
    cdf = np.broadcast_to(r.reshape(nsub, n, per), (nsub, n, L)).copy()
    return _masks(cdf, cldfr, icld)


def _masks(cdf, cldfr, icld):
    L = cldfr.shape[0]
    cf = np.where(cldfr < 1e-20, 0.0, cldfr)
    if icld == 2:
        for lay in range(1, L):
            keep = cdf[:, :, lay - 1] > 1.0 - cf[lay - 1]
            cdf[:, :, lay] = np.where(keep, cdf[:, :, lay - 1], cdf[:, :, lay] * (1.0 - cf[lay - 1]))
    return (cdf >= 1.0 - cf.T[None]).transpose(2, 1, 0).astype(np.float64)


@pytest.mark.parametrize("icld", [1, 2, 3])
def test_masks_match_numpy_restatement(orc, icld):
    """Both generators' masks, LW (140) and SW (112) sub-columns, equal a
    numpy restatement of the generator bit for bit."""
    atm = A.small_atmosphere(48, 40, seed=57)
    rng = np.random.default_rng(58)
    # kissvec seeds each column from its pressures: give every column its own
    atm.play = atm.play + rng.uniform(0.0, 1e-3, atm.play.shape)
    cl = _clouds(atm, rng)
    for side, nsub in (("lw", 140), ("sw", 112)):
        c = cl if side == "lw" else dict(cl, taucld=np.ones((atm.nlay, atm.ncol, 14)),
                                         ssacld=np.ones((atm.nlay, atm.ncol, 14)),
                                         asmcld=np.zeros((atm.nlay, atm.ncol, 14)),
                                         fsfcld=np.zeros((atm.nlay, atm.ncol, 14)))
        for irng, want in ((0, _kiss_masks_numpy(atm.play, cl["cldfr"], nsub, icld, 3)),
                           (1, _mt_masks_numpy(cl["cldfr"], nsub, icld, 3))):
            assert 0.02 < want.mean() < 0.98
            s = orc.mcica_subcol(side, atm, c, icld=icld, irng=irng, permuteseed=3)
            assert np.array_equal(s["cldfr"], want), (side, irng)


@pytest.mark.parametrize("irng", [0, 1])
@pytest.mark.parametrize("icld", [1, 2])
def test_lw_mcica_mean_is_the_deterministic_overlap(orc, icld, irng):
    """McICA samples the overlap that rtrn (random) and rtrnmr
    (maximum/random) treat exactly, layer by layer: over 512 copies of a
    column with three partly cloudy decks (covers 0.6, 0.3, 0.4), each
    drawing its own sub-columns, the mean fluxes at every level and the mean
    heating of every layer equal the deterministic ones within 4.5 standard
    errors of the mean."""
    n = 512
    atm = A.small_atmosphere(1, 40, seed=61).subset(np.zeros(n, dtype=np.int64))
    rng = np.random.default_rng(62)
    atm.play = atm.play + rng.uniform(0.0, 1e-3, atm.play.shape)   # kissvec: a seed per column
    L = atm.nlay
    cf = np.zeros((L, n))
    cf[5:9], cf[9:11], cf[20:24] = 0.6, 0.3, 0.4
    tau = np.broadcast_to(rng.uniform(0.3, 3.0, (L, 1, 16)), (L, n, 16)).copy()
    ref = orc.rrtmg_lw(atm, cloud=dict(cldfr=cf, taucld=tau), icld=icld)
    sub = orc.mcica_subcol("lw", atm, dict(cldfr=cf, cicewp=cf * 0, cliqwp=cf * 0, taucld=tau), icld=icld,
                           irng=irng)
    mc = orc.rrtmg_lw_mcica(atm, sub)
    for k in ("uflx", "dflx", "hr"):
        d = mc[k] - ref[k]
        se = d.std(axis=1) / np.sqrt(n)
        noisy = se > 1e-9
        assert np.all(np.abs(d.mean(axis=1)[noisy]) < 4.5 * se[noisy]), k
        assert np.all(np.abs(d.mean(axis=1)[~noisy]) < 1e-9), k


def _numpy_mt_after(seed, jump, n):
    bg = np.random.MT19937()
    bg._legacy_seeding(seed)
    left = jump
    while left:
        c = min(left, 1 << 23)
        bg.random_raw(c)
        left -= c
    return bg.random_raw(n).astype(np.uint32)


@pytest.mark.parametrize("jump", [0, 1, 623, 624, 625, 100003, 140 * 8192 * 40])
def test_mersenne_twister_jump_ahead(orc, jump):
    """The F2-linear jump-ahead that lets each McICA sub-column start its
    draws at its own offset of the one Mersenne Twister stream (sub-column g
    of a T42 x 40 call starts g x 8192 x 40 words in): Berlekamp-Massey finds
    the degree-19937 characteristic polynomial, and the draws after a jump
    equal the serial stream's (numpy's MT19937 drawn through the skipped
    words)."""
    got, deg = orc.mt_jump_ints(7, jump, 64)
    assert deg == 19937
    assert np.array_equal(got, _numpy_mt_after(7, jump, 64))


def test_mersenne_twister_subcolumn_starts(orc):
    """The 140 sub-column start states of a McICA call (1000 columns x 40
    layers: 40000 words apart), reached by one jump polynomial applied in a
    chain, give the serial stream's words at every start."""
    stride, nsub, n = 1000 * 40, 140, 48
    got = orc.mt_subcol_starts(3, stride, nsub, n)
    bg = np.random.MT19937()
    bg._legacy_seeding(3)
    serial = bg.random_raw(stride * nsub).astype(np.uint32).reshape(nsub, stride)
    assert np.array_equal(got, serial[:, :n])


def test_mcica_results_do_not_depend_on_threads(orc):
    """The McICA paths keep their per-g-point cloud state in each thread's own
    column: one thread and four give the same fluxes bit for bit."""
    atm = A.small_atmosphere(40, 40, seed=63)
    rng = np.random.default_rng(64)
    lw_cl = _clouds(atm, rng)
    sw_cl = _sw_clouds(atm, rng, binary=False)
    lw_sub = orc.mcica_subcol("lw", atm, lw_cl, icld=2, irng=1)
    sw_sub = orc.mcica_subcol("sw", atm, sw_cl, icld=2, irng=1)
    for f, sub in ((orc.rrtmg_lw_mcica, lw_sub), (orc.rrtmg_sw_mcica, sw_sub)):
        one, four = f(atm, sub, nthreads=1), f(atm, sub, nthreads=4)
        for k in one:
            assert np.array_equal(one[k], four[k]), k


@pytest.mark.parametrize("icld", [1, 2, 3])
def test_mt_masks_from_jumped_subcolumn_streams(orc, icld):
    """The device plan for the Mersenne Twister path, emulated: each
    sub-column draws its block from its own start, stride ncol x nlay words
    apart (ncol under maximum overlap), the starts reached by jump-ahead; the
    masks equal the serial generator's bit for bit."""
    atm = A.small_atmosphere(16, 40, seed=65)
    cl = _clouds(atm, np.random.default_rng(66))
    L, n, nsub = atm.nlay, atm.ncol, 140
    per = 1 if icld == 3 else L
    blocks = orc.mt_subcol_starts(5, n * per, nsub, n * per)
    cdf = np.broadcast_to((blocks.astype(np.float64) / 4294967295.0).reshape(nsub, n, per), (nsub, n, L)).copy()
    want = orc.mcica_subcol("lw", atm, cl, icld=icld, irng=1, permuteseed=5)["cldfr"]
    got = _masks(cdf, cl["cldfr"], icld)
    assert 0.02 < got.mean() < 0.98
    assert np.array_equal(got, want)


@pytest.mark.parametrize("iceflag", [2, 3])
def test_lw_mcica_gray_liquid_binary_covers(orc, iceflag):
    """Gray liquid (liqflag 0) with a 16-band ice scheme in every cloudy
    layer: cldprmc equals cldprop bit for bit.  (Where the two routines of the
    reference differ: cldprop / rtrn scale each of the column's ncbands cloud
    bands by secdiff of that cloud band's index, so with 1 or 5 cloud bands --
    gray ice, iceflag 1 -- bands share a diffusivity where cldprmc / rtrnmc
    take secdiff(ngb(g)); and cldprop's count of cloud bands runs across the
    layers, so a layer filled while it was 1 keeps its depth in band 1 only.)"""
    atm = A.small_atmosphere(16, 40, seed=43)
    rng = np.random.default_rng(44)
    cl = _clouds(atm, rng, binary=True)
    cf = cl["cldfr"]
    cl["cliqwp"] = np.where(cf > 0, rng.uniform(1.0, 40.0, cf.shape), 0.0)
    cl["cicewp"] = np.where(cf > 0, rng.uniform(0.5, 30.0, cf.shape), 0.0)
    rei, rel = rng.uniform(20.0, 120.0, cf.shape), rng.uniform(4.0, 40.0, cf.shape)
    sub = orc.mcica_subcol("lw", atm, dict(cl, taucld=np.zeros_like(cl["taucld"])), icld=1, irng=1)
    mc = orc.rrtmg_lw_mcica(atm, sub, inflag=2, iceflag=iceflag, liqflag=0, reice=rei, reliq=rel)
    ref = orc.rrtmg_lw(atm, icld=1, cloud=dict(cldfr=cf, cicewp=cl["cicewp"], cliqwp=cl["cliqwp"], reice=rei,
                                               reliq=rel, inflag=2, iceflag=iceflag, liqflag=0))
    for k in ref:
        assert np.array_equal(mc[k], ref[k]), k
