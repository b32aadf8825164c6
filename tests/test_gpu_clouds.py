"""Clouds on the GPU against the oracle's restatement of the reference: LW
with cloud optical depths given (inflglw = 0, rrtmg_lw_cldprop.f90:155-174),
icld = 1 (random overlap, rrtmg_lw_rtrn.f90) and icld = 2 / 3
(maximum/random overlap, rrtmg_lw_rtrnmr.f90); SW icld = 1 (cloud
optics given, inflgsw = 0, clear or overcast layers;
rrtmg_sw_cldprop.f90:120-156, rrtmg_sw_spcvrt.f90's clear and total passes).

Tolerances: the FP64 path as every FP64 parity test (fluxes 1e-10 relative,
heating 1e-8 K/day + 1e-9 relative), total and clear-sky outputs and the
surface-temperature derivatives; the split path within the split bars
(tests/split_bars.py: 0.1 W/m2 at every level, 0.05 K/day heating, its
net-flux-divergence form in layers thinner than 0.01 hPa).
"""
import numpy as np
import pytest

import split_bars as SB
from conftest import rel_err
from mima_gb300 import atmosphere as A
from mima_gb300 import rrtmg as R
from test_gpu_parity import check_lw, check_sw, hr_ok
from test_oracle import sw_cloud_fields

pytestmark = pytest.mark.gpu


def cloud_fields(atm, rng):
    """Seeded clouds below 100 hPa: about 40 % of the layers cloudy with a
    cover up to 1, 5 % overcast, per-band optical depths up to 75 (a layer's
    spectral shape times a heavy-tailed layer depth); among them layers whose
    cover is below rtrn's 1e-6 (clear for the solver) and layers with cover but
    no optical depth or water path (cldprop keeps no depth)."""
    L, n = atm.nlay, atm.ncol
    cf = rng.uniform(0.0, 1.0, (L, n)) * (rng.uniform(size=(L, n)) < 0.4)
    cf[rng.uniform(size=(L, n)) < 0.05] = 1.0
    cf[rng.uniform(size=(L, n)) < 0.02] = 5e-7
    cf = np.where(atm.play > 100.0, cf, 0.0)
    tau = (rng.uniform(0.0, 1.0, (L, n, 1)) ** 3 * 50.0) * rng.uniform(0.5, 1.5, (L, n, 16))
    tau[rng.uniform(size=(L, n)) < 0.03] = 0.0
    return dict(cldfr=cf, taucld=tau)


def _case(nlay, seed, n=384):
    rng = np.random.default_rng(seed)
    atm = A.small_atmosphere(n, nlay, seed=seed, ts_sigma=5.0, rh_random=True)
    atm.emis = rng.uniform(0.8, 1.0, size=(16, n))
    return atm, cloud_fields(atm, rng)


def _check_clear_outputs(out, ref, idrv):
    for k in ("uflxc", "dflxc"):
        assert rel_err(out[k], ref[k], 1e-3) < 1e-10, k
    assert hr_ok(out["hrc"], ref["hrc"]), "hrc"
    if idrv == 1:
        assert rel_err(out["duflxc_dt"], ref["duflxc_dt"], 1e-6) < 1e-10


@pytest.mark.parametrize("nlay", [40, 60])
@pytest.mark.parametrize("mode", ["table", "analytic"])
@pytest.mark.parametrize("idrv", [0, 1])
@pytest.mark.parametrize("icld", [1, 2])
def test_lw_clouds_fp64_matches_oracle(gpu, orc, nlay, mode, idrv, icld):
    atm, cl = _case(nlay, 900 + nlay + idrv + 10 * icld)
    orc.set_table_mode(mode == "table")
    try:
        ref = orc.rrtmg_lw(atm, idrv=idrv, cloud=cl, icld=icld)
    finally:
        orc.set_table_mode(True)
    gpu.set_precision("fp64")
    gpu.set_transcendentals(mode)
    try:
        out = gpu.lw(atm, idrv=idrv, cloud=cl, icld=icld)
    finally:
        gpu.set_transcendentals("table")
    check_lw(out, ref, idrv=idrv)
    _check_clear_outputs(out, ref, idrv)
    # the clouds matter: OLR and the surface downward flux move
    clear = orc.rrtmg_lw(atm)
    assert np.abs(ref["uflx"][-1] - clear["uflx"][-1]).max() > 10.0


@pytest.mark.parametrize("nlay", [40, 60])
@pytest.mark.parametrize("icld", [1, 2])
def test_lw_clouds_split_within_bars(gpu, orc, nlay, icld):
    atm, cl = _case(nlay, 950 + nlay + 10 * icld, n=768)
    ref = orc.rrtmg_lw(atm, idrv=1, cloud=cl, icld=icld)
    gpu.set_precision("split")
    try:
        out = gpu.lw(atm, idrv=1, cloud=cl, icld=icld)
    finally:
        gpu.set_precision("fp64")
    bar = SB.hr_bar(atm)
    for k in ("uflx", "dflx", "uflxc", "dflxc"):
        assert np.abs(out[k] - ref[k]).max() <= SB.FLUX_BAR, (k, np.abs(out[k] - ref[k]).max())
    for k in ("hr", "hrc"):
        assert np.all(np.abs(out[k] - ref[k]) <= bar), (k, np.abs(out[k] - ref[k]).max())
    assert np.abs(out["duflx_dt"] - ref["duflx_dt"]).max() <= 1e-3


@pytest.mark.parametrize("icld", [1, 2])
def test_lw_clouds_without_clouds_equal_clear_sky(gpu, icld):
    """Clouds with no cloud (cover 0, or below the solvers' 1e-6) take the clear
    branch everywhere: the FP64 results are the clear-sky call's bit for bit,
    the split ones within FP32 rounding."""
    atm = A.small_atmosphere(200, 40, seed=17)
    L, n = atm.nlay, atm.ncol
    cl = dict(cldfr=np.full((L, n), 5e-7), taucld=np.full((L, n, 16), 3.0))
    for prec in ("fp64", "split"):
        gpu.set_precision(prec)
        try:
            a, b = gpu.lw(atm, idrv=1), gpu.lw(atm, idrv=1, cloud=cl, icld=icld)
        finally:
            gpu.set_precision("fp64")
        for k in a:
            if k == "status":
                continue
            if prec == "fp64":
                assert np.array_equal(a[k], b[k]), k
            else:
                assert np.abs(a[k] - b[k]).max() <= 1e-3, k


def test_lw_maximum_random_overlap_icld_3_is_icld_2(gpu):
    """The non-McICA driver sends icld = 2 and 3 to the same solver."""
    atm, cl = _case(40, 41, n=256)
    for prec in ("fp64", "split"):
        gpu.set_precision(prec)
        try:
            a, b = gpu.lw(atm, idrv=1, cloud=cl, icld=2), gpu.lw(atm, idrv=1, cloud=cl, icld=3)
        finally:
            gpu.set_precision("fp64")
        for k in a:
            assert np.array_equal(a[k], b[k]), (prec, k)


@pytest.mark.parametrize("icld", [1, 2])
def test_lw_clouds_host_entry_matches_device_entry(gpu, icld):
    """rrtmg_lw_c (page-locked arrays, 40000 columns: two column chunks on two
    streams, taucld copied 16 values per column) against rrtmg_lw_dev on the
    same arrays, bit for bit."""
    torch = pytest.importorskip("torch")
    atm, cl = _case(40, 77 + icld, n=40000)
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
    L, n = atm.nlay, atm.ncol
    outs = {k: pin(np.zeros((L + 1 if k not in ("hr", "hrc") else L, n))) for k in
            ("uflx", "dflx", "hr", "uflxc", "dflxc", "hrc", "duflx_dt", "duflxc_dt")}
    gpu.set_precision("split")
    try:
        host = gpu.rrtmg_lw(n, L, icld, 1, *[pin(a) for a in (atm.play, atm.plev, atm.tlay, atm.tlev, atm.tsfc, atm.h2o,
                                                            atm.o3, atm.co2, atm.ch4, atm.n2o, atm.o2, atm.cfc11,
                                                            atm.cfc12, atm.cfc22, atm.ccl4, atm.emis)],
                            out=outs, cldfr=pin(cl["cldfr"]), taucld=pin(cl["taucld"]))
        d = R.atm_device_inputs(atm)
        d["cldfr"] = torch.from_numpy(cl["cldfr"]).cuda()
        d["taucld"] = torch.from_numpy(np.ascontiguousarray(cl["taucld"])).cuda()
        o, _ = R.device_outputs(n, L, idrv=1)
        s = torch.cuda.Stream()
        with torch.cuda.stream(s):
            gpu.rrtmg_lw_dev(s.cuda_stream, n, L, icld, 1, d, o)
        s.synchronize()
    finally:
        gpu.set_precision("fp64")
    for k in o:
        assert np.array_equal(o[k].cpu().numpy(), host[k]), k


def test_lw_cloud_options_not_computed_are_refused(gpu):
    atm, cl = _case(40, 5, n=16)
    args = (atm.ncol, atm.nlay)
    base = (atm.play, atm.plev, atm.tlay, atm.tlev, atm.tsfc, atm.h2o, atm.o3, atm.co2)
    o = gpu.rrtmg_lw(*args, 4, 0, *base, check=False, cldfr=cl["cldfr"], taucld=cl["taucld"])
    assert o["status"] == R.RRTMG_ERR_UNSUPPORTED  # icld outside 0..3
    o = gpu.rrtmg_lw(*args, 1, 0, *base, check=False, inflglw=3, cldfr=cl["cldfr"], taucld=cl["taucld"])
    assert o["status"] == R.RRTMG_ERR_UNSUPPORTED  # cldprop has no inflag = 3
    o = gpu.rrtmg_lw(*args, 1, 0, *base, check=False, inflglw=2, cldfr=cl["cldfr"], taucld=cl["taucld"])
    assert o["status"] == R.RRTMG_ERR_ARG  # cloud physics without water paths and sizes
    o = gpu.rrtmg_lw(*args, 1, 0, *base, check=False, cldfr=cl["cldfr"])
    assert o["status"] == R.RRTMG_ERR_ARG  # no cloud optical depths
    assert gpu.lw(atm, cloud=cl)["status"] == R.RRTMG_OK


# ---------------------------------------------------------------------------
# SW clouds
# ---------------------------------------------------------------------------
def _sw_case(nlay, seed, n=384, night=0.15):
    rng = np.random.default_rng(seed)
    atm = A.small_atmosphere(n, nlay, seed=seed, ts_sigma=5.0, rh_random=True)
    atm.coszen = np.where(rng.uniform(size=n) < night, 0.0, rng.uniform(0.02, 1.0, n))
    return atm, sw_cloud_fields(atm, rng)


@pytest.mark.parametrize("nlay", [40, 60])
@pytest.mark.parametrize("mode", ["table", "analytic"])
def test_sw_clouds_fp64_matches_oracle(gpu, orc, nlay, mode):
    atm, cl = _sw_case(nlay, 700 + nlay)
    orc.set_table_mode(mode == "table")
    try:
        ref = orc.rrtmg_sw(atm, cloud=cl)
        clear = orc.rrtmg_sw(atm)
    finally:
        orc.set_table_mode(True)
    gpu.set_precision("fp64")
    gpu.set_transcendentals(mode)
    try:
        out = gpu.sw(atm, cloud=cl)
    finally:
        gpu.set_transcendentals("table")
    check_sw(out, ref)
    # the clouds matter, and the clear-sky outputs are the clear-sky call's
    assert np.abs(ref["swuflx"][-1] - clear["swuflx"][-1]).max() > 50.0
    for k in ("swuflxc", "swdflxc"):
        assert rel_err(out[k], clear[k[:-1]], 1e-3) < 1e-10, k


def test_sw_clouds_with_aerosols_fp64(gpu, orc):
    """Clouds and aerosols (iaer = 10) together: the clear pass carries the
    aerosols, the total pass both."""
    atm, cl = _sw_case(40, 31)
    rng = np.random.default_rng(32)
    L, n = atm.nlay, atm.ncol
    prof = (atm.play / atm.play[0]) ** 3.75
    aer = dict(tauaer=rng.uniform(0.0, 0.05, (14, L, n)) * prof, ssaaer=rng.uniform(0.8, 1.0, (14, L, n)),
               asmaer=rng.uniform(0.5, 0.8, (14, L, n)))
    ref = orc.rrtmg_sw(atm, iaer=10, cloud=cl, **aer)
    gpu.set_precision("fp64")
    check_sw(gpu.sw(atm, iaer=10, cloud=cl, **aer), ref)


@pytest.mark.parametrize("nlay", [40, 60])
def test_sw_clouds_split_within_bars(gpu, orc, nlay):
    """The split path with clouds within the split bars, a column that misses
    them justified by the backward-error criterion (gas amounts or cloud
    optical depths within FP32 rounding reproduce it)."""
    atm, cl = _sw_case(nlay, 750 + nlay, n=768)
    ref = orc.rrtmg_sw(atm, cloud=cl)
    gpu.set_precision("split")
    try:
        out = gpu.sw(atm, cloud=cl)
    finally:
        gpu.set_precision("fp64")
    SB.check_sw(orc, atm, out, ref, cloud=cl)


def test_sw_clouds_analytic_split_strict(gpu, orc):
    """Analytic exponentials: no table steps, so no backward-error allowance."""
    atm, cl = _sw_case(40, 811, n=512)
    orc.set_table_mode(False)
    try:
        ref = orc.rrtmg_sw(atm, cloud=cl)
    finally:
        orc.set_table_mode(True)
    gpu.set_precision("split")
    gpu.set_transcendentals("analytic")
    try:
        out = gpu.sw(atm, cloud=cl)
    finally:
        gpu.set_transcendentals("table")
        gpu.set_precision("fp64")
    bar = SB.hr_bar(atm)
    for k in ("swuflx", "swdflx", "swuflxc", "swdflxc"):
        assert np.abs(out[k] - ref[k]).max() <= SB.FLUX_BAR, (k, np.abs(out[k] - ref[k]).max())
    for k in ("swhr", "swhrc"):
        assert np.all(np.abs(out[k] - ref[k]) <= bar), (k, np.abs(out[k] - ref[k]).max())


def test_sw_clouds_without_clouds_equal_clear_sky(gpu):
    """icld = 1 with cover 0 everywhere: the total pass combines nothing; the
    FP64 results are the clear-sky call's bit for bit, the split ones within
    FP32 rounding."""
    atm = A.small_atmosphere(200, 40, seed=18)
    L, n = atm.nlay, atm.ncol
    z = np.zeros((L, n, 14))
    cl = dict(cldfr=np.zeros((L, n)), taucld=z + 3.0, ssacld=z + 0.9, asmcld=z + 0.8, fsfcld=z + 0.64)
    for prec in ("fp64", "split"):
        gpu.set_precision(prec)
        try:
            a, b = gpu.sw(atm), gpu.sw(atm, cloud=cl)
        finally:
            gpu.set_precision("fp64")
        for k in a:
            if k == "status":
                continue
            if prec == "fp64":
                assert np.array_equal(a[k], b[k]), k
            else:
                assert np.abs(a[k] - b[k]).max() <= 1e-3, k


def test_sw_partial_cloud_is_refused(gpu, orc):
    """A partly cloudy sunlit layer: the reference stops, the library reports
    invalid input (RRTMG_ERR_INPUT) and the handle stays usable; partly cloudy
    layers of unlit columns are not looked at (the reference skips them)."""
    atm, cl = _sw_case(40, 5, n=64, night=0.3)
    lit = np.asarray(atm.coszen) >= 1e-10
    bad = dict(cl)
    bad["cldfr"] = cl["cldfr"].copy()
    bad["cldfr"][20, np.flatnonzero(lit)[3]] = 0.5
    for prec in ("fp64", "split"):
        gpu.set_precision(prec)
        try:
            assert gpu.sw(atm, cloud=bad, check=False)["status"] == R.RRTMG_ERR_INPUT
            out = gpu.sw(atm, cloud=cl)
        finally:
            gpu.set_precision("fp64")
        assert out["status"] == R.RRTMG_OK
    check_sw(gpu.sw(atm, cloud=cl), orc.rrtmg_sw(atm, cloud=cl))


def test_sw_clouds_host_entry_matches_device_entry(gpu):
    """rrtmg_sw_c (page-locked arrays, 40000 columns: two column chunks on two
    streams, the 14-band cloud optics copied 14 values per column) against
    rrtmg_sw_dev on the same arrays, bit for bit."""
    torch = pytest.importorskip("torch")
    atm, cl = _sw_case(40, 78, n=40000)
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
    L, n = atm.nlay, atm.ncol
    outs = {k: pin(np.zeros((L + 1 if k not in ("swhr", "swhrc") else L, n))) for k in
            ("swuflx", "swdflx", "swhr", "swuflxc", "swdflxc", "swhrc")}
    gpu.set_precision("split")
    try:
        host = gpu.rrtmg_sw(n, L, 1, 0, *[pin(a) for a in (atm.play, atm.plev, atm.tlay, atm.tlev, atm.tsfc,
                                                            atm.h2o, atm.o3, atm.co2, atm.ch4, atm.n2o, atm.o2,
                                                            atm.asdir, atm.asdif, atm.aldir, atm.aldif,
                                                            atm.coszen)],
                            atm.adjes, atm.dyofyr, atm.scon, out=outs, **{k: pin(v) for k, v in cl.items()})
        d = R.atm_device_inputs(atm)
        dc = {k: torch.from_numpy(np.ascontiguousarray(v)).cuda() for k, v in cl.items()}
        o = {k: torch.zeros(v.shape, dtype=torch.float64, device="cuda") for k, v in outs.items()}
        s = torch.cuda.Stream()
        with torch.cuda.stream(s):
            gpu.rrtmg_sw_dev(s.cuda_stream, n, L, 1, 0, d, o, atm.adjes, atm.dyofyr, atm.scon, cloud=dc)
        s.synchronize()
    finally:
        gpu.set_precision("fp64")
    for k in o:
        assert np.array_equal(o[k].cpu().numpy(), host[k]), k


def test_sw_cloud_options_not_computed_are_refused(gpu):
    atm, cl = _sw_case(40, 6, n=16)
    base = (atm.play, atm.plev, atm.tlay, atm.tlev, atm.tsfc, atm.h2o, atm.o3, atm.co2, atm.ch4, atm.n2o,
            atm.o2, atm.asdir, atm.asdif, atm.aldir, atm.aldif, atm.coszen, atm.adjes, atm.dyofyr, atm.scon)
    args = (atm.ncol, atm.nlay)
    o = gpu.rrtmg_sw(*args, 1, 0, *base, check=False, inflgsw=1, **cl)
    assert o["status"] == R.RRTMG_ERR_UNSUPPORTED  # cldprop_sw has no inflag = 1 branch
    o = gpu.rrtmg_sw(*args, 1, 0, *base, check=False, inflgsw=2, **cl)
    assert o["status"] == R.RRTMG_ERR_UNSUPPORTED  # cloud physics with iceflgsw = 0
    o = gpu.rrtmg_sw(*args, 4, 0, *base, check=False, **cl)
    assert o["status"] == R.RRTMG_ERR_UNSUPPORTED  # icld outside 0..3
    o = gpu.rrtmg_sw(*args, 1, 0, *base, check=False, cldfr=cl["cldfr"], taucld=cl["taucld"])
    assert o["status"] == R.RRTMG_ERR_ARG  # no ssacld / asmcld / fsfcld
    # icld = 2 and 3 are icld = 1 without McICA (only clear and overcast layers)
    gpu.set_precision("fp64")
    a = gpu.rrtmg_sw(*args, 1, 0, *base, **cl)
    for icld in (2, 3):
        b = gpu.rrtmg_sw(*args, icld, 0, *base, **cl)
        for k in ("swuflx", "swdflx", "swhr"):
            assert np.array_equal(a[k], b[k]), (icld, k)
