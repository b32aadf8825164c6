"""Cloud physics on the GPU against the oracle: the LW cloud depths formed
from water paths (cldprop inflag = 1) or from the ice and liquid
parameterisations with effective sizes (inflag = 2, iceflag 0-3, liqflag
0-1, rrtmg_lw_cldprop.f90:155-270) with the column's running count of cloud
bands and rtrn / rtrnmr's band map; the SW optics of cldprop_sw inflag = 2
(iceflag 1-3, liqflag 1, rrtmg_sw_cldprop.f90:158-340).

Tolerances as every FP64 parity test (fluxes 1e-10 relative, heating 1e-8
K/day + 1e-9 relative); the split path within the split bars (0.1 W/m2 at
every level, tests/split_bars.py's heating bar).
"""
import numpy as np
import pytest

import split_bars as SB
from mima_gb300 import atmosphere as A
from mima_gb300 import rrtmg as R
from test_gpu_parity import check_lw, check_sw
from test_oracle_cloud_physics import physics_fields

pytestmark = pytest.mark.gpu

LW_OPTIONS = [(1, 0, 0), (2, 0, 0), (2, 0, 1), (2, 1, 0), (2, 1, 1), (2, 2, 1), (2, 3, 1)]


def _lw_case(nlay, seed, n=384):
    rng = np.random.default_rng(seed)
    atm = A.small_atmosphere(n, nlay, seed=seed, ts_sigma=5.0, rh_random=True)
    atm.emis = rng.uniform(0.8, 1.0, size=(16, n))
    return atm, physics_fields(atm, rng)


def _phys(cl, inflag, iceflag, liqflag):
    return dict(cl, inflag=inflag, iceflag=iceflag, liqflag=liqflag)


@pytest.mark.parametrize("opt", LW_OPTIONS)
@pytest.mark.parametrize("icld", [1, 2])
def test_lw_cloud_physics_fp64_matches_oracle(gpu, orc, opt, icld):
    """Every LW option, both overlaps, idrv = 1.  iceflag = 1 (5 ice bands)
    exercises the running count: a column whose highest formed layer holds
    ice alone ends with 5 cloud bands, which the layers below it then use."""
    atm, cl = _lw_case(40, 300 + 10 * icld + opt[1] + 4 * opt[2])
    cloud = _phys(cl, *opt)
    ref = orc.rrtmg_lw(atm, idrv=1, cloud=cloud, icld=icld)
    gpu.set_precision("fp64")
    out = gpu.lw(atm, idrv=1, cloud=cloud, icld=icld)
    check_lw(out, ref, idrv=1)
    clear = orc.rrtmg_lw(atm)
    assert np.abs(ref["uflx"][-1] - clear["uflx"][-1]).max() > 5.0


def test_lw_cloud_physics_fp64_deep_columns(gpu, orc):
    atm, cl = _lw_case(60, 345)
    cloud = _phys(cl, 2, 3, 1)
    gpu.set_precision("fp64")
    check_lw(gpu.lw(atm, idrv=1, cloud=cloud, icld=2), orc.rrtmg_lw(atm, idrv=1, cloud=cloud, icld=2), idrv=1)


@pytest.mark.parametrize("opt", [(1, 0, 0), (2, 1, 1), (2, 3, 1)])
def test_lw_cloud_physics_split_within_bars(gpu, orc, opt):
    atm, cl = _lw_case(40, 360 + opt[1], n=768)
    cloud = _phys(cl, *opt)
    ref = orc.rrtmg_lw(atm, idrv=1, cloud=cloud, icld=2)
    gpu.set_precision("split")
    try:
        out = gpu.lw(atm, idrv=1, cloud=cloud, icld=2)
    finally:
        gpu.set_precision("fp64")
    bar = SB.hr_bar(atm)
    for k in ("uflx", "dflx", "uflxc", "dflxc"):
        assert np.abs(out[k] - ref[k]).max() <= SB.FLUX_BAR, (k, np.abs(out[k] - ref[k]).max())
    for k in ("hr", "hrc"):
        assert np.all(np.abs(out[k] - ref[k]) <= bar), (k, np.abs(out[k] - ref[k]).max())


def _sw_case(nlay, seed, n=384):
    rng = np.random.default_rng(seed)
    atm = A.small_atmosphere(n, nlay, seed=seed)
    return atm, physics_fields(atm, rng, overcast=True)


@pytest.mark.parametrize("iceflag", [1, 2, 3])
@pytest.mark.parametrize("nlay", [40, 60])
def test_sw_cloud_physics_fp64_matches_oracle(gpu, orc, iceflag, nlay):
    atm, cl = _sw_case(nlay, 400 + iceflag + nlay)
    cloud = _phys(cl, 2, iceflag, 1)
    ref = orc.rrtmg_sw(atm, cloud=cloud)
    gpu.set_precision("fp64")
    check_sw(gpu.sw(atm, cloud=cloud), ref)
    clear = orc.rrtmg_sw(atm)
    assert np.abs(ref["swuflx"][-1] - clear["swuflx"][-1]).max() > 20.0


@pytest.mark.parametrize("iceflag", [1, 3])
def test_sw_cloud_physics_split_within_bars(gpu, orc, iceflag):
    atm, cl = _sw_case(40, 450 + iceflag, n=768)
    cloud = _phys(cl, 2, iceflag, 1)
    ref = orc.rrtmg_sw(atm, cloud=cloud)
    gpu.set_precision("split")
    try:
        out = gpu.sw(atm, cloud=cloud)
    finally:
        gpu.set_precision("fp64")
    bar = SB.hr_bar(atm)
    for k in ("swuflx", "swdflx", "swuflxc", "swdflxc"):
        assert np.abs(out[k] - ref[k]).max() <= SB.FLUX_BAR, (k, np.abs(out[k] - ref[k]).max())
    for k in ("swhr", "swhrc"):
        assert np.all(np.abs(out[k] - ref[k]) <= bar), (k, np.abs(out[k] - ref[k]).max())


def test_lw_cloud_physics_host_entry_matches_device_entry(gpu):
    """rrtmg_lw_c (page-locked arrays, 40000 columns in two chunks, the sizes
    copied with the water paths) against rrtmg_lw_dev, bit for bit."""
    torch = pytest.importorskip("torch")
    atm, cl = _lw_case(40, 370, n=40000)
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
    L, n = atm.nlay, atm.ncol
    outs = {k: pin(np.zeros((L + 1 if k not in ("hr", "hrc") else L, n))) for k in
            ("uflx", "dflx", "hr", "uflxc", "dflxc", "hrc", "duflx_dt", "duflxc_dt")}
    gpu.set_precision("split")
    try:
        host = gpu.rrtmg_lw(n, L, 2, 1, *[pin(a) for a in (atm.play, atm.plev, atm.tlay, atm.tlev, atm.tsfc, atm.h2o,
                                                         atm.o3, atm.co2, atm.ch4, atm.n2o, atm.o2, atm.cfc11,
                                                         atm.cfc12, atm.cfc22, atm.ccl4, atm.emis)],
                            out=outs, inflglw=2, iceflglw=1, liqflglw=1,
                            **{k: pin(v) for k, v in cl.items()})
        d = R.atm_device_inputs(atm)
        d.update({k: torch.from_numpy(np.ascontiguousarray(v)).cuda() for k, v in cl.items()})
        o, _ = R.device_outputs(n, L, idrv=1)
        s = torch.cuda.Stream()
        with torch.cuda.stream(s):
            gpu.rrtmg_lw_dev(s.cuda_stream, n, L, 2, 1, d, o, inflglw=2, iceflglw=1, liqflglw=1)
        s.synchronize()
    finally:
        gpu.set_precision("fp64")
    for k in o:
        assert np.array_equal(o[k].cpu().numpy(), host[k]), k


def test_sw_cloud_physics_host_entry_matches_device_entry(gpu):
    torch = pytest.importorskip("torch")
    atm, cl = _sw_case(40, 380, n=40000)
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
                            atm.adjes, atm.dyofyr, atm.scon, out=outs, inflgsw=2, iceflgsw=2, liqflgsw=1,
                            **{k: pin(v) for k, v in cl.items()})
        d = R.atm_device_inputs(atm)
        dc = {k: torch.from_numpy(np.ascontiguousarray(v)).cuda() for k, v in cl.items()}
        dc.update(inflag=2, iceflag=2, liqflag=1)
        o = {k: torch.zeros(v.shape, dtype=torch.float64, device="cuda") for k, v in outs.items()}
        s = torch.cuda.Stream()
        with torch.cuda.stream(s):
            gpu.rrtmg_sw_dev(s.cuda_stream, n, L, 1, 0, d, o, atm.adjes, atm.dyofyr, atm.scon, cloud=dc)
        s.synchronize()
    finally:
        gpu.set_precision("fp64")
    for k in o:
        assert np.array_equal(o[k].cpu().numpy(), host[k]), k


@pytest.mark.parametrize("side,opt,key,bad", [
    ("lw", (2, 0, 0), "reice", 9.0),
    ("lw", (2, 1, 1), "reice", 131.0),
    ("lw", (2, 3, 1), "reliq", 61.0),
    ("lw", (2, 2, 1), "reice", np.nan),
    ("sw", (2, 1, 1), "reice", 12.0),
    ("sw", (2, 3, 1), "reice", 141.0),
    ("sw", (2, 2, 1), "reliq", 2.0),
])
@pytest.mark.parametrize("precision", ["fp64", "split"])
def test_cloud_physics_size_out_of_range_is_invalid_input(gpu, orc, side, opt, key, bad, precision):
    """A size outside its table in a formed layer (where the reference stops)
    returns invalid input; the handle stays usable and the same size in a
    layer without that water is not looked at (nor, in the SW, in an unlit
    column)."""
    atm = A.small_atmosphere(64, 40, seed=17)
    cl = physics_fields(atm, np.random.default_rng(8), overcast=side == "sw")
    water = "cicewp" if key == "reice" else "cliqwp"
    col = int(np.argmax(atm.coszen))
    lay = int(np.argmin(np.abs(atm.play[:, col] - 450.0)))
    cl["cldfr"][lay, col] = 1.0
    cl[water][lay, col] = 5.0
    cl[key][lay, col] = bad
    call = gpu.lw if side == "lw" else gpu.sw
    gpu.set_precision(precision)
    try:
        assert call(atm, cloud=_phys(cl, *opt), check=False)["status"] == R.RRTMG_ERR_INPUT
        assert "effective size" in gpu.last_error()
        if side == "sw":
            dark = (col + 1) % atm.ncol
            atm.coszen = np.where(np.arange(atm.ncol) == dark, 0.0, atm.coszen)
            c2 = {k: v.copy() for k, v in cl.items()}
            c2[water][lay, col] = 0.0
            lay2 = int(np.argmin(np.abs(atm.play[:, dark] - 450.0)))
            c2["cldfr"][lay2, dark], c2[water][lay2, dark], c2[key][lay2, dark] = 1.0, 5.0, bad
            assert call(atm, cloud=_phys(c2, *opt))["status"] == R.RRTMG_OK
        cl[water][lay, col] = 0.0
        out = call(atm, cloud=_phys(cl, *opt))
        assert out["status"] == R.RRTMG_OK
    finally:
        gpu.set_precision("fp64")
    if precision == "fp64":
        ref = orc.rrtmg_lw(atm, cloud=_phys(cl, *opt)) if side == "lw" else orc.rrtmg_sw(atm, cloud=_phys(cl, *opt))
        (check_lw if side == "lw" else check_sw)(call(atm, cloud=_phys(cl, *opt)), ref)


def test_cloud_physics_options_refused(gpu):
    atm = A.small_atmosphere(16, 40, seed=18)
    cl = physics_fields(atm, np.random.default_rng(9), overcast=True)
    for bad in [(3, 0, 0), (2, 4, 0), (2, 0, 2)]:
        assert gpu.lw(atm, cloud=_phys(cl, *bad), check=False)["status"] == R.RRTMG_ERR_UNSUPPORTED, bad
    for bad in [(1, 0, 0), (2, 0, 1), (2, 1, 0), (2, 4, 1)]:
        assert gpu.sw(atm, cloud=_phys(cl, *bad), check=False)["status"] == R.RRTMG_ERR_UNSUPPORTED, bad
    no_sizes = {k: v for k, v in cl.items() if k not in ("reice", "reliq")}
    assert gpu.lw(atm, cloud=_phys(no_sizes, 2, 2, 1), check=False)["status"] == R.RRTMG_ERR_ARG
    assert gpu.sw(atm, cloud=_phys(no_sizes, 2, 2, 1), check=False)["status"] == R.RRTMG_ERR_ARG
    assert gpu.lw(atm, cloud=_phys(no_sizes, 1, 0, 0))["status"] == R.RRTMG_OK  # inflag 1 needs no sizes


def test_cloud_physics_split_t85_full_grid(gpu, orc):
    """The benchmark's cloudy step (T85 x 40, every column, the seeded
    overcast clouds of atmosphere.cloud_physics_fields with Fu ice and
    Hu-Stamnes liquid): the split path within the split bars of the oracle.
    Among its columns a thick ice cloud at 112 hPa under a low sun, whose
    albedo lies within 1e-6 of 1 in several bands: its absorptance follows
    the co-albedo, which the split total-sky pass forms without cancellation."""
    atm = A.config_atmosphere(1)
    cl = A.cloud_physics_fields(atm, seed=2024)
    cloud = _phys(cl, 2, 3, 1)
    rlw = orc.rrtmg_lw(atm, cloud=cloud, icld=2)
    rsw = orc.rrtmg_sw(atm, cloud=cloud)
    gpu.set_precision("split")
    try:
        lw, sw = gpu.lw(atm, cloud=cloud, icld=2), gpu.sw(atm, cloud=cloud)
    finally:
        gpu.set_precision("fp64")
    bar = SB.hr_bar(atm)
    for out, ref, keys, hk in ((lw, rlw, ("uflx", "dflx"), "hr"), (sw, rsw, ("swuflx", "swdflx"), "swhr")):
        for k in keys:
            assert np.abs(out[k] - ref[k]).max() <= SB.FLUX_BAR, (k, np.abs(out[k] - ref[k]).max())
        assert np.all(np.abs(out[hk] - ref[hk]) <= bar), (hk, np.abs(out[hk] - ref[hk]).max())


@pytest.mark.parametrize("precision", ["fp64", "split"])
def test_cloud_physics_deep_and_ragged(gpu, orc, precision):
    """120 layers (the deep-column build of the solvers; the split LW cloud
    physics keeps 120 layer records per column in shared memory) and 77
    columns (warps with idle lanes in the SW cloud kernel, which computes a
    warp's formed layers together): LW maximum/random overlap with iceflag 1
    and liquid, SW Fu ice."""
    atm = A.small_atmosphere(77, 120, seed=19)
    cl = physics_fields(atm, np.random.default_rng(10), overcast=True)
    lw_c, sw_c = _phys(cl, 2, 1, 1), _phys(cl, 2, 3, 1)
    rlw = orc.rrtmg_lw(atm, idrv=1, cloud=lw_c, icld=2)
    rsw = orc.rrtmg_sw(atm, cloud=sw_c)
    gpu.set_precision(precision)
    try:
        lw, sw = gpu.lw(atm, idrv=1, cloud=lw_c, icld=2), gpu.sw(atm, cloud=sw_c)
    finally:
        gpu.set_precision("fp64")
    if precision == "fp64":
        check_lw(lw, rlw, idrv=1)
        check_sw(sw, rsw)
        return
    bar = SB.hr_bar(atm)
    for out, ref, keys, hk in ((lw, rlw, ("uflx", "dflx"), "hr"), (sw, rsw, ("swuflx", "swdflx"), "swhr")):
        for k in keys:
            assert np.abs(out[k] - ref[k]).max() <= SB.FLUX_BAR, (k, np.abs(out[k] - ref[k]).max())
        assert np.all(np.abs(out[hk] - ref[hk]) <= bar), (hk, np.abs(out[hk] - ref[hk]).max())
