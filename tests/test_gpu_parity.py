"""GPU parity: the sm_103a path through the C-ABI against the CPU oracle.

Tolerances (FP64 path): fluxes within 1e-10 relative (floor 1e-3 W/m2 for
levels where the flux vanishes, e.g. LW downward flux at the top), heating
rates within 1e-8 K/day absolute.  FP32-split path: heating rates within
0.05 K/day, OLR and surface fluxes within 0.1 W/m2 of the FP64 oracle.
"""
import json
from pathlib import Path

import numpy as np
import pytest

from conftest import rel_err
from mima_gb300 import atmosphere as A
from mima_gb300 import rrtmg as R

pytestmark = pytest.mark.gpu

FLUX_TOL = 1e-10
HR_TOL = 1e-8
HR_REL = 1e-9


def hr_ok(out, ref):
    """Heating within HR_TOL K/day plus HR_REL relative: a heating rate is a
    flux difference over the layer's pressure thickness, so over the
    0.002 hPa layers of deep columns it amplifies the relative agreement of
    the fluxes (1e-14 there) by the flux over the difference."""
    return bool(np.all(np.abs(out - ref) <= HR_TOL + HR_REL * np.abs(ref)))


def check_lw(out, ref, idrv=0):
    for k in ("uflx", "dflx", "uflxc", "dflxc"):
        assert rel_err(out[k], ref[k], 1e-3) < FLUX_TOL, k
    for k in ("hr", "hrc"):
        assert hr_ok(out[k], ref[k]), k
    if idrv == 1:
        for k in ("duflx_dt", "duflxc_dt"):
            assert rel_err(out[k], ref[k], 1e-6) < FLUX_TOL, k


def check_sw(out, ref):
    for k in ("swuflx", "swdflx", "swuflxc", "swdflxc"):
        assert rel_err(out[k], ref[k], 1e-3) < FLUX_TOL, k
    for k in ("swhr", "swhrc"):
        assert hr_ok(out[k], ref[k]), k


@pytest.mark.parametrize("nlay", [40, 60])
def test_lw_fp64_matches_oracle(gpu, orc, nlay):
    atm = A.small_atmosphere(1024, nlay, seed=11 + nlay)
    gpu.set_precision("fp64")
    check_lw(gpu.lw(atm), orc.rrtmg_lw(atm))


@pytest.mark.parametrize("nlay", [40, 60])
def test_sw_fp64_matches_oracle(gpu, orc, nlay):
    atm = A.small_atmosphere(1024, nlay, seed=21 + nlay)
    gpu.set_precision("fp64")
    check_sw(gpu.sw(atm), orc.rrtmg_sw(atm))


def test_t42_full_grid_fp64(gpu, orc):
    """Configuration 0 of the benchmark set: T42 x 40 layers, 8192 columns."""
    atm = A.config_atmosphere(0)
    gpu.set_precision("fp64")
    check_lw(gpu.lw(atm), orc.rrtmg_lw(atm))
    check_sw(gpu.sw(atm), orc.rrtmg_sw(atm))


def test_t85_full_grid_fp64_and_split(gpu, orc):
    """Configuration 1, the benchmark's headline workload: T85 x 40 layers,
    32768 columns, every column.  FP64 within the FP64 parity tolerance of
    the oracle; FP32-split within the split bars (0.1 W/m2 at every level,
    the heating bar of tests/split_bars.py) against the same oracle outputs."""
    import split_bars as SB
    atm = A.config_atmosphere(1)
    rlw, rsw = orc.rrtmg_lw(atm), orc.rrtmg_sw(atm)
    gpu.set_precision("fp64")
    check_lw(gpu.lw(atm), rlw)
    check_sw(gpu.sw(atm), rsw)
    gpu.set_precision("split")
    try:
        lw, sw = gpu.lw(atm), gpu.sw(atm)
    finally:
        gpu.set_precision("fp64")
    bar = SB.hr_bar(atm)
    for out, ref, keys, hk in ((lw, rlw, ("uflx", "dflx"), "hr"), (sw, rsw, ("swuflx", "swdflx"), "swhr")):
        for k in keys:
            assert np.abs(out[k] - ref[k]).max() <= SB.FLUX_BAR, (k, np.abs(out[k] - ref[k]).max())
        assert np.all(np.abs(out[hk] - ref[hk]) <= bar), (hk, np.abs(out[hk] - ref[hk]).max())


def test_lw_idrv_surface_derivative(gpu, orc):
    atm = A.small_atmosphere(256, 40, seed=5)
    gpu.set_precision("fp64")
    check_lw(gpu.lw(atm, idrv=1), orc.rrtmg_lw(atm, idrv=1), idrv=1)


def test_lw_surface_flux_known_answers(gpu):
    """The surface upward LW flux of the reference's standalone RRTMG_LW runs
    (tests/golden/rrtm_lw_std_atm.json; emissivity 1, so only the
    Planck tables, the band constants and, for the idrv = 1 run, the Planck
    derivative enter), one column per run, through the FP64 and the split path:
    within 1e-5 (FP64) and 5e-5 (split) of the printed values."""
    runs = json.loads((Path(__file__).resolve().parent / "golden" / "rrtm_lw_std_atm.json")
                      .read_text())["runs"]
    names = sorted(runs)
    atm = A.small_atmosphere(len(names), 40, seed=3)
    atm.tsfc = np.array([runs[n]["tbound"] for n in names])
    atm.emis = np.ones_like(atm.emis)
    dt = np.array([runs[n].get("dtbound", 0.0) for n in names])
    ref = np.array([runs[n]["surface_up"][0][2] for n in names])
    for prec, tol in (("fp64", 1e-5), ("split", 5e-5)):
        gpu.set_precision(prec)
        try:
            out = gpu.lw(atm, idrv=1)
        finally:
            gpu.set_precision("fp64")
        up = out["uflx"][0] + dt * out["duflx_dt"][0]
        assert np.all(np.abs(up - ref) <= tol * ref), (prec, up - ref)


def test_standard_atmospheres(gpu, orc):
    """The reference's clear-sky standard atmospheres (the TAPE5 profiles of
    doc_rrtm/runs_std_atm: midlatitude summer and winter, subarctic winter,
    tropical; 51-60 layers to 0.07 hPa) as columns: the FP64 path against the
    oracle at the FP64 tolerances, with idrv = 1; the split path within the
    split bars (0.05 K/day heating, 0.1 W/m2 OLR and surface fluxes)."""
    from test_oracle_std_atm import PROFILES, RUNS, std_atm_column
    for name in PROFILES:
        atm = std_atm_column(RUNS[name])
        rlw, rsw = orc.rrtmg_lw(atm, idrv=1), orc.rrtmg_sw(atm)
        gpu.set_precision("fp64")
        check_lw(gpu.lw(atm, idrv=1), rlw, idrv=1)
        check_sw(gpu.sw(atm), rsw)
        gpu.set_precision("split")
        try:
            lw, sw = gpu.lw(atm), gpu.sw(atm)
        finally:
            gpu.set_precision("fp64")
        assert np.abs(lw["hr"] - rlw["hr"]).max() <= 0.05, name
        assert np.abs(sw["swhr"] - rsw["swhr"]).max() <= 0.05, name
        assert abs(lw["uflx"][-1, 0] - rlw["uflx"][-1, 0]) <= 0.1, name
        for k in ("uflx", "dflx"):
            assert abs(lw[k][0, 0] - rlw[k][0, 0]) <= 0.1, (name, k)
        for k in ("swuflx", "swdflx"):
            assert abs(sw[k][0, 0] - rsw[k][0, 0]) <= 0.1, (name, k)


def test_trace_gases_emissivity_and_aerosol(gpu, orc):
    """All optional gases non-zero, spectral emissivity < 1, LW and SW aerosols."""
    rng = np.random.default_rng(9)
    atm = A.small_atmosphere(512, 40, seed=9)
    shp = atm.play.shape
    atm.ch4 = np.full(shp, 1.8e-6)
    atm.n2o = np.full(shp, 3.2e-7)
    atm.o2 = np.full(shp, 0.209)
    atm.cfc11 = np.full(shp, 2.5e-10)
    atm.cfc12 = np.full(shp, 5.0e-10)
    atm.cfc22 = np.full(shp, 1.5e-10)
    atm.ccl4 = np.full(shp, 1.0e-10)
    atm.co2 = rng.uniform(200e-6, 1500e-6, size=shp)  # exercises the CO2 column adjustments
    atm.emis = rng.uniform(0.85, 1.0, size=(16, atm.ncol))
    lw_aer = rng.uniform(0.0, 0.05, size=(16, atm.nlay, atm.ncol))
    sw_tau = rng.uniform(0.0, 0.1, size=(14, atm.nlay, atm.ncol))
    sw_ssa = rng.uniform(0.8, 1.0, size=(14, atm.nlay, atm.ncol))
    sw_asm = rng.uniform(0.0, 0.8, size=(14, atm.nlay, atm.ncol))
    gpu.set_precision("fp64")
    check_lw(gpu.lw(atm, tauaer=lw_aer), orc.rrtmg_lw(atm, tauaer=lw_aer))
    check_sw(gpu.sw(atm, iaer=10, tauaer=sw_tau, ssaaer=sw_ssa, asmaer=sw_asm),
             orc.rrtmg_sw(atm, iaer=10, tauaer=sw_tau, ssaaer=sw_ssa, asmaer=sw_asm))


def test_dark_columns_and_ragged_sizes(gpu, orc):
    gpu.set_precision("fp64")
    for n in (1, 3, 33, 127):
        atm = A.small_atmosphere(n, 40, seed=100 + n)
        atm.coszen[::2] = 0.0  # MiMA skips columns with coszen < 1e-10
        sw = gpu.sw(atm)
        ref = orc.rrtmg_sw(atm)
        check_sw(sw, ref)
        assert np.all(sw["swdflx"][:, ::2] == 0.0)
        check_lw(gpu.lw(atm), orc.rrtmg_lw(atm))


def test_extreme_temperatures(gpu, orc):
    """Table-index clamps (Planck 1..180, jt 1..4) at MiMA's T limits 100..370 K."""
    atm = A.small_atmosphere(64, 40, seed=77)
    atm.tlay[:, :16] = 100.0
    atm.tlev[:, :16] = 100.0
    atm.tsfc[:16] = 100.0
    atm.tlay[:, 16:32] = 370.0
    atm.tlev[:, 16:32] = 370.0
    atm.tsfc[16:32] = 370.0
    gpu.set_precision("fp64")
    check_lw(gpu.lw(atm), orc.rrtmg_lw(atm))
    check_sw(gpu.sw(atm), orc.rrtmg_sw(atm))


def test_split_precision_error_budget(gpu, orc):
    """FP32-split vs the FP64 oracle on T170-like columns (60 layers, top 0.01 hPa)."""
    atm = A.small_atmosphere(2048, 60, seed=31, ts_sigma=5.0, rh_random=True)
    rlw, rsw = orc.rrtmg_lw(atm), orc.rrtmg_sw(atm)
    gpu.set_precision("split")
    try:
        lw, sw = gpu.lw(atm), gpu.sw(atm)
    finally:
        gpu.set_precision("fp64")
    hr = np.abs(lw["hr"] - rlw["hr"]) + 0.0
    shr = np.abs(sw["swhr"] - rsw["swhr"])
    assert hr.max() <= 0.05, hr.max()
    assert shr.max() <= 0.05, shr.max()
    assert np.abs(lw["uflx"][-1] - rlw["uflx"][-1]).max() <= 0.1  # OLR
    for k in ("uflx", "dflx"):
        assert np.abs(lw[k][0] - rlw[k][0]).max() <= 0.1
    for k in ("swuflx", "swdflx"):
        assert np.abs(sw[k][0] - rsw[k][0]).max() <= 0.1


def test_device_api_matches_host_api_and_graph_capture(gpu):
    import torch
    atm = A.small_atmosphere(300, 40, seed=4)
    gpu.set_precision("fp64")
    hlw, hsw = gpu.lw(atm), gpu.sw(atm)
    d = R.atm_device_inputs(atm)
    olw, osw = R.device_outputs(atm.ncol, atm.nlay)
    s = torch.cuda.Stream()
    gpu.reserve(atm.ncol, atm.nlay)
    with torch.cuda.stream(s):
        gpu.rrtmg_lw_dev(s.cuda_stream, atm.ncol, atm.nlay, 0, 0, d, olw)
        gpu.rrtmg_sw_dev(s.cuda_stream, atm.ncol, atm.nlay, 0, 0, d, osw, atm.adjes, atm.dyofyr, atm.scon)
    s.synchronize()
    for k in olw:
        assert np.array_equal(olw[k].cpu().numpy(), hlw[k]), k
    for k in osw:
        assert np.array_equal(osw[k].cpu().numpy(), hsw[k]), k
    # the same two calls captured once in a CUDA graph and replayed
    for t in list(olw.values()) + list(osw.values()):
        t.zero_()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        gpu.rrtmg_lw_dev(s.cuda_stream, atm.ncol, atm.nlay, 0, 0, d, olw)
        gpu.rrtmg_sw_dev(s.cuda_stream, atm.ncol, atm.nlay, 0, 0, d, osw, atm.adjes, atm.dyofyr, atm.scon)
    g.replay()
    torch.cuda.synchronize()
    for k in olw:
        assert np.array_equal(olw[k].cpu().numpy(), hlw[k]), k
    assert gpu.sync_status(s.cuda_stream) == 0


@pytest.mark.parametrize("precision", ["fp64", "split"])
def test_fused_step_equals_separate_calls_and_captures(gpu, precision):
    """rrtmg_step_dev (SW forked onto the handle's second stream) gives the
    results of rrtmg_lw_dev + rrtmg_sw_dev bit for bit, directly and replayed
    from a CUDA graph, with idrv = 1 and aerosols on both sides."""
    import torch
    rng = np.random.default_rng(31)
    atm = A.small_atmosphere(700, 40, seed=31)
    gpu.set_precision(precision)
    try:
        d = R.atm_device_inputs(atm)
        t = lambda a: torch.from_numpy(a).cuda()
        aer_lw = t(rng.uniform(0.0, 0.05, size=(16, atm.nlay, atm.ncol)))
        d["tauaer"] = t(rng.uniform(0.0, 0.1, size=(14, atm.nlay, atm.ncol)))
        d["ssaaer"] = t(rng.uniform(0.8, 1.0, size=(14, atm.nlay, atm.ncol)))
        d["asmaer"] = t(rng.uniform(0.0, 0.8, size=(14, atm.nlay, atm.ncol)))
        s = torch.cuda.Stream()
        gpu.reserve(atm.ncol, atm.nlay)
        rlw, rsw = R.device_outputs(atm.ncol, atm.nlay, idrv=1)
        olw, osw = R.device_outputs(atm.ncol, atm.nlay, idrv=1)
        with torch.cuda.stream(s):
            gpu.rrtmg_lw_dev(s.cuda_stream, atm.ncol, atm.nlay, 0, 1, d, rlw, tauaer=aer_lw)
            gpu.rrtmg_sw_dev(s.cuda_stream, atm.ncol, atm.nlay, 0, 10, d, rsw, atm.adjes, atm.dyofyr, atm.scon)
            gpu.rrtmg_step_dev(s.cuda_stream, atm.ncol, atm.nlay, d, olw, osw, atm.adjes, atm.dyofyr, atm.scon,
                               idrv=1, iaer=10, tauaer_lw=aer_lw)
        s.synchronize()
        for k in olw:
            assert torch.equal(olw[k], rlw[k]), k
        for k in osw:
            assert torch.equal(osw[k], rsw[k]), k
        for x in list(olw.values()) + list(osw.values()):
            x.zero_()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=s):
            gpu.rrtmg_step_dev(s.cuda_stream, atm.ncol, atm.nlay, d, olw, osw, atm.adjes, atm.dyofyr, atm.scon,
                               idrv=1, iaer=10, tauaer_lw=aer_lw)
        before = gpu.launch_count()
        g.replay()
        torch.cuda.synchronize()
        assert gpu.launch_count() == before  # a replay issues no new library calls
        for k in olw:
            assert torch.equal(olw[k], rlw[k]), k
        for k in osw:
            assert torch.equal(osw[k], rsw[k]), k
        assert gpu.sync_status(s.cuda_stream) == 0
    finally:
        gpu.set_precision("fp64")


def test_invalid_input_and_unsupported_configurations(gpu):
    atm = A.small_atmosphere(8, 40, seed=1)
    atm.tlay[5, 3] = np.nan
    out = gpu.lw(atm, check=False)
    assert out["status"] == R.RRTMG_ERR_INPUT
    atm = A.small_atmosphere(8, 40, seed=1)
    o = gpu.rrtmg_lw(atm.ncol, atm.nlay, 4, 0, atm.play, atm.plev, atm.tlay, atm.tlev, atm.tsfc, atm.h2o,
                     atm.o3, atm.co2, check=False)
    assert o["status"] == R.RRTMG_ERR_UNSUPPORTED  # icld outside 0..3
    o = gpu.rrtmg_lw(atm.ncol, atm.nlay, 2, 0, atm.play, atm.plev, atm.tlay, atm.tlev, atm.tsfc, atm.h2o,
                     atm.o3, atm.co2, check=False)
    assert o["status"] == R.RRTMG_ERR_ARG  # clouds without cloud arrays
    o = gpu.rrtmg_sw(atm.ncol, atm.nlay, 0, 6, atm.play, atm.plev, atm.tlay, atm.tlev, atm.tsfc, atm.h2o,
                     atm.o3, atm.co2, None, None, None, atm.asdir, atm.asdif, atm.aldir, atm.aldif,
                     atm.coszen, 1.0, 0, 1360.0, check=False)
    assert o["status"] == R.RRTMG_ERR_UNSUPPORTED
    # a valid call after the failures still works
    assert gpu.lw(atm)["status"] == R.RRTMG_OK


def test_launch_count_is_native(gpu):
    atm = A.small_atmosphere(16, 40, seed=2)
    before = gpu.launch_count()
    gpu.lw(atm)
    gpu.sw(atm)
    assert gpu.launch_count() - before == 8


def test_allocation_failure_is_reported_and_recoverable(blob, monkeypatch):
    """An injected workspace allocation failure (RRTMG_GPU_FAIL_ALLOC=1, made on
    the host) is reported as RRTMG_ERR_NOMEM by the host and device calls; the
    handle stays usable, and once allocations succeed again the results are
    those of an undisturbed handle."""
    import torch
    atm = A.small_atmosphere(96, 40, seed=61)
    ref = R.RRTMG(blob)
    r = R.RRTMG(blob)  # a fresh handle: no workspace yet
    try:
        monkeypatch.setenv("RRTMG_GPU_FAIL_ALLOC", "1")
        for call in (lambda: r.lw(atm), lambda: r.sw(atm)):
            with pytest.raises(R.RRTMGError) as ei:
                call()
            assert "allocation" in str(ei.value)
        d = R.atm_device_inputs(atm)
        olw, _ = R.device_outputs(atm.ncol, atm.nlay)
        with pytest.raises(R.RRTMGError):
            r.rrtmg_lw_dev(torch.cuda.current_stream().cuda_stream, atm.ncol, atm.nlay, 0, 0, d, olw)
        monkeypatch.delenv("RRTMG_GPU_FAIL_ALLOC")
        got, want = r.lw(atm), ref.lw(atm)
        for k in want:
            assert np.array_equal(got[k], want[k]), k
        assert np.array_equal(r.sw(atm)["swdflx"], ref.sw(atm)["swdflx"])
    finally:
        r.close()
        ref.close()


@pytest.mark.gpu
def test_fp64_path_reproduces_golden_fixtures(gpu):
    """The committed oracle regression fixtures (tests/golden) at the FP64 tolerance."""
    from pathlib import Path
    ref = np.load(Path(__file__).with_name("golden") / "oracle_regression.npz")
    gpu.set_precision("fp64")
    for name, (ncol, nlay, seed, sig, rh) in {"l40": (8, 40, 101, 2.0, False), "l60": (6, 60, 202, 5.0, True)}.items():
        atm = A.small_atmosphere(ncol, nlay, seed=seed, ts_sigma=sig, rh_random=rh)
        lw, sw = gpu.lw(atm, idrv=1), gpu.sw(atm)
        for k in ("uflx", "dflx", "duflx_dt"):
            assert rel_err(lw[k], ref[f"{name}_{k}"], 1e-6) <= FLUX_TOL, (name, k)
        assert rel_err(lw["hr"], ref[f"{name}_hr"], 1e-3) <= HR_TOL, name
        for k in ("swuflx", "swdflx"):
            assert rel_err(sw[k], ref[f"{name}_{k}"], 1e-6) <= FLUX_TOL, (name, k)
        assert rel_err(sw["swhr"], ref[f"{name}_swhr"], 1e-3) <= HR_TOL, name


def test_sw_conserves_energy_without_absorbers(gpu, orc):
    """Pure Rayleigh scattering over a white surface (no absorbers): the net SW
    flux is zero at every level and no layer absorbs.  FP64 (equal to the
    oracle): net flux within 1e-3 W/m2 (the reference's single-scattering-albedo
    cap of 1 - 1e-6), heating within 1e-5 K/day.  Split (delta-Eddington terms
    for nearly conservative layers reformulated for FP32): net flux within
    0.1 W/m2 and each layer's net-flux divergence within 0.01 W/m2 -- stated as
    a flux because the top layers here are 0.003 hPa thin, where 1e-4 W/m2 of
    FP32 rounding already reads as 0.3 K/day."""
    from test_oracle import scattering_only
    atm = scattering_only(ncol=64)
    gpu.set_precision("fp64")
    sw = gpu.sw(atm)
    check_sw(sw, orc.rrtmg_sw(atm))
    net = sw["swdflx"] - sw["swuflx"]
    assert np.abs(net).max() <= 1e-3 and np.abs(sw["swhr"]).max() <= 1e-5
    gpu.set_precision("split")
    try:
        sw = gpu.sw(atm)
    finally:
        gpu.set_precision("fp64")
    net = sw["swdflx"] - sw["swuflx"]
    assert np.abs(net).max() <= 0.1, np.abs(net).max()
    assert np.abs(np.diff(net, axis=0)).max() <= 0.01, np.abs(np.diff(net, axis=0)).max()


@pytest.mark.parametrize("nlay", [100, 203])
def test_deep_columns(gpu, orc, nlay):
    """Columns deeper than 64 layers (the solvers' 208-level variants), up to
    the reference's maximum of 203 layers (mxlay, parrrtm.f90 / parrrsw.f90):
    the FP64 path against the oracle at the FP64 tolerances, with idrv = 1;
    the split path within 0.1 W/m2 of the oracle at every level.  (The split
    heating-rate bar is stated for 40 layers; at 203 layers to 0.01 hPa a layer
    is down to 6e-4 hPa thick, and the same flux error is a larger rate.)"""
    atm = A.small_atmosphere(96, nlay, seed=300 + nlay)
    rlw, rsw = orc.rrtmg_lw(atm, idrv=1), orc.rrtmg_sw(atm)
    gpu.set_precision("fp64")
    check_lw(gpu.lw(atm, idrv=1), rlw, idrv=1)
    check_sw(gpu.sw(atm), rsw)
    gpu.set_precision("split")
    try:
        lw, sw = gpu.lw(atm, idrv=1), gpu.sw(atm)
    finally:
        gpu.set_precision("fp64")
    for k in ("uflx", "dflx"):
        assert np.abs(lw[k] - rlw[k]).max() <= 0.1, k
    for k in ("swuflx", "swdflx"):
        assert np.abs(sw[k] - rsw[k]).max() <= 0.1, k
    assert np.isfinite(lw["hr"]).all() and np.isfinite(sw["swhr"]).all()


def test_edge_columns(gpu, orc):
    """The fewest layers (2, 3) and columns wholly below or wholly above the
    troposphere boundary (laytrop = nlay: the solar-source search reads past the
    last layer, as the reference's jp(lay+1); laytrop = 0: the lower-atmosphere
    loops are empty): FP64 against the oracle at the FP64 tolerances, split
    within 0.1 W/m2 at every level."""
    from test_oracle import edge_columns
    for name, atm in edge_columns().items():
        rlw, rsw = orc.rrtmg_lw(atm, idrv=1), orc.rrtmg_sw(atm)
        gpu.set_precision("fp64")
        check_lw(gpu.lw(atm, idrv=1), rlw, idrv=1)
        check_sw(gpu.sw(atm), rsw)
        gpu.set_precision("split")
        try:
            lw, sw = gpu.lw(atm), gpu.sw(atm)
        finally:
            gpu.set_precision("fp64")
        for k in ("uflx", "dflx"):
            assert np.abs(lw[k] - rlw[k]).max() <= 0.1, (name, k)
        for k in ("swuflx", "swdflx"):
            assert np.abs(sw[k] - rsw[k]).max() <= 0.1, (name, k)


def _random_case(rng):
    """One seeded random case of test_random_columns (the draw order is part of
    the case definition)."""
    nlay = int(rng.choice([2, 5, 17, 40, 64, 65, 90]))
    ncol = int(rng.integers(1, 200))
    atm = A.small_atmosphere(ncol, nlay, seed=int(rng.integers(1 << 30)), ts_sigma=float(rng.uniform(0.0, 15.0)),
                             rh_random=bool(rng.integers(2)))
    shp = atm.play.shape
    atm.co2 = rng.uniform(100e-6, 2000e-6, size=shp)
    atm.o3 = atm.o3 * rng.uniform(0.0, 3.0)
    atm.h2o = np.clip(atm.h2o * rng.uniform(0.05, 1.5), 1e-7, 0.05)
    if rng.integers(2):
        atm.ch4, atm.n2o, atm.o2 = np.full(shp, 1.8e-6), np.full(shp, 3.2e-7), np.full(shp, 0.209)
        atm.cfc11, atm.cfc12 = np.full(shp, 2.5e-10), np.full(shp, 5.0e-10)
        atm.cfc22, atm.ccl4 = np.full(shp, 1.5e-10), np.full(shp, 1.0e-10)
    atm.emis = rng.uniform(0.8, 1.0, size=(16, ncol))
    atm.coszen = rng.uniform(0.0, 1.0, ncol) * (rng.uniform(size=ncol) > 0.3)
    for k in ("asdir", "asdif", "aldir", "aldif"):
        setattr(atm, k, rng.uniform(0.0, 0.9, ncol))
    idrv = int(rng.integers(2))
    lw_aer = rng.uniform(0.0, 0.05, size=(16, nlay, ncol)) if rng.integers(2) else None
    if rng.integers(2):
        aer = dict(iaer=10, tauaer=rng.uniform(0.0, 0.1, size=(14, nlay, ncol)),
                   ssaaer=rng.uniform(0.8, 1.0, size=(14, nlay, ncol)),
                   asmaer=rng.uniform(0.0, 0.8, size=(14, nlay, ncol)))
    else:
        aer = {}
    return atm, idrv, lw_aer, aer


def test_random_columns(gpu, orc):
    """Seeded random cases across the inputs: layer counts on both sides of the
    solvers' 64 / 208-level switch, ragged column counts, surface-temperature
    spread, gas amounts (CO2 100-2000 ppmv, O3 and H2O scaled, the secondary
    gases on or off), spectral emissivity, albedos up to 0.9, dark and sunlit
    columns, idrv, LW and SW aerosols.

    FP64 path: against the oracle at the FP64 tolerances.  Split path: the bars
    of tests/split_bars.py (0.1 W/m2 at every level; 0.05 K/day heating up to
    60 layers, where the bar is stated, in layers heated or cooled by less than
    100 K/day: the aerosol depths here are drawn per layer, up to 0.1 even in
    the 0.003 hPa layers near the top, which heats those layers by up to 10^4
    K/day, where the flux bar at every level is the meaningful one), in both
    transcendental modes.  With the
    analytic exponentials every column must meet them.  With the reference's
    tables a column may miss them only where the reference itself is
    ill-conditioned (the delta-Eddington resonance k mu0 = 1 amplifying one
    table step): then the oracle on inputs within FP32 rounding of the given
    ones must reproduce the split result within the bars.  Case 3 holds such a
    column (band 25, k mu0 = 0.9993: a 1e-6 relative change of the aerosol
    depth moves the oracle's surface flux by 2.15 W/m2)."""
    import split_bars as SB
    rng = np.random.default_rng(2024)
    gpu.set_precision("fp64")
    excused = {}
    for case in range(12):
        atm, idrv, lw_aer, aer = _random_case(rng)
        heating = atm.nlay <= 60
        rlw, rsw = orc.rrtmg_lw(atm, idrv=idrv, tauaer=lw_aer), orc.rrtmg_sw(atm, **aer)
        check_lw(gpu.lw(atm, idrv=idrv, tauaer=lw_aer), rlw, idrv=idrv)
        check_sw(gpu.sw(atm, **aer), rsw)
        gpu.set_precision("split")
        try:
            slw, ssw = gpu.lw(atm, idrv=idrv, tauaer=lw_aer), gpu.sw(atm, **aer)
            gpu.set_transcendentals("analytic")
            alw, asw = gpu.lw(atm, idrv=idrv, tauaer=lw_aer), gpu.sw(atm, **aer)
        finally:
            gpu.set_transcendentals("table")
            gpu.set_precision("fp64")
        excused[case] = (SB.check_lw(orc, atm, slw, rlw, idrv=idrv, tauaer=lw_aer, heating=heating, hr_limit=100.0)
                         + SB.check_sw(orc, atm, ssw, rsw, aer=aer, heating=heating, hr_limit=100.0))
        orc.set_table_mode(False)
        try:
            blw, bsw = orc.rrtmg_lw(atm, idrv=idrv, tauaer=lw_aer), orc.rrtmg_sw(atm, **aer)
        finally:
            orc.set_table_mode(True)
        for k in ("swuflx", "swdflx"):
            assert np.abs(asw[k] - bsw[k]).max() <= SB.FLUX_BAR, (case, "analytic", k)
        for k in ("uflx", "dflx"):
            assert np.abs(alw[k] - blw[k]).max() <= SB.FLUX_BAR, (case, "analytic", k)
        if heating:
            for o, b, k in ((asw, bsw, "swhr"), (alw, blw, "hr")):
                plausible = np.abs(b[k]) <= 100.0
                assert np.all((np.abs(o[k] - b[k]) <= SB.hr_bar(atm))[plausible]), (case, "analytic", k)
    # the resonance column of case 3 needed the allowance; few others may
    assert 20 in [c for c, _, _ in excused[3]], excused
    assert sum(len(v) for v in excused.values()) <= 4, excused


def test_grazing_sun(gpu, orc):
    """Sun just above the horizon (coszen 2e-10 ... 0.05, above MiMA's 1e-10
    skip): direct-beam transmittances underflow and the exp-table index
    saturates.  FP64 against the oracle at the FP64 tolerances; split within
    0.1 W/m2 and 0.05 K/day."""
    atm = A.small_atmosphere(6, 40, seed=81)
    atm.coszen = np.array([2e-10, 1e-8, 1e-5, 1e-3, 0.01, 0.05])
    ref = orc.rrtmg_sw(atm)
    gpu.set_precision("fp64")
    check_sw(gpu.sw(atm), ref)
    gpu.set_precision("split")
    try:
        sw = gpu.sw(atm)
    finally:
        gpu.set_precision("fp64")
    for k in ("swuflx", "swdflx"):
        assert np.abs(sw[k] - ref[k]).max() <= 0.1, k
    assert np.abs(sw["swhr"] - ref["swhr"]).max() <= 0.05
