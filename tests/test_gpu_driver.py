"""GPU parity of the device-resident radiation driver (rrtmg_run_c /
rrtmg_run_dev, include/rrtmg_run.h) against the CPU restatement of MiMA's
run_rrtmg, interp_temp and compute_zenith (oracle/driver.py).

Bit-exact chain: the library's driver output equals, bit for bit, the
oracle's input side -> the library's own rrtmg_lw / rrtmg_sw on the
oracle-prepared columns -> the oracle's output side, fed the device's zenith
angle.  Any difference in the GCM -> RRTM column preparation would change the
RRTMG results; any in the output side, the tendencies.  Tolerances: the
device zenith angle within 1e-12 of the oracle's (CUDA's sin/cos/tan/acos vs
the host's); against the all-CPU oracle (C++ RRTMG), the FP64 tendencies
within 1e-12 K/s and the fluxes within 1e-10 relative.
"""
import numpy as np
import pytest

from conftest import rel_err
from mima_gb300 import atmosphere as A
from mima_gb300 import rrtmg as R
from oracle import driver as D

pytestmark = pytest.mark.gpu

CASES = {
    "defaults": dict(),
    "lonstep4_zm_rad": dict(lonstep=4, do_zm_rad=1),
    "tracers_water_precip": dict(lonstep=2, do_zm_tracers=1, do_fixed_water=1, fixed_water_pres=30.0,
                                 fixed_water_lat=0.6, do_precip_albedo=1, num_precip=4, precip_lat=15.0),
    "secondary_instantaneous": dict(include_secondary_gases=1, ch4_val=1.8e-6, n2o_val=3.2e-7, o2_val=0.209,
                                    cfc11_val=2.5e-10, cfc12_val=5e-10, cfc22_val=1.5e-10, ccl4_val=1e-10,
                                    dt_rad_avg=0),
    "timeavg_dyofyr_slowdown": dict(dt_rad_avg=10800, use_dyofyr=1, slowdown_rad=0.7),
    "perpetual_no_ozone": dict(solday=172, dt_rad_avg=3600, o3_val=2e-7),
}
OUTS = ("tdt", "tdt_rad", "tdt_sw", "tdt_lw", "olr", "isr", "flux_sw", "flux_lw", "t_half")
SECONDS, DAYS = 30000, 200


def slab_for(case, seed):
    s = A.gcm_slab(64, 12, 40, seed=seed, ozone=(case != "perpetual_no_ozone"))
    s.t[5, 3, 8] = 80.0    # below temp_lower_limit
    s.q[7, 2, 4] = 1e-9    # below h2o_lower_limit
    return s


@pytest.mark.parametrize("precision", ["fp64", "split"])
@pytest.mark.parametrize("case", list(CASES))
def test_driver_bit_exact_chain(gpu, case, precision):
    slab = slab_for(case, 100 + len(case))
    prm = R.run_params(**CASES[case])
    gpu.set_precision(precision)
    try:
        out = gpu.run_rrtmg(prm, slab, SECONDS, DAYS)
        ref = D.run_rrtmg(None, prm, slab, SECONDS, DAYS, coszen=out["coszen"],
                          lw_sw=lambda atm: (gpu.lw(atm), gpu.sw(atm)))
    finally:
        gpu.set_precision("fp64")
    sec, day = D.model_time(prm, SECONDS, DAYS)
    cz = D.compute_zenith(prm, sec, day, 365, slab.lat, slab.lon)
    assert np.max(np.abs(out["coszen"] - cz)) <= 1e-12
    for k in OUTS:
        np.testing.assert_array_equal(out[k], ref[k], err_msg=k)


def test_driver_fp64_matches_cpu_oracle(gpu, orc):
    """The whole step against the all-CPU oracle (numpy driver + C++ RRTMG)."""
    slab = slab_for("defaults", 7)
    prm = R.run_params(lonstep=2, dt_rad_avg=10800)
    out = gpu.run_rrtmg(prm, slab, SECONDS, DAYS)
    ref = D.run_rrtmg(orc, prm, slab, SECONDS, DAYS)
    assert np.max(np.abs(out["coszen"] - ref["coszen"])) <= 1e-12
    for k in ("tdt", "tdt_rad", "tdt_sw", "tdt_lw"):
        assert np.max(np.abs(out[k] - ref[k])) < 1e-12, k
    for k in ("olr", "isr", "flux_sw", "flux_lw"):
        assert rel_err(out[k], ref[k], 1e-3) < 1e-10, k
    np.testing.assert_array_equal(out["t_half"], ref["t_half"])
    # the step does radiative work: OLR and SW heating are physical
    assert 100.0 < out["olr"].min() and out["olr"].max() < 400.0
    assert out["tdt_sw"].max() > 0.0


def test_driver_device_entry_matches_host_entry(gpu):
    torch = pytest.importorskip("torch")
    slab = slab_for("defaults", 9)
    prm = R.run_params(lonstep=2)
    host = gpu.run_rrtmg(prm, slab, SECONDS, DAYS)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    d = {k: dev(getattr(slab, k)) for k in R.RUN_IN if getattr(slab, k) is not None}
    out = {k: torch.empty(host[k].shape, dtype=torch.float64, device="cuda") for k in R.RUN_OUT}
    out["tdt"] = dev(slab.tdt.copy())
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        gpu.run_rrtmg_dev(s.cuda_stream, prm, slab.si, slab.sj, slab.sk, SECONDS, DAYS, 365, d, out)
    s.synchronize()
    assert gpu.sync_status(s.cuda_stream) == R.RRTMG_OK
    for k in R.RUN_OUT:
        np.testing.assert_array_equal(out[k].cpu().numpy(), host[k], err_msg=k)


def test_driver_argument_errors(gpu):
    slab = A.gcm_slab(30, 4, 10, seed=1)
    with pytest.raises(R.RRTMGError) as e:
        gpu.run_rrtmg(R.run_params(lonstep=4), slab, 0, 0)  # 30 longitudes, lonstep 4
    assert e.value.code == R.RRTMG_ERR_ARG
    with pytest.raises(R.RRTMGError) as e:
        gpu.run_rrtmg(R.run_params(dt_rad_avg=-1), slab, 0, 0)
    assert e.value.code == R.RRTMG_ERR_ARG
    slab.rrtm_precip = None
    with pytest.raises(R.RRTMGError) as e:
        gpu.run_rrtmg(R.run_params(do_precip_albedo=1, num_precip=2), slab, 0, 0)
    assert e.value.code == R.RRTMG_ERR_ARG
    # invalid state values are caught by the RRTM input validation
    bad = A.gcm_slab(16, 4, 10, seed=2)
    bad.p_full[3, 1, 0] = np.nan
    with pytest.raises(R.RRTMGError) as e:
        gpu.run_rrtmg(R.run_params(), bad, 0, 0)
    assert e.value.code == R.RRTMG_ERR_INPUT


@pytest.mark.parametrize("si,sj,case", [(256, 128, "lonstep4_zm_rad"), (512, 128, "tracers_water_precip"),
                                         (256, 128, "secondary_instantaneous")])
def test_driver_host_chunks_match_device_entry(gpu, si, sj, case):
    """rrtmg_run_c on page-locked arrays of 32768 and 65536 columns runs the
    slab in 2 and 4 latitude chunks alternating between two streams; its
    results equal rrtmg_run_dev's on the whole slab bit for bit.  One slab has
    its top interfaces above 0 Pa, so the slab-wide top-interface test the
    host makes for the chunks is checked both ways."""
    torch = pytest.importorskip("torch")
    slab = A.gcm_slab(si, sj, 40, seed=si + sj, ozone=True)
    if case == "secondary_instantaneous":
        slab.p_half[0] = 1.0  # every top interface at 1 Pa
    prm = R.run_params(**dict(CASES[case], lonstep=1))
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
    for k in R.RUN_IN:
        if getattr(slab, k) is not None:
            setattr(slab, k, pin(getattr(slab, k)))
    out = {}
    for k in R.RUN_OUT:
        shape = slab.p_half.shape if k == "t_half" else slab.tdt.shape if k.startswith("tdt") else slab.t_surf_rad.shape
        out[k] = pin(np.zeros(shape))
    out["tdt"][...] = slab.tdt
    gpu.set_precision("split")
    try:
        host = gpu.run_rrtmg(prm, slab, SECONDS, DAYS, out=out)
        dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
        d = {k: dev(getattr(slab, k)) for k in R.RUN_IN if getattr(slab, k) is not None}
        dout = {k: torch.empty(host[k].shape, dtype=torch.float64, device="cuda") for k in R.RUN_OUT}
        dout["tdt"] = dev(slab.tdt.copy())
        s = torch.cuda.Stream()
        with torch.cuda.stream(s):
            gpu.run_rrtmg_dev(s.cuda_stream, prm, slab.si, slab.sj, slab.sk, SECONDS, DAYS, 365, d, dout)
        s.synchronize()
    finally:
        gpu.set_precision("fp64")
    assert gpu.sync_status(s.cuda_stream) == R.RRTMG_OK
    for k in R.RUN_OUT:
        np.testing.assert_array_equal(dout[k].cpu().numpy(), host[k], err_msg=k)
    assert host["olr"].min() > 100.0
