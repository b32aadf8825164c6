"""The allocation-free LW entry point ``rrtmg_lw_dev_static`` (scratch in the
library's static device array) against the workspace-owning ``rrtmg_lw_dev``,
through the C-ABI, on two calls in a row with different inputs and sizes.

Collected last so that it runs both after every other GPU test and, on its
own, in a fresh process."""
import ctypes as C

import numpy as np
import pytest

from mima_gb300 import atmosphere as A
from mima_gb300 import rrtmg as R

FLUX_TOL = 1e-10   # relative, as for the FP64 parity tests
HR_TOL = 1e-8      # K/day relative with a 1e-3 K/day floor


def _close(got, ref, key):
    floor = 1e-3 if key.startswith("hr") else 1e-6
    tol = HR_TOL if key.startswith("hr") else FLUX_TOL
    err = np.max(np.abs(got - ref) / np.maximum(np.abs(ref), floor))
    assert err <= tol, (key, err)


@pytest.mark.gpu
def test_static_scratch_entry_point_matches_dev_entry_point(gpu):
    import torch
    gpu.set_precision("fp64")
    cases = [(A.small_atmosphere(300, 40, seed=41), 0), (A.small_atmosphere(257, 60, seed=42, ts_sigma=5.0), 1)]
    s = torch.cuda.Stream()
    # every device buffer exists before the first call, so that device memory
    # seen after the set-up call is the library's alone
    bufs = []
    for atm, idrv in cases:
        d = R.atm_device_inputs(atm)
        ref, _ = R.device_outputs(atm.ncol, atm.nlay, idrv=idrv)
        got, _ = R.device_outputs(atm.ncol, atm.nlay, idrv=idrv)
        for t in got.values():
            t.fill_(float("nan"))
        bufs.append((atm, idrv, d, ref, got))
    torch.cuda.synchronize()
    free = []
    for atm, idrv, d, ref, got in bufs:
        with torch.cuda.stream(s):
            gpu.rrtmg_lw_dev(s.cuda_stream, atm.ncol, atm.nlay, 0, idrv, d, ref)
        s.synchronize()
        free.append(torch.cuda.mem_get_info()[0])
        with torch.cuda.stream(s):
            gpu.rrtmg_lw_dev_static(s.cuda_stream, atm.ncol, atm.nlay, 0, idrv, d, got)
        assert gpu.sync_status(s.cuda_stream) == R.RRTMG_OK
        free.append(torch.cuda.mem_get_info()[0])
        for k in ref:
            _close(got[k].cpu().numpy(), ref[k].cpu().numpy(), k)
    # the second static call (after the first call's one-time set-up) changed
    # no device allocation
    assert free[3] == free[2], free


@pytest.mark.gpu
def test_static_scratch_entry_point_split_precision(gpu):
    """The FP32-split path reads the same static array as FP32 fields.  After a
    larger FP64 call has left its data in the array, split calls through
    rrtmg_lw_dev_static give rrtmg_lw_dev's split results bit for bit (two
    calls in a row, different sizes, idrv 1 then 0)."""
    import torch
    s = torch.cuda.Stream()
    big = A.small_atmosphere(1500, 40, seed=44)
    d = R.atm_device_inputs(big)
    out, _ = R.device_outputs(big.ncol, big.nlay, idrv=1)
    gpu.set_precision("fp64")
    with torch.cuda.stream(s):
        gpu.rrtmg_lw_dev_static(s.cuda_stream, big.ncol, big.nlay, 0, 1, d, out)
    s.synchronize()
    gpu.set_precision("split")
    try:
        for atm, idrv in ((A.small_atmosphere(700, 40, seed=45), 1), (A.small_atmosphere(333, 60, seed=46), 0)):
            d = R.atm_device_inputs(atm)
            ref, _ = R.device_outputs(atm.ncol, atm.nlay, idrv=idrv)
            got, _ = R.device_outputs(atm.ncol, atm.nlay, idrv=idrv)
            for t in got.values():
                t.fill_(float("nan"))
            with torch.cuda.stream(s):
                gpu.rrtmg_lw_dev(s.cuda_stream, atm.ncol, atm.nlay, 0, idrv, d, ref)
                gpu.rrtmg_lw_dev_static(s.cuda_stream, atm.ncol, atm.nlay, 0, idrv, d, got)
            assert gpu.sync_status(s.cuda_stream) == R.RRTMG_OK
            for k in ref:
                assert torch.equal(got[k], ref[k]), k
    finally:
        gpu.set_precision("fp64")


@pytest.mark.gpu
def test_static_scratch_entry_point_rejects_sizes_beyond_the_limit(gpu):
    import torch
    nlay = 40
    # LW scratch per column: indices, 25 fields, Planck terms by layer and level, three band-partial
    # arrays of 20 rows (the split path's slots), surface terms, laytrop, column sums
    per_col = (4 * nlay + 8 * 25 * nlay + 8 * 16 * nlay + 8 * 16 * (nlay + 1) + 3 * 8 * 20 * (nlay + 1)
               + 3 * 8 * 16 + 4 + 2 * 8 * nlay)
    ncol = R.STATIC_SCRATCH_BYTES // per_col + 64
    atm = A.small_atmosphere(ncol, nlay, seed=43)
    d = R.atm_device_inputs(atm)
    out, _ = R.device_outputs(ncol, nlay)
    with pytest.raises(R.RRTMGError) as e:
        gpu.rrtmg_lw_dev_static(0, ncol, nlay, 0, 0, d, out)
    assert e.value.code == R.RRTMG_ERR_ARG
    assert "static limit" in gpu.lib.rrtmg_gpu_last_error(gpu._h).decode()
    torch.cuda.synchronize()
