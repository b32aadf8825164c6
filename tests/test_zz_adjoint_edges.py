"""The adjoint at the ends of the layer range: columns deeper than 64 layers
(the reverse sweeps' 208-level variants) and of 3 layers.  The FP64 Jacobians
against central differences of the analytic FP64 forward with the tolerances
of tests/test_gpu_adjoint.py; the VJP against cot^T J; the split VJP against
the FP64 VJP within bounds that catch a broken variant (the split adjoint's
FP32 error grows with depth; 40-layer columns meet 1e-4 at the 99th
percentile).  Collected after the adjoint, driver and parity test files."""
import numpy as np
import pytest

from mima_gb300 import atmosphere as A
from mima_gb300 import rrtmg as R
from test_gpu_adjoint import JAC_TOL, compare, fd_jacobian, off_knots

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("nlay", [3, 100])
def test_jacobian_matches_central_differences_at_the_ends(gpu, nlay):
    atm = off_knots(A.small_atmosphere(4, nlay, seed=90 + nlay))
    jac = gpu.jacobian(atm)
    fd, step, y0 = fd_jacobian(gpu, atm)
    err, kink = compare(jac, fd, step, y0)
    ok = ~kink
    print(f"\nnlay {nlay}: entries {err.size}, kink-masked {kink.mean():.2%}, max err {err[ok].max():.3e}")
    assert np.isfinite(jac).all()
    assert kink.mean() < 0.3
    assert err[ok].max() <= JAC_TOL


@pytest.mark.parametrize("nlay", [3, 100])
def test_vjp_and_split_adjoint_at_the_ends(gpu, nlay):
    atm = off_knots(A.small_atmosphere(4, nlay, seed=95 + nlay))
    nx, ny = R.adjoint_shape(nlay)
    cot = np.random.default_rng(nlay).standard_normal((ny, atm.ncol))
    j64 = gpu.jacobian(atm)
    g64 = gpu.vjp(atm, cot)
    ref = np.einsum("xrc,rc->xc", j64, cot)
    assert np.max(np.abs(g64 - ref)) <= 1e-10 * np.max(np.abs(ref))
    gpu.set_precision("split")
    try:
        g32 = gpu.vjp(atm, cot)
    finally:
        gpu.set_precision("fp64")
    assert np.isfinite(g32).all()
    err = np.abs(g32 - g64) / np.max(np.abs(g64), axis=1, keepdims=True)
    print(f"\nnlay {nlay}: split vs fp64 VJP: max {err.max():.2e}, 99% {np.quantile(err, 0.99):.2e}")
    assert np.quantile(err, 0.99) <= 1e-3
    assert err.max() <= 5e-2
