"""Adjoint (reverse-mode) Jacobians and vector-Jacobian products against
central finite differences of the analytic-transcendental FP64 forward:
T42 x 40 columns, dT = 0.01 K, dq = 1e-3 q.  Entries within a step of a kink
or jump of the forward (Planck-table and setcoef interpolation knots, eta
knots, the 0.06 optical-depth series switch, secdiff clamps) are detected by
disagreeing one-sided differences and left out; their count is reported."""
import numpy as np
import pytest

from mima_gb300 import atmosphere as A
from mima_gb300 import rrtmg as R

DT = 0.01          # K, tlay / tlev / tsfc step
DQ_REL = 1e-3      # relative q step
JAC_TOL = 1e-4     # relative tolerance of the Jacobian vs central differences
FLOOR = 1e-3       # entries below FLOOR * (largest entry of their row) compare absolutely


def replicate(atm, k):
    return atm.subset(np.tile(np.arange(atm.ncol), k))


STEPS = (1.0, 0.5, 0.25, 0.1)  # central differences at the configured step and fractions of it


def fd_jacobian(gpu, atm, chunk=16):
    """Central differences (len(STEPS), nx, ny, ncol) of the analytic FP64
    forward, the configured steps (nx, ncol) and the base rows (ny, ncol)."""
    L, n = atm.nlay, atm.ncol
    nx, ny = R.adjoint_shape(L)
    step = np.zeros((nx, n))
    step[:L] = DT
    step[L:2 * L] = DQ_REL * atm.h2o
    step[2 * L:] = DT
    fd = np.zeros((len(STEPS), nx, ny, n))
    gpu.set_precision("fp64")
    gpu.set_transcendentals("analytic")
    try:
        y0 = R.output_rows(gpu.lw(atm), gpu.sw(atm))
        for x0 in range(0, nx, chunk):
            xs = range(x0, min(nx, x0 + chunk))
            nb = 2 * len(STEPS)
            big = replicate(atm, nb * len(xs))
            for i, x in enumerate(xs):
                for k in range(nb):
                    h = (1.0 if k % 2 == 0 else -1.0) * STEPS[k // 2] * step[x]
                    sl = slice((nb * i + k) * n, (nb * i + k + 1) * n)
                    if x < L:
                        big.tlay[x, sl] += h
                    elif x < 2 * L:
                        big.h2o[x - L, sl] += h
                    elif x <= 3 * L:
                        big.tlev[x - 2 * L, sl] += h
                    else:
                        big.tsfc[sl] += h
            y = R.output_rows(gpu.lw(big), gpu.sw(big)).reshape(ny, len(xs), nb, n)
            for j, f in enumerate(STEPS):
                fd[j, x0:x0 + len(xs)] = ((y[:, :, 2 * j] - y[:, :, 2 * j + 1]) /
                                          (2 * f * step[x0:x0 + len(xs)][None])).transpose(1, 0, 2)
    finally:
        gpu.set_transcendentals("table")
    return fd, step, y0


def off_knots(atm, seed=3):
    """The columns with seeded 0.1-0.9 K offsets on every temperature.  The
    generator's isothermal 200 K stratosphere lies exactly on the 1 K knots of
    the Planck-table interpolation, where the forward has a kink at the point
    itself: every central difference there returns the mean of the two
    one-sided slopes, while the adjoint returns the slope of the branch the
    forward takes."""
    a = atm.subset(np.arange(atm.ncol))
    rng = np.random.default_rng(seed)
    a.tlay = a.tlay + rng.uniform(0.1, 0.9, a.tlay.shape)
    a.tlev = a.tlev + rng.uniform(0.1, 0.9, a.tlev.shape)
    a.tsfc = a.tsfc + rng.uniform(0.1, 0.9, a.tsfc.shape)
    return a


def compare(jac, fd, step, y0):
    """Relative errors against the central difference at the configured step,
    and the mask of entries that difference cannot judge: a kink or jump of
    the forward within the step (central differences at the three steps
    disagree) or a difference swamped by the forward's rounding."""
    d = fd[0]
    rowmax = np.max(np.abs(d), axis=0, keepdims=True)
    scale = np.maximum(np.abs(d), FLOOR * rowmax) + 1e-300
    bad = np.zeros(d.shape, bool)
    for j, f in enumerate(STEPS):
        noise = 1e-12 * np.maximum(np.abs(y0)[None], 1.0) / (f * step[:, None, :])
        if j == 0:
            bad |= noise > 0.1 * JAC_TOL * scale
        else:
            bad |= np.abs(d - fd[j]) > 0.25 * JAC_TOL * scale + noise
    err = np.abs(jac - d) / scale
    return err, bad


@pytest.fixture(scope="module")
def cfg3():
    """256 seeded T42 x 40 columns (the adjoint configuration), off the knots."""
    return off_knots(A.config_atmosphere(3))


@pytest.mark.gpu
def test_jacobian_matches_central_differences(gpu, cfg3):
    atm = cfg3
    jac = gpu.jacobian(atm)
    fd, step, y0 = fd_jacobian(gpu, atm)
    err, kink = compare(jac, fd, step, y0)
    fd, fd_half = fd[0], fd[1]
    ok = ~kink
    L = atm.nlay
    print(f"\nentries {err.size}, kink-masked {kink.sum()} ({kink.mean():.2%}), "
          f"max err unmasked {err[ok].max():.3e}, 99.9th pct {np.quantile(err[ok], 0.999):.3e}")
    for name, xs in (("tlay", slice(0, L)), ("q", slice(L, 2 * L)), ("tlev", slice(2 * L, 3 * L + 1)),
                     ("tsfc", slice(3 * L + 1, 3 * L + 2))):
        e = np.where(ok[xs], err[xs], 0)
        print(f"  {name:5s} max {e.max():.3e}")
    for name, rs in (("hr_lw", slice(0, L)), ("olr", slice(L, L + 1)), ("sfc_lw", slice(L + 1, L + 2)),
                     ("hr_sw", slice(L + 2, 2 * L + 2)), ("sfc_sw", slice(2 * L + 2, 2 * L + 3))):
        e = np.where(ok[:, rs], err[:, rs], 0)
        print(f"  row {name:6s} max {e.max():.3e}")
    worst = np.argsort(np.where(ok, err, 0).ravel())[-8:]
    for w in worst:
        x, r, c = np.unravel_index(w, err.shape)
        print(f"  x={x} r={r} c={c} err={err[x, r, c]:.2e} jac={jac[x, r, c]:.6e} fd={fd[x, r, c]:.6e} "
              f"half={fd_half[x, r, c]:.6e} y0={y0[r, c]:.4e} step={step[x, c]:.3e}")
    assert kink.mean() < 0.15
    assert err[ok].max() <= JAC_TOL


@pytest.mark.gpu
def test_vjp_equals_cotangent_times_jacobian(gpu, cfg3):
    atm = cfg3.subset(np.arange(32))
    jac = gpu.jacobian(atm)
    nx, ny = R.adjoint_shape(atm.nlay)
    cot = np.random.default_rng(5).standard_normal((ny, atm.ncol))
    grad = gpu.vjp(atm, cot)
    ref = np.einsum("xrc,rc->xc", jac, cot)
    assert np.max(np.abs(grad - ref)) <= 1e-10 * np.max(np.abs(ref))


class RadiationFn:
    """torch.autograd.Function over the C-ABI, for the tests only: forward is
    the analytic FP64 LW+SW forward (rows of R.output_rows), backward the
    adjoint's vector-Jacobian product."""

    @staticmethod
    def build(gpu, atm):
        import torch

        class Fn(torch.autograd.Function):
            @staticmethod
            def forward(ctx, tlay, q, tlev, tsfc):
                a = atm.subset(np.arange(atm.ncol))
                a.tlay, a.h2o = tlay.detach().cpu().numpy().copy(), q.detach().cpu().numpy().copy()
                a.tlev, a.tsfc = tlev.detach().cpu().numpy().copy(), tsfc.detach().cpu().numpy().copy()
                ctx.atm = a
                gpu.set_transcendentals("analytic")
                try:
                    y = R.output_rows(gpu.lw(a), gpu.sw(a))
                finally:
                    gpu.set_transcendentals("table")
                return torch.from_numpy(y).to(tlay.device)

            @staticmethod
            def backward(ctx, gy):
                a, L = ctx.atm, ctx.atm.nlay
                g = torch.from_numpy(gpu.vjp(a, gy.detach().cpu().numpy())).to(gy.device)
                return g[:L], g[L:2 * L], g[2 * L:3 * L + 1], g[3 * L + 1]

        return Fn


@pytest.mark.gpu
def test_autograd_function_backward_is_the_adjoint(gpu, cfg3):
    import torch
    atm = cfg3.subset(np.arange(16))
    Fn = RadiationFn.build(gpu, atm)
    t = lambda a: torch.tensor(a, dtype=torch.float64, device="cuda", requires_grad=True)
    tlay, q, tlev, tsfc = t(atm.tlay), t(atm.h2o), t(atm.tlev), t(atm.tsfc)
    y = Fn.apply(tlay, q, tlev, tsfc)
    w = torch.randn_like(y)
    gl, gq, gv, gs = torch.autograd.grad((w * y).sum(), (tlay, q, tlev, tsfc))
    jac = gpu.jacobian(atm)
    L = atm.nlay
    ref = np.einsum("xrc,rc->xc", jac, w.cpu().numpy())
    got = np.concatenate([gl.cpu().numpy(), gq.cpu().numpy(), gv.cpu().numpy(), gs.cpu().numpy()[None]])
    assert np.max(np.abs(got - ref)) <= 1e-10 * np.max(np.abs(ref))


@pytest.mark.gpu
def test_olr_surface_temperature_derivative_matches_idrv(gpu, cfg3):
    """d OLR / d tsfc against the reference's own idrv = 1 derivative
    (rrtmg_lw_rtrnmr.f90:628-745), which uses the separately tabulated
    totplnkderiv, hence the 2 % tolerance."""
    atm = cfg3.subset(np.arange(32))
    L = atm.nlay
    jac = gpu.jacobian(atm)
    out = gpu.lw(atm, idrv=1)
    np.testing.assert_allclose(jac[3 * L + 1, L], out["duflx_dt"][L], rtol=2e-2)


@pytest.mark.gpu
def test_jacobian_against_oracle_differences(gpu, cfg3, orc):
    """Central differences of the FP64 C++ restatement (analytic mode) at small
    steps, where two step sizes agree, for a sample of entries."""
    atm = cfg3.subset(np.array([0, 101, 202]))
    L = atm.nlay
    jac = gpu.jacobian(atm)
    rng = np.random.default_rng(11)
    xs = np.concatenate([rng.choice(L, 4, replace=False), L + rng.choice(L, 4, replace=False),
                         2 * L + rng.choice(L + 1, 3, replace=False), [3 * L + 1]])
    orc.set_table_mode(False)
    try:
        checked = 0
        for c in range(atm.ncol):
            col = atm.subset(np.array([c]))
            for x in xs:
                def rows(h):
                    a = col.subset(np.array([0]))
                    if x < L:
                        a.tlay[x, 0] += h
                    elif x < 2 * L:
                        a.h2o[x - L, 0] += h
                    elif x <= 3 * L:
                        a.tlev[x - 2 * L, 0] += h
                    else:
                        a.tsfc[0] += h
                    return R.output_rows(orc.rrtmg_lw(a), orc.rrtmg_sw(a))[:, 0]
                base = 1e-4 * col.h2o[x - L, 0] if L <= x < 2 * L else 2e-3
                d1 = (rows(base) - rows(-base)) / (2 * base)
                d2 = (rows(base / 2) - rows(-base / 2)) / base
                scale = np.maximum(np.abs(d1), FLOOR * np.abs(d1).max()) + 1e-300
                ok = np.abs(d1 - d2) <= 2e-5 * scale
                err = np.abs(jac[x, :, c] - d1) / scale
                assert np.all(err[ok] <= JAC_TOL), (c, x, err[ok].max())
                checked += ok.sum()
        assert checked > 0.8 * len(xs) * atm.ncol * (2 * L + 3)
    finally:
        orc.set_table_mode(True)


@pytest.mark.gpu
def test_split_adjoint_against_fp64_adjoint(gpu, cfg3):
    """FP32/FP64-split adjoint (FP32 dual numbers and reverse sweeps, FP64 sums)
    against the FP64 adjoint, relative to each row's scale as above."""
    gpu.set_precision("fp64")
    j64 = gpu.jacobian(cfg3)
    gpu.set_precision("split")
    try:
        j32 = gpu.jacobian(cfg3)
    finally:
        gpu.set_precision("fp64")
    rowmax = np.max(np.abs(j64), axis=0, keepdims=True)
    err = np.abs(j32 - j64) / (np.maximum(np.abs(j64), FLOOR * rowmax) + 1e-300)
    print(f"\nsplit vs fp64 Jacobian: max {err.max():.2e}, 99.9% {np.quantile(err, 0.999):.2e}, "
          f"99% {np.quantile(err, 0.99):.2e}")
    assert np.isfinite(j32).all()
    assert np.quantile(err, 0.99) <= 1e-4
    assert np.quantile(err, 0.999) <= 1e-3
    assert err.max() <= 1e-2


@pytest.mark.gpu
def test_split_vjp_against_split_jacobian_and_fp64_vjp(gpu, cfg3):
    """The split VJP (its own lean reverse: layer cotangents contracted with
    tangents recomputed at the end) equals cot^T J of the split Jacobian to
    FP32 rounding, and the FP64 VJP to the accuracy of the split adjoint."""
    atm = cfg3.subset(np.arange(64))
    nx, ny = R.adjoint_shape(atm.nlay)
    cot = np.random.default_rng(8).standard_normal((ny, atm.ncol))
    g64 = gpu.vjp(atm, cot)
    gpu.set_precision("split")
    try:
        j32 = gpu.jacobian(atm)
        g32 = gpu.vjp(atm, cot)
    finally:
        gpu.set_precision("fp64")
    ref = np.einsum("xrc,rc->xc", j32, cot)
    scale = np.max(np.abs(ref), axis=1, keepdims=True)  # per input kind and layer
    assert np.isfinite(g32).all()
    assert np.max(np.abs(g32 - ref) / scale) <= 1e-4
    err = np.abs(g32 - g64) / np.max(np.abs(g64), axis=1, keepdims=True)
    print(f"\nsplit vs fp64 VJP: max {err.max():.2e}, 99% {np.quantile(err, 0.99):.2e}")
    assert np.quantile(err, 0.99) <= 1e-4
    assert err.max() <= 1e-2
