"""The oracle's tangent-linear model (dual numbers through the FP64 restatement of the reference's
SLIC step, fixed time steps) against central finite differences of its own forward, and its value
part against the plain oracle sweeps: this pins the derivative that the GPU adjoint is checked
against."""
import numpy as np
import pytest

import cases


def forward_loss(oracle, p, target, dx, dts, lim, bc):
    """1/2 sum (rho_T - target)^2 from plain oracle sweeps (X(dt/2) Y(dt) X(dt/2) in 2D)."""
    q = p.copy()
    for dt in dts:
        if q.ndim == 2:
            q = oracle.sweep(0, q, 0, 2, dx, dt, 0.0, lim, 1.4, bc)
        else:
            q = oracle.sweep(0, q, 0, 2, dx, 0.5 * dt, 0.0, lim, 1.4, bc)
            q = oracle.sweep(0, q, 1, 2, dx, dt, 0.0, lim, 1.4, bc)
            q = oracle.sweep(0, q, 0, 2, dx, 0.5 * dt, 0.0, lim, 1.4, bc)
    e = (q[..., 0] - target).ravel()
    L = 0.0
    for v in 0.5 * (e * e):  # cell order, like the oracle's accumulation
        L = L + float(v)
    return L, q


@pytest.mark.parametrize("dims", [1, 2])
@pytest.mark.parametrize("lim", [0, 1, 2])
@pytest.mark.parametrize("bc", [0, 1])
def test_oracle_tlm_matches_finite_differences(oracle, dims, lim, bc):
    shape = (24,) if dims == 1 else (10, 12)
    p0 = cases.smooth_state(shape, 3 + lim)
    target = cases.smooth_state(shape, 11)[..., 0]
    dx = 1.0 / shape[-1]
    dts = np.full(6, 0.15 * dx)
    L_plain, _ = forward_loss(oracle, p0, target, dx, dts, lim, bc)
    rng = np.random.default_rng(dims * 10 + lim + 100 * bc)
    for _ in range(3):
        d = rng.standard_normal(p0.shape)
        L0, dL = oracle.tlm_newton(p0, d, target, dx, dts, 0.0, lim, 1.4, bc)
        assert L0 == L_plain  # the dual numbers' value part is the plain FP64 forward
        h = 1e-7  # the map is piecewise smooth (limiter branches, the 1e-5 clamp): keep the step small
        Lp, _ = oracle.tlm_newton(p0 + h * d, np.zeros_like(d), target, dx, dts, 0.0, lim, 1.4, bc)
        Lm, _ = oracle.tlm_newton(p0 - h * d, np.zeros_like(d), target, dx, dts, 0.0, lim, 1.4, bc)
        fd = (Lp - Lm) / (2 * h)
        assert abs(fd - dL) <= 1e-6 * abs(dL) + 1e-10, (fd, dL)


def sr_smooth_state(shape, seed):
    """Smooth periodic special-relativistic data (|v| <= 0.36, rho and p near 1)."""
    rng = np.random.default_rng(seed)
    x = np.linspace(0, 1, shape[-1], endpoint=False)
    ph = rng.uniform(0, 2 * np.pi, 4)
    s = np.zeros(shape + (5,))
    s[..., 0] = 1.0 + 0.2 * np.sin(2 * np.pi * x + ph[0])
    s[..., 1] = 0.3 * np.sin(2 * np.pi * x + ph[1])
    s[..., 4] = 1.0 + 0.1 * np.cos(2 * np.pi * x + ph[3])
    if len(shape) == 2:
        y = np.linspace(0, 1, shape[0], endpoint=False)[:, None]
        s[..., 2] = 0.2 * np.cos(2 * np.pi * y + ph[2]) + 0.0 * x
        s[..., 0] += 0.1 * np.sin(2 * np.pi * y)
    return s


def sr_forward_loss(oracle, p, target, dx, dts, lim, bc, g):
    q = p.copy()
    for dt in dts:
        if q.ndim == 2:
            q = oracle.sweep(1, q, 0, 2, dx, dt, 0.0, lim, g, bc)
        else:
            q = oracle.sweep(1, q, 0, 2, dx, 0.5 * dt, 0.0, lim, g, bc)
            q = oracle.sweep(1, q, 1, 2, dx, dt, 0.0, lim, g, bc)
            q = oracle.sweep(1, q, 0, 2, dx, 0.5 * dt, 0.0, lim, g, bc)
    e = (q[..., 0] - target).ravel()
    L = 0.0
    for v in 0.5 * (e * e):
        L = L + float(v)
    return L


@pytest.mark.parametrize("dims", [1, 2])
@pytest.mark.parametrize("lim", [0, 1, 2])
@pytest.mark.parametrize("bc", [0, 1])
def test_oracle_sr_tlm_matches_finite_differences(oracle, dims, lim, bc):
    """The special-relativistic tangent-linear model (dual numbers through every primitive
    recovery's Newton iteration): value part = the plain SR forward, derivative = central
    differences (h = 1e-7: larger steps leave the reference's 1e-5 slope clamp on rows where a field
    is constant)."""
    g = 5.0 / 3.0
    shape = (24,) if dims == 1 else (10, 12)
    p0 = sr_smooth_state(shape, 3 + lim)
    target = sr_smooth_state(shape, 11)[..., 0]
    dx = 1.0 / shape[-1]
    dts = np.full(5, 0.15 * dx)
    L_plain = sr_forward_loss(oracle, p0, target, dx, dts, lim, bc, g)
    rng = np.random.default_rng(dims * 10 + lim + 100 * bc)
    for _ in range(2):
        d = rng.standard_normal(p0.shape)
        L0, dL = oracle.tlm_sr(p0, d, target, dx, dts, 0.0, lim, g, bc)
        assert L0 == L_plain
        h = 1e-7
        Lp, _ = oracle.tlm_sr(p0 + h * d, np.zeros_like(d), target, dx, dts, 0.0, lim, g, bc)
        Lm, _ = oracle.tlm_sr(p0 - h * d, np.zeros_like(d), target, dx, dts, 0.0, lim, g, bc)
        fd = (Lp - Lm) / (2 * h)
        assert abs(fd - dL) <= 1e-6 * abs(dL) + 1e-10, (fd, dL)


def gr_smooth_state(shape, seed):
    """Gentle data for the black-hole scheme (|v| <= 0.15, p near 0.5, varying along both axes).  The
    reference's GR half-step evolution drives faster flows superluminal at the grid edges within a
    few steps; this stays physical over the test's steps."""
    rng = np.random.default_rng(seed)
    ph = rng.uniform(0, 2 * np.pi, 5)
    x = np.linspace(0, 1, shape[-1], endpoint=False)
    s = np.zeros(shape + (5,))
    s[..., 0] = 1.0 + 0.2 * np.sin(2 * np.pi * x + ph[0])
    s[..., 1] = 0.1 * np.cos(2 * np.pi * x + ph[1])
    s[..., 4] = 0.5 + 0.05 * np.sin(4 * np.pi * x + ph[3])
    if len(shape) == 2:
        y = np.linspace(0, 1, shape[0], endpoint=False)[:, None]
        s[..., 0] += 0.1 * np.sin(2 * np.pi * y + ph[4])
        s[..., 2] = 0.05 * np.cos(2 * np.pi * y + ph[2]) + 0.0 * x
        s[..., 4] += 0.03 * np.cos(2 * np.pi * y + ph[2])
    return s


def gr_forward_loss(oracle, p, target, dx, dts, lim, g, bh):
    q = p.copy()
    for dt in dts:
        if q.ndim == 2:
            q = oracle.sweep(2, q, 0, 2, dx, dt, 0.0, lim, g, bh=bh)
        else:
            q = oracle.sweep(2, q, 0, 2, dx, 0.5 * dt, 0.0, lim, g, bh=bh)
            q = oracle.sweep(2, q, 1, 2, dx, dt, 0.0, lim, g, bh=bh)
            q = oracle.sweep(2, q, 0, 2, dx, 0.5 * dt, 0.0, lim, g, bh=bh)
    e = (q[..., 0] - target).ravel()
    L = 0.0
    for v in 0.5 * (e * e):
        L = L + float(v)
    return L


@pytest.mark.parametrize("dims,bh", [(1, (0.05, 0.0, 0.5, 0.0, 0.0)), (2, (0.05, 0.0, 0.5, 0.5, 0.0)),
                                     (2, (0.08, 0.6, 0.4, 0.6, 0.0))])
@pytest.mark.parametrize("lim", [0, 1, 2])
def test_oracle_gr_tlm_matches_finite_differences(oracle, dims, bh, lim):
    """The black-hole flux step's tangent-linear model (no source terms; the hole excises cells on
    the grid): value part = the plain GR sweeps, derivative = central differences (fields vary along
    both axes, so no neighbour difference grows out of zero through the 1e-5 slope clamp)."""
    g = 5.0 / 3.0
    shape = (24,) if dims == 1 else (10, 12)
    p0 = gr_smooth_state(shape, 5 + lim)
    target = gr_smooth_state(shape, 13)[..., 0]
    dx = 1.0 / shape[-1]
    dts = np.full(4, 0.1 * dx)
    L_plain = gr_forward_loss(oracle, p0, target, dx, dts, lim, g, bh)
    rng = np.random.default_rng(dims * 10 + lim)
    for _ in range(2):
        d = rng.standard_normal(p0.shape)
        L0, dL = oracle.tlm_gr(p0, d, target, dx, dts, 0.0, lim, g, bh)
        assert L0 == L_plain
        h = 1e-7
        Lp, _ = oracle.tlm_gr(p0 + h * d, np.zeros_like(d), target, dx, dts, 0.0, lim, g, bh)
        Lm, _ = oracle.tlm_gr(p0 - h * d, np.zeros_like(d), target, dx, dts, 0.0, lim, g, bh)
        fd = (Lp - Lm) / (2 * h)
        assert abs(fd - dL) <= 1e-6 * abs(dL) + 1e-10, (fd, dL)


def gr_step_loss(oracle, p, target, dx, dts, lim, g, bh, sub):
    """Plain oracle forward of the black-hole step: `sub` RK source half-steps, the flux sweeps, `sub` more."""
    q = p.copy()
    for dt in dts:
        for _ in range(sub):
            q = oracle.rk_source(q, dx, 0.5 * (dt / sub), 0.0, 1, g, bh)
        if q.ndim == 2:
            q = oracle.sweep(2, q, 0, 2, dx, dt, 0.0, lim, g, bh=bh)
        else:
            q = oracle.sweep(2, q, 0, 2, dx, 0.5 * dt, 0.0, lim, g, bh=bh)
            q = oracle.sweep(2, q, 1, 2, dx, dt, 0.0, lim, g, bh=bh)
            q = oracle.sweep(2, q, 0, 2, dx, 0.5 * dt, 0.0, lim, g, bh=bh)
        for _ in range(sub):
            q = oracle.rk_source(q, dx, 0.5 * (dt / sub), 0.0, 1, g, bh)
    e = (q[..., 0] - target).ravel()
    L = 0.0
    for v in 0.5 * (e * e):
        L = L + float(v)
    return L


@pytest.mark.parametrize("dims,bh", [(1, (0.05, 0.0, 0.5, 0.0, 0.0)), (2, (0.05, 0.0, 0.5, 0.5, 0.0)),
                                     (2, (0.08, 0.6, 0.4, 0.6, 0.0))])
@pytest.mark.parametrize("sub", [1, 2])
@pytest.mark.parametrize("lim", [0, 1, 2])
def test_oracle_gr_source_tlm_matches_finite_differences(oracle, dims, bh, sub, lim):
    """The whole black-hole step with its RK source half-steps (the source term, the fractional
    flux evolutions inside each RK stage) in dual numbers: value part = the plain oracle forward;
    derivative = central differences.  Near the horizon the map is stiff: at one step size a
    central difference may cross a limiter branch or lose digits to rounding, so the best of three
    step sizes must agree to 1e-6 (measured: 3e-9 to 2.3e-7)."""
    g = 5.0 / 3.0
    shape = (24,) if dims == 1 else (10, 12)
    p0 = gr_smooth_state(shape, 5 + lim)
    target = gr_smooth_state(shape, 13)[..., 0]
    dx = 1.0 / shape[-1]
    dts = np.full(3, 0.1 * dx)
    d = np.random.default_rng(sub * 10 + lim + dims).standard_normal(p0.shape)
    L0, dL = oracle.tlm_gr(p0, d, target, dx, dts, 0.0, lim, g, bh, sub)
    assert L0 == gr_step_loss(oracle, p0, target, dx, dts, lim, g, bh, sub)
    err = []
    for h in (1e-6, 1e-7, 1e-8):
        Lp, _ = oracle.tlm_gr(p0 + h * d, np.zeros_like(d), target, dx, dts, 0.0, lim, g, bh, sub)
        Lm, _ = oracle.tlm_gr(p0 - h * d, np.zeros_like(d), target, dx, dts, 0.0, lim, g, bh, sub)
        err.append(abs((Lp - Lm) / (2 * h) - dL) / abs(dL))
    assert min(err) <= 1e-6, err
