"""Seeded synthetic states shared by the golden-fixture generator and the tests.

Shapes and value ranges follow the benchmark configurations: Newtonian states with
rho in [0.1, 1.5], |u|, |v| <= 1, p in [0.03, 1.5]; SR states with |v| well below 1; GR states
around a Schwarzschild/Kerr hole with some cells inside the excision radius.
"""
import numpy as np

SYS_GAMMA = {0: 1.4, 1: 5.0 / 3.0, 2: 5.0 / 3.0}


def newton_state(rng, shape, vz=0.2):
    p = np.zeros(tuple(shape) + (5,))
    p[..., 0] = rng.uniform(0.1, 1.5, shape)
    p[..., 1] = rng.uniform(-1.0, 1.0, shape)
    p[..., 2] = rng.uniform(-1.0, 1.0, shape)
    p[..., 3] = rng.uniform(-vz, vz, shape)
    p[..., 4] = rng.uniform(0.03, 1.5, shape)
    return p


def sr_state(rng, shape):
    p = np.zeros(tuple(shape) + (5,))
    p[..., 0] = rng.uniform(0.5, 2.0, shape)
    p[..., 1] = rng.uniform(-0.4, 0.4, shape)
    p[..., 2] = rng.uniform(-0.4, 0.4, shape)
    p[..., 3] = rng.uniform(-0.1, 0.1, shape)
    p[..., 4] = rng.uniform(0.1, 1.5, shape)
    return p


def sr_mild_state(rng, shape):
    """SR states with moderate cell-to-cell jumps: every slope-extrapolated state stays physical
    (positive pressure, (tau + D)^2 > |S|^2) under all three limiters."""
    p = np.zeros(tuple(shape) + (5,))
    p[..., 0] = rng.uniform(0.8, 1.25, shape)
    p[..., 1] = rng.uniform(-0.3, 0.3, shape)
    p[..., 2] = rng.uniform(-0.3, 0.3, shape)
    p[..., 3] = rng.uniform(-0.05, 0.05, shape)
    p[..., 4] = rng.uniform(0.8, 1.25, shape)
    return p


def gr_state(rng, shape):
    p = np.zeros(tuple(shape) + (5,))
    p[..., 0] = rng.uniform(0.5, 1.5, shape)
    p[..., 1] = rng.uniform(-0.2, 0.2, shape)
    p[..., 2] = rng.uniform(-0.2, 0.2, shape)
    p[..., 3] = rng.uniform(-0.05, 0.05, shape)
    p[..., 4] = rng.uniform(0.05, 0.5, shape)
    return p


def state(system, rng, shape):
    return {0: newton_state, 1: sr_state, 2: gr_state}[system](rng, shape)


def sod(n=1000):
    """Sod shock tube (Tests/EulerTests.cpp:3-30): left (1, 0, 1) for i <= n/2, right (0.125, 0, 0.1)."""
    p = np.zeros((n, 5))
    for i in range(n):
        p[i] = (1.0, 0.0, 0.0, 0.0, 1.0) if i <= 0.5 * n else (0.125, 0.0, 0.0, 0.0, 0.1)
    return p


def four_quadrant(n, seed):
    """2D four-quadrant Riemann problem, per-quadrant (rho, u, v, p) drawn by seed."""
    rng = np.random.default_rng(seed)
    q = np.zeros((4, 5))
    q[:, 0] = rng.uniform(0.1, 1.5, 4)
    q[:, 1] = rng.uniform(-1.0, 1.0, 4)
    q[:, 2] = rng.uniform(-1.0, 1.0, 4)
    q[:, 4] = rng.uniform(0.03, 1.5, 4)
    p = np.zeros((n, n, 5))
    h = n // 2
    p[:h, :h] = q[0]
    p[:h, h:] = q[1]
    p[h:, :h] = q[2]
    p[h:, h:] = q[3]
    return p


# GR test hole: a Schwarzschild (and a spinning) hole inside a unit box, so that a small grid has
# excised cells, stencils crossing the horizon and plain cells.
GR_BH = (0.1, 0.0, 0.5, 0.5, 0.0)
GR_BH_SPIN = (0.1, 0.9, 0.47, 0.52, 0.0)


def riemann(shape, seed):
    """Seeded Riemann problem on a 1D (nx,) or 2D (ny, nx) grid: two states split at the middle
    in 1D, four quadrants in 2D, each (rho, u, v, p) drawn like four_quadrant's."""
    rng = np.random.default_rng(seed)
    q = np.zeros((4, 5))
    q[:, 0] = rng.uniform(0.1, 1.5, 4)
    q[:, 1] = rng.uniform(-1.0, 1.0, 4)
    q[:, 2] = rng.uniform(-1.0, 1.0, 4)
    q[:, 4] = rng.uniform(0.03, 1.5, 4)
    p = np.zeros(tuple(shape) + (5,))
    if len(shape) == 1:
        h = shape[0] // 2
        p[:h], p[h:] = q[0], q[1]
        return p
    hy, hx = shape[0] // 2, shape[1] // 2
    p[:hy, :hx], p[:hy, hx:], p[hy:, :hx], p[hy:, hx:] = q[0], q[1], q[2], q[3]
    return p


def batch_shapes(count=256, lo=128, hi=2048, seed=5):
    """Grid shapes of the batched workload: half 1D, half 2D (by seed), every side drawn
    log-uniform from [lo, hi] cells."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        side = lambda: int(round(float(np.exp(rng.uniform(np.log(lo), np.log(hi))))))  # noqa: E731
        out.append((side(),) if rng.random() < 0.5 else (side(), side()))
    return out


def smooth_state(shape, seed):
    """Smooth periodic Newtonian state (sines of random phase), for derivative checks by finite
    differences: no limiter branch lies within a small perturbation of most cells."""
    rng = np.random.default_rng(seed)
    nx = shape[-1]
    ny = shape[0] if len(shape) == 2 else 1
    x = (np.arange(nx) + 0.5) / nx
    y = (np.arange(ny) + 0.5) / ny
    X, Y = np.meshgrid(x, y)
    ph = rng.uniform(0, 2 * np.pi, 6)
    p = np.zeros((ny, nx, 5))
    p[..., 0] = 1.0 + 0.3 * np.sin(2 * np.pi * X + ph[0]) * np.cos(2 * np.pi * Y + ph[1])
    p[..., 1] = 0.3 * np.sin(2 * np.pi * (X + Y) + ph[2])
    p[..., 2] = 0.2 * np.cos(2 * np.pi * X + ph[3]) if len(shape) == 2 else 0.0
    p[..., 3] = 0.05 * np.sin(2 * np.pi * Y + ph[4])
    p[..., 4] = 1.0 + 0.2 * np.cos(2 * np.pi * X + ph[5])
    return p.reshape(tuple(shape) + (5,))


def kelvin_helmholtz(n, seed, width=0.01, amp=0.01, modes=2):
    """Special-relativistic Kelvin-Helmholtz shear layers on the periodic unit square: a band
    0.25 < y < 0.75 with vx = +0.5 and rho = 2 inside, vx = -0.5 and rho = 1 outside, joined by
    tanh profiles of the given width; p = 1; vy = amp * sin(2 pi modes x + phase), phase by seed.
    The Lorentz factor stays below 1.16."""
    rng = np.random.default_rng(seed)
    phase = rng.uniform(0.0, 2.0 * np.pi)
    x = (np.arange(n) + 0.5) / n
    y = (np.arange(n) + 0.5) / n
    X, Y = np.meshgrid(x, y)
    s = np.tanh((Y - 0.25) / width) - np.tanh((Y - 0.75) / width) - 1.0
    p = np.zeros((n, n, 5))
    p[..., 0] = 1.5 + 0.5 * s
    p[..., 1] = 0.5 * s
    p[..., 2] = amp * np.sin(2.0 * np.pi * modes * X + phase)
    p[..., 4] = 1.0
    return p
