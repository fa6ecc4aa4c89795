"""The relativistic sweep adjoint's cell function (the body of the device kernel), built for the
host, against the oracle's tangent-linear models: forward sweeps by the oracle, the sweep adjoints
in reverse by the host build, and <grad, d> against the tangent model's directional derivative
along random d -- the SR sweep (`tlm_sr`) and the black-hole flux sweep with excision (`tlm_gr`).
The storage copy in between is padded with NaN, so this also checks that every cell reads only its
stencil."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT
from test_oracle_adjoint import gr_smooth_state, sr_smooth_state

G = 5.0 / 3.0
HOLES = [(0.05, 0.0, 0.5, 0.5, 0.0), (0.08, 0.6, 0.4, 0.6, 0.0)]


@pytest.fixture(scope="module")
def host_adjoint(tmp_path_factory):
    so = str(tmp_path_factory.mktemp("radj") / "librel_host.so")
    subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-shared", "-fPIC",
                    os.path.join(ROOT, "tests", "cpp", "rel_adjoint_host.cpp"), "-o", so], check=True)
    lib = ctypes.CDLL(so)
    d, i, p = ctypes.c_double, ctypes.c_int, ctypes.c_void_p
    lib.rel_host_sweep_adjoint.argtypes = [i, i, p, p, p, i, i, i, i, d, p, d, d, d, i]
    lib.rel_host_sweep_adjoint.restype = i
    lib.rel_host_rk_adjoint.argtypes = [i, p, p, p, i, i, d, p, d, d]
    lib.rel_host_rk_adjoint.restype = i

    def run(system, state, pbar_out, axis, bc, dx, dt, bias, lim, bh=None):
        s = np.ascontiguousarray(state, dtype=np.float64)
        po = np.ascontiguousarray(pbar_out, dtype=np.float64)
        out = np.empty_like(s)
        ny, nx = (1, s.shape[0]) if s.ndim == 2 else s.shape[:2]
        hole = None if bh is None else np.ascontiguousarray(bh, dtype=np.float64)
        rc = lib.rel_host_sweep_adjoint(system, s.ndim - 1, s.ctypes.data, po.ctypes.data, out.ctypes.data, ny, nx,
                                        axis, bc, G, None if hole is None else hole.ctypes.data, dx, dt, bias, lim)
        assert rc == 0
        return out

    def rk(state, pbar_out, dx, dt, bh):
        s = np.ascontiguousarray(state, dtype=np.float64)
        po = np.ascontiguousarray(pbar_out, dtype=np.float64)
        out = np.empty_like(s)
        ny, nx = (1, s.shape[0]) if s.ndim == 2 else s.shape[:2]
        hole = np.ascontiguousarray(bh, dtype=np.float64)
        assert lib.rel_host_rk_adjoint(s.ndim - 1, s.ctypes.data, po.ctypes.data, out.ctypes.data, ny, nx, G,
                                       hole.ctypes.data, dx, dt) == 0
        return out
    run.rk = rk
    return run


def ops_of(dims, dts, sub=0):
    """(axis, dt) of every operation in order: X(dt) per 1D step, X(dt/2) Y(dt) X(dt/2) per 2D step,
    with `sub` black-hole RK source half-steps (axis None, dt / (2 sub)) before and after."""
    out = []
    for dt in dts:
        rk = [(None, 0.5 * (dt / sub))] * sub if sub else []
        out += rk + ([(0, dt)] if dims == 1 else [(0, 0.5 * dt), (1, dt), (0, 0.5 * dt)]) + rk
    return out


def reverse_gradient(oracle, adj, system, p0, target, dx, dts, bias, lim, bc, bh=None, sub=0):
    seq = ops_of(p0.ndim - 1, dts, sub)
    inputs, q = [], p0.copy()
    for axis, dt in seq:
        inputs.append(q)
        if axis is None:
            q = oracle.rk_source(q, dx, dt, 0.0, 1, G, bh)
        else:
            q = oracle.sweep(system, q, axis, 2, dx, dt, bias, lim, G, bc, bh=bh)
    pbar = np.zeros_like(q)
    pbar[..., 0] = q[..., 0] - target
    for (axis, dt), s in zip(reversed(seq), reversed(inputs)):
        if axis is None:
            pbar = adj.rk(s, pbar, dx, dt, bh)
        else:
            pbar = adj(system, s, pbar, axis, bc, dx, dt, bias, lim, bh)
    return pbar


def check_directions(grad, tlm, shape, seed, n=3):
    rng = np.random.default_rng(seed)
    for _ in range(n):
        d = rng.standard_normal(shape)
        dL = tlm(d)
        got = float(np.sum(grad * d))
        assert abs(got - dL) <= 1e-10 * max(1.0, abs(dL)), (got, dL)


@pytest.mark.parametrize("dims", [1, 2])
@pytest.mark.parametrize("lim", [0, 1, 2])
@pytest.mark.parametrize("bc,bias", [(0, 0.0), (1, 0.0), (0, 0.4)])
def test_sr_sweep_adjoint_matches_tangent_model(oracle, host_adjoint, dims, lim, bc, bias):
    shape = (20,) if dims == 1 else (8, 10)
    p0 = sr_smooth_state(shape, 3 + lim)
    target = sr_smooth_state(shape, 11)[..., 0]
    dx = 1.0 / shape[-1]
    dts = np.full(3, 0.15 * dx)
    grad = reverse_gradient(oracle, host_adjoint, 1, p0, target, dx, dts, bias, lim, bc)
    assert np.isfinite(grad).all()
    check_directions(grad, lambda d: oracle.tlm_sr(p0, d, target, dx, dts, bias, lim, G, bc)[1], p0.shape,
                     dims * 100 + lim * 10 + bc)


@pytest.mark.parametrize("shape", [(2,), (3,), (4,), (2, 5), (4, 3), (3, 2)])
@pytest.mark.parametrize("bc", [0, 1])
def test_sr_sweep_adjoint_tiny_lines(oracle, host_adjoint, shape, bc):
    """Lines of two to four cells: the mirror reaches past the far end and the periodic wrap
    aliases one cell into several window positions (each counted once per output cell)."""
    p0 = sr_smooth_state(shape, 6)
    target = sr_smooth_state(shape, 12)[..., 0]
    dx = 1.0 / shape[-1]
    dts = np.full(3, 0.1 * dx)
    grad = reverse_gradient(oracle, host_adjoint, 1, p0, target, dx, dts, 0.0, 1, bc)
    check_directions(grad, lambda d: oracle.tlm_sr(p0, d, target, dx, dts, 0.0, 1, G, bc)[1], p0.shape,
                     len(shape) * 10 + shape[0] + bc)


@pytest.mark.parametrize("dims,bh", [(1, (0.05, 0.0, 0.5, 0.0, 0.0))] + [(2, h) for h in HOLES])
@pytest.mark.parametrize("lim", [0, 1, 2])
def test_gr_sweep_adjoint_matches_tangent_model(oracle, host_adjoint, dims, bh, lim):
    """The black-hole flux sweeps around holes that excise cells of the grid (those cells, and the
    cells whose stencil reaches them, keep their state and pass their adjoint through)."""
    shape = (24,) if dims == 1 else (10, 12)
    p0 = gr_smooth_state(shape, 5 + lim)
    target = gr_smooth_state(shape, 13)[..., 0]
    dx = 1.0 / shape[-1]
    dts = np.full(3, 0.1 * dx)
    grad = reverse_gradient(oracle, host_adjoint, 2, p0, target, dx, dts, 0.0, lim, 0, bh)
    assert np.isfinite(grad).all()
    check_directions(grad, lambda d: oracle.tlm_gr(p0, d, target, dx, dts, 0.0, lim, G, bh)[1], p0.shape,
                     dims * 10 + lim)


@pytest.mark.parametrize("dims,bh", [(1, (0.05, 0.0, 0.5, 0.0, 0.0))] + [(2, h) for h in HOLES])
@pytest.mark.parametrize("sub", [1, 2])
@pytest.mark.parametrize("lim", [0, 1])
def test_gr_step_adjoint_with_source_matches_tangent_model(oracle, host_adjoint, dims, bh, sub, lim):
    """The whole black-hole step: `sub` RK source half-steps (source term, fractional evolutions in
    each RK stage, excision) around the flux sweeps."""
    shape = (24,) if dims == 1 else (10, 12)
    p0 = gr_smooth_state(shape, 5 + lim)
    target = gr_smooth_state(shape, 13)[..., 0]
    dx = 1.0 / shape[-1]
    dts = np.full(2, 0.1 * dx)
    grad = reverse_gradient(oracle, host_adjoint, 2, p0, target, dx, dts, 0.0, lim, 0, bh, sub)
    assert np.isfinite(grad).all()
    check_directions(grad, lambda d: oracle.tlm_gr(p0, d, target, dx, dts, 0.0, lim, G, bh, sub)[1], p0.shape,
                     dims * 10 + sub * 3 + lim, n=2)


def test_gr_sweep_adjoint_passes_excised_cells_through(oracle, host_adjoint):
    """A cell of the excision region keeps its state: its input adjoint is its output adjoint."""
    bh = HOLES[0]
    p = gr_smooth_state((10, 12), 4)
    dx = 1.0 / 12
    pbar = np.random.default_rng(2).standard_normal(p.shape)
    for axis in (0, 1):
        got = host_adjoint(2, p, pbar, axis, 0, dx, 0.1 * dx, 0.0, 1, bh)
        # cell (6, 6) sits on the hole; its neighbours within two cells are frozen too, so the
        # adjoint of (6, 6) receives nothing but its own
        assert np.array_equal(got[6, 6], pbar[6, 6])


def test_sr_sweep_adjoint_is_local(oracle, host_adjoint):
    """A unit output adjoint at one cell reaches exactly the five cells of its window."""
    p = sr_smooth_state((9, 12), 4)
    dx = 1.0 / 12
    for axis in (0, 1):
        pbar = np.zeros_like(p)
        pbar[4, 6, 0] = 1.0
        got = host_adjoint(1, p, pbar, axis, 0, dx, 0.1 * dx, 0.0, 1)
        hit = np.argwhere(np.abs(got).sum(-1) > 0)
        exp = [(4, 6 + t) if axis == 0 else (4 + t, 6) for t in range(-2, 3)]
        assert sorted(map(tuple, hit)) == sorted(exp)
