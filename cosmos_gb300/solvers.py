"""Reference-named host API over the C ABI.

Mirrors the reference's static solver classes (Solvers/*.hpp) with the same method names and
argument meaning, on numpy arrays of primitive states: shape (nx, 5) for 1D and (ny, nx, 5) for
2D with (rho, vx, vy, vz, p) per cell -- the reference's vector<StateVector> /
vector<vector<StateVector>> indexed [row i = y][column j = x].

  * solve / solve2D return a new array (the reference returns grids by value);
  * the per-sweep functions (computeSLICTimeStep, computeXSLICTimeStep2D, ...) update the array
    in place (the reference takes vector& and mutates it);
  * every call runs on the GPU through libcosmos_gb300.so; extra keyword arguments select the
    precision (FP64 reproduces the reference bit for bit; FP32 is the Newtonian bulk path) and
    the boundary (transmissive as in the reference, or periodic).
"""
import ctypes
import sys
import threading

import numpy as np

from . import _lib
from ._lib import SPACETIME_WIDTH  # noqa: F401
from ._lib import (BC_PERIODIC, BC_TRANSMISSIVE, FP32, FP64, GR, NEWTONIAN, SR, Params, SolveOpts,  # noqa: F401
                   SolveResult, check, load)

_tls = threading.local()


class EulerMaterialParameters:
    """Euler/EulerMaterialParameters.cpp:3-21 (default adiabatic index 1.0)."""

    def __init__(self, adiabaticIndex=1.0):
        self.adiabaticIndex = float(adiabaticIndex)

    def setAdiabaticIndex(self, g):
        self.adiabaticIndex = float(g)

    def getAdiabaticIndex(self):
        return self.adiabaticIndex


class BlackHoleSpacetime:
    """BlackHoleEuler/BlackHoleSpacetime.cpp:3-52 constructors: (), (M), (M, x, y, z), (M, a),
    (M, a, x, y, z); defaults M = 1, a = 0, position (0.5, 0.5, 0)."""

    def __init__(self, *args):
        m, a, x, y, z = 1.0, 0.0, 0.5, 0.5, 0.0
        if len(args) == 1:
            m = args[0]
        elif len(args) == 2:
            m, a = args
        elif len(args) == 4:
            m, x, y, z = args
        elif len(args) == 5:
            m, a, x, y, z = args
        elif len(args) != 0:
            raise TypeError("BlackHoleSpacetime takes 0, 1, 2, 4 or 5 arguments")
        self.mass, self.spin, self.x, self.y, self.z = map(float, (m, a, x, y, z))

    def getBlackHoleMass(self):
        return self.mass

    def getBlackHoleSpin(self):
        return self.spin

    def getBlackHoleXPosition(self):
        return self.x

    def getBlackHoleYPosition(self):
        return self.y

    def getBlackHoleZPosition(self):
        return self.z

    def setBlackHoleMass(self, v):
        self.mass = float(v)

    def setBlackHoleSpin(self, v):
        self.spin = float(v)

    def setBlackHoleXPosition(self, v):
        self.x = float(v)

    def setBlackHoleYPosition(self, v):
        self.y = float(v)

    def setBlackHoleZPosition(self, v):
        self.z = float(v)

    # ---- the metric (BlackHoleEuler/BlackHoleSpacetime.hpp:16-42), evaluated on the device
    # (cosmos_spacetime_eval, bit for bit with the reference); coordinates may be arrays
    def record(self, x, y, z, cellSpacing=1.0, ctx=None):
        """Every public quantity at the points (x, y, z): array (..., 125) in the layout of the
        COSMOS_ST_* offsets; the derivative entries use cellSpacing."""
        xb, yb, zb = np.broadcast_arrays(*(np.asarray(v, dtype=np.float64) for v in (x, y, z)))
        q = np.ascontiguousarray(np.stack([xb, yb, zb], axis=-1).reshape(-1, 3))
        p = Params()
        load().cosmos_params_default(ctypes.byref(p))
        p.system, p.dx = GR, float(cellSpacing)
        p.bh_mass, p.bh_spin, p.bh_x, p.bh_y, p.bh_z = self.mass, self.spin, self.x, self.y, self.z
        out = np.empty((q.shape[0], SPACETIME_WIDTH))
        check(load().cosmos_spacetime_eval((ctx or default_context()).h, ctypes.byref(p), q.shape[0],
                                           q.ctypes.data, out.ctypes.data))
        return out.reshape(xb.shape + (SPACETIME_WIDTH,))

    def _part(self, at, shape, x, y, z, h=1.0):
        r = self.record(x, y, z, h)[..., at:at + int(np.prod(shape))]
        r = r.reshape(r.shape[:-1] + shape)
        return float(r) if np.ndim(x) == 0 and shape == () else r

    def computeKerrSchildScalar(self, x, y, z):
        return self._part(0, (), x, y, z)

    def computeKerrSchildVector(self, x, y, z):
        return self._part(1, (3,), x, y, z)

    def computeKerrSchildSpacetimeVector(self, x, y, z):
        return self._part(4, (4,), x, y, z)

    def computeKerrSchildScalarDerivative(self, x, y, z, cellSpacing):
        return self._part(8, (3,), x, y, z, cellSpacing)

    def computeKerrSchildVectorDerivative(self, x, y, z, cellSpacing):
        return self._part(11, (3, 3), x, y, z, cellSpacing)

    def computeSpatialMetricTensor(self, x, y, z):
        return self._part(20, (3, 3), x, y, z)

    def computeSpacetimeMetricTensor(self, x, y, z):
        return self._part(29, (4, 4), x, y, z)

    def computeInverseSpatialMetricTensor(self, x, y, z):
        return self._part(45, (3, 3), x, y, z)

    def computeInverseSpacetimeMetricTensor(self, x, y, z):
        return self._part(54, (4, 4), x, y, z)

    def computeSpatialMetricDeterminant(self, x, y, z):
        return self._part(70, (), x, y, z)

    def computeSpacetimeMetricDeterminant(self, x, y, z):
        return self._part(71, (), x, y, z)

    def computeSpatialMetricTensorDerivative(self, x, y, z, cellSpacing):
        return self._part(72, (3, 3, 3), x, y, z, cellSpacing)

    def computeLapseFunction(self, x, y, z):
        return self._part(99, (), x, y, z)

    def computeShiftVector(self, x, y, z):
        return self._part(100, (3,), x, y, z)

    def computeLapseFunctionDerivative(self, x, y, z, cellSpacing):
        return self._part(103, (3,), x, y, z, cellSpacing)

    def computeShiftVectorDerivative(self, x, y, z, cellSpacing):
        return self._part(106, (3, 3), x, y, z, cellSpacing)

    def computeExtrinsicCurvatureTensor(self, x, y, z, cellSpacing):
        return self._part(115, (3, 3), x, y, z, cellSpacing)

    def inExcisionRegion(self, x, y, z):
        """BlackHoleEuler/BlackHoleSpacetime.cpp:372-386, on the host (no device call)."""
        r = np.sqrt((np.asarray(x) - self.x) ** 2 + (np.asarray(y) - self.y) ** 2 + (np.asarray(z) - self.z) ** 2)
        e = r <= self.mass * (1.0 + np.sqrt(1.0 - self.spin * self.spin))
        return bool(e) if np.ndim(e) == 0 else e


class Context:
    """A CUDA stream on one device (cosmos_ctx)."""

    def __init__(self, device=0):
        L = load()
        h = ctypes.c_void_p()
        check(L.cosmos_ctx_create(device, ctypes.byref(h)))
        self.h = h

    def synchronize(self):
        check(load().cosmos_ctx_synchronize(self.h))

    @property
    def stream(self):
        return load().cosmos_ctx_stream(self.h)

    def close(self):
        if self.h and not sys.is_finalizing():
            load().cosmos_ctx_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def set_tensor_maps(enable):
    """FP32 sweeps stage rows through TMA tensor maps (True, the default) or one copy per field
    (False); results are bit-identical.  Read when a sweep is launched or captured and when a batch
    is created.  Returns the previous setting."""
    return bool(load().cosmos_set_tensor_maps(1 if enable else 0))


def default_context():
    c = getattr(_tls, "ctx", None)
    if c is None:
        c = _tls.ctx = Context(0)
    return c


class Grid:
    """A device-resident grid (cosmos_grid)."""

    def __init__(self, system, shape, dx, gamma, precision=FP64, boundary=BC_TRANSMISSIVE, black_hole=None,
                 ctx=None, sr_c2p64_above=2.0):
        self.ctx = ctx or default_context()
        p = Params()
        load().cosmos_params_default(ctypes.byref(p))
        p.sr_c2p64_above = float(sr_c2p64_above)
        p.system = system
        if len(shape) == 1:
            p.dims, p.nx, p.ny = 1, shape[0], 1
        else:
            p.dims, p.ny, p.nx = 2, shape[0], shape[1]
        p.precision, p.boundary, p.gamma, p.dx = precision, boundary, float(gamma), float(dx)
        if black_hole is not None:
            p.bh_mass, p.bh_spin = black_hole.mass, black_hole.spin
            p.bh_x, p.bh_y, p.bh_z = black_hole.x, black_hole.y, black_hole.z
        self.params = p
        self.shape = tuple(shape)
        h = ctypes.c_void_p()
        check(load().cosmos_grid_create(self.ctx.h, ctypes.byref(p), ctypes.byref(h)))
        self.h = h

    @property
    def ncell(self):
        return int(np.prod(self.shape))

    def set_prim(self, prim):
        a = np.ascontiguousarray(prim, dtype=np.float64)
        if a.shape != self.shape + (5,):
            raise ValueError(f"expected shape {self.shape + (5,)}, got {a.shape}")
        check(load().cosmos_grid_set_prim(self.h, a.ctypes.data, a.size))

    def get_prim(self, out=None):
        o = np.empty(self.shape + (5,), dtype=np.float64) if out is None else out
        check(load().cosmos_grid_get_prim(self.h, o.ctypes.data, o.size))
        return o

    def sweep(self, axis, order, dt, bias, limiter):
        check(load().cosmos_grid_sweep(self.h, axis, order, float(dt), float(bias), int(limiter)))

    def rk_source(self, dt, bias, limiter):
        check(load().cosmos_grid_rk_source(self.h, float(dt), float(bias), int(limiter)))

    def max_wavespeed(self):
        v = ctypes.c_double()
        check(load().cosmos_grid_max_wavespeed(self.h, ctypes.byref(v)))
        return v.value

    def stable_dt(self, cfl, t, t_final, iteration):
        v = ctypes.c_double()
        check(load().cosmos_grid_stable_dt(self.h, float(cfl), float(t), float(t_final), int(iteration),
                                           ctypes.byref(v)))
        return v.value

    @staticmethod
    def opts(order, cfl, t_final, bias, limiter, subcycles=1, max_steps=-1):
        o = SolveOpts()
        o.order, o.cfl, o.t_final, o.bias = int(order), float(cfl), float(t_final), float(bias)
        o.limiter, o.subcycles, o.max_steps = int(limiter), int(subcycles), int(max_steps)
        return o

    def solve(self, order, cfl, t_final, bias, limiter, subcycles=1, max_steps=-1):
        o = self.opts(order, cfl, t_final, bias, limiter, subcycles, max_steps)
        r = SolveResult()
        check(load().cosmos_grid_solve(self.h, ctypes.byref(o), ctypes.byref(r)))
        return r

    def run_begin(self, order, cfl, t_final, bias, limiter, subcycles=1, max_steps=-1):
        o = self.opts(order, cfl, t_final, bias, limiter, subcycles, max_steps)
        check(load().cosmos_grid_run_begin(self.h, ctypes.byref(o)))

    def run_steps(self, n):
        check(load().cosmos_grid_run_steps(self.h, int(n)))

    def run_end(self):
        r = SolveResult()
        check(load().cosmos_grid_run_end(self.h, ctypes.byref(r)))
        return r

    def field_sums(self):
        o = np.zeros(5)
        check(load().cosmos_grid_field_sums(self.h, o.ctypes.data))
        return o

    def set_adjoint_keep(self, nbytes):
        """Device bytes adjoint() may use to keep sweep inputs from its forward pass (the last
        checkpoint segments that fit are not recomputed); -1: half the free device memory (the
        default), 0: the last segment only.  The gradient does not depend on it."""
        check(load().cosmos_grid_set_adjoint_keep(self.h, int(nbytes)))

    def adjoint(self, target, nsteps, cfl, bias, limiter, checkpoint_every=10, dts=None, subcycles=1):
        """Gradient of L = 1/2 sum (rho_T - target)^2 after `nsteps` SLIC steps from the current
        state with respect to its primitives (dt of each step held fixed: `dts` if given, else the
        CFL rule's).  Black-hole grids take `subcycles` RK source half-steps before and after each
        flux step (0: the flux step alone).  Returns (loss, grad with the shape of get_prim(), dts,
        (forward_ms, backward_ms)).  The grid holds the final state afterwards."""
        tgt = np.ascontiguousarray(target, dtype=np.float64)
        if tgt.shape != self.shape:
            raise ValueError(f"target must have shape {self.shape}, got {tgt.shape}")
        o = self.opts(2, cfl, 1e300, bias, limiter, int(subcycles), nsteps)
        grad = np.empty(self.shape + (5,), dtype=np.float64)
        dts_out = np.empty(int(nsteps), dtype=np.float64)
        din = None if dts is None else np.ascontiguousarray(dts, dtype=np.float64)
        if din is not None and din.size < nsteps:
            raise ValueError("dts must hold nsteps entries")
        loss = ctypes.c_double()
        ms = np.zeros(2)
        check(load().cosmos_grid_adjoint(self.h, ctypes.byref(o), int(nsteps), int(checkpoint_every), tgt.ctypes.data,
                                         None if din is None else din.ctypes.data, grad.ctypes.data,
                                         ctypes.byref(loss), dts_out.ctypes.data, ms.ctypes.data))
        return loss.value, grad, dts_out, (float(ms[0]), float(ms[1]))

    def amr_flags(self, tol, coarse=None, fine=None):
        nc = self.ncell
        nf = nc * (4 if len(self.shape) == 2 else 2)
        c = np.ones(nc, np.uint8) if coarse is None else np.ascontiguousarray(coarse, np.uint8).reshape(-1).copy()
        f = np.zeros(nf, np.uint8) if fine is None else np.ascontiguousarray(fine, np.uint8).reshape(-1).copy()
        check(load().cosmos_grid_amr_flags(self.h, float(tol), c.ctypes.data, f.ctypes.data))
        return c, f

    def amr_derefine(self, fine_grid, tol, coarse, fine):
        c = np.ascontiguousarray(coarse, np.uint8).reshape(-1).copy()
        f = np.ascontiguousarray(fine, np.uint8).reshape(-1).copy()
        check(load().cosmos_grid_amr_derefine(self.h, fine_grid.h, float(tol), c.ctypes.data, f.ctypes.data))
        return c, f

    def close(self):
        # at interpreter exit the process releases the device; no native teardown then
        if getattr(self, "h", None) and not sys.is_finalizing():
            load().cosmos_grid_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """Many independent Newtonian grids of uneven sizes advanced by one persistent launch
    (cosmos_batch).  `shapes` holds one entry per grid: (nx,) for 1D, (ny, nx) for 2D; each grid
    keeps its own dt and step count, as if the reference's solve / solve2D ran on it alone."""

    def __init__(self, shapes, dx, gamma, precision=FP32, boundary=BC_TRANSMISSIVE, ctx=None):
        self.ctx = ctx or default_context()
        self.shapes = [tuple(int(v) for v in s) for s in shapes]
        n = len(self.shapes)
        dxs = np.broadcast_to(np.asarray(dx, dtype=np.float64), (n,)).copy()
        dims = np.array([len(s) for s in self.shapes], dtype=np.int32)
        nx = np.array([s[-1] for s in self.shapes], dtype=np.int32)
        ny = np.array([s[0] if len(s) == 2 else 1 for s in self.shapes], dtype=np.int32)
        h = ctypes.c_void_p()
        check(load().cosmos_batch_create(self.ctx.h, n, dims.ctypes.data, nx.ctypes.data, ny.ctypes.data,
                                         dxs.ctypes.data, float(gamma), int(boundary), int(precision),
                                         ctypes.byref(h)))
        self.h = h
        self.dx = dxs

    def __len__(self):
        return len(self.shapes)

    @property
    def cells(self):
        c = ctypes.c_longlong()
        check(load().cosmos_batch_size(self.h, None, ctypes.byref(c)))
        return c.value

    def set_prim(self, k, prim):
        a = np.ascontiguousarray(prim, dtype=np.float64)
        if a.shape != self.shapes[k] + (5,):
            raise ValueError(f"grid {k}: expected shape {self.shapes[k] + (5,)}, got {a.shape}")
        check(load().cosmos_batch_set_prim(self.h, int(k), a.ctypes.data, a.size))

    def get_prim(self, k, out=None):
        o = np.empty(self.shapes[k] + (5,), dtype=np.float64) if out is None else out
        check(load().cosmos_batch_get_prim(self.h, int(k), o.ctypes.data, o.size))
        return o

    def run_begin(self, cfl, t_final, bias, limiter, max_steps=-1):
        o = Grid.opts(2, cfl, t_final, bias, limiter, 1, max_steps)
        check(load().cosmos_batch_run_begin(self.h, ctypes.byref(o)))

    def run_steps(self, n):
        check(load().cosmos_batch_run_steps(self.h, int(n)))

    def run_end(self):
        r = (SolveResult * len(self.shapes))()
        check(load().cosmos_batch_run_end(self.h, r))
        return list(r)

    def set_wait_limit(self, polls):
        """Bound each grid-barrier wait to `polls` polls of about 64 ns (0: the default, about 4 s);
        takes effect at the next run_begin."""
        check(load().cosmos_batch_set_wait_limit(self.h, int(polls)))

    def set_shape(self, threads, rows, cap=0):
        check(load().cosmos_batch_set_shape(self.h, int(threads), int(rows), int(cap)))

    def time_shape(self, threads, rows, cap=0, steps=3):
        ms = ctypes.c_double()
        check(load().cosmos_batch_time_shape(self.h, int(threads), int(rows), int(cap), int(steps), ctypes.byref(ms)))
        return ms.value

    def autotune(self, cache_path=None):
        """Times every tile shape (threads, rows, cap), keeps the fastest; returns it and its ms/step."""
        nt, seg, cap, ms = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_double()
        path = cache_path.encode() if cache_path else None
        check(load().cosmos_batch_autotune(self.h, path, ctypes.byref(nt), ctypes.byref(seg), ctypes.byref(cap),
                                           ctypes.byref(ms)))
        return (nt.value, seg.value, cap.value), ms.value

    def close(self):
        # at interpreter exit the process releases the device; no native teardown then
        if getattr(self, "h", None) and not sys.is_finalizing():
            load().cosmos_batch_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _shape(cells):
    a = np.asarray(cells)
    if a.ndim == 2 and a.shape[1] == 5:
        return (a.shape[0],)
    if a.ndim == 3 and a.shape[2] == 5:
        return (a.shape[0], a.shape[1])
    raise ValueError("cells must have shape (nx, 5) or (ny, nx, 5)")


def _solve(system, cells, dx, cfl, t_final, bias, lim, mp, order, bh=None, subcycles=1, precision=FP64,
           boundary=BC_TRANSMISSIVE, max_steps=-1):
    g = Grid(system, _shape(cells), dx, mp.getAdiabaticIndex(), precision, boundary, bh)
    try:
        g.set_prim(cells)
        r = g.solve(order, cfl, t_final, bias, lim, subcycles, max_steps)
        out = g.get_prim()
    finally:
        g.close()
    out_steps = r.steps
    return out, out_steps


def _sweep_inplace(system, cells, dx, dt, axis, order, bias, lim, mp, bh=None, precision=FP64,
                   boundary=BC_TRANSMISSIVE):
    g = Grid(system, _shape(cells), dx, mp.getAdiabaticIndex(), precision, boundary, bh)
    try:
        g.set_prim(cells)
        g.sweep(axis, order, dt, bias, lim)
        cells[...] = g.get_prim()
    finally:
        g.close()


def _family(system, name):
    """Build the First/SecondOrderSolver and Solvers classes of one system."""
    bh_kw = system == GR

    class SecondOrder:
        __qualname__ = f"{name}SecondOrderSolver"

        @staticmethod
        def solve(initialCells, cellSpacing, CFLCoefficient, finalTime, bias, slopeLimiter, *rest, **kw):
            sub, mp, bh = _unpack(rest, bh_kw)
            return _solve(system, initialCells, cellSpacing, CFLCoefficient, finalTime, bias, slopeLimiter, mp, 2,
                          bh, sub, **kw)[0]

        solve2D = solve

        @staticmethod
        def computeSLICTimeStep(currentCells, cellSpacing, timeStep, bias, slopeLimiter, *rest, **kw):
            _, mp, bh = _unpack(rest, bh_kw, has_sub=False)
            _sweep_inplace(system, currentCells, cellSpacing, timeStep, 0, 2, bias, slopeLimiter, mp, bh, **kw)

        computeXSLICTimeStep2D = computeSLICTimeStep

        @staticmethod
        def computeYSLICTimeStep2D(currentCells, cellSpacing, timeStep, bias, slopeLimiter, *rest, **kw):
            _, mp, bh = _unpack(rest, bh_kw, has_sub=False)
            _sweep_inplace(system, currentCells, cellSpacing, timeStep, 1, 2, bias, slopeLimiter, mp, bh, **kw)

    class FirstOrder:
        __qualname__ = f"{name}FirstOrderSolver"

        @staticmethod
        def solve(initialCells, cellSpacing, CFLCoefficient, finalTime, *rest, **kw):
            sub, mp, bh = _unpack(rest, bh_kw)
            return _solve(system, initialCells, cellSpacing, CFLCoefficient, finalTime, 0.0, 1, mp, 1, bh, sub,
                          **kw)[0]

        solve2D = solve

        @staticmethod
        def computeFORCETimeStep(currentCells, cellSpacing, timeStep, *rest, **kw):
            _, mp, bh = _unpack(rest, bh_kw, has_sub=False)
            _sweep_inplace(system, currentCells, cellSpacing, timeStep, 0, 1, 0.0, 1, mp, bh, **kw)

        computeXFORCETimeStep2D = computeFORCETimeStep

        @staticmethod
        def computeYFORCETimeStep2D(currentCells, cellSpacing, timeStep, *rest, **kw):
            _, mp, bh = _unpack(rest, bh_kw, has_sub=False)
            _sweep_inplace(system, currentCells, cellSpacing, timeStep, 1, 1, 0.0, 1, mp, bh, **kw)

    class Utilities:
        __qualname__ = f"{name}Solvers"

        @staticmethod
        def computeMaximumWaveSpeed(currentCells, materialParameters, blackHole=None, **kw):
            g = Grid(system, _shape(currentCells), 1.0, materialParameters.getAdiabaticIndex(), black_hole=blackHole,
                     **kw)
            try:
                g.set_prim(currentCells)
                return g.max_wavespeed()
            finally:
                g.close()

        computeMaximumWaveSpeed2D = computeMaximumWaveSpeed

        @staticmethod
        def computeStableTimeStep(*args, **kw):
            if len(args) == 4:  # (timeStep, currentTime, finalTime, currentIteration)
                return load().cosmos_stable_dt_rule(*map(float, args[:3]), int(args[3]))
            cells, dx, cfl, t, tf, it, mp = args[:7]
            bh = args[7] if len(args) > 7 else None
            g = Grid(system, _shape(cells), dx, mp.getAdiabaticIndex(), black_hole=bh, **kw)
            try:
                g.set_prim(cells)
                return g.stable_dt(cfl, t, tf, it)
            finally:
                g.close()

        computeStableTimeStep2D = computeStableTimeStep

    return SecondOrder, FirstOrder, Utilities


def _unpack(rest, gr, has_sub=True):
    """Positional tail after the common arguments: Newtonian/SR (materialParameters); GR
    ([subcyclingIterations,] materialParameters, blackHole)."""
    if not gr:
        return 1, rest[0], None
    if has_sub:
        return int(rest[0]), rest[1], rest[2]
    return 1, rest[0], rest[1]


EulerSecondOrderSolver, EulerFirstOrderSolver, EulerSolvers = _family(NEWTONIAN, "Euler")
RelativisticEulerSecondOrderSolver, RelativisticEulerFirstOrderSolver, RelativisticEulerSolvers = _family(
    SR, "RelativisticEuler")
BlackHoleEulerSecondOrderSolver, BlackHoleEulerFirstOrderSolver, BlackHoleEulerSolvers = _family(GR, "BlackHoleEuler")


class BlackHoleEulerForcingSolver:
    """Solvers/BlackHoleEulerForcingSolver.hpp: RK4 source step (in place)."""

    @staticmethod
    def computeRungeKuttaTimeStep(currentCells, cellSpacing, timeStep, bias, slopeLimiter, materialParameters,
                                  blackHole):
        g = Grid(GR, _shape(currentCells), cellSpacing, materialParameters.getAdiabaticIndex(), black_hole=blackHole)
        try:
            g.set_prim(currentCells)
            g.rk_source(timeStep, bias, slopeLimiter)
            currentCells[...] = g.get_prim()
        finally:
            g.close()

    computeRungeKuttaTimeStep2D = computeRungeKuttaTimeStep


def solve_with_steps(system, cells, dx, cfl, t_final, bias, limiter, gamma, order=2, black_hole=None, subcycles=1,
                     precision=FP64, boundary=BC_TRANSMISSIVE, max_steps=-1):
    """solve() that also returns the step count (the reference prints it per step)."""
    return _solve(system, cells, dx, cfl, t_final, bias, limiter, EulerMaterialParameters(gamma), order, black_hole,
                  subcycles, precision, boundary, max_steps)


class AMR:
    """A device-resident AMR hierarchy (cosmos_amr) with one flag per cell (Newtonian or SR,
    transmissive boundaries): levels=1 is the Level-1 driver (a coarse grid of `shape` and its 2x
    refinement), levels=2 the Level-2 driver (coarse, 2x intermediate, 4x fine)."""

    def __init__(self, system, shape, dx, gamma, precision=FP64, ctx=None, sr_c2p64_above=2.0, levels=1):
        self.ctx = ctx or default_context()
        p = Params()
        load().cosmos_params_default(ctypes.byref(p))
        p.sr_c2p64_above = float(sr_c2p64_above)
        p.system = system
        if len(shape) == 1:
            p.dims, p.nx, p.ny = 1, shape[0], 1
        else:
            p.dims, p.ny, p.nx = 2, shape[0], shape[1]
        p.precision, p.boundary, p.gamma, p.dx = precision, BC_TRANSMISSIVE, float(gamma), float(dx)
        if levels not in (1, 2):
            raise ValueError("levels must be 1 or 2")
        self.levels = levels
        self.shape = tuple(shape)
        self.shapes = [tuple((1 << l) * n for n in shape) for l in range(levels + 1)]
        self.fine_shape = self.shapes[-1]
        h = ctypes.c_void_p()
        create = load().cosmos_amr_create if levels == 1 else load().cosmos_amr_create_level2
        check(create(self.ctx.h, ctypes.byref(p), ctypes.byref(h)))
        self.h = h

    def set_prim(self, prim):
        a = np.ascontiguousarray(prim, dtype=np.float64)
        if a.shape != self.shape + (5,):
            raise ValueError(f"expected shape {self.shape + (5,)}, got {a.shape}")
        check(load().cosmos_amr_set_prim(self.h, a.ctypes.data, a.size))

    def solve(self, cfl, t_final, tol, order):
        """Runs the driver from t = 0; returns (coarse steps, fine steps, final time, status bits) with
        the reference's counters.  self.fine_run holds the number of fine steps actually taken."""
        r = _lib.AmrResult()
        check(load().cosmos_amr_solve(self.h, float(cfl), float(t_final), float(tol), int(order), ctypes.byref(r)))
        self.fine_run, self.mid_run = r.fine_run, r.mid_run
        return r.coarse_steps, r.fine_steps, r.t, r.status

    def get_level(self, level):
        """(cells, flags) of one level: 0 coarse, up to `levels` (the finest)."""
        sh = self.shapes[level]
        cells = np.empty(sh + (5,))
        fl = np.empty(sh, np.uint8)
        check(load().cosmos_amr_get_level(self.h, int(level), cells.ctypes.data, fl.ctypes.data))
        return cells, fl.astype(bool)

    def get(self):
        """The reference driver's tuple: Level 1 (coarse, fine cells, coarse, fine flags); Level 2
        (coarse, intermediate, fine cells, coarse, intermediate, fine flags)."""
        got = [self.get_level(l) for l in range(self.levels + 1)]
        return tuple(c for c, _ in got) + tuple(f for _, f in got)

    def close(self):
        if getattr(self, "h", None) and not sys.is_finalizing():
            load().cosmos_amr_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _amr_family(system, name):
    """The reference's AMR driver class of one system (AMR/EulerAMR.hpp, AMR/RelativisticEulerAMR.hpp):
    solveLevel1AMR / solve2DLevel1AMR return (coarse cells, fine cells, coarse flags, fine flags);
    solveLevel2AMR / solve2DLevel2AMR (coarse, intermediate, fine cells, and their three flag sets)."""

    class Driver:
        __qualname__ = f"{name}AMR"

        @staticmethod
        def solveLevel1AMR(initialCells, cellSpacing, CFLCoefficient, finalTime, AMRTolerance, order,
                           materialParameters, precision=FP64):
            a = AMR(system, _shape(initialCells), cellSpacing, materialParameters.getAdiabaticIndex(), precision)
            try:
                a.set_prim(initialCells)
                a.solve(CFLCoefficient, finalTime, AMRTolerance, order)
                return a.get()
            finally:
                a.close()

        solve2DLevel1AMR = solveLevel1AMR

        @staticmethod
        def solveLevel2AMR(initialCells, cellSpacing, CFLCoefficient, finalTime, AMRTolerance, order,
                           materialParameters, precision=FP64):
            a = AMR(system, _shape(initialCells), cellSpacing, materialParameters.getAdiabaticIndex(), precision,
                    levels=2)
            try:
                a.set_prim(initialCells)
                a.solve(CFLCoefficient, finalTime, AMRTolerance, order)
                return a.get()
            finally:
                a.close()

        solve2DLevel2AMR = solveLevel2AMR

    return Driver


EulerAMR = _amr_family(NEWTONIAN, "Euler")
RelativisticEulerAMR = _amr_family(SR, "RelativisticEuler")


def state_eval(op, items, system=NEWTONIAN, gamma=1.4, xyz=None, black_hole=None, dx=0.0, bias=0.0, limiter=1,
               ctx=None):
    """The reference's state-level functions for an array of items on the device (cosmos_state_eval):
    op is a COSMOS_STATE_* code (cosmos_gb300._lib.STATE_*), items an array whose last axis holds
    the op's input width (5 for states, 1 for ratios, 15 for slope triples); xyz (..., 3) holds the
    black-hole items' coordinates.  Returns an array of the op's output width."""
    ctx = ctx or default_context()
    wi, wo = ctypes.c_size_t(0), ctypes.c_size_t(0)
    check(load().cosmos_state_width(int(op), ctypes.byref(wi), ctypes.byref(wo)))
    a = np.ascontiguousarray(items, dtype=np.float64).reshape(-1, wi.value)
    n = a.shape[0]
    p = Params()
    load().cosmos_params_default(ctypes.byref(p))
    p.system, p.gamma, p.dx = int(system), float(gamma), float(dx)
    if black_hole is not None:
        p.bh_mass, p.bh_spin = black_hole.mass, black_hole.spin
        p.bh_x, p.bh_y, p.bh_z = black_hole.x, black_hole.y, black_hole.z
    q = None if xyz is None else np.ascontiguousarray(xyz, dtype=np.float64).reshape(n, 3)
    out = np.empty((n, wo.value))
    check(load().cosmos_state_eval(ctx.h, ctypes.byref(p), int(op), n, a.ctypes.data,
                                   None if q is None else q.ctypes.data, float(bias), int(limiter), out.ctypes.data))
    return out


def interface_eval(op, items, system=NEWTONIAN, gamma=1.4, dx=1.0, dt=1.0, xyz=None, black_hole=None, bias=0.0,
                   limiter=1, frac=0.5, side=0, ctx=None):
    """The reference's per-interface solver functions (computeXSLICFlux, computeLaxFriedrichsFlux,
    evolveStateByHalfXTimeStep, ..., cosmos_interface_eval) for an array of items on the device,
    bit for bit with the reference: op is a COSMOS_IF_* code (cosmos_gb300._lib.IF_*), items an
    array whose last axis holds the op's inputs back to back (5-vectors: conserved vectors, flux
    vectors or primitive states), dx the cellSpacing, dt the timeStep; xyz (..., 3) holds the
    black-hole items' coordinate arguments.  Returns (n, 5): the vectors, or the primitives of the
    returned states."""
    ctx = ctx or default_context()
    wi = ctypes.c_size_t(0)
    check(load().cosmos_interface_width(int(op), ctypes.byref(wi), None))
    a = np.ascontiguousarray(items, dtype=np.float64).reshape(-1, wi.value)
    n = a.shape[0]
    p = Params()
    load().cosmos_params_default(ctypes.byref(p))
    p.system, p.gamma, p.dx = int(system), float(gamma), float(dx)
    if black_hole is not None:
        p.bh_mass, p.bh_spin = black_hole.mass, black_hole.spin
        p.bh_x, p.bh_y, p.bh_z = black_hole.x, black_hole.y, black_hole.z
    q = None if xyz is None else np.ascontiguousarray(xyz, dtype=np.float64).reshape(n, 3)
    out = np.empty((n, 5))
    check(load().cosmos_interface_eval(ctx.h, ctypes.byref(p), int(op), n, a.ctypes.data,
                                       None if q is None else q.ctypes.data, float(dt), float(bias), int(limiter),
                                       float(frac), int(side), out.ctypes.data))
    return out


def _scalar_or_array(out, like):
    return float(out[0, 0]) if np.ndim(like) == 0 else out[:, 0].reshape(np.shape(like))


def _rho_p_items(rho, p):
    r, q = np.broadcast_arrays(np.asarray(rho, dtype=np.float64), np.asarray(p, dtype=np.float64))
    items = np.zeros(r.shape + (5,))
    items[..., 0], items[..., 4] = r, q
    return items, r


class EulerEquationOfState:
    """Euler/EulerEquationOfState.hpp on the device; scalars or arrays."""

    @staticmethod
    def computeSpecificInternalEnergy(density, pressure, materialParameters):
        items, r = _rho_p_items(density, pressure)
        return _scalar_or_array(state_eval(_lib.STATE_INTERNAL_ENERGY, items, NEWTONIAN,
                                           materialParameters.getAdiabaticIndex()), r)

    @staticmethod
    def computePressure(density, specificInternalEnergy, materialParameters):
        items, r = _rho_p_items(density, specificInternalEnergy)
        return _scalar_or_array(state_eval(_lib.STATE_PRESSURE, items, NEWTONIAN,
                                           materialParameters.getAdiabaticIndex()), r)

    @staticmethod
    def computeSoundSpeed(density, pressure, materialParameters):
        items, r = _rho_p_items(density, pressure)
        return _scalar_or_array(state_eval(_lib.STATE_SOUND, items, NEWTONIAN, materialParameters.getAdiabaticIndex()),
                                r)


class RelativisticEulerEquationOfState:
    """RelativisticEuler/RelativisticEulerEquationOfState.hpp on the device; scalars or arrays."""

    @staticmethod
    def computeSpecificEnthalpy(density, pressure, materialParameters):
        items, r = _rho_p_items(density, pressure)
        return _scalar_or_array(state_eval(_lib.STATE_ENTHALPY, items, SR, materialParameters.getAdiabaticIndex()), r)

    @staticmethod
    def computeSoundSpeed(density, pressure, materialParameters):
        items, r = _rho_p_items(density, pressure)
        return _scalar_or_array(state_eval(_lib.STATE_SOUND, items, SR, materialParameters.getAdiabaticIndex()), r)


class SlopeLimiters:
    """Solvers/SlopeLimiters.hpp on the device: limiter functions of a steepness r (scalar or array)
    and slope vectors of conserved (left, middle, right) vectors ((..., 5) arrays)."""

    @staticmethod
    def computeGradientRatio(steepness, bias):
        r = np.asarray(steepness, dtype=np.float64)
        return _scalar_or_array(state_eval(_lib.STATE_GRADIENT_RATIO, r.reshape(-1, 1), bias=bias), r)

    @staticmethod
    def computeSlopeLimiter(steepness, bias, slopeLimiter):
        r = np.asarray(steepness, dtype=np.float64)
        return _scalar_or_array(state_eval(_lib.STATE_LIMITER, r.reshape(-1, 1), bias=bias, limiter=slopeLimiter), r)

    @staticmethod
    def computeSuperBeeSlopeLimiter(steepness, bias):
        return SlopeLimiters.computeSlopeLimiter(steepness, bias, 0)

    @staticmethod
    def computeVanLeerSlopeLimiter(steepness, bias):
        return SlopeLimiters.computeSlopeLimiter(steepness, bias, 1)

    @staticmethod
    def computeMinBeeSlopeLimiter(steepness, bias):
        return SlopeLimiters.computeSlopeLimiter(steepness, bias, 2)

    @staticmethod
    def computeSlopeVector(left, middle, right, bias, slopeLimiter):
        l, m, r = np.broadcast_arrays(*(np.asarray(v, dtype=np.float64) for v in (left, middle, right)))
        out = state_eval(_lib.STATE_SLOPE, np.concatenate([l.reshape(-1, 5), m.reshape(-1, 5), r.reshape(-1, 5)], axis=1),
                         bias=bias, limiter=slopeLimiter)
        return out.reshape(l.shape)
