"""TEST INFRASTRUCTURE ONLY -- ctypes access to the CPU oracle and to the reference build.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg import this module.

``Oracle`` wraps ``oracle/liboracle.so`` (the FP64 restatement of the reference's SLIC/FORCE
path, oracle/cosmos_oracle.cpp).  ``Reference`` wraps ``oracle/_ref/libcosmos_ref.so``, the
reference itself compiled from its own sources by oracle/ref/Makefile; it exists only where the
reference checkout is present (not on the GPU host), so callers must handle ``available()``.

Grids are float64 arrays of primitive states shaped (ny, nx, 5) (or (nx, 5) in 1D):
(rho, vx, vy, vz, p).  bh = (mass, spin, x, y, z).
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libcosmos_ref.so")

_d, _i, _p = ctypes.c_double, ctypes.c_int, ctypes.c_void_p
SYSTEMS = {"newton": 0, "sr": 1, "gr": 2}


def _ptr(a):
    return a.ctypes.data if a is not None else None


def _sys(s):
    return SYSTEMS[s] if isinstance(s, str) else int(s)


def _shape(prim):
    if prim.ndim == 2:
        return 1, prim.shape[0], 1
    return prim.shape[0], prim.shape[1], 2


def _bh(bh):
    return np.ascontiguousarray(np.asarray(bh if bh is not None else (1.0, 0.0, 0.5, 0.5, 0.0), dtype=np.float64))


IFACE_WIDTH = (20, 20, 10, 15, 10, 10, 10, 10, 10, 10, 10, 10, 20, 20, 15, 15, 15, 15, 15, 15, 10, 15, 25)


def _iface(fn, op, system, items, xyz, gamma, bh, dx, dt, bias, lim, frac, side):
    """Shared driver of orc_interface_eval / ref_interface_eval: items (n, in_width), xyz (n, 3) or
    None; returns (n, 5)."""
    a = np.ascontiguousarray(items, dtype=np.float64).reshape(-1, IFACE_WIDTH[op])
    n = a.shape[0]
    q = None if xyz is None else np.ascontiguousarray(xyz, dtype=np.float64).reshape(n, 3)
    o = np.zeros((n, 5))
    rc = fn(op, _sys(system), n, _ptr(a), _ptr(q), gamma, _ptr(_bh(bh)), dx, dt, bias, lim, frac, side, _ptr(o))
    if rc:
        raise ValueError(f"interface op {op} is not defined for system {system}")
    return o


class Oracle:
    """The FP64 restatement (always available once built)."""

    def __init__(self, path=ORACLE_SO):
        if not os.path.exists(path):
            raise RuntimeError(f"oracle library not built: {path} (run make -C oracle)")
        L = self.L = ctypes.CDLL(path)
        L.orc_sweep.argtypes = [_i, _p, _i, _i, _i, _i, _i, _d, _d, _d, _i, _d, _i, _p, _p]
        L.orc_max_wavespeed.argtypes = [_i, _p, _i, _i, _i, _d, _p]
        L.orc_max_wavespeed.restype = _d
        L.orc_stable_dt.argtypes = [_i, _p, _i, _i, _i, _d, _d, _d, _d, _i, _d, _p]
        L.orc_stable_dt.restype = _d
        L.orc_interface_eval.argtypes = [_i, _i, ctypes.c_size_t, _p, _p, _d, _p, _d, _d, _d, _i, _d, _i, _p]
        L.orc_interface_eval.restype = _i
        L.orc_spacetime_record.argtypes = [_d, _d, _d, _d, _p, _p]
        L.orc_gr_eigenvalues.argtypes = [_p, _d, _d, _d, _d, _p, _p]
        L.orc_stable_dt_rule.argtypes = [_d, _d, _d, _i]
        L.orc_stable_dt_rule.restype = _d
        L.orc_rk_source.argtypes = [_p, _i, _i, _i, _d, _d, _d, _i, _d, _p]
        L.orc_solve.argtypes = [_i, _p, _i, _i, _i, _i, _d, _d, _d, _d, _i, _d, _i, _i, _p, _i, _p, _p]
        L.orc_solve.restype = _i
        for n in ("orc_cons", "orc_prim"):
            getattr(L, n).argtypes = [_i, _p, _d, _d, _d, _p, _d, _p]
        L.orc_flux.argtypes = [_i, _p, _i, _d, _d, _d, _p, _d, _p]
        L.orc_gr_source.argtypes = [_p, _d, _d, _d, _d, _p, _p]
        L.orc_gr_sound_speed.argtypes = [_p, _d, _d, _d, _p]
        L.orc_gr_sound_speed.restype = _d
        L.orc_limiter.argtypes = [_d, _d, _i]
        L.orc_limiter.restype = _d
        L.orc_slope.argtypes = [_p, _p, _p, _d, _i, _p]
        L.orc_gr_metric.argtypes = [_d, _d, _d, _d, _p, _p]
        L.orc_amr_flags.argtypes = [_i, _p, _i, _i, _i, _d, _d, _d, _p, _p, _p]
        L.orc_amr_derefine.argtypes = [_i, _p, _p, _i, _i, _i, _d, _d, _d, _p, _p, _p]
        L.orc_amr_level1.argtypes = [_i, _p, _i, _i, _i, _d, _d, _d, _d, _i, _d, _p, _p, _p, _p, _p, _p]
        L.orc_amr_level1.restype = _i
        L.orc_amr_level2.argtypes = [_i, _p, _i, _i, _i, _d, _d, _d, _d, _i, _d, _p, _p, _p, _p, _p, _p, _p]
        L.orc_amr_level2.restype = _i
        L.orc_tlm_newton.argtypes = [_p, _p, _p, _i, _i, _i, _d, _p, _i, _d, _i, _d, _i, _p]
        L.orc_tlm_newton.restype = _d
        L.orc_tlm_sr.argtypes = [_p, _p, _p, _i, _i, _i, _d, _p, _i, _d, _i, _d, _i, _p]
        L.orc_tlm_sr.restype = _d
        L.orc_tlm_gr.argtypes = [_p, _p, _p, _i, _i, _i, _d, _p, _i, _d, _i, _d, _p, _i, _p]
        L.orc_tlm_gr.restype = _d
        L.orc_set_threads.argtypes = [_i]

    def set_threads(self, n):
        """Line-parallel sweeps on n host threads (results do not depend on n)."""
        self.L.orc_set_threads(int(n))

    # ---- grid operations (in place on a float64 copy; returns the new array)
    def sweep(self, system, prim, axis, order, dx, dt, bias, lim, gamma, bc=0, mask=None, bh=None):
        p = np.ascontiguousarray(prim, dtype=np.float64).copy()
        ny, nx, dims = _shape(p)
        m = None if mask is None else np.ascontiguousarray(mask, dtype=np.uint8)
        self.L.orc_sweep(_sys(system), _ptr(p), ny, nx, dims, axis, order, dx, dt, bias, lim, gamma, bc,
                         _ptr(m), _ptr(_bh(bh)))
        return p

    def max_wavespeed(self, system, prim, gamma, bh=None):
        p = np.ascontiguousarray(prim, dtype=np.float64)
        ny, nx, dims = _shape(p)
        return self.L.orc_max_wavespeed(_sys(system), _ptr(p), ny, nx, dims, gamma, _ptr(_bh(bh)))

    def stable_dt(self, system, prim, dx, cfl, t, tf, it, gamma, bh=None):
        p = np.ascontiguousarray(prim, dtype=np.float64)
        ny, nx, dims = _shape(p)
        return self.L.orc_stable_dt(_sys(system), _ptr(p), ny, nx, dims, dx, cfl, t, tf, it, gamma, _ptr(_bh(bh)))

    def stable_dt_rule(self, dt, t, tf, it):
        return self.L.orc_stable_dt_rule(dt, t, tf, it)

    def rk_source(self, prim, dx, dt, bias, lim, gamma, bh):
        p = np.ascontiguousarray(prim, dtype=np.float64).copy()
        ny, nx, dims = _shape(p)
        self.L.orc_rk_source(_ptr(p), ny, nx, dims, dx, dt, bias, lim, gamma, _ptr(_bh(bh)))
        return p

    def solve(self, system, prim, order, dx, cfl, tf, bias, lim, gamma, bc=0, subcycles=1, bh=None, max_steps=-1):
        """Returns (prim, steps, t, dts)."""
        p = np.ascontiguousarray(prim, dtype=np.float64).copy()
        ny, nx, dims = _shape(p)
        cap = max_steps if max_steps >= 0 else 1 << 20
        dts = np.zeros(min(cap, 1 << 20), dtype=np.float64)
        t = _d(0.0)
        n = self.L.orc_solve(_sys(system), _ptr(p), ny, nx, dims, order, dx, cfl, tf, bias, lim, gamma, bc,
                             subcycles, _ptr(_bh(bh)), max_steps, _ptr(dts), ctypes.byref(t))
        return p, n, t.value, dts[:n].copy()

    # ---- state level
    def cons(self, system, prim, gamma, x=0.0, y=0.0, bh=None, h=0.0):
        p = np.ascontiguousarray(prim, dtype=np.float64); o = np.zeros(5)
        self.L.orc_cons(_sys(system), _ptr(p), x, y, gamma, _ptr(_bh(bh)), h, _ptr(o)); return o

    def prim(self, system, cons, gamma, x=0.0, y=0.0, bh=None, h=0.0):
        u = np.ascontiguousarray(cons, dtype=np.float64); o = np.zeros(5)
        self.L.orc_prim(_sys(system), _ptr(u), x, y, gamma, _ptr(_bh(bh)), h, _ptr(o)); return o

    def flux(self, system, cons, axis, gamma, x=0.0, y=0.0, bh=None, h=0.0):
        u = np.ascontiguousarray(cons, dtype=np.float64); o = np.zeros(5)
        self.L.orc_flux(_sys(system), _ptr(u), axis, x, y, gamma, _ptr(_bh(bh)), h, _ptr(o)); return o

    def gr_source(self, cons, x, y, h, gamma, bh):
        u = np.ascontiguousarray(cons, dtype=np.float64); o = np.zeros(5)
        self.L.orc_gr_source(_ptr(u), x, y, h, gamma, _ptr(_bh(bh)), _ptr(o)); return o

    def gr_sound_speed(self, prim, x, y, gamma, bh):
        p = np.ascontiguousarray(prim, dtype=np.float64)
        return self.L.orc_gr_sound_speed(_ptr(p), x, y, gamma, _ptr(_bh(bh)))

    def gr_metric(self, x, y, z, h, bh):
        o = np.zeros(57); self.L.orc_gr_metric(x, y, z, h, _ptr(_bh(bh)), _ptr(o)); return o

    def limiter(self, r, bias, lim):
        return self.L.orc_limiter(r, bias, lim)

    def interface(self, op, system, items, xyz=None, gamma=1.4, bh=None, dx=0.01, dt=0.004, bias=0.0, lim=1,
                  frac=0.5, side=0):
        """The per-interface solver function `op` (orc_interface_eval) on each item."""
        return _iface(self.L.orc_interface_eval, op, system, items, xyz, gamma, bh, dx, dt, bias, lim, frac, side)

    def _st(self, *a):
        self.L.orc_spacetime_record(*a)

    def _eig(self, *a):
        self.L.orc_gr_eigenvalues(*a)

    def spacetime_record(self, xyz, h, bh):
        """Every public BlackHoleSpacetime quantity at each point of xyz (n, 3): (n, 125)."""
        q = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
        o = np.zeros((q.shape[0], 125))
        b = _bh(bh)
        for i in range(q.shape[0]):
            self._st(q[i, 0], q[i, 1], q[i, 2], h, _ptr(b), o[i].ctypes.data)
        return o

    def gr_eigenvalues(self, prims, xyz, gamma, bh):
        """Material, fast and slow acoustic eigenvalues (3 each) of each primitive state: (n, 9)."""
        p = np.ascontiguousarray(prims, dtype=np.float64).reshape(-1, 5)
        q = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
        o = np.zeros((p.shape[0], 9))
        b = _bh(bh)
        for i in range(p.shape[0]):
            self._eig(p[i].ctypes.data, q[i, 0], q[i, 1], q[i, 2], gamma, _ptr(b), o[i].ctypes.data)
        return o


    def slope(self, ul, uc, ur, bias, lim):
        a, b, c = (np.ascontiguousarray(v, dtype=np.float64) for v in (ul, uc, ur)); o = np.zeros(5)
        self.L.orc_slope(_ptr(a), _ptr(b), _ptr(c), bias, lim, _ptr(o)); return o

    # ---- AMR
    def amr_flags(self, system, prim, dx, tol, gamma, coarse=None, fine=None, bh=None):
        p = np.ascontiguousarray(prim, dtype=np.float64)
        ny, nx, dims = _shape(p)
        nc = nx * (ny if dims == 2 else 1)
        c = np.ones(nc, np.uint8) if coarse is None else np.ascontiguousarray(coarse, np.uint8).reshape(-1).copy()
        f = np.zeros(nc * (4 if dims == 2 else 2), np.uint8) if fine is None else \
            np.ascontiguousarray(fine, np.uint8).reshape(-1).copy()
        self.L.orc_amr_flags(_sys(system), _ptr(p), ny, nx, dims, dx, tol, gamma, _ptr(_bh(bh)), _ptr(c), _ptr(f))
        return c, f

    def amr_derefine(self, system, coarse_prim, fine_prim, dx, tol, gamma, coarse, fine, bh=None):
        cp = np.ascontiguousarray(coarse_prim, dtype=np.float64).copy()
        fp = np.ascontiguousarray(fine_prim, dtype=np.float64)
        ny, nx, dims = _shape(cp)
        c = np.ascontiguousarray(coarse, np.uint8).reshape(-1).copy()
        f = np.ascontiguousarray(fine, np.uint8).reshape(-1).copy()
        self.L.orc_amr_derefine(_sys(system), _ptr(cp), _ptr(fp), ny, nx, dims, dx, tol, gamma, _ptr(_bh(bh)),
                                _ptr(c), _ptr(f))
        return cp, c, f

    def amr_level1(self, system, prim, dx, cfl, tf, tol, order, gamma, fine_run=None):
        """The Level-1 AMR driver: (coarse steps, fine steps, coarse prims, fine prims, coarse flags,
        fine flags), grids flattened like Reference.amr_level1.  fine_run (a list) receives the number
        of fine steps actually taken."""
        p = np.ascontiguousarray(prim, dtype=np.float64)
        ny, nx, dims = _shape(p)
        nc = nx * (ny if dims == 2 else 1)
        nf = nc * (4 if dims == 2 else 2)
        cp = np.zeros(nc * 5); fp = np.zeros(nf * 5)
        cf = np.zeros(nc, np.uint8); ff = np.zeros(nf, np.uint8)
        fs, fr = ctypes.c_int(0), ctypes.c_int(0)
        n = self.L.orc_amr_level1(_sys(system), _ptr(p), ny, nx, dims, dx, cfl, tf, tol, order, gamma, _ptr(cp),
                                  _ptr(fp), _ptr(cf), _ptr(ff), ctypes.byref(fs), ctypes.byref(fr))
        if fine_run is not None:
            fine_run.append(fr.value)
        return n, fs.value, cp, fp, cf, ff

    def amr_level2(self, system, prim, dx, cfl, tf, tol, order, gamma):
        """The Level-2 AMR driver: (coarse steps, [total fine count, intermediate steps taken, fine
        steps taken], coarse, intermediate, fine prims, and the three flag sets), flattened."""
        p = np.ascontiguousarray(prim, dtype=np.float64)
        ny, nx, dims = _shape(p)
        nc = nx * (ny if dims == 2 else 1)
        r = 4 if dims == 2 else 2
        cp, mp, fp = np.zeros(nc * 5), np.zeros(nc * r * 5), np.zeros(nc * r * r * 5)
        cf, mf, ff = np.zeros(nc, np.uint8), np.zeros(nc * r, np.uint8), np.zeros(nc * r * r, np.uint8)
        counts = np.zeros(3, np.int32)
        n = self.L.orc_amr_level2(_sys(system), _ptr(p), ny, nx, dims, dx, cfl, tf, tol, order, gamma, _ptr(cp),
                                  _ptr(mp), _ptr(fp), _ptr(cf), _ptr(mf), _ptr(ff), counts.ctypes.data)
        return n, [int(c) for c in counts], cp, mp, fp, cf, mf, ff

    # ---- tangent-linear of the Newtonian SLIC loss
    def tlm_sr(self, prim0, dprim, target, dx, dts, bias, lim, gamma, bc=0):
        """The SR tangent-linear model: (loss, directional derivative) like tlm_newton."""
        p = np.ascontiguousarray(prim0, dtype=np.float64)
        d = np.ascontiguousarray(dprim, dtype=np.float64)
        t = np.ascontiguousarray(target, dtype=np.float64)
        ds = np.ascontiguousarray(dts, dtype=np.float64)
        ny, nx, dims = _shape(p)
        out = _d(0.0)
        L = self.L.orc_tlm_sr(_ptr(p), _ptr(d), _ptr(t), ny, nx, dims, dx, _ptr(ds), len(ds), bias, lim, gamma, bc,
                              ctypes.byref(out))
        return L, out.value

    def tlm_gr(self, prim0, dprim, target, dx, dts, bias, lim, gamma, bh, subcycles=0):
        """The black-hole step's tangent-linear model (`subcycles` RK source half-steps around the flux
        step; 0: the flux step alone): (loss, directional derivative)."""
        p = np.ascontiguousarray(prim0, dtype=np.float64)
        d = np.ascontiguousarray(dprim, dtype=np.float64)
        t = np.ascontiguousarray(target, dtype=np.float64)
        ds = np.ascontiguousarray(dts, dtype=np.float64)
        ny, nx, dims = _shape(p)
        out = _d(0.0)
        L = self.L.orc_tlm_gr(_ptr(p), _ptr(d), _ptr(t), ny, nx, dims, dx, _ptr(ds), len(ds), bias, lim, gamma,
                              _ptr(_bh(bh)), int(subcycles), ctypes.byref(out))
        return L, out.value

    def tlm_newton(self, prim0, dprim, target, dx, dts, bias, lim, gamma, bc=0):
        p = np.ascontiguousarray(prim0, dtype=np.float64)
        d = np.ascontiguousarray(dprim, dtype=np.float64)
        t = np.ascontiguousarray(target, dtype=np.float64)
        ds = np.ascontiguousarray(dts, dtype=np.float64)
        ny, nx, dims = _shape(p)
        out = _d(0.0)
        L = self.L.orc_tlm_newton(_ptr(p), _ptr(d), _ptr(t), ny, nx, dims, dx, _ptr(ds), len(ds), bias, lim, gamma,
                                  bc, ctypes.byref(out))
        return L, out.value


class Reference:
    """The reference compiled from its own sources (present only where the checkout is)."""

    @staticmethod
    def available(path=REF_SO):
        return os.path.exists(path)

    def __init__(self, path=REF_SO):
        L = self.L = ctypes.CDLL(path)
        L.ref_sweep.argtypes = [_i, _p, _i, _i, _i, _i, _i, _d, _d, _d, _i, _d, _i]
        L.ref_stable_dt.argtypes = [_i, _p, _i, _i, _i, _d, _d, _d, _d, _i, _d]
        L.ref_stable_dt.restype = _d
        L.ref_max_wavespeed.argtypes = [_i, _p, _i, _i, _i, _d]
        L.ref_max_wavespeed.restype = _d
        L.ref_solve.argtypes = [_i, _p, _i, _i, _i, _i, _d, _d, _d, _d, _i, _d]
        L.ref_solve.restype = _i
        for n in ("ref_euler_cons", "ref_euler_prim", "ref_sr_cons", "ref_sr_prim"):
            getattr(L, n).argtypes = [_p, _d, _p]
        for n in ("ref_euler_flux", "ref_sr_flux"):
            getattr(L, n).argtypes = [_p, _i, _d, _p]
        L.ref_interface_eval.argtypes = [_i, _i, ctypes.c_size_t, _p, _p, _d, _p, _d, _d, _d, _i, _d, _i, _p]
        L.ref_interface_eval.restype = _i
        L.ref_spacetime_record.argtypes = [_d, _d, _d, _d, _p, _p]
        L.ref_gr_eigenvalues.argtypes = [_p, _d, _d, _d, _d, _p, _p]
        L.ref_limiter.argtypes = [_d, _d, _i]
        L.ref_limiter.restype = _d
        L.ref_slope.argtypes = [_p, _p, _p, _d, _i, _p]
        L.ref_gr_metric.argtypes = [_d, _d, _d, _d, _p, _p]
        L.ref_gr_cons.argtypes = [_p, _d, _d, _d, _d, _p, _p]
        L.ref_gr_prim.argtypes = [_p, _d, _d, _d, _d, _p, _p]
        L.ref_gr_flux.argtypes = [_p, _i, _d, _d, _d, _d, _p, _p]
        L.ref_gr_source.argtypes = [_p, _d, _d, _d, _d, _d, _p, _p]
        L.ref_gr_sound_speed.argtypes = [_p, _d, _d, _d, _d, _p]
        L.ref_gr_sound_speed.restype = _d
        L.ref_gr_sweep.argtypes = [_p, _i, _i, _i, _i, _i, _d, _d, _d, _i, _d, _p]
        L.ref_gr_rk_source.argtypes = [_p, _i, _i, _i, _d, _d, _d, _i, _d, _p]
        L.ref_gr_stable_dt.argtypes = [_p, _i, _i, _i, _d, _d, _d, _d, _i, _d, _p]
        L.ref_gr_stable_dt.restype = _d
        L.ref_gr_solve.argtypes = [_p, _i, _i, _i, _i, _d, _d, _d, _d, _i, _i, _d, _p]
        L.ref_gr_solve.restype = _i
        L.ref_amr_level1.argtypes = [_i, _p, _i, _i, _i, _d, _d, _d, _d, _i, _d, _p, _p, _p, _p, _p]
        L.ref_amr_level1.restype = _i
        L.ref_amr_level2.argtypes = [_i, _p, _i, _i, _i, _d, _d, _d, _d, _i, _d, _p, _p, _p, _p, _p, _p]
        L.ref_amr_level2.restype = _i

    def sweep(self, system, prim, axis, order, dx, dt, bias, lim, gamma, bc=0, bh=None):
        p = np.ascontiguousarray(prim, dtype=np.float64).copy()
        ny, nx, dims = _shape(p)
        if _sys(system) == 2:
            self.L.ref_gr_sweep(_ptr(p), ny, nx, dims, axis, order, dx, dt, bias, lim, gamma, _ptr(_bh(bh)))
        else:
            self.L.ref_sweep(_sys(system), _ptr(p), ny, nx, dims, axis, order, dx, dt, bias, lim, gamma, bc)
        return p

    def stable_dt(self, system, prim, dx, cfl, t, tf, it, gamma, bh=None):
        p = np.ascontiguousarray(prim, dtype=np.float64)
        ny, nx, dims = _shape(p)
        if _sys(system) == 2:
            return self.L.ref_gr_stable_dt(_ptr(p), ny, nx, dims, dx, cfl, t, tf, it, gamma, _ptr(_bh(bh)))
        return self.L.ref_stable_dt(_sys(system), _ptr(p), ny, nx, dims, dx, cfl, t, tf, it, gamma)

    def max_wavespeed(self, system, prim, gamma):
        p = np.ascontiguousarray(prim, dtype=np.float64)
        ny, nx, dims = _shape(p)
        return self.L.ref_max_wavespeed(_sys(system), _ptr(p), ny, nx, dims, gamma)

    def rk_source(self, prim, dx, dt, bias, lim, gamma, bh):
        p = np.ascontiguousarray(prim, dtype=np.float64).copy()
        ny, nx, dims = _shape(p)
        self.L.ref_gr_rk_source(_ptr(p), ny, nx, dims, dx, dt, bias, lim, gamma, _ptr(_bh(bh)))
        return p

    def solve(self, system, prim, order, dx, cfl, tf, bias, lim, gamma, subcycles=1, bh=None):
        p = np.ascontiguousarray(prim, dtype=np.float64).copy()
        ny, nx, dims = _shape(p)
        if _sys(system) == 2:
            n = self.L.ref_gr_solve(_ptr(p), ny, nx, dims, order, dx, cfl, tf, bias, lim, subcycles, gamma,
                                    _ptr(_bh(bh)))
        else:
            n = self.L.ref_solve(_sys(system), _ptr(p), ny, nx, dims, order, dx, cfl, tf, bias, lim, gamma)
        return p, n

    def cons(self, system, prim, gamma, x=0.0, y=0.0, bh=None):
        p = np.ascontiguousarray(prim, dtype=np.float64); o = np.zeros(5)
        s = _sys(system)
        if s == 2: self.L.ref_gr_cons(_ptr(p), x, y, 0.0, gamma, _ptr(_bh(bh)), _ptr(o))
        else: (self.L.ref_euler_cons if s == 0 else self.L.ref_sr_cons)(_ptr(p), gamma, _ptr(o))
        return o

    def prim(self, system, cons, gamma, x=0.0, y=0.0, bh=None):
        u = np.ascontiguousarray(cons, dtype=np.float64); o = np.zeros(5)
        s = _sys(system)
        if s == 2: self.L.ref_gr_prim(_ptr(u), x, y, 0.0, gamma, _ptr(_bh(bh)), _ptr(o))
        else: (self.L.ref_euler_prim if s == 0 else self.L.ref_sr_prim)(_ptr(u), gamma, _ptr(o))
        return o

    def flux(self, system, cons, axis, gamma, x=0.0, y=0.0, bh=None):
        u = np.ascontiguousarray(cons, dtype=np.float64); o = np.zeros(5)
        s = _sys(system)
        if s == 2: self.L.ref_gr_flux(_ptr(u), axis, x, y, 0.0, gamma, _ptr(_bh(bh)), _ptr(o))
        else: (self.L.ref_euler_flux if s == 0 else self.L.ref_sr_flux)(_ptr(u), axis, gamma, _ptr(o))
        return o

    def gr_source(self, cons, x, y, h, gamma, bh):
        u = np.ascontiguousarray(cons, dtype=np.float64); o = np.zeros(5)
        self.L.ref_gr_source(_ptr(u), x, y, 0.0, h, gamma, _ptr(_bh(bh)), _ptr(o)); return o

    def gr_sound_speed(self, prim, x, y, gamma, bh):
        p = np.ascontiguousarray(prim, dtype=np.float64)
        return self.L.ref_gr_sound_speed(_ptr(p), x, y, 0.0, gamma, _ptr(_bh(bh)))

    def gr_metric(self, x, y, z, h, bh):
        o = np.zeros(57); self.L.ref_gr_metric(x, y, z, h, _ptr(_bh(bh)), _ptr(o)); return o

    def limiter(self, r, bias, lim):
        return self.L.ref_limiter(r, bias, lim)

    def interface(self, op, system, items, xyz=None, gamma=1.4, bh=None, dx=0.01, dt=0.004, bias=0.0, lim=1,
                  frac=0.5, side=0):
        """The reference's own static function for `op` (ref_interface_eval) on each item."""
        return _iface(self.L.ref_interface_eval, op, system, items, xyz, gamma, bh, dx, dt, bias, lim, frac, side)

    def _st(self, *a):
        self.L.ref_spacetime_record(*a)

    def _eig(self, *a):
        self.L.ref_gr_eigenvalues(*a)

    def spacetime_record(self, xyz, h, bh):
        """Every public BlackHoleSpacetime quantity at each point of xyz (n, 3): (n, 125)."""
        q = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
        o = np.zeros((q.shape[0], 125))
        b = _bh(bh)
        for i in range(q.shape[0]):
            self._st(q[i, 0], q[i, 1], q[i, 2], h, _ptr(b), o[i].ctypes.data)
        return o

    def gr_eigenvalues(self, prims, xyz, gamma, bh):
        """Material, fast and slow acoustic eigenvalues (3 each) of each primitive state: (n, 9)."""
        p = np.ascontiguousarray(prims, dtype=np.float64).reshape(-1, 5)
        q = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
        o = np.zeros((p.shape[0], 9))
        b = _bh(bh)
        for i in range(p.shape[0]):
            self._eig(p[i].ctypes.data, q[i, 0], q[i, 1], q[i, 2], gamma, _ptr(b), o[i].ctypes.data)
        return o


    def slope(self, ul, uc, ur, bias, lim):
        a, b, c = (np.ascontiguousarray(v, dtype=np.float64) for v in (ul, uc, ur)); o = np.zeros(5)
        self.L.ref_slope(_ptr(a), _ptr(b), _ptr(c), bias, lim, _ptr(o)); return o

    def amr_level1(self, system, prim, dx, cfl, tf, tol, order, gamma, bh=None):
        p = np.ascontiguousarray(prim, dtype=np.float64)
        ny, nx, dims = _shape(p)
        nc = nx * (ny if dims == 2 else 1)
        nf = nc * (4 if dims == 2 else 2)
        cp = np.zeros(nc * 5); fp = np.zeros(nf * 5)
        cf = np.zeros(nc, np.uint8); ff = np.zeros(nf, np.uint8)
        n = self.L.ref_amr_level1(_sys(system), _ptr(p), ny, nx, dims, dx, cfl, tf, tol, order, gamma,
                                  _ptr(_bh(bh)), _ptr(cp), _ptr(fp), _ptr(cf), _ptr(ff))
        return n, cp, fp, cf, ff

    def amr_level2(self, system, prim, dx, cfl, tf, tol, order, gamma):
        """The reference's Level-2 driver: (coarse steps, coarse, intermediate, fine prims, and the three
        flag sets), flattened."""
        p = np.ascontiguousarray(prim, dtype=np.float64)
        ny, nx, dims = _shape(p)
        nc = nx * (ny if dims == 2 else 1)
        r = 4 if dims == 2 else 2
        cp, mp, fp = np.zeros(nc * 5), np.zeros(nc * r * 5), np.zeros(nc * r * r * 5)
        cf, mf, ff = np.zeros(nc, np.uint8), np.zeros(nc * r, np.uint8), np.zeros(nc * r * r, np.uint8)
        n = self.L.ref_amr_level2(_sys(system), _ptr(p), ny, nx, dims, dx, cfl, tf, tol, order, gamma, _ptr(cp),
                                  _ptr(mp), _ptr(fp), _ptr(cf), _ptr(mf), _ptr(ff))
        return n, cp, mp, fp, cf, mf, ff
