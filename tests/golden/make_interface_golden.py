"""Generate tests/golden/interface_golden.npz: the reference's per-interface solver functions
(computeXSLICFlux, computeLaxFriedrichsFlux, evolveStateByHalfXTimeStep, the black-hole forcing
solver's cell update, ...) evaluated by the reference itself on seeded inputs.

The reference is compiled from its own sources by oracle/ref/Makefile; ref_interface_eval
(oracle/ref/ref_harness.cpp) calls its public static functions once per item.  Each case stores
the op, the system, the scalar arguments, the inputs, the coordinates (black hole) and the
reference's outputs; tests/test_oracle_golden.py checks the oracle against them and
tests/test_gpu_interface.py the device functions.

    make -C oracle && make -C oracle/ref && python tests/golden/make_interface_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, os.path.dirname(HERE))

from oracle.pyoracle import IFACE_WIDTH, Oracle, Reference  # noqa: E402
import cases  # noqa: E402

BH = (1.0, 0.0, 0.5, 0.5, 0.0)  # the reference's default hole (BlackHoleEuler/BlackHoleSpacetime.cpp:3-11)
SPIN = (1.0, 0.6, 0.5, 0.5, 0.0)
N_ITEMS = 48


def points(rng, n, bh):
    """Coordinates 3M < r < 8M from the hole, z = 0."""
    r = rng.uniform(3.0, 8.0, n) * bh[0]
    a = rng.uniform(0.0, 2.0 * np.pi, n)
    return np.stack([bh[2] + r * np.cos(a), bh[3] + r * np.sin(a), np.zeros(n)], axis=1)


def items(O, op, system, rng, n, dx, bh):
    """Seeded inputs for `op` (IFACE_WIDTH[op] doubles per item) and the GR coordinates."""
    g = cases.SYS_GAMMA[system]
    xyz = points(rng, n, bh) if system == 2 else None
    if op <= 5:  # vectors: conserved states and fluxes of physical states (any values are valid)
        flat = min(system, 1)  # the vector forms are the same arithmetic for every system
        s = cases.state(flat, rng, (n * IFACE_WIDTH[op] // 5,))
        v = np.stack([O.cons(flat, p, cases.SYS_GAMMA[flat]) for p in s])
        return v.reshape(n, -1), xyz
    if op in (16, 17, 20):  # conserved vectors at the state's point plus a small evolution vector
        k = 2 if op != 20 else 1
        axis = 1 if op == 17 else 0
        s = cases.state(system, rng, (n, k))
        out = np.zeros((n, IFACE_WIDTH[op]))
        for i in range(n):
            for j in range(k):
                x, y = (xyz[i, 0], xyz[i, 1]) if xyz is not None else (0.0, 0.0)
                if op != 20 and system == 2:  # the extrapolated values belong to the cell's faces
                    d = (-0.5 if j == 0 else 0.5) * dx
                    x, y = (x + d, y) if axis == 0 else (x, y + d)
                out[i, 5 * j:5 * j + 5] = O.cons(system, s[i, j], g, x, y, bh, dx)
            out[i, 5 * k:5 * k + 5] = 1e-3 * rng.standard_normal(5) * np.abs(out[i, :5]).max()
        return out, xyz
    if op in (21, 22):  # conserved neighbours at their own points (l, m, r[, t, b])
        k = 3 if op == 21 else 5
        s = cases.state(2, rng, (n, k))
        off = [(-dx, 0.0), (0.0, 0.0), (dx, 0.0), (0.0, -dx), (0.0, dx)]
        out = np.zeros((n, 5 * k))
        for i in range(n):
            for j in range(k):
                out[i, 5 * j:5 * j + 5] = O.cons(2, s[i, j], g, xyz[i, 0] + off[j][0], xyz[i, 1] + off[j][1], bh, dx)
        return out, xyz
    # primitive states
    k = IFACE_WIDTH[op] // 5
    return cases.state(system, rng, (n, k)).reshape(n, -1), xyz


def cases_for(system):
    """(op, lim, bias, side, frac) combinations: every op the system has, every limiter where the op
    takes one, both sides where it takes one."""
    ops = range(23) if system == 2 else range(18)
    out = []
    for op in ops:
        lims = (0, 1, 2) if op in (12, 13, 14, 15, 18, 19, 21, 22) else (1,)
        sides = (0, 1) if op in (14, 15, 16, 17) else (0,)
        for lim in lims:
            for side in sides:
                bias = 0.3 if lim == 2 else 0.0
                frac = 0.25 if op in (4, 18, 19) else 0.5
                out.append((op, lim, bias, side, frac))
    return out


def main():
    R, O = Reference(), Oracle()
    rng = np.random.default_rng(20260911)
    out = {}
    for system in (0, 1, 2):
        for hole, bh in ((("schw", BH), ("kerr", SPIN)) if system == 2 else (("none", BH),)):
            dx = 0.05 if system == 2 else 1.0 / 64
            dt = 0.4 * dx
            g = cases.SYS_GAMMA[system]
            for (op, lim, bias, side, frac) in cases_for(system):
                a, xyz = items(O, op, system, rng, N_ITEMS if op < 21 else 16, dx, bh)
                key = f"if_s{system}_{hole}_op{op}_l{lim}_side{side}"
                out[key + "_in"] = a
                if xyz is not None:
                    out[key + "_xyz"] = xyz
                out[key + "_args"] = np.array([op, system, g, dx, dt, bias, lim, frac, side, *bh])
                out[key + "_out"] = R.interface(op, system, a, xyz, g, bh, dx, dt, bias, lim, frac, side)
    # BlackHoleSpacetime's public quantities and BlackHoleEulerEigenvalues, around a Schwarzschild
    # and a spinning hole, off the plane z = 0 as well (the spin couples z)
    for hole, bh in (("schw", BH), ("kerr", SPIN)):
        q = points(rng, 64, bh)
        q[32:, 2] = rng.uniform(-1.5, 1.5, 32)
        out[f"st_{hole}_xyz"] = q
        out[f"st_{hole}_bh"] = np.array(bh)
        out[f"st_{hole}_h"] = np.array(0.05)
        out[f"st_{hole}_out"] = R.spacetime_record(q, 0.05, bh)
        p = cases.gr_state(rng, (64,))
        out[f"eig_{hole}_in"] = p
        out[f"eig_{hole}_out"] = R.gr_eigenvalues(p, q, 5.0 / 3.0, bh)
    path = os.path.join(HERE, "interface_golden.npz")
    np.savez_compressed(path, **out)
    print(f"{path}: {len(out)} arrays")


if __name__ == "__main__":
    main()
