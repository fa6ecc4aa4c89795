"""The CPU oracle reproduces the reference's own outputs bit for bit.

The fixtures in tests/golden/reference_golden.npz were produced by running the reference itself
(compiled from its sources, tests/golden/make_golden.py).  These tests run everywhere (no GPU, no
reference checkout needed) and pin the oracle that the GPU parity tests compare against.
"""
import os
import re

import numpy as np
import pytest

import cases
from conftest import bit_equal


def _keys(golden, prefix, suffix="_in"):
    return sorted(k[: -len(suffix)] for k in golden if k.startswith(prefix) and k.endswith(suffix))


def parse_sweep_key(k):
    """'newton_d2_o2_l1_bc0_a1' -> dict(d=2, o=2, l=1, bc=0, a=1)"""
    m = re.match(r"^\w+?_d(\d)_o(\d)_l(\d)_bc(\d)_a(\d)$", k)
    return dict(zip(("d", "o", "l", "bc", "a"), map(int, m.groups())))


def test_sod_1000_cells(oracle, golden):
    p, n, t, _ = oracle.solve(0, cases.sod(1000), 2, 1.0 / 1000, 0.9, 0.25, 0.0, 1, 1.4)
    assert n == int(golden["sod1000_steps"]) == 613
    assert bit_equal(p, golden["sod1000_final"])
    assert p[500, 0] == 0.4263927017295945  # anchor recorded from the reference build


@pytest.mark.parametrize("tag,system", [("newton", 0), ("sr", 1)])
def test_sweeps(oracle, golden, tag, system):
    keys = [k for k in _keys(golden, tag + "_d") if re.match(r"^\w+?_d\d_o", k)]
    assert len(keys) >= 20
    for k in keys:
        q = parse_sweep_key(k)
        s = golden[k + "_in"]
        out = oracle.sweep(system, s, q["a"], q["o"], 1.0 / 64, 0.004, float(golden[k + "_bias"]), q["l"],
                           cases.SYS_GAMMA[system], q["bc"])
        assert bit_equal(out, golden[k + "_out"]), k


@pytest.mark.parametrize("tag,system", [("newton", 0), ("sr", 1)])
def test_solves_and_dt(oracle, golden, tag, system):
    g = cases.SYS_GAMMA[system]
    p, n, _, _ = oracle.solve(system, golden[f"{tag}_solve2d_in"], 2, 1.0 / 12, 0.9, 0.05, 0.0, 2, g)
    assert n == int(golden[f"{tag}_solve2d_steps"]) and bit_equal(p, golden[f"{tag}_solve2d_out"])
    p, n, _, _ = oracle.solve(system, golden[f"{tag}_solve1d_force_in"], 1, 1.0 / 24, 0.8, 0.05, 0.0, 1, g)
    assert n == int(golden[f"{tag}_solve1d_force_steps"]) and bit_equal(p, golden[f"{tag}_solve1d_force_out"])
    for dims in (1, 2):
        s = golden[f"{tag}_dt_d{dims}_in"]
        dts = [oracle.stable_dt(system, s, 0.01, 0.9, 0.0, 1.0, it, g) for it in (0, 7)]
        assert bit_equal(np.array(dts), golden[f"{tag}_dt_d{dims}"])


@pytest.mark.parametrize("bhname,bh", [("bh", cases.GR_BH), ("spin", cases.GR_BH_SPIN)])
def test_gr(oracle, golden, bhname, bh):
    g = cases.SYS_GAMMA[2]
    for dims in (1, 2):
        dx = 1.0 / 12
        for order in (1, 2):
            for axis in ((0,) if dims == 1 else (0, 1)):
                k = f"gr_{bhname}_d{dims}_o{order}_a{axis}"
                out = oracle.sweep(2, golden[k + "_in"], axis, order, dx, 0.002, 0.0, 1, g, bh=bh)
                assert bit_equal(out, golden[k + "_out"]), k
        s = golden[f"gr_{bhname}_rk_d{dims}_in"]
        assert bit_equal(oracle.rk_source(s, dx, 0.002, 0.0, 1, g, bh), golden[f"gr_{bhname}_rk_d{dims}_out"])
        assert oracle.stable_dt(2, s, dx, 0.9, 0.0, 1.0, 0, g, bh=bh) == float(golden[f"gr_{bhname}_dt_d{dims}"])


def test_gr_solve_and_metric(oracle, golden):
    p, n, _, _ = oracle.solve(2, golden["gr_solve_in"], 2, 2.0, 0.9, 0.3, 0.0, 1, 5.0 / 3.0, subcycles=1,
                              bh=(1.0, 0.0, 10.0, 10.0, 0.0))
    assert n == int(golden["gr_solve_steps"]) and bit_equal(p, golden["gr_solve_out"])
    for bhname, bh in (("bh", cases.GR_BH), ("spin", cases.GR_BH_SPIN), ("cfg4", (1.0, 0.0, 10.0, 10.0, 0.0))):
        ref = golden[f"gr_metric_{bhname}"]
        for row, (x, y, z) in zip(ref, golden["gr_metric_pts"]):
            assert np.array_equal(oracle.gr_metric(x, y, z, 0.05, bh), row, equal_nan=True), (bhname, x, y, z)


def _emulate_amr_first_step(O, system, p0, dx, cfl, T, tol, g):
    """The reference Level-1 driver's first coarse step when dt < 1e-4 (no fine sub-steps):
    flag pass, masked coarse step, restriction, injection, derefinement (AMR/EulerAMR.cpp:169-350)."""
    dims = 1 if p0.ndim == 2 else 2
    c, f = O.amr_flags(system, p0, dx, tol, g)
    dt = O.stable_dt(system, p0, dx, cfl, 0.0, T, 0, g)
    m = c.reshape(p0.shape[:-1])
    if dims == 1:
        cp = O.sweep(system, p0, 0, 2, dx, dt, 0.0, 1, g, mask=m)
        fp = np.repeat(p0, 2, axis=0)
    else:
        cp = O.sweep(system, p0, 0, 2, dx, dt * 0.5, 0.0, 1, g, mask=m)
        cp = O.sweep(system, cp, 1, 2, dx, dt, 0.0, 1, g, mask=m)
        cp = O.sweep(system, cp, 0, 2, dx, dt * 0.5, 0.0, 1, g, mask=m)
        fp = np.repeat(np.repeat(p0, 2, axis=0), 2, axis=1)
    cpf, fpf = cp.reshape(-1, 5).copy(), fp.reshape(-1, 5).copy()
    ny, nx = (1, p0.shape[0]) if dims == 1 else p0.shape[:2]
    fnx = 2 * nx
    for i in range(ny):
        for j in range(nx):
            k = i * nx + j
            kids = [2 * j, 2 * j + 1] if dims == 1 else \
                [(2 * i) * fnx + 2 * j, (2 * i) * fnx + 2 * j + 1, (2 * i + 1) * fnx + 2 * j, (2 * i + 1) * fnx + 2 * j + 1]
            if not c[k]:
                us = [O.cons(system, fpf[q], g) for q in kids]
                avg = 0.5 * (us[0] + us[1]) if dims == 1 else 0.25 * (((us[0] + us[1]) + us[2]) + us[3])
                cpf[k] = O.prim(system, avg, g)
            for q in kids:
                if not f[q]:
                    fpf[q] = cpf[k]
    cp2, c2, f2 = O.amr_derefine(system, cpf.reshape(cp.shape), fpf.reshape(fp.shape), dx, tol, g, c, f)
    return cp2, fpf.reshape(fp.shape), c2, f2


@pytest.mark.parametrize("tag,system", [("newton", 0), ("sr", 1)])
def test_amr_flag_and_derefine_passes(oracle, golden, tag, system):
    g = cases.SYS_GAMMA[system]
    n = 0
    for k in _keys(golden, f"amr_{tag}_"):
        s = golden[k + "_in"]
        tol = float(k.split("_t")[-1])
        cp, fp, c, f = _emulate_amr_first_step(oracle, system, s, 1.0 / s.shape[-2], 0.9, 1e-5, tol, g)
        assert bit_equal(c, golden[k + "_cflags"]) and bit_equal(f, golden[k + "_fflags"]), k
        assert bit_equal(cp.reshape(-1), golden[k + "_coarse"]) and bit_equal(fp.reshape(-1), golden[k + "_fine"]), k
        n += 1
    assert n == 6


def amr_golden():
    import os
    return dict(np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "amr_golden.npz")))


def test_amr_level1_driver(oracle):
    """The oracle's Level-1 AMR driver against the reference's solveLevel1AMR / solve2DLevel1AMR runs
    (Newtonian and SR, 1D and 2D, FORCE and SLIC; several coarse steps with fine sub-cycles)."""
    G = amr_golden()
    keys = [k for k in _keys(G, "amr") if k[3:].isdigit()]  # Level-1 runs: amr<k>
    assert len(keys) == 8
    for k in keys:
        s = G[k + "_in"]
        system, dims, T, order, tol, nsteps = G[k + "_args"]
        system, order = int(system), int(order)
        n, nf, cp, fp, cf, ff = oracle.amr_level1(system, s, 1.0 / s.shape[-2], 0.9, T, tol, order,
                                                  cases.SYS_GAMMA[system])
        assert n == int(nsteps) and nf > n, k
        assert bit_equal(cp, G[k + "_coarse"]) and bit_equal(fp, G[k + "_fine"]), k
        assert bit_equal(cf, G[k + "_cflags"]) and bit_equal(ff, G[k + "_fflags"]), k


def test_amr_level2_driver(oracle):
    """The oracle's Level-2 driver (three levels) against the reference's solveLevel2AMR /
    solve2DLevel2AMR runs: every grid, flag set and the coarse step count, bit for bit."""
    G = amr_golden()
    keys = [k for k in _keys(G, "amr2_") if k[5:].isdigit()]  # Level-2 runs: amr2_<k>
    assert len(keys) == 8
    for k in keys:
        s = G[k + "_in"]
        system, dims, T, order, tol, nsteps = G[k + "_args"]
        system, order = int(system), int(order)
        n, counts, cp, mp, fp, cf, mf, ff = oracle.amr_level2(system, s, 1.0 / s.shape[-2], 0.9, T, tol, order,
                                                              cases.SYS_GAMMA[system])
        assert n == int(nsteps) and counts[1] > n, k
        for name, got in (("coarse", cp), ("mid", mp), ("fine", fp), ("cflags", cf), ("mflags", mf), ("fflags", ff)):
            assert bit_equal(got, G[f"{k}_{name}"]), (k, name)


def _interface_cases():
    d = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "interface_golden.npz"))
    return d, sorted(k[:-5] for k in d.files if k.endswith("_args"))


def test_oracle_interface_functions_match_reference(oracle):
    """The oracle's per-interface solver functions (orc_interface_eval) reproduce the reference's own
    static functions (computeXSLICFlux, computeLaxFriedrichsFlux, evolveStateByHalfXTimeStep, the
    forcing solver's cell update, ...) bit for bit on every golden case: every op of every system,
    every limiter, both sides, a Schwarzschild and a spinning hole."""
    d, keys = _interface_cases()
    assert len(keys) == 162
    for k in keys:
        a = d[k + "_args"]
        op, system, g, dx, dt, bias, lim, frac, side = a[:9]
        xyz = d[k + "_xyz"] if k + "_xyz" in d.files else None
        got = oracle.interface(int(op), int(system), d[k + "_in"], xyz, g, a[9:], dx, dt, bias, int(lim), frac, int(side))
        want = d[k + "_out"]
        assert np.isfinite(want).all(), k
        assert np.array_equal(got.view(np.uint64), want.view(np.uint64)), k


def test_oracle_spacetime_and_eigenvalues_match_reference(oracle):
    """Every public BlackHoleSpacetime quantity (BlackHoleEuler/BlackHoleSpacetime.hpp:16-42) and the
    three BlackHoleEulerEigenvalues vectors, restated by the oracle, against the reference's own
    outputs around a Schwarzschild and a spinning hole."""
    d, _ = _interface_cases()
    for hole in ("schw", "kerr"):
        q, bh, h = d[f"st_{hole}_xyz"], d[f"st_{hole}_bh"], float(d[f"st_{hole}_h"])
        want = d[f"st_{hole}_out"]
        assert want.shape == (64, 125) and np.isfinite(want).all()
        assert np.array_equal(oracle.spacetime_record(q, h, bh).view(np.uint64), want.view(np.uint64)), hole
        want = d[f"eig_{hole}_out"]
        got = oracle.gr_eigenvalues(d[f"eig_{hole}_in"], q, 5.0 / 3.0, bh)
        assert np.array_equal(got.view(np.uint64), want.view(np.uint64)), hole
