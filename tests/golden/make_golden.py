"""Generate the golden fixtures in tests/golden/ by running the reference itself.

The reference (JonathanGorard/Cosmos) is compiled from its own sources by oracle/ref/Makefile into
oracle/_ref/libcosmos_ref.so; this script drives its public static API through that build and
stores inputs and outputs as .npz files.  The fixtures let the oracle be checked against the
reference on machines where the reference checkout is absent (the GPU host).

    make -C oracle/ref && python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, os.path.dirname(HERE))

from oracle.pyoracle import Reference  # noqa: E402
import cases  # noqa: E402


def main():
    R = Reference()
    rng = np.random.default_rng(20240611)
    out = {}

    # Sod shock tube: SLIC van Leer, N=1000, CFL 0.9, t=0.25
    p0 = cases.sod(1000)
    p, n = R.solve(0, p0, 2, 1.0 / 1000, 0.9, 0.25, 0.0, 1, 1.4)
    out["sod1000_final"] = p
    out["sod1000_steps"] = np.array(n)

    # Newtonian and SR sweeps: every axis/order/limiter/boundary on small grids
    for system, tag in ((0, "newton"), (1, "sr")):
        g = cases.SYS_GAMMA[system]
        for dims in (1, 2):
            shape = (17,) if dims == 1 else (7, 9)
            for order in (1, 2):
                for lim in ((0, 1, 2) if order == 2 else (1,)):
                    for bc in (0, 1):
                        for axis in ((0,) if dims == 1 else (0, 1)):
                            bias = 0.3 if (lim == 2 and bc == 0) else 0.0
                            s = cases.state(system, rng, shape)
                            key = f"{tag}_d{dims}_o{order}_l{lim}_bc{bc}_a{axis}"
                            out[key + "_in"] = s
                            out[key + "_out"] = R.sweep(system, s, axis, order, 1.0 / 64, 0.004, bias, lim, g, bc)
                            out[key + "_bias"] = np.array(bias)
        # solve: 2D Strang SLIC on a four-quadrant problem
        s = cases.four_quadrant(12, 7) if system == 0 else cases.sr_state(rng, (10, 12))
        p, n = R.solve(system, s, 2, 1.0 / 12, 0.9, 0.05, 0.0, 2, g)
        out[f"{tag}_solve2d_in"], out[f"{tag}_solve2d_out"], out[f"{tag}_solve2d_steps"] = s, p, np.array(n)
        s = cases.state(system, rng, (24,))
        p, n = R.solve(system, s, 1, 1.0 / 24, 0.8, 0.05, 0.0, 1, g)
        out[f"{tag}_solve1d_force_in"], out[f"{tag}_solve1d_force_out"] = s, p
        out[f"{tag}_solve1d_force_steps"] = np.array(n)
        for dims, shape in ((1, (19,)), (2, (8, 11))):
            s = cases.state(system, rng, shape)
            out[f"{tag}_dt_d{dims}_in"] = s
            out[f"{tag}_dt_d{dims}"] = np.array([R.stable_dt(system, s, 0.01, 0.9, 0.0, 1.0, it, g) for it in (0, 7)])

    # GR: sweeps around the hole, RK source, dt, one full step
    g = cases.SYS_GAMMA[2]
    for bhname, bh in (("bh", cases.GR_BH), ("spin", cases.GR_BH_SPIN)):
        for dims in (1, 2):
            n = 12
            shape = (n,) if dims == 1 else (n, n)
            dx = 1.0 / n
            for order in (1, 2):
                for axis in ((0,) if dims == 1 else (0, 1)):
                    s = cases.gr_state(rng, shape)
                    key = f"gr_{bhname}_d{dims}_o{order}_a{axis}"
                    out[key + "_in"] = s
                    out[key + "_out"] = R.sweep(2, s, axis, order, dx, 0.002, 0.0, 1, g, bh=bh)
            s = cases.gr_state(rng, shape)
            out[f"gr_{bhname}_rk_d{dims}_in"] = s
            out[f"gr_{bhname}_rk_d{dims}_out"] = R.rk_source(s, dx, 0.002, 0.0, 1, g, bh)
            out[f"gr_{bhname}_dt_d{dims}"] = np.array(R.stable_dt(2, s, dx, 0.9, 0.0, 1.0, 0, g, bh=bh))
    s = cases.gr_state(rng, (10, 10))
    bh = (1.0, 0.0, 10.0, 10.0, 0.0)
    p, n = R.solve(2, s, 2, 2.0, 0.9, 0.3, 0.0, 1, g, subcycles=1, bh=bh)
    out["gr_solve_in"], out["gr_solve_out"], out["gr_solve_steps"] = s, p, np.array(n)

    # metric probes (determinant, lapse, shift, metrics, K_ij, ...)
    pts = np.array([[0.3, 0.2, 0.0], [0.62, 0.41, 0.0], [0.5, 0.75, 0.05], [9.0, 12.5, 0.0], [13.0, 8.0, 0.0]])
    out["gr_metric_pts"] = pts
    for bhname, bh in (("bh", cases.GR_BH), ("spin", cases.GR_BH_SPIN), ("cfg4", (1.0, 0.0, 10.0, 10.0, 0.0))):
        out[f"gr_metric_{bhname}"] = np.array([R.gr_metric(x, y, z, 0.05, bh) for x, y, z in pts])

    # AMR Level-1, one coarse step shorter than the 1e-4 sub-cycling slack (no fine steps)
    for system, tag in ((0, "newton"), (1, "sr")):
        gg = cases.SYS_GAMMA[system]
        for dims in (1, 2):
            shape = (40,) if dims == 1 else (12, 14)
            x = np.linspace(0, 1, shape[-1])
            s = np.zeros(shape + (5,))
            s[..., 0] = 1.0 + 0.3 * np.sin(6 * x) + np.where(x > 0.6, 0.8, 0.0) + (0.2 * rng.uniform(0, 1, shape) if dims == 2 else 0)
            s[..., 1] = 0.1 * rng.uniform(-1, 1, shape)
            s[..., 4] = 1.0 + 0.2 * np.cos(5 * x)
            for tol in (1.0, 3.0, 8.0):
                _, cp, fp, cf, ff = R.amr_level1(system, s, 1.0 / shape[-1], 0.9, 1e-5, tol, 2, gg)
                key = f"amr_{tag}_d{dims}_t{int(tol)}"
                out[key + "_in"] = s
                out[key + "_coarse"], out[key + "_fine"], out[key + "_cflags"], out[key + "_fflags"] = cp, fp, cf, ff

    path = os.path.join(HERE, "reference_golden.npz")
    np.savez_compressed(path, **out)
    print(f"wrote {path}: {len(out)} arrays, {os.path.getsize(path)} bytes")


if __name__ == "__main__":
    main()
