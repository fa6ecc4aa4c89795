"""Minimal launch driver for profiler captures of single kernels.

    python bench_profile.py --kernel sweep --n 4096 --precision fp32 --axis 0 --launches 3
    python bench_profile.py --kernel step --n 4096 --precision fp32 --launches 4
    python bench_profile.py --kernel step --system 2 --n 1024 --warm 60 --launches 1
    python bench_profile.py --kernel adjoint --n 1024 --precision fp32 --launches 2
    python bench_profile.py --kernel adjoint --system 2 --n 256 --precision fp64 --subcycles 1 --launches 1
    python bench_profile.py --kernel batch --grids 64 --launches 2

Creates one grid of the system's benchmark problem (Newtonian: four-quadrant Riemann
data, periodic; SR: Kelvin-Helmholtz layers, periodic; GR: accretion onto a
Schwarzschild hole, transmissive; MinBee) and launches the requested kernels a few times, so that a profiler can capture exactly those launches on a
bounded device footprint (two state buffers plus one staging buffer).  `adjoint` runs the
gradient of `launches` SLIC steps (checkpoint every step: launches X and Y sweep adjoints per
step; FP64 SR and black-hole grids run the relativistic adjoints, the latter with `subcycles` RK
source half-steps around each flux step); `batch` runs `launches` chunks of 10 steps of the first `grids` grids of the batched
workload (256 grids, sides log-uniform in [128, 2048]).
"""
import argparse
import os
import sys

import numpy as np


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--kernel", choices=["sweep", "step", "rk", "adjoint", "batch"], default="sweep")
    ap.add_argument("--grids", type=int, default=64)
    ap.add_argument("--system", type=int, default=0)
    ap.add_argument("--precision", choices=["fp32", "fp64"], default="fp32")
    ap.add_argument("--n", type=int, default=4096)
    ap.add_argument("--axis", type=int, default=0)
    ap.add_argument("--order", type=int, default=2)
    ap.add_argument("--launches", type=int, default=3)
    ap.add_argument("--subcycles", type=int, default=1, help="`adjoint` on a black-hole grid: RK source half-steps")
    ap.add_argument("--warm", type=int, default=0,
                    help="`step` only: steps run before the captured ones (evolved states)")
    ap.add_argument("--c2p64-above", type=float, default=2.0,
                    help="FP32 SR and black-hole grids: Lorentz factor above which a primitive recovery "
                         "finishes in FP64 (0: every recovery)")
    ap.add_argument("--shape", type=int, nargs=3, default=[256, 64, 1], metavar=("NT", "SEG", "CAP"),
                    help="`batch`: tile shape (threads per block, Y rows per item, register cap)")
    a = ap.parse_args()
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    import cosmos_gb300 as cg

    if a.kernel == "batch":
        sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "tests"))
        import cases
        shapes = cases.batch_shapes()[:a.grids]
        b = cg.Batch(shapes, [1.0 / sh[-1] for sh in shapes], 1.4, cg.FP32, cg.BC_TRANSMISSIVE)
        for k, sh in enumerate(shapes):
            b.set_prim(k, cases.riemann(sh, 1000 + k))
        b.run_begin(0.9, 1e30, 0.0, cg.MINBEE)
        b.set_shape(*a.shape)
        b.run_steps(10 * a.launches)
        b.run_end()
        b.ctx.synchronize()
        print(f"ok: {a.launches} x batch chunk ({len(shapes)} grids, {b.cells} cells)")
        return
    n = a.n
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "tests"))
    import cases
    prec = cg.FP32 if a.precision == "fp32" else cg.FP64
    bh = None
    dx = 1.0 / n
    if a.system == cg.NEWTONIAN:  # four-quadrant Riemann data
        s = cases.four_quadrant(n, 2)
    elif a.system == cg.SR:  # Kelvin-Helmholtz layers
        s = cases.kelvin_helmholtz(n, 3)
    else:  # accretion: [-10, 10]^2 with the hole at the centre, M = 1
        rng = np.random.default_rng(4)
        s = np.zeros((n, n, 5))
        s[..., 0] = np.exp(0.01 * rng.standard_normal((n, n)))
        s[..., 4] = 0.01
        dx = 20.0 / n
        bh = cg.BlackHoleSpacetime(1.0, 0.0, 10.0, 10.0, 0.0)
    bc = cg.BC_PERIODIC if a.system != cg.GR else cg.BC_TRANSMISSIVE
    g = cg.Grid(a.system, (n, n), dx, 1.4 if a.system == 0 else 5.0 / 3.0, prec, bc, bh,
                sr_c2p64_above=a.c2p64_above)
    g.set_prim(s)
    dt = 0.25 * dx
    if a.kernel == "sweep":
        for _ in range(a.launches):
            g.sweep(a.axis, a.order, dt, 0.0, cg.MINBEE)
    elif a.kernel == "adjoint":
        tgt = s[..., 0] * 0.9
        g.adjoint(tgt, a.launches, 0.8, 0.0, cg.MINBEE, checkpoint_every=1, subcycles=a.subcycles)
    elif a.kernel == "rk":
        for _ in range(a.launches):
            g.rk_source(dt, 0.0, 1)
    else:  # the workload's solve: MinBee (Newtonian 4096^2, SR 2048^2); van Leer and the RK source (GR 1024^2)
        lim = cg.VANLEER if a.system == cg.GR else cg.MINBEE
        g.run_begin(2, 0.9, 1e30, 0.0, lim)
        if a.warm:
            g.run_steps(a.warm)
        g.run_steps(a.launches)
        g.run_end()
    g.ctx.synchronize()
    print(f"ok: {a.launches} x {a.kernel} ({a.precision}, n={n})")


if __name__ == "__main__":
    main()
