"""Minimal launch driver for profiler captures of single kernels.

    python -m cosmos_gb300.profile --kernel sweep --n 4096 --precision fp32 --axis 0 --launches 3
    python -m cosmos_gb300.profile --kernel step --n 4096 --precision fp32 --launches 4

Creates one grid of the config-2 problem (four-quadrant data, periodic, MinBee) and launches the
requested kernels a few times, so that a profiler can capture exactly those launches on a
bounded device footprint (two state buffers plus one staging buffer).
"""
import argparse
import os
import sys

import numpy as np


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--kernel", choices=["sweep", "step", "rk"], default="sweep")
    ap.add_argument("--system", type=int, default=0)
    ap.add_argument("--precision", choices=["fp32", "fp64"], default="fp32")
    ap.add_argument("--n", type=int, default=4096)
    ap.add_argument("--axis", type=int, default=0)
    ap.add_argument("--order", type=int, default=2)
    ap.add_argument("--launches", type=int, default=3)
    a = ap.parse_args()
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import cosmos_gb300 as cg

    n = a.n
    rng = np.random.default_rng(2)
    q = np.zeros((4, 5))
    q[:, 0] = rng.uniform(0.1, 1.5, 4)
    q[:, 1] = rng.uniform(-1.0, 1.0, 4)
    q[:, 2] = rng.uniform(-1.0, 1.0, 4)
    q[:, 4] = rng.uniform(0.03, 1.5, 4)
    s = np.zeros((n, n, 5))
    h = n // 2
    s[:h, :h], s[:h, h:], s[h:, :h], s[h:, h:] = q
    prec = cg.FP32 if a.precision == "fp32" else cg.FP64
    bc = cg.BC_PERIODIC if a.system != cg.GR else cg.BC_TRANSMISSIVE
    g = cg.Grid(a.system, (n, n), 1.0 / n, 1.4 if a.system == 0 else 5.0 / 3.0, prec, bc)
    g.set_prim(s)
    dt = 0.25 / n
    if a.kernel == "sweep":
        for _ in range(a.launches):
            g.sweep(a.axis, a.order, dt, 0.0, cg.MINBEE)
    elif a.kernel == "rk":
        for _ in range(a.launches):
            g.rk_source(dt, 0.0, 1)
    else:
        g.run_begin(2, 0.9, 1e30, 0.0, cg.MINBEE)
        g.run_steps(a.launches)
        g.run_end()
    g.ctx.synchronize()
    print(f"ok: {a.launches} x {a.kernel} ({a.precision}, n={n})")


if __name__ == "__main__":
    main()
