"""Writes amr_level1_golden.npz: runs of the reference's Level-1 AMR drivers
(EulerAMR::solveLevel1AMR / solve2DLevel1AMR, RelativisticEulerAMR twins; AMR/EulerAMR.cpp:169-592)
over many coarse steps with fine sub-cycles, from the reference compiled from its own sources
(oracle/ref/Makefile -> oracle/_ref/libcosmos_ref.so).  Needs the reference checkout; the committed
fixture is what the tests read.

    make -C oracle/ref && python tests/golden/make_amr_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from oracle.pyoracle import Reference  # noqa: E402
import cases  # noqa: E402

# (system, dims, shape, final time, order, tolerance)
CASES = [(0, 1, (64,), 0.2, 2, 2.0), (0, 1, (64,), 0.2, 1, 5.0), (0, 2, (20, 24), 0.1, 2, 3.0),
         (0, 2, (20, 24), 0.1, 1, 5.0), (1, 1, (64,), 0.2, 2, 2.0), (1, 1, (64,), 0.2, 1, 5.0),
         (1, 2, (20, 24), 0.1, 2, 3.0), (1, 2, (20, 24), 0.1, 1, 5.0)]


def amr_state(shape, system, rng):
    """Two-level density and pressure jumps with a sinusoid and seeded noise in density and velocity."""
    x = np.linspace(0, 1, shape[-1])
    s = np.zeros(shape + (5,))
    s[..., 0] = 1.0 + 0.3 * np.sin(6 * x) + np.where(x > 0.5, 0.8, 0.0) + 0.1 * rng.uniform(0, 1, shape)
    s[..., 1] = (0.3 if system == 0 else 0.2) * rng.uniform(-1, 1, shape)
    if len(shape) == 2:
        s[..., 2] = 0.1 * rng.uniform(-1, 1, shape)
    s[..., 4] = 1.0 + 0.5 * np.where(x < 0.3, 1.0, 0.0)
    return s


def main():
    R = Reference()
    rng = np.random.default_rng(2024)
    out = {}
    for k, (system, dims, shape, T, order, tol) in enumerate(CASES):
        s = amr_state(shape, system, rng)
        n, cp, fp, cf, ff = R.amr_level1(system, s, 1.0 / shape[-1], 0.9, T, tol, order, cases.SYS_GAMMA[system])
        key = f"amr{k}"
        out[key + "_in"] = s
        out[key + "_args"] = np.array([system, dims, T, order, tol, n], dtype=np.float64)
        out[key + "_coarse"], out[key + "_fine"], out[key + "_cflags"], out[key + "_fflags"] = cp, fp, cf, ff
        print(key, system, dims, shape, "coarse steps", n, "refined fine cells", int(ff.sum()))
    path = os.path.join(HERE, "amr_level1_golden.npz")
    np.savez_compressed(path, **out)
    print(f"wrote {path}: {len(out)} arrays, {os.path.getsize(path)} bytes")


if __name__ == "__main__":
    main()
