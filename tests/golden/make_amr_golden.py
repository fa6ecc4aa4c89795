"""Writes amr_golden.npz: runs of the reference's Level-1 AMR drivers
(EulerAMR::solveLevel1AMR / solve2DLevel1AMR, RelativisticEulerAMR twins; AMR/EulerAMR.cpp:169-592)
over many coarse steps with fine sub-cycles (keys amr<k>_*), and of its Level-2 drivers
(solveLevel2AMR / solve2DLevel2AMR, AMR/EulerAMR.cpp:593-1379; keys amr2_<k>_*), from the reference
compiled from its own sources (oracle/ref/Makefile -> oracle/_ref/libcosmos_ref.so).  Needs the
reference checkout; the committed fixture is what the tests read.

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
# Level-2 runs: (system, dims, shape, final time, order, tolerance)
CASES2 = [(0, 1, (40,), 0.12, 2, 2.0), (0, 1, (40,), 0.12, 1, 0.5), (0, 2, (8, 10), 0.08, 2, 2.0),
          (0, 2, (8, 10), 0.08, 1, 0.5), (1, 1, (40,), 0.12, 2, 2.0), (1, 1, (40,), 0.12, 1, 0.5),
          (1, 2, (8, 10), 0.08, 2, 2.0), (1, 2, (8, 10), 0.08, 1, 0.5)]


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
    rng2 = np.random.default_rng(2025)
    for k, (system, dims, shape, T, order, tol) in enumerate(CASES2):
        s = amr_state(shape, system, rng2)
        n, cp, mp, fp, cf, mf, ff = R.amr_level2(system, s, 1.0 / shape[-1], 0.9, T, tol, order,
                                                 cases.SYS_GAMMA[system])
        key = f"amr2_{k}"
        out[key + "_in"] = s
        out[key + "_args"] = np.array([system, dims, T, order, tol, n], dtype=np.float64)
        out[key + "_coarse"], out[key + "_mid"], out[key + "_fine"] = cp, mp, fp
        out[key + "_cflags"], out[key + "_mflags"], out[key + "_fflags"] = cf, mf, ff
        print(key, system, dims, shape, "coarse steps", n, "intermediate on", int(mf.sum()), "fine on", int(ff.sum()))
    path = os.path.join(HERE, "amr_golden.npz")
    np.savez_compressed(path, **out)
    print(f"wrote {path}: {len(out)} arrays, {os.path.getsize(path)} bytes")


if __name__ == "__main__":
    main()
