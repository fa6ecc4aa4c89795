"""Writes dat_golden.npz: the reference's own scenario drivers (Tests/*.cpp: EulerTests,
RelativisticEulerTests, BlackHoleEulerTests, EulerAMRTests, RelativisticEulerAMRTests) run at small
sizes, and its solution writers (outputSolution, outputSolution2D, the black-hole and AMR writers)
on seeded level data, with the text of every .dat file they write.  The reference is compiled from
its own sources with its fixed output paths redirected into a scratch directory
(oracle/ref/Makefile, oracle/ref/redirect_ofstream.hpp).  Needs the reference checkout; the
committed fixture is what the tests read.

    make -C oracle/ref && python tests/golden/make_dat_golden.py
"""
import ctypes
import os
import shutil
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(HERE))

FILES = ("density.dat", "xVelocity.dat", "yVelocity.dat", "zVelocity.dat", "pressure.dat")

# (reference scenario, cellCount, order, subcycles, AMRTolerance, AMRLevel)
SCENARIOS = []
for order in (1, 2):
    for t in (1, 2, 3):
        SCENARIOS.append((f"EulerTests::solveToroTest{t}", 64, order, 1, 0.0, 1))
    for fn in ("solveMildlyRelativisticShock", "solveStronglyRelativisticBlast", "solvePerturbedDensityTest"):
        SCENARIOS.append((f"RelativisticEulerTests::{fn}", 64, order, 1, 0.0, 1))
    for fn in ("solve1DSphericalAccretionTest", "solve1DSpinningSphericalAccretionTest"):
        SCENARIOS.append((f"BlackHoleEulerTests::{fn}", 40, order, 1, 0.0, 1))
for t in (1, 2, 3):
    SCENARIOS.append((f"EulerTests::solve2DToroTest{t}", 10, 2, 1, 0.0, 1))
for fn in ("solve2DMildlyRelativisticShock", "solve2DStronglyRelativisticBlast", "solve2DPerturbedDensityTest"):
    SCENARIOS.append((f"RelativisticEulerTests::{fn}", 10, 2, 1, 0.0, 1))
for fn in ("solve2DSphericalAccretionTest", "solve2DSpinningSphericalAccretionTest", "solve2DSpheroidalAccretionTest",
           "solve2DSpinningSpheroidalAccretionTest"):
    SCENARIOS.append((f"BlackHoleEulerTests::{fn}", 10, 2, 1, 0.0, 1))
for level in (1, 2):
    SCENARIOS.append(("EulerAMRTests::solveToroTest1AMR", 48, 2, 1, 20.0, level))
    SCENARIOS.append(("EulerAMRTests::solve2DToroTest1AMR", 8, 2, 1, 3.0, level))
    for fn in ("solveMildlyRelativisticShock", "solveStronglyRelativisticBlast", "solvePerturbedDensityTest"):
        SCENARIOS.append((f"RelativisticEulerAMRTests::{fn}", 48, 2, 1, 20.0, level))
    for fn in ("solve2DMildlyRelativisticShock", "solve2DStronglyRelativisticBlast", "solve2DPerturbedDensityTest"):
        SCENARIOS.append((f"RelativisticEulerAMRTests::{fn}", 8, 2, 1, 3.0, level))

# the reference's own main.cpp runs the accretion tests with subcyclingIterations = 0 (no source step)
SCENARIOS.append(("BlackHoleEulerTests::solve1DSphericalAccretionTest", 40, 2, 0, 0.0, 1))
SCENARIOS.append(("BlackHoleEulerTests::solve2DSpinningSphericalAccretionTest", 10, 2, 0, 0.0, 1))

# writer cases: (kind, system, dims, ny, nx); kind 0 plain, 1 Level-1 AMR, 2 Level-2 AMR
WRITERS = [(0, 0, 1, 1, 23), (0, 1, 2, 7, 9), (0, 2, 1, 1, 31), (0, 2, 2, 9, 11), (1, 0, 1, 1, 29), (1, 0, 2, 6, 7),
           (1, 1, 2, 6, 7), (2, 0, 1, 1, 37), (2, 1, 1, 1, 37), (2, 0, 2, 7, 8), (2, 1, 2, 7, 8)]


def writer_inputs(kind, dims, ny, nx, rng):
    """Seeded level data with values of many magnitudes and flags that reach every writer branch."""
    r = 4 if dims == 2 else 2
    n0 = nx * (ny if dims == 2 else 1)
    sizes = [n0, n0 * r, n0 * r * r]
    levels = []
    for n in sizes:
        mag = 10.0 ** rng.integers(-7, 6, size=(n, 5))
        levels.append(rng.uniform(-1, 1, size=(n, 5)) * mag)
    flags = [rng.integers(0, 2, size=n).astype(np.uint8) for n in sizes]
    if kind == 2:  # make the all-children-on branches likely
        for q in range(sizes[2]):
            if rng.uniform() < 0.6:
                flags[2][q] = 1
    return levels, flags


def main():
    L = ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", "libcosmos_ref.so"))
    L.ref_tests_set_dir.argtypes = [ctypes.c_char_p]
    L.ref_tests_run.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                ctypes.c_int]
    L.ref_tests_run.restype = ctypes.c_int
    L.ref_tests_write.argtypes = [ctypes.c_int] * 5 + [ctypes.c_void_p] * 7
    scratch = os.path.join(HERE, ".dat_scratch")
    out = {}

    def collect(key):
        for f in FILES:
            p = os.path.join(scratch, f)
            if os.path.exists(p):
                out[f"{key}/{f}"] = np.frombuffer(open(p, "rb").read(), dtype=np.uint8)

    def fresh():
        shutil.rmtree(scratch, ignore_errors=True)
        os.makedirs(scratch)
        L.ref_tests_set_dir(scratch.encode())

    for k, (name, n, order, sub, tol, level) in enumerate(SCENARIOS):
        fresh()
        rc = L.ref_tests_run(name.encode(), n, order, sub, tol, level)
        assert rc == 0, name
        key = f"scenario{k}"
        out[key + "/args"] = np.frombuffer(f"{name} {n} {order} {sub} {tol!r} {level}".encode(), dtype=np.uint8)
        collect(key)
        print(key, name, n, order, tol, level, sum(v.size for kk, v in out.items() if kk.startswith(key + "/")))
    rng = np.random.default_rng(77)
    bh = np.array([0.05, 0.3, 0.5, 0.5, 0.0])
    for k, (kind, system, dims, ny, nx) in enumerate(WRITERS):
        fresh()
        levels, flags = writer_inputs(kind, dims, ny, nx, rng)
        ptr = lambda a: a.ctypes.data
        L.ref_tests_write(kind, system, dims, ny, nx, ptr(levels[0]), ptr(levels[1]), ptr(levels[2]), ptr(flags[0]),
                          ptr(flags[1]), ptr(flags[2]), ptr(bh))
        key = f"writer{k}"
        out[key + "/args"] = np.array([kind, system, dims, ny, nx])
        out[key + "/bh"] = bh
        for q in range(3):
            out[f"{key}/level{q}"] = levels[q]
            out[f"{key}/flags{q}"] = flags[q]
        collect(key)
    shutil.rmtree(scratch, ignore_errors=True)
    path = os.path.join(HERE, "dat_golden.npz")
    np.savez_compressed(path, **out)
    print(f"wrote {path}: {len(out)} arrays, {os.path.getsize(path)} bytes")


if __name__ == "__main__":
    main()
