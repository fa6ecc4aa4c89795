"""The C++ drop-in shim (include/cosmos_gb300_compat.hpp): a reference-style driver compiles against it
(CPU check) and, on the GPU, produces the oracle's results bit for bit."""
import os
import subprocess

import numpy as np
import pytest

import cases
from conftest import ROOT, bit_equal


def _compile(out, syntax_only=False):
    src = os.path.join(ROOT, "tests", "cpp", "compat_driver.cpp")
    cmd = ["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), src]
    if syntax_only:
        cmd += ["-fsyntax-only"]
    else:
        lib = os.path.join(ROOT, "cosmos_gb300")
        cmd += ["-o", out, "-L", lib, "-lcosmos_gb300", f"-Wl,-rpath,{lib}"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)


def test_compat_header_compiles():
    _compile(None, syntax_only=True)


@pytest.mark.gpu
def test_compat_driver_matches_oracle(cosmos_lib, oracle, tmp_path):
    exe = str(tmp_path / "compat_driver")
    _compile(exe)
    r = subprocess.run([exe, str(tmp_path)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    load = lambda n, shape: np.fromfile(str(tmp_path / n), dtype=np.float64).reshape(shape)

    want, _, _, _ = oracle.solve(0, cases.sod(1000), 2, 1e-3, 0.9, 0.25, 0.0, 1, 1.4)
    assert bit_equal(load("sod.bin", (1000, 5)), want)

    n = 40
    s = np.zeros((n, n, 5))
    for i in range(n):
        for j in range(n):
            r2 = (i - 0.5 * n) ** 2 + (j - 0.5 * n) ** 2
            s[i, j] = (1.0, 0, 0, 0, 1.0) if r2 <= (0.2 * n) ** 2 else (0.125, 0, 0, 0, 0.1)
    want, _, _, _ = oracle.solve(0, s, 1, 1.0 / n, 0.9, 0.05, 0.0, 1, 1.4)
    assert bit_equal(load("cyl_force.bin", (n, n, 5)), want)
    assert bit_equal(load("cyl_xsweep.bin", (n, n, 5)), oracle.sweep(0, s, 0, 2, 1.0 / n, 0.001, 0.0, 2, 1.4))

    m = 200
    s = np.array([(10.0, 0, 0, 0, 13.3) if i <= 0.5 * m else (1.0, 0, 0, 0, 1e-6) for i in range(m)])
    want, _, _, _ = oracle.solve(1, s, 2, 1.0 / m, 0.8, 0.1, 0.0, 1, 5.0 / 3.0)
    assert bit_equal(load("sr_shock.bin", (m, 5)), want)

    k = 60
    s = np.array([(10.0, 0, 0, 0, 0.1) if 0.1 * k <= i <= 0.9 * k else (0.1, 0, 0, 0, 0.1) for i in range(k)])
    want, _, _, _ = oracle.solve(2, s, 2, 1.0 / k, 0.9, 0.02, 0.0, 1, 5.0 / 3.0, subcycles=1,
                                 bh=(0.05, 0.0, 0.5, 0.0, 0.0))
    assert bit_equal(load("bh_accretion.bin", (k, 5)), want)

    n = 20
    s = np.zeros((n, n, 5))
    for i in range(n):
        for j in range(n):
            r2 = (i - 0.5 * n) ** 2 + (j - 0.5 * n) ** 2
            s[i, j] = (1.0, 0, 0, 0, 1.0) if r2 <= (0.2 * n) ** 2 else (0.125, 0, 0, 0, 0.1)
    _, _, cp, fp, cf, ff = oracle.amr_level1(0, s, 1.0 / n, 0.9, 0.05, 4.0, 2, 1.4)
    assert bit_equal(load("amr_coarse.bin", (n * n * 5,)), cp)
    assert bit_equal(load("amr_fine.bin", (4 * n * n * 5,)), fp)
    assert bit_equal(load("amr_flags.bin", (5 * n * n,)), np.concatenate([cf, ff]).astype(np.float64))

    m = 50
    s = np.array([(10.0, 0, 0, 0, 13.3) if i <= 0.5 * m else (1.0, 0, 0, 0, 1e-6) for i in range(m)])
    _, _, cp, mp, fp, cf, mf, ff = oracle.amr_level2(1, s, 1.0 / m, 0.8, 0.1, 20.0, 2, 5.0 / 3.0)
    want = np.concatenate([cp, mp, fp, cf, mf, ff]).astype(np.float64)
    assert bit_equal(load("amr2_sr.bin", want.shape), want)
