"""Host-only parts of the C++ shim (include/cosmos_gb300_compat.hpp): boundary-cell insertion as in
Solvers/EulerSolvers.cpp:3-85 (corners of 2D grids keep default-constructed states, density 1),
the spacetime's excision test (BlackHoleEuler/BlackHoleSpacetime.cpp:372-386) and the status line
(Solvers/EulerSolvers.cpp:225-228)."""
import math
import os
import subprocess

from conftest import ROOT


def test_boundary_cells_excision_and_status(tmp_path):
    exe = str(tmp_path / "compat_host")
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "compat_host.cpp"), "-o", exe], check=True)
    lines = subprocess.run([exe], check=True, capture_output=True, text=True).stdout.splitlines()
    d = {l.split()[0]: [float(v) for v in l.split()[1:]] for l in lines[:4]}
    assert d["1d1"] == [0, 0, 1, 2, 3, 4, 4]
    assert d["1d2"] == [1, 0, 0, 1, 2, 3, 4, 4, 3]

    def padded(b):
        rows, cols = 3 + 2 * b, 4 + 2 * b
        out = [[1.0] * cols for _ in range(rows)]
        src = lambda i, j: 10 * i + j
        mir = (lambda k, n: [0, n - 1]) if b == 1 else (lambda k, n: [1, 0, n - 1, n - 2])
        for i in range(3):
            for j in range(4):
                out[i + b][j + b] = src(i, j)
            left, right = mir(0, 4)[:b], mir(0, 4)[b:]
            for k, jj in enumerate(left):
                out[i + b][k] = src(i, jj)
            for k, jj in enumerate(right):
                out[i + b][4 + b + k] = src(i, jj)
        for j in range(4):
            top, bottom = mir(0, 3)[:b], mir(0, 3)[b:]
            for k, ii in enumerate(top):
                out[k][j + b] = src(ii, j)
            for k, ii in enumerate(bottom):
                out[3 + b + k][j + b] = src(ii, j)
        return [v for r in out for v in r]

    assert d["2d1"] == padded(1) and d["2d2"] == padded(2)
    horizon = 0.1 * (1.0 + math.sqrt(1.0 - 0.99 * 0.99))
    assert lines[4] == "excised 1 %d %d" % (int(0.1 <= horizon), int(0.11 <= horizon))
    assert lines[5] == "Iteration = 3; Time = 0.25; Timestep = 0.001"
