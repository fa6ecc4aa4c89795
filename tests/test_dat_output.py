"""The reference's scenario drivers and .dat writers (include/cosmos_gb300_tests.hpp).

Fixtures (tests/golden/dat_golden.npz, tests/golden/make_dat_golden.py) hold the text the
reference's own Tests/*.cpp wrote: its writers on seeded level data, and its scenarios run at small
sizes.  On the host: the writers reproduce the reference's files byte for byte, and each scenario's
problem (initial cells, material, CFL, final times, hole) run through the oracle and written by the
writers reproduces the reference's scenario files byte for byte.  On the GPU: the scenario drivers
themselves (initial cells, GPU solve, writer) reproduce them."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT

FILES = ("density.dat", "xVelocity.dat", "yVelocity.dat", "zVelocity.dat", "pressure.dat")


@pytest.fixture(scope="module")
def golden():
    return dict(np.load(os.path.join(ROOT, "tests", "golden", "dat_golden.npz")))


@pytest.fixture(scope="module")
def tool(cosmos_lib, tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("dat_tool") / "dat_tool")
    lib = os.path.join(ROOT, "cosmos_gb300")
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "dat_tool.cpp"), "-o", exe, "-L", lib, "-lcosmos_gb300",
                    f"-Wl,-rpath,{lib}"], check=True, capture_output=True, text=True)
    return exe


def expected_files(golden, key):
    return {f: golden[f"{key}/{f}"].tobytes() for f in FILES if f"{key}/{f}" in golden}


def written_files(d):
    return {f: open(os.path.join(d, f), "rb").read() for f in FILES if os.path.exists(os.path.join(d, f))}


def run_writer(tool, d, kind, system, dims, ny, nx, levels, flags, bh):
    os.makedirs(d, exist_ok=True)
    src = os.path.join(d, "input.bin")
    with open(src, "wb") as f:
        for lv in levels:
            f.write(np.ascontiguousarray(lv, dtype=np.float64).tobytes())
        f.write(np.ascontiguousarray(bh, dtype=np.float64).tobytes())
        for fl in flags:
            f.write(np.ascontiguousarray(fl, dtype=np.uint8).tobytes())
    r = subprocess.run([tool, "write", str(kind), str(system), str(dims), str(ny), str(nx), src, d],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    os.remove(src)
    return written_files(d)


def scenarios(golden):
    out = []
    k = 0
    while f"scenario{k}/args" in golden:
        name, n, order, sub, tol, level = golden[f"scenario{k}/args"].tobytes().decode().split()
        out.append((f"scenario{k}", name, int(n), int(order), int(sub), float(tol), int(level)))
        k += 1
    return out


def test_writers_match_the_reference(golden, tool, tmp_path):
    k = 0
    while f"writer{k}/args" in golden:
        key = f"writer{k}"
        kind, system, dims, ny, nx = (int(v) for v in golden[key + "/args"])
        levels = [golden[f"{key}/level{q}"] for q in range(3)]
        flags = [golden[f"{key}/flags{q}"] for q in range(3)]
        got = run_writer(tool, str(tmp_path / key), kind, system, dims, ny, nx, levels, flags, golden[key + "/bh"])
        want = expected_files(golden, key)
        assert sorted(got) == sorted(want), key
        for f in want:
            assert got[f] == want[f], (key, f)
        k += 1
    assert k == 11


def read_problem(tool, d, name, n):
    path = os.path.join(d, "problem.bin")
    r = subprocess.run([tool, "problem", name, str(n), path], capture_output=True, text=True)
    assert r.returncode == 0, (name, r.stderr)
    raw = open(path, "rb").read()
    system, dims, nx, ny = np.frombuffer(raw[:16], dtype=np.int32)
    par = np.frombuffer(raw[16:16 + 88], dtype=np.float64)
    prim = np.frombuffer(raw[16 + 88:], dtype=np.float64).reshape((nx, 5) if dims == 1 else (ny, nx, 5))
    return dict(system=int(system), dims=int(dims), nx=int(nx), ny=int(ny), dx=par[0], gamma=par[1], cfl=par[2],
                t=(par[3], par[4]), t_amr=par[5], bh=tuple(par[6:11]), prim=prim.copy())


def test_scenario_problems_through_the_oracle_match_the_reference(golden, tool, oracle, tmp_path):
    """Each scenario's problem data, solved by the oracle with the scenario's solver arguments and
    written by the writers, gives the reference's scenario files byte for byte."""
    cases = scenarios(golden)
    assert len(cases) == 44
    for key, name, n, order, sub, tol, level in cases:
        d = str(tmp_path / key)
        os.makedirs(d)
        P = read_problem(tool, d, name, n)
        s, dims, sysid = P["prim"], P["dims"], P["system"]
        ny = 1 if dims == 1 else P["ny"]
        r = 4 if dims == 2 else 2
        sizes = [P["nx"] * ny * r ** q for q in range(3)]
        levels = [np.zeros(5 * m) for m in sizes]
        flags = [np.zeros(m, np.uint8) for m in sizes]
        if "AMR" in name:
            run = oracle.amr_level1 if level == 1 else oracle.amr_level2
            res = run(sysid, s, P["dx"], P["cfl"], P["t_amr"], tol, order, P["gamma"])
            nlev = level + 1
            levels[:nlev], flags[:nlev] = res[2:2 + nlev], res[2 + nlev:]
            kind = level
        else:
            out, _, _, _ = oracle.solve(sysid, s, order, P["dx"], P["cfl"], P["t"][order - 1], 0.0, 1, P["gamma"],
                                        subcycles=sub, bh=P["bh"] if sysid == 2 else None)
            levels[0] = out.reshape(-1)
            kind = 0
        got = run_writer(tool, d, kind, sysid, dims, ny, P["nx"], levels, flags, np.array(P["bh"]))
        want = expected_files(golden, key)
        assert sorted(got) == sorted(want), (key, name)
        for f in want:
            assert got[f] == want[f], (key, name, f)


def numbers_close(a, b):
    """Same layout, numbers equal to the six printed digits (initial data from sin/cos/atan2 may
    differ in the last bit between hosts)."""
    la, lb = a.decode().split("\n"), b.decode().split("\n")
    if len(la) != len(lb):
        return False
    for x, y in zip(la, lb):
        tx, ty = x.split(), y.split()
        if len(tx) != len(ty):
            return False
        if tx != ty and not np.allclose(np.array(tx, float), np.array(ty, float), rtol=2e-5, atol=1e-9):
            return False
    return True


@pytest.mark.gpu
def test_scenario_drivers_on_the_gpu_match_the_reference(golden, tool, tmp_path):
    transcendental = ("solve2DToroTest2", "PerturbedDensity")
    for key, name, n, order, sub, tol, level in scenarios(golden):
        d = str(tmp_path / key)
        os.makedirs(d)
        r = subprocess.run([tool, "run", name, str(n), str(order), str(sub), repr(tol), str(level), d],
                           capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, (name, r.stderr)
        got, want = written_files(d), expected_files(golden, key)
        assert sorted(got) == sorted(want), (key, name)
        for f in want:
            if any(t in name for t in transcendental):
                assert numbers_close(got[f], want[f]), (key, name, f)
            else:
                assert got[f] == want[f], (key, name, f)
