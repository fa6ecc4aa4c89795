"""The reference's per-interface solver functions on the device (cosmos_interface_eval) and through the
C++ shim's reference-named methods (include/cosmos_gb300_compat.hpp), bit for bit against the
reference itself (tests/golden/interface_golden.npz, written by the reference's own static
functions: Solvers/EulerFirstOrderSolver.hpp:11-31, Solvers/EulerSecondOrderSolver.hpp:9-14,
Solvers/EulerSolvers.hpp:25-34, their special-relativistic and black-hole twins,
Solvers/BlackHoleEulerSolvers.hpp:22-49 and Solvers/BlackHoleEulerForcingSolver.hpp:9-17)."""
import os
import struct
import subprocess

import numpy as np
import pytest

from conftest import ROOT, bit_equal

GOLDEN = os.path.join(ROOT, "tests", "golden", "interface_golden.npz")
EINVAL, EUNSUPPORTED = 1, 4


def _cases():
    d = np.load(GOLDEN)
    keys = sorted(k[:-5] for k in d.files if k.endswith("_args"))
    out = []
    for k in keys:
        a = d[k + "_args"]
        out.append(dict(key=k, op=int(a[0]), system=int(a[1]), gamma=a[2], dx=a[3], dt=a[4], bias=a[5], lim=int(a[6]),
                        frac=a[7], side=int(a[8]), bh=tuple(a[9:]), items=d[k + "_in"],
                        xyz=d[k + "_xyz"] if k + "_xyz" in d.files else None, want=d[k + "_out"]))
    return out


def _driver(out):
    src = os.path.join(ROOT, "tests", "cpp", "interface_driver.cpp")
    lib = os.path.join(ROOT, "cosmos_gb300")
    cmd = ["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), src]
    cmd += ["-fsyntax-only"] if out is None else ["-o", out, "-L", lib, "-lcosmos_gb300", f"-Wl,-rpath,{lib}"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)


def test_interface_driver_compiles():
    _driver(None)


@pytest.fixture(scope="module")
def cg(cosmos_lib):
    import cosmos_gb300
    return cosmos_gb300


@pytest.mark.gpu
def test_interface_functions_bit_exact(cg):
    cases = _cases()
    assert len(cases) == 162
    for c in cases:
        bh = cg.BlackHoleSpacetime(*c["bh"]) if c["system"] == 2 else None
        got = cg.interface_eval(c["op"], c["items"], c["system"], c["gamma"], c["dx"], c["dt"], c["xyz"], bh,
                                c["bias"], c["lim"], c["frac"], c["side"])
        assert bit_equal(got, c["want"]), c["key"]


@pytest.mark.gpu
def test_compat_methods_bit_exact(cosmos_lib, tmp_path):
    """Every reference-named method, called one item at a time from C++ as the reference's callers
    do (AMR/EulerAMR.cpp:96-101 calls computeXSLICFlux and computeFORCEUpdate this way)."""
    exe = str(tmp_path / "interface_driver")
    _driver(exe)
    cases = _cases()
    blob = bytearray()
    for c in cases:
        n, w = c["items"].shape
        blob += struct.pack("<5i", c["op"], c["system"], n, w, int(c["xyz"] is not None))
        blob += struct.pack("<5d", c["gamma"], c["dx"], c["dt"], c["bias"], c["frac"])
        blob += struct.pack("<5d", *c["bh"])
        blob += struct.pack("<2i", c["lim"], c["side"])
        blob += np.ascontiguousarray(c["items"], dtype="<f8").tobytes()
        if c["xyz"] is not None:
            blob += np.ascontiguousarray(c["xyz"], dtype="<f8").tobytes()
    (tmp_path / "cases.bin").write_bytes(bytes(blob))
    r = subprocess.run([exe, str(tmp_path / "cases.bin"), str(tmp_path / "out.bin")], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr
    got = np.fromfile(str(tmp_path / "out.bin"), dtype=np.float64)
    k = 0
    for c in cases:
        n = c["items"].shape[0]
        assert bit_equal(got[k:k + 5 * n].reshape(n, 5), c["want"]), c["key"]
        k += 5 * n
    assert k == got.size


@pytest.mark.gpu
def test_spacetime_and_eigenvalues_bit_exact(cg, cosmos_lib, tmp_path):
    """BlackHoleSpacetime's metric methods (BlackHoleEuler/BlackHoleSpacetime.hpp:16-42) and
    BlackHoleEulerEigenvalues (BlackHoleEuler/BlackHoleEulerEigenvalues.hpp:9-18) around a
    Schwarzschild and a spinning hole, off the plane z = 0 too: the device record, the Python
    methods and the C++ shim's methods against the reference's outputs."""
    from cosmos_gb300 import _lib
    d = np.load(GOLDEN)
    blob, want_cpp = bytearray(), []
    for hole in ("schw", "kerr"):
        q, bh, h = d[f"st_{hole}_xyz"], d[f"st_{hole}_bh"], float(d[f"st_{hole}_h"])
        B = cg.BlackHoleSpacetime(*bh)
        rec = B.record(q[:, 0], q[:, 1], q[:, 2], h)
        assert bit_equal(rec, d[f"st_{hole}_out"]), hole
        k = 7
        assert B.computeLapseFunction(*q[k]) == d[f"st_{hole}_out"][k, 99]
        assert bit_equal(B.computeSpatialMetricTensorDerivative(*q[k], h), d[f"st_{hole}_out"][k, 72:99].reshape(3, 3, 3))
        assert bit_equal(B.computeInverseSpacetimeMetricTensor(*q[k]), d[f"st_{hole}_out"][k, 54:70].reshape(4, 4))
        eig = cg.state_eval(_lib.STATE_EIGENVALUES, d[f"eig_{hole}_in"], cg.GR, 5.0 / 3.0, xyz=q, black_hole=B)
        assert bit_equal(eig, d[f"eig_{hole}_out"]), hole
        for op, items, out in ((100, q, d[f"st_{hole}_out"]), (101, np.hstack([d[f"eig_{hole}_in"], q]), d[f"eig_{hole}_out"])):
            n, w = items.shape
            blob += struct.pack("<5i", op, 2, n, w, 0)
            blob += struct.pack("<5d", 5.0 / 3.0, h, 1.0, 0.0, 0.5)
            blob += struct.pack("<5d", *bh)
            blob += struct.pack("<2i", 1, 0)
            blob += np.ascontiguousarray(items, dtype="<f8").tobytes()
            want_cpp.append(out)
    exe = str(tmp_path / "interface_driver")
    _driver(exe)
    (tmp_path / "cases.bin").write_bytes(bytes(blob))
    r = subprocess.run([exe, str(tmp_path / "cases.bin"), str(tmp_path / "out.bin")], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr
    got = np.fromfile(str(tmp_path / "out.bin"), dtype=np.float64)
    want = np.concatenate([w.reshape(-1) for w in want_cpp])
    assert bit_equal(got, want)


@pytest.mark.gpu
def test_interface_argument_errors(cg):
    prim = np.tile(np.array([1.0, 0.1, 0.0, 0.0, 1.0]), (3, 2))
    with pytest.raises(cg.CosmosError) as e:  # fractional evolutions exist for the black-hole system only
        cg.interface_eval(cg._lib.IF_EVOLVE_FRACTION_X, np.tile(prim, (1, 2))[:, :15], cg.NEWTONIAN, 1.4, 0.1, 0.01)
    assert e.value.code == EUNSUPPORTED
    with pytest.raises(cg.CosmosError) as e:  # black-hole functions need their coordinates
        cg.interface_eval(cg._lib.IF_X_FORCE_FLUX, prim, cg.GR, 5.0 / 3.0, 0.1, 0.01)
    assert e.value.code == EINVAL
    with pytest.raises(cg.CosmosError) as e:
        cg.interface_eval(cg._lib.IF_EVOLVE_HALF_X, np.tile(prim, (1, 2))[:, :15], cg.NEWTONIAN, 1.4, 0.1, 0.01, side=2)
    assert e.value.code == EINVAL
    with pytest.raises(cg.CosmosError) as e:
        cg.interface_eval(cg._lib.IF_X_FORCE_FLUX, prim, cg.NEWTONIAN, 1.4, 0.1, 0.0)
    assert e.value.code == EINVAL
    with pytest.raises(cg.CosmosError):
        cg.interface_eval(23, prim, cg.NEWTONIAN, 1.4, 0.1, 0.01)
