"""C ABI checks that need no GPU: the library builds and loads, exports every function that
include/cosmos_gb300.h declares, the Python binding covers the same set, and the host-side
functions agree with the oracle."""
import ctypes
import os
import re

import numpy as np
import pytest

import cases

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    text = open(os.path.join(ROOT, "include", "cosmos_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(cosmos_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_abi():
    fns = header_functions()
    assert len(fns) >= 25
    for must in ("cosmos_grid_sweep", "cosmos_grid_solve", "cosmos_grid_rk_source", "cosmos_grid_amr_flags", "cosmos_amr_solve",
                 "cosmos_stable_dt_rule", "cosmos_last_error"):
        assert must in fns


def test_library_exports_every_declared_symbol(cosmos_lib):
    for name in header_functions():
        assert hasattr(cosmos_lib, name), name


def test_binding_matches_header():
    from cosmos_gb300 import _lib
    assert sorted(_lib.SIGNATURES) == header_functions()


def test_stable_dt_rule_matches_oracle(cosmos_lib, oracle):
    rng = np.random.default_rng(0)
    for _ in range(200):
        dt, t, tf = rng.uniform(1e-4, 1e-2), rng.uniform(0, 1), rng.uniform(0, 1.2)
        it = int(rng.integers(0, 10))
        assert cosmos_lib.cosmos_stable_dt_rule(dt, t, tf, it) == oracle.stable_dt_rule(dt, t, tf, it)


def test_defaults_mirror_the_reference(cosmos_lib):
    from cosmos_gb300._lib import Params, SolveOpts
    p = Params()
    cosmos_lib.cosmos_params_default(ctypes.byref(p))
    # BlackHoleSpacetime() defaults, BlackHoleEuler/BlackHoleSpacetime.cpp:3-11
    assert (p.bh_mass, p.bh_spin, p.bh_x, p.bh_y, p.bh_z) == (1.0, 0.0, 0.5, 0.5, 0.0)
    o = SolveOpts()
    cosmos_lib.cosmos_solve_opts_default(ctypes.byref(o))
    assert o.order == 2 and o.max_steps == -1


def test_error_paths_without_gpu(cosmos_lib):
    """Argument errors are reported before any device work; with no GPU the context call fails
    cleanly with a message instead of crashing."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = ctypes.c_void_p()
    rc = cosmos_lib.cosmos_ctx_create(0, ctypes.byref(h))
    assert rc != 0 and len(cosmos_lib.cosmos_last_error()) > 0
    assert cosmos_lib.cosmos_grid_create(None, None, None) == 1
    assert cosmos_lib.cosmos_grid_sweep(None, 0, 2, 0.1, 0.0, 1) == 1
    assert b"null" in cosmos_lib.cosmos_last_error()


def test_python_api_names_mirror_reference():
    import cosmos_gb300 as cg
    for cls, methods in (
        (cg.EulerSecondOrderSolver, ("solve", "solve2D", "computeSLICTimeStep", "computeXSLICTimeStep2D",
                                     "computeYSLICTimeStep2D")),
        (cg.EulerFirstOrderSolver, ("solve", "solve2D", "computeFORCETimeStep", "computeXFORCETimeStep2D",
                                    "computeYFORCETimeStep2D")),
        (cg.EulerSolvers, ("computeMaximumWaveSpeed", "computeMaximumWaveSpeed2D", "computeStableTimeStep",
                           "computeStableTimeStep2D")),
        (cg.RelativisticEulerSecondOrderSolver, ("solve", "solve2D", "computeXSLICTimeStep2D")),
        (cg.BlackHoleEulerSecondOrderSolver, ("solve", "solve2D", "computeXSLICTimeStep2D")),
        (cg.BlackHoleEulerForcingSolver, ("computeRungeKuttaTimeStep", "computeRungeKuttaTimeStep2D")),
    ):
        for m in methods:
            assert callable(getattr(cls, m)), (cls, m)
    assert cg.EulerMaterialParameters(1.4).getAdiabaticIndex() == 1.4
    assert cg.BlackHoleSpacetime(0.05, 0.5, 0.0, 0.0).mass == 0.05


def test_state_operation_widths(cosmos_lib):
    """cosmos_state_width: the input and output doubles per item of every state operation (host
    only, no device)."""
    from cosmos_gb300 import _lib
    want = {_lib.STATE_CONS: (5, 5), _lib.STATE_PRIM: (5, 5), _lib.STATE_FLUX_X: (5, 5), _lib.STATE_FLUX_Y: (5, 5),
            _lib.STATE_SOUND: (5, 1), _lib.STATE_INTERNAL_ENERGY: (5, 1), _lib.STATE_TOTAL_ENERGY: (5, 1),
            _lib.STATE_PRESSURE: (5, 1), _lib.STATE_ENTHALPY: (5, 1), _lib.STATE_SOURCE: (5, 5),
            _lib.STATE_EIGENVALUES: (5, 9), _lib.STATE_GRADIENT_RATIO: (1, 1), _lib.STATE_LIMITER: (1, 1),
            _lib.STATE_SLOPE: (15, 5)}
    for op, (wi, wo) in want.items():
        a, b = ctypes.c_size_t(0), ctypes.c_size_t(0)
        assert cosmos_lib.cosmos_state_width(op, ctypes.byref(a), ctypes.byref(b)) == 0
        assert (a.value, b.value) == (wi, wo), op
    assert cosmos_lib.cosmos_state_width(14, None, None) == _lib.EINVAL
    assert cosmos_lib.cosmos_state_width(-1, None, None) == _lib.EINVAL
