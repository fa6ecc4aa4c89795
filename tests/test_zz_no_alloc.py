"""cosmos_field_sums_noalloc: the allocation-free conservation sums.

Callers that cannot allocate device memory (runtimes that own the device allocator and its pool,
embedded callers with a fixed memory budget, pipelines that must not stall on cudaMalloc's device
synchronisation) use this entry point; its scratch is a fixed device array.  The
test calls it through the C ABI on caller-owned device buffers, twice in a row (the second call
runs on the scratch left by the first), and checks both results against cosmos_grid_field_sums on
a grid holding the same state.  It lives in its own file, collected last, and also passes alone.
"""
import ctypes

import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu

REL_TOL = 1e-12  # compensated FP64 sums of the same values, different summation order


def _call(L, torch, state, precision, nx, ny, out):
    fn = L.cosmos_field_sums_noalloc
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_size_t,
                   ctypes.c_void_p, ctypes.c_void_p]
    rc = fn(state.data_ptr(), precision, nx, ny, nx, nx * ny, out.data_ptr(), torch.cuda.current_stream().cuda_stream)
    return rc


def _cons_f32(prim, gamma):
    """Conserved FP32 state exactly as the library forms it from primitives (FP64, rounded once)."""
    rho, vx, vy, vz, p = (prim[..., k] for k in range(5))
    v2 = ((vx * vx) + (vy * vy)) + (vz * vz)
    e = p / ((gamma - 1.0) * rho)
    u = np.stack([rho, rho * vx, rho * vy, rho * vz, rho * ((0.5 * v2) + e)], axis=0)
    return u.astype(np.float32)


@pytest.mark.parametrize("precision", [0, 1])
def test_noalloc_matches_grid_sums(cosmos_lib, precision):
    torch = pytest.importorskip("torch")
    import cosmos_gb300 as cg
    L = cg.load()
    ny, nx = 300, 517
    rng = np.random.default_rng(99 + precision)
    prim = cases.newton_state(rng, (ny, nx))
    g = cg.Grid(cg.NEWTONIAN, (ny, nx), 1.0 / nx, 1.4, precision)
    g.set_prim(prim)
    want = g.field_sums()
    soa = np.ascontiguousarray(np.moveaxis(prim, -1, 0)) if precision == 0 else _cons_f32(prim, 1.4)
    state = torch.from_numpy(soa.reshape(-1)).cuda()
    for _ in range(2):
        out = torch.full((5,), float("nan"), dtype=torch.float64, device="cuda")
        assert _call(L, torch, state, precision, nx, ny, out) == 0, L.cosmos_last_error()
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        np.testing.assert_allclose(got, want, rtol=REL_TOL, atol=0)


def test_noalloc_rejects_oversized(cosmos_lib):
    torch = pytest.importorskip("torch")
    import cosmos_gb300 as cg
    L = cg.load()
    ny = 16385  # one row more than COSMOS_NOALLOC_MAX_ROWS
    state = torch.zeros((5 * ny * 2,), dtype=torch.float64, device="cuda")
    out = torch.zeros((5,), dtype=torch.float64, device="cuda")
    assert _call(L, torch, state, 0, 2, ny, out) == 1
    assert b"COSMOS_NOALLOC_MAX_ROWS" in L.cosmos_last_error()
