"""Batched persistent launch (cosmos_batch): many independent grids of uneven sizes, one
cooperative launch per chunk of steps.  Every grid must evolve exactly as the reference's
EulerSecondOrderSolver::solve / solve2D would evolve it alone (Solvers/EulerSecondOrderSolver.cpp:
102-147): bit for bit with FP64, within FP32 rounding of the single-grid FP32 path with FP32."""
import numpy as np
import pytest

import cases
from conftest import bit_equal

pytestmark = pytest.mark.gpu

# 1D and 2D grids crossing every tile boundary (X tiles of 126/254 cells, X items of several rows,
# Y items of 128/256 columns x 7/64 rows) plus the 2-cell minimum; grids finish at different steps.
SHAPES = [(301,), (2,), (37, 53), (130, 9), (2, 2), (5, 600), (64, 64), (600,), (33, 257)]


@pytest.fixture(scope="module")
def cg(cosmos_lib):
    import cosmos_gb300
    return cosmos_gb300


def make_batch(cg, states, dxs, precision, bc):
    b = cg.solvers.Batch([s.shape[:-1] for s in states], dxs, 1.4, precision, bc)
    for k, s in enumerate(states):
        b.set_prim(k, s)
    return b


def states_for(seed, shapes):
    rng = np.random.default_rng(seed)
    return [cases.newton_state(rng, sh) for sh in shapes]


@pytest.mark.parametrize("shape", [(128, 7), (256, 64)])
@pytest.mark.parametrize("bc", [0, 1])
def test_fp64_batch_bit_exact_per_grid(cg, oracle, shape, bc):
    states = states_for(17 + bc, SHAPES)
    dxs = [1.0 / sh[-1] for sh in SHAPES]
    b = make_batch(cg, states, dxs, 0, bc)
    b.set_shape(*shape)
    b.run_begin(0.9, 0.03, 0.0, 2)
    for n in (7, 23, 40, 130):  # chunks of 10 replayed from a graph plus direct remainders
        b.run_steps(n)
    res = b.run_end()
    for k, s in enumerate(states):
        want, n, t, _ = oracle.solve(0, s, 2, dxs[k], 0.9, 0.03, 0.0, 2, 1.4, bc)
        assert n < 200, "the batch ran 200 steps; every grid must have finished"
        assert res[k].steps == n and res[k].t == t, (k, res[k].steps, n)
        assert bit_equal(b.get_prim(k), want), (k, SHAPES[k])


@pytest.mark.parametrize("lim", [0, 1, 2])
def test_fp64_batch_max_steps_and_resume(cg, oracle, lim):
    """A step cap stops every grid at the same iteration; a second run_begin restarts the
    controllers (t = 0) from the state reached, like a second call of the reference's solve."""
    shapes = SHAPES[:6]
    states = states_for(5 + lim, shapes)
    dxs = [0.7 / sh[-1] for sh in shapes]
    b = make_batch(cg, states, dxs, 0, 0)
    b.run_begin(0.8, 1e9, 0.0, lim, max_steps=9)
    b.run_steps(13)
    res = b.run_end()
    b.run_begin(0.8, 1e9, 0.0, lim, max_steps=4)
    b.run_steps(4)
    res2 = b.run_end()
    for k, s in enumerate(states):
        mid, n, t, _ = oracle.solve(0, s, 2, dxs[k], 0.8, 1e9, 0.0, lim, 1.4, max_steps=9)
        want, n2, t2, _ = oracle.solve(0, mid, 2, dxs[k], 0.8, 1e9, 0.0, lim, 1.4, max_steps=4)
        assert res[k].steps == n == 9 and res[k].t == t
        assert res2[k].steps == n2 == 4 and res2[k].t == t2
        assert bit_equal(b.get_prim(k), want), k


@pytest.mark.parametrize("cap", [0, 1])
@pytest.mark.parametrize("bc", [0, 1])
def test_fp32_batch_matches_single_grid(cg, oracle, cap, bc):
    """The FP32 batch runs the same per-cell arithmetic as the single-grid FP32 path (only the
    tiling differs), so the two agree to FP32 rounding; both stay near the FP64 oracle."""
    shapes = [(700,), (64, 300), (130, 9), (3, 3), (48, 48)]
    states = states_for(29 + bc, shapes)
    dxs = [1.0 / sh[-1] for sh in shapes]
    b = make_batch(cg, states, dxs, 1, bc)
    b.set_shape(256, 32, cap)
    b.run_begin(0.9, 1e9, 0.0, 2, max_steps=20)
    b.run_steps(20)
    res = b.run_end()
    for k, s in enumerate(states):
        g = cg.Grid(0, shapes[k], dxs[k], 1.4, 1, bc)
        g.set_prim(s)
        r = g.solve(2, 0.9, 1e9, 0.0, 2, max_steps=20)
        single = g.get_prim()
        got = b.get_prim(k)
        assert res[k].steps == r.steps == 20
        assert abs(res[k].t - r.t) <= 1e-6 * r.t, (res[k].t, r.t)
        rel = np.abs(got - single) / (np.abs(single) + 1e-3)
        assert np.median(rel) < 1e-6 and rel.max() < 1e-3, (k, np.median(rel), rel.max())
        want, _, _, _ = oracle.solve(0, s, 2, dxs[k], 0.9, 1e9, 0.0, 2, 1.4, bc, max_steps=20)
        l1 = np.abs(got[..., 0] - want[..., 0]).mean() / np.abs(want[..., 0]).mean()
        assert l1 < 1e-4, (k, l1)


def test_time_shape_restores_state_and_autotune_cache(cg, oracle, tmp_path):
    shapes = SHAPES[:5]
    states = states_for(41, shapes)
    dxs = [1.0 / sh[-1] for sh in shapes]
    b = make_batch(cg, states, dxs, 0, 0)
    b.run_begin(0.9, 0.02, 0.0, 1)
    b.run_steps(3)
    before = [b.get_prim(k) for k in range(len(shapes))]
    ms = b.time_shape(256, 32, 0, steps=4)
    assert ms > 0.0
    assert all(bit_equal(b.get_prim(k), before[k]) for k in range(len(shapes)))
    cache = str(tmp_path / "batch_tune.txt")
    (nt, seg, cap), ms1 = b.autotune(cache)
    assert (nt, seg) in [(128, 32), (128, 64), (256, 32), (256, 64)] and cap == 0  # FP64 has no capped shape
    assert all(bit_equal(b.get_prim(k), before[k]) for k in range(len(shapes)))
    shape2, ms2 = b.autotune(cache)  # second call: read back from the cache file
    assert shape2 == (nt, seg, cap) and ms2 == ms1
    assert len(open(cache).read().strip().splitlines()) == 1
    # the run continues from where it was, unaffected by the timing runs
    b.run_steps(200)
    res = b.run_end()
    for k, s in enumerate(states):
        want, n, t, _ = oracle.solve(0, s, 2, dxs[k], 0.9, 0.02, 0.0, 1, 1.4)
        assert res[k].steps == n and res[k].t == t and bit_equal(b.get_prim(k), want), k


def test_fp32_autotune_considers_capped_shapes(cg):
    rng = np.random.default_rng(3)
    shapes = [(256, 256), (1000,), (77, 130)]
    b = make_batch(cg, [cases.newton_state(rng, sh) for sh in shapes], 0.01, 1, 1)
    b.run_begin(0.9, 1e9, 0.0, 2)
    # the autotuner's shapes: threads {128, 256} x Y rows {32, 64} x cap {0, 1}, and 128 rows capped
    grid = [(nt, seg, cap) for nt in (128, 256) for seg in (32, 64) for cap in (0, 1)]
    grid += [(128, 128, 1), (256, 128, 1)]
    times = {sh: b.time_shape(*sh, steps=3) for sh in grid}
    assert all(v > 0.0 for v in times.values())
    shape, ms = b.autotune(None)
    assert shape in times and ms > 0.0


def test_batch_errors(cg):
    with pytest.raises(cg.CosmosError):
        cg.solvers.Batch([(1,)], 0.1, 1.4)  # fewer than 2 cells
    with pytest.raises(cg.CosmosError):
        cg.solvers.Batch([(8,)], 0.1, 1.0)  # gamma must exceed 1
    b = cg.solvers.Batch([(8,), (4, 4)], 0.1, 1.4, precision=0)
    with pytest.raises(cg.CosmosError):
        b.run_steps(1)  # run_begin not called
    with pytest.raises(cg.CosmosError) as e:
        b.set_shape(256, 32, 1)  # FP64 has no register-capped variant
    assert e.value.code == 4  # COSMOS_EUNSUPPORTED
    with pytest.raises(cg.CosmosError):
        b.set_shape(64, 16)
    with pytest.raises(ValueError):
        b.set_prim(1, np.zeros((4, 5, 5)))
    buf = np.zeros((4, 4, 5))
    assert cg.load().cosmos_batch_get_prim(b.h, 2, buf.ctypes.data, buf.size) == 1  # grid index out of range
    assert cg.load().cosmos_batch_get_prim(b.h, 1, buf.ctypes.data, buf.size - 5) == 1  # size mismatch


def test_context_outlives_its_objects(cg):
    """Destroying the context first leaves its grids and batches usable until they are destroyed."""
    ctx = cg.Context(0)
    g = cg.Grid(0, (16,), 1.0 / 16, 1.4, ctx=ctx)
    b = cg.solvers.Batch([(8,), (6, 6)], 0.1, 1.4, precision=0, ctx=ctx)
    s = cases.sod(16)
    g.set_prim(s)
    ctx.close()
    r = g.solve(2, 0.9, 0.01, 0.0, 1)
    assert r.steps > 0
    b.set_prim(0, cases.sod(8))
    b.run_begin(0.9, 0.01, 0.0, 1)
    b.run_steps(3)
    b.run_end()
    g.close()
    b.close()


@pytest.mark.parametrize("shape", [(37, 300), (130, 61), (700,), (2, 2), (5, 3), (64, 121)])
@pytest.mark.parametrize("bc", [0, 1])
@pytest.mark.parametrize("lim", [0, 1, 2])
def test_fp32_pair_kernels_match_one_cell_kernels(cg, shape, bc, lim):
    """Single FP32 grids sweep on cell pairs (paired FP32 instructions; X across warp lanes by
    shuffles, Y two columns per thread), the batched launch with the one-cell tile functions.
    Both evaluate the same explicitly rounded operation sequence; they agree to FP32 rounding
    (a last-bit difference in an extrapolated state can flip a limiter branch in a few cells)."""
    rng = np.random.default_rng(hash((shape, bc, lim)) % 2**32)
    s = cases.newton_state(rng, shape)
    dx = 1.0 / shape[-1]
    b = cg.solvers.Batch([shape], dx, 1.4, 1, bc)
    b.set_prim(0, s)
    b.run_begin(0.9, 1e9, 0.0, lim, max_steps=12)
    b.run_steps(12)
    res = b.run_end()
    g = cg.Grid(0, shape, dx, 1.4, 1, bc)
    g.set_prim(s)
    r = g.solve(2, 0.9, 1e9, 0.0, lim, max_steps=12)
    assert res[0].steps == r.steps == 12 and abs(res[0].t - r.t) <= 1e-6 * r.t
    got, want = b.get_prim(0), g.get_prim()
    rel = np.abs(got - want) / (np.abs(want) + 1e-3)
    assert np.median(rel) < 1e-6 and rel.max() < 1e-2, (np.median(rel), rel.max())


def test_fp32_batch_uneven_step_counts(cg):
    """The FP32 warps take items through per-phase counters that alternate with the step parity:
    runs of 3, 10 (one replayed chunk) and 7 steps, and again after a time_shape (which restores the
    state), give the same states as 20 single steps."""
    rng = np.random.default_rng(8)
    shapes = [(64, 96), (300,), (45, 70)]
    states = [cases.newton_state(rng, sh) for sh in shapes]
    results = []
    for plan in ((3, 10, 7), (1,) * 20):
        b = make_batch(cg, states, [1.0 / sh[-1] for sh in shapes], 1, 1)
        b.run_begin(0.8, 1e9, 0.0, 2, max_steps=20)
        if len(plan) > 3:
            b.time_shape(128, 32, 1, steps=3)
        for k in plan:
            b.run_steps(k)
        res = b.run_end()
        assert all(r.steps == 20 for r in res)
        results.append([b.get_prim(k) for k in range(len(shapes))])
        b.close()
    assert all(bit_equal(x, y) for x, y in zip(*results))
