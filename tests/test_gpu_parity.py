"""GPU parity: the FP64 path through the C ABI reproduces the reference (via the pinned oracle and the
reference-generated golden fixtures) bit for bit; the FP32 path stays within its stated error."""
import re

import numpy as np
import pytest

import cases
from conftest import bit_equal

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cg(cosmos_lib):
    import cosmos_gb300
    return cosmos_gb300


def grid_from(cg, system, prim, dx, precision=0, bc=0, bh=None):
    g = cg.Grid(system, prim.shape[:-1], dx, cases.SYS_GAMMA[system], precision, bc,
                cg.BlackHoleSpacetime(*bh) if bh is not None else None)
    g.set_prim(prim)
    return g


def test_sod_1000_cells_bit_exact(cg, golden):
    """Sod shock tube: SLIC van Leer, N=1000, CFL 0.9, t=0.25 (613 steps in the reference)."""
    g = grid_from(cg, 0, cases.sod(1000), 1.0 / 1000)
    r = g.solve(2, 0.9, 0.25, 0.0, 1)
    p = g.get_prim()
    assert r.steps == 613 and r.t == 0.25
    assert bit_equal(p, golden["sod1000_final"])
    # the same through the reference-named entry point
    q = cg.EulerSecondOrderSolver.solve(cases.sod(1000), 1.0 / 1000, 0.9, 0.25, 0.0, 1, cg.EulerMaterialParameters(1.4))
    assert bit_equal(q, golden["sod1000_final"])


@pytest.mark.parametrize("tag,system", [("newton", 0), ("sr", 1)])
def test_golden_sweeps(cg, golden, tag, system):
    keys = sorted(k[:-3] for k in golden if re.match(rf"^{tag}_d\d_o\d_l\d_bc\d_a\d_in$", k))
    assert len(keys) >= 20
    for k in keys:
        d, o, l, bc, a = map(int, re.match(r"^\w+?_d(\d)_o(\d)_l(\d)_bc(\d)_a(\d)$", k).groups())
        g = grid_from(cg, system, golden[k + "_in"], 1.0 / 64, bc=bc)
        g.sweep(a, o, 0.004, float(golden[k + "_bias"]), l)
        assert bit_equal(g.get_prim(), golden[k + "_out"]), k


@pytest.mark.parametrize("system", [0, 1])
@pytest.mark.parametrize("shape", [(2,), (3,), (301,), (2, 2), (37, 53), (130, 9)])
def test_random_sweeps_vs_oracle(cg, oracle, system, shape):
    """Odd sizes cross tile boundaries (126-cell X tiles, 16-row Y segments) and the 2-cell minimum."""
    rng = np.random.default_rng(hash((system, shape)) % 2**32)
    gam = cases.SYS_GAMMA[system]
    for order in (1, 2):
        for lim in ((0, 1, 2) if order == 2 else (1,)):
            for bc in (0, 1):
                for axis in ((0,) if len(shape) == 1 else (0, 1)):
                    s = cases.state(system, rng, shape)
                    g = grid_from(cg, system, s, 0.02, bc=bc)
                    g.sweep(axis, order, 0.003, 0.0, lim)
                    want = oracle.sweep(system, s, axis, order, 0.02, 0.003, 0.0, lim, gam, bc)
                    assert bit_equal(g.get_prim(), want), (order, lim, bc, axis)


@pytest.mark.parametrize("tag,system", [("newton", 0), ("sr", 1)])
def test_golden_solves_and_dt(cg, golden, tag, system):
    g = grid_from(cg, system, golden[f"{tag}_solve2d_in"], 1.0 / 12)
    r = g.solve(2, 0.9, 0.05, 0.0, 2)
    assert r.steps == int(golden[f"{tag}_solve2d_steps"]) and bit_equal(g.get_prim(), golden[f"{tag}_solve2d_out"])
    g = grid_from(cg, system, golden[f"{tag}_solve1d_force_in"], 1.0 / 24)
    r = g.solve(1, 0.8, 0.05, 0.0, 1)
    assert r.steps == int(golden[f"{tag}_solve1d_force_steps"])
    assert bit_equal(g.get_prim(), golden[f"{tag}_solve1d_force_out"])
    for dims in (1, 2):
        g = grid_from(cg, system, golden[f"{tag}_dt_d{dims}_in"], 0.01)
        dts = np.array([g.stable_dt(0.9, 0.0, 1.0, it) for it in (0, 7)])
        assert bit_equal(dts, golden[f"{tag}_dt_d{dims}"])


@pytest.mark.parametrize("system,bc", [(0, 0), (0, 1), (1, 0), (1, 1)])
def test_solve_2d_vs_oracle(cg, oracle, system, bc):
    """Device-side dt, graph-replayed steps: same step count, same final state, same t."""
    rng = np.random.default_rng(11 + system + 2 * bc)
    s = cases.four_quadrant(40, 3) if system == 0 else cases.sr_state(rng, (33, 40))
    gam = cases.SYS_GAMMA[system]
    g = grid_from(cg, system, s, 1.0 / 40, bc=bc)
    r = g.solve(2, 0.9, 0.08, 0.0, 2)
    want, n, t, _ = oracle.solve(system, s, 2, 1.0 / 40, 0.9, 0.08, 0.0, 2, gam, bc)
    assert r.steps == n and r.t == t
    assert bit_equal(g.get_prim(), want)


def test_max_steps_and_resume(cg, oracle):
    s = cases.four_quadrant(24, 5)
    g = grid_from(cg, 0, s, 1.0 / 24)
    r = g.solve(2, 0.9, 10.0, 0.0, 2, max_steps=7)
    want, n, t, _ = oracle.solve(0, s, 2, 1.0 / 24, 0.9, 10.0, 0.0, 2, 1.4, max_steps=7)
    assert r.steps == n == 7 and r.t == t and bit_equal(g.get_prim(), want)


@pytest.mark.parametrize("bhname,bh", [("bh", cases.GR_BH), ("spin", cases.GR_BH_SPIN)])
def test_gr_golden(cg, golden, bhname, bh):
    for dims in (1, 2):
        dx = 1.0 / 12
        for order in (1, 2):
            for axis in ((0,) if dims == 1 else (0, 1)):
                k = f"gr_{bhname}_d{dims}_o{order}_a{axis}"
                g = grid_from(cg, 2, golden[k + "_in"], dx, bh=bh)
                g.sweep(axis, order, 0.002, 0.0, 1)
                assert bit_equal(g.get_prim(), golden[k + "_out"]), k
        s = golden[f"gr_{bhname}_rk_d{dims}_in"]
        g = grid_from(cg, 2, s, dx, bh=bh)
        assert g.stable_dt(0.9, 0.0, 1.0, 0) == float(golden[f"gr_{bhname}_dt_d{dims}"])
        g.rk_source(0.002, 0.0, 1)
        assert bit_equal(g.get_prim(), golden[f"gr_{bhname}_rk_d{dims}_out"]), (bhname, dims)


def test_gr_solve_golden(cg, golden):
    g = grid_from(cg, 2, golden["gr_solve_in"], 2.0, bh=(1.0, 0.0, 10.0, 10.0, 0.0))
    r = g.solve(2, 0.9, 0.3, 0.0, 1, subcycles=1)
    assert r.steps == int(golden["gr_solve_steps"]) and bit_equal(g.get_prim(), golden["gr_solve_out"])


@pytest.mark.parametrize("sub", [0, 2])
def test_gr_solve_vs_oracle_accretion_shape(cg, oracle, sub):
    """The 1024^2 accretion geometry at reduced size: [-10,10]^2 as [0,20]^2 with the hole at (10,10), M=1,
    excision r <= 2M, rho = 1 + 1% log-normal noise, p = 0.01; two subcycles, or none (the flux
    sweeps alone, as the reference's own driver runs its accretion tests)."""
    n = 24
    rng = np.random.default_rng(4)
    s = np.zeros((n, n, 5))
    s[..., 0] = np.exp(0.01 * rng.standard_normal((n, n)))
    s[..., 4] = 0.01
    bh = (1.0, 0.0, 10.0, 10.0, 0.0)
    g = grid_from(cg, 2, s, 20.0 / n, bh=bh)
    r = g.solve(2, 0.9, 1e9, 0.0, 1, subcycles=sub, max_steps=3)
    want, n_, t, _ = oracle.solve(2, s, 2, 20.0 / n, 0.9, 1e9, 0.0, 1, 5.0 / 3.0, subcycles=sub, bh=bh, max_steps=3)
    assert r.steps == n_ == 3 and r.t == t
    assert bit_equal(g.get_prim(), want)


@pytest.mark.parametrize("system", [0, 1, 2])
@pytest.mark.parametrize("dims", [1, 2])
def test_amr_flags_vs_oracle(cg, oracle, system, dims):
    rng = np.random.default_rng(7 * system + dims)
    shape = (50,) if dims == 1 else (21, 26)
    s = cases.state(system, rng, shape)
    s[..., 0] += np.where(np.arange(shape[-1]) > shape[-1] // 2, 0.7, 0.0)
    dx = 1.0 / shape[-1]
    bh = cases.GR_BH if system == 2 else None
    g = grid_from(cg, system, s, dx, bh=bh)
    gam = cases.SYS_GAMMA[system]
    for tol in (0.5, 5.0, 40.0):
        c0 = rng.integers(0, 2, int(np.prod(shape))).astype(np.uint8)
        f0 = np.zeros(c0.size * (2 if dims == 1 else 4), np.uint8)
        c, f = g.amr_flags(tol, c0, f0)
        wc, wf = oracle.amr_flags(system, s, dx, tol, gam, c0, f0, bh=bh)
        assert bit_equal(c, wc) and bit_equal(f, wf), tol


@pytest.mark.parametrize("system", [0, 1])
@pytest.mark.parametrize("dims", [1, 2])
def test_amr_derefine_vs_oracle(cg, oracle, system, dims):
    rng = np.random.default_rng(3 + system + dims)
    shape = (20,) if dims == 1 else (9, 12)
    fshape = (40,) if dims == 1 else (18, 24)
    gam = cases.SYS_GAMMA[system]
    cs = cases.state(system, rng, shape)
    fs = cases.state(system, rng, fshape) * 0.02 + cases.state(system, rng, fshape) * 0.0
    fs[..., 0] += 1.0
    fs[..., 4] += 0.5
    dx = 1.0 / shape[-1]
    for tol in (0.1, 2.0):
        c0 = rng.integers(0, 2, int(np.prod(shape))).astype(np.uint8)
        f0 = rng.integers(0, 2, int(np.prod(fshape))).astype(np.uint8)
        gc, gf = grid_from(cg, system, cs, dx), grid_from(cg, system, fs, dx * 0.5)
        c, f = gc.amr_derefine(gf, tol, c0, f0)
        wp, wc, wf = oracle.amr_derefine(system, cs, fs, dx, tol, gam, c0, f0)
        assert bit_equal(c, wc) and bit_equal(f, wf)
        assert bit_equal(gc.get_prim(), wp)


def test_fp32_four_quadrant_error(cg, oracle):
    """FP32 bulk path vs the FP64 oracle on the 4096^2 four-quadrant problem at reduced size (128^2, 30 steps,
    MinBee, periodic): relative L1 density error and conservation drift stated here."""
    n = 128
    s = cases.four_quadrant(n, 2)
    g = grid_from(cg, 0, s, 1.0 / n, precision=1, bc=1)
    m0 = g.field_sums()
    r = g.solve(2, 0.9, 1e9, 0.0, 2, max_steps=30)
    p32 = g.get_prim()
    m1 = g.field_sums()
    want, nsteps, _, _ = oracle.solve(0, s, 2, 1.0 / n, 0.9, 1e9, 0.0, 2, 1.4, 1, max_steps=30)
    assert r.steps == nsteps == 30
    l1 = np.abs(p32[..., 0] - want[..., 0]).mean() / np.abs(want[..., 0]).mean()
    assert l1 < 1e-5, l1
    # mass and energy are conserved by the periodic flux form up to FP32 rounding
    assert abs(m1[0] - m0[0]) / abs(m0[0]) < 1e-6 and abs(m1[4] - m0[4]) / abs(m0[4]) < 1e-6


@pytest.mark.parametrize("precision", [0, 1])
def test_chunk_replay_equals_single_steps(cg, precision):
    """A run replays 8-step graphs where it can and single-step graphs for the rest: 21 steps in
    one call (two chunks and five single steps) and in 21 calls of one step give the same state,
    time and step count bit for bit; a run that reaches its final time inside a chunk stops there."""
    rng = np.random.default_rng(12)
    s = cases.newton_state(rng, (40, 56))
    out = []
    for split in (False, True):
        g = grid_from(cg, 0, s, 1.0 / 56, precision=precision, bc=1)
        g.run_begin(2, 0.8, 1e9, 0.0, 2, max_steps=21)
        if split:
            for _ in range(21):
                g.run_steps(1)
        else:
            g.run_steps(21)
        r = g.run_end()
        out.append((r.steps, r.t, g.get_prim()))
    assert out[0][0] == out[1][0] == 21 and out[0][1] == out[1][1]
    assert bit_equal(out[0][2], out[1][2])
    g = grid_from(cg, 0, s, 1.0 / 56, precision=precision, bc=1)
    g.run_begin(2, 0.8, 1e9, 0.0, 2, max_steps=11)
    g.run_steps(16)  # two chunks; the controller stops the run after step 11
    r = g.run_end()
    assert r.steps == 11


@pytest.mark.parametrize("bc", [0, 1])
def test_tensor_map_staging_is_bit_identical(cg, bc):
    """FP32 rows staged through TMA tensor maps (one copy of a row's five fields: the Y sweep and the
    CFL-reducing X sweep of single grids, the batch's Y items) and by one copy per field give the
    same states bit for bit: a grid whose rows hold several inside segments and whose last column
    run passes nx (300 columns), and a batch of uneven grids."""
    rng = np.random.default_rng(21)
    s = cases.newton_state(rng, (136, 300))
    shapes = [(130, 260), (300,), (70, 190), (64, 64)]
    states = [cases.newton_state(rng, sh) for sh in shapes]
    out = []
    try:
        for on in (True, False):
            cg.set_tensor_maps(on)
            g = grid_from(cg, 0, s, 1.0 / 300, precision=1, bc=bc)
            g.run_begin(2, 0.8, 1e9, 0.0, 2, max_steps=9)
            g.run_steps(9)
            r = g.run_end()
            b = cg.solvers.Batch(shapes, [1.0 / sh[-1] for sh in shapes], 1.4, 1, bc)
            for k, st in enumerate(states):
                b.set_prim(k, st)
            b.run_begin(0.9, 1e9, 0.0, 2, max_steps=12)
            b.run_steps(12)
            rb = b.run_end()
            out.append((r.steps, r.t, g.get_prim(), [(x.steps, x.t) for x in rb],
                        [b.get_prim(k) for k in range(len(shapes))]))
            b.close()
    finally:
        cg.set_tensor_maps(True)
    assert out[0][0] == out[1][0] == 9 and out[0][1] == out[1][1]
    assert bit_equal(out[0][2], out[1][2])
    assert out[0][3] == out[1][3] and all(n == 12 for n, _ in out[0][3])
    for a, c in zip(out[0][4], out[1][4]):
        assert bit_equal(a, c)


def test_fp32_sod_error(cg, golden):
    g = grid_from(cg, 0, cases.sod(1000), 1.0 / 1000, precision=1)
    r = g.solve(2, 0.9, 0.25, 0.0, 1)
    p = g.get_prim()
    ref = golden["sod1000_final"]
    assert abs(r.steps - 613) <= 2
    assert np.abs(p[:, 0] - ref[:, 0]).mean() < 1e-4


def test_errors_are_reported(cg):
    with pytest.raises(cg.CosmosError) as e:
        cg.Grid(0, (1,), 0.1, 1.4)
    assert e.value.code == 1 and "2 cells" in str(e.value)
    with pytest.raises(cg.CosmosError):
        cg.Grid(2, (8, 8), 0.1, 5 / 3, precision=1, boundary=1)  # GR: transmissive boundaries only
    g = cg.Grid(0, (8,), 0.1, 1.4)
    with pytest.raises(ValueError):
        g.set_prim(np.zeros((7, 5)))
    with pytest.raises(cg.CosmosError):
        g.sweep(1, 2, 0.01, 0.0, 1)  # no y axis in 1D
    with pytest.raises(cg.CosmosError):
        g.run_steps(1)  # run_begin not called


@pytest.mark.parametrize("shape,axis", [((5, 600), 0), ((600, 5), 1), ((700,), 0), ((3, 3), 0), ((3, 3), 1)])
def test_fp32_single_sweeps_vs_oracle(cg, oracle, shape, axis):
    """FP32 X tiles (254 updated cells per block) and Y segments (32 rows) crossing boundaries:
    one sweep against the FP64 oracle.  On random discontinuous data a few cells may take the
    other branch of a limiter (FP32 vs FP64 rounding near r = 1 or the 1e-5 clamp); a tiling
    error would instead give O(1) errors along whole tile edges."""
    rng = np.random.default_rng(shape[0] * 1000 + axis)
    for lim in (0, 1, 2):
        for bc in (0, 1):
            s = cases.newton_state(rng, shape)
            g = grid_from(cg, 0, s, 0.01, precision=1, bc=bc)
            g.sweep(axis, 2, 0.002, 0.0, lim)
            got = g.get_prim()
            want = oracle.sweep(0, s, axis, 2, 0.01, 0.002, 0.0, lim, 1.4, bc)
            rel = (np.abs(got - want) / (np.abs(want) + 1e-3)).max(axis=-1)
            assert np.median(rel) < 1e-6, (lim, bc, np.median(rel))
            assert rel.max() < 1e-2, (lim, bc, rel.max())
            assert (rel > 1e-5).mean() < 0.01, (lim, bc, (rel > 1e-5).mean())
