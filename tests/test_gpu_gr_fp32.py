"""FP32 bulk path of the black-hole system (FP64 metric tables, FP32 sweeps / RK4 source, primitive
recovery finishing in FP64 above Lorentz factor 2) against the FP64 oracle.  Stated error: the
relative L1 density error over the cells outside the excision region is below 1e-4 after the
steps below (the FP32 path evaluates the metric at exact geometric points, the reference at
separately rounded face coordinates, so it is not bit-identical even in exact arithmetic)."""
import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu
G53 = 5.0 / 3.0


@pytest.fixture(scope="module")
def cg(cosmos_lib):
    import cosmos_gb300
    return cosmos_gb300


def accretion(n, seed):
    rng = np.random.default_rng(seed)
    s = np.zeros((n, n, 5))
    s[..., 0] = np.exp(0.01 * rng.standard_normal((n, n)))
    s[..., 4] = 0.01
    return s


def l1_outside(got, want, mask):
    g, w = got[..., 0][mask], want[..., 0][mask]
    return np.abs(g - w).mean() / np.abs(w).mean()


@pytest.mark.parametrize("above", [2.0, 0.0])
def test_gr_fp32_accretion_vs_oracle(cg, oracle, above):
    """The accretion benchmark's geometry at reduced size: [-10,10]^2 as [0,20]^2 with the hole at (10,10), M = 1,
    excision r <= 2M, rho = 1 + 1% log-normal noise, p = 0.01; 6 steps, RK4 source on both sides."""
    n = 48
    s = accretion(n, 4)
    bh = (1.0, 0.0, 10.0, 10.0, 0.0)
    dx = 20.0 / n
    g = cg.Grid(2, (n, n), dx, G53, 1, 0, cg.BlackHoleSpacetime(*bh), sr_c2p64_above=above)
    g.set_prim(s)
    r = g.solve(2, 0.9, 1e9, 0.0, 1, subcycles=1, max_steps=6)
    got = g.get_prim()
    want, n_, _, _ = oracle.solve(2, s, 2, dx, 0.9, 1e9, 0.0, 1, G53, subcycles=1, bh=bh, max_steps=6)
    assert r.steps == n_ == 6
    x = np.arange(n) * dx
    X, Y = np.meshgrid(x, x)
    outside = np.sqrt((X - 10.0) ** 2 + (Y - 10.0) ** 2) > 2.0 + 3 * dx
    assert np.all(np.isfinite(got[outside]))
    l1 = l1_outside(got, want, outside)
    assert l1 < 1e-4, l1


def test_gr_fp32_long_accretion_stays_finite(cg):
    """The accretion benchmark's geometry at 256^2 for 40 steps: after about a dozen steps the inflow next to the
    horizon reaches the reference's rootless recovery states (density floor, superluminal garbage
    velocities whose conserved values outgrow FP32's range); the FP32 path hands those to its FP64
    stage and keeps every cell and the CFL time step finite."""
    n = 256
    s = accretion(n, 4)
    g = cg.Grid(2, (n, n), 20.0 / n, G53, 1, 0, cg.BlackHoleSpacetime(1.0, 0.0, 10.0, 10.0, 0.0))
    g.set_prim(s)
    r = g.solve(2, 0.9, 1e9, 0.0, 1, subcycles=1, max_steps=40)
    assert r.steps == 40 and np.isfinite(r.t)
    assert np.isfinite(g.get_prim()).all()


def test_gr_fp32_lorentz_cap_keeps_states_finite(cg):
    """Primitives with gamma_ij v^i v^j >= 1 (the density floor next to the horizon reaches them):
    the conserved state caps W at 1e4 as the reference does (v^2 clamped to 1 - 1e-8).  In FP32 the
    clamp value 1 - 1e-8 rounds to 1 (W would be infinite), so the cap is applied to 1 - v^2.  A
    source step and both sweeps on such cells stay finite wherever the FP64 path does."""
    n = 32
    s = accretion(n, 5)
    s[20, 10:20, 0] = 1e-8
    s[20, 10:20, 1] = 1.5
    s[20, 10:20, 4] = 1e-8
    dx = 20.0 / n
    out = {}
    for prec in (0, 1):
        g = cg.Grid(2, (n, n), dx, G53, prec, 0, cg.BlackHoleSpacetime(1.0, 0.0, 10.0, 10.0, 0.0))
        g.set_prim(s)
        g.rk_source(0.01, 0.0, 1)
        g.sweep(0, 2, 0.01, 0.0, 1)
        g.sweep(1, 2, 0.01, 0.0, 1)
        out[prec] = g.get_prim()
        g.close()
    fin64 = np.isfinite(out[0]).all(axis=-1)
    assert fin64[20, 10:20].all()
    assert np.isfinite(out[1][fin64]).all()


@pytest.mark.parametrize("bhname,bh", [("bh", cases.GR_BH), ("spin", cases.GR_BH_SPIN)])
@pytest.mark.parametrize("dims", [1, 2])
def test_gr_fp32_sweeps_and_source_vs_oracle(cg, oracle, bhname, bh, dims):
    """Single X / Y sweeps and one source step around a Schwarzschild and a spinning hole inside a
    small box (excised cells, stencils crossing the horizon and plain cells)."""
    shape = (40,) if dims == 1 else (24, 26)
    rng = np.random.default_rng(7 + dims)
    s = cases.gr_state(rng, shape)
    dx = 1.0 / shape[-1]
    bhs = cg.BlackHoleSpacetime(*bh)
    for axis in ((0,) if dims == 1 else (0, 1)):
        g = cg.Grid(2, shape, dx, G53, 1, 0, bhs)
        g.set_prim(s)
        g.sweep(axis, 2, 0.002, 0.0, 1)
        want = oracle.sweep(2, s, axis, 2, dx, 0.002, 0.0, 1, G53, bh=bh)
        got = g.get_prim()
        rel = (np.abs(got - want) / (np.abs(want) + 1e-3)).max(axis=-1)
        assert np.median(rel) < 1e-5 and (rel > 1e-3).mean() < 0.02, (axis, np.median(rel), (rel > 1e-3).mean())
    g = cg.Grid(2, shape, dx, G53, 1, 0, bhs)
    g.set_prim(s)
    g.rk_source(0.002, 0.0, 1)
    want = oracle.rk_source(s, dx, 0.002, 0.0, 1, G53, bh)
    got = g.get_prim()
    rel = (np.abs(got - want) / (np.abs(want) + 1e-3)).max(axis=-1)
    assert np.median(rel) < 1e-5 and (rel > 1e-3).mean() < 0.02, (np.median(rel), (rel > 1e-3).mean())
