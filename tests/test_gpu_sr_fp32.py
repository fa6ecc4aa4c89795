"""FP32 bulk path of the special-relativistic system (conserved FP32 storage, primitive recovery
finishing in FP64) against the FP64 oracle.  Stated error: relative L1 density error below 1e-5
after 20 steps of the Kelvin-Helmholtz problem; mass and energy conserved to FP32 rounding."""
import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu
G53 = 5.0 / 3.0


@pytest.fixture(scope="module")
def cg(cosmos_lib):
    import cosmos_gb300
    return cosmos_gb300


@pytest.mark.parametrize("above", [0.0, 2.0])
def test_sr_fp32_kelvin_helmholtz_vs_oracle(cg, oracle, above):
    """above = 0: every primitive recovery finishes in FP64; 2.0 (the default): only states with
    W > 2 do (none here, so the recovery stays in FP32)."""
    n = 64
    s = cases.kelvin_helmholtz(n, 3)
    g = cg.Grid(1, (n, n), 1.0 / n, G53, 1, 1, sr_c2p64_above=above)
    g.set_prim(s)
    m0 = g.field_sums()
    r = g.solve(2, 0.8, 1e9, 0.0, 2, max_steps=20)
    got = g.get_prim()
    m1 = g.field_sums()
    want, nsteps, _, _ = oracle.solve(1, s, 2, 1.0 / n, 0.8, 1e9, 0.0, 2, G53, 1, max_steps=20)
    assert r.steps == nsteps == 20 and r.status == 0
    l1 = np.abs(got[..., 0] - want[..., 0]).mean() / np.abs(want[..., 0]).mean()
    assert l1 < 1e-5, l1
    assert np.abs(got - want).max() < 1e-3
    assert abs(m1[0] - m0[0]) <= 1e-6 * abs(m0[0]) and abs(m1[4] - m0[4]) <= 1e-6 * abs(m0[4])


@pytest.mark.parametrize("shape,axis", [((5, 600), 0), ((600, 5), 1), ((700,), 0), ((3, 3), 0), ((3, 3), 1)])
def test_sr_fp32_single_sweeps_vs_oracle(cg, oracle, shape, axis):
    """One sweep on random data across FP32 X tiles (254 cells) and Y segments (32 rows).  The data
    keep every extrapolated state physical: where SuperBee extrapolates a wild jump to negative
    pressure, the reference's Newton iteration runs on a quartic without a physical root and its
    result (floored at 1e-8) depends on rounding along the iteration, which no other arithmetic
    reproduces."""
    rng = np.random.default_rng(shape[0] * 7 + axis)
    for lim in (0, 1, 2):
        for bc in (0, 1):
            s = cases.sr_mild_state(rng, shape)
            g = cg.Grid(1, shape, 0.01, G53, 1, bc, sr_c2p64_above=0.0)
            g.set_prim(s)
            g.sweep(axis, 2, 0.002, 0.0, lim)
            got = g.get_prim()
            want = oracle.sweep(1, s, axis, 2, 0.01, 0.002, 0.0, lim, G53, bc)
            rel = (np.abs(got - want) / (np.abs(want) + 1e-3)).max(axis=-1)
            assert np.median(rel) < 1e-5, (lim, bc, np.median(rel))
            assert rel.max() < 1e-2, (lim, bc, rel.max())
            assert (rel > 1e-4).mean() < 0.01, (lim, bc, (rel > 1e-4).mean())


def test_sr_fp32_dt_and_wavespeed(cg, oracle):
    n = 48
    s = cases.kelvin_helmholtz(n, 5)
    g = cg.Grid(1, (n, n), 1.0 / n, G53, 1, 1)
    g.set_prim(s)
    h = cg.Grid(1, (n, n), 1.0 / n, G53, 0, 1)
    h.set_prim(s)
    a, b = g.max_wavespeed(), h.max_wavespeed()
    assert abs(a - b) <= 1e-6 * b
