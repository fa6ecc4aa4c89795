"""Failure detection on the GPU, exercised without faulting or hanging the device.

* Bounded waits: the batched launch's grid-barrier wait is bounded; with its limit set to one poll
  (cosmos_batch_set_wait_limit) the waits run out, the launch ends at the next barrier and
  cosmos_batch_run_end reports the timeout (COSMOS_ECUDA); with the default limit restored the same
  batch runs again.
* Poison inputs through every path (FP64 and FP32; Newtonian, special-relativistic, black hole;
  single grids, the batched launch and the AMR driver): a NaN density makes the run stop with
  COSMOS_ENONFINITE and COSMOS_STATUS_NONFINITE, where the reference would carry the NaN on.
  Negative pressure and superluminal velocities are states the reference runs through without a
  check: the FP64 path reproduces the reference's arithmetic on them bit for bit (oracle), the FP32
  path keeps them finite.
* A Newton solve that hits its iteration cap sets COSMOS_STATUS_NEWTON_CAP (black-hole accretion,
  where the reference's primitive recovery finds no physical root next to the horizon).
The reference's floors and cap: RelativisticEuler/RelativisticEulerStateVector.cpp:45-100.
"""
import numpy as np
import pytest

import cases
from conftest import bit_equal

pytestmark = pytest.mark.gpu

ENONFINITE, ECUDA = 3, 2
STATUS_NONFINITE, STATUS_NEWTON_CAP = 1, 2
BH = (1.0, 0.0, 10.0, 10.0, 0.0)


@pytest.fixture(scope="module")
def cg(cosmos_lib):
    import cosmos_gb300
    return cosmos_gb300


def _batch(cg, precision):
    shapes = [(96,), (40, 56), (72, 24)]
    b = cg.Batch(shapes, [1.0 / sh[-1] for sh in shapes], 1.4, precision, cg.BC_TRANSMISSIVE)
    states = [cases.riemann(sh, 40 + i) for i, sh in enumerate(shapes)]
    for i, st in enumerate(states):
        b.set_prim(i, st)
    return b, states


@pytest.mark.parametrize("precision", [0, 1])
def test_batch_barrier_wait_runs_out(cg, precision):
    b, states = _batch(cg, precision)
    b.set_wait_limit(1)
    b.run_begin(0.9, 1e30, 0.0, cg.MINBEE)
    b.run_steps(10)
    with pytest.raises(cg.CosmosError) as e:
        b.run_end()
    assert e.value.code == ECUDA and "timed out" in str(e.value)
    # the default limit restored, the same batch runs again from fresh data
    b.set_wait_limit(0)
    for i, st in enumerate(states):
        b.set_prim(i, st)
    b.run_begin(0.9, 1e30, 0.0, cg.MINBEE, max_steps=3)
    b.run_steps(3)
    res = b.run_end()
    assert all(r.steps == 3 for r in res)
    with pytest.raises(cg.CosmosError):
        b.set_wait_limit(-1)
    b.close()


def _grid(cg, system, precision, shape):
    rng = np.random.default_rng(11)
    if system == cg.GR:
        n = shape[-1]
        g = cg.Grid(cg.GR, shape, 20.0 / n, 5.0 / 3.0, precision, cg.BC_TRANSMISSIVE,
                    cg.BlackHoleSpacetime(*BH))
        s = cases.gr_state(rng, shape)
    else:
        g = cg.Grid(system, shape, 1.0 / shape[-1], 1.4 if system == cg.NEWTONIAN else 5.0 / 3.0, precision,
                    cg.BC_PERIODIC)
        s = cases.state(system, rng, shape)
    return g, s


@pytest.mark.parametrize("system", [0, 1, 2])
@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("dims", [1, 2])
def test_nan_density_stops_the_run(cg, system, precision, dims):
    shape = (48,) if dims == 1 else (32, 48)
    g, s = _grid(cg, system, precision, shape)
    s[(3,) if dims == 1 else (3, 5)][0] = np.nan  # far from the hole at (10, 10)
    g.set_prim(s)
    with pytest.raises(cg.CosmosError) as e:
        g.solve(2, 0.9, 1e9, 0.0, cg.MINBEE, max_steps=4)
    assert e.value.code == ENONFINITE and "non-finite" in str(e.value)
    g.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_nan_in_one_batched_grid_is_reported(cg, precision):
    b, states = _batch(cg, precision)
    states[1][10, 20, 0] = np.nan
    b.set_prim(1, states[1])
    b.run_begin(0.9, 1e30, 0.0, cg.MINBEE, max_steps=4)
    b.run_steps(4)
    with pytest.raises(cg.CosmosError) as e:
        b.run_end()
    assert e.value.code == ENONFINITE
    b.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_nan_in_amr_run_is_reported(cg, precision):
    a = cg.AMR(cg.NEWTONIAN, (12, 16), 1.0 / 16, 1.4, precision)
    s = cases.riemann((12, 16), 8)
    s[4, 4, 4] = np.nan
    a.set_prim(s)
    with pytest.raises(cg.CosmosError):
        a.solve(0.9, 0.03, 3.0, 2)
    a.close()


def test_negative_pressure_runs_as_the_reference(cg, oracle):
    """The reference has no check on pressure: its sound speed is NaN there and drops out of the
    CFL maximum (`if (w > max)`).  The FP64 path takes the same steps bit for bit."""
    rng = np.random.default_rng(5)
    s = cases.newton_state(rng, (24, 32))
    s[7, 9, 4] = -0.05
    s[2, 30, 4] = -0.2
    g = cg.Grid(cg.NEWTONIAN, (24, 32), 1.0 / 32, 1.4)
    g.set_prim(s)
    r = g.solve(2, 0.9, 1e9, 0.0, cg.VANLEER, max_steps=6)
    want, steps, t, _ = oracle.solve(0, s, 2, 1.0 / 32, 0.9, 1e9, 0.0, 1, 1.4, 0, max_steps=6)
    assert r.steps == steps == 6 and r.t == t
    assert bit_equal(g.get_prim(), want)
    g32 = cg.Grid(cg.NEWTONIAN, (24, 32), 1.0 / 32, 1.4, cg.FP32)
    g32.set_prim(s)
    g32.solve(2, 0.9, 1e9, 0.0, cg.VANLEER, max_steps=6)
    assert np.isfinite(g32.get_prim()).all()


def test_superluminal_sr_input_runs_as_the_reference(cg, oracle):
    """|v| >= 1 in the primitives: the reference clamps v^2 to 1 - 1e-8 when it forms the conserved
    state (W = 1e4), whose primitive recovery then has no physical root; it leaves the density at
    its 1e-8 floor and superluminal velocities (|v| about 3.5 here) and carries on.  The FP64 path
    does the same bit for bit; the FP32 path stays finite."""
    rng = np.random.default_rng(6)
    s = cases.sr_state(rng, (40,))
    s[17, 1] = 1.2
    s[23, 1] = -1.0
    g = cg.Grid(cg.SR, (40,), 1.0 / 40, 5.0 / 3.0)
    g.set_prim(s)
    r = g.solve(2, 0.5, 1e9, 0.0, cg.MINBEE, max_steps=3)
    want, steps, t, _ = oracle.solve(1, s, 2, 1.0 / 40, 0.5, 1e9, 0.0, 2, 5.0 / 3.0, 0, max_steps=3)
    assert r.steps == steps == 3 and r.t == t
    assert bit_equal(g.get_prim(), want)
    g32 = cg.Grid(cg.SR, (40,), 1.0 / 40, 5.0 / 3.0, cg.FP32)
    g32.set_prim(s)
    g32.solve(2, 0.5, 1e9, 0.0, cg.MINBEE, max_steps=3)
    assert np.isfinite(g32.get_prim()).all()


@pytest.mark.parametrize("precision", [0, 1])
def test_newton_cap_is_reported(cg, precision):
    """Accretion onto the hole: after a few dozen steps the inflow next to the horizon reaches
    states for which the reference's primitive recovery has no physical root; its Newton solves
    stop at their cap and the run's status carries COSMOS_STATUS_NEWTON_CAP.  (A few steps later the
    reference-exact run produces a non-finite state there -- at 128^2 at step 32 -- and stops with
    COSMOS_ENONFINITE; the cap must be reported before that.)"""
    n = 128
    rng = np.random.default_rng(4)
    s = np.zeros((n, n, 5))
    s[..., 0] = np.exp(0.01 * rng.standard_normal((n, n)))
    s[..., 4] = 0.01
    seen = None
    for k in (8, 12, 16, 20, 24, 28):
        g = cg.Grid(cg.GR, (n, n), 20.0 / n, 5.0 / 3.0, precision, cg.BC_TRANSMISSIVE, cg.BlackHoleSpacetime(*BH))
        g.set_prim(s)
        try:
            r = g.solve(2, 0.9, 1e9, 0.0, cg.VANLEER, max_steps=k)
        except cg.CosmosError as e:
            assert e.code == ENONFINITE
            break
        finally:
            g.close()
        assert r.steps == k
        if r.status & STATUS_NEWTON_CAP:
            seen = k
            break
    assert seen is not None, "no Newton cap reported before the run stopped"
