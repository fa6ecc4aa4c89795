"""GPU adjoints of the relativistic SLIC steps (cosmos_grid_adjoint on FP64 SR grids, and on FP64
black-hole grids for the flux step alone and with its RK source half-steps) against the host build of the same
sweep-adjoint cell function and against the oracle's tangent-linear models (dual numbers through
every primitive recovery's Newton iteration, same fixed time steps).

Tolerances: the GPU gradient runs the host build's arithmetic in the same order (IEEE FP64, no
contraction on either side) on states from the reference-exact forward: within 1e-12 of the largest
component.  Directional derivatives <g, d> against the tangent model to 1e-10 relative; the loss to
1e-13."""
import numpy as np
import pytest

from test_oracle_adjoint import gr_smooth_state, sr_smooth_state
from test_rel_adjoint_host import G, HOLES, host_adjoint, reverse_gradient  # noqa: F401  (module fixture)

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cg(cosmos_lib):
    import cosmos_gb300
    return cosmos_gb300


def rel_grid(cg, system, p0, bc=0, precision=0, bh=None):
    hole = None if bh is None else cg.BlackHoleSpacetime(*bh)
    g = cg.Grid(system, p0.shape[:-1], 1.0 / p0.shape[-2], G, precision, bc, black_hole=hole)
    g.set_prim(p0)
    return g


def check(cg, oracle, host_adjoint, system, p0, target, dts, lim, bc, bh, bias=0.0, seed=0, sub=0):
    dx = 1.0 / p0.shape[-2]
    g = rel_grid(cg, system, p0, bc, bh=bh)
    g.set_adjoint_keep(0)  # earlier segments recomputed (keeping them is checked bit for bit below)
    loss, grad, dts_out, _ = g.adjoint(target, len(dts) if dts is not None else 5, 0.6, bias, lim, checkpoint_every=3,
                                       dts=dts, subcycles=sub)
    if dts is None:
        assert (dts_out > 0).all()
        dts = dts_out
    host = reverse_gradient(oracle, host_adjoint, system, p0, target, dx, dts, bias, lim, bc, bh, sub)
    assert np.abs(grad - host).max() <= 1e-12 * np.abs(host).max()
    rng = np.random.default_rng(seed)
    for _ in range(2):
        d = rng.standard_normal(p0.shape)
        if system == 1:
            L0, dL = oracle.tlm_sr(p0, d, target, dx, dts, bias, lim, G, bc)
        else:
            L0, dL = oracle.tlm_gr(p0, d, target, dx, dts, bias, lim, G, bh, sub)
        assert abs(loss - L0) <= 1e-13 * abs(L0), (loss, L0)
        got = float(np.sum(grad * d))
        assert abs(got - dL) <= 1e-10 * max(1.0, abs(dL)), (got, dL)


@pytest.mark.parametrize("shape", [(20,), (2,), (3,), (8, 10), (2, 5), (4, 3)])
@pytest.mark.parametrize("lim", [0, 1, 2])
@pytest.mark.parametrize("bc", [0, 1])
def test_sr_adjoint_matches_host_build_and_tangent_model(cg, oracle, host_adjoint, shape, lim, bc):
    p0 = sr_smooth_state(shape, 3 + lim)
    target = sr_smooth_state(shape, 11)[..., 0]
    dts = np.full(4, 0.15 / shape[-1])
    check(cg, oracle, host_adjoint, 1, p0, target, dts, lim, bc, None, seed=hash((shape, lim, bc)) % 2**32)


def test_sr_adjoint_cfl_steps_and_bias(cg, oracle, host_adjoint):
    """Time steps from the CFL rule of the forward run (returned and then held fixed), biased slopes."""
    p0 = sr_smooth_state((12, 16), 21)
    check(cg, oracle, host_adjoint, 1, p0, sr_smooth_state((12, 16), 22)[..., 0], None, 1, 0, None, bias=0.3, seed=23)


@pytest.mark.parametrize("dims,bh", [(1, (0.05, 0.0, 0.5, 0.0, 0.0))] + [(2, h) for h in HOLES])
@pytest.mark.parametrize("lim", [0, 1, 2])
def test_gr_adjoint_matches_host_build_and_tangent_model(cg, oracle, host_adjoint, dims, bh, lim):
    """Black-hole flux steps (zero subcycles) around holes that excise cells of the grid."""
    shape = (24,) if dims == 1 else (10, 12)
    p0 = gr_smooth_state(shape, 5 + lim)
    target = gr_smooth_state(shape, 13)[..., 0]
    dts = np.full(4, 0.1 / shape[-1])
    check(cg, oracle, host_adjoint, 2, p0, target, dts, lim, 0, bh, seed=dims * 10 + lim)


@pytest.mark.parametrize("dims,bh", [(1, (0.05, 0.0, 0.5, 0.0, 0.0)), (2, HOLES[1])])
@pytest.mark.parametrize("sub", [1, 2])
def test_gr_adjoint_with_source_steps(cg, oracle, host_adjoint, dims, bh, sub):
    """The whole black-hole step: `sub` RK source half-steps before and after each flux step; four
    steps with checkpoints every three, so the first segment is recomputed (RK steps included)."""
    shape = (24,) if dims == 1 else (10, 12)
    p0 = gr_smooth_state(shape, 7 + sub)
    target = gr_smooth_state(shape, 13)[..., 0]
    dts = np.full(4, 0.1 / shape[-1])
    check(cg, oracle, host_adjoint, 2, p0, target, dts, 1, 0, bh, seed=dims * 10 + sub, sub=sub)


def test_relativistic_adjoint_rejects_fp32_grids(cg):
    from cosmos_gb300._lib import CosmosError
    p0 = sr_smooth_state((16,), 1)
    with pytest.raises(CosmosError):
        rel_grid(cg, 1, p0, precision=1).adjoint(p0[..., 0], 2, 0.5, 0.0, 1)
    q0 = gr_smooth_state((16,), 1)
    with pytest.raises(CosmosError):
        rel_grid(cg, 2, q0, precision=1, bh=HOLES[0]).adjoint(q0[..., 0], 2, 0.5, 0.0, 1)


def test_keep_budget_does_not_change_the_relativistic_gradient(cg):
    """Sweep inputs kept from the forward pass (the default) or recomputed from the checkpoints:
    the same gradient bit for bit, SR and black hole with source half-steps."""
    from conftest import bit_equal
    p0 = sr_smooth_state((8, 10), 4)
    q0 = gr_smooth_state((8, 10), 5)
    for system, s0, bh, sub in ((1, p0, None, 0), (2, q0, HOLES[1], 1)):
        out = []
        for keep in (-1, 0):
            g = rel_grid(cg, system, s0, bh=bh)
            g.set_adjoint_keep(keep)
            out.append(g.adjoint(s0[..., 0] * 1.05, 5, 0.5, 0.0, 1, checkpoint_every=2, subcycles=sub))
        assert bit_equal(out[0][1], out[1][1]) and out[0][0] == out[1][0]
