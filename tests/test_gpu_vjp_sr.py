"""GPU adjoint of the special-relativistic SLIC step (cosmos_grid_adjoint on an FP64 SR grid)
against the host build of the same sweep-adjoint cell function and against the oracle's SR
tangent-linear model (dual numbers through every primitive recovery's Newton iteration, same fixed
time steps).

Tolerances: the GPU gradient runs the host build's arithmetic in the same order (IEEE FP64, no
contraction on either side) on states from the reference-exact forward: within 1e-12 of the largest
component.  Directional derivatives <g, d> against the tangent model to 1e-10 relative; the loss to
1e-13."""
import numpy as np
import pytest

from test_oracle_adjoint import sr_smooth_state
from test_sr_adjoint_host import G, host_adjoint, reverse_gradient  # noqa: F401  (module fixture)

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cg(cosmos_lib):
    import cosmos_gb300
    return cosmos_gb300


def sr_grid(cg, p0, bc, precision=0):
    g = cg.Grid(1, p0.shape[:-1], 1.0 / p0.shape[-2], G, precision, bc)
    g.set_prim(p0)
    return g


@pytest.mark.parametrize("shape", [(20,), (2,), (3,), (8, 10), (2, 5), (4, 3)])
@pytest.mark.parametrize("lim", [0, 1, 2])
@pytest.mark.parametrize("bc", [0, 1])
def test_sr_adjoint_matches_host_build_and_tangent_model(cg, oracle, host_adjoint, shape, lim, bc):
    p0 = sr_smooth_state(shape, 3 + lim)
    target = sr_smooth_state(shape, 11)[..., 0]
    dx = 1.0 / shape[-1]
    dts = np.full(4, 0.15 * dx)
    loss, grad, _, _ = sr_grid(cg, p0, bc).adjoint(target, len(dts), 0.5, 0.0, lim, checkpoint_every=3, dts=dts)
    host = reverse_gradient(oracle, host_adjoint, p0, target, dx, dts, 0.0, lim, bc)
    assert np.abs(grad - host).max() <= 1e-12 * np.abs(host).max()
    rng = np.random.default_rng(hash((shape, lim, bc)) % 2**32)
    for _ in range(2):
        d = rng.standard_normal(p0.shape)
        L0, dL = oracle.tlm_sr(p0, d, target, dx, dts, 0.0, lim, G, bc)
        assert abs(loss - L0) <= 1e-13 * abs(L0), (loss, L0)
        got = float(np.sum(grad * d))
        assert abs(got - dL) <= 1e-10 * max(1.0, abs(dL)), (got, dL)


def test_sr_adjoint_cfl_steps_and_bias(cg, oracle, host_adjoint):
    """Time steps from the CFL rule of the forward run (returned and then held fixed), biased slopes."""
    shape = (12, 16)
    p0 = sr_smooth_state(shape, 21)
    target = sr_smooth_state(shape, 22)[..., 0]
    dx = 1.0 / shape[-1]
    loss, grad, dts, _ = sr_grid(cg, p0, 0).adjoint(target, 5, 0.6, 0.3, 1, checkpoint_every=2)
    assert (dts > 0).all()
    host = reverse_gradient(oracle, host_adjoint, p0, target, dx, dts, 0.3, 1, 0)
    assert np.abs(grad - host).max() <= 1e-12 * np.abs(host).max()
    d = np.random.default_rng(23).standard_normal(p0.shape)
    L0, dL = oracle.tlm_sr(p0, d, target, dx, dts, 0.3, 1, G, 0)
    assert abs(loss - L0) <= 1e-13 * abs(L0)
    assert abs(float(np.sum(grad * d)) - dL) <= 1e-10 * max(1.0, abs(dL))


def test_sr_adjoint_rejects_fp32_and_black_hole_grids(cg):
    from cosmos_gb300._lib import CosmosError
    p0 = sr_smooth_state((16,), 1)
    with pytest.raises(CosmosError):
        sr_grid(cg, p0, 0, precision=1).adjoint(p0[..., 0], 2, 0.5, 0.0, 1)
    hole = cg.BlackHoleSpacetime(0.05, 0.0, 0.5, 0.0, 0.0)
    g = cg.Grid(2, (16,), 1.0 / 16, G, 0, 0, black_hole=hole)
    g.set_prim(p0 * np.array([1.0, 0.3, 0.3, 0.3, 0.5]))
    with pytest.raises(CosmosError):
        g.adjoint(p0[..., 0], 2, 0.5, 0.0, 1)
