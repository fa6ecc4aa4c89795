"""GPU adjoint of the Newtonian SLIC step (cosmos_grid_adjoint) against the oracle's
tangent-linear model (dual numbers through the FP64 restatement of the reference, same fixed
time steps) and against central finite differences of the GPU forward.

Tolerances: FP64 gradient vs the oracle TLM, directional derivatives <g, d> to 1e-10 relative on
smooth data (different but mathematically equal evaluation orders: conserved-variable adjoint vs
primitive-storage dual numbers) and 1e-7 on discontinuous data; vs finite differences to 1e-4;
FP32 gradient within 3e-3 (relative L2) of the FP64 gradient: over 20 steps the piecewise limiter takes
a different branch in FP32 than in FP64 at a few near-tie cells, which moves the gradient there by
O(1) relative amounts (measured: 2e-4 to 1.4e-3 on the shapes below)."""
import numpy as np
import pytest

import cases
from conftest import bit_equal

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cg(cosmos_lib):
    import cosmos_gb300
    return cosmos_gb300


def grid(cg, prim, precision=0, bc=0):
    g = cg.Grid(0, prim.shape[:-1], 1.0 / prim.shape[-2], 1.4, precision, bc)
    g.set_prim(prim)
    return g


def check_vs_tlm(cg, oracle, p0, target, nsteps, K, lim, bc, tol, seed):
    g = grid(cg, p0, 0, bc)
    dx = 1.0 / p0.shape[-2]
    loss, grad, dts, _ = g.adjoint(target, nsteps, 0.6, 0.0, lim, checkpoint_every=K)
    rng = np.random.default_rng(seed)
    for _ in range(3):
        d = rng.standard_normal(p0.shape)
        L0, dL = oracle.tlm_newton(p0, d, target, dx, dts, 0.0, lim, 1.4, bc)
        assert abs(loss - L0) <= 1e-13 * abs(L0), (loss, L0)
        got = float(np.sum(grad * d))
        assert abs(got - dL) <= tol * abs(dL) + 1e-14, (got, dL, abs(got - dL) / abs(dL))
    return grad, dts


@pytest.mark.parametrize("shape", [(37,), (2,), (3,), (5,), (9, 13), (2, 5), (4, 3)])
@pytest.mark.parametrize("lim", [0, 1, 2])
@pytest.mark.parametrize("bc", [0, 1])
def test_fp64_adjoint_matches_oracle_tlm_smooth(cg, oracle, shape, lim, bc):
    """Tiny lines exercise the ghost-cell pull-back (mirror, and periodic aliasing for n <= 4)."""
    p0 = cases.smooth_state(shape, 7 + lim)
    target = cases.smooth_state(shape, 8)[..., 0] * 0.9
    check_vs_tlm(cg, oracle, p0, target, 7, 3, lim, bc, 1e-10, hash((shape, lim, bc)) % 2**32)


@pytest.mark.parametrize("shape", [(130,), (21, 140), (70, 9)])
@pytest.mark.parametrize("lim", [0, 1, 2])
def test_fp64_adjoint_matches_oracle_tlm_discontinuous(cg, oracle, shape, lim):
    """Random discontinuous data across several X tiles (120 cells) and Y tiles (56 cells)."""
    rng = np.random.default_rng(5 + lim)
    p0 = cases.newton_state(rng, shape)
    target = cases.newton_state(rng, shape)[..., 0]
    for bc in (0, 1):
        check_vs_tlm(cg, oracle, p0, target, 5, 2, lim, bc, 1e-7, lim + 10 * bc)


def segment_bytes(shape, K, elem=8, ops=3):
    """Device bytes of one checkpoint segment's sweep inputs (the library's padded layout)."""
    pitch = -(-shape[1] // 64) * 64
    fstride = -(-pitch * shape[0] // 64) * 64
    return K * ops * fstride * 5 * elem


@pytest.mark.parametrize("precision", [0, 1])
def test_checkpoint_interval_and_keep_budget_do_not_change_the_gradient(cg, precision):
    """Every checkpoint interval, and every keep budget: all segments' sweep inputs kept from the
    forward pass (the default), the last segment only (each earlier one recomputed), and two."""
    p0 = cases.smooth_state((20, 24), 3)
    target = p0[..., 0] * 1.1
    grads = []
    for K in (1, 4, 11, 11 + 5):
        for keep in (-1, 0, 2 * segment_bytes((20, 24), K, 8 if precision == 0 else 4)):
            g = grid(cg, p0, precision)
            g.set_adjoint_keep(keep)
            _, gr, dts, _ = g.adjoint(target, 11, 0.8, 0.0, 2, checkpoint_every=K)
            grads.append(gr)
    assert all(bit_equal(grads[0], x) for x in grads[1:])
    if precision == 1:
        return
    # the caller's dts reproduce the CFL run exactly, and the grid ends in the final state
    g = grid(cg, p0)
    loss2, gr2, dts2, _ = g.adjoint(target, 11, 0.8, 0.0, 2, checkpoint_every=4, dts=dts)
    assert bit_equal(gr2, grads[0]) and bit_equal(dts2, dts)
    h = grid(cg, p0)
    h.solve(2, 0.8, 1e300, 0.0, 2, max_steps=11)
    assert bit_equal(g.get_prim(), h.get_prim())


@pytest.mark.parametrize("shape,nsteps,K", [((48,), 30, 7), ((16, 20), 20, 6), ((24, 24), 100, 10)])
def test_fp64_adjoint_vs_finite_differences(cg, shape, nsteps, K):
    """Central differences of the GPU FP64 forward with the same fixed dts (the last case is the
    100-step, checkpoint-every-10 setting of the batched workload at reduced size)."""
    p0 = cases.smooth_state(shape, 21)
    target = cases.smooth_state(shape, 22)[..., 0]
    g = grid(cg, p0)
    loss, grad, dts, _ = g.adjoint(target, nsteps, 0.8, 0.0, 2, checkpoint_every=K)
    rng = np.random.default_rng(9)
    h = 1e-7
    for _ in range(2):
        d = rng.standard_normal(p0.shape)
        Ls = []
        for sgn in (1, -1):
            gg = grid(cg, p0 + sgn * h * d)
            Ls.append(gg.adjoint(target, nsteps, 0.8, 0.0, 2, checkpoint_every=K, dts=dts)[0])
        fd = (Ls[0] - Ls[1]) / (2 * h)
        got = float(np.sum(grad * d))
        assert abs(fd - got) <= 1e-4 * abs(got), (fd, got)


@pytest.mark.parametrize("shape", [(200,), (40, 48), (37, 45), (61, 253), (130, 7)])
def test_fp32_adjoint_close_to_fp64(cg, shape):
    """FP32 runs two lines per thread: odd line counts leave the last pair incomplete in X (odd
    rows) and in Y (odd columns); (61, 253) spans two X tiles and two Y tiles.  A wrong lane would
    show as an error concentrated in the last row or column, well above the tolerance."""
    p0 = cases.smooth_state(shape, 31)
    target = cases.smooth_state(shape, 32)[..., 0]
    g64 = grid(cg, p0, 0)
    l64, gr64, dts, _ = g64.adjoint(target, 20, 0.8, 0.0, 2, checkpoint_every=5)
    g32 = grid(cg, p0, 1)
    l32, gr32, _, _ = g32.adjoint(target, 20, 0.8, 0.0, 2, checkpoint_every=5, dts=dts)
    assert abs(l32 - l64) <= 1e-5 * abs(l64)
    err = np.linalg.norm(gr32 - gr64) / np.linalg.norm(gr64)
    assert err < 3e-3, err


def test_adjoint_errors(cg):
    g = grid(cg, cases.smooth_state((8, 8), 1))
    with pytest.raises(ValueError):
        g.adjoint(np.zeros((8, 9)), 3, 0.8, 0.0, 2)
    with pytest.raises(cg.CosmosError):
        g.adjoint(np.zeros((8, 8)), 0, 0.8, 0.0, 2)
    with pytest.raises(cg.CosmosError):
        g.adjoint(np.zeros((8, 8)), 3, 0.8, 0.0, 2, dts=np.array([0.01, -1.0, 0.01]))
    sr = cg.Grid(1, (8,), 0.1, 5.0 / 3.0, cg.FP32)  # the SR adjoint covers FP64 grids
    sr.set_prim(cases.sr_state(np.random.default_rng(0), (8,)))
    with pytest.raises(cg.CosmosError) as e:
        sr.adjoint(np.zeros(8), 3, 0.8, 0.0, 2)
    assert e.value.code == 4
