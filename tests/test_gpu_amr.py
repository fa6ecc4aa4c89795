"""The Level-1 AMR driver on the GPU (cosmos_amr_*): FP64 runs equal the reference's own
solveLevel1AMR / solve2DLevel1AMR runs (committed fixtures) and the oracle's driver bit for bit --
coarse and fine cells, both flag sets and the step counts; FP32 runs keep the level invariants and
stay near the FP64 run."""
import os

import numpy as np
import pytest

import cases
from conftest import bit_equal

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def cg(cosmos_lib):
    import cosmos_gb300
    return cosmos_gb300


def run_amr(cg, system, s, T, tol, order, precision=0):
    shape = s.shape[:-1]
    a = cg.AMR(system, shape, 1.0 / shape[-1], cases.SYS_GAMMA[system], precision)
    try:
        a.set_prim(s)
        n, nf, t, status = a.solve(0.9, T, tol, order)
        cp, fp, cf, ff = a.get()
    finally:
        a.close()
    return n, nf, t, status, cp, fp, cf, ff


def amr_state(shape, system, seed):
    rng = np.random.default_rng(seed)
    x = np.linspace(0, 1, shape[-1])
    s = np.zeros(shape + (5,))
    s[..., 0] = 1.0 + 0.3 * np.sin(6 * x) + np.where(x > 0.5, 0.8, 0.0) + 0.1 * rng.uniform(0, 1, shape)
    s[..., 1] = (0.3 if system == 0 else 0.2) * rng.uniform(-1, 1, shape)
    if len(shape) == 2:
        s[..., 2] = 0.1 * rng.uniform(-1, 1, shape)
    s[..., 4] = 1.0 + 0.5 * np.where(x < 0.3, 1.0, 0.0)
    return s


def check_invariants(cf, ff):
    """Every coarse cell is either active (its children off) or refined (all children on)."""
    kids = ff.reshape(-1, 2) if cf.ndim == 1 else \
        ff.reshape(cf.shape[0], 2, cf.shape[1], 2).transpose(0, 2, 1, 3).reshape(cf.shape + (4,))
    kids = kids.reshape(cf.shape + (-1,))
    assert np.all(kids.all(-1) | ~kids.any(-1))
    assert np.array_equal(cf, ~kids.any(-1))


def test_amr_level1_matches_reference_runs(cg):
    G = dict(np.load(os.path.join(HERE, "golden", "amr_golden.npz")))
    keys = sorted(k[:-3] for k in G if k.endswith("_in") and k[3:-3].isdigit())  # Level-1 runs: amr<k>
    assert len(keys) == 8
    for k in keys:
        s = G[k + "_in"]
        system, dims, T, order, tol, nsteps = G[k + "_args"]
        n, nf, t, status, cp, fp, cf, ff = run_amr(cg, int(system), s, T, tol, int(order))
        assert n == int(nsteps) and status == 0, k
        assert bit_equal(cp.reshape(-1), G[k + "_coarse"]) and bit_equal(fp.reshape(-1), G[k + "_fine"]), k
        assert np.array_equal(cf.reshape(-1), G[k + "_cflags"].astype(bool)), k
        assert np.array_equal(ff.reshape(-1), G[k + "_fflags"].astype(bool)), k


@pytest.mark.parametrize("system", [0, 1])
@pytest.mark.parametrize("shape,T", [((37,), 0.15), ((96,), 0.1), ((13, 17), 0.06), ((24, 9), 0.05)])
@pytest.mark.parametrize("order", [1, 2])
def test_amr_level1_matches_oracle(cg, oracle, system, shape, T, order):
    s = amr_state(shape, system, 31 + len(shape) + order)
    tol = 3.0
    n, nf, t, status, cp, fp, cf, ff = run_amr(cg, system, s, T, tol, order)
    wn, wnf, wcp, wfp, wcf, wff = oracle.amr_level1(system, s, 1.0 / shape[-1], 0.9, T, tol, order,
                                                    cases.SYS_GAMMA[system])
    assert (n, nf) == (wn, wnf) and t >= T
    assert bit_equal(cp.reshape(-1), wcp) and bit_equal(fp.reshape(-1), wfp)
    assert np.array_equal(cf.reshape(-1), wcf.astype(bool)) and np.array_equal(ff.reshape(-1), wff.astype(bool))
    check_invariants(cf, ff)


@pytest.mark.parametrize("system", [0, 1])
def test_amr_without_refinement_is_the_plain_solver(cg, oracle, system):
    """With a tolerance no gradient reaches, nothing refines: the coarse grid follows the plain
    SLIC solve with bias 0 and limiter 1, and the fine grid holds the injected coarse cells."""
    shape = (16, 20)
    s = amr_state(shape, system, 5)
    n, nf, t, status, cp, fp, cf, ff = run_amr(cg, system, s, 0.04, 1e30, 2)
    want, wn, _, _ = oracle.solve(system, s, 2, 1.0 / shape[-1], 0.9, 0.04, 0.0, 1, cases.SYS_GAMMA[system])
    assert n == wn == nf and cf.all() and not ff.any()
    assert bit_equal(cp, want)
    assert bit_equal(fp, np.repeat(np.repeat(cp, 2, axis=0), 2, axis=1))


@pytest.mark.parametrize("system", [0, 1])
@pytest.mark.parametrize("shape,T", [((128,), 0.1), ((32, 40), 0.05)])
def test_amr_fp32_keeps_levels_consistent(cg, system, shape, T):
    s = amr_state(shape, system, 77)
    r64 = run_amr(cg, system, s, T, 3.0, 2, precision=0)
    r32 = run_amr(cg, system, s, T, 3.0, 2, precision=1)
    n, nf, t, status, cp, fp, cf, ff = r32
    assert np.isfinite(cp).all() and np.isfinite(fp).all() and t >= T
    check_invariants(cf, ff)
    rho64, rho32 = r64[4][..., 0], cp[..., 0]
    assert np.abs(rho32 - rho64).sum() / np.abs(rho64).sum() < 2e-3
    assert np.mean(cf == r64[6]) > 0.95


def test_amr_rejects_unsupported_setups(cg):
    from cosmos_gb300._lib import CosmosError, EUNSUPPORTED
    with pytest.raises(CosmosError) as e:
        cg.AMR(cg.GR, (16,), 1.0 / 16, 5.0 / 3.0)
    assert e.value.code == EUNSUPPORTED


def test_reference_named_amr_entry_points(cg, oracle):
    s = amr_state((40,), 1, 9)
    cp, fp, cf, ff = cg.RelativisticEulerAMR.solveLevel1AMR(s, 1.0 / 40, 0.9, 0.1, 2.0, 2,
                                                             cg.EulerMaterialParameters(5.0 / 3.0))
    _, _, wcp, wfp, wcf, wff = oracle.amr_level1(1, s, 1.0 / 40, 0.9, 0.1, 2.0, 2, 5.0 / 3.0)
    assert bit_equal(cp.reshape(-1), wcp) and bit_equal(fp.reshape(-1), wfp)
    assert np.array_equal(cf, wcf.astype(bool)) and np.array_equal(ff, wff.astype(bool))


def run_amr2(cg, system, s, T, tol, order, precision=0):
    shape = s.shape[:-1]
    a = cg.AMR(system, shape, 1.0 / shape[-1], cases.SYS_GAMMA[system], precision, levels=2)
    try:
        a.set_prim(s)
        n, nf, t, status = a.solve(0.9, T, tol, order)
        out = a.get()
        runs = (a.mid_run, a.fine_run)
    finally:
        a.close()
    return (n, nf, t, status, runs) + out


def test_amr_level2_matches_reference_runs(cg):
    """Level-2 drivers (three levels): the reference's own solveLevel2AMR / solve2DLevel2AMR runs."""
    G = dict(np.load(os.path.join(HERE, "golden", "amr_golden.npz")))
    keys = sorted(k[:-3] for k in G if k.startswith("amr2_") and k.endswith("_in") and k[5:-3].isdigit())
    assert len(keys) == 8
    for k in keys:
        s = G[k + "_in"]
        system, dims, T, order, tol, nsteps = G[k + "_args"]
        n, nf, t, status, runs, cp, mp, fp, cf, mf, ff = run_amr2(cg, int(system), s, T, tol, int(order))
        assert n == int(nsteps) and status == 0, k
        for name, got in (("coarse", cp), ("mid", mp), ("fine", fp)):
            assert bit_equal(got.reshape(-1), G[f"{k}_{name}"]), (k, name)
        for name, got in (("cflags", cf), ("mflags", mf), ("fflags", ff)):
            assert np.array_equal(got.reshape(-1), G[f"{k}_{name}"].astype(bool)), (k, name)


@pytest.mark.parametrize("system", [0, 1])
@pytest.mark.parametrize("shape,T,tol", [((37,), 0.1, 1.0), ((13, 11), 0.04, 1.0), ((9, 14), 0.04, 4.0)])
@pytest.mark.parametrize("order", [1, 2])
def test_amr_level2_matches_oracle(cg, oracle, system, shape, T, tol, order):
    s = amr_state(shape, system, 51 + len(shape) + order)
    n, nf, t, status, runs, cp, mp, fp, cf, mf, ff = run_amr2(cg, system, s, T, tol, order)
    wn, counts, wcp, wmp, wfp, wcf, wmf, wff = oracle.amr_level2(system, s, 1.0 / shape[-1], 0.9, T, tol, order,
                                                                 cases.SYS_GAMMA[system])
    assert (n, nf, runs[0], runs[1]) == (wn, counts[0], counts[1], counts[2]) and t >= T
    for got, want in ((cp, wcp), (mp, wmp), (fp, wfp)):
        assert bit_equal(got.reshape(-1), want)
    for got, want in ((cf, wcf), (mf, wmf), (ff, wff)):
        assert np.array_equal(got.reshape(-1), want.astype(bool))


@pytest.mark.parametrize("system", [0, 1])
def test_amr_level2_fp32_stays_near_fp64(cg, system):
    s = amr_state((24, 28), system, 78)
    r64 = run_amr2(cg, system, s, 0.04, 1.0, 2, precision=0)
    r32 = run_amr2(cg, system, s, 0.04, 1.0, 2, precision=1)
    assert all(np.isfinite(x).all() for x in r32[5:8]) and r32[2] >= 0.04
    rho64, rho32 = r64[5][..., 0], r32[5][..., 0]
    assert np.abs(rho32 - rho64).sum() / np.abs(rho64).sum() < 2e-3


def test_reference_named_level2_entry_points(cg, oracle):
    s = amr_state((10, 12), 0, 19)
    out = cg.EulerAMR.solve2DLevel2AMR(s, 1.0 / 12, 0.9, 0.03, 1.0, 2, cg.EulerMaterialParameters(1.4))
    want = oracle.amr_level2(0, s, 1.0 / 12, 0.9, 0.03, 1.0, 2, 1.4)[2:]
    for got, w in zip(out[:3], want[:3]):
        assert bit_equal(got.reshape(-1), w)
    for got, w in zip(out[3:], want[3:]):
        assert np.array_equal(got.reshape(-1), w.astype(bool))
