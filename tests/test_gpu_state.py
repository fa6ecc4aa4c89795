"""The state-level functions (cosmos_state_eval): the reference's state-vector, equation-of-state,
slope-limiter and black-hole eigenvalue functions evaluated on the device, bit for bit against the
oracle's restatement of the same functions (and, where the oracle has no entry, against the
reference's formula evaluated in the same operation order)."""
import math

import numpy as np
import pytest

import cases
from conftest import bit_equal

pytestmark = pytest.mark.gpu

BH = (1.0, 0.3, 0.5, 0.5, 0.0)


@pytest.fixture(scope="module")
def cg(cosmos_lib):
    import cosmos_gb300
    return cosmos_gb300


def states(system, n, seed):
    rng = np.random.default_rng(seed)
    s = np.zeros((n, 5))
    s[:, 0] = rng.uniform(0.2, 2.0, n)
    s[:, 1:4] = rng.uniform(-0.4, 0.4, (n, 3)) * (1.0 if system else 3.0)
    s[:, 4] = rng.uniform(0.1, 2.0, n)
    return s


def coords(n, seed):
    """Points at least 3 M from the hole (outside the horizon, where the metric is regular)."""
    rng = np.random.default_rng(seed)
    out = []
    while len(out) < n:
        x, y = rng.uniform(-8, 8, 2)
        if math.hypot(x - BH[2], y - BH[3]) > 3.0:
            out.append((x, y, 0.0))
    return np.array(out)


@pytest.mark.parametrize("system", [0, 1, 2])
def test_conserved_primitive_and_fluxes(cg, oracle, system):
    from cosmos_gb300 import _lib
    g = cases.SYS_GAMMA[system]
    n = 64
    p = states(system, n, 3 + system)
    q = coords(n, 9) if system == 2 else None
    hole = cg.BlackHoleSpacetime(*BH) if system == 2 else None
    kw = dict(system=system, gamma=g, xyz=q, black_hole=hole, dx=0.05)
    u = cg.state_eval(_lib.STATE_CONS, p, **kw)
    back = cg.state_eval(_lib.STATE_PRIM, u, **kw)
    fx = cg.state_eval(_lib.STATE_FLUX_X, u, **kw)
    fy = cg.state_eval(_lib.STATE_FLUX_Y, u, **kw)
    bh = BH if system == 2 else None
    for k in range(n):
        x, y = (q[k, 0], q[k, 1]) if system == 2 else (0.0, 0.0)
        assert bit_equal(u[k], oracle.cons(system, p[k], g, x, y, bh, 0.05)), k
        assert bit_equal(back[k], oracle.prim(system, u[k], g, x, y, bh, 0.05)), k
        assert bit_equal(fx[k], oracle.flux(system, u[k], 0, g, x, y, bh, 0.05)), k
        assert bit_equal(fy[k], oracle.flux(system, u[k], 1, g, x, y, bh, 0.05)), k


def test_equation_of_state_functions(cg):
    from cosmos_gb300 import _lib
    p = states(0, 40, 5)
    g = 1.4
    c = cg.state_eval(_lib.STATE_SOUND, p, system=0, gamma=g)[:, 0]
    e = cg.state_eval(_lib.STATE_INTERNAL_ENERGY, p, system=0, gamma=g)[:, 0]
    E = cg.state_eval(_lib.STATE_TOTAL_ENERGY, p, system=0, gamma=g)[:, 0]
    pe = p.copy()
    pe[:, 4] = e
    pr = cg.state_eval(_lib.STATE_PRESSURE, pe, system=0, gamma=g)[:, 0]
    sr = states(1, 40, 6)
    gs = 5.0 / 3.0
    h = cg.state_eval(_lib.STATE_ENTHALPY, sr, system=1, gamma=gs)[:, 0]
    cs = cg.state_eval(_lib.STATE_SOUND, sr, system=1, gamma=gs)[:, 0]
    for k in range(40):
        rho, vx, vy, vz, P = p[k]
        assert c[k] == math.sqrt((g * P) / rho)                      # Euler/EulerEquationOfState.cpp:17-22
        assert e[k] == P / ((g - 1.0) * rho)                          # :3-8
        v2 = ((vx * vx) + (vy * vy)) + (vz * vz)
        assert E[k] == rho * ((0.5 * v2) + e[k])                      # Euler/EulerStateVector.cpp:129-134
        assert pr[k] == (e[k] * (g - 1.0)) * rho                      # Euler/EulerEquationOfState.cpp:10-15
        r2, P2 = sr[k, 0], sr[k, 4]
        assert h[k] == 1.0 + ((P2 / r2) * (gs / (gs - 1.0)))          # RelativisticEulerEquationOfState.cpp:3-8
        assert cs[k] == math.sqrt(((gs * P2) / r2) / (1.0 + ((P2 / r2) * (gs / (gs - 1.0)))))  # :10-18


def test_black_hole_source_sound_speed_and_eigenvalues(cg, oracle):
    from cosmos_gb300 import _lib
    n, g = 32, 5.0 / 3.0
    p = states(2, n, 8)
    q = coords(n, 10)
    hole = cg.BlackHoleSpacetime(*BH)
    kw = dict(system=2, gamma=g, xyz=q, black_hole=hole, dx=0.05)
    u = cg.state_eval(_lib.STATE_CONS, p, **kw)
    src = cg.state_eval(_lib.STATE_SOURCE, u, **kw)
    snd = cg.state_eval(_lib.STATE_SOUND, p, **kw)[:, 0]
    eig = cg.state_eval(_lib.STATE_EIGENVALUES, p, **kw)
    for k in range(n):
        x, y = q[k, 0], q[k, 1]
        assert bit_equal(src[k], oracle.gr_source(u[k], x, y, 0.05, g, BH)), k
        assert snd[k] == oracle.gr_sound_speed(p[k], x, y, g, BH), k
        assert snd[k] == max(0.0, *eig[k]), k                         # the largest signed eigenvalue
        m = oracle.gr_metric(x, y, 0.0, 0.05, BH)
        al, be = m[1], m[2:5]
        assert [al * p[k, 1 + i] - be[i] for i in range(3)] == list(eig[k, :3]), k  # material


def test_slope_limiters(cg, oracle):
    from cosmos_gb300 import _lib
    rng = np.random.default_rng(12)
    r = np.concatenate([rng.uniform(-2, 4, 200), [0.0, 0.5, 1.0, 2.0, -0.0]])
    for bias in (0.0, 0.4, -0.7):
        gr = cg.state_eval(_lib.STATE_GRADIENT_RATIO, r[:, None], bias=bias)[:, 0]
        assert list(gr) == [2.0 / ((1.0 - bias) + ((1.0 + bias) * v)) for v in r]  # SlopeLimiters.cpp:3-6
        for lim in (0, 1, 2, 7):
            got = cg.state_eval(_lib.STATE_LIMITER, r[:, None], bias=bias, limiter=lim)[:, 0]
            assert list(got) == [oracle.limiter(v, bias, lim) for v in r], (bias, lim)
    u = rng.uniform(-1, 1, (50, 15))
    u[:10, 5:10] = u[:10, 0:5] + rng.uniform(-1e-6, 1e-6, (10, 5))  # differences inside the 1e-5 clamp
    for lim in (0, 1, 2):
        got = cg.state_eval(_lib.STATE_SLOPE, u, bias=0.3, limiter=lim)
        for k in range(50):
            assert bit_equal(got[k], oracle.slope(u[k, :5], u[k, 5:10], u[k, 10:], 0.3, lim)), (lim, k)


def test_state_eval_rejects_misuse(cg):
    from cosmos_gb300 import _lib
    from cosmos_gb300._lib import CosmosError
    with pytest.raises(CosmosError):
        cg.state_eval(_lib.STATE_INTERNAL_ENERGY, states(1, 2, 1), system=1, gamma=5.0 / 3.0)
    with pytest.raises(CosmosError):
        cg.state_eval(_lib.STATE_SOURCE, states(0, 2, 1), system=0)
    with pytest.raises(CosmosError):
        cg.state_eval(_lib.STATE_CONS, states(2, 2, 1), system=2, gamma=5.0 / 3.0)  # no coordinates


def test_reference_named_python_classes(cg, oracle):
    mp = cg.EulerMaterialParameters(1.4)
    assert cg.EulerEquationOfState.computeSoundSpeed(0.8, 0.6, mp) == math.sqrt((1.4 * 0.6) / 0.8)
    e = cg.EulerEquationOfState.computeSpecificInternalEnergy(np.array([0.8, 1.2]), np.array([0.6, 0.3]), mp)
    assert list(e) == [0.6 / ((1.4 - 1.0) * 0.8), 0.3 / ((1.4 - 1.0) * 1.2)]
    assert cg.EulerEquationOfState.computePressure(0.8, e[0], mp) == (e[0] * (1.4 - 1.0)) * 0.8
    r = np.linspace(-1, 3, 17)
    assert list(cg.SlopeLimiters.computeVanLeerSlopeLimiter(r, 0.2)) == [oracle.limiter(v, 0.2, 1) for v in r]
    u = np.random.default_rng(3).uniform(-1, 1, (3, 4, 5))
    s = cg.SlopeLimiters.computeSlopeVector(u[0], u[1], u[2], 0.0, 2)
    for k in range(4):
        assert bit_equal(s[k], oracle.slope(u[0, k], u[1, k], u[2, k], 0.0, 2))
    g = 5.0 / 3.0
    h = cg.RelativisticEulerEquationOfState.computeSpecificEnthalpy(1.0, 2.0, cg.EulerMaterialParameters(g))
    assert h == 1.0 + ((2.0 / 1.0) * (g / (g - 1.0)))


def test_compat_state_classes_from_cpp(cosmos_lib, oracle, tmp_path):
    import os
    import subprocess
    from conftest import ROOT
    exe, out = str(tmp_path / "state_driver"), str(tmp_path / "state.bin")
    lib = os.path.join(ROOT, "cosmos_gb300")
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "state_driver.cpp"), "-o", exe, "-L", lib, "-lcosmos_gb300",
                    f"-Wl,-rpath,{lib}"], check=True)
    subprocess.run([exe, out], check=True, timeout=120)
    st = np.fromfile(out, dtype=np.float64)
    assert st.shape == (18,)
    prim = np.array([0.8, 0.3, -0.2, 0.1, 0.6])
    u = oracle.cons(0, prim, 1.4)
    assert bit_equal(st[:5], u) and bit_equal(st[5:10], oracle.flux(0, u, 0, 1.4))
    assert bit_equal(st[10:15], oracle.prim(0, u, 1.4))
    assert st[15] == oracle.limiter(0.7, 0.0, 1) and st[16] == math.sqrt((1.4 * 0.6) / 0.8)
    g = 5.0 / 3.0
    assert st[17] == math.sqrt(((g * 1.0) / 1.0) / (1.0 + ((1.0 / 1.0) * (g / (g - 1.0)))))
