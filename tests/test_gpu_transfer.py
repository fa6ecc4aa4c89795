"""Host transfers from and to page-locked (pinned) and pageable host buffers: the states and the
primitives read back are bit-identical (the same conversion kernels on the same staged data; the
copy engine moves both kinds of buffer)."""
import numpy as np
import pytest

import cases
from conftest import bit_equal

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cg(cosmos_lib):
    import cosmos_gb300
    return cosmos_gb300


def pinned_like(a):
    torch = pytest.importorskip("torch")
    h = torch.empty(a.shape, dtype=torch.float64, pin_memory=True).numpy()
    h[...] = a
    return h


@pytest.mark.parametrize("system,precision", [(0, 0), (0, 1), (1, 0), (1, 1), (2, 1)])
def test_page_locked_grid_transfers_match_pageable(cg, system, precision):
    shape = (37, 53)
    rng = np.random.default_rng(11 + system)
    s = cases.state(system, rng, shape)
    bh = cg.BlackHoleSpacetime(*cases.GR_BH) if system == 2 else None
    gamma = 1.4 if system == 0 else 5.0 / 3.0
    outs = []
    for page_locked in (False, True):
        g = cg.Grid(system, shape, 1.0 / shape[1], gamma, precision, 0, bh)
        g.set_prim(pinned_like(s) if page_locked else s)
        g.sweep(0, 2, 0.2 / shape[1], 0.0, 1)
        out = pinned_like(np.zeros(shape + (5,))) if page_locked else None
        outs.append(np.array(g.get_prim(out=out)))
        g.close()
    assert bit_equal(outs[0], outs[1])


@pytest.mark.parametrize("precision", [0, 1])
def test_page_locked_batch_transfers_match_pageable(cg, precision):
    shapes = [(40,), (23, 31), (64, 17)]
    states = [cases.riemann(sh, 30 + k) for k, sh in enumerate(shapes)]
    outs = []
    for page_locked in (False, True):
        b = cg.Batch(shapes, [1.0 / sh[-1] for sh in shapes], 1.4, precision, cg.BC_TRANSMISSIVE)
        for k, s in enumerate(states):
            b.set_prim(k, pinned_like(s) if page_locked else s)
        b.run_begin(0.9, 1e30, 0.0, cg.MINBEE)
        b.run_steps(3)
        b.run_end()
        got = []
        for k, sh in enumerate(shapes):
            out = pinned_like(np.zeros(sh + (5,))) if page_locked else None
            got.append(np.array(b.get_prim(k, out=out)))
        outs.append(got)
        b.close()
    assert all(bit_equal(a, c) for a, c in zip(*outs))
