"""Tile-shape autotuner: every candidate shape computes the same gradient,
and the tuned plan matches the oracle like any other."""
import numpy as np
import pytest

import helpers
from fwi_cuda_gb300 import engine

pytestmark = pytest.mark.gpu


def _grad(sv, init, uz, ux, **opt):
    with engine.Plan(sv, precision=32, **opt) as p:
        p.set_model(*init)
        p.set_observed(uz, ux)
        L2, g = p.gradient()
        return L2, g, p


def test_autotune_shape_and_parity(gpu, orc):
    sv, true, init = helpers.case(fdorder=4, stencil="holberg", nshot=2, nt=300, nz=81, nx=121)
    uz, ux = orc.simulate_fwd(sv, *true)
    L2_ref, g_ref, _ = helpers.oracle_gradient(orc, sv, init, uz, ux)
    with engine.Plan(sv, precision=32) as p:
        p.set_model(*init)
        p.set_observed(uz, ux)
        rpt, by = p.autotune(8)
        assert rpt in (1, 2, 4, -2, -4) and by in (2, 4, 8)
        L2, g = p.gradient()
    assert L2 == pytest.approx(L2_ref, rel=1e-4)
    for a, b in zip(g, g_ref):
        assert helpers.rel_l2(a, b) < 1e-4


@pytest.mark.parametrize("rpt,by", [(2, 4), (4, 2), (-2, 4), (-4, 8)])
def test_every_shape_gives_the_same_gradient(gpu, orc, rpt, by):
    # register blocking and warp shuffles change which thread loads a value,
    # not the arithmetic on it: results agree to rounding of the FP32 sums
    sv, true, init = helpers.case(fdorder=8, stencil="holberg", nshot=2, nt=200, nz=75, nx=97)
    uz, ux = orc.simulate_fwd(sv, *true)
    L2a, ga, _ = _grad(sv, init, uz, ux, rows_per_thread=1, block=(32, 8))
    L2b, gb, _ = _grad(sv, init, uz, ux, rows_per_thread=rpt, block=(32, by))
    assert L2b == pytest.approx(L2a, rel=1e-6)
    for a, b in zip(ga, gb):
        assert helpers.rel_l2(b, a) < 1e-6
