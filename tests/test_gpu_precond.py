"""Optional preconditioners on the device against the oracle: smoothing
(bit for bit: same FP64 sum order), Fletcher-Reeves (reduction order differs:
1e-13), and both inside the plan's gradient / FWI iteration."""
import numpy as np
import pytest

import helpers
from fwi_cuda_gb300 import engine

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("shape,hfs", [((37, 53), 2), ((64, 48), 3), ((41, 90), 5)])
def test_apply_gauss_filter_matches_the_oracle(gpu, orc, shape, hfs):
    m = np.random.default_rng(hfs).standard_normal(shape) * 1e9
    assert np.array_equal(engine.apply_gauss_filter(m, hfs), orc.apply_gauss_filter(m, hfs))


def test_pcg_matches_the_oracle_over_three_calls(gpu, orc):
    rng = np.random.default_rng(3)
    d1, o1 = np.zeros((50, 70)), np.zeros((50, 70))
    d2, o2 = d1.copy(), o1.copy()
    for _ in range(3):
        g = rng.standard_normal((50, 70))
        a, b = g.copy(), g.copy()
        engine.PCG_PSV(d1, o1, a)
        orc.PCG_PSV(d2, o2, b)
        assert helpers.rel_l2(a, b) < 1e-13 and helpers.rel_l2(d1, d2) < 1e-13
        assert np.array_equal(o1, o2)


@pytest.mark.parametrize("precision,tol", [(64, 1e-9), (32, 1e-4)])
def test_plan_smooths_shot_gradients(gpu, orc, precision, tol):
    sv, true, init = helpers.case(fdorder=4, stencil="holberg", nshot=2, nt=300)
    uz, ux = orc.simulate_fwd(sv, *true)
    L2r, gr, _ = helpers.oracle_gradient(orc, sv, init, uz, ux, smooth_hfs=3)
    _, g0, _ = helpers.oracle_gradient(orc, sv, init, uz, ux)
    assert helpers.rel_l2(gr[0], g0[0]) > 1e-3  # smoothing changes the gradient
    with engine.Plan(sv, precision=precision, smooth_hfs=3) as p:
        p.set_model(*init)
        p.set_observed(uz, ux)
        L2, g = p.gradient()
    assert L2 == pytest.approx(L2r, rel=tol)
    for a, b in zip(g, gr):
        assert helpers.rel_l2(a, b) < tol


def test_plan_pcg_direction_follows_the_oracle(gpu, orc):
    sv, true, init = helpers.case(fdorder=4, stencil="holberg", nshot=2, nt=300)
    uz, ux = orc.simulate_fwd(sv, *true)
    state = [(np.zeros((sv.nz, sv.nx)), np.zeros((sv.nz, sv.nx))) for _ in range(3)]
    models = [init, [1.01 * a for a in init]]
    with engine.Plan(sv, precision=64) as p:
        p.set_observed(uz, ux)
        for model in models:
            p.set_model(*model)
            p.reset_gradient()  # gradients accumulate across calls, as in the reference
            _, g = p.gradient()
            p.pcg_gradient()
            d = p.get_gradient()
            for k in range(3):
                ref = g[k].copy()
                orc.PCG_PSV(state[k][0], state[k][1], ref)
                assert helpers.rel_l2(d[k], ref) < 1e-12


def test_fwi_iteration_with_preconditioners(gpu, orc):
    sv, true, init = helpers.case(fdorder=4, stencil="holberg", nshot=2, nt=300)
    uz, ux = orc.simulate_fwd(sv, *true)
    with engine.Plan(sv, precision=32, smooth_hfs=2, pcg=True) as p:
        p.set_model(*init)
        p.set_observed(uz, ux)
        out = [p.fwi_iteration(0.01) for _ in range(2)]
    for r in out:
        assert all(np.isfinite(x) for x in (r["step"], r["L2"])) and r["step"] > 0
