"""FWI iterations (gradient, taper, step-length search with trial forwards,
clamped update) on the GPU against the reference's golden run and the
oracle.  Accepted steps and misfits must follow the same branch sequence
(identical trial counts)."""
import numpy as np
import pytest

import helpers
from fwi_cuda_gb300 import engine

pytestmark = pytest.mark.gpu


def test_fwi_fp64_matches_reference_golden(gpu):
    # ten iterations of the reference's own CPU FWI (tests/golden): misfit and
    # accepted step of every iteration, final model and gradient
    z = np.load(helpers.GOLDEN)
    name = "fwi_crosswell"
    sv = helpers.load_case(z, name)
    with engine.Plan(sv, precision=64) as p:
        p.set_model(*z[f"{name}/init"])
        p.set_observed(z[f"{name}/obs_uz"], z[f"{name}/obs_ux"])
        step = 0.01
        for it in range(10):
            r = p.fwi_iteration(step)
            step = r["step"]
            assert r["L2"] == pytest.approx(z[f"{name}/L2"][it], rel=1e-9)
            assert step == pytest.approx(z[f"{name}/step"][it], rel=1e-7)
        lam, mu, rho = p.get_model()
        g = p.get_gradient()
    assert helpers.rel_l2(lam, z[f"{name}/lam"]) < 1e-9
    assert helpers.rel_l2(mu, z[f"{name}/mu"]) < 1e-9
    assert helpers.rel_l2(rho, z[f"{name}/rho"]) < 1e-9
    assert helpers.rel_l2(g[0], z[f"{name}/grad_lam"]) < 1e-8


def test_fwi_fp32_follows_reference_sequence(gpu, orc):
    # FP32 engine over the same ten iterations: the same number of trial
    # forwards in every step-length search (the oracle, pinned bit for bit to
    # the reference, supplies the counts), accepted steps and misfits within
    # FP32 error of the reference's
    z = np.load(helpers.GOLDEN)
    name = "fwi_crosswell"
    sv = helpers.load_case(z, name)
    ro = orc.simulate_fwi(sv, *z[f"{name}/init"], z[f"{name}/obs_uz"], z[f"{name}/obs_ux"],
                          niter=10)
    assert ro["rc"] == 0 and np.array_equal(ro["step"], z[f"{name}/step"])
    with engine.Plan(sv, precision=32) as p:
        p.set_model(*z[f"{name}/init"])
        p.set_observed(z[f"{name}/obs_uz"], z[f"{name}/obs_ux"])
        step = 0.01
        for it in range(10):
            r = p.fwi_iteration(step)
            step = r["step"]
            assert r["ntrials"] == ro["trials"][it], it
            assert r["L2"] == pytest.approx(z[f"{name}/L2"][it], rel=1e-4), it
            assert step == pytest.approx(z[f"{name}/step"][it], rel=2e-3), it


@pytest.mark.parametrize("precision", [64, 32])
def test_fwi_iterations_match_oracle(gpu, orc, precision):
    sv, true, init = helpers.case(fdorder=4, stencil="holberg", nshot=2, nt=300, imaging_sign=1)
    uz, ux = orc.simulate_fwd(sv, *true)
    niter = 4
    r = orc.simulate_fwi(sv, *init, uz, ux, niter=niter)
    assert r["rc"] == 0
    with engine.Plan(sv, precision=precision) as p:
        p.set_model(*init)
        p.set_observed(uz, ux)
        step = 0.01
        for it in range(niter):
            o = p.fwi_iteration(step)
            step = o["step"]
            assert o["ntrials"] == r["trials"][it]
            rtol = 1e-9 if precision == 64 else 1e-4
            assert o["L2"] == pytest.approx(r["L2"][it], rel=rtol)
            assert step == pytest.approx(r["step"][it], rel=1e-6 if precision == 64 else 2e-3)
