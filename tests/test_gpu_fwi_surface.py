"""Ten FWI iterations of the surface configuration at full size: 301 x 601,
8 shots, nt = 4000, 4th-order Holberg, free surface on the first interior
row (fwi_cuda_gb300.survey.surface_fwi_case), each iteration a gradient of
all shots, the taper, the parabolic step-length search with its trial
forwards and the clamped model update (src/cpu/n_simulate_PSV.cpp:249-582,
src/cpu/n_step_length_PSV.cpp:13-209).

The FP64 oracle's sequence is the fixture tests/golden/fwi_surface_301x601.npz
(made once by tests/golden/make_fwi_sequence.py, about three hours on 8 CPU
cores): misfit, accepted step, trial count and every trial's (step, misfit)
per iteration, the global gradients of the first iteration in full, and
gradient and model values at 2048 seeded cells after every iteration.  The
observed data here come from the FP64 engine; they are checked against the
oracle's norms and samples first (1e-9).

Bars.  FP64 engine: identical trial counts, misfits within 1e-9, accepted
steps within 1e-7, gradients within 1e-6 (the fixture stores the first
gradient in float32).  FP32 engine: identical trial counts in every
iteration (the same branches of the search), misfits within FP32_L2 and
accepted steps within FP32_STEP of the oracle's.  An accepted step is the
vertex of a parabola through three trial misfits, so it carries the misfit
error divided by the parabola's relative curvature: with misfits within
~2e-5 the steps differ by up to a few 1e-3 (measured values are printed,
run with -s)."""
import os

import numpy as np
import pytest

import helpers
from fwi_cuda_gb300 import engine
from fwi_cuda_gb300 import survey as S

pytestmark = pytest.mark.gpu

FIXTURE = os.path.join(os.path.dirname(__file__), "golden", "fwi_surface_301x601.npz")
FP32_L2 = 1e-4
FP32_STEP = 2e-2


@pytest.fixture(scope="module")
def case():
    if not os.path.exists(FIXTURE):
        pytest.skip("the oracle's sequence has not been generated (tests/golden/make_fwi_sequence.py)")
    z = np.load(FIXTURE)
    sv, true, init = S.surface_fwi_case()
    with engine.Plan(sv, precision=64) as p:
        p.set_model(*true)
        uz, ux = p.forward()
    r, t = z["trace_rec"], z["trace_t"]
    np.testing.assert_allclose(np.linalg.norm(uz.reshape(sv.nshot, -1), axis=1), z["obs_norm_uz"],
                               rtol=1e-9)
    np.testing.assert_allclose(np.linalg.norm(ux.reshape(sv.nshot, -1), axis=1), z["obs_norm_ux"],
                               rtol=1e-9)
    assert helpers.rel_l2(uz[:, r, t], z["obs_sample_uz"]) < 1e-9
    assert helpers.rel_l2(ux[:, r, t], z["obs_sample_ux"]) < 1e-9
    return z, sv, init, (uz, ux)


def _run(sv, init, obs, precision, niter):
    rows = []
    with engine.Plan(sv, precision=precision) as p:
        p.set_model(*init)
        p.set_observed(*obs)
        step = 0.01
        for it in range(niter):
            r = p.fwi_iteration(step)
            step = r["step"]
            g = p.get_gradient()
            m = p.get_model()
            rows.append(dict(L2=r["L2"], step=step, ntrials=r["ntrials"], grad=g, model=m))
    return rows


def _sample(arrs, z):
    return np.stack([a[z["cells_z"], z["cells_x"]] for a in arrs])


def test_fp64_engine_follows_the_oracle_sequence(gpu, case):
    z, sv, init, obs = case
    niter = 4  # the FP64 kernels are slow on this part; four iterations already cover the search's branches
    rows = _run(sv, init, obs, 64, niter)
    for it, r in enumerate(rows):
        assert r["ntrials"] == z["trials"][it], it
        assert r["L2"] == pytest.approx(z["L2"][it], rel=1e-9), it
        assert r["step"] == pytest.approx(z["step"][it], rel=1e-7), it
        assert helpers.rel_l2(_sample(r["grad"], z), z["grad_sample"][it]) < 1e-7, it
        assert helpers.rel_l2(_sample(r["model"], z), z["model_sample"][it]) < 1e-9, it
    for k in range(3):
        assert helpers.rel_l2(rows[0]["grad"][k], z["grad_iter0"][k]) < 1e-6


def test_fp32_engine_follows_the_oracle_sequence(gpu, case):
    z, sv, init, obs = case
    niter = int(z["niter"])
    rows = _run(sv, init, obs, 32, niter)
    e_L2 = [abs(r["L2"] - z["L2"][i]) / z["L2"][i] for i, r in enumerate(rows)]
    e_step = [abs(r["step"] - z["step"][i]) / z["step"][i] for i, r in enumerate(rows)]
    e_grad = [helpers.rel_l2(_sample(r["grad"], z), z["grad_sample"][i]) for i, r in enumerate(rows)]
    print("\nFP32 vs the FP64 oracle over", niter, "iterations")
    print("  trials  engine", [r["ntrials"] for r in rows], "oracle", list(z["trials"]))
    print("  misfit  rel. error", " ".join(f"{e:.1e}" for e in e_L2))
    print("  step    rel. error", " ".join(f"{e:.1e}" for e in e_step))
    print("  gradient sample rel. L2", " ".join(f"{e:.1e}" for e in e_grad))
    print("  first gradient rel. L2 (lam, mu, rho)",
          " ".join(f"{helpers.rel_l2(rows[0]['grad'][k], z['grad_iter0'][k]):.1e}" for k in range(3)))
    for it, r in enumerate(rows):
        assert r["ntrials"] == z["trials"][it], it
    assert max(e_L2) <= FP32_L2
    assert max(e_step) <= FP32_STEP
