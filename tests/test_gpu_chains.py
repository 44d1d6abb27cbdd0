"""Chained time loops: the batch's shots split into groups whose launches run
on their own streams.  Each shot's arithmetic is unchanged, so gradients,
traces and misfits equal the single-stream schedule bit for bit."""
import numpy as np
import pytest

import helpers
from fwi_cuda_gb300 import _lib, engine

pytestmark = pytest.mark.gpu

SHAPE = dict(precision=32, kernels="direct", rows_per_thread=1, block=(32, 4))


def _run(sv, init, uz, ux, **opt):
    with engine.Plan(sv, **dict(SHAPE, **opt)) as p:
        p.set_model(*init)
        p.set_observed(uz, ux)
        L2, g = p.gradient()
        fwd = p.forward()
        return p.chains, L2, g, fwd


@pytest.mark.parametrize("nshot,max_batch,chains", [(8, 0, 2), (8, 0, 4), (5, 0, 2), (5, 0, 4),
                                                     (7, 3, 2), (7, 3, 4)])
def test_chains_equal_one_stream(gpu, orc, nshot, max_batch, chains):
    # 5 shots in 4 groups: ceil(5 / 4) = 2 slots a group, the last group empty;
    # 7 shots in batches of 3: the last batch holds one shot
    sv, true, init = helpers.case(fdorder=4, stencil="holberg", nshot=nshot, nt=200, snap_dt=2)
    uz, ux = orc.simulate_fwd(sv, *true)
    c1, L1, g1, f1 = _run(sv, init, uz, ux, max_batch=max_batch, chains=1)
    c2, L2, g2, f2 = _run(sv, init, uz, ux, max_batch=max_batch, chains=chains)
    assert c1 == 1 and c2 == (chains if chains <= (max_batch or nshot) else 2)
    assert L1 == L2
    for a, b in zip(g1 + list(f1), g2 + list(f2)):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("storage,kw", [("full", {}), ("binomial", dict(checkpoint_slots=2))])
def test_fp64_chains_equal_one_stream(gpu, orc, storage, kw):
    # FP64 plans run the direct family, so they chain too; 6 shots in 4
    # groups of 2, 2, 2 and none
    sv, true, init = helpers.case(fdorder=4, stencil="holberg", nshot=6, nt=150, snap_dt=3)
    uz, ux = orc.simulate_fwd(sv, *true)
    c1, L1, g1, f1 = _run(sv, init, uz, ux, precision=64, storage=storage, chains=1, **kw)
    c2, L2, g2, f2 = _run(sv, init, uz, ux, precision=64, storage=storage, chains=4, **kw)
    assert c1 == 1 and c2 == 4
    assert L1 == L2
    for a, b in zip(g1 + list(f1), g2 + list(f2)):
        assert np.array_equal(a, b)
    L_ref, g_ref, _ = helpers.oracle_gradient(orc, sv, init, uz, ux)
    assert L2 == pytest.approx(L_ref, rel=1e-9)
    for a, b in zip(g2, g_ref):
        assert helpers.rel_l2(a, b) < 1e-9


@pytest.mark.parametrize("storage,kw", [("checkpoint", dict(checkpoint_interval=37)),
                                        ("binomial", dict(checkpoint_slots=3))])
def test_checkpointed_chains_equal_one_stream(gpu, orc, storage, kw):
    # the forward saves states between chained segments; the adjoint's
    # recomputations and reversals run chained between the state copies
    sv, true, init = helpers.case(fdorder=4, stencil="holberg", nshot=4, nt=200, snap_dt=2)
    uz, ux = orc.simulate_fwd(sv, *true)
    c1, L1, g1, _ = _run(sv, init, uz, ux, storage=storage, chains=1, **kw)
    c2, L2, g2, _ = _run(sv, init, uz, ux, storage=storage, chains=4, **kw)
    assert c1 == 1 and c2 == 4
    assert L1 == L2 and all(np.array_equal(a, b) for a, b in zip(g1, g2))
    with engine.Plan(sv, **dict(SHAPE, storage="full")) as p:
        p.set_model(*init)
        p.set_observed(uz, ux)
        L0, g0 = p.gradient()
    assert L0 == L1 and all(np.array_equal(a, b) for a, b in zip(g0, g1))


def test_autotuner_picks_a_chain_count(gpu, orc):
    sv, true, init = helpers.case(fdorder=4, stencil="holberg", nshot=4, nt=100)
    uz, ux = orc.simulate_fwd(sv, *true)
    with engine.Plan(sv, precision=32, kernels="direct") as p:
        p.set_model(*init)
        p.set_observed(uz, ux)
        p.autotune(8)
        assert p.chains in (1, 2, 4)


def test_bad_chain_count_is_rejected(gpu):
    sv, _, _ = helpers.case(nshot=2, nt=20)
    with pytest.raises(_lib.PSVError, match="chains"):
        engine.Plan(sv, precision=32, chains=3)


def test_fwi_iterations_do_not_depend_on_chains(gpu, orc):
    # gradient, taper, the step-length search's trial forwards and the update
    sv, true, init = helpers.case(fdorder=4, stencil="holberg", nshot=4, nt=250)
    uz, ux = orc.simulate_fwd(sv, *true)
    out = []
    for chains in (1, 4):
        with engine.Plan(sv, **dict(SHAPE, chains=chains)) as p:
            p.set_model(*init)
            p.set_observed(uz, ux)
            steps = [p.fwi_iteration(0.01) for _ in range(2)]
            out.append((steps, p.get_model()))
    (s1, m1), (s2, m2) = out
    for a, b in zip(s1, s2):
        assert a["step"] == b["step"] and a["L2"] == b["L2"] and a["ntrials"] == b["ntrials"]
    for a, b in zip(m1, m2):
        assert np.array_equal(a, b)
