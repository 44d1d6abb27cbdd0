"""FWI gradient on the GPU (forward with snapshots, residual, time-reversed
adjoint with the imaging condition, energy-weight preconditioning) against
the FP64 oracle.  Tolerances: FP64 engine 1e-9 relative L2; FP32 engine 1e-4
relative L2 on the gradients (the stated target)."""
import numpy as np
import pytest

import helpers
from fwi_cuda_gb300 import engine

pytestmark = pytest.mark.gpu
RTOL64 = 1e-9
RTOL32_GRAD = 1e-4


def _setup(orc, **kw):
    sv, true, init = helpers.case(**kw)
    uz, ux = orc.simulate_fwd(sv, *true)
    return sv, true, init, uz, ux


@pytest.mark.parametrize("kw", [dict(fdorder=4, stencil="holberg", nshot=2, nt=300),
                                dict(fdorder=2, stencil="reference", nshot=1, nt=300),
                                dict(fdorder=8, stencil="holberg", nshot=1, nt=250,
                                     imaging_sign=1)])
@pytest.mark.parametrize("precision", [64, 32])
def test_shot_and_global_gradient(gpu, orc, kw, precision):
    sv, true, init, uz, ux = _setup(orc, **kw)
    L2_ref, g_ref, shots = helpers.oracle_gradient(orc, sv, init, uz, ux)  # oracle honours imaging_sign
    tol = RTOL64 if precision == 64 else RTOL32_GRAD
    with engine.Plan(sv, precision=precision) as p:
        p.set_model(*init)
        p.set_observed(uz, ux)
        L2, g = p.gradient()
        assert L2 == pytest.approx(L2_ref, rel=1e-9 if precision == 64 else 1e-4)
        for a, b in zip(g, g_ref):
            assert helpers.rel_l2(a, b) < tol
        for s in range(sv.nshot):
            o = p.shot_gradient(s)
            for k in ("grad_lam", "grad_mu", "grad_rho"):
                assert helpers.rel_l2(o[k], shots[s][k]) < tol, k
            for k in ("We", "We_adj"):
                assert helpers.rel_l2(o[k], shots[s][k]) < (1e-9 if precision == 64 else 1e-4), k


def test_gradient_accumulates_across_calls_like_reference(gpu, orc):
    # the reference never resets the global gradient (n_simulate_PSV.cpp:260)
    sv, true, init, uz, ux = _setup(orc, fdorder=4, stencil="holberg", nt=200)
    with engine.Plan(sv, precision=64) as p:
        p.set_model(*init)
        p.set_observed(uz, ux)
        _, g1 = p.gradient()
        _, g2 = p.gradient()
        for a, b in zip(g1, g2):
            assert helpers.rel_l2(b, 2 * a) < 1e-12
        p.reset_gradient()
        _, g3 = p.gradient()
        for a, b in zip(g1, g3):
            assert np.array_equal(a, b)


def test_subsampled_snapshots_and_interpolation(gpu, orc):
    # snap_dt, snap_dz, snap_dx > 1, window not divisible by the steps
    sv, true, init = helpers.case(fdorder=4, stencil="holberg", nt=240)
    sv.snap_dt, sv.snap_dz, sv.snap_dx = 3, 2, 3
    sv.snap_z1, sv.snap_z2, sv.snap_x1, sv.snap_x2 = 5, sv.nz - 9, 7, sv.nx - 10
    uz, ux = orc.simulate_fwd(sv, *true)
    L2_ref, g_ref, _ = helpers.oracle_gradient(orc, sv, init, uz, ux)
    with engine.Plan(sv, precision=64) as p:
        p.set_model(*init)
        p.set_observed(uz, ux)
        L2, g = p.gradient()
    for a, b in zip(g, g_ref):
        assert helpers.rel_l2(a, b) < RTOL64


def test_batched_gradient_equals_one_shot_at_a_time(gpu, orc):
    sv, true, init, uz, ux = _setup(orc, fdorder=4, stencil="holberg", nshot=3, nt=200)
    res = []
    for mb in (0, 1, 2):
        # one kernel shape for all batch sizes (the autotuner may pick per batch
        # size, and shapes agree only to FP32 rounding)
        with engine.Plan(sv, precision=32, max_batch=mb, kernels="direct",
                         rows_per_thread=1, block=(32, 4)) as p:
            p.set_model(*init)
            p.set_observed(uz, ux)
            res.append(p.gradient())
    for L2, g in res[1:]:
        assert L2 == res[0][0]
        for a, b in zip(g, res[0][1]):
            assert np.array_equal(a, b)


@pytest.mark.parametrize("precision,interval", [(32, 0), (32, 7), (64, 50)])
def test_checkpointed_gradient_bitwise_equals_full_storage(gpu, orc, precision, interval):
    # recomputation from checkpoints is deterministic: stated bound = 0
    sv, true, init, uz, ux = _setup(orc, fdorder=4, stencil="holberg", nshot=2, nt=301,
                                    snap_dt=2)
    res = {}
    for storage in ("full", "checkpoint"):
        with engine.Plan(sv, precision=precision, storage=storage,
                         checkpoint_interval=interval) as p:
            p.set_model(*init)
            p.set_observed(uz, ux)
            res[storage] = (p.gradient(), [p.shot_gradient(s) for s in range(sv.nshot)])
    (L2a, ga), sa = res["full"]
    (L2b, gb), sb = res["checkpoint"]
    assert L2a == L2b
    for a, b in zip(ga, gb):
        assert np.array_equal(a, b)
    for x, y in zip(sa, sb):
        for k in ("grad_lam", "grad_mu", "grad_rho", "We", "We_adj"):
            assert np.array_equal(x[k], y[k]), k


@pytest.mark.parametrize("precision,interval,slots", [(32, 0, 1), (32, 0, 3), (32, 7, 2),
                                                      (64, 0, 4), (32, 11, 0)])
def test_binomial_checkpoints_bitwise_equal_full_storage(gpu, orc, precision, interval, slots):
    # fewer state slots than segments: segments are reached again by advancing
    # from earlier states (Griewank's schedule); still deterministic, bound 0
    sv, true, init, uz, ux = _setup(orc, fdorder=4, stencil="holberg", nshot=2, nt=301,
                                    snap_dt=2)
    res = {}
    for storage in ("full", "binomial"):
        with engine.Plan(sv, precision=precision, storage=storage, checkpoint_interval=interval,
                         checkpoint_slots=slots) as p:
            kind, K, S, adv = p.storage
            assert kind == storage
            if storage == "binomial":
                nseg = -(-sv.nt // K)
                assert K == (interval or sv.snap_dt) and S < nseg and adv > 0
                assert S == slots or slots == 0
            p.set_model(*init)
            p.set_observed(uz, ux)
            res[storage] = (p.gradient(), [p.shot_gradient(s) for s in range(sv.nshot)])
    (L2a, ga), sa = res["full"]
    (L2b, gb), sb = res["binomial"]
    assert L2a == L2b
    for a, b in zip(ga, gb):
        assert np.array_equal(a, b)
    for x, y in zip(sa, sb):
        for k in ("grad_lam", "grad_mu", "grad_rho", "We", "We_adj"):
            assert np.array_equal(x[k], y[k]), k


def test_auto_storage_falls_back_to_binomial(gpu, orc):
    # a budget below what the two-level scheme needs for one shot
    sv, true, init, uz, ux = _setup(orc, fdorder=4, stencil="holberg", nshot=1, nt=400)
    with engine.Plan(sv, storage="checkpoint", max_batch=1) as p:
        p.set_model(*init)
        p.set_observed(uz, ux)
        p.gradient(fetch=False)  # checkpoints are allocated by the first gradient
        need = p.device_bytes
    kinds = []
    for f in (0.9, 0.8, 0.7, 0.6, 0.5, 0.4):
        try:
            with engine.Plan(sv, storage="auto", max_batch=1, hbm_budget_gb=f * need / 1e9) as p:
                kinds.append(p.storage[0])
                if kinds[-1] != "binomial":
                    continue
                p.set_model(*init)
                p.set_observed(uz, ux)
                L2, g = p.gradient()
                assert p.device_bytes < need
            break
        except Exception as e:  # too small for any storage
            kinds.append(str(e))
            break
    assert "binomial" in kinds, kinds
    with engine.Plan(sv, storage="full") as p:
        p.set_model(*init)
        p.set_observed(uz, ux)
        L2f, gf = p.gradient()
    assert L2 == L2f
    for a, b in zip(g, gf):
        assert np.array_equal(a, b)


def test_checkpoint_storage_uses_less_memory(gpu, orc):
    sv, true, init, uz, ux = _setup(orc, fdorder=4, stencil="holberg", nshot=2, nt=600)
    mem = {}
    for storage in ("full", "checkpoint"):
        with engine.Plan(sv, storage=storage) as p:
            p.set_model(*init)
            p.set_observed(uz, ux)
            p.gradient(fetch=False)
            mem[storage] = p.device_bytes
    assert mem["checkpoint"] < 0.5 * mem["full"]


def test_misfit_entry_point_matches_oracle(gpu, orc):
    rng = np.random.default_rng(5)
    mod = rng.standard_normal((3, 17, 301)) * 1e-9
    obs = mod + rng.standard_normal(mod.shape) * 1e-11
    modx, obsx = mod[:, ::-1].copy(), obs[:, ::-1].copy()
    L2, rz, rx = engine.misfit(mod, modx, obs, obsx, 5e-5)
    for s in range(3):
        L2o, az, ax = orc.adjsrc2(mod[s], modx[s], obs[s], obsx[s], 5e-5)
        assert L2[s] == pytest.approx(L2o, rel=1e-13)
        assert np.array_equal(rz[s], az) and np.array_equal(rx[s], ax)


def test_survey_without_receivers(gpu, orc):
    # no receivers: forward modelling runs (empty traces); observed data, and
    # so a gradient, is refused with an error status instead of a zero misfit
    from fwi_cuda_gb300 import _lib
    sv, true, init = helpers.case(fdorder=4, stencil="holberg", nshot=2, nt=120)
    sv.z_rec = np.zeros(0, np.int32)
    sv.x_rec = np.zeros(0, np.int32)
    sv.finalize()
    for precision in (32, 64):
        with engine.Plan(sv, precision=precision) as p:
            p.set_model(*true)
            uz, ux = p.forward()
            assert uz.shape == (2, 0, sv.nt) and ux.shape == (2, 0, sv.nt)
            with pytest.raises(_lib.PSVError, match="no receivers"):
                p.set_observed(uz, ux)
            with pytest.raises(_lib.PSVError):
                p.gradient()


def test_silent_shot_follows_the_reference(gpu, orc):
    # every source fires in shot 0, so shot 1 has no source: its traces and
    # energies are zero, and the reference's scale_grad_E2
    # (src/cpu/n_kernel_lib_PSV.cpp:760-783) divides its zero gradient by a
    # zero energy weight, 0 / 0, over the whole energy window.  The engine
    # does the same: NaN at the oracle's cells, its values elsewhere.
    sv, true, init = helpers.case(fdorder=4, stencil="holberg", nshot=2, nt=120, nz=41,
                                  nx=61, nrec=6)
    sv.src_shot_to_fire = np.zeros(sv.nsrc, np.int32)
    sv.finalize()
    uz, ux = orc.simulate_fwd(sv, *true)
    assert not np.abs(uz[1]).any() and not np.abs(ux[1]).any()
    with np.errstate(invalid="ignore", divide="ignore"):
        L2_ref, g_ref, _ = helpers.oracle_gradient(orc, sv, init, uz, ux)
    nan_ref = [np.isnan(g) for g in g_ref]
    assert all(m.any() for m in nan_ref)
    for precision, tol in ((64, RTOL64), (32, RTOL32_GRAD)):
        with engine.Plan(sv, precision=precision) as p:
            p.set_model(*true)
            fu, fx = p.forward()
            assert not np.abs(fu[1]).any() and not np.abs(fx[1]).any()
            p.set_model(*init)
            p.set_observed(uz, ux)
            L2, g = p.gradient()
        assert L2 == pytest.approx(L2_ref, rel=tol)
        for a, b, m in zip(g, g_ref, nan_ref):
            assert np.array_equal(np.isnan(a), m)
            assert helpers.rel_l2(a[~m], b[~m]) < tol


def test_single_shot_with_chains_requested(gpu, orc):
    # one shot a batch: nothing to split, the plan runs one stream
    sv, true, init = helpers.case(fdorder=4, stencil="holberg", nshot=1, nt=150)
    uz, ux = orc.simulate_fwd(sv, *true)
    out = []
    for chains in (1, 4):
        with engine.Plan(sv, precision=32, kernels="direct", rows_per_thread=1, block=(32, 4),
                         chains=chains) as p:
            assert p.chains == 1
            p.set_model(*init)
            p.set_observed(uz, ux)
            out.append(p.gradient())
    assert out[0][0] == out[1][0]
    for a, b in zip(out[0][1], out[1][1]):
        assert np.array_equal(a, b)
