"""Joint passes (psv_joint_*, psv_joint.cu): several surveys of uneven grid
size, shot count, step count and stencil order stepped in one stress and
one velocity launch per time step must give each survey's own traces and
gradients (the same block bodies as the plan's direct launches with the
same tile shape) to rounding: traces to relative L2 <= 1e-6 in FP32 (the
joint kernels' compiled multiply-add contraction may differ from the
single-survey kernels'), <= 1e-12 in FP64; gradients to 1e-4 in FP32 (the
near-source imaging sum cancels and magnifies rounding differences),
1e-10 in FP64, misfits to 1e-6 / 1e-12.  Repeated calls (graph replays)
repeat themselves bit for bit, and the traces match the FP64 oracle."""
import numpy as np
import pytest

import helpers
from fwi_cuda_gb300 import _lib, engine

pytestmark = pytest.mark.gpu

CASES = [dict(fdorder=4, nz=61, nx=91, nt=300, nshot=2),                       # mirrored rows above the surface
         dict(fdorder=8, nz=83, nx=157, nt=220, nshot=3, surf_offset=0),       # surface on the first interior row
         dict(fdorder=2, stencil="reference", nz=50, nx=70, nt=350, nshot=1),
         dict(fdorder=6, nz=47, nx=133, nt=260, nshot=2, snap_dt=3)]


def _surveys():
    out = []
    for kw in CASES:
        kw = dict(dict(stencil="holberg"), **kw)
        out.append(helpers.case(**kw))
    sv, true, init = helpers.crosswell(nt=280, nshot=2)  # CPML on four sides, x-force sources
    out.append((sv, true, init))
    return out


def _shape(precision, rpt, by):
    return dict(precision=precision, kernels="direct", rows_per_thread=rpt, block=(32, by),
                autotune=False)


def _separate(surveys, **shape):
    res = []
    for sv, true, _ in surveys:
        with engine.Plan(sv, **shape) as p:
            p.set_model(*true)
            res.append(p.forward())
    return res


@pytest.mark.parametrize("precision,rpt,by", [(32, 1, 4), (32, 2, 4), (32, 2, 2), (64, 1, 8)])
def test_joint_forward_equals_each_plan(gpu, precision, rpt, by):
    surveys = _surveys()
    shape = _shape(precision, rpt, by)
    ref = _separate(surveys, **shape)
    plans = [engine.Plan(sv, **shape) for sv, *_ in surveys]
    try:
        for p, (sv, true, _) in zip(plans, surveys):
            p.set_model(*true)
        bar = 1e-6 if precision == 32 else 1e-12
        with engine.Joint(plans, rows_per_thread=rpt, block_y=by) as J:
            first = J.forward()
            again = J.forward()  # replays the captured graph
            assert J.launches() == 2 * max(sv.nt for sv, *_ in surveys)
            assert J.ms > 0
        err = []
        for k, ((uz, ux), (az, ax), (rz, rx)) in enumerate(zip(first, again, ref)):
            assert np.array_equal(uz, az) and np.array_equal(ux, ax), k
            err.append(max(helpers.rel_l2(uz, rz), helpers.rel_l2(ux, rx)))
        print(f"\nFP{precision} rpt {rpt} by {by}: joint vs each plan, rel. L2 per survey",
              " ".join(f"{e:.1e}" for e in err))
        assert max(err) <= bar
        # the plans' own passes afterwards are unaffected
        for p, (rz, rx) in zip(plans, ref):
            uz, ux = p.forward()
            assert np.array_equal(uz, rz) and np.array_equal(ux, rx)
    finally:
        for p in plans:
            p.close()


@pytest.mark.parametrize("precision,rpt,by", [(32, 1, 4), (32, 2, 4), (64, 1, 4)])
def test_joint_gradient_equals_each_plan(gpu, orc, precision, rpt, by):
    # five surveys (orders 2-8, snapshots every step and every third step,
    # uneven step counts): each plan's own full-storage gradient against the
    # joint gradient forward + adjoint passes (two launches per joint step)
    surveys = _surveys()
    shape = dict(_shape(precision, rpt, by), storage="full")
    obs = [orc.simulate_fwd(sv, *true) for sv, true, _ in surveys]
    ref = []
    for (sv, _, init), o in zip(surveys, obs):
        with engine.Plan(sv, **shape) as p:
            p.set_model(*init)
            p.set_observed(*o)
            ref.append(p.gradient())
    plans = [engine.Plan(sv, **shape) for sv, *_ in surveys]
    try:
        for p, (sv, _, init), o in zip(plans, surveys, obs):
            p.set_model(*init)
            p.set_observed(*o)
        with engine.Joint(plans, rows_per_thread=rpt, block_y=by) as J:
            L2 = J.gradient()
            assert J.ms > 0 and J.launches() == 4 * max(sv.nt for sv, *_ in surveys)
            g1 = [p.get_gradient() for p in plans]
            for p in plans:
                p.reset_gradient()
            L2b = J.gradient()  # replays the captured passes
            g2 = [p.get_gradient() for p in plans]
        # FP32: measured 2.5e-5 at one row per thread on the order-8 survey
        # whose source sits two rows below the surface (bit for bit at two)
        bar_l2, bar_g = (1e-6, 1e-4) if precision == 32 else (1e-12, 1e-10)
        err = []
        for k, ((L2r, gr), a, b) in enumerate(zip(ref, g1, g2)):
            assert L2b[k] == L2[k], k
            assert all(np.array_equal(x, y) for x, y in zip(a, b)), k
            assert L2[k] == pytest.approx(L2r, rel=bar_l2), k
            err.append(max(helpers.rel_l2(x, y) for x, y in zip(a, gr)))
        print(f"\nFP{precision} rpt {rpt} by {by}: joint gradient vs each plan, rel. L2 per survey",
              " ".join(f"{e:.1e}" for e in err))
        assert max(err) <= bar_g
    finally:
        for p in plans:
            p.close()


@pytest.mark.parametrize("rpt", [2, 1])
def test_joint_checkpointed_gradient_equals_each_plan(gpu, orc, rpt):
    # checkpointed plans (two-level, binomial, full history mixed): the joint
    # passes run each survey's own schedule (state copies between the
    # launches, recomputed segments beside other surveys' adjoint steps)
    s = _surveys()[:4]
    storages = [dict(storage="checkpoint", checkpoint_interval=20),
                dict(storage="binomial", checkpoint_interval=9, checkpoint_slots=4),
                dict(storage="full"),
                dict(storage="checkpoint", checkpoint_interval=37)]
    obs = [orc.simulate_fwd(sv, *true) for sv, true, _ in s]
    ref = []
    for (sv, _, init), o, st in zip(s, obs, storages):
        with engine.Plan(sv, **_shape(32, rpt, 4), **st) as p:
            p.set_model(*init)
            p.set_observed(*o)
            ref.append(p.gradient())
    plans = [engine.Plan(sv, **_shape(32, rpt, 4), **st) for (sv, *_), st in zip(s, storages)]
    try:
        kinds = [p.storage[0] for p in plans]
        assert kinds == ["checkpoint", "binomial", "full", "checkpoint"]
        for p, (sv, _, init), o in zip(plans, s, obs):
            p.set_model(*init)
            p.set_observed(*o)
        with engine.Joint(plans, rows_per_thread=rpt, block_y=4) as J:
            L2 = J.gradient()
            assert J.launches() >= 4 * max(sv.nt for sv, *_ in s) > 0
        err = []
        for k, ((L2r, gr), p) in enumerate(zip(ref, plans)):
            assert L2[k] == pytest.approx(L2r, rel=1e-6), k
            err.append(max(helpers.rel_l2(x, y) for x, y in zip(p.get_gradient(), gr)))
        print(f"\nFP32 rpt {rpt}: joint checkpointed gradient vs each plan, rel. L2 per survey",
              " ".join(f"{e:.1e}" for e in err))
        assert max(err) <= 1e-4
    finally:
        for p in plans:
            p.close()


def test_joint_gradient_needs_observed_traces(gpu, orc):
    s = _surveys()[:2]
    obs = orc.simulate_fwd(s[0][0], *s[0][1])
    a = engine.Plan(s[0][0], **_shape(32, 1, 4))
    c = engine.Plan(s[1][0], **_shape(32, 1, 4))
    try:
        a.set_model(*s[0][2])
        a.set_observed(*obs)
        c.set_model(*s[1][2])  # no observed traces
        with engine.Joint([a, c], rows_per_thread=1) as J:
            with pytest.raises(_lib.PSVError, match="observed"):
                J.gradient()
    finally:
        a.close()
        c.close()


def test_joint_forward_against_oracle(gpu, orc):
    surveys = _surveys()[:3]
    plans = [engine.Plan(sv, **_shape(32, 1, 4)) for sv, *_ in surveys]
    try:
        for p, (sv, true, _) in zip(plans, surveys):
            p.set_model(*true)
        with engine.Joint(plans) as J:  # shape autotuned on the first forward
            assert J.shape == (0, 0)
            out = J.forward()
            r, b = J.shape
            assert r in (1, 2) and b in (2, 4, 8)
            assert all(p.shape == ("direct", r, b) for p in plans)
        for (uz, ux), (sv, true, _) in zip(out, surveys):
            rz, rx = orc.simulate_fwd(sv, *true)
            assert helpers.rel_l2(uz, rz) < 1e-5 and helpers.rel_l2(ux, rx) < 1e-5
    finally:
        for p in plans:
            p.close()


def test_joint_switches_autotuned_plans_to_its_shape(gpu):
    # plans created with the default options (any family) are set to the
    # direct family with the joint shape and give that shape's traces
    surveys = _surveys()[:2]
    ref = _separate(surveys, **_shape(32, 2, 4))
    plans = [engine.Plan(sv, precision=32) for sv, *_ in surveys]
    try:
        for p, (sv, true, _) in zip(plans, surveys):
            p.set_model(*true)
        with engine.Joint(plans, rows_per_thread=2, block_y=4) as J:
            out = J.forward()
        for p, (uz, ux), (rz, rx) in zip(plans, out, ref):
            assert p.shape == ("direct", 2, 4)
            assert helpers.rel_l2(uz, rz) <= 1e-6 and helpers.rel_l2(ux, rx) <= 1e-6
            fz, fx = p.forward()  # the plan's own pass now has the joint shape
            assert np.array_equal(fz, rz) and np.array_equal(fx, rx)
    finally:
        for p in plans:
            p.close()


def test_joint_rejects_what_it_does_not_run(gpu):
    s = _surveys()
    a = engine.Plan(s[0][0], precision=32)
    b = engine.Plan(s[1][0], precision=64)
    try:
        for p, k in ((a, 0), (b, 1)):
            p.set_model(*s[k][1])
        with pytest.raises(_lib.PSVError, match="precision"):
            engine.Joint([a, b])
        with pytest.raises(_lib.PSVError, match="twice"):
            engine.Joint([a, a])
        with pytest.raises(_lib.PSVError, match="1 to 8"):
            engine.Joint([])
        with pytest.raises(_lib.PSVError, match="rows_per_thread"):
            engine.Joint([a], rows_per_thread=3)
        with pytest.raises(_lib.PSVError, match="block_y"):
            engine.Joint([a], rows_per_thread=1, block_y=9)
        with pytest.raises(_lib.PSVError, match="FP64"):
            engine.Joint([b], rows_per_thread=2)
        d = engine.Plan(s[2][0], precision=32)  # no model
        try:
            with engine.Joint([a, d], rows_per_thread=1) as J:
                with pytest.raises(_lib.PSVError, match="no model"):
                    J.forward()
        finally:
            d.close()
    finally:
        for p in (a, b):
            p.close()


def test_joint_plans_with_several_shot_batches(gpu, orc):
    # plans whose shots do not fit one batch (max_batch below nshot) step
    # batch by batch, batch b of every plan that has one in the same joint
    # launches; traces and gradients as each plan's own
    s = _surveys()
    batch = [dict(max_batch=1), dict(max_batch=2), dict(), dict(max_batch=1), dict(max_batch=1)]
    shape = _shape(32, 2, 4)
    obs = [orc.simulate_fwd(sv, *true) for sv, true, _ in s]
    ref_f, ref_g = [], []
    for (sv, true, init), o, mb in zip(s, obs, batch):
        with engine.Plan(sv, **shape, **mb) as p:
            p.set_model(*true)
            ref_f.append(p.forward())
            p.set_model(*init)
            p.set_observed(*o)
            ref_g.append(p.gradient())
    plans = [engine.Plan(sv, **shape, **mb) for (sv, *_), mb in zip(s, batch)]
    try:
        with engine.Joint(plans, rows_per_thread=2, block_y=4) as J:
            for p, (sv, true, _) in zip(plans, s):
                p.set_model(*true)
            out = J.forward()
            for p, (sv, _, init), o in zip(plans, s, obs):
                p.set_model(*init)
                p.set_observed(*o)
            L2 = J.gradient()
        for k, p in enumerate(plans):
            (rz, rx), (L2r, gr) = ref_f[k], ref_g[k]
            assert helpers.rel_l2(out[k][0], rz) <= 1e-6 and helpers.rel_l2(out[k][1], rx) <= 1e-6, k
            assert L2[k] == pytest.approx(L2r, rel=1e-6), k
            for x, y in zip(p.get_gradient(), gr):
                assert helpers.rel_l2(x, y) <= 1e-4, k
    finally:
        for p in plans:
            p.close()
