"""Time-step kernel families and shapes: every candidate the autotuner may
pick computes the same gradient, and the tuned plan matches the oracle."""
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
        fam, rpt, _ = p.shape
        assert fam == opt["kernels"] and rpt == opt["rows_per_thread"]  # the shape asked for ran
        return L2, g


def test_autotune_shape_and_parity(gpu, orc):
    # nt = 600: data residual 0.74 % of the traces (at nt = 300 it is 0.27 %
    # and the FP32 gradient error, trace error / residual, sits at the bar)
    sv, true, init = helpers.case(fdorder=4, stencil="holberg", nshot=2, nt=600, nz=81, nx=121)
    uz, ux = orc.simulate_fwd(sv, *true)
    L2_ref, g_ref, _ = helpers.oracle_gradient(orc, sv, init, uz, ux)
    with engine.Plan(sv, precision=32) as p:
        p.set_model(*init)
        p.set_observed(uz, ux)
        fam, rpt, by = p.autotune(8)
        assert (fam == "direct" and rpt in (1, 2, 4, -2, -4) and by in (2, 4, 8)) or \
               (fam == "tma" and rpt in (2, 4, 8)) or \
               (fam == "vec4" and rpt in (1, 2, 4) and by in (2, 4, 8)) or \
               (fam == "fused" and rpt in (16, 32) and by == 0) or \
               (fam == "march" and rpt in (32, 64, 128) and by in (2, 4))
        assert p.shape == (fam, rpt, by)
        L2, g = p.gradient()
    assert L2 == pytest.approx(L2_ref, rel=1e-4)
    for a, b in zip(g, g_ref):
        assert helpers.rel_l2(a, b) < 1e-4


SHAPES = [("direct", 2, 4), ("direct", 4, 2), ("direct", -2, 4), ("direct", -4, 8),
          ("tma", 2, 0), ("tma", 4, 0), ("tma", 8, 0),
          ("vec4", 1, 4), ("vec4", 2, 2), ("vec4", 4, 8),
          ("fused", 16, 0), ("fused", 32, 0)]


@pytest.mark.parametrize("fam,rpt,by", SHAPES)
@pytest.mark.parametrize("fdorder", [4, 8])
def test_every_shape_gives_the_same_gradient(gpu, orc, fam, rpt, by, fdorder):
    # register blocking, warp shuffles and shared-memory staging change which
    # thread loads a value and how the compiler contracts multiply-adds, not
    # the operations: shapes agree to FP32 rounding (1e-5, ten times tighter
    # than the bar against the FP64 oracle)
    sv, true, init = helpers.case(fdorder=fdorder, stencil="holberg", nshot=2, nt=200, nz=75,
                                  nx=97)
    uz, ux = orc.simulate_fwd(sv, *true)
    L2a, ga = _grad(sv, init, uz, ux, kernels="direct", rows_per_thread=1, block=(32, 8))
    L2b, gb = _grad(sv, init, uz, ux, kernels=fam, rows_per_thread=rpt, block=(32, by))
    assert L2b == pytest.approx(L2a, rel=1e-6)
    for a, b in zip(ga, gb):
        assert helpers.rel_l2(b, a) < 1e-5


@pytest.mark.parametrize("fam,rpt", [("tma", 4), ("vec4", 2), ("fused", 32), ("fused", 16)])
@pytest.mark.parametrize("kw", [dict(fdorder=2, stencil="reference", nshot=3, nt=300),
                                dict(fdorder=6, stencil="holberg", nshot=2, nt=250,
                                     imaging_sign=1),
                                dict(fdorder=4, stencil="holberg", nshot=1, nt=250,
                                     surf_offset=3),
                                dict(fdorder=8, stencil="holberg", nshot=2, nt=450, nz=96,
                                     nx=300)])
def test_tiled_families_against_oracle(gpu, orc, kw, fam, rpt):
    # The 96 x 300 case has plain blocks (interior, away from CPML and the
    # surface) in both families.  Its data residual is 0.45 % of the traces:
    # the FP32 gradient error against the oracle grows like the FP32 trace
    # error divided by the relative residual, so a case whose waves have not
    # yet reached the model perturbation (residual at round-off) cannot be
    # compared at all.
    kw = dict(dict(nz=70, nx=130), **kw)
    sv, true, init = helpers.case(**kw)
    uz_ref, ux_ref = orc.simulate_fwd(sv, *true)
    L2_ref, g_ref, _ = helpers.oracle_gradient(orc, sv, init, uz_ref, ux_ref)
    with engine.Plan(sv, precision=32, kernels=fam, rows_per_thread=rpt) as p:
        assert p.shape[:2] == (fam, rpt)
        p.set_model(*true)
        uz, ux = p.forward()
        assert helpers.rel_l2(uz, uz_ref) < 1e-5 and helpers.rel_l2(ux, ux_ref) < 1e-5
        p.set_model(*init)
        p.set_observed(uz_ref, ux_ref)
        L2, g = p.gradient()
    assert L2 == pytest.approx(L2_ref, rel=1e-4)
    for a, b in zip(g, g_ref):
        assert helpers.rel_l2(a, b) < 1e-4


@pytest.mark.parametrize("fam", ["tma", "vec4", "fused"])
def test_tiled_families_checkpointed_equal_full(gpu, orc, fam):
    sv, true, init = helpers.case(fdorder=4, stencil="holberg", nshot=2, nt=300, snap_dt=3)
    uz, ux = orc.simulate_fwd(sv, *true)
    out = []
    for storage, slots in (("full", 0), ("checkpoint", 0), ("binomial", 3)):
        with engine.Plan(sv, precision=32, kernels=fam, rows_per_thread=16 if fam == "fused" else 2,
                         storage=storage, checkpoint_interval=40, checkpoint_slots=slots) as p:
            assert p.shape[0] == fam and p.storage[0] == storage
            p.set_model(*init)
            p.set_observed(uz, ux)
            out.append(p.gradient())
    (La, ga), *rest = out
    for Lb, gb in rest:
        assert La == Lb
        for a, b in zip(ga, gb):
            assert np.array_equal(a, b)


@pytest.mark.parametrize("rpt", [16, 32])
def test_fused_step_without_free_surface(gpu, orc, rpt):
    # CPML on all four sides (the top strip included), no free surface, odd
    # step count (the pass ends on the second field copy), snapshots every
    # third step
    sv, true, init = helpers.case(fdorder=4, stencil="holberg", nt=301, nshot=2, snap_dt=3)
    sv.surf = False
    sv.npml = (10, 10, 10, 10)
    sv.finalize()
    uz_ref, ux_ref = orc.simulate_fwd(sv, *true)
    L2_ref, g_ref, _ = helpers.oracle_gradient(orc, sv, init, uz_ref, ux_ref)
    with engine.Plan(sv, precision=32, kernels="fused", rows_per_thread=rpt) as p:
        assert p.shape == ("fused", rpt, 0)
        p.set_model(*true)
        uz, ux = p.forward()
        assert helpers.rel_l2(uz, uz_ref) < 1e-5 and helpers.rel_l2(ux, ux_ref) < 1e-5
        p.set_model(*init)
        p.set_observed(uz_ref, ux_ref)
        L2, g = p.gradient()
    assert L2 == pytest.approx(L2_ref, rel=1e-4)
    for a, b in zip(g, g_ref):
        assert helpers.rel_l2(a, b) < 1e-4


def test_fused_step_rejects_a_bottom_surface(gpu):
    from fwi_cuda_gb300 import _lib
    sv, true, _ = helpers.case(fdorder=4, stencil="holberg", nt=60)
    sv.isurf = (0, sv.nz - 8, 0, 0)
    sv.npml = (10, 0, 10, 10)
    sv.z_src = np.full(sv.nsrc, 20, np.int32)
    sv.z_rec = np.full(sv.nrec, sv.nz - 12, np.int32)
    sv.finalize()
    with pytest.raises(_lib.PSVError, match="fused"):
        engine.Plan(sv, precision=32, kernels="fused")
    with engine.Plan(sv, precision=32) as p:  # the autotuner leaves it out
        p.set_model(*true)
        p.set_observed(*p.forward())
        assert p.autotune(4)[0] != "fused"
