"""The MARCH time-step family (psv_march.cu): one launch per step, each CTA
walking down a strip of columns.  It must give the direct family's gradient
to FP32 rounding, match the FP64 oracle at the stated bars, recompute the
checkpointed gradient bit for bit, and refuse the free-surface placements it
does not handle."""
import numpy as np
import pytest

import helpers
from fwi_cuda_gb300 import _lib, engine

pytestmark = pytest.mark.gpu

SHAPES = [(32, 2), (64, 4), (128, 4), (128, 2)]


def _grad(sv, init, uz, ux, **opt):
    with engine.Plan(sv, precision=32, **opt) as p:
        p.set_model(*init)
        p.set_observed(uz, ux)
        L2, g = p.gradient()
        return L2, g, p.shape


@pytest.mark.parametrize("rows,warps", SHAPES)
@pytest.mark.parametrize("fdorder", [2, 4, 6, 8])
def test_march_gives_the_direct_family_gradient(gpu, orc, rows, warps, fdorder):
    # surface on the first interior row (the benchmark placement); a grid
    # whose width and height are not multiples of the strip width or march
    # length, so partial strips and segments are exercised
    sv, true, init = helpers.case(fdorder=fdorder, stencil="holberg", nshot=2, nt=220, nz=83,
                                  nx=157, surf_offset=0, snap_dt=3)
    uz, ux = orc.simulate_fwd(sv, *true)
    L2a, ga, _ = _grad(sv, init, uz, ux, kernels="direct", rows_per_thread=1, block=(32, 4))
    L2b, gb, shape = _grad(sv, init, uz, ux, kernels="march", rows_per_thread=rows,
                           block=(32, warps))
    assert shape == ("march", rows, warps)
    assert L2b == pytest.approx(L2a, rel=1e-6)
    # the two families contract different multiply-adds; with the source two
    # cells below the surface the near-source imaging sum cancels strongly
    # and magnifies that rounding difference (measured 1.3e-5 at order 2)
    for a, b in zip(ga, gb):
        assert helpers.rel_l2(b, a) < 5e-5


@pytest.mark.parametrize("kw", [dict(fdorder=4, stencil="holberg", nshot=2, nt=450, nz=96,
                                     nx=300, surf_offset=0),
                                dict(fdorder=8, stencil="holberg", nshot=2, nt=450, nz=96,
                                     nx=300, surf_offset=0, imaging_sign=1),
                                dict(fdorder=2, stencil="reference", nshot=3, nt=300,
                                     surf_offset=0)])
def test_march_against_oracle(gpu, orc, kw):
    kw = dict(dict(nz=70, nx=130), **kw)
    sv, true, init = helpers.case(**kw)
    uz_ref, ux_ref = orc.simulate_fwd(sv, *true)
    L2_ref, g_ref, shots = helpers.oracle_gradient(orc, sv, init, uz_ref, ux_ref)
    with engine.Plan(sv, precision=32, kernels="march", rows_per_thread=32, block=(32, 4)) as p:
        p.set_model(*true)
        uz, ux = p.forward()
        assert helpers.rel_l2(uz, uz_ref) < 1e-5 and helpers.rel_l2(ux, ux_ref) < 1e-5
        p.set_model(*init)
        p.set_observed(uz_ref, ux_ref)
        L2, g = p.gradient()
        o = p.shot_gradient(0)
    assert L2 == pytest.approx(L2_ref, rel=1e-4)
    for a, b in zip(g, g_ref):
        assert helpers.rel_l2(a, b) < 1e-4
    for k in ("We", "We_adj"):
        assert helpers.rel_l2(o[k], shots[0][k]) < 1e-4, k


def test_march_without_free_surface_odd_steps(gpu, orc):
    # CPML on all four sides (the top strip included), no free surface, an
    # odd step count (the pass ends on the second field copy)
    sv, true, init = helpers.case(fdorder=4, stencil="holberg", nt=301, nshot=2, snap_dt=3)
    sv.surf = False
    sv.npml = (10, 10, 10, 10)
    sv.finalize()
    uz_ref, ux_ref = orc.simulate_fwd(sv, *true)
    L2_ref, g_ref, _ = helpers.oracle_gradient(orc, sv, init, uz_ref, ux_ref)
    with engine.Plan(sv, precision=32, kernels="march", rows_per_thread=64, block=(32, 2)) as p:
        assert p.shape == ("march", 64, 2)
        p.set_model(*true)
        uz, ux = p.forward()
        assert helpers.rel_l2(uz, uz_ref) < 1e-5 and helpers.rel_l2(ux, ux_ref) < 1e-5
        p.set_model(*init)
        p.set_observed(uz_ref, ux_ref)
        L2, g = p.gradient()
    assert L2 == pytest.approx(L2_ref, rel=1e-4)
    for a, b in zip(g, g_ref):
        assert helpers.rel_l2(a, b) < 1e-4


def test_march_checkpointed_equal_full(gpu, orc):
    sv, true, init = helpers.case(fdorder=4, stencil="holberg", nshot=2, nt=300, snap_dt=3,
                                  surf_offset=0)
    uz, ux = orc.simulate_fwd(sv, *true)
    out = []
    for storage, slots in (("full", 0), ("checkpoint", 0), ("binomial", 3)):
        with engine.Plan(sv, precision=32, kernels="march", rows_per_thread=32, block=(32, 4),
                         storage=storage, checkpoint_interval=40, checkpoint_slots=slots) as p:
            assert p.shape[0] == "march" and p.storage[0] == storage
            p.set_model(*init)
            p.set_observed(uz, ux)
            out.append(p.gradient())
    (La, ga), *rest = out
    for Lb, gb in rest:
        assert La == Lb
        for a, b in zip(ga, gb):
            assert np.array_equal(a, b)


def test_march_rejects_mirrored_rows_and_other_surfaces(gpu):
    # a top surface with rows mirrored above it, and a bottom surface
    sv, true, _ = helpers.case(fdorder=4, stencil="holberg", nt=60)  # surface 2 rows down
    with pytest.raises(_lib.PSVError, match="march"):
        engine.Plan(sv, precision=32, kernels="march")
    sv.isurf = (0, sv.nz - 8, 0, 0)
    sv.npml = (10, 0, 10, 10)
    sv.z_src = np.full(sv.nsrc, 20, np.int32)
    sv.z_rec = np.full(sv.nrec, sv.nz - 12, np.int32)
    sv.finalize()
    with pytest.raises(_lib.PSVError, match="march"):
        engine.Plan(sv, precision=32, kernels="march")
    with engine.Plan(sv, precision=32) as p:  # the autotuner leaves it out
        p.set_model(*true)
        p.set_observed(*p.forward())
        assert p.autotune(4)[0] != "march"
