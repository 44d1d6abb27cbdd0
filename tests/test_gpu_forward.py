"""Forward modelling on the GPU against the FP64 oracle and the reference's
golden traces.  Tolerances: FP64 engine 1e-10 relative L2 (FMA contraction
and summation order are the only differences); FP32 engine 1e-5 relative L2
on seismograms (the stated target)."""
import numpy as np
import pytest

import helpers
from fwi_cuda_gb300 import engine

pytestmark = pytest.mark.gpu
RTOL64 = 1e-10
RTOL32_SEISMO = 1e-5


@pytest.mark.parametrize("fd,stencil", [(2, "reference"), (4, "reference"), (8, "reference"),
                                        (4, "holberg"), (6, "holberg"), (8, "holberg")])
def test_forward_fp64_matches_oracle(gpu, orc, fd, stencil):
    sv, true, _ = helpers.case(fdorder=fd, stencil=stencil, nt=300, nshot=2)
    ref_uz, ref_ux = orc.simulate_fwd(sv, *true)
    with engine.Plan(sv, precision=64) as p:
        p.set_model(*true)
        uz, ux = p.forward()
    assert helpers.rel_l2(uz, ref_uz) < RTOL64
    assert helpers.rel_l2(ux, ref_ux) < RTOL64


@pytest.mark.parametrize("fd,stencil", [(4, "holberg"), (2, "reference"), (8, "holberg")])
def test_forward_fp32_seismogram_tolerance(gpu, orc, fd, stencil):
    sv, true, _ = helpers.case(fdorder=fd, stencil=stencil, nt=800, nz=101, nx=151, nrec=40)
    ref_uz, ref_ux = orc.simulate_fwd(sv, *true)
    with engine.Plan(sv, precision=32) as p:
        p.set_model(*true)
        uz, ux = p.forward()
    e = max(helpers.rel_l2(uz, ref_uz), helpers.rel_l2(ux, ref_ux))
    assert e < RTOL32_SEISMO, e


@pytest.mark.parametrize("name", ["fwd_surface_o2", "fwd_surface_o4"])
def test_forward_matches_reference_golden(gpu, name):
    z = np.load(helpers.GOLDEN)
    sv = helpers.load_case(z, name)
    with engine.Plan(sv, precision=64) as p:
        p.set_model(*z[f"{name}/model"])
        uz, ux = p.forward()
    assert helpers.rel_l2(uz[0], z[f"{name}/rtf_uz"]) < RTOL64
    assert helpers.rel_l2(ux[0], z[f"{name}/rtf_ux"]) < RTOL64
    with engine.Plan(sv, precision=32) as p:
        p.set_model(*z[f"{name}/model"])
        uz, ux = p.forward()
    assert helpers.rel_l2(uz[0], z[f"{name}/rtf_uz"]) < RTOL32_SEISMO


def test_batching_and_graphs_do_not_change_results(gpu):
    sv, true, _ = helpers.case(fdorder=4, stencil="holberg", nt=200, nshot=3)
    out = []
    for kw in (dict(max_batch=0), dict(max_batch=1), dict(max_batch=2, use_graphs=False),
               dict(max_batch=0, block=(64, 4))):
        with engine.Plan(sv, **kw) as p:
            p.set_model(*true)
            out.append(p.forward())
    for uz, ux in out[1:]:
        assert np.array_equal(uz, out[0][0]) and np.array_equal(ux, out[0][1])


def test_other_surfaces_and_no_pml(gpu, orc):
    # bottom free surface with CPML top, then no CPML at all (reflecting box)
    sv, true, _ = helpers.case(fdorder=4, stencil="holberg", nt=250)
    sv.isurf = (0, sv.nz - 8, 0, 0)
    sv.npml = (10, 0, 10, 10)
    sv.z_src = np.full(sv.nsrc, 20, np.int32)
    sv.z_rec = np.full(sv.nrec, sv.nz - 12, np.int32)
    sv.finalize()
    for s in (sv, ):
        a = orc.simulate_fwd(s, *true)
        with engine.Plan(s, precision=64) as p:
            p.set_model(*true)
            b = p.forward()
        assert helpers.rel_l2(b[0], a[0]) < RTOL64
    sv.surf = False
    sv.npml = (0, 0, 0, 0)
    sv.finalize()
    a = orc.simulate_fwd(sv, *true)
    with engine.Plan(sv, precision=64) as p:
        p.set_model(*true)
        b = p.forward()
    assert helpers.rel_l2(b[0], a[0]) < RTOL64


def test_left_right_surfaces(gpu, orc):
    sv, true, _ = helpers.case(fdorder=2, stencil="reference", nt=250)
    sv.isurf = (0, 0, 4, sv.nx - 6)
    sv.npml = (10, 10, 0, 0)
    sv.x_src = np.full(sv.nsrc, 12, np.int32)
    sv.z_src = np.full(sv.nsrc, 30, np.int32)
    sv.finalize()
    a = orc.simulate_fwd(sv, *true)
    with engine.Plan(sv, precision=64) as p:
        p.set_model(*true)
        b = p.forward()
    assert helpers.rel_l2(b[0], a[0]) < RTOL64


def test_velocity_source_and_shared_cells(gpu, orc):
    # stf_type 1 (v += s) and two sources of one shot in the same cell
    sv, true, _ = helpers.case(fdorder=4, stencil="holberg", nt=200)
    sv.stf_type = 1
    sv.z_src = np.array([10, 10], np.int32)
    sv.x_src = np.array([40, 40], np.int32)
    sv.src_shot_to_fire = np.array([0, 0], np.int32)
    sv.stf_z = np.stack([sv.stf_z[0], 0.5 * sv.stf_z[0]])
    sv.stf_x = np.stack([0.3 * sv.stf_z[0], sv.stf_z[0]])
    sv.finalize()
    a = orc.simulate_fwd(sv, *true)
    with engine.Plan(sv, precision=64) as p:
        p.set_model(*true)
        b = p.forward()
    assert helpers.rel_l2(b[0], a[0]) < RTOL64 and helpers.rel_l2(b[1], a[1]) < RTOL64
