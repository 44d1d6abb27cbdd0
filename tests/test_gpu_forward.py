"""Forward modelling on the GPU against the FP64 oracle and the reference's
golden traces.  Tolerances: FP64 engine 1e-10 relative L2 (FMA contraction
and summation order are the only differences); FP32 engine 1e-5 relative L2
on seismograms (the stated target)."""
import numpy as np
import pytest

import helpers
from fwi_cuda_gb300 import engine
from fwi_cuda_gb300 import survey as S

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


def _topography_case(nt=400):
    # a ground profile with air above it (lam = mu = 0, rho = 1.25), a softer
    # layer along the surface, CPML on all sides, sources and receivers on the
    # ground: the layout of the reference's field scripts
    x = np.linspace(-2.0, 12.0, 30)
    z = 1.0 + 0.3 * np.sin(x / 2.0)
    t = S.topography_grid(x, z, 0.0, 8.0, 0.1, 0.1, npml=(10, 10, 10, 10), fpad=2, z_above=6,
                          z_below=25)
    layers = ((1.0, 700.0, 300.0, 1200.0),)
    true = S.topography_model(t, (1200.0, 500.0, 2000.0), layers=layers, perturb=0.1, sigma=1.5,
                              rng=np.random.default_rng(3))
    zs, xs = t.on_surface([2.0, 6.0])
    zr, xr = t.on_surface(np.linspace(1.0, 7.0, 12))
    dt, fpad = 2e-5, 2
    sv = S.Survey(nt=nt, nz=t.nz, nx=t.nx, dt=dt, dz=t.dz, dx=t.dx, fdorder=4, stencil="holberg",
                  npml=(10, 10, 10, 10), damp_v_pml=1200.0, freq_pml=150.0,
                  snap_z1=10 + fpad, snap_z2=t.nz - 10 - fpad - 1, snap_x1=10 + fpad,
                  snap_x2=t.nx - 10 - fpad - 1, snap_dt=2,
                  taper=(14, 16, t.nz - 15, t.nz - 17, 14, 16, t.nx - 15, t.nx - 17),
                  imaging_sign=-1, nshot=2, stf_type=1, z_src=zs, x_src=xs,
                  src_shot_to_fire=np.arange(2), stf_z=np.stack([S.ricker(nt, dt, 150.0)] * 2),
                  stf_x=np.zeros((2, nt)), z_rec=zr, x_rec=xr)
    return sv.finalize(), true


@pytest.mark.parametrize("precision,tol,kw", [(64, RTOL64, {}), (32, 1e-5, {}),
                                              (32, 1e-5, dict(kernels="fused", rows_per_thread=32))])
def test_topography_with_air_cells(gpu, orc, precision, tol, kw):
    sv, true = _topography_case()
    assert (true[1] == 0).any()  # vacuum cells take mat_av2's special cases
    a = orc.simulate_fwd(sv, *true)
    with engine.Plan(sv, precision=precision, **kw) as p:
        p.set_model(*true)
        b = p.forward()
    assert np.abs(a[0]).max() > 0
    for x, y in zip(b, a):
        assert helpers.rel_l2(x, y) < tol
