"""Largest grids: the 32-bit in-shot offset limit of the time-step kernels.

An FP32 plan holds 14 field planes per shot (the FUSED family's second copy
of v and sigma included) and the interior paths of the time-step kernels
address them with 32-bit offsets, so nz x padded nx x 14 must stay at or
below 2^31 - 1.  A grid one row above the limit is refused at plan creation.
The largest grid of nx = 4032 at the limit (38043 x 4032, 153 M points) runs
a forward (DIRECT and FUSED families) and a gradient from a source near its
far corner, where the offsets are highest, and its traces, imaging and
energies equal those of a 512 x 512
grid with the same corner: the medium is homogeneous, the bottom and right
CPML profiles depend only on the distance to the edge, and within nt steps
nothing reaches a cell where the two grids differ (each step widens the
domain of dependence by at most 2N cells, here 4; the small grid keeps 430
cells between the source and its top / left strips).  FP32 tolerances as
elsewhere: 1e-5 relative L2 on seismograms, 1e-4 on gradients."""
import numpy as np
import pytest

import helpers
from fwi_cuda_gb300 import _lib, engine
from fwi_cuda_gb300 import survey as S

pytestmark = pytest.mark.gpu

NX_BIG = 4032               # a multiple of 32: the FP32 pitch equals nx
PLANES_FP32 = 14
NZ_BIG = _lib.PSV_MAX_SHOT_ELEMS // (PLANES_FP32 * NX_BIG)   # 38043
NT, D = 40, 60              # steps; source distance from the bottom / right edges
W0, W1 = 110, 30            # imaging window: rows / columns [n - W0, n - W1]


def _corner_survey(nz, nx):
    zs, xs = nz - D, nx - D
    rz = zs + np.array([-6, 6, 0, 0, -4, 4])
    rx = xs + np.array([0, 0, -6, 6, 4, -4])
    rng = np.random.default_rng(11)
    return S.Survey(nt=NT, nz=nz, nx=nx, dt=1.5e-4, dz=1.0, dx=1.0, fdorder=4,
                    stencil="holberg", npml=(20, 20, 20, 20), damp_v_pml=2000.0,
                    freq_pml=500.0, snap_z1=nz - W0, snap_z2=nz - W1, snap_x1=nx - W0,
                    snap_x2=nx - W1, snap_dt=1, nshot=1, stf_type=0, z_src=[zs], x_src=[xs],
                    src_shot_to_fire=[0], stf_z=rng.standard_normal((1, NT)),
                    stf_x=rng.standard_normal((1, NT)), z_rec=rz, x_rec=rx).finalize()


def _model(nz, nx):
    vp = np.full((nz, nx), 2000.0)
    return S.elastic_from_velocity(vp, vp / 1.73, np.full((nz, nx), 2000.0))


def _run(nz, nx, kernels, rpt):
    sv = _corner_survey(nz, nx)
    out = {}
    with engine.Plan(sv, precision=32, storage="full", kernels=kernels, rows_per_thread=rpt,
                     block=(32, 4) if kernels == "direct" else (0, 0)) as p:
        p.set_model(*_model(nz, nx))
        out["uz"], out["ux"] = p.forward()
        if kernels == "direct":
            p.set_observed(np.zeros_like(out["uz"]), np.zeros_like(out["ux"]))
            p.gradient(fetch=False)
            g = p.shot_gradient(0)
            for k in ("grad_lam", "grad_mu", "grad_rho"):
                out[k] = g[k]
            out["We"] = g["We"][-W0 - 20:, -W0 - 20:].copy()
            out["We_adj"] = g["We_adj"][-W0 - 20:, -W0 - 20:].copy()
            out["L2"] = g["L2"]
    return out


def test_grid_above_the_offset_limit_is_refused(gpu):
    assert PLANES_FP32 * NZ_BIG * NX_BIG <= _lib.PSV_MAX_SHOT_ELEMS
    assert PLANES_FP32 * (NZ_BIG + 1) * NX_BIG > _lib.PSV_MAX_SHOT_ELEMS
    with pytest.raises(_lib.PSVError) as e:
        engine.Plan(_corner_survey(NZ_BIG + 1, NX_BIG), precision=32, storage="full")
    assert e.value.status == _lib.PSV_ERR_UNSUPPORTED


@pytest.mark.parametrize("kernels,rpt", [("direct", 1), ("fused", 16)])
def test_largest_grid_equals_small_grid_at_the_far_corner(gpu, kernels, rpt):
    small = _run(512, 512, kernels, rpt)
    big = _run(NZ_BIG, NX_BIG, kernels, rpt)
    assert np.abs(small["uz"]).max() > 0 and np.abs(small["ux"]).max() > 0
    for k in ("uz", "ux"):
        assert helpers.rel_l2(big[k], small[k]) < 1e-5, k
    if kernels == "direct":
        assert big["L2"] == pytest.approx(small["L2"], rel=1e-5)
        for k in ("grad_lam", "grad_mu", "grad_rho", "We", "We_adj"):
            assert np.abs(small[k]).max() > 0, k
            assert helpers.rel_l2(big[k], small[k]) < 1e-4, k
