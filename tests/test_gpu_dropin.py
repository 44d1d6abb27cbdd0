"""The reference-shaped drop-in psv_kernel_PSV (kernel_PSV's argument list)
against the oracle's kernel_PSV: every output array, forward and adjoint."""
import numpy as np
import pytest

import helpers
from fwi_cuda_gb300 import engine

pytestmark = pytest.mark.gpu


def _call(sv, lam, mu, mz, rz, rx, grad=False, accu=False, history=None, stf=None, src=None,
          precision=64, stencil=None):
    if stf is None:
        stf = (sv.stf_z, sv.stf_x)
        src = (sv.z_src, sv.x_src, sv.src_shot_to_fire, sv.stf_type)
    return engine.kernel_PSV(
        0, sv.nt, sv.nz, sv.nx, sv.dt, sv.dx, sv.dz, sv.surf, sv.isurf, sv.hc, sv.fdorder,
        lam, mu, mz, rz, rx, grad, sv.pml_z,
        (sv.a_z, sv.b_z, sv.K_z, sv.a_half_z, sv.b_half_z, sv.K_half_z), sv.pml_x,
        (sv.a_x, sv.b_x, sv.K_x, sv.a_half_x, sv.b_half_x, sv.K_half_x),
        len(src[0]), src[3], stf[0], stf[1], src[0], src[1], src[2],
        0 if grad else sv.nrec, sv.rtf_type, sv.z_rec, sv.x_rec, accu,
        (sv.snap_z1, sv.snap_z2, sv.snap_x1, sv.snap_x2, sv.snap_dt, sv.snap_dz, sv.snap_dx),
        history=history, stencil=stencil or sv.stencil, precision=precision)


@pytest.mark.parametrize("fd,stencil", [(2, "reference"), (4, "holberg")])
def test_dropin_forward_and_adjoint(gpu, orc, fd, stencil):
    sv, true, _ = helpers.case(fdorder=fd, stencil=stencil, nt=200, snap_dt=2)
    lam, mu, rho = true
    mz, rz, rx, _ = orc.mat_av2(lam, mu, rho)
    a = orc.kernel_PSV(sv, 0, lam, mu, mz, rz, rx, accu=True)
    b = _call(sv, lam, mu, mz, rz, rx, accu=True)
    for k in ("vz", "vx", "uz", "ux", "szz", "szx", "sxx", "We", "rtf_uz", "rtf_ux"):
        assert helpers.rel_l2(b[k], a[k]) < 1e-10, k
    for k in a["history"]:
        assert helpers.rel_l2(b["history"][k], a["history"][k]) < 1e-10, k
    # adjoint with residual-like sources at the receivers and the forward history
    src = (sv.z_rec, sv.x_rec, np.zeros(sv.nrec, np.int32), 0)
    stf = (a["rtf_uz"] * 1e3, a["rtf_ux"] * 1e3)
    ga = orc.kernel_PSV(sv, 0, lam, mu, mz, rz, rx, grad=True, history=a["history"], stf=stf,
                        src=src, rec=False)
    gb = _call(sv, lam, mu, mz, rz, rx, grad=True, history=a["history"], stf=stf, src=src)
    for k in ("grad_lam", "grad_mu", "grad_rho", "uz", "ux", "We", "szz", "vx"):
        assert helpers.rel_l2(gb[k], ga[k]) < 1e-9, k
    # FP32 drop-in within the stated tolerances
    c = _call(sv, lam, mu, mz, rz, rx, accu=True, precision=32)
    assert helpers.rel_l2(c["rtf_uz"], a["rtf_uz"]) < 1e-5
    gc = _call(sv, lam, mu, mz, rz, rx, grad=True, history=a["history"], stf=stf, src=src,
               precision=32)
    for k in ("grad_lam", "grad_mu", "grad_rho"):
        assert helpers.rel_l2(gc[k], ga[k]) < 1e-4, k
