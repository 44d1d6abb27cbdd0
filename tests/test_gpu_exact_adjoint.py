"""The exact discrete adjoint (PSV_ADJOINT_EXACT, psv_exact.cu): the
gradient it returns must be the derivative of the misfit the engine
computes.  Checked by directional derivatives against central finite
differences of L2 along random smooth model perturbations, one parameter at
a time, on layouts that exercise every transposed piece: CPML on three or
four sides, a free surface with mirrored rows and one on the first interior
row, orders 2 to 8, both source types, several shots.

Bar: |FD - <grad, dm>| <= 1e-6 |FD|.  With h = 1e-4 relative the central
difference's truncation error is O(h^2) ~ 1e-8 relative and FP64 rounding of
L2 contributes ~1e-12 / 1e-4; a transposition error of one operator, one
boundary row or one average shows up at 1e-3 or more."""
import numpy as np
import pytest

import helpers
from fwi_cuda_gb300 import _lib, engine

pytestmark = pytest.mark.gpu


def _misfit(sv, model, obs):
    with engine.Plan(sv, precision=64) as p:
        p.set_model(*model)
        uz, ux = p.forward()
    return 0.5 * sv.dt * (np.sum((uz - obs[0]) ** 2) + np.sum((ux - obs[1]) ** 2))


def _smooth_direction(shape, seed, scale):
    from scipy.ndimage import gaussian_filter
    rng = np.random.default_rng(seed)
    d = gaussian_filter(rng.standard_normal(shape), 3.0, mode="nearest")
    return d / np.abs(d).max() * scale


def _check(sv, true, init, params=("lam", "mu", "rho"), h=1e-4):
    with engine.Plan(sv, precision=64) as p:
        p.set_model(*true)
        obs = p.forward()
    with engine.Plan(sv, precision=64, adjoint="exact") as p:
        p.set_model(*init)
        p.set_observed(*obs)
        L2, g = p.gradient()
    orient = -1.0 if sv.imaging_sign > 0 else 1.0  # the plan stores -imaging_sign dL2/dm
    grad = [orient * x for x in g]
    assert L2 == pytest.approx(_misfit(sv, init, obs), rel=1e-12)
    out = {}
    for k, name in enumerate(("lam", "mu", "rho")):
        if name not in params:
            continue
        d = _smooth_direction(init[k].shape, 10 + k, h * np.abs(init[k]).max())
        mp = [a.copy() for a in init]
        mm = [a.copy() for a in init]
        mp[k] = mp[k] + d
        mm[k] = mm[k] - d
        fd = (_misfit(sv, mp, obs) - _misfit(sv, mm, obs)) / 2.0
        an = float(np.sum(grad[k] * d))
        out[name] = (fd, an)
        assert an == pytest.approx(fd, rel=1e-6), (name, fd, an)
    return out


@pytest.mark.parametrize("kw", [
    dict(fdorder=4, stencil="holberg", nshot=2, nt=300),                  # mirrored rows above the surface
    dict(fdorder=4, stencil="holberg", nshot=1, nt=300, surf_offset=0),   # surface on the first interior row
    dict(fdorder=2, stencil="reference", nshot=1, nt=250),
    dict(fdorder=8, stencil="holberg", nshot=1, nt=250, imaging_sign=1),
    dict(fdorder=6, stencil="holberg", nshot=2, nt=220, snap_dt=3),
])
def test_exact_gradient_is_the_derivative_of_the_misfit(gpu, kw):
    sv, true, init = helpers.case(nz=61, nx=91, **kw)
    _check(sv, true, init)


def test_exact_gradient_without_surface_and_with_force_sources(gpu):
    # CPML on all four sides, no free surface; x-force sources injected
    # without the dt / rho scaling (stf_type 1)
    sv, true, init = helpers.case(fdorder=4, stencil="holberg", nz=61, nx=91, nt=300, nshot=2)
    sv.surf = False
    sv.npml = (10, 10, 10, 10)
    sv.stf_type = 1
    sv.stf_x, sv.stf_z = np.array(sv.stf_z) * 1e-9, np.zeros_like(sv.stf_z)
    sv.finalize()
    _check(sv, true, init)


def test_exact_mode_fwi_iteration_descends(gpu):
    sv, true, init = helpers.case(fdorder=4, stencil="holberg", nz=61, nx=91, nt=300, nshot=2,
                                  imaging_sign=1)
    with engine.Plan(sv, precision=64) as p:
        p.set_model(*true)
        obs = p.forward()
    with engine.Plan(sv, precision=64, adjoint="exact") as p:
        p.set_model(*init)
        p.set_observed(*obs)
        r = p.fwi_iteration(0.01)
        L2_next, _ = p.gradient(fetch=False)
    assert r["L2"] > 0 and L2_next < r["L2"]


def test_exact_mode_limits(gpu):
    sv, true, init = helpers.case(fdorder=4, stencil="holberg", nz=41, nx=61, nt=60)
    with pytest.raises(_lib.PSVError, match="FP64"):
        engine.Plan(sv, precision=32, adjoint="exact")
    with engine.Plan(sv, precision=64, adjoint="exact") as p:
        p.set_model(*true)
        p.set_observed(*p.forward())
        p.set_model(*init)
        p.gradient(fetch=False)
        with pytest.raises(_lib.PSVError, match="per-shot"):
            p.shot_gradient(0)
    sv.isurf = (0, sv.nz - 8, 0, 0)
    sv.npml = (10, 0, 10, 10)
    sv.z_src = np.full(sv.nsrc, 20, np.int32)
    sv.z_rec = np.full(sv.nrec, sv.nz - 12, np.int32)
    sv.finalize()
    with pytest.raises(_lib.PSVError, match="top one"):
        engine.Plan(sv, precision=64, adjoint="exact")
