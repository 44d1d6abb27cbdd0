"""Parity on the batched-survey configuration's grid: 1001 x 2001 cells of
0.5 m, 8th-order Holberg, 30-cell CPML, free surface on the first interior
row, dt = 2.5e-5 s, 500 receivers, one shot, the time axis cropped to 800
steps (20 ms), snapshots every 3 steps on every second row and column.  The
true model is 24 dipping layers (vp 1500-4500 m/s, 21 m apart, so that
their reflections return within the cropped record) with a +10 % Gaussian
anomaly of 15 cells 60 rows below the source; the initial model is the true
one smoothed with sigma = 15 cells.  FP32 with the TMA tile kernels (two
rows per thread, the autotuner's choice on this grid) and FP64 with the
direct kernels, against the FP64 oracle (all host cores, about a minute).

Bars.  FP64: 1e-9 on everything.  FP32: seismogram 1e-5 and every
gradient 1e-4 over the whole grid (measured 1.1e-7 and at most 1.1e-5);
misfit 2 kappa e_seis, kappa = |observed traces| / |residual| (529 here),
e_seis the seismogram error: the modelled traces' FP32 error is a kappa
times larger part of the residual, and the misfit, quadratic in the
residual, moves by at most twice that (measured 1.3e-5 against a bound of
1.2e-4).  The measured errors are printed (run with -s).  With the anomaly
alone as the model error (kappa ~1e4, residuals of its weak reflections
only) the FP32 misfit and gradients were measured 6e-4 and 3e-4 from the
oracle's, the seismograms 8e-8: FP32 gradients are as good as the residual
is large against the traces."""
import os

import numpy as np
import pytest

import helpers
from fwi_cuda_gb300 import engine
from fwi_cuda_gb300 import survey as S

pytestmark = pytest.mark.gpu


def _case():
    nz, nx, fd, npml = 1001, 2001, 8, 30
    rng = np.random.default_rng(31)
    vp = S.layered_vp(nz, nx, 24, 1500.0, 4500.0, rng, dip_cells=60.0, top=2 * (fd // 2))
    sv = S.surface_survey(nz, nx, 0.5, 0.5, 800, 2.5e-5, fdorder=fd, npml=npml, nshot=1, nrec=500,
                          rec_spacing=3, fc=100.0, vp_max=float(vp.max()), snap_dt=3,
                          surf_offset=0, seed=7)
    sv.snap_dz = sv.snap_dx = 2
    sv.imaging_sign = 1
    sv.finalize()
    iz = np.arange(nz)[:, None]
    ix = np.arange(nx)[None, :]
    z0, x0 = int(sv.z_src[0]) + 60, int(sv.x_src[0])
    bump = np.exp(-((iz - z0) ** 2 + (ix - x0) ** 2) / (2.0 * 15.0 ** 2))
    vpt = vp * (1.0 + 0.10 * bump)
    return sv, S.model_from_vp(vpt), S.smoothed(vpt, 15.0)


@pytest.fixture(scope="module")
def large(orc):
    sv, true, init = _case()
    orc.set_threads(os.cpu_count() or 1)
    try:
        uz, ux = orc.simulate_fwd(sv, *true)
        L2, g, _ = helpers.oracle_gradient(orc, sv, init, uz, ux)
    finally:
        orc.set_threads(1)
    return sv, true, init, uz, ux, L2, g


@pytest.mark.parametrize("precision,kernels,rpt", [(32, "tma", 2), (64, "direct", 1)])
def test_large_grid_forward_and_gradient(gpu, large, precision, kernels, rpt):
    sv, true, init, uz, ux, L2_ref, g_ref = large
    assert (sv.nz, sv.nx, sv.nt, sv.fdorder) == (1001, 2001, 800, 8)
    with engine.Plan(sv, precision=precision, kernels=kernels, rows_per_thread=rpt,
                     autotune=False) as p:
        assert p.shape[0] == kernels
        p.set_model(*true)
        fz, fx = p.forward()
        p.set_model(*init)
        p.set_observed(uz, ux)
        L2, g = p.gradient()
    e_seis = max(helpers.rel_l2(fz, uz), helpers.rel_l2(fx, ux))
    e_grad = [helpers.rel_l2(a, b) for a, b in zip(g, g_ref)]
    deep = slice(int(sv.z_src[0]) + 24, None)
    e_deep = [helpers.rel_l2(a[deep], b[deep]) for a, b in zip(g, g_ref)]
    e_L2 = abs(L2 - L2_ref) / L2_ref
    kappa = np.sqrt((np.sum(uz ** 2) + np.sum(ux ** 2)) / (2.0 * L2_ref / sv.dt))
    print(f"\nFP{precision} {kernels} vs FP64 oracle, 1001x2001 nt=800: seismogram {e_seis:.2e}, "
          f"gradient lam/mu/rho {e_grad[0]:.2e}/{e_grad[1]:.2e}/{e_grad[2]:.2e} "
          f"(below the near field {e_deep[0]:.2e}/{e_deep[1]:.2e}/{e_deep[2]:.2e}), "
          f"misfit {e_L2:.2e} (L2 {L2_ref:.6e}, |traces| / |residual| {kappa:.1f})")
    assert L2_ref > 0 and np.isfinite(L2)
    if precision == 32:
        assert e_seis <= 1e-5
        assert e_L2 <= max(1e-5, 2.0 * kappa * e_seis)
        assert max(e_grad) <= 1e-4
        assert max(e_deep) <= 1e-4
    else:
        assert e_seis <= 1e-9
        assert max(e_grad) <= 1e-9
        assert e_L2 <= 1e-9
