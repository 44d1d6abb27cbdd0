"""Degenerate surveys against the FP64 oracle: a grid smaller than one thread
block, a single time step, a one-cell imaging window, sources and receivers
in the stencil padding rows / columns (the reference injects and records
there like anywhere else; those cells are never updated by the stencil), a
source and a receiver on the same cell.  FP64 engine 1e-9 relative L2, FP32
1e-5 on seismograms and 1e-4 on gradients, as in the other parity tests."""
import numpy as np
import pytest

import helpers
from fwi_cuda_gb300 import engine
from fwi_cuda_gb300 import survey as S

pytestmark = pytest.mark.gpu
TOL = {64: (1e-9, 1e-9), 32: (1e-5, 1e-4)}   # seismograms, gradients


def _survey(nz, nx, nt, z_src, x_src, z_rec, x_rec, npml=(0, 0, 0, 0), window=None,
            snap_dt=1, fdorder=4, seed=5):
    rng = np.random.default_rng(seed)
    n = len(z_src)
    fpad = fdorder // 2
    z1, z2, x1, x2 = window or (fpad, nz - fpad - 1, fpad, nx - fpad - 1)
    return S.Survey(nt=nt, nz=nz, nx=nx, dt=1e-4, dz=1.0, dx=1.0, fdorder=fdorder,
                    stencil="holberg", npml=npml, damp_v_pml=2000.0, freq_pml=500.0,
                    snap_z1=z1, snap_z2=z2, snap_x1=x1, snap_x2=x2, snap_dt=snap_dt, nshot=n,
                    z_src=z_src, x_src=x_src, src_shot_to_fire=np.arange(n),
                    stf_z=rng.standard_normal((n, nt)), stf_x=rng.standard_normal((n, nt)),
                    z_rec=z_rec, x_rec=x_rec).finalize()


def _models(nz, nx, seed=5):
    rng = np.random.default_rng(seed)
    vp = 2000.0 + 300.0 * rng.random((nz, nx))
    true = S.model_from_vp(vp)
    init = S.model_from_vp(np.full((nz, nx), float(vp.mean())))
    return true, init


def _check(orc, sv, precision):
    true, init = _models(sv.nz, sv.nx)
    uz, ux = orc.simulate_fwd(sv, *true)
    L2_ref, g_ref, _ = helpers.oracle_gradient(orc, sv, init, uz, ux)
    ts, tg = TOL[precision]
    with engine.Plan(sv, precision=precision) as p:
        p.set_model(*true)
        fu, fx = p.forward()
        assert helpers.rel_l2(fu, uz) < ts and helpers.rel_l2(fx, ux) < ts
        p.set_model(*init)
        p.set_observed(uz, ux)
        L2, g = p.gradient()
    assert L2 == pytest.approx(L2_ref, rel=tg)
    for a, b in zip(g, g_ref):
        m = np.isnan(b)  # the reference's 0 / 0 where no forward energy arrived
        assert np.array_equal(np.isnan(a), m)
        assert helpers.rel_l2(a[~m], b[~m]) < tg
    return uz, g_ref


@pytest.mark.parametrize("precision", [64, 32])
def test_grid_smaller_than_a_block(gpu, orc, precision):
    # 12 x 13 cells: one partial 32 x 4 block column, no CPML, two shots
    sv = _survey(12, 13, 60, [5, 7], [6, 4], [3, 8, 9], [2, 10, 6])
    uz, g = _check(orc, sv, precision)
    assert np.abs(uz).max() > 0 and np.abs(g[0]).max() > 0


@pytest.mark.parametrize("precision", [64, 32])
@pytest.mark.parametrize("nt", [1, 2])
def test_one_and_two_time_steps(gpu, orc, precision, nt):
    # nt = 1: the forward energy (accumulated from the old velocities) is
    # still zero after the only step, so the reference's gradient is 0 / 0
    # over the whole energy window
    sv = _survey(40, 50, nt, [20], [25], [20, 21], [25, 24], npml=(8, 8, 8, 8))
    _, g = _check(orc, sv, precision)
    assert np.isnan(g[0]).any() == (nt == 1)


@pytest.mark.parametrize("precision", [64, 32])
@pytest.mark.parametrize("window,cells", [((19, 19, 24, 24), 0), ((19, 20, 24, 25), 1)])
def test_smallest_imaging_windows(gpu, orc, precision, window, cells):
    # snapshots cover [z1, z2] x [x1, x2]; energy_weights2 and scale_grad_E2
    # (src/cpu/n_kernel_lib_PSV.cpp:696-783) loop over [z1, z2) x [x1, x2),
    # so a one-cell window images nothing and the next size one cell
    sv = _survey(40, 50, 80, [20], [25], [18, 22], [27, 23], npml=(8, 8, 8, 8),
                 window=window, snap_dt=3)
    _, g = _check(orc, sv, precision)
    assert np.count_nonzero(g[2]) == cells


@pytest.mark.parametrize("precision", [64, 32])
def test_sources_and_receivers_in_the_padding(gpu, orc, precision):
    # fpad = 2: rows / columns 0, 1 and the last two take injections and
    # recordings; a third source shares its cell with a receiver
    sv = _survey(36, 44, 70, [1, 20, 30], [20, 0, 15], [0, 35, 18, 30], [5, 43, 1, 15])
    uz, _ = _check(orc, sv, precision)
    assert np.abs(uz[:, 3]).max() > 0
