"""The oracle (oracle/psv_oracle.c) pinned to the reference.

* against the golden vectors in tests/golden/reference_cases.npz, generated
  by the reference's own CPU code (tests/golden/make_golden.py): bit for bit;
* against the reference library itself when it is built here
  (oracle/_ref/libref_psv.so): bit for bit, including the FWI loop.
"""
import numpy as np
import pytest

import helpers
from oracle import oracle as O


@pytest.fixture(scope="module")
def golden():
    return np.load(helpers.GOLDEN)


def test_host_preprocessing_matches_golden(orc, golden):
    for fd in (2, 4, 6, 8):
        assert np.array_equal(orc.holbergcoeff(fd), golden[f"hc/{fd}"])
    prof = orc.cpml(2.0, 3000.0, 0.001, 1.0, 100.0, 20, 20, 2, 141, 5e-5, 0.5)
    assert np.array_equal(np.stack(prof), golden["cpml"])
    assert np.array_equal(orc.wavelet(800, 5e-5, 1.0, 100.0), golden["wavelet"])


@pytest.mark.parametrize("name", ["fwd_surface_o2", "fwd_surface_o4"])
def test_forward_matches_golden_bitwise(orc, golden, name):
    sv = helpers.load_case(golden, name)
    lam, mu, rho = golden[f"{name}/model"]
    mz, rz, rx, _ = orc.mat_av2(lam, mu, rho)
    o = orc.kernel_PSV(sv, 0, lam, mu, mz, rz, rx, accu=True)
    for k in ("rtf_uz", "rtf_ux", "vz", "vx", "szz", "szx", "sxx", "We", "uz", "ux"):
        assert np.array_equal(o[k], golden[f"{name}/{k}"]), k
    assert np.array_equal(o["history"]["szz"][::25], golden[f"{name}/hist_szz"])


def test_fwi_iterations_match_golden_bitwise(orc, golden):
    name = "fwi_crosswell"
    sv = helpers.load_case(golden, name)
    r = orc.simulate_fwi(sv, *golden[f"{name}/init"], golden[f"{name}/obs_uz"],
                         golden[f"{name}/obs_ux"], niter=10)
    assert r["rc"] == 0
    for k in ("L2", "step", "lam", "mu", "rho", "grad_lam", "grad_mu", "grad_rho"):
        assert np.array_equal(r[k], golden[f"{name}/{k}"]), k


def test_calc_opt_step_is_parabola_vertex(orc):
    # L2 = 3 (a - 0.25)^2 + 1 sampled at 0, 0.2, 0.5: vertex 0.25 inside (0, 0.5]
    sl = np.array([0.0, 0.2, 0.5])
    L2 = 3.0 * (sl - 0.25) ** 2 + 1.0
    assert orc.calc_opt_step(L2, sl) == pytest.approx(0.25, rel=1e-12)
    # monotone decrease -> the largest step (n_step_length_PSV.cpp:508-510)
    assert orc.calc_opt_step(np.array([3.0, 2.0, 1.0]), sl) == 0.5


def test_step_length_control_flow(orc):
    # quadratic misfit with minimum at 0.037: halve from 0.1? no - 0.1 is worse
    # than 0 only if L2(0.1) >= L2(0); here L2(0.1) < L2(0) so it grows.
    f = lambda a: (a - 0.037) ** 2
    rc, step, n, log = orc.step_length(0.01, f(0.0), f)
    assert rc == 0 and n >= 2
    assert step == pytest.approx(0.037, rel=1e-9)
    # every trial misfit larger than L2_0 -> 31 halvings then failure (the reference exits)
    rc, _, n, _ = orc.step_length(0.01, 0.0, lambda a: 1.0 + a)
    assert rc == -1 and n == 31


ref_only = pytest.mark.skipif(not O.ref_available(), reason="reference library not built here")


def _in_child(fn, *args):
    """Run fn(*args) in a spawned child process: the reference's error paths
    print and call exit(0), which in this process would end the test run
    early with a success status; in a child it breaks the pool instead."""
    import concurrent.futures as cf
    import multiprocessing as mp
    with cf.ProcessPoolExecutor(1, mp_context=mp.get_context("spawn")) as pool:
        return pool.submit(fn, *args).result(timeout=600)


def _libraries():
    from oracle import oracle as O2
    O2.build()
    orc = O2.oracle()
    orc.set_threads(1)
    ref = O2.reference()
    ref.set_threads(1)
    return orc, ref


def _kernel_against_reference(fd):
    orc, ref = _libraries()
    sv, true, _ = helpers.case(fdorder=fd, stencil="reference", nt=200, nz=51, nx=71, npml=8,
                               nrec=12)
    lam, mu, rho = true
    mz, rz, rx, C = orc.mat_av2(lam, mu, rho)
    mz2, rz2, rx2, C2 = ref.mat_av2(lam, mu, rho)
    same = {"mat_av2": bool(np.array_equal(mz[:-1, :-1], mz2[:-1, :-1]) and np.array_equal(C, C2))}
    a = orc.kernel_PSV(sv, 0, lam, mu, mz, rz, rx, accu=True)
    b = ref.kernel_PSV(sv, 0, lam, mu, mz, rz, rx, accu=True)
    for k in ("rtf_uz", "rtf_ux", "vz", "vx", "szz", "szx", "sxx", "We", "uz", "ux"):
        same["fwd " + k] = bool(np.array_equal(a[k], b[k]))
    # adjoint: residual-like sources at the receivers, time reversed, imaging
    nrec = sv.nrec
    src = (sv.z_rec, sv.x_rec, np.zeros(nrec, np.int32), 0)
    stf = (a["rtf_uz"] * 1e3, a["rtf_ux"] * 1e3)
    ga = orc.kernel_PSV(sv, 0, lam, mu, mz, rz, rx, grad=True, history=a["history"], stf=stf,
                        src=src, rec=False)
    gb = ref.kernel_PSV(sv, 0, lam, mu, mz, rz, rx, grad=True, history=a["history"], stf=stf,
                        src=src, rec=False)
    for k in ("grad_lam", "grad_mu", "grad_rho", "uz", "ux", "We", "szz"):
        same["adj " + k] = bool(np.array_equal(ga[k], gb[k]))
    return same


@ref_only
@pytest.mark.parametrize("fd", [2, 4, 8])
def test_forward_and_adjoint_match_reference_library(fd):
    same = _in_child(_kernel_against_reference, fd)
    assert all(same.values()), same


def _fwi2_against_reference():
    orc, ref = _libraries()
    sv, true, init = helpers.case(fdorder=4, stencil="reference", nshot=2, nt=250, nz=51,
                                  nx=71, npml=8, nrec=12, imaging_sign=1)
    uz, ux = orc.simulate_fwd(sv, *true)
    r1 = orc.simulate_fwi(sv, *init, uz, ux, niter=2)
    r2 = ref.simulate_fwi(sv, *init, uz, ux, niter=2)
    same = {k: bool(np.array_equal(r1[k], r2[k])) for k in
            ("L2", "step", "lam", "mu", "rho", "grad_lam", "grad_mu", "grad_rho")}
    return int(r1["rc"]), int(r2["rc"]), same


@ref_only
def test_fwi_matches_reference_library_surface_layout():
    rc1, rc2, same = _in_child(_fwi2_against_reference)
    assert rc1 == 0 and rc2 == 0
    assert all(same.values()), same


def _layout(name):
    """FWI layouts for the reference-library pins; imaging_sign = 1 (the
    reference's CUDA sign), the sign whose update lowers the misfit, so the
    reference's step search succeeds."""
    if name == "order6":
        return helpers.case(fdorder=6, stencil="reference", nt=180, nz=51, nx=71, npml=8,
                            nrec=12, imaging_sign=1)
    if name == "subsampled":
        sv, true, init = helpers.case(fdorder=4, stencil="reference", nt=180, nz=51, nx=71,
                                      npml=8, nrec=12, snap_dt=3, imaging_sign=1)
        sv.snap_dz, sv.snap_dx = 2, 3
        sv.snap_z1, sv.snap_z2, sv.snap_x1, sv.snap_x2 = 5, sv.nz - 9, 7, sv.nx - 10
        return sv, true, init
    if name == "velocity_sources":
        return helpers.crosswell(fdorder=2, stencil="reference", nt=250, nz=61, nx=51, nshot=2,
                                 nrec=10)
    if name == "side_surfaces":
        sv, true, init = helpers.case(fdorder=2, stencil="reference", nt=180, nz=51, nx=71,
                                      nrec=12, imaging_sign=1)
        sv.isurf = (0, 0, 4, sv.nx - 6)
        sv.npml = (10, 10, 0, 0)
        sv.x_src = np.full(sv.nsrc, 12, np.int32)
        sv.z_src = np.full(sv.nsrc, 30, np.int32)
        return sv.finalize(), true, init
    raise KeyError(name)


def _fwi_against_reference(name):
    """Run in a child process (the reference's error paths call exit):
    one FWI iteration of the oracle and of the reference library."""
    orc, ref = _libraries()
    sv, true, init = _layout(name)
    uz, ux = orc.simulate_fwd(sv, *true)
    r1 = orc.simulate_fwi(sv, *init, uz, ux, niter=1)
    r2 = ref.simulate_fwi(sv, *init, uz, ux, niter=1)
    same = {k: bool(np.array_equal(r1[k], r2[k])) for k in
            ("L2", "step", "lam", "mu", "rho", "grad_lam", "grad_mu", "grad_rho")}
    return int(r1["rc"]), int(r2["rc"]), same


@ref_only
@pytest.mark.parametrize("name", ["order6", "subsampled", "velocity_sources", "side_surfaces"])
def test_more_layouts_match_reference_library(name):
    # one FWI iteration (forward, residuals, adjoint, imaging with the
    # snapshot interpolation, energy preconditioning, step-length trials,
    # update) of the oracle and of the reference's own code, bit for bit
    rc1, rc2, same = _in_child(_fwi_against_reference, name)
    assert rc1 == 0 and rc2 == 0
    assert all(same.values()), same


@pytest.mark.parametrize("cause", ["silent_shot", "zero_gradient"])
def test_fwi_with_a_nan_update_stops(orc, cause):
    # silent_shot: the gradient is NaN (0 / 0 in scale_grad_E2); zero_gradient
    # (a one-cell window images nothing): update_mat2 scales by
    # max|mat| / max|grad| = inf and inf * 0 is NaN.  Either way the first
    # trial's misfit is NaN: the reference's step search would loop for ever,
    # the oracle (like the engine) reports a failed search
    sv, true, init = helpers.case(fdorder=4, stencil="reference", nshot=2, nt=120, nz=41,
                                  nx=61, nrec=6, imaging_sign=1)
    if cause == "silent_shot":
        sv.src_shot_to_fire = np.zeros(sv.nsrc, np.int32)
    else:
        sv.snap_z1 = sv.snap_z2 = 20
        sv.snap_x1 = sv.snap_x2 = 30
    sv.finalize()
    uz, ux = orc.simulate_fwd(sv, *true)
    r = orc.simulate_fwi(sv, *init, uz, ux, niter=1)
    assert r["rc"] != 0 and np.isnan(r["lam"]).any()
