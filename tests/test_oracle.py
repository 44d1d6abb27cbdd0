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


@ref_only
@pytest.mark.parametrize("fd", [2, 4, 8])
def test_forward_and_adjoint_match_reference_library(orc, fd):
    ref = O.reference()
    ref.set_threads(1)
    sv, true, _ = helpers.case(fdorder=fd, stencil="reference", nt=200, nz=51, nx=71, npml=8,
                               nrec=12)
    lam, mu, rho = true
    mz, rz, rx, C = orc.mat_av2(lam, mu, rho)
    mz2, rz2, rx2, C2 = ref.mat_av2(lam, mu, rho)
    assert np.array_equal(mz[:-1, :-1], mz2[:-1, :-1]) and np.array_equal(C, C2)
    a = orc.kernel_PSV(sv, 0, lam, mu, mz, rz, rx, accu=True)
    b = ref.kernel_PSV(sv, 0, lam, mu, mz, rz, rx, accu=True)
    for k in ("rtf_uz", "rtf_ux", "vz", "vx", "szz", "szx", "sxx", "We", "uz", "ux"):
        assert np.array_equal(a[k], b[k]), k
    # adjoint: residual-like sources at the receivers, time reversed, imaging
    nrec = sv.nrec
    src = (sv.z_rec, sv.x_rec, np.zeros(nrec, np.int32), 0)
    stf = (a["rtf_uz"] * 1e3, a["rtf_ux"] * 1e3)
    ga = orc.kernel_PSV(sv, 0, lam, mu, mz, rz, rx, grad=True, history=a["history"], stf=stf,
                        src=src, rec=False)
    gb = ref.kernel_PSV(sv, 0, lam, mu, mz, rz, rx, grad=True, history=a["history"], stf=stf,
                        src=src, rec=False)
    for k in ("grad_lam", "grad_mu", "grad_rho", "uz", "ux", "We", "szz"):
        assert np.array_equal(ga[k], gb[k]), k


@ref_only
def test_fwi_matches_reference_library_surface_layout(orc):
    ref = O.reference()
    ref.set_threads(1)
    sv, true, init = helpers.case(fdorder=4, stencil="reference", nshot=2, nt=250, nz=51,
                                  nx=71, npml=8, nrec=12, imaging_sign=1)
    uz, ux = orc.simulate_fwd(sv, *true)
    r1 = orc.simulate_fwi(sv, *init, uz, ux, niter=2)
    r2 = ref.simulate_fwi(sv, *init, uz, ux, niter=2)
    assert r1["rc"] == 0 and r2["rc"] == 0
    for k in ("L2", "step", "lam", "mu", "rho", "grad_lam", "grad_mu", "grad_rho"):
        assert np.array_equal(r1[k], r2[k]), k
