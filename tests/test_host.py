"""Host side of the engine library, no GPU needed: exported symbols, the
FP64 preprocessing (bitwise against the oracle), the step-length control
flow, and argument validation."""
import ctypes as C
import re

import numpy as np
import pytest

import helpers
from fwi_cuda_gb300 import _lib, engine
from fwi_cuda_gb300 import survey as S
from fwi_cuda_gb300._lib import dptr


def header_symbols():
    text = open(helpers.__file__.replace("tests/helpers.py", "include/fwi_psv.h")).read()
    return sorted(set(re.findall(r"^[\w\s\*]*?\b(psv_\w+)\s*\(", text, flags=re.M)))


def test_library_exports_every_declared_symbol():
    lib = _lib.lib()
    names = header_symbols()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert set(names) <= set(_lib.SIGNATURES), set(names) - set(_lib.SIGNATURES)


def test_holberg_cpml_wavelet_bitwise(orc):
    for fd in (2, 4, 6, 8):
        assert np.array_equal(S.holbergcoeff(fd), orc.holbergcoeff(fd))
    for args in [(2.0, 3000.0, 0.001, 1.0, 100.0, 20, 20, 2, 301, 5e-5, 0.5),
                 (2.0, 800.0, 0.001, 1.0, 200.0, 20, 0, 1, 601, 4e-5, 0.1),
                 (3.0, 4500.0, 0.0001, 2.0, 60.0, 0, 40, 4, 401, 1e-4, 1.0)]:
        for a, b in zip(S.cpml_profiles(*args), orc.cpml(*args)):
            assert np.array_equal(a, b)
    assert np.array_equal(S.ricker(4000, 5e-5, 100.0), orc.wavelet(4000, 5e-5, 1.0, 100.0))


def test_checkfd_matches_oracle(orc):
    sv, true, _ = helpers.case()
    lam, mu, rho = true
    out = np.zeros(4)
    rc = _lib.lib().psv_checkfd_ssg_elastic(sv.nz, sv.nx, sv.dz, sv.dt, sv.freq_pml,
                                            sv.npml[1], dptr(rho), dptr(lam), dptr(mu),
                                            dptr(sv.hc), dptr(out))
    rc2, out2 = orc.checkfd(sv, lam, mu, rho)
    assert rc == 0 and rc2 == 0
    assert np.array_equal(out, out2)
    # a time step above the limit is reported
    rc = _lib.lib().psv_checkfd_ssg_elastic(sv.nz, sv.nx, sv.dz, out[0] * 1.01, sv.freq_pml,
                                            sv.npml[1], dptr(rho), dptr(lam), dptr(mu),
                                            dptr(sv.hc), dptr(out))
    assert rc == _lib.PSV_ERR_CFL


def _step_length(est, L2_0, f):
    cb = _lib.TRIAL_FN(lambda a, L, _: (L.__setitem__(0, f(a)), 0)[1])
    e = C.c_double(est)
    n = C.c_int()
    log = np.zeros((64, 2))
    rc = _lib.lib().psv_step_length(C.byref(e), L2_0, C.cast(cb, C.c_void_p), None, C.byref(n),
                                    dptr(log), 64)
    return rc, e.value, n.value, log[:min(n.value, 64)]


@pytest.mark.parametrize("fun,est,L0", [
    (lambda a: (a - 0.037) ** 2, 0.01, 0.037 ** 2),          # grows, brackets, parabola
    (lambda a: (a - 0.001) ** 2 + 1e-9, 0.01, 1e-6 + 1e-9),  # halves first
    (lambda a: -a, 0.01, 0.0),                                # never brackets (4 growths)
    (lambda a: 1.0 + a, 0.01, 0.0),                           # fails after 31 halvings
])
def test_step_length_control_flow_matches_oracle(orc, fun, est, L0):
    rc, step, n, log = _step_length(est, L0, fun)
    rc2, step2, n2, log2 = orc.step_length(est, L0, fun)
    assert (rc == 0) == (rc2 == 0)
    assert n == n2 and np.array_equal(log, log2)
    if rc == 0:
        assert step == step2
    else:
        assert rc == _lib.PSV_ERR_STEP_SEARCH


def test_step_length_stops_at_a_failing_trial():
    # a trial forward that fails (e.g. a device error) ends the search with
    # its status; the estimate is left as it was and the trials done counted
    calls = []

    def trial(a, L, _):
        calls.append(a)
        if len(calls) == 3:
            return _lib.PSV_ERR_CUDA
        L[0] = (a - 0.037) ** 2
        return 0

    cb = _lib.TRIAL_FN(trial)
    e, n = C.c_double(0.01), C.c_int(-1)
    rc = _lib.lib().psv_step_length(C.byref(e), 0.037 ** 2, C.cast(cb, C.c_void_p), None,
                                    C.byref(n), None, 0)
    assert rc == _lib.PSV_ERR_CUDA and n.value == 2 and e.value == 0.01 and len(calls) == 3
    assert _lib.lib().psv_step_length(C.byref(e), 1.0, None, None, None, None, 0) == \
        _lib.PSV_ERR_ARG


def test_step_length_fails_on_a_misfit_that_is_not_a_number(orc):
    # the reference's search would loop for ever (every comparison with NaN
    # is false); the engine and the oracle stop with a failure
    nan = float("nan")
    for L0, fun, trials in ((0.037 ** 2, lambda a: nan, 1), (nan, lambda a: a, 0),
                            (0.037 ** 2, lambda a: (a - 0.037) ** 2 if a < 0.012 else nan, 2)):
        rc, step, n, log = _step_length(0.01, L0, fun)
        assert rc == _lib.PSV_ERR_STEP_SEARCH and n == trials and step == 0.01
        assert b"not a number" in _lib.lib().psv_last_error()
        rc2, _, n2, log2 = orc.step_length(0.01, L0, fun)
        assert rc2 != 0 and n2 == trials
        assert np.array_equal(log, log2, equal_nan=True)


def test_calc_opt_step_matches_oracle(orc):
    rng = np.random.default_rng(0)
    for _ in range(50):
        sl = np.sort(rng.uniform(0, 0.1, 3))
        sl[0] = 0.0
        L2 = rng.uniform(1, 2, 3)
        assert _lib.lib().psv_calc_opt_step(dptr(L2), dptr(sl)) == orc.calc_opt_step(L2, sl)


def _create(sv, **kw):
    keep = []
    g, s = sv.grid_struct(keep), sv.shots_struct(keep)
    o = engine.options(**kw)
    h = C.c_void_p()
    rc = _lib.lib().psv_plan_create(C.byref(g), C.byref(s), C.byref(o), C.byref(h))
    if rc == 0:
        _lib.lib().psv_plan_destroy(h)
    return rc


def test_plan_validation_errors():
    sv, _, _ = helpers.case()
    bad = helpers.case()[0]
    bad.fdorder = 10
    assert _create(bad) == _lib.PSV_ERR_UNSUPPORTED
    bad = helpers.case()[0]
    bad.x_src = np.array([bad.nx + 3], np.int32)
    assert _create(bad) == _lib.PSV_ERR_ARG
    bad = helpers.case()[0]
    bad.isurf = (bad.isurf[0], 0, 5, 0)  # horizontal + vertical surface
    assert _create(bad) == _lib.PSV_ERR_UNSUPPORTED
    bad = helpers.case()[0]
    bad.snap_z2 = bad.nz + 4
    assert _create(bad) == _lib.PSV_ERR_ARG
    assert _create(sv, precision=16) == _lib.PSV_ERR_ARG
    if not _lib.device_available():
        assert _create(sv) == _lib.PSV_ERR_CUDA  # valid survey, no device: no CPU fallback


def _tiny_survey(nz=40, nx=40, nshot=1, nt=4):
    return S.Survey(nt=nt, nz=nz, nx=nx, dt=1e-4, dz=1.0, dx=1.0, npml=(0, 0, 0, 0),
                    nshot=nshot, z_src=np.full(nshot, 5), x_src=np.full(nshot, 5),
                    src_shot_to_fire=np.arange(nshot), stf_z=np.zeros((nshot, nt)),
                    stf_x=np.zeros((nshot, nt))).finalize()


def test_survey_size_limits():
    """Blocks of grid rows and the shots of a batch map to CUDA grid
    dimensions (at most 65535 each): larger surveys are refused before any
    device work; the limits themselves are accepted."""
    no_device = _lib.PSV_ERR_CUDA if not _lib.device_available() else _lib.PSV_OK
    assert _create(_tiny_survey(nz=_lib.PSV_MAX_NZ + 1)) == _lib.PSV_ERR_UNSUPPORTED
    assert b"nz above 65535" in _lib.lib().psv_last_error()
    assert _create(_tiny_survey(nshot=_lib.PSV_MAX_SHOTS + 1)) == _lib.PSV_ERR_UNSUPPORTED
    assert b"nshot above 65535" in _lib.lib().psv_last_error()
    if no_device:
        assert _create(_tiny_survey(nz=_lib.PSV_MAX_NZ)) == no_device
        assert _create(_tiny_survey(nshot=_lib.PSV_MAX_SHOTS)) == no_device


def _header_struct_fields(name):
    """Field names of `typedef struct name {...} name;` in declaration order."""
    text = open(helpers.__file__.replace("tests/helpers.py", "include/fwi_psv.h")).read()
    body = re.search(r"typedef struct %s \{(.*?)\} %s;" % (name, name), text, flags=re.S).group(1)
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    names = []
    for decl in body.split(";"):
        decl = decl.strip()
        if not decl:
            continue
        # "int a, b" / "double hc[7]" / "const double *a_z, *b_z"
        first, *rest = decl.split(",")
        names.append(re.findall(r"(\w+)\s*(?:\[\d+\])?\s*$", first)[0])
        names += [re.findall(r"(\w+)\s*(?:\[\d+\])?\s*$", r)[0] for r in rest]
    return names


@pytest.mark.parametrize("cname,pyclass", [("psv_grid", _lib.PsvGrid), ("psv_shots", _lib.PsvShots),
                                           ("psv_options", _lib.PsvOptions)])
def test_ctypes_structs_match_the_header(cname, pyclass):
    # a field out of order silently hands the library the wrong option
    assert [f[0] for f in pyclass._fields_] == _header_struct_fields(cname)


def test_python_constants_match_the_header():
    text = open(helpers.__file__.replace("tests/helpers.py", "include/fwi_psv.h")).read()
    defs = dict(re.findall(r"#define (PSV_[A-Z0-9_]+) (\d+)(?:LL)?\b", text))
    for name in ("PSV_MAX_NZ", "PSV_MAX_SHOTS", "PSV_MAX_SHOT_ELEMS"):
        assert getattr(_lib, name) == int(defs[name]), name
    for key, name in (("full", "PSV_STORE_FULL"), ("checkpoint", "PSV_STORE_CHECKPOINT"),
                      ("binomial", "PSV_STORE_BINOMIAL")):
        assert _lib.STORAGE[key] == int(defs[name])


def test_options_reach_the_library_in_order():
    o = engine.options(precision=32, kernels="tma", autotune=False, rows_per_thread=8)
    raw = C.string_at(C.addressof(o), C.sizeof(o))
    fields = dict(_lib.PsvOptions._fields_)
    off = {n: getattr(_lib.PsvOptions, n).offset for n in fields}
    as_int = lambda n: int.from_bytes(raw[off[n]:off[n] + 4], "little", signed=True)
    assert as_int("kernel_family") == 2 and as_int("autotune") == 0 and as_int("rows_per_thread") == 8


def test_host_mat_av2_matches_oracle(orc):
    sv, true, _ = helpers.case(nz=41, nx=57)
    lam, mu, rho = (a.copy() for a in true)
    mu[5, 7] = 0.0  # vacuum cells take the reference's special cases
    rho[9, 3] = rho[10, 3] = rho[9, 4] = 0.0
    a = S.mat_av2(lam, mu, rho)
    b = orc.mat_av2(lam, mu, rho)
    for x, y in zip(a[:3], b[:3]):
        assert np.array_equal(x, y)
    assert np.allclose(a[3], b[3], rtol=1e-12)


def test_host_preprocessing_argument_errors():
    # where the reference would index out of range or exit, the ABI returns
    # a status and leaves a message
    L = _lib.lib()
    hc = np.zeros(7)
    for fd, mre in ((3, 1), (14, 1), (0, 1), (4, 5), (4, -1)):
        assert L.psv_holbergcoeff(fd, mre, dptr(hc)) == _lib.PSV_ERR_ARG, (fd, mre)
    assert L.psv_holbergcoeff(12, 4, dptr(hc)) == _lib.PSV_OK
    p = [np.zeros(40) for _ in range(6)]
    args = (2.0, 3000.0, 0.001, 1.0, 100.0)
    assert L.psv_cpml_PSV(*[dptr(a) for a in p], *args, 10, 10, 2, 40, 1e-4, 1.0) == _lib.PSV_OK
    assert L.psv_cpml_PSV(*[dptr(a) for a in p], *args, 38, 0, 2, 40, 1e-4, 1.0) == _lib.PSV_ERR_ARG
    assert b"do not fit" in L.psv_last_error()
    assert L.psv_cpml_PSV(*[dptr(a) for a in p], *args, 0, 38, 2, 40, 1e-4, 1.0) == _lib.PSV_ERR_ARG
    assert L.psv_cpml_PSV(*[dptr(a) for a in p], *args, 1, 1, 2, 0, 1e-4, 1.0) == _lib.PSV_ERR_ARG
    s = np.zeros(10)
    assert L.psv_wavelet(dptr(s), 10, 1e-4, 1.0, 100.0, 0.0, 2) == _lib.PSV_ERR_UNSUPPORTED
    assert L.psv_wavelet(dptr(s), -1, 1e-4, 1.0, 100.0, 0.0, 1) == _lib.PSV_ERR_ARG
    m = np.full((20, 20), 2000.0)
    out = np.zeros(4)
    L.psv_holbergcoeff(4, 1, dptr(hc))
    assert L.psv_checkfd_ssg_elastic(20, 20, 1.0, 1e-5, 1e-2, 11, dptr(m), dptr(m * 1e6),
                                     dptr(m * 1e6), dptr(hc), dptr(out)) == _lib.PSV_ERR_ARG
    assert b"absorbing frame" in L.psv_last_error()
    assert L.psv_checkfd_ssg_elastic(20, 20, 1.0, 1e-5, 1e-2, 5, dptr(m), dptr(m * 1e6),
                                     dptr(m * 1e6), dptr(hc), dptr(out)) == _lib.PSV_OK


def test_every_plan_call_refuses_a_null_plan():
    # the status-returning plan calls give PSV_ERR_ARG for a null handle
    # (never a crash), destroy accepts it, the queries give 0 / NULL
    L = _lib.lib()
    plan_calls = [n for n, (_, a) in _lib.SIGNATURES.items()
                  if a and a[0] is C.c_void_p and n != "psv_misfit_noalloc"]
    assert len(plan_calls) >= 20
    for n in plan_calls:
        res, argt = _lib.SIGNATURES[n]
        args = [None] + [0 if t in (C.c_int, C.c_double) else None for t in argt[1:]]
        got = getattr(L, n)(*args)
        if n in ("psv_plan_destroy", "psv_joint_destroy"):
            assert got == _lib.PSV_OK
        elif res is C.c_int:
            assert got == _lib.PSV_ERR_ARG, n
        else:
            assert not got, n


def test_compute_calls_refuse_null_arguments():
    # checked before any device work: the CPU container gives the same
    # statuses as a GPU machine
    L = _lib.lib()
    assert L.psv_multi_forward(None, 0, None, None) == _lib.PSV_ERR_ARG
    assert L.psv_multi_gradient(None, 0, None) == _lib.PSV_ERR_ARG
    assert L.psv_multi_forward((C.c_void_p * 2)(None, None), 2, None, None) == _lib.PSV_ERR_ARG
    out = C.c_void_p()
    assert L.psv_joint_create(None, 0, 1, 4, C.byref(out)) == _lib.PSV_ERR_ARG
    assert L.psv_joint_create((C.c_void_p * 9)(), 9, 1, 4, C.byref(out)) == _lib.PSV_ERR_ARG
    assert b"1 to 8" in L.psv_last_error()
    assert L.psv_joint_create((C.c_void_p * 2)(None, None), 2, 1, 4, C.byref(out)) == _lib.PSV_ERR_ARG
    assert L.psv_joint_create((C.c_void_p * 1)(None), 1, 1, 4, None) == _lib.PSV_ERR_ARG
    assert not out
    assert L.psv_misfit(None, None, None, None, None, None, 1, 1, 1, 1.0, None) == _lib.PSV_ERR_ARG
    assert L.psv_misfit_noalloc(None, None, None, None, None, None, 1, 1, 1, 1.0, None,
                                None) == _lib.PSV_ERR_ARG
    assert L.psv_simulate_PSV(None, 0, -1, None) == _lib.PSV_ERR_ARG
    assert L.psv_apply_gauss_filter(None, 5, 5, 2) == _lib.PSV_ERR_ARG
    assert L.psv_PCG_PSV(None, None, None, 5, 5) == _lib.PSV_ERR_ARG


def test_misfit_refuses_more_shots_than_a_launch_grid_holds():
    # the shots of the misfit reduction map to gridDim.y: above 65535 the call
    # fails with its own status before any device work, not a launch error
    L = _lib.lib()
    one = np.zeros(1)
    rc = L.psv_misfit(dptr(one), dptr(one), dptr(one), dptr(one), None, None,
                      _lib.PSV_MAX_SHOTS + 1, 1, 1, 1.0, dptr(one))
    assert rc == _lib.PSV_ERR_UNSUPPORTED
    assert b"65535" in L.psv_last_error()
