"""ctypes front-end of the test oracle (test infrastructure only).

Two libraries share one interface:

* ``liboracle_psv.so`` (``oracle/psv_oracle.c``): the FP64 C restatement of
  the reference's CPU path.  Built by ``make -C oracle`` anywhere.
* ``libref_psv.so`` (``oracle/ref_shim.cpp`` + the reference's own sources):
  built by ``make -C oracle ref`` only where the reference checkout exists.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` use this module, always as the checker.

A *case* is any object with the survey attributes of
``fwi_cuda_gb300.survey.Survey`` (grid, CPML profiles, sources, receivers,
snapshot window, taper); :func:`grid_struct` and :func:`shots_struct` turn it
into the C structs.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "liboracle_psv.so")
REF_SO = os.path.join(HERE, "_ref", "libref_psv.so")

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


class OrcGrid(C.Structure):
    _fields_ = [
        ("nt", C.c_int), ("nz", C.c_int), ("nx", C.c_int),
        ("dt", C.c_double), ("dx", C.c_double), ("dz", C.c_double),
        ("surf", C.c_int), ("isurf", C.c_int * 4),
        ("hc", C.c_double * 7), ("fdorder", C.c_int), ("stencil", C.c_int),
        ("pml_z", C.c_int), ("pml_x", C.c_int),
        ("a_z", _dp), ("b_z", _dp), ("K_z", _dp), ("a_half_z", _dp), ("b_half_z", _dp),
        ("K_half_z", _dp),
        ("a_x", _dp), ("b_x", _dp), ("K_x", _dp), ("a_half_x", _dp), ("b_half_x", _dp),
        ("K_half_x", _dp),
        ("snap_z1", C.c_int), ("snap_z2", C.c_int), ("snap_x1", C.c_int), ("snap_x2", C.c_int),
        ("snap_dt", C.c_int), ("snap_dz", C.c_int), ("snap_dx", C.c_int),
        ("grad_sign", C.c_int),
    ]


class OrcShots(C.Structure):
    _fields_ = [
        ("nshot", C.c_int), ("nsrc", C.c_int), ("nrec", C.c_int), ("stf_type", C.c_int),
        ("rtf_type", C.c_int),
        ("z_src", _ip), ("x_src", _ip), ("src_shot_to_fire", _ip),
        ("stf_z", _dp), ("stf_x", _dp),
        ("z_rec", _ip), ("x_rec", _ip),
    ]


def build(ref: bool = False) -> None:
    """Compile the oracle (and the reference library when ``ref``)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    if ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref"], check=True)


def ref_available() -> bool:
    return os.path.exists(REF_SO)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def dptr(a):
    return a.ctypes.data_as(_dp) if a is not None else None


def iptr(a):
    return a.ctypes.data_as(_ip) if a is not None else None


class Lib:
    """One of the two libraries; ``prefix`` is ``orc_`` or ``ref_``."""

    def __init__(self, path: str, prefix: str):
        if not os.path.exists(path):
            raise FileNotFoundError(f"{path} not built (run make -C oracle{' ref' if prefix == 'ref_' else ''})")
        self.lib = C.CDLL(path)
        self.p = prefix
        self.keep = []  # arrays referenced by the C structs
        f = self.fn
        f("set_threads").argtypes = [C.c_int]
        f("holbergcoeff").argtypes = [C.c_int, C.c_int, _dp]
        f("cpml_PSV").argtypes = [_dp] * 6 + [C.c_double] * 5 + [C.c_int] * 4 + [C.c_double] * 2
        f("wavelet").argtypes = [_dp, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int]
        f("mat_av2").argtypes = [_dp] * 7 + [C.c_int, C.c_int]
        f("adjsrc2").argtypes = [_dp] * 6 + [C.c_double, C.c_int, C.c_int]
        f("adjsrc2").restype = C.c_double
        f("calc_opt_step").argtypes = [_dp, _dp]
        f("calc_opt_step").restype = C.c_double
        f("update_mat2").argtypes = [_dp] * 3 + [C.c_double] * 3 + [C.c_int] * 2
        kargs = ([C.POINTER(OrcGrid), C.c_int] + [_dp] * 13 + [C.c_int] + [_dp] * 3
                 + [C.c_int, C.c_int, _dp, _dp, _ip, _ip, _ip]
                 + [C.c_int, C.c_int, _dp, _dp, _ip, _ip]
                 + [C.c_int] + [_dp] * 5)
        f("kernel_PSV").argtypes = kargs
        fwi = [C.POINTER(OrcGrid), C.POINTER(OrcShots), _dp, _dp, _dp, _dp, _dp, _ip,
               C.c_int, C.c_double, _dp, _dp, _dp, _dp, _dp]
        if prefix == "orc_":
            fwi += [_ip, _dp]
            f("taper2").argtypes = [_dp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _ip]
            f("interpol_grad2").argtypes = [_dp, _dp] + [C.c_int] * 7
            f("energy_weights2").argtypes = [_dp, _dp] + [C.c_int] * 5 + [_dp]
            f("scale_grad_E2").argtypes = [_dp, _dp, C.c_double, _dp] + [C.c_int] * 5
            f("shot_gradient").argtypes = ([C.POINTER(OrcGrid), C.POINTER(OrcShots), C.c_int]
                                           + [_dp] * 12)
            f("shot_gradient").restype = C.c_double
            f("simulate_fwd").argtypes = [C.POINTER(OrcGrid), C.POINTER(OrcShots)] + [_dp] * 5
            f("checkfd_ssg_elastic").argtypes = ([C.c_int, C.c_int, C.c_double, C.c_double,
                                                  C.c_double, C.c_int] + [_dp] * 5)
            f("checkfd_ssg_elastic").restype = C.c_int
            f("step_length_cb").argtypes = [_dp, C.c_double, C.c_void_p, C.c_void_p, _ip, _dp]
            f("step_length_cb").restype = C.c_int
            f("gauss_filter_kernel").argtypes = [C.c_int, _dp]
            f("gauss_filter_kernel").restype = C.c_int
            f("apply_gauss_filter").argtypes = [_dp, C.c_int, C.c_int, _dp, C.c_int]
            f("PCG_PSV").argtypes = [_dp, _dp, _dp, C.c_int, C.c_int]
        else:
            f("taper2").argtypes = [_dp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _ip]
            f("interpol_grad2").argtypes = [_dp, _dp] + [C.c_int] * 8
            f("energy_weights2").argtypes = [_dp, _dp] + [C.c_int] * 6
            f("scale_grad_E2").argtypes = [_dp, _dp, C.c_double, _dp] + [C.c_int] * 6
            f("simulate_PSV_in_dir").argtypes = [C.c_char_p]
            f("simulate_PSV_in_dir").restype = C.c_int
        f("simulate_fwi").argtypes = fwi
        f("simulate_fwi").restype = C.c_int

    def fn(self, name):
        return getattr(self.lib, self.p + name)

    # ---- host preprocessing ----
    def set_threads(self, n: int) -> None:
        self.fn("set_threads")(int(n))

    def holbergcoeff(self, fdorder: int, maxrelerror: int = 1) -> np.ndarray:
        hc = np.zeros(7)
        self.fn("holbergcoeff")(fdorder, maxrelerror, dptr(hc))
        return hc

    def cpml(self, npower, damp, rcoef, kmax, freq, n1, n2, fpad, nh, dt, dh):
        arrs = [np.zeros(nh) for _ in range(6)]
        self.fn("cpml_PSV")(*[dptr(a) for a in arrs], npower, damp, rcoef, kmax, freq,
                            n1, n2, fpad, nh, dt, dh)
        return arrs  # a, b, K, a_half, b_half, K_half

    def wavelet(self, nt, dt, amp, fc, ts=0.0, shape=1):
        s = np.zeros(nt)
        self.fn("wavelet")(dptr(s), nt, dt, amp, fc, ts, shape)
        return s

    # ---- kernel library ----
    def mat_av2(self, lam, mu, rho):
        lam, mu, rho = _f64(lam), _f64(mu), _f64(rho)
        nz, nx = lam.shape
        out = [np.zeros((nz, nx)) for _ in range(3)]
        Cs = np.zeros(3)
        self.fn("mat_av2")(dptr(lam), dptr(mu), dptr(rho), *[dptr(o) for o in out], dptr(Cs), nz, nx)
        return out[0], out[1], out[2], Cs

    def adjsrc2(self, mod_uz, mod_ux, true_uz, true_ux, dt):
        mod_uz, mod_ux = _f64(mod_uz).copy(), _f64(mod_ux).copy()
        true_uz, true_ux = _f64(true_uz), _f64(true_ux)
        nseis, nt = mod_uz.shape
        L2 = self.fn("adjsrc2")(dptr(mod_uz), dptr(mod_ux), dptr(true_uz), dptr(true_ux),
                                dptr(mod_uz), dptr(mod_ux), dt, nseis, nt)
        return L2, mod_uz, mod_ux

    def calc_opt_step(self, L2, sl):
        return self.fn("calc_opt_step")(dptr(_f64(L2)), dptr(_f64(sl)))

    def update_mat2(self, mat_old, grad, mat_max, mat_min, step):
        mat_old, grad = _f64(mat_old), _f64(grad)
        nz, nx = mat_old.shape
        out = np.zeros_like(mat_old)
        self.fn("update_mat2")(dptr(out), dptr(mat_old), dptr(grad), mat_max, mat_min, step, nz, nx)
        return out

    def taper2(self, A, snap, taper8):
        A = _f64(A).copy()
        nz, nx = A.shape
        z1, z2, x1, x2 = snap
        self.fn("taper2")(dptr(A), nz, nx, z1, z2, x1, x2, iptr(_i32(taper8)))
        return A

    def interpol_grad2(self, grad, grad_shot, snap, sdz, sdx):
        grad = _f64(grad).copy()
        gs = _f64(grad_shot)
        nz, nx = grad.shape
        z1, z2, x1, x2 = snap
        if self.p == "orc_":
            self.fn("interpol_grad2")(dptr(grad), dptr(gs), nx, z1, z2, x1, x2, sdz, sdx)
        else:
            self.fn("interpol_grad2")(dptr(grad), dptr(gs), nz, nx, z1, z2, x1, x2, sdz, sdx)
        return grad

    def energy_weights2(self, We, We_adj, snap):
        We = _f64(We).copy()
        Wa = _f64(We_adj).copy()
        nz, nx = We.shape
        z1, z2, x1, x2 = snap
        if self.p == "orc_":
            self.fn("energy_weights2")(dptr(We), dptr(Wa), nx, z1, z2, x1, x2, None)
        else:
            self.fn("energy_weights2")(dptr(We), dptr(Wa), nz, nx, z1, z2, x1, x2)
        return We

    def scale_grad_E2(self, grad, grad_shot, mat_av, We, snap):
        grad = _f64(grad).copy()
        gs, W = _f64(grad_shot), _f64(We)
        nz, nx = grad.shape
        z1, z2, x1, x2 = snap
        if self.p == "orc_":
            self.fn("scale_grad_E2")(dptr(grad), dptr(gs), mat_av, dptr(W), nx, z1, z2, x1, x2)
        else:
            self.fn("scale_grad_E2")(dptr(grad), dptr(gs), mat_av, dptr(W), nz, nx, z1, z2, x1, x2)
        return grad

    # ---- time loop ----
    def kernel_PSV(self, case, ishot, lam, mu, mu_zx, rho_zp, rho_xp, *, grad=False,
                   accu=False, history=None, stf=None, src=None, rec=True):
        """One call of kernel_PSV.  Returns a dict of every output array.

        ``stf``/``src`` override the case's sources (used for the adjoint:
        residuals fired at the receivers); ``history`` supplies the forward
        snapshot arrays for ``grad`` mode.
        """
        g = grid_struct(case, self.keep)
        nz, nx, nt = case.nz, case.nx, case.nt
        f = {k: np.zeros((nz, nx)) for k in ("vz", "vx", "uz", "ux", "szz", "szx", "sxx", "We")}
        snt, snz, snx = case.snap_dims()
        gr = {k: np.zeros((snz, snx)) for k in ("grad_lam", "grad_mu", "grad_rho")}
        if history is None:
            history = {k: np.zeros((snt, snz, snx) if accu else (1,))
                       for k in ("vz", "vx", "szz", "szx", "sxx")}
        if stf is None:
            stf_z, stf_x = _f64(case.stf_z), _f64(case.stf_x)
            z_src, x_src, fire = _i32(case.z_src), _i32(case.x_src), _i32(case.src_shot_to_fire)
            stf_type = case.stf_type
        else:
            stf_z, stf_x = _f64(stf[0]), _f64(stf[1])
            z_src, x_src, fire, stf_type = (_i32(src[0]), _i32(src[1]), _i32(src[2]), src[3])
        nsrc = stf_z.shape[0]
        nrec = case.nrec if rec else 0
        rtf_uz = np.zeros((max(case.nrec, 1), nt))
        rtf_ux = np.zeros((max(case.nrec, 1), nt))
        args = [C.byref(g), ishot] + [dptr(f[k]) for k in ("vz", "vx", "uz", "ux", "szz", "szx", "sxx", "We")]
        args += [dptr(_f64(a)) for a in (lam, mu, mu_zx, rho_zp, rho_xp)]
        args += [int(grad)] + [dptr(gr[k]) for k in ("grad_lam", "grad_mu", "grad_rho")]
        args += [nsrc, stf_type, dptr(stf_z), dptr(stf_x), iptr(z_src), iptr(x_src), iptr(fire)]
        args += [nrec, case.rtf_type, dptr(rtf_uz), dptr(rtf_ux), iptr(_i32(case.z_rec)),
                 iptr(_i32(case.x_rec))]
        args += [int(accu)] + [dptr(history[k]) for k in ("vz", "vx", "szz", "szx", "sxx")]
        self.fn("kernel_PSV")(*args)
        out = dict(f)
        out.update(gr)
        out["rtf_uz"], out["rtf_ux"] = rtf_uz, rtf_ux
        out["history"] = history
        return out

    def gauss_filter_kernel(self, hfs):
        k = np.zeros((2 * abs(hfs) + 1, 2 * abs(hfs) + 1))
        if self.fn("gauss_filter_kernel")(int(hfs), dptr(k)) != 0:
            raise ValueError("hfs must be at least 2")
        return k

    def apply_gauss_filter(self, mat, hfs):
        """Filtered copy of mat (orc_ only)."""
        out = _f64(mat).copy()
        k = self.gauss_filter_kernel(hfs)
        self.fn("apply_gauss_filter")(dptr(out), out.shape[0], out.shape[1], dptr(k), int(hfs))
        return out

    def PCG_PSV(self, dir_, old, grad):
        """One Fletcher-Reeves step; updates the three arrays in place (orc_ only)."""
        for a in (dir_, old, grad):
            assert a.dtype == np.float64 and a.flags.c_contiguous
        self.fn("PCG_PSV")(dptr(dir_), dptr(old), dptr(grad), grad.shape[0], grad.shape[1])

    def shot_gradient(self, case, ishot, lam, mu, rho, true_uz, true_ux):
        """Forward + residual + adjoint of one shot (orc_ only)."""
        g = grid_struct(case, self.keep)
        s = shots_struct(case, self.keep)
        snt, snz, snx = case.snap_dims()
        out = {k: np.zeros((snz, snx)) for k in ("grad_lam", "grad_mu", "grad_rho")}
        out["We"] = np.zeros((case.nz, case.nx))
        out["We_adj"] = np.zeros((case.nz, case.nx))
        out["rtf_uz"] = np.zeros((case.nrec, case.nt))
        out["rtf_ux"] = np.zeros((case.nrec, case.nt))
        L2 = self.fn("shot_gradient")(
            C.byref(g), C.byref(s), ishot, dptr(_f64(lam)), dptr(_f64(mu)), dptr(_f64(rho)),
            dptr(_f64(true_uz)), dptr(_f64(true_ux)), dptr(out["grad_lam"]), dptr(out["grad_mu"]),
            dptr(out["grad_rho"]), dptr(out["We"]), dptr(out["We_adj"]), dptr(out["rtf_uz"]),
            dptr(out["rtf_ux"]))
        out["L2"] = L2
        return out

    def simulate_fwd(self, case, lam, mu, rho):
        g = grid_struct(case, self.keep)
        s = shots_struct(case, self.keep)
        uz = np.zeros((case.nshot, case.nrec, case.nt))
        ux = np.zeros_like(uz)
        self.fn("simulate_fwd")(C.byref(g), C.byref(s), dptr(_f64(lam)), dptr(_f64(mu)),
                                dptr(_f64(rho)), dptr(uz), dptr(ux))
        return uz, ux

    def simulate_fwi(self, case, lam, mu, rho, true_uz, true_ux, niter, step0=0.01, grads=None):
        g = grid_struct(case, self.keep)
        s = shots_struct(case, self.keep)
        lam, mu, rho = _f64(lam).copy(), _f64(mu).copy(), _f64(rho).copy()
        if grads is None:
            grads = [np.zeros((case.nz, case.nx)) for _ in range(3)]
        grads = [_f64(x).copy() for x in grads]
        L2 = np.zeros(niter)
        step = np.zeros(niter)
        args = [C.byref(g), C.byref(s), dptr(lam), dptr(mu), dptr(rho), dptr(_f64(true_uz)),
                dptr(_f64(true_ux)), iptr(_i32(case.taper)), niter, step0,
                dptr(grads[0]), dptr(grads[1]), dptr(grads[2]), dptr(L2), dptr(step)]
        trials = np.zeros(niter, dtype=np.int32)
        tlog = np.zeros((niter, 64, 2))
        if self.p == "orc_":
            args += [iptr(trials), dptr(tlog)]
        rc = self.fn("simulate_fwi")(*args)
        return dict(rc=rc, lam=lam, mu=mu, rho=rho, grad_lam=grads[0], grad_mu=grads[1],
                    grad_rho=grads[2], L2=L2, step=step, trials=trials, trial_log=tlog)

    def step_length(self, est, L2_0, fn):
        """step_length_PSV's control flow with L2 = fn(step) (orc_ only)."""
        cb = C.CFUNCTYPE(C.c_double, C.c_double, C.c_void_p)(lambda a, _: float(fn(a)))
        e = C.c_double(est)
        n = C.c_int()
        tlog = np.zeros((64, 2))
        rc = self.fn("step_length_cb")(C.byref(e), L2_0, C.cast(cb, C.c_void_p), None, C.byref(n),
                                       dptr(tlog))
        return rc, e.value, n.value, tlog[:min(n.value, 64)].copy()

    def checkfd(self, case, lam, mu, rho):
        out = np.zeros(4)
        rc = self.fn("checkfd_ssg_elastic")(case.nz, case.nx, case.dz, case.dt, case.freq_pml,
                                            int(case.npml[1]), dptr(_f64(rho)), dptr(_f64(lam)),
                                            dptr(_f64(mu)), dptr(_f64(case.hc)), dptr(out))
        return rc, out


def grid_struct(case, keep: list) -> OrcGrid:
    g = OrcGrid()
    g.nt, g.nz, g.nx = case.nt, case.nz, case.nx
    g.dt, g.dx, g.dz = case.dt, case.dx, case.dz
    g.surf = int(case.surf)
    for i in range(4):
        g.isurf[i] = int(case.isurf[i])
    for i in range(7):
        g.hc[i] = float(case.hc[i])
    g.fdorder = case.fdorder
    g.stencil = 1 if case.stencil == "holberg" else 0
    g.pml_z, g.pml_x = int(case.pml_z), int(case.pml_x)
    for name in ("a_z", "b_z", "K_z", "a_half_z", "b_half_z", "K_half_z",
                 "a_x", "b_x", "K_x", "a_half_x", "b_half_x", "K_half_x"):
        arr = _f64(getattr(case, name))
        keep.append(arr)
        setattr(g, name, dptr(arr))
    (g.snap_z1, g.snap_z2, g.snap_x1, g.snap_x2, g.snap_dt, g.snap_dz, g.snap_dx) = (
        case.snap_z1, case.snap_z2, case.snap_x1, case.snap_x2, case.snap_dt, case.snap_dz,
        case.snap_dx)
    g.grad_sign = int(getattr(case, "imaging_sign", -1))
    return g


def shots_struct(case, keep: list) -> OrcShots:
    s = OrcShots()
    s.nshot, s.nsrc, s.nrec = case.nshot, case.nsrc, case.nrec
    s.stf_type, s.rtf_type = case.stf_type, case.rtf_type
    arrs = dict(z_src=_i32(case.z_src), x_src=_i32(case.x_src),
                src_shot_to_fire=_i32(case.src_shot_to_fire), z_rec=_i32(case.z_rec),
                x_rec=_i32(case.x_rec), stf_z=_f64(case.stf_z), stf_x=_f64(case.stf_x))
    keep.extend(arrs.values())
    for k, v in arrs.items():
        setattr(s, k, iptr(v) if v.dtype == np.int32 else dptr(v))
    return s


_cache = {}


def oracle() -> Lib:
    """The FP64 restatement (builds it on first use)."""
    if "orc" not in _cache:
        if not os.path.exists(ORACLE_SO):
            build()
        _cache["orc"] = Lib(ORACLE_SO, "orc_")
    return _cache["orc"]


def reference() -> Lib:
    """The reference's own CPU code (only where it has been built)."""
    if "ref" not in _cache:
        _cache["ref"] = Lib(REF_SO, "ref_")
    return _cache["ref"]
