"""Python front-end of the GB300 engine (thin wrapper over the C ABI).

* :class:`Plan` -- a device-resident survey: forward modelling, FWI gradient,
  FWI iteration with the reference's step-length search
  (``simulate_fwd_PSV`` / ``simulate_fwi_PSV``, include/cpu/n_simulate_PSV.hpp).
* :func:`kernel_PSV` -- the reference's per-shot time loop (``kernel_PSV``,
  include/cpu/n_kernel_PSV.hpp:8-43) with the same argument meaning.
* :func:`simulate_PSV` -- the reference's whole program on the GPU
  (``simulate_PSV``, include/h_simulate_PSV.hpp:23).

Every call goes to ``libfwi_psv.so``; nothing here computes on the CPU.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import PsvOptions, check, dptr, f64, i32, iptr


FAMILIES = {1: "direct", 2: "tma", 3: "vec4", 4: "fused", 5: "march"}


def options(precision=32, storage="auto", hbm_budget_gb=180.0, max_batch=0, use_graphs=True,
            block=(0, 0), checkpoint_interval=0, rows_per_thread=0, autotune=True,
            kernels="any", checkpoint_slots=0, smooth_hfs=0, pcg=False, chains=0,
            adjoint="reference") -> PsvOptions:
    o = PsvOptions()
    _lib.lib().psv_options_default(C.byref(o))
    o.precision = int(precision)
    o.storage = _lib.STORAGE[storage]
    o.hbm_budget_gb = float(hbm_budget_gb)
    o.max_batch = int(max_batch)
    o.use_graphs = int(bool(use_graphs))
    o.block_x, o.block_y = int(block[0]), int(block[1])
    o.checkpoint_interval = int(checkpoint_interval)
    o.checkpoint_slots = int(checkpoint_slots)
    o.smooth_hfs = int(smooth_hfs)
    o.pcg = int(bool(pcg))
    o.chains = int(chains)
    o.rows_per_thread = int(rows_per_thread)
    o.autotune = int(bool(autotune))
    o.kernel_family = {"any": 0, "direct": 1, "tma": 2, "vec4": 3, "fused": 4, "march": 5}[kernels]
    o.adjoint = {"reference": 0, "exact": 1}[adjoint]
    return o


def gauss_filter_kernel(hfs):
    """gauss_filter_kernel: the (2 hfs + 1)^2 smoothing weights (host only)."""
    k = np.zeros((2 * abs(hfs) + 1, 2 * abs(hfs) + 1))
    check(_lib.lib().psv_gauss_filter_kernel(int(hfs), dptr(k)))
    return k


def apply_gauss_filter(mat, hfs):
    """apply_gauss_filter: a smoothed copy of the [nz][nx] array."""
    out = f64(mat).copy()
    check(_lib.lib().psv_apply_gauss_filter(dptr(out), out.shape[0], out.shape[1], int(hfs)))
    return out


def PCG_PSV(dir_, old, grad):
    """PCG_PSV: one Fletcher-Reeves step, the three float64 arrays updated in place."""
    for a in (dir_, old, grad):
        if a.dtype != np.float64 or not a.flags.c_contiguous:
            raise TypeError("PCG_PSV needs C-contiguous float64 arrays")
    check(_lib.lib().psv_PCG_PSV(dptr(dir_), dptr(old), dptr(grad), grad.shape[0], grad.shape[1]))


def checkpoint_schedule(nseg, slots):
    """Griewank's binomial schedule for nseg segments and `slots` state slots
    (host only): (actions, advances), actions an (n, 3) array of
    (op, segment, slot) -- op 1 forward-pass save, 2 restore, 3 advance,
    4 save the working state, 5 recompute + reverse a segment."""
    n, adv = C.c_int(), C.c_longlong()
    check(_lib.lib().psv_checkpoint_schedule(int(nseg), int(slots), None, 0, C.byref(n), C.byref(adv)))
    a = np.zeros((max(n.value, 1), 3), np.int32)
    check(_lib.lib().psv_checkpoint_schedule(int(nseg), int(slots), iptr(a), n.value, C.byref(n),
                                             C.byref(adv)))
    return a[:n.value], adv.value


class Plan:
    def __init__(self, survey, **opts):
        self.sv = survey
        self._keep = []
        g = survey.grid_struct(self._keep)
        s = survey.shots_struct(self._keep)
        o = options(**opts)
        h = C.c_void_p()
        check(_lib.lib().psv_plan_create(C.byref(g), C.byref(s), C.byref(o), C.byref(h)))
        self.h = h
        self.n = survey.nz * survey.nx
        self.adjoint = opts.get("adjoint", "reference")

    def close(self):
        if getattr(self, "h", None):
            _lib.lib().psv_plan_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def device_bytes(self) -> int:
        return int(_lib.lib().psv_plan_device_bytes(self.h))

    def set_model(self, lam, mu, rho):
        self._model = [f64(lam), f64(mu), f64(rho)]
        check(_lib.lib().psv_plan_set_model(self.h, *[dptr(a) for a in self._model]))

    def get_model(self):
        out = [np.zeros((self.sv.nz, self.sv.nx)) for _ in range(3)]
        check(_lib.lib().psv_plan_get_model(self.h, *[dptr(a) for a in out]))
        return out

    def set_observed(self, uz, ux):
        self._obs = [f64(uz), f64(ux)]
        check(_lib.lib().psv_plan_set_observed(self.h, dptr(self._obs[0]), dptr(self._obs[1])))

    def forward(self):
        sv = self.sv
        uz = np.zeros((sv.nshot, sv.nrec, sv.nt))
        ux = np.zeros_like(uz)
        check(_lib.lib().psv_forward(self.h, dptr(uz), dptr(ux)))
        return uz, ux

    def gradient(self, fetch=True):
        L2 = C.c_double()
        if fetch:
            g = [np.zeros((self.sv.nz, self.sv.nx)) for _ in range(3)]
            check(_lib.lib().psv_gradient(self.h, C.byref(L2), *[dptr(a) for a in g]))
            return L2.value, g
        check(_lib.lib().psv_gradient(self.h, C.byref(L2), None, None, None))
        return L2.value, None

    def reset_gradient(self):
        check(_lib.lib().psv_reset_gradient(self.h))

    def get_gradient(self):
        g = [np.zeros((self.sv.nz, self.sv.nx)) for _ in range(3)]
        check(_lib.lib().psv_get_gradient(self.h, *[dptr(a) for a in g]))
        return g

    def set_gradient(self, gl, gm, gr):
        arrs = [f64(gl), f64(gm), f64(gr)]
        check(_lib.lib().psv_set_gradient(self.h, *[dptr(a) for a in arrs]))

    def shot_gradient(self, ishot):
        sv = self.sv
        snt, snz, snx = sv.snap_dims()
        out = {k: np.zeros((snz, snx)) for k in ("grad_lam", "grad_mu", "grad_rho")}
        out["We"] = np.zeros((sv.nz, sv.nx))
        out["We_adj"] = np.zeros((sv.nz, sv.nx))
        out["rtf_uz"] = np.zeros((sv.nrec, sv.nt))
        out["rtf_ux"] = np.zeros((sv.nrec, sv.nt))
        L2 = C.c_double()
        check(_lib.lib().psv_get_shot_gradient(
            self.h, ishot, dptr(out["grad_lam"]), dptr(out["grad_mu"]), dptr(out["grad_rho"]),
            dptr(out["We"]), dptr(out["We_adj"]), dptr(out["rtf_uz"]), dptr(out["rtf_ux"]),
            C.byref(L2)))
        out["L2"] = L2.value
        return out

    def fwi_iteration(self, step, max_trials=64):
        st = C.c_double(step)
        L2 = C.c_double()
        nt = C.c_int()
        tlog = np.zeros((max_trials, 2))
        check(_lib.lib().psv_fwi_iteration(self.h, C.byref(st), C.byref(L2), C.byref(nt),
                                           dptr(tlog), max_trials))
        n = nt.value
        return dict(step=st.value, L2=L2.value, ntrials=n, trials=tlog[:min(n, max_trials)].copy())

    # pieces of fwi_iteration, for distributed drivers
    def save_model(self):
        check(_lib.lib().psv_save_model(self.h))

    def taper_gradient(self):
        check(_lib.lib().psv_taper_gradient(self.h))

    def pcg_gradient(self):
        """PCG_PSV on the plan's global gradients (direction state kept by the plan)."""
        check(_lib.lib().psv_pcg_gradient(self.h))

    def trial_misfit(self, step):
        L2 = C.c_double()
        check(_lib.lib().psv_trial_misfit(self.h, float(step), C.byref(L2)))
        return L2.value

    def update_model(self, step):
        check(_lib.lib().psv_update_model(self.h, float(step)))

    @property
    def stream(self) -> int:
        """cudaStream_t of the plan (for torch.cuda.ExternalStream)."""
        return int(_lib.lib().psv_plan_stream(self.h) or 0)

    @property
    def kernel_launches(self) -> int:
        return int(_lib.lib().psv_plan_kernel_launches(self.h))

    def autotune(self, nsteps=24):
        """Pick the fastest time-step kernels; returns (family, rows_per_thread,
        block_y) with family "direct" or "tma"."""
        f, r, b = C.c_int(), C.c_int(), C.c_int()
        check(_lib.lib().psv_plan_autotune(self.h, int(nsteps), C.byref(f), C.byref(r), C.byref(b)))
        return FAMILIES[f.value], r.value, b.value

    @property
    def shape(self):
        """(family, rows_per_thread, block_y) of the kernels the plan launches now."""
        f, r, b = C.c_int(), C.c_int(), C.c_int()
        check(_lib.lib().psv_plan_shape(self.h, C.byref(f), C.byref(r), C.byref(b)))
        return FAMILIES[f.value], r.value, b.value

    @property
    def chains(self):
        """Shot groups (streams) the time loops run in."""
        c = C.c_int()
        check(_lib.lib().psv_plan_chains(self.h, C.byref(c)))
        return c.value

    @property
    def storage(self):
        """(storage, segment_steps, slots, advances): "full", "checkpoint" or
        "binomial"; steps per checkpoint segment and state slots per shot;
        segment advances the adjoint pass recomputes beyond one
        recomputation of every segment."""
        k, K, S, a = C.c_int(), C.c_int(), C.c_int(), C.c_longlong()
        check(_lib.lib().psv_plan_storage(self.h, C.byref(k), C.byref(K), C.byref(S), C.byref(a)))
        name = {v: n for n, v in _lib.STORAGE.items()}[k.value]
        return name, K.value, S.value, a.value

    def profile_kernels(self, nsteps=100):
        ms = np.zeros(6)
        check(_lib.lib().psv_profile_kernels(self.h, int(nsteps), dptr(ms)))
        return dict(stress_fwd=ms[0], velocity_fwd=ms[1], stress_adj=ms[3], velocity_adj=ms[4])

    def timing(self):
        t = np.zeros(3)
        check(_lib.lib().psv_last_timing(self.h, dptr(t)))
        return dict(forward_ms=t[0], adjoint_ms=t[1], other_ms=t[2])


def misfit(mod_uz, mod_ux, true_uz, true_ux, dt, residual=True):
    """adjsrc2 for [nshot][nrec][nt] traces on the GPU: (L2 per shot, res_z, res_x)."""
    m = [f64(a) for a in (mod_uz, mod_ux, true_uz, true_ux)]
    if m[0].ndim == 2:
        m = [a[None] for a in m]
    nshot, nrec, nt = m[0].shape
    L2 = np.zeros(nshot)
    rz = np.zeros_like(m[0]) if residual else None
    rx = np.zeros_like(m[0]) if residual else None
    check(_lib.lib().psv_misfit(*[dptr(a) for a in m], dptr(rz), dptr(rx), nshot, nrec, nt, dt,
                                dptr(L2)))
    return L2, rz, rx


def kernel_PSV(ishot, nt, nz, nx, dt, dx, dz, surf, isurf, hc, fdorder, lam, mu, mu_zx, rho_zp,
               rho_xp, grad, pml_z, cpml_z, pml_x, cpml_x, nsrc, stf_type, stf_z, stf_x, z_src,
               x_src, src_shot_to_fire, nrec, rtf_type, z_rec, x_rec, accu, snap, history=None,
               stencil="reference", precision=32):
    """One shot, nt steps, forward (grad=False) or time-reversed adjoint
    (grad=True), arguments as the reference's kernel_PSV.  ``cpml_z`` /
    ``cpml_x`` are the six profiles (a, b, K, a_half, b_half, K_half);
    ``snap`` = (snap_z1, snap_z2, snap_x1, snap_x2, snap_dt, snap_dz, snap_dx);
    ``history`` = the forward snapshots {vz, vx, szz, szx, sxx} (adjoint).
    Returns every array the reference leaves filled."""
    n = (nz, nx)
    f = {k: np.zeros(n) for k in ("vz", "vx", "uz", "ux", "szz", "szx", "sxx", "We")}
    mem = {k: np.zeros(n) for k in ("mem_vz_z", "mem_vx_z", "mem_szz_z", "mem_szx_z",
                                    "mem_vz_x", "mem_vx_x", "mem_szx_x", "mem_sxx_x")}
    z1, z2, x1, x2, sdt, sdz, sdx = snap
    snt, snz, snx = 1 + (nt - 1) // sdt, 1 + (z2 - z1) // sdz, 1 + (x2 - x1) // sdx
    gr = {k: np.zeros((snz, snx)) for k in ("grad_lam", "grad_mu", "grad_rho")}
    hist = {}
    for k in ("vz", "vx", "szz", "szx", "sxx"):
        if history is not None:
            hist[k] = f64(history[k]).copy()
        else:
            hist[k] = np.zeros((snt, snz, snx) if accu else (1,))
    rtf_uz = np.zeros((max(nrec, 1), nt))
    rtf_ux = np.zeros_like(rtf_uz)
    keep = [f64(a) for a in (lam, mu, mu_zx, rho_zp, rho_xp)]
    cz = [f64(a) for a in cpml_z] if pml_z else [np.ones(nz)] * 6
    cx = [f64(a) for a in cpml_x] if pml_x else [np.ones(nx)] * 6
    src = [f64(stf_z), f64(stf_x), i32(z_src), i32(x_src), i32(src_shot_to_fire)]
    rec = [i32(z_rec), i32(x_rec)]
    isurf_a = i32(isurf if isurf is not None else [0, 0, 0, 0])
    hc_a = f64(hc)
    args = [ishot, nt, nz, nx, dt, dx, dz, int(surf), iptr(isurf_a), dptr(hc_a), fdorder]
    args += [dptr(f[k]) for k in ("vz", "vx", "uz", "ux", "szz", "szx", "sxx", "We")]
    args += [None] * 4
    args += [dptr(a) for a in keep]
    args += [int(grad)] + [dptr(gr[k]) for k in ("grad_lam", "grad_mu", "grad_rho")]
    args += [int(pml_z)] + [dptr(a) for a in cz] + [int(pml_x)] + [dptr(a) for a in cx]
    args += [dptr(mem[k]) for k in mem]
    args += [nsrc, stf_type, dptr(src[0]), dptr(src[1]), iptr(src[2]), iptr(src[3]), iptr(src[4])]
    args += [nrec, rtf_type, dptr(rtf_uz), dptr(rtf_ux), iptr(rec[0]), iptr(rec[1])]
    args += [int(accu)] + [dptr(hist[k]) for k in ("vz", "vx", "szz", "szx", "sxx")]
    args += [z1, z2, x1, x2, sdt, sdz, sdx, _lib.STENCIL[stencil], int(precision)]
    check(_lib.lib().psv_kernel_PSV(*args))
    out = dict(f)
    out.update(mem)
    out.update(gr)
    out["rtf_uz"], out["rtf_ux"] = rtf_uz[:nrec], rtf_ux[:nrec]
    out["history"] = hist
    return out


def simulate_PSV(workdir: str, max_iter: int = 0, imaging_sign: int = -1, **opts) -> None:
    """Run the reference's program (inputs under workdir/bin, workdir/io) on the GPU."""
    o = options(**opts)
    check(_lib.lib().psv_simulate_PSV(workdir.encode(), int(max_iter), int(imaging_sign),
                                      C.byref(o)))


def multi_forward(plans):
    """psv_multi_forward: forward modelling of several surveys (one Plan each,
    uneven sizes allowed) concurrently; returns [(uz, ux)] per plan."""
    n = len(plans)
    hs = (C.c_void_p * n)(*[p.h for p in plans])
    out = [(np.zeros((p.sv.nshot, p.sv.nrec, p.sv.nt)), np.zeros((p.sv.nshot, p.sv.nrec, p.sv.nt)))
           for p in plans]
    uz = (_lib._dp * n)(*[dptr(o[0]) for o in out])
    ux = (_lib._dp * n)(*[dptr(o[1]) for o in out])
    check(_lib.lib().psv_multi_forward(hs, n, uz, ux))
    return out


class Joint:
    """psv_joint_*: forward modelling or FWI gradients of up to 8 surveys
    (one Plan each, one precision; batch b of every plan at once) in one stress and
    one velocity launch per time step; grid sizes, stencil orders, shot and
    step counts may differ.  The plans run the direct kernel family with the joint tile
    shape (rows_per_thread x 32 x block_y threads; rows_per_thread 0: chosen
    by timing the first steps on the first forward)."""

    def __init__(self, plans, rows_per_thread=0, block_y=4):
        self.plans = list(plans)
        n = len(self.plans)
        self._hs = (C.c_void_p * n)(*[p.h for p in self.plans])
        self.h = C.c_void_p()
        check(_lib.lib().psv_joint_create(self._hs, n, int(rows_per_thread), int(block_y),
                                          C.byref(self.h)))
        self.ms = 0.0

    def forward(self, fetch=True):
        """One joint pass; returns [(uz, ux)] per plan ([] with fetch=False).
        self.ms holds the device time of the joint time loop."""
        n = len(self.plans)
        out = []
        uz = ux = None
        if fetch:
            out = [(np.zeros((p.sv.nshot, p.sv.nrec, p.sv.nt)), np.zeros((p.sv.nshot, p.sv.nrec, p.sv.nt)))
                   for p in self.plans]
            uz = (_lib._dp * n)(*[dptr(o[0]) for o in out])
            ux = (_lib._dp * n)(*[dptr(o[1]) for o in out])
        ms = np.zeros(1)
        check(_lib.lib().psv_joint_forward(self.h, uz, ux, dptr(ms)))
        self.ms = float(ms[0])
        return out

    def gradient(self):
        """One FWI gradient of every survey (any storage) through the two
        joint passes of each shot batch; returns L2 per plan, the gradients
        stay on the plans.  self.ms holds the device time of the passes."""
        L2 = np.zeros(len(self.plans))
        ms = np.zeros(1)
        check(_lib.lib().psv_joint_gradient(self.h, dptr(L2), dptr(ms)))
        self.ms = float(ms[0])
        return L2

    def launches(self) -> int:
        return int(_lib.lib().psv_joint_launches(self.h))

    @property
    def shape(self):
        """(rows_per_thread, block_y) of the joint launches ((0, 0) before an
        autotuning first forward)."""
        r, b = np.zeros(1, np.int32), np.zeros(1, np.int32)
        check(_lib.lib().psv_joint_shape(self.h, iptr(r), iptr(b)))
        return int(r[0]), int(b[0])

    def close(self):
        if self.h:
            _lib.lib().psv_joint_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def multi_gradient(plans):
    """psv_multi_gradient: one FWI gradient of every survey (one Plan each)
    concurrently; returns L2 per plan, gradients stay on the plans."""
    n = len(plans)
    hs = (C.c_void_p * n)(*[p.h for p in plans])
    L2 = np.zeros(n)
    check(_lib.lib().psv_multi_gradient(hs, n, dptr(L2)))
    return L2
