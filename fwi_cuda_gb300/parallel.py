"""Shot-parallel FWI over several GPUs, one process (rank) per GPU.

Shots are independent in the reference (the shot loop of simulate_fwi_PSV,
src/cpu/n_simulate_PSV.cpp:270-419), so rank r owns a disjoint block of
shots and its own plan.  Per FWI iteration the only exchanges are one sum of
the three global gradients plus the L2 misfit, and one L2 sum per
step-length trial; every rank then takes the same branches of the line
search because it sees the same sums.

The reference's global gradient is never reset between iterations and is
tapered in place (:260, :443-450): G_k = taper(G_{k-1} + sum of this
iteration's shot contributions).  Each rank therefore computes its shots'
contributions from zero, the contributions are summed across ranks, and the
sum is added to the previous global gradient kept by the driver.

`plan` is any object with the methods of fwi_cuda_gb300.engine.Plan used
below (reset_gradient, gradient, set_gradient, get_gradient, save_model,
taper_gradient, trial_misfit, update_model).
"""
from __future__ import annotations

import ctypes as C

import numpy as np


def shard_shots(nshot: int, world: int, rank: int) -> list[int]:
    """Balanced contiguous blocks of shot indices."""
    base, extra = divmod(nshot, world)
    start = rank * base + min(rank, extra)
    return list(range(start, start + base + (1 if rank < extra else 0)))


def shard_survey(sv, shots):
    """A copy of survey `sv` holding only `shots`, renumbered 0..len-1 (the
    sources keep their src_shot_to_fire mapping, remapped)."""
    import copy
    loc = copy.copy(sv)
    remap = {g: i for i, g in enumerate(shots)}
    keep = [i for i, s in enumerate(sv.src_shot_to_fire) if int(s) in remap]
    loc.z_src = np.asarray(sv.z_src)[keep]
    loc.x_src = np.asarray(sv.x_src)[keep]
    loc.src_shot_to_fire = np.array([remap[int(sv.src_shot_to_fire[i])] for i in keep], np.int32)
    loc.stf_z = np.asarray(sv.stf_z)[keep]
    loc.stf_x = np.asarray(sv.stf_x)[keep]
    loc.nshot = len(shots)
    return loc


class DistributedFWI:
    """FWI iterations of a survey whose shots are split over ranks.

    Every rank enters every collective, also after a local failure: a rank
    whose gradient or trial forward raises contributes zeros and a failure
    mark to the same all-reduce, so all ranks learn of it from that sum and
    leave the iteration together with an error, instead of the others
    waiting in a collective the failing rank never joins."""

    NSTATUS = 16  # psv_status values are below this

    def __init__(self, plan, nz: int, nx: int, allreduce):
        """allreduce(np.ndarray float64) -> element-wise sum over ranks."""
        self.plan = plan
        self.allreduce = allreduce
        self.G = [np.zeros((nz, nx)) for _ in range(3)]  # global gradient, after the taper

    def _reduce(self, payload, status: int):
        """Sum payload over ranks together with a count of the ranks that
        failed, per status.  Returns (sum, highest failing status or 0)."""
        marks = np.zeros(self.NSTATUS)
        if status:
            marks[min(int(status), self.NSTATUS - 1)] = 1.0
        buf = self.allreduce(np.concatenate([np.ravel(payload), marks]))
        counts = buf[-self.NSTATUS:]
        failed = [k for k in range(1, self.NSTATUS) if counts[k] > 0.5]
        return buf[:-self.NSTATUS], (max(failed) if failed else 0)

    def iteration(self, step: float, max_trials: int = 64):
        from . import _lib
        p = self.plan
        p.save_model()
        p.reset_gradient()
        try:
            L2_loc, c = p.gradient()
            status, err = 0, None
        except _lib.PSVError as e:
            status, err = e.status, e
            L2_loc, c = np.nan, [np.zeros_like(g) for g in self.G]
        buf, failed = self._reduce(np.concatenate([np.ravel(x) for x in c] + [np.array([L2_loc])]),
                                   status)
        if failed:
            if err is not None:
                raise err
            raise _lib.PSVError(failed, "gradient failed on another rank")
        n = c[0].size
        L2 = float(buf[-1])
        self.G = [g + buf[k * n:(k + 1) * n].reshape(g.shape) for k, g in enumerate(self.G)]
        p.set_gradient(*self.G)
        p.taper_gradient()
        self.G = p.get_gradient()

        def trial(a, L, _ctx):
            try:
                v, st = float(p.trial_misfit(a)), 0
            except _lib.PSVError as e:
                v, st = np.nan, e.status
            tot, failed = self._reduce(np.array([v]), st)
            if failed:
                return failed
            L[0] = float(tot[0])
            return 0

        cb = _lib.TRIAL_FN(trial)
        est = C.c_double(step)
        nt = C.c_int()
        log = np.zeros((max_trials, 2))
        _lib.check(_lib.lib().psv_step_length(C.byref(est), L2, C.cast(cb, C.c_void_p), None,
                                              C.byref(nt), _lib.dptr(log), max_trials))
        p.update_model(est.value)
        return dict(L2=L2, step=est.value, ntrials=nt.value, trials=log[:min(nt.value, max_trials)])


def torch_allreduce(device=None):
    """Sum over the default torch.distributed group (gloo on CPU, nccl on GPU)."""
    import torch
    import torch.distributed as dist

    def f(a):
        t = torch.from_numpy(np.ascontiguousarray(a, np.float64))
        if device is not None:
            t = t.to(device)
        dist.all_reduce(t)
        return t.cpu().numpy()
    return f
