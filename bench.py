"""Benchmark: FWI gradient throughput of the GB300 P/SV engine.

Workload (the reference's FWI-iteration configuration): 301 x 601 grid,
dx = dz = 0.5 m, 8 shots along a free surface, 120 receivers, 4th-order
Holberg stencil, 20-cell CPML on three sides, dt = 5e-5 s, nt = 4000, FP32
wavefields, snapshots every 3 steps (the reference's example setting,
scripts/pre_proc_fwi.py:68).  Seeded synthetic layered-plus-anomaly model.

One step = one FWI gradient over all 8 shots: forward with snapshot storage,
residual and L2, time-reversed adjoint with the imaging condition, energy
weights and scaling into the global gradients.
metric = grid-point updates per second, forward + adjoint
       = 8 shots * 2 passes * nt * nz * nx / step time.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
Prints one JSON line (rank 0).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "grid-pt updates/s fwd+adj (FWI gradient)"
UNIT = "updates/s"
CFG = dict(nz=301, nx=601, dx=0.5, nt=4000, dt=5e-5, nshot=8, fdorder=4, stencil="holberg",
           npml=20, nrec=120, snap_dt=3)
L2_BYTES = 129 * 2 ** 20


def workload(nt=None, nshot=None, setup=None):
    """The surface FWI case (fwi_cuda_gb300.survey.surface_fwi_case): the
    free surface sits on the first interior row, where the reference's
    stress-image surface is stable with the full 4th-order stencil."""
    from fwi_cuda_gb300 import survey as S
    return S.surface_fwi_case(nt=nt or CFG["nt"], nshot=nshot or CFG["nshot"], setup=setup)


def config_dict(n_gpus, extra=None):
    d = {"workload": "FWI gradient, 301x601 layered+anomaly, 8 shots, nt=4000, order-4 Holberg, "
                     "free surface (first interior row) + 20-cell CPML, snap_dt=3",
         "nz": CFG["nz"], "nx": CFG["nx"], "nt": CFG["nt"], "shots_per_gpu": CFG["nshot"],
         "fdorder": CFG["fdorder"], "stencil": CFG["stencil"], "snap_dt": CFG["snap_dt"],
         "precision": "fp32 wavefields, fp64 model/traces", "l2_flush": True,
         "parallelism": f"shots sharded over {n_gpus} GPU(s), gradient all-reduce"}
    if extra:
        d.update(extra)
    return d


def updates_per_step(nt, nshot):
    return 2.0 * nshot * nt * CFG["nz"] * CFG["nx"]


# ----------------------------------------------------------------------------- CPU baseline
def product_library_loaded():
    """True when the engine's libfwi_psv.so is mapped into this process."""
    try:
        with open("/proc/self/maps") as f:
            return any("libfwi_psv" in line for line in f)
    except OSError:
        return False


def cpu_baseline(nt_sample=1000, threads=None, stencil="reference"):
    """One shot, forward + adjoint gradient, cropped to nt_sample steps, on the
    host cores: the reference's own code when oracle/_ref is built here, else
    the oracle port (same loop structure and OpenMP placement).  The survey's
    set-up arrays come from that library's own functions, so the engine's
    library is never loaded.  stencil "reference": the reference as written
    (2-point difference x hc[1]); "holberg": the full 4th-order stencil the
    engine runs (oracle port only: the reference has no such stencil)."""
    from oracle import oracle as O
    O.build()
    kind = "reference" if O.ref_available() and stencil == "reference" else "port"
    lib = O.reference() if kind == "reference" else O.oracle()
    cores = threads or os.cpu_count()
    lib.set_threads(cores)
    sv, true, init = workload(nt=nt_sample, nshot=1, setup=lib)
    sv.stencil = stencil
    lam, mu, rho = init
    mz, rz, rx, _ = lib.mat_av2(lam, mu, rho)
    t0 = time.perf_counter()
    fwd = lib.kernel_PSV(sv, 0, lam, mu, mz, rz, rx, accu=True)
    src = (sv.z_rec, sv.x_rec, np.zeros(sv.nrec, np.int32), 0)
    lib.kernel_PSV(sv, 0, lam, mu, mz, rz, rx, grad=True, history=fwd["history"],
                   stf=(fwd["rtf_uz"], fwd["rtf_ux"]), src=src, rec=False)
    dt = time.perf_counter() - t0
    upd = 2.0 * nt_sample * CFG["nz"] * CFG["nx"]
    what = ("reference 2-point stencil at fdorder 4" if stencil == "reference"
            else "4th-order Holberg stencil (the engine's work)")
    return dict(value=upd / dt, unit=UNIT, cores=cores, kind=kind,
                sample=f"1 shot forward+adjoint gradient, 301x601, nt={nt_sample} "
                       f"(of 4000), {what}, FP64, {dt:.1f} s")


# ----------------------------------------------------------------------------- clocks
class Clocks:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={gpu_index}", f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        self.p.wait()
        self.f.seek(0)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.f.read().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.f.name)
        load = [s for s in sm if smax and s > 0.5 * max(smax)] or sm
        return {"sm_mhz": statistics.median(load) if load else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": sorted(reasons),
                "samples": len(sm)}


# ----------------------------------------------------------------------------- roofline
def algorithmic_bytes(prof_kernel, snap_dt):
    """Bytes per grid-point update each kernel must move (FP32) when every
    field it touches crosses HBM exactly once: stress reads vz, vx (8 B),
    reads and writes szz, szx, sxx (24 B), reads dt*lam, dt*(lam+2mu),
    dt*mu_zx (12 B); velocity reads the 3 stresses (12 B), reads and writes
    vz, vx (16 B), reads dt/rho_z, dt/rho_x (8 B), plus the energy (8 B),
    displacement (16 B, adjoint) and the snapshot store or imaging terms
    amortised over snap_dt."""
    store = 20.0 / snap_dt           # 5 snapshot planes written every snap_dt steps
    image = (20.0 + 24.0 + 8.0) / snap_dt  # history read + 3 gradients RW + 2 factors
    return {"stress_fwd": 44.0, "stress_adj": 44.0,
            "velocity_fwd": 36.0 + 8.0 + store,          # sigma R, v RW, 2 coef, We RW
            "velocity_adj": 36.0 + 16.0 + 8.0 + image}[prof_kernel]  # + u RW, We_adj RW


def read_traffic(kernel, name="dram_traffic.txt"):
    """DRAM bytes per launch of `kernel` from a committed ncu summary, or None."""
    path = os.path.join(ROOT, "profiles", name)
    if not os.path.exists(path):
        return None
    for line in open(path):
        parts = line.split()
        if len(parts) >= 2 and parts[0] == kernel and not line.startswith("#"):
            try:
                return float(parts[1])
            except ValueError:
                return None
    return None


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        d = json.load(open(path))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# ----------------------------------------------------------------------------- our arm
def run_profile(args):
    """One FWI gradient of a reduced case for ncu captures (--profile):
    nt / shots from --nt / --nshot; prints nothing measured."""
    from fwi_cuda_gb300 import engine
    if args.grid == "large":
        sv, true, init = large_workload(nt=args.nt, nshot=args.nshot)
    else:
        sv, true, init = workload(nt=args.nt, nshot=args.nshot)
    with engine.Plan(sv, precision=32, **plan_kernels(args)) as p:
        p.set_model(*true)
        obs = p.forward()
        p.set_model(*init)
        p.set_observed(*obs)
        L2, _ = p.gradient(fetch=False)
    print(json.dumps({"profile_case": {"nt": sv.nt, "nshot": sv.nshot, "L2": L2,
                                       "kernels": args.kernels, "rows_per_thread": args.rpt,
                                       "block_y": args.by}}))


def plan_kernels(args):
    """Plan options for --kernels / --rpt (auto: the autotuner chooses)."""
    if args.kernels == "auto":
        return {}
    dflt = {"tma": 4, "fused": 32, "march": 64}.get(args.kernels, 1)
    return dict(kernels=args.kernels, rows_per_thread=args.rpt or dflt, block=(32, args.by))


def run_ours(args, rank, world):
    import torch
    from fwi_cuda_gb300 import _lib, engine

    dev = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(dev)
    sv, true, init = workload()
    nt, nshot = sv.nt, sv.nshot
    with engine.Plan(sv, precision=32, **plan_kernels(args)) as p:
        p.set_model(*true)
        obs_uz, obs_ux = p.forward()          # observed data from the true model
        p.set_model(*init)
        p.set_observed(obs_uz, obs_ux)
        fam, rpt, by = p.autotune() if args.kernels == "auto" else p.shape
        kernels = {"family": fam, "rows_per_thread": rpt, "block_y": by, "chains": p.chains}
        stream = torch.cuda.ExternalStream(p.stream)
        flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device="cuda")

        def barrier():
            if world > 1:
                import torch.distributed as dist
                dist.barrier()
            torch.cuda.synchronize()

        for _ in range(args.warmup):
            p.gradient(fetch=False)
        # ---- value: inputs resident, CUDA events on the plan's stream
        barrier()
        clk = Clocks(dev)
        l0 = p.kernel_launches
        times = []
        for _ in range(args.steps):
            flush.fill_(1.0)                    # evict L2 between steps
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            p.gradient(fetch=False)
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
        barrier()
        clocks = clk.stop()
        launches = p.kernel_launches - l0
        ms = float(np.mean(times))
        if world > 1:
            import torch.distributed as dist
            t = torch.tensor([ms], device="cuda")
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            ms = float(t.item())
        value = updates_per_step(nt, nshot) * world / (ms / 1e3)
        split = p.timing()

        # ---- e2e: through the C ABI with pinned host buffers each step
        h_model = [torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy() for a in init]
        h_obs = [torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy() for a in (obs_uz, obs_ux)]
        h_grad = [torch.empty((sv.nz, sv.nx), dtype=torch.float64).pin_memory().numpy() for _ in range(3)]
        import ctypes as C
        lib = _lib.lib()
        L2 = C.c_double()
        e2e_t = []
        for it in range(max(2, args.steps)):
            barrier()
            t0 = time.perf_counter()
            _lib.check(lib.psv_plan_set_model(p.h, *[_lib.dptr(a) for a in h_model]))
            _lib.check(lib.psv_plan_set_observed(p.h, _lib.dptr(h_obs[0]), _lib.dptr(h_obs[1])))
            _lib.check(lib.psv_gradient(p.h, C.byref(L2), *[_lib.dptr(a) for a in h_grad]))
            if world > 1:
                import torch.distributed as dist
                g = torch.from_numpy(np.stack(h_grad)).cuda()
                dist.all_reduce(g)
            torch.cuda.synchronize()
            e2e_t.append(time.perf_counter() - t0)
        e2e_s = float(np.mean(e2e_t[1:]))
        if world > 1:
            import torch.distributed as dist
            t = torch.tensor([e2e_s], device="cuda")
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            e2e_s = float(t.item())
        h2d = sum(a.nbytes for a in h_model) + sum(a.nbytes for a in h_obs)
        d2h = sum(a.nbytes for a in h_grad) + 8

        # ---- roofline of the dominant kernel (event-timed launches)
        prof = p.profile_kernels(nsteps=min(300, nt))
        fwi = None
        if rank == 0 and not args.no_fwi:
            t0 = time.perf_counter()
            r = p.fwi_iteration(0.01)
            fwi = dict(seconds=time.perf_counter() - t0, trials=r["ntrials"], step=r["step"])
    large = large_grid(args) if rank == 0 and not args.no_large else None
    c3 = c3_cropped(args) if rank == 0 and not args.no_c3 else None
    uneven = uneven_batch(args) if rank == 0 and not args.no_uneven else None
    small = small_surveys(args) if rank == 0 and not args.no_uneven else None
    batching = None
    if rank == 0 and not args.no_batching:
        shape = dict(kernels=fam, rows_per_thread=rpt, block=(32, by), chains=kernels["chains"])
        batching = batching_compare(sv, init, obs_uz, obs_ux, shape, nshot / (ms / 1e3))

    if rank != 0:
        return None
    peak, src = peaks()
    pts = CFG["nz"] * CFG["nx"] * nshot
    bench_kernels = {}
    for k, v in prof.items():
        if v <= 0:
            continue
        alg = algorithmic_bytes(k, CFG["snap_dt"]) * pts
        bench_kernels[k] = {"ms": round(v, 5), "algorithmic_bytes": alg,
                            "achieved_gbs": alg / (v * 1e-3) / 1e9,
                            "frac": alg / (v * 1e-3) / 1e9 / peak}
    if large:
        roofline = large.pop("roofline")
    else:  # no HBM-bound leg: the bench grid's dominant kernel, whose fields stay in L2
        top = max(prof, key=prof.get)
        alg = algorithmic_bytes(top, CFG["snap_dt"]) * pts
        roofline = {"bound": "hbm", "kernel": top, "grid": "301x601x8 (L2-resident)",
                    "achieved": alg / (prof[top] * 1e-3) / 1e9, "peak": peak, "unit": "GB/s",
                    "frac": alg / (prof[top] * 1e-3) / 1e9 / peak, "peak_source": src,
                    "traffic": None, "algorithmic_bytes_per_launch": alg, "launch_ms": prof[top]}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded layered model)",
        "config": config_dict(world, {"kernels": kernels}),
        "shots_per_s": nshot * world / (ms / 1e3),
        "split_ms": {k: round(v, 3) for k, v in split.items()},
        # forward-only and adjoint-only rates of the same gradient (device time)
        "updates_per_s_forward": nshot * world * nt * CFG["nz"] * CFG["nx"] / (split["forward_ms"] * 1e-3),
        "updates_per_s_adjoint": nshot * world * nt * CFG["nz"] * CFG["nx"] / (split["adjoint_ms"] * 1e-3),
        "e2e": {"value": updates_per_step(nt, nshot) * world / e2e_s, "unit": UNIT,
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": e2e_s * 1e3},
        "roofline": roofline,
        # the bench grid's kernels: their 55 MB of wavefields stay in the L2, so
        # these fractions of the HBM peak say little about HBM efficiency
        "bench_grid_kernels": bench_kernels,
        "gpu_launches": launches,
        "clocks": clocks,
    }
    if fwi:
        line["fwi_iteration_s"] = fwi["seconds"]
        line["fwi_trials"] = fwi["trials"]
    if batching:
        line["batching"] = batching
    if large:
        line["large_grid"] = large
    if c3:
        line["c3_cropped"] = c3
    if uneven:
        line["uneven_batch"] = uneven
    if small:
        line["small_surveys"] = small
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(nt_sample=args.cpu_nt)
        line["cpu_one_thread"] = cpu_baseline(nt_sample=max(20, args.cpu_nt // 4), threads=1)
    return line


def batching_compare(sv, init, obs_uz, obs_ux, shape, batched_shots_s):
    """Shots/s of one FWI gradient of the bench survey along the plain and the
    batched paths on this GPU:
    plain        - the reference's GPU structure: one shot per launch
                   (kernel_PSV_GPU, src/cuda/d_kernel_PSV.cu:16-220), the
                   snapshot history resident on the device
                   (src/cuda/d_alloc_PSV.cu:104): the plan with max_batch = 1
                   and full storage;
    checkpointed - every shot in one launch per half-step, checkpointed
                   snapshot storage (two-level: one extra forward);
    batched_full - every shot in one launch, full storage (the bench's value);
    dropin_host_history - one shot through psv_kernel_PSV (kernel_PSV's
                   interface) with the FP64 snapshot history returned to the
                   host and fed back, host residual: the drop-in's price.
    batched_vs_plain = checkpointed / plain."""
    from fwi_cuda_gb300 import engine, survey as S
    lam, mu, rho = init
    mz, rz, rx, _ = S.mat_av2(lam, mu, rho)
    snap = (sv.snap_z1, sv.snap_z2, sv.snap_x1, sv.snap_x2, sv.snap_dt, sv.snap_dz, sv.snap_dx)
    cz = (sv.a_z, sv.b_z, sv.K_z, sv.a_half_z, sv.b_half_z, sv.K_half_z)
    cx = (sv.a_x, sv.b_x, sv.K_x, sv.a_half_x, sv.b_half_x, sv.K_half_x)

    def call(grad, stf, src, nrec, history=None):
        return engine.kernel_PSV(0, sv.nt, sv.nz, sv.nx, sv.dt, sv.dx, sv.dz, sv.surf, sv.isurf,
                                 sv.hc, sv.fdorder, lam, mu, mz, rz, rx, grad, sv.pml_z, cz,
                                 sv.pml_x, cx, len(src[0]), src[3], stf[0], stf[1], src[0],
                                 src[1], src[2], nrec, sv.rtf_type, sv.z_rec, sv.x_rec,
                                 not grad, snap, history=history, stencil=sv.stencil,
                                 precision=32)

    fire = np.asarray(sv.src_shot_to_fire)
    own = np.nonzero(fire == 0)[0]
    src0 = (np.asarray(sv.z_src)[own], np.asarray(sv.x_src)[own], np.zeros(len(own), np.int32),
            sv.stf_type)
    stf0 = (np.asarray(sv.stf_z)[own], np.asarray(sv.stf_x)[own])
    t0 = time.perf_counter()
    f = call(False, stf0, src0, sv.nrec)
    res = (f["rtf_uz"] - obs_uz[0], f["rtf_ux"] - obs_ux[0])   # adjsrc2 residual
    call(True, res, (sv.z_rec, sv.x_rec, np.zeros(sv.nrec, np.int32), sv.rtf_type), 0,
         history=f["history"])
    dropin = 1.0 / (time.perf_counter() - t0)
    del f

    def plan_rate(**kw):
        with engine.Plan(sv, precision=32, **dict(shape, **kw)) as p:
            p.set_model(*init)
            p.set_observed(obs_uz, obs_ux)
            p.gradient(fetch=False)  # warm-up (graph capture)
            t = []
            for _ in range(3):
                t0 = time.perf_counter()
                p.gradient(fetch=False)  # returns after the stream is idle
                t.append(time.perf_counter() - t0)
            return sv.nshot / min(t), p.storage[0]

    plain, kind_p = plan_rate(max_batch=1, storage="full", chains=1)
    ck, kind_c = plan_rate(storage="checkpoint")
    return {"plain_shots_s": plain, "checkpointed_shots_s": ck,
            "batched_full_shots_s": batched_shots_s, "batched_vs_plain": ck / plain,
            "batched_full_vs_plain": batched_shots_s / plain,
            "dropin_host_history_shots_s": dropin, "storage": [kind_p, kind_c],
            "note": "plain: one shot per launch, history on the device (the reference's GPU "
                    "structure); batched_vs_plain = checkpointed batch / plain"}


LARGE = dict(nz=1001, nx=2001, dx=0.5, nt=300, dt=2.5e-5, nshot=8, fdorder=8, npml=30,
             nrec=500, snap_dt=3)


def large_workload(nt=None, nshot=None):
    from fwi_cuda_gb300 import survey as S
    c = dict(LARGE)
    c["nt"] = nt or c["nt"]
    c["nshot"] = nshot or c["nshot"]
    sv, true, init = S.config_layered(nz=c["nz"], nx=c["nx"], dx=c["dx"], nt=c["nt"], dt=c["dt"],
                                      nshot=c["nshot"], fdorder=c["fdorder"], npml=c["npml"],
                                      nrec=c["nrec"], snap_dt=c["snap_dt"], n_layers=8,
                                      vp_range=(1500.0, 4500.0), seed=77, surf_offset=0)
    sv.imaging_sign = 1
    return sv, true, init


STEP_BYTES = {  # algorithmic bytes per grid-point update of a whole time step (FP32)
    "forward": 60.0,   # v, sigma read + written once (40 B), 5 coefficients (20 B)
    "adjoint": 84.0,   # + adjoint displacement u RW (16 B), We_adj RW (8 B)
}


def step_terms(snap_dt):
    """Per-update bytes reported beside the step's: forward We RW (8 B) and
    snapshot store (5 planes every snap_dt steps), adjoint imaging (history
    read 20 B + 3 shot gradients RW 24 B every snap_dt steps)."""
    return {"forward": 8.0 + 20.0 / snap_dt, "adjoint": 44.0 / snap_dt}


def large_grid(args):
    """HBM-bound kernels: the 1001 x 2001, order-8 Holberg, 30-cell CPML grid
    of the batched-survey configuration, 8 shots (577 MB of wavefields, far
    above the 126 MB L2), time axis cropped to 300 steps.  Reports
    - the headline roofline object: the dominant kernel's per-kernel
      algorithmic bytes (algorithmic_bytes x points) / its CUDA-event launch
      time, against the measured HBM copy bandwidth, with the ncu DRAM
      traffic per launch (profiles/dram_traffic_large.txt, captured on two
      shots and scaled to eight by the points processed);
    - the forward and adjoint time steps' fractions on the whole-step bytes
      (60 and 84 B per update), and with the We / snapshot-store and imaging
      terms added;
    - gradient throughput."""
    from fwi_cuda_gb300 import engine
    c = LARGE
    sv, true, init = large_workload()
    with engine.Plan(sv, precision=32, **plan_kernels(args)) as p:
        p.set_model(*true)
        obs = p.forward()
        p.set_model(*init)
        p.set_observed(*obs)
        fam, rpt, by = p.autotune() if args.kernels == "auto" else p.shape
        p.gradient(fetch=False)
        t0 = time.perf_counter()
        p.gradient(fetch=False)
        sec = time.perf_counter() - t0
        tm = p.timing()
        prof = p.profile_kernels(nsteps=100)
    pts = c["nz"] * c["nx"] * c["nshot"]
    peak, src = peaks()
    kern = {}
    for k, ms in prof.items():
        if ms <= 0:  # one-launch families time the whole step as the velocity launch
            continue
        alg = algorithmic_bytes(k, c["snap_dt"]) * pts
        kern[k] = {"ms": round(ms, 4), "algorithmic_bytes": alg,
                   "achieved_gbs": alg / (ms * 1e-3) / 1e9, "frac": alg / (ms * 1e-3) / 1e9 / peak}
    step_ms = {"forward": prof["stress_fwd"] + prof["velocity_fwd"],
               "adjoint": prof["stress_adj"] + prof["velocity_adj"]}
    terms = step_terms(c["snap_dt"])
    steps = {}
    for d in ("forward", "adjoint"):
        t = step_ms[d] * 1e-3
        steps[d] = {"ms": round(step_ms[d], 4), "bytes_per_update": STEP_BYTES[d],
                    "frac": STEP_BYTES[d] * pts / t / 1e9 / peak,
                    "bytes_per_update_with_terms": STEP_BYTES[d] + terms[d],
                    "frac_with_terms": (STEP_BYTES[d] + terms[d]) * pts / t / 1e9 / peak}
    top = max(kern, key=lambda k: kern[k]["ms"])
    fam_kernel = {"tma": "k_{}_tma", "direct": "k_{}", "vec4": "k_{}_v4", "fused": "k_step_fused",
                  "march": "k_step_march"}[fam]
    traffic = read_traffic(f"{fam_kernel.format(top.split('_')[0])}_{top.split('_')[1]}",
                           "dram_traffic_large.txt")
    roofline = {"bound": "hbm", "kernel": top, "family": fam,
                "grid": "1001x2001x8 shots, order 8 (HBM-bound)",
                "achieved": kern[top]["achieved_gbs"], "peak": peak, "unit": "GB/s",
                "frac": kern[top]["frac"], "peak_source": src, "traffic": traffic,
                "algorithmic_bytes_per_launch": kern[top]["algorithmic_bytes"],
                "launch_ms": kern[top]["ms"], "step": steps}
    return {"workload": "1001x2001, order-8 Holberg, 30-cell CPML, 8 shots, nt=300 (cropped), "
                        "FP32, snap_dt=3", "kernels": {"family": fam, "rows_per_thread": rpt,
                                                        "block_y": by},
            "updates_per_s": 2.0 * pts * c["nt"] / sec, "gradient_s": sec,
            "updates_per_s_forward": pts * c["nt"] / (tm["forward_ms"] * 1e-3),
            "updates_per_s_adjoint": pts * c["nt"] / (tm["adjoint_ms"] * 1e-3),
            "peak_gbs": peak, "peak_source": src, "per_kernel": kern, "roofline": roofline}


def c3_cropped(args, nt=240):
    """The batched-survey configuration's 64 shots on its 1001 x 2001,
    order-8 grid, time axis cropped to `nt` steps: one FWI gradient with the
    full snapshot history and one with 64 checkpoints per shot (two-level),
    both in two batches of 32 shots (the full history of 64 shots does not
    fit the 180 GB budget at once, and the global gradient sums the batches
    in order, so equal batches are what makes the comparison exact); the two
    gradients must be equal bit for bit (recomputation is deterministic)."""
    from fwi_cuda_gb300 import engine
    c = dict(LARGE, nshot=64, nt=nt)
    sv, true, init = large_workload(nt=nt, nshot=64)
    out = {}
    obs = None
    for storage in ("full", "checkpoint"):
        kw = dict(plan_kernels(args), storage=storage, max_batch=32)
        if storage == "checkpoint":
            kw["checkpoint_interval"] = -(-nt // 64)
        with engine.Plan(sv, precision=32, **kw) as p:
            if obs is None:
                p.set_model(*true)
                obs = p.forward()
            p.set_model(*init)
            p.set_observed(*obs)
            p.gradient(fetch=False)  # tunes, captures the graphs
            p.reset_gradient()
            t0 = time.perf_counter()
            L2, g = p.gradient()
            sec = time.perf_counter() - t0
            kind, seg, slots, _ = p.storage
            out[storage] = dict(L2=L2, g=g, s=sec, kind=kind, seg=seg, slots=slots,
                                gb=p.device_bytes / 1e9, shape=p.shape)
    f, k = out["full"], out["checkpoint"]
    equal = f["L2"] == k["L2"] and all(np.array_equal(a, b) for a, b in zip(f["g"], k["g"]))
    diff = max(float(np.linalg.norm(b - a) / max(np.linalg.norm(a), 1e-300))
               for a, b in zip(f["g"], k["g"]))
    upd = 2.0 * c["nshot"] * nt * c["nz"] * c["nx"]
    return {"workload": f"1001x2001, order 8, 64 shots, nt={nt} (cropped from 10000), FP32",
            "full_s": f["s"], "checkpoint_s": k["s"],
            "full_updates_per_s": upd / f["s"], "checkpoint_updates_per_s": upd / k["s"],
            "checkpoint_segment_steps": k["seg"], "checkpoint_slots_per_shot": k["slots"],
            "device_gb": {"full": f["gb"], "checkpoint": k["gb"]},
            "kernels": dict(zip(("family", "rows_per_thread", "block_y"), f["shape"])),
            "checkpointed_equals_full_bitwise": bool(equal), "max_rel_l2_difference": diff}


UNEVEN_SHOTS = 32
UNEVEN = [  # (nz, nx, nt cropped, fdorder, npml, peak Hz): the uneven-batch grids
    (401, 801, 200, 4, 20, 60.0), (601, 1201, 300, 8, 30, 80.0),
    (1001, 2001, 400, 4, 30, 100.0), (1501, 3001, 600, 8, 40, 120.0)]


def uneven_batch(args):
    """Four surveys of the uneven-batch configuration's shape (32 shots on
    each of its grids, 401x801 to 1501x3001, time axes cropped to 200-600
    steps, orders 4 and 8 mixed, CPML 20-40 cells, Ricker peaks 60-120 Hz, at
    most 40 GB of device memory each): one FWI gradient of all four through
    psv_multi_gradient (concurrent) against the same plans one after another;
    then forward modelling of all four concurrently, one after another and
    in one launch per half-step (forward_modes)."""
    from fwi_cuda_gb300 import engine, survey as S
    plans, models, pts = [], [], 0.0
    try:
        for k, (nz, nx, nt, fd, npml, fc) in enumerate(UNEVEN):
            sv, true, init = S.config_layered(nz=nz, nx=nx, dx=0.5, nt=nt, dt=5e-5, nshot=UNEVEN_SHOTS,
                                              fdorder=fd, npml=npml, nrec=200, snap_dt=3,
                                              fc=fc, seed=100 + k, surf_offset=0)
            sv.imaging_sign = 1
            p = engine.Plan(sv, precision=32, hbm_budget_gb=40.0, **plan_kernels(args))
            plans.append(p)
            models.append((sv, true))
            p.set_model(*true)
            obs = p.forward()
            p.set_model(*init)
            p.set_observed(*obs)
            pts += 2.0 * UNEVEN_SHOTS * nt * nz * nx
        engine.multi_gradient(plans)  # tunes and captures graphs
        t0 = time.perf_counter()
        engine.multi_gradient(plans)
        conc = time.perf_counter() - t0
        t0 = time.perf_counter()
        for p in plans:
            p.gradient(fetch=False)
        seq = time.perf_counter() - t0
        kernels = [dict(zip(("family", "rows_per_thread", "block_y"), p.shape)) for p in plans]
        storage = [p.storage[0] for p in plans]
        for p in plans:
            p.close()
        # forward modelling: plans holding every shot in one batch (their
        # history is never allocated), each with the gradient plans' tuned shape
        plans = []
        for (sv, true), kk in zip(models, kernels):
            p = engine.Plan(sv, precision=32, hbm_budget_gb=250.0, max_batch=UNEVEN_SHOTS,
                            kernels=kk["family"], rows_per_thread=kk["rows_per_thread"],
                            block=(32, kk["block_y"]), autotune=False)
            plans.append(p)
            p.set_model(*true)
        fwd = forward_modes(plans, pts / 2.0)
        return {"workload": "4 surveys: 401x801 (nt 200), 601x1201 (300), 1001x2001 (400), "
                            f"1501x3001 (600; cropped from 4000-12000), {UNEVEN_SHOTS} shots each, "
                            "orders 4/8, FP32",
                "storage": storage,
                "concurrent_s": conc, "sequential_s": seq,
                "concurrent_updates_per_s": pts / conc, "sequential_updates_per_s": pts / seq,
                "kernels": kernels, "forward_modelling": fwd}
    finally:
        for p in plans:
            p.close()


def forward_modes(plans, updates, rpt=0, by=4):
    """Forward modelling of every survey of `plans` three ways: concurrently
    (psv_multi_forward, each plan's own kernels), one after another, and in
    one stress + one velocity launch per time step over all surveys
    (psv_joint_forward: direct family, rpt rows per thread and 32 x by
    blocks, rpt 0: the joint autotuner's shape; the plans keep that shape
    afterwards).  Seconds per pass of all surveys (host clock around warm
    calls; the joint pass also by CUDA events)."""
    from fwi_cuda_gb300 import engine
    engine.multi_forward(plans)
    t0 = time.perf_counter()
    engine.multi_forward(plans)
    conc = time.perf_counter() - t0
    t0 = time.perf_counter()
    for p in plans:
        p.forward()
    seq = time.perf_counter() - t0
    out = {"concurrent_s": conc, "sequential_s": seq,
           "concurrent_updates_per_s": updates / conc, "sequential_updates_per_s": updates / seq}
    try:
        with engine.Joint(plans, rows_per_thread=rpt, block_y=by) as J:
            J.forward()  # captures the joint graph
            t0 = time.perf_counter()
            J.forward()
            joint = time.perf_counter() - t0
            jr, jb = J.shape
            out.update(joint_s=joint, joint_device_s=J.ms * 1e-3, joint_launches=J.launches(),
                       joint_shape={"rows_per_thread": jr, "block_y": jb},
                       joint_updates_per_s=updates / joint)
    except _lib_error() as e:
        out["joint_error"] = str(e)
    return out


def _lib_error():
    from fwi_cuda_gb300 import _lib
    return _lib.PSVError


def small_surveys(args):
    """Eight small surveys (101 x 201, 2 shots, nt 500, order 4, one model
    each): one FWI gradient of all eight through psv_multi_gradient (one
    stream per survey), one after another, and one survey holding all 16
    shots (one launch per half-step: the most a single launch over the eight
    surveys could reach); then forward modelling the same ways and through
    the joint launch over the eight surveys (forward_modes), and the
    gradient of all eight through the joint passes."""
    from fwi_cuda_gb300 import engine, survey as S
    plans = []

    def plan(nshot, seed):
        sv, true, init = S.config_layered(nz=101, nx=201, dx=0.5, nt=500, dt=5e-5, nshot=nshot,
                                          fdorder=4, npml=10, nrec=40, snap_dt=3, seed=seed,
                                          surf_offset=0)
        p = engine.Plan(sv, precision=32, **plan_kernels(args))
        plans.append(p)
        p.set_model(*true)
        obs = p.forward()
        p.set_model(*init)
        p.set_observed(*obs)
        return p

    try:
        each = [plan(2, 200 + k) for k in range(8)]
        one16 = plan(16, 300)
        engine.multi_gradient(each)  # tunes and captures graphs
        one16.gradient(fetch=False)
        t0 = time.perf_counter()
        engine.multi_gradient(each)
        conc = time.perf_counter() - t0
        t0 = time.perf_counter()
        for p in each:
            p.gradient(fetch=False)
        seq = time.perf_counter() - t0
        t0 = time.perf_counter()
        one16.gradient(fetch=False)
        one = time.perf_counter() - t0
        upd = 2.0 * 16 * 500 * 101 * 201
        one16.forward()
        t0 = time.perf_counter()
        one16.forward()
        one_fwd = time.perf_counter() - t0
        fwd = forward_modes(each, upd / 2.0)
        fwd["one_survey_16_shots_s"] = one_fwd
        fwd["one_survey_updates_per_s"] = upd / 2.0 / one_fwd
        out = {"workload": "8 surveys of 101x201, 2 shots each, nt 500, order 4, FP32",
               "concurrent_s": conc, "sequential_s": seq, "one_survey_16_shots_s": one,
               "concurrent_updates_per_s": upd / conc, "sequential_updates_per_s": upd / seq,
               "one_survey_updates_per_s": upd / one, "forward_modelling": fwd}
        # the gradient of all eight through the joint passes (autotuned shape)
        try:
            with engine.Joint(each) as J:
                J.gradient()  # tunes and captures the passes
                for p in each:
                    p.reset_gradient()
                t0 = time.perf_counter()
                J.gradient()
                jg = time.perf_counter() - t0
                jr, jb = J.shape
                out.update(joint_s=jg, joint_device_s=J.ms * 1e-3, joint_updates_per_s=upd / jg,
                           joint_shape={"rows_per_thread": jr, "block_y": jb})
        except _lib_error() as e:
            out["joint_error"] = str(e)
        return out
    finally:
        for p in plans:
            p.close()


FULL = {  # the batched-survey and the large single-model configurations
    "c3": dict(nz=1001, nx=2001, dx=0.5, dt=2.5e-5, nt=10000, nshot=64, nrec=500, rec_spacing=3,
               fdorder=8, npml=30, layers=8, dip=60.0, fault=None, anomalies=6, radius=(10, 30),
               checkpoint_interval=157),   # 64 checkpoints per shot
    "c5": dict(nz=2001, nx=4001, dx=1.0, dt=1e-4, nt=12000, nshot=32, nrec=800, rec_spacing=4,
               fdorder=8, npml=40, layers=8, dip=40.0, fault=(2000, 40), anomalies=10,
               radius=(10, 30), checkpoint_interval=0),  # checkpoints sized to the 180 GB budget
}


UNEVEN_FULL_NT = (4000, 6000, 8000, 12000)


def run_uneven_full(args):
    """The uneven batch at its stated shape (--config c4): the four surveys
    of the uneven-batch leg (401x801 to 1501x3001, 32 shots each, orders 4
    and 8 mixed, CPML 20-40, Ricker peaks 60-120 Hz) with their full time
    axes (4000, 6000, 8000, 12000 steps; --crop-nt M caps each), 45 GB of
    device memory per plan (checkpointed storage where the history does not
    fit).  Observed data from the true models, then one FWI gradient of all
    four through psv_multi_gradient (concurrent), or with --joint through
    psv_joint_gradient (one stress and one velocity launch per joint step
    over batch b of all four surveys, the direct family).
    Prints one JSON line: wall seconds, forward + adjoint updates/s over the
    four surveys (the recomputed forwards not counted), each plan's storage,
    kernels and device time (concurrent), or the joint shape and launches."""
    from fwi_cuda_gb300 import engine, survey as S
    plans, pts = [], 0.0
    nts = [min(n, args.crop_nt) if args.crop_nt else n for n in UNEVEN_FULL_NT]
    try:
        t0 = time.perf_counter()
        for k, ((nz, nx, _, fd, npml, fc), nt) in enumerate(zip(UNEVEN, nts)):
            sv, true, init = S.config_layered(nz=nz, nx=nx, dx=0.5, nt=nt, dt=5e-5, nshot=UNEVEN_SHOTS,
                                              fdorder=fd, npml=npml, nrec=200, snap_dt=3,
                                              fc=fc, seed=100 + k, surf_offset=0)
            sv.imaging_sign = 1
            p = engine.Plan(sv, precision=32, hbm_budget_gb=45.0, **plan_kernels(args))
            plans.append(p)
            p.set_model(*true)
            obs = p.forward()
            p.set_model(*init)
            p.set_observed(*obs)
            pts += 2.0 * UNEVEN_SHOTS * nt * nz * nx
        t_obs = time.perf_counter() - t0
        if args.joint:
            with engine.Joint(plans) as J:
                t1 = time.perf_counter()
                L2 = J.gradient()
                sec = time.perf_counter() - t1
                shape, nl, dev = J.shape, J.launches(), J.ms
            print(json.dumps({"config": "c4", "joint": True, "cropped_nt": bool(args.crop_nt), "nt": nts,
                              "shots": 4 * UNEVEN_SHOTS, "gradient_s": sec,
                              "gradient_s_includes": "the joint shape autotune and graph captures",
                              "updates_per_s": pts / sec, "device_s": dev * 1e-3,
                              "device_updates_per_s": pts / (dev * 1e-3), "observed_data_s": t_obs,
                              "joint_shape": shape, "launches": nl,
                              "storage": [p.storage[0] for p in plans],
                              "L2": [float(x) for x in L2]}), flush=True)
            return
        for p in plans:  # tune serially, as psv_multi_gradient does
            p.autotune()
        t1 = time.perf_counter()
        L2 = engine.multi_gradient(plans)
        sec = time.perf_counter() - t1
        per = []
        for p, (nz, nx, *_), nt in zip(plans, UNEVEN, nts):
            kind, seg, slots, _ = p.storage
            per.append({"grid": f"{nz}x{nx}", "nt": nt, "storage": kind, "segment_steps": seg,
                        "slots_per_shot": slots, "device_gb": p.device_bytes / 1e9,
                        "kernels": dict(zip(("family", "rows_per_thread", "block_y"), p.shape)),
                        "device_ms": p.timing()})
        print(json.dumps({"config": "c4", "cropped_nt": bool(args.crop_nt), "nt": nts,
                          "shots": 4 * UNEVEN_SHOTS, "gradient_s": sec,
                          "updates_per_s": pts / sec, "observed_data_s": t_obs,
                          "L2": [float(x) for x in L2], "surveys": per}), flush=True)
    finally:
        for p in plans:
            p.close()


def run_full_config(args):
    """One FWI gradient of a full configuration (--config c3 | c5): seeded
    dipping layered model (vp in [1500, 4500] m/s, Gardner rho, vs = vp/1.73,
    c5 with a fault), +-10 % Gaussian anomalies, initial model smoothed with
    sigma = 15 cells, surface sources and receivers, checkpointed storage
    (two-level, or binomial with --storage binomial).
    Prints one JSON line: seconds per gradient, forward + adjoint updates/s
    (the recomputed forward is extra work, not counted), shots/s.  With
    --fwi-iterations N, then N FWI iterations from the initial model (the
    step-length search with its trial forwards and the update included): the
    misfit, accepted step, trial count and seconds of each.  --crop-nt M runs
    the configuration on its first M time steps (labelled in the line)."""
    import numpy as np
    from fwi_cuda_gb300 import engine, survey as S
    c = dict(FULL[args.config])
    if args.crop_nt:
        c["nt"] = min(c["nt"], args.crop_nt)
    rng = np.random.default_rng(2024)
    fpad = c["fdorder"] // 2
    vp = S.layered_vp(c["nz"], c["nx"], c["layers"], 1500.0, 4500.0, rng, dip_cells=c["dip"],
                      top=2 * fpad, fault=c["fault"])
    vp = S.add_anomalies(vp, rng, c["anomalies"], amp=0.10, radius=c["radius"], signs=(1, -1),
                         margin=c["npml"] + fpad)
    true, init = S.model_from_vp(vp), S.smoothed(vp, 15.0)
    sv = S.surface_survey(c["nz"], c["nx"], c["dx"], c["dx"], c["nt"], c["dt"],
                          fdorder=c["fdorder"], npml=c["npml"], nshot=c["nshot"], nrec=c["nrec"],
                          rec_spacing=c["rec_spacing"], fc=100.0, vp_max=float(vp.max()),
                          snap_dt=3, surf_offset=0, seed=7)
    sv.imaging_sign = 1
    t0 = time.perf_counter()
    ck = dict(storage="checkpoint", checkpoint_interval=c["checkpoint_interval"])
    if args.storage == "binomial":
        ck = dict(storage="binomial", checkpoint_slots=args.slots)
    with engine.Plan(sv, precision=32, **ck, **plan_kernels(args)) as p:
        p.set_model(*true)
        obs = p.forward()
        t_obs = time.perf_counter() - t0
        p.set_model(*init)
        p.set_observed(*obs)
        fam, rpt, by = p.autotune() if args.kernels == "auto" else p.shape
        t1 = time.perf_counter()
        L2, _ = p.gradient(fetch=False)
        sec = time.perf_counter() - t1
        tm = p.timing()
        mem = p.device_bytes
        kind, seg, slots, adv = p.storage
        fwi = []
        if args.fwi_iterations:
            p.reset_gradient()
            step = 0.01
            from fwi_cuda_gb300 import _lib
            for _ in range(args.fwi_iterations):
                t2 = time.perf_counter()
                try:
                    r = p.fwi_iteration(step)
                except _lib.PSVError as e:  # a search that finds no decrease ends the run
                    fwi.append({"error": str(e), "seconds": time.perf_counter() - t2})
                    break
                step = r["step"]
                fwi.append({"L2": r["L2"], "step": step, "trials": r["ntrials"],
                            "seconds": time.perf_counter() - t2})
                # progress on stderr, so a run stopped from outside keeps its record
                print(json.dumps({"iteration": len(fwi) - 1, **fwi[-1]}), file=sys.stderr,
                      flush=True)
                if args.time_budget and time.perf_counter() - t0 > args.time_budget:
                    break
    upd = 2.0 * c["nshot"] * c["nt"] * c["nz"] * c["nx"]
    print(json.dumps({"config": args.config, "cropped_nt": bool(args.crop_nt),
                      "fwi_iterations": fwi, "workload": {k: v for k, v in c.items()},
                      "kernels": {"family": fam, "rows_per_thread": rpt, "block_y": by},
                      "storage": {"kind": kind, "segment_steps": seg, "slots_per_shot": slots,
                                  "extra_segment_advances": adv},
                      "gradient_s": sec, "updates_per_s_fwd_adj": upd / sec,
                      "shots_per_s": c["nshot"] / sec, "forward_ms": tm["forward_ms"],
                      "adjoint_ms": tm["adjoint_ms"], "observed_data_s": t_obs,
                      "device_gb": mem / 1e9, "L2": L2, "finite": bool(np.isfinite(L2))}))


# ----------------------------------------------------------------------------- reference arm
def run_reference(args):
    """The reference's CPU implementation of the path on the host cores: each
    step is a bounded sample (one shot forward + adjoint, nt cropped).  Beside
    it: the same sample on one thread, and the oracle port running the
    engine's own 4th-order stencil on all cores.  The engine's library is
    never loaded in this process (checked)."""
    for _ in range(args.warmup):
        cpu_baseline(nt_sample=args.ref_nt)
    vals = [cpu_baseline(nt_sample=args.ref_nt) for _ in range(args.steps)]
    v = float(np.mean([x["value"] for x in vals]))
    b = vals[-1]
    one = cpu_baseline(nt_sample=max(20, args.ref_nt // 4), threads=1)
    hol = cpu_baseline(nt_sample=args.ref_nt, stencil="holberg")
    if product_library_loaded():
        raise RuntimeError("the engine's library was loaded by the reference arm")
    upd = 2.0 * args.ref_nt * CFG["nz"] * CFG["nx"]
    return {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": 0,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": upd / v * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded layered model)", "config": config_dict(1),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": b["cores"], "kind": b["kind"],
                             "sample": b["sample"]},
            "cpu_one_thread": one, "cpu_same_stencil": hol,
            "engine_library_loaded": False,
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def flush_c_stdio():
    """Flush the C stdio buffers of loaded libraries (the compiled reference
    prints progress with printf), so the JSON line is the last one."""
    import ctypes
    try:
        ctypes.CDLL(None).fflush(None)
    except (OSError, AttributeError):
        pass
    sys.stdout.flush()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--grid", choices=["bench", "large"], default="bench",
                    help="--profile workload: the 301x601 bench grid or the 1001x2001 grid")
    ap.add_argument("--config", choices=["c3", "c4", "c5"], default=None,
                    help="run one gradient of a full configuration instead of the bench")
    ap.add_argument("--storage", choices=["checkpoint", "binomial"], default="checkpoint",
                    help="snapshot storage of the --config runs")
    ap.add_argument("--fwi-iterations", type=int, default=0,
                    help="with --config: FWI iterations after the gradient")
    ap.add_argument("--time-budget", type=float, default=0.0,
                    help="with --fwi-iterations: start no iteration after this many seconds")
    ap.add_argument("--crop-nt", type=int, default=0,
                    help="with --config: run the first N time steps only")
    ap.add_argument("--slots", type=int, default=0,
                    help="state slots per shot with --storage binomial (0 = the library's choice)")
    ap.add_argument("--joint", action="store_true",
                    help="--config c4: the gradient through the joint launches")
    ap.add_argument("--no-uneven", action="store_true",
                    help="skip the multi-survey legs (uneven grids, small surveys)")
    ap.add_argument("--no-large", action="store_true",
                    help="skip the 1001x2001 per-kernel bandwidth leg")
    ap.add_argument("--no-c3", action="store_true",
                    help="skip the 64-shot cropped batched-survey leg (full vs checkpointed)")
    ap.add_argument("--no-batching", action="store_true",
                    help="skip the plain-vs-batched shots/s comparison")
    ap.add_argument("--kernels", choices=["auto", "direct", "tma", "vec4", "fused", "march"], default="auto",
                    help="time-step kernel family (auto: the plan's autotuner picks)")
    ap.add_argument("--rpt", type=int, default=0, help="rows per thread with --kernels")
    ap.add_argument("--by", type=int, default=4, help="thread-block height with --kernels")
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-nt", type=int, default=1000)
    ap.add_argument("--ref-nt", type=int, default=400)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fwi", action="store_true")
    ap.add_argument("--profile", action="store_true", help="one gradient of a reduced case (ncu)")
    ap.add_argument("--nt", type=int, default=400, help="time steps of the --profile case")
    ap.add_argument("--nshot", type=int, default=2, help="shots of the --profile case")
    args = ap.parse_args()
    if args.config == "c4":
        return run_uneven_full(args)
    if args.config:
        return run_full_config(args)
    if args.profile:
        run_profile(args)
        return
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    if args.impl == "reference":
        if rank == 0:
            line = run_reference(args)
            flush_c_stdio()  # the reference's own prints come before the JSON line
            print(json.dumps(line), flush=True)
        return
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
        dist.init_process_group("nccl")
    line = run_ours(args, rank, world)
    if rank == 0:
        flush_c_stdio()
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
