"""Generate tests/golden/fwi_surface_301x601.npz: the FP64 oracle's ten FWI
iterations on the full-size surface FWI case (301 x 601, 8 shots,
nt = 4000, order-4 Holberg; fwi_cuda_gb300.survey.surface_fwi_case).

The oracle restates the reference's CPU FWI loop
(src/cpu/n_simulate_PSV.cpp:249-582) and step-length search
(src/cpu/n_step_length_PSV.cpp:13-209) and is pinned bit for bit to the
reference's own code on smaller cases (tests/test_oracle.py).  This script
runs it once, one iteration per call with the step, the model and the
accumulating global gradients carried from call to call (the same sequence
as one ten-iteration call), and stores per iteration:

* misfit, accepted step, number of trial forwards, the (step, misfit) of
  every trial;
* the global gradients' norms and their values at 2048 seeded cells, the
  updated model's values at the same cells;
* the first iteration's global gradients in full (float32);
* per shot, the norms of the observed traces and their values at 512
  seeded (receiver, step) pairs, so a test can check that its own observed
  data are the oracle's.

The survey's set-up arrays (Holberg coefficients, CPML profiles, wavelet)
come from the oracle's own functions, so the fixture does not depend on the
engine.  Run time: about three hours on 8 x86 cores.

Usage: python tests/golden/make_fwi_sequence.py [--threads N] [--niter 10]
"""
import argparse
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from fwi_cuda_gb300 import survey as S  # noqa: E402
from oracle import oracle as O  # noqa: E402

OUT = os.path.join(HERE, "fwi_surface_301x601.npz")
NSAMPLE = 2048
NSAMPLE_TRACE = 512


def sample_cells(sv, n, seed=11):
    rng = np.random.default_rng(seed)
    iz = rng.integers(sv.snap_z1, sv.snap_z2 + 1, n)
    ix = rng.integers(sv.snap_x1, sv.snap_x2 + 1, n)
    return iz.astype(np.int32), ix.astype(np.int32)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--threads", type=int, default=max(1, (os.cpu_count() or 2) - 1))
    ap.add_argument("--niter", type=int, default=10)
    ap.add_argument("--out", default=OUT)
    ap.add_argument("--nt", type=int, default=4000, help="shorter records check the script quickly")
    args = ap.parse_args()
    O.build()
    orc = O.oracle()
    orc.set_threads(args.threads)
    sv, true, init = S.surface_fwi_case(nt=args.nt, setup=orc)
    t0 = time.time()
    obs_uz, obs_ux = orc.simulate_fwd(sv, *true)
    print(f"observed data: {time.time() - t0:.0f} s", flush=True)
    iz, ix = sample_cells(sv, NSAMPLE)
    rng = np.random.default_rng(12)
    tr_r = rng.integers(0, sv.nrec, NSAMPLE_TRACE).astype(np.int32)
    tr_t = rng.integers(0, sv.nt, NSAMPLE_TRACE).astype(np.int32)
    out = dict(cells_z=iz, cells_x=ix, trace_rec=tr_r, trace_t=tr_t,
               obs_norm_uz=np.linalg.norm(obs_uz.reshape(sv.nshot, -1), axis=1),
               obs_norm_ux=np.linalg.norm(obs_ux.reshape(sv.nshot, -1), axis=1),
               obs_sample_uz=obs_uz[:, tr_r, tr_t], obs_sample_ux=obs_ux[:, tr_r, tr_t],
               niter=args.niter, threads=args.threads, nt=args.nt)
    lam, mu, rho = (np.array(a, np.float64) for a in init)
    grads = [np.zeros((sv.nz, sv.nx)) for _ in range(3)]
    step = 0.01
    L2s, steps, trials, tlogs, gnorm, gsamp, msamp = [], [], [], [], [], [], []
    for it in range(args.niter):
        t1 = time.time()
        r = orc.simulate_fwi(sv, lam, mu, rho, obs_uz, obs_ux, niter=1, step0=step, grads=grads)
        if r["rc"] != 0:
            raise SystemExit(f"iteration {it}: step-length search failed (rc {r['rc']})")
        lam, mu, rho = r["lam"], r["mu"], r["rho"]
        grads = [r["grad_lam"], r["grad_mu"], r["grad_rho"]]
        step = float(r["step"][0])
        L2s.append(r["L2"][0])
        steps.append(step)
        trials.append(int(r["trials"][0]))
        tlogs.append(r["trial_log"][0])
        gnorm.append([np.linalg.norm(g) for g in grads])
        gsamp.append(np.stack([g[iz, ix] for g in grads]))
        msamp.append(np.stack([m[iz, ix] for m in (lam, mu, rho)]))
        if it == 0:
            out["grad_iter0"] = np.stack(grads).astype(np.float32)
        print(f"iteration {it}: L2 {L2s[-1]:.10e} step {step:.10e} trials {trials[-1]} "
              f"({time.time() - t1:.0f} s)", flush=True)
    out.update(L2=np.array(L2s), step=np.array(steps), trials=np.array(trials, np.int32),
               trial_log=np.array(tlogs), grad_norm=np.array(gnorm), grad_sample=np.array(gsamp),
               model_sample=np.array(msamp),
               model_norm=np.array([np.linalg.norm(m) for m in (lam, mu, rho)]))
    np.savez_compressed(args.out, **out)
    print(f"wrote {args.out} ({os.path.getsize(args.out) / 1e6:.2f} MB) "
          f"in {time.time() - t0:.0f} s", flush=True)


if __name__ == "__main__":
    main()
