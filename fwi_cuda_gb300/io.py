"""The reference's binary files (src/h_io_PSV.cpp; written by
scripts/pre_proc_fwi.py:240-276).

Inputs under <workdir>/bin:
  metaint.bin    8 flags (gpu, surf, pml_z, pml_x, accu_save, seismo_save,
                 fwinv, rtf_meas_true) then 29 int32 (nt nz nx snap_t1 snap_t2
                 snap_z1 snap_z2 snap_x1 snap_x2 snap_dt snap_dz snap_dx,
                 taper t1 t2 b1 b2 l1 l2 r1 r2, nsrc nrec nshot stf_type
                 rtf_type fdorder fpad mat_save_interval mat_grid)
  intarray.bin   npml[4] isurf[4] z_src x_src src_shot_to_fire z_rec x_rec (int32)
  metafloat.bin  dt dz dx npower damp_v_pml rcoef k_max_pml freq_pml
                 scalar_lam scalar_mu scalar_rho (float64)
  mat.bin        lam, mu, rho [nz][nx] float64
Observed traces (FWI): <workdir>/io/shot{i}_rtf_u{z,x}.bin, [nrec][nt] float64.
Outputs: bin/shot{i}_rtf_u{z,x}.bin, bin/shot{i}_{vz,vx,szz,szx,sxx}.bin,
bin/iter{n}_mat.bin.
"""
from __future__ import annotations

import os

import numpy as np


def write_inputs(workdir, sv, lam, mu, rho, *, fwinv=False, accu_save=False, seismo_save=True,
                 gpu_code=True, rtf_meas_true=None, mat_save_interval=1, mat_grid=1,
                 scalar=(0.0, 0.0, 0.0)):
    """Write a survey and model the way the reference's preprocessing does."""
    b = os.path.join(workdir, "bin")
    os.makedirs(b, exist_ok=True)
    if rtf_meas_true is None:
        rtf_meas_true = fwinv
    flags = [gpu_code, sv.surf, sv.pml_z, sv.pml_x, accu_save, seismo_save, fwinv, rtf_meas_true]
    ints = [sv.nt, sv.nz, sv.nx, 0, sv.nt - 1, sv.snap_z1, sv.snap_z2, sv.snap_x1, sv.snap_x2,
            sv.snap_dt, sv.snap_dz, sv.snap_dx, *sv.taper, sv.nsrc, sv.nrec, sv.nshot,
            sv.stf_type, sv.rtf_type, sv.fdorder, sv.fpad, mat_save_interval, mat_grid]
    np.array([int(bool(f)) for f in flags] + [int(v) for v in ints], np.int32).tofile(
        os.path.join(b, "metaint.bin"))
    ia = np.concatenate([np.asarray(sv.npml, np.int32), np.asarray(sv.isurf, np.int32),
                         np.asarray(sv.z_src, np.int32), np.asarray(sv.x_src, np.int32),
                         np.asarray(sv.src_shot_to_fire, np.int32),
                         np.asarray(sv.z_rec, np.int32), np.asarray(sv.x_rec, np.int32)])
    ia.tofile(os.path.join(b, "intarray.bin"))
    np.array([sv.dt, sv.dz, sv.dx, sv.npower, sv.damp_v_pml, sv.rcoef, sv.k_max_pml, sv.freq_pml,
              *scalar], np.float64).tofile(os.path.join(b, "metafloat.bin"))
    np.concatenate([np.ravel(np.asarray(a, np.float64)) for a in (lam, mu, rho)]).tofile(
        os.path.join(b, "mat.bin"))


def write_observed(workdir, uz, ux):
    """Field measurements io/shot{i}_rtf_u{z,x}.bin from [nshot][nrec][nt]."""
    d = os.path.join(workdir, "io")
    os.makedirs(d, exist_ok=True)
    for s in range(uz.shape[0]):
        np.asarray(uz[s], np.float64).tofile(os.path.join(d, f"shot{s}_rtf_uz.bin"))
        np.asarray(ux[s], np.float64).tofile(os.path.join(d, f"shot{s}_rtf_ux.bin"))


def read_seismo(workdir, ishot, nrec, nt):
    b = os.path.join(workdir, "bin", f"shot{ishot}")
    return (np.fromfile(b + "_rtf_uz.bin", np.float64).reshape(nrec, nt),
            np.fromfile(b + "_rtf_ux.bin", np.float64).reshape(nrec, nt))


def read_accu(workdir, ishot, shape):
    """Snapshot histories (write_accu) of one shot, each `shape` = (snap_nt, snap_nz, snap_nx)."""
    b = os.path.join(workdir, "bin", f"shot{ishot}")
    return {k: np.fromfile(b + f"_{k}.bin", np.float64).reshape(shape)
            for k in ("vz", "vx", "szz", "szx", "sxx")}


def read_mat(workdir, iterstep, nz, nx):
    a = np.fromfile(os.path.join(workdir, "bin", f"iter{iterstep}_mat.bin"), np.float64)
    return a.reshape(3, nz, nx)
