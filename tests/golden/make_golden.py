"""Generate tests/golden/reference_cases.npz from the reference's own CPU code.

Run where the reference checkout is present (``make -C oracle ref`` builds
oracle/_ref/libref_psv.so from its sources):

    python tests/golden/make_golden.py

Every case stores its inputs (survey scalars, sources, receivers, models,
observed traces) and the reference's outputs, so the tests can re-run the
oracle (and, on a GPU, the engine) on exactly these inputs without the
reference being present.
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

from oracle import oracle as O  # noqa: E402
import helpers  # noqa: E402

SCALARS = ("nt", "nz", "nx", "dt", "dz", "dx", "fdorder", "surf", "npower", "damp_v_pml", "rcoef",
           "k_max_pml", "freq_pml", "snap_z1", "snap_z2", "snap_x1", "snap_x2", "snap_dt",
           "snap_dz", "snap_dx", "imaging_sign", "nshot", "stf_type", "rtf_type", "fpad")
ARRAYS = ("npml", "isurf", "taper", "z_src", "x_src", "src_shot_to_fire", "stf_z", "stf_x",
          "z_rec", "x_rec")


def pack(prefix, sv, out):
    for k in SCALARS:
        out[f"{prefix}/{k}"] = np.asarray(getattr(sv, k))
    out[f"{prefix}/stencil"] = np.asarray(sv.stencil)
    for k in ARRAYS:
        out[f"{prefix}/{k}"] = np.asarray(getattr(sv, k))


def main():
    O.build(ref=True)
    ref = O.reference()
    ref.set_threads(1)
    out = {}
    # host preprocessing
    for fd in (2, 4, 6, 8):
        out[f"hc/{fd}"] = ref.holbergcoeff(fd)
    prof = ref.cpml(2.0, 3000.0, 0.001, 1.0, 100.0, 20, 20, 2, 141, 5e-5, 0.5)
    out["cpml"] = np.stack(prof)
    out["wavelet"] = ref.wavelet(800, 5e-5, 1.0, 100.0)

    # forward: surface layout, reference stencil at orders 2 and 4
    for name, fd in (("fwd_surface_o2", 2), ("fwd_surface_o4", 4)):
        sv, true, _ = helpers.case(fdorder=fd, stencil="reference", nt=300, nz=51, nx=71,
                                   npml=10, nrec=16, seed=11)
        lam, mu, rho = true
        mz, rz, rx, _ = ref.mat_av2(lam, mu, rho)
        o = ref.kernel_PSV(sv, 0, lam, mu, mz, rz, rx, accu=True)
        pack(name, sv, out)
        out[f"{name}/model"] = np.stack(true)
        for k in ("rtf_uz", "rtf_ux", "vz", "vx", "szz", "szx", "sxx", "We", "uz", "ux"):
            out[f"{name}/{k}"] = o[k]
        out[f"{name}/hist_szz"] = o["history"]["szz"][::25]

    # FWI: the reference's crosswell layout, CUDA-path sign (the CPU sign's
    # search fails on physical cases), 10 iterations
    sv, true, init = helpers.crosswell(nt=300, nz=51, nx=41, nshot=2, nrec=12, npml=8)
    mz, rz, rx, _ = ref.mat_av2(*true)
    uz = np.zeros((sv.nshot, sv.nrec, sv.nt))
    ux = np.zeros_like(uz)
    for s in range(sv.nshot):  # observed data: the reference's forward of the true model
        o = ref.kernel_PSV(sv, s, true[0], true[1], mz, rz, rx)
        uz[s], ux[s] = o["rtf_uz"], o["rtf_ux"]
    r = ref.simulate_fwi(sv, *init, uz, ux, niter=10)
    assert r["rc"] == 0
    name = "fwi_crosswell"
    pack(name, sv, out)
    out[f"{name}/true"] = np.stack(true)
    out[f"{name}/init"] = np.stack(init)
    out[f"{name}/obs_uz"], out[f"{name}/obs_ux"] = uz, ux
    for k in ("L2", "step", "lam", "mu", "rho", "grad_lam", "grad_mu", "grad_rho"):
        out[f"{name}/{k}"] = r[k]
    # whole program: the reference's simulate_PSV() on its binary inputs
    # (forward modelling with snapshot and seismogram output)
    import tempfile
    from fwi_cuda_gb300 import io as fio
    sv, true, _ = helpers.crosswell(nt=200, nz=45, nx=37, nshot=2, nrec=10, npml=8, snap_dt=5)
    sv.snap_dz = sv.snap_dx = 3
    work = tempfile.mkdtemp()
    fio.write_inputs(work, sv, *true, fwinv=False, accu_save=True, seismo_save=True, gpu_code=False)
    name = "program_fwd"
    for f in ("metaint", "intarray", "metafloat", "mat"):
        out[f"{name}/{f}.bin"] = np.fromfile(os.path.join(work, "bin", f + ".bin"), np.uint8)
    assert ref.lib.ref_simulate_PSV_in_dir(work.encode()) == 0
    snt, snz, snx = sv.snap_dims()
    for s in range(sv.nshot):
        uz, ux = fio.read_seismo(work, s, sv.nrec, sv.nt)
        out[f"{name}/shot{s}_rtf_uz"], out[f"{name}/shot{s}_rtf_ux"] = uz, ux
        acc = fio.read_accu(work, s, (snt, snz, snx))
        for k in ("vz", "szx"):
            out[f"{name}/shot{s}_{k}"] = acc[k]
    pack(name, sv, out)
    out[f"{name}/model"] = np.stack(true)

    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_cases.npz")
    np.savez_compressed(path, **out)
    print(path, os.path.getsize(path))


if __name__ == "__main__":
    main()
