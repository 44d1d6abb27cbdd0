"""Small seeded survey cases shared by the tests."""
import numpy as np

from fwi_cuda_gb300 import survey as S


def rel_l2(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (nb if nb > 0 else 1.0))


def case(fdorder=4, stencil="holberg", nshot=1, nt=250, nz=61, nx=91, npml=10, nrec=20,
         seed=7, snap_dt=1, imaging_sign=-1, surf_offset=None):
    """Layered model with a free surface on top and CPML on three sides."""
    sv, true, init = S.config_layered(nz=nz, nx=nx, nt=nt, nshot=nshot, fdorder=fdorder,
                                      stencil=stencil, npml=npml, nrec=nrec, seed=seed,
                                      anomaly_radius=5, smooth_sigma=3, snap_dt=snap_dt)
    sv.imaging_sign = imaging_sign
    if surf_offset is not None:
        fpad = fdorder // 2
        sv.isurf = (fpad + surf_offset, 0, 0, 0)
        sv.z_src = np.full(sv.nsrc, sv.isurf[0] + 4, np.int32)
        sv.z_rec = np.full(sv.nrec, sv.isurf[0] + 2, np.int32)
    return sv, true, init


def crosswell(fdorder=2, stencil="reference", nt=400, nz=81, nx=61, nshot=3, nrec=16, seed=3,
              snap_dt=3, stf_type=1, imaging_sign=1, npml=10, bottom_surface=False):
    """The reference's own example layout (scripts/pre_proc_fwi.py): CPML on
    all sides, sources in a column on the left, receivers in a column on the
    right, x-force Ricker sources."""
    rng = np.random.default_rng(seed)
    dt, dx = 4e-5, 0.5
    vp = S.layered_vp(nz, nx, 4, 1500.0, 2500.0, rng)
    vpt = S.add_anomalies(vp, rng, 1, amp=0.1, radius=(6, 6), margin=npml + 4)
    true, init = S.model_from_vp(vpt), S.model_from_vp(vp)
    fpad = fdorder // 2
    xs, xr = npml + fpad + 4, nx - npml - fpad - 5
    z_src = np.linspace(npml + 8, nz - npml - 9, nshot).astype(int)
    sv = S.Survey(nt=nt, nz=nz, nx=nx, dt=dt, dz=dx, dx=dx, fdorder=fdorder, stencil=stencil,
                  npml=(npml, npml, npml, npml), damp_v_pml=2500.0, freq_pml=200.0,
                  snap_z1=npml + fpad, snap_z2=nz - npml - fpad - 1, snap_x1=npml + fpad,
                  snap_x2=nx - npml - fpad - 1, snap_dt=snap_dt,
                  taper=(npml + 4, npml + 8, nz - npml - 5, nz - npml - 9,
                         npml + 4, npml + 8, nx - npml - 5, nx - npml - 9),
                  imaging_sign=imaging_sign, nshot=nshot, stf_type=stf_type,
                  z_src=z_src, x_src=np.full(nshot, xs), src_shot_to_fire=np.arange(nshot),
                  stf_z=np.zeros((nshot, nt)), stf_x=np.stack([S.ricker(nt, dt, 200.0)] * nshot),
                  z_rec=np.linspace(npml + 4, nz - npml - 5, nrec).astype(int),
                  x_rec=np.full(nrec, xr))
    return sv.finalize(), true, init


GOLDEN = __import__("os").path.join(__import__("os").path.dirname(__file__), "golden",
                                    "reference_cases.npz")


def load_case(z, name):
    """Rebuild the Survey of a golden case from its stored inputs."""
    kw = {}
    for k in ("nt", "nz", "nx", "fdorder", "snap_z1", "snap_z2", "snap_x1", "snap_x2", "snap_dt",
              "snap_dz", "snap_dx", "imaging_sign", "nshot", "stf_type", "rtf_type", "fpad"):
        kw[k] = int(z[f"{name}/{k}"])
    for k in ("dt", "dz", "dx", "npower", "damp_v_pml", "rcoef", "k_max_pml", "freq_pml"):
        kw[k] = float(z[f"{name}/{k}"])
    kw["surf"] = bool(z[f"{name}/surf"])
    kw["stencil"] = str(z[f"{name}/stencil"])
    for k in ("npml", "isurf", "taper"):
        kw[k] = tuple(int(v) for v in z[f"{name}/{k}"])
    for k in ("z_src", "x_src", "src_shot_to_fire", "stf_z", "stf_x", "z_rec", "x_rec"):
        kw[k] = z[f"{name}/{k}"]
    return S.Survey(**kw).finalize()


def oracle_gradient(orc, sv, model, obs_uz, obs_ux, smooth_hfs=0):
    """Global gradients of one FWI gradient pass (simulate_fwi_PSV :270-417)
    from the oracle's building blocks, before the taper; smooth_hfs >= 2
    smooths every shot gradient first (the commented-out apply_gauss_filter
    calls, :377-379)."""
    lam, mu, rho = model
    _, _, _, Cs = orc.mat_av2(lam, mu, rho)
    snap = (sv.snap_z1, sv.snap_z2, sv.snap_x1, sv.snap_x2)
    grads = [np.zeros((sv.nz, sv.nx)) for _ in range(3)]
    L2 = 0.0
    shots = []
    for s in range(sv.nshot):
        o = orc.shot_gradient(sv, s, lam, mu, rho, obs_uz, obs_ux)
        shots.append(o)
        L2 += o["L2"]
        We = orc.energy_weights2(o["We"], o["We_adj"], snap)
        for p, k in enumerate(("grad_lam", "grad_mu", "grad_rho")):
            if smooth_hfs:
                o[k] = orc.apply_gauss_filter(o[k], smooth_hfs)
            tmp = orc.interpol_grad2(o["We_adj"], o[k], snap, sv.snap_dz, sv.snap_dx)
            grads[p] = orc.scale_grad_E2(grads[p], tmp, Cs[p], We, snap)
    return L2, grads, shots
