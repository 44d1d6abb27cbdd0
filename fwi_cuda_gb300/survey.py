"""Survey description and seeded synthetic models.

A :class:`Survey` holds what the reference reads from its binary inputs
(``scripts/pre_proc_fwi.py:240-276`` / ``src/h_simulate_PSV.cpp:99-185``):
grid, CPML parameters, snapshot window, taper, sources and receivers.
:meth:`Survey.finalize` derives the Holberg coefficients and the CPML
profiles with the engine's host functions (``psv_holbergcoeff``,
``psv_cpml_PSV``), exactly as ``simulate_PSV`` does.  Every builder takes
an optional ``setup`` object with the same three set-up functions
(``holbergcoeff(fdorder, maxrelerror)``, ``cpml(...)``, ``wavelet(...)``) in
their place, so a caller that must not load the engine's library (a CPU
baseline timed beside it) builds the same survey from its own copies.

The generators below build the layered-plus-anomaly models of the
benchmark configurations from a seed (no dataset is involved): horizontal
or dipping layers with vp drawn uniformly and sorted with depth,
vs = vp / 1.73, Gardner density rho = 310 vp^0.25, Gaussian vp anomalies.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from ._lib import PsvGrid, PsvShots, dptr, f64, i32, iptr


def ricker(nt: int, dt: float, fc: float, amp: float = 1.0, ts: float = 0.0,
           setup=None) -> np.ndarray:
    """Ricker wavelet of the reference (wavelet, src/h_preproc_PSV.cpp:267-286)."""
    if setup is not None:
        return np.asarray(setup.wavelet(nt, dt, amp, fc, ts, 1), np.float64)
    s = np.zeros(nt)
    _lib.check(_lib.lib().psv_wavelet(dptr(s), nt, dt, amp, fc, ts, 1))
    return s


def holbergcoeff(fdorder: int, maxrelerror: int = 1) -> np.ndarray:
    hc = np.zeros(7)
    _lib.check(_lib.lib().psv_holbergcoeff(fdorder, maxrelerror, dptr(hc)))
    return hc


def cpml_profiles(npower, damp, rcoef, kmax, freq, n1, n2, fpad, nh, dt, dh):
    arrs = [np.zeros(nh) for _ in range(6)]
    _lib.check(_lib.lib().psv_cpml_PSV(*[dptr(a) for a in arrs], npower, damp, rcoef, kmax, freq,
                                       n1, n2, fpad, nh, dt, dh))
    return arrs


@dataclass
class Survey:
    nt: int
    nz: int
    nx: int
    dt: float
    dz: float
    dx: float
    fdorder: int = 4
    stencil: str = "reference"       # "reference" (2-point x hc[1]) or "holberg"
    npml: tuple = (0, 20, 20, 20)    # top, bottom, left, right
    fpad: int | None = None          # CPML padding (metaint's fpad); default fdorder // 2
    surf: bool = False
    isurf: tuple = (0, 0, 0, 0)
    npower: float = 2.0
    damp_v_pml: float = 3000.0
    rcoef: float = 0.001
    k_max_pml: float = 1.0
    freq_pml: float = 100.0
    snap_z1: int = 0
    snap_z2: int = 0
    snap_x1: int = 0
    snap_x2: int = 0
    snap_dt: int = 1
    snap_dz: int = 1
    snap_dx: int = 1
    taper: tuple = (0, 0, 0, 0, 0, 0, 0, 0)
    imaging_sign: int = -1           # -1: reference CPU path (grad -=); +1: its CUDA path (+=)
    nshot: int = 1
    stf_type: int = 0
    rtf_type: int = 0
    z_src: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    x_src: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    src_shot_to_fire: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    stf_z: np.ndarray = field(default_factory=lambda: np.zeros((0, 0)))
    stf_x: np.ndarray = field(default_factory=lambda: np.zeros((0, 0)))
    z_rec: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    x_rec: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))

    def finalize(self, setup=None) -> "Survey":
        """Holberg coefficients and CPML profiles (h_simulate_PSV.cpp:155-170),
        from the engine's host functions or from ``setup``'s."""
        if self.fpad is None:
            self.fpad = self.fdorder // 2
        hc_fn = setup.holbergcoeff if setup is not None else holbergcoeff
        cpml_fn = setup.cpml if setup is not None else cpml_profiles
        self.hc = np.asarray(hc_fn(self.fdorder, 1), np.float64)
        self.pml_z = bool(self.npml[0] or self.npml[1])
        self.pml_x = bool(self.npml[2] or self.npml[3])
        z = cpml_fn(self.npower, self.damp_v_pml, self.rcoef, self.k_max_pml, self.freq_pml,
                    self.npml[0], self.npml[1], self.fpad, self.nz, self.dt, self.dz)
        x = cpml_fn(self.npower, self.damp_v_pml, self.rcoef, self.k_max_pml, self.freq_pml,
                    self.npml[2], self.npml[3], self.fpad, self.nx, self.dt, self.dx)
        (self.a_z, self.b_z, self.K_z, self.a_half_z, self.b_half_z, self.K_half_z) = z
        (self.a_x, self.b_x, self.K_x, self.a_half_x, self.b_half_x, self.K_half_x) = x
        self.z_src, self.x_src = i32(self.z_src), i32(self.x_src)
        self.src_shot_to_fire = i32(self.src_shot_to_fire)
        self.z_rec, self.x_rec = i32(self.z_rec), i32(self.x_rec)
        self.stf_z = f64(self.stf_z).reshape(len(self.z_src), self.nt)
        self.stf_x = f64(self.stf_x).reshape(len(self.z_src), self.nt)
        return self

    @property
    def nsrc(self) -> int:
        return int(len(self.z_src))

    @property
    def nrec(self) -> int:
        return int(len(self.z_rec))

    def snap_dims(self):
        return (1 + (self.nt - 1) // self.snap_dt,
                1 + (self.snap_z2 - self.snap_z1) // self.snap_dz,
                1 + (self.snap_x2 - self.snap_x1) // self.snap_dx)

    def grid_struct(self, keep: list) -> PsvGrid:
        g = PsvGrid()
        g.nt, g.nz, g.nx = self.nt, self.nz, self.nx
        g.dt, g.dx, g.dz = self.dt, self.dx, self.dz
        g.fdorder = self.fdorder
        g.stencil = _lib.STENCIL[self.stencil]
        g.surf = int(self.surf)
        for i in range(4):
            g.isurf[i] = int(self.isurf[i])
        for i in range(7):
            g.hc[i] = float(self.hc[i])
        g.pml_z, g.pml_x = int(self.pml_z), int(self.pml_x)
        for name in ("a_z", "b_z", "K_z", "a_half_z", "b_half_z", "K_half_z",
                     "a_x", "b_x", "K_x", "a_half_x", "b_half_x", "K_half_x"):
            a = f64(getattr(self, name))
            keep.append(a)
            setattr(g, name, dptr(a))
        (g.snap_z1, g.snap_z2, g.snap_x1, g.snap_x2, g.snap_dt, g.snap_dz, g.snap_dx) = (
            self.snap_z1, self.snap_z2, self.snap_x1, self.snap_x2, self.snap_dt, self.snap_dz,
            self.snap_dx)
        for i in range(8):
            g.taper[i] = int(self.taper[i])
        g.imaging_sign = int(self.imaging_sign)
        return g

    def shots_struct(self, keep: list) -> PsvShots:
        s = PsvShots()
        s.nshot, s.nsrc, s.nrec = self.nshot, self.nsrc, self.nrec
        s.stf_type, s.rtf_type = self.stf_type, self.rtf_type
        arrs = dict(z_src=i32(self.z_src), x_src=i32(self.x_src),
                    src_shot_to_fire=i32(self.src_shot_to_fire), z_rec=i32(self.z_rec),
                    x_rec=i32(self.x_rec), stf_z=f64(self.stf_z), stf_x=f64(self.stf_x))
        keep.extend(arrs.values())
        for k, v in arrs.items():
            setattr(s, k, iptr(v) if v.dtype == np.int32 else dptr(v))
        return s


# ----------------------------------------------------------------------------
# Seeded synthetic models
# ----------------------------------------------------------------------------

def elastic_from_velocity(vp, vs, rho):
    """lam, mu from velocities (Pa): mu = rho vs^2, lam = rho vp^2 - 2 mu."""
    mu = rho * vs * vs
    lam = rho * vp * vp - 2.0 * mu
    return f64(lam), f64(mu), f64(rho)


def layered_vp(nz, nx, n_layers, vp_lo, vp_hi, rng, dip_cells=0.0, top=0, fault=None):
    """Layers with vp ~ U[vp_lo, vp_hi] sorted increasing with depth.

    dip_cells: depth change of each interface across the model (cells).
    fault: (x_index, throw_cells) shifts the interfaces right of x_index.
    """
    vps = np.sort(rng.uniform(vp_lo, vp_hi, n_layers))
    cuts = np.sort(rng.uniform(0.15, 0.9, n_layers - 1)) * (nz - top) + top
    iz = np.arange(nz)[:, None].astype(np.float64)
    ix = np.arange(nx)[None, :].astype(np.float64)
    vp = np.full((nz, nx), vps[0])
    for k in range(n_layers - 1):
        depth = cuts[k] + dip_cells * (ix / max(nx - 1, 1) - 0.5)
        if fault is not None:
            depth = depth + np.where(ix >= fault[0], fault[1], 0.0)
        vp = np.where(iz >= depth, vps[k + 1], vp)
    return vp


def add_anomalies(vp, rng, n, amp=0.10, radius=(15, 15), signs=(1,), margin=0):
    nz, nx = vp.shape
    iz = np.arange(nz)[:, None]
    ix = np.arange(nx)[None, :]
    out = vp.copy()
    for _ in range(n):
        r = rng.uniform(radius[0], radius[1])
        cz = rng.uniform(margin + r, nz - margin - r)
        cx = rng.uniform(margin + r, nx - margin - r)
        sgn = signs[int(rng.integers(len(signs)))]
        out = out * (1.0 + sgn * amp * np.exp(-((iz - cz) ** 2 + (ix - cx) ** 2) / (r * r)))
    return out


def model_from_vp(vp, vs_ratio=1.73):
    vs = vp / vs_ratio
    rho = 310.0 * vp ** 0.25
    return elastic_from_velocity(vp, vs, rho)


def smoothed(vp, sigma, vs_ratio=1.73):
    from scipy.ndimage import gaussian_filter
    return model_from_vp(gaussian_filter(vp, sigma, mode="nearest"), vs_ratio)


# ----------------------------------------------------------------------------
# Field geometry (topography and acquisition coordinates)
# ----------------------------------------------------------------------------

def v_lami(cp, cs, rho):
    """Lame constants from velocities (scripts/seismic_def.py, v_lami)."""
    mu = cs * cs * rho
    return cp * cp * rho - 2.0 * mu, mu


def e_lami(E, nu):
    """Lame constants from Young's modulus and Poisson's ratio (e_lami)."""
    return E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu)), 0.5 * E / (1.0 + nu)


def w_vel(lam, mu, rho):
    """P and S velocities from Lame constants and density (w_vel)."""
    return np.sqrt((lam + 2 * mu) / rho), np.sqrt(mu / rho)


@dataclass
class Topography:
    """A ground profile on the model grid: nz x nx cells of dz x dx, the x
    coordinate of column 0 and the first ground row of every column."""
    nz: int
    nx: int
    xmin: float
    dz: float
    dx: float
    surf_idz: np.ndarray  # [nx] int

    def cell_x(self, x):
        """Column of each x coordinate (floor, as the reference's int())."""
        return ((np.asarray(x, np.float64) - self.xmin) / self.dx).astype(np.int32)

    def on_surface(self, x):
        """(z, x) grid indices of points placed on the ground at x."""
        ix = self.cell_x(x)
        if ix.size and (ix.min() < 0 or ix.max() >= self.nx):
            raise ValueError("a coordinate lies outside the model")
        return self.surf_idz[ix].astype(np.int32), ix


def topography_grid(profile_x, profile_z, x0, x1, dz, dx, *, npml=(20, 20, 20, 20), fpad=1,
                    z_above=10, z_below=20) -> Topography:
    """Grid around a ground profile (elevations profile_z at profile_x, in
    metres, up positive), the layout of scripts/pre_proc_dyke_4000.py:93-130:
    columns for [x0, x1] plus CPML (npml = top, bottom, left, right) and fpad
    cells; rows for the profile's relief plus z_above air and z_below ground
    cells, CPML and fpad; the profile is flipped to depths, shifted below
    the added rows and interpolated linearly at every column centre (the
    edge elevations continue beyond the profile's ends, where the
    reference's interpolation raises)."""
    pt, pb, pl, pr = npml
    px = np.asarray(profile_x, np.float64)
    depth = np.max(profile_z) - np.asarray(profile_z, np.float64)  # top at depth 0
    relief = abs(float(np.max(profile_z) - np.min(profile_z)))
    nx = fpad + pl + int(abs(x1 - x0) / dx) + pr + fpad + 1
    nz = fpad + pt + z_above + int(relief / dz) + z_below + pb + fpad + 1
    xmin = x0 - (pl + fpad) * dx
    xmax = x1 + (pr + fpad) * dx
    zmin = np.min(depth) - (z_above + pt + fpad) * dz
    depth = depth + (np.min(depth) - zmin)
    order = np.argsort(px)
    zc = np.interp(np.linspace(xmin, xmax, nx), px[order], depth[order])
    return Topography(nz=nz, nx=nx, xmin=xmin, dz=dz, dx=dx,
                      surf_idz=(zc / dz).astype(np.int64))


def topography_model(topo: Topography, ground, air=(0.0, 0.0, 1.25), *, layers=(),
                     perturb=0.0, sigma=0.0, rng=None):
    """lam, mu, rho of a model with air above the ground profile and the
    ground material (cp, cs, rho) below it; layers = ((depth_m, cp, cs, rho),
    ...) put other materials within depth_m of the surface, in order; perturb
    scales every cell by 1 + perturb * U(-1, 1); sigma > 0 smooths with a
    Gaussian (constant mode) and restores the air, as
    scripts/pre_proc_dyke_4000.py:170-205 does."""
    from scipy.ndimage import gaussian_filter
    rng = rng if rng is not None else np.random.default_rng(0)
    iz = np.arange(topo.nz)[:, None]
    below = iz >= topo.surf_idz[None, :]
    out = []
    for k in range(3):
        def prop(m):
            lam, mu = v_lami(m[0], m[1], m[2])
            return (lam, mu, m[2])[k]
        a = np.where(below, prop(ground), prop(air)).astype(np.float64)
        for depth_m, *m in layers:
            inside = below & (iz < topo.surf_idz[None, :] + depth_m / topo.dz)
            a = np.where(inside, prop(m), a)
        if perturb:
            a = np.where(below, a * (1.0 + perturb * rng.uniform(-1, 1, a.shape)), a)
        if sigma:
            a = gaussian_filter(a, sigma, mode="constant")
            a = np.where(below, a, prop(air))
        out.append(a)
    return tuple(out)


def load_profile_csv(path):
    """A ground profile file of the reference's layout (two comma-separated
    columns x, z; scripts/pre_proc_dyke_4000.py:45): (x, z)."""
    xz = np.loadtxt(path, delimiter=",").T
    return xz[0], xz[1]


def surface_survey(nz, nx, dz, dx, nt, dt, *, fdorder=4, stencil="holberg", npml=20, nshot=1,
                   nrec=120, rec_spacing=4, src_depth=4, rec_depth=2, fc=100.0, vp_max=3000.0,
                   snap_dt=1, surf_offset=None, force="z", seed=0, setup=None) -> Survey:
    """Free surface on top, CPML on the other three sides, shots evenly
    spread along the surface, receivers on a line below the surface."""
    fpad = fdorder // 2
    isurf = fpad + (surf_offset if surf_offset is not None else fpad)
    span = rec_spacing * (nrec - 1)
    x0 = (nx - 1 - span) // 2
    x_rec = x0 + rec_spacing * np.arange(nrec)
    if nshot == 1:
        x_src = np.array([(nx - 1) // 2])
    else:
        x_src = np.linspace(x_rec[0] if nrec else npml + fpad + 4,
                            x_rec[-1] if nrec else nx - npml - fpad - 5, nshot).round()
    w = ricker(nt, dt, fc, setup=setup)
    stf = np.stack([w] * nshot)
    zero = np.zeros_like(stf)
    snap_z1, snap_z2 = fpad, nz - fpad - 1
    snap_x1, snap_x2 = fpad, nx - fpad - 1
    t = max(1, npml // 2)
    taper = (isurf + 1, isurf + 1 + t, nz - npml - fpad - 1, nz - npml - fpad - 1 - t,
             npml + fpad + 1, npml + fpad + 1 + t, nx - npml - fpad - 1, nx - npml - fpad - 1 - t)
    sv = Survey(nt=nt, nz=nz, nx=nx, dt=dt, dz=dz, dx=dx, fdorder=fdorder, stencil=stencil,
                npml=(0, npml, npml, npml), surf=True, isurf=(isurf, 0, 0, 0),
                damp_v_pml=vp_max, freq_pml=fc,
                snap_z1=snap_z1, snap_z2=snap_z2, snap_x1=snap_x1, snap_x2=snap_x2,
                snap_dt=snap_dt, taper=taper, nshot=nshot, stf_type=0, rtf_type=0,
                z_src=np.full(nshot, isurf + src_depth), x_src=x_src.astype(np.int32),
                src_shot_to_fire=np.arange(nshot), stf_z=stf if force == "z" else zero,
                stf_x=zero if force == "z" else stf,
                z_rec=np.full(nrec, isurf + rec_depth), x_rec=x_rec)
    return sv.finalize(setup)


def config_layered(nz=301, nx=601, dx=0.5, nt=4000, dt=5e-5, nshot=1, fdorder=4,
                   stencil="holberg", npml=20, nrec=120, seed=1234, snap_dt=1, n_layers=5,
                   vp_range=(1800.0, 3000.0), anomaly_radius=15, smooth_sigma=15.0, fc=100.0,
                   surf_offset=None, setup=None):
    """The 301 x 601 layered-plus-anomaly survey (one shot: forward + one
    adjoint gradient; eight shots: the FWI iteration case).  Smaller sizes
    give the same structure for tests.  surf_offset: free-surface row below
    the frame (None: fdorder/2 rows, so the surface has mirrored rows above
    it).  Returns (survey, true model, initial model) with models as
    (lam, mu, rho)."""
    rng = np.random.default_rng(seed)
    fpad = fdorder // 2
    vp = layered_vp(nz, nx, n_layers, *vp_range, rng, top=2 * fpad)
    vp = add_anomalies(vp, rng, 1, amp=0.10, radius=(anomaly_radius, anomaly_radius),
                       margin=npml + fpad)
    true = model_from_vp(vp)
    init = smoothed(vp, smooth_sigma)
    rec_spacing = max(1, min(4, (nx - 2 * (npml + fpad) - 8) // max(nrec - 1, 1)))
    sv = surface_survey(nz, nx, dx, dx, nt, dt, fdorder=fdorder, stencil=stencil, npml=npml,
                        nshot=nshot, nrec=nrec, rec_spacing=rec_spacing, fc=fc,
                        vp_max=float(vp.max()), snap_dt=snap_dt, seed=seed,
                        surf_offset=surf_offset, setup=setup)
    return sv, true, init


def surface_fwi_case(nt=4000, nshot=8, setup=None):
    """The reference's surface FWI configuration at full size: 301 x 601
    cells of 0.5 m, five horizontal layers (vp uniform in [1800, 3000] m/s,
    increasing with depth) plus one +10 % Gaussian vp anomaly of 15-cell
    radius (seed 1234), initial model = the true vp Gaussian-smoothed with
    sigma = 15 cells; 4th-order Holberg stencil, free surface on the first
    interior row and 20-cell CPML on the other sides; z-force 100 Hz Ricker
    sources 2 m below the surface (one shot: x = 150 m; eight shots: evenly
    along the receiver line), 120 receivers every 2 m at 1 m depth,
    dt = 5e-5 s, nt = 4000, snapshots every 3 steps (the reference's example
    setting, scripts/pre_proc_fwi.py:68), imaging sign +1 (the descent
    direction).  The surface sits on the first interior row because with
    rows mirrored above it the reference's stress-image free surface and
    the full 4th-order Holberg stencil grow without bound over 4000 steps
    (x80 every 500 steps in the FP64 oracle).
    Returns (survey, true model, initial model)."""
    sv, true, init = config_layered(nz=301, nx=601, dx=0.5, nt=nt, dt=5e-5, nshot=nshot,
                                    fdorder=4, stencil="holberg", npml=20, nrec=120,
                                    snap_dt=3, seed=1234, surf_offset=0, setup=setup)
    sv.imaging_sign = 1
    return sv, true, init


def mat_av2(lam, mu, rho):
    """Staggered material averages the reference's host computes before each
    kernel_PSV call (mat_av2, src/cpu/n_kernel_lib_PSV.cpp:853-922): harmonic
    mu at (z+1/2, x+1/2), reciprocal arithmetic rho at (z+1/2, x) and
    (z, x+1/2), zero in the last row and column (left unset there by the
    reference), and the model means C = (C_lam, C_mu, C_rho) over the other
    cells.  The reference's vacuum test for rho_xp writes rho_zp
    (:894-897); kept.  Returns (mu_zx, rho_zp, rho_xp, C)."""
    lam, mu, rho = (np.asarray(a, np.float64) for a in (lam, mu, rho))
    nz, nx = mu.shape
    mu_zx, rho_zp, rho_xp = np.zeros((nz, nx)), np.zeros((nz, nx)), np.zeros((nz, nx))
    m00, m01, m10, m11 = mu[:-1, :-1], mu[:-1, 1:], mu[1:, :-1], mu[1:, 1:]
    with np.errstate(divide="ignore"):
        v = 4.0 / ((1.0 / m00) + (1.0 / m01) + (1.0 / m10) + (1.0 / m11))
    v[(m00 == 0) | (m01 == 0) | (m10 == 0) | (m11 == 0)] = 0.0
    mu_zx[:-1, :-1] = v
    r00, r10, r01 = rho[:-1, :-1], rho[1:, :-1], rho[:-1, 1:]
    with np.errstate(divide="ignore"):
        zp = 1.0 / (0.5 * (r00 + r10))
        xp = 1.0 / (0.5 * (r00 + r01))
    zp[(r00 < 1e-4) & (r10 < 1e-4)] = 0.0
    zp[(r00 < 1e-4) & (r01 < 1e-4)] = 0.0
    rho_zp[:-1, :-1], rho_xp[:-1, :-1] = zp, xp
    n = (nz - 1) * (nx - 1)
    C = np.array([lam[:-1, :-1].sum() / n, mu[:-1, :-1].sum() / n, rho[:-1, :-1].sum() / n])
    return mu_zx, rho_zp, rho_xp, C
