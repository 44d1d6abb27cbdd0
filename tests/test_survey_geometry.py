"""Field-geometry helpers of the survey builder (the layout of
scripts/pre_proc_dyke_4000.py and scripts/seismic_def.py), on the CPU."""
import numpy as np
import pytest

from fwi_cuda_gb300 import survey as S


def test_lame_and_velocity_round_trip():
    lam, mu = S.v_lami(1200.0, 500.0, 2000.0)
    assert (lam, mu) == (1200.0 ** 2 * 2000 - 2 * 500.0 ** 2 * 2000, 500.0 ** 2 * 2000)
    cp, cs = S.w_vel(lam, mu, 2000.0)
    assert cp == pytest.approx(1200.0) and cs == pytest.approx(500.0)
    lam2, mu2 = S.e_lami(2.0 * mu * 1.25, 0.25)  # E = 2 mu (1 + nu)
    assert mu2 == pytest.approx(mu) and lam2 == pytest.approx(2 * mu * 0.25 / 0.5)


def test_flat_profile_grid():
    x = np.array([-5.0, 30.0])
    t = S.topography_grid(x, [3.0, 3.0], 0.0, 10.0, 0.5, 0.25, npml=(4, 5, 6, 7), fpad=2,
                          z_above=3, z_below=8)
    assert t.nx == 2 + 6 + 40 + 7 + 2 + 1
    assert t.nz == 2 + 4 + 3 + 0 + 8 + 5 + 2 + 1
    assert t.xmin == pytest.approx(-(6 + 2) * 0.25)
    assert np.all(t.surf_idz == 3 + 4 + 2)  # air rows, CPML, fpad above the ground


def test_sloping_profile_surface_rows():
    # ground falls 1 m over 10 m; depth below the highest point grows with x
    x = np.array([-10.0, 20.0])
    z = np.array([6.0, 3.0])
    dz = 0.07  # keeps the depths off cell boundaries, where flooring is a rounding coin toss
    t = S.topography_grid(x, z, 0.0, 10.0, dz, 0.1, npml=(0, 0, 0, 0), fpad=0, z_above=2,
                          z_below=2)
    xc = t.xmin + 0.1 * np.arange(t.nx)
    depth = 0.1 * (xc + 10.0) + 2 * dz  # below the highest point, under 2 added air rows
    assert np.array_equal(t.surf_idz, (depth / dz).astype(np.int64))
    zs, xs = t.on_surface([0.05, 5.05])
    assert list(xs) == [0, 50] and list(zs) == list(t.surf_idz[[0, 50]])
    with pytest.raises(ValueError):
        t.on_surface([11.0])


def test_topography_model_regions():
    t = S.Topography(nz=30, nx=20, xmin=0.0, dz=0.5, dx=0.5,
                     surf_idz=np.full(20, 10, np.int64))
    ground, near = (1200.0, 500.0, 2000.0), (700.0, 300.0, 1200.0)
    lam, mu, rho = S.topography_model(t, ground, layers=((2.0, *near),))
    assert np.all(rho[:10] == 1.25) and np.all(mu[:10] == 0.0) and np.all(lam[:10] == 0.0)
    assert np.all(rho[10:14] == 1200.0) and np.all(rho[14:] == 2000.0)
    lam2, mu2, rho2 = S.topography_model(t, ground, perturb=0.25, sigma=2.0,
                                         rng=np.random.default_rng(1))
    assert np.all(rho2[:10] == 1.25)  # air restored after smoothing
    assert rho2[10:].min() > 0 and rho2[20:].max() < 2000.0 * 1.25


def test_profile_csv(tmp_path):
    f = tmp_path / "profile.csv"
    np.savetxt(f, np.array([[0.0, 1.0, 2.0], [5.0, 5.5, 5.2]]).T, delimiter=",")
    x, z = S.load_profile_csv(f)
    assert list(x) == [0.0, 1.0, 2.0] and list(z) == [5.0, 5.5, 5.2]


def test_surface_fwi_case_matches_the_configuration():
    # the benchmark's survey: 301 x 601 cells of 0.5 m, 120 receivers every
    # 2 m at 1 m depth, z-force Ricker sources 2 m below the surface (one
    # shot at x = 150 m; eight shots spread along the receiver line), free
    # surface on the first interior row with 20-cell CPML on the other sides,
    # dt = 5e-5 s, nt = 4000, order-4 Holberg, snapshots every 3 steps
    from fwi_cuda_gb300 import survey as S
    sv, true, init = S.surface_fwi_case(nshot=1)
    assert (sv.nz, sv.nx, sv.dz, sv.dx) == (301, 601, 0.5, 0.5)
    assert (sv.nt, sv.dt, sv.fdorder, sv.stencil, sv.snap_dt) == (4000, 5e-5, 4, "holberg", 3)
    fpad = sv.fdorder // 2
    assert sv.surf and sv.isurf[0] == fpad and tuple(sv.npml) == (0, 20, 20, 20)
    assert sv.nrec == 120 and np.all(np.diff(sv.x_rec) * sv.dx == 2.0)
    assert np.all((sv.z_rec - sv.isurf[0]) * sv.dz == 1.0)
    assert (sv.z_src[0] - sv.isurf[0]) * sv.dz == 2.0 and sv.x_src[0] * sv.dx == 150.0
    assert np.allclose(sv.stf_x, 0.0) and np.abs(sv.stf_z).max() > 0  # vertical force
    lam, mu, rho = true
    vp = np.sqrt((lam + 2 * mu) / rho)
    assert 1800 * 0.999 <= vp.min() and vp.max() <= 3000 * 1.1 * 1.001  # layers + a +10 % anomaly
    np.testing.assert_allclose(rho, 310.0 * vp ** 0.25, rtol=1e-12)
    np.testing.assert_allclose(np.sqrt(mu / rho), vp / 1.73, rtol=1e-12)
    sv8, _, _ = S.surface_fwi_case(nshot=8, nt=10)
    assert sv8.nshot == 8 and len(set(sv8.x_src)) == 8
    assert sv8.x_src.min() >= sv8.x_rec.min() and sv8.x_src.max() <= sv8.x_rec.max()
