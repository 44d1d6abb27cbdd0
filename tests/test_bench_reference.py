"""The reference arm of bench.py on the CPU: one bounded sample of the
reference's CPU path (the compiled reference where it was built, else the
oracle port), printed as one JSON line with the bench's keys."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _run(*args, env=None):
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *args], cwd=ROOT,
                         capture_output=True, text=True, timeout=300, env=env)
    assert out.returncode == 0, out.stderr[-2000:]
    return out.stdout.strip().splitlines()


def test_reference_arm_json_line():
    lines = _run("--impl", "reference", "--steps", "1", "--warmup", "0", "--ref-nt", "12")
    r = json.loads(lines[-1])
    assert r["impl"] == "reference" and r["higher_is_better"] is True
    assert r["value"] > 0 and r["unit"] == "updates/s" and r["steps"] == 1
    cb = r["cpu_baseline"]
    assert cb["kind"] in ("reference", "port") and cb["cores"] >= 1 and cb["value"] == r["value"]
    assert r["e2e"] == {"value": r["value"], "unit": r["unit"], "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}
    assert r["config"]["nz"] == 301 and r["config"]["nx"] == 601
    # a one-thread sample and the engine's own stencil on the port beside it;
    # the engine's library stays out of the reference arm's process
    assert r["cpu_one_thread"]["cores"] == 1 and r["cpu_one_thread"]["value"] > 0
    assert r["cpu_same_stencil"]["kind"] == "port" and "Holberg" in r["cpu_same_stencil"]["sample"]
    assert r["engine_library_loaded"] is False


def test_reference_arm_builds_its_survey_without_the_engine():
    # the oracle's set-up functions give the engine's survey bit for bit
    from fwi_cuda_gb300 import survey as S
    from oracle import oracle as O
    a, ta, ia = S.surface_fwi_case(nt=40, nshot=2)
    b, tb, ib = S.surface_fwi_case(nt=40, nshot=2, setup=O.oracle())
    for k in ("hc", "a_z", "b_z", "K_z", "a_half_z", "b_half_z", "K_half_z", "a_x", "b_x", "K_x",
              "a_half_x", "b_half_x", "K_half_x", "stf_z", "stf_x", "z_src", "x_src", "z_rec"):
        assert (getattr(a, k) == getattr(b, k)).all(), k
    for x, y in zip(ta + ia, tb + ib):
        assert (x == y).all()


def test_reference_arm_prints_on_rank_zero_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2")
    assert _run("--impl", "reference", "--steps", "1", "--warmup", "0", "--ref-nt", "4",
                env=env) == []


def _bench_module():
    import importlib.util
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_roofline_byte_model_and_committed_traffic():
    # the per-update byte model of the roofline and the ncu traffic it is
    # compared with (profiles/dram_traffic.txt, read by the bench)
    import pytest
    b = _bench_module()
    assert b.algorithmic_bytes("stress_fwd", 3) == b.algorithmic_bytes("stress_adj", 3) == 44.0
    assert b.algorithmic_bytes("velocity_fwd", 3) == pytest.approx(44.0 + 20.0 / 3)
    assert b.algorithmic_bytes("velocity_adj", 3) == pytest.approx(60.0 + 52.0 / 3)  # 77.3 B
    assert b.algorithmic_bytes("velocity_adj", 1) == 112.0
    tv, ts = b.read_traffic("k_velocity_adj"), b.read_traffic("k_stress_adj")
    # below the algorithmic bytes of one 301 x 601 x 8 launch: the wavefields stay in L2
    updates = 8 * 301 * 601  # 111.9 MB a velocity_adj launch at snap_dt = 3
    assert b.algorithmic_bytes("velocity_adj", 3) * updates == pytest.approx(111.917e6, rel=1e-4)
    assert 0 < tv < b.algorithmic_bytes("velocity_adj", 3) * updates
    assert 0 < ts < b.algorithmic_bytes("stress_adj", 3) * updates
    assert b.read_traffic("no_such_kernel") is None


def test_step_byte_model():
    # whole-step bytes per grid-point update behind the roofline's step
    # fractions: 60 forward, 84 adjoint, plus the separately reported terms
    b = _bench_module()
    assert b.STEP_BYTES == {"forward": 60.0, "adjoint": 84.0}
    t = b.step_terms(3)
    assert t["forward"] == 8.0 + 20.0 / 3 and t["adjoint"] == 44.0 / 3
    assert b.read_traffic("k_velocity_tma_adj", "dram_traffic_large.txt") == 1062.8e6
    assert b.read_traffic("k_stress_tma_fwd", "dram_traffic_large.txt") == 528.6e6


def test_uneven_batch_configuration():
    # the uneven batch at its stated shape (bench.py --config c4): four
    # seeded layered surveys 401x801, 601x1201, 1001x2001, 1501x3001 with
    # nt 4000, 6000, 8000, 12000, 32 shots each (128), orders 4 and 8 mixed,
    # 20-40-cell CPML, Ricker peaks in [60, 120] Hz; each time step below
    # its survey's stability limit (checkfd_ssg_elastic)
    import numpy as np
    sys.path.insert(0, ROOT)
    import bench
    from fwi_cuda_gb300 import _lib, survey as S
    from fwi_cuda_gb300._lib import dptr
    assert bench.UNEVEN_SHOTS == 32 and bench.UNEVEN_FULL_NT == (4000, 6000, 8000, 12000)
    grids = [(nz, nx) for nz, nx, *_ in bench.UNEVEN]
    assert grids == [(401, 801), (601, 1201), (1001, 2001), (1501, 3001)]
    assert {fd for _, _, _, fd, _, _ in bench.UNEVEN} == {4, 8}
    assert all(20 <= npml <= 40 and 60.0 <= fc <= 120.0 for *_, npml, fc in bench.UNEVEN)
    for k, ((nz, nx, _, fd, npml, fc), nt) in enumerate(zip(bench.UNEVEN, bench.UNEVEN_FULL_NT)):
        sv, true, _ = S.config_layered(nz=nz, nx=nx, dx=0.5, nt=nt, dt=5e-5, nshot=bench.UNEVEN_SHOTS,
                                       fdorder=fd, npml=npml, nrec=200, snap_dt=3, fc=fc,
                                       seed=100 + k, surf_offset=0)
        assert (sv.nz, sv.nx, sv.nt, sv.fdorder, sv.nshot) == (nz, nx, nt, fd, 32)
        lam, mu, rho = true
        out = np.zeros(4)
        rc = _lib.lib().psv_checkfd_ssg_elastic(sv.nz, sv.nx, sv.dz, sv.dt, sv.freq_pml, npml,
                                                dptr(rho), dptr(lam), dptr(mu), dptr(sv.hc),
                                                dptr(out))
        assert rc == _lib.PSV_OK and sv.dt < out[0], (k, out)
