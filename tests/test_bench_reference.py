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


def test_reference_arm_prints_on_rank_zero_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2")
    assert _run("--impl", "reference", "--steps", "1", "--warmup", "0", "--ref-nt", "4",
                env=env) == []
