"""The reference arm of bench.py on the host cores: its one JSON line keeps the
benchmark contract (metric, unit, step counts, cpu_baseline, a zero-copy e2e),
and ranks other than 0 exit cleanly without output.  Small workload (32^3,
64 x 64 rays) so it runs in about a second."""
import json
import os
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
ARGS = ["--impl", "reference", "--size", "32", "--rays", "64", "--steps", "2", "--warmup", "1"]


def _run(env_extra=None):
    env = dict(os.environ)
    env.update(env_extra or {})
    return subprocess.run([sys.executable, str(ROOT / "bench.py"), *ARGS], cwd=ROOT, env=env,
                          capture_output=True, text=True, timeout=300)


def test_reference_arm_line():
    r = _run()
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["unit"] == "s" and d["higher_is_better"] is False
    assert d["n_gpus"] == 1 and d["steps"] == 2 and d["warmup"] == 1
    assert d["value"] > 0 and abs(d["ms_per_step"] - 1e3 * d["value"]) <= 1e-3 * d["ms_per_step"] + 1e-3
    assert d["vs_baseline"] is None
    assert "32^3" in d["config"]["workload"]
    # the timed runs stop at K*, the first iteration within 1e-3 of the oracle's solution
    assert d["config"]["output_relerr_vs_oracle"] <= 1e-3
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == d["value"]
    e2e = d["e2e"]
    assert e2e["value"] == d["value"] and e2e["unit"] == "s"
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_reference_arm_other_ranks_exit_quietly():
    r = _run({"RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1"})
    assert r.returncode == 0, r.stderr[-2000:]
    assert not [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
