"""bench.py's reference arm on the CPU: one JSON line with the contract's keys,
the metric and config of our own arm, a cpu_baseline describing the run, and
an e2e object with no host-device traffic."""
import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def test_reference_arm_line():
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--dx", "0.04",
                        "--steps", "2", "--warmup", "1"], capture_output=True, text=True, cwd=ROOT, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    j = json.loads(lines[0])
    assert j["impl"] == "reference"
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in j, k
    assert j["metric"] == "particle-steps/s" and j["higher_is_better"] is True
    assert (j["steps"], j["warmup"], j["n_gpus"]) == (2, 1, 1)
    assert j["value"] > 0 and j["config"]["workload"].startswith("3-D dam break")
    cb = j["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == j["value"]
    assert j["e2e"]["value"] == j["value"]
    assert j["e2e"]["h2d_bytes_per_step"] == 0 and j["e2e"]["d2h_bytes_per_step"] == 0
    # the same config object as our own arm prints for this workload
    sys.path.insert(0, str(ROOT))
    import bench
    from mysph_gb300 import cases
    assert j["config"] == json.loads(json.dumps(bench.bench_config(cases.dam_break_3d(dx=0.04), "fp64")))
