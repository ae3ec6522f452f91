"""bench.py's reference arm on the CPU: `--impl reference` times the C
restatement of WalkRay's traversal on a bounded sample of the kd workload
and prints one JSON line with the keys the benchmark contract asks for, on
the same workload description as the GPU arm."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_contract_line(built):
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--workload", "kd", "--steps", "1",
                        "--warmup", "3", "--cpu-sample", "65536"], cwd=ROOT, capture_output=True, text=True,
                       timeout=600, check=True)
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    line = json.loads(lines[0])
    sys.path.insert(0, ROOT)
    import bench

    assert line["impl"] == "reference"
    assert line["metric"] == "Mrays/s (closest hit, bit-exact vs reference)" and line["unit"] == "Mrays/s"
    assert line["value"] > 0 and line["higher_is_better"] is True
    assert line["steps"] == 1 and line["warmup"] >= 3
    assert line["config"]["workload"] == bench.KD_WORKLOAD
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"] and cb["sample"]
