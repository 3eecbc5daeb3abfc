"""bench.py's reference arm on the CPU: one small step of the CPU
restatement, printed as the benchmark's JSON line (same metric and unit as
the GPU arm, a cpu_baseline object and an end-to-end entry without copies)."""
import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def test_reference_arm_prints_the_contract_line():
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0", "--cpu-rows", "2"], capture_output=True, text=True, timeout=600,
                       cwd=str(ROOT))
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads([l for l in r.stdout.splitlines() if l.startswith("{")][-1])
    sys.path.insert(0, str(ROOT))
    import bench
    assert line["impl"] == "reference"
    assert line["metric"] == bench.METRIC and line["unit"] == bench.UNIT
    assert line["higher_is_better"] is True and line["steps"] == 1 and line["warmup"] == 0
    assert line["value"] > 0.0 and line["ms_per_step"] > 0.0
    cb = line["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == line["value"]
    assert cb["unit"] == line["unit"] and cb["sample"]
    # the timed build is the CPU-tuned one, with its flags and the CPU model stated
    assert "native" in cb["flags"] and cb["cpu_model"]
    assert cb["bit_identical_to_portable_build"] is True
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["unit"] == line["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
