"""The host BVH code (build, validation, binary and wide collapse) compiled
with AddressSanitizer and UndefinedBehaviorSanitizer and run over random and
degenerate triangle sets (tests/native/bvh_host_check.cpp)."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


@pytest.mark.timeout(600)
def test_host_bvh_code_under_sanitizers(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    cuda_inc = next((p for p in ("/usr/local/cuda/include", "/usr/include") if Path(p, "vector_types.h").exists()),
                    None)
    if cuda_inc is None:
        pytest.skip("CUDA headers not found")
    exe = tmp_path / "bvh_host_check"
    cmd = [gxx, "-std=c++17", "-O1", "-g", "-ffp-contract=off", "-fsanitize=address,undefined",
           "-fno-sanitize-recover=all", f"-I{cuda_inc}", str(ROOT / "tests/native/bvh_host_check.cpp"),
           str(ROOT / "pyre_gb300/csrc/bvh_host.cpp"), "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=500,
                       env={"ASAN_OPTIONS": "detect_leaks=1", "UBSAN_OPTIONS": "print_stacktrace=1"})
    assert r.returncode == 0 and r.stdout.strip() == "ok", (r.stdout + r.stderr)[-4000:]
