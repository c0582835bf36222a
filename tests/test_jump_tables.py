"""Host check of the mrg32k3a skip-ahead (no GPU): radix-16 records against the recurrences (small
skips) and binary matrix powers (large skips), and the kernels' folded modular reduction against
exact arithmetic; see tests/cpp/jump_test.cpp."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_jump_tables(tmp_path):
    exe = str(tmp_path / "jump_test")
    csrc = os.path.join(ROOT, "compfinance_gb300", "csrc")
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-I", csrc, os.path.join(ROOT, "tests", "cpp", "jump_test.cpp"),
                           os.path.join(csrc, "host_math.cpp"), "-o", exe])
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    bad = [l for l in r.stdout.splitlines() if not l.startswith("ok")]
    assert r.returncode == 0 and not bad, r.stdout + r.stderr
    assert len(r.stdout.splitlines()) >= 15
