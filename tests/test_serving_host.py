"""Host-side tests of the serving scheduler (no GPU): a fake executor drives
compfinance_gb300/csrc/serving_core.h through admission, rejection, cancellation,
time-outs, injected failures and concurrent submitters."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_scheduler_with_fake_executor(tmp_path):
    exe = str(tmp_path / "sched_test")
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-pthread", os.path.join(ROOT, "tests", "cpp", "sched_test.cpp"),
                           "-o", exe])
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    bad = [l for l in r.stdout.splitlines() if not l.startswith("ok")]
    assert r.returncode == 0 and not bad, r.stdout + r.stderr
    assert len(r.stdout.splitlines()) >= 18
