"""bench.py's command line: it parses without a GPU and offers the options
the measurements in the design notes use (the network's gate and grid
level, the schedule, tuning on or off, the profile run)."""
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_bench_help_lists_the_options():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--help"], capture_output=True, text=True,
                       timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stderr
    for opt in ("--impl", "--gpus", "--steps", "--warmup", "--net-gate", "--unet-level", "--schedule",
                "--autotune", "--no-autotune", "--profile-run", "--history"):
        assert opt in r.stdout, opt
