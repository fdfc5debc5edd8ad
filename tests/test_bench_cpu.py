"""The bench's reference arm and its timed window, on the CPU (no GPU needed)."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


def _args(*argv):
    old = sys.argv
    sys.argv = ["bench.py", *argv]
    try:
        return bench.parse()
    finally:
        sys.argv = old


def test_timed_window_starts_after_the_transient():
    a = _args("--steps", "20", "--warmup", "5")
    # steps 1..195 untimed, 196..200 warm-up, 201..220 timed
    assert bench.window_pre(a) == 195
    assert "steps 201..220" in bench.bench_config(98304, 1, a)["timed_steps"]
    # a window that starts at the impulsive start keeps one untimed step
    b = _args("--steps", "20", "--warmup", "5", "--window-start", "0")
    assert bench.window_pre(b) == 1
    assert "steps 7..26" in bench.bench_config(98304, 1, b)["timed_steps"]


@pytest.mark.skipif(not os.path.exists(os.path.join(ROOT, "oracle", "liboracle.so")),
                    reason="the oracle is built by build()")
def test_reference_arm_prints_one_line_on_the_same_config():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "2",
                        "--warmup", "1", "--window-start", "3"], capture_output=True, text=True, timeout=600,
                       cwd=ROOT)
    assert r.returncode == 0, r.stderr
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0 and d["steps"] == 2 and d["warmup"] == 1
    a = _args("--steps", "2", "--warmup", "1", "--window-start", "3")
    assert d["config"] == bench.bench_config(d["config"]["cells"], 1, a)
    assert d["cpu_baseline"]["value"] == d["value"] and d["e2e"]["value"] == d["value"]
