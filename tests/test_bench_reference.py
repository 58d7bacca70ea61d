"""The reference arm of bench.py on the CPU: the reference step (the compiled reference where
its tree exists, else the FP64 restatement) times the same workload as the GPU arm and prints
one JSON line in the GPU arm's format."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_line_on_the_same_workload(oracle_built):
    out = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--scale", "0.125", "--steps", "2",
                          "--warmup", "1"], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "particle-steps/s" and d["value"] > 0
    assert d["config"]["workload"] == "dam_break_3d_newtonian" and d["config"]["same_config"]
    assert "19950 particles" in d["config"]["sample"]  # the GPU arm's scene at this scale
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["value"] == d["value"]
    assert d["cpu_baseline"]["kind"] in ("reference", "port") and d["cpu_baseline"]["cores"] >= 1
