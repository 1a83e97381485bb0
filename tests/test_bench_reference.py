"""CPU: the reference arm of bench.py (`--impl reference`) prints the bench
contract's JSON line -- the reference's own CPU code (or, where its sources
are absent, the oracle's restatement) timed on the host cores on one tile
sample of the GPU arm's workload, with its cpu_baseline and a zero-copy e2e
-- on the small workload (seconds)."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_json_line():
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload",
                          "small", "--steps", "1", "--warmup", "0"], cwd=ROOT, env=env, capture_output=True,
                         text=True, timeout=300)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
                "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference"
    assert line["unit"] == "depth maps/s" and line["higher_is_better"] is True
    assert line["value"] > 0 and line["cpu_baseline"]["value"] == line["value"]
    import oracle as O

    # the reference's own sources where this host has them (or their staged
    # copy), else the oracle's restatement -- and the line says which
    want_kind = "reference" if O.reference_available() else "port"
    assert line["cpu_baseline"]["kind"] == want_kind and line["cpu_baseline"]["cores"] >= 1
    assert line["ms_per_step"] > 0 and line["config"]["seconds_per_map_estimate"] > 0
    assert line["e2e"] == {"value": line["value"], "unit": "depth maps/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    assert line["config"]["workload"].startswith("sphere 640x480, 4 sources")
