"""bench.py's reference arm (CPU): it prints the bench's one JSON line with the GPU arm's config
for the same workload and the reference's plain-ELP time to a 1 %/95 % triangle answer, and it runs
the oracle alone: neither the GPU library nor its Python binding is loaded in its process."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROBE = r"""
import runpy, sys
sys.argv = ["bench.py", "--impl", "reference", "--workload", "rmat13", "--steps", "1", "--warmup", "1"]
runpy.run_path("bench.py", run_name="__main__")
maps = open("/proc/self/maps").read()
print("LOADED", "zgraph" in sys.modules, "libzgraph_gpu" in maps, "libzgoracle" in maps)
"""


def test_reference_arm_line_and_isolation():
    p = subprocess.run([sys.executable, "-c", PROBE], cwd=ROOT, stdout=subprocess.PIPE, stderr=subprocess.PIPE,
                       text=True, timeout=600)
    assert p.returncode == 0, p.stderr
    lines = p.stdout.strip().splitlines()
    line = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "config", "cpu_baseline", "e2e", "impl"):
        assert k in line, k
    assert line["impl"] == "reference" and line["value"] > 0 and line["unit"] == "samples/s"
    assert line["cpu_baseline"]["value"] == line["value"] and line["cpu_baseline"]["kind"] == "port"
    assert "79403 undirected edges" in line["config"]["workload"]
    sys.path.insert(0, ROOT)
    import bench
    assert line["config"] == bench.workload_config("rmat13", 79403)  # what the GPU arm prints
    assert lines[1] == "LOADED False False True"
    # each program's samples/s and closure checks per second (the triangle closes one edge per sample)
    (prog,) = line["per_program"]
    assert prog["program"] == "triangle" and prog["samples_per_s"] > 0
    assert 0.5 < prog["closure_checks_per_sample"] <= 1.0
    # the reference's own way to a 1 %/95 % triangle answer: ErrorProfile::get_num_estimators timed on
    # the host, then calculate(n_required) at the measured rate
    ttb = line["time_to_bound"]
    assert "error" not in ttb, ttb
    assert ttb["pattern"] == "triangle" and ttb["n_required"] > 0 and ttb["samples_per_s"] > 0
    assert abs(ttb["seconds"] - ttb["profile_s"] - ttb["n_required"] / ttb["samples_per_s"]) < 1e-6 * ttb["seconds"]
