"""bench.py's output contract on the CPU: the reference arm's JSON line (the oracle on the host
cores, small C1 workload) carries every key of the contract with the right types, and the
launch count the GPU arm claims follows the kernels each timed slot launches."""
import json
import os
import subprocess
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, REPO)


# runs bench.py's reference arm in this process, then lists the shared objects of the repository it mapped
_RUN_AND_LIST = """
import os, runpy, sys
sys.argv = ["bench.py", "--impl", "reference", "--workload", "c1", "--steps", "1", "--warmup", "0"]
try:
    runpy.run_path("bench.py", run_name="__main__")
except SystemExit as e:
    if e.code:
        raise
maps = open("/proc/self/maps").read().split("\\n")
libs = sorted({l.split()[-1] for l in maps if l.endswith(".so") and os.path.realpath(os.getcwd()) in l})
print("LOADED " + " ".join(os.path.relpath(p) for p in libs))
"""


def test_reference_arm_line_has_the_contract_keys():
    """The reference arm's JSON line carries the contract's keys, and the arm runs on the oracle's
    libraries only: its scene arrays and cameras come from the oracle-side generator library, so
    no part of libgrisrt is loaded."""
    out = subprocess.run([sys.executable, "-c", _RUN_AND_LIST], capture_output=True, text=True, timeout=600, cwd=REPO)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    loaded = [l for l in out.stdout.splitlines() if l.startswith("LOADED")][0].split()[1:]
    assert loaded and all(p.startswith("oracle" + os.sep) for p in loaded), loaded
    assert not any("libgrisrt" in p for p in loaded)
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference"
    assert d["unit"] == "frames/s" and d["higher_is_better"] is True
    assert d["steps"] == 1 and d["warmup"] == 0 and d["n_gpus"] == 1
    assert d["value"] > 0 and d["ms_per_step"] == pytest.approx(1000.0 / d["value"])
    assert "workload" in d["config"]
    # the workload only: how an arm ran it (host cores, GPU form, graphs) is in "run"
    assert not {"parallelism", "api", "path_form", "graphs", "autotune"} & set(d["config"])
    assert d["run"]["parallelism"]
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["sample"]
    e = d["e2e"]
    assert e["value"] == d["value"] and e["unit"] == d["unit"]
    assert e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0


def test_launch_count_counts_both_traversal_kernels_of_a_refilling_level():
    import bench
    slots = ["gbuffer", "temporal", "spatial", "wave_begin", "wave_extend", "wave_shade", "wave_shadow", "wave_post"]
    per_frame = {"gbuffer": 1, "temporal": 1, "spatial": 1, "wave_begin": 1, "wave_extend": 7, "wave_shade": 7,
                 "wave_shadow": 7, "wave_post": 7}
    frames = 30
    prof = {s: {"launches": n * frames} for s, n in per_frame.items()}
    assert bench.kernel_launches_per_frame(prof, slots, frames, True, False) == 32
    assert bench.kernel_launches_per_frame(prof, slots, frames, True, True) == 46
    mk = ["gbuffer", "path_trace", "temporal", "spatial"]
    prof_mk = {s: {"launches": frames} for s in mk}
    assert bench.kernel_launches_per_frame(prof_mk, mk, frames, False, True) == 4
