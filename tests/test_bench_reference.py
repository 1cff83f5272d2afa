"""The bench's reference arm runs on the host alone (the oracle's OpenMP FP32
path): its JSON line carries the contract's keys, every step evaluates a fixed
sample of at least 128 whole cells whatever --steps is, ms_per_step is the
time of the steps actually run, and the GPU library is never loaded in that
process.  A small grid keeps it to seconds; no GPU needed."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

RUN = """
import json, sys
sys.path.insert(0, {root!r})
sys.argv = ["bench.py"] + {argv!r}
import bench
bench.main()
maps = open("/proc/self/maps").read()
print(json.dumps({{"gpu_library_loaded": "libgpu_determ" in maps}}))
"""


def _run(argv):
    r = subprocess.run([sys.executable, "-c", RUN.format(root=ROOT, argv=argv)], capture_output=True, text=True,
                       cwd=ROOT, timeout=600)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.strip().splitlines()
    return json.loads(lines[-2]), json.loads(lines[-1])


def test_reference_arm_json_line(gdlib):
    line, maps = _run(["--impl", "reference", "--grid", "8", "--radius", "16.5", "--cells", "256",
                       "--steps", "20", "--warmup", "2"])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference" and line["value"] > 0 and line["higher_is_better"] is True
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["value"] == line["value"]
    # a fixed sample of >= 128 whole cells per step, independent of --steps
    assert line["config"]["sample_cells"] >= 128 and line["config"]["cells"] == 256
    assert line["cpu_baseline"]["sample"].startswith("128 cell(s)")
    # ms_per_step is the measured time of one step of those cells
    assert abs(line["ms_per_step"] - 1000.0 * 128 / line["value"]) < 1e-6 * line["ms_per_step"]
    assert maps["gpu_library_loaded"] is False
