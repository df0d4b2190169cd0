"""The reference arm of bench.py on CPU (a small case): one JSON line with the contract's keys, the same
workload config as the GPU arm apart from the precision, whole steps timed."""
import json
import os
import subprocess
import sys

from conftest import ROOT


def test_reference_arm_line():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--n", "12",
                          "--steps", "2", "--warmup", "1"], capture_output=True, text=True, timeout=600, check=True,
                         cwd=ROOT).stdout.strip().splitlines()
    line = json.loads(out[-1])
    assert line["impl"] == "reference"
    assert line["unit"] == "DoF/s" and line["value"] > 0 and line["higher_is_better"] is True
    assert line["steps"] == 2 and line["warmup"] == 1
    assert line["config"]["dofs"] == 13 ** 3 and line["config"]["precision"] == "fp64"
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"] and cb["sample"]
    assert line["e2e"] == {"value": line["value"], "unit": "DoF/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    assert line["consistency"]["same_config"] is True and line["consistency"]["fits_in_driver_run"] is True
    assert line["single_thread"]["cores"] == 1 and line["single_thread"]["iterations"] > 0
