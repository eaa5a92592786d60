"""The benchmark's reference arm on the host: `bench.py --impl reference`
prints one JSON line with the keys of the benchmark line, the reference
marker, a CPU baseline describing the run and an end-to-end block with no
host-device copies.  (The reference arm runs the reference CPU program, or
the oracle's restatement when that program was not built; no GPU.)"""
import json
import os
import subprocess
import sys

from conftest import ROOT

KEYS = ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
        "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e")


def test_reference_arm_prints_one_contract_line(built):
    env = dict(os.environ, PYTHONPATH=ROOT)
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "3"], cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert all(k in line for k in KEYS), [k for k in KEYS if k not in line]
    assert line["impl"] == "reference" and line["higher_is_better"] is True and line["n_gpus"] == 1
    assert line["value"] > 0 and line["metric"] == line["unit"] == "Gcell-updates/s"
    assert line["steps"] == 1 and line["warmup"] >= 3
    cpu = line["cpu_baseline"]
    assert cpu["value"] == line["value"] and cpu["cores"] >= 1 and cpu["kind"] in ("reference", "port")
    assert line["e2e"] == {"value": line["value"], "unit": line["unit"], "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    assert line["config"]["grid"] == [256, 256, 256]
