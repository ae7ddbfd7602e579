"""The benchmark's reference arm (`bench.py --impl reference`) runs on the host cores alone: the
CPU path of the reference's algorithm (the oracle) on the benchmark's workload, one JSON line
with the contract's keys, its end-to-end entry equal to its value with no device traffic."""
import json
import os
import subprocess
import sys

from conftest import ROOT


def test_reference_arm_prints_the_contract_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "3"], cwd=ROOT, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-2000:]
    d = json.loads(r.stdout.strip().splitlines()[-1])
    assert d["impl"] == "reference"
    assert d["metric"] == "cell_updates_per_s" and d["unit"] == "cell-updates/s" and d["higher_is_better"] is True
    assert d["value"] > 0 and d["steps"] == 1 and d["warmup"] >= 3
    assert d["config"]["workload"] == "rotor_passage_129x49x49_2level_multigrid"
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    base = d["cpu_baseline"]
    assert base["value"] == d["value"] and base["kind"] in ("port", "reference") and base["cores"] >= 1
