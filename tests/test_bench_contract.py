"""The bench's CPU arm (no GPU): `bench.py --impl reference` runs the CPU
implementation of the path (the FP64 oracle on every host thread) on a
bounded sample of a workload and prints one JSON line with the keys the
measurement contract asks for; ranks other than 0 print nothing."""
import json
import os
import subprocess
import sys

from conftest import ROOT


def _run(extra_env=None, workload=("--workload", "er800")):
    env = dict(os.environ)
    env.update(extra_env or {})
    return subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                           *workload, "--steps", "1", "--warmup", "0"],
                          capture_output=True, text=True, timeout=300, env=env, cwd=ROOT)


def test_reference_arm_prints_one_contract_line():
    p = _run()
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [l for l in p.stdout.splitlines() if l.strip().startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["metric"] == "nnz*agent*steps/s" and d["unit"] == "nnz*agent*steps/s"
    assert d["value"] > 0 and d["higher_is_better"] is True
    assert d["steps"] == 1 and d["warmup"] == 0 and d["ms_per_step"] > 0
    assert d["config"]["workload"].startswith("maxcut-er-800")
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] == "port" and cb["cores"] >= 1 and cb["sample"]
    e2e = d["e2e"]
    assert e2e["value"] == d["value"] and e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_reference_arm_other_ranks_exit_quietly():
    p = _run({"RANK": "1", "WORLD_SIZE": "2"})
    assert p.returncode == 0, p.stderr[-2000:]
    assert not [l for l in p.stdout.splitlines() if l.strip().startswith("{")]


def test_reference_arm_batch_loads_no_engine_code():
    # The default (batched) workload: its instances come from the oracle's
    # generators, so the arm never maps the engine's library.
    code = ("import runpy, sys; sys.argv = ['bench.py', '--impl', 'reference', '--instances', '12', "
            "'--steps', '1', '--warmup', '0']; runpy.run_path('bench.py', run_name='__main__'); "
            "print('MAPS', open('/proc/self/maps').read().count('libsbx'))")
    p = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300,
                       cwd=ROOT)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [l for l in p.stdout.splitlines() if l.strip().startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0
    assert d["config"]["workload"].startswith("batch-512")
    assert "12 instances" in d["cpu_baseline"]["sample"]
    assert "MAPS 0" in p.stdout
