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


def test_restart_copies_keep_a_round_near_a_tenth_of_the_batch():
    # the batch time-to-target's restart rounds: copies of each missed
    # instance sized to the round's rows, clamped to [1, 32]
    sys.path.insert(0, ROOT)
    import bench
    n = 1_908_368
    assert bench.restart_copies(139_000, n) == 1      # many misses: one copy each
    assert bench.restart_copies(50_000, n) == 3
    assert bench.restart_copies(5_000, n) == 32       # a few small ones: the cap
    assert bench.restart_copies(n, n) == 1
    assert bench.restart_copies(0, n) == 32           # nothing missed: never divides by zero
    for rows in (100, 1_000, 10_000, 100_000, 1_000_000):
        c = bench.restart_copies(rows, n)
        assert 1 <= c <= bench.RESTART_MAX_COPIES
        assert c == 1 or c * rows <= bench.RESTART_ROWS * n
