"""The drop-in CLI end to end on the GPU: `program` with the reference's
arguments appends the reference's output-file line, every field checked
against the oracle's statistics of the same run, formatted as std::ofstream
formats a double by default (6 significant digits, %g).

  MaxCut line: time,min,max,avg,std,ps,   (src/ising.cu:267)
               file,n,nnz,max_steps,time_step,agents   (src/main.cu:223)
  TSP line:    time, min, max, mean, std, valid,   (src/ising_tsp.cu:248)
"""
import os
import subprocess

import numpy as np
import pytest

import sbx
from conftest import GOLDEN, PKG

pytestmark = pytest.mark.gpu

PROGRAM = os.path.join(PKG, "program")


def g6(v):
    return "%g" % v


def run_program(args, tmp_path):
    out = tmp_path / "out.csv"
    p = subprocess.run([PROGRAM, *args[:1], args[1], str(out), *args[2:]], capture_output=True,
                       text=True, timeout=600)
    assert p.returncode == 0, p.stdout + p.stderr
    lines = out.read_text().splitlines()
    assert len(lines) == 1
    return lines[0], p.stdout


def test_maxcut_output_line_matches_the_oracle(oracle, tmp_path):
    mtx = os.path.join(GOLDEN, "er40_pm1.mtx")
    seed, steps, dt, A = 4321, 300, 0.1, 64
    line, stdout = run_program(["0", mtx, "maxcut", "0", "1", "0", str(dt), str(steps), str(A),
                                "--seed=%d" % seed, "--precision=f64"], tmp_path)
    g = oracle.mtx_load(mtx)
    o = oracle.maxcut_solve(g, oracle.params(dt=dt, steps=steps, agents=A, seed=seed))["result"]
    f = line.split(",")
    assert len(f) == 12
    assert int(f[0]) >= 0                               # microseconds of the SB loop
    assert f[1:6] == [g6(o["min"]), g6(o["max"]), g6(o["mean"]), g6(o["std"]), g6(o["ps"])]
    assert f[6:] == [mtx, str(g.n), str(g.nnz), str(steps), g6(dt), str(A)]
    assert "max: %s" % g6(o["max"]) in stdout


def test_maxcut_unfused_update_window_line(oracle, tmp_path):
    mtx = os.path.join(GOLDEN, "er40_pm1.mtx")
    seed, steps, dt, A = 77, 5000, 0.3, 40
    line, _ = run_program(["0", mtx, "maxcut", "1", "0", "1", str(dt), str(steps), str(A),
                           "--seed=%d" % seed, "--precision=f64"], tmp_path)
    g = oracle.mtx_load(mtx)
    o = oracle.maxcut_solve(g, oracle.params(dt=dt, steps=steps, agents=A, seed=seed, uw=1,
                                             fused=0))["result"]
    f = line.split(",")
    assert f[1:6] == [g6(o["min"]), g6(o["max"]), g6(o["mean"]), g6(o["std"]), g6(o["ps"])]


def test_tsp_default_settings_line_matches_the_oracle(oracle, tmp_path):
    # `program 1 file.tsp out`: the reference's fixed TSP settings (dt 0.1,
    # 10,000 steps, 10,000 agents), FP64 state
    tsp = os.path.join(GOLDEN, "euc5.tsp")
    seed = 99
    line, stdout = run_program(["1", tsp, "--seed=%d" % seed, "--precision=f64"], tmp_path)
    xc, yc, kind = oracle.tsplib_load(tsp)
    t = oracle.Tsp(xc, yc, kind)
    o = t.solve(oracle.params(dt=0.1, steps=10000, agents=10000, seed=seed, threshold=50))
    r = o["result"]
    f = [v.strip() for v in line.split(",")]
    assert f[-1] == "" and len(f) == 7
    assert int(f[0]) >= 0
    assert f[1:6] == [g6(r["min"]), g6(r["max"]), g6(r["mean"]), g6(r["std"]), str(r["valid"])]
    assert "vagents: %d" % r["valid"] in stdout
