"""sbx_fused_steps_noalloc: SB steps for callers that cannot allocate device
memory (all of it held by their own arena, or a loop that cannot take the
synchronisation cudaMalloc may bring).  The entry point is called through the
C ABI on buffers the caller owns; its result must match sbx_solve's, call
after call, because it shares one static scratch array between calls.

This file is collected last on purpose: if it fails, a run that stops at the
first failure has already run every other test."""
import ctypes as C

import numpy as np
import pytest

import sbx

pytestmark = pytest.mark.gpu

TOL = 1e-4


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-30))


def _entry():
    f = sbx.lib().sbx_fused_steps_noalloc
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_int32, C.c_void_p,
                  C.c_void_p, C.c_double, C.c_double, C.c_int32, C.c_int32, C.c_int32,
                  C.c_void_p]
    f.restype = C.c_int
    return f


def test_noalloc_steps_match_sbx_solve_on_two_calls():
    torch = pytest.importorskip("torch")
    f = _entry()
    g = sbx.gen_er(600, 0.05, pm1=True, seed=3)
    A, max_steps, dt, seed = 64, 1000, 0.2, 5
    ctx = sbx.Context(0)
    prob = ctx.problem(g)
    # period 1: the reference run can stop after any number of steps
    base = dict(dt=dt, steps=max_steps, period=1, agents=A, seed=seed, precision=sbx.F32,
                kernel=sbx.KERNEL_STREAM)
    r, _ = ctx.solve(prob, sbx.params(run_steps=1, **base))
    x0, y0, _ = ctx.state(g.n, A)

    dev = torch.device("cuda", 0)
    rowptr = torch.tensor(g.rowptr, dtype=torch.int32, device=dev)
    col = torch.tensor(g.col, dtype=torch.int32, device=dev)
    val = torch.tensor(g.val.astype(np.float32), device=dev)
    x = torch.tensor(x0.astype(np.float32).reshape(g.n, A), device=dev)
    y = torch.tensor(y0.astype(np.float32).reshape(g.n, A), device=dev)
    stream = torch.cuda.current_stream().cuda_stream

    done = 1
    for nsteps in (40, 60):
        rc = f(rowptr.data_ptr(), col.data_ptr(), val.data_ptr(), g.n, A, x.data_ptr(),
               y.data_ptr(), dt, r["xi0"], done, nsteps, max_steps, stream)
        assert rc == sbx.OK, sbx.lib().sbx_last_error()
        torch.cuda.synchronize()
        done += nsteps
        ctx.solve(prob, sbx.params(run_steps=done, **base))
        xe, ye, _ = ctx.state(g.n, A)
        assert rel(x.cpu().numpy().ravel(), xe) < TOL
        assert rel(y.cpu().numpy().ravel(), ye) < TOL

    # beyond the static array: refused before any work, with the reason
    n_big = sbx.NOALLOC_MAX_WORDS + 1   # agents = 32: one word per row
    rc = f(rowptr.data_ptr(), col.data_ptr(), val.data_ptr(), n_big, 32, x.data_ptr(),
           y.data_ptr(), dt, r["xi0"], 0, 1, max_steps, stream)
    assert rc == -1 and b"exceeds SBX_NOALLOC_MAX_WORDS" in sbx.lib().sbx_last_error()
    ctx.close()
