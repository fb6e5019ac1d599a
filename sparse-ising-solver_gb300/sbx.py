"""ctypes binding of libsbx.so (include/sbx.h) for Python callers.

The engine is the C ABI; this module only marshals numpy arrays across it.
It loads the in-tree libsbx.so and raises if it is missing: there is no
Python or CPU fallback for the solver.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libsbx.so")

OK = 0
ERR_ARG, ERR_CUDA, ERR_NOMEM, ERR_IO, ERR_FORMAT, ERR_UNSUPPORTED, ERR_NODEVICE, ERR_STATE = \
    -1, -2, -3, -4, -5, -6, -7, -8
F32, BF16, F16, F64 = 0, 1, 2, 3
KERNEL_AUTO, KERNEL_STREAM, KERNEL_RESIDENT, KERNEL_RESIDENT_SPLIT, KERNEL_TENSOR = 0, 1, 2, 3, 4
DIST_EUC_2D, DIST_GEO, DIST_EUC_2D_FLOAT = 0, 1, 2
FLAG_NO_PDL, FLAG_NO_GRAPH, FLAG_PROFILE, FLAG_NO_TUNE, FLAG_TEST_GIVEUP = 1, 2, 4, 8, 16
PRECISIONS = {"f32": F32, "bf16": BF16, "f16": F16, "f64": F64}
NOALLOC_MAX_WORDS = 1 << 21   # SBX_NOALLOC_MAX_WORDS in include/sbx.h

# Every function include/sbx.h declares (checked by the CPU tests).
EXPORTS = [
    "sbx_strerror", "sbx_last_error", "sbx_version", "sbx_params_default", "sbx_create",
    "sbx_destroy", "sbx_set_stream", "sbx_problem_csr", "sbx_problem_tsp",
    "sbx_problem_destroy", "sbx_problem_info", "sbx_solve", "sbx_get_state", "sbx_get_tours",
    "sbx_get_trace", "sbx_solve_batch", "sbx_load_mtx", "sbx_load_tsplib",
    "sbx_tsp_distances", "sbx_gen_er", "sbx_gen_torus", "sbx_gen_rmat", "sbx_gen_rgg",
    "sbx_gen_cities", "sbx_fused_steps_noalloc", "sbx_get_batch_state",
    "sbx_problem_tsp_cities",
]


class Params(C.Structure):
    _fields_ = [("dt", C.c_double), ("steps", C.c_int32), ("agents", C.c_int32),
                ("fused", C.c_int32), ("update_window", C.c_int32), ("period", C.c_int32),
                ("threshold", C.c_int32), ("precision", C.c_int32), ("seed", C.c_uint32),
                ("kernel", C.c_int32), ("agents_per_block", C.c_int32), ("trace", C.c_int32),
                ("flags", C.c_uint32), ("run_steps", C.c_int32), ("lane_agents", C.c_int32),
                ("row_lanes", C.c_int32), ("block_threads", C.c_int32), ("count_mode", C.c_int32),
                ("staging", C.c_int32), ("target", C.c_double)]


class Result(C.Structure):
    _fields_ = [("time_us", C.c_double), ("min", C.c_double), ("max", C.c_double),
                ("mean", C.c_double), ("std", C.c_double), ("ps", C.c_double),
                ("xi0", C.c_double), ("steps_run", C.c_int64), ("windows_run", C.c_int64),
                ("bifurcated", C.c_int64), ("valid", C.c_int64), ("best_agent", C.c_int32),
                ("kernel_used", C.c_int32), ("agents_per_block", C.c_int32),
                ("lane_agents", C.c_int32), ("row_lanes", C.c_int32), ("block_threads", C.c_int32),
                ("count_mode", C.c_int32), ("staging", C.c_int32), ("kernel_ms", C.c_double), ("kernel_launches", C.c_int64),
                ("gpu_launches", C.c_int64), ("time_to_target_us", C.c_double),
                ("steps_to_target", C.c_int64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class SbxError(RuntimeError):
    def __init__(self, what, rc):
        msg = lib().sbx_strerror(rc).decode()
        detail = lib().sbx_last_error().decode()
        super().__init__("%s: %s (%d)%s" % (what, msg, rc, (": " + detail) if detail else ""))
        self.rc = rc


def build():
    subprocess.run(["make", "-s", "-C", HERE, "-j8"], check=True)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libsbx.so is not built (run __graft_entry__.build() or make -C %s)" % HERE)
        _lib = C.CDLL(LIB_PATH)
        _lib.sbx_strerror.restype = C.c_char_p
        _lib.sbx_last_error.restype = C.c_char_p
        _lib.sbx_version.restype = C.c_char_p
    return _lib


def _check(what, rc):
    if rc != OK:
        raise SbxError(what, rc)


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def params(**kw):
    p = Params()
    lib().sbx_params_default(C.byref(p))
    for k, v in kw.items():
        if k == "precision" and isinstance(v, str):
            v = PRECISIONS[v]
        setattr(p, k, v)
    return p


class Graph:
    """Host CSR (int32 row pointers and columns, float64 weights) + W."""

    def __init__(self, n, rowptr, col, val, wsum):
        self.n = int(n)
        self.rowptr = np.ascontiguousarray(rowptr, np.int32)
        self.col = np.ascontiguousarray(col, np.int32)
        self.val = np.ascontiguousarray(val, np.float64)
        self.wsum = float(wsum)

    @property
    def nnz(self):
        return int(self.col.size)


def _two_call(fn, *args):
    nnz = C.c_int64()
    w = C.c_double()
    _check(fn.__name__, fn(*args, C.byref(nnz), None, None, None, C.byref(w)))
    return nnz.value


def load_mtx(path):
    n = C.c_int64()
    nnz = C.c_int64()
    w = C.c_double()
    _check("sbx_load_mtx", lib().sbx_load_mtx(path.encode(), C.byref(n), C.byref(nnz), None, None,
                                                None, C.byref(w)))
    rp = np.empty(n.value + 1, np.int32)
    col = np.empty(nnz.value, np.int32)
    val = np.empty(nnz.value)
    _check("sbx_load_mtx", lib().sbx_load_mtx(path.encode(), C.byref(n), C.byref(nnz), _p(rp),
                                                _p(col), _p(val), C.byref(w)))
    return Graph(n.value, rp, col, val, w.value)


def load_tsplib(path):
    N = C.c_int32()
    kind = C.c_int32()
    _check("sbx_load_tsplib", lib().sbx_load_tsplib(path.encode(), C.byref(N), None, None,
                                                      C.byref(kind)))
    xc = np.empty(N.value)
    yc = np.empty(N.value)
    _check("sbx_load_tsplib", lib().sbx_load_tsplib(path.encode(), C.byref(N), _p(xc), _p(yc),
                                                      C.byref(kind)))
    return xc, yc, kind.value


def tsp_distances(xc, yc, kind):
    xc = np.ascontiguousarray(xc, np.float64)
    yc = np.ascontiguousarray(yc, np.float64)
    N = xc.size
    out = np.empty(N * (N - 1) // 2)
    _check("sbx_tsp_distances", lib().sbx_tsp_distances(C.c_int32(N), _p(xc), _p(yc),
                                                          C.c_int32(kind), _p(out)))
    return out


def _gen(name, n, argtypes_and_values):
    fn = getattr(lib(), name)
    nnz = C.c_int64()
    w = C.c_double()
    _check(name, fn(*argtypes_and_values, C.byref(nnz), None, None, None, C.byref(w)))
    rp = np.empty(n + 1, np.int32)
    col = np.empty(nnz.value, np.int32)
    val = np.empty(nnz.value)
    _check(name, fn(*argtypes_and_values, C.byref(nnz), _p(rp), _p(col), _p(val), C.byref(w)))
    return Graph(n, rp, col, val, w.value)


def gen_er(n, p, pm1=False, seed=1234):
    return _gen("sbx_gen_er", n, [C.c_int64(n), C.c_double(p), C.c_int32(int(pm1)),
                                  C.c_uint64(seed)])


def gen_torus(rows, cols, seed=1234):
    return _gen("sbx_gen_torus", rows * cols, [C.c_int32(rows), C.c_int32(cols), C.c_uint64(seed)])


def gen_rmat(scale, edge_factor=4, a=0.57, b=0.19, c=0.19, seed=1234):
    return _gen("sbx_gen_rmat", 1 << scale, [C.c_int32(scale), C.c_int32(edge_factor),
                                             C.c_double(a), C.c_double(b), C.c_double(c),
                                             C.c_uint64(seed)])


def gen_rgg(n, avg_degree, seed=1234):
    return _gen("sbx_gen_rgg", n, [C.c_int64(n), C.c_double(avg_degree), C.c_uint64(seed)])


def gen_cities(N, scale=1.0, seed=1234):
    xc = np.empty(N)
    yc = np.empty(N)
    _check("sbx_gen_cities", lib().sbx_gen_cities(C.c_int32(N), C.c_double(scale),
                                                    C.c_uint64(seed), _p(xc), _p(yc)))
    return xc, yc


class Context:
    """An engine context on one CUDA device (sbx_create)."""

    def __init__(self, device=0):
        self._c = C.c_void_p()
        _check("sbx_create", lib().sbx_create(C.byref(self._c), C.c_int(device)))

    def close(self):
        if self._c:
            lib().sbx_destroy(self._c)
            self._c = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream_handle):
        _check("sbx_set_stream", lib().sbx_set_stream(self._c, C.c_void_p(stream_handle)))

    def problem(self, g):
        p = C.c_void_p()
        _check("sbx_problem_csr", lib().sbx_problem_csr(
            self._c, C.c_int64(g.n), C.c_int64(g.nnz), _p(g.rowptr), _p(g.col), _p(g.val),
            C.c_double(g.wsum), C.byref(p)))
        return Problem(self, p, g.n, False)

    def tsp_problem(self, packed, N, A=1.0, B=None, C_=None):
        packed = np.ascontiguousarray(packed, np.float64)
        mx = float(packed.max()) if packed.size else 0.0
        B = mx if B is None else B
        C_ = mx if C_ is None else C_
        p = C.c_void_p()
        _check("sbx_problem_tsp", lib().sbx_problem_tsp(
            self._c, C.c_int32(N), _p(packed), C.c_double(A), C.c_double(B), C.c_double(C_),
            C.byref(p)))
        return Problem(self, p, N * N, True, N=N, packed=packed)

    def tsp_problem_cities(self, xc, yc, kind, A=1.0, penalty_scale=1.0):
        """TSP problem from city coordinates, distances computed on the device."""
        xc = np.ascontiguousarray(xc, np.float64)
        yc = np.ascontiguousarray(yc, np.float64)
        N = int(xc.size)
        p = C.c_void_p()
        _check("sbx_problem_tsp_cities", lib().sbx_problem_tsp_cities(
            self._c, C.c_int32(N), _p(xc), _p(yc), C.c_int32(kind), C.c_double(A),
            C.c_double(penalty_scale), C.byref(p)))
        return Problem(self, p, N * N, True, N=N)

    def solve(self, prob, prm, want_values=True):
        r = Result()
        vals = np.empty(prm.agents) if want_values else None
        _check("sbx_solve", lib().sbx_solve(self._c, prob._p, C.byref(prm), C.byref(r), _p(vals)))
        return r.as_dict(), vals

    def solve_batch(self, probs, agents, prm, targets=None):
        n = len(probs)
        arr = (C.c_void_p * n)(*[p._p for p in probs])
        ag = np.ascontiguousarray(agents, np.int32)
        tg = None if targets is None else np.ascontiguousarray(targets, np.float64)
        res = (Result * n)()
        vals = np.empty(int(ag.sum()))
        t = C.c_double()
        _check("sbx_solve_batch", lib().sbx_solve_batch(self._c, C.c_int32(n), arr, _p(ag),
                                                        C.byref(prm), _p(tg), res, _p(vals),
                                                        C.byref(t)))
        return [r.as_dict() for r in res], vals, t.value

    def state(self, n, agents):
        x = np.empty(n * agents)
        y = np.empty(n * agents)
        s = np.empty(n * agents, np.int32)
        _check("sbx_get_state", lib().sbx_get_state(self._c, _p(x), _p(y), _p(s)))
        return x, y, s

    def batch_state(self, index, n, agents):
        """x, y, window spins of instance `index` of the last batched solve."""
        x = np.empty(n * agents)
        y = np.empty(n * agents)
        s = np.empty(n * agents, np.int32)
        _check("sbx_get_batch_state", lib().sbx_get_batch_state(self._c, C.c_int32(index), _p(x),
                                                                _p(y), _p(s)))
        return x, y, s

    def trace(self, cap=1 << 16):
        """Per-window (steps, best cut, microseconds) of the last traced solve."""
        st = np.empty(cap, np.int64)
        b = np.empty(cap)
        t = np.empty(cap)
        cnt = C.c_int64()
        _check("sbx_get_trace", lib().sbx_get_trace(self._c, C.c_int64(cap), _p(st), _p(b), _p(t),
                                                    C.byref(cnt)))
        k = min(cnt.value, cap)
        return st[:k].copy(), b[:k].copy(), t[:k].copy()

    def tours(self, N, agents):
        t = np.empty(N * agents, np.int32)
        v = np.empty(agents, np.int32)
        _check("sbx_get_tours", lib().sbx_get_tours(self._c, _p(t), _p(v)))
        return t.reshape(agents, N), v


class Problem:
    def __init__(self, ctx, handle, n, tsp, N=0, packed=None):
        self.ctx = ctx
        self._p = handle
        self.n = n
        self.tsp = tsp
        self.N = N
        self.packed = packed

    def close(self):
        if self._p:
            lib().sbx_problem_destroy(self._p)
            self._p = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
