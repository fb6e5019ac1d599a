"""Host-side checks of the C ABI (no GPU): the library loads and exports
every declared entry point, the loaders reproduce the reference's CSR / TSPLIB
parse (fixtures from the reference's own csr.cpp / tsp_cpu.cpp), errors come
back as status codes, and the generators are seeded and well formed."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, PKG, ROOT

import sbx


def test_library_exports_every_declared_symbol():
    hdr = open(os.path.join(ROOT, "include", "sbx.h")).read()
    declared = set(re.findall(r"\b(sbx_[a-z0-9_]+)\s*\(", hdr))
    assert declared == set(sbx.EXPORTS)
    out = subprocess.run(["nm", "-D", "--defined-only", sbx.LIB_PATH], capture_output=True,
                         text=True, check=True).stdout
    exported = set(re.findall(r" T (sbx_[a-z0-9_]+)", out))
    missing = declared - exported
    assert not missing, missing
    lib = sbx.lib()
    for name in declared:
        assert hasattr(lib, name)


def test_struct_layout_matches_header(tmp_path):
    """The ctypes mirror of sbx_params / sbx_result has the C layout: every
    field at the offset gcc gives it, and the same total size."""
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "sbx.h"', 'int main(void) {']
    for cname, py in (("sbx_params", sbx.Params), ("sbx_result", sbx.Result)):
        lines.append('printf("%s size %%zu\\n", sizeof(%s));' % (cname, cname))
        for f, _ in py._fields_:
            lines.append('printf("%s %s %%zu\\n", offsetof(%s, %s));' % (cname, f, cname, f))
    lines += ['return 0;', '}']
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = dict(l.rsplit(" ", 1) for l in subprocess.run([str(exe)], capture_output=True, text=True,
                                                          check=True).stdout.splitlines())
    for cname, py in (("sbx_params", sbx.Params), ("sbx_result", sbx.Result)):
        assert int(got[cname + " size"]) == C.sizeof(py)
        for f, _ in py._fields_:
            assert int(got["%s %s" % (cname, f)]) == getattr(py, f).offset, (cname, f)


def test_version_and_strerror():
    assert b"sm_103a" in sbx.lib().sbx_version()
    for rc in range(0, -9, -1):
        assert sbx.lib().sbx_strerror(rc)


@pytest.mark.parametrize("name,src", [("load_er40_pm1", "er40_pm1.mtx"),
                                      ("load_er40_real", "er40_real.mtx"),
                                      ("load_ring24_pattern", "ring24_pattern.mtx"),
                                      ("load_gen4_integer", "gen4_integer.mtx")])
def test_mtx_loader_matches_reference(name, src):
    ref = dict(np.load(os.path.join(GOLDEN, name + ".npz")))
    g = sbx.load_mtx(os.path.join(GOLDEN, src))
    assert g.n == ref["size_nnz"][0] and g.nnz == ref["size_nnz"][1]
    np.testing.assert_array_equal(g.rowptr, ref["rowptr"])
    np.testing.assert_array_equal(g.col, ref["col"])
    np.testing.assert_array_equal(g.val, ref["val"])
    assert g.wsum == ref["wsum"][0]


def test_mtx_loader_keeps_empty_rows(tmp_path, oracle):
    # vertex 2 (1-based 3) is isolated: the reference's construct_csr would
    # drop its row pointer (csr.cpp:168-186); both here keep it.
    p = tmp_path / "iso.mtx"
    p.write_text("%%MatrixMarket matrix coordinate pattern symmetric\n4 4 2\n1 2\n2 4\n")
    g = sbx.load_mtx(str(p))
    o = oracle.mtx_load(str(p))
    assert g.n == 4 and list(g.rowptr) == [0, 1, 3, 3, 4]
    np.testing.assert_array_equal(g.rowptr, o.rowptr)
    np.testing.assert_array_equal(g.col, o.col)


@pytest.mark.parametrize("text,rc", [
    (None, -4),
    ("%%MatrixMarket matrix coordinate integer skew\n", -5),
    ("%%MatrixMarket matrix coordinate integer symmetric\n3 3 2\n1 2 1\n", -5),
    ("%%MatrixMarket matrix coordinate integer symmetric\n3 3 1\n1 9 1\n", -5),
])
def test_mtx_errors_are_statuses(tmp_path, text, rc):
    p = tmp_path / "bad.mtx"
    if text is not None:
        p.write_text(text)
    with pytest.raises(sbx.SbxError) as e:
        sbx.load_mtx(str(p))
    assert e.value.rc == rc


@pytest.mark.parametrize("name,src", [("load_euc5", "euc5.tsp"), ("load_geo6", "geo6.tsp")])
def test_tsplib_loader_and_distances(oracle, name, src):
    ref = dict(np.load(os.path.join(GOLDEN, name + ".npz")))
    xc, yc, kind = sbx.load_tsplib(os.path.join(GOLDEN, src))
    np.testing.assert_array_equal(xc, ref["lat"])
    np.testing.assert_array_equal(yc, ref["lon"])
    assert kind == (sbx.DIST_GEO if ref["n_geo"][1] else sbx.DIST_EUC_2D)
    t = oracle.Tsp(xc, yc, kind)
    np.testing.assert_array_equal(sbx.tsp_distances(xc, yc, kind), t.packed)


def test_tsplib_spaced_colon(tmp_path):
    p = tmp_path / "s.tsp"
    p.write_text("NAME : s\nTYPE : TSP\nDIMENSION : 3\nEDGE_WEIGHT_TYPE : EUC_2D\n"
                 "NODE_COORD_SECTION\n1 0 0\n2 3 4\n3 6 8\nEOF\n")
    xc, yc, kind = sbx.load_tsplib(str(p))
    assert list(xc) == [0, 3, 6] and list(yc) == [0, 4, 8] and kind == sbx.DIST_EUC_2D
    assert list(sbx.tsp_distances(xc, yc, kind)) == [5.0, 10.0, 5.0]


def _check_symmetric(g):
    n = g.n
    assert g.rowptr[0] == 0 and g.rowptr[-1] == g.nnz
    assert np.all(np.diff(g.rowptr) >= 0)
    rows = np.repeat(np.arange(n), np.diff(g.rowptr))
    assert np.all(rows != g.col)
    fwd = set(zip(rows.tolist(), g.col.tolist(), g.val.tolist()))
    assert all((c, r, v) in fwd for r, c, v in fwd)
    assert abs(g.wsum - g.val.sum() / 2) < 1e-9


def test_generators_are_seeded_and_well_formed():
    g = sbx.gen_er(800, 0.0601, pm1=False, seed=1234)
    _check_symmetric(g)
    assert 34000 < g.nnz < 43000 and np.all(g.val == 1.0)
    g2 = sbx.gen_er(800, 0.0601, pm1=False, seed=1234)
    np.testing.assert_array_equal(g.col, g2.col)
    t = sbx.gen_torus(100, 100, seed=1234)
    _check_symmetric(t)
    assert t.nnz == 40000 and set(np.diff(t.rowptr).tolist()) == {4}
    assert set(np.unique(t.val).tolist()) == {-1.0, 1.0}
    r = sbx.gen_rmat(12, 4, seed=7)
    _check_symmetric(r)
    rows = np.repeat(np.arange(r.n), np.diff(r.rowptr))
    assert len(set(zip(rows.tolist(), r.col.tolist()))) == r.nnz   # no duplicates
    q = sbx.gen_rgg(2000, 10.0, seed=3)
    _check_symmetric(q)
    assert 6 < q.nnz / q.n < 12
    xc, yc = sbx.gen_cities(30, 1.0, seed=5)
    assert xc.min() >= 0 and xc.max() < 1 and yc.min() >= 0 and yc.max() < 1


def test_cli_usage_and_errors(tmp_path):
    prog = os.path.join(PKG, "program")
    r = subprocess.run([prog], capture_output=True, text=True)
    assert r.returncode != 0 and "usage: ./program" in r.stdout
    r = subprocess.run([prog, "0", "x.mtx", "o.csv", "maxcut"], capture_output=True, text=True)
    assert r.returncode != 0 and "usage" in r.stdout
    r = subprocess.run([prog, "1", str(tmp_path / "missing.mtx"), str(tmp_path / "o.csv")],
                       capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "cannot open" in r.stderr


def _big_mtx(path, n=200000, m=1200000, seed=4, real=True, split_one=False):
    rng = np.random.default_rng(seed)
    r = rng.integers(1, n + 1, m)
    c = rng.integers(1, n + 1, m)
    c[::97] = r[::97]                      # some diagonal entries, dropped on load
    v = np.round(rng.normal(0, 1, m), 4)
    with open(path, "w") as f:
        f.write("%%MatrixMarket matrix coordinate real symmetric\n%% generated\n")
        f.write("%d %d %d\n" % (n, n, m))
        lines = ["%d %d %.4f" % t for t in zip(r, c, v)] if real else ["%d %d" % t for t in zip(r, c)]
        if split_one:
            k = len(lines) // 2
            a, b, w = lines[k].split(" ")
            lines[k] = a + "\n" + b + " " + w   # one entry over two lines
        f.write("\n".join(lines) + "\n")


@pytest.mark.parametrize("split_one", [False, True])
def test_large_mtx_parallel_parse_matches_oracle(tmp_path, oracle, split_one):
    # bodies over 8 MB are parsed by every host thread; an entry spread over
    # two lines sends the file back to the sequential parse
    path = str(tmp_path / "big.mtx")
    _big_mtx(path, split_one=split_one)
    assert os.path.getsize(path) > 8 << 20
    g = sbx.load_mtx(path)
    ref = oracle.mtx_load(path)
    assert g.n == ref.n
    np.testing.assert_array_equal(g.rowptr, ref.rowptr)
    np.testing.assert_array_equal(g.col, ref.col)
    np.testing.assert_array_equal(g.val, ref.val)
    assert g.wsum == ref.wsum


def test_large_mtx_errors(tmp_path):
    path = str(tmp_path / "bad.mtx")
    _big_mtx(path)
    with open(path) as f:
        text = f.read()
    k = len(text) * 3 // 4
    k = text.index("\n", k) + 1
    with open(path, "w") as f:
        f.write(text[:k] + "12 x 0.5\n" + text[k:])      # a malformed entry in a late piece
    n = C.c_int64()
    nnz = C.c_int64()
    w = C.c_double()
    rc = sbx.lib().sbx_load_mtx(path.encode(), C.byref(n), C.byref(nnz), None, None, None, C.byref(w))
    assert rc == -5
    with open(path, "w") as f:
        f.write(text[:len(text) // 2])                   # fewer entries than announced
    rc = sbx.lib().sbx_load_mtx(path.encode(), C.byref(n), C.byref(nnz), None, None, None, C.byref(w))
    assert rc == -5
