"""Host-side engine logic without a GPU: the library loads and exports the
C ABI, the load balancer matches the reference's, and the phase flattening
of reference zone trees reproduces the reference execution order."""
import ctypes as C
import pathlib
import re

import numpy as np
import pytest

from cases import COLOR3_CASES, COLOR_CASES, EXEC_CASES, digest, key_color, key_color3
from oracle import oracle as orc
from oracle.refpy import parse_zone_tree
from race_gb300 import _lib, matgen

ROOT = pathlib.Path(__file__).resolve().parents[1]


def _header_functions():
    text = (ROOT / "include" / "race_gb300.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(race_[a-z_0-9]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    L = _lib.lib()
    declared = _header_functions()
    assert declared, "no functions parsed from the header"
    for name in declared:
        assert hasattr(L, name), name
    assert sorted(_lib.EXPORTS) == declared


def test_every_handle_entry_point_rejects_a_null_handle():
    """Every entry point taking an engine, batch or MLP handle returns
    RACE_ERR_INVALID_ARG for NULL (no GPU needed, nothing dereferenced);
    the destroy calls accept NULL as a no-op, like free."""
    L = _lib.lib()
    text = re.sub(r"/\*.*?\*/", "", (ROOT / "include" / "race_gb300.h").read_text(), flags=re.S)
    names = sorted(set(re.findall(
        r"int\s+(race_[a-z_0-9]+)\s*\(\s*(?:const\s+)?race_(?:engine|batch|mlp)\s*\*\s*\w+\s*[,)]", text)))
    assert len(names) >= 40
    for name in names:
        f = getattr(L, name)
        args = [0 if t in (C.c_int, C.c_longlong) else 0.0 if t in (C.c_double, C.c_float) else None
                for t in f.argtypes]
        want = _lib.RACE_SUCCESS if name.endswith("destroy") else _lib.RACE_ERR_INVALID_ARG
        assert f(*args) == want, name


def _lb(levelRow, levelNnz, nt, eff, dist, tgt, base=7, d2type=0):
    L = _lib.lib()
    lr = np.ascontiguousarray(levelRow, np.int32)
    ln = np.ascontiguousarray(levelNnz, np.int32)
    n = C.c_int()
    _lib.check(L.race_lb_balance(lr.ctypes.data, ln.ctypes.data, lr.size, nt, eff, dist, d2type, tgt, base, None, 0,
                                 C.byref(n)))
    out = np.zeros(n.value, np.int32)
    _lib.check(L.race_lb_balance(lr.ctypes.data, ln.ctypes.data, lr.size, nt, eff, dist, d2type, tgt, base,
                                 out.ctypes.data, n.value, C.byref(n)))
    return out


def test_load_balancer_three_block_matches_reference(golden):
    """RACE::THREE_BLOCK (three blocks per thread, gap 1; macros.h:29-38)."""
    idx = golden["lb3__index"]
    off = golden["lb3__offsets"]
    data = golden["lb3__data"]
    for i, key in enumerate(idx):
        m, nt, eff, tgt = str(key).split("|")
        k = f"trav__{m}__d2"
        got = _lb(golden[k + "__levelRow"], golden[k + "__levelNnz"], int(nt), float(eff), 2, int(tgt), d2type=1)
        np.testing.assert_array_equal(got, data[off[i]:off[i + 1]], err_msg=str(key))


def test_load_balancer_matches_reference(golden):
    idx = golden["lb__index"]
    off = golden["lb__offsets"]
    data = golden["lb__data"]
    for i, key in enumerate(idx):
        m, d, nt, eff, tgt = str(key).split("|")
        k = f"trav__{m}__d{d}"
        got = _lb(golden[k + "__levelRow"], golden[k + "__levelNnz"], int(nt), float(eff), int(d), int(tgt))
        np.testing.assert_array_equal(got, data[off[i]:off[i + 1]], err_msg=str(key))


def _flatten(tree_flat, dist, rev, n, d2type=0):
    L = _lib.lib()
    t = np.ascontiguousarray(tree_flat, np.int32)
    npz, nl = C.c_int(), C.c_int()
    _lib.check(L.race_flatten_zone_tree(t.ctypes.data, t.size, dist, d2type, int(rev), n, n, None, None, None, 0,
                                        C.byref(npz), C.byref(nl)))
    cap = max(nl.value, npz.value + 1)
    pp = np.zeros(cap, np.int32); lo = np.zeros(cap, np.int32); hi = np.zeros(cap, np.int32)
    _lib.check(L.race_flatten_zone_tree(t.ctypes.data, t.size, dist, d2type, int(rev), n, n, pp.ctypes.data,
                                        lo.ctypes.data, hi.ctypes.data, cap, C.byref(npz), C.byref(nl)))
    return pp[:npz.value + 1], lo[:nl.value], hi[:nl.value]


@pytest.mark.parametrize("m,d,t", COLOR_CASES)
def test_phases_cover_every_row_once(golden, mats, m, d, t):
    A = mats[m]
    k = key_color(m, d, t)
    for rev in (False, True):
        pp, lo, hi = _flatten(golden[k + "__tree"], d, rev, A.n)
        seen = np.zeros(A.n, np.int32)
        for a, b in zip(lo, hi):
            if a <= b:
                seen[a:b] += 1
            else:
                seen[b + 1:a + 1] += 1
        assert (seen == 1).all()


def _run_phases(pp, lo, hi, kern, mat, x, b):
    for p in range(len(pp) - 1):
        for l in range(pp[p], pp[p + 1]):
            orc.run_kernel(kern, int(lo[l]), int(hi[l]), mat, x, b)


@pytest.mark.parametrize("m,d,t", sorted(EXEC_CASES) + [("lap7_32", 2, 1024), ("lap7_32", 1, 256)])
def test_phases_reproduce_reference_order(golden, mats, m, d, t):
    """Running the kernels phase by phase over the flattened phases gives the
    same bits as the reference's recursive execution order."""
    A = mats[m]
    k = key_color(m, d, t)
    perm = golden[k + "__perm"]
    inv = np.empty_like(perm); inv[perm] = np.arange(A.n, dtype=np.int32)
    P = A.permuted(perm, inv)
    U = P.upper()
    nodes = parse_zone_tree(golden[k + "__tree"])
    x0 = matgen.uniform_vector(A.n, 0)
    b0 = matgen.uniform_vector(A.n, 1)
    kernels = [(orc.K_GS, P, False), (orc.K_GS, P, True)]
    if d == 2:
        kernels += [(orc.K_SYMMSPMV, U, False), (orc.K_KACZ, P, False), (orc.K_KACZ, P, True)]
    for kern, mat, rev in kernels:
        x1, b1 = x0.copy(), (np.zeros(A.n) if kern == orc.K_SYMMSPMV else b0.copy())
        x2, b2 = x1.copy(), b1.copy()
        orc.exec_tree(nodes, 2, golden[k + "__serial"], kern, rev, mat, x1, b1)
        pp, lo, hi = _flatten(golden[k + "__tree"], d, rev, A.n)
        _run_phases(pp, lo, hi, kern, mat, x2, b2)
        np.testing.assert_array_equal(x1, x2)
        np.testing.assert_array_equal(b1, b2)


def test_cpp_header_compiles(tmp_path):
    """The header-only C++ Interface (include/race_gb300.hpp) compiles against
    the C ABI and exposes the reference's method names."""
    import shutil
    import subprocess
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    src = tmp_path / "use.cpp"
    src.write_text("""
#include "race_gb300.hpp"
int use(int n, int *rp, int *col, race_operands ops) {
    RACE::gb300::Interface ce(n, 8, RACE::gb300::POWER, rp, col, true);
    int rc = ce.RACEColor(4, 1e6);
    int *perm = nullptr, len = 0;
    ce.getPerm(&perm, &len);
    delete[] perm;
    int f = ce.registerFunction(RACE::gb300::MPK, ops, 4);
    int g = ce.registerMpkBlock(ops, 4, 16);
    RACE::gb300::Batch b;
    b.add(ce, g);
    b.graphLaunch();
    int scol[8] = {0}, cs[2] = {0, 8}, rl[4] = {2, 2, 2, 2}, clp[1] = {2};
    double sval[8] = {0};
    float fval[8] = {0};
    bool ok = ce.simdify(4, 4, 4, scol, cs, rl, clp, sval, true) && ce.simdifyD1(4, 4, 4, scol, cs, rl, clp, fval);
    int *split = nullptr, splitLen = 0;
    ce.getNumaSplitting(&split, &splitLen);
    free(split);
    ce.printZoneTree();
    ce.setSerial(f);
    ce.unsetSerial(f);
    ce.numaInitMtxVec(rp, col, nullptr, nullptr, 4);
    int best = ce.tuneFunction(f);
    return rc + f + ce.executeFunctionAsync(f) + ce.getStatus() + b.getStatus() + ce.getNumThreads() +
           ce.getHighestPower() + (ok ? 1 : 0) + best;
}
""")
    root = pathlib.Path(__file__).resolve().parents[1]
    r = subprocess.run([gxx, "-std=c++17", "-fsyntax-only", "-I", str(root / "include"), str(src)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def _wave_plan(kernel, mat, pp, lo, hi):
    L = _lib.lib()
    rp, cl = np.ascontiguousarray(mat.row_ptr, np.int32), np.ascontiguousarray(mat.col, np.int32)
    pp, lo, hi = (np.ascontiguousarray(a, np.int32) for a in (pp, lo, hi))
    nw, nr = C.c_int(), C.c_int()
    args = [kernel, mat.n, rp.ctypes.data, cl.ctypes.data, pp.ctypes.data, lo.ctypes.data, hi.ctypes.data,
            len(pp) - 1]
    _lib.check(L.race_wave_plan(*args, None, None, 0, C.byref(nw), C.byref(nr)))
    cap = max(nr.value, nw.value + 1)
    wp, rows = np.zeros(cap, np.int32), np.zeros(cap, np.int32)
    _lib.check(L.race_wave_plan(*args, wp.ctypes.data, rows.ctypes.data, cap, C.byref(nw), C.byref(nr)))
    return wp[: nw.value + 1], rows[: nr.value]


@pytest.mark.parametrize("m,d,t", sorted(EXEC_CASES) + [("lap7_32", 2, 1024), ("lap7_32", 1, 256)])
def test_wave_plans_reproduce_the_sequential_walk(golden, mats, m, d, t):
    """The wave compiler behind the GPU's bit-exact sweeps: every row of a
    wave is run on its own, in REVERSED order inside each wave, and the
    result still equals the sequential walk of the reference's phases bit
    for bit, for every kernel (and both directions of the sweeps): rows of one wave do not
    conflict and the order of conflicting accesses is RACE's."""
    A = mats[m]
    k = key_color(m, d, t)
    perm = golden[k + "__perm"]
    inv = np.empty_like(perm)
    inv[perm] = np.arange(A.n, dtype=np.int32)
    P = A.permuted(perm, inv)
    U = P.upper()
    x0 = matgen.uniform_vector(A.n, 0)
    b0 = matgen.uniform_vector(A.n, 1)
    kernels = [(orc.K_GS, P), (orc.K_SPMV, P)]
    if d == 2:
        kernels += [(orc.K_SYMMSPMV, U), (orc.K_KACZ, P), (orc.K_SPMTV, P)]
    for kern, mat in kernels:
        # only the sweeps run backward (the oracle's product kernels take forward ranges)
        for rev in ((False, True) if kern in (orc.K_GS, orc.K_KACZ) else (False,)):
            zero_b = kern in (orc.K_SPMV, orc.K_SYMMSPMV, orc.K_SPMTV)
            x1, b1 = x0.copy(), (np.zeros(A.n) if zero_b else b0.copy())
            x2, b2 = x1.copy(), b1.copy()
            pp, lo, hi = _flatten(golden[k + "__tree"], d, rev, A.n)
            _run_phases(pp, lo, hi, kern, mat, x1, b1)
            wp, rows = _wave_plan(kern, mat, pp, lo, hi)
            assert np.array_equal(np.sort(rows), np.arange(A.n))
            for w in range(len(wp) - 1):
                for r in rows[wp[w]:wp[w + 1]][::-1]:
                    orc.run_kernel(kern, int(r), int(r) + 1, mat, x2, b2)
            np.testing.assert_array_equal(x1, x2, err_msg=f"{kern} rev={rev}")
            np.testing.assert_array_equal(b1, b2, err_msg=f"{kern} rev={rev}")


def test_wave_plan_rejects_bad_phase_tables():
    L = _lib.lib()
    rp = np.array([0, 1, 2], np.int32)
    cl = np.array([0, 1], np.int32)
    nw, nr = C.c_int(), C.c_int()

    def call(kernel, pp, lo, hi):
        pp, lo, hi = (np.ascontiguousarray(a, np.int32) for a in (pp, lo, hi))
        return L.race_wave_plan(kernel, 2, rp.ctypes.data, cl.ctypes.data, pp.ctypes.data, lo.ctypes.data,
                                hi.ctypes.data, len(pp) - 1, None, None, 0, C.byref(nw), C.byref(nr))

    assert call(orc.K_GS, [0, 1], [0], [2]) == _lib.RACE_SUCCESS and (nw.value, nr.value) == (1, 2)  # diagonal: one wave
    assert call(orc.K_GS, [0, 1], [1], [-1]) == _lib.RACE_SUCCESS and nr.value == 2  # backward leaf
    bad = _lib.RACE_ERR_INVALID_ARG
    assert call(orc.K_GS, [0, 1], [0], [3]) == bad      # past the last row
    assert call(orc.K_GS, [0, 1], [2], [0]) == bad      # backward leaf from row n
    assert call(orc.K_GS, [1, 1], [0], [2]) == bad      # phase table not from 0
    assert call(orc.K_GS, [0, 1, 0], [0], [2]) == bad   # phases not monotonic
    assert call(5, [0, 1], [0], [2]) == bad             # MPK has no wave plan


def test_print_zone_tree_cpp_and_python_agree(golden, tmp_path):
    """printZoneTree of the C++ wrapper and of the Python mirror print the
    same lines for the reference's zone trees (one line per node, ranges
    and children as stored)."""
    import shutil
    import subprocess
    from race_gb300.interface import format_zone_tree
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    src = tmp_path / "pz.cpp"
    src.write_text("""
#include <iostream>
#include "race_gb300.hpp"
int main() {
    std::vector<int> t;
    int v;
    while (std::cin >> v) t.push_back(v);
    RACE::gb300::printZoneTreeFlat(t);
    return 0;
}
""")
    root = pathlib.Path(__file__).resolve().parents[1]
    exe = tmp_path / "pz"
    r = subprocess.run([gxx, "-std=c++17", "-O1", "-I", str(root / "include"), str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    for key in ("color__lap7_16__d2__t16__tree", "color__islands_330__d1__t8__tree", "color__tiny_1__d1__t4__tree"):
        tree = golden[key]
        out = subprocess.run([str(exe)], input=" ".join(map(str, tree)), capture_output=True, text=True).stdout
        py = format_zone_tree(tree)
        assert out == py
        assert len(py.splitlines()) == int(tree[0])
        assert py.startswith("0. Range:[")


def test_params_from_env_reads_recursion_stages(monkeypatch):
    """race_params_from_env reads RACE_MAX_RECURSION_STAGES like the
    reference (matrixPowerRecursive.cpp:50-60): -1 when unset."""
    L = _lib.lib()
    p = _lib.race_params()
    monkeypatch.delenv("RACE_MAX_RECURSION_STAGES", raising=False)
    _lib.check(L.race_params_from_env(C.byref(p)))
    assert p.max_recursion_stages == -1 and p.cache_violation_cutoff == 50 and p.n_eff == 1 and p.eff[0] == 40.0
    monkeypatch.setenv("RACE_MAX_RECURSION_STAGES", "0")
    _lib.check(L.race_params_from_env(C.byref(p)))
    assert p.max_recursion_stages == 0
    # the per-stage list RACE_CACHE_VIOLATION_CUTOFF after the default
    # (matrixPowerRecursive.cpp:39-48)
    assert p.n_cutoffs == 0
    monkeypatch.setenv("RACE_CACHE_VIOLATION_CUTOFF_DEFAULT", "30")
    monkeypatch.setenv("RACE_CACHE_VIOLATION_CUTOFF", "50,2,1")
    _lib.check(L.race_params_from_env(C.byref(p)))
    assert p.cache_violation_cutoff == 30 and p.n_cutoffs == 3 and list(p.cutoffs[:3]) == [50, 2, 1]


def _conflicts(P, pp, lo, hi, dist):
    """Rows of different leaves of one phase that are neighbours (dist 1) or
    share a neighbour (dist 2) in the symmetrised pattern of P; RACE's
    coloring guarantee, which the reference checks with
    Interface::detectConflict (interface.cpp:655-815)."""
    import scipy.sparse as sp
    n = P.n
    phase = np.full(n, -1, np.int64)
    leaf = np.full(n, -1, np.int64)
    for p in range(len(pp) - 1):
        for l in range(pp[p], pp[p + 1]):
            a, b = int(lo[l]), int(hi[l])
            rows = np.arange(a, b) if a <= b else np.arange(b + 1, a + 1)
            phase[rows], leaf[rows] = p, l
    assert (phase >= 0).all()
    S = sp.csr_matrix((np.ones(P.nnz), P.col, P.row_ptr), shape=(n, n))
    S = ((S + S.T + sp.identity(n, format="csr")) > 0).tocoo()
    i, j = S.row.astype(np.int64), S.col.astype(np.int64)
    if dist == 1:
        return int(((phase[i] == phase[j]) & (leaf[i] != leaf[j])).sum())
    # distance 2: every row k sees the rows of {k} + N(k); per (phase, k)
    # they must all lie in one leaf
    key = phase[j] * n + i
    order = np.lexsort((leaf[j], key))
    k2, l2 = key[order], leaf[j][order]
    return int(((k2[1:] == k2[:-1]) & (l2[1:] != l2[:-1])).sum())


@pytest.mark.parametrize("m,d,t", COLOR_CASES)
def test_phases_are_conflict_free(golden, mats, m, d, t):
    """Leaves that run concurrently (one phase of the flattened zone tree)
    never touch the same row's neighbourhood: no distance-1 neighbours for
    D1 coloring, no shared neighbour for D2, in both sweep directions."""
    A = mats[m]
    k = key_color(m, d, t)
    perm = golden[k + "__perm"]
    inv = np.empty_like(perm)
    inv[perm] = np.arange(A.n, dtype=np.int32)
    P = A.permuted(perm, inv)
    for rev in (False, True):
        pp, lo, hi = _flatten(golden[k + "__tree"], d, rev, A.n)
        assert _conflicts(P, pp, lo, hi, d) == 0


def test_conflict_check_detects_a_bad_phase(golden, mats):
    """The checker itself: merging two consecutive phases of a D2 schedule
    (red and black blocks together) creates conflicts."""
    A = mats["lap7_16"]
    k = key_color("lap7_16", 2, 16)
    perm = golden[k + "__perm"]
    inv = np.empty_like(perm)
    inv[perm] = np.arange(A.n, dtype=np.int32)
    P = A.permuted(perm, inv)
    pp, lo, hi = _flatten(golden[k + "__tree"], 2, False, A.n)
    assert len(pp) > 2
    merged = np.concatenate([[0], pp[2:]])  # phases 0 and 1 run together
    assert _conflicts(P, merged, lo, hi, 2) > 0
    assert _conflicts(P, pp, lo, hi, 2) == 0


def test_integration_examples_compile(tmp_path):
    """The C++ examples under tests/examples compile against the headers."""
    import shutil
    import subprocess
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    root = pathlib.Path(__file__).resolve().parents[1]
    srcs = sorted((root / "tests" / "examples").glob("*.cpp"))
    assert srcs
    for src in srcs:
        r = subprocess.run([gxx, "-std=c++17", "-fsyntax-only", "-Wno-unused-variable", "-I", str(root / "include"),
                            str(src)], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr


@pytest.mark.parametrize("m,t", COLOR3_CASES)
def test_three_block_phases_reproduce_reference(golden, mats, m, t):
    """THREE_BLOCK zone trees of the reference, flattened with three blocks
    per thread: every row once, distance-2 conflict-free phases in both
    directions, and the phase walk gives the reference executor's outputs
    bit for bit (GS both ways, KACZ, SymmSpMV, SpMTV)."""
    A = mats[m]
    k = key_color3(m, t)
    assert str(golden[k + "__digest"]) == digest(A)
    perm = golden[k + "__perm"]
    inv = np.empty_like(perm)
    inv[perm] = np.arange(A.n, dtype=np.int32)
    P = A.permuted(perm, inv)
    U = P.upper()
    assert int(golden[k + "__serial"][1]) <= int(golden[k + "__serial"][0])  # no serial part
    for rev in (False, True):
        pp, lo, hi = _flatten(golden[k + "__tree"], 2, rev, A.n, d2type=1)
        assert _conflicts(P, pp, lo, hi, 2) == 0
    x0 = matgen.uniform_vector(A.n, 0)
    b0 = matgen.uniform_vector(A.n, 1)
    for kern, name, mat, rev in [(orc.K_SYMMSPMV, "symmspmv", U, False), (orc.K_GS, "gs", P, False),
                                 (orc.K_GS, "gsrev", P, True), (orc.K_KACZ, "kacz", P, False),
                                 (orc.K_SPMTV, "spmtv", P, False)]:
        scatter = kern in (orc.K_SYMMSPMV, orc.K_SPMTV)
        x, b = x0.copy(), (np.zeros(A.n) if scatter else b0.copy())
        pp, lo, hi = _flatten(golden[k + "__tree"], 2, rev, A.n, d2type=1)
        _run_phases(pp, lo, hi, kern, mat, x, b)
        np.testing.assert_array_equal(b if scatter else x, golden[k + f"__out_{name}"], err_msg=name)



def _host_traverse(A, d, lo, hi, tp, ti):
    """The engine's host traversal (race_traverse_host) in the oracle's
    calling convention: (totalPerm, totalInvPerm, levelRow, levelNnz)."""
    L = _lib.lib()
    rp, cl = np.ascontiguousarray(A.row_ptr, np.int32), np.ascontiguousarray(A.col, np.int32)
    tp, ti = np.array(tp, np.int32), np.array(ti, np.int32)
    total = C.c_int()
    args = [A.n, rp.ctypes.data, cl.ctypes.data, tp.ctypes.data, ti.ctypes.data, lo, hi, d]
    # the first call only sizes the level arrays (distance 2 can count more
    # levels than the range has rows); the second traverses
    before = tp.copy()
    _lib.check(L.race_traverse_host(*args, None, None, 0, C.byref(total)))
    np.testing.assert_array_equal(tp, before)  # nothing written without room
    lr = np.zeros(max(total.value, 1), np.int32)
    ln = np.zeros_like(lr)
    _lib.check(L.race_traverse_host(*args, lr.ctypes.data, ln.ctypes.data, lr.size, C.byref(total)))
    return tp, ti, lr[: total.value], ln[: total.value]


def _zone_tree_host(A, d, t, d2type, cap, init=None, params=None, lb_target=1, host_traverse=False):
    """The engine's level recursion (race_zone_tree_host) driven by the
    oracle's traversal (or, with host_traverse, the engine's own host
    traversal), which keeps the running permutation here (starting from
    `init`, the identity by default)."""
    L = _lib.lib()
    lens = np.diff(A.row_ptr).astype(np.int64)
    tp0 = np.arange(A.n, dtype=np.int32) if init is None else np.ascontiguousarray(init, np.int32)
    ti0 = np.empty_like(tp0)
    ti0[tp0] = np.arange(A.n, dtype=np.int32)
    state = {"tp": tp0, "ti": ti0, "err": None}

    @_lib.TRAVERSE_FN
    def trav(user, lo, hi, lr_ptr, ln_ptr, lcap, total):
        try:
            if host_traverse:
                tp, ti, lr, ln = _host_traverse(A, d, lo, hi, state["tp"], state["ti"])
            else:
                tp, ti, lr, ln, _ = orc.traverse(A, d, lo, hi, state["tp"], state["ti"])
            state["tp"], state["ti"] = tp, ti
            if len(lr) > lcap:
                return 1
            np.ctypeslib.as_array(lr_ptr, shape=(lcap,))[: len(lr)] = lr
            np.ctypeslib.as_array(ln_ptr, shape=(lcap,))[: len(ln)] = ln
            total[0] = len(lr)
            return 0
        except Exception as ex:  # report instead of unwinding through C
            state["err"] = ex
            return 1

    @_lib.RANGE_NNZ_FN
    def rnnz(user, lo, hi):
        return int(lens[state["tp"][lo:hi]].sum())

    buf = np.zeros(cap, np.int32)
    tlen, avail = C.c_int(), C.c_int()
    rc = L.race_zone_tree_host(A.n, t, d, d2type, lb_target, None if params is None else C.byref(params), trav, rnnz,
                               None, buf.ctypes.data, cap, C.byref(tlen), C.byref(avail))
    assert state["err"] is None, state["err"]
    _lib.check(rc)
    assert tlen.value <= cap
    return buf[: tlen.value], avail.value, state["tp"]


@pytest.mark.parametrize("m,d,t,d2type", [c + (0,) for c in COLOR_CASES]
                         + [(m, 2, t, 1) for m, t in COLOR3_CASES])
def test_level_recursion_on_host_matches_reference(golden, mats, m, d, t, d2type, monkeypatch):
    """The engine's restatement of RACE's level recursion and zone tree
    (coloring.cpp), run on the CPU with the oracle's traversal in place of
    the GPU BFS: the zone tree, the thread count and the permutation equal
    the reference's (TWO_BLOCK and THREE_BLOCK)."""
    for var in ("RACE_EFFICIENCY", "RACE_THREADS", "RACE_CACHE_VIOLATION_CUTOFF", "RACE_MAX_RECURSION_STAGES"):
        monkeypatch.delenv(var, raising=False)
    A = mats[m]
    k = key_color(m, d, t) if d2type == 0 else key_color3(m, t)
    gold = golden[k + "__tree"]
    tree, avail, perm = _zone_tree_host(A, d, t, d2type, 2 * gold.size + 1024)
    np.testing.assert_array_equal(tree, gold)
    assert avail == int(golden[k + "__threads"])
    np.testing.assert_array_equal(perm, golden[k + "__perm"])


def _stage_partition(lr, ln, n, nnz, power, cache, cutoff=50, safety=2.0):
    L = _lib.lib()
    lr = np.ascontiguousarray(lr, np.int32)
    ln = np.ascontiguousarray(ln, np.int32)
    ng, nh = C.c_int(), C.c_int()
    args = [lr.ctypes.data, ln.ctypes.data, lr.size, n, nnz, power, float(cache), float(safety), cutoff]
    _lib.check(L.race_mpk_stage_partition(*args, None, None, 0, C.byref(ng), C.byref(nh)))
    cap = max(ng.value + 1, nh.value, 1)
    gp, hid = np.zeros(cap, np.int32), np.zeros(cap, np.int32)
    _lib.check(L.race_mpk_stage_partition(*args, gp.ctypes.data, hid.ctypes.data, cap, C.byref(ng), C.byref(nh)))
    return gp[: ng.value + 1], hid[: nh.value]


def test_stage_partition_matches_reference(golden, mats):
    """The single-stage MPK partition with hopeless regions
    (race_mpk_stage_partition) on the BFS levels of the oracle's traversal
    gives the reference's level groups (MPLeaf::lp) and hopeless groups
    (MPLeaf::hid): cases without hopeless regions, cases with them (whose
    reference partition then recurses inside those groups), and partitions
    without recursion (cut-off disabled)."""
    from cases import HOPELESS_CASES, POWER_CASES, POWER_FLAT_CASES, key_hopeless, key_power, key_power_flat
    cases = [(mpc, key_power(*mpc), 50, golden[key_power(*mpc) + "__hid"][:-1]) for mpc in POWER_CASES]  # -1 ends
    cases += [(mpc, key_hopeless(*mpc), 50, golden[key_hopeless(*mpc) + "__hid"]) for mpc in HOPELESS_CASES]
    cases += [(mpc, key_power_flat(*mpc), 2**31 - 1, np.zeros(0, np.int32)) for mpc in POWER_FLAT_CASES]
    with_hopeless = 0
    for (m, p, c), k, cutoff, want_hid in cases:
        A = mats[m]
        _, _, lr, ln, _ = orc.traverse(A, 3, 0, A.n)
        gp, hid = _stage_partition(lr, ln, A.n, A.nnz, p, c, cutoff)
        np.testing.assert_array_equal(gp, golden[k + "__lp"], err_msg=k)
        np.testing.assert_array_equal(hid, want_hid, err_msg=k)
        with_hopeless += hid.size > 0
    assert with_hopeless >= 6
    # triangular matrices (mtxType L / U): one row per level
    from cases import POWER_TRI_CASES, key_power_tri, triangle
    for m, tri, p, c in POWER_TRI_CASES:
        T = triangle(mats[m], tri)
        lens = np.diff(T.row_ptr).astype(np.int32)
        order = lens if tri == "L" else lens[::-1]
        gp, hid = _stage_partition(np.ones(T.n, np.int32), order, T.n, T.nnz, p, c)
        np.testing.assert_array_equal(gp, golden[key_power_tri(m, tri, p, c) + "__lp"])


def test_mpk_recursion_matches_reference(golden, mats):
    """The engine's partition of a matrix with hopeless regions, computed on
    the host from the oracle's stage-0 BFS: level groups and hopeless groups
    (race_mpk_stage_partition) and the recursion's permutation
    (race_mpk_recursion_permute) equal the reference's default partition."""
    from cases import HOPELESS_CASES, key_hopeless
    L = _lib.lib()
    for m, p, c in HOPELESS_CASES:
        A = mats[m]
        k = key_hopeless(m, p, c)
        tp, ti, lr, ln, _ = orc.traverse(A, 3, 0, A.n)
        gp, hid = _stage_partition(lr, ln, A.n, A.nnz, p, c)
        np.testing.assert_array_equal(gp, golden[k + "__lp"])
        rp, cl = np.ascontiguousarray(A.row_ptr, np.int32), np.ascontiguousarray(A.col, np.int32)
        tp, ti = np.ascontiguousarray(tp, np.int32), np.ascontiguousarray(ti, np.int32)
        hid = np.ascontiguousarray(hid, np.int32)
        _lib.check(L.race_mpk_recursion_permute(A.n, rp.ctypes.data, cl.ctypes.data, tp.ctypes.data, ti.ctypes.data,
                                                gp.ctypes.data, gp.size - 1, hid.ctypes.data, hid.size, p))
        np.testing.assert_array_equal(tp, golden[k + "__perm"], err_msg=k)
        np.testing.assert_array_equal(ti[tp], np.arange(A.n))


def _recursive_partition(A, p, c, stage_cutoffs, safety=2.0):
    """Stage 0 from the oracle's BFS (race_mpk_stage_partition), then the
    engine's recursion below it (race_mpk_recursive_partition): the flat
    leaf tree and the permutation."""
    L = _lib.lib()
    tp, ti, lr, ln, _ = orc.traverse(A, 3, 0, A.n)
    c0 = stage_cutoffs[0] if stage_cutoffs else 2**31 - 1
    gp, hid = _stage_partition(lr, ln, A.n, A.nnz, p, c, c0, safety)
    gp, hid = np.ascontiguousarray(gp, np.int32), np.ascontiguousarray(hid, np.int32)
    rp, cl = np.ascontiguousarray(A.row_ptr, np.int32), np.ascontiguousarray(A.col, np.int32)
    tp, ti = np.ascontiguousarray(tp, np.int32), np.ascontiguousarray(ti, np.int32)
    sc = np.ascontiguousarray(list(stage_cutoffs) or [0], np.int32)
    tl = C.c_int()
    tree = np.zeros(1 << 16, np.int32)
    _lib.check(L.race_mpk_recursive_partition(A.n, rp.ctypes.data, cl.ctypes.data, tp.ctypes.data, ti.ctypes.data,
                                              gp.ctypes.data, gp.size - 1, hid.ctypes.data, hid.size, p, A.nnz,
                                              float(c), float(safety), sc.ctypes.data, len(stage_cutoffs),
                                              tree.ctypes.data, tree.size, C.byref(tl)))
    assert 0 < tl.value <= tree.size
    return tree[: tl.value], tp, ti


def test_mpk_deep_recursion_matches_reference(golden, mats):
    """The MPK partition's recursion deeper than one stage
    (RACE_MAX_RECURSION_STAGES > 1, a list of cut-offs per stage;
    mtxPowerRecursive::recursivePartition, matrixPowerRecursive.cpp:156-338)
    computed by the engine on the host gives the reference's whole leaf tree
    (each leaf's rows, stage, parent, level groups and hopeless groups) and
    its permutation, for boundary widths 0 to 3 and up to three stages."""
    from cases import DEEP_CASES, deep_stage_cutoffs, key_deep
    deepest = 0
    for m, p, c, stages, cuts in DEEP_CASES:
        A = mats[m]
        k = key_deep(m, p, c, stages, cuts)
        assert str(golden[k + "__digest"]) == digest(A)
        tree, tp, ti = _recursive_partition(A, p, c, deep_stage_cutoffs(stages, cuts))
        np.testing.assert_array_equal(tree, golden[k + "__tree"], err_msg=k)
        np.testing.assert_array_equal(tp, golden[k + "__perm"], err_msg=k)
        np.testing.assert_array_equal(ti[tp], np.arange(A.n))
        deepest = max(deepest, max(int(v) for v in _leaf_stages(tree)))
    assert deepest == 3


def _leaf_stages(tree):
    k, out = 1, []
    for _ in range(int(tree[0])):
        out.append(tree[k + 2])
        k += 5 + int(tree[k + 4]) + 1
        k += 1 + int(tree[k])
    return out


def test_mpk_partition_at_edge_parameters(golden, mats):
    """Power 1 and high powers, a budget that holds the whole matrix, tiny
    budgets (hopeless regions, also with power 1), a one-row matrix: the
    engine's host partition and recursion give the reference's whole leaf
    tree and permutation."""
    from cases import POWER_EDGE_CASES, key_power_edge
    with_hopeless = 0
    for m, p, c in POWER_EDGE_CASES:
        A = mats[m]
        k = key_power_edge(m, p, c)
        assert str(golden[k + "__digest"]) == digest(A)
        tree, tp, _ = _recursive_partition(A, p, c, [50])
        np.testing.assert_array_equal(tree, golden[k + "__tree"], err_msg=k)
        np.testing.assert_array_equal(tp, golden[k + "__perm"], err_msg=k)
        with_hopeless += int(tree[0]) > 1
    assert with_hopeless == 3


def test_mpk_one_stage_recursion_is_the_general_one(golden, mats):
    """At the default depth (one stage past the cut-off list: stage 1 has no
    cut-off) the general recursion gives the one-stage permutation of the
    reference's default partitions, and one leaf per hopeless group."""
    from cases import HOPELESS_CASES, key_hopeless
    for m, p, c in HOPELESS_CASES:
        A = mats[m]
        k = key_hopeless(m, p, c)
        tree, tp, _ = _recursive_partition(A, p, c, [50])
        np.testing.assert_array_equal(tp, golden[k + "__perm"], err_msg=k)
        assert int(tree[0]) == int(golden[k + "__leaves"]) == 1 + len(golden[k + "__hid"])


def test_mpk_recursive_partition_rejects_invalid_input():
    """Group offsets that do not cover the rows, hopeless indices outside
    the groups and missing arrays are refused before any work."""
    L = _lib.lib()
    A = matgen.laplace3d_7pt(4)
    rp, cl = np.ascontiguousarray(A.row_ptr, np.int32), np.ascontiguousarray(A.col, np.int32)
    tp = np.arange(A.n, dtype=np.int32)
    ti = tp.copy()
    sc = np.array([50, 50], np.int32)
    tl = C.c_int()

    def call(gp, hid, n=A.n, stages=2):
        gp, hid = np.ascontiguousarray(gp, np.int32), np.ascontiguousarray(hid, np.int32)
        return L.race_mpk_recursive_partition(n, rp.ctypes.data, cl.ctypes.data, tp.ctypes.data, ti.ctypes.data,
                                              gp.ctypes.data, gp.size - 1, hid.ctypes.data, hid.size, 4, A.nnz, 1e4,
                                              2.0, sc.ctypes.data, stages, None, 0, C.byref(tl))
    assert call([0, 10, A.n], []) == _lib.RACE_SUCCESS and int(tl.value) == 1 + 5 + 3 + 1  # the root alone
    assert call([0, 10, A.n - 1], []) == _lib.RACE_ERR_INVALID_ARG
    assert call([0, 10, 5, A.n], []) == _lib.RACE_ERR_INVALID_ARG
    assert call([0, 10, A.n], [2]) == _lib.RACE_ERR_INVALID_ARG
    assert call([0, 10, A.n], [], stages=-1) == _lib.RACE_ERR_INVALID_ARG
    # a hopeless group without p-1 groups on either side has no boundaries to take
    assert call([0, 10, A.n], [0]) == _lib.RACE_ERR_GRAPH_TRAVERSAL
    np.testing.assert_array_equal(tp, np.arange(A.n))  # untouched on errors


def test_level_recursion_from_an_initial_permutation(golden, mats):
    """Coloring that starts from an initial permutation (the Interface
    ctor's initPerm, graph_SoA.cpp:63-79): the engine's level recursion
    gives the reference's zone tree, thread count and composed permutation."""
    from cases import COLOR_INIT_CASES, key_color_init
    for m, d, t in COLOR_INIT_CASES:
        A = mats[m]
        k = key_color_init(m, d, t)
        assert str(golden[k + "__digest"]) == digest(A)
        gold = golden[k + "__tree"]
        tree, avail, perm = _zone_tree_host(A, d, t, 0, 2 * gold.size + 1024, init=golden[k + "__init"])
        np.testing.assert_array_equal(tree, gold, err_msg=k)
        assert avail == int(golden[k + "__threads"])
        np.testing.assert_array_equal(perm, golden[k + "__perm"], err_msg=k)


def test_level_recursion_under_environment_knobs(golden, mats, monkeypatch):
    """RACE_EFFICIENCY (per-stage list after the default 40) and
    RACE_THREADS (per-stage thread requests, which zero that stage's
    efficiency), read by the engine like the reference
    (level_recursion.cpp:48-90): same zone tree, threads and permutation."""
    from cases import COLOR_ENV_CASES, key_color_env
    for m, d, t, env in COLOR_ENV_CASES:
        for var in ("RACE_EFFICIENCY", "RACE_THREADS"):
            monkeypatch.delenv(var, raising=False)
        for var, val in env.items():
            monkeypatch.setenv(var, val)
        A = mats[m]
        k = key_color_env(m, d, t, env)
        gold = golden[k + "__tree"]
        tree, avail, perm = _zone_tree_host(A, d, t, 0, 2 * gold.size + 1024)
        np.testing.assert_array_equal(tree, gold, err_msg=k)
        assert avail == int(golden[k + "__threads"]), k
        np.testing.assert_array_equal(perm, golden[k + "__perm"], err_msg=k)


def test_level_recursion_with_explicit_params(golden, mats, monkeypatch):
    """The same knobs passed in race_params instead of the environment
    (thread requests zero their stages' efficiency there too)."""
    from cases import COLOR_ENV_CASES, key_color_env
    for var in ("RACE_EFFICIENCY", "RACE_THREADS", "RACE_CACHE_VIOLATION_CUTOFF", "RACE_MAX_RECURSION_STAGES"):
        monkeypatch.delenv(var, raising=False)
    for m, d, t, env in COLOR_ENV_CASES:
        prm = _lib.race_params()
        _lib.check(_lib.lib().race_params_from_env(C.byref(prm)))
        eff = [40] + [int(v) for v in env.get("RACE_EFFICIENCY", "").split(",") if v]
        thr = [int(v) for v in env.get("RACE_THREADS", "").split(",") if v]
        prm.n_eff = len(eff)
        for i, v in enumerate(eff):
            prm.eff[i] = v
        prm.n_lvl_threads = len(thr)
        for i, v in enumerate(thr):
            prm.lvl_threads[i] = v
        A = mats[m]
        k = key_color_env(m, d, t, env)
        gold = golden[k + "__tree"]
        tree, avail, perm = _zone_tree_host(A, d, t, 0, 2 * gold.size + 1024, params=prm)
        np.testing.assert_array_equal(tree, gold, err_msg=k)
        np.testing.assert_array_equal(perm, golden[k + "__perm"], err_msg=k)


def test_level_recursion_balancing_rows(golden, mats, monkeypatch):
    """LBTarget ROW (balance rows, not non-zeros): the engine's level
    recursion equals the reference's zone tree, threads and permutation."""
    from cases import COLOR_ROW_CASES, key_color_row
    for var in ("RACE_EFFICIENCY", "RACE_THREADS"):
        monkeypatch.delenv(var, raising=False)
    for m, d, t in COLOR_ROW_CASES:
        A = mats[m]
        k = key_color_row(m, d, t)
        gold = golden[k + "__tree"]
        tree, avail, perm = _zone_tree_host(A, d, t, 0, 2 * gold.size + 1024, lb_target=0)
        np.testing.assert_array_equal(tree, gold, err_msg=k)
        assert avail == int(golden[k + "__threads"]), k
        np.testing.assert_array_equal(perm, golden[k + "__perm"], err_msg=k)


@pytest.mark.parametrize("m,d", [c for c in __import__("cases").TRAVERSE_CASES if c[1] in (1, 2)])
def test_host_traversal_matches_reference(golden, mats, m, d):
    """The engine's host traversal (run for short coloring ranges with
    RACE_GPU_HOST_TRAVERSE_BELOW) of the whole matrix gives the reference's
    permutation and level histogram."""
    from cases import key_trav
    A = mats[m]
    k = key_trav(m, d)
    ident = np.arange(A.n, dtype=np.int32)
    tp, ti, lr, ln = _host_traverse(A, d, 0, A.n, ident, ident)
    np.testing.assert_array_equal(tp, golden[k + "__perm"])
    np.testing.assert_array_equal(lr, golden[k + "__levelRow"])
    np.testing.assert_array_equal(ln, golden[k + "__levelNnz"])
    np.testing.assert_array_equal(ti[tp], np.arange(A.n))


def test_level_recursion_with_host_traversal_matches_reference(golden, mats, monkeypatch):
    """The engine's level recursion driven by the engine's own host
    traversal on every sub-range (what RACE_GPU_HOST_TRAVERSE_BELOW does for
    short ranges) gives the reference's zone trees, thread counts and
    permutations: all coloring cases and the thread-count edges."""
    from cases import COLOR_EDGE_CASES, key_color_edge
    for var in ("RACE_EFFICIENCY", "RACE_THREADS"):
        monkeypatch.delenv(var, raising=False)
    cases = [(m, d, t, key_color(m, d, t)) for m, d, t in COLOR_CASES]
    cases += [(m, d, t, key_color_edge(m, d, t)) for m, d, t in COLOR_EDGE_CASES]
    for m, d, t, k in cases:
        A = mats[m]
        gold = golden[k + "__tree"]
        tree, avail, perm = _zone_tree_host(A, d, t, 0, 2 * gold.size + 1024, host_traverse=True)
        np.testing.assert_array_equal(tree, gold, err_msg=k)
        assert avail == int(golden[k + "__threads"]), k
        np.testing.assert_array_equal(perm, golden[k + "__perm"], err_msg=k)


def test_level_recursion_at_thread_count_edges(golden, mats, monkeypatch):
    """The engine's level recursion at the edges of the thread count (one
    thread, odd and prime counts, far more threads than the matrix can
    use) gives the reference's zone tree, threads and permutation."""
    from cases import COLOR_EDGE_CASES, key_color_edge
    for var in ("RACE_EFFICIENCY", "RACE_THREADS"):
        monkeypatch.delenv(var, raising=False)
    for m, d, t in COLOR_EDGE_CASES:
        A = mats[m]
        k = key_color_edge(m, d, t)
        assert str(golden[k + "__digest"]) == digest(A)
        gold = golden[k + "__tree"]
        tree, avail, perm = _zone_tree_host(A, d, t, 0, 2 * gold.size + 1024)
        np.testing.assert_array_equal(tree, gold, err_msg=k)
        assert avail == int(golden[k + "__threads"]), k
        np.testing.assert_array_equal(perm, golden[k + "__perm"], err_msg=k)


def test_level_recursion_on_unsymmetric_patterns(golden, mats, monkeypatch):
    """Matrices whose pattern is not symmetric, colored with symm_hint
    false: with RACE's symmetrisation (the missing transposed entries added,
    graph.cpp:47-142) as the traversal graph, the engine's level recursion
    gives the reference's zone tree, threads and permutation."""
    from cases import COLOR_UNSYM_CASES, key_color_unsym, symmetrized_pattern, triangle
    for var in ("RACE_EFFICIENCY", "RACE_THREADS"):
        monkeypatch.delenv(var, raising=False)
    for m, tri, d, t in COLOR_UNSYM_CASES:
        T = triangle(mats[m], tri)
        k = key_color_unsym(m, tri, d, t)
        assert str(golden[k + "__digest"]) == digest(T)
        S = symmetrized_pattern(T)
        gold = golden[k + "__tree"]
        tree, avail, perm = _zone_tree_host(S, d, t, 0, 2 * gold.size + 1024)
        np.testing.assert_array_equal(tree, gold, err_msg=k)
        assert avail == int(golden[k + "__threads"]), k
        np.testing.assert_array_equal(perm, golden[k + "__perm"], err_msg=k)


def test_host_partition_entry_points_reject_bad_input():
    L = _lib.lib()
    bad = _lib.RACE_ERR_INVALID_ARG
    lr = np.array([1, 2], np.int32)
    ln = np.array([3, 5], np.int32)
    ng, nh = C.c_int(), C.c_int()
    ok = L.race_mpk_stage_partition(lr.ctypes.data, ln.ctypes.data, 2, 3, 8, 2, 1e6, 2.0, 50, None, None, 0,
                                    C.byref(ng), C.byref(nh))
    assert ok == _lib.RACE_SUCCESS and (ng.value, nh.value) == (1, 0)
    assert L.race_mpk_stage_partition(lr.ctypes.data, ln.ctypes.data, 2, 0, 8, 2, 1e6, 2.0, 50, None, None, 0,
                                      C.byref(ng), C.byref(nh)) == bad  # no rows
    assert L.race_mpk_stage_partition(lr.ctypes.data, ln.ctypes.data, 2, 3, 8, 0, 1e6, 2.0, 50, None, None, 0,
                                      C.byref(ng), C.byref(nh)) == bad  # power 0
    assert L.race_mpk_stage_partition(None, None, 2, 3, 8, 2, 1e6, 2.0, 50, None, None, 0, C.byref(ng),
                                      C.byref(nh)) == bad
    rp = np.array([0, 1, 2, 3], np.int32)
    cl = np.array([0, 1, 2], np.int32)
    tp = np.arange(3, dtype=np.int32)
    ti = np.arange(3, dtype=np.int32)
    gp = np.array([0, 1, 3], np.int32)
    hid = np.array([5], np.int32)
    args = [3, rp.ctypes.data, cl.ctypes.data, tp.ctypes.data, ti.ctypes.data, gp.ctypes.data, 2]
    assert L.race_mpk_recursion_permute(*args, None, 0, 2) == _lib.RACE_SUCCESS  # nothing hopeless: unchanged
    np.testing.assert_array_equal(tp, [0, 1, 2])
    assert L.race_mpk_recursion_permute(*args, hid.ctypes.data, 1, 2) != _lib.RACE_SUCCESS  # no group 5
    gp_bad = np.array([0, 2, 1], np.int32)
    assert L.race_mpk_recursion_permute(3, rp.ctypes.data, cl.ctypes.data, tp.ctypes.data, ti.ctypes.data,
                                        gp_bad.ctypes.data, 2, None, 0, 2) == bad  # groups not monotonic
    tl, av = C.c_int(), C.c_int()
    assert L.race_zone_tree_host(3, 4, 3, 0, 1, None, _lib.TRAVERSE_FN(0), _lib.RANGE_NNZ_FN(0), None, None, 0,
                                 C.byref(tl), C.byref(av)) == bad  # dist POWER has no zone tree


def _gather_plan(kernel, mat, pp, lo, hi):
    L = _lib.lib()
    rp, cl = np.ascontiguousarray(mat.row_ptr, np.int32), np.ascontiguousarray(mat.col, np.int32)
    pp, lo, hi = (np.ascontiguousarray(a, np.int32) for a in (pp, lo, hi))
    nu = C.c_int()
    args = [kernel, mat.n, rp.ctypes.data, cl.ctypes.data, pp.ctypes.data, lo.ctypes.data, hi.ctypes.data,
            len(pp) - 1]
    _lib.check(L.race_gather_plan(*args, None, None, None, 0, C.byref(nu)))
    cap = max(nu.value, mat.n + 1)
    ptr, entry, row = (np.zeros(cap, np.int32) for _ in range(3))
    _lib.check(L.race_gather_plan(*args, ptr.ctypes.data, entry.ctypes.data, row.ctypes.data, cap, C.byref(nu)))
    return ptr[: mat.n + 1], entry[: nu.value], row[: nu.value]


def _replay_gather(mat, x, b, ptr, entry, row):
    """The gather kernel's operations in exact arithmetic with one rounding
    per fused multiply-add (fma(a, b, c) = round(a*b + c))."""
    from fractions import Fraction

    def fma(a, b, c):
        return float(Fraction(a) * Fraction(b) + Fraction(c))

    out = b.copy()
    val, col, rp = mat.val, mat.col, mat.row_ptr
    for y in range(mat.n):
        acc = float(out[y])
        for k in range(ptr[y], ptr[y + 1]):
            e = int(entry[k])
            if e >= 0:
                acc = fma(val[e], x[row[k]], acc)
            else:
                s = int(rp[y])
                acc = fma(val[s], x[y], acc)
                t = 0.0
                for j in range(s + 1, int(rp[y + 1])):
                    t = fma(val[j], x[col[j]], t)
                acc = acc + t
        out[y] = acc
    return out


@pytest.mark.parametrize("m,d,t", [("lap7_16", 2, 16), ("islands_330", 2, 16), ("aniso5_120x90", 2, 48)])
def test_gather_plans_reproduce_the_sequential_walk(golden, mats, m, d, t):
    """RACE_SWEEP_GATHER's plans: replaying each entry of b's updates in the
    plan's order gives RACE's sequential walk bit for bit (SpMTV on the full
    matrix, SymmSpMV on the upper triangle; forward schedule, and the reverse
    phase order)."""
    A = mats[m]
    k = key_color(m, d, t)
    perm = golden[k + "__perm"]
    inv = np.empty_like(perm)
    inv[perm] = np.arange(A.n, dtype=np.int32)
    P = A.permuted(perm, inv)
    U = P.upper()
    x0 = matgen.uniform_vector(A.n, 0)
    b0 = matgen.uniform_vector(A.n, 1)  # accumulate onto a nonzero b
    for kern, mat in ((orc.K_SPMTV, P), (orc.K_SYMMSPMV, U)):
        for rev in (False, True):
            pp, lo, hi = _flatten(golden[k + "__tree"], d, rev, A.n)
            xs, bs = x0.copy(), b0.copy()
            if rev:  # the oracle's scatter bodies take forward ranges: reversed phase order, forward leaves
                lo, hi = np.minimum(lo, hi) + (lo > hi), np.maximum(lo, hi) + (lo > hi)
            _run_phases(pp, lo, hi, kern, mat, xs, bs)
            ptr, entry, row = _gather_plan(kern, mat, pp, lo, hi)
            assert ptr[-1] == entry.size
            got = _replay_gather(mat, x0, b0, ptr, entry, row)
            np.testing.assert_array_equal(got, bs, err_msg=f"{kern} rev={rev}")


def test_stage_partition_with_other_safety_factors(golden, mats):
    """RACEColor's safetyFactor (interface.cpp:205) scales every level's
    budget: the level groups and hopeless groups follow the reference."""
    from cases import POWER_SAFETY_CASES, key_power_safety
    for m, p, c, sf in POWER_SAFETY_CASES:
        A = mats[m]
        k = key_power_safety(m, p, c, sf)
        _, _, lr, ln, _ = orc.traverse(A, 3, 0, A.n)
        gp, hid = _stage_partition(lr, ln, A.n, A.nnz, p, c, safety=sf)
        np.testing.assert_array_equal(gp, golden[k + "__lp"], err_msg=k)
        np.testing.assert_array_equal(hid, golden[k + "__hid"], err_msg=k)


@pytest.mark.parametrize("m,d,t", [("lap7_32", 2, 8), ("lap7_32", 2, 64), ("lap7_16", 2, 16), ("st27_16", 2, 128),
                                   ("lap7_32", 1, 256)])
def test_openmp_phase_executor_matches_sequential_walk(golden, mats, m, d, t):
    """The C1 CPU baseline's executor (orc.exec_phases_omp: leaves of a phase
    on parallel OpenMP threads, a barrier between phases) gives the
    sequential phase walk's bits: the leaves of a phase never conflict."""
    A = mats[m]
    k = key_color(m, d, t)
    perm = golden[k + "__perm"]
    inv = np.empty_like(perm)
    inv[perm] = np.arange(A.n, dtype=np.int32)
    P = A.permuted(perm, inv)
    U = P.upper()
    x0 = matgen.uniform_vector(A.n, 0)
    b0 = matgen.uniform_vector(A.n, 1)
    kernels = [(orc.K_GS, P, False), (orc.K_GS, P, True)]
    if d == 2:
        kernels += [(orc.K_SYMMSPMV, U, False), (orc.K_KACZ, P, False)]
    for kern, mat, rev in kernels:
        pp, lo, hi = _flatten(golden[k + "__tree"], d, rev, A.n)
        xs, bs = x0.copy(), (np.zeros(A.n) if kern == orc.K_SYMMSPMV else b0.copy())
        _run_phases(pp, lo, hi, kern, mat, xs, bs)
        for threads in (1, 4, 8):
            xp, bp = x0.copy(), (np.zeros(A.n) if kern == orc.K_SYMMSPMV else b0.copy())
            orc.exec_phases_omp(kern, pp, lo, hi, threads, 1, mat, xp, bp)
            assert np.array_equal(xp, xs) and np.array_equal(bp, bs), (kern, rev, threads)
