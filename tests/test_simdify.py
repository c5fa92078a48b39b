"""SELL-C-sigma preparation (simdify / simdifyD1) against the reference.

The golden entries hold the reference's own output (Interface::simdify and
simdifyD1 run through a colored RACE::Interface, tests/golden/make_golden.py)
for SELL-C-1 matrices in RACE order whose values number the slots; the
engine's host implementation must give the same columns and the same slot
moves, and the same failures. The distance-2 pass uses the forward schedule
flattened from the reference's own zone tree (race_flatten_zone_tree), as the
engine does with its own tree.
"""
import ctypes as C

import numpy as np
import pytest

from cases import SIMDIFY_CASES, digest, key_simdify, sell_layout
from race_gb300 import _lib
from race_gb300 import interface as ri
from race_gb300.interface import VAL_BF16, VAL_F32, VAL_F64

EXPECT = {True: _lib.RACE_SUCCESS, False: _lib.RACE_ERR_INCOMPATIBILITY}

# The reference's simdifyD1 swaps with slot clp[c]-(k+1) of the row's chunk
# without checking that it is >= 0 (include/simdify.h:426). In this case the
# slot lies in the previous chunk and the reference's output trades entries
# between two rows; the engine refuses the input instead.
REF_CROSSES_ROWS = {key_simdify("islands_330", 1, 8, 7, 14, 0, False, "d1")}


def _forward_leaves(tree_flat, dist, n):
    L = _lib.lib()
    t = np.ascontiguousarray(tree_flat, np.int32)
    npz, nl = C.c_int(), C.c_int()
    args = [t.ctypes.data, t.size, dist, 0, 0, n, n]
    _lib.check(L.race_flatten_zone_tree(*args, None, None, None, 0, C.byref(npz), C.byref(nl)))
    cap = max(nl.value, npz.value + 1)
    pp, lo, hi = (np.zeros(cap, np.int32) for _ in range(3))
    _lib.check(L.race_flatten_zone_tree(*args, pp.ctypes.data, lo.ctypes.data, hi.ctypes.data, cap, C.byref(npz),
                                        C.byref(nl)))
    return lo[: nl.value], hi[: nl.value]


def _run(kind, d, w, c, flag, sell, val, val_type, leaves, n):
    col, _, cs, rl, clp = sell
    L = _lib.lib()
    vp = None if val is None else val.ctypes.data
    if kind == "d2":
        lo, hi = leaves
        coll = C.c_int(-1)
        rc = L.race_simdify_schedule(w, c, n, col.ctypes.data, cs.ctypes.data, rl.ctypes.data, clp.ctypes.data, vp,
                                     val_type, int(flag), lo.ctypes.data, hi.ctypes.data, lo.size, C.byref(coll))
        assert coll.value >= 0
        return rc
    return L.race_simdify_d1(w, c, n, col.ctypes.data, cs.ctypes.data, rl.ctypes.data, clp.ctypes.data, vp,
                             val_type, int(flag))


def _case(golden, mats, case):
    m, d, t, w, c, extra, flag, kind = case
    A = mats[m]
    k = key_simdify(*case)
    assert str(golden[k + "__digest"]) == digest(A)
    perm = golden[k + "__perm"]
    inv = np.empty_like(perm)
    inv[perm] = np.arange(A.n, dtype=np.int32)
    sell = sell_layout(A.permuted(perm, inv), c, extra, diag_first=(kind == "d2" and flag))
    leaves = _forward_leaves(golden[k + "__tree"], d, A.n) if kind == "d2" else None
    return k, A.n, sell, leaves


@pytest.mark.parametrize("case", SIMDIFY_CASES, ids=[key_simdify(*c) for c in SIMDIFY_CASES])
def test_simdify_matches_reference(golden, mats, case):
    m, d, t, w, c, extra, flag, kind = case
    k, n, sell, leaves = _case(golden, mats, case)
    ok = bool(golden[k + "__ok"])
    rows = _slot_rows(sell, c, n)
    rc = _run(kind, d, w, c, flag, sell, sell[1], VAL_F64, leaves, n)
    if k in REF_CROSSES_ROWS:
        src = golden[k + "__src"]
        assert ((rows[src] != rows) & (rows >= 0)).any()  # the reference moved entries between rows
        assert rc == _lib.RACE_ERR_INVALID_ARG
        return
    assert rc == EXPECT[ok]
    np.testing.assert_array_equal(sell[0], golden[k + "__col"])
    np.testing.assert_array_equal(sell[1].astype(np.int32), golden[k + "__src"])


@pytest.mark.parametrize("case", [c for c in SIMDIFY_CASES if c[0] in ("lap7_16", "islands_330", "arrow_64")
                                  and key_simdify(*c) not in REF_CROSSES_ROWS],
                         ids=lambda c: key_simdify(*c))
def test_simdify_value_types(golden, mats, case):
    """Values move with their columns whatever their width: FP32 slot
    numbers, BF16 bit patterns, or no values at all."""
    m, d, t, w, c, extra, flag, kind = case
    k, n, sell, leaves = _case(golden, mats, case)
    ok = bool(golden[k + "__ok"])
    src = golden[k + "__src"]
    base_col = sell[0].copy()
    for val_type, val in ((VAL_F32, sell[1].astype(np.float32)), (VAL_BF16, (sell[1].astype(np.int64) & 0xFFFF)
                                                                  .astype(np.uint16)), (VAL_F64, None)):
        s = (base_col.copy(),) + sell[1:]
        assert _run(kind, d, w, c, flag, s, val, val_type, leaves, n) == EXPECT[ok]
        np.testing.assert_array_equal(s[0], golden[k + "__col"])
        if val_type == VAL_F32:
            np.testing.assert_array_equal(val.astype(np.int32), src)
        elif val_type == VAL_BF16:
            np.testing.assert_array_equal(val, (src.astype(np.int64) & 0xFFFF).astype(np.uint16))


def test_simdify_d2_lanes_differ_and_rows_keep_their_entries(golden, mats):
    """The property simdify exists for: after it, the rows of every SIMD
    group hold pairwise different columns in every slot, and every row
    still holds exactly its own entries (slots moved inside the row)."""
    for case in SIMDIFY_CASES:
        m, d, t, w, c, extra, flag, kind = case
        k = key_simdify(*case)
        if kind != "d2" or not golden[k + "__ok"]:
            continue
        _, n, sell, leaves = _case(golden, mats, case)
        slot_row_before = _slot_rows(sell, c, n)
        assert _run(kind, d, w, c, flag, sell, sell[1], VAL_F64, leaves, n) == _lib.RACE_SUCCESS
        col, val, cs, rl, clp = sell
        src = val.astype(np.int64)
        owner = slot_row_before[src]
        here = _slot_rows(sell, c, n)
        assert np.array_equal(owner[here >= 0], here[here >= 0]), k
        first = 1 if flag else 0
        for ch in range(len(clp)):
            for g in range(c // w):
                base = ch * c + g * w
                lanes = min(w, n - base)
                if lanes <= 0:
                    break
                for j in range(first, clp[ch]):
                    s = cs[ch] + j * c + g * w
                    assert len(set(col[s:s + lanes])) == lanes, (k, ch, g, j)


def _slot_rows(sell, c, n):
    """Row of every SELL slot (-1 for the padding rows of the last chunk)."""
    col, val, cs, rl, clp = sell
    rows = np.full(col.size, -1, np.int64)
    for ch in range(len(clp)):
        r = np.arange(ch * c, ch * c + c)
        r = np.where(r < n, r, -1)
        rows[cs[ch]:cs[ch + 1]] = np.tile(r, clp[ch])
    return rows


def test_simdify_rejects_bad_arguments():
    L = _lib.lib()
    col = np.zeros(8, np.int32)
    cs = np.array([0, 8], np.int32)
    rl = np.full(4, 2, np.int32)
    clp = np.array([2], np.int32)
    lo, hi = np.array([0], np.int32), np.array([4], np.int32)

    def d2(w, c, lo=lo, hi=hi, val_type=VAL_F64):
        return L.race_simdify_schedule(w, c, 4, col.ctypes.data, cs.ctypes.data, rl.ctypes.data, clp.ctypes.data,
                                       None, val_type, 0, lo.ctypes.data, hi.ctypes.data, lo.size, None)

    bad = _lib.RACE_ERR_INVALID_ARG
    assert d2(3, 4) == bad                                   # C not a multiple of simdWidth
    assert d2(0, 4) == bad
    assert d2(4, 4, val_type=7) == bad
    assert d2(4, 4, hi=np.array([5], np.int32)) == bad        # leaf beyond the rows
    assert L.race_simdify_d1(3, 4, 4, col.ctypes.data, cs.ctypes.data, None, clp.ctypes.data, None, VAL_F64,
                             0) == bad
    assert L.race_simdify(None, 4, 4, 4, col.ctypes.data, cs.ctypes.data, rl.ctypes.data, clp.ctypes.data, None,
                          VAL_F64, 0, None) == bad


def test_python_mirror_simdify_d1(golden, mats):
    """Interface.simdifyD1 needs no engine: the Python mirror runs on the
    host and gives the reference's output."""
    case = ("aniso9_100x80", 1, 16, 4, 8, 0, True, "d1")
    k, n, sell, _ = _case(golden, mats, case)
    col, val, cs, rl, clp = sell
    iface = ri.Interface.__new__(ri.Interface)  # no engine
    iface._h = None
    assert iface.simdifyD1(4, 8, n, col, cs, rl, clp, val, dist2Compatible=True) is True
    np.testing.assert_array_equal(col, golden[k + "__col"])
    np.testing.assert_array_equal(val.astype(np.int32), golden[k + "__src"])
    with pytest.raises(TypeError):
        iface.simdifyD1(4, 8, n, col.astype(np.int64), cs, rl, clp, val)
    with pytest.raises(_lib.RaceError):
        iface.simdify(4, 8, n, col, cs, rl, clp, val)  # distance-2 needs a colored engine


@pytest.mark.gpu
def test_engine_simdify_matches_reference(golden, mats):
    """Interface.simdify on the engine's own coloring (its forward schedule
    pads the rows) equals the reference's Interface::simdify."""
    for case in [c for c in SIMDIFY_CASES if c[0] == "lap7_16" and c[7] == "d2"]:
        m, d, t, w, c, extra, flag, kind = case
        k, n, sell, _ = _case(golden, mats, case)
        A = mats[m]
        iface = ri.Interface(A.n, t, d, A.row_ptr, A.col, symm_hint=True)
        assert iface.RACEColor() == 0
        np.testing.assert_array_equal(iface.getPerm(), golden[k + "__perm"])
        col, val, cs, rl, clp = sell
        assert iface.simdify(w, c, n, col, cs, rl, clp, val, diagFirst=flag) is bool(golden[k + "__ok"])
        np.testing.assert_array_equal(col, golden[k + "__col"])
        np.testing.assert_array_equal(val.astype(np.int32), golden[k + "__src"])
        assert iface.getHighestPower() == 1
