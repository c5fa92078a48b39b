"""Issue order of the persistent matrix-power kernel (host only).

The GPU executor takes runs of (chunk, power) items from one ticket per L2
die queue, in the order race_mpk_issue_order returns; a run waits until the
chunks of its intervals are complete at the previous power. These tests
check, on the chunk dependency intervals of real RACE partitions (the
oracle's BFS levels and level groups, src/matrixPower.cpp:685-940), that

* every (chunk, power) item appears exactly once, in runs of consecutive
  chunks at one power of at most runLen chunks, each run on one die;
* each die's queue follows the global order;
* every chunk a run reads (its columns) is covered by its intervals;
* every chunk in a run's intervals was issued, at the previous power, in a
  run of smaller global rank, so no run waits on work behind it and the
  kernel cannot deadlock;
* for the chunk-level order, the live window: the matrix entries issued
  between two consecutive powers of one chunk, which is what has to stay in
  L2 for the second use to hit.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from oracle import oracle as orc
from race_gb300 import _lib, matgen


def chunk_tables(P, gp):
    """Chunks of <= 32 rows inside level groups and, per chunk, the chunk
    intervals its columns fall in within the previous/own/next group (the
    host restatement of mpk.cu's chunking and kChunkRanges)."""
    starts, groups = [], []
    for g in range(len(gp) - 1):
        for r in range(gp[g], gp[g + 1], 32):
            starts.append(r)
            groups.append(g)
    starts = np.array(starts + [P.n], np.int64)
    C_ = len(groups)
    groups = np.array(groups, np.int32)
    chunk_of_row = np.repeat(np.arange(C_), np.diff(starts))
    dep = np.zeros((C_, 6), np.int32)
    dep[:, 1::2] = -1
    reads = []
    for c in range(C_):
        cols = P.col[P.row_ptr[starts[c]]:P.row_ptr[starts[c + 1]]]
        ch = np.unique(chunk_of_row[cols])
        reads.append(ch)
        d = groups[ch] - groups[c] + 1
        assert d.min() >= 0 and d.max() <= 2
        for j in range(3):
            sel = ch[d == j]
            if len(sel):
                dep[c, 2 * j], dep[c, 2 * j + 1] = sel.min(), sel.max()
    return dep, groups, reads, starts


def issue_order(dep, groups, power, order=0, stride=2, seg=0, run=2, lag=0, dies=None, pass_groups=True):
    """Runs in queue order (die 0's queue, then die 1's), their global ranks
    and the queue bounds (pass_groups False: no chunk groups, so completion
    blocks follow the chunk index alone)."""
    L = _lib.lib()
    C_ = len(groups)
    dep = np.ascontiguousarray(dep, np.int32)
    groups = np.ascontiguousarray(groups, np.int32)
    gptr = groups.ctypes.data if pass_groups else None
    dies_a = None if dies is None else np.ascontiguousarray(dies, np.int32)
    dp = None if dies_a is None else dies_a.ctypes.data
    nr = C.c_int(0)
    _lib.check(L.race_mpk_issue_order(dep.ctypes.data, gptr, dp, C_, power, order, stride, seg, run,
                                      lag, None, None, None, None, 0, C.byref(nr)))
    head = np.zeros((nr.value, 4), np.int32)
    deps = np.zeros((nr.value, 8), np.int32)
    rank = np.zeros(nr.value, np.int32)
    ds = np.zeros(3, np.int32)
    _lib.check(L.race_mpk_issue_order(dep.ctypes.data, gptr, dp, C_, power, order, stride, seg, run,
                                      lag, head.ctypes.data, deps.ctypes.data, rank.ctypes.data, ds.ctypes.data,
                                      nr.value, C.byref(nr)))
    return head, deps, rank, ds


def partition(A, power, cache):
    perm, inv, lr, ln, _ = orc.traverse(A, 3, 0, A.n)
    P = A.permuted(perm, inv)
    lp = np.concatenate([[0], np.cumsum(lr)]).astype(np.int32)
    groups = orc.mpk_groups(power, A.n, A.nnz, cache, 2.0, 1 << 30, lp, ln)
    assert groups is not None
    return P, groups[0]


def two_dies(C_, s0, s1, block=16):
    """The engine's chunk-to-die rule (mpk_order.cpp chunkDies), restated:
    blocks of 16 chunks, block b on die 0 when die 0's share of blocks
    0..b grows by one."""
    b = np.arange(C_) // block
    return np.where((b + 1) * s0 // (s0 + s1) > b * s0 // (s0 + s1), 0, 1).astype(np.int32)


def check_order(head, deps, reads, power, run, rank, die_start, dies=None):
    C_ = len(reads)
    nr = len(head)
    assert sorted(rank.tolist()) == list(range(nr))
    assert die_start[0] == 0 and die_start[2] == nr
    for d in range(2):
        q = rank[die_start[d]:die_start[d + 1]]
        assert (np.diff(q) > 0).all(), "queue not in global order"
        for c0, c1, _, _ in head[die_start[d]:die_start[d + 1]]:
            assert ((dies[c0:c1] if dies is not None else np.zeros(c1 - c0)) == d).all(), "run on the wrong die"
    pos = -np.ones((power, C_), np.int64)  # rank of the run computing every item
    for i, (c0, c1, k, _) in enumerate(head):
        assert 0 <= k < power and 0 <= c0 < c1 <= C_ and c1 - c0 <= run
        assert (pos[k, c0:c1] < 0).all(), "item issued twice"
        pos[k, c0:c1] = rank[i]
    assert (pos >= 0).all(), "item missing"
    for i, (c0, c1, k, _) in enumerate(head):
        iv = deps[i].reshape(4, 2)
        if k == 0:
            assert (iv[:, 1] < iv[:, 0]).all()
            continue
        waited = np.zeros(C_, bool)
        for lo, hi in iv:
            if hi >= lo:
                waited[lo:hi + 1] = True
        assert (pos[k - 1, waited] < rank[i]).all(), "run waits on a later run"
        for c in range(c0, c1):
            assert waited[reads[c]].all(), "a read chunk is not waited for"


CASES = [
    ("st27_24", lambda: matgen.stencil3d_27pt(24), 8, 2e6),
    ("lap7_20", lambda: matgen.laplace3d_7pt(20), 4, 1e6),
    ("plaw_8k", lambda: matgen.powerlaw_chung_lu(8000, seed=4), 3, 4e6),
    ("band_6k", lambda: matgen.banded_scrambled(6000, 24, seed=5), 5, 1e6),
    ("aniso9_90x70", lambda: matgen.aniso2d(90, 70, 9, 12.0), 6, 5e5),
]


@pytest.mark.parametrize("name,gen,power,cache", CASES, ids=[c[0] for c in CASES])
def test_issue_orders_are_valid(name, gen, power, cache):
    A = gen()
    P, gp = partition(A, power, cache)
    dep, groups, reads, _ = chunk_tables(P, gp)
    dies = two_dies(len(groups), 72, 80)  # the SM split of a GB300's two dies
    for seg in (0, 1, 2, power):
        for run, lag in ((1, 0), (2, 0), (4, 0), (32, 0), (2, 7), (4, 300)):
            for dd in (None, dies):
                head, deps, rank, ds = issue_order(dep, groups, power, 0, seg=seg, run=run, lag=lag, dies=dd)
                check_order(head, deps, reads, power, run, rank, ds, dd)
                # flag bit 0 marks the last power of each segment
                s = power if seg in (0, power) else seg
                k = head[:, 2]
                assert np.array_equal(head[:, 3] & 1, ((k == power - 1) | ((k + 1) % s == 0)).astype(np.int32))
    for stride in (1, 2):
        head, deps, rank, ds = issue_order(dep, groups, power, 1, stride=stride)
        check_order(head, deps, reads, power, 1, rank, ds)


def test_completion_blocks_widen_dependencies():
    """The kernel counts finished chunks per completion block (at most 16
    consecutive chunks, inside one level group when groups are given), so
    every dependency interval is widened to whole blocks; the widened
    orders stay valid (every chunk of every polled block comes earlier),
    with groups and by chunk index alone."""
    power = 4
    A = matgen.stencil3d_27pt(20)
    P, gp = partition(A, power, 1e6)
    dep, groups, reads, _ = chunk_tables(P, gp)
    dies = two_dies(len(groups), 72, 80)
    starts = np.flatnonzero((np.arange(len(groups)) % 16 == 0) | np.r_[True, groups[1:] != groups[:-1]])
    for pass_groups in (True, False):
        for run, lag in ((1, 0), (4, 0), (4, 300)):
            head, deps, rank, ds = issue_order(dep, groups, power, 0, run=run, lag=lag, dies=dies,
                                               pass_groups=pass_groups)
            check_order(head, deps, reads, power, run, rank, ds, dies)
            iv = deps.reshape(-1, 2)
            iv = iv[iv[:, 1] >= iv[:, 0]]
            block_starts = starts if pass_groups else np.arange(0, len(groups), 16)
            assert np.isin(iv[:, 0], block_starts).all()  # every interval begins a block
            ends = np.r_[block_starts[1:], len(groups)] - 1
            assert np.isin(iv[:, 1], ends).all()  # and ends one
    head, deps, rank, ds = issue_order(dep, groups, power, 1, stride=1)
    check_order(head, deps, reads, power, 1, rank, ds)


def test_chunk_wavefront_live_window():
    """On the 27-point stencil the chunk-level order keeps a chunk's
    consecutive powers about one level apart, where RACE's level-group order
    with stride 2 keeps them 2p-1 groups apart: fewer matrix entries are
    issued between two uses of a chunk."""
    power = 8
    A = matgen.stencil3d_27pt(32)
    P, gp = partition(A, power, 2e6)
    dep, groups, reads, starts = chunk_tables(P, gp)
    nnz_chunk = P.row_ptr[starts[1:]] - P.row_ptr[starts[:-1]]

    def reuse_nnz(head):
        seq = np.concatenate([np.arange(a, b) for a, b, _, _ in head])
        cum = np.concatenate([[0], np.cumsum(nnz_chunk[seq])])
        slot, t = {}, 0
        for a, b, k, _ in head:
            for c in range(a, b):
                slot[(k, c)] = t
                t += 1
        gaps = [cum[slot[(k + 1, c)]] - cum[slot[(k, c)]] for c in range(len(reads)) for k in range(power - 1)]
        return float(np.median(gaps))

    chunk = reuse_nnz(issue_order(dep, groups, power, 0, run=2)[0])
    group2 = reuse_nnz(issue_order(dep, groups, power, 1, stride=2)[0])
    assert chunk < 0.75 * group2, (chunk, group2)


def test_issue_order_rejects_bad_input():
    L = _lib.lib()
    nr = C.c_int(0)
    g = np.zeros(1, np.int32)

    def call(dep, die, power, run):
        return L.race_mpk_issue_order(dep.ctypes.data, g.ctypes.data, die, 1, power, 0, 2, 0, run, 0, None, None,
                                      None, None, 0, C.byref(nr))

    assert call(np.array([0, 0, 0, 5, 0, -1], np.int32), None, 2, 2) == _lib.RACE_ERR_INVALID_ARG  # past the end
    ok = np.array([0, 0, 0, 0, 0, -1], np.int32)
    assert call(ok, None, 2, 33) == _lib.RACE_ERR_INVALID_ARG  # a run is at most a warp's 32 flags
    assert call(ok, None, 0, 2) == _lib.RACE_ERR_INVALID_ARG  # power 0
    bad_die = np.array([2], np.int32)
    assert call(ok, bad_die.ctypes.data, 2, 2) == _lib.RACE_ERR_INVALID_ARG
    assert call(ok, None, 2, 2) == _lib.RACE_SUCCESS and nr.value == 2
