"""ctypes bindings for the C restatement oracle (oracle/race_oracle.c).

TEST INFRASTRUCTURE ONLY: loaded by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py to check or time the reference algorithm. The
product never imports this module.
"""
from __future__ import annotations

import ctypes as C
import os
import pathlib
import subprocess

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
SRC = HERE / "race_oracle.c"
OUT_DIR = HERE / "_build"
LIB = OUT_DIR / "librace_oracle.so"

IP = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
DP = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")

K_SPMV, K_SPMTV, K_SYMMSPMV, K_GS, K_KACZ = 0, 1, 2, 3, 4

_lib = None


def build(force: bool = False) -> pathlib.Path:
    """Compile the oracle with -O3 -fopenmp and no floating-point contraction
    (every fused multiply-add in the source is an explicit fma())."""
    OUT_DIR.mkdir(exist_ok=True)
    if force or not LIB.exists() or LIB.stat().st_mtime < SRC.stat().st_mtime:
        tmp = LIB.with_suffix(f".{os.getpid()}.tmp")
        subprocess.check_call(["gcc", "-O3", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", "-std=c11",
                               str(SRC), "-o", str(tmp), "-lm"])
        os.replace(tmp, LIB)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB))
        L.orc_bfs.restype = C.c_int
        L.orc_bfs.argtypes = [C.c_int, IP, IP, IP, IP, C.c_int, C.c_int, C.c_int, IP]
        L.orc_bfs_boundary.restype = C.c_int
        L.orc_bfs_boundary.argtypes = [C.c_int, IP, IP, IP, IP, C.c_int, C.c_int, C.c_int, IP, IP, IP]
        L.orc_level_data.argtypes = [IP, IP, IP, C.c_int, C.c_int, C.c_int, IP, IP]
        L.orc_level_permute.argtypes = [C.c_int, IP, C.c_int, C.c_int, C.c_int, IP, IP]
        for nm in ["orc_spmv_range", "orc_spmtv_range", "orc_symmspmv_range"]:
            getattr(L, nm).argtypes = [C.c_int, C.c_int, IP, IP, DP, DP, DP]
        for nm in ["orc_gs_range", "orc_kacz_range"]:
            getattr(L, nm).argtypes = [C.c_int, C.c_int, IP, IP, DP, DP, DP]
        L.orc_exec_tree.argtypes = [C.c_int, IP, IP, IP, IP, IP, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                    IP, IP, DP, DP, DP]
        L.orc_exec_phases_omp.argtypes = [C.c_int, C.c_int, IP, IP, IP, C.c_int, C.c_int, IP, IP, DP, DP, DP]
        L.orc_mpk_plain.argtypes = [C.c_int, C.c_int, IP, IP, DP, DP]
        FP = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
        L.orc_mpk_block.argtypes = [C.c_int, C.c_int, C.c_int, IP, IP, DP, DP]
        L.orc_mpk_block_f32.argtypes = [C.c_int, C.c_int, C.c_int, IP, IP, FP, FP]
        L.orc_mpk_groups.restype = C.c_int
        L.orc_mpk_groups.argtypes = [C.c_int, C.c_int, C.c_longlong, C.c_double, C.c_double, C.c_int, C.c_int,
                                     IP, IP, IP, IP, IP]
        L.orc_mpk_partition.restype = C.c_int
        L.orc_mpk_partition.argtypes = [C.c_int, C.c_int, C.c_longlong, C.c_double, C.c_double, C.c_int, C.c_int,
                                        IP, IP, C.c_int, IP, IP, IP, C.POINTER(C.c_int), IP]
        L.orc_mpk_unlock_ctr.argtypes = [C.c_int, IP, IP, C.c_int, IP]
        L.orc_mpk_wavefront.argtypes = [C.c_int, C.c_int, C.c_int, IP, IP, IP, C.c_int, IP, IP, DP, DP]
        _lib = L
    return _lib


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def bfs(csr, dist: int, lo: int, hi: int, total_perm=None, total_inv=None):
    """Distances of rows [lo,hi) in the current permuted space."""
    n = csr.n
    tp = _i32(np.arange(n) if total_perm is None else total_perm)
    ti = _i32(np.arange(n) if total_inv is None else total_inv)
    d = np.zeros(n, np.int32)
    L = lib().orc_bfs(n, _i32(csr.row_ptr), _i32(csr.col), tp, ti, dist, lo, hi, d)
    if L < 0:
        raise RuntimeError("oracle BFS: some rows went missing")
    return d, L


def traverse(csr, dist: int, lo: int, hi: int, total_perm=None, total_inv=None):
    """One RACE traversal step: distances, level histograms and the composed
    permutation (same outputs as the reference's Traverse on [lo,hi))."""
    n = csr.n
    tp = _i32(np.arange(n) if total_perm is None else total_perm).copy()
    ti = _i32(np.arange(n) if total_inv is None else total_inv).copy()
    d, L = bfs(csr, dist, lo, hi, tp, ti)
    lr = np.zeros(max(L, 1), np.int32); ln = np.zeros(max(L, 1), np.int32)
    lib().orc_level_data(_i32(csr.row_ptr), tp, d, lo, hi, L, lr, ln)
    lib().orc_level_permute(n, d, lo, hi, L, tp, ti)
    return tp, ti, lr[:L], ln[:L], d


def traverse_boundary(csr, lo: int, hi: int, regions, total_perm, total_inv, region_levels: bool = False):
    """One traversal of a recursion stage of the MPK partition: rows [lo,hi)
    with boundary regions [(lo_k, hi_k), ...] (orc_bfs_boundary), then the
    range and every boundary region each stably sorted by level and composed
    into the running permutation (permuteGraph, traverse_GAP_graphSoA.cpp:
    506-575). Returns the new (total_perm, total_inv, level rows and level
    non-zeros of [lo,hi), number of levels), and with region_levels also the
    (level rows, level non-zeros) of every boundary region
    (createLevelData, :449-504)."""
    n = csr.n
    tp = _i32(total_perm).copy()
    ti = _i32(total_inv).copy()
    blo = _i32([a for a, _ in regions] or [0])
    bhi = _i32([b for _, b in regions] or [0])
    d = np.zeros(n, np.int32)
    L = lib().orc_bfs_boundary(n, _i32(csr.row_ptr), _i32(csr.col), tp, ti, lo, hi, len(regions), blo, bhi, d)
    if L < 0:
        raise RuntimeError("oracle BFS: some rows went missing")
    lr = np.zeros(L, np.int32)
    ln = np.zeros(L, np.int32)
    lib().orc_level_data(_i32(csr.row_ptr), tp, d, lo, hi, L, lr, ln)
    per_region = []
    for a, b in regions:
        rr, rn = np.zeros(L, np.int32), np.zeros(L, np.int32)
        lib().orc_level_data(_i32(csr.row_ptr), tp, d, a, b, L, rr, rn)
        per_region.append((rr, rn))
    for a, b in [(lo, hi)] + list(regions):
        lib().orc_level_permute(n, d, a, b, L, tp, ti)
    if region_levels:
        return tp, ti, lr, ln, L, per_region
    return tp, ti, lr, ln, L


INT_MAX = 2**31 - 1


def mpk_partition(p: int, nrow: int, nnz: int, cache_bytes: float, safety: float, cutoff: int, level_ptr, level_nnz,
                  bnd_ptrs=()):
    """One stage of the MPK partition with hopeless regions
    (orc_mpk_partition): (group row offsets, hopeless group indices, each
    boundary region's offsets at the group starts), or None."""
    L = len(level_nnz)
    nb = len(bnd_ptrs)
    gp = np.zeros(L + 1, np.int32)
    hid = np.zeros(max(L, 1), np.int32)
    nh = C.c_int()
    bp = np.ascontiguousarray(np.concatenate([_i32(b) for b in bnd_ptrs]) if nb else np.zeros(1, np.int32), np.int32)
    bgp = np.zeros(max(nb * (L + 1), 1), np.int32)
    ng = lib().orc_mpk_partition(p, nrow, nnz, float(cache_bytes), float(safety), int(cutoff), L, _i32(level_ptr),
                                 _i32(level_nnz), nb, bp, gp, hid, C.byref(nh), bgp)
    if ng < 0:
        return None
    bgps = [bgp[k * (L + 1): k * (L + 1) + ng + 1].copy() for k in range(nb)]
    return gp[: ng + 1].copy(), hid[: nh.value].copy(), bgps


def mpk_recursive(csr, p: int, cache_bytes: float, safety: float, stage_cutoffs):
    """RACE's MPK partition with its recursion into hopeless groups
    (mtxPowerRecursive::findPartition / recursivePartition,
    matrixPowerRecursive.cpp:156-436), composed from the oracle's traversals
    and orc_mpk_partition. stage_cutoffs[s] is the cut-off of stage s
    (INT_MAX beyond the list). Depth first, each hopeless group h of a leaf
    becomes a leaf whose boundaries are the leaf's groups h-w..h+w but h and,
    of each of the leaf's boundary regions, its groups h-w..h+w with h-1..h+1
    as one range (w = ceil(p/2)-1, empty ranges left out); the leaf is
    traversed with them, partitioned (boundary non-zeros counted per level)
    and recursed into before its next sibling. Returns (tree, total_perm,
    total_inv): tree is a list of dicts lo, hi, stage, parent, lp, hid in the
    reference's order; None if a partition fails."""
    n = csr.n
    nnz = int(csr.row_ptr[-1])
    cut = list(stage_cutoffs)
    tp, ti, lr, ln, L = traverse(csr, 3, 0, n)
    lp0 = np.concatenate([[0], np.cumsum(lr)]).astype(np.int32)
    part = mpk_partition(p, n, nnz, cache_bytes, safety, cut[0] if cut else INT_MAX, lp0, ln)
    if part is None:
        return None
    tree = [dict(lo=0, hi=n, stage=0, parent=-1, lp=[int(v) for v in part[0]], hid=[int(v) for v in part[1]])]
    w = (p + 1) // 2 - 1
    state = {"tp": tp, "ti": ti}

    def recurse(parent, bgps):
        leaf = tree[parent]
        gp, stage = leaf["lp"], leaf["stage"] + 1
        cutoff = cut[stage] if stage < len(cut) else INT_MAX
        for h in list(leaf["hid"]):
            regions = []
            if w > 0:
                for bp in bgps:
                    r = -w
                    while r <= w:
                        if r == -1:
                            a, b = bp[h - 1], bp[h + 2]
                            r = 1
                        else:
                            a, b = bp[h + r], bp[h + r + 1]
                        if b > a:
                            regions.append((int(a), int(b)))
                        r += 1
            regions += [(gp[h + r], gp[h + r + 1]) for r in range(-w, w + 1) if r != 0 and gp[h + r + 1] > gp[h + r]]
            lo, hi = gp[h], gp[h + 1]
            state["tp"], state["ti"], clr, cln, CL, reg = traverse_boundary(csr, lo, hi, regions, state["tp"],
                                                                            state["ti"], region_levels=True)
            lvl_ptr = np.concatenate([[lo], lo + np.cumsum(clr)]).astype(np.int32)
            lvl_nnz = cln.astype(np.int64) + sum((rn.astype(np.int64) for _, rn in reg), np.zeros(CL, np.int64))
            bnd = [np.concatenate([[a], a + np.cumsum(rr)]).astype(np.int32) for (a, _), (rr, _) in zip(regions, reg)]
            part = mpk_partition(p, n, nnz, cache_bytes, safety, cutoff, lvl_ptr, lvl_nnz.astype(np.int32), bnd)
            if part is None:
                return False
            tree.append(dict(lo=int(lo), hi=int(hi), stage=stage, parent=parent, lp=[int(v) for v in part[0]],
                             hid=[int(v) for v in part[1]]))
            if part[1].size and not recurse(len(tree) - 1, part[2]):
                return False
        return True

    if not recurse(0, []):
        return None
    return tree, state["tp"], state["ti"]


def flat_power_tree(tree):
    """A tree of mpk_recursive flattened like the golden fixtures: count,
    then per leaf lo, hi, stage, parent, groups, lp, hopeless count, hid."""
    flat = [len(tree)]
    for leaf in tree:
        flat += [leaf["lo"], leaf["hi"], leaf["stage"], leaf["parent"], len(leaf["lp"]) - 1] + list(leaf["lp"])
        flat += [len(leaf["hid"])] + list(leaf["hid"])
    return np.array(flat, np.int32)


def run_kernel(kernel: int, start: int, end: int, csr, x, b):
    fn = {K_SPMV: "orc_spmv_range", K_SPMTV: "orc_spmtv_range", K_SYMMSPMV: "orc_symmspmv_range",
          K_GS: "orc_gs_range", K_KACZ: "orc_kacz_range"}[kernel]
    getattr(lib(), fn)(start, end, _i32(csr.row_ptr), _i32(csr.col), _f64(csr.val), x, b)


def tree_arrays(nodes):
    """Flatten a parsed zone tree (list of dicts with value/children/subblocks)."""
    vs = np.zeros(len(nodes) + 1, np.int32)
    cs = np.zeros(len(nodes) + 1, np.int32)
    for i, z in enumerate(nodes):
        vs[i + 1] = vs[i] + len(z["value"])
        cs[i + 1] = cs[i] + len(z["children"])
    val = np.array([v for z in nodes for v in z["value"]] or [0], np.int32)
    ch = np.array([c for z in nodes for c in z["children"]] or [0], np.int32)
    sb = np.array([z["subblocks"] for z in nodes], np.int32)
    return vs, val, cs, ch, sb


def exec_tree(nodes, block_per_thread: int, serial_part, kernel: int, rev: bool, pcsr, x, b):
    """Run `kernel` over the zone tree sequentially in RACE's execution order."""
    vs, val, cs, ch, sb = tree_arrays(nodes)
    lib().orc_exec_tree(len(nodes), vs, val, cs, ch, sb, block_per_thread, int(serial_part[0]),
                        int(serial_part[1]), kernel, int(rev), _i32(pcsr.row_ptr), _i32(pcsr.col),
                        _f64(pcsr.val), x, b)


def exec_phases_omp(kernel: int, phase_ptr, leaf_lo, leaf_hi, nthreads: int, reps: int, pcsr, x, b):
    """The colored executor on `nthreads` OpenMP threads over a phase table
    (x and b float64 arrays, updated in place; `reps` calls)."""
    lib().orc_exec_phases_omp(kernel, len(phase_ptr) - 1, _i32(phase_ptr), _i32(leaf_lo), _i32(leaf_hi),
                              int(nthreads), int(reps), _i32(pcsr.row_ptr), _i32(pcsr.col), _f64(pcsr.val), x, b)


def mpk_plain(csr, x0, p: int):
    x = np.zeros((p + 1) * csr.n)
    x[: csr.n] = x0
    lib().orc_mpk_plain(csr.n, p, _i32(csr.row_ptr), _i32(csr.col), _f64(csr.val), x)
    return x.reshape(p + 1, csr.n)


def mpk_block(csr, x0, p: int, val=None):
    """Block matrix power: x0 is (n, nrhs); returns (p+1, n, nrhs). FP64
    fma chains, or FP32 fmaf chains when x0 is float32 (then ``val`` may give
    the float32 values, e.g. BF16 values widened exactly)."""
    x0 = np.asarray(x0)
    n, nrhs = x0.shape
    if x0.dtype == np.float32:
        v = np.ascontiguousarray(csr.val if val is None else val, dtype=np.float32)
        x = np.zeros((p + 1) * n * nrhs, np.float32)
        x[: n * nrhs] = x0.reshape(-1)
        lib().orc_mpk_block_f32(n, p, nrhs, _i32(csr.row_ptr), _i32(csr.col), v, x)
    else:
        x = np.zeros((p + 1) * n * nrhs)
        x[: n * nrhs] = x0.reshape(-1)
        lib().orc_mpk_block(n, p, nrhs, _i32(csr.row_ptr), _i32(csr.col), _f64(csr.val), x)
    return x.reshape(p + 1, n, nrhs)


def mpk_groups(p: int, nrow: int, nnz: int, cache_bytes: float, safety: float, cutoff: int, level_ptr, level_nnz):
    L = len(level_nnz)
    gp = np.zeros(L + 2, np.int32); ur = np.zeros(L + 2, np.int32); dr = np.zeros(L + 2, np.int32)
    ng = lib().orc_mpk_groups(p, nrow, nnz, float(cache_bytes), float(safety), cutoff, L, _i32(level_ptr),
                              _i32(level_nnz), gp, ur, dr)
    if ng < 0:
        return None
    return gp[: ng + 1].copy(), ur[:ng].copy(), dr[:ng].copy()


def mpk_wavefront(pcsr, x0, p: int, group_ptr, unlock_row, danger_row, nthreads: int):
    """Run the reference's level-group wavefront on `nthreads` OpenMP threads
    (the CPU baseline)."""
    ng = len(group_ptr) - 1
    x = np.zeros((p + 1) * pcsr.n)
    x[: pcsr.n] = x0
    lib().orc_mpk_wavefront(pcsr.n, p, ng, _i32(group_ptr), _i32(unlock_row), _i32(danger_row), int(nthreads),
                            _i32(pcsr.row_ptr), _i32(pcsr.col), _f64(pcsr.val), x)
    return x.reshape(p + 1, pcsr.n)
