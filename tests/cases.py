"""Parity cases shared by the golden generator and the tests.

Matrices are regenerated from race_gb300.matgen (seeded, platform
independent); each golden entry also stores a digest of the matrix so a
change in a generator is caught instead of silently comparing different
inputs.
"""
from __future__ import annotations

import hashlib

import numpy as np

from race_gb300 import matgen

def _arrow(n: int):
    """Arrow matrix: row 0 full, every other row its diagonal and column 0."""
    cols = [np.arange(n)] + [np.array([0, r]) for r in range(1, n)]
    rp = np.concatenate([[0], np.cumsum([len(c) for c in cols])]).astype(np.int32)
    col = np.concatenate(cols).astype(np.int32)
    val = np.where(col == np.repeat(np.arange(n), np.diff(rp)), float(n), -1.0)
    return matgen.Csr(n, rp, col, val, f"arrow_{n}")


# name -> generator
MATRICES = {
    "lap7_32": lambda: matgen.laplace3d_7pt(32),          # 32^3 7-point Laplacian (n=32,768)
    "lap7_16": lambda: matgen.laplace3d_7pt(16),
    "st27_16": lambda: matgen.stencil3d_27pt(16),
    "st27_24": lambda: matgen.stencil3d_27pt(24),
    "st27_40": lambda: matgen.stencil3d_27pt(40),
    "plaw_20k": lambda: matgen.powerlaw_chung_lu(20000, seed=2),
    "plaw_3k": lambda: matgen.powerlaw_chung_lu(3000, seed=1),
    "band_5k": lambda: matgen.banded_scrambled(5000, 16, seed=3),
    "aniso5_120x90": lambda: matgen.aniso2d(120, 90, 5, 30.0),
    "aniso9_100x80": lambda: matgen.aniso2d(100, 80, 9, 7.0),
    # edge cases: disconnected pieces and diagonal-only rows (islands), rows scrambled
    "islands_330": lambda: matgen.islands(0),
    # a single row
    "tiny_1": lambda: matgen.Csr(1, np.array([0, 1], np.int32), np.array([0], np.int32), np.array([3.0]), "tiny_1"),
    # rows of two entries that share column 0: too few columns for wide SIMD groups
    "arrow_64": lambda: _arrow(64),
}

# (matrix, dist, nthreads)
COLOR_CASES = [
    ("lap7_32", 2, 8), ("lap7_32", 2, 64), ("lap7_32", 2, 1024), ("lap7_32", 1, 8), ("lap7_32", 1, 256),
    ("lap7_16", 2, 16), ("st27_16", 2, 128), ("plaw_20k", 2, 64), ("plaw_3k", 1, 32), ("band_5k", 2, 32),
    ("aniso9_100x80", 1, 16), ("aniso5_120x90", 2, 48), ("islands_330", 1, 8), ("islands_330", 2, 16),
    ("tiny_1", 1, 4),
]

# distance-2 colorings with RACE::THREE_BLOCK (three blocks per thread,
# macros.h:29-38): (matrix, nthreads); reference sweep outputs are stored for
# all of them
COLOR3_CASES = [("lap7_16", 16), ("band_5k", 32), ("plaw_3k", 16), ("islands_330", 8), ("aniso5_120x90", 48)]


# colorings that start from an initial permutation (the Interface ctor's
# initPerm): (matrix, dist, nthreads); the permutation is a seeded shuffle
COLOR_INIT_CASES = [("lap7_16", 2, 16), ("aniso9_100x80", 1, 16), ("plaw_3k", 2, 16), ("islands_330", 1, 8)]


def init_perm(n: int, seed: int = 5) -> np.ndarray:
    return np.random.default_rng(seed).permutation(n).astype(np.int32)


def key_color_init(m, d, t):
    return f"colorinit__{m}__d{d}__t{t}"


# colorings with RACE's environment knobs (level_recursion.cpp:48-90: a
# per-stage efficiency list after the default 40, and per-stage thread
# requests that drop that stage's efficiency to 0): (matrix, dist, nthreads,
# environment)
COLOR_ENV_CASES = [
    ("lap7_32", 2, 64, {"RACE_EFFICIENCY": "60,30"}),
    ("lap7_32", 1, 256, {"RACE_EFFICIENCY": "10"}),
    ("band_5k", 2, 32, {"RACE_THREADS": "4", "RACE_EFFICIENCY": "40"}),
    ("plaw_3k", 1, 32, {"RACE_THREADS": "8,2", "RACE_EFFICIENCY": "50,50"}),
    ("lap7_16", 2, 16, {"RACE_EFFICIENCY": "80"}),
]


# colorings that balance rows instead of non-zeros (RACE::ROW load-balancer
# target): (matrix, dist, nthreads)
COLOR_ROW_CASES = [("lap7_32", 2, 64), ("plaw_3k", 1, 32), ("band_5k", 2, 32), ("aniso5_120x90", 2, 48)]


def key_color_row(m, d, t):
    return f"colorrow__{m}__d{d}__t{t}"


# colorings at the edges of the thread count: one thread, odd and prime
# counts, far more threads than the matrix can use: (matrix, dist, nthreads)
COLOR_EDGE_CASES = [("lap7_16", 2, 1), ("lap7_16", 1, 1), ("band_5k", 1, 3), ("aniso5_120x90", 2, 7),
                    ("plaw_3k", 2, 1000), ("islands_330", 1, 2), ("arrow_64", 2, 5), ("st27_16", 2, 13),
                    ("aniso9_100x80", 2, 4096), ("tiny_1", 2, 1)]


# edge colorings whose reference sweep outputs are stored
COLOR_EDGE_EXEC = {("aniso5_120x90", 2, 7), ("plaw_3k", 2, 1000), ("st27_16", 2, 13), ("arrow_64", 2, 5),
                   ("band_5k", 1, 3)}


def key_color_edge(m, d, t):
    return f"coloredge__{m}__d{d}__t{t}"


# colorings of matrices whose pattern is not symmetric (a triangle), with
# symm_hint false, so that RACE first adds the missing transposed entries
# (makeSymmetricGraph, graph.cpp:47-142): (matrix, triangle, dist, nthreads)
COLOR_UNSYM_CASES = [("lap7_16", "U", 2, 16), ("plaw_3k", "L", 1, 32), ("aniso9_100x80", "L", 2, 16)]


def key_color_unsym(m, tri, d, t):
    return f"colorunsym__{m}__{tri}__d{d}__t{t}"


def symmetrized_pattern(csr):
    """makeSymmetricGraph: every entry (r, c), c != r, without its pair adds
    (c, r) after row c's own entries (in the order the entries are met)."""
    n = csr.n
    rp = np.asarray(csr.row_ptr, np.int64)
    col = np.asarray(csr.col, np.int64)
    rows = np.repeat(np.arange(n), np.diff(rp))
    present = set(zip(rows.tolist(), col.tolist()))
    extra = [[] for _ in range(n)]
    for r, c in zip(rows.tolist(), col.tolist()):
        if c != r and (c, r) not in present:
            extra[c].append(r)
    cols = [np.concatenate([col[rp[r]:rp[r + 1]], np.array(extra[r], np.int64)]) for r in range(n)]
    nrp = np.concatenate([[0], np.cumsum([len(c) for c in cols])]).astype(np.int32)
    ncol = np.concatenate(cols).astype(np.int32)
    return matgen.Csr(n, nrp, ncol, np.ones(ncol.size), csr.name + "_sym")


def key_color_env(m, d, t, env):
    return f"colorenv__{m}__d{d}__t{t}__" + "_".join(f"{k}={v}" for k, v in sorted(env.items()))


def key_color3(m, t):
    return f"color3__{m}__t{t}"


# coloring cases whose reference sweep outputs are stored
EXEC_CASES = {("lap7_16", 2, 16), ("aniso9_100x80", 1, 16), ("plaw_3k", 1, 32), ("islands_330", 2, 16)}

# (matrix, power, cacheBytes)
POWER_CASES = [
    ("st27_24", 8, 2e6), ("st27_40", 8, 8e6), ("lap7_32", 4, 1e6), ("aniso5_120x90", 4, 5e5),
    ("plaw_20k", 4, 1e6), ("band_5k", 6, 3e5), ("islands_330", 3, 2e4), ("tiny_1", 2, 1e4),
    # levels over the cache cut-off, none of them consecutive: no hopeless
    # region, so the reference partitions without recursion
    ("band_5k", 8, 3300), ("band_5k", 6, 2500),
]

# (matrix, power, cacheBytes) with consecutive levels over the cut-off: the
# reference recurses into the hopeless region by default; with
# RACE_MAX_RECURSION_STAGES=0 it partitions without recursion, as the engine
# does with max_recursion_stages = 0
POWER_FLAT_CASES = [("plaw_20k", 4, 1e4), ("lap7_32", 4, 1e4)]

# (matrix, power, cacheBytes) with hopeless regions at the default settings:
# the reference's stage-0 level groups and hopeless groups (before its
# recursion, which reorders rows inside groups only) are stored
HOPELESS_CASES = POWER_FLAT_CASES + [("band_5k", 8, 3000), ("band_5k", 8, 2500), ("band_5k", 8, 3200),
                                     ("plaw_3k", 4, 2e3), ("lap7_16", 4, 2e4), ("st27_24", 8, 1e5)]


# MPK partitions with other safety factors (RACEColor's safetyFactor,
# interface.cpp:205): (matrix, power, cacheBytes, safety)
POWER_SAFETY_CASES = [("st27_24", 8, 2e6, 1.0), ("band_5k", 6, 3e5, 4.0), ("plaw_20k", 4, 1e6, 1.5),
                      ("lap7_32", 4, 1e5, 8.0)]


def key_power_safety(m, p, c, safety):
    return f"powersafety__{m}__p{p}__c{int(c)}__s{safety:g}"


def key_hopeless(m, p, c):
    return f"hopeless__{m}__p{p}__c{int(c)}"


# MPK partitions that recurse deeper than one stage: (matrix, power,
# cacheBytes, RACE_MAX_RECURSION_STAGES (-1: unset), RACE_CACHE_VIOLATION_CUTOFF
# list). The reference's whole leaf tree and permutation are stored. Powers
# 2, 3-4, 5-6 and 8 give boundary widths ceil(p/2)-1 = 0, 1, 2 and 3.
DEEP_CASES = [("band_5k", 8, 3000, 2, ()), ("band_5k", 8, 3000, -1, (50, 1)), ("band_5k", 8, 3000, 3, (50, 1, 1)),
              ("plaw_3k", 3, 2000, 3, (50, 2, 1)), ("st27_24", 2, 2000, 3, (50, 2, 1)),
              ("st27_24", 5, 20000, 3, (50, 2, 1)), ("lap7_32", 4, 10000, 2, ()),
              ("aniso5_120x90", 6, 2000, 3, (50, 2, 1)), ("plaw_20k", 4, 10000, 2, ())]
# deep cases whose reference MPK outputs are stored
DEEP_EXEC_CASES = {("band_5k", 8, 3000, -1, (50, 1)), ("plaw_3k", 3, 2000, 3, (50, 2, 1))}


# MPK partitions at edge parameters (default recursion): power 1 and high
# powers, a budget that holds the whole matrix in one group, tiny budgets
# (hopeless regions, also with power 1), a one-row matrix, islands:
# (matrix, power, cacheBytes). The whole leaf tree and permutation are stored.
POWER_EDGE_CASES = [("lap7_16", 1, 1e4), ("band_5k", 16, 1e5), ("st27_16", 8, 1e9), ("lap7_32", 3, 1e3),
                    ("islands_330", 5, 1e3), ("tiny_1", 4, 1e2), ("aniso9_100x80", 12, 2e4), ("plaw_20k", 2, 1e3),
                    ("arrow_64", 3, 50), ("st27_24", 1, 1e3)]


def key_power_edge(m, p, c):
    return f"poweredge__{m}__p{p}__c{int(c)}"


def key_deep(m, p, c, stages, cuts):
    return f"deep__{m}__p{p}__c{int(c)}__s{stages}__k{'-'.join(str(v) for v in cuts)}"


def deep_stage_cutoffs(stages, cuts, default=50):
    """The cut-off of each recursion stage s < the maximal depth
    (get_cache_violation_cutoff, matrixPowerRecursive.cpp:81-100); deeper
    stages have none (INT_MAX)."""
    cv = [default] + list(cuts)
    depth = stages if stages >= 0 else len(cv)
    return [cv[s + 1] if s < len(cv) - 1 else cv[0] for s in range(depth)]


# (matrix, triangle, power, cacheBytes): the lower ("L") or upper ("U")
# triangle of the matrix, partitioned with mtxType L / U (one row per level,
# traverse_GAP_graphSoA.cpp:316-335)
POWER_TRI_CASES = [("lap7_16", "L", 4, 2e4), ("lap7_16", "U", 4, 2e4), ("plaw_3k", "L", 3, 1e5),
                   ("plaw_3k", "U", 8, 5e4)]

# simdify cases on colored matrices (each golden entry stores its own
# permutation and zone tree): (matrix, dist, nthreads, simdWidth, C, extra padded slots per chunk, flag, pass)
# pass "d2": Interface::simdify, flag = diagFirst; pass "d1": simdifyD1,
# flag = dist2Compatible. islands_330 with simdWidth 7 and tiny_1 have a
# last SIMD group of one row; arrow_64 cannot be simdified for 4 lanes.
SIMDIFY_CASES = [
    ("lap7_16", 2, 16, 4, 8, 0, False, "d2"), ("lap7_16", 2, 16, 4, 8, 2, True, "d2"),
    ("islands_330", 2, 16, 4, 4, 1, False, "d2"), ("band_5k", 2, 32, 8, 32, 0, True, "d2"),
    ("aniso5_120x90", 2, 48, 32, 32, 0, False, "d2"), ("plaw_3k", 2, 16, 4, 8, 0, False, "d2"),
    ("lap7_16", 2, 64, 8, 8, 0, False, "d2"),
    ("aniso9_100x80", 1, 16, 4, 8, 0, False, "d1"), ("aniso9_100x80", 1, 16, 4, 8, 0, True, "d1"),
    ("plaw_3k", 1, 32, 8, 32, 1, False, "d1"), ("lap7_16", 1, 8, 4, 4, 0, True, "d1"),
    ("islands_330", 1, 8, 7, 14, 0, False, "d1"), ("tiny_1", 1, 4, 4, 4, 0, False, "d1"),
    ("arrow_64", 2, 4, 4, 4, 0, False, "d2"), ("arrow_64", 1, 4, 4, 8, 0, False, "d1"),
]


def key_simdify(m, d, t, w, c, extra, flag, kind):
    return f"simd__{kind}__{m}__d{d}__t{t}__w{w}__c{c}__e{extra}__f{int(flag)}"


def sell_layout(csr, C, extra=0, diag_first=False):
    """SELL-C-1 arrays of a CRS matrix in RACE simdify's layout (entry j of
    row r at chunkStart[r // C] + r % C + j * C): col, val, chunkStart
    (chunks + 1), rl, clp. Every chunk is `extra` slots longer than its
    longest row; a row's padding points at the row itself, the padding rows
    of the last chunk at column 0. val numbers the slots (0, 1, ...) so that
    a rearranged val records where each entry came from. diag_first moves
    each row's diagonal entry to slot 0."""
    n = csr.n
    rp = np.asarray(csr.row_ptr, np.int64)
    rl = np.diff(rp).astype(np.int32)
    nch = (n + C - 1) // C
    padded = np.zeros(nch * C, np.int32)
    padded[:n] = rl
    clp = (padded.reshape(nch, C).max(axis=1) + extra).astype(np.int32)
    cs = np.zeros(nch + 1, np.int64)
    cs[1:] = np.cumsum(clp.astype(np.int64) * C)
    col = np.zeros(int(cs[-1]), np.int32)
    for c in range(nch):
        own = np.arange(c * C, c * C + C)
        col[cs[c]:cs[c + 1]] = np.tile(np.where(own < n, own, 0), clp[c])
    src = np.asarray(csr.col, np.int32).copy()
    if diag_first:
        for r in range(n):
            seg = src[rp[r]:rp[r + 1]]
            d = np.flatnonzero(seg == r)
            if d.size:
                seg[[0, d[0]]] = seg[[d[0], 0]]
    rows = np.repeat(np.arange(n), rl)
    slot = np.arange(rp[-1]) - rp[rows]
    col[cs[rows // C] + rows % C + slot * C] = src
    val = np.arange(col.size, dtype=np.float64)
    return col, val, cs.astype(np.int32), rl, clp


# (matrix, dist) traversals of the whole range
TRAVERSE_CASES = [(m, d) for m in ["lap7_16", "st27_16", "plaw_3k", "band_5k", "aniso9_100x80", "islands_330"] for d in (1, 2, 3)]


def digest(csr) -> str:
    h = hashlib.sha256()
    for a in (np.asarray(csr.row_ptr, np.int32), np.asarray(csr.col, np.int32), np.asarray(csr.val, np.float64)):
        h.update(a.tobytes())
    return h.hexdigest()[:16]


def arr_digest(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, np.int32).tobytes()).hexdigest()[:16]


def f64_digest(a) -> str:
    """A checksum of the exact bits of a float64 array (outputs stored as
    digests where the arrays themselves would be large)."""
    return hashlib.sha256(np.ascontiguousarray(a, np.float64).tobytes()).hexdigest()[:16]


def key_color(m, d, t):
    return f"color__{m}__d{d}__t{t}"


def key_power(m, p, c):
    return f"power__{m}__p{p}__c{int(c)}"


def key_power_tri(m, tri, p, c):
    return f"powertri__{m}__{tri}__p{p}__c{int(c)}"


def triangle(csr, tri: str):
    """Lower ("L", col <= row) or upper ("U", col >= row) triangle of a CRS
    matrix, entries in their original order within each row."""
    rows = np.repeat(np.arange(csr.n), np.diff(csr.row_ptr))
    keep = csr.col <= rows if tri == "L" else csr.col >= rows
    rp = np.zeros(csr.n + 1, np.int32)
    np.cumsum(np.bincount(rows[keep], minlength=csr.n), out=rp[1:])
    return matgen.Csr(csr.n, rp, csr.col[keep].astype(np.int32), csr.val[keep].copy(), f"{csr.name}_{tri}")


def key_power_flat(m, p, c):
    return f"powerflat__{m}__p{p}__c{int(c)}"


def key_trav(m, d):
    return f"trav__{m}__d{d}"
