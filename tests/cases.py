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
}

# (matrix, dist, nthreads)
COLOR_CASES = [
    ("lap7_32", 2, 8), ("lap7_32", 2, 64), ("lap7_32", 2, 1024), ("lap7_32", 1, 8), ("lap7_32", 1, 256),
    ("lap7_16", 2, 16), ("st27_16", 2, 128), ("plaw_20k", 2, 64), ("plaw_3k", 1, 32), ("band_5k", 2, 32),
    ("aniso9_100x80", 1, 16), ("aniso5_120x90", 2, 48), ("islands_330", 1, 8), ("islands_330", 2, 16),
    ("tiny_1", 1, 4),
]

# coloring cases whose reference sweep outputs are stored
EXEC_CASES = {("lap7_16", 2, 16), ("aniso9_100x80", 1, 16), ("plaw_3k", 1, 32), ("islands_330", 2, 16)}

# (matrix, power, cacheBytes)
POWER_CASES = [
    ("st27_24", 8, 2e6), ("st27_40", 8, 8e6), ("lap7_32", 4, 1e6), ("aniso5_120x90", 4, 5e5),
    ("plaw_20k", 4, 1e6), ("band_5k", 6, 3e5), ("islands_330", 3, 2e4), ("tiny_1", 2, 1e4),
]

# (matrix, dist) traversals of the whole range
TRAVERSE_CASES = [(m, d) for m in ["lap7_16", "st27_16", "plaw_3k", "band_5k", "aniso9_100x80", "islands_330"] for d in (1, 2, 3)]


def digest(csr) -> str:
    h = hashlib.sha256()
    for a in (np.asarray(csr.row_ptr, np.int32), np.asarray(csr.col, np.int32), np.asarray(csr.val, np.float64)):
        h.update(a.tobytes())
    return h.hexdigest()[:16]


def arr_digest(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, np.int32).tobytes()).hexdigest()[:16]


def key_color(m, d, t):
    return f"color__{m}__d{d}__t{t}"


def key_power(m, p, c):
    return f"power__{m}__p{p}__c{int(c)}"


def key_trav(m, d):
    return f"trav__{m}__d{d}"
