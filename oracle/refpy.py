"""ctypes view of oracle/_ref/librace_ref.so (the reference compiled in place).

TEST INFRASTRUCTURE ONLY: used by tests and by tests/golden/make_golden.py to
produce golden data. The library is built by oracle/build_ref.sh and exists
only where the reference sources are present (x86 build host).
"""
from __future__ import annotations

import ctypes as C
import os
import pathlib

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
LIB_PATH = HERE / "_ref" / "librace_ref.so"

_lib = None

IP = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
DP = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")


def available() -> bool:
    return LIB_PATH.exists()


def lib():
    global _lib
    if _lib is None:
        os.environ.setdefault("ORACLE_QUIET", "1")
        L = C.CDLL(str(LIB_PATH))
        L.refc_color.restype = C.c_void_p
        L.refc_color.argtypes = [C.c_int, IP, IP, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]
        L.refc_color_init.restype = C.c_void_p
        L.refc_color_init.argtypes = [C.c_int, IP, IP, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, IP, IP]
        L.refc_color_free.argtypes = [C.c_void_p]
        L.refc_color_perm.argtypes = [C.c_void_p, IP, IP]
        L.refc_color_threads.argtypes = [C.c_void_p]
        L.refc_color_efficiency.argtypes = [C.c_void_p]
        L.refc_color_efficiency.restype = C.c_double
        L.refc_color_max_stage.argtypes = [C.c_void_p]
        L.refc_color_serial_part.argtypes = [C.c_void_p, IP]
        L.refc_color_tree.argtypes = [C.c_void_p, C.c_void_p, C.c_int]
        L.refc_color_exec.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, IP, IP, DP, DP, DP]
        L.refc_traverse.argtypes = [C.c_int, IP, IP, C.c_int, C.c_int, C.c_int, C.c_int, IP, IP, IP, IP, C.c_int]
        L.refc_lb.argtypes = [IP, IP, C.c_int, C.c_int, C.c_double, C.c_int, C.c_int, C.c_int, C.c_int,
                              C.c_void_p, C.c_int]
        L.refc_power.restype = C.c_void_p
        L.refc_power.argtypes = [C.c_int, IP, IP, C.c_int, C.c_double, C.c_double, C.c_char_p, C.c_int]
        L.refc_power_free.argtypes = [C.c_void_p]
        L.refc_power_perm.argtypes = [C.c_void_p, IP, IP]
        L.refc_power_tree.argtypes = [C.c_void_p, C.c_void_p, C.c_int]
        L.refc_power_exec.argtypes = [C.c_void_p, C.c_int, C.c_int, IP, IP, DP, DP]
        L.refc_power_coverage.argtypes = [C.c_void_p, C.c_int, IP]
        L.refc_iface.restype = C.c_void_p
        L.refc_iface.argtypes = [C.c_int, IP, IP, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]
        L.refc_iface_free.argtypes = [C.c_void_p]
        L.refc_iface_perm.argtypes = [C.c_void_p, IP, IP]
        L.refc_simdify.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, IP, IP, IP, IP, DP, C.c_int]
        L.refc_simdify_d1.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, IP, IP, IP, IP, DP, C.c_int]
        _lib = L
    return _lib


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _flat(fn, h):
    n = fn(h, None, 0)
    buf = np.zeros(n, dtype=np.int32)
    fn(h, buf.ctypes.data, n)
    return buf


def parse_zone_tree(buf):
    """Decode refc_color_tree's flat buffer into a list of dicts."""
    nodes, k = [], 1
    for _ in range(int(buf[0])):
        d = dict(nthreads=int(buf[k]), ideal=int(buf[k + 1]), subblocks=int(buf[k + 2]), parent=int(buf[k + 3]),
                 effrow=int(buf[k + 4]), stage=int(buf[k + 5]), reached=int(buf[k + 6]))
        k += 7
        nv = int(buf[k]); d["value"] = [int(v) for v in buf[k + 1:k + 1 + nv]]; k += 1 + nv
        nc = int(buf[k]); d["children"] = [int(v) for v in buf[k + 1:k + 1 + nc]]; k += 1 + nc
        nodes.append(d)
    return nodes


def parse_power_tree(buf):
    leaves, k = [], 1
    names = ["lp", "hid", "unlockRow", "dangerRow", "unlockCtr", "nodePtr", "unitPtr", "unitNodePtr", "children"]
    for _ in range(int(buf[0])):
        d = dict(lo=int(buf[k]), hi=int(buf[k + 1]), stage=int(buf[k + 2]), parent=int(buf[k + 3]),
                 nodeId=int(buf[k + 4]))
        k += 5
        for nm in names:
            nv = int(buf[k]); d[nm] = [int(v) for v in buf[k + 1:k + 1 + nv]]; k += 1 + nv
        leaves.append(d)
    return leaves


class RefInterface:
    """A colored RACE::Interface, for simdify/simdifyD1 (interface.cpp:824-842)."""

    def __init__(self, csr, dist: int, nthreads: int, symm_hint: bool = True, d2type: int = 0, lbtarget: int = 1):
        self.n = csr.n
        self.h = lib().refc_iface(csr.n, _i32(csr.row_ptr), _i32(csr.col), dist, nthreads, int(symm_hint), d2type,
                                  lbtarget)
        if not self.h:
            raise RuntimeError("RACEColor failed")

    def close(self):
        if self.h:
            lib().refc_iface_free(self.h)
            self.h = None

    __del__ = close

    def perm(self):
        p = np.zeros(self.n, np.int32); ip = np.zeros(self.n, np.int32)
        lib().refc_iface_perm(self.h, p, ip)
        return p, ip

    def simdify(self, simd_width, C, sell, diag_first):
        """Runs Interface::simdify on sell = (col, val, chunkStart, rl, clp) in place; returns its bool."""
        col, val, cs, rl, clp = sell
        return bool(lib().refc_simdify(self.h, simd_width, C, self.n, col, cs, rl, clp, val, int(diag_first)))

    def simdify_d1(self, simd_width, C, sell, dist2_compatible):
        col, val, cs, rl, clp = sell
        return bool(lib().refc_simdify_d1(self.h, simd_width, C, self.n, col, cs, rl, clp, val,
                                          int(dist2_compatible)))


class RefColor:
    """Reference coloring of one matrix (RACE::Interface with dist ONE/TWO)."""

    def __init__(self, csr, dist: int, nthreads: int, symm_hint: bool = True, d2type: int = 0, lbtarget: int = 1,
                 init_perm=None):
        self.n = csr.n
        self._rp, self._col = _i32(csr.row_ptr), _i32(csr.col)
        if init_perm is None:
            self.h = lib().refc_color(csr.n, self._rp, self._col, dist, nthreads, int(symm_hint), d2type, lbtarget)
        else:
            self._ip = _i32(init_perm)
            self._iip = np.empty_like(self._ip)
            self._iip[self._ip] = np.arange(csr.n, dtype=np.int32)
            self.h = lib().refc_color_init(csr.n, self._rp, self._col, dist, nthreads, int(symm_hint), d2type,
                                           lbtarget, self._ip, self._iip)

    def close(self):
        if self.h:
            lib().refc_color_free(self.h)
            self.h = None

    __del__ = close

    def perm(self):
        p = np.zeros(self.n, np.int32); ip = np.zeros(self.n, np.int32)
        lib().refc_color_perm(self.h, p, ip)
        return p, ip

    def threads(self):
        return lib().refc_color_threads(self.h)

    def efficiency(self):
        return lib().refc_color_efficiency(self.h)

    def max_stage(self):
        return lib().refc_color_max_stage(self.h)

    def serial_part(self):
        o = np.zeros(2, np.int32)
        lib().refc_color_serial_part(self.h, o)
        return o

    def tree(self):
        return parse_zone_tree(_flat(lib().refc_color_tree, self.h))

    def tree_flat(self):
        return _flat(lib().refc_color_tree, self.h)

    def execute(self, kernel: int, rev: bool, pcsr, x, b):
        lib().refc_color_exec(self.h, kernel, int(rev), pcsr.n, _i32(pcsr.row_ptr), _i32(pcsr.col),
                              np.ascontiguousarray(pcsr.val), x, b)


def traverse(csr, dist: int, lo: int, hi: int, symm_hint: bool = True, level_cap: int | None = None):
    n = csr.n
    cap = level_cap or n + 2
    p = np.zeros(n, np.int32); ip = np.zeros(n, np.int32)
    lr = np.zeros(cap, np.int32); ln = np.zeros(cap, np.int32)
    L = lib().refc_traverse(n, _i32(csr.row_ptr), _i32(csr.col), dist, lo, hi, int(symm_hint), p, ip, lr, ln, cap)
    return p, ip, lr[:L].copy(), ln[:L].copy()


def lb(level_row, level_nnz, nthreads: int, eff: float, dist: int, d2type: int = 0, lbtarget: int = 1, base: int = 0):
    L = lib()
    lr, ln = _i32(level_row), _i32(level_nnz)
    n = L.refc_lb(lr, ln, lr.size, nthreads, eff, dist, d2type, lbtarget, base, None, 0)
    buf = np.zeros(n, np.int32)
    L.refc_lb(lr, ln, lr.size, nthreads, eff, dist, d2type, lbtarget, base, buf.ctypes.data, n)
    k = 0
    ns = int(buf[k]); scale = buf[k + 1:k + 1 + ns].tolist(); k += 1 + ns
    tb = int(buf[k]); zone = buf[k + 1:k + 2 + tb].tolist(); k += 2 + tb
    tsb = int(buf[k]); sub = buf[k + 1:k + 2 + tsb].tolist(); k += 2 + tsb
    nb = buf[k:k + tb].tolist()
    return dict(scale=scale, zonePtr=zone, subZonePtr=sub, numBlocks=nb)


class RefPower:
    """Reference MPK pre-processing (RACE::Interface with dist POWER)."""

    def __init__(self, csr, power: int, cache_bytes: float, safety: float = 2.0, mtx_type: str = "N",
                 symm_hint: bool = True):
        self.n = csr.n
        self.power = power
        self._rp, self._col = _i32(csr.row_ptr), _i32(csr.col)
        self.h = lib().refc_power(csr.n, self._rp, self._col, power, float(cache_bytes), float(safety),
                                  mtx_type.encode(), int(symm_hint))

    def close(self):
        if self.h:
            lib().refc_power_free(self.h)
            self.h = None

    __del__ = close

    def perm(self):
        p = np.zeros(self.n, np.int32); ip = np.zeros(self.n, np.int32)
        lib().refc_power_perm(self.h, p, ip)
        return p, ip

    def tree(self):
        return parse_power_tree(_flat(lib().refc_power_tree, self.h))

    def execute(self, pcsr, x0, power: int | None = None):
        p = power or self.power
        x = np.zeros((p + 1) * self.n)
        x[: self.n] = x0
        lib().refc_power_exec(self.h, p, self.n, _i32(pcsr.row_ptr), _i32(pcsr.col), np.ascontiguousarray(pcsr.val), x)
        return x.reshape(p + 1, self.n)

    def coverage(self, power: int | None = None):
        p = power or self.power
        cov = np.zeros(p * self.n, np.int32)
        lib().refc_power_coverage(self.h, p, cov)
        return cov.reshape(p, self.n)
