"""Python mirror of RACE::Interface (include/interface.h of the reference)
over the engine's C ABI.

Names, argument meaning and return codes follow the reference:
``RACEColor`` returns a RACE_error code, ``registerFunction`` returns a
function id (or an error code), ``executeFunction`` returns a code. The
difference is the callback: instead of a host function pointer,
``registerFunction`` takes a built-in device kernel (``SPMV``, ``SYMMSPMV``,
``GS``, ``KACZ``, ``SPMTV``, ``MPK``) and its device operands. Device memory
is managed with torch tensors; the engine never allocates user vectors.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import time
from typing import Optional

import numpy as np
import torch

from . import _lib
from ._lib import check, lib, race_operands, race_params

ONE, TWO, POWER = 1, 2, 3
TWO_BLOCK, THREE_BLOCK = 0, 1
ROW, NNZ = 0, 1
FILL, SCATTER = 0, 1
SPMV, SPMTV, SYMMSPMV, GS, KACZ, MPK = 0, 1, 2, 3, 4, 5
SWEEP_AUTO, SWEEP_WAVE, SWEEP_LEAF, SWEEP_GATHER = 0, 1, 2, 3
# RACE_MPK_AUTO / WAVEFRONT / SWEEPS
MPK_SCHEDULES = ("auto", "wavefront", "sweeps")
VAL_F64, VAL_F32, VAL_BF16 = 0, 1, 2
_VAL_TYPE = {torch.float64: VAL_F64, torch.float32: VAL_F32, torch.bfloat16: VAL_BF16}


def _ptr(t: Optional[torch.Tensor]):
    return None if t is None else C.c_void_p(t.data_ptr())


def _host_i32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.int32)


def format_zone_tree(flat) -> str:
    """printZoneTree's text (interface.cpp:328-331, zone_tree.cpp:307-339)
    for a zone tree in race_get_zone_tree's flat form, one line per node;
    the reference's pinning and timing fields have no GPU meaning and are
    left out."""
    t = [int(v) for v in flat]
    lines, k = [], 1
    for i in range(t[0]):
        nth, ideal, sub, parent, eff, stage, reached = t[k:k + 7]
        k += 7
        nv = t[k]
        rng = t[k + 1:k + 1 + nv]
        k += 1 + nv
        nc = t[k]
        ch = t[k + 1:k + 1 + nc]
        k += 1 + nc
        lines.append(f"{i}. Range:[{''.join(f'{v}, ' for v in rng)}] Children:[{''.join(f'{c}, ' for c in ch)}], "
                     f"Parent: {parent}, nthreads: {nth}, idealNThreads:{ideal}, stage:{stage}, subBLocks:{sub}, "
                     f"effRow: {eff}, reachedLimit: {'true' if reached else 'false'}")
    return "\n".join(lines) + ("\n" if lines else "")


_SELL_VAL_TYPE = {np.dtype(np.float64): VAL_F64, np.dtype(np.float32): VAL_F32, np.dtype(np.uint16): VAL_BF16}


def _sell_args(col, chunkStart, rl, clp, val):
    """C arguments of the simdify calls: col and val are rewritten in place,
    so they must be writable C-contiguous host arrays (col int32; val
    float64, float32, uint16 holding BF16 bits, or None)."""
    for name, a in (("col", col), ("val", val)):
        if a is not None and not (isinstance(a, np.ndarray) and a.flags.c_contiguous and a.flags.writeable):
            raise TypeError(f"simdify: {name} must be a writable C-contiguous numpy array")
    if col.dtype != np.int32:
        raise TypeError("simdify: col must be int32")
    if val is not None and val.dtype not in _SELL_VAL_TYPE:
        raise TypeError("simdify: val must be float64, float32 or uint16 (BF16 bits)")
    keep = [_host_i32(chunkStart), _host_i32(rl), _host_i32(clp)]
    args = [col.ctypes.data] + [k.ctypes.data for k in keep] + \
           [None if val is None else val.ctypes.data, VAL_F64 if val is None else _SELL_VAL_TYPE[val.dtype]]
    return args, keep


@dataclasses.dataclass
class DeviceCsr:
    """A CRS matrix in device memory (torch tensors)."""
    n: int
    row_ptr: torch.Tensor
    col: torch.Tensor
    val: torch.Tensor

    @staticmethod
    def from_csr(csr, device="cuda", dtype=torch.float64) -> "DeviceCsr":
        return DeviceCsr(csr.n, torch.as_tensor(_host_i32(csr.row_ptr), device=device),
                         torch.as_tensor(_host_i32(csr.col), device=device),
                         torch.as_tensor(np.asarray(csr.val), device=device).to(dtype))


@dataclasses.dataclass
class Operands:
    """The ``args`` of registerFunction: a device matrix and vectors.
    For MPK, ``x`` holds (power+1)*n doubles, power-major."""
    mat: DeviceCsr
    x: torch.Tensor
    b: Optional[torch.Tensor] = None

    def to_c(self) -> race_operands:
        vt = _VAL_TYPE[self.mat.val.dtype]
        xt = VAL_F32 if self.x.dtype == torch.float32 else VAL_F64
        return race_operands(self.mat.n, self.mat.row_ptr.data_ptr(), self.mat.col.data_ptr(),
                             self.mat.val.data_ptr(), vt, self.x.data_ptr(),
                             None if self.b is None else self.b.data_ptr(), xt)


class Interface:
    """RACE::Interface(nrow, nthreads, dist, rowPtr, col, symm_hint, SMT,
    pinMethod, initPerm, initInvPerm, d2Type, lbTarget) (interface.h:124).
    SMT and pinMethod are accepted for signature parity; thread pinning has no
    meaning on the GPU. ``params`` overrides the reference's environment
    knobs (read from the environment otherwise): ``efficiency`` and
    ``lvl_threads`` (RACE_EFFICIENCY, RACE_THREADS), ``cache_violation_cutoff``
    (RACE_CACHE_VIOLATION_CUTOFF_DEFAULT), ``cache_violation_cutoffs`` (the
    list RACE_CACHE_VIOLATION_CUTOFF: entry k is the cut-off of MPK
    recursion stage k) and ``max_recursion_stages`` (RACE_MAX_RECURSION_STAGES)."""

    def __init__(self, nrow: int, nthreads: int, dist: int, rowPtr, col, symm_hint: bool = False, SMT: int = 1,
                 pinMethod: int = SCATTER, initPerm=None, initInvPerm=None, d2Type: int = TWO_BLOCK,
                 lbTarget: int = NNZ, params: Optional[dict] = None, stream: Optional[torch.cuda.Stream] = None):
        self.nrow = int(nrow)
        self.dist = dist
        self._funcs = {}
        self._tuned = {}
        rp, cl = _host_i32(rowPtr), _host_i32(col)
        ip = _host_i32(initPerm) if initPerm is not None else None
        iip = _host_i32(initInvPerm) if initInvPerm is not None else None
        cparams = None
        if params is not None:
            cparams = race_params()
            check(lib().race_params_from_env(C.byref(cparams)))
            if "efficiency" in params:
                eff = list(params["efficiency"])
                cparams.n_eff = len(eff)
                for i, v in enumerate(eff):
                    cparams.eff[i] = v
            if "lvl_threads" in params:
                lt = list(params["lvl_threads"])
                cparams.n_lvl_threads = len(lt)
                for i, v in enumerate(lt):
                    cparams.lvl_threads[i] = v
            if "cache_violation_cutoff" in params:
                cparams.cache_violation_cutoff = int(params["cache_violation_cutoff"])
            if "max_recursion_stages" in params:
                cparams.max_recursion_stages = int(params["max_recursion_stages"])
            if "cache_violation_cutoffs" in params:
                cuts = [int(v) for v in params["cache_violation_cutoffs"]][:16]
                cparams.n_cutoffs = len(cuts)
                for i, v in enumerate(cuts):
                    cparams.cutoffs[i] = v
        h = C.c_void_p()
        check(lib().race_create(C.byref(h), self.nrow, int(nthreads), int(dist), rp.ctypes.data, cl.ctypes.data,
                                int(bool(symm_hint)), None if ip is None else ip.ctypes.data,
                                None if iip is None else iip.ctypes.data, int(d2Type), int(lbTarget),
                                None if cparams is None else C.byref(cparams)))
        self._h = h
        self.stream = stream
        if stream is not None:
            check(lib().race_set_stream(self._h, C.c_void_p(stream.cuda_stream)), self._h)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().race_destroy(h)
            self._h = None

    close = __del__

    def _check(self, rc):
        check(rc, self._h)

    # ---- pre-processing (interface.h:127-135)
    def RACEColor(self, highestPower: Optional[int] = None, cacheSize: Optional[float] = None,
                  safetyFactor: float = 2.0, mtxType: str = "N", highestSubPower: int = 1) -> int:
        """RACEColor() for coloring, RACEColor(highestPower, cacheSize [bytes], ...)
        for the matrix-power partition. Returns a RACE_error code."""
        if highestPower is None:
            return lib().race_color(self._h)
        return lib().race_power_prepare(self._h, int(highestPower), float(cacheSize), float(safetyFactor),
                                        mtxType.encode(), int(highestSubPower))

    def RACEing(self, *args, **kwargs) -> int:
        """RACEColor under the name the RACE papers use for the coloring /
        partitioning step (same arguments, same result)."""
        return self.RACEColor(*args, **kwargs)

    def getPerm(self) -> np.ndarray:
        p = np.zeros(self.nrow, np.int32)
        self._check(lib().race_get_perm(self._h, p.ctypes.data, None))
        return p

    def getInvPerm(self) -> np.ndarray:
        p = np.zeros(self.nrow, np.int32)
        self._check(lib().race_get_perm(self._h, None, p.ctypes.data))
        return p

    def getNumThreads(self) -> int:
        v = C.c_int()
        self._check(lib().race_get_num_threads(self._h, C.byref(v)))
        return v.value

    def getEfficiency(self) -> float:
        v = C.c_double()
        self._check(lib().race_get_efficiency(self._h, C.byref(v)))
        return v.value

    def getMaxStageDepth(self) -> int:
        v = C.c_int()
        self._check(lib().race_get_max_stage_depth(self._h, C.byref(v)))
        return v.value

    def getHighestPower(self) -> int:
        v = C.c_int()
        self._check(lib().race_get_highest_power(self._h, C.byref(v)))
        return v.value

    # ---- SELL-C-sigma preparation (interface.h:179-185)
    def simdify(self, simdWidth: int, C: int, nrows: int, col: np.ndarray, chunkStart, rl, clp,
                val: Optional[np.ndarray], diagFirst: bool = False) -> bool:
        """Interface::simdify: pads each row of each forward leaf, then orders
        every SIMD group's entries so that its lanes hold different columns in
        each slot. Host arrays in SELL-C layout, col/val rewritten in place.
        False when a row cannot be placed (as the reference; the arrays are
        then partly rearranged)."""
        args, _keep = _sell_args(col, chunkStart, rl, clp, val)
        rc = lib().race_simdify(self._h, int(simdWidth), int(C), int(nrows), *args, int(bool(diagFirst)), None)
        if rc == _lib.RACE_ERR_INCOMPATIBILITY:
            return False
        self._check(rc)
        return True

    def simdifyD1(self, simdWidth: int, C: int, nrows: int, col: np.ndarray, chunkStart, rl, clp,
                  val: Optional[np.ndarray], dist2Compatible: bool = False) -> bool:
        """Interface::simdifyD1: moves each row's entries on the earlier rows
        of its SIMD group to the row's last slots."""
        args, _keep = _sell_args(col, chunkStart, rl, clp, val)
        check(lib().race_simdify_d1(int(simdWidth), int(C), int(nrows), *args, int(bool(dist2Compatible))))
        return True

    def printZoneTree(self):
        print(format_zone_tree(self.getZoneTreeFlat()), end="")

    def getNumaSplitting(self) -> np.ndarray:
        """Row split of the level groups over shared-cache domains; the
        reference always uses one domain (interface.cpp:207, 1042-1053)."""
        return np.array([0, self.nrow], np.int32)

    def getZoneTreeFlat(self) -> np.ndarray:
        n = C.c_int()
        self._check(lib().race_get_zone_tree(self._h, None, 0, C.byref(n)))
        buf = np.zeros(n.value, np.int32)
        self._check(lib().race_get_zone_tree(self._h, buf.ctypes.data, n.value, C.byref(n)))
        return buf

    def getPhases(self, rev: bool = False):
        npz, nl = C.c_int(), C.c_int()
        self._check(lib().race_get_phases(self._h, int(rev), None, None, None, 0, C.byref(npz), C.byref(nl)))
        cap = max(nl.value, npz.value + 1)
        pp = np.zeros(cap, np.int32); lo = np.zeros(cap, np.int32); hi = np.zeros(cap, np.int32)
        self._check(lib().race_get_phases(self._h, int(rev), pp.ctypes.data, lo.ctypes.data, hi.ctypes.data, cap,
                                          C.byref(npz), C.byref(nl)))
        return pp[: npz.value + 1], lo[: nl.value], hi[: nl.value]

    def getPowerTree(self) -> np.ndarray:
        """The MPK partition's leaf tree, flat (race_get_power_tree)."""
        n = C.c_int()
        self._check(lib().race_get_power_tree(self._h, None, 0, C.byref(n)))
        buf = np.zeros(n.value, np.int32)
        self._check(lib().race_get_power_tree(self._h, buf.ctypes.data, n.value, C.byref(n)))
        return buf

    def getPowerGroups(self) -> np.ndarray:
        n = C.c_int()
        self._check(lib().race_get_power_groups(self._h, None, 0, C.byref(n)))
        buf = np.zeros(n.value, np.int32)
        self._check(lib().race_get_power_groups(self._h, buf.ctypes.data, n.value, C.byref(n)))
        return buf

    # ---- execution (interface.h:149-174)
    def registerFunction(self, kernel: int, args: Operands, power: int = 1) -> int:
        fid = C.c_int(-1)
        if kernel == MPK and (args.x.dtype != torch.float64 or args.x.numel() < (power + 1) * args.mat.n):
            return _lib.RACE_ERR_INVALID_ARG  # x must hold (power+1)*n doubles
        ops = args.to_c()
        rc = lib().race_register_function(self._h, int(kernel), C.byref(ops), int(power), C.byref(fid))
        if rc != _lib.RACE_SUCCESS:
            return rc  # the reference returns the error code in place of an id (interface.cpp:429)
        self._funcs[fid.value] = args  # keep operand tensors alive
        return fid.value

    def registerMpkBlock(self, args: Operands, power: int, nrhs: int) -> int:
        """Matrix power over nrhs right-hand sides (race_register_mpk_block):
        ``args.x`` holds (power+1)*n*nrhs values, power-major, then row, then
        right-hand side; FP64 values with FP64 x or FP32/BF16 values with FP32
        x. Returns a function id, or an error code like registerFunction."""
        if args.x.numel() < (power + 1) * args.mat.n * nrhs or not args.x.is_contiguous():
            return _lib.RACE_ERR_INVALID_ARG
        fid = C.c_int(-1)
        ops = args.to_c()
        rc = lib().race_register_mpk_block(self._h, C.byref(ops), int(power), int(nrhs), C.byref(fid))
        if rc != _lib.RACE_SUCCESS:
            return rc
        self._funcs[fid.value] = args
        return fid.value

    def executeFunction(self, funcId: int, rev: bool = False) -> int:
        return lib().race_execute_function(self._h, int(funcId), int(bool(rev)))

    def executeFunctionAsync(self, funcId: int, rev: bool = False) -> int:
        """Enqueue without waiting; getStatus() reports device-side waits."""
        return lib().race_execute_function_async(self._h, int(funcId), int(bool(rev)))

    def getStatus(self) -> int:
        return lib().race_get_status(self._h)

    def setSweepMode(self, mode: int):
        """SWEEP_AUTO, SWEEP_WAVE (bit-exact wave plans), SWEEP_LEAF, or
        SWEEP_GATHER (SpMV, SpMTV, SymmSpMV in one launch, bit-exact)."""
        self._check(lib().race_set_sweep_mode(self._h, int(mode)))

    def getMpkLayout(self, funcId: int) -> dict:
        """Device layout and schedule of a registered MPK function
        (race_get_mpk_layout)."""
        v = [C.c_int() for _ in range(3)]
        w = [C.c_longlong() for _ in range(2)]
        sch = C.c_int()
        self._check(lib().race_get_mpk_layout(self._h, int(funcId), *[C.byref(a) for a in v + w], C.byref(sch)))
        return dict(chunks=v[0].value, col_bits=v[1].value, wide_chunks=v[2].value, sell_slots=w[0].value,
                    matrix_bytes=w[1].value, schedule=MPK_SCHEDULES[sch.value])

    def setMpkSchedule(self, funcId: int, schedule: str):
        """race_set_mpk_schedule: "auto", "wavefront" or "sweeps"."""
        self._check(lib().race_set_mpk_schedule(self._h, int(funcId), MPK_SCHEDULES.index(schedule)))

    def getSweepInfo(self, funcId: int, rev: bool = False) -> dict:
        v = [C.c_int() for _ in range(5)]
        self._check(lib().race_get_sweep_info(self._h, int(funcId), int(bool(rev)), *[C.byref(a) for a in v]))
        return dict(waves=v[0].value, max_wave_rows=v[1].value, phases=v[2].value, max_leaf_rows=v[3].value,
                    wave_mode=v[4].value == 1, mode={0: "leaf", 1: "wave", 2: "gather"}[v[4].value])

    def setStream(self, stream: torch.cuda.Stream):
        self.stream = stream
        self._check(lib().race_set_stream(self._h, C.c_void_p(stream.cuda_stream)))

    def setPower(self, funcId: int, pow: int):
        self._check(lib().race_set_power(self._h, int(funcId), int(pow)))

    def getPower(self, funcId: int) -> int:
        v = C.c_int()
        self._check(lib().race_get_power(self._h, int(funcId), C.byref(v)))
        return v.value

    def setSubPower(self, funcId: int, subPow: int):
        """Interface::setSubPower: built-in kernels have no sub-steps, so
        only 1 is accepted (RACE_ERR_INCOMPATIBILITY otherwise)."""
        self._check(lib().race_set_sub_power(self._h, int(funcId), int(subPow)))

    def getSubPower(self, funcId: int) -> int:
        v = C.c_int()
        self._check(lib().race_get_sub_power(self._h, int(funcId), C.byref(v)))
        return v.value

    def tuneFunction(self, funcId: int, rev: bool = False, highestPower: Optional[int] = None) -> int:
        """Interface::tuneFunction (interface.cpp:605-647): time powers
        1..highestPower for >= 0.2 s each, keep the fastest time per power."""
        if funcId in self._tuned:
            self.setPower(funcId, self._tuned[funcId])
            return self._tuned[funcId]
        hp = highestPower or self.getPower(funcId)
        times = []
        for p in range(1, hp + 1):
            self.setPower(funcId, p)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            it = 0
            while True:
                self._check(self.executeFunction(funcId, rev))
                torch.cuda.synchronize()
                it += 1
                el = time.perf_counter() - t0
                if el >= 0.2:
                    break
            times.append(el / (it * p))
        best = int(np.argmin(times)) + 1
        self._tuned[funcId] = best
        self.setPower(funcId, best)
        return best

    def symmGsIr(self, innerFuncId: int, mat64: DeviceCsr, b: torch.Tensor, x: torch.Tensor, tol: float = 1e-10,
                 maxIter: int = 100, sweeps: int = 1):
        """FP64 iterative refinement around symmetric GS sweeps of a
        registered (reduced-precision) RACE_K_GS function; returns
        (refinements, final relative residual)."""
        it, rel = C.c_int(), C.c_double()
        self._check(lib().race_symmgs_ir(self._h, int(innerFuncId), mat64.n, _ptr(mat64.row_ptr), _ptr(mat64.col),
                                         _ptr(mat64.val), _ptr(b), _ptr(x), float(tol), int(maxIter), int(sweeps),
                                         C.byref(it), C.byref(rel)))
        return it.value, rel.value

    # ---- convenience
    def spmvPowerLayout(self, funcId: int, k: int):
        """x_{k+1} = A x_k for a registered MPK function, as a plain SpMV on
        the same internal layout (no level blocking)."""
        self._check(lib().race_spmv_power_layout(self._h, int(funcId), int(k)))

    def spmv_plain(self, mat: DeviceCsr, x: torch.Tensor, b: torch.Tensor):
        self._check(lib().race_spmv_plain(self._h, mat.n, _ptr(mat.row_ptr), _ptr(mat.col), _ptr(mat.val), _ptr(x),
                                          _ptr(b)))


def _stream_ptr(stream: Optional[torch.cuda.Stream]):
    s = stream if stream is not None else torch.cuda.current_stream()
    return C.c_void_p(s.cuda_stream)


class Batch:
    """Block-MPK functions of several Interfaces run by one persistent launch
    (race_batch_*); ``graphLaunch`` replays a CUDA graph of that launch.
    The Interfaces and operand tensors must outlive the batch; prepare() again
    after changing a member (setPower)."""

    def __init__(self):
        h = C.c_void_p()
        check(lib().race_batch_create(C.byref(h)))
        self._h = h
        self._members = []

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().race_batch_destroy(h)
            self._h = None

    close = __del__

    def _check(self, rc):
        if rc != _lib.RACE_SUCCESS:
            m = lib().race_batch_last_error(self._h)
            raise _lib.RaceError(rc, m.decode() if m else "")

    def add(self, iface: Interface, funcId: int):
        self._check(lib().race_batch_add(self._h, iface._h, int(funcId)))
        self._members.append(iface)

    def prepare(self, stream: Optional[torch.cuda.Stream] = None):
        self._check(lib().race_batch_prepare(self._h, _stream_ptr(stream)))

    def execute(self, stream: Optional[torch.cuda.Stream] = None):
        self._check(lib().race_batch_execute(self._h, _stream_ptr(stream)))

    def graphLaunch(self, stream: Optional[torch.cuda.Stream] = None):
        self._check(lib().race_batch_graph_launch(self._h, _stream_ptr(stream)))

    def getStatus(self, stream: Optional[torch.cuda.Stream] = None) -> int:
        return lib().race_batch_get_status(self._h, _stream_ptr(stream))

    def info(self) -> dict:
        v = [C.c_int() for _ in range(3)]
        self._check(lib().race_batch_info(self._h, *[C.byref(a) for a in v]))
        return dict(members=v[0].value, chunks=v[1].value, items=v[2].value)
