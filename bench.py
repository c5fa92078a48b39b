"""Benchmark of the level-blocked matrix-power kernel (RACE MPK) on GB300.

Workload (one GPU): y_k = A^k x for k = 1..8 on the 27-point stencil of a
128^3 grid (n = 2,097,152, nnz = 55,742,968; the HPCG-128 shape the reference
publishes MPK numbers for), FP64 values, permuted with RACE's MPK ordering
and level groups (cacheSize 300 MB, safety 2: the fastest of 50-500 MB on
GB300; the host-core reference runs equally fast at 100 and 300 MB).
Synthetic data: off-diagonals
U[-1,0) mirrored, diagonal = sum|off| + 1, x ~ U[-1,1] (seeded).

Metric: effective GB/s = p * (nnz*12 + 4(n+1) + 8n + 8n) bytes per call
divided by the time (the FP64 CRS SpMV traffic model the reference's
published GFlop/s convert to). The matrix (669 MB) is larger than the L2,
so no flush is needed between iterations.

--impl reference times the reference algorithm on the host cores instead:
the C restatement of RACE's level-group wavefront executor on OpenMP
threads (oracle/race_oracle.c), since the reference library itself cannot be
built on the GPU host.

N > 1 GPUs (torchrun): every rank runs an independent replica of the same
workload (the reference's MPK has no multi-GPU path); value = total effective
bytes over all ranks / max rank time.
"""
from __future__ import annotations

import argparse
import json
import os
import pathlib
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "MPK/SymmGS effective GB/s & % HBM peak, mixed vs FP64 at 1e-10 rel err"
GRID = 128
POWER = 8
CACHE_BYTES = 300e6
# Published RACE MPK p=8 on HPCG-128 (the same shape), best CPU result in the
# reference's perf data: AMD Rome 49.85 GF/s = 317.9 GB/s effective
# (examples/matrixPower_perf_test/21_Jan_2021_rome1_nps1/mtxPower.csv:2131).
PUBLISHED_GBS = 317.9
# GB300's nominal FP64 (non-tensor) rate, 1/64 of FP32
FP64_PEAK_TFLOPS = 1.25


def spmv_bytes(n: int, nnz: int, val_bytes: int = 8) -> int:
    return nnz * (val_bytes + 4) + 4 * (n + 1) + 8 * n + 8 * n


def max_over_ranks(ms: float, world: int, device) -> float:
    """The slowest rank's time: every rank runs a replica, so the job ends
    when the last one does (an all-reduce MAX over the process group)."""
    if world <= 1:
        return ms
    import torch
    import torch.distributed as dist
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_gbs(bytes_per_rank: float, ms_max: float, world: int) -> float:
    """Whole-job throughput: the bytes of all ranks' replicas over the
    slowest rank's time."""
    return bytes_per_rank * world / (ms_max * 1e-3) / 1e9


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock/throttle samples while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        rows = []
        try:
            for line in open(self.path):
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        except OSError:
            pass
        finally:
            try:
                os.unlink(self.path)
            except OSError:
                pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": reasons, "samples": len(rows)}


def build_workload():
    from race_gb300 import matgen
    A = matgen.stencil3d_27pt(GRID)
    return A


# cache budgets the CPU legs choose from: RACE's cacheSize is the host's own
# (the reference's examples take it per machine), so the CPU runs the
# fastest of these on the host it runs on
CPU_CACHE_CANDIDATES = (25e6, 50e6, 100e6, 300e6)


def cpu_partition(A, x0, threads):
    """The RACE partition of the workload for the CPU legs: BFS levels and
    permutation (shared by every budget), then the level groups of each
    candidate budget, each timed on a median of three full MPK calls after a
    warm-up call; returns (P, groups, budget, times) for the fastest."""
    from oracle import oracle as orc
    perm, inv, lr, ln, _ = orc.traverse(A, 3, 0, A.n)
    P = A.permuted(perm, inv)
    lp = np.concatenate([[0], np.cumsum(lr)]).astype(np.int32)
    best, times = None, {}
    for c in CPU_CACHE_CANDIDATES:
        groups = orc.mpk_groups(POWER, A.n, A.nnz, c, 2.0, 50, lp, ln)
        if groups is None:
            continue
        orc.mpk_wavefront(P, x0, POWER, *groups, threads)
        ts = []
        for _ in range(3):
            t0 = time.perf_counter()
            orc.mpk_wavefront(P, x0, POWER, *groups, threads)
            ts.append(time.perf_counter() - t0)
        times[c] = statistics.median(ts)
        if best is None or times[c] < times[best[1]]:
            best = (groups, c)
    if best is None:
        raise RuntimeError("no cache budget gives a partition without hopeless regions for the CPU wavefront")
    return P, best[0], best[1], times, perm


def run_reference(args, rank, world):
    """RACE's level-group wavefront on the host cores (oracle port)."""
    if rank != 0:
        return
    from oracle import oracle as orc
    from race_gb300 import matgen
    A = build_workload()
    threads = os.cpu_count() or 1
    x0 = matgen.uniform_vector(A.n, 0)
    P, (gp, ur, dr), budget, _, _ = cpu_partition(A, x0, threads)
    for _ in range(args.warmup):
        orc.mpk_wavefront(P, x0, POWER, gp, ur, dr, threads)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        orc.mpk_wavefront(P, x0, POWER, gp, ur, dr, threads)
        times.append(time.perf_counter() - t0)
    t = statistics.median(times)
    eff = POWER * spmv_bytes(A.n, A.nnz)
    gbs = eff / t / 1e9
    line = {
        "impl": "reference", "metric": METRIC, "value": gbs, "unit": "GB/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": gbs / PUBLISHED_GBS, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"MPK p={POWER}, 27-point stencil {GRID}^3, FP64, RACE level groups "
                               f"(cacheSize {budget / 1e6:.0f} MB, the fastest on this host of "
                               f"{'/'.join(f'{c / 1e6:.0f}' for c in CPU_CACHE_CANDIDATES)} MB)",
                   "parallelism": "host cores"},
        "cpu_baseline": {"value": gbs, "unit": "GB/s", "cores": threads, "kind": "port",
                         "sample": f"{args.steps} full MPK calls (median), RACE wavefront restated in C, "
                                   f"OpenMP {threads} threads, cacheSize {budget / 1e6:.0f} MB"},
        "e2e": {"value": gbs, "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_profile_case(args):
    """Short, fixed sequences of launches for ncu.
    mpk: --steps MPK calls of the wavefront kernel, then --steps rounds of
    the p plain SpMVs on the same SELL-32 layout (27-point stencil,
    --grid^3).
    batch: the batched block MPK of --batch-count matrices, --steps graph
    replays, then --steps rounds of the plain per-matrix launches.
    symmgs: --steps forward+backward GS sweeps (FP32 values) on the
    --symmgs-rows power-law system of the SymmGS measurement."""
    import torch
    from race_gb300 import interface as ri
    from race_gb300 import matgen
    if args.profile == "batch":
        p, nrhs = 4, 16
        dt = torch.float32 if args.values == "f32" else torch.float64
        batch, fns = ri.Batch(), []
        for i, A in enumerate(matgen.aniso2d_batch(args.batch_count, seed=0)):
            rc = ri.Interface(A.n, 1, ri.POWER, A.row_ptr, A.col, symm_hint=True)
            assert rc.RACEColor(p, args.batch_cache_mb * 1e6) == 0
            P = A.permuted(rc.getPerm(), rc.getInvPerm())
            dm = ri.DeviceCsr.from_csr(P, "cuda", dt)
            x = torch.zeros((p + 1) * P.n * nrhs, dtype=dt, device="cuda")
            x[: P.n * nrhs] = torch.tensor(matgen.uniform_block(P.n, nrhs, seed=100 + i).reshape(-1), dtype=dt,
                                           device="cuda")
            fid = rc.registerMpkBlock(ri.Operands(dm, x), p, nrhs)
            assert rc.executeFunction(fid) == 0
            batch.add(rc, fid)
            fns.append((rc, fid, dm, x))
        for _ in range(args.steps):
            batch.graphLaunch()
        assert batch.getStatus() == 0
        for _ in range(args.steps):
            for rc, fid, _, _ in fns:
                for k in range(p):
                    rc.spmvPowerLayout(fid, k)
        torch.cuda.synchronize()
        print(f"profile case done: batch of {args.batch_count}, values {args.values}")
        return
    if args.profile == "symmgs":
        A = matgen.powerlaw_chung_lu(args.symmgs_rows, seed=0)
        rc = ri.Interface(A.n, 4096, ri.TWO, A.row_ptr, A.col, symm_hint=True)
        assert rc.RACEColor() == 0
        P = A.permuted(rc.getPerm(), rc.getInvPerm())
        m32 = ri.DeviceCsr.from_csr(P, "cuda", torch.float32)
        d = torch.zeros(A.n, dtype=torch.float32, device="cuda")
        r = torch.ones(A.n, dtype=torch.float32, device="cuda")
        fid = rc.registerFunction(ri.GS, ri.Operands(m32, d, r))
        for _ in range(args.steps):
            assert rc.executeFunction(fid) == 0
            assert rc.executeFunction(fid, True) == 0
        print(f"profile case done: symmetric GS on power-law n={A.n}")
        return
    dt = torch.float32 if args.values == "f32" else torch.float64
    A = matgen.stencil3d_27pt(args.grid)
    rc = ri.Interface(A.n, 1, ri.POWER, A.row_ptr, A.col, symm_hint=True)
    assert rc.RACEColor(POWER, CACHE_BYTES) == 0
    P = A.permuted(rc.getPerm(), rc.getInvPerm())
    dm = ri.DeviceCsr.from_csr(P, "cuda", dt)
    x = torch.zeros((POWER + 1) * A.n, dtype=torch.float64, device="cuda")
    x[:A.n] = torch.tensor(matgen.uniform_vector(A.n, 0), device="cuda")
    fid = rc.registerFunction(ri.MPK, ri.Operands(dm, x), power=POWER)
    assert fid >= 0
    rc.setMpkSchedule(fid, "wavefront")  # the persistent kernel, not the timed choice
    for _ in range(args.steps):
        assert rc.executeFunction(fid) == 0
    for _ in range(args.steps):
        for k in range(POWER):
            rc.spmvPowerLayout(fid, k)
    torch.cuda.synchronize()
    assert rc.getStatus() == 0
    print(f"profile case done: grid {args.grid}^3, values {args.values}, {args.steps} MPK calls")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=10.0, help="budget of the CPU baseline sample")
    ap.add_argument("--symmgs-rows", type=int, default=4194304,
                    help="rows of the power-law SymmGS system (the configuration's 4,194,304; 0 skips it)")
    ap.add_argument("--profile", choices=["mpk", "batch", "symmgs"], default=None,
                    help="profiling case (mpk, batch or symmgs; see run_profile_case); prints no JSON")
    ap.add_argument("--no-tuner", action="store_true", help="skip the MLP tuner training/evaluation")
    ap.add_argument("--batch-count", type=int, default=64,
                    help="matrices of the batched block-MPK measurement (0 skips it)")
    ap.add_argument("--batch-cache-mb", type=float, default=256.0,
                    help="RACE cacheSize of each batched matrix (256 MB: fastest of 1-1000 MB on GB300)")
    ap.add_argument("--grid", type=int, default=GRID)
    ap.add_argument("--values", choices=["f64", "f32"], default="f64")
    ap.add_argument("--c1-no-gather", action="store_true",
                    help="leave the gather sweep mode out of the 32^3 SymmSpMV search")
    ap.add_argument("--mpk-per-call", type=int, default=0,
                    help="also time the 8 powers as 8/K chained calls of power K (K in 1, 2, 4), as "
                         "tuneFunction would choose; reported as a separate item, the headline stays one call")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    if args.profile:
        run_profile_case(args)
        return
    if args.impl == "reference":
        run_reference(args, rank, world)
        return

    import torch
    import torch.distributed as dist

    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    from race_gb300 import interface as ri
    from race_gb300 import matgen

    A = build_workload()
    n, nnz = A.n, A.nnz
    stream = torch.cuda.current_stream()
    rc = ri.Interface(n, 1, ri.POWER, A.row_ptr, A.col, symm_hint=True, stream=stream)
    assert rc.RACEColor(POWER, CACHE_BYTES) == 0
    perm, inv = rc.getPerm(), rc.getInvPerm()
    P = A.permuted(perm, inv)
    x0 = matgen.uniform_vector(n, 0)
    dm64 = ri.DeviceCsr.from_csr(P, "cuda", torch.float64)
    dm32 = ri.DeviceCsr(n, dm64.row_ptr, dm64.col, dm64.val.to(torch.float32))
    x64 = torch.zeros((POWER + 1) * n, dtype=torch.float64, device="cuda")
    x64[:n] = torch.tensor(x0, device="cuda")
    x32 = x64.clone()
    f64 = rc.registerFunction(ri.MPK, ri.Operands(dm64, x64), power=POWER)
    f32 = rc.registerFunction(ri.MPK, ri.Operands(dm32, x32), power=POWER)
    assert f64 >= 0 and f32 >= 0
    layout = {"f64": rc.getMpkLayout(f64), "f32": rc.getMpkLayout(f32)}

    # correctness on the benchmark inputs: FP64 MPK == plain fma SpMV chain
    assert rc.executeFunction(f64) == 0
    y = torch.zeros_like(x64)
    y[:n] = x64[:n]
    for k in range(1, POWER + 1):
        rc.spmv_plain(dm64, y[(k - 1) * n:k * n], y[k * n:(k + 1) * n])
    assert rc.executeFunction(f32) == 0
    torch.cuda.synchronize()
    exact = bool(torch.equal(x64, y))
    x64_check = x64.clone()
    ref_last = y[POWER * n:]
    rel32 = float(((x32[POWER * n:] - ref_last).abs().max() / ref_last.abs().max()).item())

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    def timed(fn, steps):
        for _ in range(args.warmup):
            fn()
        barrier()
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        for _ in range(steps):
            fn()
        ev1.record(stream)
        barrier()
        ms = ev0.elapsed_time(ev1) / steps
        return max_over_ranks(ms, world, "cuda")

    def mpk64():
        rc.executeFunctionAsync(f64)

    def mpk32():
        rc.executeFunctionAsync(f32)

    def plain64():
        # the traditional path: p separate SpMVs on the same SELL-32 layout
        for k in range(POWER):
            rc.spmvPowerLayout(f64, k)

    blocked = None
    K = args.mpk_per_call
    if K in (1, 2, 4):
        # function j runs powers jK+1 .. jK+K on the view of x that starts
        # at power jK, so the calls chain without copies
        fids = [rc.registerFunction(ri.MPK, ri.Operands(dm64, x64[j * K * n:]), power=K) for j in range(POWER // K)]
        assert min(fids) >= 0
        x64.zero_()
        x64[:n] = torch.tensor(x0, device="cuda")
        for f in fids:
            assert rc.executeFunction(f) == 0
        torch.cuda.synchronize()
        blocked_exact = bool(torch.equal(x64, y))

        def mpk_blocks():
            for f in fids:
                rc.executeFunctionAsync(f)

        ms_b = timed(mpk_blocks, args.steps)
        assert rc.getStatus() == 0
        blocked = {"power_per_call": K, "ms_per_step": ms_b,
                   "effective_gbs": POWER * spmv_bytes(n, nnz) / (ms_b * 1e-3) / 1e9,
                   "bit_exact_vs_plain_chain": blocked_exact}

    # both MPK schedules of each function, forced, then the default (auto:
    # the faster of the two, timed at the first call, inside the warm-up)
    schedules = {}
    for name, fid, fn in (("f64", f64, mpk64), ("f32", f32, mpk32)):
        sched = {}
        for sc in ("wavefront", "sweeps"):
            rc.setMpkSchedule(fid, sc)
            sched[f"{sc}_ms"] = timed(fn, args.steps)
            assert rc.getStatus() == 0
        rc.setMpkSchedule(fid, "auto")
        schedules[name] = sched
    with ClockSampler(local) as clk:
        ms64 = timed(mpk64, args.steps)
    clocks = clk.summary()
    assert rc.getStatus() == 0
    ms32 = timed(mpk32, args.steps)
    assert rc.getStatus() == 0
    ms_plain = timed(plain64, args.steps)
    for name, fid in (("f64", f64), ("f32", f32)):
        schedules[name]["auto_chose"] = rc.getMpkLayout(fid)["schedule"]

    # End to end through the public API with host buffers, every step: the
    # step's x0 from pinned host memory to the device, the MPK, all p powers
    # back to pinned host memory. Two registered operand sets alternate, as a
    # caller streaming many vectors would run them: one step's powers drain
    # to the host (copy-out stream) while the next step computes and loads
    # its input (copy-in stream); events order every reuse of a buffer.
    xB = torch.zeros_like(x64)
    fB = rc.registerFunction(ri.MPK, ri.Operands(dm64, xB), power=POWER)
    assert fB >= 0
    bufs = [(x64, f64), (xB, fB)]
    h_in = [torch.tensor(x0, dtype=torch.float64).pin_memory() for _ in range(2)]
    h_out = [torch.empty(POWER * n, dtype=torch.float64).pin_memory() for _ in range(2)]
    s_in, s_out = torch.cuda.Stream(), torch.cuda.Stream()
    ev_in = [torch.cuda.Event() for _ in range(2)]
    ev_done = [torch.cuda.Event() for _ in range(2)]
    ev_out = [torch.cuda.Event() for _ in range(2)]
    for e in ev_out:
        e.record(stream)
    step_no = [0]

    def e2e():
        j = step_no[0] % 2
        step_no[0] += 1
        x, f = bufs[j]
        s_in.wait_event(ev_out[j])  # this buffer's previous powers have left
        with torch.cuda.stream(s_in):
            x[:n].copy_(h_in[j], non_blocking=True)
        ev_in[j].record(s_in)
        stream.wait_event(ev_in[j])
        rc.executeFunctionAsync(f)
        ev_done[j].record(stream)
        s_out.wait_event(ev_done[j])
        with torch.cuda.stream(s_out):
            h_out[j].copy_(x[n:], non_blocking=True)
        ev_out[j].record(s_out)

    for _ in range(args.warmup):
        e2e()
    barrier()
    e_start, e_end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e_start.record(stream)
    for _ in range(args.steps):
        e2e()
    for e in ev_out:  # the timed region ends when the last powers are on the host
        stream.wait_event(e)
    e_end.record(stream)
    barrier()
    ms_e2e = max_over_ranks(e_start.elapsed_time(e_end) / args.steps, world, "cuda")
    assert rc.getStatus() == 0
    e2e_ok = all(torch.equal(h_out[j].to("cuda"), bufs[j][0][n:]) for j in range(2))

    eff_bytes = POWER * spmv_bytes(n, nnz)
    plain_bytes = POWER * (layout["f64"]["matrix_bytes"] + 16 * n)
    compulsory = (nnz * 12 + 4 * (n + 1)) + 8 * n + POWER * 8 * n
    gbs = whole_job_gbs(eff_bytes, ms64, world)
    peak, peak_kind = measured_peaks()
    achieved = compulsory / (ms64 * 1e-3) / 1e9

    traffic = None
    tpath = ROOT / "profiles" / "mpk_traffic.json"
    if tpath.exists():
        traffic = json.loads(tpath.read_text()).get("dram_bytes_per_launch")

    # the GPU's FP64 powers in original row order, for the CPU leg's comparison
    g = x64_check.reshape(POWER + 1, n)[1:].cpu().numpy()
    gpu_powers = np.empty_like(g)
    gpu_powers[:, perm] = g
    del g
    cpu = cpu_baseline(A, x0, args.cpu_seconds, gpu_powers) if rank == 0 else None
    del dm32, x32
    symmgs = bench_symmgs(args, ri, matgen, torch) if args.symmgs_rows > 0 else None
    batched = bench_batch(args, ri, matgen, torch) if args.batch_count > 0 else None
    tuned = bench_tuner(torch) if not args.no_tuner else None
    c1 = bench_c1(ri, matgen, torch, gather=not args.c1_no_gather) if rank == 0 else None
    if rank == 0:
        line = {
            "metric": METRIC, "value": gbs, "unit": "GB/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms64, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": gbs / PUBLISHED_GBS, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"MPK p={POWER}, 27-point stencil {GRID}^3 (n={n}, nnz={nnz}), FP64 values, "
                                   f"RACE level groups (cacheSize {CACHE_BYTES / 1e6:.0f} MB, safety 2)",
                       "l2": "inputs larger than L2 (669 MB matrix), no flush", "parallelism": f"replicas x{world}"},
            "e2e": {"value": whole_job_gbs(eff_bytes, ms_e2e, world), "unit": "GB/s",
                    "h2d_bytes_per_step": 8 * n, "d2h_bytes_per_step": POWER * 8 * n,
                    "host_results_match_device": e2e_ok,
                    "note": "two registered operand sets alternate; copies on their own streams overlap "
                            "the next step's MPK"},
            "gpu_launches": args.steps,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "note": f"achieved = compulsory bytes ({compulsory}) per launch / launch time; "
                                 f"peak {peak_kind}",
                         # one FP64 fma per non-zero and power: the FP64 pipe bounds this kernel too
                         "fp64_pipe": {"achieved_tflops": 2 * nnz * POWER / (ms64 * 1e-3) / 1e12,
                                       "peak_tflops": FP64_PEAK_TFLOPS,
                                       "frac": 2 * nnz * POWER / (ms64 * 1e-3) / 1e12 / FP64_PEAK_TFLOPS,
                                       "peak_kind": "nominal GB300 FP64"}},
            "cpu_baseline": cpu,
            "clocks": clocks,
            "fp64_bit_exact_vs_plain_chain": exact,
            "fp64_bit_exact_vs_cpu_reference": cpu["fp64_powers_equal_gpu"] if cpu else None,
            "mpk_kernel": mpk_kernel_info(),
            "mixed_f32": {"ms_per_step": ms32, "effective_gbs": eff_bytes / (ms32 * 1e-3) / 1e9,
                          "rel_err_vs_f64": rel32, "meets_1e-10": rel32 <= 1e-10},
            "plain_f64": {"ms_per_step": ms_plain, "effective_gbs": eff_bytes / (ms_plain * 1e-3) / 1e9,
                          "hbm_frac": plain_bytes / (ms_plain * 1e-3) / 1e9 / peak,
                          "note": "hbm_frac from the bytes p SpMVs move on the registered layout "
                                  f"({plain_bytes} B: p x (layout matrix bytes + x_k + x_k+1))"},
            "mpk_layout": layout,
            "mpk_schedules": schedules,
            "symmgs_ir": symmgs,
            "batched_mpk": batched,
            "mlp_tuner": tuned,
            "symmspmv_c1": c1,
            "mpk_per_call": blocked,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def mpk_kernel_info():
    """The MPK kernel's schedule settings and the L2 die map it used."""
    import ctypes
    from race_gb300 import _lib
    nd, ns = ctypes.c_int(0), ctypes.c_int(0)
    smd = (ctypes.c_int * 4096)()
    _lib.check(_lib.lib().race_device_dies(ctypes.byref(nd), smd, 4096, ctypes.byref(ns)))
    env = {k: v for k, v in os.environ.items() if k.startswith("RACE_GPU_MPK")}
    return {"order": "chunk-level wavefront, per-die run queues", "lag_chunks": int(env.get("RACE_GPU_MPK_LAG", 32768)),
            "chunks_per_run": int(env.get("RACE_GPU_MPK_RUN", 4)), "l2_dies": nd.value,
            "sms_per_die": [sum(1 for i in range(ns.value) if smd[i] == d) for d in range(nd.value)],
            "env_overrides": env}


def bench_symmgs(args, ri, matgen, torch):
    """Symmetric Gauss-Seidel as the smoother of an FP64 iterative refinement
    on a symmetric power-law system (Chung-Lu, Pareto 2.1 weights, mean
    degree 16, off-diagonals N(0,1), diagonal = sum|off| + 1), RACE
    distance-2 coloring, b = A 1, x0 = 0, stop at relative residual 1e-10.
    Inner sweeps with FP64, FP32 and BF16 values (FP32 vectors for the
    latter two); residual and update always FP64. Effective bytes use the
    FP64 model for every variant (one symmetric sweep = 2 (12 nnz + 4(n+1) +
    24 n), one residual = 12 nnz + 4(n+1) + 16 n per refinement), so the
    ratio of the GB/s figures is the ratio of the solve speeds."""
    A = matgen.powerlaw_chung_lu(args.symmgs_rows, seed=0)
    n, nnz = A.n, A.nnz
    t0 = time.perf_counter()
    rc = ri.Interface(n, 4096, ri.TWO, A.row_ptr, A.col, symm_hint=True)
    assert rc.RACEColor() == 0
    prep = time.perf_counter() - t0
    P = A.permuted(rc.getPerm(), rc.getInvPerm())
    m64 = ri.DeviceCsr.from_csr(P)
    ones = torch.ones(n, dtype=torch.float64, device="cuda")
    b = torch.zeros(n, dtype=torch.float64, device="cuda")
    rc.spmv_plain(m64, ones, b)
    per_it = 2 * (12 * nnz + 4 * (n + 1) + 24 * n) + (12 * nnz + 4 * (n + 1) + 16 * n)
    out = {"workload": f"power-law n={n} nnz={nnz}, RACE D2 (4096 threads requested -> {rc.getNumThreads()}, "
                       f"efficiency {rc.getEfficiency():.4f}), b=A*1, tol 1e-10",
           "preprocessing_s": prep}
    for name, vdt in [("f64", torch.float64), ("f32", torch.float32), ("bf16", torch.bfloat16)]:
        xdt = torch.float64 if name == "f64" else torch.float32
        d = torch.zeros(n, dtype=xdt, device="cuda")
        r = torch.zeros(n, dtype=xdt, device="cuda")
        fid = rc.registerFunction(ri.GS, ri.Operands(ri.DeviceCsr(n, m64.row_ptr, m64.col, m64.val.to(vdt)), d, r))
        x = torch.zeros(n, dtype=torch.float64, device="cuda")
        rc.symmGsIr(fid, m64, b, x, tol=1e-10, maxIter=1, sweeps=1)  # warm-up
        x.zero_()
        torch.cuda.synchronize()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record()
        its, rel = rc.symmGsIr(fid, m64, b, x, tol=1e-10, maxIter=300, sweeps=1)
        ev1.record()
        torch.cuda.synchronize()
        sec = ev0.elapsed_time(ev1) / 1e3
        info = rc.getSweepInfo(fid)
        out[name] = {"refinements": its, "rel_residual": rel, "seconds": sec,
                     "effective_gbs": per_it * its / sec / 1e9,
                     "max_err_vs_exact": float((x - 1).abs().max()), "waves_per_sweep": info["waves"],
                     "wave_mode": info["wave_mode"]}
    out["mixed_f32_speedup_vs_f64"] = out["f64"]["seconds"] / out["f32"]["seconds"]
    out["mixed_bf16_speedup_vs_f64"] = out["f64"]["seconds"] / out["bf16"]["seconds"]
    return out


def bench_batch(args, ri, matgen, torch):
    """Batched block MPK: ``--batch-count`` 2D anisotropic 5/9-point
    stencils (grid sides U{100..700}, coefficient ratio log-uniform 1-100),
    16 right-hand sides U[-1,1] each, p = 4, every matrix with its own RACE
    level groups; all matrices in ONE persistent launch replayed from a CUDA
    graph, FP64 (values and vectors) and FP32. Compared with the same
    functions launched one matrix at a time, and with the plain path (p
    multi-vector SpMV launches per matrix). Compulsory bytes: matrix once
    (nnz (s+4) + 4 (n+1)) plus the input block and p output blocks
    (16 (p+1) n xs); the plain path's bytes are p (nnz (s+4) + 4 (n+1) +
    2 16 n xs)."""
    p, nrhs = 4, 16
    mats = matgen.aniso2d_batch(args.batch_count, seed=0)
    t0 = time.perf_counter()
    members = []
    for i, A in enumerate(mats):
        rc = ri.Interface(A.n, 1, ri.POWER, A.row_ptr, A.col, symm_hint=True)
        assert rc.RACEColor(p, args.batch_cache_mb * 1e6) == 0
        P = A.permuted(rc.getPerm(), rc.getInvPerm())
        members.append((rc, P))
    prep = time.perf_counter() - t0
    n_tot = sum(P.n for _, P in members)
    nnz_tot = sum(P.nnz for _, P in members)
    out = {"workload": f"{len(mats)} matrices (aniso 5/9-point, {n_tot} rows, {nnz_tot} nnz in total), "
                       f"{nrhs} right-hand sides, p={p}, cacheSize {args.batch_cache_mb} MB each",
           "preprocessing_s": prep}
    results = {}
    for name, vdt, xdt, vs, xs in [("f64", torch.float64, torch.float64, 8, 8),
                                   ("f32", torch.float32, torch.float32, 4, 4)]:
        batch = ri.Batch()
        fns = []
        for i, (rc, P) in enumerate(members):
            dm = ri.DeviceCsr.from_csr(P, "cuda", vdt)
            x = torch.zeros((p + 1) * P.n * nrhs, dtype=xdt, device="cuda")
            x[: P.n * nrhs] = torch.tensor(matgen.uniform_block(P.n, nrhs, seed=100 + i).reshape(-1),
                                           dtype=xdt, device="cuda")
            fid = rc.registerMpkBlock(ri.Operands(dm, x), p, nrhs)
            assert fid >= 0
            batch.add(rc, fid)
            fns.append((rc, fid, dm, x))
        batch.prepare()
        compulsory = nnz_tot * (vs + 4) + 4 * (n_tot + len(mats)) + nrhs * (p + 1) * n_tot * xs
        plain_bytes = p * (nnz_tot * (vs + 4) + 4 * (n_tot + len(mats)) + 2 * nrhs * n_tot * xs)

        def timeit(fn, steps):
            for _ in range(3):
                fn()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(steps):
                fn()
            e1.record()
            torch.cuda.synchronize()
            return e0.elapsed_time(e1) / steps

        def per_matrix():
            for rc, fid, _, _ in fns:
                rc.executeFunctionAsync(fid)

        def plain():
            for rc, fid, _, _ in fns:
                for k in range(p):
                    rc.spmvPowerLayout(fid, k)

        steps = max(3, args.steps)
        ms_graph = timeit(batch.graphLaunch, steps)
        assert batch.getStatus() == 0
        ms_launch = timeit(batch.execute, steps)
        assert batch.getStatus() == 0
        snap = [x[P.n * nrhs:].clone() for (_, _, _, x), (_, P) in zip(fns, members)]
        ms_per = timeit(per_matrix, steps)
        ms_plain = timeit(plain, steps)
        same = all(torch.equal(s, x[P.n * nrhs:]) for s, (_, _, _, x), (_, P) in zip(snap, fns, members))
        results[name] = {"ms_graph": ms_graph, "ms_one_launch": ms_launch, "ms_per_matrix_launches": ms_per,
                         "ms_plain": ms_plain,
                         "compulsory_gbs": compulsory / (ms_graph * 1e-3) / 1e9,
                         "plain_equiv_gbs": plain_bytes / (ms_graph * 1e-3) / 1e9,
                         "plain_path_gbs": plain_bytes / (ms_plain * 1e-3) / 1e9,
                         "speedup_vs_plain": ms_plain / ms_graph, "speedup_vs_per_matrix": ms_per / ms_graph,
                         "bit_identical_to_plain_path": bool(same), "launches_per_step": 1}
        results[name]["_x"] = [x for (_, _, _, x) in fns]
        del batch
    rel = 0.0
    for x64, x32, (_, P) in zip(results["f64"].pop("_x"), results["f32"].pop("_x"), members):
        a, b = x64[p * P.n * nrhs:], x32[p * P.n * nrhs:].double()
        rel = max(rel, float((a - b).abs().max() / a.abs().max()))
    results["f32"]["rel_err_vs_f64"] = rel
    out.update(results)
    out["mixed_f32_speedup_vs_f64_plain"] = results["f64"]["ms_plain"] / results["f32"]["ms_graph"]
    return out


def bench_c1(ri, matgen, torch, reps: int = 100, gather: bool = True):
    """SymmSpMV with RACE distance-2 coloring on the 32^3 7-point Laplacian
    (n = 32,768, upper triangle 128,000 entries incl. the diagonal), x
    U[-1,1] seed 0, 100 calls per setting. Bytes per call: 12 nnz_u + 4(n+1)
    + 8n (x) + 16n (b read and written) = 2,453,508 B; the working set
    (2.5 MB) lives in L2, so "% of HBM" does not apply and the time is the
    latency of RACE's phases. Requested threads (RACE_THREADS, 256/1024/4096)
    and sweep mode (wave, leaf, gather) are searched as a user tunes them; the
    best is reported with all settings. The CPU baseline is RACE's colored
    executor (the oracle's port: leaves of a phase on parallel OpenMP threads,
    a barrier between phases) on all host cores, with the coloring RACE makes
    for that many threads, median of 10 trials of `reps` calls (the
    reference's practice, examples/src/colorSymmSpMV.cpp:71-99); the
    sequential kernel body on one core is reported beside it."""
    from oracle import oracle as orc
    A = matgen.laplace3d_7pt(32)
    x0 = matgen.uniform_vector(A.n, 0)
    nbytes = None
    settings = []
    for threads in (256, 1024, 4096):
        rc = ri.Interface(A.n, threads, ri.TWO, A.row_ptr, A.col, symm_hint=True)
        assert rc.RACEColor() == 0
        P = A.permuted(rc.getPerm(), rc.getInvPerm())
        U = P.upper()
        nbytes = 12 * U.nnz + 4 * (A.n + 1) + 24 * A.n
        x = torch.tensor(x0, device="cuda")
        b = torch.zeros(A.n, dtype=torch.float64, device="cuda")
        fid = rc.registerFunction(ri.SYMMSPMV, ri.Operands(ri.DeviceCsr.from_csr(U), x, b))
        assert fid >= 0
        info = rc.getSweepInfo(fid)
        modes = [(ri.SWEEP_WAVE, "wave"), (ri.SWEEP_LEAF, "leaf")] + ([(ri.SWEEP_GATHER, "gather")] if gather else [])
        for mode, mname in modes:
            rc.setSweepMode(mode)
            for _ in range(5):
                rc.executeFunctionAsync(fid)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(reps):
                rc.executeFunctionAsync(fid)
            e1.record()
            torch.cuda.synchronize()
            assert rc.getStatus() == 0
            settings.append({"threads": threads, "threads_used": rc.getNumThreads(), "mode": mname,
                             "waves": info["waves"], "phases": info["phases"],
                             "ms": e0.elapsed_time(e1) / reps})
        rc.close()
    best = min(settings, key=lambda d: d["ms"])
    # CPU: RACE's colored executor on all host cores
    cores = os.cpu_count() or 1
    rc = ri.Interface(A.n, cores, ri.TWO, A.row_ptr, A.col, symm_hint=True)
    assert rc.RACEColor() == 0
    perm = rc.getPerm()
    P = A.permuted(perm, rc.getInvPerm())
    U = P.upper()
    pp, lo, hi = rc.getPhases()
    cpu_threads_used = rc.getNumThreads()
    rc.close()
    xr, br = x0[perm].copy(), np.zeros(A.n)
    trials = []
    orc.exec_phases_omp(orc.K_SYMMSPMV, pp, lo, hi, cores, 5, U, xr, br)
    for _ in range(10):
        t0 = time.perf_counter()
        orc.exec_phases_omp(orc.K_SYMMSPMV, pp, lo, hi, cores, reps, U, xr, br)
        trials.append((time.perf_counter() - t0) / reps * 1e3)
    cpu_ms = statistics.median(trials)
    U1 = A.upper()
    xs, bs = x0.copy(), np.zeros(A.n)
    t0 = time.perf_counter()
    for _ in range(reps):
        orc.run_kernel(orc.K_SYMMSPMV, 0, A.n, U1, xs, bs)
    seq_ms = (time.perf_counter() - t0) / reps * 1e3
    return {"workload": f"SymmSpMV, 7-point Laplacian 32^3, RACE D2, {reps} calls per setting",
            "bytes_per_call": nbytes, "best": best, "gpu_gbs_best": nbytes / (best["ms"] * 1e-3) / 1e9,
            "settings": settings,
            "cpu_reference_ms_per_call": cpu_ms, "cpu_reference_cores": cores,
            "cpu_reference_threads_used": cpu_threads_used,
            "cpu_reference": "RACE colored executor (oracle port), leaves of a phase on OpenMP threads, "
                             f"D2 coloring for {cores} threads, median of 10 trials of {reps} calls",
            "gpu_speedup_vs_cpu_reference": cpu_ms / best["ms"],
            "cpu_sequential_body_ms_per_call": seq_ms}


def bench_tuner(torch, retime: int = 8):
    """The MLP cost model (matrix and config features -> 3 x 128 ReLU -> log
    time), trained by the engine's CUDA kernels on committed search timings
    and evaluated on the held-out matrices against the searched optimum and
    against the best single config. Tasks: A^8 x over power per block x
    cache budget x recursion depth (tuner_search.npz) and a symmetric GS
    sweep over requested threads x efficiency threshold
    (tuner_search_symmgs.npz). For up to `retime` held-out matrices of the
    MPK set (the smallest, up to 200k rows), the MLP's pick and the
    searched optimum are timed again here on fresh engines and the regret
    is recomputed from those times."""
    from race_gb300 import tuner
    out = {}
    for name, fname in [("mpk", "tuner_search.npz"), ("symmgs", "tuner_search_symmgs.npz")]:
        path = ROOT / "tests" / "golden" / fname
        if not path.exists():
            continue
        ds = tuner.Dataset.load(path)
        held = tuner.held_out(len(ds.times), ds.task)
        train, test = ds.subset(~held), ds.subset(held)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        model = tuner.CostModel(seed=0, task=tuner.TASKS[ds.task])
        hist = model.fit(train, seed=0)
        torch.cuda.synchronize()
        res = tuner.evaluate(model, test, tuner.best_fixed_config(train))
        res.update({"train_matrices": len(train.times), "train_seconds": time.perf_counter() - t0,
                    "final_train_loss": hist[-1]})
        if name == "mpk" and retime > 0:
            rows = [i for i in np.flatnonzero(held) if ds.sizes[i][0] <= 200_000]
            rows = sorted(rows, key=lambda i: ds.sizes[i][0])[:retime]
            regrets, details = [], []
            for i in rows:
                fam, A = tuner.dataset_matrix(int(ds.index[i]))
                feas = np.isfinite(ds.times[i])
                pick = model.choose(ds.features[i], feas)
                best = int(np.argmin(ds.times[i]))
                t_pick = tuner.time_config(A, tuner.CONFIGS[pick])
                t_best = t_pick if best == pick else tuner.time_config(A, tuner.CONFIGS[best])
                regrets.append(t_pick / min(t_pick, t_best) - 1.0)
                details.append({"matrix": int(ds.index[i]), "family": fam, "n": A.n, "pick": list(tuner.CONFIGS[pick]),
                                "searched_best": list(tuner.CONFIGS[best]), "t_pick_ms": t_pick * 1e3,
                                "t_best_ms": t_best * 1e3})
            res["retimed_here"] = {"matrices": len(regrets), "mean_regret": float(np.mean(regrets)) if regrets else None,
                                   "within_10pct": float(np.mean(np.asarray(regrets) <= 0.10)) if regrets else None,
                                   "cases": details}
        out[name] = res
    return out or None


def cpu_baseline(A, x0, budget_s: float, gpu_powers=None):
    """The reference algorithm (RACE wavefront, oracle port) on all host
    cores, with the host's fastest cache budget, on full MPK calls of the
    same workload until the time budget is spent. With gpu_powers (the GPU's
    FP64 powers 1..p in original row order) it also reports whether the CPU
    wavefront's powers equal them bit for bit."""
    from oracle import oracle as orc
    threads = os.cpu_count() or 1
    P, (gp, ur, dr), cache, _, perm = cpu_partition(A, x0, threads)
    times = []
    t_start = time.perf_counter()
    y = None
    while time.perf_counter() - t_start < budget_s and len(times) < 50:
        t0 = time.perf_counter()
        y = orc.mpk_wavefront(P, x0, POWER, gp, ur, dr, threads)
        times.append(time.perf_counter() - t0)
    t = statistics.median(times)
    same = None
    if gpu_powers is not None:
        y_orig = np.empty_like(y[1:])
        y_orig[:, perm] = y[1:]
        same = bool(np.array_equal(y_orig, gpu_powers))
    return {"value": POWER * spmv_bytes(A.n, A.nnz) / t / 1e9, "unit": "GB/s", "cores": threads, "kind": "port",
            "fp64_powers_equal_gpu": same,
            "sample": f"{len(times)} full MPK p={POWER} calls (median), RACE level-group wavefront "
                      f"restated in C on {threads} OpenMP threads, cacheSize {cache / 1e6:.0f} MB (the fastest "
                      f"on this host of {'/'.join(f'{c / 1e6:.0f}' for c in CPU_CACHE_CANDIDATES)} MB)"}


if __name__ == "__main__":
    main()
