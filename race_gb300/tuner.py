"""Learned tuning of the matrix-power kernel: an MLP cost model trained on the
engine's own parameter search.

The reference tunes one knob by wall clock: Interface::tuneFunction
(src/interface.cpp:605-647) runs powers 1..p and keeps the fastest. Its other
knobs are the cache budget of RACEColor(power, cacheSize, ...)
(interface.cpp:205), the power per block and the depth of the recursion into
hopeless regions (RACE_MAX_RECURSION_STAGES, src/matrixPowerRecursive.cpp).
This module searches those knobs on the GPU for A^8 x (computed as 8/p
chained MPK calls of power p, each in the engine's default schedule) and
learns from the search:

* ``CONFIGS``: power per block p in {1, 2, 4, 8} times cache budget in
  {8, 32, 128, 512} MB times recursion stages in {0, 1, 2} (p = 1 takes one
  budget and depth: it has no blocking);
* ``search``: times every config on the engine (median of repetitions);
  where the default depth's partition has no hopeless region every depth
  gives the same partition, and the other depths take its time; configs
  whose partition the engine refuses are infeasible;
* ``matrix_features`` / ``config_features``: 24 structural features of the
  matrix (sizes, row lengths, index distances, BFS level profile from row 0,
  RACE's root) and 10 of the config, 34 inputs in total;
* ``CostModel``: an MLP 34 -> 3 x 128 (ReLU) -> 1 predicting the log time,
  trained with the engine's own CUDA kernels (race_mlp_* in the C ABI:
  forward, MSE gradient, Adam); it picks the feasible config with the
  lowest predicted time;
* ``Tuner.choose``: the MLP's choice, or the search (the fallback when no
  model is loaded, and the yardstick of the model's regret:
  regret = t(chosen) / t(best searched) - 1).

A second task, ``SWEEP_TASK``, tunes RACE's coloring for a symmetric
Gauss-Seidel sweep (forward + backward, FP64, distance-2 coloring): requested
threads in {64, 256, 1024} times the efficiency threshold RACE_EFFICIENCY in
{20, 40, 80} (src/level_recursion.cpp:48-70).

The seeded matrix set (``dataset_matrix``): 3D 7-point and 27-point
stencils, banded matrices (bandwidth 8-512) with scrambled rows, Chung-Lu
power-law graphs, n log-uniform in [50k, 2M] rows by default.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import math
import time
from typing import Optional

import numpy as np

from . import matgen

TOTAL_POWER = 8
CACHE_MB = (8, 32, 128, 512)
RECURSION_STAGES = (0, 1, 2)  # RACE_MAX_RECURSION_STAGES; 1 is the default
CONFIGS = [(1, 512, 1)] + [(p, c, r) for p in (2, 4, 8) for c in CACHE_MB for r in RECURSION_STAGES]
L2_BYTES = 126.5 * 2 ** 20
N_MATRIX_FEATURES = 24
N_CONFIG_FEATURES = 10
N_FEATURES = N_MATRIX_FEATURES + N_CONFIG_FEATURES
HIDDEN, HIDDEN_LAYERS = 128, 3


# ---------------------------------------------------------------- features
def bfs_levels(A) -> np.ndarray:
    """BFS distance of every row from row 0 over the symmetric pattern
    (unreached rows: -1)."""
    import scipy.sparse as sp
    from scipy.sparse.csgraph import shortest_path
    M = sp.csr_matrix((np.ones(A.nnz, np.float32), A.col, A.row_ptr), shape=(A.n, A.n))
    d = shortest_path(M, method="D", directed=False, unweighted=True, indices=0)
    out = np.full(A.n, -1, np.int64)
    ok = np.isfinite(d)
    out[ok] = d[ok].astype(np.int64)
    return out


def matrix_features(A) -> np.ndarray:
    n, nnz = A.n, A.nnz
    rl = np.diff(A.row_ptr).astype(np.float64)
    rows = np.repeat(np.arange(n), np.diff(A.row_ptr))
    dist = np.abs(rows - A.col.astype(np.int64)).astype(np.float64)
    lev = bfs_levels(A)
    reached = lev >= 0
    L = int(lev.max()) + 1 if reached.any() else 1
    lrow = np.bincount(lev[reached], minlength=L).astype(np.float64)
    lnnz = np.bincount(lev[reached], weights=rl[reached], minlength=L)
    bytes64 = nnz * 12.0 + 4.0 * n
    mean = rl.mean()
    f = [
        math.log2(n) / 20, math.log2(max(nnz, 1)) / 25, mean / 32, math.log2(1 + rl.std() / max(mean, 1e-9)),
        math.log2(max(rl.max(), 1)) / 10, rl.min() / 32, float((rl > 2 * mean).mean()),
        math.log2(bytes64 / L2_BYTES) / 5, math.log2((nnz * 8.0 + 4.0 * n) / L2_BYTES) / 5,
        dist.mean() / n, float(np.percentile(dist, 90)) / n, dist.max() / n,
        float((dist <= 1).mean()), float((dist <= 32).mean()), float((dist <= 1024).mean()),
        math.log2(L) / 20, math.log2(n / L) / 20, lrow.max() / n, lnnz.max() / max(nnz, 1),
        lrow.std() / max(lrow.mean(), 1e-9) / 4, float(reached.mean()),
        math.log2(max(lnnz.max() * 12.0, 1.0) / L2_BYTES) / 10,
        float(np.sort(lrow)[::-1][: max(1, L // 10)].sum() / n), 1.0,
    ]
    assert len(f) == N_MATRIX_FEATURES
    return np.asarray(f, np.float32)


def config_features(mf: np.ndarray, p: int, cache_mb: float, stages: int = 1) -> np.ndarray:
    """Features of one config given the matrix features (log sizes are
    recovered from them)."""
    lp = math.log2(p)
    cb = cache_mb * 1e6
    bytes64 = L2_BYTES * 2 ** (mf[7] * 5)
    maxlev = L2_BYTES * 2 ** (mf[21] * 10)
    blocked = p > 1
    c3 = math.log2(cb / bytes64) / 10 if blocked else 0.0
    f = [lp / 3, 0.0 if blocked else 1.0, (math.log2(cache_mb) / 9) if blocked else 0.0, c3,
         (math.log2(cb / (2 * (p + 1) * maxlev)) / 10) if blocked else 0.0, lp * c3,
         (math.log2(cb / L2_BYTES) / 5) if blocked else 0.0, TOTAL_POWER / p / 8,
         stages / 2 if blocked else 0.0, stages * c3 / 2 if blocked else 0.0]
    assert len(f) == N_CONFIG_FEATURES
    return np.asarray(f, np.float32)


def sweep_config_features(mf: np.ndarray, threads: int, eff: float) -> np.ndarray:
    """Features of a coloring config: requested threads and efficiency
    threshold, alone and against the matrix size and BFS level count."""
    lt = math.log2(threads)
    log_n = mf[0] * 20
    log_levels = mf[15] * 20
    e = eff / 100.0
    f = [lt / 12, e, e * e, lt * e / 12, (log_n - lt) / 20, (log_levels - lt) / 20, lt * lt / 144, 1.0]
    return np.asarray(f, np.float32)


SWEEP_CONFIGS = [(t, e) for t in (64, 256, 1024) for e in (20.0, 40.0, 80.0)]


def feature_rows(mf: np.ndarray, task=None) -> np.ndarray:
    task = task or MPK_TASK
    return np.stack([np.concatenate([mf, task.config_features(mf, *c)]) for c in task.configs])


# ---------------------------------------------------------------- search
def has_hopeless(tree: np.ndarray) -> bool:
    """Whether an MPK leaf tree (Interface.getPowerTree: count, then per
    leaf lo, hi, stage, parent, numGroups, groupPtr[numGroups+1],
    numHopeless, ...) holds hopeless regions: more leaves than the root, or
    hopeless groups in the root."""
    if len(tree) == 0:
        return False
    if tree[0] > 1:
        return True
    ng = int(tree[5])
    return int(tree[6 + ng + 1]) > 0


def search(A, reps: int = 5, warmup: int = 2, stream=None) -> np.ndarray:
    """Seconds of A^8 x per config (np.inf where RACE rejects the
    partition), timed with CUDA events on the engine's stream. One engine
    per recursion depth; depths other than the default are timed only where
    the default's partition has hopeless regions."""
    import torch

    from . import interface as ri
    times = np.full(len(CONFIGS), np.inf)
    x0 = torch.tensor(matgen.uniform_vector(A.n, 0), device="cuda")
    engines = {}

    def engine(r):
        if r not in engines:
            engines[r] = [ri.Interface(A.n, 1, ri.POWER, A.row_ptr, A.col, symm_hint=True,
                                       params={"max_recursion_stages": r}), None, None]
        return engines[r]

    def timed(r, p, c):
        """(seconds or inf, whether the partition has hopeless regions)"""
        eng = engine(r)
        rc = eng[0]
        if rc.RACEColor(p, c * 1e6) != 0:
            return np.inf, False
        hopeless = has_hopeless(rc.getPowerTree())
        # The permutation normally stays the one of the first partition; a
        # partition with hopeless regions reorders rows inside groups.
        cur = rc.getPerm()
        if eng[1] is None or not np.array_equal(cur, eng[1]):
            eng[1] = cur
            eng[2] = ri.DeviceCsr.from_csr(A.permuted(cur, rc.getInvPerm()), "cuda", torch.float64)
        dm = eng[2]
        x = torch.zeros((p + 1) * A.n, dtype=torch.float64, device="cuda")
        fid = rc.registerFunction(ri.MPK, ri.Operands(dm, x), power=p)
        x[: A.n].copy_(x0)
        if rc.executeFunction(fid) != 0:  # also catches an error code returned in place of an id
            return np.inf, hopeless

        def run():
            x[: A.n].copy_(x0)
            for j in range(TOTAL_POWER // p):
                if j:
                    x[: A.n].copy_(x[p * A.n:])
                rc.executeFunctionAsync(fid)

        for _ in range(warmup):
            run()
        ts = []
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            run()
            e1.record()
            e1.synchronize()
            ts.append(e0.elapsed_time(e1) * 1e-3)
        if rc.getStatus() != 0:
            return np.inf, hopeless
        return float(np.median(ts)), hopeless

    index = {cfg: i for i, cfg in enumerate(CONFIGS)}
    times[index[(1, 512, 1)]] = timed(1, 1, 512)[0]
    for p in (2, 4, 8):
        for c in CACHE_MB:
            t, hopeless = timed(1, p, c)
            times[index[(p, c, 1)]] = t
            for r in RECURSION_STAGES:
                if r != 1:
                    times[index[(p, c, r)]] = timed(r, p, c)[0] if hopeless else t
    for eng in engines.values():
        eng[0].close()
    return times


def time_config(A, config, reps: int = 5, warmup: int = 2) -> float:
    """Seconds of A^8 x in one MPK config (p, cacheMB, recursion stages) on
    a fresh engine, timed as the search times it (np.inf if refused)."""
    import torch

    from . import interface as ri
    p, c, r = config
    rc = ri.Interface(A.n, 1, ri.POWER, A.row_ptr, A.col, symm_hint=True, params={"max_recursion_stages": r})
    try:
        if rc.RACEColor(p, c * 1e6) != 0:
            return np.inf
        P = A.permuted(rc.getPerm(), rc.getInvPerm())
        dm = ri.DeviceCsr.from_csr(P, "cuda", torch.float64)
        x0 = torch.tensor(matgen.uniform_vector(A.n, 0), device="cuda")
        x = torch.zeros((p + 1) * A.n, dtype=torch.float64, device="cuda")
        fid = rc.registerFunction(ri.MPK, ri.Operands(dm, x), power=p)
        x[: A.n].copy_(x0)
        if rc.executeFunction(fid) != 0:
            return np.inf

        def run():
            x[: A.n].copy_(x0)
            for j in range(TOTAL_POWER // p):
                if j:
                    x[: A.n].copy_(x[p * A.n:])
                rc.executeFunctionAsync(fid)

        for _ in range(warmup):
            run()
        ts = []
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            run()
            e1.record()
            e1.synchronize()
            ts.append(e0.elapsed_time(e1) * 1e-3)
        return float(np.median(ts)) if rc.getStatus() == 0 else np.inf
    finally:
        rc.close()


def search_sweep(A, reps: int = 5, warmup: int = 2) -> np.ndarray:
    """Seconds of one symmetric GS sweep (forward + backward, FP64) per
    coloring config (np.inf where RACEColor fails)."""
    import torch

    from . import interface as ri
    times = np.full(len(SWEEP_CONFIGS), np.inf)
    x0 = torch.tensor(matgen.uniform_vector(A.n, 0), device="cuda")
    b0 = torch.tensor(matgen.uniform_vector(A.n, 1), device="cuda")
    for ci, (threads, eff) in enumerate(SWEEP_CONFIGS):
        rc = ri.Interface(A.n, threads, ri.TWO, A.row_ptr, A.col, symm_hint=True, params={"efficiency": [eff]})
        if rc.RACEColor() != 0:
            rc.close()
            continue
        P = A.permuted(rc.getPerm(), rc.getInvPerm())
        x, b = x0.clone(), b0.clone()
        fid = rc.registerFunction(ri.GS, ri.Operands(ri.DeviceCsr.from_csr(P, "cuda", torch.float64), x, b))
        if rc.executeFunction(fid) != 0:  # also catches an error code returned in place of an id
            rc.close()
            continue

        def run():
            rc.executeFunctionAsync(fid)
            rc.executeFunctionAsync(fid, True)

        for _ in range(warmup):
            run()
        ts = []
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            run()
            e1.record()
            e1.synchronize()
            ts.append(e0.elapsed_time(e1) * 1e-3)
        if rc.getStatus() == 0:
            times[ci] = float(np.median(ts))
        rc.close()
    return times


def dataset_matrix(index: int, seed: int = 0, nmin: int = 50_000, nmax: int = 2_000_000):
    """Matrix `index` of the seeded tuning set: 3D 7-point or 27-point
    stencil, random banded (bandwidth 8-512, rows scrambled) or power-law
    graph, n log-uniform in [nmin, nmax]."""
    rng = np.random.Generator(np.random.PCG64([seed, index]))
    fam = int(rng.integers(0, 4))
    n = int(math.exp(rng.uniform(math.log(nmin), math.log(nmax))))
    if fam == 0:
        g = max(8, round(n ** (1 / 3)))
        return "lap7", matgen.laplace3d_7pt(g)
    if fam == 1:
        g = max(8, round(n ** (1 / 3)))
        return "st27", matgen.stencil3d_27pt(g, seed=int(rng.integers(1 << 30)))
    if fam == 2:
        bw = int(math.exp(rng.uniform(math.log(8), math.log(512))))
        return "band", matgen.banded_scrambled(n, bw, seed=int(rng.integers(1 << 30)), fill=min(0.5, 32.0 / bw))
    return "plaw", matgen.powerlaw_chung_lu(n, seed=int(rng.integers(1 << 30)))


# ---------------------------------------------------------------- the network
def init_params(seed: int = 0, n_in: int = N_FEATURES, hidden: int = HIDDEN, layers: int = HIDDEN_LAYERS,
                n_out: int = 1) -> np.ndarray:
    """He-uniform weights, zero biases, in the C ABI's flat layout."""
    rng = np.random.Generator(np.random.PCG64(seed))
    dims = [n_in] + [hidden] * layers + [n_out]
    parts = []
    for i, o in zip(dims[:-1], dims[1:]):
        lim = math.sqrt(6.0 / i)
        parts.append(rng.uniform(-lim, lim, size=o * i))
        parts.append(np.zeros(o))
    return np.concatenate(parts).astype(np.float32)


class Mlp:
    """The C ABI's race_mlp: parameters, forward, gradient, Adam on the GPU."""

    def __init__(self, n_in: int = N_FEATURES, hidden: int = HIDDEN, layers: int = HIDDEN_LAYERS, n_out: int = 1,
                 seed: int = 0):
        from ._lib import check, lib
        self._lib, self._checkfn = lib(), check
        self.dims = (n_in, hidden, layers, n_out)
        h = C.c_void_p()
        check(self._lib.race_mlp_create(C.byref(h), n_in, hidden, layers, n_out))
        self._h = h
        cnt = C.c_longlong()
        self._check(self._lib.race_mlp_num_params(self._h, C.byref(cnt)))
        self.num_params = cnt.value
        self.set_params(init_params(seed, n_in, hidden, layers, n_out))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            self._lib.race_mlp_destroy(h)
            self._h = None

    def _check(self, rc):
        if rc != 0:
            m = self._lib.race_mlp_last_error(self._h)
            from ._lib import RaceError
            raise RaceError(rc, m.decode() if m else "")

    def set_params(self, theta: np.ndarray):
        theta = np.ascontiguousarray(theta, np.float32)
        self._check(self._lib.race_mlp_set_params(self._h, theta.ctypes.data, theta.size))

    def get_params(self) -> np.ndarray:
        out = np.zeros(self.num_params, np.float32)
        self._check(self._lib.race_mlp_get_params(self._h, out.ctypes.data, out.size))
        return out

    def forward(self, X):
        """X: torch float32 (batch, n_in) on the GPU -> (batch, n_out)."""
        import torch
        X = X.contiguous()
        Y = torch.empty((X.shape[0], self.dims[3]), dtype=torch.float32, device=X.device)
        self._check(self._lib.race_mlp_forward(self._h, C.c_void_p(X.data_ptr()), X.shape[0],
                                               C.c_void_p(Y.data_ptr()), C.c_void_p(torch.cuda.current_stream()
                                                                                    .cuda_stream)))
        return Y

    def loss_grad(self, X, T, want_grad: bool = True):
        import torch
        X, T = X.contiguous(), T.contiguous()
        loss = C.c_float()
        g = np.zeros(self.num_params, np.float32) if want_grad else None
        self._check(self._lib.race_mlp_loss_grad(self._h, C.c_void_p(X.data_ptr()), C.c_void_p(T.data_ptr()),
                                                 X.shape[0], C.byref(loss), None if g is None else g.ctypes.data,
                                                 C.c_void_p(torch.cuda.current_stream().cuda_stream)))
        return loss.value, g

    def train(self, X, T, epochs: int = 200, batch: int = 256, lr: float = 2e-3, seed: int = 0):
        """Minibatch Adam on (X, T) (torch float32 on the GPU); returns the
        loss history per epoch (full-data loss)."""
        import torch
        g = torch.Generator(device="cpu")
        g.manual_seed(seed)
        s = C.c_void_p(torch.cuda.current_stream().cuda_stream)
        hist = []
        n = X.shape[0]
        for ep in range(epochs):
            order = torch.randperm(n, generator=g).to(X.device)
            for i in range(0, n, batch):
                idx = order[i: i + batch]
                xb, tb = X[idx].contiguous(), T[idx].contiguous()
                self._check(self._lib.race_mlp_loss_grad(self._h, C.c_void_p(xb.data_ptr()),
                                                         C.c_void_p(tb.data_ptr()), xb.shape[0], None, None, s))
                self._check(self._lib.race_mlp_adam_step(self._h, lr, 0.9, 0.999, 1e-8, s))
            if ep == epochs - 1 or ep % 10 == 0:
                hist.append(self.loss_grad(X, T, want_grad=False)[0])
        return hist


# ---------------------------------------------------------------- the tuner
@dataclasses.dataclass(frozen=True)
class Task:
    name: str
    configs: list
    config_features: object
    search: object


MPK_TASK = Task("mpk", CONFIGS, config_features, search)
SWEEP_TASK = Task("symmgs", SWEEP_CONFIGS, sweep_config_features, search_sweep)
TASKS = {t.name: t for t in (MPK_TASK, SWEEP_TASK)}


@dataclasses.dataclass
class Dataset:
    features: np.ndarray   # (matrices, 24)
    times: np.ndarray      # (matrices, len(CONFIGS)) seconds, inf = infeasible
    families: np.ndarray
    sizes: np.ndarray      # (matrices, 2): n, nnz
    task: str = "mpk"      # configs of the times' columns: TASKS[task].configs
    index: Optional[np.ndarray] = None  # each row's matrix in the seeded set (dataset_matrix)

    def __post_init__(self):
        if self.index is None:
            self.index = np.arange(len(self.times), dtype=np.int64)

    def save(self, path):
        np.savez_compressed(path, features=self.features, times=self.times, families=self.families,
                            sizes=self.sizes, configs=np.asarray(TASKS[self.task].configs),
                            task=np.array(self.task), index=np.asarray(self.index, np.int64))

    @staticmethod
    def load(path) -> "Dataset":
        d = np.load(path)
        task = str(d["task"]) if "task" in d.files else "mpk"
        assert [tuple(c) for c in d["configs"]] == [tuple(c) for c in TASKS[task].configs], "config space changed"
        return Dataset(d["features"], d["times"], d["families"], d["sizes"], task,
                       d["index"] if "index" in d.files else None)

    def subset(self, idx) -> "Dataset":
        return Dataset(self.features[idx], self.times[idx], self.families[idx], self.sizes[idx], self.task,
                       self.index[idx])


def regret(times_row: np.ndarray, choice: int) -> float:
    return float(times_row[choice] / np.min(times_row) - 1.0)


class CostModel:
    """MLP regression of log time on (matrix, config) features: an ensemble
    of `members` networks from consecutive seeds, trained alike, whose
    predictions are averaged (in the normalised log domain), which steadies
    the choice between seeds."""

    def __init__(self, seed: int = 0, task: Task = None, members: int = 3):
        self.task = task or MPK_TASK
        n_in = feature_rows(np.zeros(N_MATRIX_FEATURES, np.float32), self.task).shape[1]
        self.seed = seed
        self.nets = [Mlp(n_in=n_in, seed=seed + m) for m in range(max(1, members))]
        self.mu = 0.0
        self.sd = 1.0

    def _rows(self, ds: Dataset):
        X, T = [], []
        for mf, tr in zip(ds.features, ds.times):
            rows = feature_rows(mf, self.task)
            ok = np.isfinite(tr)
            X.append(rows[ok])
            T.append(np.log(tr[ok]))
        return np.concatenate(X).astype(np.float32), np.concatenate(T).astype(np.float32)

    def fit(self, ds: Dataset, epochs: int = 300, batch: int = 64, lr: float = 1e-3, seed: int = 0):
        """Adam on the MSE of the normalised log times; the batch grows with
        the data (at most ~128 steps an epoch) so large searches train in
        seconds."""
        import torch
        X, T = self._rows(ds)
        batch = max(batch, len(T) // 128)
        self.mu, self.sd = float(T.mean()), float(T.std() + 1e-6)
        Xt = torch.tensor(X, device="cuda")
        Tt = torch.tensor(((T - self.mu) / self.sd)[:, None], device="cuda")
        hists = [net.train(Xt, Tt, epochs=epochs, batch=batch, lr=lr, seed=seed + m)
                 for m, net in enumerate(self.nets)]
        return [float(np.mean(h)) for h in zip(*hists)]

    def predict(self, mf: np.ndarray) -> np.ndarray:
        """Predicted seconds of every config (the members' mean)."""
        import torch
        rows = torch.tensor(feature_rows(mf, self.task), device="cuda")
        y = np.mean([net.forward(rows).cpu().numpy()[:, 0] for net in self.nets], axis=0)
        return np.exp(y * self.sd + self.mu)

    def choose(self, mf: np.ndarray, feasible: Optional[np.ndarray] = None) -> int:
        pred = self.predict(mf)
        if feasible is not None:
            pred = np.where(feasible, pred, np.inf)
        return int(np.argmin(pred))


def held_out(count: int, task: str = "mpk") -> np.ndarray:
    """The evaluation split: every k-th row is held out, k = count // 200
    (at least 2) for the MPK task, so that 200 of the configured 2,000
    matrices (and at least 200 of any set of 400 or more) are held out, and
    every fifth row for the coloring task."""
    k = max(2, count // 200) if task == "mpk" else 5
    return np.arange(count) % k == k - 1


def best_fixed_config(ds: Dataset) -> int:
    """The single config with the lowest mean regret over a dataset (the
    method without the model)."""
    best, arg = np.inf, 0
    for ci in range(len(TASKS[ds.task].configs)):
        r = [regret(t, ci) if np.isfinite(t[ci]) else 10.0 for t in ds.times]
        if np.mean(r) < best:
            best, arg = float(np.mean(r)), ci
    return arg


def evaluate(model: CostModel, ds: Dataset, fixed: int) -> dict:
    rm, rf, rs = [], [], []
    for mf, tr in zip(ds.features, ds.times):
        feas = np.isfinite(tr)
        c = model.choose(mf, feas)
        rm.append(regret(tr, c))
        rf.append(regret(tr, fixed) if feas[fixed] else regret(tr, 0))
        # MLP then time its two best guesses (a short search)
        pred = np.where(feas, model.predict(mf), np.inf)
        top = np.argsort(pred)[:2]
        rs.append(regret(tr, top[np.argmin(tr[top])]))
    rm, rf, rs = map(np.asarray, (rm, rf, rs))
    return {"matrices": len(rm), "mlp_mean_regret": float(rm.mean()), "mlp_median_regret": float(np.median(rm)),
            "mlp_p90_regret": float(np.percentile(rm, 90)), "mlp_within_10pct": float((rm <= 0.10).mean()),
            "mlp_top2_mean_regret": float(rs.mean()), "mlp_top2_within_10pct": float((rs <= 0.10).mean()),
            "fixed_config": list(TASKS[ds.task].configs[fixed]), "fixed_mean_regret": float(rf.mean()),
            "fixed_within_10pct": float((rf <= 0.10).mean())}


class Tuner:
    """Parameter choice for one task (A^8 x by default): the trained cost
    model when one is given, else (and on request) the exhaustive search."""

    def __init__(self, model: Optional[CostModel] = None, task: Task = None):
        self.model = model
        self.task = model.task if model is not None else (task or MPK_TASK)

    def choose(self, A, mode: str = "auto"):
        """Returns (config, info); config is (p, cacheMB) for the MPK task and
        (threads, efficiency) for the sweep task. mode: 'mlp', 'search' or
        'auto' (the model when loaded, else the search)."""
        if mode == "search" or (mode == "auto" and self.model is None):
            t0 = time.perf_counter()
            tr = self.task.search(A)
            return self.task.configs[int(np.argmin(tr))], {"how": "search", "seconds": time.perf_counter() - t0}
        t0 = time.perf_counter()
        c = self.model.choose(matrix_features(A))
        return self.task.configs[c], {"how": "mlp", "seconds": time.perf_counter() - t0}


def _lower_priority():
    """Pool initializer: matrix generation yields the host to the search
    process, whose launch timing it would otherwise perturb."""
    import os
    try:
        os.nice(19)
    except OSError:
        pass


def _generate(job):
    i, seed, nmin, nmax = job
    fam, A = dataset_matrix(i, seed, nmin, nmax)
    return i, fam, A, matrix_features(A)


def build_dataset(count: int, seed: int = 0, nmin: int = 50_000, nmax: int = 2_000_000, log=None,
                  out=None, save_every: int = 10, task: str = "mpk", start: int = 0, workers: int = 0,
                  max_seconds: float = math.inf) -> Dataset:
    """Search matrices start .. start+count-1 of the seeded set for one task;
    with `out`, the partial dataset is saved every `save_every` matrices.
    workers > 0 makes the matrices and their features in that many spawned
    processes, at most 2 x workers ahead of the GPU search; the search stops
    after the matrix that passes max_seconds."""
    import collections
    import itertools

    feats, times, fams, sizes, idx = [], [], [], [], []
    tk = TASKS[task]
    jobs = [(i, seed, nmin, nmax) for i in range(start, start + count)]

    def ds():
        return Dataset(np.stack(feats), np.stack(times), np.asarray(fams), np.asarray(sizes, np.int64), task,
                       np.asarray(idx, np.int64))

    def made():
        if workers <= 0:
            for j in jobs:
                yield _generate(j)
            return
        import multiprocessing as mp
        with mp.get_context("spawn").Pool(workers, initializer=_lower_priority) as pool:
            it = iter(jobs)
            pending = collections.deque(pool.apply_async(_generate, (j,)) for j in itertools.islice(it, 2 * workers))
            while pending:
                r = pending.popleft().get()
                nxt = next(it, None)
                if nxt is not None:
                    pending.append(pool.apply_async(_generate, (nxt,)))
                yield r

    t_start = time.perf_counter()
    for i, fam, A, mf in made():
        t0 = time.perf_counter()
        try:
            tr = tk.search(A)
        except Exception as exc:  # one failing matrix is recorded as infeasible, the search goes on
            if log:
                log(f"{i} {fam} n={A.n}: search failed: {exc}")
            tr = np.full(len(tk.configs), np.inf)
        feats.append(mf)
        times.append(tr)
        fams.append(fam)
        sizes.append((A.n, A.nnz))
        idx.append(i)
        if log:
            log(f"{i} {fam} n={A.n} nnz={A.nnz} best={tk.configs[int(np.argmin(tr))]} "
                f"{time.perf_counter() - t0:.1f}s")
        if out is not None and len(times) % save_every == 0:
            ds().save(out)
        if time.perf_counter() - t_start > max_seconds:
            break
    d = ds()
    if out is not None:
        d.save(out)
    return d


def main(argv=None):
    import argparse
    ap = argparse.ArgumentParser(description="parameter search for the MPK tuner (needs a GPU)")
    ap.add_argument("command", choices=["search", "merge"],
                    help="search: time every config of --count matrices; merge: concatenate saved datasets "
                         "(the inputs) of one task into --out")
    ap.add_argument("inputs", nargs="*")
    ap.add_argument("--count", type=int, default=2000)
    ap.add_argument("--start", type=int, default=0, help="index of the first matrix of the seeded set")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--nmin", type=int, default=50_000)
    ap.add_argument("--nmax", type=int, default=2_000_000)
    ap.add_argument("--task", choices=sorted(TASKS), default="mpk")
    ap.add_argument("--workers", type=int, default=0, help="processes that make the matrices ahead of the search")
    ap.add_argument("--max-seconds", type=float, default=math.inf, help="stop the search after this long")
    ap.add_argument("--out", required=True)
    a = ap.parse_intermixed_args(argv)
    if a.command == "merge":
        parts = [Dataset.load(p) for p in a.inputs]
        assert parts and len({d.task for d in parts}) == 1, "merge needs datasets of one task"
        Dataset(np.concatenate([d.features for d in parts]), np.concatenate([d.times for d in parts]),
                np.concatenate([d.families for d in parts]), np.concatenate([d.sizes for d in parts]),
                parts[0].task, np.concatenate([d.index for d in parts])).save(a.out)
        return
    build_dataset(a.count, a.seed, a.nmin, a.nmax, log=lambda s: print(s, flush=True), out=a.out, task=a.task,
                  start=a.start, workers=a.workers, max_seconds=a.max_seconds)


if __name__ == "__main__":
    main()
