"""GPU engine parity: structure bit-exact against the reference (golden
fixtures), numerics against the C oracle. Needs a GB300."""
import numpy as np
import pytest

from cases import COLOR_CASES, POWER_CASES, POWER_FLAT_CASES, arr_digest, digest, key_color, key_power, key_power_flat
from oracle import oracle as orc
from oracle.refpy import parse_zone_tree
from race_gb300 import matgen

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from race_gb300 import _lib  # noqa: E402
from race_gb300 import interface as ri  # noqa: E402


def _rel_err(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.mark.parametrize("m,d,t", COLOR_CASES)
def test_coloring_matches_reference(golden, mats, m, d, t):
    A = mats[m]
    k = key_color(m, d, t)
    assert str(golden[k + "__digest"]) == digest(A)
    rc = ri.Interface(A.n, t, d, A.row_ptr, A.col, symm_hint=True)
    assert rc.RACEColor() == 0
    np.testing.assert_array_equal(rc.getPerm(), golden[k + "__perm"])
    inv = rc.getInvPerm()
    np.testing.assert_array_equal(inv[rc.getPerm()], np.arange(A.n))
    np.testing.assert_array_equal(rc.getZoneTreeFlat(), golden[k + "__tree"])
    assert rc.getNumThreads() == int(golden[k + "__threads"])
    assert rc.getEfficiency() == float(golden[k + "__eff"])
    assert rc.getMaxStageDepth() == int(golden[k + "__stage"])


@pytest.mark.parametrize("m,p,c", POWER_CASES)
def test_power_partition_matches_reference(golden, mats, m, p, c):
    A = mats[m]
    k = key_power(m, p, c)
    rc = ri.Interface(A.n, 1, ri.POWER, A.row_ptr, A.col, symm_hint=True)
    assert rc.RACEColor(p, c) == 0
    np.testing.assert_array_equal(rc.getPerm(), golden[k + "__perm"])
    np.testing.assert_array_equal(rc.getPowerGroups(), golden[k + "__lp"])


@pytest.mark.parametrize("m,p,c", POWER_FLAT_CASES)
def test_power_partition_without_recursion(golden, mats, m, p, c):
    """Consecutive levels over the cache cut-off: the reference recurses into
    the hopeless region by default (tests/test_zz_recursion.py); with
    max_recursion_stages = 0 both partition without recursion, and the
    permutation, the level groups and the MPK agree."""
    A = mats[m]
    k = key_power_flat(m, p, c)
    assert str(golden[k + "__digest"]) == digest(A)
    assert int(golden[k + "__default_leaves"]) > 1 and int(golden[k + "__leaves"]) == 1
    rc = ri.Interface(A.n, 1, ri.POWER, A.row_ptr, A.col, symm_hint=True, params={"max_recursion_stages": 0})
    assert rc.RACEColor(p, c) == 0
    np.testing.assert_array_equal(rc.getPerm(), golden[k + "__perm"])
    np.testing.assert_array_equal(rc.getPowerGroups(), golden[k + "__lp"])
    _check_mpk(rc, A, p)


def _upload(P, dtype=torch.float64):
    return ri.DeviceCsr.from_csr(P, "cuda", dtype)


SWEEP_CASES = [("lap7_16", 2, 16), ("lap7_32", 2, 1024), ("lap7_32", 1, 256), ("aniso9_100x80", 1, 16),
               ("plaw_3k", 1, 32), ("band_5k", 2, 32), ("st27_16", 2, 128), ("aniso5_120x90", 2, 48),
               ("islands_330", 2, 16), ("islands_330", 1, 8), ("tiny_1", 1, 4)]


@pytest.mark.parametrize("m,d,t", SWEEP_CASES)
def test_sweeps_match_oracle(golden, mats, m, d, t):
    """Every built-in kernel through the persistent colored sweep, forward
    and reverse, against the oracle's sequential walk of the reference zone
    tree. FP64, wave executor: identical bit for bit."""
    A = mats[m]
    k = key_color(m, d, t)
    rc = ri.Interface(A.n, t, d, A.row_ptr, A.col, symm_hint=True)
    assert rc.RACEColor() == 0
    rc.setSweepMode(ri.SWEEP_WAVE)
    perm, inv = rc.getPerm(), rc.getInvPerm()
    P = A.permuted(perm, inv)
    U = P.upper()
    nodes = parse_zone_tree(golden[k + "__tree"])
    x0 = matgen.uniform_vector(A.n, 0)
    b0 = matgen.uniform_vector(A.n, 1)
    kernels = [(ri.GS, P, False), (ri.GS, P, True), (ri.SPMV, P, False)]
    if d == 2:
        kernels += [(ri.SYMMSPMV, U, False), (ri.KACZ, P, False), (ri.KACZ, P, True), (ri.SPMTV, P, False)]
    for kern, mat, rev in kernels:
        zero_b = kern in (ri.SPMV, ri.SYMMSPMV, ri.SPMTV)
        xr, br = x0.copy(), (np.zeros(A.n) if zero_b else b0.copy())
        orc.exec_tree(nodes, 2, golden[k + "__serial"], kern, rev, mat, xr, br)
        dm = _upload(mat)
        x = torch.tensor(x0, device="cuda")
        b = torch.zeros(A.n, dtype=torch.float64, device="cuda") if zero_b else torch.tensor(b0, device="cuda")
        fid = rc.registerFunction(kern, ri.Operands(dm, x, b))
        assert fid >= 0
        assert rc.executeFunction(fid, rev) == 0
        torch.cuda.synchronize()
        out_ref = br if zero_b else xr
        out = (b if zero_b else x).cpu().numpy()
        if np.diff(mat.row_ptr).max() <= 512:
            assert np.array_equal(out, out_ref), (kern, rev, _rel_err(out, out_ref))
        else:  # rows above 512 entries run with a warp reduction
            assert _rel_err(out, out_ref) <= 1e-12, (kern, rev, _rel_err(out, out_ref))


@pytest.mark.parametrize("m", ["plaw_20k", "band_5k"])
def test_wave_sweep_layouts_agree(mats, monkeypatch, m):
    """Wave-mode sweeps hand a row to one thread or to a warp by its length
    (RACE_GPU_SWEEP_MIDROW) and read thread rows from the SELL copy of the
    wave plan or from the caller's CRS (RACE_GPU_SWEEP_SELL); every
    combination keeps each row's operation order, so GS, Kaczmarz and SpMV
    give the same vectors bit for bit, with FP64 and FP32 values."""
    A = mats[m]
    x0 = matgen.uniform_vector(A.n, 0)
    b0 = matgen.uniform_vector(A.n, 1)
    ref = {}
    for sell in ("1", "0"):
        for mid in ("0", "8", "32", "-1"):
            monkeypatch.setenv("RACE_GPU_SWEEP_SELL", sell)
            monkeypatch.setenv("RACE_GPU_SWEEP_MIDROW", mid)
            rc = ri.Interface(A.n, 64, ri.TWO, A.row_ptr, A.col, symm_hint=True)
            assert rc.RACEColor() == 0
            rc.setSweepMode(ri.SWEEP_WAVE)
            P = A.permuted(rc.getPerm(), rc.getInvPerm())
            for vdt in (torch.float64, torch.float32):
                xdt = torch.float64 if vdt == torch.float64 else torch.float32
                for kern in (ri.GS, ri.KACZ, ri.SPMV):
                    x = torch.tensor(x0, dtype=xdt, device="cuda")
                    b = torch.zeros(A.n, dtype=xdt, device="cuda") if kern == ri.SPMV else \
                        torch.tensor(b0, dtype=xdt, device="cuda")
                    fid = rc.registerFunction(kern, ri.Operands(_upload(P, vdt), x, b))
                    assert fid >= 0 and rc.getSweepInfo(fid)["wave_mode"]
                    assert rc.executeFunction(fid) == 0
                    if kern != ri.SPMV:
                        assert rc.executeFunction(fid, True) == 0
                    out = (b if kern == ri.SPMV else x).cpu().numpy()
                    key = (str(vdt), kern)
                    if key not in ref:
                        ref[key] = out
                    assert np.array_equal(out, ref[key]), (sell, mid, key)
            rc.close()


@pytest.mark.parametrize("m,d,t", [("lap7_32", 2, 1024), ("aniso9_100x80", 1, 16), ("plaw_3k", 1, 32)])
def test_leaf_mode_sweeps(golden, mats, m, d, t):
    """Leaf mode (warp per RACE leaf, shuffle reductions): within 1e-12 of
    the oracle's sequential walk."""
    A = mats[m]
    k = key_color(m, d, t)
    rc = ri.Interface(A.n, t, d, A.row_ptr, A.col, symm_hint=True)
    assert rc.RACEColor() == 0
    rc.setSweepMode(ri.SWEEP_LEAF)
    P = A.permuted(rc.getPerm(), rc.getInvPerm())
    nodes = parse_zone_tree(golden[k + "__tree"])
    x0 = matgen.uniform_vector(A.n, 0)
    b0 = matgen.uniform_vector(A.n, 1)
    kernels = [(ri.GS, P, False), (ri.GS, P, True)]
    if d == 2:
        kernels += [(ri.SYMMSPMV, P.upper(), False), (ri.KACZ, P, False)]
    for kern, mat, rev in kernels:
        zero_b = kern == ri.SYMMSPMV
        xr, br = x0.copy(), (np.zeros(A.n) if zero_b else b0.copy())
        orc.exec_tree(nodes, 2, golden[k + "__serial"], kern, rev, mat, xr, br)
        x = torch.tensor(x0, device="cuda")
        b = torch.zeros(A.n, dtype=torch.float64, device="cuda") if zero_b else torch.tensor(b0, device="cuda")
        fid = rc.registerFunction(kern, ri.Operands(_upload(mat), x, b))
        assert not rc.getSweepInfo(fid, rev)["wave_mode"]
        assert rc.executeFunction(fid, rev) == 0
        out = (b if zero_b else x).cpu().numpy()
        assert _rel_err(out, br if zero_b else xr) <= 1e-12


def test_long_rows_use_warp_path(mats):
    """A power-law graph has hub rows above 512 entries (warp reduction) and
    above 2048 (segments summed by all warps of the grid in waves of their
    own): every kernel's sweep stays within 1e-12 of the oracle's sequential
    walk of the engine's phases, and repeated runs are identical."""
    A = matgen.powerlaw_chung_lu(20000, seed=2)
    assert np.diff(A.row_ptr).max() > 2048
    rc = ri.Interface(A.n, 64, ri.TWO, A.row_ptr, A.col, symm_hint=True)
    assert rc.RACEColor() == 0
    rc.setSweepMode(ri.SWEEP_WAVE)
    P = A.permuted(rc.getPerm(), rc.getInvPerm())
    U = P.upper()
    pp, lo, hi = rc.getPhases(False)
    x0 = matgen.uniform_vector(A.n, 0)
    b0 = matgen.uniform_vector(A.n, 1)
    okern = {ri.GS: orc.K_GS, ri.KACZ: orc.K_KACZ, ri.SPMV: orc.K_SPMV, ri.SYMMSPMV: orc.K_SYMMSPMV,
             ri.SPMTV: orc.K_SPMTV}
    for kern, mat in [(ri.GS, P), (ri.KACZ, P), (ri.SPMV, P), (ri.SYMMSPMV, U), (ri.SPMTV, P)]:
        zero_b = kern in (ri.SPMV, ri.SYMMSPMV, ri.SPMTV)
        xr, br = x0.copy(), (np.zeros(A.n) if zero_b else b0.copy())
        for ph in range(len(pp) - 1):
            for leaf in range(pp[ph], pp[ph + 1]):
                orc.run_kernel(okern[kern], int(lo[leaf]), int(hi[leaf]), mat, xr, br)
        outs = []
        for _ in range(2):
            x = torch.tensor(x0, device="cuda")
            b = torch.zeros(A.n, dtype=torch.float64, device="cuda") if zero_b else torch.tensor(b0, device="cuda")
            fid = rc.registerFunction(kern, ri.Operands(_upload(mat), x, b))
            assert fid >= 0 and rc.executeFunction(fid) == 0
            outs.append((b if zero_b else x).cpu().numpy())
        assert _rel_err(outs[0], br if zero_b else xr) <= 1e-12, kern
        assert np.array_equal(outs[0], outs[1]), kern


def test_symmgs_refinement_power_law():
    """Refinement on a power-law system (hub rows: the FP64 residual runs
    them as warp-summed segments): FP32 inner sweeps reach 1e-10, and two
    solves give identical results (fixed reduction orders)."""
    sp = pytest.importorskip("scipy.sparse")
    A = matgen.powerlaw_chung_lu(20000, seed=2)
    rc = ri.Interface(A.n, 64, ri.TWO, A.row_ptr, A.col, symm_hint=True)
    assert rc.RACEColor() == 0
    P = A.permuted(rc.getPerm(), rc.getInvPerm())
    S = sp.csr_matrix((P.val, P.col, P.row_ptr), shape=(A.n, A.n))
    m64 = _upload(P)
    bh = S @ np.ones(A.n)
    b = torch.tensor(bh, device="cuda")
    d = torch.zeros(A.n, dtype=torch.float32, device="cuda")
    r = torch.zeros(A.n, dtype=torch.float32, device="cuda")
    fid = rc.registerFunction(ri.GS, ri.Operands(_upload(P, torch.float32), d, r))
    xs = []
    for _ in range(2):
        x = torch.zeros(A.n, dtype=torch.float64, device="cuda")
        its, rel = rc.symmGsIr(fid, m64, b, x, tol=1e-10, maxIter=300, sweeps=1)
        assert rel <= 1e-10, (its, rel)
        xs.append(x.cpu().numpy())
    assert np.linalg.norm(bh - S @ xs[0]) <= 1.01e-10 * np.linalg.norm(bh)
    assert np.array_equal(xs[0], xs[1])


@pytest.mark.parametrize("vdtype,tol", [(torch.float32, 1e-5), (torch.bfloat16, 3e-2)])
def test_reduced_precision_sweeps(golden, mats, vdtype, tol):
    """GS and KACZ with FP32/BF16 values and FP32 vectors against the FP64
    oracle (error of the storage precision, reported by the tolerance)."""
    m, d, t = "lap7_16", 2, 16
    A = mats[m]
    k = key_color(m, d, t)
    rc = ri.Interface(A.n, t, d, A.row_ptr, A.col, symm_hint=True)
    assert rc.RACEColor() == 0
    P = A.permuted(rc.getPerm(), rc.getInvPerm())
    nodes = parse_zone_tree(golden[k + "__tree"])
    x0 = matgen.uniform_vector(A.n, 0)
    b0 = matgen.uniform_vector(A.n, 1)
    for kern, rev in [(ri.GS, False), (ri.GS, True), (ri.KACZ, False)]:
        xr, br = x0.copy(), b0.copy()
        orc.exec_tree(nodes, 2, golden[k + "__serial"], kern, rev, P, xr, br)
        x = torch.tensor(x0, dtype=torch.float32, device="cuda")
        b = torch.tensor(b0, dtype=torch.float32, device="cuda")
        fid = rc.registerFunction(kern, ri.Operands(_upload(P, vdtype), x, b))
        assert fid >= 0 and rc.executeFunction(fid, rev) == 0
        assert _rel_err(x.double().cpu().numpy(), xr) < tol


@pytest.mark.parametrize("inner", ["f64", "f32", "bf16"])
def test_symmgs_iterative_refinement(mats, inner):
    """Symmetric GS with FP64 iterative refinement reaches 1e-10 relative
    residual with FP64, FP32 or BF16 inner sweeps; the solution agrees with
    the FP64-inner solve."""
    sp = pytest.importorskip("scipy.sparse")
    A = matgen.stencil3d_27pt(20)
    rc = ri.Interface(A.n, 512, ri.ONE, A.row_ptr, A.col, symm_hint=True)
    assert rc.RACEColor() == 0
    P = A.permuted(rc.getPerm(), rc.getInvPerm())
    S = sp.csr_matrix((P.val, P.col, P.row_ptr), shape=(A.n, A.n))
    m64 = _upload(P)
    bh = S @ np.ones(A.n)  # b = A 1, the reference drivers' convention (colorSymmGS.cpp:147-188)
    b = torch.tensor(bh, device="cuda")
    x = torch.zeros(A.n, dtype=torch.float64, device="cuda")
    vdt = {"f64": torch.float64, "f32": torch.float32, "bf16": torch.bfloat16}[inner]
    xdt = torch.float64 if inner == "f64" else torch.float32
    d = torch.zeros(A.n, dtype=xdt, device="cuda")
    r = torch.zeros(A.n, dtype=xdt, device="cuda")
    fid = rc.registerFunction(ri.GS, ri.Operands(_upload(P, vdt), d, r))
    assert fid >= 0
    its, rel = rc.symmGsIr(fid, m64, b, x, tol=1e-10, maxIter=200, sweeps=1)
    assert rel <= 1e-10, (its, rel)
    xh = x.cpu().numpy()
    assert np.linalg.norm(bh - S @ xh) <= 1.01e-10 * np.linalg.norm(bh)
    assert np.max(np.abs(xh - 1.0)) < 1e-8  # the exact solution is all ones


HUB_ROW_LEN = 256  # rows longer than this are summed by a warp (mpk.cu kHubRowLen)


@pytest.mark.parametrize("m,p,c", POWER_CASES)
def test_mpk_fp64_bit_exact(golden, mats, m, p, c):
    """Level-blocked MPK in FP64 equals p sequential fma SpMVs bit for bit;
    with rows above HUB_ROW_LEN entries (warp-summed) every power stays
    within 1e-12 relative, and the other rows of the first power are still
    exact."""
    A = mats[m]
    rc = ri.Interface(A.n, 1, ri.POWER, A.row_ptr, A.col, symm_hint=True)
    assert rc.RACEColor(p, c) == 0
    _check_mpk(rc, A, p)


def _check_mpk(rc, A, p):
    perm, inv = rc.getPerm(), rc.getInvPerm()
    P = A.permuted(perm, inv)
    x0 = matgen.uniform_vector(A.n, 0)
    Y = orc.mpk_plain(P, x0, p)
    dm = _upload(P)
    x = torch.zeros((p + 1) * A.n, dtype=torch.float64, device="cuda")
    x[: A.n] = torch.tensor(x0, device="cuda")
    fid = rc.registerFunction(ri.MPK, ri.Operands(dm, x), power=p)
    assert fid >= 0
    lens = np.diff(P.row_ptr)
    hubs = lens > HUB_ROW_LEN
    for _ in range(2):  # repeated calls reuse the plan
        assert rc.executeFunction(fid) == 0
        torch.cuda.synchronize()
        got = x.cpu().numpy().reshape(p + 1, A.n)
        if not hubs.any():
            np.testing.assert_array_equal(got, Y)
        else:
            np.testing.assert_array_equal(got[1][~hubs], Y[1][~hubs])
            for kk in range(1, p + 1):
                assert _rel_err(got[kk], Y[kk]) <= 1e-12


def test_mpk_full_size_c2(golden):
    """128^3 27-point stencil, p=8 (the benchmark's configuration):
    permutation and level groups equal the reference's (digests), and all 8
    powers of the GPU MPK equal the CPU oracle's p sequential fma SpMVs
    (orc.mpk_plain, the reference's MAT_SPMV_KERNEL order) bit for bit, on
    repeated calls and at the benchmark's cache budget too."""
    A = matgen.stencil3d_27pt(128)
    k = key_power("st27_128", 8, 100e6)
    assert str(golden[k + "__digest"]) == digest(A)
    rc = ri.Interface(A.n, 1, ri.POWER, A.row_ptr, A.col, symm_hint=True)
    assert rc.RACEColor(8, 100e6) == 0
    perm, inv = rc.getPerm(), rc.getInvPerm()
    assert arr_digest(perm) == str(golden[k + "__perm_digest"])
    np.testing.assert_array_equal(rc.getPowerGroups(), golden[k + "__lp"])
    P = A.permuted(perm, inv)
    dm = _upload(P)
    x = torch.zeros(9 * A.n, dtype=torch.float64, device="cuda")
    x[: A.n] = torch.tensor(matgen.uniform_vector(A.n, 0), device="cuda")
    fid = rc.registerFunction(ri.MPK, ri.Operands(dm, x), power=8)
    y = torch.zeros_like(x)
    y[: A.n] = x[: A.n]
    for kk in range(1, 9):
        rc.spmv_plain(dm, y[(kk - 1) * A.n: kk * A.n], y[kk * A.n:(kk + 1) * A.n])
    x0 = matgen.uniform_vector(A.n, 0)
    ref = torch.tensor(orc.mpk_plain(P, x0, 8).reshape(-1), device="cuda")
    assert torch.equal(y, ref)  # the GPU plain chain, pinned to the oracle
    for rep in range(3):  # repeated calls: stale cached values would show up as mismatches
        x[A.n:] = 0
        assert rc.executeFunction(fid) == 0
        torch.cuda.synchronize()
        assert torch.equal(x, ref), rep
    # the benchmark's cache budget (300 MB): other level groups, same powers
    rc3 = ri.Interface(A.n, 1, ri.POWER, A.row_ptr, A.col, symm_hint=True)
    assert rc3.RACEColor(8, 300e6) == 0
    np.testing.assert_array_equal(rc3.getPerm(), perm)
    x3 = torch.zeros_like(x)
    x3[: A.n] = x[: A.n]
    f3 = rc3.registerFunction(ri.MPK, ri.Operands(dm, x3), power=8)
    assert rc3.executeFunction(f3) == 0
    torch.cuda.synchronize()
    assert torch.equal(x3, ref)
    # the same p SpMVs without level blocking on the registered layout
    x[A.n:] = 0
    for kk in range(8):
        rc.spmvPowerLayout(fid, kk)
    torch.cuda.synchronize()
    assert torch.equal(x, y)


def _col_layout(P, gp, window, hub=HUB_ROW_LEN):
    """Restatement of the MPK's column layout choice: chunks of <= 32 rows
    inside the level groups gp, each chunk's columns (hub rows excluded)
    covered greedily by windows of `window` rows; chunks needing more than
    four windows keep 32-bit columns, and the plan stays 32-bit when those
    chunks hold more than half of the SELL slots. Returns (chunks, chunks
    with 32-bit columns, column bits)."""
    lens = np.diff(P.row_ptr)
    cr = [0]
    for g in range(len(gp) - 1):
        for r in range(gp[g], gp[g + 1], 32):
            cr.append(min(gp[g + 1], r + 32))
    slots = wide = wide_slots = 0
    for c in range(len(cr) - 1):
        rows = [r for r in range(cr[c], cr[c + 1]) if lens[r] <= hub]
        L = int(max((lens[r] for r in rows), default=0))
        slots += 32 * L
        v = np.unique(np.concatenate([P.col[P.row_ptr[r]:P.row_ptr[r + 1]] for r in rows] or [np.zeros(0, int)]))
        i = w = 0
        while i < len(v):
            w += 1
            i = int(np.searchsorted(v, v[i] + window, "left"))
        if w > 4:
            wide += 1
            wide_slots += 32 * L
    return (len(cr) - 1, 0, 32) if 2 * wide_slots > slots else (len(cr) - 1, wide, 16)


def test_mpk_column_layouts(monkeypatch):
    """The 16-bit column layout (per chunk four window bases, per entry a
    2-bit window and a 14-bit offset) and the 32-bit one give identical
    powers: FP64 equal to the oracle's p sequential fma SpMVs, FP32 equal to
    the 32-bit layout's, for the MPK and the plain SpMV on the layout. Small
    windows force plans that mix 16-bit chunks with chunks that keep 32-bit
    columns (window 512 on the 40^3 stencil) and plans that fall back to 32
    bits (window 64); the reported layout matches the restatement."""
    A = matgen.stencil3d_27pt(40)
    p = 4
    x0 = matgen.uniform_vector(A.n, 0)
    ref32 = None
    mixed = False
    for col16, window in [("0", None), ("1", None), ("1", "512"), ("1", "64")]:
        monkeypatch.setenv("RACE_GPU_MPK_COL16", col16)
        if window:
            monkeypatch.setenv("RACE_GPU_MPK_COL_WINDOW", window)
        else:
            monkeypatch.delenv("RACE_GPU_MPK_COL_WINDOW", raising=False)
        rc = ri.Interface(A.n, 1, ri.POWER, A.row_ptr, A.col, symm_hint=True)
        assert rc.RACEColor(p, 2e6) == 0
        P = A.permuted(rc.getPerm(), rc.getInvPerm())
        Y = orc.mpk_plain(P, x0, p)
        outs = []
        for dtype in (torch.float64, torch.float32):
            x = torch.zeros((p + 1) * A.n, dtype=torch.float64, device="cuda")
            x[: A.n] = torch.tensor(x0, device="cuda")
            fid = rc.registerFunction(ri.MPK, ri.Operands(_upload(P, dtype), x), power=p)
            assert fid >= 0
            lay = rc.getMpkLayout(fid)
            want = (lay["chunks"], 0, 32) if col16 == "0" else _col_layout(P, rc.getPowerGroups(),
                                                                             int(window or 16384))
            assert (lay["chunks"], lay["wide_chunks"], lay["col_bits"]) == want, (col16, window, lay)
            mixed |= lay["col_bits"] == 16 and 0 < lay["wide_chunks"] < lay["chunks"]
            assert rc.executeFunction(fid) == 0
            got = x.clone()
            x[A.n:] = 0
            for kk in range(p):
                rc.spmvPowerLayout(fid, kk)
            torch.cuda.synchronize()
            assert torch.equal(x, got)  # plain SpMVs on the layout == MPK
            outs.append(got.cpu().numpy().reshape(p + 1, A.n))
        np.testing.assert_array_equal(outs[0], Y)
        if ref32 is None:
            ref32 = outs[1]
        np.testing.assert_array_equal(outs[1], ref32)
    assert mixed


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32, torch.bfloat16])
def test_mpk_schedules_agree(mats, dtype):
    """The wavefront kernel, the p plain sweeps and the automatic choice
    (timed at the first call) give bit-identical powers; FP64 equals the
    oracle's p sequential fma SpMVs. The layout query reports the schedule
    that ran."""
    A = mats["st27_24"]
    p = 5
    rc = ri.Interface(A.n, 1, ri.POWER, A.row_ptr, A.col, symm_hint=True)
    assert rc.RACEColor(p, 2e6) == 0
    P = A.permuted(rc.getPerm(), rc.getInvPerm())
    x0 = matgen.uniform_vector(A.n, 3)
    x = torch.zeros((p + 1) * A.n, dtype=torch.float64, device="cuda")
    x[: A.n] = torch.tensor(x0, device="cuda")
    fid = rc.registerFunction(ri.MPK, ri.Operands(_upload(P, dtype), x), power=p)
    assert rc.getMpkLayout(fid)["schedule"] == "auto"
    outs = {}
    for sc in ("wavefront", "sweeps", "auto"):
        rc.setMpkSchedule(fid, sc)
        x[A.n:] = 0
        for _ in range(2):
            assert rc.executeFunction(fid) == 0
        outs[sc] = x.cpu().numpy()
    assert rc.getMpkLayout(fid)["schedule"] in ("wavefront", "sweeps")
    np.testing.assert_array_equal(outs["wavefront"], outs["sweeps"])
    np.testing.assert_array_equal(outs["auto"], outs["sweeps"])
    if dtype == torch.float64:
        np.testing.assert_array_equal(outs["auto"].reshape(p + 1, A.n), orc.mpk_plain(P, x0, p))
    with pytest.raises(_lib.RaceError):
        rc.setMpkSchedule(fid + 1, "sweeps")


@pytest.mark.parametrize("dtype,tol", [(torch.float32, 1e-5), (torch.bfloat16, 5e-2)])
def test_mpk_reduced_precision_error(mats, dtype, tol):
    """FP32/BF16 value storage with FP32 accumulation: error against the FP64
    oracle stays within the storage precision (reported, not hidden)."""
    A = mats["st27_24"]
    p = 4
    rc = ri.Interface(A.n, 1, ri.POWER, A.row_ptr, A.col, symm_hint=True)
    assert rc.RACEColor(p, 2e6) == 0
    P = A.permuted(rc.getPerm(), rc.getInvPerm())
    x0 = matgen.uniform_vector(A.n, 0)
    Y = orc.mpk_plain(P, x0, p)
    dm = _upload(P, dtype)
    x = torch.zeros((p + 1) * A.n, dtype=torch.float64, device="cuda")
    x[: A.n] = torch.tensor(x0, device="cuda")
    fid = rc.registerFunction(ri.MPK, ri.Operands(dm, x), power=p)
    assert rc.executeFunction(fid) == 0
    out = x.cpu().numpy().reshape(p + 1, A.n)
    for kk in range(1, p + 1):
        assert _rel_err(out[kk], Y[kk]) < tol


def test_error_codes(mats):
    A = mats["lap7_16"]
    rc = ri.Interface(A.n, 8, ri.TWO, A.row_ptr, A.col, symm_hint=True)
    assert rc.RACEColor(4, 1e6) == 1  # power partition needs dist POWER (interface.cpp:218-221)
    assert rc.RACEColor() == 0
    dm = _upload(A)
    x = torch.zeros((5) * A.n, dtype=torch.float64, device="cuda")
    assert rc.registerFunction(ri.MPK, ri.Operands(dm, x), power=4) == 1
    assert rc.executeFunction(12345) == 1
    rp = ri.Interface(A.n, 1, ri.POWER, A.row_ptr, A.col, symm_hint=True)
    assert rp.RACEColor() == 1  # coloring needs dist ONE/TWO (interface.cpp:264-267)
    assert rp.RACEColor(4, 1e6, 2.0, "N", 0) == 1  # sub power < 1
    assert rp.RACEColor(4, 1e6) == 0
    dmp = _upload(A.permuted(rp.getPerm(), rp.getInvPerm()))
    xp = torch.zeros(257 * A.n, dtype=torch.float64, device="cuda")
    assert rp.registerFunction(ri.MPK, ri.Operands(dmp, xp), power=256) == 1  # powers are stored in 8 bits
    fp = rp.registerFunction(ri.MPK, ri.Operands(dmp, xp), power=4)
    assert rp.getPower(fp) == 4  # a real function id, not an error code
    with pytest.raises(Exception):
        rp.setPower(fp, 300)
    assert rp.getPower(fp) == 4
    d1 = ri.Interface(A.n, 8, ri.ONE, A.row_ptr, A.col, symm_hint=True)
    assert d1.RACEColor() == 0
    b = torch.zeros(A.n, dtype=torch.float64, device="cuda")
    assert d1.registerFunction(ri.KACZ, ri.Operands(dm, x[: A.n], b)) == 3  # needs distance-2


def test_unsymmetric_pattern_is_symmetrised(mats):
    """symm_hint=False on a matrix with one-sided entries: the traversal graph
    gains the transposed pattern (graph.cpp:47-142) and levels match the
    oracle on the symmetrised pattern."""
    A = mats["band_5k"]
    rows = np.repeat(np.arange(A.n), np.diff(A.row_ptr))
    keep = (A.col >= rows) | (np.arange(A.nnz) % 3 == 0)  # drop two thirds of the lower triangle
    counts = np.bincount(rows[keep], minlength=A.n)
    rp = np.concatenate([[0], np.cumsum(counts)]).astype(np.int32)
    B = matgen.Csr(A.n, rp, A.col[keep].astype(np.int32), A.val[keep])
    rc = ri.Interface(B.n, 1, ri.POWER, B.row_ptr, B.col, symm_hint=False)
    assert rc.RACEColor(4, 3e5) == 0
    # oracle on the explicitly symmetrised pattern
    r2 = np.concatenate([rows[keep], B.col]); c2 = np.concatenate([B.col, rows[keep]])
    S = matgen._assemble(B.n, r2[r2 != c2], c2[r2 != c2].astype(np.int32), np.ones((r2 != c2).sum()), np.ones(B.n), "s")
    key = np.unique(S.col.astype(np.int64) + np.repeat(np.arange(S.n), np.diff(S.row_ptr)).astype(np.int64) * S.n)
    rr, cc = key // S.n, key % S.n
    off = rr != cc
    S2 = matgen._assemble(S.n, rr[off], cc[off].astype(np.int32), np.ones(off.sum()), np.ones(S.n), "s2")
    perm, _, _, _, _ = orc.traverse(S2, 3, 0, S2.n)
    np.testing.assert_array_equal(rc.getPerm(), perm)


def test_empty_rows_spmv_and_mpk():
    """Rows without any entry (not even a diagonal) are undefined input for
    the reference (its graph build reads each row's first entry,
    src/graph_SoA.cpp:121-130), so there is no golden; the engine must still
    color and permute such a matrix and give empty rows a zero result in
    SpMV and every power of the MPK."""
    A = matgen.chain_with_empty_rows(300, (0, 150, 299))
    for d, t in ((1, 8), (2, 16)):
        rc = ri.Interface(A.n, t, d, A.row_ptr, A.col, symm_hint=True)
        assert rc.RACEColor() == 0
        perm, inv = rc.getPerm(), rc.getInvPerm()
        assert np.array_equal(np.sort(perm), np.arange(A.n))
        P = A.permuted(perm, inv)
        x0 = matgen.uniform_vector(A.n, 0)
        x = torch.tensor(x0, device="cuda")
        b = torch.zeros(A.n, dtype=torch.float64, device="cuda")
        fid = rc.registerFunction(ri.SPMV, ri.Operands(_upload(P), x, b))
        assert rc.executeFunction(fid) == 0
        ref = np.zeros(A.n)
        orc.run_kernel(orc.K_SPMV, 0, A.n, P, x0.copy(), ref)
        np.testing.assert_array_equal(b.cpu().numpy(), ref)
    p = 4
    rc = ri.Interface(A.n, 1, ri.POWER, A.row_ptr, A.col, symm_hint=True)
    assert rc.RACEColor(p, 1e4) == 0
    P = A.permuted(rc.getPerm(), rc.getInvPerm())
    x0 = matgen.uniform_vector(A.n, 0)
    x = torch.zeros((p + 1) * A.n, dtype=torch.float64, device="cuda")
    x[: A.n] = torch.tensor(x0, device="cuda")
    fid = rc.registerFunction(ri.MPK, ri.Operands(_upload(P), x), power=p)
    assert rc.executeFunction(fid) == 0
    np.testing.assert_array_equal(x.cpu().numpy().reshape(p + 1, A.n), orc.mpk_plain(P, x0, p))


def test_medium_rows_warp_path_is_bit_exact():
    """Rows of 33..512 entries run as one warp that keeps the sequential
    order (gathers 32 entries at a time, folds them in order): every kernel's
    forward sweep stays identical bit for bit to the sequential walk of the
    engine's phases."""
    A = matgen.banded_scrambled(4000, 48, seed=5, fill=1.0)
    lens = np.diff(A.row_ptr)
    assert lens.max() <= 512 and (lens > 32).mean() > 0.9
    rc = ri.Interface(A.n, 64, ri.TWO, A.row_ptr, A.col, symm_hint=True)
    assert rc.RACEColor() == 0
    rc.setSweepMode(ri.SWEEP_WAVE)
    P = A.permuted(rc.getPerm(), rc.getInvPerm())
    U = P.upper()
    pp, lo, hi = rc.getPhases(False)
    x0 = matgen.uniform_vector(A.n, 0)
    b0 = matgen.uniform_vector(A.n, 1)
    for kern, mat in [(ri.GS, P), (ri.KACZ, P), (ri.SPMV, P), (ri.SYMMSPMV, U), (ri.SPMTV, P)]:
        zero_b = kern in (ri.SPMV, ri.SYMMSPMV, ri.SPMTV)
        xr, br = x0.copy(), (np.zeros(A.n) if zero_b else b0.copy())
        okern = {ri.GS: orc.K_GS, ri.KACZ: orc.K_KACZ, ri.SPMV: orc.K_SPMV, ri.SYMMSPMV: orc.K_SYMMSPMV,
                 ri.SPMTV: orc.K_SPMTV}[kern]
        for ph in range(len(pp) - 1):
            for leaf in range(pp[ph], pp[ph + 1]):
                orc.run_kernel(okern, int(lo[leaf]), int(hi[leaf]), mat, xr, br)
        x = torch.tensor(x0, device="cuda")
        b = torch.zeros(A.n, dtype=torch.float64, device="cuda") if zero_b else torch.tensor(b0, device="cuda")
        fid = rc.registerFunction(kern, ri.Operands(_upload(mat), x, b))
        assert fid >= 0 and rc.getSweepInfo(fid)["wave_mode"]
        assert rc.executeFunction(fid) == 0
        out = (b if zero_b else x).cpu().numpy()
        assert np.array_equal(out, br if zero_b else xr), (kern, _rel_err(out, br if zero_b else xr))


def test_tune_function_on_registered_mpk(mats):
    """tuneFunction (src/interface.cpp:605-647) on a registered matrix power:
    it times powers 1..p, keeps the fastest in its tuned map (a second call
    returns it without timing again) and leaves the function at that power;
    the results are then the oracle's first `best` powers, and after
    setPower back to p all p powers again."""
    import time
    A, p = mats["st27_24"], 8
    rc = ri.Interface(A.n, 1, ri.POWER, A.row_ptr, A.col, symm_hint=True)
    assert rc.RACEColor(p, 2e6) == 0
    P = A.permuted(rc.getPerm(), rc.getInvPerm())
    x0 = matgen.uniform_vector(A.n, 0)
    ref = orc.mpk_plain(P, x0, p)
    x = torch.zeros((p + 1) * A.n, dtype=torch.float64, device="cuda")
    x[: A.n] = torch.tensor(x0, device="cuda")
    fid = rc.registerFunction(ri.MPK, ri.Operands(_upload(P), x), power=p)
    best = rc.tuneFunction(fid)
    assert 1 <= best <= p and rc.getPower(fid) == best
    t0 = time.perf_counter()
    assert rc.tuneFunction(fid) == best  # from the tuned map
    assert time.perf_counter() - t0 < 0.1
    x[A.n:] = 0
    assert rc.executeFunction(fid) == 0
    got = x.cpu().numpy().reshape(p + 1, A.n)
    np.testing.assert_array_equal(got[: best + 1], ref[: best + 1])
    assert not got[best + 1:].any()
    rc.setPower(fid, p)
    assert rc.executeFunction(fid) == 0
    np.testing.assert_array_equal(x.cpu().numpy().reshape(p + 1, A.n), ref)
