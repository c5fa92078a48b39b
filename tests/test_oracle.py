"""The C restatement oracle against golden data produced by the reference
(tests/golden/make_golden.py). CPU only."""
import numpy as np
import pytest

from cases import (COLOR_CASES, EXEC_CASES, POWER_CASES, POWER_FLAT_CASES, POWER_TRI_CASES, TRAVERSE_CASES, digest,
                   key_color, key_power, key_power_flat, key_power_tri, key_trav, triangle)
from oracle import oracle as orc
from oracle.refpy import parse_zone_tree
from race_gb300 import matgen


@pytest.mark.parametrize("m,d", TRAVERSE_CASES)
def test_traverse_matches_reference(golden, mats, m, d):
    A = mats[m]
    k = key_trav(m, d)
    assert str(golden[k + "__digest"]) == digest(A)
    perm, inv, lr, ln, _ = orc.traverse(A, d, 0, A.n)
    np.testing.assert_array_equal(perm, golden[k + "__perm"])
    np.testing.assert_array_equal(lr, golden[k + "__levelRow"])
    np.testing.assert_array_equal(ln, golden[k + "__levelNnz"])
    np.testing.assert_array_equal(inv[perm], np.arange(A.n))


def _tree(golden, k):
    from oracle.refpy import parse_zone_tree
    return parse_zone_tree(golden[k + "__tree"])


def _edge_exec_cases():
    from cases import COLOR_EDGE_EXEC, key_color_edge
    return [(m, d, t, key_color_edge(m, d, t)) for m, d, t in sorted(COLOR_EDGE_EXEC)]


@pytest.mark.parametrize("m,d,t,k", [(m, d, t, key_color(m, d, t)) for m, d, t in sorted(EXEC_CASES)]
                         + _edge_exec_cases())
def test_executor_walk_matches_reference(golden, mats, m, d, t, k):
    """The sequential zone-tree walk reproduces the reference's threaded
    executor bit for bit on its own schedule (also at the thread-count
    edges: 3, 5, 7, 13 and 1000 requested threads)."""
    A = mats[m]
    checked = 0
    perm = golden[k + "__perm"]
    inv = np.empty_like(perm); inv[perm] = np.arange(A.n, dtype=np.int32)
    P = A.permuted(perm, inv)
    U = P.upper()
    nodes = _tree(golden, k)
    x0 = matgen.uniform_vector(A.n, 0)
    b0 = matgen.uniform_vector(A.n, 1)
    for kern, name, mat, rev in [(orc.K_SYMMSPMV, "symmspmv", U, False), (orc.K_GS, "gs", P, False),
                                 (orc.K_GS, "gsrev", P, True), (orc.K_KACZ, "kacz", P, False),
                                 (orc.K_SPMV, "spmv", P, False)]:
        key = k + f"__out_{name}"
        if key not in golden:
            continue
        x = x0.copy()
        b = np.zeros(A.n) if kern in (orc.K_SPMV, orc.K_SYMMSPMV) else b0.copy()
        orc.exec_tree(nodes, 2, golden[k + "__serial"], kern, rev, mat, x, b)
        out = b if kern in (orc.K_SPMV, orc.K_SYMMSPMV) else x
        np.testing.assert_array_equal(out, golden[key], err_msg=name)
        checked += 1
    assert checked == (5 if d == 2 else 3)


@pytest.mark.parametrize("m,p,c", POWER_CASES)
def test_mpk_partition_matches_reference(golden, mats, m, p, c):
    A = mats[m]
    k = key_power(m, p, c)
    assert str(golden[k + "__digest"]) == digest(A)
    perm, inv, lr, ln, _ = orc.traverse(A, 3, 0, A.n)
    np.testing.assert_array_equal(perm, golden[k + "__perm"])
    lp = np.concatenate([[0], np.cumsum(lr)]).astype(np.int32)
    g = orc.mpk_groups(p, A.n, A.nnz, c, 2.0, 50, lp, ln)
    assert g is not None
    np.testing.assert_array_equal(g[0], golden[k + "__lp"])


@pytest.mark.parametrize("m,p,c", POWER_FLAT_CASES)
def test_mpk_flat_partition_matches_reference(golden, mats, m, p, c):
    """A hopeless region (consecutive levels over the cut-off) makes the
    single-stage grouping refuse; without recursion (cut-off disabled, as
    RACE_MAX_RECURSION_STAGES=0 does) it equals the reference's groups."""
    A = mats[m]
    k = key_power_flat(m, p, c)
    assert str(golden[k + "__digest"]) == digest(A)
    perm, inv, lr, ln, _ = orc.traverse(A, 3, 0, A.n)
    np.testing.assert_array_equal(perm, golden[k + "__perm"])
    lp = np.concatenate([[0], np.cumsum(lr)]).astype(np.int32)
    assert orc.mpk_groups(p, A.n, A.nnz, c, 2.0, 50, lp, ln) is None
    g = orc.mpk_groups(p, A.n, A.nnz, c, 2.0, 2**31 - 1, lp, ln)
    np.testing.assert_array_equal(g[0], golden[k + "__lp"])


@pytest.mark.parametrize("m,tri,p,c", POWER_TRI_CASES)
def test_mpk_triangular_partition_matches_reference(golden, mats, m, tri, p, c):
    """mtxType L / U: one row per level, forward or backward
    (traverse_GAP_graphSoA.cpp:316-335), so the permutation is the identity
    or the reversal and the single-stage grouping of the rows' non-zeros
    gives the reference's level groups."""
    T = triangle(mats[m], tri)
    k = key_power_tri(m, tri, p, c)
    assert str(golden[k + "__digest"]) == digest(T)
    rows = np.arange(T.n, dtype=np.int32)
    order = rows if tri == "L" else rows[::-1]
    np.testing.assert_array_equal(golden[k + "__perm"], order)
    lens = np.diff(T.row_ptr)[order]
    g = orc.mpk_groups(p, T.n, T.nnz, c, 2.0, 50, np.arange(T.n + 1, dtype=np.int32), lens)
    np.testing.assert_array_equal(g[0], golden[k + "__lp"])


@pytest.mark.parametrize("m,p,c", [pc for pc in POWER_CASES if pc[0] in ("st27_24", "aniso5_120x90")])
def test_mpk_output_matches_reference(golden, mats, m, p, c):
    """The reference MPK executor's output equals p sequential fma SpMVs, and
    the oracle's threaded wavefront port gives the same bits."""
    A = mats[m]
    k = key_power(m, p, c)
    perm = golden[k + "__perm"]
    inv = np.empty_like(perm); inv[perm] = np.arange(A.n, dtype=np.int32)
    P = A.permuted(perm, inv)
    x0 = matgen.uniform_vector(A.n, 0)
    Y = orc.mpk_plain(P, x0, p)
    np.testing.assert_array_equal(Y[1:], golden[k + "__out"])
    perm2, inv2, lr, ln, _ = orc.traverse(A, 3, 0, A.n)
    lp = np.concatenate([[0], np.cumsum(lr)]).astype(np.int32)
    gp, ur, dr = orc.mpk_groups(p, A.n, A.nnz, c, 2.0, 50, lp, ln)
    Z = orc.mpk_wavefront(P, x0, p, gp, ur, dr, int(__import__("os").environ.get("OMP_NUM_THREADS", "4")))
    np.testing.assert_array_equal(Z, Y)


def test_oracle_detects_planted_schedule_error(mats):
    """A schedule that drops a level group must not match: the checker can fail."""
    A = mats["st27_16"]
    x0 = matgen.uniform_vector(A.n, 0)
    perm, inv, lr, ln, _ = orc.traverse(A, 3, 0, A.n)
    P = A.permuted(perm, inv)
    lp = np.concatenate([[0], np.cumsum(lr)]).astype(np.int32)
    gp, ur, dr = orc.mpk_groups(4, A.n, A.nnz, 2e5, 2.0, 50, lp, ln)
    Y = orc.mpk_plain(P, x0, 4)
    assert len(gp) > 2
    Z = orc.mpk_wavefront(P, x0, 4, gp[:-1].copy(), ur, dr, 1)  # last group dropped
    assert not np.array_equal(Z, Y)


def test_block_mpk_oracle_is_per_column_chain(mats):
    """The block matrix power restatement equals the single-vector fma chain
    (MAT_SPMV_KERNEL, kernels.cpp:749-777) on every right-hand side."""
    from race_gb300 import matgen
    A = mats["aniso9_100x80"]
    X0 = matgen.uniform_block(A.n, 4, seed=7)
    blk = orc.mpk_block(A, X0, 3)
    for j in range(4):
        np.testing.assert_array_equal(blk[:, :, j], orc.mpk_plain(A, X0[:, j], 3))
    X32 = X0.astype(np.float32)
    blk32 = orc.mpk_block(A, X32, 3)
    assert blk32.dtype == np.float32
    np.testing.assert_allclose(blk32[3], blk[3], rtol=0, atol=1e-4 * np.abs(blk[3]).max())


def test_mlp_oracle_gradient_matches_finite_differences():
    """The tuner network's CPU gradient (oracle/mlp_ref.py) against central
    differences in float64: pins the oracle the GPU kernels are checked
    against."""
    from oracle import mlp_ref
    dims = (5, 7, 2, 2)
    rng = np.random.Generator(np.random.PCG64(4))
    theta = rng.normal(0, 0.5, mlp_ref.num_params(*dims))
    X = rng.normal(size=(6, 5))
    T = rng.normal(size=(6, 2))
    loss, g = mlp_ref.loss_grad(theta, X, T, dims)
    h = 1e-6
    fd = np.zeros_like(theta)
    for i in range(theta.size):
        tp, tm = theta.copy(), theta.copy()
        tp[i] += h
        tm[i] -= h
        fd[i] = (mlp_ref.loss_grad(tp, X, T, dims)[0] - mlp_ref.loss_grad(tm, X, T, dims)[0]) / (2 * h)
    assert np.max(np.abs(fd - g)) <= 1e-6 * max(1.0, np.max(np.abs(g)))
    assert loss > 0


def test_mpk_recursion_permutation_matches_reference(golden, mats):
    """The reference's default MPK partition recurses once into every
    hopeless group (RACE_MAX_RECURSION_STAGES unset: one stage past the
    cut-off list, matrixPowerRecursive.cpp:50-60). Its permutation is the
    stage-0 BFS permutation followed, per hopeless group h of the level
    groups lp, by a BFS of the group's rows from its first row through the
    boundary groups h-w..h+w (w = ceil(p/2)-1, matrixPowerRecursive.cpp:
    199-298), each region then sorted by level. The oracle restates this and
    must give the reference's permutation."""
    import math

    from cases import HOPELESS_CASES, key_hopeless
    for m, p, c in HOPELESS_CASES:
        A = mats[m]
        k = key_hopeless(m, p, c)
        assert int(golden[k + "__leaves"]) == 1 + len(golden[k + "__hid"])  # one recursion stage
        tp, ti, lr, ln, _ = orc.traverse(A, 3, 0, A.n)
        lp = golden[k + "__lp"]
        w = math.ceil(p / 2) - 1
        for h in golden[k + "__hid"]:
            regions = [(int(lp[h + r]), int(lp[h + r + 1])) for r in range(-w, w + 1)
                       if r != 0 and lp[h + r + 1] > lp[h + r]]
            tp, ti, _, _, _ = orc.traverse_boundary(A, int(lp[h]), int(lp[h + 1]), regions, tp, ti)
        np.testing.assert_array_equal(tp, golden[k + "__perm"], err_msg=k)


def test_reference_mpk_on_recursive_partitions_equals_spmv_chain(golden, mats):
    """On the reference's own recursive partitions (hopeless groups
    re-traversed), its MPK executor still gives p sequential SpMVs bit for
    bit, so an engine with the same permutation gives the same outputs."""
    from cases import HOPELESS_CASES, key_hopeless
    checked = 0
    for m, p, c in HOPELESS_CASES:
        k = key_hopeless(m, p, c)
        if k + "__out" not in golden:
            continue
        A = mats[m]
        perm = golden[k + "__perm"]
        inv = np.empty_like(perm)
        inv[perm] = np.arange(A.n, dtype=np.int32)
        Y = orc.mpk_plain(A.permuted(perm, inv), matgen.uniform_vector(A.n, 0), p)
        np.testing.assert_array_equal(Y[1:], golden[k + "__out"], err_msg=k)
        checked += 1
    assert checked == 2


def test_oracle_stage_partition_matches_reference(golden, mats):
    """The oracle's own stage-0 MPK partition with hopeless regions
    (orc_mpk_partition, restated from what identifyHopelessRegions and
    consolidatePartition compute) gives the reference's level groups and
    hopeless groups: partitions without hopeless regions, with them, without
    recursion (cut-off disabled) and with other safety factors."""
    from cases import HOPELESS_CASES, POWER_SAFETY_CASES, key_hopeless, key_power_safety
    cases = [((m, p, c, 2.0), key_power(m, p, c), 50, golden[key_power(m, p, c) + "__hid"][:-1])
             for m, p, c in POWER_CASES]  # -1 ends the stored list
    cases += [((m, p, c, 2.0), key_hopeless(m, p, c), 50, golden[key_hopeless(m, p, c) + "__hid"])
              for m, p, c in HOPELESS_CASES]
    cases += [((m, p, c, 2.0), key_power_flat(m, p, c), orc.INT_MAX, np.zeros(0, np.int32))
              for m, p, c in POWER_FLAT_CASES]
    cases += [((m, p, c, sf), key_power_safety(m, p, c, sf), 50, golden[key_power_safety(m, p, c, sf) + "__hid"])
              for m, p, c, sf in POWER_SAFETY_CASES]
    with_hopeless = 0
    for (m, p, c, sf), k, cutoff, want_hid in cases:
        A = mats[m]
        _, _, lr, ln, _ = orc.traverse(A, 3, 0, A.n)
        lp = np.concatenate([[0], np.cumsum(lr)]).astype(np.int32)
        gp, hid, _ = orc.mpk_partition(p, A.n, A.nnz, c, sf, cutoff, lp, ln)
        np.testing.assert_array_equal(gp, golden[k + "__lp"], err_msg=k)
        np.testing.assert_array_equal(hid, want_hid, err_msg=k)
        with_hopeless += hid.size > 0
    assert with_hopeless >= 6


def test_oracle_mpk_recursion_matches_reference(golden, mats):
    """The oracle's MPK recursion (mpk_recursive: its traversals with
    boundaries and orc_mpk_partition, depth first) gives the reference's
    whole leaf tree and permutation, for the default single stage (also at
    edge parameters) and for recursion up to three stages deep."""
    from cases import DEEP_CASES, HOPELESS_CASES, deep_stage_cutoffs, key_deep, key_hopeless
    for m, p, c, stages, cuts in DEEP_CASES:
        k = key_deep(m, p, c, stages, cuts)
        tree, tp, _ = orc.mpk_recursive(mats[m], p, c, 2.0, deep_stage_cutoffs(stages, cuts))
        np.testing.assert_array_equal(orc.flat_power_tree(tree), golden[k + "__tree"], err_msg=k)
        np.testing.assert_array_equal(tp, golden[k + "__perm"], err_msg=k)
    from cases import POWER_EDGE_CASES, key_power_edge
    for m, p, c in POWER_EDGE_CASES:
        k = key_power_edge(m, p, c)
        tree, tp, _ = orc.mpk_recursive(mats[m], p, c, 2.0, [50])
        np.testing.assert_array_equal(orc.flat_power_tree(tree), golden[k + "__tree"], err_msg=k)
        np.testing.assert_array_equal(tp, golden[k + "__perm"], err_msg=k)
    for m, p, c in HOPELESS_CASES:
        k = key_hopeless(m, p, c)
        tree, tp, _ = orc.mpk_recursive(mats[m], p, c, 2.0, [50])
        assert len(tree) == int(golden[k + "__leaves"])
        np.testing.assert_array_equal(tree[0]["lp"], golden[k + "__lp"])
        np.testing.assert_array_equal(tp, golden[k + "__perm"], err_msg=k)


def test_reference_mpk_at_edge_parameters_equals_spmv_chain(golden, mats):
    """The reference's MPK executor at edge parameters (power 1 and 16, one
    group for the whole matrix, tiny budgets with hopeless regions, a
    one-row matrix) gives p sequential SpMVs of the permuted matrix bit for
    bit (its outputs are stored as a checksum of their exact bits)."""
    from cases import POWER_EDGE_CASES, f64_digest, key_power_edge
    for m, p, c in POWER_EDGE_CASES:
        k = key_power_edge(m, p, c)
        A = mats[m]
        perm = golden[k + "__perm"]
        inv = np.empty_like(perm)
        inv[perm] = np.arange(A.n, dtype=np.int32)
        Y = orc.mpk_plain(A.permuted(perm, inv), matgen.uniform_vector(A.n, 0), p)
        assert f64_digest(Y[1:]) == str(golden[k + "__out_digest"]), k


def test_reference_mpk_on_deep_partitions_equals_spmv_chain(golden, mats):
    """With recursion deeper than one stage too, the reference's MPK executor
    (recursivePowerCallSerial over the whole leaf tree) gives p sequential
    SpMVs of the permuted matrix bit for bit."""
    from cases import DEEP_EXEC_CASES, key_deep
    for m, p, c, stages, cuts in sorted(DEEP_EXEC_CASES):
        k = key_deep(m, p, c, stages, cuts)
        A = mats[m]
        perm = golden[k + "__perm"]
        inv = np.empty_like(perm)
        inv[perm] = np.arange(A.n, dtype=np.int32)
        Y = orc.mpk_plain(A.permuted(perm, inv), matgen.uniform_vector(A.n, 0), p)
        np.testing.assert_array_equal(Y[1:], golden[k + "__out"], err_msg=k)


@pytest.mark.parametrize("m,d,t", [c for c in COLOR_CASES if c[1] == 2])
def test_validated_coloring_invariant(golden, mats, m, d, t):
    """The reference's own validation of a coloring (colorSymmSpMV.cpp:
    230-260, checkEqual in densemat.cpp:147-180): a plain SpMV, the colored
    SpMV and the colored SymmSpMV on the upper triangle agree, here within
    1e-12 of the largest entry (the SymmSpMV sums in another order)."""
    A = mats[m]
    k = key_color(m, d, t)
    perm = golden[k + "__perm"]
    inv = np.empty_like(perm)
    inv[perm] = np.arange(A.n, dtype=np.int32)
    P = A.permuted(perm, inv)
    U = P.upper()
    x = matgen.uniform_vector(A.n, 0)
    plain = np.zeros(A.n)
    orc.run_kernel(orc.K_SPMV, 0, A.n, P, x, plain)
    nodes = parse_zone_tree(golden[k + "__tree"])
    colored, symm = np.zeros(A.n), np.zeros(A.n)
    orc.exec_tree(nodes, 2, golden[k + "__serial"], orc.K_SPMV, False, P, x.copy(), colored)
    orc.exec_tree(nodes, 2, golden[k + "__serial"], orc.K_SYMMSPMV, False, U, x.copy(), symm)
    np.testing.assert_array_equal(colored, plain)  # rows are independent: same sums
    assert np.max(np.abs(symm - plain)) <= 1e-12 * np.max(np.abs(plain))
