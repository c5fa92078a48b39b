"""Coloring variants on the GPU, against the reference: distance-2 coloring
with RACE::THREE_BLOCK (permutation, zone tree, thread count, and bit-exact
sweeps reproducing the reference executor's outputs), coloring from an
initial permutation, of unsymmetric patterns and balancing rows. (Their host parts, the load balancer, the level
recursion and the phase semantics, are checked on the CPU in
test_host_logic.py; this file runs after the other GPU tests.)"""
import numpy as np
import pytest

from cases import (COLOR3_CASES, COLOR_EDGE_CASES, COLOR_INIT_CASES, COLOR_ROW_CASES, COLOR_UNSYM_CASES, digest,
                   key_color3, key_color_edge, key_color_init, key_color_row, key_color_unsym, triangle)
from race_gb300 import matgen

torch = pytest.importorskip("torch")

from race_gb300 import interface as ri  # noqa: E402


@pytest.mark.gpu
@pytest.mark.parametrize("m,t", COLOR3_CASES)
def test_three_block_coloring_and_sweeps(golden, mats, m, t):
    A = mats[m]
    k = key_color3(m, t)
    assert str(golden[k + "__digest"]) == digest(A)
    rc = ri.Interface(A.n, t, ri.TWO, A.row_ptr, A.col, symm_hint=True, d2Type=ri.THREE_BLOCK)
    assert rc.RACEColor() == 0
    np.testing.assert_array_equal(rc.getPerm(), golden[k + "__perm"])
    np.testing.assert_array_equal(rc.getZoneTreeFlat(), golden[k + "__tree"])
    assert rc.getNumThreads() == int(golden[k + "__threads"])
    assert rc.getEfficiency() == float(golden[k + "__eff"])
    rc.setSweepMode(ri.SWEEP_WAVE)
    perm, inv = rc.getPerm(), rc.getInvPerm()
    P = A.permuted(perm, inv)
    U = P.upper()
    x0 = matgen.uniform_vector(A.n, 0)
    b0 = matgen.uniform_vector(A.n, 1)
    for kern, name, mat, rev in [(ri.SYMMSPMV, "symmspmv", U, False), (ri.GS, "gs", P, False),
                                 (ri.GS, "gsrev", P, True), (ri.KACZ, "kacz", P, False),
                                 (ri.SPMTV, "spmtv", P, False)]:
        scatter = kern in (ri.SYMMSPMV, ri.SPMTV)
        dm = ri.DeviceCsr.from_csr(mat, "cuda", torch.float64)
        x = torch.tensor(x0, device="cuda")
        b = torch.zeros(A.n, dtype=torch.float64, device="cuda") if scatter else torch.tensor(b0, device="cuda")
        fid = rc.registerFunction(kern, ri.Operands(dm, x, b))
        assert fid >= 0
        assert rc.executeFunction(fid, rev) == 0
        torch.cuda.synchronize()
        out = (b if scatter else x).cpu().numpy()
        ref = golden[k + f"__out_{name}"]
        if np.diff(mat.row_ptr).max() <= 512:
            np.testing.assert_array_equal(out, ref, err_msg=name)
        else:  # rows above 512 entries run with a warp reduction
            assert np.max(np.abs(out - ref)) <= 1e-12 * np.max(np.abs(ref)), name


@pytest.mark.gpu
@pytest.mark.parametrize("m,d,t", COLOR_INIT_CASES)
def test_coloring_from_an_initial_permutation(golden, mats, m, d, t):
    """Interface(..., initPerm, initInvPerm): the coloring starts from the
    caller's permutation, and the permutation, zone tree and thread count
    equal the reference's."""
    A = mats[m]
    k = key_color_init(m, d, t)
    ip0 = golden[k + "__init"]
    inv0 = np.empty_like(ip0)
    inv0[ip0] = np.arange(A.n, dtype=np.int32)
    rc = ri.Interface(A.n, t, d, A.row_ptr, A.col, symm_hint=True, initPerm=ip0, initInvPerm=inv0)
    assert rc.RACEColor() == 0
    np.testing.assert_array_equal(rc.getPerm(), golden[k + "__perm"])
    np.testing.assert_array_equal(rc.getZoneTreeFlat(), golden[k + "__tree"])
    assert rc.getNumThreads() == int(golden[k + "__threads"])
    assert rc.getEfficiency() == float(golden[k + "__eff"])


@pytest.mark.gpu
@pytest.mark.parametrize("m,tri,d,t", COLOR_UNSYM_CASES)
def test_coloring_of_unsymmetric_patterns(golden, mats, m, tri, d, t):
    """symm_hint false on a pattern that is not symmetric: the engine adds
    the missing transposed entries on the GPU and colors like the
    reference."""
    T = triangle(mats[m], tri)
    k = key_color_unsym(m, tri, d, t)
    rc = ri.Interface(T.n, t, d, T.row_ptr, T.col, symm_hint=False)
    assert rc.RACEColor() == 0
    np.testing.assert_array_equal(rc.getPerm(), golden[k + "__perm"])
    np.testing.assert_array_equal(rc.getZoneTreeFlat(), golden[k + "__tree"])
    assert rc.getNumThreads() == int(golden[k + "__threads"])


@pytest.mark.gpu
@pytest.mark.parametrize("m,d,t", COLOR_ROW_CASES)
def test_coloring_balancing_rows(golden, mats, m, d, t):
    """LBTarget ROW on the GPU engine."""
    A = mats[m]
    k = key_color_row(m, d, t)
    rc = ri.Interface(A.n, t, d, A.row_ptr, A.col, symm_hint=True, lbTarget=ri.ROW)
    assert rc.RACEColor() == 0
    np.testing.assert_array_equal(rc.getPerm(), golden[k + "__perm"])
    np.testing.assert_array_equal(rc.getZoneTreeFlat(), golden[k + "__tree"])


@pytest.mark.gpu
@pytest.mark.parametrize("m,d,t", COLOR_EDGE_CASES)
def test_coloring_at_thread_count_edges(golden, mats, m, d, t):
    """One thread, odd and prime thread counts, and far more threads than
    the matrix can use: the reference's permutation, zone tree, thread
    count and efficiency, and (where stored) the reference executor's sweep
    outputs from the engine's wave mode."""
    A = mats[m]
    k = key_color_edge(m, d, t)
    assert str(golden[k + "__digest"]) == digest(A)
    rc = ri.Interface(A.n, t, d, A.row_ptr, A.col, symm_hint=True)
    assert rc.RACEColor() == 0
    np.testing.assert_array_equal(rc.getPerm(), golden[k + "__perm"])
    np.testing.assert_array_equal(rc.getZoneTreeFlat(), golden[k + "__tree"])
    assert rc.getNumThreads() == int(golden[k + "__threads"])
    assert rc.getEfficiency() == float(golden[k + "__eff"])
    if k + "__out_gs" not in golden:
        return
    rc.setSweepMode(ri.SWEEP_WAVE)
    P = A.permuted(rc.getPerm(), rc.getInvPerm())
    U = P.upper()
    x0 = matgen.uniform_vector(A.n, 0)
    b0 = matgen.uniform_vector(A.n, 1)
    for kern, name, mat, rev in [(ri.SYMMSPMV, "symmspmv", U, False), (ri.GS, "gs", P, False),
                                 (ri.GS, "gsrev", P, True), (ri.KACZ, "kacz", P, False),
                                 (ri.SPMV, "spmv", P, False)]:
        if k + f"__out_{name}" not in golden:
            continue
        zero_b = kern in (ri.SYMMSPMV, ri.SPMV)
        dm = ri.DeviceCsr.from_csr(mat, "cuda", torch.float64)
        x = torch.tensor(x0, device="cuda")
        b = torch.zeros(A.n, dtype=torch.float64, device="cuda") if zero_b else torch.tensor(b0, device="cuda")
        fid = rc.registerFunction(kern, ri.Operands(dm, x, b))
        assert fid >= 0
        assert rc.executeFunction(fid, rev) == 0
        torch.cuda.synchronize()
        out = (b if zero_b else x).cpu().numpy()
        ref = golden[k + f"__out_{name}"]
        if np.diff(mat.row_ptr).max() <= 512:
            np.testing.assert_array_equal(out, ref, err_msg=name)
        else:  # rows above 512 entries run with a warp reduction
            assert np.max(np.abs(out - ref)) <= 1e-12 * np.max(np.abs(ref)), name


@pytest.mark.gpu
@pytest.mark.parametrize("below", [1000, 1 << 30])
@pytest.mark.parametrize("m,d,t", [("plaw_3k", 2, 1000), ("lap7_32", 2, 64), ("aniso9_100x80", 1, 16)])
def test_host_traversal_of_short_ranges(golden, mats, monkeypatch, below, m, d, t):
    """RACE_GPU_HOST_TRAVERSE_BELOW: ranges shorter than the threshold are
    traversed on the host (all of them with a huge threshold); the coloring
    is the reference's all the same."""
    from cases import COLOR_EDGE_CASES
    monkeypatch.setenv("RACE_GPU_HOST_TRAVERSE_BELOW", str(below))
    A = mats[m]
    k = key_color_edge(m, d, t) if (m, d, t) in COLOR_EDGE_CASES else f"color__{m}__d{d}__t{t}"
    rc = ri.Interface(A.n, t, d, A.row_ptr, A.col, symm_hint=True)
    assert rc.RACEColor() == 0
    np.testing.assert_array_equal(rc.getPerm(), golden[k + "__perm"])
    np.testing.assert_array_equal(rc.getZoneTreeFlat(), golden[k + "__tree"])
    assert rc.getNumThreads() == int(golden[k + "__threads"])
