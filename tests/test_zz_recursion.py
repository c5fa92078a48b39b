"""MPK partitions with hopeless regions on the GPU: the engine's
RACEColor(p, cacheSize) gives the reference's level groups and, after its
recursion into the hopeless groups (one stage by default, deeper with
max_recursion_stages or a list of cut-offs), the reference's permutation;
the MPK on that partition equals p sequential SpMVs bit for bit. (The host
parts are checked on the CPU in test_host_logic.py; this file runs last
among the GPU tests.)"""
import numpy as np
import pytest

from cases import (DEEP_CASES, HOPELESS_CASES, POWER_EDGE_CASES, POWER_SAFETY_CASES, digest, key_deep, key_hopeless,
                   key_power_edge, key_power_safety)
from oracle import oracle as orc
from race_gb300 import matgen

torch = pytest.importorskip("torch")

from race_gb300 import interface as ri  # noqa: E402

HUB_ROW_LEN = 256  # rows longer than this are summed by a warp (mpk.cu kHubRowLen)


@pytest.mark.gpu
@pytest.mark.parametrize("m,p,c", HOPELESS_CASES)
def test_default_partition_with_hopeless_regions(golden, mats, m, p, c):
    A = mats[m]
    k = key_hopeless(m, p, c)
    assert str(golden[k + "__digest"]) == digest(A)
    rc = ri.Interface(A.n, 1, ri.POWER, A.row_ptr, A.col, symm_hint=True)
    assert rc.RACEColor(p, c) == 0
    np.testing.assert_array_equal(rc.getPowerGroups(), golden[k + "__lp"])
    tree = rc.getPowerTree()
    assert int(tree[0]) == int(golden[k + "__leaves"])  # the root and one leaf per hopeless group
    ng = int(tree[5])
    np.testing.assert_array_equal(tree[7 + ng:8 + ng + int(tree[7 + ng])][1:], golden[k + "__hid"])
    _check_mpk(rc, A, p, golden[k + "__perm"])


def _check_mpk(rc, A, p, want_perm):
    """The engine's permutation is want_perm and its MPK on the permuted
    matrix gives the oracle's p sequential SpMVs (bit for bit without hub
    rows, which a warp sums in another order)."""
    perm, inv = rc.getPerm(), rc.getInvPerm()
    np.testing.assert_array_equal(perm, want_perm)
    np.testing.assert_array_equal(inv[perm], np.arange(A.n))
    P = A.permuted(perm, inv)
    x0 = matgen.uniform_vector(A.n, 0)
    Y = orc.mpk_plain(P, x0, p)
    x = torch.zeros((p + 1) * A.n, dtype=torch.float64, device="cuda")
    x[: A.n] = torch.tensor(x0, device="cuda")
    fid = rc.registerFunction(ri.MPK, ri.Operands(ri.DeviceCsr.from_csr(P), x), power=p)
    assert fid >= 0
    assert rc.executeFunction(fid) == 0
    got = x.cpu().numpy().reshape(p + 1, A.n)
    hubs = np.diff(P.row_ptr) > HUB_ROW_LEN
    if not hubs.any():
        np.testing.assert_array_equal(got, Y)
    else:
        for kk in range(1, p + 1):
            assert np.max(np.abs(got[kk] - Y[kk])) <= 1e-12 * np.max(np.abs(Y[kk]))


@pytest.mark.gpu
@pytest.mark.parametrize("m,p,c,stages,cuts", DEEP_CASES)
def test_deep_recursion(golden, mats, m, p, c, stages, cuts):
    """Recursion deeper than one stage (RACE_MAX_RECURSION_STAGES and the
    per-stage RACE_CACHE_VIOLATION_CUTOFF list, given as params): the
    reference's stage-0 groups and its permutation after every stage."""
    A = mats[m]
    k = key_deep(m, p, c, stages, cuts)
    params = {"cache_violation_cutoffs": list(cuts)}
    if stages >= 0:
        params["max_recursion_stages"] = stages
    rc = ri.Interface(A.n, 1, ri.POWER, A.row_ptr, A.col, symm_hint=True, params=params)
    assert rc.RACEColor(p, c) == 0
    tree = golden[k + "__tree"]
    ng = int(tree[5])  # the root leaf: lo, hi, stage, parent, groups, lp
    np.testing.assert_array_equal(rc.getPowerGroups(), tree[6:7 + ng])
    np.testing.assert_array_equal(rc.getPowerTree(), tree)  # every leaf of every stage
    _check_mpk(rc, A, p, golden[k + "__perm"])


@pytest.mark.gpu
@pytest.mark.parametrize("m,p,c", POWER_EDGE_CASES)
def test_partition_at_edge_parameters(golden, mats, m, p, c):
    """Power 1 and high powers, a budget that holds the whole matrix, tiny
    budgets, a one-row matrix: the reference's groups and permutation, and
    the MPK on them."""
    A = mats[m]
    k = key_power_edge(m, p, c)
    assert str(golden[k + "__digest"]) == digest(A)
    rc = ri.Interface(A.n, 1, ri.POWER, A.row_ptr, A.col, symm_hint=True)
    assert rc.RACEColor(p, c) == 0
    tree = golden[k + "__tree"]
    np.testing.assert_array_equal(rc.getPowerGroups(), tree[6:7 + int(tree[5])])
    np.testing.assert_array_equal(rc.getPowerTree(), tree)
    _check_mpk(rc, A, p, golden[k + "__perm"])


@pytest.mark.gpu
@pytest.mark.parametrize("m,p,c,sf", POWER_SAFETY_CASES)
def test_partition_with_other_safety_factors(golden, mats, m, p, c, sf):
    """RACEColor(p, cacheSize, safetyFactor): the engine's permutation and
    level groups equal the reference's."""
    A = mats[m]
    k = key_power_safety(m, p, c, sf)
    rc = ri.Interface(A.n, 1, ri.POWER, A.row_ptr, A.col, symm_hint=True)
    assert rc.RACEColor(p, c, safetyFactor=sf) == 0
    np.testing.assert_array_equal(rc.getPerm(), golden[k + "__perm"])
    np.testing.assert_array_equal(rc.getPowerGroups(), golden[k + "__lp"])


@pytest.mark.gpu
@pytest.mark.parametrize("split", [4, 2, 3])
def test_split_wavefront_order(mats, monkeypatch, split):
    """RACE_GPU_MPK_SPLIT: the issue order in power segments inside one
    launch still gives p sequential SpMVs bit for bit."""
    monkeypatch.setenv("RACE_GPU_MPK_SPLIT", str(split))
    A = mats["st27_24"]
    p = 8
    rc = ri.Interface(A.n, 1, ri.POWER, A.row_ptr, A.col, symm_hint=True)
    assert rc.RACEColor(p, 2e6) == 0
    P = A.permuted(rc.getPerm(), rc.getInvPerm())
    x0 = matgen.uniform_vector(A.n, 0)
    x = torch.zeros((p + 1) * A.n, dtype=torch.float64, device="cuda")
    x[: A.n] = torch.tensor(x0, device="cuda")
    fid = rc.registerFunction(ri.MPK, ri.Operands(ri.DeviceCsr.from_csr(P), x), power=p)
    assert fid >= 0 and rc.executeFunction(fid) == 0
    np.testing.assert_array_equal(x.cpu().numpy().reshape(p + 1, A.n), orc.mpk_plain(P, x0, p))
