"""Matrix-power cases on the GPU (after the other GPU tests): triangular
partitions (mtxType L / U) and their MPK through device functors and the
built-in kernel, and sub-powers. Their host parts are checked on the CPU
(test_oracle.py, test_device_functors.py)."""
import numpy as np
import pytest

from cases import POWER_TRI_CASES, digest, key_power_tri, triangle
from oracle import oracle as orc
from race_gb300 import matgen

torch = pytest.importorskip("torch")

from race_gb300 import interface as ri  # noqa: E402

HUB_ROW_LEN = 256  # rows longer than this are summed by a warp (mpk.cu kHubRowLen)


@pytest.mark.gpu
@pytest.mark.parametrize("m,tri,p,c", POWER_TRI_CASES)
def test_triangular_partition_and_functor_mpk(golden, mats, fnlib, m, tri, p, c):
    """The engine's L / U partition equals the reference's, and the MPK body
    as a device power functor on the permuted triangle (lower triangular in
    RACE's order) equals p sequential SpMVs bit for bit."""
    T = triangle(mats[m], tri)
    k = key_power_tri(m, tri, p, c)
    assert str(golden[k + "__digest"]) == digest(T)
    rc = ri.Interface(T.n, 1, ri.POWER, T.row_ptr, T.col, symm_hint=True)
    assert rc.RACEColor(p, c, mtxType=tri) == 0
    np.testing.assert_array_equal(rc.getPerm(), golden[k + "__perm"])
    np.testing.assert_array_equal(rc.getPowerGroups(), golden[k + "__lp"])
    P = T.permuted(rc.getPerm(), rc.getInvPerm())
    dm = ri.DeviceCsr.from_csr(P)
    x0 = matgen.uniform_vector(T.n, 0)
    Y = orc.mpk_plain(P, x0, p)
    x = torch.zeros((p + 1) * T.n, dtype=torch.float64, device="cuda")
    x[: T.n] = torch.tensor(x0, device="cuda")
    assert fnlib.fn_mpk(rc._h, dm.row_ptr.data_ptr(), dm.col.data_ptr(), dm.val.data_ptr(), x.data_ptr(), T.n,
                        p, 32) == 0
    np.testing.assert_array_equal(x.cpu().numpy().reshape(p + 1, T.n), Y)


@pytest.mark.gpu
@pytest.mark.parametrize("m,tri,p,c", POWER_TRI_CASES)
def test_triangular_builtin_mpk(golden, mats, m, tri, p, c):
    """The built-in MPK on a triangular partition (run one launch per
    wavefront step, since a row may read any earlier group) equals p
    sequential SpMVs bit for bit."""
    T = triangle(mats[m], tri)
    rc = ri.Interface(T.n, 1, ri.POWER, T.row_ptr, T.col, symm_hint=True)
    assert rc.RACEColor(p, c, mtxType=tri) == 0
    np.testing.assert_array_equal(rc.getPerm(), golden[key_power_tri(m, tri, p, c) + "__perm"])
    P = T.permuted(rc.getPerm(), rc.getInvPerm())
    x0 = matgen.uniform_vector(T.n, 0)
    x = torch.zeros((p + 1) * T.n, dtype=torch.float64, device="cuda")
    x[: T.n] = torch.tensor(x0, device="cuda")
    fid = rc.registerFunction(ri.MPK, ri.Operands(ri.DeviceCsr.from_csr(P), x), power=p)
    assert fid >= 0 and rc.executeFunction(fid) == 0
    got, Y = x.cpu().numpy().reshape(p + 1, T.n), orc.mpk_plain(P, x0, p)
    if np.diff(P.row_ptr).max() <= HUB_ROW_LEN:
        np.testing.assert_array_equal(got, Y)
    else:  # hub rows are summed by a warp, in another order
        for kk in range(1, p + 1):
            assert np.max(np.abs(got[kk] - Y[kk])) <= 1e-12 * np.max(np.abs(Y[kk]))


@pytest.mark.gpu
@pytest.mark.parametrize("m,p,sub,c", [("st27_24", 4, 2, 2e6), ("aniso5_120x90", 2, 3, 5e5)])
def test_subpower_functor_visits_every_row_in_order(mats, fnlib, m, p, sub, c):
    """registerFunction(f, args, power, subPower) counterpart: every row is
    called once per (pow, subPow), in order (the reference example's
    counting kernel)."""
    A = mats[m]
    rc = ri.Interface(A.n, 1, ri.POWER, A.row_ptr, A.col, symm_hint=True)
    assert rc.RACEColor(p, c, highestSubPower=sub) == 0
    x = torch.zeros(A.n, dtype=torch.float64, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    assert fnlib.fn_count_subpower(rc._h, x.data_ptr(), p, sub, err.data_ptr()) == 0
    assert int(err.item()) == 0
    assert bool((x == p * sub).all())


@pytest.mark.gpu
def test_set_power_and_subpower_rebuild_the_schedule(mats, fnlib):
    """Interface::setPower / setSubPower on a device power function: after
    both, every row is called once per (pow, subPow), in order."""
    A = mats["st27_24"]
    p, sub = 4, 2
    rc = ri.Interface(A.n, 1, ri.POWER, A.row_ptr, A.col, symm_hint=True)
    assert rc.RACEColor(p, 2e6, highestSubPower=sub) == 0
    x = torch.zeros(A.n, dtype=torch.float64, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    assert fnlib.fn_count_after_set(rc._h, x.data_ptr(), p, sub, err.data_ptr()) == 0
    assert int(err.item()) == 0
    assert bool((x == p * sub).all())


@pytest.mark.gpu
@pytest.mark.parametrize("m,p,c", [("st27_24", 8, 2e6), ("plaw_3k", 4, 2e3), ("band_5k", 8, 3000)])
def test_check_power_coverage(mats, fnlib, m, p, c):
    """Interface::checkPowerCoverage: the reference's counting kernel over
    the engine's level groups (also with hopeless regions) finds every row
    computed once per power, in order."""
    import ctypes as C
    A = mats[m]
    rc = ri.Interface(A.n, 1, ri.POWER, A.row_ptr, A.col, symm_hint=True)
    assert rc.RACEColor(p, c) == 0
    errors = C.c_int(-2)
    assert fnlib.fn_check_coverage(rc._h, C.byref(errors)) == 0
    assert errors.value == 0


@pytest.mark.gpu
def test_builtin_functions_have_subpower_one(mats):
    """Interface::setSubPower / getSubPower on a built-in function: sub-power
    1 only (the built-in kernels have no sub-steps)."""
    A = mats["lap7_16"]
    rc = ri.Interface(A.n, 1, ri.POWER, A.row_ptr, A.col, symm_hint=True)
    assert rc.RACEColor(2, 1e6) == 0
    P = A.permuted(rc.getPerm(), rc.getInvPerm())
    x = torch.zeros(3 * A.n, dtype=torch.float64, device="cuda")
    fid = rc.registerFunction(ri.MPK, ri.Operands(ri.DeviceCsr.from_csr(P), x), power=2)
    assert fid >= 0
    assert rc.getSubPower(fid) == 1
    rc.setSubPower(fid, 1)
    with pytest.raises(RuntimeError):
        rc.setSubPower(fid, 2)
    assert rc.executeFunction(fid) == 0
