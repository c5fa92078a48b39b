"""race_mpk_noalloc: the matrix-power entry point that allocates no device
memory, for callers that cannot allocate when they run the kernel (memory
owned by their own pool, fixed real-time budgets, code that must not trigger
a cudaMalloc). Its scratch is a built-in device array, so it is checked here
against the registered matrix-power path through the C ABI, on two calls in
a row (the first call on a device also resolves the array's address).
Collected last on purpose: it runs after every other GPU test."""
import ctypes as C

import numpy as np
import pytest

from race_gb300 import _lib, matgen

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from race_gb300 import interface as ri  # noqa: E402


def _call(A, groups_dev, groups_host, power, x):
    return _lib.lib().race_mpk_noalloc(A.n, C.c_void_p(A.row_ptr.data_ptr()), C.c_void_p(A.col.data_ptr()),
                                       C.c_void_p(A.val.data_ptr()), C.c_void_p(groups_dev.data_ptr()),
                                       groups_host.ctypes.data, int(groups_host.size - 1), int(power),
                                       C.c_void_p(x.data_ptr()), None)


@pytest.mark.parametrize("grid,power,cache", [(24, 8, 2e6), (40, 4, 8e6)])
def test_noalloc_matches_registered_mpk(grid, power, cache):
    A = matgen.stencil3d_27pt(grid)
    rc = ri.Interface(A.n, 1, ri.POWER, A.row_ptr, A.col, symm_hint=True)
    assert rc.RACEColor(power, cache) == 0
    P = A.permuted(rc.getPerm(), rc.getInvPerm())
    dm = ri.DeviceCsr.from_csr(P)
    x0 = torch.tensor(matgen.uniform_vector(A.n, 0), device="cuda")
    ref = torch.zeros((power + 1) * A.n, dtype=torch.float64, device="cuda")
    ref[: A.n] = x0
    fid = rc.registerFunction(ri.MPK, ri.Operands(dm, ref), power=power)
    assert fid >= 0 and rc.executeFunction(fid) == 0
    groups = np.ascontiguousarray(rc.getPowerGroups(), np.int32)
    groups_dev = torch.tensor(groups, device="cuda")
    for call in range(2):
        x = torch.full(((power + 1) * A.n,), float("nan"), dtype=torch.float64, device="cuda")
        x[: A.n] = x0
        assert _call(dm, groups_dev, groups, power, x) == 0, call
        torch.cuda.synchronize()
        assert torch.equal(x, ref), call


def test_noalloc_rejects_oversized_problem():
    """A problem beyond the built-in scratch array is refused, not run."""
    n = 32 * (1 << 20)  # 2^20 chunks per power: 255 powers cannot fit in 2^22 ints
    groups = np.array([0, n], np.int32)
    groups_dev = torch.tensor(groups, device="cuda")
    dummy_i = torch.zeros(8, dtype=torch.int32, device="cuda")
    dummy_d = torch.zeros(8, dtype=torch.float64, device="cuda")
    rc = _lib.lib().race_mpk_noalloc(n, C.c_void_p(dummy_i.data_ptr()), C.c_void_p(dummy_i.data_ptr()),
                                     C.c_void_p(dummy_d.data_ptr()), C.c_void_p(groups_dev.data_ptr()),
                                     groups.ctypes.data, 1, 255, C.c_void_p(dummy_d.data_ptr()), None)
    assert rc == 1  # RACE_ERR_INVALID_ARG
