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


def _registered(A, power, cache):
    """The registered RACE_K_MPK path's result and the operands."""
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
    return P, dm, x0, ref, groups


@pytest.mark.parametrize("name,power,cache", [("st27_24", 8, 2e6), ("st27_40", 4, 8e6), ("plaw_30k", 4, 4e6)])
def test_noalloc_matches_registered_mpk(name, power, cache):
    """Bit for bit equal to the registered path on two calls in a row. The
    power-law matrix has rows of more than 256 entries, which both paths sum
    with the whole warp in the same order."""
    if name == "plaw_30k":
        A = matgen.powerlaw_chung_lu(30000, seed=2)
        assert np.diff(A.row_ptr).max() > 256
    else:
        A = matgen.stencil3d_27pt(int(name.split("_")[1]))
    P, dm, x0, ref, groups = _registered(A, power, cache)
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


def test_noalloc_refuses_a_matrix_out_of_level_order_and_recovers():
    """A matrix whose columns reach beyond the neighbouring level groups
    (here: the unpermuted stencil with the permuted matrix's groups) is
    refused with RACE_ERR_INVALID_ARG before anything waits; group offsets
    whose device copy differs from the host copy are refused the same way;
    the next valid call is bit for bit right again (flags and status reset)."""
    A = matgen.stencil3d_27pt(24)
    power = 4
    P, dm, x0, ref, groups = _registered(A, power, 2e6)
    groups_dev = torch.tensor(groups, device="cuda")
    raw = ri.DeviceCsr.from_csr(A)
    x = torch.zeros_like(ref)
    x[: A.n] = x0
    assert _call(raw, groups_dev, groups, power, x) == _lib.RACE_ERR_INVALID_ARG
    # device copies that differ from the host copy: decreasing offsets, and
    # a last offset other than n (the kernel would index rows past the end)
    dev_dec = groups.copy()
    dev_dec[1], dev_dec[2] = dev_dec[2], dev_dec[1]
    assert _call(dm, torch.tensor(dev_dec, device="cuda"), groups, power, x) == _lib.RACE_ERR_INVALID_ARG
    dev_end = groups.copy()
    dev_end[-1] = A.n + 32
    assert _call(dm, torch.tensor(dev_end, device="cuda"), groups, power, x) == _lib.RACE_ERR_INVALID_ARG
    # decreasing host offsets
    dec = groups.copy()
    dec[1], dec[2] = dec[2], dec[1]
    assert _call(dm, groups_dev, dec, power, x) == _lib.RACE_ERR_INVALID_ARG
    for call in range(2):
        x = torch.full_like(ref, float("nan"))
        x[: A.n] = x0
        assert _call(dm, groups_dev, groups, power, x) == 0, call
        torch.cuda.synchronize()
        assert torch.equal(x, ref), call
