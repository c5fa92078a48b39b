"""Block matrix power over many right-hand sides and batches of matrices in
one persistent launch (and its CUDA graph), against the C oracle's fma
chains per right-hand side. Needs a GB300."""
import numpy as np
import pytest

from oracle import oracle as orc
from race_gb300 import matgen

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from race_gb300 import _lib  # noqa: E402
from race_gb300 import interface as ri  # noqa: E402


def _setup(A, p, cache):
    rc = ri.Interface(A.n, 1, ri.POWER, A.row_ptr, A.col, symm_hint=True)
    assert rc.RACEColor(p, cache) == 0
    return rc, A.permuted(rc.getPerm(), rc.getInvPerm())


def _block(rc, P, p, nrhs, X0, vdt=torch.float64, xdt=torch.float64):
    dm = ri.DeviceCsr.from_csr(P, "cuda", vdt)
    x = torch.zeros((p + 1) * P.n * nrhs, dtype=xdt, device="cuda")
    x[: P.n * nrhs] = torch.tensor(np.ascontiguousarray(X0).reshape(-1), dtype=xdt, device="cuda")
    fid = rc.registerMpkBlock(ri.Operands(dm, x), p, nrhs)
    assert fid >= 0
    return dm, x, fid


def _powers(x, p, n, nrhs):
    return x.cpu().numpy().reshape(p + 1, n, nrhs)


@pytest.mark.parametrize("nrhs", [1, 4, 16])
@pytest.mark.parametrize("m", ["aniso5_120x90", "aniso9_100x80", "st27_24"])
def test_block_mpk_fp64_bit_exact(mats, m, nrhs):
    A, p = mats[m], 4
    rc, P = _setup(A, p, 5e5)
    X0 = matgen.uniform_block(A.n, nrhs, seed=1)
    dm, x, fid = _block(rc, P, p, nrhs, X0)
    assert rc.executeFunction(fid) == 0
    ref = orc.mpk_block(P, X0, p)
    np.testing.assert_array_equal(_powers(x, p, A.n, nrhs), ref)
    # the plain p-SpMV path on the same operands gives the same bits
    x[A.n * nrhs:] = 0
    for k in range(p):
        rc.spmvPowerLayout(fid, k)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(_powers(x, p, A.n, nrhs), ref)
    # right-hand side j equals the single-vector chain
    j = nrhs - 1
    np.testing.assert_array_equal(ref[:, :, j], orc.mpk_plain(P, X0[:, j], p))


@pytest.mark.parametrize("vdt", [torch.float32, torch.bfloat16])
def test_block_mpk_reduced_precision_bit_exact(mats, vdt):
    A, p, nrhs = mats["aniso9_100x80"], 4, 8
    rc, P = _setup(A, p, 5e5)
    X0 = matgen.uniform_block(A.n, nrhs, seed=2).astype(np.float32)
    dm, x, fid = _block(rc, P, p, nrhs, X0, vdt, torch.float32)
    assert rc.executeFunction(fid) == 0
    got = _powers(x, p, A.n, nrhs)
    vals32 = dm.val.float().cpu().numpy()  # BF16 -> FP32 widening is exact
    np.testing.assert_array_equal(got, orc.mpk_block(P, X0, p, val=vals32))
    # error against the FP64 chain on the FP64 matrix
    ref64 = orc.mpk_block(P, X0.astype(np.float64), p)
    rel = np.abs(got[p] - ref64[p]).max() / np.abs(ref64[p]).max()
    assert rel < (1e-5 if vdt == torch.float32 else 2e-2)


def _make_batch(mats, p, nrhs, cache, vdt=torch.float64, xdt=torch.float64, seed=10):
    b = ri.Batch()
    members = []
    for i, A in enumerate(mats):
        rc, P = _setup(A, p, cache)
        X0 = matgen.uniform_block(A.n, nrhs, seed=seed + i)
        if xdt == torch.float32:
            X0 = X0.astype(np.float32)
        dm, x, fid = _block(rc, P, p, nrhs, X0, vdt, xdt)
        b.add(rc, fid)
        members.append((rc, P, X0, dm, x, fid))
    return b, members


def test_batch_uneven_matrices_one_launch_and_graph():
    mats = matgen.aniso2d_batch(7, seed=5, lo=20, hi=120)
    p, nrhs = 4, 16
    b, members = _make_batch(mats, p, nrhs, 2e5)
    b.execute()
    assert b.getStatus() == 0
    info = b.info()
    assert info["members"] == 7 and info["items"] == p * info["chunks"]
    for rc, P, X0, dm, x, fid in members:
        np.testing.assert_array_equal(_powers(x, p, P.n, nrhs), orc.mpk_block(P, X0, p))
    # graph replay: clear the outputs, give member 0 a new input block,
    # replay twice; every member is recomputed from its current input
    new0 = matgen.uniform_block(members[0][1].n, nrhs, seed=99)
    for i, (rc, P, X0, dm, x, fid) in enumerate(members):
        x[P.n * nrhs:] = 0
        if i == 0:
            x[: P.n * nrhs] = torch.tensor(new0.reshape(-1), device="cuda")
    b.graphLaunch()
    b.graphLaunch()
    assert b.getStatus() == 0
    for i, (rc, P, X0, dm, x, fid) in enumerate(members):
        np.testing.assert_array_equal(_powers(x, p, P.n, nrhs), orc.mpk_block(P, new0 if i == 0 else X0, p))


def test_batch_members_with_different_powers_fp32():
    mats = matgen.aniso2d_batch(3, seed=8, lo=30, hi=80)
    nrhs = 4
    b = ri.Batch()
    members = []
    for i, (A, p) in enumerate(zip(mats, (2, 5, 3))):
        rc, P = _setup(A, p, 1e5)
        X0 = matgen.uniform_block(A.n, nrhs, seed=20 + i).astype(np.float32)
        dm, x, fid = _block(rc, P, p, nrhs, X0, torch.float32, torch.float32)
        b.add(rc, fid)
        members.append((P, X0, dm, x, p))
    b.graphLaunch()
    assert b.getStatus() == 0
    for P, X0, dm, x, p in members:
        np.testing.assert_array_equal(_powers(x, p, P.n, nrhs), orc.mpk_block(P, X0, p))


def test_batch_and_block_errors(mats):
    A, p = mats["aniso5_120x90"], 3
    rc, P = _setup(A, p, 5e5)
    dm = ri.DeviceCsr.from_csr(P, "cuda", torch.float64)
    x = torch.zeros((p + 1) * A.n * 4, dtype=torch.float64, device="cuda")
    # nrhs outside {1,2,4,8,16,32}; x too small; FP64 values with FP32 x
    assert rc.registerMpkBlock(ri.Operands(dm, x), p, 3) == _lib.RACE_ERR_INVALID_ARG
    assert rc.registerMpkBlock(ri.Operands(dm, x[:10]), p, 4) == _lib.RACE_ERR_INVALID_ARG
    assert rc.registerMpkBlock(ri.Operands(dm, x.float()), p, 4) == _lib.RACE_ERR_INVALID_ARG
    # a matrix not in the engine's level order (rows scrambled)
    perm = np.random.Generator(np.random.PCG64(3)).permutation(A.n).astype(np.int32)
    inv = np.empty_like(perm)
    inv[perm] = np.arange(A.n, dtype=np.int32)
    dm_raw = ri.DeviceCsr.from_csr(A.permuted(perm, inv), "cuda", torch.float64)
    assert rc.registerMpkBlock(ri.Operands(dm_raw, x), p, 4) == _lib.RACE_ERR_INVALID_ARG
    fid64 = rc.registerMpkBlock(ri.Operands(dm, x), p, 4)
    assert fid64 >= 0
    # members must share types and nrhs
    dm32 = ri.DeviceCsr(A.n, dm.row_ptr, dm.col, dm.val.float())
    x32 = torch.zeros((p + 1) * A.n * 4, dtype=torch.float32, device="cuda")
    fid32 = rc.registerMpkBlock(ri.Operands(dm32, x32), p, 4)
    b = ri.Batch()
    b.add(rc, fid64)
    b.add(rc, fid32)
    with pytest.raises(_lib.RaceError) as ei:
        b.prepare()
    assert ei.value.code == 6  # RACE_ERR_INCOMPATIBILITY
    # only block-MPK functions can join a batch
    fid_single = rc.registerFunction(ri.MPK, ri.Operands(dm, torch.zeros((p + 1) * A.n, dtype=torch.float64,
                                                                           device="cuda")), power=p)
    assert fid_single >= 0
    with pytest.raises(_lib.RaceError):
        ri.Batch().add(rc, fid_single)


def test_batch_configured_64_matrices_against_oracle():
    """The benchmark's batch: 64 anisotropic 2D stencils (aniso2d_batch(64,
    seed 0), 10k-490k rows), 16 right-hand sides each, p = 4, FP64, RACE
    level groups at 256 MB each, all in one persistent launch replayed from
    its CUDA graph. Eight members spread over the batch (the largest among
    them) are compared with the CPU oracle's fma chains per right-hand side
    (orc.mpk_block) bit for bit; every member must equal its plain path."""
    p, nrhs = 4, 16
    mats = matgen.aniso2d_batch(64, seed=0)
    b, members = _make_batch(mats, p, nrhs, 256e6, seed=100)
    b.graphLaunch()
    assert b.getStatus() == 0
    torch.cuda.synchronize()
    largest = int(np.argmax([P.n for _, P, *_ in members]))
    pick = sorted({0, 9, 21, 33, 47, 58, 63, largest})
    for i in pick:
        rc, P, X0, dm, x, fid = members[i]
        np.testing.assert_array_equal(_powers(x, p, P.n, nrhs), orc.mpk_block(P, X0, p), err_msg=f"member {i}")
    for rc, P, X0, dm, x, fid in members:
        got = x[P.n * nrhs:].clone()
        x[P.n * nrhs:] = 0
        for k in range(p):
            rc.spmvPowerLayout(fid, k)
        torch.cuda.synchronize()
        assert torch.equal(got, x[P.n * nrhs:])
