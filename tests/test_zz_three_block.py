"""Distance-2 coloring with RACE::THREE_BLOCK on the GPU: the engine's
permutation, zone tree and thread count equal the reference's, and its
bit-exact sweeps reproduce the reference executor's outputs. (The load
balancer, the level recursion and the phase semantics for THREE_BLOCK are
checked on the CPU in test_host_logic.py; this file runs after the other
GPU tests.)"""
import numpy as np
import pytest

from cases import COLOR3_CASES, digest, key_color3
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
