"""RACE_SWEEP_GATHER on the GPU: SpMV, SpMTV and SymmSpMV in one launch
without phases. FP64 results equal RACE's sequential walk (the oracle on
the engine's own phases) bit for bit; with FP32/BF16 values they equal the
wave executor's. (The gather plans are checked against the sequential walk
on the CPU in test_host_logic.py; this file runs after the other GPU
tests.)"""
import numpy as np
import pytest

from oracle import oracle as orc
from race_gb300 import matgen

torch = pytest.importorskip("torch")

from race_gb300 import interface as ri  # noqa: E402


def _run(rc, kern, dm, x0, b0, xdt, mode):
    rc.setSweepMode(mode)
    x = torch.tensor(x0, device="cuda").to(xdt)
    b = torch.tensor(b0, device="cuda").to(xdt)
    fid = rc.registerFunction(kern, ri.Operands(dm, x, b))
    assert fid >= 0
    for _ in range(2):  # the plan is built at the first gather call, then reused
        assert rc.executeFunction(fid) == 0
    torch.cuda.synchronize()
    return b.cpu().numpy()


@pytest.mark.gpu
@pytest.mark.parametrize("m,d,t", [("lap7_32", 2, 1024), ("lap7_16", 2, 16), ("band_5k", 2, 32),
                                   ("islands_330", 2, 16), ("plaw_3k", 1, 32)])
def test_gather_mode(mats, m, d, t):
    A = mats[m]
    rc = ri.Interface(A.n, t, d, A.row_ptr, A.col, symm_hint=True)
    assert rc.RACEColor() == 0
    P = A.permuted(rc.getPerm(), rc.getInvPerm())
    U = P.upper()
    x0 = matgen.uniform_vector(A.n, 0)
    b0 = matgen.uniform_vector(A.n, 1)
    pp, lo, hi = rc.getPhases(False)
    kernels = [(ri.SPMV, P)] + ([(ri.SPMTV, P), (ri.SYMMSPMV, U)] if d == 2 else [])
    for kern, mat in kernels:
        # FP64 against the sequential walk of the engine's phases (twice, as on the GPU)
        xs, bs = x0.copy(), b0.copy()
        for _ in range(2):
            for ph in range(len(pp) - 1):
                for leaf in range(pp[ph], pp[ph + 1]):
                    orc.run_kernel(kern, int(lo[leaf]), int(hi[leaf]), mat, xs, bs)
        got = _run(rc, kern, ri.DeviceCsr.from_csr(mat, "cuda", torch.float64), x0, b0, torch.float64,
                   ri.SWEEP_GATHER)
        np.testing.assert_array_equal(got, bs, err_msg=f"{kern} f64")
        # reduced precision against the wave executor (rows of at most 512 entries: both sequential)
        if np.diff(mat.row_ptr).max() <= 512:
            for vdt in (torch.float32, torch.bfloat16):
                dm = ri.DeviceCsr.from_csr(mat, "cuda", vdt)
                w = _run(rc, kern, dm, x0, b0, torch.float32, ri.SWEEP_WAVE)
                g = _run(rc, kern, dm, x0, b0, torch.float32, ri.SWEEP_GATHER)
                np.testing.assert_array_equal(g, w, err_msg=f"{kern} {vdt}")
    rc.setSweepMode(ri.SWEEP_AUTO)
