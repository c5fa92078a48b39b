"""Custom device functions through the engine's schedule
(include/race_gb300_device.cuh), the GPU counterpart of the reference's
host callbacks: the example GS body as a colored functor must equal the
sequential walk of the engine's phases bit for bit, and the MPK body as a
power functor must equal p sequential SpMVs bit for bit. The functors live
in tests/device_functors.cu, compiled with nvcc for sm_103a (the fnlib
fixture of conftest.py)."""
import ctypes as C
import pathlib
import subprocess

import numpy as np
import pytest

from oracle import oracle as orc
from race_gb300 import _lib, build, matgen

ROOT = pathlib.Path(__file__).resolve().parents[1]
SRC = ROOT / "tests" / "device_functors.cu"
NVCC = ["-std=c++17", "-O3", "--fmad=false", *build.ARCH, "-I", str(ROOT / "include")]


def _nvcc():
    try:
        return build._nvcc()
    except RuntimeError:
        pytest.skip("no nvcc")


def test_device_header_compiles(tmp_path):
    """The header-only templates instantiate and compile for sm_103a."""
    r = subprocess.run([_nvcc(), *NVCC, "-c", str(SRC), "-o", str(tmp_path / "fn.o")], capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stderr


def test_device_functions_link_and_reject_a_null_engine(fnlib):
    """The functor library links against the engine and loads; without an
    engine the schedule queries fail before any launch."""
    bad = _lib.RACE_ERR_INVALID_ARG
    assert fnlib.fn_gs(None, None, None, None, None, None, 0) == bad
    assert fnlib.fn_mpk(None, None, None, None, None, 10, 2, 32) == bad
    assert fnlib.fn_mpk(None, None, None, None, None, 10, 0, 32) == bad  # power below 1
    assert fnlib.fn_count_subpower(None, None, 2, 2, None) == bad
    assert fnlib.fn_count_after_set(None, None, 2, 2, None) == bad
    errors = C.c_int(7)
    assert fnlib.fn_check_coverage(None, C.byref(errors)) == bad and errors.value == -1


@pytest.mark.gpu
@pytest.mark.parametrize("m,d,t", [("lap7_16", 2, 16), ("aniso9_100x80", 1, 16), ("plaw_3k", 1, 32),
                                   ("islands_330", 2, 16)])
def test_device_function_gs_matches_sequential_walk(mats, fnlib, m, d, t):
    import torch

    from race_gb300 import interface as ri
    A = mats[m]
    rc = ri.Interface(A.n, t, d, A.row_ptr, A.col, symm_hint=True)
    assert rc.RACEColor() == 0
    P = A.permuted(rc.getPerm(), rc.getInvPerm())
    dm = ri.DeviceCsr.from_csr(P)
    x0 = matgen.uniform_vector(A.n, 0)
    b0 = matgen.uniform_vector(A.n, 1)
    for rev in (False, True):
        x = torch.tensor(x0, device="cuda")
        b = torch.tensor(b0, device="cuda")
        assert fnlib.fn_gs(rc._h, dm.row_ptr.data_ptr(), dm.col.data_ptr(), dm.val.data_ptr(), b.data_ptr(),
                           x.data_ptr(), int(rev)) == 0
        xr, br = x0.copy(), b0.copy()
        pp, lo, hi = rc.getPhases(rev)
        for p in range(len(pp) - 1):
            for leaf in range(pp[p], pp[p + 1]):
                orc.run_kernel(orc.K_GS, int(lo[leaf]), int(hi[leaf]), P, xr, br)
        np.testing.assert_array_equal(x.cpu().numpy(), xr)


@pytest.mark.gpu
@pytest.mark.parametrize("m,p,c", [("st27_24", 8, 2e6), ("aniso5_120x90", 4, 5e5), ("band_5k", 8, 3300),
                                   ("plaw_20k", 4, 1e6)])
def test_device_power_function_matches_spmv_chain(mats, fnlib, m, p, c):
    import torch

    from race_gb300 import interface as ri
    A = mats[m]
    rc = ri.Interface(A.n, 1, ri.POWER, A.row_ptr, A.col, symm_hint=True)
    assert rc.RACEColor(p, c) == 0
    P = A.permuted(rc.getPerm(), rc.getInvPerm())
    dm = ri.DeviceCsr.from_csr(P)
    x0 = matgen.uniform_vector(A.n, 0)
    Y = orc.mpk_plain(P, x0, p)
    for rows in (32, 7):
        x = torch.zeros((p + 1) * A.n, dtype=torch.float64, device="cuda")
        x[: A.n] = torch.tensor(x0, device="cuda")
        assert fnlib.fn_mpk(rc._h, dm.row_ptr.data_ptr(), dm.col.data_ptr(), dm.val.data_ptr(), x.data_ptr(), A.n,
                            p, rows) == 0
        np.testing.assert_array_equal(x.cpu().numpy().reshape(p + 1, A.n), Y)


def test_integration_cuda_examples_compile(tmp_path):
    """The CUDA examples under tests/examples compile for sm_103a."""
    srcs = sorted((ROOT / "tests" / "examples").glob("*.cu"))
    assert srcs
    for src in srcs:
        r = subprocess.run([_nvcc(), *NVCC, "-c", str(src), "-o", str(tmp_path / (src.stem + ".o"))],
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stderr


@pytest.mark.parametrize("key,power,sub,rows", [("power__st27_24__p8__c2000000", 8, 1, 32),
                                                ("power__band_5k__p8__c3300", 2, 3, 7),
                                                ("power__tiny_1__p2__c10000", 2, 2, 32),
                                                ("power__islands_330__p3__c20000", 3, 2, 5),
                                                ("powertri__lap7_16__L__p4__c20000", 4, 1, 32),
                                                ("powertri__plaw_3k__U__p8__c50000", 8, 1, 16)])
def test_power_call_schedule(golden, tmp_path, key, power, sub, rows):
    """The matrix-power call table on the reference's level groups: every
    row gets every (power, sub-power) exactly once, in order; the call of
    group g at flat step q runs in wavefront step g + 2(q-1), so everything it
    reads (flat step q-1 of groups up to g+1, any earlier group included, as
    triangular partitions need) ran in an earlier step; and a four-argument
    functor sees (pow, subPow) = ((q-1)/sub+1, (q-1)%sub+1)."""
    exe = tmp_path / "pc"
    r = subprocess.run([_nvcc(), *NVCC, str(ROOT / "tests" / "power_calls_check.cu"), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    gp = golden[key + "__lp"]
    out = subprocess.run([str(exe), str(power), str(sub), str(rows)], input=" ".join(map(str, gp)),
                         capture_output=True, text=True, check=True).stdout.split("\n")
    steps = int(out[0])
    T = power * sub
    G = len(gp) - 1
    assert steps == G + 2 * (T - 1)
    n = int(gp[-1])
    seen = np.zeros((T, n), np.int32)
    group_of = np.searchsorted(gp, np.arange(n), side="right") - 1
    for line in out[1:]:
        if not line:
            continue
        s, start, end, q, pw, sp = map(int, line.split())
        assert 0 <= start < end <= n and end - start <= rows
        g = group_of[start]
        assert group_of[end - 1] == g and s == g + 2 * (q - 1)
        seen[q - 1, start:end] += 1
        assert (pw, sp) == ((q - 1) // sub + 1, (q - 1) % sub + 1)
    assert (seen == 1).all()
