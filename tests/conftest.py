import os
import pathlib
import sys

import numpy as np
import pytest

ROOT = pathlib.Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))
os.environ.setdefault("ORACLE_QUIET", "1")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


@pytest.fixture(scope="session")
def golden():
    path = ROOT / "tests" / "golden" / "golden.npz"
    return dict(np.load(path, allow_pickle=False))


_MATS = {}


@pytest.fixture(scope="session")
def mats():
    from cases import MATRICES

    class _M:
        def __getitem__(self, name):
            if name not in _MATS:
                _MATS[name] = MATRICES[name]()
            return _MATS[name]

    return _M()


@pytest.fixture(scope="session")
def fnlib(tmp_path_factory):
    """tests/device_functors.cu (functors through the engine's schedule,
    include/race_gb300_device.cuh) built with nvcc for sm_103a and linked
    against the engine library."""
    import ctypes as C
    import subprocess

    from race_gb300 import _lib, build
    try:
        nvcc = build._nvcc()
    except RuntimeError:
        pytest.skip("no nvcc")
    out = tmp_path_factory.mktemp("fn") / "libdevice_functors.so"
    lib_path = _lib.LIB_PATH
    subprocess.check_call([nvcc, "-std=c++17", "-O3", "--fmad=false", *build.ARCH, "-I", str(ROOT / "include"),
                           "-shared", "-Xcompiler", "-fPIC", "--cudart", "shared",
                           str(ROOT / "tests" / "device_functors.cu"), str(lib_path), "-Xlinker",
                           f"-rpath,{lib_path.parent}", "-o", str(out)])
    _lib.lib()  # the engine library first, so both refer to one copy
    L = C.CDLL(str(out))
    vp = C.c_void_p
    L.fn_gs.argtypes = [vp, vp, vp, vp, vp, vp, C.c_int]
    L.fn_mpk.argtypes = [vp, vp, vp, vp, vp, C.c_int, C.c_int, C.c_int]
    L.fn_count_subpower.argtypes = [vp, vp, C.c_int, C.c_int, vp]
    L.fn_count_after_set.argtypes = [vp, vp, C.c_int, C.c_int, vp]
    L.fn_check_coverage.argtypes = [vp, C.POINTER(C.c_int)]
    return L
