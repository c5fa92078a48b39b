"""Builds race_gb300/_build/librace_gb300.so with nvcc for sm_103a.

Host code is compiled without floating-point contraction (-ffp-contract=off)
so the load balancer's double arithmetic is identical on x86 and Arm hosts;
device code uses --fmad=false so every fused multiply-add in the kernels is an
explicit fma() (the same operation the CPU oracle performs).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import pathlib
import shutil
import subprocess

PKG = pathlib.Path(__file__).resolve().parent
CSRC = PKG / "csrc"
OUT = PKG / "_build"
LIB = OUT / "librace_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not pathlib.Path(cand).exists():
        raise RuntimeError("nvcc not found")
    return cand


def sources():
    return sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")))


def _compile(src: pathlib.Path) -> pathlib.Path:
    obj = OUT / (src.name + ".o")
    deps = [src] + list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + [PKG.parent / "include" / "race_gb300.h"]
    if obj.exists() and obj.stat().st_mtime > max(d.stat().st_mtime for d in deps):
        return obj
    cmd = [_nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "--fmad=false", "-Xcompiler", "-fPIC,-ffp-contract=off",
           "-I", str(CSRC), "-I", str(PKG.parent / "include"), "-c", str(src), "-o", str(obj)]
    if src.suffix == ".cpp":
        cmd[cmd.index(str(src)) - 1:cmd.index(str(src)) - 1] = ["-x", "cu"]
    if os.environ.get("RACE_PTXAS_VERBOSE"):
        cmd.insert(1, "-Xptxas=-v")
    subprocess.check_call(cmd)
    return obj


def build(force: bool = False) -> pathlib.Path:
    OUT.mkdir(exist_ok=True)
    if force:
        for o in OUT.glob("*.o"):
            o.unlink()
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(_compile, srcs))
    if force or not LIB.exists() or LIB.stat().st_mtime < max(o.stat().st_mtime for o in objs):
        tmp = LIB.with_suffix(f".{os.getpid()}.tmp")
        subprocess.check_call([_nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart"])
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
