"""Build recipe of libspr.so, in tree, for sm_103a.

CUDA sources are compiled with nvcc for sm_103a only, with --fmad=false so
that no multiply-add is fused (the fragment, intersection and resolve
arithmetic must match the host restatement bit for bit) and with IEEE
division / square root (the nvcc defaults; fast math is never enabled).
Host sources use -ffp-contract=off for the same reason.  Objects go to
_build/ and the library next to this file; both are git-ignored.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import pathlib
import platform
import shutil
import subprocess
import sys

PKG = pathlib.Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libspr.so"
CUDA_HOME = pathlib.Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
NVCC = str(CUDA_HOME / "bin" / "nvcc")
CXX = shutil.which("g++") or "g++"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "--fmad=false", "-Xcompiler", "-fPIC,-ffp-contract=off",
              "-Xptxas", "-warn-spills"]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-Wall", "-Wno-unused-function",
             f"-I{CUDA_HOME / 'include'}"]


def sources():
    return sorted(CSRC.glob("*.cu")), sorted(CSRC.glob("*.cpp"))


def _compile(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed:\n" + " ".join(cmd) + "\n" + r.stdout[-3000:] + r.stderr[-6000:])
    return r.stderr


def _stale(out: pathlib.Path, deps) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> pathlib.Path:
    BUILD.mkdir(exist_ok=True)
    stamp = BUILD / "MACHINE"
    if not stamp.exists() or stamp.read_text() != platform.machine():
        force = True  # objects from another host architecture
    stamp.write_text(platform.machine())
    cus, cpps = sources()
    headers = list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + [PKG.parent / "include" / "spr.h"]
    jobs, objs = [], []
    for src in cus:
        obj = BUILD / (src.stem + ".cu.o")
        objs.append(obj)
        if force or _stale(obj, [src, *headers]):
            jobs.append([NVCC, *ARCH, *NVCC_FLAGS, "-c", str(src), "-o", str(obj)])
    for src in cpps:
        obj = BUILD / (src.stem + ".o")
        objs.append(obj)
        if force or _stale(obj, [src, *headers]):
            jobs.append([CXX, *CXX_FLAGS, "-c", str(src), "-o", str(obj)])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for err in ex.map(_compile, jobs):
                if verbose and err:
                    print(err, file=sys.stderr)
    if force or jobs or _stale(LIB, objs):
        _compile([CXX, "-shared", "-o", str(LIB), *map(str, objs), f"-L{CUDA_HOME / 'lib64'}",
                  "-lcudart_static", "-lrt", "-lpthread", "-ldl"])
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
