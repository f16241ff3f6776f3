"""Build recipe of the CPU oracle (test infrastructure).

  liboracle.so     -- oracle/spr_oracle.cpp, the CPU restatement (always built)
  _ref/libref.so   -- the reference's own ras_cut.h / ras_qm_mask.h compiled in
                      place from /root/reference through oracle/ref/ (built only
                      where the reference tree is mounted; nothing is copied)

Both are compiled with -ffp-contract=off so that no multiply-add is fused,
matching the CUDA kernels built with --fmad=false.
"""
from __future__ import annotations

import pathlib
import platform
import shutil
import subprocess
import sys

HERE = pathlib.Path(__file__).resolve().parent
REFERENCE_SRC = pathlib.Path("/root/reference/gpu-scanline/src")
CXX = shutil.which("g++") or "g++"
FLAGS = ["-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared"]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stderr[-4000:])


def _stale(out: pathlib.Path, srcs) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(pathlib.Path(s).stat().st_mtime > t for s in srcs)


def _arch_changed() -> bool:
    stamp = HERE / ".machine"
    changed = not stamp.exists() or stamp.read_text() != platform.machine()
    stamp.write_text(platform.machine())
    return changed


def build_oracle(force=False) -> pathlib.Path:
    force = _arch_changed() or force
    out = HERE / "liboracle.so"
    srcs = [HERE / "spr_oracle.cpp", HERE / "spr_oracle.h", HERE.parent / "include" / "spr.h"]
    if force or _stale(out, srcs):
        _run([CXX, *FLAGS, "-pthread", "-o", str(out), str(HERE / "spr_oracle.cpp")])
    return out


def build_ref(force=False):
    """Compiles the reference's intersection and mask code; None if absent."""
    if not (REFERENCE_SRC / "rasterizer" / "shared" / "ras_cut.h").exists():
        return None
    outdir = HERE / "_ref"
    outdir.mkdir(exist_ok=True)
    out = outdir / "libref.so"
    srcs = [HERE / "ref" / "ref_driver.cpp", HERE / "ref" / "ref_shim.h",
            HERE / "ref" / "shim_include" / "mochimazui" / "glpp.h"]
    if force or _stale(out, srcs):
        cuda_inc = "/usr/local/cuda/include"
        _run([CXX, *FLAGS, "-w", "-I", str(HERE / "ref" / "shim_include"), "-I", str(HERE / "ref"),
              "-I", str(REFERENCE_SRC), "-I", str(REFERENCE_SRC / "rasterizer" / "shared"),
              "-I", cuda_inc, "-o", str(out), str(HERE / "ref" / "ref_driver.cpp")])
    return out


if __name__ == "__main__":
    force = "--force" in sys.argv
    print(build_oracle(force))
    print(build_ref(force))
