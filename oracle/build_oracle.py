"""Build recipe of the CPU oracle (test infrastructure).

  liboracle.so     -- oracle/spr_oracle.cpp, the CPU restatement (always built)
  _ref/libref.so   -- the reference's own ras_cut.h / ras_qm_mask.h compiled in
                      place from /root/reference through oracle/ref/ (built only
                      where the reference tree is mounted; nothing is copied)

Both are compiled with -ffp-contract=off so that no multiply-add is fused,
matching the CUDA kernels built with --fmad=false.
"""
from __future__ import annotations

import os
import pathlib
import platform
import shutil
import subprocess
import sys

HERE = pathlib.Path(__file__).resolve().parent
# The reference's source tree: SPR_REFERENCE_SRC, or the read-only mount of
# this build's container by default (absent on machines without it, where
# build_ref() builds nothing).
DEFAULT_REFERENCE_SRC = "/root/reference/gpu-scanline/src"
REFERENCE_SRC = pathlib.Path(os.environ.get("SPR_REFERENCE_SRC", DEFAULT_REFERENCE_SRC))
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


def build_ref(force=False, reference_src=None):
    """Compiles the reference's intersection and mask code from
    `reference_src` (default REFERENCE_SRC); None if absent."""
    src = pathlib.Path(reference_src) if reference_src else REFERENCE_SRC
    if not (src / "rasterizer" / "shared" / "ras_cut.h").exists():
        return None
    outdir = HERE / "_ref"
    outdir.mkdir(exist_ok=True)
    out = outdir / "libref.so"
    srcs = [HERE / "ref" / "ref_driver.cpp", HERE / "ref" / "ref_shim.h",
            HERE / "ref" / "shim_include" / "mochimazui" / "glpp.h"]
    if force or _stale(out, srcs):
        cuda_inc = "/usr/local/cuda/include"
        _run([CXX, *FLAGS, "-w", "-I", str(HERE / "ref" / "shim_include"), "-I", str(HERE / "ref"),
              "-I", str(src), "-I", str(src / "rasterizer" / "shared"),
              "-I", cuda_inc, "-o", str(out), str(HERE / "ref" / "ref_driver.cpp")])
    return out


if __name__ == "__main__":
    import argparse

    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--reference-src", default=None,
                    help=f"the reference's gpu-scanline/src directory (default: $SPR_REFERENCE_SRC or "
                         f"{DEFAULT_REFERENCE_SRC})")
    args = ap.parse_args()
    print(build_oracle(args.force))
    print(build_ref(args.force, args.reference_src))
