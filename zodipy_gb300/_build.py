"""Build ``libzodigb.so`` (the CUDA kernels + C ABI) in-tree for sm_103a.

Each translation unit is compiled by nvcc in parallel, then linked into one
shared library next to this file.  The library links the CUDA runtime
statically and exports only the ``zl_*`` C symbols of ``include/zodigb.h``.
"""

from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
REPO_DIR = os.path.dirname(PKG_DIR)
CSRC = os.path.join(PKG_DIR, "csrc")
BUILD_DIR = os.path.join(PKG_DIR, "_build")
LIB_PATH = os.path.join(PKG_DIR, "libzodigb.so")
SOURCES = [
    "zl_api.cu",
    "zl_fwd_f64.cu",
    "zl_fwd_f64_warp.cu",
    "zl_fwd_f32.cu",
    "zl_fwd_f32_dirbe.cu",
    "zl_fwd_f32_planck.cu",
    "zl_fwd_f32_generic.cu",
    "zl_fwd_f32_rrm.cu",
    "zl_fwd_f32x2_dirbe.cu",
    "zl_fwd_f32x2_dirbe_scat.cu",
    "zl_fwd_f32x2_planck.cu",
    "zl_fwd_dirbe_cp.cu",
    "zl_bwd_f32.cu",
    "zl_bwd_f32_dirbe.cu",
    "zl_bwd_f32_dirbe34.cu",
    "zl_bwd_dirbe_cp.cu",
    "zl_bwd_dirbe_cp34.cu",
    "zl_bwd_f32_planck.cu",
    "zl_bwd_rrm.cu",
    "zl_diag.cu",
    "zl_static.cu",
    "zl_tod.cu",
]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Per-file code-generation flags, kept where they measured faster on GB300: ptxas's most
# register-hungry scheduling took the Kelsall adjoint kernels 0.7-2.1 % faster (and the
# forward kernels up to 4.6 % slower, so they keep the default).
FILE_FLAGS = {
    src: ["-Xptxas=--register-usage-level=10"]
    for src in ("zl_bwd_f32_dirbe.cu", "zl_bwd_f32_dirbe34.cu", "zl_bwd_dirbe_cp.cu", "zl_bwd_dirbe_cp34.cu",
                "zl_bwd_f32_planck.cu")
}


def nvcc_path() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libzodigb.so")


def _inputs() -> list[str]:
    deps = [os.path.join(CSRC, s) for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]
    deps += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cuh")]
    deps.append(os.path.join(REPO_DIR, "include", "zodigb.h"))
    deps.append(os.path.abspath(__file__))
    return deps


def up_to_date() -> bool:
    if not os.path.exists(LIB_PATH):
        return False
    t = os.path.getmtime(LIB_PATH)
    return all(os.path.getmtime(p) <= t for p in _inputs())


def build(force: bool = False, verbose: bool = False, extra_flags: list[str] | None = None) -> str:
    """Compile and link; returns the library path.  Raises on any nvcc error."""
    if not force and up_to_date():
        return LIB_PATH
    nvcc = nvcc_path()
    os.makedirs(BUILD_DIR, exist_ok=True)
    flags = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-fvisibility=hidden", *ARCH]
    flags += list(extra_flags or [])
    srcs = [s for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]

    def compile_one(src: str) -> str:
        obj = os.path.join(BUILD_DIR, src.replace(".cu", ".o"))
        cmd = [nvcc, *flags, *FILE_FLAGS.get(src, []), "-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{res.stdout}\n{res.stderr}")
        if verbose and res.stderr:
            print(res.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB_PATH + ".tmp"
    cmd = [nvcc, "-shared", *ARCH, "-o", tmp, *objs, "-Xcompiler", "-fPIC"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    import sys

    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
