"""Builds libwakis_fit.so (the C-ABI library with the sm_103a kernels) in-tree.

    python -m wakis_gb300.build          # or wakis_gb300.build.build()

The library is written to wakis_gb300/_lib/libwakis_fit.so next to the sources, so the
package finds it without installation.  One translation unit, one -gencode target.
"""

import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
SRC = os.path.join(PKG, "csrc", "fit_capi.cu")
DEPS = [SRC, os.path.join(PKG, "csrc", "fit_kernels.cuh"), os.path.join(PKG, "csrc", "fit_pool.cuh"),
        os.path.join(PKG, "csrc", "fit_tma.cuh"),
        os.path.join(ROOT, "include", "wakis_fit.h")]
OUT_DIR = os.path.join(PKG, "_lib")
LIB = os.path.join(OUT_DIR, "libwakis_fit.so")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def nvcc_path():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libwakis_fit.so")


def needs_build():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(p) > t for p in DEPS)


def build(force=False, verbose=False, extra=()):
    if not force and not needs_build():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = [nvcc_path(), ARCH, "-O3", "-lineinfo", "-std=c++17", "-shared", "-Xcompiler", "-fPIC",
           "-Xcompiler", "-fvisibility=hidden", "-I", os.path.join(ROOT, "include"),
           "-DFIT_EXPORT", *extra, SRC, "-o", tmp, "-lcudart"]
    if verbose:
        print(" ".join(cmd))
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed building libwakis_fit.so:\n" + r.stdout + r.stderr)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
