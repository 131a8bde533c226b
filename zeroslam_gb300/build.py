"""Builds the sm_103a CUDA library ``zeroslam_gb300/_lib/libzeroslam_ba.so``.

Each ``csrc/*.cu`` is compiled by nvcc in parallel with one ``-gencode``
(compute_103a / sm_103a) and linked into one shared library that exports the
C ABI of ``include/zeroslam_ba.h``. The build is in-tree and incremental.
"""

from __future__ import annotations

import glob
import hashlib
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ_DIR = os.path.join(HERE, "_build")
LIB_DIR = os.path.join(HERE, "_lib")
LIB_PATH = os.path.join(LIB_DIR, "libzeroslam_ba.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Host code is compiled without floating-point contraction, so that it rounds
# the same on x86-64 and aarch64 (and as the reference, built as ISO C++17).
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-O2,-ffp-contract=off", "--expt-relaxed-constexpr",
              "-I", os.path.join(ROOT, "include")]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build zeroslam_gb300")


def _headers() -> list[str]:
    return sorted(glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) +
                  [os.path.join(ROOT, "include", "zeroslam_ba.h")])


def _sig(paths: list[str], extra: list[str]) -> str:
    h = hashlib.sha1()
    for p in paths:
        with open(p, "rb") as f:
            h.update(f.read())
    h.update(" ".join(extra).encode())
    return h.hexdigest()


def _compile(src: str, extra: list[str]) -> str:
    obj = os.path.join(OBJ_DIR, os.path.basename(src)[:-3] + ".o")
    stamp = obj + ".sig"
    sig = _sig([src] + _headers(), ARCH + NVCC_FLAGS + extra)
    if os.path.exists(obj) and os.path.exists(stamp) and open(stamp).read() == sig:
        return obj
    cmd = [nvcc(), "-c", src, "-o", obj] + ARCH + NVCC_FLAGS + extra
    subprocess.check_call(cmd)
    with open(stamp, "w") as f:
        f.write(sig)
    return obj


def build(verbose_ptxas: bool = False, jobs: int | None = None) -> str:
    os.makedirs(OBJ_DIR, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    extra = ["-Xptxas", "-v"] if verbose_ptxas else []
    with ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 1)) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), srcs))
    sig = _sig(objs, [])
    stamp = LIB_PATH + ".sig"
    if not (os.path.exists(LIB_PATH) and os.path.exists(stamp) and open(stamp).read() == sig):
        tmp = LIB_PATH + f".{os.getpid()}.tmp"
        subprocess.check_call([nvcc(), "-shared", "-o", tmp] + ARCH + objs + ["-lcudart"])
        os.replace(tmp, LIB_PATH)
        with open(stamp, "w") as f:
            f.write(sig)
    return LIB_PATH


if __name__ == "__main__":
    print(build(verbose_ptxas="-v" in sys.argv))
