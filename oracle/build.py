"""Build recipe for the oracle (test infrastructure, never the product).

* ``build_oracle()`` compiles the C restatement ``ba_oracle.c`` into
  ``oracle/_build/libzsoracle.so`` with the system C compiler. It runs on any
  host (x86-64 here, aarch64 on the GPU host).
* ``build_ref()`` compiles ``ref_driver.cpp`` against the unmodified
  zeroslam headers where they lie (``$ZS_REFERENCE_ROOT/source``) into
  ``oracle/_ref/libzsref.so``, with the reference's release flags
  (-O3 -DNDEBUG -std=c++17 -fno-exceptions -fno-rtti, CMakeLists.txt:17-43).
  Nothing is copied out of the reference tree. When the reference tree is
  absent this is a no-op.

Run ``ZS_REFERENCE_ROOT=<zeroslam checkout> python oracle/build.py`` to build
both (without the variable only the restatement is built).
"""

from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
REF_DIR = os.path.join(HERE, "_ref")
ORACLE_SO = os.path.join(BUILD_DIR, "libzsoracle.so")
REF_SO = os.path.join(REF_DIR, "libzsref.so")
# The zeroslam source tree to build the reference driver against: the
# ZS_REFERENCE_ROOT environment variable, else the tree of the last build in
# this checkout (recorded in oracle/_ref, which is not version-controlled),
# else none (no reference build; the tests that need the tree skip).
ROOT_RECORD = os.path.join(REF_DIR, "reference_root")


def _reference_root() -> str:
    env = os.environ.get("ZS_REFERENCE_ROOT", "")
    if env:
        return env
    try:
        with open(ROOT_RECORD) as f:
            return f.read().strip()
    except OSError:
        return ""


REFERENCE_ROOT = _reference_root()


def _stale(target: str, sources: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def build_oracle(force: bool = False) -> str:
    src = os.path.join(HERE, "ba_oracle.c")
    hdr = os.path.join(HERE, "ba_oracle.h")
    if force or _stale(ORACLE_SO, [src, hdr]):
        os.makedirs(BUILD_DIR, exist_ok=True)
        tmp = ORACLE_SO + f".{os.getpid()}.tmp"
        # -ffp-contract=off keeps the restatement's rounding the same on hosts
        # with and without fused multiply-add.
        subprocess.check_call(["gcc", "-O2", "-std=c99", "-fPIC", "-shared", "-ffp-contract=off", "-pthread",
                               "-o", tmp, src, "-lm"])
        os.replace(tmp, ORACLE_SO)
    return ORACLE_SO


def reference_available() -> bool:
    return bool(REFERENCE_ROOT) and os.path.isfile(os.path.join(REFERENCE_ROOT, "source", "factor_graph.hpp"))


def build_ref(force: bool = False) -> str | None:
    if not reference_available():
        return REF_SO if os.path.exists(REF_SO) else None
    src = os.path.join(HERE, "ref_driver.cpp")
    inc = os.path.join(REFERENCE_ROOT, "source")
    deps = [src] + [os.path.join(inc, f) for f in ("factor_graph.hpp", "camera.hpp", "lie.hpp", "matrix.hpp",
                                                   "matrix_sparse_block.hpp", "matrix_sparse_block_diagonal.hpp",
                                                   "matrix_decomposition_cholesky.hpp", "math.hpp", "map.hpp",
                                                   "frame.hpp", "landmark.hpp", "feature.hpp", "image.hpp")]
    if force or _stale(REF_SO, deps):
        os.makedirs(REF_DIR, exist_ok=True)
        tmp = REF_SO + f".{os.getpid()}.tmp"
        subprocess.check_call(["g++", "-O3", "-DNDEBUG", "-std=c++17", "-fno-exceptions", "-fno-rtti", "-fPIC",
                               "-shared", "-I", inc, "-o", tmp, src])
        os.replace(tmp, REF_SO)
    with open(ROOT_RECORD, "w") as f:
        f.write(REFERENCE_ROOT + "\n")
    return REF_SO


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_ref(force="--force" in sys.argv))
