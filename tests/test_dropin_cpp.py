"""The C++ drop-in factor graph (include/zeroslam_gb300/factor_graph.hpp).

It is compiled against zeroslam's own matrix / lie / camera headers, so these
checks run where the zeroslam source tree is (they skip elsewhere):
  * the drop-in's host checks (tests/cpp/dropin_host_test.cpp): single-edge
    residuals and Jacobians with the values of zeroslam's
    tests/factor_graph.test.cpp:229-276, structure-of-arrays export and
    write-back, unsupported graphs, and solve() returning ZS_ERR_CUDA with the
    vertices untouched when no GPU is usable (no CPU fallback);
  * zeroslam's own tests/factor_graph.test.cpp compiles unmodified against
    the drop-in (its solve sections need a GPU to pass);
  * the drop-in's robust losses print bit-identical values to zeroslam's;
  * the map-level glue (include/zeroslam_gb300/map_glue.hpp) compiles against
    zeroslam's map, frame, landmark and feature types and lays a map out as
    the C ABI expects (tests/cpp/map_glue_test.cpp);
  * the stand-in matrix / lie / camera headers (tests/cpp/standin), which
    let the drop-in build where zeroslam's tree is absent (the GPU tests,
    tests/test_gpu_dropin.py), print the same values as zeroslam's headers
    (tests/cpp/standin_values.cpp), and the drop-in's host checks pass
    against them.
"""

import os
import shutil
import subprocess

import pytest

from oracle import build as ob

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CPP = os.path.join(ROOT, "tests", "cpp")
DROPIN = os.path.join(ROOT, "include", "zeroslam_gb300")

STANDIN = os.path.join(CPP, "standin")

pytestmark = pytest.mark.skipif(not shutil.which("g++"), reason="needs g++")
needs_reference = pytest.mark.skipif(not ob.reference_available(), reason="needs the zeroslam source tree")


def _lib_dir():
    from zeroslam_gb300 import build

    return os.path.dirname(build.build())


def _compile(src, out, dropin=True, link=True, standin=False):
    cmd = ["g++", "-std=c++17", "-O1", "-Wall"]
    if dropin:
        cmd += ["-I", DROPIN]
    cmd += ["-I", STANDIN if standin else os.path.join(ob.REFERENCE_ROOT, "source"), src, "-o", out]
    if link:
        lib = _lib_dir()
        cmd += ["-L", lib, "-lzeroslam_ba", f"-Wl,-rpath,{lib}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return out


@needs_reference
def test_dropin_host_checks(tmp_path):
    exe = _compile(os.path.join(CPP, "dropin_host_test.cpp"), str(tmp_path / "dropin_host_test"))
    args = [exe] + (["--gpu"] if os.environ.get("ZS_DROPIN_EXPECT_GPU") == "1" else [])
    r = subprocess.run(args, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == "OK", r.stderr


@needs_reference
def test_reference_test_compiles_against_dropin(tmp_path):
    _compile(os.path.join(ob.REFERENCE_ROOT, "tests", "factor_graph.test.cpp"), str(tmp_path / "fg_test"))


@needs_reference
def test_losses_match_reference(tmp_path):
    mine = _compile(os.path.join(CPP, "loss_values.cpp"), str(tmp_path / "loss_mine"))
    ref = _compile(os.path.join(CPP, "loss_values.cpp"), str(tmp_path / "loss_ref"), dropin=False, link=False)
    a = subprocess.run([mine], capture_output=True, text=True, check=True).stdout
    b = subprocess.run([ref], capture_output=True, text=True, check=True).stdout
    assert a == b and len(a.splitlines()) == 27


@needs_reference
def test_map_glue_host_checks(tmp_path):
    exe = _compile(os.path.join(CPP, "map_glue_test.cpp"), str(tmp_path / "map_glue_test"))
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip().splitlines()[-1] == "OK", r.stderr


@needs_reference
def test_standins_match_reference(tmp_path):
    mine = _compile(os.path.join(CPP, "standin_values.cpp"), str(tmp_path / "sv_mine"), dropin=False, link=False,
                    standin=True)
    ref = _compile(os.path.join(CPP, "standin_values.cpp"), str(tmp_path / "sv_ref"), dropin=False, link=False)
    a = subprocess.run([mine], capture_output=True, text=True, check=True).stdout.split("\n")
    b = subprocess.run([ref], capture_output=True, text=True, check=True).stdout.split("\n")
    assert len(a) == len(b) and len(a) > 60
    for x, y in zip(a, b):
        if not y:
            continue
        kx, vx = x.split()
        ky, vy = y.split()
        assert kx == ky
        assert abs(float(vx) - float(vy)) <= 1e-12 * max(1.0, abs(float(vy))), (x, y)


def test_dropin_host_checks_standins(tmp_path):
    """The drop-in against the stand-in headers, without a usable device:
    solve() reports ZS_ERR_CUDA and leaves the vertices alone."""
    exe = _compile(os.path.join(CPP, "dropin_host_test.cpp"), str(tmp_path / "dropin_standin"), standin=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120, env={**os.environ, "CUDA_VISIBLE_DEVICES": ""})
    assert r.returncode == 0 and r.stdout.strip() == "OK", r.stderr
