"""The C++ drop-in factor graph (include/zeroslam_gb300/factor_graph.hpp)
solving on the device: factor_graph::solve() (source/factor_graph.hpp:489)
through the C ABI it wraps.

zeroslam's source tree is not on the GPU machines, so the drop-in is built
here against the stand-in matrix / lie / camera headers of tests/cpp/standin
(pinned to zeroslam's own headers by tests/test_dropin_cpp.py where that tree
is available):
  * tests/cpp/dropin_host_test.cpp with --gpu: the host checks, and a small
    graph's solve() accepting steps and lowering the cost on the device;
  * tests/cpp/dropin_solve.cpp: every golden solve (solve_*.npz, written by
    zeroslam's own factor_graph::solve) rebuilt as vertices and edges the way
    zeroslam's map code builds them, solved by the drop-in's solve(), and the
    vertices it writes back compared with zeroslam's result at the
    tolerances of the C-ABI parity tests (tests/test_gpu_parity.py); the mixed
    form on the loss-free fixtures at the mixed-form cost tolerance.
"""
import os
import shutil
import struct
import subprocess

import numpy as np
import pytest

from conftest import SOLVE_FIXTURES, cost_tol, load_npz, rel_err, state_tol

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not shutil.which("g++"), reason="needs g++")]

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CPP = os.path.join(ROOT, "tests", "cpp")
STEP_TOL = 1e-9
MIXED_COST_TOL = 1e-6


def _build(zs_lib, src, out):
    lib = os.path.dirname(zs_lib._name)
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-I", os.path.join(ROOT, "include", "zeroslam_gb300"), "-I",
           os.path.join(CPP, "standin"), src, "-o", out, "-L", lib, "-lzeroslam_ba", f"-Wl,-rpath,{lib}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return out


@pytest.fixture(scope="module")
def solver(zs_lib, tmp_path_factory):
    d = tmp_path_factory.mktemp("dropin")
    return _build(zs_lib, os.path.join(CPP, "dropin_solve.cpp"), str(d / "dropin_solve"))


def _write_scene(path, g, precision):
    K, L, M = g["poses"].shape[0], g["landmarks"].shape[0], g["obs_pose"].shape[0]
    has_info = "obs_info" in g
    with open(path, "wb") as f:
        f.write(struct.pack("<8i", K, L, M, int(g["iterations"]), int(bool(g["use_relative"])), int(g["loss_kind"]),
                            int(has_info), precision))
        f.write(struct.pack("<d", float(g["loss_delta"])))
        f.write(np.asarray(g["intrinsics"], "<f8").tobytes())
        f.write(np.ascontiguousarray(g["poses"], "<f8").tobytes())
        f.write(np.ascontiguousarray(g["landmarks"], "<f8").tobytes())
        f.write(np.ascontiguousarray(g["pose_fixed"], np.uint8).tobytes())
        f.write(np.ascontiguousarray(g["landmark_fixed"], np.uint8).tobytes())
        f.write(np.ascontiguousarray(g["obs_pose"], "<i4").tobytes())
        f.write(np.ascontiguousarray(g["obs_landmark"], "<i4").tobytes())
        f.write(np.ascontiguousarray(g["obs_uv"], "<f8").tobytes())
        if has_info:
            f.write(np.ascontiguousarray(g["obs_info"], "<f8").tobytes())
    return K, L


def _solve(solver, tmp_path, g, precision=0):
    scene, result = str(tmp_path / "scene.bin"), str(tmp_path / "result.bin")
    K, L = _write_scene(scene, g, precision)
    r = subprocess.run([solver, scene, result], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    raw = open(result, "rb").read()
    ret = struct.unpack_from("<i", raw, 0)[0]
    chi_before, chi_after = struct.unpack_from("<2d", raw, 4)
    vals = np.frombuffer(raw, "<f8", offset=20)
    return ret, chi_before, chi_after, vals[:7 * K].reshape(K, 7), vals[7 * K:].reshape(L, 3)


def test_host_checks_on_device(zs_lib, tmp_path):
    exe = _build(zs_lib, os.path.join(CPP, "dropin_host_test.cpp"), str(tmp_path / "dropin_host_test"))
    r = subprocess.run([exe, "--gpu"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.strip() == "OK", r.stderr


@pytest.mark.parametrize("name", SOLVE_FIXTURES)
def test_solve_matches_reference(solver, tmp_path, name):
    g = load_npz(name)
    ret, chi_before, chi_after, poses, lms = _solve(solver, tmp_path, g)
    assert abs(chi_before - float(g["chi2_before"])) <= 1e-12 * abs(float(g["chi2_before"]))
    assert ret == int(g["accepted"])
    c_ref = float(g["chi2_after"])
    assert abs(chi_after - c_ref) <= cost_tol(g) * abs(c_ref) + 1e-12
    if int(g["iterations"]) == 1:
        assert rel_err(poses - g["poses"], g["out_poses"] - g["poses"]) < STEP_TOL
        assert rel_err(lms - g["landmarks"], g["out_landmarks"] - g["landmarks"]) < STEP_TOL
    elif state_tol(g) is not None:
        assert rel_err(poses, g["out_poses"]) < state_tol(g)


@pytest.mark.parametrize("name", [n for n in SOLVE_FIXTURES if n.startswith(("solve_arc_small", "solve_fixed_mix"))])
def test_solve_mixed_form(solver, tmp_path, name):
    """set_precision(ZS_PRECISION_MIXED), the drop-in's extension: the final
    cost at the mixed form's tolerance."""
    g = load_npz(name)
    ret, _, chi_after, _, _ = _solve(solver, tmp_path, g, precision=1)
    assert ret >= 1
    c_ref = float(g["chi2_after"])
    assert abs(chi_after - c_ref) <= MIXED_COST_TOL * abs(c_ref) + 1e-12
