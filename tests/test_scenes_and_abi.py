"""CPU checks: the scene generator, and that the CUDA library loads and
exports every entry point include/zeroslam_ba.h declares (no compute)."""

import ctypes
import os
import re

import numpy as np

from conftest import ROOT
from zeroslam_gb300 import scenes


def test_pcg_streams_deterministic():
    a = scenes.Pcg32Streams(5).raw(10000)
    b = scenes.Pcg32Streams(5).raw(10000)
    c = scenes.Pcg32Streams(6).raw(10000)
    assert np.array_equal(a, b) and not np.array_equal(a, c)
    u = scenes.Pcg32Streams(1).uniform(200000)
    assert 0.0 < u.min() and u.max() < 1.0 and abs(u.mean() - 0.5) < 0.01
    z = scenes.Pcg32Streams(2).normal(200000)
    assert abs(z.mean()) < 0.01 and abs(z.std() - 1.0) < 0.01


def test_small_scene_shape():
    sc = scenes.small_scene()
    assert sc.K == 10 and sc.L == 500 and 3500 < sc.M < 5000
    assert sc.pose_fixed[0] == 1 and sc.pose_fixed[1:].sum() == 0
    assert np.all(np.diff(sc.obs_landmark) >= 0)
    assert np.all((sc.obs_pose >= 0) & (sc.obs_pose < sc.K))
    q = sc.poses[:, 3:7]
    assert np.allclose(np.linalg.norm(q, axis=1), 1.0, atol=1e-12)
    # every kept landmark is observed
    assert np.unique(sc.obs_landmark).size == sc.L


def test_scene_reproducible():
    a, b = scenes.arc_scene(7, 200, seed=3), scenes.arc_scene(7, 200, seed=3)
    assert np.array_equal(a.poses, b.poses) and np.array_equal(a.obs_uv, b.obs_uv)


def test_window_batch_sizes():
    ws = scenes.window_batch(8)
    assert len(ws) == 8
    for w in ws:
        assert 5 <= w.K <= 30 and 200 <= w.L <= 3000


def _declared_functions():
    src = open(os.path.join(ROOT, "include", "zeroslam_ba.h")).read()
    return sorted(set(re.findall(r"\b(zs_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    from zeroslam_gb300 import ba, build

    path = build.build()
    lib = ctypes.CDLL(path)
    declared = _declared_functions()
    assert set(ba.ABI_FUNCTIONS) == set(declared)
    for name in declared:
        assert hasattr(lib, name), name


def test_default_options_are_the_reference_constants():
    from zeroslam_gb300 import ba

    o = ba.default_options()
    assert o.tau == 1e-5 and o.diagonal_clamp == 5e10 and o.max_failures == 10
    assert o.legacy_stop == 1e-10 and o.relative_tolerance == 1e-6 and o.chi2_floor == 1e-12
    assert o.precision == ba.FP64


def test_status_strings_and_no_device_behaviour():
    from zeroslam_gb300 import ba

    lib = ba.load()
    assert lib.zs_ba_status_string(ba.ZS_ERR_CHOLESKY) == b"Cholesky solver failed"
    try:
        import torch

        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if not has_gpu:
        # no CPU fallback: without a device the handle cannot be created
        h = ctypes.c_void_p()
        assert lib.zs_ba_create(ctypes.byref(h), None) == ba.ZS_ERR_CUDA
