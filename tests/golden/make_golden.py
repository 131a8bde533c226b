"""Writes the golden fixtures under tests/golden/ from zeroslam's own solver.

Run where the reference tree is present (it is compiled by oracle/build.py
into oracle/_ref): ``python tests/golden/make_golden.py``. Every fixture
stores its inputs next to the reference's outputs, so tests that read them
need neither the reference tree nor the scene generator's libm.

Fixtures:
  edges.npz        residuals and analytic Jacobians of edge_reprojection<pinhole>
                   (source/factor_graph.hpp:990-1048), incl. the literal case
                   of tests/factor_graph.test.cpp:236-276 and behind-camera points
  losses.npz       rho of loss_huber / cauchy / tukey (source/factor_graph.hpp:851-934)
  invert3.npz      matrix::invert<3> incl. singular blocks (source/matrix.hpp:749-774)
  cholesky.npz     decompose_cholesky / solve_cholesky on SPD, indefinite and NaN
                   inputs (source/matrix_decomposition_cholesky.hpp:26-95)
  pose_plus.npz    vertex_pose::plus (source/factor_graph.hpp:947-960)
  solve_*.npz      factor_graph::solve on whole problems: state before and after,
                   chi2 before / after and the accepted-step count
  map_optimise.npz map::optimise (source/map.hpp:65-267) on an array map: the
                   frames and landmarks it writes back; the vertex poses it
                   builds from the frames (so3 from a rotation matrix)
  matches.npz      feature::find_matches (source/feature.hpp:1190-1235): two
                   descriptor sets and the matches of several threshold / k /
                   size cases
  cull_*.npz       map::cull (source/map.hpp:269-323) on array maps: inputs and
                   the landmarks it erased; the frame rotations and translations
                   map::optimise writes back from vertex poses (map.hpp:247-251)
"""

from __future__ import annotations

import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.oracle import Reference  # noqa: E402
from zeroslam_gb300 import scenes  # noqa: E402


class Pcg32:
    """Scalar PCG32 with the constants of tests/factor_graph.test.cpp:62-83."""

    def __init__(self):
        self.state = 0x853C49E6748FEA9B
        self.inc = 0xDA3E39CB94B95BDB

    def raw(self) -> int:
        old = self.state
        self.state = (old * 0x5851F42D4C957F2D + self.inc) & ((1 << 64) - 1)
        xs = (((old >> 18) ^ old) >> 27) & 0xFFFFFFFF
        rot = old >> 59
        return ((xs >> rot) | (xs << ((-rot) & 31))) & 0xFFFFFFFF


def seven_camera_scene() -> scenes.Scene:
    """The end-to-end problem of tests/factor_graph.test.cpp:61-155: 7 poses
    (the first fixed), 3 landmarks, PCG-seeded landmark and pixel noise, pinhole
    (1, 1, 0, 0)."""
    rng = Pcg32()
    cams_t = [(0, 0, 0), (0.1, 0, 0), (0, 0.1, 0), (0, 0, 0.1), (-0.1, 0, 0), (0, -0.1, 0), (0, 0, -0.1)]
    lms = [(0.0, 0.0, 1.0), (0.0, 1.0, 1.0), (1.0, 0.0, 1.0)]
    noisy = []
    for lm in lms:
        noisy.append([lm[j] + ((rng.raw() % 10) - 5) * 0.01 for j in range(3)])
    obs_pose, obs_lm, uv = [], [], []
    for c, t in enumerate(cams_t):
        for li, lm in enumerate(lms):
            X = np.array(lm) + np.array(t)
            u, v = X[0] / X[2], X[1] / X[2]
            du = ((rng.raw() % 10) - 5) * 0.0001
            dv = ((rng.raw() % 10) - 5) * 0.0001
            obs_pose.append(c)
            obs_lm.append(li)
            uv.append((u + du, v + dv))
    poses = np.array([[t[0], t[1], t[2], 0.0, 0.0, 0.0, 1.0] for t in cams_t])
    pf = np.zeros(7, dtype=np.uint8)
    pf[0] = 1
    return scenes.Scene(name="seven_camera", poses=poses, pose_fixed=pf, landmarks=np.array(noisy),
                        landmark_fixed=np.zeros(3, dtype=np.uint8), obs_pose=np.array(obs_pose, dtype=np.int32),
                        obs_landmark=np.array(obs_lm, dtype=np.int32), obs_uv=np.array(uv),
                        intrinsics=(1.0, 1.0, 0.0, 0.0), iterations=50,
                        gt_landmarks=np.array(lms))


def negative_information_scene() -> scenes.Scene:
    """tests/factor_graph.test.cpp:182-224: a negative-definite information
    matrix makes the reduced system indefinite until the damping is large."""
    return scenes.Scene(name="negative_information",
                        poses=np.array([[0, 0, 0, 0, 0, 0, 1.0], [0.1, 0, 0, 0, 0, 0, 1.0]]),
                        pose_fixed=np.array([1, 0], dtype=np.uint8), landmarks=np.array([[0.1, 0.2, 1.0]]),
                        landmark_fixed=np.array([1], dtype=np.uint8), obs_pose=np.array([1], dtype=np.int32),
                        obs_landmark=np.array([0], dtype=np.int32), obs_uv=np.array([[0.15, 0.25]]),
                        obs_info=np.array([[-1.0, 0.0, 0.0, -1.0]]), intrinsics=(1.0, 1.0, 0.0, 0.0),
                        iterations=10)


def scene_arrays(sc: scenes.Scene) -> dict:
    d = dict(poses=sc.poses, pose_fixed=sc.pose_fixed, landmarks=sc.landmarks, landmark_fixed=sc.landmark_fixed,
             obs_pose=sc.obs_pose, obs_landmark=sc.obs_landmark, obs_uv=sc.obs_uv,
             intrinsics=np.array(sc.intrinsics, dtype=np.float64), loss_kind=np.int32(sc.loss_kind),
             loss_delta=np.float64(sc.loss_delta))
    if sc.obs_info is not None:
        d["obs_info"] = sc.obs_info
    return d


def write_edges(ref: Reference, rng: np.random.Generator):
    cases = []
    # literal case of tests/factor_graph.test.cpp:236-276 and the behind-camera case :278-323
    cases.append(([0, 0, 0, 0, 0, 0, 1.0], [0, 0, 1.0], [0.1, -0.2], [1, 1, 0, 0.0]))
    cases.append(([0, 0, 0, 0, 0, 0, 1.0], [0.1, 0.2, -10.0], [0.1, -0.2], [1, 1, 0, 0.0]))
    for _ in range(64):
        q = rng.normal(size=4)
        q /= np.linalg.norm(q)
        if rng.random() < 0.3:
            q *= 1.0 + 0.01 * rng.normal()  # un-normalised quaternions are used as given
        t = rng.normal(size=3)
        X = rng.normal(size=3) * 3.0
        if rng.random() < 0.5:
            X[2] = abs(X[2]) + 2.0
        pose = [t[0], t[1], t[2], q[1], q[2], q[3], q[0]]
        cases.append((pose, list(X), list(rng.uniform(0, 640, 2)), [525.0, 525.0, 320.0, 240.0]))
    P = np.array([c[0] for c in cases], dtype=np.float64)
    X = np.array([c[1] for c in cases], dtype=np.float64)
    UV = np.array([c[2] for c in cases], dtype=np.float64)
    IN = np.array([c[3] for c in cases], dtype=np.float64)
    R = np.zeros((len(cases), 2))
    JP = np.zeros((len(cases), 2, 6))
    JL = np.zeros((len(cases), 2, 3))
    for i in range(len(cases)):
        R[i], JP[i], JL[i] = ref.edge(P[i], X[i], UV[i], IN[i])
    np.savez_compressed(os.path.join(HERE, "edges.npz"), pose=P, X=X, uv=UV, intr=IN, r=R, Jp=JP, Jl=JL)


def write_losses(ref: Reference):
    e2 = np.array([0.0, 1e-6, 0.5, 1.0, 5.0, 5.991, 6.0, 30.0, 1e4])
    rows = []
    for kind in (0, 1, 2, 3):
        for delta in (1.0, math.sqrt(5.991), 3.0):
            for v in e2:
                rows.append([kind, delta, v] + list(ref.loss(kind, delta, v)))
    np.savez_compressed(os.path.join(HERE, "losses.npz"), table=np.array(rows))


def write_invert3(ref: Reference, rng: np.random.Generator):
    As, outs, oks = [], [], []
    for i in range(40):
        A = rng.normal(size=(3, 3))
        if i % 4 == 0:
            A = A @ A.T + 1e-3 * np.eye(3)
        if i % 10 == 5:
            A[2] = A[0] + A[1]  # singular
        if i % 10 == 7:
            A = np.zeros((3, 3))
        ok, out = ref.invert3(A)
        As.append(A)
        outs.append(out)
        oks.append(ok)
    np.savez_compressed(os.path.join(HERE, "invert3.npz"), A=np.array(As), inv=np.array(outs), ok=np.array(oks))


def write_cholesky(ref: Reference, rng: np.random.Generator):
    out = {}
    idx = 0
    mats = []
    # the 6x6 system and exact 2x2 case of tests/matrix_decomposition_cholesky.test.cpp are
    # covered by random SPD systems of those sizes plus larger ones
    for n in (2, 6, 20, 60, 97, 150):
        G = rng.normal(size=(n, n))
        mats.append(G @ G.T + n * np.eye(n))
    mats.append(np.array([[4.0, 2.0], [2.0, 3.0]]))
    mats.append(np.array([[1.0, 2.0], [2.0, 1.0]]))  # indefinite: must fail
    bad = np.eye(3)
    bad[1, 1] = np.nan
    mats.append(bad)  # NaN: must fail
    G = rng.normal(size=(40, 40))
    ill = G @ G.T
    ill[39] = ill[38]
    ill[:, 39] = ill[:, 38]
    mats.append(ill)  # singular
    for A in mats:
        n = A.shape[0]
        b = rng.normal(size=n)
        ok, Lm = ref.cholesky(A)
        okx, x = ref.cholesky_solve(Lm, b) if ok else (False, np.zeros(n))
        out[f"A{idx}"] = A
        out[f"b{idx}"] = b
        out[f"L{idx}"] = Lm
        out[f"x{idx}"] = x
        out[f"ok{idx}"] = np.array([ok, okx])
        idx += 1
    out["count"] = np.array(idx)
    np.savez_compressed(os.path.join(HERE, "cholesky.npz"), **out)


def write_pose_plus(ref: Reference, rng: np.random.Generator):
    P, D, O = [], [], []
    for i in range(40):
        q = rng.normal(size=4)
        q /= np.linalg.norm(q)
        t = rng.normal(size=3)
        pose = np.array([t[0], t[1], t[2], q[1], q[2], q[3], q[0]])
        d = rng.normal(size=6) * (10.0 ** -rng.integers(0, 8))
        if i == 0:
            d = np.zeros(6)
        P.append(pose)
        D.append(d)
        O.append(ref.pose_plus(pose, d))
    np.savez_compressed(os.path.join(HERE, "pose_plus.npz"), pose=np.array(P), delta=np.array(D), out=np.array(O))


def write_solve(ref: Reference, name: str, sc: scenes.Scene, iterations: int, use_relative: bool = False):
    poses, lms, acc, c0, c1, _, _ = ref.solve(sc, iterations, use_relative)
    d = scene_arrays(sc)
    d.update(out_poses=poses, out_landmarks=lms, accepted=np.int32(acc), chi2_before=np.float64(c0),
             chi2_after=np.float64(c1), iterations=np.int32(iterations), use_relative=np.int32(use_relative))
    np.savez_compressed(os.path.join(HERE, f"solve_{name}.npz"), **d)
    print(f"solve_{name}: K={sc.K} L={sc.L} M={sc.M} accepted={acc} chi2 {c0:.6g} -> {c1:.6g}")


def write_cull(ref: Reference):
    """map::cull (source/map.hpp:269-323) on maps with every branch made to
    occur (scenes.cull_map), and the frame rotations map::optimise writes
    back (source/map.hpp:247-251)."""
    for name, (K, L, seed) in {"arc": (8, 600, 61), "arc_b": (10, 900, 62)}.items():
        sc = scenes.arc_scene(K, L, seed=seed)
        cm = scenes.cull_map(sc, seed=seed, truth=True)
        erase, n = ref.map_cull(cm)
        d = {f: getattr(cm, f) for f in cm.__dataclass_fields__}
        d.update(ref_erase=erase, pose=sc.poses, pose_rt=ref.pose_rt(sc.poses))
        np.savez_compressed(os.path.join(HERE, f"cull_{name}.npz"), **d)
        print(f"cull_{name}: F={cm.F} L={cm.L} M={cm.M} erased={n}")


MAP_OPTIMISE_CASES = {  # name: (local_window, fix_landmarks, rounds)
    "global_1": (0, False, 1),
    "window4_1": (4, False, 1),
    "tracking_50": (1, True, 50),
}


def write_map_optimise(ref: Reference):
    """map::optimise (source/map.hpp:65-267) on the map of a light-noise arc
    scene: a global and a windowed round, and the tracking mode (landmarks
    fixed, edges to fixed frames dropped) to convergence."""
    sc = scenes.arc_scene(12, 1000, seed=7, min_obs=2, **scenes.ADJOINT_INIT_NOISE)
    cm = scenes.slam_map(sc)
    d = {f: getattr(cm, f) for f in cm.__dataclass_fields__}
    d["rt_pose"] = ref.rt_pose(cm.frame_pose)
    for name, (lw, fixl, rounds) in MAP_OPTIMISE_CASES.items():
        fp, X = ref.map_optimise(cm, lw, fixl, rounds)
        d[f"{name}_frame_pose"] = fp
        d[f"{name}_landmarks"] = X
    np.savez_compressed(os.path.join(HERE, "map_optimise.npz"), **d)
    print(f"map_optimise: F={cm.F} L={cm.L} M={cm.M}")


MATCH_CASES = [  # (threshold, k, size): zeroslam's call (32, 2, 2 max(n)), ties and wide thresholds,
    (32.0, 2, 1600),  # the capacity rule, k = 1 and the largest k
    (32.0, 1, 1600),
    (100.0, 3, 2400),
    (32.5, 2, 301),
    (130.0, 8, 6400),
]


def write_matches(ref: Reference):
    """feature::find_matches (source/feature.hpp:1190-1235) on descriptor sets
    with near copies (true matches around the threshold) and exact duplicate
    rhs descriptors (ties)."""
    lhs, rhs = scenes.descriptor_pair(700, 800, seed=3)
    d = {"lhs": lhs, "rhs": rhs, "cases": np.array(MATCH_CASES, dtype=np.float64)}
    for c, (thr, k, size) in enumerate(MATCH_CASES):
        m = ref.find_matches(lhs, rhs, thr, k, size)
        d[f"case{c}_lhs"] = m["lhs_index"]
        d[f"case{c}_rhs"] = m["rhs_index"]
        d[f"case{c}_score"] = m["score"]
        print(f"matches case {c}: threshold {thr} k {k} size {size}: {len(m)} matches")
    np.savez_compressed(os.path.join(HERE, "matches.npz"), **d)


def main():
    ref = Reference()
    write_cull(ref)
    write_map_optimise(ref)
    write_matches(ref)
    rng = np.random.default_rng(20261203)
    write_edges(ref, rng)
    write_losses(ref)
    write_invert3(ref, rng)
    write_cholesky(ref, rng)
    write_pose_plus(ref, rng)
    write_solve(ref, "seven_camera", seven_camera_scene(), 50, True)
    write_solve(ref, "negative_information", negative_information_scene(), 10)
    small = scenes.small_scene()
    write_solve(ref, "arc_small_10", small, 10)
    write_solve(ref, "arc_small_1", small, 1)
    write_solve(ref, "arc_huber_1", scenes.arc_scene(10, 500, seed=5, huber=True), 1)
    write_solve(ref, "arc_huber_5", scenes.arc_scene(10, 500, seed=5, huber=True), 5)
    write_solve(ref, "window_k20_1", scenes.arc_scene(20, 1000, seed=11), 1)
    fixed = scenes.arc_scene(12, 400, seed=13)
    fixed.pose_fixed[1] = 1
    fixed.landmark_fixed[::7] = 1
    write_solve(ref, "fixed_mix_3", fixed, 3)


if __name__ == "__main__":
    main()
