"""Seeded synthetic bundle-adjustment scenes.

Every scene is a problem in the structure-of-arrays form that the C ABI
(`include/zeroslam_ba.h`, `zs_ba_problem`) consumes:

* ``poses``      float64 [K, 7]  (tx, ty, tz, qx, qy, qz, qw), world->camera,
  the parameter order of zeroslam's ``vertex_pose`` (source/factor_graph.hpp:941);
* ``pose_fixed`` uint8 [K]; pose 0 is fixed (the gauge, as in
  tests/factor_graph.test.cpp:118 and source/map.hpp:134);
* ``landmarks``  float64 [L, 3]; ``landmark_fixed`` uint8 [L];
* ``obs_pose``, ``obs_landmark`` int32 [M]; ``obs_uv`` float64 [M, 2];
* ``intrinsics`` (fx, fy, cx, cy) = (525, 525, 320, 240), image 640 x 480.

Random numbers come from PCG32 (the generator and constants of
tests/factor_graph.test.cpp:62-83), run as many independent streams in
lock-step so that numpy can vectorise it, and Gaussian noise from the
Box-Muller transform. The same seed gives the same scene on x86-64 and
aarch64 up to the last bit of libm's log/cos.

Workloads (sizes follow the headline configurations of the bundle-adjustment
benchmark; each builder records the choices it makes in ``meta``):

* ``arc``        K keyframes on a 1 m radius arc spanning 36 degrees, looking
  at the origin; landmarks uniform in x, y in [-2, 2], z in [1, 7] (depth 2-8 m
  from the arc). K=10, L=500 is the small FP64 scene; K=50, L=10000 the
  differentiable-BA scene; random K, L give the batched local windows.
* ``walk``       200 keyframes on a 20 m random walk (0.1 m steps, 3 degree yaw
  jitter), 50,000 landmarks in a 30 x 10 x 30 m box, ~1M observations.
* ``loop``       1,000 keyframes on a 100 m loop, 200,000 landmarks in a
  60 x 15 x 60 m box, ~4M observations, drift growing to 0.5 m / 2 degrees.
"""

from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

WIDTH = 640
HEIGHT = 480
INTRINSICS = (525.0, 525.0, 320.0, 240.0)

_PCG_MULT = np.uint64(0x5851F42D4C957F2D)
_PCG_STATE0 = 0x853C49E6748FEA9B
_PCG_INC0 = 0xDA3E39CB94B95BDB
_GOLDEN = 0x9E3779B97F4A7C15
_M64 = (1 << 64) - 1


class Pcg32Streams:
    """``n`` PCG32 generators advanced together.

    Stream ``s`` of seed ``seed`` starts from the reference test's state and
    increment, offset by the stream and seed numbers (the increment must stay
    odd). Draws are taken step-major: step 0 of every stream, then step 1 ...
    """

    def __init__(self, seed: int, streams: int = 4096):
        s = np.arange(streams, dtype=np.uint64)
        seed_mix = (int(seed) * _GOLDEN) & _M64
        self.state = (np.uint64(_PCG_STATE0 ^ seed_mix) + s * np.uint64(_GOLDEN)).astype(np.uint64)
        self.inc = ((np.uint64(_PCG_INC0) + s * np.uint64(2)) | np.uint64(1)).astype(np.uint64)
        self.n = streams
        for _ in range(3):  # decorrelate neighbouring streams
            self._step()

    def _step(self) -> np.ndarray:
        old = self.state
        with np.errstate(over="ignore"):
            self.state = old * _PCG_MULT + self.inc
        xs = (((old >> np.uint64(18)) ^ old) >> np.uint64(27)).astype(np.uint32)
        rot = (old >> np.uint64(59)).astype(np.uint32)
        return ((xs >> rot) | (xs << ((np.uint32(32) - rot) & np.uint32(31)))).astype(np.uint32)

    def raw(self, count: int) -> np.ndarray:
        steps = (count + self.n - 1) // self.n
        out = np.empty((steps, self.n), dtype=np.uint32)
        for i in range(steps):
            out[i] = self._step()
        return out.reshape(-1)[:count]

    def uniform(self, count: int, lo: float = 0.0, hi: float = 1.0) -> np.ndarray:
        """Uniform in (lo, hi): (x + 0.5) / 2^32 never reaches either end."""
        u = (self.raw(count).astype(np.float64) + 0.5) * (1.0 / 4294967296.0)
        return lo + (hi - lo) * u

    def normal(self, count: int, sigma: float = 1.0) -> np.ndarray:
        half = (count + 1) // 2
        u1 = self.uniform(half)
        u2 = self.uniform(half)
        rad = np.sqrt(-2.0 * np.log(u1))
        z = np.concatenate([rad * np.cos(2.0 * math.pi * u2), rad * np.sin(2.0 * math.pi * u2)])
        return sigma * z[:count]


# ----------------------------------------------------------------------------
# Small SE(3) helpers (quaternion w, x, y, z), following the formulas of
# source/lie.hpp so3::exp (:247-264), so3::left_jacobian (:284-294),
# so3 * so3 (:337-344), so3 * point (:347-362) and se3 * se3 (:521-526).
# ----------------------------------------------------------------------------

def so3_exp(omega: np.ndarray) -> np.ndarray:
    omega = np.atleast_2d(omega)
    th2 = np.sum(omega * omega, axis=1)
    th = np.sqrt(th2)
    small = th2 < 1e-12
    th_safe = np.where(small, 1.0, th)
    real = np.where(small, 1.0 - th2 / 8.0 + th2 * th2 / 384.0, np.cos(0.5 * th_safe))
    scale = np.where(small, 0.5 - th2 / 48.0 + th2 * th2 / 3840.0, np.sin(0.5 * th_safe) / th_safe)
    return np.concatenate([real[:, None], omega * scale[:, None]], axis=1)


def _hat(v: np.ndarray) -> np.ndarray:
    z = np.zeros(v.shape[0])
    return np.stack([np.stack([z, -v[:, 2], v[:, 1]], 1),
                     np.stack([v[:, 2], z, -v[:, 0]], 1),
                     np.stack([-v[:, 1], v[:, 0], z], 1)], 1)


def so3_left_jacobian(omega: np.ndarray) -> np.ndarray:
    omega = np.atleast_2d(omega)
    th2 = np.sum(omega * omega, axis=1)
    th = np.sqrt(th2)
    small = th2 < 1e-12
    th_safe = np.where(small, 1.0, th)
    a = np.where(small, 0.5, (1.0 - np.cos(th_safe)) / np.where(small, 1.0, th2))
    b = np.where(small, 1.0 / 6.0, (th_safe - np.sin(th_safe)) / np.where(small, 1.0, th2 * th_safe))
    h = _hat(omega)
    return np.eye(3)[None] + a[:, None, None] * h + b[:, None, None] * (h @ h)


def quat_mul(p: np.ndarray, q: np.ndarray) -> np.ndarray:
    pw, px, py, pz = p[:, 0], p[:, 1], p[:, 2], p[:, 3]
    qw, qx, qy, qz = q[:, 0], q[:, 1], q[:, 2], q[:, 3]
    return np.stack([pw * qw - px * qx - py * qy - pz * qz,
                     pw * qx + px * qw + py * qz - pz * qy,
                     pw * qy - px * qz + py * qw + pz * qx,
                     pw * qz + px * qy - py * qx + pz * qw], axis=1)


def quat_to_matrix(q: np.ndarray) -> np.ndarray:
    w, x, y, z = q[:, 0], q[:, 1], q[:, 2], q[:, 3]
    return np.stack([
        np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)], 1),
        np.stack([2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)], 1),
        np.stack([2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)], 1)], 1)


def se3_exp(xi: np.ndarray):
    """xi = (omega, upsilon) -> (quaternion wxyz [N,4], translation [N,3])."""
    xi = np.atleast_2d(xi)
    q = so3_exp(xi[:, :3])
    t = np.einsum("nij,nj->ni", so3_left_jacobian(xi[:, :3]), xi[:, 3:])
    return q, t


def se3_compose(qa, ta, qb, tb):
    """(a * b): rotation qa*qb, translation Ra tb + ta."""
    return quat_mul(qa, qb), np.einsum("nij,nj->ni", quat_to_matrix(qa), tb) + ta


def yaw_pose(centre: np.ndarray, heading: np.ndarray):
    """World->camera pose of a camera at ``centre`` looking along yaw ``heading``
    (look direction (sin h, 0, cos h), image y along world +y)."""
    q = so3_exp(np.stack([np.zeros_like(heading), -heading, np.zeros_like(heading)], 1))
    R = quat_to_matrix(q)
    t = -np.einsum("nij,nj->ni", R, centre)
    return q, t


def pack_poses(q: np.ndarray, t: np.ndarray) -> np.ndarray:
    return np.ascontiguousarray(np.concatenate([t, q[:, 1:4], q[:, 0:1]], axis=1))


def unpack_poses(p: np.ndarray):
    q = np.concatenate([p[:, 6:7], p[:, 3:6]], axis=1)
    return q, p[:, 0:3]


def project(q: np.ndarray, t: np.ndarray, X: np.ndarray, intr=INTRINSICS):
    """Camera-frame points and pixels of every (pose, landmark) pair.

    Returns Xc [K, L, 3] and uv [K, L, 2]; callers mask invisible pairs."""
    R = quat_to_matrix(q)
    Xc = np.einsum("kij,lj->kli", R, X) + t[:, None, :]
    z = Xc[..., 2]
    zs = np.where(np.abs(z) < 1e-12, 1e-12, z)
    u = intr[0] * Xc[..., 0] / zs + intr[2]
    v = intr[1] * Xc[..., 1] / zs + intr[3]
    return Xc, np.stack([u, v], axis=-1)


@dataclass
class Scene:
    name: str
    poses: np.ndarray
    pose_fixed: np.ndarray
    landmarks: np.ndarray
    landmark_fixed: np.ndarray
    obs_pose: np.ndarray
    obs_landmark: np.ndarray
    obs_uv: np.ndarray
    intrinsics: tuple = INTRINSICS
    loss_kind: int = 0
    loss_delta: float = 0.0
    obs_info: np.ndarray | None = None
    iterations: int = 10
    gt_poses: np.ndarray | None = None
    gt_landmarks: np.ndarray | None = None
    meta: dict = field(default_factory=dict)

    @property
    def K(self) -> int:
        return int(self.poses.shape[0])

    @property
    def L(self) -> int:
        return int(self.landmarks.shape[0])

    @property
    def M(self) -> int:
        return int(self.obs_pose.shape[0])

    def copy(self) -> "Scene":
        import copy
        return copy.deepcopy(self)


def _observe(q, t, X, rng: Pcg32Streams, sigma_px: float, zmin: float, zmax: float,
             keep: int, min_obs: int = 1, pose_window=None):
    """Visible (pose, landmark) pairs, landmark-major with poses ascending, for
    the first ``keep`` candidate landmarks that at least ``min_obs`` cameras
    see. Visible: zmin <= Z <= zmax and the projection inside [0, 640) x
    [0, 480). Pixel noise N(0, sigma_px^2) is added afterwards.

    ``pose_window(X_chunk) -> int [n, W]`` optionally restricts the poses
    tested for each candidate (it must include every pose that can see it).

    Returns (kept landmark indices into X, obs_pose, obs_landmark, obs_uv);
    obs_landmark indexes the kept landmarks."""
    K = q.shape[0]
    R = quat_to_matrix(q)
    W = K if pose_window is None else pose_window(X[:1]).shape[1]
    chunk = max(256, int(4e6 // W))
    poses, lms, uvs, kept = [], [], [], []
    n_kept = 0
    for l0 in range(0, X.shape[0], chunk):
        Xb = X[l0:l0 + chunk]
        n = Xb.shape[0]
        ks = np.broadcast_to(np.arange(K), (n, K)) if pose_window is None else pose_window(Xb)
        Xc = np.einsum("nwij,nj->nwi", R[ks], Xb) + t[ks]
        z = Xc[..., 2]
        zs = np.where(np.abs(z) < 1e-12, 1e-12, z)
        uv = np.stack([INTRINSICS[0] * Xc[..., 0] / zs + INTRINSICS[2],
                       INTRINSICS[1] * Xc[..., 1] / zs + INTRINSICS[3]], -1)
        vis = (z >= zmin) & (z <= zmax) & (uv[..., 0] >= 0) & (uv[..., 0] < WIDTH) \
            & (uv[..., 1] >= 0) & (uv[..., 1] < HEIGHT)
        good = np.nonzero(vis.sum(axis=1) >= min_obs)[0][: keep - n_kept]
        vis, ks, uv = vis[good], ks[good], uv[good]
        # pose-ascending within each landmark
        order = np.argsort(np.where(vis, ks, K + 1), axis=1, kind="stable")
        vis = np.take_along_axis(vis, order, 1)
        ks = np.take_along_axis(ks, order, 1)
        uv = np.take_along_axis(uv, order[..., None], 1)
        li, wi = np.nonzero(vis)
        poses.append(ks[li, wi].astype(np.int32))
        lms.append((li + n_kept).astype(np.int32))
        uvs.append(uv[li, wi])
        kept.append(good + l0)
        n_kept += good.size
        if n_kept >= keep:
            break
    if n_kept < keep:
        raise ValueError(f"only {n_kept} of {keep} landmarks are visible; enlarge the candidate set")
    obs_pose = np.concatenate(poses)
    obs_lm = np.concatenate(lms)
    obs_uv = np.concatenate(uvs)
    obs_uv = obs_uv + rng.normal(obs_uv.size, sigma_px).reshape(obs_uv.shape)
    return np.concatenate(kept), obs_pose, obs_lm, np.ascontiguousarray(obs_uv)


def _finish(name, q_gt, t_gt, X_gt, obs_pose, obs_lm, obs_uv, q0, t0, X0, iterations, meta,
            loss_kind=0, loss_delta=0.0):
    K = q_gt.shape[0]
    pose_fixed = np.zeros(K, dtype=np.uint8)
    pose_fixed[0] = 1
    return Scene(
        name=name,
        poses=pack_poses(q0, t0),
        pose_fixed=pose_fixed,
        landmarks=np.ascontiguousarray(X0),
        landmark_fixed=np.zeros(X0.shape[0], dtype=np.uint8),
        obs_pose=np.ascontiguousarray(obs_pose, dtype=np.int32),
        obs_landmark=np.ascontiguousarray(obs_lm, dtype=np.int32),
        obs_uv=obs_uv,
        iterations=iterations,
        loss_kind=loss_kind,
        loss_delta=loss_delta,
        gt_poses=pack_poses(q_gt, t_gt),
        gt_landmarks=np.ascontiguousarray(X_gt),
        meta=meta,
    )


def _map_gauge(sc: Scene) -> Scene:
    """zeroslam's gauge for a map with more than two frames: frames 0 and 1
    fixed (source/map.hpp:134). With pose 0 alone the monocular scale is free,
    S is singular along it and only the damping regularises it; at small
    lambda the steps then blow up along that direction and the accept /
    reject sequence of LM depends on rounding."""
    if sc.K > 2:
        sc.pose_fixed[1] = 1
    return sc


def _depth_relative_noise(X, centre, obs_pose, obs_lm, rng, rel):
    """Isotropic Gaussian landmark noise with sigma = rel x the distance from
    the landmark to the first camera that observes it."""
    L = X.shape[0]
    first = np.full(L, -1, dtype=np.int64)
    order = np.argsort(obs_lm, kind="stable")
    lm_sorted = obs_lm[order]
    starts = np.searchsorted(lm_sorted, np.arange(L))
    first = obs_pose[order][np.minimum(starts, len(order) - 1)]
    dist = np.linalg.norm(X - centre[first], axis=1)
    return rel * dist[:, None] * rng.normal(3 * L).reshape(L, 3)


def _perturb_poses(q, t, rng, sig_rot, sig_trans, drift=None):
    """Left-multiplicative perturbation exp(xi) * T for every pose but pose 0."""
    K = q.shape[0]
    xi = np.concatenate([rng.normal(3 * K, sig_rot).reshape(K, 3),
                         rng.normal(3 * K, sig_trans).reshape(K, 3)], axis=1)
    if drift is not None:
        xi = xi + drift
    xi[0] = 0.0
    dq, dt = se3_exp(xi)
    qn, tn = se3_compose(dq, dt, q, t)
    qn[0], tn[0] = q[0], t[0]
    return qn, tn


def arc_scene(K: int = 10, L: int = 500, seed: int = 0, iterations: int = 10,
              sigma_px: float = 1.0, rot_sigma: float = 0.02, trans_sigma: float = 0.05,
              landmark_rel_noise: float = 0.05, huber: bool = False, name: str | None = None,
              min_obs: int = 1) -> Scene:
    """K keyframes on a 1 m radius arc (36 degree span) in the x-z plane, each
    optical axis through the origin; L landmarks uniform in [-2,2]^2 x [1,7]."""
    rng = Pcg32Streams(seed)
    theta = np.deg2rad(-18.0 + 36.0 * np.arange(K) / max(1, K - 1))
    centre = np.stack([np.sin(theta), np.zeros(K), -np.cos(theta)], 1)
    q_gt, t_gt = yaw_pose(centre, -theta)
    C = 2 * L + 64  # candidates; the first L that some camera sees are kept
    X = np.stack([rng.uniform(C, -2.0, 2.0), rng.uniform(C, -2.0, 2.0), rng.uniform(C, 1.0, 7.0)], 1)
    kept, obs_pose, obs_lm, obs_uv = _observe(q_gt, t_gt, X, rng, sigma_px, 1e-12, np.inf, L, min_obs)
    X = X[kept]
    q0, t0 = _perturb_poses(q_gt, t_gt, rng, rot_sigma, trans_sigma)
    X0 = X * (1.0 + landmark_rel_noise * rng.normal(3 * L).reshape(L, 3))
    meta = dict(generator="arc", K=K, L_requested=L, seed=seed, sigma_px=sigma_px,
                rot_sigma=rot_sigma, trans_sigma=trans_sigma)
    kind, delta = (1, math.sqrt(5.991)) if huber else (0, 0.0)
    return _finish(name or f"arc_K{K}_L{L}_s{seed}", q_gt, t_gt, X, obs_pose, obs_lm, obs_uv,
                   q0, t0, X0, iterations, meta, kind, delta)


WALK_DMAX = 7.0


def walk_scene(K: int = 200, L: int = 50000, seed: int = 1, iterations: int = 20,
               dmax: float = WALK_DMAX, sigma_px: float = 1.0, landmark_rel_noise: float = 0.02) -> Scene:
    """20 m random walk (0.1 m steps, yaw jitter N(0, 3 deg) per step) through
    a 30 x 10 x 30 m box of landmarks; observations with depth in [0.5, dmax]."""
    rng = Pcg32Streams(seed)
    yaw = np.cumsum(np.concatenate([[0.0], rng.normal(K - 1, math.radians(3.0))]))
    step = 0.1 * np.stack([np.sin(yaw), np.zeros(K), np.cos(yaw)], 1)
    centre = np.array([0.0, 0.0, -10.0]) + np.concatenate([np.zeros((1, 3)), np.cumsum(step[:-1], 0)])
    q_gt, t_gt = yaw_pose(centre, yaw)
    C = 9 * L  # candidates; the first L seen by two or more cameras are kept
    X = np.stack([rng.uniform(C, -15.0, 15.0), rng.uniform(C, -5.0, 5.0), rng.uniform(C, -15.0, 15.0)], 1)
    kept, obs_pose, obs_lm, obs_uv = _observe(q_gt, t_gt, X, rng, sigma_px, 0.5, dmax, L, 2)
    X = X[kept]
    q0, t0 = _perturb_poses(q_gt, t_gt, rng, 0.01, 0.03)
    X0 = X + _depth_relative_noise(X, centre, obs_pose, obs_lm, rng, landmark_rel_noise)
    meta = dict(generator="walk", K=K, L_requested=L, seed=seed, dmax=dmax, sigma_px=sigma_px,
                landmark_rel_noise=landmark_rel_noise)
    sc = _finish(f"walk_K{K}_L{L}_s{seed}", q_gt, t_gt, X, obs_pose, obs_lm, obs_uv,
                 q0, t0, X0, iterations, meta)
    return _map_gauge(sc)


LOOP_DMAX = 5.6


def loop_scene(K: int = 1000, L: int = 200000, seed: int = 4, iterations: int = 30,
               dmax: float = LOOP_DMAX, sigma_px: float = 0.5, landmark_rel_noise: float = 0.02) -> Scene:
    """K keyframes on a 100 m circular loop looking along the direction of
    travel, landmarks in a 60 x 15 x 60 m box; initial drift grows linearly to
    0.5 m / 2 degrees at the end of the loop."""
    rng = Pcg32Streams(seed)
    r = 100.0 / (2.0 * math.pi)
    a = 2.0 * math.pi * np.arange(K) / K
    centre = np.stack([r * np.cos(a), np.zeros(K), r * np.sin(a)], 1)
    heading = -a  # look along the tangent (-sin a, 0, cos a)
    q_gt, t_gt = yaw_pose(centre, heading)
    # Candidates uniform in the part of the box that the loop's cameras can
    # see (radius r +- 4 m, |y| <= 3 m); the first L seen by two or more
    # cameras are kept. Each candidate is tested against the poses whose arc
    # position is within dmax + 4 m of its own.
    C = 4 * L
    rad = np.sqrt(rng.uniform(C, (r - 4.0) ** 2, (r + 4.0) ** 2))
    ang = rng.uniform(C, 0.0, 2.0 * math.pi)
    X = np.stack([rad * np.cos(ang), rng.uniform(C, -3.0, 3.0), rad * np.sin(ang)], 1)
    half = int(math.ceil((dmax + 4.0) / (r - 4.0) / (2.0 * math.pi) * K)) + 1

    def window(Xb):
        kc = np.round(np.arctan2(Xb[:, 2], Xb[:, 0]) / (2.0 * math.pi) * K).astype(np.int64)
        return (kc[:, None] + np.arange(-half, half + 1)[None, :]) % K

    kept, obs_pose, obs_lm, obs_uv = _observe(q_gt, t_gt, X, rng, sigma_px, 0.5, dmax, L, 2, window)
    X = X[kept]
    axis = rng.normal(3)
    axis /= np.linalg.norm(axis)
    tdir = rng.normal(3)
    tdir /= np.linalg.norm(tdir)
    s = (np.arange(K) / max(1, K - 1))[:, None]
    drift = np.concatenate([s * math.radians(2.0) * axis[None], s * 0.5 * tdir[None]], axis=1)
    q0, t0 = _perturb_poses(q_gt, t_gt, rng, 0.001, 0.003, drift=drift)
    X0 = X + _depth_relative_noise(X, centre, obs_pose, obs_lm, rng, landmark_rel_noise)
    meta = dict(generator="loop", K=K, L_requested=L, seed=seed, dmax=dmax, sigma_px=sigma_px,
                landmark_rel_noise=landmark_rel_noise)
    sc = _finish(f"loop_K{K}_L{L}_s{seed}", q_gt, t_gt, X, obs_pose, obs_lm, obs_uv,
                 q0, t0, X0, iterations, meta)
    return _map_gauge(sc)


def window_batch(n_windows: int = 256, seed: int = 2, iterations: int = 10,
                 k_range=(5, 30), l_range=(200, 3000)) -> list[Scene]:
    """Independent local windows built by the arc generator with keyframe and
    landmark counts drawn uniformly from the given inclusive ranges."""
    rng = Pcg32Streams(seed, streams=64)
    ks = k_range[0] + (rng.raw(n_windows) % (k_range[1] - k_range[0] + 1)).astype(int)
    ls = l_range[0] + (rng.raw(n_windows) % (l_range[1] - l_range[0] + 1)).astype(int)
    return [arc_scene(int(k), int(l), seed=1000 + seed * 10007 + w, iterations=iterations,
                      name=f"window{w}_K{k}_L{l}") for w, (k, l) in enumerate(zip(ks, ls))]


# Named workloads: the small FP64 scene, the 1M-observation scene, the batched
# windows, the differentiable scene and the 4M-observation loop.
def small_scene(seed: int = 0) -> Scene:
    return arc_scene(10, 500, seed=seed, iterations=10)


def large_scene(seed: int = 1) -> Scene:
    return walk_scene(seed=seed)


ADJOINT_INIT_NOISE = dict(rot_sigma=0.002, trans_sigma=0.005, landmark_rel_noise=0.005)


def adjoint_scene(K: int = 50, L: int = 10000, seed: int = 3) -> Scene:
    """The differentiable-BA scene: the arc generator at 50 keyframes and
    10,000 landmarks, every landmark seen at least twice, and poses 0 and 1
    fixed (zeroslam's own gauge for windows of more than two frames,
    source/map.hpp:134), so the converged solution is an isolated point.
    The initial guess is close to the truth (0.1 degree, 5 mm, 0.5% of the
    landmark coordinates), as for a tracked estimate that is refined: from
    the generator's default 5% landmark noise a few landmarks settle in poor
    local minima (behind a camera, or on a near-degenerate ray) and the
    Hessian at the solution is singular to working precision."""
    sc = arc_scene(K, L, seed=seed, iterations=50, min_obs=2, name=f"adjoint_K{K}_L{L}_s{seed}",
                   **ADJOINT_INIT_NOISE)
    sc.pose_fixed[1] = 1
    return sc


def loop_large_scene(seed: int = 4) -> Scene:
    return loop_scene(seed=seed)


# ---------------------------------------------------------------- map culling

@dataclass
class CullMap:
    """A zeroslam map as the arrays of ``zs_map_cull_input`` (include/zeroslam_ba.h):
    frames (rotation and translation [F, 12], intrinsics [F, 4], ids [F]),
    landmarks (ids [L], locations [L, 3]), each landmark's observations in
    order (ranges ``landmark_obs`` [L+1]; observing frame index, -1 for a
    frame not in the map; observing frame id; float32 keypoint [M, 2]) and
    the two id generators."""
    frame_pose: np.ndarray
    frame_intrinsics: np.ndarray
    frame_id: np.ndarray
    landmark_id: np.ndarray
    landmarks: np.ndarray
    landmark_obs: np.ndarray
    obs_frame: np.ndarray
    obs_frame_id: np.ndarray
    obs_keypoint: np.ndarray
    landmark_id_generator: int
    frame_id_generator: int

    @property
    def F(self) -> int:
        return int(self.frame_pose.shape[0])

    @property
    def L(self) -> int:
        return int(self.landmarks.shape[0])

    @property
    def M(self) -> int:
        return int(self.obs_frame.shape[0])


def frames_from_poses(poses: np.ndarray) -> np.ndarray:
    """[K, 12] rotation (row-major) and translation of [K, 7] poses."""
    q, t = unpack_poses(poses)
    R = quat_to_matrix(q)
    return np.ascontiguousarray(np.concatenate([R.reshape(-1, 9), t], axis=1))


def cull_map(sc: Scene, seed: int = 0, frame_pose: np.ndarray | None = None, plain: bool = False,
             truth: bool = False) -> CullMap:
    """The map of a scene at its current state (``truth``: at its ground
    truth, where the pixel errors are the observation noise), for map culling.

    Each landmark's observations keep the scene's order. ``plain`` gives the
    scene itself: every frame in the map, the scene's pixels rounded to
    float32 (zeroslam's keypoints are float), one camera, every landmark and
    frame recent. Otherwise every branch of the cull is made to occur, in
    proportions drawn from ``seed``: half the landmark ids older than the
    newest 500; landmarks cut to 1-4 observations, a frame id generator that
    leaves most frames older than the newest 7; landmarks without
    observations; observations whose frame is not in the map (and landmarks
    with no frame in the map at all); landmarks moved behind a camera that
    sees them; keypoints shifted by up to 10 px so that the mean errors
    straddle 5.991; and intrinsics that differ between frames.
    ``frame_pose`` overrides the frames' rotations and translations."""
    K, L = sc.K, sc.L
    order = np.argsort(sc.obs_landmark, kind="stable")
    obs_lm = sc.obs_landmark[order].astype(np.int64)
    obs_pose = sc.obs_pose[order].astype(np.int32)
    uv = sc.obs_uv[order].astype(np.float64)
    poses = sc.gt_poses if truth else sc.poses
    X = np.array(sc.gt_landmarks if truth else sc.landmarks, dtype=np.float64, copy=True)
    Rt = frames_from_poses(poses) if frame_pose is None else np.ascontiguousarray(frame_pose, dtype=np.float64)
    intr = np.tile(np.asarray(sc.intrinsics, dtype=np.float64), (K, 1))
    frame_id = np.arange(K, dtype=np.int32) + 10
    landmark_id = np.arange(L, dtype=np.int32) + 1000
    obs_frame = obs_pose.copy()
    keep = np.ones(obs_lm.shape[0], dtype=bool)
    if plain:
        kp = uv.astype(np.float32)
        counts = np.bincount(obs_lm, minlength=L)
        ptr = np.zeros(L + 1, dtype=np.int64)
        np.cumsum(counts, out=ptr[1:])
        return CullMap(Rt, intr, frame_id, landmark_id, X, ptr, obs_frame, frame_id[obs_frame], kp,
                       int(landmark_id[0]), int(frame_id[0]))
    rng = np.random.default_rng(seed)
    intr[:, 0] *= 1.0 + 0.01 * (np.arange(K) % 3)
    # keypoints shifted per landmark: a third by up to 10 px
    shift = np.where(rng.random(L) < 0.35, rng.uniform(0.0, 10.0, L), 0.0)
    ang = rng.uniform(0.0, 2.0 * math.pi, L)
    uv = uv + (shift[:, None] * np.stack([np.cos(ang), np.sin(ang)], 1))[obs_lm]
    kp = uv.astype(np.float32)
    counts = np.bincount(obs_lm, minlength=L)
    first = np.zeros(L + 1, dtype=np.int64)
    np.cumsum(counts, out=first[1:])
    rank = np.arange(obs_lm.shape[0]) - first[obs_lm]
    # 20% of the landmarks keep only their first 1-4 observations, 5% none
    cut = rng.random(L)
    nkeep = np.where(cut < 0.20, rng.integers(1, 5, L), np.where(cut < 0.25, 0, counts))
    keep &= rank < nkeep[obs_lm]
    # observations from frames that are not in the map: 5% of all, and every
    # observation of 2% of the landmarks
    gone = rng.random(obs_lm.shape[0]) < 0.05
    gone |= (rng.random(L) < 0.02)[obs_lm]
    obs_frame[gone] = -1
    obs_frame_id = np.where(gone, 100000 + rng.integers(0, 1000, obs_lm.shape[0]), frame_id[obs_pose]).astype(np.int32)
    # 3% of the landmarks behind the first camera that sees them (2 m along
    # its optical axis backwards, from its centre)
    back = np.flatnonzero((rng.random(L) < 0.03) & (counts > 0))
    k0 = obs_pose[first[back]]
    R = Rt[k0, :9].reshape(-1, 3, 3)
    c = -np.einsum("nji,nj->ni", R, Rt[k0, 9:])
    X[back] = c - 2.0 * R[:, 2, :]
    obs_frame, obs_frame_id, kp, obs_lm = obs_frame[keep], obs_frame_id[keep], kp[keep], obs_lm[keep]
    ptr = np.zeros(L + 1, dtype=np.int64)
    np.cumsum(np.bincount(obs_lm, minlength=L), out=ptr[1:])
    return CullMap(Rt, intr, frame_id, landmark_id, X, ptr, np.ascontiguousarray(obs_frame, dtype=np.int32),
                   np.ascontiguousarray(obs_frame_id), np.ascontiguousarray(kp), 1000 + L // 2 + 500,
                   int(frame_id[-1]) + 4)


def slam_map(sc: Scene) -> CullMap:
    """A scene at its current state as a zeroslam map for map::optimise:
    frame ids 0..K-1 (0 and 1 are the map's gauge, source/map.hpp:89,134),
    landmark ids 0..L-1, one camera, float32 keypoints, every observing
    frame in the map, both id generators one past the last id."""
    cm = cull_map(sc, plain=True)
    cm.frame_id = np.arange(sc.K, dtype=np.int32)
    cm.obs_frame_id = cm.frame_id[cm.obs_frame].astype(np.int32)
    cm.landmark_id = np.arange(sc.L, dtype=np.int32)
    cm.landmark_id_generator = sc.L
    cm.frame_id_generator = sc.K
    return cm


# ---------------------------------------------------------------- descriptors

def descriptor_pair(n_lhs: int, n_rhs: int, seed: int = 0, near: float = 0.6, dup: float = 0.05):
    """Two sets of 256-bit binary descriptors (uint8 [n, 32]) for matching.
    rhs: uniform random bits, with a fraction ``dup`` of them exact copies of
    other rhs descriptors (equal distances, so ties occur). lhs: a fraction
    ``near`` are copies of a random rhs descriptor with 0-40 bits flipped
    (true matches near zeroslam's threshold of 32), the rest uniform random
    (distance ~128 to everything)."""
    rng = np.random.default_rng(seed)
    rhs = rng.integers(0, 256, size=(n_rhs, 32), dtype=np.uint8)
    if n_rhs > 1:
        d = np.flatnonzero(rng.random(n_rhs) < dup)
        rhs[d] = rhs[rng.integers(0, n_rhs, d.size)]
    lhs = rng.integers(0, 256, size=(n_lhs, 32), dtype=np.uint8)
    if n_rhs > 0:
        nr = np.flatnonzero(rng.random(n_lhs) < near)
        lhs[nr] = rhs[rng.integers(0, n_rhs, nr.size)]
        bits = np.unpackbits(lhs[nr], axis=1)
        flips = rng.integers(0, 41, nr.size)
        for row, f in enumerate(flips):
            bits[row, rng.choice(256, size=f, replace=False)] ^= 1
        lhs[nr] = np.packbits(bits, axis=1)
    return lhs, rhs
