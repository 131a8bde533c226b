"""Gradient-check harness for the bundle-adjustment adjoint (test code).

* SE(3) log and its left-Jacobian inverse in numpy, following
  source/lie.hpp:267-308 (so3 log, so3 left-Jacobian inverse), :453-457
  (se3 log) and :459-485 (se3 left Jacobian by its series).
* `converge`: LM solve on the device, then Gauss-Newton polishing steps
  (zs_ba_linear_step with a tiny damping and a host-side exp-map update) until
  the state is the stationary point to machine precision, as finite
  differences of whole solves need.
* `PoseLogLoss`: L = sum over free poses of ||log T_k - log T_k^target||^2
  and its gradient in the solver's local coordinates, 2 J_l^-1(xi)^T (xi - xi_t).
* `BAFunction`: a torch.autograd.Function whose forward converges the problem
  for given pixels and intrinsics and returns the poses' log coordinates, and
  whose backward calls the C ABI adjoint.
* `reference_gradient`: an FP64 reference built from the oracle: the exact
  Hessian and dF/dtheta by central differences of the oracle's analytic
  gradient F = -b (zso_linear_step), then a dense solve.
"""

from __future__ import annotations

import math

import numpy as np

from zeroslam_gb300 import scenes


def _hat(w):
    return np.array([[0.0, -w[2], w[1]], [w[2], 0.0, -w[0]], [-w[1], w[0], 0.0]])


def so3_log(q):
    """q = (w, x, y, z)."""
    w, v = q[0], np.asarray(q[1:4], dtype=np.float64)
    n2 = float(v @ v)
    if n2 < 1e-12:
        mult = 2.0 / w - (2.0 * n2) / (3.0 * w * w * w)
    else:
        n = math.sqrt(n2)
        sgn = 1.0 if w >= 0 else -1.0
        mult = 2.0 * math.atan2(sgn * n, sgn * w) / n
    return mult * v


def so3_left_jacobian_inverse(w):
    th2 = float(w @ w)
    H = _hat(w)
    if th2 < 1e-12:
        return np.eye(3) - 0.5 * H + (H @ H) / 12.0
    th = math.sqrt(th2)
    h = 0.5 * th
    return np.eye(3) - 0.5 * H + ((1.0 - th * math.cos(h) / (2.0 * math.sin(h))) / th2) * (H @ H)


def se3_log(pose7):
    """pose7 = (tx, ty, tz, qx, qy, qz, qw) -> (omega, upsilon)."""
    q = np.array([pose7[6], pose7[3], pose7[4], pose7[5]])
    w = so3_log(q)
    u = so3_left_jacobian_inverse(w) @ np.asarray(pose7[0:3])
    return np.concatenate([w, u])


def se3_left_jacobian(xi):
    ad = np.zeros((6, 6))
    ad[0:3, 0:3] = _hat(xi[0:3])
    ad[3:6, 0:3] = _hat(xi[3:6])
    ad[3:6, 3:6] = _hat(xi[0:3])
    J = np.eye(6)
    P = ad.copy()
    f = 1.0
    for n in range(1, 20):
        f *= n + 1
        J = J + P / f
        P = P @ ad
    return J


def apply_step(poses, lms, delta, pose_fixed, lm_fixed):
    """T <- exp(d) T for free poses, X <- X + d for free landmarks."""
    K = poses.shape[0]
    n = 6 * K
    dp = delta[:n].reshape(K, 6)
    dq, dt = scenes.se3_exp(dp)
    q, t = scenes.unpack_poses(poses)
    qn, tn = scenes.se3_compose(dq, dt, q, t)
    newp = scenes.pack_poses(qn, tn)
    newp[pose_fixed != 0] = poses[pose_fixed != 0]
    newl = lms + delta[n:].reshape(-1, 3) * (lm_fixed == 0)[:, None]
    return newp, newl


def converge(h, sc, lm_iterations=50, polish_steps=4):
    """LM to convergence on the device, then exact Newton polishing."""
    h.set_problem(sc)
    if lm_iterations:
        h.solve(lm_iterations, True)
    return converge_from_state(h, sc, polish_steps)


class PoseLogLoss:
    def __init__(self, targets, pose_fixed):
        self.targets = np.asarray(targets)
        self.free = np.nonzero(np.asarray(pose_fixed) == 0)[0]

    def value(self, poses):
        return float(sum(np.sum((se3_log(poses[k]) - self.targets[k]) ** 2) for k in self.free))

    def grad_local(self, poses):
        """dL/d(left perturbation) per pose, [K, 6]."""
        g = np.zeros((poses.shape[0], 6))
        for k in self.free:
            xi = se3_log(poses[k])
            Jinv = np.linalg.inv(se3_left_jacobian(xi))
            g[k] = 2.0 * Jinv.T @ (xi - self.targets[k])
        return g


def targets_for(sc, seed=7, sigma=0.01):
    rng = np.random.default_rng(seed)
    base = sc.gt_poses if sc.gt_poses is not None else sc.poses
    return np.array([se3_log(p) for p in base]) + sigma * rng.normal(size=(sc.K, 6))


def with_params(sc, uv=None, intrinsics=None):
    s2 = sc.copy()
    if uv is not None:
        s2.obs_uv = np.ascontiguousarray(uv, dtype=np.float64)
    if intrinsics is not None:
        s2.intrinsics = tuple(float(v) for v in intrinsics)
    return s2


def loss_at(h, sc, x_star, loss, uv=None, intrinsics=None, polish_steps=4):
    """L(x*(theta)) re-converged from x* for perturbed pixels / intrinsics."""
    s2 = with_params(sc, uv, intrinsics)
    h.set_problem(s2)
    h.set_state(*x_star)
    s2.poses, s2.landmarks = x_star[0].copy(), x_star[1].copy()
    poses, _ = converge_from_state(h, s2, polish_steps)
    return loss.value(poses)


def converge_from_state(h, sc, polish_steps=4):
    """Newton steps x <- x (+) H^-1 b with the exact Hessian: the adjoint
    solve with a = b (b = -gradient, from zs_ba_linear_step) returns the
    Newton step, so convergence is quadratic."""
    poses, lms = h.get_state()
    K = sc.K
    for _ in range(polish_steps):
        b = h.linear_step(1.0, want_S=False)["b"]
        _, _, rep, v = h.adjoint(b[:6 * K].reshape(K, 6), b[6 * K:].reshape(-1, 3), want_state=True)
        poses, lms = apply_step(poses, lms, v, sc.pose_fixed, sc.landmark_fixed)
        h.set_state(poses, lms)
    return poses, lms


def reference_gradient(oracle, sc, x_star, a_pose, a_lm, hstep=1e-6):
    """FP64 reference dL/duv and dL/dtheta from the oracle (dense, small scenes).

    F(x) = -b(x) is the oracle's analytic gradient in local coordinates; H and
    dF/dtheta come from its central differences; then v = H^-1 a on the free
    variables, dL/duv_o = -J_o v_o (J from the oracle's edge Jacobians)."""
    K, L = sc.K, sc.L
    n = 6 * K
    N = n + 3 * L
    free = np.concatenate([np.repeat(sc.pose_fixed == 0, 6), np.repeat(sc.landmark_fixed == 0, 3)])
    base = sc.copy()
    base.poses, base.landmarks = x_star[0].copy(), x_star[1].copy()

    def F(s):
        return -oracle.linear_step(s, 1.0, want_S=False)["b"]

    H = np.zeros((N, N))
    for j in np.nonzero(free)[0]:
        d = np.zeros(N)
        cols = []
        for sgn in (1.0, -1.0):
            d[:] = 0.0
            d[j] = sgn * hstep
            s = base.copy()
            s.poses, s.landmarks = apply_step(base.poses, base.landmarks, d, sc.pose_fixed, sc.landmark_fixed)
            cols.append(F(s))
        H[:, j] = (cols[0] - cols[1]) / (2.0 * hstep)
    Hf = H[np.ix_(free, free)]
    Hf = 0.5 * (Hf + Hf.T)
    a = np.concatenate([a_pose.reshape(-1), a_lm.reshape(-1)])
    v = np.zeros(N)
    v[free] = np.linalg.solve(Hf, a[free])
    # dL/dtheta = -v^T dF/dtheta
    dth = np.zeros(4)
    for c in range(4):
        Fs = []
        for sgn in (1.0, -1.0):
            intr = list(sc.intrinsics)
            intr[c] += sgn * hstep
            s = with_params(base, intrinsics=intr)
            Fs.append(F(s))
        dth[c] = -v @ ((Fs[0] - Fs[1]) / (2.0 * hstep))
    duv = np.zeros((sc.M, 2))
    for o in range(sc.M):
        pi, li = sc.obs_pose[o], sc.obs_landmark[o]
        _, Jp, Jl, _ = oracle.edge(base.poses[pi], base.landmarks[li], sc.obs_uv[o], sc.intrinsics)
        vo = np.concatenate([v[6 * pi:6 * pi + 6], v[n + 3 * li:n + 3 * li + 3]])
        duv[o] = -(np.concatenate([Jp, Jl], axis=1) @ vo)
    return duv, dth


def make_autograd_function():
    """The torch.autograd.Function over (pixels, intrinsics) -> pose logs."""
    import torch

    from zeroslam_gb300 import ba

    class BAFunction(torch.autograd.Function):
        @staticmethod
        def forward(ctx, uv, intrinsics, scene, lm_iterations):
            s2 = with_params(scene, uv.detach().cpu().numpy(), intrinsics.detach().cpu().numpy())
            h = ba.BundleAdjuster(precision=ba.FP64)
            poses, lms = converge(h, s2, lm_iterations)
            ctx.h, ctx.poses, ctx.scene = h, poses, s2
            logs = np.array([se3_log(p) for p in poses])
            return torch.from_numpy(logs)

        @staticmethod
        def backward(ctx, grad_logs):
            g = grad_logs.detach().cpu().numpy()
            a = np.zeros((ctx.scene.K, 6))
            for k in range(ctx.scene.K):
                if ctx.scene.pose_fixed[k]:
                    continue
                xi = se3_log(ctx.poses[k])
                a[k] = np.linalg.inv(se3_left_jacobian(xi)).T @ g[k]
            duv, dint, _ = ctx.h.adjoint(a, None)
            return torch.from_numpy(duv), torch.from_numpy(dint), None, None

    return BAFunction
