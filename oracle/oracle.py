"""ctypes access to the oracle (test infrastructure only).

``Oracle`` wraps the C restatement ``ba_oracle.c``; ``Reference`` wraps the
reference's own solver compiled by ``build.py`` into ``oracle/_ref``. Both
take scenes in the structure-of-arrays form of ``zeroslam_gb300.scenes``.
Only tests/, the smoke check and bench.py's CPU-baseline leg use this module.
"""

from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_up = C.POINTER(C.c_ubyte)


def _ptr(a: np.ndarray | None, t):
    if a is None:
        return None
    return a.ctypes.data_as(t)


class _Problem(C.Structure):
    _fields_ = [("num_poses", C.c_int), ("num_landmarks", C.c_int), ("num_obs", C.c_longlong),
                ("poses", _dp), ("pose_fixed", _up), ("landmarks", _dp), ("landmark_fixed", _up),
                ("obs_pose", _ip), ("obs_landmark", _ip), ("obs_uv", _dp), ("obs_info", _dp),
                ("intrinsics", C.c_double * 4), ("loss_kind", C.c_int), ("loss_delta", C.c_double)]


class Report(C.Structure):
    _fields_ = [("iterations", C.c_int), ("accepted", C.c_int), ("attempts", C.c_int),
                ("chol_failures", C.c_int), ("chi2_initial", C.c_double), ("chi2_final", C.c_double),
                ("lambda_final", C.c_double)]


class _Arrays:
    """Contiguous copies of a scene's arrays that stay alive with the struct."""

    def __init__(self, scene):
        self.poses = np.ascontiguousarray(scene.poses, dtype=np.float64).copy()
        self.landmarks = np.ascontiguousarray(scene.landmarks, dtype=np.float64).copy()
        self.pose_fixed = np.ascontiguousarray(scene.pose_fixed, dtype=np.uint8)
        self.landmark_fixed = np.ascontiguousarray(scene.landmark_fixed, dtype=np.uint8)
        self.obs_pose = np.ascontiguousarray(scene.obs_pose, dtype=np.int32)
        self.obs_landmark = np.ascontiguousarray(scene.obs_landmark, dtype=np.int32)
        self.obs_uv = np.ascontiguousarray(scene.obs_uv, dtype=np.float64)
        self.obs_info = None if scene.obs_info is None else np.ascontiguousarray(scene.obs_info, dtype=np.float64)
        self.intrinsics = np.ascontiguousarray(scene.intrinsics, dtype=np.float64)
        self.loss_kind = int(scene.loss_kind)
        self.loss_delta = float(scene.loss_delta)

    def struct(self) -> _Problem:
        p = _Problem()
        p.num_poses = self.poses.shape[0]
        p.num_landmarks = self.landmarks.shape[0]
        p.num_obs = self.obs_pose.shape[0]
        p.poses = _ptr(self.poses, _dp)
        p.pose_fixed = _ptr(self.pose_fixed, _up)
        p.landmarks = _ptr(self.landmarks, _dp)
        p.landmark_fixed = _ptr(self.landmark_fixed, _up)
        p.obs_pose = _ptr(self.obs_pose, _ip)
        p.obs_landmark = _ptr(self.obs_landmark, _ip)
        p.obs_uv = _ptr(self.obs_uv, _dp)
        p.obs_info = _ptr(self.obs_info, _dp)
        for i in range(4):
            p.intrinsics[i] = self.intrinsics[i]
        p.loss_kind = self.loss_kind
        p.loss_delta = self.loss_delta
        return p


class _CullMap(C.Structure):
    _fields_ = [("num_frames", C.c_int), ("frame_pose", _dp), ("frame_intrinsics", _dp),
                ("num_landmarks", C.c_int), ("landmark_id", _ip), ("landmarks", _dp),
                ("landmark_obs", C.POINTER(C.c_longlong)), ("obs_frame", _ip), ("obs_frame_id", _ip),
                ("obs_keypoint", C.POINTER(C.c_float)), ("landmark_id_generator", C.c_int),
                ("frame_id_generator", C.c_int)]


def _cull_arrays(cm) -> dict:
    return dict(
        frame_pose=np.ascontiguousarray(cm.frame_pose, dtype=np.float64),
        frame_intrinsics=np.ascontiguousarray(cm.frame_intrinsics, dtype=np.float64),
        frame_id=np.ascontiguousarray(cm.frame_id, dtype=np.int32),
        landmark_id=np.ascontiguousarray(cm.landmark_id, dtype=np.int32),
        landmarks=np.ascontiguousarray(cm.landmarks, dtype=np.float64),
        landmark_obs=np.ascontiguousarray(cm.landmark_obs, dtype=np.int64),
        obs_frame=np.ascontiguousarray(cm.obs_frame, dtype=np.int32),
        obs_frame_id=np.ascontiguousarray(cm.obs_frame_id, dtype=np.int32),
        obs_keypoint=np.ascontiguousarray(cm.obs_keypoint, dtype=np.float32),
    )


MATCH_DTYPE = np.dtype([("lhs_index", np.uint64), ("rhs_index", np.uint64), ("score", np.float32)], align=True)


def _find_matches(fn, lhs, rhs, threshold, k, size):
    lhs = np.ascontiguousarray(lhs, dtype=np.uint8).reshape(-1, 32)
    rhs = np.ascontiguousarray(rhs, dtype=np.uint8).reshape(-1, 32)
    out = np.zeros(max(int(size), 1), dtype=MATCH_DTYPE)
    n = fn(_ptr(lhs, _up), lhs.shape[0], _ptr(rhs, _up), rhs.shape[0], float(threshold), int(k),
           out.ctypes.data_as(C.c_void_p), int(size))
    return out[:n].copy()


def default_threads() -> int:
    """Host threads for the restatement's loops: every core, at most 16
    (its results do not depend on the count)."""
    return max(1, min(16, os.cpu_count() or 1))


class Oracle:
    def __init__(self, threads: int | None = None):
        self.lib = C.CDLL(_build.build_oracle())
        L = self.lib
        L.zso_set_threads.restype = None
        L.zso_set_threads.argtypes = [C.c_int]
        L.zso_get_threads.restype = C.c_int
        L.zso_get_threads.argtypes = []
        self.set_threads(default_threads() if threads is None else threads)
        L.zso_chi2.restype = C.c_double
        L.zso_chi2.argtypes = [C.POINTER(_Problem)]
        L.zso_solve.restype = C.c_int
        L.zso_solve.argtypes = [C.POINTER(_Problem), C.c_int, C.c_int, C.POINTER(Report)]
        L.zso_lm_begin.restype = C.c_void_p
        L.zso_lm_begin.argtypes = [C.POINTER(_Problem), C.c_int]
        L.zso_lm_iteration.restype = C.c_int
        L.zso_lm_iteration.argtypes = [C.c_void_p]
        L.zso_lm_end.restype = C.c_int
        L.zso_lm_end.argtypes = [C.c_void_p, C.POINTER(Report)]
        L.zso_lm_report.restype = None
        L.zso_lm_report.argtypes = [C.c_void_p, C.POINTER(Report)]
        L.zso_linear_step.restype = C.c_int
        L.zso_linear_step.argtypes = [C.POINTER(_Problem), C.c_double, _dp, _dp, _dp, _dp, _dp, _dp]
        L.zso_initial_lambda.restype = C.c_double
        L.zso_initial_lambda.argtypes = [C.POINTER(_Problem)]
        L.zso_edge.restype = C.c_int
        L.zso_edge.argtypes = [_dp, _dp, _dp, _dp, _dp, _dp, _dp]
        L.zso_cholesky.restype = C.c_int
        L.zso_cholesky.argtypes = [_dp, C.c_int, _dp]
        L.zso_cholesky_solve.restype = C.c_int
        L.zso_cholesky_solve.argtypes = [_dp, _dp, C.c_int, _dp]
        L.zso_invert3.restype = C.c_int
        L.zso_invert3.argtypes = [_dp, _dp]
        L.zso_pose_plus.restype = None
        L.zso_pose_plus.argtypes = [_dp, _dp]
        L.zso_loss.restype = None
        L.zso_loss.argtypes = [C.c_int, C.c_double, C.c_double, _dp]
        L.zso_map_cull.restype = C.c_longlong
        L.zso_map_cull.argtypes = [C.POINTER(_CullMap), _up, C.POINTER(C.c_float)]
        L.zso_pose_rt.restype = None
        L.zso_pose_rt.argtypes = [_dp, _dp]
        L.zso_rt_pose.restype = None
        L.zso_rt_pose.argtypes = [_dp, _dp]
        L.zso_find_matches.restype = C.c_longlong
        L.zso_find_matches.argtypes = [_up, C.c_longlong, _up, C.c_longlong, C.c_float, C.c_longlong, C.c_void_p,
                                       C.c_longlong]

    def set_threads(self, n: int) -> None:
        """Host threads of the restatement's loops (process-wide)."""
        self.lib.zso_set_threads(int(n))

    @property
    def threads(self) -> int:
        return int(self.lib.zso_get_threads())

    def find_matches(self, lhs, rhs, threshold: float, k: int, size: int):
        """feature::find_matches: structured array of (lhs_index, rhs_index, score)."""
        return _find_matches(self.lib.zso_find_matches, lhs, rhs, threshold, k, size)

    def rt_pose(self, frame_pose):
        """[F, 7] vertex_pose parameters map::optimise builds from [F, 12] frames."""
        Rt = np.ascontiguousarray(frame_pose, dtype=np.float64).reshape(-1, 12)
        out = np.zeros((Rt.shape[0], 7))
        for f in range(Rt.shape[0]):
            self.lib.zso_rt_pose(_ptr(Rt[f], _dp), _ptr(out[f], _dp))
        return out

    def map_optimise(self, cm, local_window: int, fix_landmarks: bool, rounds: int, use_relative: bool = False):
        """map::map::optimise (source/map.hpp:65-267) restated over a
        ``scenes.CullMap``: window selection (79-127), the graph (129-179,
        frames in array order, landmarks in array order, each landmark's
        edges in observation order), removal of poses without edges
        (181-192), the two early returns (195-233), the solve with
        loss_huber(sqrt(5.991)) (236) and the write-back (239-252).
        Returns (frame_pose [F, 12], landmarks [L, 3], info); the inputs are
        not modified."""
        from zeroslam_gb300.scenes import Scene

        F, L = cm.F, cm.L
        fp = np.array(cm.frame_pose, dtype=np.float64, copy=True)
        X = np.array(cm.landmarks, dtype=np.float64, copy=True)
        info = {"status": 1, "frames": 0, "landmarks": 0, "edges": 0}
        if F == 0:
            return fp, X, info
        fid = [int(v) for v in cm.frame_id]
        ptr = cm.landmark_obs
        below = int(cm.frame_id_generator) - 1 - local_window
        fixed_below = below + 1

        def is_fixed(i, windowed):
            return i == 0 or (i == 1 and F > 2) or (windowed and i < fixed_below)

        if local_window > 0:
            active = [not is_fixed(i, True) for i in fid]
            horizon = int(cm.frame_id_generator) - 1 - 2 * local_window
            relevant = [False] * F
            active_lm = [False] * L
            for l in range(L):
                obs = range(int(ptr[l]), int(ptr[l + 1]))
                if any(cm.obs_frame[o] >= 0 and active[cm.obs_frame[o]] for o in obs):
                    active_lm[l] = True
                    for o in obs:
                        if cm.obs_frame[o] >= 0 and cm.obs_frame_id[o] >= horizon:
                            relevant[cm.obs_frame[o]] = True
            relevant = [r or a for r, a in zip(relevant, active)]
        else:
            relevant = [True] * F
            active_lm = [True] * L
        pose_fixed = [is_fixed(fid[f], local_window > 0) for f in range(F)]
        poses7 = self.rt_pose(fp)
        lm_of, obs_pose, obs_lm, obs_uv, edge_obs = {}, [], [], [], []
        for l in range(L):
            if not active_lm[l]:
                continue
            for o in range(int(ptr[l]), int(ptr[l + 1])):
                f = int(cm.obs_frame[o])
                if f < 0 or not relevant[f]:
                    continue
                if pose_fixed[f] and fix_landmarks:
                    continue
                if l not in lm_of:
                    lm_of[l] = len(lm_of)
                obs_pose.append(f)
                obs_lm.append(lm_of[l])
                edge_obs.append(o)
                obs_uv.append([float(cm.obs_keypoint[o, 0]), float(cm.obs_keypoint[o, 1])])
        has_edge = [False] * F
        for f in obs_pose:
            has_edge[f] = True
        problem_frames = [f for f in range(F) if relevant[f] and has_edge[f]]
        nf_poses = sum(1 for f in problem_frames if not pose_fixed[f])
        nf_lms = 0 if fix_landmarks else len(lm_of)
        info.update(frames=nf_poses, landmarks=nf_lms, edges=len(obs_pose), problem_frames=problem_frames,
                    problem_landmarks=sorted(lm_of, key=lambda l: lm_of[l]), edge_obs=edge_obs,
                    written=[bool(r) for r in relevant])
        if nf_poses == 0 and nf_lms == 0:
            info["status"] = 2
            return fp, X, info
        if not any(relevant) or not lm_of:
            info["status"] = 1
            return fp, X, info
        pidx = {f: i for i, f in enumerate(problem_frames)}
        lms = sorted(lm_of, key=lambda l: lm_of[l])
        sc = Scene(name="map", poses=poses7[problem_frames].copy(),
                   pose_fixed=np.array([pose_fixed[f] for f in problem_frames], dtype=np.uint8),
                   landmarks=X[lms].copy(), landmark_fixed=np.full(len(lms), int(bool(fix_landmarks)), dtype=np.uint8),
                   obs_pose=np.array([pidx[f] for f in obs_pose], dtype=np.int32),
                   obs_landmark=np.array(obs_lm, dtype=np.int32), obs_uv=np.array(obs_uv, dtype=np.float64),
                   intrinsics=tuple(float(v) for v in cm.frame_intrinsics[0]), loss_kind=1,
                   loss_delta=float(np.sqrt(5.991)))
        P, Lm, rep = self.solve(sc, rounds, use_relative)
        for f in range(F):
            if relevant[f]:
                fp[f] = self.pose_rt(P[pidx[f]] if f in pidx else poses7[f])[0]
        X[lms] = Lm
        info.update(status=0, accepted=rep.accepted, chi2_initial=rep.chi2_initial, chi2_final=rep.chi2_final,
                    scene=sc, problem_frames=problem_frames, problem_landmarks=lms)
        return fp, X, info

    def map_cull(self, cm):
        """map::cull of a ``scenes.CullMap``: (erase uint8 [L], mean error float32 [L], erased)."""
        a = _cull_arrays(cm)
        m = _CullMap(a["frame_pose"].shape[0], _ptr(a["frame_pose"], _dp), _ptr(a["frame_intrinsics"], _dp),
                     a["landmark_id"].shape[0], _ptr(a["landmark_id"], _ip), _ptr(a["landmarks"], _dp),
                     _ptr(a["landmark_obs"], C.POINTER(C.c_longlong)), _ptr(a["obs_frame"], _ip),
                     _ptr(a["obs_frame_id"], _ip), _ptr(a["obs_keypoint"], C.POINTER(C.c_float)),
                     int(cm.landmark_id_generator), int(cm.frame_id_generator))
        L = a["landmark_id"].shape[0]
        erase = np.zeros(L, dtype=np.uint8)
        mean = np.zeros(L, dtype=np.float32)
        n = self.lib.zso_map_cull(C.byref(m), _ptr(erase, _up), _ptr(mean, C.POINTER(C.c_float)))
        return erase, mean, int(n)

    def pose_rt(self, poses):
        """[K, 12] rotation and translation map::optimise writes back from [K, 7] poses."""
        P = np.ascontiguousarray(poses, dtype=np.float64).reshape(-1, 7)
        out = np.zeros((P.shape[0], 12))
        for k in range(P.shape[0]):
            self.lib.zso_pose_rt(_ptr(P[k], _dp), _ptr(out[k], _dp))
        return out

    def chi2(self, scene) -> float:
        a = _Arrays(scene)
        p = a.struct()
        return self.lib.zso_chi2(C.byref(p))

    def solve(self, scene, iterations: int, use_relative: bool = False):
        """Returns (poses, landmarks, Report)."""
        a = _Arrays(scene)
        p = a.struct()
        rep = Report()
        self.lib.zso_solve(C.byref(p), int(iterations), int(bool(use_relative)), C.byref(rep))
        return a.poses, a.landmarks, rep

    def stepwise(self, scene, use_relative: bool = False) -> "StepwiseSolve":
        """The solve of ``solve`` one outer LM iteration at a time (for timing
        a solve iteration by iteration)."""
        return StepwiseSolve(self, scene, use_relative)

    def initial_lambda(self, scene) -> float:
        a = _Arrays(scene)
        p = a.struct()
        return self.lib.zso_initial_lambda(C.byref(p))

    def linear_step(self, scene, lam: float, want_S: bool = True):
        """One linearisation + damped solve. Returns dict(ok, S, bs, delta, b, hpp, hll)."""
        a = _Arrays(scene)
        p = a.struct()
        K, L = scene.K, scene.L
        n = 6 * K
        S = np.zeros((n, n)) if want_S else None
        bs = np.zeros(n)
        delta = np.zeros(n + 3 * L)
        b = np.zeros(n + 3 * L)
        hpp = np.zeros((K, 6, 6))
        hll = np.zeros((L, 3, 3))
        ok = self.lib.zso_linear_step(C.byref(p), float(lam), _ptr(S, _dp), _ptr(bs, _dp), _ptr(delta, _dp),
                                      _ptr(b, _dp), _ptr(hpp, _dp), _ptr(hll, _dp))
        return dict(ok=bool(ok), S=S, bs=bs, delta=delta, b=b, hpp=hpp, hll=hll)

    def edge(self, pose7, X3, uv2, intr4):
        pose7, X3, uv2, intr4 = (np.ascontiguousarray(v, dtype=np.float64) for v in (pose7, X3, uv2, intr4))
        r = np.zeros(2)
        Jp = np.zeros((2, 6))
        Jl = np.zeros((2, 3))
        front = self.lib.zso_edge(_ptr(pose7, _dp), _ptr(X3, _dp), _ptr(uv2, _dp), _ptr(intr4, _dp),
                                  _ptr(r, _dp), _ptr(Jp, _dp), _ptr(Jl, _dp))
        return r, Jp, Jl, bool(front)

    def cholesky(self, A):
        A = np.ascontiguousarray(A, dtype=np.float64)
        n = A.shape[0]
        Lm = np.zeros_like(A)
        ok = self.lib.zso_cholesky(_ptr(A, _dp), n, _ptr(Lm, _dp))
        return bool(ok), Lm

    def cholesky_solve(self, Lm, b):
        Lm = np.ascontiguousarray(Lm, dtype=np.float64)
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.zeros_like(b)
        ok = self.lib.zso_cholesky_solve(_ptr(Lm, _dp), _ptr(b, _dp), Lm.shape[0], _ptr(x, _dp))
        return bool(ok), x

    def invert3(self, A):
        A = np.ascontiguousarray(A, dtype=np.float64)
        out = np.zeros((3, 3))
        ok = self.lib.zso_invert3(_ptr(A, _dp), _ptr(out, _dp))
        return bool(ok), out

    def pose_plus(self, pose7, d6):
        pose = np.ascontiguousarray(pose7, dtype=np.float64).copy()
        d6 = np.ascontiguousarray(d6, dtype=np.float64)
        self.lib.zso_pose_plus(_ptr(pose, _dp), _ptr(d6, _dp))
        return pose

    def loss(self, kind, delta, e2):
        rho = np.zeros(3)
        self.lib.zso_loss(int(kind), float(delta), float(e2), _ptr(rho, _dp))
        return rho


class StepwiseSolve:
    """Oracle.solve split into its parts: construction linearises and sets the
    initial damping (zso_lm_begin), ``iteration()`` runs one outer LM
    iteration and returns False once a stop rule has fired, ``report()``
    reads the Report so far and ``finish()`` returns (poses, landmarks,
    Report)."""

    def __init__(self, oracle: "Oracle", scene, use_relative: bool = False):
        self.lib = oracle.lib
        self.a = _Arrays(scene)
        self.p = self.a.struct()
        self.m = self.lib.zso_lm_begin(C.byref(self.p), int(bool(use_relative)))
        if not self.m:
            raise MemoryError("zso_lm_begin")

    def iteration(self) -> bool:
        return bool(self.lib.zso_lm_iteration(self.m))

    def report(self):
        """The Report of the iterations run so far."""
        rep = Report()
        self.lib.zso_lm_report(self.m, C.byref(rep))
        return rep

    def finish(self):
        rep = Report()
        self.lib.zso_lm_end(self.m, C.byref(rep))
        self.m = None
        return self.a.poses, self.a.landmarks, rep

    def __del__(self):
        if getattr(self, "m", None):
            self.lib.zso_lm_end(self.m, None)
            self.m = None


class Reference:
    """zeroslam's own factor_graph, compiled from the reference tree."""

    def __init__(self, path: str | None = None):
        path = path or _build.build_ref()
        if path is None or not os.path.exists(path):
            raise FileNotFoundError("the reference solver has not been built (oracle/_ref)")
        self.lib = C.CDLL(path)
        L = self.lib
        args = [C.c_int, C.c_int, C.c_longlong, _dp, _up, _dp, _up, _ip, _ip, _dp, _dp, _dp, C.c_int, C.c_double]
        L.zsref_solve.restype = C.c_int
        L.zsref_solve.argtypes = args + [C.c_int, C.c_int, _dp]
        L.zsref_chi2.restype = C.c_double
        L.zsref_chi2.argtypes = args
        L.zsref_edge.restype = None
        L.zsref_edge.argtypes = [_dp] * 7
        L.zsref_cholesky.restype = C.c_int
        L.zsref_cholesky.argtypes = [_dp, C.c_int, _dp]
        L.zsref_cholesky_solve.restype = C.c_int
        L.zsref_cholesky_solve.argtypes = [_dp, _dp, C.c_int, _dp]
        L.zsref_invert3.restype = C.c_int
        L.zsref_invert3.argtypes = [_dp, _dp]
        L.zsref_pose_plus.restype = None
        L.zsref_pose_plus.argtypes = [_dp, _dp]
        L.zsref_loss.restype = None
        L.zsref_loss.argtypes = [C.c_int, C.c_double, C.c_double, _dp]
        L.zsref_map_cull.restype = C.c_longlong
        L.zsref_map_cull.argtypes = [C.c_int, _dp, _dp, _ip, C.c_int, _ip, _dp, C.POINTER(C.c_longlong), _ip, _ip,
                                     C.POINTER(C.c_float), C.c_int, C.c_int, _up, _dp]
        L.zsref_pose_rt.restype = None
        L.zsref_pose_rt.argtypes = [_dp, _dp]
        L.zsref_rt_pose.restype = None
        L.zsref_rt_pose.argtypes = [_dp, _dp]
        L.zsref_find_matches.restype = C.c_longlong
        L.zsref_find_matches.argtypes = [_up, C.c_longlong, _up, C.c_longlong, C.c_float, C.c_longlong, C.c_void_p,
                                         C.c_longlong]

    def find_matches(self, lhs, rhs, threshold: float, k: int, size: int):
        return _find_matches(self.lib.zsref_find_matches, lhs, rhs, threshold, k, size)
        L.zsref_map_optimise.restype = None
        L.zsref_map_optimise.argtypes = [C.c_int, _dp, _dp, _ip, C.c_int, _ip, _dp, C.POINTER(C.c_longlong), _ip,
                                         C.POINTER(C.c_float), C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]

    def rt_pose(self, frame_pose):
        Rt = np.ascontiguousarray(frame_pose, dtype=np.float64).reshape(-1, 12)
        out = np.zeros((Rt.shape[0], 7))
        for f in range(Rt.shape[0]):
            self.lib.zsref_rt_pose(_ptr(Rt[f], _dp), _ptr(out[f], _dp))
        return out

    def map_optimise(self, cm, local_window: int, fix_landmarks: bool, rounds: int, use_relative: bool = False):
        """zeroslam's map::optimise on the map of a ``scenes.CullMap`` (every
        observing frame in the map): (frame_pose [F, 12], landmarks [L, 3])."""
        a = _cull_arrays(cm)
        fp = a["frame_pose"].copy()
        X = a["landmarks"].copy()
        self.lib.zsref_map_optimise(fp.shape[0], _ptr(fp, _dp), _ptr(a["frame_intrinsics"], _dp),
                                    _ptr(a["frame_id"], _ip), X.shape[0], _ptr(a["landmark_id"], _ip), _ptr(X, _dp),
                                    _ptr(a["landmark_obs"], C.POINTER(C.c_longlong)), _ptr(a["obs_frame"], _ip),
                                    _ptr(a["obs_keypoint"], C.POINTER(C.c_float)), int(cm.frame_id_generator),
                                    int(local_window), int(bool(fix_landmarks)), int(rounds), int(bool(use_relative)))
        return fp, X

    def map_cull(self, cm, timing: bool = False):
        """Which landmarks zeroslam's map::cull erases from the map of a
        ``scenes.CullMap``: (erase uint8 [L], erased[, seconds cull() took])."""
        a = _cull_arrays(cm)
        L = a["landmark_id"].shape[0]
        erase = np.zeros(L, dtype=np.uint8)
        secs = C.c_double(0.0)
        n = self.lib.zsref_map_cull(a["frame_pose"].shape[0], _ptr(a["frame_pose"], _dp),
                                    _ptr(a["frame_intrinsics"], _dp), _ptr(a["frame_id"], _ip), L,
                                    _ptr(a["landmark_id"], _ip), _ptr(a["landmarks"], _dp),
                                    _ptr(a["landmark_obs"], C.POINTER(C.c_longlong)), _ptr(a["obs_frame"], _ip),
                                    _ptr(a["obs_frame_id"], _ip), _ptr(a["obs_keypoint"], C.POINTER(C.c_float)),
                                    int(cm.landmark_id_generator), int(cm.frame_id_generator), _ptr(erase, _up),
                                    C.byref(secs))
        return (erase, int(n), secs.value) if timing else (erase, int(n))

    def pose_rt(self, poses):
        P = np.ascontiguousarray(poses, dtype=np.float64).reshape(-1, 7)
        out = np.zeros((P.shape[0], 12))
        for k in range(P.shape[0]):
            self.lib.zsref_pose_rt(_ptr(P[k], _dp), _ptr(out[k], _dp))
        return out

    @staticmethod
    def available() -> bool:
        return _build.reference_available() or os.path.exists(_build.REF_SO)

    def _args(self, a: _Arrays):
        return (a.poses.shape[0], a.landmarks.shape[0], a.obs_pose.shape[0], _ptr(a.poses, _dp),
                _ptr(a.pose_fixed, _up), _ptr(a.landmarks, _dp), _ptr(a.landmark_fixed, _up),
                _ptr(a.obs_pose, _ip), _ptr(a.obs_landmark, _ip), _ptr(a.obs_uv, _dp), _ptr(a.obs_info, _dp),
                _ptr(a.intrinsics, _dp), a.loss_kind, a.loss_delta)

    def solve(self, scene, iterations: int, use_relative: bool = False):
        """Returns (poses, landmarks, accepted, chi2_before, chi2_after, build_s, solve_s)."""
        a = _Arrays(scene)
        out = np.zeros(4)
        acc = self.lib.zsref_solve(*self._args(a), int(iterations), int(bool(use_relative)), _ptr(out, _dp))
        return a.poses, a.landmarks, acc, out[0], out[1], out[2], out[3]

    def chi2(self, scene) -> float:
        return self.lib.zsref_chi2(*self._args(_Arrays(scene)))

    def edge(self, pose7, X3, uv2, intr4):
        pose7, X3, uv2, intr4 = (np.ascontiguousarray(v, dtype=np.float64) for v in (pose7, X3, uv2, intr4))
        r = np.zeros(2)
        Jp = np.zeros((2, 6))
        Jl = np.zeros((2, 3))
        self.lib.zsref_edge(_ptr(pose7, _dp), _ptr(X3, _dp), _ptr(uv2, _dp), _ptr(intr4, _dp), _ptr(r, _dp),
                            _ptr(Jp, _dp), _ptr(Jl, _dp))
        return r, Jp, Jl

    def cholesky(self, A):
        A = np.ascontiguousarray(A, dtype=np.float64)
        Lm = np.zeros_like(A)
        ok = self.lib.zsref_cholesky(_ptr(A, _dp), A.shape[0], _ptr(Lm, _dp))
        return bool(ok), Lm

    def cholesky_solve(self, Lm, b):
        Lm = np.ascontiguousarray(Lm, dtype=np.float64)
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.zeros_like(b)
        ok = self.lib.zsref_cholesky_solve(_ptr(Lm, _dp), _ptr(b, _dp), Lm.shape[0], _ptr(x, _dp))
        return bool(ok), x

    def invert3(self, A):
        A = np.ascontiguousarray(A, dtype=np.float64)
        out = np.zeros((3, 3))
        ok = self.lib.zsref_invert3(_ptr(A, _dp), _ptr(out, _dp))
        return bool(ok), out

    def pose_plus(self, pose7, d6):
        pose = np.ascontiguousarray(pose7, dtype=np.float64).copy()
        d6 = np.ascontiguousarray(d6, dtype=np.float64)
        self.lib.zsref_pose_plus(_ptr(pose, _dp), _ptr(d6, _dp))
        return pose

    def loss(self, kind, delta, e2):
        rho = np.zeros(3)
        self.lib.zsref_loss(int(kind), float(delta), float(e2), _ptr(rho, _dp))
        return rho
