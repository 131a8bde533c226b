"""Python access to the C ABI of ``include/zeroslam_ba.h`` (ctypes).

The CUDA library is the only implementation: if ``_lib/libzeroslam_ba.so``
is missing or no CUDA device is usable, every call that needs one raises
``ZsError``. There is no CPU fallback.
"""

from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

ZS_OK = 0
ZS_ERR_INVALID = -1
ZS_ERR_CUDA = -2
ZS_ERR_UNSUPPORTED = -3
ZS_ERR_TIMEOUT = -4
ZS_ERR_NONFINITE = -5
ZS_ERR_NO_PROBLEM = -6
ZS_ERR_OUT_OF_MEMORY = -7
ZS_ERR_CHOLESKY = -8

FP64 = 0
MIXED = 1

LOSS_NONE, LOSS_HUBER, LOSS_CAUCHY, LOSS_TUKEY = 0, 1, 2, 3

_dp = C.POINTER(C.c_double)
_fp = C.POINTER(C.c_float)
_ip = C.POINTER(C.c_int32)
_up = C.POINTER(C.c_uint8)


class Options(C.Structure):
    _fields_ = [("precision", C.c_int32), ("max_failures", C.c_int32), ("tau", C.c_double),
                ("diagonal_clamp", C.c_double), ("legacy_stop", C.c_double), ("relative_tolerance", C.c_double),
                ("chi2_floor", C.c_double), ("refine_iterations", C.c_int32), ("refine_tolerance", C.c_double),
                ("device", C.c_int32), ("verbose", C.c_int32), ("profile", C.c_int32),
                ("batch_graph", C.c_int32), ("autotune_cache", C.c_char_p), ("pose_only_path", C.c_int32)]


class Problem(C.Structure):
    _fields_ = [("num_poses", C.c_int32), ("num_landmarks", C.c_int32), ("num_obs", C.c_int64),
                ("poses", _dp), ("pose_fixed", _up), ("landmarks", _dp), ("landmark_fixed", _up),
                ("obs_pose", _ip), ("obs_landmark", _ip), ("obs_uv", _dp), ("obs_info", _dp),
                ("intrinsics", C.c_double * 4), ("loss_kind", C.c_int32), ("loss_delta", C.c_double)]


class Report(C.Structure):
    _fields_ = [("status", C.c_int32), ("iterations", C.c_int32), ("accepted", C.c_int32), ("attempts", C.c_int32),
                ("cholesky_failures", C.c_int32), ("refine_sweeps", C.c_int32), ("chi2_initial", C.c_double),
                ("chi2_final", C.c_double), ("lambda_final", C.c_double), ("ms_total", C.c_double),
                ("ms_phase", C.c_double * 8), ("phase_calls", C.c_int32 * 8), ("kernel_launches", C.c_int64),
                ("preconditioner_retries", C.c_int32)]

    PHASES = ("linearize", "invert", "schur", "factor", "trisolve", "update", "cost", "other")

    def as_dict(self) -> dict:
        d = {k: getattr(self, k) for k, _ in self._fields_ if k not in ("ms_phase", "phase_calls")}
        d["ms_phase"] = {p: self.ms_phase[i] for i, p in enumerate(self.PHASES)}
        d["phase_calls"] = {p: self.phase_calls[i] for i, p in enumerate(self.PHASES)}
        return d


class BatchReport(C.Structure):
    _fields_ = [("status", C.c_int32), ("windows", C.c_int32), ("rounds", C.c_int32), ("graph_launches", C.c_int32),
                ("kernel_launches", C.c_int64), ("attempts", C.c_int64), ("accepted", C.c_int64),
                ("ms_total", C.c_double), ("bucket_windows", C.c_int32 * 5), ("bucket_threads", C.c_int32 * 5),
                ("bucket_tune_us", C.c_float * 5)]

    def as_dict(self) -> dict:
        d = {k: getattr(self, k) for k, _ in self._fields_ if not k.startswith("bucket_")}
        for k in ("bucket_windows", "bucket_threads", "bucket_tune_us"):
            d[k] = list(getattr(self, k))
        return d


class Attempt(C.Structure):
    _fields_ = [("iteration", C.c_int32), ("attempt", C.c_int32), ("solved", C.c_int32), ("accepted", C.c_int32),
                ("chi2", C.c_double), ("rho", C.c_double), ("lambda", C.c_double)]


class AdjointReport(C.Structure):
    _fields_ = [("status", C.c_int32), ("iterations", C.c_int32), ("rel_residual", C.c_double),
                ("ms_total", C.c_double)]


class MapCullInput(C.Structure):
    _fields_ = [("num_frames", C.c_int32), ("frame_pose", _dp), ("frame_intrinsics", _dp),
                ("num_landmarks", C.c_int32), ("landmark_id", _ip), ("landmarks", _dp),
                ("landmark_obs", C.POINTER(C.c_int64)), ("obs_frame", _ip), ("obs_frame_id", _ip),
                ("obs_keypoint", C.POINTER(C.c_float)), ("landmark_id_generator", C.c_int32),
                ("frame_id_generator", C.c_int32)]


MATCH_DTYPE = np.dtype([("lhs_index", np.uint64), ("rhs_index", np.uint64), ("score", np.float32)], align=True)


class MapOptimiseInput(C.Structure):
    _fields_ = [("num_frames", C.c_int32), ("frame_id", _ip), ("frame_pose", _dp), ("frame_intrinsics", _dp),
                ("num_landmarks", C.c_int32), ("landmark_id", _ip), ("landmarks", _dp),
                ("landmark_obs", C.POINTER(C.c_int64)), ("obs_frame", _ip), ("obs_keypoint", C.POINTER(C.c_float)),
                ("frame_id_generator", C.c_int32)]


class MapOptimiseReport(C.Structure):
    _fields_ = [("outcome", C.c_int32), ("frames", C.c_int32), ("landmarks", C.c_int32), ("edges", C.c_int32),
                ("problem_poses", C.c_int32), ("problem_landmarks", C.c_int32), ("ms_select", C.c_double),
                ("solve", Report)]


MAP_OPTIMISED, MAP_NOTHING_TO_OPTIMISE, MAP_ALL_FIXED = 0, 1, 2


class CullReport(C.Structure):
    _fields_ = [("erased", C.c_int64), ("error_passes", C.c_int64), ("ms_device", C.c_double)]


class ZsError(RuntimeError):
    def __init__(self, status: int, what: str = ""):
        self.status = status
        msg = _LIB.zs_ba_status_string(status).decode() if _LIB is not None else str(status)
        if _LIB is not None and status in (ZS_ERR_CUDA, ZS_ERR_OUT_OF_MEMORY):
            detail = _LIB.zs_last_error().decode()
            if detail:
                msg += f" [{detail}]"
        super().__init__(f"{what}: {msg} ({status})" if what else f"{msg} ({status})")


_LIB = None

ABI_FUNCTIONS = ("zs_ba_default_options", "zs_ba_create", "zs_ba_destroy", "zs_ba_set_problem", "zs_ba_set_state",
                 "zs_ba_get_state", "zs_ba_reset_state", "zs_ba_solve", "zs_ba_chi2", "zs_ba_linear_step",
                 "zs_ba_initial_lambda", "zs_dense_cholesky_solve", "zs_pipe_peaks", "zs_ba_status_string",
                 "zs_last_error", "zs_dense_cholesky_solve_noalloc", "zs_dense_gemm_nt_tf32x3", "zs_dense_chol_inverse_f32", "zs_ba_adjoint",
                 "zs_ba_set_batch", "zs_ba_solve_batch", "zs_ba_get_window_state", "zs_ba_batch_solve_profile", "zs_map_cull",
                 "zs_ba_cull", "zs_map_optimise", "zs_find_matches", "zs_map_optimise_plan",
                 "zs_frame_to_pose", "zs_pose_to_frame", "zs_ba_get_history")


def library_path() -> str:
    return _build.LIB_PATH


def load(path: str | None = None) -> C.CDLL:
    """Loads (building first if needed and nvcc is present) the CUDA library."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = path or library_path()
    if not os.path.exists(path):
        path = _build.build()
    lib = C.CDLL(path)
    lib.zs_ba_default_options.restype = None
    lib.zs_ba_default_options.argtypes = [C.POINTER(Options)]
    lib.zs_ba_create.restype = C.c_int
    lib.zs_ba_create.argtypes = [C.POINTER(C.c_void_p), C.POINTER(Options)]
    lib.zs_ba_destroy.restype = None
    lib.zs_ba_destroy.argtypes = [C.c_void_p]
    lib.zs_ba_set_problem.restype = C.c_int
    lib.zs_ba_set_problem.argtypes = [C.c_void_p, C.POINTER(Problem)]
    lib.zs_ba_set_state.restype = C.c_int
    lib.zs_ba_set_state.argtypes = [C.c_void_p, _dp, _dp]
    lib.zs_ba_get_state.restype = C.c_int
    lib.zs_ba_get_state.argtypes = [C.c_void_p, _dp, _dp]
    lib.zs_ba_reset_state.restype = C.c_int
    lib.zs_ba_reset_state.argtypes = [C.c_void_p]
    lib.zs_pipe_peaks.restype = C.c_int
    lib.zs_pipe_peaks.argtypes = [C.c_int, _dp, _dp]
    lib.zs_ba_solve.restype = C.c_int
    lib.zs_ba_solve.argtypes = [C.c_void_p, C.c_int, C.c_int, C.POINTER(Report)]
    lib.zs_ba_chi2.restype = C.c_int
    lib.zs_ba_chi2.argtypes = [C.c_void_p, _dp]
    lib.zs_ba_linear_step.restype = C.c_int
    lib.zs_ba_linear_step.argtypes = [C.c_void_p, C.c_double, _dp, _dp, _dp, _dp]
    lib.zs_ba_initial_lambda.restype = C.c_int
    lib.zs_ba_initial_lambda.argtypes = [C.c_void_p, _dp]
    lib.zs_dense_cholesky_solve.restype = C.c_int
    lib.zs_dense_cholesky_solve.argtypes = [_dp, C.c_int, _dp, _dp, _dp, C.c_int]
    lib.zs_ba_status_string.restype = C.c_char_p
    lib.zs_ba_status_string.argtypes = [C.c_int]
    lib.zs_last_error.restype = C.c_char_p
    lib.zs_last_error.argtypes = []
    lib.zs_ba_adjoint.restype = C.c_int
    lib.zs_ba_adjoint.argtypes = [C.c_void_p, _dp, _dp, _dp, _dp, _dp, C.POINTER(AdjointReport)]
    lib.zs_ba_set_batch.restype = C.c_int
    lib.zs_ba_set_batch.argtypes = [C.c_void_p, C.c_int, C.POINTER(Problem)]
    lib.zs_ba_solve_batch.restype = C.c_int
    lib.zs_ba_solve_batch.argtypes = [C.c_void_p, C.c_int, C.c_int, C.POINTER(Report), C.POINTER(BatchReport)]
    lib.zs_ba_batch_solve_profile.restype = C.c_int
    lib.zs_ba_batch_solve_profile.argtypes = [C.c_void_p, C.POINTER(C.c_longlong)]
    lib.zs_ba_get_window_state.restype = C.c_int
    lib.zs_ba_get_window_state.argtypes = [C.c_void_p, C.c_int, _dp, _dp]
    lib.zs_dense_cholesky_solve_noalloc.restype = C.c_int
    lib.zs_dense_cholesky_solve_noalloc.argtypes = [_dp, C.c_int, _dp, _dp, _dp]
    lib.zs_dense_gemm_nt_tf32x3.restype = C.c_int
    lib.zs_dense_gemm_nt_tf32x3.argtypes = [_fp, _fp, _fp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _dp]
    lib.zs_dense_chol_inverse_f32.restype = C.c_int
    lib.zs_dense_chol_inverse_f32.argtypes = [_fp, C.c_int, _fp, _fp, C.c_int, _dp]
    lib.zs_map_cull.restype = C.c_int
    lib.zs_map_cull.argtypes = [C.c_void_p, C.POINTER(MapCullInput), _up, C.POINTER(C.c_float),
                                C.POINTER(CullReport)]
    lib.zs_find_matches.restype = C.c_int
    lib.zs_find_matches.argtypes = [C.c_void_p, _up, C.c_int64, _up, C.c_int64, C.c_float, C.c_int64, C.c_void_p,
                                    C.c_int64, C.POINTER(C.c_int64), _dp]
    lib.zs_ba_get_history.restype = C.c_int
    lib.zs_ba_get_history.argtypes = [C.c_void_p, C.POINTER(Attempt), C.c_int32, C.POINTER(C.c_int32)]
    lib.zs_frame_to_pose.restype = None
    lib.zs_frame_to_pose.argtypes = [_dp, _dp]
    lib.zs_pose_to_frame.restype = None
    lib.zs_pose_to_frame.argtypes = [_dp, _dp]
    lib.zs_map_optimise_plan.restype = C.c_int
    lib.zs_map_optimise_plan.argtypes = [C.POINTER(MapOptimiseInput), C.c_int32, C.c_int32, _ip, _ip,
                                         C.POINTER(C.c_int64), _up, C.POINTER(MapOptimiseReport)]
    lib.zs_map_optimise.restype = C.c_int
    lib.zs_map_optimise.argtypes = [C.c_void_p, C.POINTER(MapOptimiseInput), C.c_int32, C.c_int32, C.c_int32,
                                    C.c_int32, C.POINTER(MapOptimiseReport)]
    lib.zs_ba_cull.restype = C.c_int
    lib.zs_ba_cull.argtypes = [C.c_void_p, _ip, _ip, C.c_int32, C.c_int32, _up, C.POINTER(C.c_float),
                               C.POINTER(CullReport)]
    _LIB = lib
    return lib


def _p(a, t):
    return None if a is None else a.ctypes.data_as(t)


def default_options(**kw) -> Options:
    lib = load()
    o = Options()
    lib.zs_ba_default_options(C.byref(o))
    for k, v in kw.items():
        setattr(o, k, v)
    return o


class BundleAdjuster:
    """One device handle (zs_ba_handle): problem upload, LM solve, state access."""

    def __init__(self, precision: int = FP64, **options):
        self.lib = load()
        self.options = default_options(precision=precision, **options)
        h = C.c_void_p()
        st = self.lib.zs_ba_create(C.byref(h), C.byref(self.options))
        if st != ZS_OK:
            raise ZsError(st, "zs_ba_create")
        self.h = h
        self.K = self.L = self.M = 0

    def close(self):
        if getattr(self, "h", None):
            self.lib.zs_ba_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @staticmethod
    def _problem(scene, p=None):
        """Fills a Problem from a scene; returns (problem, arrays that must stay alive)."""
        k = dict(
            poses=np.ascontiguousarray(scene.poses, dtype=np.float64),
            pose_fixed=np.ascontiguousarray(scene.pose_fixed, dtype=np.uint8),
            landmarks=np.ascontiguousarray(scene.landmarks, dtype=np.float64),
            landmark_fixed=np.ascontiguousarray(scene.landmark_fixed, dtype=np.uint8),
            obs_pose=np.ascontiguousarray(scene.obs_pose, dtype=np.int32),
            obs_landmark=np.ascontiguousarray(scene.obs_landmark, dtype=np.int32),
            obs_uv=np.ascontiguousarray(scene.obs_uv, dtype=np.float64),
            obs_info=None if scene.obs_info is None else np.ascontiguousarray(scene.obs_info, dtype=np.float64),
        )
        p = Problem() if p is None else p
        p.num_poses = k["poses"].shape[0]
        p.num_landmarks = k["landmarks"].shape[0]
        p.num_obs = k["obs_pose"].shape[0]
        p.poses = _p(k["poses"], _dp)
        p.pose_fixed = _p(k["pose_fixed"], _up)
        p.landmarks = _p(k["landmarks"], _dp)
        p.landmark_fixed = _p(k["landmark_fixed"], _up)
        p.obs_pose = _p(k["obs_pose"], _ip)
        p.obs_landmark = _p(k["obs_landmark"], _ip)
        p.obs_uv = _p(k["obs_uv"], _dp)
        p.obs_info = _p(k["obs_info"], _dp)
        for i in range(4):
            p.intrinsics[i] = float(scene.intrinsics[i])
        p.loss_kind = int(scene.loss_kind)
        p.loss_delta = float(scene.loss_delta)
        return p, k

    def set_batch(self, scenes) -> None:
        """Uploads independent windows (zs_ba_set_batch)."""
        arr = (Problem * len(scenes))()
        keep = []
        for i, sc in enumerate(scenes):
            keep.append(self._problem(sc, arr[i])[1])
        st = self.lib.zs_ba_set_batch(self.h, len(scenes), arr)
        if st != ZS_OK:
            raise ZsError(st, "zs_ba_set_batch")
        self._keep = keep
        self.windows = [(a["poses"].shape[0], a["landmarks"].shape[0]) for a in keep]
        self.K = sum(k for k, _ in self.windows)
        self.L = sum(l for _, l in self.windows)
        self.M = sum(a["obs_pose"].shape[0] for a in keep)

    def solve_batch(self, iterations: int, use_relative: bool = False):
        """(accepted summed over windows, [Report per window], BatchReport)."""
        reps = (Report * len(self.windows))()
        brep = BatchReport()
        v = self.lib.zs_ba_solve_batch(self.h, int(iterations), int(bool(use_relative)), reps, C.byref(brep))
        if v < 0:
            raise ZsError(v, "zs_ba_solve_batch")
        return v, list(reps), brep

    def batch_solve_profile(self) -> np.ndarray:
        """[windows, 5]: SM cycles per reduced-solve phase (load, factor, first
        solve, refinement) and refinement sweeps of the last batched solve
        (needs profile=1)."""
        out = np.zeros((len(self.windows), 5), dtype=np.int64)
        st = self.lib.zs_ba_batch_solve_profile(self.h, out.ctypes.data_as(C.POINTER(C.c_longlong)))
        if st != ZS_OK:
            raise ZsError(st, "zs_ba_batch_solve_profile")
        return out

    def get_window_state(self, w: int):
        K, L = self.windows[w]
        P = np.zeros((K, 7))
        Lm = np.zeros((L, 3))
        st = self.lib.zs_ba_get_window_state(self.h, int(w), _p(P, _dp), _p(Lm, _dp))
        if st != ZS_OK:
            raise ZsError(st, "zs_ba_get_window_state")
        return P, Lm

    def set_problem(self, scene) -> None:
        p, self._keep = self._problem(scene)
        st = self.lib.zs_ba_set_problem(self.h, C.byref(p))
        if st != ZS_OK:
            raise ZsError(st, "zs_ba_set_problem")
        self.K, self.L, self.M = p.num_poses, p.num_landmarks, p.num_obs

    def set_state(self, poses=None, landmarks=None) -> None:
        P = None if poses is None else np.ascontiguousarray(poses, dtype=np.float64)
        Lm = None if landmarks is None else np.ascontiguousarray(landmarks, dtype=np.float64)
        st = self.lib.zs_ba_set_state(self.h, _p(P, _dp), _p(Lm, _dp))
        if st != ZS_OK:
            raise ZsError(st, "zs_ba_set_state")

    def get_state(self):
        P = np.zeros((self.K, 7))
        Lm = np.zeros((self.L, 3))
        st = self.lib.zs_ba_get_state(self.h, _p(P, _dp), _p(Lm, _dp))
        if st != ZS_OK:
            raise ZsError(st, "zs_ba_get_state")
        return P, Lm

    def reset_state(self) -> None:
        st = self.lib.zs_ba_reset_state(self.h)
        if st != ZS_OK:
            raise ZsError(st, "zs_ba_reset_state")

    def solve(self, iterations: int, use_relative: bool = False) -> Report:
        rep = Report()
        v = self.lib.zs_ba_solve(self.h, int(iterations), int(bool(use_relative)), C.byref(rep))
        if v < 0:
            raise ZsError(v, "zs_ba_solve")
        return rep

    def history(self) -> list:
        """The last solve's attempts (zs_ba_get_history) as dicts."""
        n = C.c_int32()
        st = self.lib.zs_ba_get_history(self.h, None, 0, C.byref(n))
        if st != ZS_OK:
            raise ZsError(st, "zs_ba_get_history")
        buf = (Attempt * max(n.value, 1))()
        st = self.lib.zs_ba_get_history(self.h, buf, n.value, C.byref(n))
        if st != ZS_OK:
            raise ZsError(st, "zs_ba_get_history")
        return [dict(iteration=a.iteration, attempt=a.attempt, solved=bool(a.solved), accepted=bool(a.accepted),
                     chi2=a.chi2, rho=a.rho, lam=getattr(a, "lambda")) for a in buf[:n.value]]

    def chi2(self) -> float:
        out = C.c_double()
        st = self.lib.zs_ba_chi2(self.h, C.byref(out))
        if st != ZS_OK:
            raise ZsError(st, "zs_ba_chi2")
        return out.value

    def initial_lambda(self) -> float:
        out = C.c_double()
        st = self.lib.zs_ba_initial_lambda(self.h, C.byref(out))
        if st != ZS_OK:
            raise ZsError(st, "zs_ba_initial_lambda")
        return out.value

    def adjoint(self, dloss_dpose=None, dloss_dlandmark=None, want_state=False):
        """(dL/duv [M,2], dL/d(fx,fy,cx,cy) [4], AdjointReport[, v [6K+3L]]) at the current state."""
        dp = None if dloss_dpose is None else np.ascontiguousarray(dloss_dpose, dtype=np.float64)
        dl = None if dloss_dlandmark is None else np.ascontiguousarray(dloss_dlandmark, dtype=np.float64)
        duv = np.zeros((self.M, 2))
        dint = np.zeros(4)
        v = np.zeros(6 * self.K + 3 * self.L) if want_state else None
        rep = AdjointReport()
        st = self.lib.zs_ba_adjoint(self.h, _p(dp, _dp), _p(dl, _dp), _p(duv, _dp), _p(dint, _dp), _p(v, _dp),
                                    C.byref(rep))
        if st != ZS_OK:
            raise ZsError(st, "zs_ba_adjoint")
        return (duv, dint, rep, v) if want_state else (duv, dint, rep)

    def cull(self, landmark_id, pose_frame_id, landmark_id_generator: int, frame_id_generator: int):
        """map::cull of the resident problem at the current state (zs_ba_cull):
        (erase uint8 [L], mean error float32 [L], CullReport)."""
        lid = np.ascontiguousarray(landmark_id, dtype=np.int32)
        fid = np.ascontiguousarray(pose_frame_id, dtype=np.int32)
        if lid.shape != (self.L,) or fid.shape != (self.K,):
            raise ValueError("landmark_id must have L entries and pose_frame_id K")
        erase = np.zeros(self.L, dtype=np.uint8)
        mean = np.zeros(self.L, dtype=np.float32)
        rep = CullReport()
        st = self.lib.zs_ba_cull(self.h, _p(lid, _ip), _p(fid, _ip), int(landmark_id_generator),
                                 int(frame_id_generator), _p(erase, _up), _p(mean, C.POINTER(C.c_float)),
                                 C.byref(rep))
        if st != ZS_OK:
            raise ZsError(st, "zs_ba_cull")
        return erase, mean, rep

    def map_optimise(self, cm, local_window: int, fix_landmarks: bool, rounds: int, use_relative: bool = False):
        """map::optimise of a map given as arrays (zs_map_optimise, ``scenes.CullMap``):
        (frame_pose [F, 12], landmarks [L, 3], MapOptimiseReport); the map is not modified.
        The handle's problem becomes the map's window."""
        fp = np.array(cm.frame_pose, dtype=np.float64, copy=True, order="C")
        X = np.array(cm.landmarks, dtype=np.float64, copy=True, order="C")
        fid = np.ascontiguousarray(cm.frame_id, dtype=np.int32)
        intr = np.ascontiguousarray(cm.frame_intrinsics, dtype=np.float64)
        lid = np.ascontiguousarray(cm.landmark_id, dtype=np.int32)
        ptr = np.ascontiguousarray(cm.landmark_obs, dtype=np.int64)
        of = np.ascontiguousarray(cm.obs_frame, dtype=np.int32)
        kp = np.ascontiguousarray(cm.obs_keypoint, dtype=np.float32)
        inp = MapOptimiseInput(fp.shape[0], _p(fid, _ip), _p(fp, _dp), _p(intr, _dp), X.shape[0], _p(lid, _ip),
                               _p(X, _dp), _p(ptr, C.POINTER(C.c_int64)), _p(of, _ip),
                               _p(kp, C.POINTER(C.c_float)), int(cm.frame_id_generator))
        rep = MapOptimiseReport()
        st = self.lib.zs_map_optimise(self.h, C.byref(inp), int(local_window), int(bool(fix_landmarks)),
                                      int(rounds), int(bool(use_relative)), C.byref(rep))
        if st != ZS_OK:
            raise ZsError(st, "zs_map_optimise")
        if rep.outcome == MAP_OPTIMISED:
            self.K, self.L, self.M = rep.problem_poses, rep.problem_landmarks, rep.edges
        return fp, X, rep

    def find_matches(self, lhs, rhs, threshold: float, k: int, size: int, timing: bool = False):
        """feature::find_matches on the device (zs_find_matches): a structured
        array of (lhs_index, rhs_index, score) [, device ms]."""
        lhs = np.ascontiguousarray(lhs, dtype=np.uint8).reshape(-1, 32)
        rhs = np.ascontiguousarray(rhs, dtype=np.uint8).reshape(-1, 32)
        out = np.zeros(max(int(size), 1), dtype=MATCH_DTYPE)
        n = C.c_int64()
        ms = C.c_double()
        st = self.lib.zs_find_matches(self.h, _p(lhs, _up), lhs.shape[0], _p(rhs, _up), rhs.shape[0], float(threshold),
                                      int(k), out.ctypes.data_as(C.c_void_p), int(size), C.byref(n), C.byref(ms))
        if st != ZS_OK:
            raise ZsError(st, "zs_find_matches")
        res = out[:n.value].copy()
        return (res, ms.value) if timing else res

    def map_cull(self, cm):
        """map::cull of a map given as arrays (zs_map_cull, ``scenes.CullMap``):
        (erase uint8 [L], mean error float32 [L], CullReport)."""
        inp, keep = cull_input(cm)
        L = inp.num_landmarks
        erase = np.zeros(L, dtype=np.uint8)
        mean = np.zeros(L, dtype=np.float32)
        rep = CullReport()
        st = self.lib.zs_map_cull(self.h, C.byref(inp), _p(erase, _up), _p(mean, C.POINTER(C.c_float)),
                                  C.byref(rep))
        del keep
        if st != ZS_OK:
            raise ZsError(st, "zs_map_cull")
        return erase, mean, rep

    def linear_step(self, lam: float, want_S: bool = True) -> dict:
        n = 6 * self.K
        S = np.zeros((n, n)) if want_S else None
        bs = np.zeros(n)
        delta = np.zeros(n + 3 * self.L)
        b = np.zeros(n + 3 * self.L)
        st = self.lib.zs_ba_linear_step(self.h, float(lam), _p(S, _dp), _p(bs, _dp), _p(delta, _dp), _p(b, _dp))
        if st not in (ZS_OK, ZS_ERR_CHOLESKY):
            raise ZsError(st, "zs_ba_linear_step")
        return dict(ok=(st == ZS_OK), S=S, bs=bs, delta=delta, b=b)


def partition_windows(windows, parts: int) -> list:
    """Splits independent windows over ``parts`` devices (one process per
    GPU, no exchange between them): each window's cost is estimated as
    M + n^3 (observations, and the dense reduced system of n = 6K), windows
    are taken largest first and each goes to the part with the least cost so
    far (ties to the lower part, then the lower window index), so every
    process computes the same partition. Returns one ascending list of window
    indices per part."""
    if parts < 1:
        raise ValueError("parts must be positive")
    cost = [int(w.M) + (6 * int(w.K)) ** 3 for w in windows]
    order = sorted(range(len(windows)), key=lambda i: (-cost[i], i))
    load = [0] * parts
    out = [[] for _ in range(parts)]
    for i in order:
        p = min(range(parts), key=lambda q: (load[q], q))
        out[p].append(i)
        load[p] += cost[i]
    return [sorted(o) for o in out]


def frames_to_poses(frame_pose) -> np.ndarray:
    """[F, 7] vertex_pose parameters of [F, 12] frames (zs_frame_to_pose)."""
    lib = load()
    Rt = np.ascontiguousarray(frame_pose, dtype=np.float64).reshape(-1, 12)
    out = np.zeros((Rt.shape[0], 7))
    for f in range(Rt.shape[0]):
        lib.zs_frame_to_pose(_p(Rt[f], _dp), _p(out[f], _dp))
    return out


def poses_to_frames(poses) -> np.ndarray:
    """[K, 12] frames of [K, 7] poses (zs_pose_to_frame)."""
    lib = load()
    P = np.ascontiguousarray(poses, dtype=np.float64).reshape(-1, 7)
    out = np.zeros((P.shape[0], 12))
    for k in range(P.shape[0]):
        lib.zs_pose_to_frame(_p(P[k], _dp), _p(out[k], _dp))
    return out


def map_optimise_plan(cm, local_window: int, fix_landmarks: bool) -> dict:
    """The window and graph map::optimise would build from a map
    (zs_map_optimise_plan; host only, no device): problem poses as frame
    indices, problem landmarks as map landmark indices, the edges as
    observation indices, the frames written back, and the report."""
    lib = load()
    fid = np.ascontiguousarray(cm.frame_id, dtype=np.int32)
    fp = np.ascontiguousarray(cm.frame_pose, dtype=np.float64)
    intr = np.ascontiguousarray(cm.frame_intrinsics, dtype=np.float64)
    lid = np.ascontiguousarray(cm.landmark_id, dtype=np.int32)
    X = np.ascontiguousarray(cm.landmarks, dtype=np.float64)
    ptr = np.ascontiguousarray(cm.landmark_obs, dtype=np.int64)
    of = np.ascontiguousarray(cm.obs_frame, dtype=np.int32)
    kp = np.ascontiguousarray(cm.obs_keypoint, dtype=np.float32)
    inp = MapOptimiseInput(fp.shape[0], _p(fid, _ip), _p(fp, _dp), _p(intr, _dp), X.shape[0], _p(lid, _ip),
                           _p(X, _dp), _p(ptr, C.POINTER(C.c_int64)), _p(of, _ip), _p(kp, C.POINTER(C.c_float)),
                           int(cm.frame_id_generator))
    F, L, M = fp.shape[0], X.shape[0], of.shape[0]
    pose_frame = np.zeros(max(F, 1), dtype=np.int32)
    lm_index = np.zeros(max(L, 1), dtype=np.int32)
    edge_obs = np.zeros(max(M, 1), dtype=np.int64)
    written = np.zeros(max(F, 1), dtype=np.uint8)
    rep = MapOptimiseReport()
    st = lib.zs_map_optimise_plan(C.byref(inp), int(local_window), int(bool(fix_landmarks)), _p(pose_frame, _ip),
                                  _p(lm_index, _ip), _p(edge_obs, C.POINTER(C.c_int64)), _p(written, _up),
                                  C.byref(rep))
    if st != ZS_OK:
        raise ZsError(st, "zs_map_optimise_plan")
    return dict(report=rep, pose_frame=pose_frame[:rep.problem_poses].copy(),
                landmark_index=lm_index[:rep.problem_landmarks].copy(), edge_obs=edge_obs[:rep.edges].copy(),
                written=written[:F].astype(bool))


def cull_input(cm):
    """A MapCullInput over the arrays of a ``scenes.CullMap``; returns
    (input, arrays that must stay alive while it is used)."""
    k = dict(
        frame_pose=np.ascontiguousarray(cm.frame_pose, dtype=np.float64),
        frame_intrinsics=np.ascontiguousarray(cm.frame_intrinsics, dtype=np.float64),
        landmark_id=np.ascontiguousarray(cm.landmark_id, dtype=np.int32),
        landmarks=np.ascontiguousarray(cm.landmarks, dtype=np.float64),
        landmark_obs=np.ascontiguousarray(cm.landmark_obs, dtype=np.int64),
        obs_frame=np.ascontiguousarray(cm.obs_frame, dtype=np.int32),
        obs_frame_id=np.ascontiguousarray(cm.obs_frame_id, dtype=np.int32),
        obs_keypoint=np.ascontiguousarray(cm.obs_keypoint, dtype=np.float32),
    )
    inp = MapCullInput()
    inp.num_frames = k["frame_pose"].shape[0]
    inp.frame_pose = _p(k["frame_pose"], _dp)
    inp.frame_intrinsics = _p(k["frame_intrinsics"], _dp)
    inp.num_landmarks = k["landmark_id"].shape[0]
    inp.landmark_id = _p(k["landmark_id"], _ip)
    inp.landmarks = _p(k["landmarks"], _dp)
    inp.landmark_obs = _p(k["landmark_obs"], C.POINTER(C.c_int64))
    inp.obs_frame = _p(k["obs_frame"], _ip)
    inp.obs_frame_id = _p(k["obs_frame_id"], _ip)
    inp.obs_keypoint = _p(k["obs_keypoint"], C.POINTER(C.c_float))
    inp.landmark_id_generator = int(cm.landmark_id_generator)
    inp.frame_id_generator = int(cm.frame_id_generator)
    return inp, k


def dense_cholesky_solve(A, b, precision: int = FP64):
    """(ok, L, x) of the device Cholesky solve of A x = b."""
    lib = load()
    A = np.ascontiguousarray(A, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    n = A.shape[0]
    Lm = np.zeros_like(A)
    x = np.zeros(n)
    st = lib.zs_dense_cholesky_solve(_p(A, _dp), n, _p(b, _dp), _p(Lm, _dp), _p(x, _dp), int(precision))
    if st not in (ZS_OK, ZS_ERR_CHOLESKY):
        raise ZsError(st, "zs_dense_cholesky_solve")
    return st == ZS_OK, Lm, x


def dense_cholesky_status(A, b, precision: int = FP64) -> int:
    """The status zs_dense_cholesky_solve returns for A x = b (no results)."""
    lib = load()
    A = np.ascontiguousarray(A, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    x = np.zeros(A.shape[0])
    return int(lib.zs_dense_cholesky_solve(_p(A, _dp), A.shape[0], _p(b, _dp), None, _p(x, _dp), int(precision)))


def dense_gemm_tf32x3(A, B, lower: bool = False, max_ctas: int = 0):
    """(A B^T on the tensor cores with FP32 accuracy, the kernel's device ms);
    max_ctas > 0 caps the grid (each CTA walks several tiles)."""
    lib = load()
    A = np.ascontiguousarray(A, dtype=np.float32)
    B = np.ascontiguousarray(B, dtype=np.float32)
    M, K = A.shape
    N = B.shape[0]
    if B.shape[1] != K:
        raise ValueError("A and B need the same number of columns")
    out = np.zeros((M, N), dtype=np.float32)
    ms = C.c_double()
    st = lib.zs_dense_gemm_nt_tf32x3(_p(A, _fp), _p(B, _fp), _p(out, _fp), M, N, K, int(bool(lower)), int(max_ctas),
                                     C.byref(ms))
    if st != ZS_OK:
        raise ZsError(st, "zs_dense_gemm_nt_tf32x3")
    return out, ms.value


def dense_chol_inverse_f32(S, form: int = 0):
    """(status, L, X = L^-1, device ms) of the mixed form's FP32
    preconditioner on the symmetric matrix S (its lower triangle is read);
    form 0 as the solve chooses,
    1 the dataflow kernel alone, 2 the blocked tensor-core form."""
    lib = load()
    S = np.ascontiguousarray(S, dtype=np.float32)
    n = S.shape[0]
    L = np.zeros((n, n), dtype=np.float32)
    X = np.zeros((n, n), dtype=np.float32)
    ms = C.c_double()
    st = lib.zs_dense_chol_inverse_f32(_p(S, _fp), n, _p(L, _fp), _p(X, _fp), int(form), C.byref(ms))
    if st not in (ZS_OK, ZS_ERR_CHOLESKY):
        raise ZsError(st, "zs_dense_chol_inverse_f32")
    return st, L, X, ms.value


def pipe_peaks(device: int = 0):
    """(fp64_tflops, fp32_tflops) measured by an FMA-chain microbenchmark."""
    lib = load()
    a, b = C.c_double(), C.c_double()
    st = lib.zs_pipe_peaks(int(device), C.byref(a), C.byref(b))
    if st != ZS_OK:
        raise ZsError(st, "zs_pipe_peaks")
    return a.value, b.value
