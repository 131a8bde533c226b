/*
 * zeroslam_ba.h — C ABI of the GB300 (sm_103a) sparse-block bundle adjuster.
 *
 * This library replaces the Levenberg-Marquardt / Schur-complement solve of
 * zeroslam's factor graph for SE(3) keyframe poses and 3-D landmarks joined
 * by pinhole reprojection edges. Every entry point takes plain host pointers
 * and sizes; the handle owns all device memory and one CUDA stream. No CPU
 * fallback exists: without a usable CUDA device every call that needs one
 * returns ZS_ERR_CUDA.
 *
 * Entry point -> reference interface it replaces (paths inside gpdaniels/zeroslam):
 *   zs_ba_create / zs_ba_destroy  factor_graph::factor_graph(bool)          source/factor_graph.hpp:379
 *   zs_ba_set_problem             add_vertex / add_edge / set_observation /
 *                                 set_information / set_loss_function      source/factor_graph.hpp:385,444,
 *                                                                          198-277; graph build source/map.hpp:129-179
 *   zs_ba_solve                   int factor_graph::solve(int, bool)       source/factor_graph.hpp:489-615
 *   zs_ba_chi2                    double get_current_chi(bool)             source/factor_graph.hpp:618-629
 *   zs_ba_get_state/zs_ba_set_state vertex_base::get/set_parameters        source/factor_graph.hpp:123-129
 *   zs_ba_linear_step             make_hessian + solve_linear_system       source/factor_graph.hpp:648-806
 *   zs_dense_cholesky_solve       matrix::decompose_cholesky +
 *                                 matrix::solve_cholesky                   source/matrix_decomposition_cholesky.hpp:26-95
 *   zs_ba_reset_state             vertex_base::restore                     source/factor_graph.hpp:135-137
 *   zs_ba_status_string           (stderr diagnostics of solve)           source/factor_graph.hpp:495,786
 *   zs_map_optimise               map::map::optimise                       source/map.hpp:65-267
 *   zs_map_cull / zs_ba_cull      map::map::cull                           source/map.hpp:269-323
 *   zs_find_matches               feature::find_matches, distance<256>     source/feature.hpp:1133-1235
 *
 * Conventions: return values are status codes (0 = ok, negative = error);
 * nothing throws or aborts across this boundary. Host buffers stay owned by
 * the caller and are copied. A handle is not thread-safe; use one handle per
 * host thread. Results are bit-for-bit reproducible from run to run on the
 * same device (no floating-point atomics).
 */
#ifndef ZEROSLAM_BA_H
#define ZEROSLAM_BA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ZS_BA_ABI_VERSION 1

/* Status codes. */
#define ZS_OK 0
#define ZS_ERR_INVALID (-1)      /* bad argument or problem (index out of range, NULL pointer) */
#define ZS_ERR_CUDA (-2)         /* CUDA runtime error or no usable device */
#define ZS_ERR_UNSUPPORTED (-3)  /* vertex / edge / loss kind the device path does not implement */
#define ZS_ERR_TIMEOUT (-4)      /* a bounded device wait ran out */
#define ZS_ERR_NONFINITE (-5)    /* non-finite values in the inputs */
#define ZS_ERR_NO_PROBLEM (-6)   /* solve/get before set_problem */
#define ZS_ERR_OUT_OF_MEMORY (-7)
#define ZS_ERR_CHOLESKY (-8)     /* dense Cholesky factor or solve failed its pivot test */

/* Arithmetic of the solve. */
#define ZS_PRECISION_FP64 0  /* everything in double: the reference's arithmetic */
#define ZS_PRECISION_MIXED 1 /* FP32 Jacobians/Hessian/Schur, FP32 factor, FP64 refinement, FP64 cost */

/* Robust losses of source/factor_graph.hpp:851-934. */
#define ZS_LOSS_NONE 0
#define ZS_LOSS_HUBER 1
#define ZS_LOSS_CAUCHY 2
#define ZS_LOSS_TUKEY 3

typedef struct zs_ba_handle zs_ba_handle;

/* Solver settings. zs_ba_default_options() gives the reference's constants
 * (source/factor_graph.hpp:511-536). */
typedef struct zs_ba_options {
    int32_t precision;          /* ZS_PRECISION_* */
    int32_t max_failures;       /* 10: failed attempts per outer iteration */
    double tau;                 /* 1e-5: initial damping = tau * min(clamp, max diag) */
    double diagonal_clamp;      /* 5e10 */
    double legacy_stop;         /* 1e-10: stop when the gain < legacy_stop * chi2_initial */
    double relative_tolerance;  /* 1e-6: stop when the gain < tol * max(last, floor) */
    double chi2_floor;          /* 1e-12 */
    int32_t refine_iterations;  /* mixed form: conjugate-gradient iterations on the FP64 Schur operator
                                   (batched windows: FP64 refinement sweeps) at most (8) */
    double refine_tolerance;    /* mixed form: stop at ||b - S x|| <= tol ||b|| (1e-10) */
    int32_t device;             /* CUDA device ordinal (0) */
    int32_t verbose;            /* 1: print [INIT]/[GOOD]/[ BAD] lines to stderr; 2: also each mixed-form refinement */
    int32_t profile;            /* 1: time each phase with CUDA events into zs_ba_report.ms_phase */
    int32_t batch_graph;        /* batched solve: 1 = one CUDA graph launch (conditional WHILE
                                   node over attempt rounds), 0 = host loop over rounds (1) */
    const char* autotune_cache; /* batched solve: file of autotuned block sizes (read, and written
                                   after tuning), or NULL for a per-process cache only */
    int32_t pose_only_path;     /* 1: a single problem with every landmark fixed, at most 64 poses and
                                   at most 4 of them free (zeroslam's tracking mode) runs its whole LM
                                   loop in one launch, in FP64 in both precisions; so does a batch whose
                                   landmarks are all fixed, one CTA per window; 0: the general
                                   path (1) */
} zs_ba_options;

/* A bundle-adjustment problem as structure of arrays (host pointers).
 * Pose parameters are zeroslam's vertex_pose layout (tx, ty, tz, qx, qy, qz, qw),
 * world->camera (source/factor_graph.hpp:941). Quaternions are used as given,
 * without renormalisation, as the reference does. */
typedef struct zs_ba_problem {
    int32_t num_poses;              /* K */
    int32_t num_landmarks;          /* L */
    int64_t num_obs;                /* M: one edge_reprojection each */
    const double* poses;            /* [K*7] */
    const uint8_t* pose_fixed;      /* [K] nonzero = fixed (still ordered into the reduced system) */
    const double* landmarks;        /* [L*3] */
    const uint8_t* landmark_fixed;  /* [L] */
    const int32_t* obs_pose;        /* [M] pose index of each observation */
    const int32_t* obs_landmark;    /* [M] landmark index of each observation */
    const double* obs_uv;           /* [M*2] observed pixel */
    const double* obs_info;         /* [M*4] row-major 2x2 information, or NULL for identity */
    double intrinsics[4];           /* fx, fy, cx, cy of camera::pinhole */
    int32_t loss_kind;              /* ZS_LOSS_* shared by all edges */
    double loss_delta;
} zs_ba_problem;

/* What a solve did. */
typedef struct zs_ba_report {
    int32_t status;            /* ZS_OK or the error returned */
    int32_t iterations;        /* outer LM iterations run */
    int32_t accepted;          /* accepted steps (the reference's solve() return value) */
    int32_t attempts;          /* damped linear solves attempted */
    int32_t cholesky_failures; /* attempts whose reduced Cholesky failed */
    int32_t refine_sweeps;     /* mixed form: conjugate-gradient iterations (batched windows: refinement
                                  sweeps) over all attempts */
    double chi2_initial;
    double chi2_final;
    double lambda_final;
    double ms_total;           /* device time of the solve (CUDA events) */
    /* With options.profile: device milliseconds and launch counts per phase
     * (ZS_PHASE_*), summed over the solve. */
    double ms_phase[8];
    int32_t phase_calls[8];
    int64_t kernel_launches;   /* kernels this library launched during the solve */
    int32_t preconditioner_retries; /* mixed form: attempts whose FP32 factorisation of the FP32-formed S
                                       failed and was retried on S + 1e-5 diag(S) (the factor only
                                       preconditions the conjugate-gradient solve) */
} zs_ba_report;

/* Phases of zs_ba_report.ms_phase. */
#define ZS_PHASE_LINEARIZE 0 /* residuals, Jacobians, H_pp / H_pl / H_ll / b assembly */
#define ZS_PHASE_INVERT 1    /* damped H_ll inverses and W = H_pl H_ll^-1 */
#define ZS_PHASE_SCHUR 2     /* S = H_pp - W H_lp and b_s */
#define ZS_PHASE_FACTOR 3    /* reduced Cholesky factorisation */
#define ZS_PHASE_TRISOLVE 4  /* triangular solves and refinement */
#define ZS_PHASE_UPDATE 5    /* back-substitution, state update, gain scale */
#define ZS_PHASE_COST 6      /* robust chi2, LM decision, rollback */
#define ZS_PHASE_OTHER 7

void zs_ba_default_options(zs_ba_options* opt);

int zs_ba_create(zs_ba_handle** out, const zs_ba_options* opt);
void zs_ba_destroy(zs_ba_handle* h);

/* Uploads a problem and analyses its structure (landmark- and pose-major
 * orderings, Schur pair lists). Replaces any previous problem. */
int zs_ba_set_problem(zs_ba_handle* h, const zs_ba_problem* p);

/* Overwrites / reads the current vertex parameters ([K*7], [L*3]). */
int zs_ba_set_state(zs_ba_handle* h, const double* poses, const double* landmarks);
int zs_ba_get_state(zs_ba_handle* h, double* poses, double* landmarks);

/* Restores the vertex parameters uploaded by zs_ba_set_problem (a device
 * copy), so a problem can be solved again from the same initial guess. */
int zs_ba_reset_state(zs_ba_handle* h);

/* Levenberg-Marquardt with Schur complement, `iterations` outer iterations,
 * stop rule as source/factor_graph.hpp:608-611. Returns the accepted-step
 * count (>= 0) or a negative status; `rep` may be NULL. A ZS_PRECISION_MIXED
 * handle with a ZS_LOSS_TUKEY problem returns ZS_ERR_UNSUPPORTED: under that
 * redescending loss the mixed form's rounding moves observations across the
 * loss's threshold and the solve can settle in another nearby minimum than
 * the FP64 one, so it cannot promise the mixed form's agreement with FP64
 * (use a ZS_PRECISION_FP64 handle). */
int zs_ba_solve(zs_ba_handle* h, int iterations, int use_relative, zs_ba_report* rep);

/* Robust chi2 of the current state. */
int zs_ba_chi2(zs_ba_handle* h, double* chi2);

/* One linearisation at the current state and one damped solve at `lambda`,
 * without changing the state. Outputs (each may be NULL): S [n*n] the damped
 * reduced camera matrix (n = 6K, row-major), bs [n] its right-hand side,
 * delta [6K+3L] the step (poses then landmarks), b [6K+3L] the gradient
 * vector. Returns ZS_OK or ZS_ERR_CHOLESKY. */
int zs_ba_linear_step(zs_ba_handle* h, double lambda, double* S, double* bs, double* delta, double* b);

/* What an adjoint solve did. */
typedef struct zs_ba_adjoint_report {
    int32_t status;
    int32_t iterations;      /* preconditioned conjugate-gradient iterations */
    double rel_residual;     /* ||a - H v|| / ||a|| at exit */
    double ms_total;
} zs_ba_adjoint_report;

/* ---- Batched local windows ----
 * Many independent windows (each a complete problem as for zs_ba_set_problem)
 * solved together on one device: the reference runs one factor_graph per
 * window (map::optimise, source/map.hpp:65-267, calling
 * factor_graph::solve, source/factor_graph.hpp:489-615); here every window
 * runs the same LM control flow with its own damping, acceptance and stop
 * decisions, in one CUDA graph launch. All windows share the intrinsics, the
 * loss and the presence of obs_info; each window has at most
 * ZS_BATCH_MAX_POSES poses. */
#define ZS_BATCH_MAX_POSES 32
#define ZS_BATCH_BUCKETS 5

typedef struct zs_ba_batch_report {
    int32_t status;
    int32_t windows;
    int32_t rounds;                           /* attempt rounds run (each: one attempt per active window) */
    int32_t graph_launches;                   /* 1 when the solve ran as one graph launch, else 0 */
    int64_t kernel_launches;                  /* kernels executed: prologue + rounds x round body */
    int64_t attempts;                         /* summed over windows */
    int64_t accepted;                         /* summed over windows */
    double ms_total;                          /* device time of the batched solve (CUDA events) */
    int32_t bucket_windows[ZS_BATCH_BUCKETS]; /* windows per reduced-system size bucket (n <= 64, 96, 128, 160, 192) */
    int32_t bucket_threads[ZS_BATCH_BUCKETS]; /* autotuned block size of each bucket's reduced solve */
    float bucket_tune_us[ZS_BATCH_BUCKETS];   /* autotuner's best time (synthetic 2 x SMs windows), 0 if cached */
} zs_ba_batch_report;

/* Uploads num_windows windows (an array of problems) as one batch; replaces
 * any problem of the handle. */
int zs_ba_set_batch(zs_ba_handle* h, int num_windows, const zs_ba_problem* windows);
/* Solves every window of the batch as zs_ba_solve would (same iterations /
 * use_relative semantics per window). window_reports (may be NULL): one
 * report per window; rep (may be NULL): the batch summary. Returns the
 * accepted steps summed over windows, or a negative status. A batch whose
 * landmarks are all fixed (tracking problems) takes the pose-only path
 * (options.pose_only_path): one launch, one CTA per window, in FP64. */
int zs_ba_solve_batch(zs_ba_handle* h, int iterations, int use_relative, zs_ba_report* window_reports,
                      zs_ba_batch_report* rep);
/* With options.profile: per window, the SM cycles the last zs_ba_solve_batch
 * spent in each phase of its reduced solves (load, factor, first solve,
 * refinement; summed over attempts) and its refinement sweeps:
 * out[window * 5 + phase]. */
int zs_ba_batch_solve_profile(zs_ba_handle* h, long long* out);
/* Current state of one window ([K_w*7], [L_w*3]; either may be NULL). */
int zs_ba_get_window_state(zs_ba_handle* h, int window, double* poses, double* landmarks);

/* One attempt of the last zs_ba_solve: the values of the reference's verbose
 * [GOOD] / [ BAD] lines (source/factor_graph.hpp:583-606). */
typedef struct zs_ba_attempt {
    int32_t iteration;  /* outer iteration, from 0 */
    int32_t attempt;    /* attempt within the iteration (the reference's failure counter) */
    int32_t solved;     /* 0: the damped linear solve failed (the reference's "Cholesky solver failed!") */
    int32_t accepted;   /* 1: the step was kept */
    double chi2;        /* cost at the attempted state (the current state's when not solved) */
    double rho;         /* gain ratio (0 when not solved) */
    double lambda;      /* damping after the attempt */
} zs_ba_attempt;

/* The attempts of the last zs_ba_solve on h, in order: *count receives their
 * number, out the first min(count, capacity). */
int zs_ba_get_history(zs_ba_handle* h, zs_ba_attempt* out, int32_t capacity, int32_t* count);

/* Gradient of a scalar loss of the solved state with respect to the observed
 * pixels and the intrinsics, by the implicit-function theorem at the current
 * state (call after zs_ba_solve has converged). Inputs: a = dL/dx in the
 * solver's local coordinates, dloss_dpose [K*6] (left perturbation
 * exp(d) T, omega then upsilon) and dloss_dlandmark [L*3] (either may be
 * NULL = zero); fixed vertices are ignored. Outputs (each may be NULL):
 * dloss_duv [M*2] in the problem's observation order, dloss_dintrinsics [4]
 * (fx, fy, cx, cy) and adjoint_state [6K+3L], the solution v of H v = a.
 * H is the exact Hessian of the cost in local coordinates (Gauss-Newton term
 * plus residual curvature); H v = a is solved by conjugate gradients
 * preconditioned with the solver's Schur / reduced-Cholesky factorisation.
 * With a = the gradient vector b of zs_ba_linear_step, v is the exact Newton
 * step. FP64 handles and ZS_LOSS_NONE only (ZS_ERR_UNSUPPORTED otherwise).
 * No counterpart in the reference. */
int zs_ba_adjoint(zs_ba_handle* h, const double* dloss_dpose, const double* dloss_dlandmark, double* dloss_duv,
                  double* dloss_dintrinsics, double* adjoint_state, zs_ba_adjoint_report* rep);

/* Initial damping tau * min(clamp, max diagonal of H) at the current state. */
int zs_ba_initial_lambda(zs_ba_handle* h, double* lambda);

/* ---- descriptor matching: feature::find_matches (source/feature.hpp:1190-1235) ---- */

/* feature::match, field for field (size_t, size_t, float on LP64 hosts). */
typedef struct zs_match {
    uint64_t lhs_index;
    uint64_t rhs_index;
    float score;        /* the Hamming distance, as float */
} zs_match;

#define ZS_MATCH_MAX_K 8

/* For each lhs descriptor in order (32 bytes each, the 256-bit
 * feature::descriptor), the matches_count nearest rhs descriptors by Hamming
 * distance (distance<256>) whose distance is below threshold, nearest first,
 * equal distances in rhs order; lhs descriptors are taken while
 * found + matches_count <= matches_size (the reference's capacity rule).
 * Writes matches[0 .. *found) exactly as the reference does; entries from
 * *found on are not written (the reference leaves scratch there). Host
 * arrays; ms_device (may be NULL) receives the kernels' device time.
 * matches_count > ZS_MATCH_MAX_K returns ZS_ERR_UNSUPPORTED. */
int zs_find_matches(zs_ba_handle* h, const uint8_t* lhs, int64_t lhs_count, const uint8_t* rhs, int64_t rhs_count,
                    float threshold, int64_t matches_count, zs_match* matches, int64_t matches_size, int64_t* found,
                    double* ms_device);

/* ---- windowed bundle adjustment of a map: map::map::optimise (source/map.hpp:65-267) ----
 *
 * The map as arrays; frame_pose and landmarks are updated in place. With
 * local_window > 0 the window is selected as the reference does (79-127):
 * frames are fixed when their id is 0, 1 (maps of more than two frames) or
 * below frame_id_generator - local_window; landmarks seen by a non-fixed
 * frame are optimised with every frame that sees them within
 * 2 * local_window of the newest frame. local_window <= 0 optimises the whole
 * map (frames 0 and 1 fixed). With fix_landmarks, landmarks are fixed and
 * edges to fixed frames are dropped (the tracking mode, pose-only). Each
 * edge is a reprojection with loss_huber(sqrt(5.991)); frames are converted
 * to vertex_pose as so3(rotation matrix) (lie.hpp:159-180), frames without
 * edges leave the problem, and after `rounds` LM iterations (zs_ba_solve on
 * h, with h's options) every selected frame gets back so3::get_matrix of its
 * pose and every optimised landmark its location (239-252). The camera of
 * frame 0 is used for every edge, as the reference uses the first frame's.
 * Observations whose frame is not in the map (obs_frame -1) are skipped
 * (the reference requires every observing frame to be in the map). */
typedef struct zs_map_optimise_input {
    int32_t num_frames;               /* F */
    const int32_t* frame_id;          /* [F] frame::id */
    double* frame_pose;               /* [F*12] rotation (row-major) then translation; updated */
    const double* frame_intrinsics;   /* [F*4] fx, fy, cx, cy */
    int32_t num_landmarks;            /* L */
    const int32_t* landmark_id;       /* [L] */
    double* landmarks;                /* [L*3] updated */
    const int64_t* landmark_obs;      /* [L+1] observation ranges, map::observations order; [0] = 0 */
    const int32_t* obs_frame;         /* [M] frame index, or -1 */
    const float* obs_keypoint;        /* [M*2] */
    int32_t frame_id_generator;       /* frame::frame::id_generator */
} zs_map_optimise_input;

#define ZS_MAP_OPTIMISED 0            /* the problem was solved and written back */
#define ZS_MAP_NOTHING_TO_OPTIMISE 1  /* no frames, or no frame or landmark with an edge */
#define ZS_MAP_ALL_FIXED 2            /* no non-fixed pose or landmark */

typedef struct zs_map_optimise_report {
    int32_t outcome;     /* ZS_MAP_* */
    int32_t frames;      /* non-fixed poses in the problem (the reference's non_fixed_poses) */
    int32_t landmarks;   /* non-fixed landmarks (non_fixed_landmarks) */
    int32_t edges;       /* edges (non_fixed_edges) */
    int32_t problem_poses;      /* poses in the problem, fixed included */
    int32_t problem_landmarks;  /* landmarks in the problem */
    double ms_select;    /* host time of the window selection and problem assembly */
    zs_ba_report solve;  /* the solve (zeroed unless outcome == ZS_MAP_OPTIMISED) */
} zs_map_optimise_report;

/* Replaces map::map::optimise(local_window, fix_landmarks, rounds,
 * use_relative_convergence), source/map.hpp:65-267. Returns ZS_OK (see
 * rep->outcome), ZS_ERR_INVALID for bad arrays, or the solve's error. */
int zs_map_optimise(zs_ba_handle* h, zs_map_optimise_input* map, int32_t local_window, int32_t fix_landmarks,
                    int32_t rounds, int32_t use_relative, zs_map_optimise_report* rep);

/* The conversions zs_map_optimise applies, host only: a frame's rotation
 * matrix (row-major) and translation [12] to vertex_pose parameters
 * [tx ty tz qx qy qz qw] as so3(rotation matrix) (source/lie.hpp:159-180,
 * map.hpp:131-135), and back as so3::get_matrix (lie.hpp:188-204,
 * map.hpp:247-251); both round as the reference does. */
void zs_frame_to_pose(const double* frame_pose, double* pose);
void zs_pose_to_frame(const double* pose, double* frame_pose);

/* The window and graph zs_map_optimise would build, without a device or a
 * handle (host work only): pose_frame [F] receives the frame index of each
 * problem pose, landmark_index [L] the map landmark of each problem
 * landmark, edge_obs [M] the observation (index into the map's observation
 * arrays) of each edge, frame_written [F] 1 for the frames the optimise
 * would write back; rep the counts and the outcome (ms_select and solve
 * zero). Each output may be NULL. */
int zs_map_optimise_plan(const zs_map_optimise_input* map, int32_t local_window, int32_t fix_landmarks,
                         int32_t* pose_frame, int32_t* landmark_index, int64_t* edge_obs, uint8_t* frame_written,
                         zs_map_optimise_report* rep);

/* ---- map culling: map::map::cull (source/map.hpp:269-323) ----
 *
 * For each landmark, in the reference's order: kept untouched when
 * id + 500 < landmark_id_generator; erased when it has no observations;
 * erased when it has at most 4 and the frame id of its last one + 7 <
 * frame_id_generator; otherwise erased when none of its observations has a
 * frame in the map, or when the float mean over those that have of
 * |keypoint - projection| (5.991 where camera::pinhole::project fails) is
 * >= 5.991. Decisions and means are the reference's bit for bit. The caller
 * erases the flagged landmarks and their observation lists from its map, as
 * cull() does. */
typedef struct zs_map_cull_input {
    int32_t num_frames;               /* F */
    const double* frame_pose;         /* [F*12] frame::rotation (row-major 3x3) then frame::translation */
    const double* frame_intrinsics;   /* [F*4] fx, fy, cx, cy of each frame's camera::pinhole */
    int32_t num_landmarks;            /* L */
    const int32_t* landmark_id;       /* [L] landmark::point::id */
    const double* landmarks;          /* [L*3] landmark::point::location */
    const int64_t* landmark_obs;      /* [L+1] landmark l's observations are [landmark_obs[l], landmark_obs[l+1]),
                                         in the order of map::observations[id]; landmark_obs[0] = 0 */
    const int32_t* obs_frame;         /* [M] index of the observing frame in the frame arrays, or -1 when that
                                         frame is not in the map */
    const int32_t* obs_frame_id;      /* [M] id of the observing frame (observation::first) */
    const float* obs_keypoint;        /* [M*2] keypoint_pyramid[0][kp_index].x, .y of the observing frame */
    int32_t landmark_id_generator;    /* landmark::point::id_generator */
    int32_t frame_id_generator;       /* frame::frame::id_generator */
} zs_map_cull_input;

typedef struct zs_cull_report {
    int64_t erased;       /* landmarks flagged for erasure */
    int64_t error_passes; /* landmarks whose mean reprojection error was computed */
    double ms_device;     /* device time of the cull kernels (CUDA events) */
} zs_cull_report;

/* Culls a map given as host arrays on h's device (h needs no problem).
 * erase [L] (1 = erase), mean_error [L] (the mean compared with 5.991, -1
 * where it is not computed) and rep may each be NULL. Returns ZS_OK, or
 * ZS_ERR_INVALID for a frame index outside [-1, F) or decreasing ranges.
 * Replaces map::map::cull, source/map.hpp:269-323. */
int zs_map_cull(zs_ba_handle* h, const zs_map_cull_input* in, uint8_t* erase, float* mean_error,
                zs_cull_report* rep);

/* The same cull of the map that h's resident problem holds, at h's current
 * state, without copying it back: frames are the problem's poses, with the
 * rotation matrix and translation that map::optimise writes back into them
 * (source/map.hpp:247-251), observations are the problem's, each landmark's
 * in the problem's order, and every frame is in the map. landmark_id [L] and
 * pose_frame_id [K] give the ids. It is map::optimise (every landmark and
 * observation in the problem) followed by map::cull, with the cull's inputs
 * never leaving the device. Single problems only (ZS_ERR_UNSUPPORTED after
 * zs_ba_set_batch). */
int zs_ba_cull(zs_ba_handle* h, const int32_t* landmark_id, const int32_t* pose_frame_id,
               int32_t landmark_id_generator, int32_t frame_id_generator, uint8_t* erase, float* mean_error,
               zs_cull_report* rep);

/* Dense SPD solve on the device with the reference's pivot tests: factors the
 * row-major n x n matrix A = L L^T and solves L L^T x = b. L (n*n, lower, zero
 * above the diagonal) and x may be NULL. precision: ZS_PRECISION_FP64, or
 * ZS_PRECISION_MIXED (the mixed solve's preconditioner: FP32 factor and its
 * inverse, then FP64 refinement of x).
 * Returns ZS_OK, ZS_ERR_CHOLESKY, ZS_ERR_TIMEOUT (mixed: a bounded wait between
 * the factor's tile tasks ran out; nothing hangs) or a CUDA status. */
int zs_dense_cholesky_solve(const double* A, int n, const double* b, double* L, double* x, int precision);

/* Largest n accepted by zs_dense_cholesky_solve_noalloc. */
#define ZS_NOALLOC_MAX_N 384

/* zs_dense_cholesky_solve (FP64) for callers that must not allocate device
 * memory while they run: a real-time tracking thread that cannot block in
 * the allocator or risk an out-of-memory failure mid-sequence, or a host
 * application whose device memory belongs to another allocator. This entry
 * point has no counterpart in the reference; it calls no cudaMalloc, cudaFree
 * or other allocating routine. Its device workspace is one fixed array of
 * about 2.5 MB inside this library (sized for n <= ZS_NOALLOC_MAX_N) that
 * every device loading the library keeps until the process exits; larger n
 * returns ZS_ERR_INVALID. A, b, L and x are host pointers as in
 * zs_dense_cholesky_solve; L and x may be NULL. Runs on the current device's
 * legacy default stream and returns after the result is copied back. The
 * first call on each device looks the workspace address up, so make that
 * first call before any stream capture; the address is kept for the life of
 * the process, so after a cudaDeviceReset of a device this entry point must
 * not be called on that device again. All calls share the one workspace:
 * calls that overlap on the GPU (other host threads, other streams) race.
 * Returns ZS_OK, ZS_ERR_CHOLESKY (a pivot or solve test failed),
 * ZS_ERR_INVALID (null A or b, n <= 0 or n > ZS_NOALLOC_MAX_N) or
 * ZS_ERR_CUDA / ZS_ERR_OUT_OF_MEMORY (a CUDA call failed; zs_last_error()
 * names it). */
int zs_dense_cholesky_solve_noalloc(const double* A, int n, const double* b, double* L, double* x);

/* C = A B^T (or only its lower triangle, col <= row, with lower != 0 and
 * M >= N) for row-major FP32 host arrays A (M x K), B (N x K), C (M x N) on
 * the current device's tensor cores with FP32 accuracy (three TF32 products
 * per operand pair, FP32 accumulation): the product the mixed form's dense
 * preconditioner uses for large reduced systems. max_ctas > 0 caps the grid
 * (each CTA then walks several 128 x 128 tiles of C); 0: a CTA per tile.
 * *ms (may be NULL) receives the kernel's device time. No reference
 * counterpart: a test and measurement utility. Returns ZS_OK,
 * ZS_ERR_INVALID, ZS_ERR_TIMEOUT (a bounded wait inside the kernel ran out)
 * or a CUDA status. */
int zs_dense_gemm_nt_tf32x3(const float* A, const float* B, float* C, int M, int N, int K, int lower, int max_ctas,
                            double* ms);

/* The mixed form's FP32 preconditioner on a row-major n x n host matrix S
 * (only its lower triangle is read, as matrix::decompose_cholesky reads it):
 * the factor S = L L^T and X = L^-1 (both lower triangular; the upper
 * triangles of L and X come back zero; either may be NULL). form 0: as the
 * mixed solve chooses; 1: the dataflow kernel alone (64 x 64 tiles, any n);
 * 2: the blocked form (panels of 256 columns, the diagonal blocks by the
 * dataflow kernel and all other work as tensor-core products; needs
 * n % 4 == 0, else ZS_ERR_INVALID; the solves take it from n = 3072 on). *ms (may be NULL)
 * receives the device time of the factor and inverse. No reference
 * counterpart beyond matrix::decompose_cholesky
 * (source/matrix_decomposition_cholesky.hpp:26-61): a test and measurement
 * utility. Returns ZS_OK, ZS_ERR_CHOLESKY (a pivot was not positive),
 * ZS_ERR_INVALID, ZS_ERR_TIMEOUT or a CUDA status. */
int zs_dense_chol_inverse_f32(const float* S, int n, float* L, float* X, int form, double* ms);

/* Measures the FP64 and FP32 fused multiply-add pipe peaks of `device` with
 * a register-resident FMA chain on every SM (TFLOP/s, 2 flops per FMA). A
 * measurement utility for roofline reports; no reference counterpart. */
int zs_pipe_peaks(int device, double* fp64_tflops, double* fp32_tflops);

const char* zs_ba_status_string(int status);

/* The CUDA error behind the last ZS_ERR_CUDA / ZS_ERR_OUT_OF_MEMORY returned
 * on this host thread ("" if none). */
const char* zs_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* ZEROSLAM_BA_H */
