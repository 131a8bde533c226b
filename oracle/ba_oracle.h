/*
 * CPU restatement of zeroslam's factor-graph bundle adjustment, in plain C99.
 *
 * TEST INFRASTRUCTURE ONLY. This is the oracle that the CUDA path is checked
 * against; the product path never links or calls it. Only tests/, the smoke
 * check in __graft_entry__.py and bench.py's CPU-baseline leg load it.
 *
 * It restates, in double precision and with a fixed summation order:
 *   source/factor_graph.hpp:489-615  factor_graph::solve (LM driver)
 *   source/factor_graph.hpp:618-629  get_current_chi
 *   source/factor_graph.hpp:648-732  make_hessian
 *   source/factor_graph.hpp:736-806  solve_linear_system
 *   source/factor_graph.hpp:809-846  update_states / rollback_states
 *   source/factor_graph.hpp:851-934  loss_trivial / huber / cauchy / tukey
 *   source/factor_graph.hpp:947-960  vertex_pose::plus
 *   source/factor_graph.hpp:990-1048 edge_reprojection residual and Jacobians
 *   source/matrix.hpp:749-774        invert<3>
 *   source/matrix_decomposition_cholesky.hpp:26-95
 *   source/lie.hpp:188-204,247-264,284-294,337-362,446-450,521-531
 *   source/camera.hpp:91-142
 *   source/map.hpp:247-251,269-323   frame write-back and map::cull
 *   source/lie.hpp:159-180           so3 from a rotation matrix (map::optimise)
 *   source/feature.hpp:1133-1235     distance<256> and find_matches
 * The reference stores H_pl in a hash map and sums the Schur products in
 * hash-iteration order; this restatement sums per landmark in ascending
 * landmark order, so results agree to rounding, not bit for bit.
 */
#ifndef ZS_BA_ORACLE_H
#define ZS_BA_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct zso_problem {
    int num_poses;
    int num_landmarks;
    long long num_obs;
    double* poses;                 /* [K*7] tx ty tz qx qy qz qw, updated in place */
    const unsigned char* pose_fixed;
    double* landmarks;             /* [L*3], updated in place */
    const unsigned char* landmark_fixed;
    const int* obs_pose;           /* [M] */
    const int* obs_landmark;       /* [M] */
    const double* obs_uv;          /* [M*2] */
    const double* obs_info;        /* [M*4] row-major 2x2, or NULL for identity */
    double intrinsics[4];          /* fx fy cx cy */
    int loss_kind;                 /* 0 none, 1 huber, 2 cauchy, 3 tukey */
    double loss_delta;
} zso_problem;

typedef struct zso_report {
    int iterations;    /* outer LM iterations run */
    int accepted;      /* accepted steps: the value solve() returns */
    int attempts;      /* linear solves attempted */
    int chol_failures; /* attempts whose reduced Cholesky failed */
    double chi2_initial;
    double chi2_final;
    double lambda_final;
} zso_report;

/* Per-edge residual and Jacobians (J_p 2x6 row-major, J_l 2x3 row-major).
 * Returns 1 when the point projects (Z >= 1e-12), 0 for the behind-camera
 * penalty branch. Jp / Jl may be NULL. */
int zso_edge(const double pose[7], const double X[3], const double uv[2], const double intr[4],
             double r[2], double Jp[12], double Jl[6]);

/* rho[0..2] of the robust loss at squared error e2. */
void zso_loss(int kind, double delta, double e2, double rho[3]);

/* Sum of robust chi2 over all edges at the current state. */
double zso_chi2(const zso_problem* p);

/* Host threads the restatement may use for its loops (default 1). Results
 * are bit-for-bit the same for every thread count: threads own disjoint
 * outputs and every sum keeps its serial order. */
void zso_set_threads(int n);
int zso_get_threads(void);

/* 3x3 inverse with zeroslam's |det| > 1e-12 * max|a|^3 test; out = 0 and
 * returns 0 when singular. */
int zso_invert3(const double A[9], double out[9]);

/* Row-major dense Cholesky A = L L^T and the two triangular solves, with
 * zeroslam's pivot thresholds. Return 1 on success, 0 on failure. */
int zso_cholesky(const double* A, int n, double* L);
int zso_cholesky_solve(const double* L, const double* b, int n, double* x);

/* T <- exp(delta) * T on a [tx ty tz qx qy qz qw] pose, delta = (omega, upsilon). */
void zso_pose_plus(double pose[7], const double delta[6]);

/* Linearise at the current state and solve the damped system once at
 * `lambda`. Any output pointer may be NULL:
 *   S [n*n] reduced camera matrix (damped), bs [n], delta [6K+3L],
 *   b [6K+3L] gradient vector, hpp [K*36], hll [L*9] (undamped).
 * Returns 1 on success, 0 when the reduced Cholesky failed. */
int zso_linear_step(const zso_problem* p, double lambda, double* S, double* bs, double* delta,
                    double* b, double* hpp, double* hll);

/* Initial damping tau * min(5e10, max diagonal) at the current state. */
double zso_initial_lambda(const zso_problem* p);

/* Full Levenberg-Marquardt solve; returns the accepted-step count. */
int zso_solve(zso_problem* p, int iterations, int use_relative, zso_report* rep);

/* The same solve one outer iteration at a time (zso_solve is begin, up to
 * `iterations` calls of zso_lm_iteration, end): zso_lm_begin linearises and
 * sets the initial damping (source/factor_graph.hpp:494-536);
 * zso_lm_iteration runs one pass of the outer loop (:538-611) and returns 0
 * once a stop rule has fired; zso_lm_end fills the report, frees the state and
 * returns the accepted-step count; zso_lm_report reads the report so far.
 * p is updated in place. */
typedef struct zso_lm zso_lm;
zso_lm* zso_lm_begin(zso_problem* p, int use_relative);
int zso_lm_iteration(zso_lm* m);
int zso_lm_end(zso_lm* m, zso_report* rep);
/* The report of the iterations run so far (the solve continues). */
void zso_lm_report(const zso_lm* m, zso_report* rep);

/* Map culling, source/map.hpp:269-323, over a map given as arrays (the layout
 * of zs_map_cull_input in include/zeroslam_ba.h). */
typedef struct zso_cull_map {
    int num_frames;
    const double* frame_pose;        /* [F*12] rotation (row-major) then translation */
    const double* frame_intrinsics;  /* [F*4] fx fy cx cy */
    int num_landmarks;
    const int* landmark_id;          /* [L] */
    const double* landmarks;         /* [L*3] */
    const long long* landmark_obs;   /* [L+1] */
    const int* obs_frame;            /* [M] frame index or -1 (frame not in the map) */
    const int* obs_frame_id;         /* [M] */
    const float* obs_keypoint;       /* [M*2] */
    int landmark_id_generator;
    int frame_id_generator;
} zso_cull_map;

/* erase[l] = 1 when map::cull erases landmark l; mean_error[l] = the float
 * mean reprojection error it compares with 5.991, or -1 where the error pass
 * does not run (old landmarks, landmarks erased before it). Either output
 * may be NULL. Returns the number erased. */
long long zso_map_cull(const zso_cull_map* m, unsigned char* erase, float* mean_error);

/* Rotation matrix and translation written back to a frame from a
 * [tx ty tz qx qy qz qw] vertex, source/map.hpp:247-251 with
 * source/lie.hpp:188-204: Rt = (R row-major, t). */
void zso_pose_rt(const double pose[7], double Rt[12]);

/* The vertex_pose parameters [tx ty tz qx qy qz qw] map::optimise builds
 * from a frame's rotation matrix and translation, source/map.hpp:131-135
 * with the so3-from-matrix conversion of source/lie.hpp:159-180. */
void zso_rt_pose(const double Rt[12], double pose[7]);

/* feature::find_matches with distance<256>, source/feature.hpp:1133-1235:
 * for each lhs descriptor (32 bytes) in order, while count + k <= size, the
 * k smallest Hamming distances to the rhs descriptors (scanned in order,
 * strict improvement, so ties keep the earlier rhs) that are below the
 * threshold. matches: [size] of (lhs, rhs, score). Returns the count. */
typedef struct zso_match {
    unsigned long long lhs_index;
    unsigned long long rhs_index;
    float score;
} zso_match;
long long zso_find_matches(const unsigned char* lhs, long long n_lhs, const unsigned char* rhs, long long n_rhs,
                           float threshold, long long k, zso_match* matches, long long size);

#ifdef __cplusplus
}
#endif

#endif
