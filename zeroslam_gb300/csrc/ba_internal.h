// Internal interfaces between the C ABI layer (ba_api.cu) and the kernels
// (ba_kernels.cu, ba_cholesky.cu). Device pointers only; no torch types.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "ba_common.cuh"

#include <atomic>

struct zs_ba_attempt;

namespace zs {

// A value computed once per device (launch configurations: SM counts,
// occupancies, function attributes) so that the launch paths of the solve
// loop make no runtime queries: f() runs on the first call for the current
// device and must return a positive value, or a non-positive one that is
// not cached.
constexpr int kMaxDevices = 64;
template <typename F>
int per_device(std::atomic<int> (&slot)[kMaxDevices], F f) {
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= kMaxDevices) return f();
    int v = slot[dev].load(std::memory_order_acquire);
    if (v > 0) return v;
    v = f();
    if (v > 0) slot[dev].store(v, std::memory_order_release);
    return v;
}

// Device-resident problem and structure. Observations are stored
// landmark-major (sorted by landmark, then pose); "blocks" are the
// observations that own an H_pl block (pose and landmark both free, first
// of any duplicate (pose, landmark) run).
struct DevProblem {
    int K = 0, L = 0;
    int64_t M = 0;
    int n = 0;                     // 6K
    double* pose = nullptr;        // [K*8]
    double* pose_bk = nullptr;     // [K*8]
    double* lm = nullptr;          // [L*4]
    double* lm_bk = nullptr;       // [L*4]
    double* pose_init = nullptr;   // [K*8] state uploaded with the problem
    double* lm_init = nullptr;     // [L*4]
    uint8_t* pose_fixed = nullptr; // [K]
    uint8_t* lm_fixed = nullptr;   // [L]
    int32_t* obs_pose = nullptr;   // [M] landmark-major
    int32_t* obs_lm = nullptr;     // [M]
    double2* obs_uv = nullptr;     // [M]
    double* obs_info = nullptr;    // [M*4] or null
    int32_t* lm_ptr = nullptr;     // [L+1] observation ranges per landmark
    int32_t* pose_ptr = nullptr;   // [K+1] ranges into pose_obs
    int32_t* pose_obs = nullptr;   // [M] observations of each pose (landmark-major index), ascending
    uint8_t* blk_valid = nullptr;  // [M] 1 if the observation owns an H_pl block
    int32_t* dup_owner = nullptr;  // [M] owner of the duplicate run (== self when unique), or null
    bool has_dups = false;
    // Schur structure: pairs (i >= j) of poses sharing landmarks; triples
    // (block of pose i, block of pose j) grouped by pair, landmark order within a pair.
    int npairs = 0;
    int64_t ntriples = 0;
    int32_t* pair_i = nullptr;         // [npairs]
    int32_t* pair_j = nullptr;         // [npairs]
    int2* triples = nullptr;           // [ntriples] pose-major record positions (of pose i, of pose j)
    int64_t nsegs = 0;                 // segments: <= 512 consecutive triples of one pair
    int64_t* seg_ptr = nullptr;        // [nsegs+1] triple ranges per segment
    int32_t* seg_pair = nullptr;       // [nsegs] pair of each segment
    int64_t* pair_seg_ptr = nullptr;   // [npairs+1] segment ranges per pair
    int32_t* pm = nullptr;             // [M] pose-major position of each (landmark-major) observation
    Intrinsics intr{};
    LossParams loss{};
    // Batched windows (null / 1 for a single problem): poses, landmarks and
    // observations of window w are contiguous; S is block diagonal, window
    // w's n_w x n_w block (n_w = 6 K_w) at S + win_s_off[w].
    int nwin = 1;
    int32_t* pose_win = nullptr;   // [K] window of each pose
    int32_t* lm_win = nullptr;     // [L] window of each landmark
    int32_t* win_pose0 = nullptr;  // [nwin+1] first pose of each window
    int32_t* win_lm0 = nullptr;    // [nwin+1] first landmark of each window
    int64_t* win_s_off = nullptr;  // [nwin] offset of the window's S block
    int64_t nochunks = 0;          // observation chunks for per-window sums
    int64_t* ochunk_ptr = nullptr; // [nochunks+1] observation ranges (never across windows)
    int32_t* ochunk_win = nullptr; // [nochunks] window of each chunk
    int32_t* win_ochunk = nullptr; // [nwin+1] chunk ranges per window
    // Pose-major observation chunks of the mixed form's FP64 Schur operator:
    // chunk c covers pose-major positions [opch_q[c], opch_q[c+1]) of one pose,
    // pose k's chunks are [pose_opch[k], pose_opch[k+1]).
    int64_t nopch = 0;
    int32_t* opch_q = nullptr;     // [nopch+1]
    int32_t* pose_opch = nullptr;  // [K+1]
    // Landmark chunks of the same operator: chunk c holds landmarks
    // [lmch_l[c], lmch_l[c+1]), consecutive, <= kOpChunk observations in all
    // (or one landmark with more).
    int64_t nlmch = 0;
    int32_t* lmch_l = nullptr;     // [nlmch+1]
};

// At most this many observations per operator chunk (a warp's share).
constexpr int kOpChunk = 64;

// Per-observation record of the mixed form (landmark-major, 112 bytes): the
// FP32 Jacobian blocks J_p (2 x 6) and J_l (2 x 3) that the FP32 Schur
// records are built from, the robust weight W (2 x 2, row-major, FP32) and
// the gradient factor g = rho' Omega r as two double-float values (hi, lo,
// hi, lo). The mixed form's FP64-accurate Schur operator, b_l and H_ll are
// sums over exactly these values.
struct alignas(16) ObsJac {
    float g[4];
    float jp[12];
    float jl[6];
    float w[4];
    float pad[2];
};
static_assert(sizeof(ObsJac) == 112, "ObsJac is seven 16-byte vectors");

// Working arrays of one precision (T = double for the plain form, float for
// the mixed form).
struct TcStreams;

struct DevWork {
    void* hpl = nullptr;       // [M*RS] T, RS = 18 (double) or 20 (float, padded); pose-major positions
    void* W = nullptr;         // [M*RS] T, pose-major positions
    double* pose_aux = nullptr; // [K*24] mixed form: per-pose sandwich matrix, translation, rotation
    double* partial = nullptr; // [nsegs*36] Schur segment sums (FP64)
    void* lm_part = nullptr;   // plain form: [M*12] per-observation landmark records (9 used)
    ObsJac* jac = nullptr;     // mixed form: [M] per-observation Jacobian records
    float4* jp_pm = nullptr;   // mixed form: [3M] J_p of each record again, pose-major positions, three planes
    double* pcg = nullptr;     // mixed form: PCG vectors and operator scratch (pcg_doubles)
    void* pose_part = nullptr; // [M*28] T, per-observation pose records (27 used), pose-major positions
    double* hpp = nullptr;     // [K*36]
    double* hll = nullptr;     // [L*9]
    double* hll_inv = nullptr; // [L*9]
    float* hll_inv_f = nullptr; // mixed form: [L*12] the same in FP32, padded for 16-byte loads
    double* b = nullptr;       // [n + 3L] gradient vector (poses then landmarks)
    double* S = nullptr;       // [n*n] reduced camera matrix, FP64 in both forms
    void* F = nullptr;         // [n*n] Cholesky factor (lower): double (plain form) or float (mixed)
    void* D = nullptr;         // [ceil(n/32)*1024] T, inverses of F's diagonal blocks
    double* bs = nullptr;      // [n]
    double* work = nullptr;    // [4n + 256] triangular-solve and refinement vectors
    void* X = nullptr;         // mixed form: [n*n] L^-1 (lower)
    void* XT = nullptr;        // mixed form: [n*n] (L^-1)^T (upper)
    int* dag_flags = nullptr;  // mixed form: [dag_flag_ints(n)] tile flags of the preconditioner's launch
    int dag_epoch = 0;         // mixed form: epoch of its last launch (host side)
    float* tc_scratch = nullptr;  // mixed form at large n: panels of the blocked preconditioner
    TcStreams* tc_streams = nullptr;  // and its streams (owned by the handle)
    double* delta = nullptr;   // [n + 3L]
    double* red = nullptr;     // [kReduceBlocks * 4] reduction partials
    double* opch_sum = nullptr; // [6 nopch] per-chunk partial sums of per-pose reductions (launch_pose_sums6)
    int32_t* ired = nullptr;   // [kReduceBlocks]
};

// Device LM state (source/factor_graph.hpp:511-611), read back once per attempt.
struct LmState {
    double lambda;
    double nu;
    double chi2;       // current accepted cost
    double chi2_new;   // cost after the trial step
    double scale;      // sum delta (lambda delta + b) + 1e-3
    double rho;
    double max_diag;
    double eps_factor; // 1e-14 * max |S_ii|
    double eps_solve;  // 1e-7 * max |L_ii|
    double resid_norm; // mixed form: last refinement residual norm
    double rhs_norm;
    int32_t solve_ok;  // reduced Cholesky factor and solve passed
    int32_t good;      // trial step accepted
    int32_t nonfinite;
    int32_t refine_sweeps;  // refinement sweeps of the last reduced solve
    int32_t skip_factor;    // mixed form: the factor kernels return at once (no retry armed)
    int32_t shifted;        // mixed form: the last preconditioner factor needed the diagonal shift
    int32_t timeout;        // a bounded device wait ran out (the launch gave up; solve_ok = 0)
};

// Per-window LM control of a batched solve (source/factor_graph.hpp:538-611
// restated as a state machine advanced once per attempt round).
struct WinCtl {
    int32_t active;        // still iterating
    int32_t it;            // completed outer iterations
    int32_t iterations;    // outer iterations reported (factor_graph::solve's loop count)
    int32_t failures;      // failed attempts in the current outer iteration
    int32_t accepted;      // accepted steps (the reference's return value)
    int32_t attempts;
    int32_t chol_failures;
    int32_t refine_sweeps;
    int32_t rollback;      // the last attempt was rejected and must be undone
    int32_t pad;
    double last;           // cost at the start of the current outer iteration
    double legacy;         // legacy stop threshold (legacy_stop * initial cost)
    double chi2_initial;
};

// Records e as this host thread's zs_last_error() text, clears CUDA's
// last-error state and returns the status for it (ZS_ERR_CUDA or
// ZS_ERR_OUT_OF_MEMORY). Defined with the C ABI (ba_api.cu).
int record_cuda_error(cudaError_t e);

// ---- kernels (ba_kernels.cu) ----
template <typename T>
void launch_linearize(const DevProblem& P, DevWork& W, cudaStream_t s);
template <typename T>
void launch_invert_w(const DevProblem& P, DevWork& W, const LmState* st, cudaStream_t s);
template <typename T>
void launch_schur(const DevProblem& P, DevWork& W, const LmState* st, cudaStream_t s);
template <typename T>
void launch_backsub(const DevProblem& P, DevWork& W, const LmState* st, cudaStream_t s);
// b_s = b_p - W b_l from the current W.b (no other Schur work).
template <typename T>
void launch_bs(const DevProblem& P, DevWork& W, cudaStream_t s);
// W = H_pl H_ll^-1 from the current inverses (no inversion).
template <typename T>
void launch_w(const DevProblem& P, DevWork& W, cudaStream_t s);
// S_ij -= the pairs' W_i H_j^T sums (after the S blocks' initialisation);
// with windows, stopped windows (ctl) are skipped.
template <typename T>
void launch_schur_pairs(const DevProblem& P, DevWork& W, const WinCtl* ctl, cudaStream_t s);
void launch_update(const DevProblem& P, DevWork& W, const LmState* st, cudaStream_t s);
void launch_rollback(const DevProblem& P, const LmState* st, cudaStream_t s);
void launch_scale(const DevProblem& P, DevWork& W, LmState* st, cudaStream_t s);
// cost of the current state into st->chi2_new (when only_if_ok, skipped if !st->solve_ok)
void launch_cost(const DevProblem& P, DevWork& W, LmState* st, bool only_if_ok, cudaStream_t s);
// the mixed form's cost (per-pose sandwich matrices of the current poses, then FP64 residuals)
void launch_cost_fast(const DevProblem& P, DevWork& W, LmState* st, bool only_if_ok, cudaStream_t s);
void launch_pose_aux(const DevProblem& P, DevWork& W, cudaStream_t s);
void launch_init_lambda(const DevProblem& P, DevWork& W, LmState* st, double tau, double clamp, cudaStream_t s);
void launch_decide(LmState* st, cudaStream_t s);
void launch_set_solve_ok(LmState* st, int v, cudaStream_t s);

// ---- batched windows (ba_batch.cu) ----
constexpr int kBatchBuckets = 5;     // reduced-solve size buckets: n <= 64, 96, 128, 160, 192
constexpr int kBatchMaxK = 32;       // poses per window (n <= 192)
constexpr int kBatchObsChunk = 2048; // observations per cost chunk

inline int batch_bucket(int n) {
    const int ns = (n + 31) / 32;
    return ns <= 2 ? 0 : ns - 2;
}

struct BatchParams {
    int iterations;
    int use_relative;
    int max_failures;
    int refine_iters;
    int max_rounds;
    int use_cond;
    double relative_tolerance;
    double chi2_floor;
    double legacy_stop;
    double tau;
    double clamp;
    double refine_tol;
    cudaGraphConditionalHandle cond;
};

// What the reduced-solve kernel needs of a batch.
struct BatchView {
    double* S;
    const double* bs;
    double* delta;
    LmState* st;
    WinCtl* ctl;
    const int32_t* win_pose0;
    const int64_t* win_s_off;
    long long* prof;  // with options.profile: [nwin][kBatchProfSlots] SM cycles per phase, else null
};
// load, factor, first solve, refinement, refinement sweeps
constexpr int kBatchProfSlots = 5;

struct BatchDev {
    LmState* st = nullptr;       // [nwin]
    WinCtl* ctl = nullptr;       // [nwin]
    int* counters = nullptr;     // [kBatchBuckets] work-queue heads
    int* any_active = nullptr;   // [1]
    int* rounds = nullptr;       // [1] attempt rounds run
    long long* prof = nullptr;   // [nwin * kBatchProfSlots] (options.profile)
    int32_t* lists = nullptr;    // [nwin] windows by bucket, largest first within a bucket
    int bucket_off[kBatchBuckets + 1] = {0};
    int threads[kBatchBuckets] = {0};
    int blocks[kBatchBuckets] = {0};
    // the buckets' reduced solves run concurrently: forked from the main
    // stream by ev_fork, joined back by ev_join
    cudaStream_t streams[kBatchBuckets] = {nullptr};
    cudaEvent_t ev_fork = nullptr;
    cudaEvent_t ev_join[kBatchBuckets] = {nullptr};
};

template <typename T>
void launch_batch_prologue(const DevProblem& P, DevWork& W, BatchDev& B, const BatchParams& prm, cudaStream_t s);
template <typename T>
cudaError_t launch_batch_round(const DevProblem& P, DevWork& W, BatchDev& B, const BatchParams& prm, cudaStream_t s);
// Times the reduced-solve kernel of one bucket on synthetic SPD blocks for
// each candidate block size; returns the fastest block size and the number
// of its CTAs resident per SM.
template <typename TF>
cudaError_t bsolve_autotune(int bucket, int sms, cudaStream_t s, int* threads_out, int* blocks_per_sm_out,
                            float* us_out);
template <typename TF>
int bsolve_max_blocks_per_sm(int bucket, int threads);

// ---- adjoint (ba_adjoint.cu) ----
constexpr int kAdjRecord = 64;  // doubles per observation in the adjoint record
void launch_adj_prep(const DevProblem& P, double* rec, cudaStream_t s);
void launch_adj_residual(const DevProblem& P, const double* rec, const double* v, const double* a, double* part,
                         double* csum, double* out, cudaStream_t s);
// The adjoint's preconditioner with an explicit inverse of its fixed FP64
// reduced factor (n <= kAdjInvMaxN): Xi = L^-1 and XiT once, then
// y = XiT (Xi b) per application (tmp: n doubles).
constexpr int kAdjInvMaxN = 1024;
constexpr int kAdjInvWarps = 4;  // columns per CTA (shared memory: 8 n bytes each)
void launch_adj_tri_inverse(int n, const double* L, double* Xi, double* XiT, cudaStream_t s);
void launch_adj_apply_inverse(int n, const double* Xi, const double* XiT, const double* b, double* tmp, double* y,
                              cudaStream_t s);
void launch_adj_axpby(int64_t N, double alpha, const double* x, double beta, double* y, cudaStream_t s);
void launch_adj_dot(int64_t N, const double* x, const double* y, double* red, cudaStream_t s);
void launch_adj_copy(int64_t N, const double* src, double* dst, cudaStream_t s);
void launch_adj_out(const DevProblem& P, const double* rec, const double* v, double* duv, double* red, cudaStream_t s);
// Scalars of the adjoint's conjugate-gradient loop, kept on the device.
struct AdjCg {
    double rz, alpha, beta, rn, anorm, tol;
    int32_t it, max_it, done, pad;  // done: 1 converged, 2 H not positive along p, 3 iteration limit
};
void launch_adj_cg_pap(const double* red, AdjCg* c, cudaStream_t s);
void launch_adj_cg_rn(const double* red, AdjCg* c, cudaStream_t s);
void launch_adj_cg_rz(const double* red, AdjCg* c, cudaStream_t s);
void launch_adj_cg_axpby(int64_t N, const AdjCg* c, int which, const double* x, double* y, cudaStream_t s);

// ---- map culling (ba_cull.cu) ----
// Inputs of k_cull: L landmarks (lm, lm_stride doubles apart, ids lm_id),
// their observations (ranges obs_ptr, frame index obs_frame, -1 when the
// frame is not in the map), F frames (Rt: 12 doubles each, rotation then
// translation; intrinsics intr, intr_stride doubles apart: 4 per frame or 0
// for one camera) and the frame id of each observation (obs_frame_id) or of
// each frame (frame_id, used when obs_frame_id is null). Outputs: erase[L],
// mean[L] (-1 where no error pass runs) and counters (erased, error passes,
// invalid input), which the caller zeroes.
struct CullArgs {
    int L = 0, F = 0;
    int64_t M = 0;  // observations: every range must lie in [0, M]
    const double* Rt = nullptr;
    const double* intr = nullptr;
    int intr_stride = 0;
    const double* lm = nullptr;
    int lm_stride = 3;
    const int32_t* lm_id = nullptr;
    const int32_t* obs_frame = nullptr;
    const int32_t* obs_frame_id = nullptr;
    const int32_t* frame_id = nullptr;
    int32_t lm_gen = 0, frame_gen = 0;
    uint8_t* erase = nullptr;
    float* mean = nullptr;
    unsigned long long* counters = nullptr;
};
void launch_pose_rt(int K, const double* pose, double* Rt, cudaStream_t s);
void launch_cull(const CullArgs& a, const int64_t* obs_ptr, const float2* kp, cudaStream_t s);
void launch_cull(const CullArgs& a, const int32_t* obs_ptr, const double2* kp, cudaStream_t s);

// ---- descriptor matching (ba_match.cu) ----
// Chunks of the rhs for n_lhs x n_rhs matching; launch_match writes, per lhs,
// the k smallest keys (distance << 32 | rhs index) with distance < d_lim into
// out [n_lhs * k] (~0 where fewer), using part [chunks * n_lhs * k] when
// chunks > 1. lhs and rhs: 32-byte descriptors, 16-byte aligned.
int match_chunks(int n_lhs, int n_rhs);
void launch_match(const uint8_t* lhs, int n_lhs, const uint8_t* rhs, int n_rhs, int k, int d_lim, int chunks,
                  unsigned long long* part, unsigned long long* out, cudaStream_t s);

// ---- dense reduced system (ba_cholesky.cu) ----
// launch_factor: S (n x n row-major, type TS) -> F = L (lower, type TF) and
// D = the inverses of L's 32 x 32 diagonal blocks ([ceil(n/32) * 1024] TF);
// sets st->solve_ok = 0 on a failed pivot or solve test.
// launch_solve_refine: x = (L L^T)^-1 bs, then up to refine_iters FP64
// refinement sweeps against S until ||bs - S x|| <= tol ||bs||. work needs
// 4n + 16 doubles. Both return the launch error, if any.
template <typename TS, typename TF>
cudaError_t launch_factor(int n, const TS* S, TF* F, TF* D, LmState* st, cudaStream_t s);
template <typename TS, typename TF>
cudaError_t launch_solve_refine(int n, const TS* S, const TF* F, const TF* D, const double* bs, double* x,
                                double* work, LmState* st, int refine_iters, double tol, cudaStream_t s);
template <typename TS, typename TF>
cudaError_t launch_reduced_solve(int n, const TS* S, TF* F, TF* D, const double* bs, double* x, double* work,
                                 LmState* st, int refine_iters, double tol, cudaStream_t s);


// ---- mixed form: the preconditioner (ba_chol_dag.cu) ----
// F (n x n FP32, the matrix) -> L in F's lower triangle (zeros above the
// diagonal inside the 64 x 64 diagonal tiles), X = L^-1 (lower, with its
// diagonal) and XT = X^T (upper), in one cooperative launch of per-tile
// tasks with dependency flags; pivot test d > st->eps_factor. A failed pivot
// sets st->solve_ok = 0; a wait that runs out also sets st->timeout. flags:
// dag_flag_ints(n) ints, zero before the first launch that uses them; *epoch
// advances per launch. Returns at once when st->skip_factor is set.
int dag_flag_ints(int n);
cudaError_t launch_chol_inverse_dag(int n, float* F, float* X, float* XT, LmState* st, int* flags, int* epoch,
                                    cudaStream_t s);
// C (M x N) = alpha A B^T + beta C on the FP32 pipe in 64 x 64 tiles (small
// products; lower: only C's lower triangle); returns at once when
// st->skip_factor is set or st->solve_ok clear. A, B 16-byte aligned, lda,
// ldb multiples of 4.
cudaError_t launch_gemm_nt64(int M, int N, int K, const float* A, int lda, const float* B, int ldb, float* C, int ldc,
                             float alpha, float beta, bool lower, const LmState* st, cudaStream_t s);
// The same for the n x n block at F, X, XT of matrices with row stride ld.
cudaError_t launch_chol_inverse_dag_ld(int n, int ld, float* F, float* X, float* XT, LmState* st, int* flags,
                                       int* epoch, cudaStream_t s);
// Blocked form for large n (ba_chol_tc.cu): panels of kPanel columns, the
// diagonal blocks by the dataflow kernel and the rest on the tensor cores.
// It applies from kTcMinN on with n % 4 == 0; scratch holds
// chol_tc_scratch_floats(n) floats (16-byte aligned).
constexpr int kPanel = 256;
constexpr int kTcMinN = 3072;
bool chol_tc_applies(int n);
int chol_tc_scratch_floats(int n);
// The blocked form's streams (high priority: the factorisation's chain and
// the work beside it; low: the bulk of the products) and its events, for
// matrices up to n.
struct TcStreams {
    cudaStream_t hi = nullptr, mid = nullptr, lo = nullptr;
    std::vector<cudaEvent_t> ev;
    cudaError_t init(int n);
    void release();
    static int panels_of(int n);
    ~TcStreams();
};
// Enqueued after everything before it on s; s waits for all of it.
cudaError_t launch_chol_inverse_tc(int n, float* F, float* X, float* XT, float* scratch, LmState* st, int* flags,
                                   int* epoch, TcStreams& ts, cudaStream_t s);
// eps from S's diagonal, F = S in FP32, the factor and inverse (blocked when
// scratch and ts are given and chol_tc_applies(n), else the dataflow kernel
// alone),
// and the reference's solve test on L's diagonal.
cudaError_t launch_factor_dag(int n, const double* S, float* F, float* X, float* XT, float* scratch, TcStreams* ts,
                              LmState* st, int* flags, int* epoch, cudaStream_t s);
// The whole preconditioner of an attempt: eps from S's diagonal, F = S in
// FP32, the factor and inverse; when that fails, once more on
// S + mu diag(S) (st->shifted); then the reference's solve test on L's
// diagonal (source/matrix_decomposition_cholesky.hpp:74,80,89).
cudaError_t launch_preconditioner(int n, const double* S, float* F, float* X, float* XT, float* scratch,
                                  TcStreams* ts, LmState* st, double mu, int* flags, int* epoch, cudaStream_t s);

// ---- pose-only problems in one launch (ba_pose_only.cu) ----
// Every landmark fixed and at most kPoseOnlyMaxK poses: one cooperative
// launch of `grid` CTAs (pose_only_grid(M)) runs the whole LM loop (FP64) on
// the poses in P.pose. Device memory: out, hist (hist_cap attempt records),
// part [grid * K * 27], sums [K * 27], cpart [grid].
constexpr int kPoseOnlyMaxK = 64;
// At most this many free poses: each free pose's sums take one pass of the
// grid (the FP64 pipe bounds it), so problems with more free poses are
// faster on the general path (measured: 16 free poses 2.42 against 2.03 ms).
constexpr int kPoseOnlyMaxFree = 4;
struct PoseOnlyCtl {
    double tau, clamp, legacy_stop, rel_tol, floor;
    int max_failures, iterations, use_relative, hist_cap;
};
struct PoseOnlyOut {
    int iterations, attempts, accepted, cholesky_failures, history;
    double chi2_initial, chi2_final, lambda_final;
};
int pose_only_grid(int64_t M);
// A batch whose landmarks are all fixed: one CTA per window (at most
// kPoseOnlyMaxK poses each), reports into wctl / wst as the general batched
// path's per-window control and state.
cudaError_t launch_pose_only_windows(const DevProblem& P, const PoseOnlyCtl& ctl, WinCtl* wctl, LmState* wst,
                                    cudaStream_t s);
cudaError_t launch_pose_only_lm(const DevProblem& P, const PoseOnlyCtl& ctl, PoseOnlyOut* out, zs_ba_attempt* hist,
                                double* part, double* sums, double* cpart, int grid, cudaStream_t s);

// ---- FP32 products on the tensor cores (ba_tc_gemm.cu) ----
// C (M x N, row stride ldc) = alpha A B^T + beta C, A (M x K) and B (N x K)
// row-major with K contiguous, three TF32 products per operand pair (FP32
// accuracy). Needs lda, ldb multiples of 4 and 16-byte aligned A, B
// (tc_gemm_supported). lower: only C's lower triangle (col <= row) is
// written (C square or taller than wide). A wait that runs out sets *err = 1
// (device int). With st, the launch returns at once when st->skip_factor is
// set or st->solve_ok clear, and a wait that runs out also clears
// st->solve_ok. max_ctas > 0 caps the grid (each CTA walks several tiles),
// leaving the other SMs to concurrent streams.
bool tc_gemm_supported(int lda, int ldb, const float* A, const float* B);
cudaError_t launch_tc_gemm_nt(int M, int N, int K, const float* A, int lda, const float* B, int ldb, float* C, int ldc,
                              float alpha, float beta, bool lower, int* err, cudaStream_t s, LmState* st = nullptr,
                              int max_ctas = 0);

// ---- mixed form (ba_inverse.cu) ----
// Dense mixed solves (zs_dense_cholesky_solve): x = X^T X bs, then FP64
// refinement x += X^T X (bs - S x) until ||bs - S x|| <= tol ||bs|| or
// refine_iters sweeps; work: 4n + 256 doubles.
template <typename TS, typename TX>
cudaError_t launch_refine(int n, const TS* S, const TX* X, const TX* XT, const double* bs, double* x, double* work,
                          LmState* st, int refine_iters, double tol, cudaStream_t s);
// Mixed-form reduced solve: preconditioned conjugate gradients on the FP64
// Schur operator of the FP32 Jacobian records (W.jac), applied matrix-free,
// preconditioned by X^T X. Writes b_s (W.bs), delta_p and the landmark
// back-substitution delta_l (W.delta); stops at ||b_s - S x|| <= tol ||b_s||
// or max_it iterations.
cudaError_t launch_pcg(const DevProblem& P, DevWork& W, LmState* st, int max_it, double tol, cudaStream_t s);
size_t pcg_doubles(const DevProblem& P);

// Per-pose sums of six values over each pose's observations, spread over the
// whole GPU (a CTA per pose leaves most SMs idle at a few hundred poses) in a
// fixed order: a warp per pose-major chunk (<= kOpChunk positions of one
// pose, P.opch_q; lane i takes positions i, i + 32, then a butterfly) into
// part[6 c + a], then a thread per (pose, value) adds its pose's chunks in
// chunk order and hands the total to out(P, k, a, total). term(P, q, s) adds
// position q's six values to s.
template <typename Term>
__global__ void __launch_bounds__(kThreads) k_chunk_sums6(DevProblem P, Term term, double* __restrict__ part) {
    const int lane = threadIdx.x & 31;
    const int64_t c = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    if (c >= P.nopch) return;
    double s[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    for (int q = P.opch_q[c] + lane; q < P.opch_q[c + 1]; q += 32) term(P, q, s);
#pragma unroll
    for (int a = 0; a < 6; ++a)
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) s[a] += __shfl_xor_sync(0xffffffffu, s[a], off);
    if (lane == 0)
#pragma unroll
        for (int a = 0; a < 6; ++a) part[6 * c + a] = s[a];
}

template <typename Out>
__global__ void __launch_bounds__(kThreads) k_chunk_finish6(DevProblem P, const double* __restrict__ part, Out out) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= 6LL * P.K) return;
    const int k = (int)(i / 6), a = (int)(i % 6);
    double v = 0.0;
    for (int c = P.pose_opch[k]; c < P.pose_opch[k + 1]; ++c) v += part[6LL * c + a];
    out(P, k, a, v);
}

// part: [6 P.nopch] scratch.
template <typename Term, typename Out>
void launch_pose_sums6(const DevProblem& P, double* part, Term term, Out out, cudaStream_t s) {
    if (P.K <= 0) return;
    if (P.nopch > 0) {
        k_chunk_sums6<<<grid_for(P.nopch * 32), kThreads, 0, s>>>(P, term, part);
        note_launch();
    }
    k_chunk_finish6<<<grid_for(6LL * P.K), kThreads, 0, s>>>(P, part, out);
    note_launch();
}

}  // namespace zs
