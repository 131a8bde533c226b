// Internal interfaces between the C ABI layer (ba_api.cu) and the kernels
// (ba_kernels.cu, ba_cholesky.cu). Device pointers only; no torch types.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "ba_common.cuh"

namespace zs {

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
    // (block of pose i, block of pose j) grouped by pair, split into chunks.
    int npairs = 0;
    int64_t ntriples = 0;
    int64_t nchunks = 0;
    int32_t* pair_i = nullptr;         // [npairs]
    int32_t* pair_j = nullptr;         // [npairs]
    int64_t* pair_chunk_ptr = nullptr; // [npairs+1]
    int64_t* chunk_ptr = nullptr;      // [nchunks+1] ranges into triples
    int2* triples = nullptr;           // [ntriples] (obs of pose i, obs of pose j)
    Intrinsics intr{};
    LossParams loss{};
};

// Working arrays of one precision (T = double for the plain form, float for
// the mixed form).
struct DevWork {
    void* hpl = nullptr;       // [M*18] T
    void* W = nullptr;         // [M*18] T
    void* lm_part = nullptr;   // [9*M] T, component-major
    void* pose_part = nullptr; // [27*M] T, component-major
    double* hpp = nullptr;     // [K*36]
    double* hll = nullptr;     // [L*9]
    double* hll_inv = nullptr; // [L*9]
    double* b = nullptr;       // [n + 3L] gradient vector (poses then landmarks)
    void* partial = nullptr;   // [nchunks*36] T
    void* S = nullptr;         // [n*n] T
    void* F = nullptr;         // [n*n] T, Cholesky factor (lower)
    double* bs = nullptr;      // [n]
    double* y = nullptr;       // [2n] scratch for triangular solves
    double* r = nullptr;       // [2n] scratch: forward work vector, refinement residual
    double* delta = nullptr;   // [n + 3L]
    double* red = nullptr;     // [kReduceBlocks * 4] reduction partials
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
    int32_t pad;
};

// ---- kernels (ba_kernels.cu) ----
template <typename T>
void launch_linearize(const DevProblem& P, DevWork& W, cudaStream_t s);
template <typename T>
void launch_invert_w(const DevProblem& P, DevWork& W, const LmState* st, cudaStream_t s);
template <typename T>
void launch_schur(const DevProblem& P, DevWork& W, const LmState* st, cudaStream_t s);
template <typename T>
void launch_backsub(const DevProblem& P, DevWork& W, const LmState* st, cudaStream_t s);
void launch_update(const DevProblem& P, DevWork& W, const LmState* st, cudaStream_t s);
void launch_rollback(const DevProblem& P, const LmState* st, cudaStream_t s);
void launch_scale(const DevProblem& P, DevWork& W, LmState* st, cudaStream_t s);
// cost of the current state into st->chi2_new (when only_if_ok, skipped if !st->solve_ok)
void launch_cost(const DevProblem& P, DevWork& W, LmState* st, bool only_if_ok, cudaStream_t s);
void launch_init_lambda(const DevProblem& P, DevWork& W, LmState* st, double tau, double clamp, cudaStream_t s);
void launch_decide(LmState* st, cudaStream_t s);
void launch_set_solve_ok(LmState* st, int v, cudaStream_t s);

// ---- dense reduced system (ba_cholesky.cu) ----
// Factor S (n x n row-major, type TS) in type TF into F and solve for x
// given bs; sets st->solve_ok. With refine_iters > 0, that many FP64
// refinement sweeps x += F^-1 (bs - S x). y and r need 2n doubles.
template <typename TS, typename TF>
void launch_reduced_solve(int n, const TS* S, TF* F, const double* bs, double* x, double* y, double* r, LmState* st,
                          int refine_iters, cudaStream_t s);
// The two halves of launch_reduced_solve.
template <typename TS, typename TF>
void launch_factor(int n, const TS* S, TF* F, LmState* st, cudaStream_t s);
template <typename TS, typename TF>
void launch_solve_refine(int n, const TS* S, const TF* F, const double* bs, double* x, double* y, double* r,
                         LmState* st, int refine_iters, cudaStream_t s);

}  // namespace zs
