// Adjoint of the converged bundle adjustment (FP64): gradients of a scalar
// loss L(x*) of the solution x* with respect to the observed pixels and the
// pinhole intrinsics (fx, fy, cx, cy), by the implicit-function theorem.
//
// At a stationary point F(x*, theta) = sum_o J_o^T Omega_o r_o = 0, where x is
// perturbed in the solver's own local coordinates (poses T <- exp(d) T,
// landmarks X <- X + d; source/factor_graph.hpp:947-960, 141-145). Then
//     dL/dtheta = -v^T dF/dtheta,   H v = a = dL/dx,
// with H the exact Hessian of E = sum r^T Omega r in those coordinates:
//     H_o = J^T Omega J + sum_k (Omega r)_k d2 r_k,
//     d2 r_k = -(A^T Pi_k A + sum_i dpi_k/dP_i d2 P_i),
// P the camera-frame point, A = dP/dx = [-[P]x | I | R], Pi_k the Hessian of
// the projection (source/camera.hpp:91-142) and d2 P the second-order terms of
// exp(d) (P + R dl): 1/2 w x (w x P) + 1/2 w x u + w x (R dl).
// H v = a is solved by conjugate gradients preconditioned with the solver's
// lightly damped Gauss-Newton factorisation (Schur complement + reduced
// Cholesky): the factor is reused, only exact-Hessian products are new. H is
// symmetric positive definite at an isolated minimum; CG also converges where
// the curvature term is not small against the Gauss-Newton block (landmarks
// seen with little parallax), where a plain preconditioned iteration stalls.
// There is no counterpart in the reference; the gradient is checked against
// central finite differences of whole solves.
#include "ba_internal.h"

namespace zs {

constexpr int kAdjRec = kAdjRecord;  // per observation: J (18), Q (45 = 9x9 upper), pad

// Per observation at the current state: J = dr/dx (2 x 9, pose then landmark)
// and Q = sum_k (Omega r)_k d2 r_k (9 x 9, upper triangle row by row).
__global__ void __launch_bounds__(kThreads) k_adj_prep(DevProblem P, double* __restrict__ rec) {
    const int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (o >= P.M) return;
    const int pi = P.obs_pose[o], li = P.obs_lm[o];
    const double* pp = P.pose + (int64_t)pi * kPoseStride;
    const double* xp = P.lm + (int64_t)li * kLmStride;
    double p[7], X[3], Pc[3], r[2];
#pragma unroll
    for (int i = 0; i < 7; ++i) p[i] = pp[i];
#pragma unroll
    for (int i = 0; i < 3; ++i) X[i] = xp[i];
    const double2 uv = P.obs_uv[o];
    const int front = residual(p, X, uv.x, uv.y, P.intr, Pc, r);
    const double* om = P.obs_info ? P.obs_info + 4 * o : nullptr;
    const double w0 = om ? om[0] * r[0] + om[1] * r[1] : r[0];
    const double w1 = om ? om[2] * r[0] + om[3] * r[1] : r[1];
    // dpi/dP (2 x 3) and sum_k w_k Pi_k (3 x 3); behind the camera the
    // residual is -0.3 Z: dpi/dP = (0, 0, 0.3) for both rows, no curvature.
    double D[6], C[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    if (front) {
        const double iz = 1.0 / Pc[2], iz2 = iz * iz, iz3 = iz2 * iz;
        const double fx = P.intr.fx, fy = P.intr.fy;
        D[0] = fx * iz; D[1] = 0.0; D[2] = -fx * Pc[0] * iz2;
        D[3] = 0.0; D[4] = fy * iz; D[5] = -fy * Pc[1] * iz2;
        C[2] = C[6] = -w0 * fx * iz2;
        C[5] = C[7] = -w1 * fy * iz2;
        C[8] = 2.0 * (w0 * fx * Pc[0] + w1 * fy * Pc[1]) * iz3;
    } else {
        D[0] = D[1] = D[3] = D[4] = 0.0;
        D[2] = D[5] = kBehindPenalty;
    }
    const double c[3] = {w0 * D[0] + w1 * D[3], w0 * D[1] + w1 * D[4], w0 * D[2] + w1 * D[5]};
    double R[9];
    {
        const double q[4] = {p[6], p[3], p[4], p[5]};
        quat_matrix(q, R);
    }
    // A = [-[P]x | I | R]
    double A[27];
    A[0] = 0.0;    A[1] = Pc[2];  A[2] = -Pc[1]; A[3] = 1; A[4] = 0; A[5] = 0; A[6] = R[0]; A[7] = R[1]; A[8] = R[2];
    A[9] = -Pc[2]; A[10] = 0.0;   A[11] = Pc[0]; A[12] = 0; A[13] = 1; A[14] = 0; A[15] = R[3]; A[16] = R[4]; A[17] = R[5];
    A[18] = Pc[1]; A[19] = -Pc[0]; A[20] = 0.0;  A[21] = 0; A[22] = 0; A[23] = 1; A[24] = R[6]; A[25] = R[7]; A[26] = R[8];
    double* out = rec + o * kAdjRec;
    // J = -D A
#pragma unroll
    for (int k = 0; k < 2; ++k)
#pragma unroll
        for (int j = 0; j < 9; ++j) out[k * 9 + j] = -(D[k * 3] * A[j] + D[k * 3 + 1] * A[9 + j] + D[k * 3 + 2] * A[18 + j]);
    // CA = C A (3 x 9)
    double CA[27];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 9; ++j) CA[i * 9 + j] = C[i * 3] * A[j] + C[i * 3 + 1] * A[9 + j] + C[i * 3 + 2] * A[18 + j];
    const double cP = c[0] * Pc[0] + c[1] * Pc[1] + c[2] * Pc[2];
    // c x e_a for a = 0, 1, 2
    const double cxe[9] = {0.0, c[2], -c[1], -c[2], 0.0, c[0], c[1], -c[0], 0.0};
    int idx = 18;
#pragma unroll
    for (int a = 0; a < 9; ++a) {
#pragma unroll
        for (int b = a; b < 9; ++b) {
            double g = 0.0;  // sum_i c_i d2 P_i / dx_a dx_b
            if (a < 3 && b < 3) {
                g = 0.5 * (c[b] * Pc[a] + c[a] * Pc[b]) - (a == b ? cP : 0.0);
            } else if (a < 3 && b < 6) {
                const int bb = b - 3;  // 1/2 c . (e_a x e_b)
                g = (a == bb) ? 0.0 : 0.5 * ((((bb - a + 3) % 3) == 1) ? c[3 - a - bb] : -c[3 - a - bb]);
            } else if (a < 3) {
                const int bb = b - 6;  // c . (e_a x R e_bb) = R e_bb . (c x e_a)
                g = R[bb] * cxe[a * 3] + R[3 + bb] * cxe[a * 3 + 1] + R[6 + bb] * cxe[a * 3 + 2];
            }
            const double aca = A[a] * CA[b] + A[9 + a] * CA[9 + b] + A[18 + a] * CA[18 + b];
            out[idx++] = -(aca + g);
        }
    }
}

// y_o = (J^T Omega J + Q) v_o for v = (v_pose, v_landmark); the 9 values go
// component-major into part ([9][M]); fixed vertices contribute and receive 0.
__global__ void __launch_bounds__(kThreads) k_adj_matvec(DevProblem P, const double* __restrict__ rec,
                                                         const double* __restrict__ v, double* __restrict__ part) {
    const int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (o >= P.M) return;
    const int pi = P.obs_pose[o], li = P.obs_lm[o];
    const bool pf = P.pose_fixed[pi] != 0, lf = P.lm_fixed[li] != 0;
    double x[9];
#pragma unroll
    for (int i = 0; i < 6; ++i) x[i] = pf ? 0.0 : v[6LL * pi + i];
#pragma unroll
    for (int i = 0; i < 3; ++i) x[6 + i] = lf ? 0.0 : v[P.n + 3LL * li + i];
    const double* J = rec + o * kAdjRec;
    const double* Q = J + 18;
    double jv0 = 0.0, jv1 = 0.0;
#pragma unroll
    for (int j = 0; j < 9; ++j) {
        jv0 += J[j] * x[j];
        jv1 += J[9 + j] * x[j];
    }
    const double* om = P.obs_info ? P.obs_info + 4 * o : nullptr;
    const double u0 = om ? om[0] * jv0 + om[1] * jv1 : jv0;
    const double u1 = om ? om[2] * jv0 + om[3] * jv1 : jv1;
    double y[9];
#pragma unroll
    for (int a = 0; a < 9; ++a) y[a] = J[a] * u0 + J[9 + a] * u1;
    int idx = 0;
#pragma unroll
    for (int a = 0; a < 9; ++a) {
#pragma unroll
        for (int b = a; b < 9; ++b) {
            const double q = Q[idx++];
            y[a] += q * x[b];
            if (b != a) y[b] += q * x[a];
        }
    }
#pragma unroll
    for (int i = 0; i < 6; ++i) part[(int64_t)i * P.M + o] = pf ? 0.0 : y[i];
#pragma unroll
    for (int i = 0; i < 3; ++i) part[(int64_t)(6 + i) * P.M + o] = lf ? 0.0 : y[6 + i];
}

// out = a - (sum of parts) per vertex, zero on fixed vertices; landmarks by
// segment (a thread per landmark), poses by a fixed tree (a CTA per pose).
__global__ void __launch_bounds__(kThreads) k_adj_reduce_lm(DevProblem P, const double* __restrict__ part,
                                                            const double* __restrict__ a, double* out) {
    const int l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l >= P.L) return;
    double s[3] = {0.0, 0.0, 0.0};
    for (int o = P.lm_ptr[l]; o < P.lm_ptr[l + 1]; ++o)
#pragma unroll
        for (int i = 0; i < 3; ++i) s[i] += part[(int64_t)(6 + i) * P.M + o];
#pragma unroll
    for (int i = 0; i < 3; ++i) out[P.n + 3LL * l + i] = P.lm_fixed[l] ? 0.0 : a[P.n + 3LL * l + i] - s[i];
}

// The pose rows of a - H v (launch_pose_sums6): position q's six pose terms
// of H v, and the pose's output (zero for a fixed pose).
struct AdjPoseTerm {
    const double* part;
    __device__ void operator()(const DevProblem& P, int q, double s[6]) const {
        const int64_t o = P.pose_obs[q];
#pragma unroll
        for (int c = 0; c < 6; ++c) s[c] += part[(int64_t)c * P.M + o];
    }
};
struct AdjPoseOut {
    const double* a;
    double* out;
    __device__ void operator()(const DevProblem& P, int k, int c, double v) const {
        out[6LL * k + c] = P.pose_fixed[k] ? 0.0 : a[6LL * k + c] - v;
    }
};

// y = alpha x + beta y
__global__ void __launch_bounds__(kThreads) k_adj_axpby(int64_t N, double alpha, const double* __restrict__ x,
                                                        double beta, double* y) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < N) y[i] = alpha * x[i] + beta * y[i];
}

// ---- the conjugate-gradient loop's scalars on the device ----
// The host enqueues iterations in batches and reads c->done once per batch;
// every update below is skipped once done is set, so iterations enqueued past
// the stop change nothing.

// The kReduceBlocks partials of a dot product, added by one warp (lane l
// takes partials l, l + 32, ..., then a butterfly): a fixed order, every lane
// gets the sum. (One thread adding them in turn waited on 304 dependent FP64
// additions, three times per iteration.)
__device__ __forceinline__ double cg_sum(const double* red) {
    const int lane = threadIdx.x & 31;
    double t = 0.0;
    for (int i = lane; i < kReduceBlocks; i += 32) t += red[i];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) t += __shfl_xor_sync(0xffffffffu, t, off);
    return t;
}

// pAp = -(p . q) with q = -H p; stop (done = 2) unless pAp > 0, else alpha.
// (One warp: the sum is the warp's, lane 0 writes.)
__global__ void k_adj_cg_pap(const double* __restrict__ red, AdjCg* c) {
    if (c->done) return;  // (uniform)
    const double pAp = -cg_sum(red);
    if (threadIdx.x) return;
    if (!(pAp > 0.0)) {
        c->done = 2;
        return;
    }
    c->alpha = c->rz / pAp;
}

// |r| after the update: one more iteration done; stop at the tolerance
// (done = 1) or at the iteration limit (done = 3).
__global__ void k_adj_cg_rn(const double* __restrict__ red, AdjCg* c) {
    if (c->done) return;
    const double rn = sqrt(cg_sum(red));
    if (threadIdx.x) return;
    c->rn = rn;
    c->it += 1;
    if (c->rn <= c->tol * c->anorm) c->done = 1;
    else if (c->it >= c->max_it) c->done = 3;
}

// r . z of the new preconditioned residual: beta and the new rz.
__global__ void k_adj_cg_rz(const double* __restrict__ red, AdjCg* c) {
    if (c->done) return;
    const double rz_new = cg_sum(red);
    if (threadIdx.x) return;
    c->beta = rz_new / c->rz;
    c->rz = rz_new;
}

// y = alpha x + 1 y (which = 0) or y = 1 x + beta y (which = 1), with the
// coefficient from c; nothing once c->done.
__global__ void __launch_bounds__(kThreads) k_adj_cg_axpby(int64_t N, const AdjCg* __restrict__ c, int which,
                                                           const double* __restrict__ x, double* y) {
    if (c->done) return;
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= N) return;
    const double alpha = which == 0 ? c->alpha : 1.0, beta = which == 0 ? 1.0 : c->beta;
    y[i] = alpha * x[i] + beta * y[i];
}

// Fixed-shape partial dot products x . y into red[blockIdx.x].
__global__ void __launch_bounds__(kThreads) k_adj_dot(int64_t N, const double* __restrict__ x,
                                                      const double* __restrict__ y, double* red) {
    __shared__ double sh[kThreads];
    double v = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x)
        v += x[i] * y[i];
    v = block_sum(v, sh);
    if (threadIdx.x == 0) red[blockIdx.x] = v;
}

__global__ void __launch_bounds__(kThreads) k_adj_copy(int64_t N, const double* __restrict__ src, double* dst) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < N) dst[i] = src[i];
}

// Outputs from the converged adjoint vector v:
//   dL/duv_o = -Omega J_o v_o (uv[2M], landmark-major order), and per-block
//   partial sums of dL/dtheta_c = -sum_o [(Omega r)^T dJ/dtheta_c v_o
//                                        + (J v_o)^T Omega dr/dtheta_c]
//   for theta = (fx, fy, cx, cy) into red[4 * blockIdx.x + c].
__global__ void __launch_bounds__(kThreads) k_adj_out(DevProblem P, const double* __restrict__ rec,
                                                      const double* __restrict__ v, double* duv, double* red) {
    __shared__ double sh[kThreads];
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    for (int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o < P.M; o += (int64_t)gridDim.x * blockDim.x) {
        const int pi = P.obs_pose[o], li = P.obs_lm[o];
        const bool pf = P.pose_fixed[pi] != 0, lf = P.lm_fixed[li] != 0;
        double x[9];
#pragma unroll
        for (int i = 0; i < 6; ++i) x[i] = pf ? 0.0 : v[6LL * pi + i];
#pragma unroll
        for (int i = 0; i < 3; ++i) x[6 + i] = lf ? 0.0 : v[P.n + 3LL * li + i];
        const double* J = rec + o * kAdjRec;
        double jv0 = 0.0, jv1 = 0.0;
#pragma unroll
        for (int j = 0; j < 9; ++j) {
            jv0 += J[j] * x[j];
            jv1 += J[9 + j] * x[j];
        }
        const double* om = P.obs_info ? P.obs_info + 4 * o : nullptr;
        const double oj0 = om ? om[0] * jv0 + om[1] * jv1 : jv0;
        const double oj1 = om ? om[2] * jv0 + om[3] * jv1 : jv1;
        // recompute the camera point for the intrinsics terms
        const double* pp = P.pose + (int64_t)pi * kPoseStride;
        const double* xp = P.lm + (int64_t)li * kLmStride;
        double p[7], X[3], Pc[3], r[2];
#pragma unroll
        for (int i = 0; i < 7; ++i) p[i] = pp[i];
#pragma unroll
        for (int i = 0; i < 3; ++i) X[i] = xp[i];
        const double2 uvo = P.obs_uv[o];
        const int front = residual(p, X, uvo.x, uvo.y, P.intr, Pc, r);
        if (!front) {  // the penalty residual depends on neither the pixel nor the intrinsics
            duv[2 * o] = 0.0;
            duv[2 * o + 1] = 0.0;
            continue;
        }
        duv[2 * o] = -oj0;
        duv[2 * o + 1] = -oj1;
        const double w0 = om ? om[0] * r[0] + om[1] * r[1] : r[0];
        const double w1 = om ? om[2] * r[0] + om[3] * r[1] : r[1];
        const double iz = 1.0 / Pc[2], iz2 = iz * iz;
        // A x (3): dP for this v_o
        double q[4] = {p[6], p[3], p[4], p[5]};
        double R[9];
        quat_matrix(q, R);
        const double ax = Pc[2] * x[1] - Pc[1] * x[2] + x[3] + R[0] * x[6] + R[1] * x[7] + R[2] * x[8];
        const double ay = -Pc[2] * x[0] + Pc[0] * x[2] + x[4] + R[3] * x[6] + R[4] * x[7] + R[5] * x[8];
        const double az = Pc[1] * x[0] - Pc[0] * x[1] + x[5] + R[6] * x[6] + R[7] * x[7] + R[8] * x[8];
        // dJ/dfx v = -(1/z, 0, -x/z^2) (A v) in row 0; dJ/dfy v = -(0, 1/z, -y/z^2) (A v) in row 1
        const double dfx = -(ax * iz - Pc[0] * iz2 * az);
        const double dfy = -(ay * iz - Pc[1] * iz2 * az);
        // dr/dtheta = -[[x/z, 0, 1, 0], [0, y/z, 0, 1]]
        acc[0] -= w0 * dfx + oj0 * (-Pc[0] * iz);
        acc[1] -= w1 * dfy + oj1 * (-Pc[1] * iz);
        acc[2] -= oj0 * (-1.0);
        acc[3] -= oj1 * (-1.0);
    }
#pragma unroll 1
    for (int c = 0; c < 4; ++c) {
        const double s = block_sum(acc[c], sh);
        if (threadIdx.x == 0) red[4 * blockIdx.x + c] = s;
    }
}

// Xi = L^-1 of the reduced system's FP64 factor (row-major lower L, n x n)
// and XiT = its transpose, for the preconditioner of the adjoint's conjugate
// gradients, whose factor stays fixed for all its iterations: a warp per
// column j, forward substitution x_i = (delta_ij - sum_{j<=k<i} L_ik x_k) /
// L_ii with lanes over k and a butterfly (a fixed order), x in shared memory.
__global__ void __launch_bounds__(kAdjInvWarps * 32) k_adj_tri_inverse(int n, const double* __restrict__ L,
                                                                     double* __restrict__ Xi, double* __restrict__ XiT) {
    extern __shared__ double xs[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int j = blockIdx.x * kAdjInvWarps + warp;
    if (j >= n) return;  // (whole warps)
    double* x = xs + (size_t)warp * n;
    for (int i = j; i < n; ++i) {
        double t = 0.0;
        for (int k = j + lane; k < i; k += 32) t += L[(int64_t)i * n + k] * x[k];
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) t += __shfl_xor_sync(0xffffffffu, t, off);
        const double xi = ((i == j ? 1.0 : 0.0) - t) / L[(int64_t)i * n + i];
        if (lane == 0) x[i] = xi;
        __syncwarp();
    }
    for (int i = lane; i < n; i += 32) {
        const double v = i >= j ? x[i] : 0.0;
        Xi[(int64_t)i * n + j] = v;
        XiT[(int64_t)j * n + i] = v;
    }
}

// y = M x for a triangular M (upper = 0: columns <= row; 1: columns >= row),
// a warp per row, lanes over the row, a butterfly.
__global__ void __launch_bounds__(kThreads) k_adj_gemv_tri(int n, const double* __restrict__ M,
                                                           const double* __restrict__ x, double* __restrict__ y,
                                                           int upper) {
    const int lane = threadIdx.x & 31;
    const int64_t i = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    if (i >= n) return;
    const int lo = upper ? (int)i : 0, hi = upper ? n : (int)i + 1;
    double t = 0.0;
    for (int k = lo + lane; k < hi; k += 32) t += M[i * n + k] * x[k];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) t += __shfl_xor_sync(0xffffffffu, t, off);
    if (lane == 0) y[i] = t;
}

void launch_adj_tri_inverse(int n, const double* L, double* Xi, double* XiT, cudaStream_t s) {
    if (n <= 0) return;
    const size_t smem = sizeof(double) * (size_t)kAdjInvWarps * n;
    k_adj_tri_inverse<<<(n + kAdjInvWarps - 1) / kAdjInvWarps, kAdjInvWarps * 32, smem, s>>>(n, L, Xi, XiT);
    note_launch();
}

// y = XiT (Xi b): the reduced solve L L^T y = b with the explicit inverse.
void launch_adj_apply_inverse(int n, const double* Xi, const double* XiT, const double* b, double* tmp, double* y,
                              cudaStream_t s) {
    if (n <= 0) return;
    k_adj_gemv_tri<<<grid_for(32LL * n), kThreads, 0, s>>>(n, Xi, b, tmp, 0);
    k_adj_gemv_tri<<<grid_for(32LL * n), kThreads, 0, s>>>(n, XiT, tmp, y, 1);
    note_launch(2);
}

void launch_adj_prep(const DevProblem& P, double* rec, cudaStream_t s) {
    if (P.M > 0) {
        k_adj_prep<<<grid_for(P.M), kThreads, 0, s>>>(P, rec);
        note_launch();
    }
}

// out = a - H v (fixed vertices zero) using part [9*M] and csum [6 nopch] scratch.
void launch_adj_residual(const DevProblem& P, const double* rec, const double* v, const double* a, double* part,
                         double* csum, double* out, cudaStream_t s) {
    if (P.M > 0) {
        k_adj_matvec<<<grid_for(P.M), kThreads, 0, s>>>(P, rec, v, part);
        note_launch();
    }
    if (P.L > 0) {
        k_adj_reduce_lm<<<grid_for(P.L), kThreads, 0, s>>>(P, part, a, out);
        note_launch();
    }
    launch_pose_sums6(P, csum, AdjPoseTerm{part}, AdjPoseOut{a, out}, s);
}

void launch_adj_axpby(int64_t N, double alpha, const double* x, double beta, double* y, cudaStream_t s) {
    if (N > 0) {
        k_adj_axpby<<<grid_for(N), kThreads, 0, s>>>(N, alpha, x, beta, y);
        note_launch();
    }
}

void launch_adj_dot(int64_t N, const double* x, const double* y, double* red, cudaStream_t s) {
    k_adj_dot<<<kReduceBlocks, kThreads, 0, s>>>(N, x, y, red);
    note_launch();
}

void launch_adj_copy(int64_t N, const double* src, double* dst, cudaStream_t s) {
    if (N > 0) {
        k_adj_copy<<<grid_for(N), kThreads, 0, s>>>(N, src, dst);
        note_launch();
    }
}

void launch_adj_cg_pap(const double* red, AdjCg* c, cudaStream_t s) {
    k_adj_cg_pap<<<1, 32, 0, s>>>(red, c);
    note_launch();
}
void launch_adj_cg_rn(const double* red, AdjCg* c, cudaStream_t s) {
    k_adj_cg_rn<<<1, 32, 0, s>>>(red, c);
    note_launch();
}
void launch_adj_cg_rz(const double* red, AdjCg* c, cudaStream_t s) {
    k_adj_cg_rz<<<1, 32, 0, s>>>(red, c);
    note_launch();
}
void launch_adj_cg_axpby(int64_t N, const AdjCg* c, int which, const double* x, double* y, cudaStream_t s) {
    if (N > 0) {
        k_adj_cg_axpby<<<grid_for(N), kThreads, 0, s>>>(N, c, which, x, y);
        note_launch();
    }
}

void launch_adj_out(const DevProblem& P, const double* rec, const double* v, double* duv, double* red, cudaStream_t s) {
    k_adj_out<<<kReduceBlocks, kThreads, 0, s>>>(P, rec, v, duv, red);
    note_launch();
}

}  // namespace zs
