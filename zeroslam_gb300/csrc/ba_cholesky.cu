// Dense reduced-camera-system solve S x = b_s on the device (sm_103a).
//
// Blocked right-looking Cholesky S = L L^T on the row-major lower triangle:
// per 32-wide panel, one CTA factors the diagonal block (k_chol_diag), the
// panel below is solved against it (k_chol_trsm) and the trailing lower
// triangle is updated (k_chol_syrk). The pivot and solve tests are zeroslam's
// (source/matrix_decomposition_cholesky.hpp:40,53 and :74,80,89): a pivot
// must exceed 1e-14 * max|S_ii| and every |L_ii| must exceed
// 1e-7 * max|L_ii|. The triangular solves run block by block. The mixed form
// factors in FP32 and refines x in FP64 against S.
#include "ba_internal.h"

namespace zs {

constexpr int kNB = 32;

template <typename T>
__global__ void __launch_bounds__(kThreads) k_diag_max(int n, const T* __restrict__ A, LmState* st, double factor,
                                                       int which) {
    __shared__ double sh[kThreads];
    double m = 0.0;
    for (int i = threadIdx.x; i < n; i += kThreads) m = fmax(m, fabs((double)A[(int64_t)i * n + i]));
    sh[threadIdx.x] = m;
    __syncthreads();
    for (int s = kThreads / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) sh[threadIdx.x] = fmax(sh[threadIdx.x], sh[threadIdx.x + s]);
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        if (which == 0) {
            st->eps_factor = sh[0] * factor;
        } else {
            st->eps_solve = sh[0] * factor;
        }
    }
}

// Every |L_ii| must exceed eps_solve.
template <typename T>
__global__ void __launch_bounds__(kThreads) k_check_solve_eps(int n, const T* __restrict__ F, LmState* st) {
    __shared__ int bad;
    if (threadIdx.x == 0) bad = 0;
    __syncthreads();
    if (!st->solve_ok) return;
    const double eps = st->eps_solve;
    for (int i = threadIdx.x; i < n; i += kThreads)
        if (!(fabs((double)F[(int64_t)i * n + i]) > eps)) bad = 1;
    __syncthreads();
    if (threadIdx.x == 0 && bad) st->solve_ok = 0;
}

// Unblocked right-looking factor of the b x b diagonal block at j0.
template <typename T>
__global__ void __launch_bounds__(kThreads) k_chol_diag(int n, T* F, int j0, LmState* st) {
    __shared__ T a[kNB][kNB + 1];
    __shared__ int fail;
    if (!st->solve_ok) return;
    const int b = min(kNB, n - j0);
    const double eps = st->eps_factor;
    for (int e = threadIdx.x; e < b * b; e += blockDim.x) {
        const int i = e / b, m = e % b;
        a[i][m] = F[(int64_t)(j0 + i) * n + j0 + m];
    }
    if (threadIdx.x == 0) fail = 0;
    __syncthreads();
    for (int k = 0; k < b; ++k) {
        if (threadIdx.x == 0) {
            const T v = a[k][k];
            if (!((double)v > eps)) fail = 1;
            else a[k][k] = sqrt(v);
        }
        __syncthreads();
        if (fail) break;
        for (int i = k + 1 + threadIdx.x; i < b; i += blockDim.x) a[i][k] = a[i][k] / a[k][k];
        __syncthreads();
        const int rem = b - k - 1;
        for (int e = threadIdx.x; e < rem * rem; e += blockDim.x) {
            const int i = k + 1 + e / rem, m = k + 1 + e % rem;
            if (m <= i) a[i][m] = a[i][m] - a[i][k] * a[m][k];
        }
        __syncthreads();
    }
    if (fail) {
        if (threadIdx.x == 0) st->solve_ok = 0;
        return;
    }
    for (int e = threadIdx.x; e < b * b; e += blockDim.x) {
        const int i = e / b, m = e % b;
        F[(int64_t)(j0 + i) * n + j0 + m] = (m <= i) ? a[i][m] : T(0);
    }
}

// L21 = A21 L11^-T, one thread per row below the panel.
template <typename T>
__global__ void __launch_bounds__(64) k_chol_trsm(int n, T* F, int j0, const LmState* st) {
    __shared__ T l11[kNB][kNB + 1];
    if (!st->solve_ok) return;
    const int b = min(kNB, n - j0);
    for (int e = threadIdx.x; e < b * b; e += blockDim.x) l11[e / b][e % b] = F[(int64_t)(j0 + e / b) * n + j0 + e % b];
    __syncthreads();
    const int i = j0 + b + blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    T x[kNB];
    T* row = F + (int64_t)i * n + j0;
#pragma unroll
    for (int k = 0; k < kNB; ++k) {
        if (k < b) {
            T v = row[k];
            for (int m = 0; m < k; ++m) v -= x[m] * l11[k][m];
            x[k] = v / l11[k][k];
        }
    }
#pragma unroll
    for (int k = 0; k < kNB; ++k)
        if (k < b) row[k] = x[k];
}

// Trailing lower-triangle update A22 -= L21 L21^T over 32 x 32 tiles.
template <typename T>
__global__ void __launch_bounds__(kThreads) k_chol_syrk(int n, T* F, int j0, const LmState* st) {
    __shared__ T pa[32][kNB + 1];
    __shared__ T pm[32][kNB + 1];
    if (!st->solve_ok) return;
    const int b = min(kNB, n - j0);
    const int c0 = j0 + b;
    // blockIdx.x -> (ti, tm), tm <= ti
    const int t = blockIdx.x;
    int ti = (int)((sqrt(8.0 * t + 1.0) - 1.0) * 0.5);
    while ((ti + 1) * (ti + 2) / 2 <= t) ++ti;
    while (ti * (ti + 1) / 2 > t) --ti;
    const int tm = t - ti * (ti + 1) / 2;
    const int r0 = c0 + ti * 32, m0 = c0 + tm * 32;
    for (int e = threadIdx.x; e < 32 * kNB; e += blockDim.x) {
        const int r = e / kNB, k = e % kNB;
        const bool ok = k < b;
        pa[r][k] = (ok && r0 + r < n) ? F[(int64_t)(r0 + r) * n + j0 + k] : T(0);
        pm[r][k] = (ok && m0 + r < n) ? F[(int64_t)(m0 + r) * n + j0 + k] : T(0);
    }
    __syncthreads();
    for (int e = threadIdx.x; e < 32 * 32; e += blockDim.x) {
        const int r = e / 32, c = e % 32;
        const int row = r0 + r, col = m0 + c;
        if (row >= n || col >= n || col > row) continue;
        T acc = T(0);
#pragma unroll 8
        for (int k = 0; k < kNB; ++k) acc += pa[r][k] * pm[c][k];
        F[(int64_t)row * n + col] -= acc;
    }
}

__device__ inline double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Forward block step: solve L_JJ y_J = w_J (J = [j0, j0+b)), write y_J (block
// 0 only), and update w_i -= L_iJ y_J for the rows below, a warp per row.
template <typename T>
__global__ void __launch_bounds__(kThreads) k_trsv_fwd(int n, const T* __restrict__ F, int j0, double* w, double* y,
                                                       const LmState* st) {
    __shared__ double xs[kNB];
    if (!st->solve_ok) return;
    const int b = min(kNB, n - j0);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (warp == 0) {
        double xv = 0.0;
        for (int k = 0; k < b; ++k) {
            double part = (lane < k) ? (double)F[(int64_t)(j0 + k) * n + j0 + lane] * xv : 0.0;
            part = warp_sum(part);
            const double v = (w[j0 + k] - part) / (double)F[(int64_t)(j0 + k) * n + j0 + k];
            if (lane == k) xv = v;
        }
        if (lane < b) xs[lane] = xv;
    }
    __syncthreads();
    if (blockIdx.x == 0)
        for (int k = threadIdx.x; k < b; k += blockDim.x) y[j0 + k] = xs[k];
    const int i = j0 + b + blockIdx.x * (kThreads / 32) + warp;
    if (i >= n) return;
    double part = (lane < b) ? (double)F[(int64_t)i * n + j0 + lane] * xs[lane] : 0.0;
    part = warp_sum(part);
    if (lane == 0) w[i] -= part;
}

// Backward block step: solve L_JJ^T x_J = z_J, write x_J (block 0 only), and
// update z_i -= sum_m L_{j0+m, i} x_m for i < j0, a thread per i.
template <typename T>
__global__ void __launch_bounds__(kThreads) k_trsv_bwd(int n, const T* __restrict__ F, int j0, double* z, double* x,
                                                       const LmState* st) {
    __shared__ double xs[kNB];
    if (!st->solve_ok) return;
    const int b = min(kNB, n - j0);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (warp == 0) {
        double xv = 0.0;
        for (int k = b - 1; k >= 0; --k) {
            double part = (lane > k && lane < b) ? (double)F[(int64_t)(j0 + lane) * n + j0 + k] * xv : 0.0;
            part = warp_sum(part);
            const double v = (z[j0 + k] - part) / (double)F[(int64_t)(j0 + k) * n + j0 + k];
            if (lane == k) xv = v;
        }
        if (lane < b) xs[lane] = xv;
    }
    __syncthreads();
    if (blockIdx.x == 0)
        for (int k = threadIdx.x; k < b; k += blockDim.x) x[j0 + k] = xs[k];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= j0) return;
    double acc = 0.0;
    for (int m = 0; m < b; ++m) acc += (double)F[(int64_t)(j0 + m) * n + i] * xs[m];
    z[i] -= acc;
}

// r = bs - S x (FP64 accumulation), a warp per row; also |r|^2 and |bs|^2
// partial sums per block for the report.
template <typename T>
__global__ void __launch_bounds__(kThreads) k_residual(int n, const T* __restrict__ S, const double* __restrict__ x,
                                                       const double* __restrict__ bs, double* r, const LmState* st) {
    if (!st->solve_ok) return;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int i = blockIdx.x * (kThreads / 32) + warp;
    if (i >= n) return;
    double acc = 0.0;
    for (int c = lane; c < n; c += 32) acc += (double)S[(int64_t)i * n + c] * x[c];
    acc = warp_sum(acc);
    if (lane == 0) r[i] = bs[i] - acc;
}

__global__ void __launch_bounds__(kThreads) k_axpy_copy(int n, const double* __restrict__ a, double* __restrict__ x,
                                                        int accumulate, const LmState* st) {
    if (!st->solve_ok) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    x[i] = accumulate ? x[i] + a[i] : a[i];
}

__global__ void __launch_bounds__(kThreads) k_norms(int n, const double* __restrict__ r, const double* __restrict__ b,
                                                    LmState* st) {
    __shared__ double sh[kThreads];
    double a = 0.0, c = 0.0;
    for (int i = threadIdx.x; i < n; i += kThreads) {
        a += r[i] * r[i];
        c += b[i] * b[i];
    }
    a = block_sum(a, sh);
    c = block_sum(c, sh);
    if (threadIdx.x == 0) {
        st->resid_norm = sqrt(a);
        st->rhs_norm = sqrt(c);
    }
}

// x = L^-T L^-1 rhs using scratch w (forward work), y (forward result).
template <typename T>
static void tri_solve(int n, const T* F, const double* rhs, double* w, double* y, double* x, const LmState* st,
                      cudaStream_t s) {
    k_axpy_copy<<<grid_for(n), kThreads, 0, s>>>(n, rhs, w, 0, st); note_launch();
    for (int j0 = 0; j0 < n; j0 += kNB) {
        const int rows = n - j0 - min(kNB, n - j0);
        const int g = rows > 0 ? (rows + kThreads / 32 - 1) / (kThreads / 32) : 1;
        k_trsv_fwd<T><<<g, kThreads, 0, s>>>(n, F, j0, w, y, st); note_launch();
    }
    // backward: z starts as y (reuse w as z)
    k_axpy_copy<<<grid_for(n), kThreads, 0, s>>>(n, y, w, 0, st); note_launch();
    const int last = ((n - 1) / kNB) * kNB;
    for (int j0 = last; j0 >= 0; j0 -= kNB) {
        const int g = j0 > 0 ? grid_for(j0) : 1;
        k_trsv_bwd<T><<<g, kThreads, 0, s>>>(n, F, j0, w, x, st); note_launch();
    }
}

template <typename TS, typename TF>
__global__ void __launch_bounds__(kThreads) k_convert(int64_t N, const TS* __restrict__ src, TF* __restrict__ dst) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < N) dst[i] = (TF)src[i];
}

template <typename TS, typename TF>
void launch_factor(int n, const TS* S, TF* F, LmState* st, cudaStream_t s) {
    if (n <= 0) return;
    const int64_t nn = (int64_t)n * n;
    k_diag_max<TS><<<1, kThreads, 0, s>>>(n, S, st, 1e-14, 0); note_launch();
    k_convert<TS, TF><<<grid_for(nn), kThreads, 0, s>>>(nn, S, F); note_launch();
    for (int j0 = 0; j0 < n; j0 += kNB) {
        const int b = min(kNB, n - j0);
        k_chol_diag<TF><<<1, kThreads, 0, s>>>(n, F, j0, st); note_launch();
        const int rows = n - j0 - b;
        if (rows > 0) {
            k_chol_trsm<TF><<<(rows + 63) / 64, 64, 0, s>>>(n, F, j0, st); note_launch();
            const int nt = (rows + 31) / 32;
            k_chol_syrk<TF><<<nt * (nt + 1) / 2, kThreads, 0, s>>>(n, F, j0, st); note_launch();
        }
    }
    k_diag_max<TF><<<1, kThreads, 0, s>>>(n, F, st, 1e-7, 1); note_launch();
    k_check_solve_eps<TF><<<1, kThreads, 0, s>>>(n, F, st); note_launch();
}

template <typename TS, typename TF>
void launch_solve_refine(int n, const TS* S, const TF* F, const double* bs, double* x, double* y, double* r,
                         LmState* st, int refine_iters, cudaStream_t s) {
    if (n <= 0) return;
    // r[0..n) is the forward work vector, y[0..n) the forward result.
    tri_solve<TF>(n, F, bs, r, y, x, st, s);
    if (refine_iters <= 0) return;
    // Refinement: x += solve(bs - S x), residual in FP64 against S.
    double* d = y + n;   // y holds 2n
    double* res = r + n; // r holds 2n
    const int rg = (n + kThreads / 32 - 1) / (kThreads / 32);
    for (int it = 0; it < refine_iters; ++it) {
        k_residual<TS><<<rg, kThreads, 0, s>>>(n, S, x, bs, res, st); note_launch();
        tri_solve<TF>(n, F, res, r, y, d, st, s);
        k_axpy_copy<<<grid_for(n), kThreads, 0, s>>>(n, d, x, 1, st); note_launch();
    }
    k_residual<TS><<<rg, kThreads, 0, s>>>(n, S, x, bs, res, st); note_launch();
    k_norms<<<1, kThreads, 0, s>>>(n, res, bs, st); note_launch();
}

template <typename TS, typename TF>
void launch_reduced_solve(int n, const TS* S, TF* F, const double* bs, double* x, double* y, double* r, LmState* st,
                          int refine_iters, cudaStream_t s) {
    launch_factor<TS, TF>(n, S, F, st, s);
    launch_solve_refine<TS, TF>(n, S, F, bs, x, y, r, st, refine_iters, s);
}

#define ZS_INST(TS, TF)                                                                                          \
    template void launch_factor<TS, TF>(int, const TS*, TF*, LmState*, cudaStream_t);                             \
    template void launch_solve_refine<TS, TF>(int, const TS*, const TF*, const double*, double*, double*, double*, \
                                              LmState*, int, cudaStream_t);
ZS_INST(double, double)
ZS_INST(float, float)
ZS_INST(double, float)
#undef ZS_INST

template void launch_reduced_solve<double, double>(int, const double*, double*, const double*, double*, double*,
                                                   double*, LmState*, int, cudaStream_t);
template void launch_reduced_solve<float, float>(int, const float*, float*, const double*, double*, double*, double*,
                                                 LmState*, int, cudaStream_t);
template void launch_reduced_solve<double, float>(int, const double*, float*, const double*, double*, double*,
                                                  double*, LmState*, int, cudaStream_t);

}  // namespace zs
