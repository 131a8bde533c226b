// Mixed-precision reduced solve after the FP32 factorisation S ~ L L^T:
//
// 1. k_tri_inverse: X = L^-1 by recursive 2 x 2 block inversion,
//        inv([A 0; B C]) = [A^-1 0; -C^-1 (B A^-1)  C^-1],
//    from the 32 x 32 diagonal-block inverses D_k up, doubling the block
//    size each level (log2(n/32) levels, two grid barriers per level). Every
//    level is a set of independent 32 x 32 output tiles of GEMM work spread
//    over all SMs. X^T is stored beside X so that both products below are
//    row-wise; the lower triangle of X^T doubles as the scratch for B A^-1.
// 2. k_refine: x = X^T X b_s, then FP64 iterative refinement
//        r = b_s - S x (FP64 accumulation),  x += X^T X r
//    until ||r|| <= tol ||b_s|| or the sweep limit, all GEMVs inside one
//    cooperative launch with a deterministic grid-wide norm.
#include <cooperative_groups.h>

#include "ba_internal.h"

namespace cg = cooperative_groups;

namespace zs {

constexpr int kB = 32;

cudaError_t launch_tri_inverse64(int n, const float* F, const float* D, float* X, float* XT, LmState* st,
                                 cudaStream_t s);

template <typename T>
__device__ __forceinline__ T ldc(const T* p) {
    return __ldcg(p);
}

// acc (r, c4..c4+3) += sum over k-blocks m in [m0, m1) of
// A[rowA0 + r, 32m + kk] * B[32m + kk, colB0 + c4 + q], zero outside n.
// A and B may have been written earlier in this launch (read through L2).
template <typename T>
__device__ void tile_gemm(int n, const T* A, int rowA0, const T* B, int colB0, int m0, int m1, T (*sa)[kB + 1],
                          T (*sb)[kB + 1], T acc[4]) {
    const int r = threadIdx.x / 8, c4 = (threadIdx.x % 8) * 4;
    for (int m = m0; m < m1; ++m) {
        T va[4], vb[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int e = threadIdx.x + q * kThreads;
            const int rr = e / kB, cc = e % kB;
            const int ar = rowA0 + rr, ac = m * kB + cc;
            va[q] = (ar < n && ac < n) ? ldc(A + (int64_t)ar * n + ac) : T(0);
            const int br = m * kB + rr, bc = colB0 + cc;
            vb[q] = (br < n && bc < n) ? ldc(B + (int64_t)br * n + bc) : T(0);
        }
        __syncthreads();
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int e = threadIdx.x + q * kThreads;
            sa[e / kB][e % kB] = va[q];
            sb[e / kB][e % kB] = vb[q];
        }
        __syncthreads();
#pragma unroll 8
        for (int kk = 0; kk < kB; ++kk) {
            const T av = sa[r][kk];
            acc[0] += av * sb[kk][c4];
            acc[1] += av * sb[kk][c4 + 1];
            acc[2] += av * sb[kk][c4 + 2];
            acc[3] += av * sb[kk][c4 + 3];
        }
    }
    __syncthreads();
}

template <typename T>
__global__ void __launch_bounds__(kThreads, 1) k_tri_inverse(int n, const T* __restrict__ F, const T* __restrict__ D,
                                                             T* X, T* XT, const LmState* st) {
    cg::grid_group grid = cg::this_grid();
    __shared__ T sa[kB][kB + 1];
    __shared__ T sb[kB][kB + 1];
    if (!__ldcg(&st->solve_ok)) return;  // written by an earlier launch: uniform
    const int nblk = (n + kB - 1) / kB;
    // level 0: diagonal blocks X_kk = D_k (and their transposes)
    for (int k = blockIdx.x; k < nblk; k += gridDim.x) {
        for (int e = threadIdx.x; e < kB * kB; e += blockDim.x) {
            const int r = e / kB, c = e % kB;
            const int gr = k * kB + r, gc = k * kB + c;
            if (gr < n && gc < n) {
                const T v = D[(int64_t)k * kB * kB + e];
                X[(int64_t)gr * n + gc] = v;
                XT[(int64_t)gc * n + gr] = v;
            }
        }
    }
    grid.sync();
    const int r = threadIdx.x / 8, c4 = (threadIdx.x % 8) * 4;
    for (int s = 1; s < nblk; s *= 2) {
        const int npairs = (nblk + 2 * s - 1) / (2 * s);
        const int ntask = npairs * s * s;
        // step 1: T_ij = sum_{m=j}^{a_end-1} L_im X_mj -> XT[rows of i, cols of j] (lower scratch)
        for (int t = blockIdx.x; t < ntask; t += gridDim.x) {
            const int p = t / (s * s), w = t % (s * s);
            const int a0 = p * 2 * s, c0 = a0 + s;
            const int i = c0 + w / s, j = a0 + w % s;
            if (i >= nblk) continue;
            T acc[4] = {T(0), T(0), T(0), T(0)};
            tile_gemm<T>(n, F, i * kB, X, j * kB, j, c0, sa, sb, acc);
            const int row = i * kB + r;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int col = j * kB + c4 + q;
                if (row < n && col < n) XT[(int64_t)row * n + col] = acc[q];
            }
        }
        grid.sync();
        // step 2: X_ij = - sum_{m=c0}^{i} X_im T_mj
        for (int t = blockIdx.x; t < ntask; t += gridDim.x) {
            const int p = t / (s * s), w = t % (s * s);
            const int a0 = p * 2 * s, c0 = a0 + s;
            const int i = c0 + w / s, j = a0 + w % s;
            if (i >= nblk) continue;
            T acc[4] = {T(0), T(0), T(0), T(0)};
            tile_gemm<T>(n, X, i * kB, XT, j * kB, c0, i + 1, sa, sb, acc);
            const int row = i * kB + r;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int col = j * kB + c4 + q;
                if (row < n && col < n) {
                    X[(int64_t)row * n + col] = -acc[q];
                    XT[(int64_t)col * n + row] = -acc[q];
                }
            }
        }
        grid.sync();
    }
}

__device__ inline double wsum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// out[i] = sum_{c in [lo(i), hi(i))} M[i][c] * v[c], a warp per row (grid-stride).
// mode 0: c <= i (lower), 1: c >= i (upper), 2: all.
template <typename T>
__device__ void gemv_rows(int n, const T* __restrict__ M, const double* v, double* out, int mode, const double* b,
                          double* part2) {
    const int lane = threadIdx.x & 31;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    double p2 = 0.0;
    for (int i = gw; i < n; i += nw) {
        const int lo = (mode == 1) ? i : 0;
        const int hi = (mode == 0) ? i + 1 : n;
        double acc = 0.0;
        for (int c = lo + lane; c < hi; c += 32) acc += (double)M[(int64_t)i * n + c] * ldc(v + c);
        acc = wsum(acc);
        if (lane == 0) {
            if (b) {
                const double ri = b[i] - acc;
                out[i] = ri;
                p2 += ri * ri;
            } else {
                out[i] = acc;
            }
        }
    }
    if (part2) *part2 = p2;
}

template <typename TS, typename TX>
__global__ void __launch_bounds__(kThreads) k_refine(int n, const TS* __restrict__ S, const TX* __restrict__ X,
                                                     const TX* __restrict__ XT, const double* __restrict__ bs,
                                                     double* x, double* u, double* r, double* scratch, int refine,
                                                     double tol, LmState* st) {
    cg::grid_group grid = cg::this_grid();
    __shared__ double red[kThreads / 32];
    if (!__ldcg(&st->solve_ok)) return;  // uniform
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    // x0 = X^T (X bs)
    gemv_rows<TX>(n, X, bs, u, 0, nullptr, nullptr);
    grid.sync();
    gemv_rows<TX>(n, XT, u, x, 1, nullptr, nullptr);
    grid.sync();
    double bn2 = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) bn2 += bs[i] * bs[i];
    bn2 = wsum(bn2);
    if (lane == 0) red[warp] = bn2;
    __syncthreads();
    bn2 = 0.0;
    for (int w = 0; w < kThreads / 32; ++w) bn2 += red[w];
    __syncthreads();
    int sweeps = 0;
    double rn2 = 0.0;
    for (int it = 0;; ++it) {
        double p2 = 0.0;
        gemv_rows<TS>(n, S, x, r, 2, bs, &p2);
        if (lane == 0) red[warp] = p2;
        __syncthreads();
        if (threadIdx.x == 0) {
            double s = 0.0;
            for (int w = 0; w < kThreads / 32; ++w) s += red[w];
            scratch[blockIdx.x] = s;
        }
        grid.sync();
        rn2 = 0.0;
        for (unsigned b = 0; b < gridDim.x; ++b) rn2 += ldc(scratch + b);
        if (it >= refine || !(rn2 > tol * tol * bn2)) break;
        grid.sync();  // everyone has read scratch before it is rewritten
        gemv_rows<TX>(n, X, r, u, 0, nullptr, nullptr);
        grid.sync();
        // x += X^T u, a warp per row
        {
            const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
            const int nw = (gridDim.x * blockDim.x) >> 5;
            for (int i = gw; i < n; i += nw) {
                double acc = 0.0;
                for (int c = i + lane; c < n; c += 32) acc += (double)XT[(int64_t)i * n + c] * ldc(u + c);
                acc = wsum(acc);
                if (lane == 0) x[i] += acc;
            }
        }
        grid.sync();
        ++sweeps;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        st->resid_norm = sqrt(rn2);
        st->rhs_norm = sqrt(bn2);
        st->refine_sweeps = sweeps;
    }
}

static int sm_count() {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return sms > 0 ? sms : 1;
}

template <typename TX>
cudaError_t launch_tri_inverse(int n, const TX* F, const TX* D, TX* X, TX* XT, LmState* st, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    if (sizeof(TX) == 4 && n >= 128)  // 64-wide blocks, asynchronous tile loads (ba_chol_blk.cu)
        return launch_tri_inverse64(n, reinterpret_cast<const float*>(F), reinterpret_cast<const float*>(D),
                                    reinterpret_cast<float*>(X), reinterpret_cast<float*>(XT), st, s);
    int nn = n;
    void* args[] = {(void*)&nn, (void*)&F, (void*)&D, (void*)&X, (void*)&XT, (void*)&st};
    cudaError_t e = cudaLaunchCooperativeKernel((const void*)k_tri_inverse<TX>, dim3(sm_count()), dim3(kThreads), args,
                                                0, s);
    if (e == cudaSuccess) note_launch();
    return e;
}

template <typename TS, typename TX>
cudaError_t launch_refine(int n, const TS* S, const TX* X, const TX* XT, const double* bs, double* x, double* work,
                          LmState* st, int refine_iters, double tol, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    int nn = n, it = refine_iters;
    double* u = work;
    double* r = work + n;
    double* scratch = work + 4 * (int64_t)n;
    void* args[] = {(void*)&nn, (void*)&S, (void*)&X, (void*)&XT, (void*)&bs, (void*)&x,
                    (void*)&u,  (void*)&r, (void*)&scratch, (void*)&it, (void*)&tol, (void*)&st};
    int blocks = (n + 7) / 8;  // a row per warp when the grid is large enough
    if (blocks > sm_count()) blocks = sm_count();
    cudaError_t e =
        cudaLaunchCooperativeKernel((const void*)k_refine<TS, TX>, dim3(blocks), dim3(kThreads), args, 0, s);
    if (e == cudaSuccess) note_launch();
    return e;
}

template cudaError_t launch_tri_inverse<float>(int, const float*, const float*, float*, float*, LmState*,
                                               cudaStream_t);
template cudaError_t launch_refine<float, float>(int, const float*, const float*, const float*, const double*, double*,
                                                double*, LmState*, int, double, cudaStream_t);
template cudaError_t launch_refine<double, float>(int, const double*, const float*, const float*, const double*,
                                                 double*, double*, LmState*, int, double, cudaStream_t);

}  // namespace zs
