// Blocked Cholesky S = L L^T of the mixed form's FP32 reduced camera system
// (n >= 128): one cooperative persistent kernel, 64-wide panels.
//
// Per panel k (columns k0 .. k0 + 64):
//   stage B  (all CTAs) panel rows below: L21 = A21 L11^-T, a 64 x 64 product
//            per 64-row block with the explicit inverse of L11;
//   stage C  (all CTAs) trailing lower 64 x 64 tiles: A22 -= L21 L21^T, a
//            rank-64 update per tile; CTA 0 updates only the next diagonal
//            tile and then factors it in shared memory (32 x 32 tiles,
//            ba_tiles.cuh) and forms its inverse (look-ahead), so the next
//            panel's stage B can start after one grid barrier.
// Two grid barriers per panel (19 panels at n = 1200, 94 at n = 6000,
// against 38 / 188 with 32-wide panels). The pivot test is zeroslam's
// (source/matrix_decomposition_cholesky.hpp:40,53): a pivot must exceed
// 1e-14 max|S_ii| (st->eps_factor). The output layout is the one the solves
// read: L in F's lower triangle, zeros above the diagonal inside each
// diagonal 32 x 32 block (k_diag_inverses then forms the 32 x 32 inverses).
#include <cooperative_groups.h>

#include "ba_internal.h"
#include "ba_tiles.cuh"

namespace cg = cooperative_groups;

namespace zs {

namespace {

constexpr int kP = 64;          // panel width and tile size
constexpr int kPL = kP + 4;     // row of a shared-memory operand: 16-byte rows, conflict-free 128-bit reads
constexpr int kBlkThreads = 256;

// Dynamic shared memory: two 64 x 64 operands, the diagonal block as three
// 32 x 32 tiles, the 64 x 64 inverse, per-row pivot thresholds and 1 / L_ii.
constexpr size_t kBlkSmem = sizeof(float) * (2 * kP * kPL + 3 * kTile + kP * kPL + 2 * kP) + 64;

__device__ __forceinline__ float ldcg(const float* p) { return __ldcg(p); }

// acc[i][j] = sum_m A[ty + 16 i][m] B[tx + 16 j][m] over m < kk rounded up to
// 4 (operands zero beyond kk). Thread (ty, tx) of a 16 x 16 grid owns rows
// ty + 16 i and columns tx + 16 j; operands are read as float4 along m: the B
// reads of 8 consecutive lanes hit distinct 16-byte bank groups (row stride
// 68 floats), the A reads are broadcasts.
__device__ __forceinline__ void tile_nt_acc(const float* A, const float* B, int kk, float acc[4][4]) {
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int k4 = (kk + 3) >> 2;
#pragma unroll 1
    for (int q = 0; q < k4; ++q) {
        float4 a[4], b[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) a[i] = *reinterpret_cast<const float4*>(A + (ty + 16 * i) * kPL + 4 * q);
#pragma unroll
        for (int j = 0; j < 4; ++j) b[j] = *reinterpret_cast<const float4*>(B + (tx + 16 * j) * kPL + 4 * q);
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                acc[i][j] = fmaf(a[i].x, b[j].x, acc[i][j]);
                acc[i][j] = fmaf(a[i].y, b[j].y, acc[i][j]);
                acc[i][j] = fmaf(a[i].z, b[j].z, acc[i][j]);
                acc[i][j] = fmaf(a[i].w, b[j].w, acc[i][j]);
            }
    }
}

__device__ __forceinline__ void tile_nt(const float* A, const float* B, int kk, float acc[4][4]) {
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = 0.f;
    tile_nt_acc(A, B, kk, acc);
}

// 16-byte asynchronous global -> shared copy; src_bytes < 16 zero-fills the rest.
__device__ __forceinline__ void cp_async16(float* dst, const float* src, int src_bytes) {
    const unsigned d = static_cast<unsigned>(__cvta_generic_to_shared(dst));
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(d), "l"(src), "r"(src_bytes) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
    asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;\n" ::: "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_one() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_none() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// Rows r0 .. r0 + 64 (clipped to n), columns c0 .. c0 + kk of F into
// S[row][m] (zero outside). With n % 4 == 0 (16-byte rows) and c0 % 4 == 0:
// 16-byte asynchronous copies, four per thread, all in flight together.
// The caller waits (cp_async_wait_all) and synchronises before reading S.
__device__ __forceinline__ void load_block(const float* F, int n, int r0, int c0, int kk, float* S) {
    if ((n & 3) == 0) {
#pragma unroll
        for (int q = 0; q < (kP * kP / 4) / kBlkThreads; ++q) {
            const int e = threadIdx.x + q * kBlkThreads;
            const int r = e >> 4, c4 = (e & 15) * 4;
            const int row = r0 + r;
            int bytes = (row < n) ? 4 * min(4, kk - c4) : 0;
            if (bytes < 0) bytes = 0;
            const float* src = bytes > 0 ? F + (int64_t)row * n + c0 + c4 : F;
            cp_async16(S + r * kPL + c4, src, bytes);
        }
    } else {
        float v[(kP * kP) / kBlkThreads];
#pragma unroll
        for (int q = 0; q < (kP * kP) / kBlkThreads; ++q) {
            const int e = threadIdx.x + q * kBlkThreads;
            const int r = e >> 6, m = e & 63;
            v[q] = (r0 + r < n && m < kk) ? ldcg(F + (int64_t)(r0 + r) * n + c0 + m) : 0.f;
        }
#pragma unroll
        for (int q = 0; q < (kP * kP) / kBlkThreads; ++q) {
            const int e = threadIdx.x + q * kBlkThreads;
            S[(e >> 6) * kPL + (e & 63)] = v[q];
        }
    }
}

// Factors the diagonal block at (k0, k0) of width kb (<= 64) in shared
// memory; on success writes L (zeros above the diagonal) into F and the
// block's inverse L^-1 (64 x 64, zero-padded) into Li. Returns 1 on success
// (uniform over the CTA).
__device__ int factor_diag64(float* F, int n, int k0, int kb, float eps, float* T, float* dinv, float* epsr, float* Inv,
                             float* Li, int* s_flag) {
    const int nbw = (kb + 31) >> 5;
    // tiles (identity padding beyond kb)
    {
        float v[(kP * kP) / kBlkThreads];
#pragma unroll
        for (int q = 0; q < (kP * kP) / kBlkThreads; ++q) {
            const int e = threadIdx.x + q * kBlkThreads;
            const int i = e >> 6, j = e & 63;
            v[q] = (i < kb && j < kb && j <= i) ? ldcg(F + (int64_t)(k0 + i) * n + k0 + j) : (i == j ? 1.f : 0.f);
        }
#pragma unroll
        for (int q = 0; q < (kP * kP) / kBlkThreads; ++q) {
            const int e = threadIdx.x + q * kBlkThreads;
            const int i = e >> 6, j = e & 63;
            if (j <= i && (i >> 5) < nbw) tile_at(T, i >> 5, j >> 5)[(i & 31) * kLd + (j & 31)] = v[q];
        }
    }
    if (threadIdx.x < 64) epsr[threadIdx.x] = eps;
    __syncthreads();
    if (!cta_cholesky<float>(T, nbw, kb, epsr, dinv, s_flag)) return 0;
    // full inverse: [Xa 0; -Xc Lb Xa  Xc] from the tile inverses
    for (int e = threadIdx.x; e < 64 * 64; e += blockDim.x) {
        const int r = e >> 6, c = e & 63;
        float v = 0.f;
        if ((r >> 5) == (c >> 5) && (r >> 5) < nbw) {
            const int b = r >> 5, rr = r & 31, cc = c & 31;
            v = rr == cc ? dinv[r] : (cc < rr ? tile_at(T, b, b)[cc * kLd + rr] : 0.f);
        }
        Inv[r * kPL + c] = v;
    }
    __syncthreads();
    if (nbw == 2) {
        // W = Lb Xa (32 x 32) into the lower-left quadrant of Inv, then Xc W
        // (Xa is lower triangular and Inv holds zeros above it, so every lane
        // runs the full 32 terms: no divergence, four independent chains)
        float w[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll 8
        for (int m = 0; m < 32; ++m) {
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int e = threadIdx.x + q * blockDim.x;
                w[q] = fmaf(tile_at(T, 1, 0)[(e >> 5) * kLd + m], Inv[m * kPL + (e & 31)], w[q]);
            }
        }
        __syncthreads();
        for (int q = 0; q < 4; ++q) {
            const int e = threadIdx.x + q * blockDim.x;
            Inv[(32 + (e >> 5)) * kPL + (e & 31)] = w[q];
        }
        __syncthreads();
        // (Xc is lower triangular with zeros above it in Inv: the full 32 terms)
#pragma unroll
        for (int q = 0; q < 4; ++q) w[q] = 0.f;
#pragma unroll 8
        for (int m = 0; m < 32; ++m) {
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int e = threadIdx.x + q * blockDim.x;
                w[q] = fmaf(Inv[(32 + (e >> 5)) * kPL + 32 + m], Inv[(32 + m) * kPL + (e & 31)], w[q]);
            }
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) w[q] = -w[q];
        __syncthreads();
        for (int q = 0; q < 4; ++q) {
            const int e = threadIdx.x + q * blockDim.x;
            Inv[(32 + (e >> 5)) * kPL + (e & 31)] = w[q];
        }
        __syncthreads();
    }
    // Li = Inv, as 16-byte copies (Inv rows are 16-byte aligned)
    for (int e4 = threadIdx.x; e4 < 64 * 16; e4 += blockDim.x)
        reinterpret_cast<float4*>(Li)[e4] = *reinterpret_cast<const float4*>(Inv + (e4 >> 4) * kPL + (e4 & 15) * 4);
    // L into F: the diagonal 32-blocks (zeros above their diagonals) and the
    // lower-left block; the upper-right block keeps S
    for (int e = threadIdx.x; e < 3 * 1024; e += blockDim.x) {
        const int blk = e >> 10, rr = (e >> 5) & 31, cc = e & 31;
        const int bi = blk == 0 ? 0 : 1, bj = blk == 2 ? 1 : 0;  // (0, 0), (1, 0), (1, 1)
        const int i = 32 * bi + rr, j = 32 * bj + cc;
        if (i >= kb || j >= kb) continue;
        const float* Tb = tile_at(T, bi, bj);
        const float v = (bi != bj || cc < rr) ? Tb[rr * kLd + cc] : (cc == rr ? Tb[rr * (kLd + 1)] : 0.f);
        F[(int64_t)(k0 + i) * n + k0 + j] = v;
    }
    __syncthreads();
    return 1;
}

}  // namespace

__global__ void __launch_bounds__(kBlkThreads) k_chol_blk(int n, float* F, float* Li, LmState* st) {
    cg::grid_group grid = cg::this_grid();
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float* sA = reinterpret_cast<float*>(smem_raw);
    float* sB = sA + kP * kPL;
    float* T = sB + kP * kPL;
    float* Inv = T + 3 * kTile;
    float* dinv = Inv + kP * kPL;
    float* epsr = dinv + kP;
    __shared__ int s_flag;
    const float eps = (float)__ldcg(&st->eps_factor);
    const int G = gridDim.x;
    const int skip = __ldcg(&st->skip_factor);  // written by an earlier launch: uniform
    const int nblk = skip ? 0 : (n + kP - 1) / kP;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    if (blockIdx.x == 0 && !skip) {
        if (!factor_diag64(F, n, 0, min(kP, n), eps, T, dinv, epsr, Inv, Li, &s_flag) && threadIdx.x == 0)
            st->solve_ok = 0;
    }
    grid.sync();
    for (int k = 0; k < nblk; ++k) {
        if (!__ldcg(&st->solve_ok)) return;
        const int k0 = k * kP;
        const int kb = min(kP, n - k0);
        const int r0 = k0 + kb;
        if (r0 >= n) break;
        const int tn = (n - r0 + kP - 1) / kP;  // trailing block rows
        // stage B: L21 = A21 L11^-T
        {
            bool have_li = false;
            for (int rb = blockIdx.x; rb < tn; rb += G) {
                if (!have_li) {
                    float v[(kP * kP) / kBlkThreads];
#pragma unroll
                    for (int q = 0; q < (kP * kP) / kBlkThreads; ++q) v[q] = ldcg(Li + threadIdx.x + q * kBlkThreads);
#pragma unroll
                    for (int q = 0; q < (kP * kP) / kBlkThreads; ++q) {
                        const int e = threadIdx.x + q * kBlkThreads;
                        sB[(e >> 6) * kPL + (e & 63)] = v[q];
                    }
                    have_li = true;
                }
                const int rr = r0 + rb * kP;
                load_block(F, n, rr, k0, kb, sA);
                cp_async_wait_all();
                __syncthreads();
                float acc[4][4];
                tile_nt(sA, sB, kb, acc);
#pragma unroll
                for (int i = 0; i < 4; ++i)
#pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        const int row = rr + ty + 16 * i, col = tx + 16 * j;
                        if (row < n && col < kb) F[(int64_t)row * n + k0 + col] = acc[i][j];
                    }
                __syncthreads();
            }
        }
        grid.sync();
        // stage C: trailing tiles (ti, tj), tj <= ti; CTA 0 takes tile (0, 0)
        // and then factors it (look-ahead)
        {
            const int ntiles = tn * (tn + 1) / 2;
            const int first = (G == 1) ? 0 : (blockIdx.x == 0 ? 0 : blockIdx.x);
            const int stride = (G == 1) ? 1 : (blockIdx.x == 0 ? ntiles : G - 1);
            for (int t = first; t < ntiles; t += stride) {
                int ti = 0;
                while ((ti + 1) * (ti + 2) / 2 <= t) ++ti;
                const int tj = t - ti * (ti + 1) / 2;
                const int i0 = r0 + ti * kP, j0 = r0 + tj * kP;
                load_block(F, n, i0, k0, kb, sA);
                if (ti != tj) load_block(F, n, j0, k0, kb, sB);
                cp_async_wait_all();
                __syncthreads();
                float acc[4][4];
                tile_nt(sA, ti != tj ? sB : sA, kb, acc);
                float c[4][4];
#pragma unroll
                for (int i = 0; i < 4; ++i)
#pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        const int row = i0 + ty + 16 * i, col = j0 + tx + 16 * j;
                        c[i][j] = (row < n && col < n) ? ldcg(F + (int64_t)row * n + col) : 0.f;
                    }
#pragma unroll
                for (int i = 0; i < 4; ++i)
#pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        const int row = i0 + ty + 16 * i, col = j0 + tx + 16 * j;
                        if (row < n && col < n && (ti != tj || col <= row))
                            F[(int64_t)row * n + col] = c[i][j] - acc[i][j];
                    }
                __syncthreads();
                if (t == 0) {
                    __threadfence_block();
                    if (!factor_diag64(F, n, r0, min(kP, n - r0), eps, T, dinv, epsr, Inv, Li, &s_flag) &&
                        threadIdx.x == 0)
                        st->solve_ok = 0;
                }
            }
        }
        grid.sync();
    }
}

namespace {

constexpr size_t kInvSmem = sizeof(float) * 4 * kP * kPL;

// acc = sum over 64-wide K chunks m in [m0, m1) of A[ra rows][m] B[rb rows][m]^T
// (both row-major with row length n), two-stage asynchronous pipeline.
__device__ void tile_nt_chunks(const float* A, int ra, const float* B, int rb, int n, int m0, int m1, float* buf,
                               float acc[4][4]) {
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = 0.f;
    if (m0 >= m1) return;
    float* sa[2] = {buf, buf + 2 * kP * kPL};
    float* sb[2] = {buf + kP * kPL, buf + 3 * kP * kPL};
    load_block(A, n, ra, kP * m0, min(kP, n - kP * m0), sa[0]);
    load_block(B, n, rb, kP * m0, min(kP, n - kP * m0), sb[0]);
    cp_async_commit();
    for (int m = m0; m < m1; ++m) {
        const int cur = (m - m0) & 1;
        if (m + 1 < m1) {
            load_block(A, n, ra, kP * (m + 1), min(kP, n - kP * (m + 1)), sa[cur ^ 1]);
            load_block(B, n, rb, kP * (m + 1), min(kP, n - kP * (m + 1)), sb[cur ^ 1]);
            cp_async_commit();
            cp_async_wait_one();
        } else {
            cp_async_wait_none();
        }
        __syncthreads();
        tile_nt_acc(sa[cur], sb[cur], min(kP, n - kP * m), acc);
        __syncthreads();
    }
}

}  // namespace

// X = L^-1 (and X^T) of the mixed form's factor, by recursive 2 x 2 block
// inversion over 64-wide blocks,
//     inv([A 0; B C]) = [A^-1 0; -C^-1 (B A^-1)  C^-1],
// level 0 from the 32 x 32 diagonal inverses D_k (k_diag_inverses), then
// log2(n/64) levels of 64 x 64 output tiles, two grid barriers per level.
// Every product reads K-contiguous rows: (B A^-1)^T is kept in X's upper
// triangle (free: the refinement reads X's lower and X^T's upper triangle).
__global__ void __launch_bounds__(kBlkThreads) k_tri_inverse64(int n, const float* F, const float* D, float* X, float* XT,
                                                               const LmState* st) {
    cg::grid_group grid = cg::this_grid();
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float* buf = reinterpret_cast<float*>(smem_raw);
    if (!__ldcg(&st->solve_ok)) return;  // written by an earlier launch: uniform
    const int nb = (n + kP - 1) / kP;
    const int nb32 = (n + 31) / 32;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    // level 0: X_bb = [D0 0; -D1 Lb D0  D1] for each 64-block b
    for (int b = blockIdx.x; b < nb; b += gridDim.x) {
        float* d0 = buf;               // 32 x 33
        float* d1 = d0 + 32 * 33;
        float* lb = d1 + 32 * 33;
        float* w = lb + 32 * 33;
        float* y = w + 32 * 33;
        const bool two = 2 * b + 1 < nb32;
        for (int e = threadIdx.x; e < 1024; e += blockDim.x) {
            const int r = e >> 5, c = e & 31;
            d0[r * 33 + c] = ldcg(D + (int64_t)(2 * b) * 1024 + e);
            d1[r * 33 + c] = two ? ldcg(D + (int64_t)(2 * b + 1) * 1024 + e) : 0.f;
            const int gr = 64 * b + 32 + r, gc = 64 * b + c;
            lb[r * 33 + c] = (two && gr < n) ? ldcg(F + (int64_t)gr * n + gc) : 0.f;
        }
        __syncthreads();
        for (int e = threadIdx.x; e < 1024; e += blockDim.x) {
            const int r = e >> 5, c = e & 31;
            float s = 0.f;
            for (int m = c; m < 32; ++m) s = fmaf(lb[r * 33 + m], d0[m * 33 + c], s);
            w[r * 33 + c] = s;
        }
        __syncthreads();
        for (int e = threadIdx.x; e < 1024; e += blockDim.x) {
            const int r = e >> 5, c = e & 31;
            float s = 0.f;
            for (int m = 0; m <= r; ++m) s = fmaf(d1[r * 33 + m], w[m * 33 + c], s);
            y[r * 33 + c] = -s;
        }
        __syncthreads();
        for (int e = threadIdx.x; e < 4096; e += blockDim.x) {
            const int r = e >> 6, c = e & 63;
            const int gr = 64 * b + r, gc = 64 * b + c;
            if (gr >= n || gc >= n) continue;
            float v = 0.f;
            if (r < 32 && c < 32) v = c <= r ? d0[r * 33 + c] : 0.f;
            else if (r >= 32 && c >= 32) v = (c <= r) ? d1[(r - 32) * 33 + (c - 32)] : 0.f;
            else if (r >= 32) v = y[(r - 32) * 33 + c];
            X[(int64_t)gr * n + gc] = v;
            XT[(int64_t)gc * n + gr] = v;
        }
        __syncthreads();
    }
    grid.sync();
    float* stage = buf;  // 64 x 65 staging for the transposed store
    for (int s = 1; s < nb; s *= 2) {
        const int npairs = (nb + 2 * s - 1) / (2 * s);
        const int ntask = npairs * s * s;
        // step 1: (T_ij)^T = sum_{m=j}^{c0-1} X^T[j][m] L[i][m]^T -> X rows of j, columns of i
        for (int t = blockIdx.x; t < ntask; t += gridDim.x) {
            const int p = t / (s * s), w = t % (s * s);
            const int a0 = p * 2 * s, c0 = a0 + s;
            const int i = c0 + w / s, j = a0 + w % s;
            if (i >= nb) continue;
            float acc[4][4];
            tile_nt_chunks(XT, kP * j, F, kP * i, n, j, c0, buf, acc);
#pragma unroll
            for (int a = 0; a < 4; ++a)
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const int row = kP * j + ty + 16 * a, col = kP * i + tx + 16 * q;
                    if (row < n && col < n) X[(int64_t)row * n + col] = acc[a][q];
                }
        }
        grid.sync();
        // step 2: X_ij = - sum_{m=c0}^{i} X[i][m] (T^T)[j][m]
        for (int t = blockIdx.x; t < ntask; t += gridDim.x) {
            const int p = t / (s * s), w = t % (s * s);
            const int a0 = p * 2 * s, c0 = a0 + s;
            const int i = c0 + w / s, j = a0 + w % s;
            if (i >= nb) continue;
            float acc[4][4];
            tile_nt_chunks(X, kP * i, X, kP * j, n, c0, i + 1, buf, acc);
#pragma unroll
            for (int a = 0; a < 4; ++a)
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const int r = ty + 16 * a, c = tx + 16 * q;
                    stage[r * 65 + c] = -acc[a][q];
                    const int row = kP * i + r, col = kP * j + c;
                    if (row < n && col < n) X[(int64_t)row * n + col] = -acc[a][q];
                }
            __syncthreads();
            for (int e = threadIdx.x; e < 4096; e += blockDim.x) {
                const int c = e >> 6, r = e & 63;  // XT[col][row], rows of XT along j, coalesced over r
                const int row = kP * i + r, col = kP * j + c;
                if (row < n && col < n) XT[(int64_t)col * n + row] = stage[r * 65 + c];
            }
            __syncthreads();
        }
        grid.sync();
    }
}

cudaError_t launch_tri_inverse64(int n, const float* F, const float* D, float* X, float* XT, LmState* st,
                                 cudaStream_t s) {
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaError_t e =
        cudaFuncSetAttribute(k_tri_inverse64, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kInvSmem);
    if (e != cudaSuccess) return e;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_tri_inverse64, kBlkThreads, kInvSmem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    int nn = n;
    void* args[] = {(void*)&nn, (void*)&F, (void*)&D, (void*)&X, (void*)&XT, (void*)&st};
    e = cudaLaunchCooperativeKernel((const void*)k_tri_inverse64, dim3(sms * per_sm), dim3(kBlkThreads), args,
                                    kInvSmem, s);
    if (e != cudaSuccess) return e;
    note_launch();
    return cudaSuccess;
}

cudaError_t launch_chol_blk(int n, float* F, float* Li, LmState* st, cudaStream_t s) {
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaError_t e = cudaFuncSetAttribute(k_chol_blk, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kBlkSmem);
    if (e != cudaSuccess) return e;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_chol_blk, kBlkThreads, kBlkSmem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    const int nblk = (n + kP - 1) / kP;
    int blocks = sms * per_sm;  // all co-resident
    if (blocks > nblk * (nblk + 1) / 2 + 1) blocks = nblk * (nblk + 1) / 2 + 1;
    if (blocks < 1) blocks = 1;
    int nn = n;
    void* args[] = {(void*)&nn, (void*)&F, (void*)&Li, (void*)&st};
    e = cudaLaunchCooperativeKernel((const void*)k_chol_blk, dim3(blocks), dim3(kBlkThreads), args, kBlkSmem, s);
    if (e != cudaSuccess) return e;
    note_launch();
    return cudaSuccess;
}

}  // namespace zs
