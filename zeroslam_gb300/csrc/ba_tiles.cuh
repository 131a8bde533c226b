// Shared-memory tile routines: a symmetric matrix of up to a few hundred
// rows held in shared memory as the lower triangle of 32 x 32 tiles, factored
// by a blocked right-looking Cholesky (per-tile inverses kept), and solved.
// Used by the batched window solve and by the diagonal blocks of the large
// factorisation.
#pragma once

#include "ba_common.cuh"

namespace zs {

// A window's S lives in shared memory as the lower triangle of 32 x 32
// tiles, tile (ib, jb) (jb <= ib) at tile index ib (ib + 1) / 2 + jb, rows
// padded to kLd elements so that row- and column-wise warp accesses hit
// distinct banks. Rows and columns from n up to the next multiple of 32 are
// an identity block (zero right-hand side), so every loop runs on whole tiles.
constexpr int kLd = 33;
constexpr int kTile = 32 * kLd;

template <typename TF>
__device__ __forceinline__ TF* tile_at(TF* A, int ib, int jb) {
    return A + (ib * (ib + 1) / 2 + jb) * kTile;
}

// Blocked right-looking Cholesky of the nbw x nbw tile lower triangle.
// Per diagonal tile: warp 0 factors it (a row per lane in registers) and
// inverts it (a column of L_kk^-1 per lane, right-looking so that the 32
// accumulators are independent), storing L_kk^-1 transposed in the tile's
// unused upper triangle (tile[j][i] = (L_kk^-1)[i][j], j < i) and 1 / L_ii in
// dinv; the panel below is then the product A(ib, kb) L_kk^-T (a row per
// thread, no division chain), and the trailing tiles get a rank-32 update.
// Pivot test d > eps_i over the real rows (i < n): eps_i = 1e-14 max|S_ii| sc_i^2
// is the reference's test on the unscaled pivot
// (source/matrix_decomposition_cholesky.hpp:40,53).
// Returns 1 on success (uniform over the CTA).
// Pivot d -> (L_cc, 1 / L_cc). The mixed form (float) uses the reciprocal
// square root (its refinement corrects the factor's last bits); the plain
// form keeps the reference's sqrt and division.
__device__ __forceinline__ void pivot_root(float d, float& l, float& inv) {
    inv = rsqrtf(d);
    l = d * inv;
}
__device__ __forceinline__ void pivot_root(double d, double& l, double& inv) {
    l = sqrt(d);
    inv = 1.0 / l;
}
__device__ __forceinline__ float scale_by(float x, float l, float inv) { return x * inv; }
__device__ __forceinline__ double scale_by(double x, double l, double inv) { return x / l; }

template <typename TF>
__device__ int cta_cholesky(TF* A, int nbw, int n, const TF* eps, TF* dinv, int* s_flag) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int kb = 0; kb < nbw; ++kb) {
        TF* D = tile_at(A, kb, kb);
        // 1. diagonal tile by warp 0
        if (warp == 0) {
            TF row[32];
#pragma unroll
            for (int j = 0; j < 32; ++j) row[j] = D[lane * kLd + j];
            int fail = 0;
            TF own_inv = TF(1);
#pragma unroll
            for (int c = 0; c < 32; ++c) {
                const TF d = __shfl_sync(0xffffffffu, row[c], c);
                if (32 * kb + c < n && !(d > eps[32 * kb + c])) fail = 1;
                TF lcc, inv;
                pivot_root(d, lcc, inv);
                if (lane == c) {
                    row[c] = lcc;
                    own_inv = inv;
                }
                if (lane > c) row[c] = scale_by(row[c], lcc, inv);
                const TF lic = row[c];
#pragma unroll
                for (int j = 0; j < 32; ++j) {
                    if (j > c) {
                        const TF ljc = __shfl_sync(0xffffffffu, lic, j);
                        if (lane >= j) row[j] -= lic * ljc;
                    }
                }
            }
#pragma unroll
            for (int j = 0; j <= 31; ++j)
                if (j <= lane) D[lane * kLd + j] = row[j];
            dinv[32 * kb + lane] = own_inv;  // 1 / L_ii of this tile
            __syncwarp();
            // column `lane` of L_kk^-1, right-looking
            TF acc[32];
#pragma unroll
            for (int i = 0; i < 32; ++i) acc[i] = TF(0);
#pragma unroll
            for (int m = 0; m < 32; ++m) {
                const TF dm = dinv[32 * kb + m];
                const TF ym = (m < lane) ? TF(0) : ((m == lane) ? dm : -acc[m] * dm);
                acc[m] = ym;  // acc[m] now holds y_m
#pragma unroll
                for (int i = 0; i < 32; ++i)
                    if (i > m) acc[i] += D[i * kLd + m] * ym;
            }
            __syncwarp();
#pragma unroll
            for (int i = 0; i < 32; ++i)
                if (i > lane) D[lane * kLd + i] = acc[i];
            if (lane == 0) *s_flag = fail;
        }
        __syncthreads();
        if (*s_flag) return 0;
        // 2. panel: L(ib, kb) = A(ib, kb) L_kk^-T, four outputs of one row per
        //    item: out_j = a_j / L_jj + sum_{m < j} a_m (L_kk^-1)[j][m]; the
        //    outputs of a batch of items are kept in registers until every
        //    thread has read its row (in place)
        const int rows = 32 * (nbw - kb - 1);
        for (int base = 0; base < rows * 8; base += blockDim.x) {
            const int it = base + tid;
            TF o[4] = {TF(0), TF(0), TF(0), TF(0)};
            int ib = 0, r = 0, j0 = 0;
            const bool act = it < rows * 8;
            if (act) {
                const int row = it >> 3;
                ib = kb + 1 + (row >> 5);
                r = row & 31;
                j0 = (it & 7) * 4;
                const TF* Ar = tile_at(A, ib, kb) + r * kLd;
#pragma unroll
                for (int q = 0; q < 4; ++q) o[q] = Ar[j0 + q] * dinv[32 * kb + j0 + q];
                for (int m = 0; m < j0 + 3; ++m) {
                    const TF am = Ar[m];
#pragma unroll
                    for (int q = 0; q < 4; ++q)
                        if (m < j0 + q) o[q] += am * D[m * kLd + j0 + q];
                }
            }
            __syncthreads();
            if (act) {
                TF* Ar = tile_at(A, ib, kb) + r * kLd;
#pragma unroll
                for (int q = 0; q < 4; ++q) Ar[j0 + q] = o[q];
            }
        }
        __syncthreads();
        // 3. trailing update A(ib, jb) -= L(ib, kb) L(jb, kb)^T, 2 x 2 outputs per item
        const int m = nbw - kb - 1;
        const int items = (m * (m + 1) / 2) * 256;
        for (int it = tid; it < items; it += blockDim.x) {
            const int t = it >> 8, u = it & 255;
            int ta = 0;
            while ((ta + 1) * (ta + 2) / 2 <= t) ++ta;
            const int tb = t - ta * (ta + 1) / 2;
            const int ib = kb + 1 + ta, jb = kb + 1 + tb;
            const int ur = (u >> 4) * 2, uc = (u & 15) * 2;
            if (ib == jb && uc > ur) continue;
            const TF* Li = tile_at(A, ib, kb) + ur * kLd;
            const TF* Lj = tile_at(A, jb, kb) + uc * kLd;
            TF a00 = TF(0), a01 = TF(0), a10 = TF(0), a11 = TF(0);
#pragma unroll 8
            for (int k = 0; k < 32; ++k) {
                const TF x0 = Li[k], x1 = Li[kLd + k], y0 = Lj[k], y1 = Lj[kLd + k];
                a00 += x0 * y0;
                a01 += x0 * y1;
                a10 += x1 * y0;
                a11 += x1 * y1;
            }
            TF* O = tile_at(A, ib, jb) + ur * kLd + uc;
            O[0] -= a00;
            O[1] -= a01;
            O[kLd] -= a10;
            O[kLd + 1] -= a11;
        }
        __syncthreads();
    }
    return 1;
}

// v <- (L L^T)^-1 v over the tiles with the diagonal-tile inverses, in the
// factor's precision (the mixed form's accuracy comes from the FP64
// residual of the refinement): per tile a 32-wide product by warp 0, then
// the off-diagonal update by the whole CTA (a row per thread).
template <typename TF>
__device__ void cta_chol_solve(const TF* A, const TF* dinv, int nbw, TF* v) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int kb = 0; kb < nbw; ++kb) {
        const TF* D = tile_at(const_cast<TF*>(A), kb, kb);
        if (warp == 0) {
            const TF* vb = v + 32 * kb;
            TF y = dinv[32 * kb + lane] * vb[lane];
#pragma unroll 8
            for (int j = 0; j < 32; ++j)
                if (j < lane) y += D[j * kLd + lane] * vb[j];
            __syncwarp();
            v[32 * kb + lane] = y;
        }
        __syncthreads();
        const int rows = 32 * (nbw - kb - 1);
        for (int t = tid; t < rows; t += blockDim.x) {
            const int ib = kb + 1 + (t >> 5), r = t & 31;
            const TF* Lr = tile_at(const_cast<TF*>(A), ib, kb) + r * kLd;
            TF acc0 = TF(0), acc1 = TF(0);
#pragma unroll
            for (int c = 0; c < 32; c += 2) {
                acc0 += Lr[c] * v[32 * kb + c];
                acc1 += Lr[c + 1] * v[32 * kb + c + 1];
            }
            v[32 * ib + r] -= acc0 + acc1;
        }
        __syncthreads();
    }
    for (int kb = nbw - 1; kb >= 0; --kb) {
        const TF* D = tile_at(const_cast<TF*>(A), kb, kb);
        if (warp == 0) {
            const TF* vb = v + 32 * kb;
            TF x = dinv[32 * kb + lane] * vb[lane];
#pragma unroll 8
            for (int i = 0; i < 32; ++i)
                if (i > lane) x += D[lane * kLd + i] * vb[i];
            __syncwarp();
            v[32 * kb + lane] = x;
        }
        __syncthreads();
        const int cols = 32 * kb;
        for (int t = tid; t < cols; t += blockDim.x) {
            const int jb = t >> 5, cidx = t & 31;
            const TF* Lc = tile_at(const_cast<TF*>(A), kb, jb) + cidx;
            TF acc0 = TF(0), acc1 = TF(0);
#pragma unroll
            for (int c = 0; c < 32; c += 2) {
                acc0 += Lc[c * kLd] * v[32 * kb + c];
                acc1 += Lc[(c + 1) * kLd] * v[32 * kb + c + 1];
            }
            v[32 * jb + cidx] -= acc0 + acc1;
        }
        __syncthreads();
    }
}

}  // namespace zs
