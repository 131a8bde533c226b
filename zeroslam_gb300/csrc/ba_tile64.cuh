// 64 x 64 FP32 tiles in shared memory for the mixed form's dense
// factorisation and inverse: rows of kPL floats (16-byte aligned, so that
// 128-bit reads of eight consecutive rows hit distinct bank groups), a
// register-tiled product of two row-major tiles (each thread of a 16 x 16
// grid owns a 4 x 4 block of the output), and 16-byte asynchronous
// global -> shared copies.
#pragma once

#include <stdint.h>

namespace zs {
namespace t64 {

constexpr int kP = 64;          // tile edge
constexpr int kPL = kP + 4;     // shared-memory row of a tile
constexpr int kThreads = 256;   // threads of a CTA working on a tile
constexpr int kTileFloats = kP * kPL;

__device__ __forceinline__ float ldcg(const float* p) { return __ldcg(p); }

// acc[i][j] += sum_m A[ty + 16 i][m] B[tx + 16 j][m] over m < kk rounded up
// to 4 (operands zero beyond kk). Thread (ty, tx) = (tid / 16, tid % 16).
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

__device__ __forceinline__ void zero_acc(float acc[4][4]) {
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = 0.f;
}

__device__ __forceinline__ void tile_nt(const float* A, const float* B, int kk, float acc[4][4]) {
    zero_acc(acc);
    tile_nt_acc(A, B, kk, acc);
}

// 16-byte asynchronous global -> shared copy; src_bytes < 16 zero-fills the rest.
__device__ __forceinline__ void cp_async16(float* dst, const float* src, int src_bytes) {
    const unsigned d = static_cast<unsigned>(__cvta_generic_to_shared(dst));
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(d), "l"(src), "r"(src_bytes) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_one() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_none() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() {
    asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;\n" ::: "memory");
}

// Rows r0 .. r0 + 64 (clipped to n), columns c0 .. c0 + kk of the row-major
// matrix M (row stride ld) into S[row][m] (zero outside). With ld % 4 == 0
// (16-byte rows), c0 % 4 == 0 and M 16-byte aligned: 16-byte asynchronous
// copies, four per thread, all in flight together; the caller commits / waits
// and synchronises before reading S. Otherwise plain L2 loads, complete on
// return (after the caller's barrier).
__device__ __forceinline__ void load_block(const float* M, int n, int ld, int r0, int c0, int kk, float* S) {
    if ((ld & 3) == 0) {
#pragma unroll
        for (int q = 0; q < (kP * kP / 4) / kThreads; ++q) {
            const int e = threadIdx.x + q * kThreads;
            const int r = e >> 4, c4 = (e & 15) * 4;
            const int row = r0 + r;
            int bytes = (row < n) ? 4 * min(4, kk - c4) : 0;
            if (bytes < 0) bytes = 0;
            const float* src = bytes > 0 ? M + (int64_t)row * ld + c0 + c4 : M;
            cp_async16(S + r * kPL + c4, src, bytes);
        }
    } else {
        float v[(kP * kP) / kThreads];
#pragma unroll
        for (int q = 0; q < (kP * kP) / kThreads; ++q) {
            const int e = threadIdx.x + q * kThreads;
            const int r = e >> 6, m = e & 63;
            v[q] = (r0 + r < n && m < kk) ? ldcg(M + (int64_t)(r0 + r) * ld + c0 + m) : 0.f;
        }
#pragma unroll
        for (int q = 0; q < (kP * kP) / kThreads; ++q) {
            const int e = threadIdx.x + q * kThreads;
            S[(e >> 6) * kPL + (e & 63)] = v[q];
        }
    }
}

// The square case: an n x n matrix with row stride n.
__device__ __forceinline__ void load_block(const float* M, int n, int r0, int c0, int kk, float* S) {
    load_block(M, n, n, r0, c0, kk, S);
}

}  // namespace t64
}  // namespace zs
