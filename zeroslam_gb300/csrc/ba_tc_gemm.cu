// FP32 products C = alpha A B^T + beta C on the 5th-generation tensor cores
// with FP32 accuracy, for the mixed form's dense preconditioner at large n:
// three TF32 products per pair of operands, A_hi B_hi + A_hi B_lo + A_lo B_hi,
// where x_hi = x rounded to TF32 (10 explicit mantissa bits) and
// x_lo = x - x_hi (exact in FP32, and seen by the tensor core to TF32 as
// well), accumulated in FP32 (the "3xTF32" split; it drops A_lo B_lo and the
// low bits of the lo parts, about 2^-21 relative per product).
//
// A (M x K) and B (N x K) are row-major with K contiguous ("K-major"), row
// strides lda, ldb multiples of 4 floats, bases 16-byte aligned. A CTA walks
// 128 x 128 tiles of C (tile blockIdx.x, then every gridDim.x-th; with a grid
// capped below the SM count the rest of the GPU stays free for other
// streams), keeping its tensor memory and its ring of stages from tile to
// tile. Per tile:
//   warp 0      TMA producer: 128 x 32 FP32 boxes of A and B per K step
//               (cp.async.bulk.tensor, 128-byte swizzle) into a 3-stage ring;
//   warps 2..5  split each landed box into hi (in place) and lo (a second
//               buffer at the same offsets: the swizzled layout is kept);
//               after the last step they read the accumulator out of tensor
//               memory (tcgen05.ld, one 32-lane quarter per warp) and write C;
//   warp 1      allocates 512 tensor-memory columns; one thread issues the
//               tcgen05.mma (kind::tf32, M = N = 128, K = 8) instructions,
//               12 per K step, and commits each stage back to the producer.
// The tensor core adds each product into its FP32 accumulator with
// truncation, so an accumulator that takes thousands of products drifts by
// ~0.5 ulp of its value per product. The leading products A_hi B_hi
// therefore go into one of two 128-column accumulators per chunk of
// kChunkKb K steps (128 values of K); after each chunk warps 2..5 add that
// accumulator into a fourth region in FP32 (rounded to nearest) while the
// next chunk goes into the other one. The small correction products go into
// their own accumulator (their drift is 2^-11 of the result's), read once.
// Tensor memory: columns [0, 128) and [128, 256) the chunk accumulators,
// [256, 384) the corrections, [384, 512) the promoted sum.
// Every wait on an mbarrier is bounded: when one runs out the kernel records
// the error (*err = 1), lets its own copies and products finish (bounded),
// frees its tensor memory and returns.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <cstdint>
#include <mutex>

#include "ba_internal.h"

namespace zs {

namespace {

constexpr int kBM = 128, kBN = 128, kBK = 32, kStages = 3;
constexpr int kTcThreads = 192;
constexpr uint32_t kBoxFloats = kBM * kBK;          // 4096 floats = 16 KB, one operand box
constexpr uint32_t kBoxBytes = kBoxFloats * 4;
constexpr long long kWaitLimit = 1ll << 24;         // polls of one mbarrier phase (well over a second)
constexpr int kChunkKb = 4;                          // K steps per promoted chunk
constexpr uint32_t kColCorr = 256, kColSum = 384, kTmemCols = 512;
constexpr uint32_t kStageFloats = 4 * 32 * 33;       // the epilogue's staging blocks
constexpr size_t kTcSmem = 4ull * kStages * kBoxBytes + 4ull * kStageFloats + 256 + 1024;  // + barriers, alignment

struct TcArgs {
    int M, N, K;
    float* C;
    int ldc;
    float alpha, beta;
    int lower;  // write only C's lower triangle (col <= row); tiles above it are skipped
    int* err;
    LmState* st;  // optional: return at once when the factorisation is skipped or has failed
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* b, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* b, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(b)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* b) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(b)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* b, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(b)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait for the phase of the given parity to complete.
__device__ bool mbar_wait(uint64_t* b, uint32_t parity, int* err) {
    for (long long i = 0; i < kWaitLimit; ++i)
        if (mbar_try_wait(b, parity)) return true;
    atomicExch(err, 1);
    return false;
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
        "[%4];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Shared-memory matrix descriptor of a K-major operand box in the 128-byte
// swizzled layout (rows of 128 bytes, 8-row atoms of 1024 bytes): start
// address, leading-byte offset 16 (unused for this layout), stride-byte offset
// 1024 (from one 8-row atom to the next), descriptor version 1, swizzle mode 2
// (128 bytes). The box base is 1024-byte aligned; a K step of 8 TF32 values is
// 32 bytes further along the row (the hardware applies the swizzle).
__device__ __forceinline__ uint64_t smem_desc(const void* p) {
    const uint32_t a = smem_u32(p);
    return (uint64_t)((a & 0x3FFFF) >> 4) | ((uint64_t)(16 >> 4) << 16) | ((uint64_t)(1024 >> 4) << 32) |
           ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}

// Instruction descriptor of tcgen05.mma kind::tf32: FP32 accumulator (bits
// 4-5 = 1), A and B TF32 (bits 7-9, 10-12 = 2), both K-major (bits 15, 16 =
// 0), N >> 3 in bits 17-22, M >> 4 in bits 24-28.
constexpr uint32_t kIdesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(kBN >> 3) << 17) |
                            ((uint32_t)(kBM >> 4) << 24);

__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(kIdesc), "r"(accumulate)
        : "memory");
}
__device__ __forceinline__ void tc_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ float tf32_round(float x) {
    uint32_t h;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h) : "f"(x));
    return __uint_as_float(h);
}

// 32 consecutive accumulator columns of this thread's row (its TMEM lane).
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float v[32]) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,"
        "%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int j = 0; j < 32; ++j) v[j] = __uint_as_float(r[j]);
}

// 32 consecutive columns of this thread's TMEM lane from registers.
__device__ __forceinline__ void tmem_st32(uint32_t taddr, const float v[32]) {
    uint32_t r[32];
#pragma unroll
    for (int j = 0; j < 32; ++j) r[j] = __float_as_uint(v[j]);
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,"
        "%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,%32};" ::"r"(taddr),
        "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]), "r"(r[8]), "r"(r[9]),
        "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]), "r"(r[15]), "r"(r[16]), "r"(r[17]), "r"(r[18]),
        "r"(r[19]), "r"(r[20]), "r"(r[21]), "r"(r[22]), "r"(r[23]), "r"(r[24]), "r"(r[25]), "r"(r[26]), "r"(r[27]),
        "r"(r[28]), "r"(r[29]), "r"(r[30]), "r"(r[31])
        : "memory");
    asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
}

// Warps 2..5: chunk ch's accumulator (columns 128 (ch & 1); ch counts the
// CTA's chunks over all its tiles) into the sum (columns [384, 512)) in FP32,
// this warp's 32 lanes, then one arrival per thread on drained[ch & 1]. A
// tile's first chunk is copied.
__device__ bool drain_chunk(int ch, bool first, uint32_t tmem, uint64_t* chunk_done, uint64_t* drained, int warp,
                            int lane, int* err) {
    const int b = ch & 1;
    if (!mbar_wait(chunk_done + b, (ch >> 1) & 1, err)) return false;
    tc_fence_after();
    const uint32_t lane_base = tmem + ((uint32_t)(32 * (warp & 3)) << 16);
#pragma unroll 1
    for (int c = 0; c < kBN / 32; ++c) {
        float v[32], acc[32];
        tmem_ld32(lane_base + 128u * b + 32 * c, v);
        if (!first) {
            tmem_ld32(lane_base + kColSum + 32 * c, acc);
#pragma unroll
            for (int j = 0; j < 32; ++j) v[j] += acc[j];
        }
        tmem_st32(lane_base + kColSum + 32 * c, v);
    }
    tc_fence_before();
    (void)lane;
    mbar_arrive(drained + b);
    return true;
}

// Tile idx of C in the launch's order (row-major over tile rows); with
// lower, only tiles on or below the diagonal (tile column <= tile row) are
// counted (C square or taller than wide).
__device__ __forceinline__ void tile_coords(int idx, int ntn, bool lower, int& ti, int& tj) {
    if (!lower) {
        ti = idx / ntn;
        tj = idx - ti * ntn;
        return;
    }
    const int tri = ntn * (ntn + 1) / 2;
    if (idx < tri) {
        ti = (int)((sqrtf(8.f * (float)idx + 1.f) - 1.f) * 0.5f);
        while ((ti + 1) * (ti + 2) / 2 <= idx) ++ti;
        while (ti * (ti + 1) / 2 > idx) --ti;
        tj = idx - ti * (ti + 1) / 2;
    } else {
        ti = ntn + (idx - tri) / ntn;
        tj = (idx - tri) % ntn;
    }
}

__device__ __forceinline__ int tile_count(int ntm, int ntn, bool lower) {
    if (!lower) return ntm * ntn;
    return ntn * (ntn + 1) / 2 + (ntm > ntn ? (ntm - ntn) * ntn : 0);
}

__global__ void __launch_bounds__(kTcThreads, 1) k_tc_gemm_nt(const __grid_constant__ CUtensorMap ta,
                                                              const __grid_constant__ CUtensorMap tb, TcArgs g) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t* base = smem_raw + ((1024 - (smem_u32(smem_raw) & 1023)) & 1023);
    float* a_hi = reinterpret_cast<float*>(base);
    float* b_hi = a_hi + kStages * kBoxFloats;
    float* a_lo = b_hi + kStages * kBoxFloats;
    float* b_lo = a_lo + kStages * kBoxFloats;
    float* stg = b_lo + kStages * kBoxFloats;  // the epilogue's staging blocks, [4][32][33]
    uint64_t* bars = reinterpret_cast<uint64_t*>(stg + kStageFloats);
    uint64_t* full = bars;                 // a stage's boxes landed (TMA bytes)
    uint64_t* conv = bars + kStages;       // a stage is split (128 arrivals)
    uint64_t* empty = bars + 2 * kStages;  // a stage's products are done (commit)
    uint64_t* done = bars + 3 * kStages;   // all products of a tile are done (commit)
    uint64_t* chunk_done = done + 1;       // [2] a chunk accumulator's products are done (commit)
    uint64_t* drained = done + 3;          // [2] a chunk accumulator was added into the sum (128 arrivals)
    uint64_t* tmem_free = done + 5;        // a tile's epilogue has read tensor memory (128 arrivals)
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(done + 6);
    volatile int* s_err = reinterpret_cast<volatile int*>(tmem_slot + 1);

    if (g.st && (__ldcg(&g.st->skip_factor) || !__ldcg(&g.st->solve_ok))) return;  // written by earlier launches
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nk = (g.K + kBK - 1) / kBK;
    const int nch = (nk + kChunkKb - 1) / kChunkKb;  // promoted chunks per tile
    const int ntm = (g.M + kBM - 1) / kBM, ntn = (g.N + kBN - 1) / kBN;
    const bool lower = g.lower != 0;
    const int ntiles = tile_count(ntm, ntn, lower);

    if (threadIdx.x == 0) {
        for (int s = 0; s < kStages; ++s) {
            mbar_init(full + s, 1);
            mbar_init(conv + s, 128);
            mbar_init(empty + s, 1);
        }
        mbar_init(done, 1);
        for (int b = 0; b < 2; ++b) {
            mbar_init(chunk_done + b, 1);
            mbar_init(drained + b, 128);
        }
        mbar_init(tmem_free, 128);
        *s_err = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    // Every role walks the CTA's tiles in the same order and counts K steps
    // (gk) and chunks (gch) over all of them, so that the ring's stages and
    // the barriers' phases continue from tile to tile.
    int issued = 0;   // producer: K steps whose boxes were requested
    int commits = 0;  // MMA issuer: tiles whose products were committed to done
    if (warp == 0) {
        if (lane == 0) {
            int gk = 0;
            for (int t = blockIdx.x; t < ntiles && !*s_err; t += gridDim.x) {
                int ti, tj;
                tile_coords(t, ntn, lower, ti, tj);
                for (int kb = 0; kb < nk; ++kb, ++gk) {
                    const int s = gk % kStages, r = gk / kStages;
                    if (gk >= kStages && !mbar_wait(empty + s, (r - 1) & 1, g.err)) {
                        *s_err = 1;
                        break;
                    }
                    if (*s_err) break;
                    mbar_expect_tx(full + s, 2 * kBoxBytes);
                    tma_load_2d(a_hi + s * kBoxFloats, &ta, kb * kBK, ti * kBM, full + s);
                    tma_load_2d(b_hi + s * kBoxFloats, &tb, kb * kBK, tj * kBN, full + s);
                    ++issued;
                }
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            int gk = 0, gch = 0;
            for (int t = blockIdx.x; t < ntiles && !*s_err; t += gridDim.x, gch += nch) {
                // the previous tile's epilogue has read the sum and the corrections
                if (commits > 0 && !mbar_wait(tmem_free, (commits - 1) & 1, g.err)) {
                    *s_err = 1;
                    break;
                }
                tc_fence_after();
                for (int kb = 0; kb < nk; ++kb, ++gk) {
                    const int s = gk % kStages, r = gk / kStages;
                    const int ch = gch + kb / kChunkKb, b = ch & 1;
                    const bool chunk_first = kb % kChunkKb == 0;
                    // a chunk accumulator is reused once the chunk before last was added into the sum
                    if (chunk_first && ch >= 2 && !mbar_wait(drained + b, ((ch >> 1) - 1) & 1, g.err)) {
                        *s_err = 1;
                        break;
                    }
                    if (!mbar_wait(conv + s, r & 1, g.err)) {
                        *s_err = 1;
                        break;
                    }
                    if (*s_err) break;
                    tc_fence_after();
                    const uint64_t ah = smem_desc(a_hi + s * kBoxFloats), al = smem_desc(a_lo + s * kBoxFloats);
                    const uint64_t bh = smem_desc(b_hi + s * kBoxFloats), bl = smem_desc(b_lo + s * kBoxFloats);
                    const uint32_t acc_main = tmem + 128u * b, acc_corr = tmem + kColCorr;
#pragma unroll
                    for (int ks = 0; ks < kBK / 8; ++ks) {
                        const uint64_t o = (uint64_t)(ks * 32) >> 4;  // 8 TF32 values = 32 bytes along the row
                        tc_mma(acc_main, ah + o, bh + o, !(chunk_first && ks == 0));
                        tc_mma(acc_corr, ah + o, bl + o, (kb | ks) != 0);
                        tc_mma(acc_corr, al + o, bh + o, 1);
                    }
                    tc_commit(empty + s);
                    if (kb % kChunkKb == kChunkKb - 1 || kb == nk - 1) tc_commit(chunk_done + b);
                }
                if (*s_err) break;
                tc_commit(done);  // arrives once every product issued so far has completed
                ++commits;
            }
            if (*s_err) {
                // let every product issued so far finish before the memory is freed
                tc_commit(done);
                mbar_wait(done, commits & 1, g.err);
            }
        }
    } else {
        // warps 2..5: split the landed boxes, promote the chunks, then the epilogue
        const int ct = threadIdx.x - 64;
        const int q = warp & 3;  // this warp's 32-lane quarter of tensor memory
        const uint32_t lane_base = tmem + ((uint32_t)(32 * q) << 16);
        float* st = stg + q * 32 * 33;
        int gk = 0, gch = 0, tiles = 0;
        for (int t = blockIdx.x; t < ntiles && !*s_err; t += gridDim.x, gch += nch, ++tiles) {
            int ti, tj;
            tile_coords(t, ntn, lower, ti, tj);
            const int row0 = ti * kBM, col0 = tj * kBN;
            for (int kb = 0; kb < nk; ++kb, ++gk) {
                const int s = gk % kStages, r = gk / kStages;
                if (!mbar_wait(full + s, r & 1, g.err)) {
                    *s_err = 1;
                    break;
                }
                float4* ah4 = reinterpret_cast<float4*>(a_hi + s * kBoxFloats);
                float4* al4 = reinterpret_cast<float4*>(a_lo + s * kBoxFloats);
                float4* bh4 = reinterpret_cast<float4*>(b_hi + s * kBoxFloats);
                float4* bl4 = reinterpret_cast<float4*>(b_lo + s * kBoxFloats);
#pragma unroll
                for (int i = 0; i < (int)(kBoxFloats / 4) / 128; ++i) {
                    const int e = ct + 128 * i;
                    float4 v = ah4[e], h;
                    h.x = tf32_round(v.x); h.y = tf32_round(v.y); h.z = tf32_round(v.z); h.w = tf32_round(v.w);
                    ah4[e] = h;
                    al4[e] = make_float4(v.x - h.x, v.y - h.y, v.z - h.z, v.w - h.w);
                    v = bh4[e];
                    h.x = tf32_round(v.x); h.y = tf32_round(v.y); h.z = tf32_round(v.z); h.w = tf32_round(v.w);
                    bh4[e] = h;
                    bl4[e] = make_float4(v.x - h.x, v.y - h.y, v.z - h.z, v.w - h.w);
                }
                // the products read shared memory through the async proxy
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                mbar_arrive(conv + s);
                // after the last step of chunk c, the previous chunk's accumulator
                // (its products were issued a chunk earlier) goes into the sum
                const int c = kb / kChunkKb;
                if ((kb % kChunkKb == kChunkKb - 1 || kb == nk - 1) && c >= 1 &&
                    !drain_chunk(gch + c - 1, c == 1, tmem, chunk_done, drained, warp, lane, g.err)) {
                    *s_err = 1;
                    break;
                }
            }
            if (*s_err) break;
            if (!drain_chunk(gch + nch - 1, nch == 1, tmem, chunk_done, drained, warp, lane, g.err) ||
                !mbar_wait(done, tiles & 1, g.err)) {
                *s_err = 1;
                break;
            }
            tc_fence_after();
            // Every product of this tile has completed (the next tile's boxes
            // may already be landing in the ring): each warp stages its
            // 32 x 32 blocks in its own staging block (33-float rows,
            // conflict-free both ways) and writes C a row at a time, 32
            // consecutive columns per warp instruction.
#pragma unroll 1
            for (int cc = 0; cc < kBN / 32; ++cc) {
                float v[32], w[32];
                tmem_ld32(lane_base + kColSum + 32 * cc, v);
                tmem_ld32(lane_base + kColCorr + 32 * cc, w);
#pragma unroll
                for (int j = 0; j < 32; ++j) st[lane * 33 + j] = v[j] + w[j];
                __syncwarp();
                const int col = col0 + 32 * cc + lane;
                // the 32 old values first, all loads in flight together
                float old[32];
#pragma unroll
                for (int rr = 0; rr < 32; ++rr) {
                    const int row = row0 + 32 * q + rr;
                    old[rr] = (g.beta != 0.f && row < g.M && col < g.N && (!g.lower || col <= row))
                                  ? __ldcg(g.C + (int64_t)row * g.ldc + col)
                                  : 0.f;
                }
#pragma unroll
                for (int rr = 0; rr < 32; ++rr) {
                    const int row = row0 + 32 * q + rr;
                    if (row < g.M && col < g.N && (!g.lower || col <= row))
                        g.C[(int64_t)row * g.ldc + col] = g.alpha * st[rr * 33 + lane] + g.beta * old[rr];
                }
                __syncwarp();
            }
            tc_fence_before();
            mbar_arrive(tmem_free);
        }
    }
    // teardown: copies still in flight land before the CTA leaves; products
    // finish before their tensor memory is freed
    if (warp == 0 && lane == 0 && *s_err) {
        for (int k = (issued > kStages ? issued - kStages : 0); k < issued; ++k)
            mbar_wait(full + k % kStages, (k / kStages) & 1, g.err);
    }
    if (threadIdx.x == 0 && *s_err && g.st) g.st->solve_ok = 0;
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
    }
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
        cudaGetLastError();
    });
    return fn;
}

// A rows x cols row-major FP32 matrix (row stride ld floats) as 32 x 128
// boxes with the 128-byte swizzle; reads outside it return zeros.
bool make_map(CUtensorMap* m, const float* base, int rows, int cols, int ld) {
    PFN_cuTensorMapEncodeTiled_v12000 enc = encode_fn();
    if (!enc) return false;
    cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)ld * 4};
    cuuint32_t box[2] = {(cuuint32_t)kBK, (cuuint32_t)kBM};
    cuuint32_t estr[2] = {1, 1};
    return enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(base), dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace

bool tc_gemm_supported(int lda, int ldb, const float* A, const float* B) {
    return lda % 4 == 0 && ldb % 4 == 0 && (reinterpret_cast<uintptr_t>(A) & 15) == 0 &&
           (reinterpret_cast<uintptr_t>(B) & 15) == 0 && encode_fn() != nullptr;
}

cudaError_t launch_tc_gemm_nt(int M, int N, int K, const float* A, int lda, const float* B, int ldb, float* C, int ldc,
                              float alpha, float beta, bool lower, int* err, cudaStream_t s, LmState* st,
                              int max_ctas) {
    if (M <= 0 || N <= 0) return cudaSuccess;
    if (K <= 0 || !tc_gemm_supported(lda, ldb, A, B)) return cudaErrorInvalidValue;
    CUtensorMap ta, tb;
    if (!make_map(&ta, A, M, K, lda) || !make_map(&tb, B, N, K, ldb)) return cudaErrorInvalidValue;
    static std::atomic<int> attr_set[kMaxDevices];
    if (per_device(attr_set, [] {
            return cudaFuncSetAttribute(k_tc_gemm_nt, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTcSmem) ==
                           cudaSuccess
                       ? 1
                       : 0;
        }) < 1)
        return cudaGetLastError() != cudaSuccess ? cudaErrorInvalidValue : cudaErrorInvalidConfiguration;
    TcArgs g{M, N, K, C, ldc, alpha, beta, lower ? 1 : 0, err, st};
    const int ntm = (M + kBM - 1) / kBM, ntn = (N + kBN - 1) / kBN;
    if (lower && M < N) return cudaErrorInvalidValue;  // lower: C square or taller than wide
    int tiles = lower ? ntn * (ntn + 1) / 2 + (ntm - ntn) * ntn : ntm * ntn;
    if (max_ctas > 0 && tiles > max_ctas) tiles = max_ctas;
    k_tc_gemm_nt<<<tiles, kTcThreads, kTcSmem, s>>>(ta, tb, g);
    note_launch();
    return cudaGetLastError();
}

}  // namespace zs

// ---- C ABI: the product on host arrays (tests and measurements) ----
#include <vector>

#include "../../include/zeroslam_ba.h"

extern "C" int zs_dense_gemm_nt_tf32x3(const float* A, const float* B, float* C, int M, int N, int K, int lower,
                                       int max_ctas, double* ms) {
    using namespace zs;
    if (!A || !B || !C || M <= 0 || N <= 0 || K <= 0 || max_ctas < 0 || (lower && M < N)) return ZS_ERR_INVALID;
    const int ld = (K + 3) & ~3;  // device rows padded to 16 bytes
    float *dA = nullptr, *dB = nullptr, *dC = nullptr;
    int* derr = nullptr;
    cudaStream_t s = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int status = ZS_OK;
    auto fail = [&](cudaError_t e) { status = record_cuda_error(e); };
    cudaError_t e;
    if ((e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking)) != cudaSuccess) { fail(e); return status; }
    if ((e = cudaMalloc(&dA, 4ull * M * ld)) != cudaSuccess || (e = cudaMalloc(&dB, 4ull * N * ld)) != cudaSuccess ||
        (e = cudaMalloc(&dC, 4ull * M * N)) != cudaSuccess || (e = cudaMalloc(&derr, sizeof(int))) != cudaSuccess ||
        (e = cudaEventCreate(&e0)) != cudaSuccess || (e = cudaEventCreate(&e1)) != cudaSuccess) {
        fail(e);
    } else if ((e = cudaMemcpy2DAsync(dA, 4ull * ld, A, 4ull * K, 4ull * K, M, cudaMemcpyHostToDevice, s)) !=
                   cudaSuccess ||
               (e = cudaMemcpy2DAsync(dB, 4ull * ld, B, 4ull * K, 4ull * K, N, cudaMemcpyHostToDevice, s)) !=
                   cudaSuccess ||
               (e = cudaMemcpyAsync(dC, C, 4ull * M * N, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
               (e = cudaMemsetAsync(derr, 0, sizeof(int), s)) != cudaSuccess ||
               (e = cudaEventRecord(e0, s)) != cudaSuccess ||
               (e = launch_tc_gemm_nt(M, N, K, dA, ld, dB, ld, dC, N, 1.f, 0.f, lower != 0, derr, s, nullptr,
                                      max_ctas)) != cudaSuccess ||
               (e = cudaEventRecord(e1, s)) != cudaSuccess ||
               (e = cudaMemcpyAsync(C, dC, 4ull * M * N, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
               (e = cudaStreamSynchronize(s)) != cudaSuccess) {
        fail(e);
    } else {
        int herr = 0;
        float t = 0.f;
        if ((e = cudaMemcpy(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost)) != cudaSuccess ||
            (e = cudaEventElapsedTime(&t, e0, e1)) != cudaSuccess)
            fail(e);
        else if (herr)
            status = ZS_ERR_TIMEOUT;
        if (ms) *ms = t;
    }
    cudaFree(dA);
    cudaFree(dB);
    cudaFree(dC);
    cudaFree(derr);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaStreamDestroy(s);
    return status;
}
