// Brute-force binary descriptor matching on the device: zeroslam's
// feature::find_matches with distance<256> (source/feature.hpp:1133-1235).
//
// For every lhs descriptor the reference keeps the k smallest Hamming
// distances to the rhs descriptors below a threshold, scanning rhs in order
// and replacing only on a strict improvement, so equal distances keep the
// earlier rhs. That is the k smallest keys (distance << 32 | rhs index), which
// is what is computed here, in two launches:
//   k_match_partial: a block holds 256 lhs descriptors (two per thread, in
//     registers) and scans one chunk of the rhs through shared memory in
//     tiles of 256 descriptors (every thread reads the same descriptor: a
//     broadcast); XOR, a carry-save popcount of the 8 words, and an
//     insertion into the thread's k sorted keys. The rhs is split into chunks (gridDim.y) so that
//     a few thousand lhs descriptors still fill every SM.
//   k_match_merge: per lhs, the k smallest keys over the chunks' lists.
// The host then lays out the matches as the reference does: lhs in order,
// each with its keys below the threshold, stopping at the first lhs for
// which count + k would exceed the output size. Integer work throughout:
// the results are the reference's exactly.
#include "ba_internal.h"

namespace zs {

namespace {

constexpr int kMatchLhs = 128;   // threads per block
constexpr int kMatchPerBlock = 2 * kMatchLhs;  // lhs descriptors per block (two per thread)
constexpr int kMatchTile = 256;  // rhs descriptors per shared-memory tile
constexpr unsigned long long kNoKey = ~0ull;

// best: K keys, ascending. Keeps the K smallest of best and key, ascending
// (a min/max pass with static indices, so best stays in registers).
template <int K>
__device__ __forceinline__ void insert_key(unsigned long long (&best)[K], unsigned long long key) {
    if (key >= best[K - 1]) return;
#pragma unroll
    for (int s = 0; s < K; ++s) {
        const unsigned long long lo = min(best[s], key);
        key = max(best[s], key);
        best[s] = lo;
    }
}

// Carry-save adder: l = a ^ b ^ c (sum bits), h = majority(a, b, c) (carry
// bits), one three-input logic operation each.
__device__ __forceinline__ void csa(unsigned& h, unsigned& l, unsigned a, unsigned b, unsigned c) {
    const unsigned u = a ^ b;
    h = (a & b) | (u & c);
    l = u ^ c;
}

// Popcount of eight words with four popcounts: the words are added bit-wise
// in carry-save form into ones, twos, fours and eights (Harley and Seal's
// method, as described in W. Mula, N. Kurz and D. Lemire, "Faster population
// counts using AVX2 instructions", The Computer Journal 61 (2018)); the
// logic operations run on the ALU pipe, the popcounts on the narrower one.
__device__ __forceinline__ int popc8(unsigned x0, unsigned x1, unsigned x2, unsigned x3, unsigned x4, unsigned x5,
                                     unsigned x6, unsigned x7) {
    unsigned ta, oa, tb, ob, tc, oc, o, td, t1, fa, t, fb, f, e;
    csa(ta, oa, x0, x1, x2);
    csa(tb, ob, x3, x4, x5);
    oc = x6 ^ x7;
    tc = x6 & x7;
    csa(td, o, oa, ob, oc);
    csa(fa, t1, ta, tb, tc);
    t = t1 ^ td;
    fb = t1 & td;
    f = fa ^ fb;
    e = fa & fb;
    return __popc(o) + 2 * __popc(t) + 4 * __popc(f) + 8 * __popc(e);
}

// part: [gridDim.y][n_lhs][K] keys, kNoKey where fewer than K were found.
// Each thread holds two lhs descriptors (rows i and i + kMatchLhs of the
// block's 2 kMatchLhs), so every shared-memory read of an rhs descriptor
// serves two distances.
template <int K>
__global__ void __launch_bounds__(kMatchLhs) k_match_partial(const uint4* __restrict__ lhs, int n_lhs,
                                                             const uint4* __restrict__ rhs, int n_rhs, int chunk,
                                                             int d_lim, unsigned long long* __restrict__ part) {
    __shared__ uint4 s_rhs[2 * kMatchTile];
    const int i0 = blockIdx.x * kMatchPerBlock + threadIdx.x;
    const int i1 = i0 + kMatchLhs;
    uint4 a0 = make_uint4(0, 0, 0, 0), a1 = a0, c0 = a0, c1 = a0;
    if (i0 < n_lhs) {
        a0 = lhs[2 * (int64_t)i0];
        a1 = lhs[2 * (int64_t)i0 + 1];
    }
    if (i1 < n_lhs) {
        c0 = lhs[2 * (int64_t)i1];
        c1 = lhs[2 * (int64_t)i1 + 1];
    }
    unsigned long long best[K], best1[K];
#pragma unroll
    for (int k = 0; k < K; ++k) best[k] = best1[k] = kNoKey;
    const int j0 = blockIdx.y * chunk;
    const int j1 = min(n_rhs, j0 + chunk);
    for (int t0 = j0; t0 < j1; t0 += kMatchTile) {
        const int cnt = min(kMatchTile, j1 - t0);
        __syncthreads();
        for (int q = threadIdx.x; q < 2 * cnt; q += kMatchLhs) s_rhs[q] = rhs[2 * (int64_t)t0 + q];
        __syncthreads();
        for (int r = 0; r < cnt; ++r) {
            const uint4 b0 = s_rhs[2 * r], b1 = s_rhs[2 * r + 1];
            const int d = popc8(a0.x ^ b0.x, a0.y ^ b0.y, a0.z ^ b0.z, a0.w ^ b0.w, a1.x ^ b1.x, a1.y ^ b1.y,
                                a1.z ^ b1.z, a1.w ^ b1.w);
            const int e = popc8(c0.x ^ b0.x, c0.y ^ b0.y, c0.z ^ b0.z, c0.w ^ b0.w, c1.x ^ b1.x, c1.y ^ b1.y,
                                c1.z ^ b1.z, c1.w ^ b1.w);
            const unsigned j = (unsigned int)(t0 + r);
            if (d < d_lim) insert_key<K>(best, ((unsigned long long)d << 32) | j);
            if (e < d_lim) insert_key<K>(best1, ((unsigned long long)e << 32) | j);
        }
    }
    if (i0 < n_lhs) {
        unsigned long long* o = part + ((int64_t)blockIdx.y * n_lhs + i0) * K;
#pragma unroll
        for (int k = 0; k < K; ++k) o[k] = best[k];
    }
    if (i1 < n_lhs) {
        unsigned long long* o = part + ((int64_t)blockIdx.y * n_lhs + i1) * K;
#pragma unroll
        for (int k = 0; k < K; ++k) o[k] = best1[k];
    }
}

template <int K>
__global__ void k_match_merge(int n_lhs, int chunks, const unsigned long long* __restrict__ part,
                              unsigned long long* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_lhs) return;
    unsigned long long best[K];
#pragma unroll
    for (int k = 0; k < K; ++k) best[k] = kNoKey;
    for (int c = 0; c < chunks; ++c) {
        const unsigned long long* p = part + ((int64_t)c * n_lhs + i) * K;
#pragma unroll
        for (int k = 0; k < K; ++k) {
            const unsigned long long key = p[k];
            if (key == kNoKey) break;
            insert_key<K>(best, key);
        }
    }
#pragma unroll
    for (int k = 0; k < K; ++k) out[(int64_t)i * K + k] = best[k];
}

template <int K>
void launch_match_k(const uint8_t* lhs, int n_lhs, const uint8_t* rhs, int n_rhs, int d_lim, int chunks,
                    unsigned long long* part, unsigned long long* out, cudaStream_t s) {
    const int chunk = (n_rhs + chunks - 1) / chunks;
    const dim3 grid((n_lhs + kMatchPerBlock - 1) / kMatchPerBlock, chunks);
    unsigned long long* dst = chunks == 1 ? out : part;
    k_match_partial<K><<<grid, kMatchLhs, 0, s>>>(reinterpret_cast<const uint4*>(lhs), n_lhs,
                                                  reinterpret_cast<const uint4*>(rhs), n_rhs, chunk, d_lim, dst);
    note_launch();
    if (chunks > 1) {
        k_match_merge<K><<<grid_for(n_lhs, 128), 128, 0, s>>>(n_lhs, chunks, part, out);
        note_launch();
    }
}

}  // namespace

int match_chunks(int n_lhs, int n_rhs) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 152;
    const int lhs_blocks = (n_lhs + kMatchPerBlock - 1) / kMatchPerBlock;
    const int want = (8 * sms + lhs_blocks - 1) / std::max(lhs_blocks, 1);  // ~8 blocks of 128 threads per SM
    const int most = std::max(1, (n_rhs + 63) / 64);                         // at least 64 rhs per chunk
    return std::max(1, std::min(want, most));
}

void launch_match(const uint8_t* lhs, int n_lhs, const uint8_t* rhs, int n_rhs, int k, int d_lim, int chunks,
                  unsigned long long* part, unsigned long long* out, cudaStream_t s) {
    if (n_lhs <= 0) return;
    switch (k) {
        case 1: launch_match_k<1>(lhs, n_lhs, rhs, n_rhs, d_lim, chunks, part, out, s); break;
        case 2: launch_match_k<2>(lhs, n_lhs, rhs, n_rhs, d_lim, chunks, part, out, s); break;
        case 3: launch_match_k<3>(lhs, n_lhs, rhs, n_rhs, d_lim, chunks, part, out, s); break;
        case 4: launch_match_k<4>(lhs, n_lhs, rhs, n_rhs, d_lim, chunks, part, out, s); break;
        case 5: launch_match_k<5>(lhs, n_lhs, rhs, n_rhs, d_lim, chunks, part, out, s); break;
        case 6: launch_match_k<6>(lhs, n_lhs, rhs, n_rhs, d_lim, chunks, part, out, s); break;
        case 7: launch_match_k<7>(lhs, n_lhs, rhs, n_rhs, d_lim, chunks, part, out, s); break;
        default: launch_match_k<8>(lhs, n_lhs, rhs, n_rhs, d_lim, chunks, part, out, s); break;
    }
}

}  // namespace zs
