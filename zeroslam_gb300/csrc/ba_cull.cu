// Map culling on the device: zeroslam's map::cull (source/map.hpp:269-323).
//
// For every landmark the reference decides, in this order:
//   * landmarks older than the newest 500 ids (id + 500 < the landmark id
//     generator) are kept without a look (map.hpp:272-275);
//   * a landmark without observations is erased (277-280);
//   * a landmark seen 4 times or fewer whose last observation is older than
//     the newest 7 frames is erased (281-287);
//   * otherwise the float mean, over its observations whose frame is in the
//     map, of the pixel distance between the keypoint and the landmark
//     projected by that frame (5.991 where camera::pinhole::project fails,
//     camera.hpp:91-111), is compared with 5.991: erased at or above it, or
//     when no observation had its frame (288-318).
//
// k_cull computes the error terms one thread per observation and sums each
// landmark's terms, in its observation order, in one thread (the float mean
// is a sequential float sum); frames (96 B each) and intrinsics stay in L1 /
// L2. The terms are FP64 with the reference's rounding order and no
// contraction (the _rn intrinsics), so the means, and with them the
// decisions, are the reference's bit for bit. The kernel is bound by the
// FP64 pipe (a division and a square root per observation), not by memory.
//
// k_pose_rt gives the frames of the solver's resident poses: the rotation
// matrix and translation that map::optimise writes back into each frame
// (map.hpp:247-251, lie.hpp:188-204), so that a cull after a resident solve
// sees what the reference's cull sees after optimise.
#include "ba_internal.h"

namespace zs {

namespace {

constexpr int kCullAge = 500;           // source/map.hpp:272
constexpr int kCullFewObs = 4;          // source/map.hpp:281
constexpr int kCullRecent = 7;          // source/map.hpp:282
constexpr float kCullError = 5.991f;    // source/map.hpp:304,316
constexpr double kMinDepth = 1.0e-12;   // source/camera.hpp:98

// One observation's term: the landmark mapped into the frame, R X + t with
// the row sums of source/matrix.hpp:494-509 (starting from 0), projected as
// camera.hpp:97-111, and the distance of matrix.hpp:177-183 rounded to float.
__device__ __forceinline__ float cull_term(const double* __restrict__ Rt, const double* __restrict__ in,
                                           double X0, double X1, double X2, double kx, double ky) {
    double m[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        double s = 0.0;
        s = __dadd_rn(s, __dmul_rn(__ldg(Rt + 3 * i + 0), X0));
        s = __dadd_rn(s, __dmul_rn(__ldg(Rt + 3 * i + 1), X1));
        s = __dadd_rn(s, __dmul_rn(__ldg(Rt + 3 * i + 2), X2));
        m[i] = __dadd_rn(s, __ldg(Rt + 9 + i));
    }
    if (m[2] < kMinDepth) return kCullError;
    const double iz = __ddiv_rn(1.0, m[2]);
    const double px = __dadd_rn(__dmul_rn(__ldg(in + 0), __dmul_rn(m[0], iz)), __ldg(in + 2));
    const double py = __dadd_rn(__dmul_rn(__ldg(in + 1), __dmul_rn(m[1], iz)), __ldg(in + 3));
    const double dx = __dsub_rn(kx, px);
    const double dy = __dsub_rn(ky, py);
    double ls = 0.0;
    ls = __dadd_rn(ls, __dmul_rn(dx, dx));
    ls = __dadd_rn(ls, __dmul_rn(dy, dy));
    return __double2float_rn(__dsqrt_rn(ls));
}

__device__ __forceinline__ double kp_x(const float2& k) { return (double)k.x; }
__device__ __forceinline__ double kp_y(const float2& k) { return (double)k.y; }
__device__ __forceinline__ double kp_x(const double2& k) { return k.x; }
__device__ __forceinline__ double kp_y(const double2& k) { return k.y; }

constexpr int kCullLm = 128;     // landmarks, and threads, per block
constexpr int kCullTile = 1024;  // observations per shared-memory tile
constexpr float kNoTerm = -1.0f; // tile entry of an observation without a term (a term is >= 0 or NaN)

// A block takes kCullLm consecutive landmarks. Thread t decides the
// reference's early rules for landmark t; then the block walks the
// landmarks' observations (one contiguous stretch) in tiles: every thread
// computes the error terms of tile entries t, t + kCullLm, ... (the landmark
// of an entry by binary search over the block's ranges) into shared memory,
// and thread t adds its landmark's entries of the tile, in order, to its
// float sum, which carries over to the next tile. The FP64 terms thus run
// one per thread over all observations, evenly spread, while each float sum
// keeps the reference's sequential order.
// counters: [0] erased, [1] error passes run, [2] invalid input seen.
template <typename RangeT, typename KpT>
__global__ void __launch_bounds__(kCullLm) k_cull(CullArgs a, const RangeT* __restrict__ obs_ptr,
                                                  const KpT* __restrict__ kp) {
    __shared__ int64_t s_ptr[kCullLm + 1];
    __shared__ double s_X[3 * kCullLm];
    __shared__ unsigned char s_pass[kCullLm];
    __shared__ float s_term[kCullTile];
    const int t = threadIdx.x;
    unsigned long long erased = 0, passes = 0;
    unsigned int bad = 0;
    for (int base = blockIdx.x * kCullLm; base < a.L; base += gridDim.x * kCullLm) {
        const int n = min(kCullLm, a.L - base);
        const int l = base + t;
        int e = 0, pass = 0;
        int64_t o0 = 0, o1 = 0;
        int mine_bad = 0;
        if (t < n) {
            o0 = obs_ptr[l];
            o1 = obs_ptr[l + 1];
            mine_bad = o0 < 0 || o1 < o0 || o1 > a.M;
            if (!mine_bad && a.lm_id[l] + kCullAge >= a.lm_gen) {
                if (o1 == o0) {
                    e = 1;
                } else {
                    const int last = a.obs_frame[o1 - 1];
                    const int last_id = a.obs_frame_id ? a.obs_frame_id[o1 - 1]
                                                       : (last >= 0 && last < a.F ? a.frame_id[last] : 0);
                    if (o1 - o0 <= kCullFewObs && last_id + kCullRecent < a.frame_gen) e = 1;
                    else pass = 1;
                }
            }
            s_ptr[t] = o0;
            if (t == n - 1) s_ptr[n] = o1;
            s_pass[t] = (unsigned char)pass;
            if (pass) {
                const double* X = a.lm + (int64_t)l * a.lm_stride;
                s_X[3 * t + 0] = X[0];
                s_X[3 * t + 1] = X[1];
                s_X[3 * t + 2] = X[2];
            }
        }
        if (__syncthreads_or(mine_bad)) {  // ranges not monotone: nothing of this block is read
            bad = 1;
            if (t < n) {
                a.erase[l] = 0;
                a.mean[l] = -1.0f;
            }
            __syncthreads();
            continue;
        }
        const int64_t O0 = s_ptr[0], O1 = s_ptr[n];
        float err = 0.0f;
        int processed = 0;
        for (int64_t ts = O0; ts < O1; ts += kCullTile) {
            const int cnt = (int)min((int64_t)kCullTile, O1 - ts);
            for (int i = t; i < cnt; i += kCullLm) {
                const int64_t o = ts + i;
                int lo = 0, hi = n - 1;  // the last landmark whose range starts at or before o
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if (s_ptr[mid] <= o) lo = mid;
                    else hi = mid - 1;
                }
                float term = kNoTerm;
                if (s_pass[lo]) {
                    const int f = a.obs_frame[o];
                    if (f >= a.F) {
                        bad = 1;
                    } else if (f >= 0) {
                        const KpT k = kp[o];
                        term = cull_term(a.Rt + 12 * (int64_t)f, a.intr + (int64_t)f * a.intr_stride, s_X[3 * lo],
                                         s_X[3 * lo + 1], s_X[3 * lo + 2], kp_x(k), kp_y(k));
                    }
                }
                s_term[i] = term;
            }
            __syncthreads();
            if (pass) {
                const int64_t b0 = max(o0, ts), b1 = min(o1, ts + cnt);
                for (int64_t o = b0; o < b1; ++o) {
                    const float v = s_term[o - ts];
                    if (v != kNoTerm) {
                        err = __fadd_rn(err, v);
                        ++processed;
                    }
                }
            }
            __syncthreads();
        }
        if (t < n) {
            float mean = -1.0f;
            if (pass) {
                if (processed == 0) {
                    e = 1;
                } else {
                    mean = __fdiv_rn(err, __int2float_rn(processed));
                    e = mean >= kCullError;
                    ++passes;
                }
            }
            a.erase[l] = (uint8_t)e;
            a.mean[l] = mean;
            erased += e;
        }
        __syncthreads();
    }
    // integer counters: the totals do not depend on the order of the atomics
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
        erased += __shfl_xor_sync(0xffffffffu, erased, d);
        passes += __shfl_xor_sync(0xffffffffu, passes, d);
        bad |= __shfl_xor_sync(0xffffffffu, bad, d);
    }
    if ((t & 31) == 0) {
        if (erased) atomicAdd(a.counters + 0, erased);
        if (passes) atomicAdd(a.counters + 1, passes);
        if (bad) atomicOr(reinterpret_cast<unsigned int*>(a.counters + 2), bad);
    }
}

__global__ void k_pose_rt(int K, const double* __restrict__ pose, double* __restrict__ Rt) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= K) return;
    const double* p = pose + (int64_t)k * kPoseStride;
    const double w = p[6], x = p[3], y = p[4], z = p[5];
    // lie.hpp:188-204, term for term
    const double tx = __dmul_rn(2.0, x), ty = __dmul_rn(2.0, y), tz = __dmul_rn(2.0, z);
    const double txx = __dmul_rn(tx, x), txy = __dmul_rn(tx, y), txz = __dmul_rn(tx, z), txw = __dmul_rn(tx, w);
    const double tyy = __dmul_rn(ty, y), tyz = __dmul_rn(ty, z), tyw = __dmul_rn(ty, w);
    const double tzz = __dmul_rn(tz, z), tzw = __dmul_rn(tz, w);
    double* o = Rt + 12 * (int64_t)k;
    o[0] = __dsub_rn(1.0, __dadd_rn(tyy, tzz));
    o[1] = __dsub_rn(txy, tzw);
    o[2] = __dadd_rn(txz, tyw);
    o[3] = __dadd_rn(txy, tzw);
    o[4] = __dsub_rn(1.0, __dadd_rn(txx, tzz));
    o[5] = __dsub_rn(tyz, txw);
    o[6] = __dsub_rn(txz, tyw);
    o[7] = __dadd_rn(tyz, txw);
    o[8] = __dsub_rn(1.0, __dadd_rn(txx, tyy));
    o[9] = p[0];
    o[10] = p[1];
    o[11] = p[2];
}

int cull_grid(int L) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int g = grid_for(L, kCullLm);
    const int cap = (sms > 0 ? sms : 152) * 16;
    return g < cap ? g : cap;
}

}  // namespace

void launch_pose_rt(int K, const double* pose, double* Rt, cudaStream_t s) {
    if (K <= 0) return;
    k_pose_rt<<<grid_for(K, 128), 128, 0, s>>>(K, pose, Rt);
    note_launch();
}

void launch_cull(const CullArgs& a, const int64_t* obs_ptr, const float2* kp, cudaStream_t s) {
    if (a.L <= 0) return;
    k_cull<int64_t, float2><<<cull_grid(a.L), kCullLm, 0, s>>>(a, obs_ptr, kp);
    note_launch();
}

void launch_cull(const CullArgs& a, const int32_t* obs_ptr, const double2* kp, cudaStream_t s) {
    if (a.L <= 0) return;
    k_cull<int32_t, double2><<<cull_grid(a.L), kCullLm, 0, s>>>(a, obs_ptr, kp);
    note_launch();
}

}  // namespace zs
