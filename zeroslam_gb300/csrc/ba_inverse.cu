// Mixed-precision reduced solves with the preconditioner X = L^-1 of the
// FP32 factor S ~ L L^T (formed with the factor by k_chol_inverse_dag,
// ba_chol_dag.cu; X^T is stored beside X so that both products are row-wise):
// 1. k_pcg (bundle adjustment, mixed form): conjugate gradients on the exact
//    Schur operator of the FP32 Jacobian, applied matrix-free in double-float,
//    preconditioned by X^T X; see the section below.
// 2. k_refine (dense solves, zs_dense_cholesky_solve): x = X^T X b_s, then
//    FP64 iterative refinement r = b_s - S x, x += X^T X r until
//    ||r|| <= tol ||b_s|| or the sweep limit, in one cooperative launch with a
//    deterministic grid-wide norm.
#include <cooperative_groups.h>

#include <algorithm>

#include "ba_df.cuh"
#include "ba_internal.h"

namespace cg = cooperative_groups;

namespace zs {

template <typename T>
__device__ __forceinline__ T ldc(const T* p) {
    return __ldcg(p);
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
    static std::atomic<int> cache[kMaxDevices];
    const int v = per_device(cache, [] {
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        return sms;
    });
    return v > 0 ? v : 1;
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

// ------------------------------------------------------------ mixed-form PCG
//
// S formed from FP32 products is wrong by ~1e-7 ||H|| entrywise, which is of
// the order of its smallest eigenvalues on long trajectories (condition
// numbers ~1e8: H_pp and W H_pl^T cancel there), so refinement against it
// converges to the wrong step. The mixed form therefore solves the exact Schur
// system of its FP32 Jacobian J' (the values its FP32 records are built from;
// rounding J perturbs singular values by ~1e-7 ||J||, not eigenvalues by
// ~1e-7 ||J||^2) by conjugate gradients: the operator
//     S v = (H_pp + lambda I) v - H_pl (H_ll + lambda I)^-1 H_lp v
// is applied matrix-free from the per-observation Jacobian records in
// double-float arithmetic (ba_df.cuh: ~48 bits on the FP32 pipe; per
// observation the pose and landmark motions cancel to ~1e-4, which leaves
// ~1e-10), and X^T X (X = L^-1 of the FP32 factor of the FP32-formed S) is
// the preconditioner. The right-hand side b_s and the landmark
// back-substitution come from the same passes. CG vectors are FP64; every sum
// has a fixed order.

// Warp w of block b is the grid's warp b + gridDim.x * w: consecutive work
// items spread over all blocks (and SMs) first.
__device__ __forceinline__ int64_t spread_warp() {
    return blockIdx.x + (int64_t)gridDim.x * (threadIdx.x >> 5);
}

// Chunks of a pass are taken from a queue (an integer counter): warps that
// finish early take more, so the pass ends with the last chunk, not with the
// most loaded warp. Each chunk writes fixed locations, so the results do not
// depend on which warp takes it.
__device__ __forceinline__ int64_t next_chunk(int* queue) {
    int c = 0;
    if ((threadIdx.x & 31) == 0) c = atomicAdd(queue, 1);
    return __shfl_sync(0xffffffffu, c, 0);
}

// The claim of a warp's next chunk, issued before the current chunk's work
// and read after it, so that the atomic's round trip overlaps the work.
__device__ __forceinline__ int claim_chunk(int* queue) {
    return (threadIdx.x & 31) == 0 ? atomicAdd(queue, 1) : 0;
}
__device__ __forceinline__ int64_t claimed_chunk(int c) { return __shfl_sync(0xffffffffu, c, 0); }

__device__ __forceinline__ df ld_df(const df* p) {
    const float2 v = __ldcg(reinterpret_cast<const float2*>(p));
    return df{v.x, v.y};
}

// Landmark pass: a warp per landmark chunk (P.lmch_l), 32 consecutive
// observations (landmark-major) at a time, lane i taking observation
// base + i:
//   u_l = -sum_o J_l^T (c g_o + W_o J_p v_p)   (= c b_l - H_lp v),
//   y_l = (H_ll + lambda I)^-1 u_l,
// then ws_o = W_o (J_p v_p + J_l y_l) + c g_o for each observation (ws holds
// J_p v_p in between). The per-observation terms of u meet in a segmented
// inclusive scan over the lanes (segments: runs of one landmark; a
// Hillis-Steele scan in double-float) plus the running sum carried over from
// the previous 32; the lane holding a landmark's last observation forms y_l
// and stores it (yst, read again by the caller). ws_o goes to wsp at the
// observation's pose-major position. v (double-float) null: v = 0.
template <bool kIdW>
__device__ void op_landmarks(const DevProblem& P, const ObsJac* __restrict__ jac, const df* hinv, const df* v, bool c,
                             float4* ws, float4* wsp, df* yst, int* queue) {
    const int lane = threadIdx.x & 31;
    for (int64_t ch = next_chunk(queue), nxt; ch < P.nlmch; ch = claimed_chunk(nxt)) {
        nxt = claim_chunk(queue);
        const int l0 = P.lmch_l[ch], l1 = P.lmch_l[ch + 1];
        const int O0 = P.lm_ptr[l0], O1 = P.lm_ptr[l1];
        df carry[3] = {df_zero(), df_zero(), df_zero()};
        int carry_l = -1;
        for (int base = O0; base < O1; base += 32) {
            const int o = base + lane;
            const bool valid = o < O1;
            const int l = valid ? P.obs_lm[o] : -1 - lane;  // invalid lanes: segments of their own
            df k[3] = {df_zero(), df_zero(), df_zero()};
            if (valid) {
                const float4* r = reinterpret_cast<const float4*>(jac + o);
                const float4 G = __ldg(r);
                df t0 = df_zero(), t1 = df_zero();
                if (v) {
                    const df* vp = v + 6LL * P.obs_pose[o];
                    const float4 a = __ldg(r + 1), b = __ldg(r + 2), d = __ldg(r + 3);
                    df x[6];
#pragma unroll
                    for (int q = 0; q < 6; ++q) x[q] = ld_df(vp + q);
                    df_dot s0, s1;
                    s0.add(a.x, x[0]); s0.add(a.y, x[1]); s0.add(a.z, x[2]);
                    s0.add(a.w, x[3]); s0.add(b.x, x[4]); s0.add(b.y, x[5]);
                    s1.add(b.z, x[0]); s1.add(b.w, x[1]); s1.add(d.x, x[2]);
                    s1.add(d.y, x[3]); s1.add(d.z, x[4]); s1.add(d.w, x[5]);
                    t0 = s0.result();
                    t1 = s1.result();
                }
                const float4 e = __ldg(r + 4), f = __ldg(r + 5);
                // w = W t + c g, W = [f.z f.w; h.x h.y] (the identity when kIdW)
                df w0, w1;
                if constexpr (kIdW) {
                    w0 = c ? df_add(t0, df{G.x, G.y}) : t0;
                    w1 = c ? df_add(t1, df{G.z, G.w}) : t1;
                } else {
                    const float4 h = __ldg(r + 6);
                    df_dot q0, q1;
                    q0.add(f.z, t0); q0.add(f.w, t1);
                    q1.add(h.x, t0); q1.add(h.y, t1);
                    if (c) {
                        q0.add_df(df{G.x, G.y});
                        q1.add_df(df{G.z, G.w});
                    }
                    w0 = q0.result();
                    w1 = q1.result();
                }
                // k = -J_l^T w, J_l = [e.x e.y e.z; e.w f.x f.y]
                df_dot k0, k1, k2;
                k0.add(-e.x, w0); k0.add(-e.w, w1);
                k1.add(-e.y, w0); k1.add(-f.x, w1);
                k2.add(-e.z, w0); k2.add(-f.y, w1);
                k[0] = k0.result();
                k[1] = k1.result();
                k[2] = k2.result();
                ws[o] = make_float4(t0.hi, t0.lo, t1.hi, t1.lo);
            }
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                const int lo = __shfl_up_sync(0xffffffffu, l, off);
                df kk[3];
#pragma unroll
                for (int a = 0; a < 3; ++a) {
                    kk[a].hi = __shfl_up_sync(0xffffffffu, k[a].hi, off);
                    kk[a].lo = __shfl_up_sync(0xffffffffu, k[a].lo, off);
                }
                if (lane >= off && lo == l) {
#pragma unroll
                    for (int a = 0; a < 3; ++a) k[a] = df_add(kk[a], k[a]);
                }
            }
            if (l == carry_l) {
#pragma unroll
                for (int a = 0; a < 3; ++a) k[a] = df_add(carry[a], k[a]);
            }
            if (valid && o + 1 == P.lm_ptr[l + 1]) {  // the landmark's last observation
                const df* hi = hinv + 9LL * l;
#pragma unroll
                for (int a = 0; a < 3; ++a) {
                    df acc = df_zero();
#pragma unroll
                    for (int b = 0; b < 3; ++b) acc = df_add(acc, df_mul(ld_df(hi + 3 * a + b), k[b]));
                    yst[3LL * l + a] = acc;
                }
            }
            carry_l = __shfl_sync(0xffffffffu, l, 31);
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                carry[a].hi = __shfl_sync(0xffffffffu, k[a].hi, 31);
                carry[a].lo = __shfl_sync(0xffffffffu, k[a].lo, 31);
            }
        }
        for (int l = l0 + lane; l < l1; l += 32) {  // landmarks without observations: y = 0
            if (P.lm_ptr[l] == P.lm_ptr[l + 1]) {
#pragma unroll
                for (int a = 0; a < 3; ++a) yst[3LL * l + a] = df_zero();
            }
        }
        __syncwarp();  // yst of this chunk written by the warp's lanes
        for (int o = O0 + lane; o < O1; o += 32) {
            const int l = P.obs_lm[o];
            const float4* r = reinterpret_cast<const float4*>(jac + o);
            const float4 G = __ldg(r), e = __ldg(r + 4), f = __ldg(r + 5);
            const float4 tt = ws[o];  // this lane's own write above
            const df y0 = yst[3LL * l], y1 = yst[3LL * l + 1], y2 = yst[3LL * l + 2];
            // s = J_p v + J_l y
            df_dot m0, m1;
            m0.add_df(df{tt.x, tt.y});
            m0.add(e.x, y0); m0.add(e.y, y1); m0.add(e.z, y2);
            m1.add_df(df{tt.z, tt.w});
            m1.add(e.w, y0); m1.add(f.x, y1); m1.add(f.y, y2);
            const df s0 = m0.result(), s1 = m1.result();
            // ws = W s + c g
            df a0, a1;
            if constexpr (kIdW) {
                a0 = c ? df_add(s0, df{G.x, G.y}) : s0;
                a1 = c ? df_add(s1, df{G.z, G.w}) : s1;
            } else {
                const float4 h = __ldg(r + 6);
                df_dot n0, n1;
                n0.add(f.z, s0); n0.add(f.w, s1);
                n1.add(h.x, s0); n1.add(h.y, s1);
                if (c) {
                    n0.add_df(df{G.x, G.y});
                    n1.add_df(df{G.z, G.w});
                }
                a0 = n0.result();
                a1 = n1.result();
            }
            wsp[P.pm[o]] = make_float4(a0.hi, a0.lo, a1.hi, a1.lo);
        }
    }
}

// Pose pass: a warp per observation chunk, part[6 ch + a] = sum over the
// chunk of (J_p^T ws_o)_a, read pose-major (contiguous): lanes strided, then
// a double-float butterfly (df_add is commutative bit for bit, so every lane
// ends with the same value).
__device__ void op_pose_chunks(const DevProblem& P, const float4* __restrict__ jp_pm, const float4* wsp, df* part,
                               int* queue) {
    const int lane = threadIdx.x & 31;
    for (int64_t ch = next_chunk(queue), nxt; ch < P.nopch; ch = claimed_chunk(nxt)) {
        nxt = claim_chunk(queue);
        const int q1 = P.opch_q[ch + 1];
        df_dot acc[6];
        for (int q = P.opch_q[ch] + lane; q < q1; q += 32) {
            const float4 a = __ldg(jp_pm + q), b = __ldg(jp_pm + P.M + q), d = __ldg(jp_pm + 2 * P.M + q);
            const float4 sv = __ldcg(wsp + q);
            const df s0{sv.x, sv.y}, s1{sv.z, sv.w};
            const float j0[6] = {a.x, a.y, a.z, a.w, b.x, b.y}, j1[6] = {b.z, b.w, d.x, d.y, d.z, d.w};
#pragma unroll
            for (int k = 0; k < 6; ++k) {
                acc[k].add(j0[k], s0);
                acc[k].add(j1[k], s1);
            }
        }
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            df t = acc[k].result();
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) {
                const df o{__shfl_xor_sync(0xffffffffu, t.hi, off), __shfl_xor_sync(0xffffffffu, t.lo, off)};
                t = df_add(t, o);
            }
            if (lane == k) part[6 * ch + k] = t;
        }
    }
}

// Pose k's totals of the pose pass: a warp per pose (spread over the grid),
// lanes strided over the pose's chunks, then a double-float butterfly; every
// lane of the warp returns with tot[0..5]. Calls f(k, tot) for each pose the
// warp owns.
template <typename F>
__device__ __forceinline__ void for_pose_sums(const DevProblem& P, const df* part, F f) {
    const int lane = threadIdx.x & 31;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t k = spread_warp(); k < P.K; k += nw) {
        const int c0 = P.pose_opch[k], c1 = P.pose_opch[k + 1];
        df t[6] = {df_zero(), df_zero(), df_zero(), df_zero(), df_zero(), df_zero()};
        for (int ch = c0 + lane; ch < c1; ch += 32) {
#pragma unroll
            for (int a = 0; a < 6; ++a) t[a] = df_add(t[a], ld_df(part + 6LL * ch + a));
        }
        double tot[6];
#pragma unroll
        for (int a = 0; a < 6; ++a) {
            df v = t[a];
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) {
                const df o{__shfl_xor_sync(0xffffffffu, v.hi, off), __shfl_xor_sync(0xffffffffu, v.lo, off)};
                v = df_add(v, o);
            }
            tot[a] = df_to_double(v);
        }
        f((int)k, tot);
    }
}

// out = M v for a triangular FP32 matrix (mode 0: lower, c <= i; 1: upper,
// c >= i), a warp per row, FP32 accumulation: the conjugate-gradient
// preconditioner needs no more (the operator it preconditions is exact).
__device__ void gemv_f32(int n, const float* __restrict__ M, const float* v, float* out, int mode) {
    const int lane = threadIdx.x & 31;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int i = gw; i < n; i += nw) {
        const int lo = (mode == 1) ? i : 0;
        const int hi = (mode == 0) ? i + 1 : n;
        float acc = 0.f;
        for (int c = lo + lane; c < hi; c += 32) acc += M[(int64_t)i * n + c] * __ldcg(v + c);
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
        if (lane == 0) out[i] = acc;
    }
}

// Deterministic grid-wide sum of one value per thread, the same in every
// block: warp butterflies, the warps in order, then the block partials
// (written to slot) in a fixed lane-strided order. One grid barrier.
__device__ double grid_sum(cg::grid_group& grid, double v, double* slot, double* sh) {
    constexpr int NW = kThreads / 32;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    v = wsum(v);
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int w = 0; w < NW; ++w) s += sh[w];
        slot[blockIdx.x] = s;
    }
    grid.sync();
    if (warp == 0) {
        double t = 0.0;
        for (unsigned b = lane; b < gridDim.x; b += 32) t += __ldcg(slot + b);
        t = wsum(t);
        if (lane == 0) sh[NW] = t;
    }
    __syncthreads();
    const double t = sh[NW];
    __syncthreads();
    return t;
}

constexpr int kPcgMaxBlocks = 2048;

template <bool kIdW>
__global__ void __launch_bounds__(kThreads, 2) k_pcg(DevProblem P, const ObsJac* __restrict__ jac,
                                                  const float4* __restrict__ jp_pm,
                                                  const double* __restrict__ hinv, const float* __restrict__ X,
                                                  const float* __restrict__ XT, double* delta, double* bs, double* buf,
                                                  int max_it, double tol, LmState* st) {
    cg::grid_group grid = cg::this_grid();
    __shared__ double sh[kThreads / 32 + 1];
    if (!__ldcg(&st->solve_ok)) return;  // written by an earlier launch: uniform
    const int n = P.n;
    const double lam = __ldcg(&st->lambda);
    double* r = buf;
    double* p = r + n;
    double* q = p + n;
    float* rf = reinterpret_cast<float*>(q + n);  // FP32 r, X r and X^T X r of the preconditioner
    float* uf = rf + n;
    float* zf = uf + n;                      // (3n floats within the 2n doubles below pdf)
    df* pdf = reinterpret_cast<df*>(q + 3 * n);  // double-float copy of p
    df* part = pdf + n;                       // [6 nopch] chunk partials
    df* hdf = part + 6 * P.nopch;             // [9 L] double-float (H_ll + lambda I)^-1
    df* yst = hdf + 9LL * P.L;                // [3 L] double-float y of the landmark pass
    double* slots = reinterpret_cast<double*>(yst + 3LL * P.L);       // [2 kPcgMaxBlocks]
    int* queues = reinterpret_cast<int*>(slots + 2 * kPcgMaxBlocks);    // [4]: landmark, pose passes x 2
    float4* ws = reinterpret_cast<float4*>(slots + 2 * kPcgMaxBlocks + 2);  // [M] landmark-major
    float4* wsp = ws + P.M;                                             // [M] pose-major
    // grid sums alternate between two slot buffers: consecutive sums never
    // share one, and a barrier separates every reuse
    int red = 0;
    const int tid = blockIdx.x * blockDim.x + threadIdx.x, nth = gridDim.x * blockDim.x;

    for (int64_t i = tid; i < 9LL * P.L; i += nth) hdf[i] = df_from_double(hinv[i]);
    if (tid < 4) queues[tid] = 0;
    // pass k of a kind takes chunks from queue k & 1 and clears the other one,
    // which pass k - 1 finished with before a grid barrier and pass k + 1
    // starts on after one
    int npass = 0;
    auto queue = [&](int kind) {
        int* q = queues + 2 * kind;
        if (tid == 0) q[(npass + 1) & 1] = 0;
        return q + (npass & 1);
    };
    grid.sync();
    // r = b_s = b_p - H_pl (H_ll + lambda I)^-1 b_l, x = 0
    op_landmarks<kIdW>(P, jac, hdf, nullptr, true, ws, wsp, yst, queue(0));
    grid.sync();
    op_pose_chunks(P, jp_pm, wsp, part, queue(1));
    ++npass;
    grid.sync();
    double acc = 0.0;
    for_pose_sums(P, part, [&](int k, const double* tot) {
        const int lane = threadIdx.x & 31;
        if (lane < 6) {
            const int i = 6 * k + lane;
            const double v = -(lane == 0 ? tot[0] : lane == 1 ? tot[1] : lane == 2 ? tot[2]
                               : lane == 3 ? tot[3] : lane == 4 ? tot[4] : tot[5]);
            r[i] = v;
            bs[i] = v;
            delta[i] = 0.0;
            rf[i] = (float)v;
            acc += v * v;
        }
    });
    // landmark back-substitution delta_l = y(x) = (H_ll + lambda I)^-1 (b_l - H_lp x)
    // is linear in x: y(0) now, plus alpha y_0(p) with each step (y_0(p), the
    // landmark pass of S p, is left in yst by op_landmarks)
    for (int64_t i = tid; i < 3LL * P.L; i += nth) delta[n + i] = df_to_double(ld_df(yst + i));
    const double bn2 = grid_sum(grid, acc, slots + ((red++) & 1) * kPcgMaxBlocks, sh);
    double rn2 = bn2;
    int it = 0;
    bool indefinite = false;
    if (bn2 > 0.0 && max_it > 0) {
        // z = X^T X r, p = z
        gemv_f32(n, X, rf, uf, 0);
        grid.sync();
        gemv_f32(n, XT, uf, zf, 1);
        grid.sync();
        acc = 0.0;
        for (int i = tid; i < n; i += nth) {
            const double zi = (double)__ldcg(zf + i);
            p[i] = zi;
            pdf[i] = df_from_double(zi);
            acc += __ldcg(r + i) * zi;
        }
        double rz = grid_sum(grid, acc, slots + ((red++) & 1) * kPcgMaxBlocks, sh);
        for (;;) {
            // q = S p
            op_landmarks<kIdW>(P, jac, hdf, pdf, false, ws, wsp, yst, queue(0));
            grid.sync();
            op_pose_chunks(P, jp_pm, wsp, part, queue(1));
            ++npass;
            grid.sync();
            acc = 0.0;
            for_pose_sums(P, part, [&](int k, const double* tot) {
                const int lane = threadIdx.x & 31;
                if (lane < 6) {
                    const int i = 6 * k + lane;
                    const double pi = __ldcg(p + i);
                    const double qi = lam * pi + (lane == 0 ? tot[0] : lane == 1 ? tot[1] : lane == 2 ? tot[2]
                                                  : lane == 3 ? tot[3] : lane == 4 ? tot[4] : tot[5]);
                    q[i] = qi;
                    acc += pi * qi;
                }
            });
            const double pq = grid_sum(grid, acc, slots + ((red++) & 1) * kPcgMaxBlocks, sh);
            if (!(pq > 0.0)) {  // uniform: S is not positive definite, as a failed FP64 factorisation
                indefinite = true;
                break;
            }
            const double alpha = rz / pq;
            acc = 0.0;
            for (int i = tid; i < n; i += nth) {
                delta[i] = __ldcg(delta + i) + alpha * __ldcg(p + i);
                const double ri = __ldcg(r + i) - alpha * __ldcg(q + i);
                r[i] = ri;
                rf[i] = (float)ri;
                acc += ri * ri;
            }
            for (int64_t i = tid; i < 3LL * P.L; i += nth)
                delta[n + i] = __ldcg(delta + n + i) + alpha * df_to_double(ld_df(yst + i));
            rn2 = grid_sum(grid, acc, slots + ((red++) & 1) * kPcgMaxBlocks, sh);
            ++it;
            if (!(rn2 > tol * tol * bn2) || it >= max_it) break;
            gemv_f32(n, X, rf, uf, 0);
            grid.sync();
            gemv_f32(n, XT, uf, zf, 1);
            grid.sync();
            acc = 0.0;
            for (int i = tid; i < n; i += nth) acc += __ldcg(r + i) * (double)__ldcg(zf + i);
            const double rz1 = grid_sum(grid, acc, slots + ((red++) & 1) * kPcgMaxBlocks, sh);
            const double beta = rz1 / rz;
            rz = rz1;
            for (int i = tid; i < n; i += nth) {
                const double pi = (double)__ldcg(zf + i) + beta * __ldcg(p + i);
                p[i] = pi;
                pdf[i] = df_from_double(pi);
            }
            grid.sync();
        }
    }
    if (indefinite) {
        if (tid == 0) st->solve_ok = 0;
        return;
    }
    if (tid == 0) {
        st->resid_norm = sqrt(rn2);
        st->rhs_norm = sqrt(bn2);
        st->refine_sweeps = it;
    }
}

size_t pcg_doubles(const DevProblem& P) {
    // r p q (FP64), rf uf zf (FP32, 2n doubles' room), the double-float p,
    // chunk partials, the double-float landmark inverses and y, slots, four
    // queue counters, ws (16 B each); in 8-byte units (the sum before ws is
    // even: ws is 16-byte aligned)
    return 6 * (size_t)P.n + 6 * (size_t)P.nopch + 12 * (size_t)P.L + 2 * (size_t)kPcgMaxBlocks + 2 + 4 * (size_t)P.M;
}

cudaError_t launch_pcg(const DevProblem& P, DevWork& W, LmState* st, int max_it, double tol, cudaStream_t s) {
    if (P.n <= 0) return cudaSuccess;
    // W = I for every observation (no robust loss, no information matrices):
    // the operator skips the weight products
    const bool id_w = P.loss.kind == 0 && P.obs_info == nullptr;  // 0: no robust loss
    const void* kern = id_w ? (const void*)k_pcg<true> : (const void*)k_pcg<false>;
    static std::atomic<int> occ_cache[2][kMaxDevices];
    const int occ = per_device(occ_cache[id_w ? 1 : 0], [&] {
        int o = 0;
        return cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, kern, kThreads, 0) == cudaSuccess ? o : 0;
    });
    if (occ < 1) {
        const cudaError_t err = cudaGetLastError();
        return err != cudaSuccess ? err : cudaErrorInvalidConfiguration;
    }
    cudaError_t e;
    const int blocks = std::max(1, std::min(kPcgMaxBlocks, occ * sm_count()));
    DevProblem Pv = P;
    const ObsJac* jac = W.jac;
    const float4* jp_pm = W.jp_pm;
    const double* hinv = W.hll_inv;
    const float* X = (const float*)W.X;
    const float* XT = (const float*)W.XT;
    double* delta = W.delta;
    double* bs = W.bs;
    double* buf = W.pcg;
    void* args[] = {(void*)&Pv,  (void*)&jac, (void*)&jp_pm,  (void*)&hinv, (void*)&X,  (void*)&XT,
                    (void*)&delta, (void*)&bs, (void*)&buf, (void*)&max_it, (void*)&tol, (void*)&st};
    e = cudaLaunchCooperativeKernel(kern, dim3(blocks), dim3(kThreads), args, 0, s);
    if (e == cudaSuccess) note_launch();
    return e;
}

template cudaError_t launch_refine<double, float>(int, const double*, const float*, const float*, const double*,
                                                 double*, double*, LmState*, int, double, cudaStream_t);

}  // namespace zs
