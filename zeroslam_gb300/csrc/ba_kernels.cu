// Bundle-adjustment kernels for sm_103a: per-observation linearisation,
// deterministic segmented assembly, 3x3 landmark inverses, the Schur
// complement, landmark back-substitution, the manifold update, the cost and
// the Levenberg-Marquardt decision. No floating-point atomics anywhere: every
// sum has one owner thread or a fixed reduction tree, so results repeat bit
// for bit from run to run.
//
// Reference counterparts (gpdaniels/zeroslam):
//   k_linearize, k_reduce_lm, k_reduce_pose  make_hessian       source/factor_graph.hpp:648-732
//                                            compute_jacobians  source/factor_graph.hpp:1012-1048
//                                            robust_info        source/factor_graph.hpp:254-269
//   k_invert, k_w                            damping + invert<3> source/factor_graph.hpp:738-765,
//                                                               source/matrix.hpp:749-774
//   k_reduce_lm_jac (mixed form)             H_ll, b_l in double-float from the FP32 Jacobian records
//   k_schur_segments, k_schur_assemble, k_bs W = H_pl H_ll^-1, S = H_pp - W H_lp, b_s = b_p - W b_l
//                                            source/factor_graph.hpp:768-781,
//                                            source/matrix_sparse_block.hpp:158-196,
//                                            source/matrix_sparse_block_diagonal.hpp:107-142
//   k_backsub                                source/factor_graph.hpp:799-800
//   k_update, k_rollback                     source/factor_graph.hpp:809-846, 947-960
//   k_cost_partial                           get_current_chi    source/factor_graph.hpp:618-629
//   k_scale_partial, k_decide                LM acceptance      source/factor_graph.hpp:555-606
#include <algorithm>

#include "ba_df.cuh"
#include "ba_internal.h"

namespace zs {

// H_pl / W records per observation: 18 values, padded to a multiple of 16
// bytes so the Schur kernel can load them as vectors.
template <typename T>
struct RecStride {
    static constexpr int value = sizeof(T) == 4 ? 20 : 18;
};

// (a, c) with a <= c of a symmetric 6x6 block, row by row.
__constant__ int8_t kUp6[21][2] = {{0, 0}, {0, 1}, {0, 2}, {0, 3}, {0, 4}, {0, 5}, {1, 1}, {1, 2}, {1, 3}, {1, 4}, {1, 5},
                                   {2, 2}, {2, 3}, {2, 4}, {2, 5}, {3, 3}, {3, 4}, {3, 5}, {4, 4}, {4, 5}, {5, 5}};

// Per-observation partial records: the pose's 21 H_pp entries (upper
// triangle) and 6 b_p entries, padded to 28; the landmark's 6 H_ll entries
// and 3 b_l entries, padded to 12. Record-major, written and read as 16-byte
// vectors.
constexpr int kPoseRec = 28;
constexpr int kLmRec = 12;

template <int N>
__device__ __forceinline__ void store_rec(float* dst, const float (&v)[N]) {
    static_assert(N % 4 == 0, "record of whole float4");
#pragma unroll
    for (int i = 0; i < N / 4; ++i)
        reinterpret_cast<float4*>(dst)[i] = make_float4(v[4 * i], v[4 * i + 1], v[4 * i + 2], v[4 * i + 3]);
}
template <int N>
__device__ __forceinline__ void store_rec(double* dst, const double (&v)[N]) {
    static_assert(N % 2 == 0, "record of whole double2");
#pragma unroll
    for (int i = 0; i < N / 2; ++i) reinterpret_cast<double2*>(dst)[i] = make_double2(v[2 * i], v[2 * i + 1]);
}
template <int N>
__device__ __forceinline__ void add_rec(const float* src, float (&acc)[N]) {
#pragma unroll
    for (int i = 0; i < N / 4; ++i) {
        const float4 t = __ldg(reinterpret_cast<const float4*>(src) + i);
        acc[4 * i] += t.x; acc[4 * i + 1] += t.y; acc[4 * i + 2] += t.z; acc[4 * i + 3] += t.w;
    }
}
template <int N>
__device__ __forceinline__ void add_rec(const double* src, double (&acc)[N]) {
#pragma unroll
    for (int i = 0; i < N / 2; ++i) {
        const double2 t = __ldg(reinterpret_cast<const double2*>(src) + i);
        acc[2 * i] += t.x; acc[2 * i + 1] += t.y;
    }
}

// Per-pose data for the mixed form's linearisation: the quaternion-sandwich
// matrix M with M X = q (0, X) q* (valid for unnormalised q),
// M = (w^2 - |v|^2) I + 2 v v^T + 2 w [v]x, the translation, and the rotation
// matrix of source/lie.hpp:188-204 used by the landmark Jacobian.
// Layout per pose: M (9), t (3), R (9), pad (3).
constexpr int kAux = kPoseAux;

__global__ void __launch_bounds__(kThreads) k_pose_aux(DevProblem P, double* aux) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= P.K) return;
    const double* p = P.pose + (int64_t)k * kPoseStride;
    const double w = p[6], x = p[3], y = p[4], z = p[5];
    const double s = w * w - (x * x + y * y + z * z);
    double* a = aux + (int64_t)k * kAux;
    a[0] = s + 2.0 * x * x;      a[1] = 2.0 * (x * y - w * z); a[2] = 2.0 * (x * z + w * y);
    a[3] = 2.0 * (x * y + w * z); a[4] = s + 2.0 * y * y;      a[5] = 2.0 * (y * z - w * x);
    a[6] = 2.0 * (x * z - w * y); a[7] = 2.0 * (y * z + w * x); a[8] = s + 2.0 * z * z;
    a[9] = p[0];
    a[10] = p[1];
    a[11] = p[2];
    const double q[4] = {w, x, y, z};
    quat_matrix(q, a + 12);
}

template <typename T>
__global__ void __launch_bounds__(kThreads, sizeof(T) == 4 ? 3 : 0) k_linearize(DevProblem P, T* __restrict__ hpl, T* __restrict__ lm_part,
                                                        T* __restrict__ pose_part, const double* __restrict__ aux,
                                                        ObsJac* __restrict__ jac, float4* __restrict__ jp_pm) {
    constexpr int RS = RecStride<T>::value;
    // threads in pose-major order: the large records (H_pl, pose partials)
    // are written coalesced and neighbouring threads share the pose's data.
    // In the mixed form every lane of a warp takes part in the pose sums
    // below: a lane past the last observation repeats it and adds nothing.
    const int64_t q_id = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const bool valid = q_id < P.M;
    if (sizeof(T) == 8 && !valid) return;
    const int64_t q = valid ? q_id : P.M - 1;
    const int64_t o = P.pose_obs[q];
    const int pi = P.obs_pose[o], li = P.obs_lm[o];
    const double* xp = P.lm + (int64_t)li * kLmStride;
    const double2 uv = P.obs_uv[o];
    const double* om = P.obs_info ? P.obs_info + 4 * o : nullptr;
    T Jc[6], Xv, Yv, Zv, Rm[9];
    double r[2];
    if (sizeof(T) == 8 || P.loss.kind != 0) {
        // plain form, and the mixed form under a robust loss: residual rounded
        // exactly as the reference's. For Huber outliers rho' + 2 rho'' e2 is
        // zero in exact arithmetic and the rank-one weight term below is added
        // or not by its rounding; any other rounding of e2 takes the other
        // branch for some observations and changes their whole curvature along
        // the residual.
        const double* pp = P.pose + (int64_t)pi * kPoseStride;
        double p[7], X[3], Xc[3];
#pragma unroll
        for (int i = 0; i < 7; ++i) p[i] = __ldg(pp + i);
#pragma unroll
        for (int i = 0; i < 3; ++i) X[i] = __ldg(xp + i);
        const int front = residual(p, X, uv.x, uv.y, P.intr, Xc, r);
        if (front) {
            const T iz = (T)(1.0 / Xc[2]);
            const T iz2 = iz * iz;
            const T fx = (T)P.intr.fx, fy = (T)P.intr.fy;
            Jc[0] = fx * iz; Jc[1] = T(0); Jc[2] = -fx * (T)Xc[0] * iz2;
            Jc[3] = T(0); Jc[4] = fy * iz; Jc[5] = -fy * (T)Xc[1] * iz2;
        } else {
            Jc[0] = T(0); Jc[1] = T(0); Jc[2] = (T)kBehindPenalty;
            Jc[3] = T(0); Jc[4] = T(0); Jc[5] = (T)kBehindPenalty;
        }
        Xv = (T)Xc[0]; Yv = (T)Xc[1]; Zv = (T)Xc[2];
        double q[4] = {p[6], p[3], p[4], p[5]};
        double R[9];
        quat_matrix(q, R);
#pragma unroll
        for (int i = 0; i < 9; ++i) Rm[i] = (T)R[i];
    } else {
        // mixed form: camera-frame point in FP64 through the per-pose
        // sandwich matrix, everything after it in FP32
        const double* a = aux + (int64_t)pi * kAux;
        const double X0 = __ldg(xp), X1 = __ldg(xp + 1), X2 = __ldg(xp + 2);
        const double xc = fma(a[0], X0, fma(a[1], X1, fma(a[2], X2, a[9])));
        const double yc = fma(a[3], X0, fma(a[4], X1, fma(a[5], X2, a[10])));
        const double zc = fma(a[6], X0, fma(a[7], X1, fma(a[8], X2, a[11])));
        Xv = (T)xc; Yv = (T)yc; Zv = (T)zc;
        if (zc < 1.0e-12) {
            const double pen = -kBehindPenalty * zc;
            r[0] = pen; r[1] = pen;
            Jc[0] = T(0); Jc[1] = T(0); Jc[2] = (T)kBehindPenalty;
            Jc[3] = T(0); Jc[4] = T(0); Jc[5] = (T)kBehindPenalty;
        } else {
            const T iz = T(1) / Zv;
            const T fx = (T)P.intr.fx, fy = (T)P.intr.fy;
            // The residual subtracts two pixel coordinates of a few hundred
            // pixels to get about one, so it is formed in FP64 (in FP32 its
            // rounding, ~1e-5 px, dominates the gradient near convergence).
            // 1/z: the FP32 reciprocal refined by one Newton-Raphson step,
            // y' = y + y (1 - z y), which squares its relative error.
            double izd = (double)iz;
            izd = fma(izd, fma(-zc, izd, 1.0), izd);
            r[0] = (uv.x - P.intr.cx) - P.intr.fx * (xc * izd);
            r[1] = (uv.y - P.intr.cy) - P.intr.fy * (yc * izd);
            const T iz2 = iz * iz;
            Jc[0] = fx * iz; Jc[1] = T(0); Jc[2] = -fx * Xv * iz2;
            Jc[3] = T(0); Jc[4] = fy * iz; Jc[5] = -fy * Yv * iz2;
        }
#pragma unroll
        for (int i = 0; i < 9; ++i) Rm[i] = (T)a[12 + i];
    }

    // Robust weight W = rho' Omega (+ 2 rho'' (Omega r)(Omega r)^T), and the
    // gradient's non-robust Omega r scaled by rho'.
    double Wd[4] = {1.0, 0.0, 0.0, 1.0};
    if (om) {
        Wd[0] = om[0]; Wd[1] = om[1]; Wd[2] = om[2]; Wd[3] = om[3];
    }
    double orr0 = r[0], orr1 = r[1];
    if (om) {
        orr0 = om[0] * r[0] + om[1] * r[1];
        orr1 = om[2] * r[0] + om[3] * r[1];
    }
    double drho = 1.0;
    if (P.loss.kind) {
        const double e2 = chi2_of(r, om);
        double rho[3];
        loss_rho(P.loss, e2, rho);
        drho = rho[1];
#pragma unroll
        for (int i = 0; i < 4; ++i) Wd[i] *= rho[1];
        // For Huber outliers rho' + 2 rho'' e2 is zero in exact arithmetic, so
        // the sign comes from rounding: evaluate it as separately rounded
        // multiply and add (no FMA), as the reference does.
        if (__dadd_rn(rho[1], __dmul_rn(2.0 * rho[2], e2)) > 0.0) {
            const double k2 = 2.0 * rho[2];
            Wd[0] += k2 * orr0 * orr0;
            Wd[1] += k2 * orr0 * orr1;
            Wd[2] += k2 * orr1 * orr0;
            Wd[3] += k2 * orr1 * orr1;
        }
    }
    // J_p = -J_cam [-[Xc]x | I] (omega first), J_l = -J_cam R.
    T Jp[12], Jl[6];
#pragma unroll
    for (int rr = 0; rr < 2; ++rr) {
        const T c0 = Jc[rr * 3], c1 = Jc[rr * 3 + 1], c2 = Jc[rr * 3 + 2];
        Jp[rr * 6 + 0] = -(c2 * Yv - c1 * Zv);
        Jp[rr * 6 + 1] = -(c0 * Zv - c2 * Xv);
        Jp[rr * 6 + 2] = -(c1 * Xv - c0 * Yv);
        Jp[rr * 6 + 3] = -c0;
        Jp[rr * 6 + 4] = -c1;
        Jp[rr * 6 + 5] = -c2;
#pragma unroll
        for (int c = 0; c < 3; ++c) Jl[rr * 3 + c] = -(c0 * Rm[c] + c1 * Rm[3 + c] + c2 * Rm[6 + c]);
    }
    const T W00 = (T)Wd[0], W01 = (T)Wd[1], W10 = (T)Wd[2], W11 = (T)Wd[3];
    const T g0 = (T)(drho * orr0), g1 = (T)(drho * orr1);
    const bool pf = P.pose_fixed[pi] != 0, lf = P.lm_fixed[li] != 0;

    T prec[kPoseRec];
    T hrec[18];
#pragma unroll
    for (int k = 0; k < kPoseRec; ++k) prec[k] = T(0);
#pragma unroll
    for (int k = 0; k < 18; ++k) hrec[k] = T(0);
    if (!pf) {
        T A0[6], A1[6];  // (J_p^T W) columns
#pragma unroll
        for (int a = 0; a < 6; ++a) {
            A0[a] = Jp[a] * W00 + Jp[6 + a] * W10;
            A1[a] = Jp[a] * W01 + Jp[6 + a] * W11;
        }
#pragma unroll
        for (int k = 0; k < 21; ++k) {
            const int a = kUp6[k][0], c = kUp6[k][1];
            prec[k] = A0[a] * Jp[c] + A1[a] * Jp[6 + c];
        }
#pragma unroll
        for (int a = 0; a < 6; ++a) prec[21 + a] = -(Jp[a] * g0 + Jp[6 + a] * g1);
        if (!lf) {
#pragma unroll
            for (int a = 0; a < 6; ++a)
#pragma unroll
                for (int c = 0; c < 3; ++c) hrec[a * 3 + c] = A0[a] * Jl[c] + A1[a] * Jl[3 + c];
        }
    }
    if (valid) {
        T* hb = hpl + q * RS;
#pragma unroll
        for (int k = 0; k < 18; ++k) hb[k] = hrec[k];
    }
    if constexpr (sizeof(T) == 8) store_rec(pose_part + q * kPoseRec, prec);
    if constexpr (sizeof(T) == 4) {
        // mixed form: the Jacobian record (H_ll and b are its FP64 Gram sums)
        if (valid) {
            float4* d = reinterpret_cast<float4*>(jac + o);
            const df g0 = df_from_double(drho * orr0), g1 = df_from_double(drho * orr1);
            d[0] = make_float4(g0.hi, g0.lo, g1.hi, g1.lo);
            float jp[12], jl[6];
#pragma unroll
            for (int k = 0; k < 12; ++k) jp[k] = pf ? 0.f : (float)Jp[k];
#pragma unroll
            for (int k = 0; k < 6; ++k) jl[k] = lf ? 0.f : (float)Jl[k];
            if (jp_pm) {  // J_p is read only by the single problem's conjugate-gradient operator
                const float4 j0 = make_float4(jp[0], jp[1], jp[2], jp[3]), j1 = make_float4(jp[4], jp[5], jp[6], jp[7]),
                             j2 = make_float4(jp[8], jp[9], jp[10], jp[11]);
                d[1] = j0;
                d[2] = j1;
                d[3] = j2;
                jp_pm[q] = j0;  // pose-major copy for the operator's pose pass, three planes
                jp_pm[P.M + q] = j1;
                jp_pm[2 * P.M + q] = j2;
            }
            d[4] = make_float4(jl[0], jl[1], jl[2], jl[3]);
            d[5] = make_float4(jl[4], jl[5], (float)W00, (float)W01);
            d[6] = make_float4((float)W10, (float)W11, 0.f, 0.f);
        }
        // The pose sums, warp by warp: a segmented inclusive scan over the
        // warp's lanes keyed by pose (pose-major order, so each pose's lanes
        // are contiguous); the last lane of each pose's run stores the run's
        // 27 sums at its position, and k_reduce_pose_runs adds a pose's runs.
        const int lane = threadIdx.x & 31;
        const int key = valid ? pi : 0x7fffffff;
        if (!valid) {
#pragma unroll
            for (int k = 0; k < kPoseRec; ++k) prec[k] = T(0);
        }
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const int ko = __shfl_up_sync(0xffffffffu, key, off);
            const bool take = lane >= off && ko == key;
#pragma unroll
            for (int k = 0; k < 27; ++k) {
                const T v = __shfl_up_sync(0xffffffffu, prec[k], off);
                if (take) prec[k] += v;
            }
        }
        const int kn = __shfl_down_sync(0xffffffffu, key, 1);
        if (valid && (lane == 31 || kn != key || q + 1 == P.M)) store_rec(pose_part + q * kPoseRec, prec);
        return;
    } else {
    T lrec[kLmRec];
#pragma unroll
    for (int k = 0; k < kLmRec; ++k) lrec[k] = T(0);
    if (!lf) {
        T B0[3], B1[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            B0[a] = Jl[a] * W00 + Jl[3 + a] * W10;
            B1[a] = Jl[a] * W01 + Jl[3 + a] * W11;
        }
        lrec[0] = B0[0] * Jl[0] + B1[0] * Jl[3];
        lrec[1] = B0[0] * Jl[1] + B1[0] * Jl[4];
        lrec[2] = B0[0] * Jl[2] + B1[0] * Jl[5];
        lrec[3] = B0[1] * Jl[1] + B1[1] * Jl[4];
        lrec[4] = B0[1] * Jl[2] + B1[1] * Jl[5];
        lrec[5] = B0[2] * Jl[2] + B1[2] * Jl[5];
#pragma unroll
        for (int a = 0; a < 3; ++a) lrec[6 + a] = -(Jl[a] * g0 + Jl[3 + a] * g1);
    }
    store_rec(lm_part + o * kLmRec, lrec);
    }
}

// Duplicate (pose, landmark) observations: the run's owner gets the sum of
// the run's H_pl blocks, in order.
template <typename T>
__global__ void k_merge_dups(DevProblem P, T* hpl) {
    constexpr int RS = RecStride<T>::value;
    const int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (o >= P.M) return;
    if (P.dup_owner[o] != o) return;
    int64_t e = o + 1;
    T* own = hpl + (int64_t)P.pm[o] * RS;
    T acc[18];
#pragma unroll
    for (int k = 0; k < 18; ++k) acc[k] = own[k];
    while (e < P.M && P.dup_owner[e] == o) {
        const T* r = hpl + (int64_t)P.pm[e] * RS;
#pragma unroll
        for (int k = 0; k < 18; ++k) acc[k] += r[k];
        ++e;
    }
#pragma unroll
    for (int k = 0; k < 18; ++k) own[k] = acc[k];
}

template <typename T>
__global__ void __launch_bounds__(kThreads) k_reduce_lm(DevProblem P, const T* __restrict__ lm_part, double* hll,
                                                        double* b) {
    const int l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l >= P.L) return;
    T acc[kLmRec];
#pragma unroll
    for (int k = 0; k < kLmRec; ++k) acc[k] = T(0);
    const int e = P.lm_ptr[l + 1];
    for (int o = P.lm_ptr[l]; o < e; ++o) add_rec(lm_part + (int64_t)o * kLmRec, acc);
    double* h = hll + (int64_t)l * 9;
    h[0] = acc[0]; h[1] = acc[1]; h[2] = acc[2];
    h[3] = acc[1]; h[4] = acc[3]; h[5] = acc[4];
    h[6] = acc[2]; h[7] = acc[4]; h[8] = acc[5];
    double* bl = b + P.n + 3LL * l;
    bl[0] = acc[6]; bl[1] = acc[7]; bl[2] = acc[8];
}

// One observation's terms of the mixed form's H_ll and b_l from its
// Jacobian record: v = H_ll's upper triangle (00 01 02 11 12 22) of
// J_l^T W J_l, then -J_l^T g, in double-float (the products of FP32 values
// are exact).
__device__ __forceinline__ void lm_jac_terms(const ObsJac* __restrict__ rec, df v[9]) {
    const float4* r = reinterpret_cast<const float4*>(rec);
    const float4 G = __ldg(r), a = __ldg(r + 4), c = __ldg(r + 5), d = __ldg(r + 6);
    const float J0[3] = {a.x, a.y, a.z}, J1[3] = {a.w, c.x, c.y};
    const df g0{G.x, G.y}, g1{G.z, G.w};
    // B = J^T W (3 x 2): B0 = column 0, B1 = column 1
    df B0[3], B1[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        df_dot s0, s1;
        s0.add(J0[k], df{c.z, 0.f});
        s0.add(J1[k], df{d.x, 0.f});
        s1.add(J0[k], df{c.w, 0.f});
        s1.add(J1[k], df{d.y, 0.f});
        B0[k] = s0.result();
        B1[k] = s1.result();
    }
    // H(a, c) = B0[a] J0[c] + B1[a] J1[c], upper triangle row by row
    auto entry = [&](int ia, int ic) {
        df_dot s;
        s.add(J0[ic], B0[ia]);
        s.add(J1[ic], B1[ia]);
        return s.result();
    };
    v[0] = entry(0, 0);
    v[1] = entry(0, 1);
    v[2] = entry(0, 2);
    v[3] = entry(1, 1);
    v[4] = entry(1, 2);
    v[5] = entry(2, 2);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        df_dot sb;
        sb.add(-J0[k], g0);
        sb.add(-J1[k], g1);
        v[6 + k] = sb.result();
    }
}

// Writes landmark l's H_ll (9 doubles, symmetric) and b_l from the sums v.
__device__ __forceinline__ void store_lm_sums(const DevProblem& P, int64_t l, const df v[9], double* hll, double* b) {
    double hd[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) hd[k] = df_to_double(v[k]);
    double* o9 = hll + l * 9;
    o9[0] = hd[0]; o9[1] = hd[1]; o9[2] = hd[2];
    o9[3] = hd[1]; o9[4] = hd[3]; o9[5] = hd[4];
    o9[6] = hd[2]; o9[7] = hd[4]; o9[8] = hd[5];
    double* bo = b + P.n + 3 * l;
    bo[0] = df_to_double(v[6]); bo[1] = df_to_double(v[7]); bo[2] = df_to_double(v[8]);
}

// Mixed form: H_ll = sum J_l^T W J_l and b_l = -sum J_l^T g per landmark from
// the FP32 Jacobian records in double-float (~48 bits): H_ll must be accurate
// far beyond FP32 for the Schur operator of launch_pcg. Two layouts of the
// same sums: a thread per landmark (observations in order) where there are
// enough landmarks to fill the GPU, else a warp per landmark chunk
// (P.lmch_l), 32 consecutive observations at a time: each lane forms its
// observation's terms, a segmented inclusive scan over the lanes (runs of one
// landmark) plus the sum carried from the previous 32 gives each landmark's
// total in the lane holding its last observation.
__global__ void __launch_bounds__(kThreads) k_reduce_lm_jac_thread(DevProblem P, const ObsJac* __restrict__ jac,
                                                                   double* hll, double* b) {
    const int64_t l = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (l >= P.L) return;
    df v[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) v[k] = df_zero();
    const int e = P.lm_ptr[l + 1];
    for (int o = P.lm_ptr[l]; o < e; ++o) {
        df t[9];
        lm_jac_terms(jac + o, t);
#pragma unroll
        for (int k = 0; k < 9; ++k) v[k] = df_add(v[k], t[k]);
    }
    store_lm_sums(P, l, v, hll, b);
}

__global__ void __launch_bounds__(kThreads) k_reduce_lm_jac(DevProblem P, const ObsJac* __restrict__ jac, double* hll,
                                                            double* b) {
    const int lane = threadIdx.x & 31;
    const int64_t ch = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    if (ch >= P.nlmch) return;
    const int l0 = P.lmch_l[ch], l1 = P.lmch_l[ch + 1];
    const int O0 = P.lm_ptr[l0], O1 = P.lm_ptr[l1];
    df carry[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) carry[k] = df_zero();
    int carry_l = -1;
    for (int base = O0; base < O1; base += 32) {
        const int o = base + lane;
        const bool valid = o < O1;
        const int l = valid ? P.obs_lm[o] : -1 - lane;
        df v[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) v[k] = df_zero();
        if (valid) lm_jac_terms(jac + o, v);
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const int lo = __shfl_up_sync(0xffffffffu, l, off);
#pragma unroll
            for (int k = 0; k < 9; ++k) {
                const df u{__shfl_up_sync(0xffffffffu, v[k].hi, off), __shfl_up_sync(0xffffffffu, v[k].lo, off)};
                if (lane >= off && lo == l) v[k] = df_add(u, v[k]);
            }
        }
        if (l == carry_l) {
#pragma unroll
            for (int k = 0; k < 9; ++k) v[k] = df_add(carry[k], v[k]);
        }
        if (valid && o + 1 == P.lm_ptr[l + 1]) store_lm_sums(P, l, v, hll, b);  // the landmark's last observation
        carry_l = __shfl_sync(0xffffffffu, l, 31);
#pragma unroll
        for (int k = 0; k < 9; ++k) {
            carry[k].hi = __shfl_sync(0xffffffffu, v[k].hi, 31);
            carry[k].lo = __shfl_sync(0xffffffffu, v[k].lo, 31);
        }
    }
    for (int l = l0 + lane; l < l1; l += 32) {  // landmarks without observations
        if (P.lm_ptr[l] == P.lm_ptr[l + 1]) {
#pragma unroll
            for (int k = 0; k < 9; ++k) hll[(int64_t)l * 9 + k] = 0.0;
            b[P.n + 3LL * l] = 0.0; b[P.n + 3LL * l + 1] = 0.0; b[P.n + 3LL * l + 2] = 0.0;
        }
    }
}

// Per pose (a CTA): each thread sums its strided share of the pose's
// observation records (pose-major, contiguous) in T; the thread partials meet
// in FP64 through a fixed tree (warp shuffles, then the warps' results in
// warp order).
template <typename T>
__global__ void __launch_bounds__(kThreads) k_reduce_pose(DevProblem P, const T* __restrict__ pose_part, double* hpp,
                                                          double* b) {
    constexpr int NW = kThreads / 32;
    __shared__ double sh[NW][28];
    const int k = blockIdx.x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    T acc[kPoseRec];
#pragma unroll
    for (int c = 0; c < kPoseRec; ++c) acc[c] = T(0);
    const int e = P.pose_ptr[k + 1];
    for (int i = P.pose_ptr[k] + threadIdx.x; i < e; i += blockDim.x)
        add_rec(pose_part + (int64_t)i * kPoseRec, acc);  // the pose's records are contiguous
#pragma unroll
    for (int c = 0; c < 27; ++c) {
        double v = (double)acc[c];
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
        if (lane == 0) sh[warp][c] = v;
    }
    __syncthreads();
    if (threadIdx.x < 27) {
        const int c = threadIdx.x;
        double v = 0.0;
#pragma unroll
        for (int w = 0; w < NW; ++w) v += sh[w][c];
        if (c < 21) {
            const int a = kUp6[c][0], d = kUp6[c][1];
            hpp[(int64_t)k * 36 + a * 6 + d] = v;
            hpp[(int64_t)k * 36 + d * 6 + a] = v;
        } else {
            b[6LL * k + (c - 21)] = v;
        }
    }
}

// Mixed form: H_pp and b_p of pose k (a CTA per pose) from the runs that
// k_linearize stored: within each 32-position warp chunk of the pose's
// pose-major range, the run's sums sit at its last position. Threads take
// the chunks in turn and add in FP64; the warps' totals meet in a fixed
// order.
__global__ void __launch_bounds__(kThreads) k_reduce_pose_runs(DevProblem P, const float* __restrict__ pose_part,
                                                               double* hpp, double* b) {
    constexpr int NW = kThreads / 32;
    __shared__ double sh[NW][28];
    const int k = blockIdx.x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    double acc[27];
#pragma unroll
    for (int c = 0; c < 27; ++c) acc[c] = 0.0;
    const int s0 = P.pose_ptr[k], e = P.pose_ptr[k + 1];
    if (e > s0) {
        const int c0 = s0 >> 5, c1 = (e - 1) >> 5;
        for (int c = c0 + threadIdx.x; c <= c1; c += blockDim.x) {
            const int tail = min(e, 32 * c + 32) - 1;
            const float4* r = reinterpret_cast<const float4*>(pose_part + (int64_t)tail * kPoseRec);
#pragma unroll
            for (int i = 0; i < 7; ++i) {
                const float4 t = __ldg(r + i);
                acc[4 * i] += (double)t.x;
                acc[4 * i + 1] += (double)t.y;
                acc[4 * i + 2] += (double)t.z;
                if (4 * i + 3 < 27) acc[4 * i + 3] += (double)t.w;
            }
        }
    }
    // The warps that took no chunk hold zeros: they skip their 27 FP64
    // butterflies (warp-uniform) and their totals are written as the zeros
    // the butterflies would have produced, so the sums are unchanged.
    const int nchunks = e > s0 ? ((e - 1) >> 5) - (s0 >> 5) + 1 : 0;
    if (warp * 32 < nchunks) {
#pragma unroll
        for (int c = 0; c < 27; ++c) {
            double v = acc[c];
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
            if (lane == 0) sh[warp][c] = v;
        }
    } else if (lane < 27) {
        sh[warp][lane] = 0.0;
    }
    __syncthreads();
    if (threadIdx.x < 27) {
        const int c = threadIdx.x;
        double v = 0.0;
#pragma unroll
        for (int w = 0; w < NW; ++w) v += sh[w][c];
        if (c < 21) {
            const int a = kUp6[c][0], d = kUp6[c][1];
            hpp[(int64_t)k * 36 + a * 6 + d] = v;
            hpp[(int64_t)k * 36 + d * 6 + a] = v;
        } else {
            b[6LL * k + (c - 21)] = v;
        }
    }
}

// Damped 3x3 landmark inverses (landmark_inverse).
__global__ void __launch_bounds__(kThreads) k_invert(DevProblem P, const double* __restrict__ hll, double* hinv,
                                                     float* hinv_f, const LmState* st) {
    const int l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l >= P.L) return;
    landmark_inverse(hll + (int64_t)l * 9, st->lambda, P.lm_fixed[l] != 0, hinv + (int64_t)l * 9,
                     hinv_f ? hinv_f + (int64_t)l * 12 : nullptr);
}

// W = H_pl H_ll^-1 per block. Mixed form: the FP32 inverses (hinv_f, 12
// floats per landmark) and 16-byte record loads and stores.
template <typename T>
__global__ void __launch_bounds__(kThreads) k_w(DevProblem P, const T* __restrict__ hpl, const double* __restrict__ hinv,
                                                const float* __restrict__ hinv_f, T* __restrict__ W) {
    constexpr int RS = RecStride<T>::value;
    const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;  // pose-major position
    if (q >= P.M) return;
    const int64_t o = P.pose_obs[q];
    if (!P.blk_valid[o]) return;
    if constexpr (sizeof(T) == 4) {
        const float4* I4 = reinterpret_cast<const float4*>(hinv_f + (int64_t)P.obs_lm[o] * 12);
        const float4 i0 = __ldg(I4), i1 = __ldg(I4 + 1), i2 = __ldg(I4 + 2);
        const float iv[9] = {i0.x, i0.y, i0.z, i0.w, i1.x, i1.y, i1.z, i1.w, i2.x};
        const float4* h4 = reinterpret_cast<const float4*>(hpl + q * RS);
        float h[20];
#pragma unroll
        for (int i = 0; i < 5; ++i) {
            const float4 t = __ldg(h4 + i);
            h[4 * i] = t.x; h[4 * i + 1] = t.y; h[4 * i + 2] = t.z; h[4 * i + 3] = t.w;
        }
        float w[20];
#pragma unroll
        for (int a = 0; a < 6; ++a)
#pragma unroll
            for (int c = 0; c < 3; ++c) w[a * 3 + c] = h[a * 3] * iv[c] + h[a * 3 + 1] * iv[3 + c] + h[a * 3 + 2] * iv[6 + c];
        w[18] = 0.f;
        w[19] = 0.f;
        float4* w4 = reinterpret_cast<float4*>(W + q * RS);
#pragma unroll
        for (int i = 0; i < 5; ++i) w4[i] = make_float4(w[4 * i], w[4 * i + 1], w[4 * i + 2], w[4 * i + 3]);
    } else {
        const double* I = hinv + (int64_t)P.obs_lm[o] * 9;
        T iv[9];
#pragma unroll
        for (int i = 0; i < 9; ++i) iv[i] = (T)I[i];
        const T* h = hpl + q * RS;
        T* w = W + q * RS;
#pragma unroll
        for (int a = 0; a < 6; ++a) {
            const T h0 = h[a * 3], h1 = h[a * 3 + 1], h2 = h[a * 3 + 2];
#pragma unroll
            for (int c = 0; c < 3; ++c) w[a * 3 + c] = h0 * iv[c] + h1 * iv[3 + c] + h2 * iv[6 + c];
        }
    }
}

// Loads one 18-value record (padded stride) with 16-byte vector loads.
__device__ __forceinline__ void load_rec(const float* p, float v[20]) {
    const float4* q = reinterpret_cast<const float4*>(p);
#pragma unroll
    for (int i = 0; i < 5; ++i) {
        const float4 t = __ldg(q + i);
        v[4 * i] = t.x; v[4 * i + 1] = t.y; v[4 * i + 2] = t.z; v[4 * i + 3] = t.w;
    }
}
__device__ __forceinline__ void load_rec(const double* p, double v[20]) {
    const double2* q = reinterpret_cast<const double2*>(p);
#pragma unroll
    for (int i = 0; i < 9; ++i) {
        const double2 t = __ldg(q + i);
        v[2 * i] = t.x; v[2 * i + 1] = t.y;
    }
}

// Partial 6 x 6 sums W_i H_j^T over one segment (<= 512 consecutive triples
// of one pose pair), a warp per segment: lane t takes the segment's triples
// t, t + 32, ... (consecutive lanes read consecutive pose-major records,
// coalesced) and accumulates in T (at most 16 triples per lane); the 32 lane
// partials meet in a fixed tree (FP32: an xor-shuffle butterfly, identical in
// every lane; FP64: a transpose through shared memory and a column sum in
// lane order) and the segment sum is stored in FP64. (The mixed form's S is
// the preconditioner of its conjugate-gradient solve, launch_pcg, so FP32
// sums suffice there.) With windows, segments of stopped windows (ctl) are
// skipped.
template <typename T>
constexpr int schur_seg_threads() {
    return sizeof(T) == 8 ? 128 : 256;  // FP64: 4 warps keep the transpose buffer under 48 KB
}

template <typename T>
__global__ void __launch_bounds__(schur_seg_threads<T>()) k_schur_segments(DevProblem P, const T* __restrict__ W,
                                                                          const T* __restrict__ hpl,
                                                                          double* __restrict__ part,
                                                                          const WinCtl* __restrict__ ctl) {
    constexpr int RS = RecStride<T>::value;
    constexpr int NW = schur_seg_threads<T>() / 32;
    __shared__ double red[sizeof(T) == 8 ? NW : 1][32][37];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int64_t g = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    if (g >= P.nsegs) return;
    if (ctl && P.pose_win && !ctl[P.pose_win[P.pair_i[P.seg_pair[g]]]].active) return;
    T acc[36];
#pragma unroll
    for (int e = 0; e < 36; ++e) acc[e] = T(0);
    const int64_t t1 = P.seg_ptr[g + 1];
    for (int64_t t = P.seg_ptr[g] + lane; t < t1; t += 32) {
        const int2 tr = P.triples[t];
        T wv[20], hv[20];
        load_rec(W + (int64_t)tr.x * RS, wv);
        load_rec(hpl + (int64_t)tr.y * RS, hv);
#pragma unroll
        for (int a = 0; a < 6; ++a)
#pragma unroll
            for (int d = 0; d < 6; ++d)
                acc[a * 6 + d] += wv[a * 3] * hv[d * 3] + wv[a * 3 + 1] * hv[d * 3 + 1] + wv[a * 3 + 2] * hv[d * 3 + 2];
    }
    double* out = part + g * 36;
    if constexpr (sizeof(T) == 4) {
#pragma unroll
        for (int e = 0; e < 36; ++e) {
            T v = acc[e];
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
            if (e == lane || e == 32 + lane) out[e] = (double)v;
        }
    } else {
        double (*r)[37] = red[wib];
#pragma unroll
        for (int e = 0; e < 36; ++e) r[lane][e] = (double)acc[e];
        __syncwarp();
        double v0 = 0.0;
        for (int k = 0; k < 32; ++k) v0 += r[k][lane];
        out[lane] = v0;
        if (lane < 4) {
            double v1 = 0.0;
            for (int k = 0; k < 32; ++k) v1 += r[k][32 + lane];
            out[32 + lane] = v1;
        }
    }
}

// S_ij -= the pair's segment sums, added in FP64 in segment order: diagonal
// pairs subtract from the H_pp + lambda I block written by k_s_init,
// off-diagonal pairs write both blocks. With windows the pair's window S
// block is used and stopped windows (ctl) are skipped.
__global__ void __launch_bounds__(kThreads) k_schur_assemble(DevProblem P, const double* __restrict__ part, double* S,
                                                             const WinCtl* __restrict__ ctl) {
    const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (idx >= (int64_t)P.npairs * 36) return;
    const int p = (int)(idx / 36), e = (int)(idx % 36);
    const int i = P.pair_i[p], j = P.pair_j[p];
    int p0 = 0, nw = P.n;
    int64_t soff = 0;
    if (P.pose_win) {
        const int w = P.pose_win[i];
        if (ctl && !ctl[w].active) return;
        p0 = P.win_pose0[w];
        nw = 6 * (P.win_pose0[w + 1] - p0);
        soff = P.win_s_off[w];
    }
    double sum = 0.0;
    const int64_t g1 = P.pair_seg_ptr[p + 1];
    for (int64_t g = P.pair_seg_ptr[p]; g < g1; ++g) sum += part[g * 36 + e];
    double* Sw = S + soff;
    const int64_t n = nw;
    const int64_t row = 6LL * (i - p0) + e / 6, col = 6LL * (j - p0) + e % 6;
    if (i == j) {
        Sw[row * n + col] = Sw[row * n + col] - sum;
    } else {
        Sw[row * n + col] = -sum;
        Sw[col * n + row] = -sum;
    }
}

// S = blockdiag(H_pp + lambda I); the pair sums are subtracted next.
__global__ void __launch_bounds__(kThreads) k_s_init(DevProblem P, const double* __restrict__ hpp, double* S,
                                                     const LmState* st) {
    const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t n = P.n;
    if (idx >= n * n) return;
    const int row = (int)(idx / n), col = (int)(idx % n);
    double v = 0.0;
    if (row / 6 == col / 6) {
        v = hpp[(int64_t)(row / 6) * 36 + (row % 6) * 6 + (col % 6)];
        if (row == col) v += st->lambda;
    }
    S[idx] = v;
}

// b_s = b_p - W b_l per pose (launch_pose_sums6): position q's term W_q b_l
// (pose-major W records) and the pose's output.
template <typename T>
struct BsTerm {
    const T* W;
    const double* b;
    __device__ void operator()(const DevProblem& P, int q, double s[6]) const {
        constexpr int RS = RecStride<T>::value;
        const int64_t o = P.pose_obs[q];
        if (!P.blk_valid[o]) return;
        const T* w = W + (int64_t)q * RS;
        const double* bl = b + P.n + 3LL * P.obs_lm[o];
        const T b0 = (T)bl[0], b1 = (T)bl[1], b2 = (T)bl[2];
#pragma unroll
        for (int a = 0; a < 6; ++a) s[a] += (double)(w[a * 3] * b0 + w[a * 3 + 1] * b1 + w[a * 3 + 2] * b2);
    }
};
struct BsOut {
    const double* b;
    double* bs;
    __device__ void operator()(const DevProblem&, int k, int a, double v) const { bs[6LL * k + a] = b[6LL * k + a] - v; }
};

// The same with a CTA per pose, for batches of thousands of window poses
// (the grid is full without the chunks, and it is one launch, not two).
template <typename T>
__global__ void __launch_bounds__(kThreads) k_bs_per_pose(DevProblem P, const T* __restrict__ W,
                                                          const double* __restrict__ b, double* bs) {
    __shared__ double sh[kThreads];
    const int k = blockIdx.x;
    const BsTerm<T> term{W, b};
    double acc[6] = {0, 0, 0, 0, 0, 0};
    for (int q = P.pose_ptr[k] + threadIdx.x; q < P.pose_ptr[k + 1]; q += blockDim.x) term(P, q, acc);
#pragma unroll 1
    for (int a = 0; a < 6; ++a) {
        const double v = block_sum(acc[a], sh);
        if (threadIdx.x == 0) bs[6LL * k + a] = b[6LL * k + a] - v;
    }
}

// delta_l = H_ll^-1 (b_l - H_lp delta_p); delta[0..n) already holds delta_p.
// A warp per landmark (lanes over its observations, then a butterfly: the
// whole GPU busy at ten thousand landmarks, and a fixed order).
template <typename T>
__global__ void __launch_bounds__(kThreads) k_backsub(DevProblem P, const T* __restrict__ hpl,
                                                      const double* __restrict__ hinv, const double* __restrict__ b,
                                                      double* delta, const LmState* st) {
    constexpr int RS = RecStride<T>::value;
    if (!st->solve_ok) return;
    const int lane = threadIdx.x & 31;
    const int64_t l = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    if (l >= P.L) return;
    double u0 = 0.0, u1 = 0.0, u2 = 0.0;
    const int e = P.lm_ptr[l + 1];
    for (int o = P.lm_ptr[l] + lane; o < e; o += 32) {
        if (!P.blk_valid[o]) continue;
        const T* h = hpl + (int64_t)P.pm[o] * RS;
        const double* dp = delta + 6LL * P.obs_pose[o];
        T s0 = T(0), s1 = T(0), s2 = T(0);
#pragma unroll
        for (int a = 0; a < 6; ++a) {
            const T d = (T)dp[a];
            s0 += h[a * 3] * d;
            s1 += h[a * 3 + 1] * d;
            s2 += h[a * 3 + 2] * d;
        }
        u0 += s0; u1 += s1; u2 += s2;
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        u0 += __shfl_xor_sync(0xffffffffu, u0, off);
        u1 += __shfl_xor_sync(0xffffffffu, u1, off);
        u2 += __shfl_xor_sync(0xffffffffu, u2, off);
    }
    if (lane != 0) return;
    const double* bl = b + P.n + 3LL * l;
    const double v0 = bl[0] - u0, v1 = bl[1] - u1, v2 = bl[2] - u2;
    const double* I = hinv + (int64_t)l * 9;
    double* dl = delta + P.n + 3LL * l;
    dl[0] = I[0] * v0 + I[1] * v1 + I[2] * v2;
    dl[1] = I[3] * v0 + I[4] * v1 + I[5] * v2;
    dl[2] = I[6] * v0 + I[7] * v1 + I[8] * v2;
}

// Backup and apply the step to free vertices.
__global__ void __launch_bounds__(kThreads) k_update(DevProblem P, const double* __restrict__ delta, const LmState* st) {
    if (!st->solve_ok) return;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < P.K) {
        double* p = P.pose + (int64_t)t * kPoseStride;
        double* bk = P.pose_bk + (int64_t)t * kPoseStride;
#pragma unroll
        for (int i = 0; i < kPoseStride; ++i) bk[i] = p[i];
        if (P.pose_fixed[t]) return;
        double d[6];
#pragma unroll
        for (int i = 0; i < 6; ++i) d[i] = delta[6LL * t + i];
        pose_plus(p, d);
    } else if (t < P.K + P.L) {
        const int l = t - P.K;
        double* x = P.lm + (int64_t)l * kLmStride;
        double* bk = P.lm_bk + (int64_t)l * kLmStride;
#pragma unroll
        for (int i = 0; i < kLmStride; ++i) bk[i] = x[i];
        if (P.lm_fixed[l]) return;
        const double* d = delta + P.n + 3LL * l;
        x[0] += d[0];
        x[1] += d[1];
        x[2] += d[2];
    }
}

// A rejected step is rolled back only while lambda stays finite: the
// reference breaks out before rollback_states() otherwise (source/factor_graph.hpp:592-604).
__global__ void __launch_bounds__(kThreads) k_rollback(DevProblem P, const LmState* st) {
    if (!st->solve_ok || st->good || !isfinite(st->lambda)) return;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < P.K) {
#pragma unroll
        for (int i = 0; i < kPoseStride; ++i)
            P.pose[(int64_t)t * kPoseStride + i] = P.pose_bk[(int64_t)t * kPoseStride + i];
    } else if (t < P.K + P.L) {
        const int l = t - P.K;
#pragma unroll
        for (int i = 0; i < kLmStride; ++i) P.lm[(int64_t)l * kLmStride + i] = P.lm_bk[(int64_t)l * kLmStride + i];
    }
}

// Fixed-shape two-level sums: kReduceBlocks blocks stride over the items in
// a fixed order, then one block adds the block results in a fixed tree.
__global__ void __launch_bounds__(kThreads) k_scale_partial(DevProblem P, const double* __restrict__ delta,
                                                            const double* __restrict__ b, double* red,
                                                            const LmState* st) {
    __shared__ double sh[kThreads];
    if (!st->solve_ok) return;
    const double lam = st->lambda;
    const int64_t N = (int64_t)P.n + 3LL * P.L;
    double v = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x)
        v += delta[i] * (lam * delta[i] + b[i]);
    v = block_sum(v, sh);
    if (threadIdx.x == 0) red[blockIdx.x] = v;
}

__global__ void __launch_bounds__(kThreads) k_cost_partial(DevProblem P, double* red, const LmState* st,
                                                           int only_if_ok) {
    __shared__ double sh[kThreads];
    if (only_if_ok && !st->solve_ok) return;
    double v = 0.0;
    for (int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o < P.M; o += (int64_t)gridDim.x * blockDim.x) {
        const int pi = P.obs_pose[o], li = P.obs_lm[o];
        const double* pp = P.pose + (int64_t)pi * kPoseStride;
        const double* xp = P.lm + (int64_t)li * kLmStride;
        double p[7], X[3];
#pragma unroll
        for (int i = 0; i < 7; ++i) p[i] = pp[i];
#pragma unroll
        for (int i = 0; i < 3; ++i) X[i] = xp[i];
        const double2 uv = P.obs_uv[o];
        double Xc[3], r[2];
        residual(p, X, uv.x, uv.y, P.intr, Xc, r);
        const double e2 = chi2_of(r, P.obs_info ? P.obs_info + 4 * o : nullptr);
        if (P.loss.kind) {
            double rho[3];
            loss_rho(P.loss, e2, rho);
            v += rho[0];
        } else {
            v += e2;
        }
    }
    v = block_sum(v, sh);
    if (threadIdx.x == 0) red[blockIdx.x] = v;
}

// The mixed form's cost: FP64 through the per-pose sandwich matrices
// (k_pose_aux of the current poses), contracted multiply-adds.
__global__ void __launch_bounds__(kThreads) k_cost_partial_fast(DevProblem P, const double* __restrict__ aux,
                                                                double* red, const LmState* st, int only_if_ok) {
    __shared__ double sh[kThreads];
    if (only_if_ok && !st->solve_ok) return;
    double v = 0.0;
    for (int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o < P.M; o += (int64_t)gridDim.x * blockDim.x) {
        const double* xp = P.lm + (int64_t)P.obs_lm[o] * kLmStride;
        const double X[3] = {xp[0], xp[1], xp[2]};
        const double2 uv = P.obs_uv[o];
        v += cost_fast(aux + (int64_t)P.obs_pose[o] * kAux, X, uv.x, uv.y, P.intr,
                       P.obs_info ? P.obs_info + 4 * o : nullptr, P.loss);
    }
    v = block_sum(v, sh);
    if (threadIdx.x == 0) red[blockIdx.x] = v;
}

// target: 0 = chi2_new, 1 = scale (+1e-3)
__global__ void __launch_bounds__(kThreads) k_finish_sum(const double* red, LmState* st, int target, int only_if_ok) {
    __shared__ double sh[kThreads];
    if (only_if_ok && !st->solve_ok) return;
    double v = 0.0;
    for (int i = threadIdx.x; i < kReduceBlocks; i += kThreads) v += red[i];
    v = block_sum(v, sh);
    if (threadIdx.x == 0) {
        if (target == 0) st->chi2_new = v;
        else st->scale = v + 1e-3;
    }
}

__global__ void __launch_bounds__(kThreads) k_max_diag(DevProblem P, const double* __restrict__ hpp,
                                                       const double* __restrict__ hll, double* red) {
    __shared__ double sh[kThreads];
    double m = 0.0;
    const int64_t N = 6LL * P.K + 3LL * P.L;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x) {
        double v;
        if (i < 6LL * P.K) v = hpp[(i / 6) * 36 + (i % 6) * 7];
        else {
            const int64_t j = i - 6LL * P.K;
            v = hll[(j / 3) * 9 + (j % 3) * 4];
        }
        m = fmax(fabs(v), m);
    }
    sh[threadIdx.x] = m;
    __syncthreads();
    for (int s = kThreads / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) sh[threadIdx.x] = fmax(sh[threadIdx.x], sh[threadIdx.x + s]);
        __syncthreads();
    }
    if (threadIdx.x == 0) red[blockIdx.x] = sh[0];
}

__global__ void k_init_lambda(const double* red, LmState* st, double tau, double clamp) {
    if (threadIdx.x != 0) return;
    double m = 0.0;
    for (int i = 0; i < kReduceBlocks; ++i) m = fmax(m, red[i]);
    st->max_diag = m;
    st->lambda = tau * fmin(clamp, m);
    st->nu = 2.0;
    st->chi2 = st->chi2_new;
}

// source/factor_graph.hpp:542-591
__global__ void k_decide(LmState* st) {
    if (threadIdx.x != 0) return;
    if (!st->solve_ok) {
        st->lambda *= st->nu;
        st->nu *= 2.0;
        st->good = 0;
        return;
    }
    const double rho = (st->chi2 - st->chi2_new) / st->scale;
    st->rho = rho;
    if ((rho > 0) && isfinite(st->chi2_new)) {
        double alpha = 1.0 - pow(2.0 * rho - 1.0, 3.0);
        alpha = fmin(alpha, 2.0 / 3.0);
        st->lambda *= fmax(1.0 / 3.0, alpha);
        st->nu = 2.0;
        st->chi2 = st->chi2_new;
        st->good = 1;
    } else {
        st->lambda *= st->nu;
        st->nu *= 2.0;
        st->good = 0;
    }
}

__global__ void k_set_solve_ok(LmState* st, int v) {
    if (threadIdx.x == 0) {
        st->solve_ok = v;
        st->timeout = 0;
    }
}

// ------------------------------------------------------------------ launchers

long long& launch_counter() {
    static long long count = 0;
    return count;
}

// Landmark count from which the mixed form's H_ll / b_l sums run a thread per
// landmark (measured: 25 ns per observation at 400,000 landmarks against 72 ns
// for the warp scan, 98 against 75 at 50,000).
constexpr int kLmThreadMin = 65536;

template <typename T>
void launch_linearize(const DevProblem& P, DevWork& W, cudaStream_t s) {
    if (sizeof(T) == 4 && P.K > 0) {
        k_pose_aux<<<grid_for(P.K), kThreads, 0, s>>>(P, W.pose_aux); note_launch();
    }
    if (P.M > 0) {
        k_linearize<T><<<grid_for(P.M), kThreads, 0, s>>>(P, (T*)W.hpl, (T*)W.lm_part, (T*)W.pose_part, W.pose_aux,
                                                          W.jac, P.pose_win ? nullptr : W.jp_pm); note_launch();
        if (P.has_dups) { k_merge_dups<T><<<grid_for(P.M), kThreads, 0, s>>>(P, (T*)W.hpl); note_launch(); }
    }
    if (P.L > 0) {
        if (sizeof(T) == 4) {
            // a thread per landmark when they fill the GPU, else warps over chunks
            if (P.L >= kLmThreadMin) k_reduce_lm_jac_thread<<<grid_for(P.L), kThreads, 0, s>>>(P, W.jac, W.hll, W.b);
            else k_reduce_lm_jac<<<grid_for(32 * P.nlmch), kThreads, 0, s>>>(P, W.jac, W.hll, W.b);
        }
        else k_reduce_lm<T><<<grid_for(P.L), kThreads, 0, s>>>(P, (const T*)W.lm_part, W.hll, W.b);
        note_launch();
    }
    if (P.K > 0) {
        if constexpr (sizeof(T) == 4)
            k_reduce_pose_runs<<<P.K, kThreads, 0, s>>>(P, (const float*)W.pose_part, W.hpp, W.b);
        else
            k_reduce_pose<T><<<P.K, kThreads, 0, s>>>(P, (const T*)W.pose_part, W.hpp, W.b);
        note_launch();
    }
}

template <typename T>
void launch_invert_w(const DevProblem& P, DevWork& W, const LmState* st, cudaStream_t s) {
    if (P.L > 0) {
        k_invert<<<grid_for(P.L), kThreads, 0, s>>>(P, W.hll, W.hll_inv, sizeof(T) == 4 ? W.hll_inv_f : nullptr, st);
        note_launch();
    }
    if (P.M > 0) {
        k_w<T><<<grid_for(P.M), kThreads, 0, s>>>(P, (const T*)W.hpl, W.hll_inv, W.hll_inv_f, (T*)W.W);
        note_launch();
    }
}

template <typename T>
void launch_schur_pairs(const DevProblem& P, DevWork& W, const WinCtl* ctl, cudaStream_t s) {
    if (P.npairs > 0) {
        constexpr int nt = schur_seg_threads<T>();
        const int64_t blocks = (P.nsegs * 32 + nt - 1) / nt;
        k_schur_segments<T><<<(int)blocks, nt, 0, s>>>(P, (const T*)W.W, (const T*)W.hpl, W.partial, ctl);
        note_launch();
        k_schur_assemble<<<grid_for((int64_t)P.npairs * 36), kThreads, 0, s>>>(P, W.partial, W.S, ctl);
        note_launch();
    }
}

template <typename T>
void launch_schur(const DevProblem& P, DevWork& W, const LmState* st, cudaStream_t s) {
    const int64_t nn = (int64_t)P.n * P.n;
    if (nn > 0) { k_s_init<<<grid_for(nn), kThreads, 0, s>>>(P, W.hpp, (double*)W.S, st); note_launch(); }
    launch_schur_pairs<T>(P, W, nullptr, s);
    // (the mixed form's b_s comes from its FP64 operator, launch_pcg)
    if (sizeof(T) == 8) launch_bs<T>(P, W, s);
}

template <typename T>
void launch_bs(const DevProblem& P, DevWork& W, cudaStream_t s) {
    if (P.K >= 1024) {
        k_bs_per_pose<T><<<P.K, kThreads, 0, s>>>(P, (const T*)W.W, W.b, W.bs);
        note_launch();
    } else {
        launch_pose_sums6(P, W.opch_sum, BsTerm<T>{(const T*)W.W, W.b}, BsOut{W.b, W.bs}, s);
    }
}

template <typename T>
void launch_w(const DevProblem& P, DevWork& W, cudaStream_t s) {
    if (P.M > 0) {
        k_w<T><<<grid_for(P.M), kThreads, 0, s>>>(P, (const T*)W.hpl, W.hll_inv, W.hll_inv_f, (T*)W.W);
        note_launch();
    }
}


template <typename T>
void launch_backsub(const DevProblem& P, DevWork& W, const LmState* st, cudaStream_t s) {
    if (P.L > 0) {
        k_backsub<T><<<grid_for(32LL * P.L), kThreads, 0, s>>>(P, (const T*)W.hpl, W.hll_inv, W.b, W.delta, st);
        note_launch();
    }
}

void launch_update(const DevProblem& P, DevWork& W, const LmState* st, cudaStream_t s) {
    k_update<<<grid_for((int64_t)P.K + P.L), kThreads, 0, s>>>(P, W.delta, st); note_launch();
}

void launch_rollback(const DevProblem& P, const LmState* st, cudaStream_t s) {
    k_rollback<<<grid_for((int64_t)P.K + P.L), kThreads, 0, s>>>(P, st); note_launch();
}

void launch_scale(const DevProblem& P, DevWork& W, LmState* st, cudaStream_t s) {
    k_scale_partial<<<kReduceBlocks, kThreads, 0, s>>>(P, W.delta, W.b, W.red, st); note_launch();
    k_finish_sum<<<1, kThreads, 0, s>>>(W.red, st, 1, 1); note_launch();
}

void launch_cost(const DevProblem& P, DevWork& W, LmState* st, bool only_if_ok, cudaStream_t s) {
    k_cost_partial<<<kReduceBlocks, kThreads, 0, s>>>(P, W.red, st, only_if_ok ? 1 : 0); note_launch();
    k_finish_sum<<<1, kThreads, 0, s>>>(W.red, st, 0, only_if_ok ? 1 : 0); note_launch();
}

void launch_pose_aux(const DevProblem& P, DevWork& W, cudaStream_t s) {
    if (P.K > 0) { k_pose_aux<<<grid_for(P.K), kThreads, 0, s>>>(P, W.pose_aux); note_launch(); }
}

void launch_cost_fast(const DevProblem& P, DevWork& W, LmState* st, bool only_if_ok, cudaStream_t s) {
    launch_pose_aux(P, W, s);
    k_cost_partial_fast<<<kReduceBlocks, kThreads, 0, s>>>(P, W.pose_aux, W.red, st, only_if_ok ? 1 : 0); note_launch();
    k_finish_sum<<<1, kThreads, 0, s>>>(W.red, st, 0, only_if_ok ? 1 : 0); note_launch();
}

void launch_init_lambda(const DevProblem& P, DevWork& W, LmState* st, double tau, double clamp, cudaStream_t s) {
    k_max_diag<<<kReduceBlocks, kThreads, 0, s>>>(P, W.hpp, W.hll, W.red); note_launch();
    k_init_lambda<<<1, 32, 0, s>>>(W.red, st, tau, clamp); note_launch();
}

void launch_decide(LmState* st, cudaStream_t s) { k_decide<<<1, 32, 0, s>>>(st); note_launch(); }

void launch_set_solve_ok(LmState* st, int v, cudaStream_t s) { k_set_solve_ok<<<1, 32, 0, s>>>(st, v); note_launch(); }

template void launch_linearize<double>(const DevProblem&, DevWork&, cudaStream_t);
template void launch_linearize<float>(const DevProblem&, DevWork&, cudaStream_t);
template void launch_invert_w<double>(const DevProblem&, DevWork&, const LmState*, cudaStream_t);
template void launch_invert_w<float>(const DevProblem&, DevWork&, const LmState*, cudaStream_t);
template void launch_schur<double>(const DevProblem&, DevWork&, const LmState*, cudaStream_t);
template void launch_schur<float>(const DevProblem&, DevWork&, const LmState*, cudaStream_t);
template void launch_backsub<double>(const DevProblem&, DevWork&, const LmState*, cudaStream_t);
template void launch_bs<double>(const DevProblem&, DevWork&, cudaStream_t);
template void launch_bs<float>(const DevProblem&, DevWork&, cudaStream_t);
template void launch_w<double>(const DevProblem&, DevWork&, cudaStream_t);
template void launch_w<float>(const DevProblem&, DevWork&, cudaStream_t);
template void launch_schur_pairs<double>(const DevProblem&, DevWork&, const WinCtl*, cudaStream_t);
template void launch_schur_pairs<float>(const DevProblem&, DevWork&, const WinCtl*, cudaStream_t);

}  // namespace zs
