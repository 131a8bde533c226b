// Device-side geometry, camera and loss math shared by the bundle-adjustment
// kernels, plus small launch and error helpers.
//
// Formulas follow zeroslam (paths inside gpdaniels/zeroslam):
//   quaternion product / rotation      source/lie.hpp:337-362
//   rotation matrix of a quaternion    source/lie.hpp:188-204
//   so3::exp, so3::left_jacobian       source/lie.hpp:247-264, 284-294
//   pinhole projection + Jacobian      source/camera.hpp:91-126
//   residual / Jacobians / penalty     source/factor_graph.hpp:981, 990-1048
//   robust losses                      source/factor_graph.hpp:851-934
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace zs {

constexpr double kBehindPenalty = 0.3;  // source/factor_graph.hpp:981
constexpr int kThreads = 256;
constexpr int kReduceBlocks = 304;      // 2 x 152 SMs; fixed so reductions are reproducible

struct Intrinsics {
    double fx, fy, cx, cy;
};

struct LossParams {
    int kind;
    double delta;
};

// Pose stored on the device as 8 doubles: tx ty tz qx qy qz qw pad.
constexpr int kPoseStride = 8;
// Landmark stored as 4 doubles: x y z pad.
constexpr int kLmStride = 4;

__host__ __device__ inline void quat_mul(const double a[4], const double b[4], double o[4]) {
    o[0] = a[0] * b[0] - a[1] * b[1] - a[2] * b[2] - a[3] * b[3];
    o[1] = a[0] * b[1] + a[1] * b[0] + a[2] * b[3] - a[3] * b[2];
    o[2] = a[0] * b[2] - a[1] * b[3] + a[2] * b[0] + a[3] * b[1];
    o[3] = a[0] * b[3] + a[1] * b[2] - a[2] * b[1] + a[3] * b[0];
}

// q (0, p) q* for an unnormalised quaternion (w, x, y, z).
__host__ __device__ inline void quat_rotate(const double q[4], const double p[3], double o[3]) {
    const double pq[4] = {0.0, p[0], p[1], p[2]};
    const double qc[4] = {q[0], -q[1], -q[2], -q[3]};
    double t[4], r[4];
    quat_mul(q, pq, t);
    quat_mul(t, qc, r);
    o[0] = r[1];
    o[1] = r[2];
    o[2] = r[3];
}

__host__ __device__ inline void quat_matrix(const double q[4], double R[9]) {
    const double tx = 2.0 * q[1], ty = 2.0 * q[2], tz = 2.0 * q[3];
    const double txx = tx * q[1], txy = tx * q[2], txz = tx * q[3], txw = tx * q[0];
    const double tyy = ty * q[2], tyz = ty * q[3], tyw = ty * q[0];
    const double tzz = tz * q[3], tzw = tz * q[0];
    R[0] = 1.0 - (tyy + tzz); R[1] = txy - tzw;         R[2] = txz + tyw;
    R[3] = txy + tzw;         R[4] = 1.0 - (txx + tzz); R[5] = tyz - txw;
    R[6] = txz - tyw;         R[7] = tyz + txw;         R[8] = 1.0 - (txx + tyy);
}

__device__ inline void so3_exp(const double w[3], double q[4]) {
    const double th2 = w[0] * w[0] + w[1] * w[1] + w[2] * w[2];
    double re, sc;
    if (th2 < 1e-12) {
        const double th4 = th2 * th2;
        re = 1.0 - (1.0 / 8.0) * th2 + (1.0 / 384.0) * th4;
        sc = 0.5 - (1.0 / 48.0) * th2 + (1.0 / 3840.0) * th4;
    } else {
        const double th = sqrt(th2);
        double s, c;
        sincos(0.5 * th, &s, &c);
        re = c;
        sc = s / th;
    }
    q[0] = re;
    q[1] = w[0] * sc;
    q[2] = w[1] * sc;
    q[3] = w[2] * sc;
}

__device__ inline void so3_left_jacobian(const double w[3], double J[9]) {
    const double th2 = w[0] * w[0] + w[1] * w[1] + w[2] * w[2];
    const double H[9] = {0.0, -w[2], w[1], w[2], 0.0, -w[0], -w[1], w[0], 0.0};
    double a, b;
    if (th2 < 1e-12) {
        a = 0.5;
        b = 1.0 / 6.0;
    } else {
        const double th = sqrt(th2);
        double s, c;
        sincos(th, &s, &c);
        a = (1.0 - c) / th2;
        b = (th - s) / (th2 * th);
    }
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            const double h2 = H[i * 3 + 0] * H[0 * 3 + j] + H[i * 3 + 1] * H[1 * 3 + j] + H[i * 3 + 2] * H[2 * 3 + j];
            J[i * 3 + j] = ((i == j) ? 1.0 : 0.0) + a * H[i * 3 + j] + b * h2;
        }
}

// T <- exp(d) * T for pose p[8] (tx ty tz qx qy qz qw), d = (omega, upsilon):
// vertex_pose::plus, source/factor_graph.hpp:947-960.
__device__ inline void pose_plus(double* p, const double d[6]) {
    const double q[4] = {p[6], p[3], p[4], p[5]};
    const double t[3] = {p[0], p[1], p[2]};
    double dq[4], J[9], nq[4], rt[3];
    so3_exp(d, dq);
    so3_left_jacobian(d, J);
    const double dt0 = J[0] * d[3] + J[1] * d[4] + J[2] * d[5];
    const double dt1 = J[3] * d[3] + J[4] * d[4] + J[5] * d[5];
    const double dt2 = J[6] * d[3] + J[7] * d[4] + J[8] * d[5];
    quat_mul(dq, q, nq);
    quat_rotate(dq, t, rt);
    p[0] = rt[0] + dt0;
    p[1] = rt[1] + dt1;
    p[2] = rt[2] + dt2;
    p[3] = nq[1];
    p[4] = nq[2];
    p[5] = nq[3];
    p[6] = nq[0];
}

// Separately rounded IEEE operations (never fused into an FMA). The
// residual and the squared error go through these so that every edge's
// residual rounds exactly as the reference's double arithmetic does: the
// reference's robust-weight branch (source/factor_graph.hpp:265) is decided
// by rounding for Huber outliers, and reproducing it needs identical inputs.
__device__ __forceinline__ double rmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double radd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double rsub(double a, double b) { return __dsub_rn(a, b); }

__device__ inline void quat_mul_rn(const double a[4], const double b[4], double o[4]) {
    o[0] = rsub(rsub(rsub(rmul(a[0], b[0]), rmul(a[1], b[1])), rmul(a[2], b[2])), rmul(a[3], b[3]));
    o[1] = rsub(radd(radd(rmul(a[0], b[1]), rmul(a[1], b[0])), rmul(a[2], b[3])), rmul(a[3], b[2]));
    o[2] = radd(radd(rsub(rmul(a[0], b[2]), rmul(a[1], b[3])), rmul(a[2], b[0])), rmul(a[3], b[1]));
    o[3] = radd(rsub(radd(rmul(a[0], b[3]), rmul(a[1], b[2])), rmul(a[2], b[1])), rmul(a[3], b[0]));
}

// Camera-frame point of landmark X under pose p; returns 1 when it projects
// (Z >= 1e-12) and writes the residual uv - pi(Xc), else the penalty
// (-0.3 Z, -0.3 Z). Rounded operation by operation as the reference.
__device__ inline int residual(const double* p, const double* X, double u_obs, double v_obs, const Intrinsics& in,
                               double Xc[3], double r[2]) {
    const double q[4] = {p[6], p[3], p[4], p[5]};
    const double pq[4] = {0.0, X[0], X[1], X[2]};
    const double qc[4] = {q[0], -q[1], -q[2], -q[3]};
    double t[4], o[4];
    quat_mul_rn(q, pq, t);
    quat_mul_rn(t, qc, o);
    Xc[0] = radd(o[1], p[0]);
    Xc[1] = radd(o[2], p[1]);
    Xc[2] = radd(o[3], p[2]);
    if (Xc[2] < 1.0e-12) {
        const double pen = rmul(-kBehindPenalty, Xc[2]);
        r[0] = pen;
        r[1] = pen;
        return 0;
    }
    const double iz = 1.0 / Xc[2];
    r[0] = rsub(u_obs, radd(rmul(in.fx, rmul(Xc[0], iz)), in.cx));
    r[1] = rsub(v_obs, radd(rmul(in.fy, rmul(Xc[1], iz)), in.cy));
    return 1;
}

// rho[0..2] of the shared robust loss.
__device__ inline void loss_rho(const LossParams& L, double e2, double rho[3]) {
    const double d = L.delta;
    const double d2 = d * d;
    if (L.kind == 1) {
        if (e2 <= d2) {
            rho[0] = e2; rho[1] = 1.0; rho[2] = 0.0;
        } else {
            const double e = sqrt(e2);
            rho[0] = 2.0 * e * d - d2;
            rho[1] = d / e;
            rho[2] = -0.5 * rho[1] / e2;
        }
    } else if (L.kind == 2) {
        const double inv = 1.0 / d2;
        const double aux = inv * e2 + 1.0;
        rho[0] = d2 * log(aux);
        rho[1] = 1.0 / aux;
        rho[2] = -inv * (rho[1] * rho[1]);
    } else if (L.kind == 3) {
        if (e2 <= d2) {
            const double aux = e2 / d2;
            const double om = 1.0 - aux;
            const double om2 = om * om;
            rho[0] = d2 * (1.0 - om2 * om) / 3.0;
            rho[1] = om2;
            rho[2] = -2.0 * om / d2;
        } else {
            rho[0] = d2 / 3.0; rho[1] = 0.0; rho[2] = 0.0;
        }
    } else {
        rho[0] = e2; rho[1] = 1.0; rho[2] = 0.0;
    }
}

// r^T Omega r with Omega row-major (identity when om == nullptr), rounded
// as the reference's (r^T Omega) r.
__device__ inline double chi2_of(const double r[2], const double* om) {
    if (!om) return radd(rmul(r[0], r[0]), rmul(r[1], r[1]));
    const double a = radd(rmul(r[0], om[0]), rmul(r[1], om[2]));
    const double b = radd(rmul(r[0], om[1]), rmul(r[1], om[3]));
    return radd(rmul(a, r[0]), rmul(b, r[1]));
}

// Per-pose data of the mixed form (k_pose_aux): the quaternion-sandwich
// matrix M (M X = q (0, X) q*, valid for unnormalised q), the translation,
// the rotation matrix of source/lie.hpp:188-204, pad.
constexpr int kPoseAux = 24;

// Squared error (or robust cost) of one observation from the per-pose data,
// in FP64 with contracted multiply-adds: the mixed form's cost. Same
// quantities as residual() + chi2_of(), without the reference's operation
// order.
__device__ inline double cost_fast(const double* __restrict__ a, const double* __restrict__ X, double u_obs,
                                   double v_obs, const Intrinsics& in, const double* om, const LossParams& loss);

// matrix::invert<3> of H_ll + lambda I for one landmark
// (source/matrix.hpp:749-774): fixed landmarks and singular blocks
// (|det| <= 1e-12 max|a|^3) get a zero inverse, as solve_linear_system
// ignores the failed inversion (source/factor_graph.hpp:763). of (optional,
// mixed form) also receives the inverse in FP32, padded to 12 floats.
__device__ inline void landmark_inverse(const double* __restrict__ hll_l, double lam, bool fixed, double* o,
                                        float* of) {
    double v[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    if (!fixed) {
        double a[9];
#pragma unroll
        for (int i = 0; i < 9; ++i) a[i] = hll_l[i];
        a[0] += lam; a[4] += lam; a[8] += lam;
        const double det = +a[0] * (a[4] * a[8] - a[7] * a[5]) - a[1] * (a[3] * a[8] - a[5] * a[6]) +
                           a[2] * (a[3] * a[7] - a[4] * a[6]);
        double scale = 0.0;
#pragma unroll
        for (int i = 0; i < 9; ++i) scale = fmax(scale, fabs(a[i]));
        if (fabs(det) > scale * scale * scale * 1e-12) {
            const double id = 1.0 / det;
            v[0] = (a[4] * a[8] - a[7] * a[5]) * id;
            v[1] = (a[2] * a[7] - a[1] * a[8]) * id;
            v[2] = (a[1] * a[5] - a[2] * a[4]) * id;
            v[3] = (a[5] * a[6] - a[3] * a[8]) * id;
            v[4] = (a[0] * a[8] - a[2] * a[6]) * id;
            v[5] = (a[3] * a[2] - a[0] * a[5]) * id;
            v[6] = (a[3] * a[7] - a[6] * a[4]) * id;
            v[7] = (a[6] * a[1] - a[0] * a[7]) * id;
            v[8] = (a[0] * a[4] - a[3] * a[1]) * id;
        }
    }
#pragma unroll
    for (int i = 0; i < 9; ++i) o[i] = v[i];
    if (of) {
        float4* f = reinterpret_cast<float4*>(of);
        f[0] = make_float4((float)v[0], (float)v[1], (float)v[2], (float)v[3]);
        f[1] = make_float4((float)v[4], (float)v[5], (float)v[6], (float)v[7]);
        f[2] = make_float4((float)v[8], 0.f, 0.f, 0.f);
    }
}

// Deterministic block sum of one value per thread (fixed tree over
// blockDim.x = kThreads threads). Result valid in thread 0.
template <typename V>
__device__ inline V block_sum(V v, V* sh) {
    const int t = threadIdx.x;
    sh[t] = v;
    __syncthreads();
#pragma unroll
    for (int s = kThreads / 2; s > 0; s >>= 1) {
        if (t < s) sh[t] = sh[t] + sh[t + s];
        __syncthreads();
    }
    const V out = sh[0];
    __syncthreads();
    return out;
}

// Kernels launched by this library in this process (all handles); a solve
// reports the difference over its duration.
long long& launch_counter();
inline void note_launch(int n = 1) { launch_counter() += n; }

inline int grid_for(long long n, int threads = kThreads) {
    long long g = (n + threads - 1) / threads;
    if (g < 1) g = 1;
    return static_cast<int>(g);
}

__device__ inline double cost_fast(const double* __restrict__ a, const double* __restrict__ X, double u_obs,
                                   double v_obs, const Intrinsics& in, const double* om, const LossParams& loss) {
    const double xc = fma(a[0], X[0], fma(a[1], X[1], fma(a[2], X[2], a[9])));
    const double yc = fma(a[3], X[0], fma(a[4], X[1], fma(a[5], X[2], a[10])));
    const double zc = fma(a[6], X[0], fma(a[7], X[1], fma(a[8], X[2], a[11])));
    double r[2];
    if (zc < 1.0e-12) {
        r[0] = r[1] = -kBehindPenalty * zc;
    } else {
        const double iz = 1.0 / zc;
        r[0] = u_obs - fma(in.fx, xc * iz, in.cx);
        r[1] = v_obs - fma(in.fy, yc * iz, in.cy);
    }
    double e2;
    if (!om) {
        e2 = fma(r[0], r[0], r[1] * r[1]);
    } else {
        const double p = fma(r[0], om[0], r[1] * om[2]);
        const double q = fma(r[0], om[1], r[1] * om[3]);
        e2 = fma(p, r[0], q * r[1]);
    }
    if (!loss.kind) return e2;
    double rho[3];
    loss_rho(loss, e2, rho);
    return rho[0];
}

}  // namespace zs
