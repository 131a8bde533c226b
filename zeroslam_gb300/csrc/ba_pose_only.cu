// Pose-only problems (every landmark fixed: zeroslam's tracking mode,
// map optimise(1, true, 50), source/slam.hpp:316,387,469) solved in one
// cooperative launch that runs the whole Levenberg-Marquardt loop of
// factor_graph::solve (source/factor_graph.hpp:489-615) on the device, with no
// host round trip per attempt.
//
// With every landmark fixed the landmark blocks vanish: no H_ll, no H_pl, and
// the reduced system is H_pp + lambda I, block diagonal with one 6 x 6 block
// per pose. Per attempt:
//   * every CTA sums its share of each pose's observations into 27 terms
//     (J_p^T W J_p upper triangle and -J_p^T g, each observation's terms
//     formed exactly as the plain form's k_linearize forms them); after a
//     grid barrier a warp per sum adds the CTAs' partials (lanes over the
//     CTAs, then a butterfly), and after another every CTA reads the sums;
//   * every CTA factors the damped 6 x 6 blocks (a thread per pose) with the
//     reference's pivot test (d > 1e-14 max |S_ii|,
//     source/matrix_decomposition_cholesky.hpp:41-57) and solve test
//     (|L_ii| > 1e-7 max |L_ii|, :74-89) and solves for the step: the same
//     arithmetic on the same values in every CTA, so all of them take the
//     same decisions without exchanging them;
//   * CTA 0 backs up and updates the poses (pose_plus); after a barrier the
//     CTAs evaluate the trial cost (per-CTA partials, then every CTA adds
//     them the same way), take the reference's accept / reject decision
//     (source/factor_graph.hpp:542-606) and CTA 0 rolls a rejected step back.
// The FP64 pipe of one SM is far too slow for the per-observation work on
// GB300 (measured: one CTA took 1.30 ms for a 6,802-observation tracking
// solve, the general path 0.81 ms), hence the whole grid. The outer loop, its
// stopping rules and the attempt history follow the host loop of the general
// path (solve_impl). Both precisions take this path in FP64: there is no
// Schur complement or dense factor to make cheaper. Every sum has a fixed
// order for a given grid size: results repeat bit for bit.
//
// Batches of such windows (many tracking problems at once) run the same loop
// with one CTA per window (k_pose_only_windows): the window's sums stay in
// its CTA, and the loop is shared with the single-problem kernel through a
// team type (GridTeam / WindowTeam: who sums, who synchronises).
#include <cooperative_groups.h>

#include <algorithm>

#include "../../include/zeroslam_ba.h"
#include "ba_internal.h"

namespace cg = cooperative_groups;

namespace zs {

namespace {

constexpr int kPoWarps = kThreads / 32;

__constant__ int8_t kPoUp6[21][2] = {{0, 0}, {0, 1}, {0, 2}, {0, 3}, {0, 4}, {0, 5}, {1, 1}, {1, 2}, {1, 3}, {1, 4},
                                      {1, 5}, {2, 2}, {2, 3}, {2, 4}, {2, 5}, {3, 3}, {3, 4}, {3, 5}, {4, 4}, {4, 5},
                                      {5, 5}};
__constant__ int kDiag6[6] = {0, 6, 11, 15, 18, 20};  // the diagonal's places in that order

// Observation o's 27 pose terms: J_p^T W J_p (upper triangle, row by row)
// and -J_p^T g, formed as the plain form's k_linearize forms them.
__device__ void pose_record(const DevProblem& P, int64_t o, double rec[27]) {
    const int pi = P.obs_pose[o], li = P.obs_lm[o];
    const double* pp = P.pose + (int64_t)pi * kPoseStride;
    const double* xp = P.lm + (int64_t)li * kLmStride;
    const double2 uv = P.obs_uv[o];
    const double* om = P.obs_info ? P.obs_info + 4 * o : nullptr;
    double p[7], X[3], Xc[3], r[2], Jc[6];
#pragma unroll
    for (int i = 0; i < 7; ++i) p[i] = pp[i];
#pragma unroll
    for (int i = 0; i < 3; ++i) X[i] = xp[i];
    const int front = residual(p, X, uv.x, uv.y, P.intr, Xc, r);
    if (front) {
        const double iz = 1.0 / Xc[2];
        const double iz2 = iz * iz;
        const double fx = P.intr.fx, fy = P.intr.fy;
        Jc[0] = fx * iz; Jc[1] = 0.0; Jc[2] = -fx * Xc[0] * iz2;
        Jc[3] = 0.0; Jc[4] = fy * iz; Jc[5] = -fy * Xc[1] * iz2;
    } else {
        Jc[0] = 0.0; Jc[1] = 0.0; Jc[2] = kBehindPenalty;
        Jc[3] = 0.0; Jc[4] = 0.0; Jc[5] = kBehindPenalty;
    }
    const double Xv = Xc[0], Yv = Xc[1], Zv = Xc[2];
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
        // rho' + 2 rho'' e2 as separately rounded multiply and add (no FMA),
        // as the reference evaluates it (its sign decides the rank-one term)
        if (__dadd_rn(rho[1], __dmul_rn(2.0 * rho[2], e2)) > 0.0) {
            const double k2 = 2.0 * rho[2];
            Wd[0] += k2 * orr0 * orr0;
            Wd[1] += k2 * orr0 * orr1;
            Wd[2] += k2 * orr1 * orr0;
            Wd[3] += k2 * orr1 * orr1;
        }
    }
    double Jp[12];
#pragma unroll
    for (int rr = 0; rr < 2; ++rr) {
        const double c0 = Jc[rr * 3], c1 = Jc[rr * 3 + 1], c2 = Jc[rr * 3 + 2];
        Jp[rr * 6 + 0] = -(c2 * Yv - c1 * Zv);
        Jp[rr * 6 + 1] = -(c0 * Zv - c2 * Xv);
        Jp[rr * 6 + 2] = -(c1 * Xv - c0 * Yv);
        Jp[rr * 6 + 3] = -c0;
        Jp[rr * 6 + 4] = -c1;
        Jp[rr * 6 + 5] = -c2;
    }
    const double g0 = drho * orr0, g1 = drho * orr1;
    double A0[6], A1[6];
#pragma unroll
    for (int a = 0; a < 6; ++a) {
        A0[a] = Jp[a] * Wd[0] + Jp[6 + a] * Wd[2];
        A1[a] = Jp[a] * Wd[1] + Jp[6 + a] * Wd[3];
    }
#pragma unroll
    for (int k = 0; k < 21; ++k) {
        const int a = kPoUp6[k][0], c = kPoUp6[k][1];
        rec[k] = A0[a] * Jp[c] + A1[a] * Jp[6 + c];
    }
#pragma unroll
    for (int a = 0; a < 6; ++a) rec[21 + a] = -(Jp[a] * g0 + Jp[6 + a] * g1);
}

// Observation o's cost term (k_cost_partial's).
__device__ double obs_cost(const DevProblem& P, int64_t o) {
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
        return rho[0];
    }
    return e2;
}

struct Shared {
    double H[kPoseOnlyMaxK][27];      // per pose: the 21 upper entries of J^T W J, then b
    double delta[kPoseOnlyMaxK][6];
    double bk[kPoseOnlyMaxK][kPoseStride];
    double wpart[kPoWarps][27];
    double red[kThreads];
    double lambda, nu, chi2, rho;
    int solve_ok, good;
};

// Warp butterflies and the warps in order: the CTA's 27 sums into
// sh.wpart[0]. Threads from `active` on took no observation: the warps made
// of them skip their FP64 butterflies and give the zeros those would give.
__device__ void cta_sum27(double acc[27], int active, Shared& sh) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (warp * 32 < active) {
#pragma unroll
        for (int e = 0; e < 27; ++e) {
            double v = acc[e];
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
            if (lane == 0) sh.wpart[warp][e] = v;
        }
    } else if (lane < 27) {
        sh.wpart[warp][lane] = 0.0;
    }
    __syncthreads();
    if (threadIdx.x < 27) {
        double v = 0.0;
        for (int w = 0; w < kPoWarps; ++w) v += sh.wpart[w][threadIdx.x];
        sh.wpart[0][threadIdx.x] = v;  // (warp 0's slot, read only after the barrier below)
    }
    __syncthreads();
}

// H and b of every pose at the current state into sh.H (every CTA).
// part: [G][K][27] per-CTA partials, sums: [K][27].
__device__ void assemble(cg::grid_group& grid, const DevProblem& P, Shared& sh, double* part, double* sums) {
    const int G = gridDim.x, c = blockIdx.x;
    for (int k = 0; k < P.K; ++k) {
        if (P.pose_fixed[k]) continue;  // (uniform) a fixed pose's sums are zero
        double acc[27];
#pragma unroll
        for (int e = 0; e < 27; ++e) acc[e] = 0.0;
        const int q0 = P.pose_ptr[k], q1 = P.pose_ptr[k + 1];
        for (int q = q0 + c * blockDim.x + threadIdx.x; q < q1; q += G * blockDim.x) {
            double rec[27];
            pose_record(P, P.pose_obs[q], rec);
#pragma unroll
            for (int e = 0; e < 27; ++e) acc[e] += rec[e];
        }
        const int span = q1 - (q0 + c * (int)blockDim.x);  // this CTA's first pass covers min(span, blockDim)
        cta_sum27(acc, span <= 0 ? 0 : min(span, (int)blockDim.x), sh);
        if (threadIdx.x < 27) part[((int64_t)c * P.K + k) * 27 + threadIdx.x] = sh.wpart[0][threadIdx.x];
        __syncthreads();
    }
    grid.sync();
    // entry i of the 27 K sums: a warp adds the G partials, lane l those of
    // CTAs l, l + 32, ..., then a butterfly (a fixed order for a given G)
    {
        const int lane = threadIdx.x & 31, nw = blockDim.x >> 5;
        for (int i = c * nw + (threadIdx.x >> 5); i < 27 * P.K; i += G * nw) {
            double v = 0.0;
            if (!P.pose_fixed[i / 27])
                for (int b = lane; b < G; b += 32) v += __ldcg(part + (int64_t)b * 27 * P.K + i);
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
            if (lane == 0) sums[i] = v;
        }
    }
    grid.sync();
    for (int i = threadIdx.x; i < 27 * P.K; i += blockDim.x) sh.H[i / 27][i % 27] = __ldcg(sums + i);
    __syncthreads();
}

// The cost at the current state (every CTA gets the same value).
__device__ double cost(cg::grid_group& grid, const DevProblem& P, Shared& sh, double* cpart) {
    const int G = gridDim.x;
    double v = 0.0;
    for (int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o < P.M; o += (int64_t)G * blockDim.x)
        v += obs_cost(P, o);
    v = block_sum(v, sh.red);
    if (threadIdx.x == 0) cpart[blockIdx.x] = v;
    grid.sync();
    // every warp adds the G partials the same way: lane l those of CTAs l,
    // l + 32, ..., then a butterfly
    double t = 0.0;
    for (int b = threadIdx.x & 31; b < G; b += 32) t += __ldcg(cpart + b);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) t += __shfl_xor_sync(0xffffffffu, t, off);
    return t;
}

__device__ double cta_max(double v, double* red) {
    red[threadIdx.x] = v;
    __syncthreads();
    for (int s = kThreads / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + s]);
        __syncthreads();
    }
    const double out = red[0];
    __syncthreads();
    return out;
}

// The damped blocks' factors and the step delta (sh.solve_ok, sh.delta).
__device__ void solve_step(int K, Shared& sh) {
    const int k = threadIdx.x;
    const bool mine = k < K;
    const double lam = sh.lambda;
    double a[6][6];
#pragma unroll
    for (int i = 0; i < 6; ++i)
#pragma unroll
        for (int j = 0; j < 6; ++j) a[i][j] = 0.0;
    double dmax = 0.0;
    if (mine) {
#pragma unroll
        for (int e = 0; e < 21; ++e) {
            const int i = kPoUp6[e][0], j = kPoUp6[e][1];
            a[i][j] = sh.H[k][e];
            a[j][i] = sh.H[k][e];
        }
#pragma unroll
        for (int i = 0; i < 6; ++i) {
            a[i][i] += lam;
            dmax = fmax(dmax, fabs(a[i][i]));
        }
    }
    const double eps_f = cta_max(dmax, sh.red) * 1e-14;
    int ok = 1;
    double lmax = 0.0;
    if (mine) {
        // right-looking, as the general path's diagonal blocks; after a
        // failed pivot the remaining columns are skipped
#pragma unroll
        for (int c = 0; c < 6; ++c) {
            const double d = a[c][c];
            if (!(d > eps_f)) ok = 0;
            if (ok) {
                const double piv = sqrt(d), inv = 1.0 / piv;
                a[c][c] = piv;
#pragma unroll
                for (int i = c + 1; i < 6; ++i) a[i][c] *= inv;
#pragma unroll
                for (int i = c + 1; i < 6; ++i)
#pragma unroll
                    for (int m = c + 1; m <= i; ++m) a[i][m] -= a[i][c] * a[m][c];
            }
        }
        if (ok)
#pragma unroll
            for (int i = 0; i < 6; ++i) lmax = fmax(lmax, fabs(a[i][i]));
    }
    ok = __syncthreads_and(ok);
    const double eps_s = cta_max(lmax, sh.red) * 1e-7;
    if (ok && mine) {
#pragma unroll
        for (int i = 0; i < 6; ++i)
            if (!(fabs(a[i][i]) > eps_s)) ok = 0;
    }
    ok = __syncthreads_and(ok);
    if (ok && mine) {
        // forward and back substitution with the pivots' reciprocals (FP64
        // division is a long instruction sequence on this GPU's slow FP64 pipe)
        double y[6], x[6], rd[6];
#pragma unroll
        for (int i = 0; i < 6; ++i) rd[i] = 1.0 / a[i][i];
#pragma unroll
        for (int i = 0; i < 6; ++i) {
            double v = sh.H[k][21 + i];
#pragma unroll
            for (int m = 0; m < i; ++m) v -= a[i][m] * y[m];
            y[i] = v * rd[i];
        }
#pragma unroll
        for (int i = 5; i >= 0; --i) {
            double v = y[i];
#pragma unroll
            for (int m = i + 1; m < 6; ++m) v -= a[m][i] * x[m];
            x[i] = v * rd[i];
        }
#pragma unroll
        for (int i = 0; i < 6; ++i) sh.delta[k][i] = x[i];
    }
    if (threadIdx.x == 0) sh.solve_ok = ok;
    __syncthreads();
}

// The window's H and b (its poses k0 .. k1, sh.H[k - k0]) by one CTA.
__device__ void assemble_window(const DevProblem& P, int k0, int k1, Shared& sh) {
    for (int k = k0; k < k1; ++k) {
        if (!P.pose_fixed[k]) {  // (uniform) a fixed pose's sums are zero
            double acc[27];
#pragma unroll
            for (int e = 0; e < 27; ++e) acc[e] = 0.0;
            const int q0 = P.pose_ptr[k], q1 = P.pose_ptr[k + 1];
            for (int q = q0 + threadIdx.x; q < q1; q += blockDim.x) {
                double rec[27];
                pose_record(P, P.pose_obs[q], rec);
#pragma unroll
                for (int e = 0; e < 27; ++e) acc[e] += rec[e];
            }
            cta_sum27(acc, min(max(q1 - q0, 0), (int)blockDim.x), sh);
            if (threadIdx.x < 27) sh.H[k - k0][threadIdx.x] = sh.wpart[0][threadIdx.x];
        } else if (threadIdx.x < 27) {
            sh.H[k - k0][threadIdx.x] = 0.0;
        }
        __syncthreads();
    }
}

// The cost of the window's observations (pose-major positions q0 .. q1), by
// one CTA; every thread gets it.
__device__ double cost_window(const DevProblem& P, int64_t q0, int64_t q1, Shared& sh) {
    double v = 0.0;
    for (int64_t q = q0 + threadIdx.x; q < q1; q += blockDim.x) v += obs_cost(P, P.pose_obs[q]);
    return block_sum(v, sh.red);
}

// Who works on one problem: the whole cooperative grid (a single problem,
// poses 0 .. P.K) or one CTA (a window of a batch, poses k0 .. k0 + K).
struct GridTeam {
    cg::grid_group grid;
    double* part;
    double* sums;
    double* cpart;
    __device__ void sync() { grid.sync(); }
    __device__ bool lead() const { return blockIdx.x == 0; }
    __device__ void assemble(const DevProblem& P, Shared& sh) { zs::assemble(grid, P, sh, part, sums); }
    __device__ double cost(const DevProblem& P, Shared& sh) { return zs::cost(grid, P, sh, cpart); }
};
struct WindowTeam {
    int k0, k1;
    int64_t q0, q1;
    __device__ void sync() { __syncthreads(); }
    __device__ bool lead() const { return true; }
    __device__ void assemble(const DevProblem& P, Shared& sh) { assemble_window(P, k0, k1, sh); }
    __device__ double cost(const DevProblem& P, Shared& sh) { return cost_window(P, q0, q1, sh); }
};

// The Levenberg-Marquardt loop of factor_graph::solve
// (source/factor_graph.hpp:506-615) over poses k0 .. k0 + K (every landmark
// fixed). active = false skips the loop (the window reports no iteration).
// hist (may be null): the attempts, up to ctl.hist_cap. The lead CTA updates
// and restores the poses; every CTA takes the same decisions.
template <typename Team>
__device__ PoseOnlyOut lm_loop(const DevProblem& P, int k0, int K, const PoseOnlyCtl& ctl, bool active, Team& team,
                               Shared& sh, zs_ba_attempt* hist) {
    const int t = threadIdx.x;
    const bool lead = team.lead();
    // the initial system, cost and damping (tau min(clamp, max diag H))
    team.assemble(P, sh);
    const double c0 = team.cost(P, sh);
    double dmax = 0.0;
    if (t < K)
#pragma unroll
        for (int i = 0; i < 6; ++i) dmax = fmax(dmax, fabs(sh.H[t][kDiag6[i]]));
    const double mdiag = cta_max(dmax, sh.red);
    if (t == 0) {
        sh.chi2 = c0;
        sh.lambda = ctl.tau * fmin(ctl.clamp, mdiag);
        sh.nu = 2.0;
    }
    __syncthreads();
    int iterations = 0, attempts = 0, accepted = 0, chol_fail = 0, nhist = 0;
    const double legacy = ctl.legacy_stop * c0;
    for (int it = 0; active && it < ctl.iterations; ++it) {
        iterations = it + 1;
        const double last = sh.chi2;
        int failures = 0;
        while (failures < ctl.max_failures) {
            solve_step(K, sh);
            const bool ok = sh.solve_ok != 0;
            double chi2_new = sh.chi2, scale = 0.0;
            if (ok) {
                // trial state (poses; every landmark is fixed), the model's
                // gain delta^T (lambda delta + b) + 1e-3 and the cost there
                double sc = 0.0;
                if (t < K) {
                    double* pp = P.pose + (int64_t)(k0 + t) * kPoseStride;
#pragma unroll
                    for (int i = 0; i < kPoseStride; ++i) sh.bk[t][i] = pp[i];
#pragma unroll
                    for (int i = 0; i < 6; ++i) {
                        const double d = sh.delta[t][i];
                        sc += d * (sh.lambda * d + sh.H[t][21 + i]);
                    }
                }
                scale = block_sum(sc, sh.red) + 1e-3;
                if (lead && t < K && !P.pose_fixed[k0 + t])
                    pose_plus(P.pose + (int64_t)(k0 + t) * kPoseStride, sh.delta[t]);
                team.sync();  // the trial poses are visible to every CTA
                chi2_new = team.cost(P, sh);
            }
            // source/factor_graph.hpp:542-591 (k_decide), in every CTA
            if (t == 0) {
                if (!ok) {
                    sh.lambda *= sh.nu;
                    sh.nu *= 2.0;
                    sh.good = 0;
                } else {
                    const double rho = (sh.chi2 - chi2_new) / scale;
                    sh.rho = rho;
                    if (rho > 0 && isfinite(chi2_new)) {
                        double alpha = 1.0 - pow(2.0 * rho - 1.0, 3.0);
                        alpha = fmin(alpha, 2.0 / 3.0);
                        sh.lambda *= fmax(1.0 / 3.0, alpha);
                        sh.nu = 2.0;
                        sh.chi2 = chi2_new;
                        sh.good = 1;
                    } else {
                        sh.lambda *= sh.nu;
                        sh.nu *= 2.0;
                        sh.good = 0;
                    }
                }
            }
            __syncthreads();
            const bool good = sh.good != 0;
            const double lam = sh.lambda;
            ++attempts;
            if (hist && lead && t == 0 && nhist < ctl.hist_cap) {
                zs_ba_attempt a{};
                a.iteration = it;
                a.attempt = failures;
                a.solved = ok ? 1 : 0;
                a.accepted = ok && good ? 1 : 0;
                a.chi2 = ok ? chi2_new : sh.chi2;
                a.rho = ok ? sh.rho : 0.0;
                a.lambda = lam;
                hist[nhist] = a;
            }
            ++nhist;
            if (ok) {
                // a rejected step is rolled back while lambda stays finite
                // (k_rollback); every CTA waits for the poses it will read
                if (lead && !good && isfinite(lam) && t < K) {
                    double* pp = P.pose + (int64_t)(k0 + t) * kPoseStride;
#pragma unroll
                    for (int i = 0; i < kPoseStride; ++i) pp[i] = sh.bk[t][i];
                }
                team.sync();
            }
            if (!ok) {
                ++chol_fail;
                ++failures;
                if (!isfinite(lam)) break;
                continue;
            }
            if (good) {
                ++accepted;
                if (!isfinite(lam)) break;
                team.assemble(P, sh);  // the next iteration's system at the accepted state
                break;
            }
            if (!isfinite(lam)) break;
            ++failures;
        }
        const double thr = ctl.use_relative ? ctl.rel_tol * fmax(last, ctl.floor) : legacy;
        if (failures >= ctl.max_failures || (last - sh.chi2) < thr || !isfinite(sh.lambda)) break;
    }
    PoseOnlyOut o;
    o.iterations = iterations;
    o.attempts = attempts;
    o.accepted = accepted;
    o.cholesky_failures = chol_fail;
    o.history = nhist;
    o.chi2_initial = c0;
    o.chi2_final = sh.chi2;
    o.lambda_final = sh.lambda;
    return o;
}

__global__ void __launch_bounds__(kThreads) k_pose_only_lm(DevProblem P, PoseOnlyCtl ctl, PoseOnlyOut* out,
                                                           zs_ba_attempt* hist, double* part, double* sums,
                                                           double* cpart) {
    __shared__ Shared sh;
    GridTeam team{cg::this_grid(), part, sums, cpart};
    const PoseOnlyOut o = lm_loop(P, 0, P.K, ctl, true, team, sh, hist);
    if (blockIdx.x == 0 && threadIdx.x == 0) *out = o;
}

// A batch of windows whose landmarks are all fixed (tracking problems solved
// together): one CTA per window runs the loop above on the window's poses,
// each window with its own damping, decisions and stops, as the general
// batched path (ba_batch.cu) runs them, and reports into the batch's
// per-window control and state. A window without observations, or with
// neither poses nor landmarks, runs no iteration (k_binit's rule).
__global__ void __launch_bounds__(kThreads) k_pose_only_windows(DevProblem P, PoseOnlyCtl ctl, WinCtl* wctl,
                                                                LmState* wst) {
    __shared__ Shared sh;
    const int w = blockIdx.x;
    const int k0 = P.win_pose0[w], k1 = P.win_pose0[w + 1];
    WindowTeam team{k0, k1, P.pose_ptr[k0], P.pose_ptr[k1]};
    const bool has_obs = team.q1 > team.q0;
    const bool active = ctl.iterations > 0 && ctl.max_failures > 0 && has_obs &&
                        (k1 > k0 || P.win_lm0[w + 1] > P.win_lm0[w]);
    const PoseOnlyOut o = lm_loop(P, k0, k1 - k0, ctl, active, team, sh, nullptr);
    if (threadIdx.x == 0) {
        WinCtl c{};
        c.iterations = o.iterations;
        c.it = o.iterations;
        c.accepted = o.accepted;
        c.attempts = o.attempts;
        c.chol_failures = o.cholesky_failures;
        c.last = o.chi2_final;
        c.legacy = ctl.legacy_stop * o.chi2_initial;
        c.chi2_initial = o.chi2_initial;
        wctl[w] = c;
        LmState st{};
        st.chi2 = o.chi2_final;
        st.chi2_new = o.chi2_final;
        st.lambda = o.lambda_final;
        st.solve_ok = 1;
        wst[w] = st;
    }
}

}  // namespace

int pose_only_grid(int64_t M) {
    static std::atomic<int> cache[kMaxDevices];
    const int co = per_device(cache, [] {
        int dev = 0, sms = 0, per = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_pose_only_lm, kThreads, 0);
        cudaGetLastError();
        return std::max(1, std::min(sms, sms * per));
    });
    // about 64 observations per CTA and pass, at most one CTA per SM
    return (int)std::max<int64_t>(1, std::min<int64_t>(co, (M + 63) / 64));
}

cudaError_t launch_pose_only_windows(const DevProblem& P, const PoseOnlyCtl& ctl, WinCtl* wctl, LmState* wst,
                                    cudaStream_t s) {
    if (P.nwin < 1) return cudaSuccess;
    k_pose_only_windows<<<P.nwin, kThreads, 0, s>>>(P, ctl, wctl, wst);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_pose_only_lm(const DevProblem& P, const PoseOnlyCtl& ctl, PoseOnlyOut* out, zs_ba_attempt* hist,
                                double* part, double* sums, double* cpart, int grid, cudaStream_t s) {
    if (P.K > kPoseOnlyMaxK || grid < 1) return cudaErrorInvalidValue;
    DevProblem Pv = P;
    PoseOnlyCtl c = ctl;
    void* args[] = {(void*)&Pv, (void*)&c, (void*)&out, (void*)&hist, (void*)&part, (void*)&sums, (void*)&cpart};
    cudaError_t e = cudaLaunchCooperativeKernel((const void*)k_pose_only_lm, dim3(grid), dim3(kThreads), args, 0, s);
    if (e == cudaSuccess) note_launch();
    return e;
}

}  // namespace zs
