// The mixed form's dense preconditioner in one launch: the Cholesky factor
// S = L L^T of the FP32 reduced camera system (source/
// matrix_decomposition_cholesky.hpp:26-59, with its pivot test) and the
// explicit inverse X = L^-1 with its transpose, which the conjugate-gradient
// solve applies as X^T X.
//
// The matrix is cut into 64 x 64 tiles (N = ceil(n / 64) per side). Every
// output tile has one owner CTA that computes it completely, in a fixed
// order of terms, and then publishes it with a per-tile flag:
//   L tile (i, j), i > j:  L_ij = (S_ij - sum_{k<j} L_ik L_jk^T) L_jj^-T
//   L tile (j, j):         factor of S_jj - sum_{k<j} L_jk L_jk^T in shared
//                          memory, with L_jj^-1 (= X_jj)
//   X tile (i, j), i > j:  X_ij = -L_ii^-1 sum_{m=j}^{i-1} L_im X_mj
// A CTA adds each term as soon as that term's operand tiles are published,
// so the factorisation's diagonal chain (L_jj -> L_{j+1,j} -> L_{j+1,j+1})
// runs without grid-wide barriers, and X follows the factor a few tiles
// behind. Tasks are numbered column block by column block (L tiles of
// column c, then X tiles of row c); task t belongs to CTA t mod G, which
// takes its tasks in increasing order. Up to kFuseMaxN tile columns the task
// of L tile (c + 1, c) also factors diagonal tile c + 1 (task_LD), so the
// chain passes one flag per column. Every dependency of a task has a smaller number, and all CTAs are
// co-resident (cooperative launch), so the lowest unfinished task can always
// proceed.
//
// The matrix may be the n x n block of a larger one (row stride ld): the
// blocked form of ba_chol_tc.cu runs this kernel on its diagonal blocks.
//
// Flags hold the launch's epoch (the host advances it per launch), so they
// need no clearing. A wait gives up after a bounded number of polls: it then
// marks the launch aborted (every other wait returns) and sets st->timeout
// and st->solve_ok = 0. A failed pivot aborts the launch the same way with
// st->solve_ok = 0. Every floating-point sum has one owner and a fixed order:
// results repeat bit for bit.
#include <cooperative_groups.h>

#include <cstdlib>

#include "ba_internal.h"
#include "ba_tile64.cuh"

namespace cg = cooperative_groups;

namespace zs {

using namespace t64;

namespace {

// Polls of one flag before a wait gives up (with the back-off below, about a
// second; a legitimate wait lasts at most one factorisation, milliseconds).
constexpr long long kSpinLimit = 1ll << 20;

struct Dag {
    int n, N;
    int ld;  // row stride of F, X and XT (the matrix may be a block of a larger one)
    float* F;
    float* X;
    float* XT;
    LmState* st;
    int* flagL;  // [N * N]: epoch once L tile (i, j) is final
    int* flagX;  // [N * N]: epoch once X tile (i, j) (i > j) is final
    int* abort;  // epoch once the launch has given up
    int epoch;
    int stall;   // a task whose flag is never published (failure-path tests), else -1
    int fuse;    // task (c, 1) also factors diagonal tile c + 1 (task_LD)
};

// Up to this many tile columns the fused task of the diagonal chain pays:
// there the chain bounds the launch. Beyond it the launch is bound by its
// work, and the fused task's doubled sums on one CTA cost more than the
// flag it saves (measured: n = 1200 faster fused, n >= 3000 slower).
constexpr int kFuseMaxN = 32;

__device__ __forceinline__ int ld_acquire(const int* p) {
    int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release(int* p, int v) {
    asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Shared memory of one CTA.
// A published row of the diagonal factor: four owner groups of 16 values,
// kRowQ apart (20: the four groups' 16-byte reads fall in distinct banks).
constexpr int kRowQ = 20;

struct Smem {
    float a[2][kTileFloats];
    float b[2][kTileFloats];
    float inv[kTileFloats];
    __align__(16) float rowbuf[2][8 * kRowQ];  // row c of [C | I] (both halves), double-buffered
    float pinv[2];                             // 1 / d_c
    float rs[kP];                              // d_c^-1/2
};

// Thread 0 waits for *f == epoch; false when the launch was aborted (or this
// wait ran out and aborted it). Uniform over the CTA (thread 0's answer is
// broadcast by the barrier itself).
__device__ bool wait_flag(const Dag& d, const int* f) {
    int ok = 0;
    if (threadIdx.x == 0) {
        ok = 1;
        if (ld_acquire(f) != d.epoch) {
            long long it = 0;
            unsigned ns = 32;
            for (;;) {
                if (ld_acquire(f) == d.epoch) break;
                if (ld_acquire(d.abort) == d.epoch) {
                    ok = 0;
                    break;
                }
                if (++it > kSpinLimit) {
                    d.st->timeout = 1;
                    d.st->solve_ok = 0;
                    __threadfence();
                    st_release(d.abort, d.epoch);
                    ok = 0;
                    break;
                }
                __nanosleep(ns);
                if (ns < 256) ns *= 2;
            }
        }
    }
    return __syncthreads_or(ok) != 0;
}

// Thread 0 reads *f once: true when already final. Uniform over the CTA.
__device__ bool is_ready(const Dag& d, const int* f) {
    return __syncthreads_or(threadIdx.x == 0 && ld_acquire(f) == d.epoch) != 0;
}

__device__ void publish(const Dag& d, int* f, int task) {
    __syncthreads();
    if (threadIdx.x == 0 && task != d.stall) {
        __threadfence();
        st_release(f, d.epoch);
    }
}

__device__ void abort_launch(const Dag& d) {
    if (threadIdx.x == 0) {
        d.st->solve_ok = 0;
        __threadfence();
        st_release(d.abort, d.epoch);
    }
    __syncthreads();
}

__device__ __forceinline__ int tile_len(const Dag& d, int b) { return min(kP, d.n - kP * b); }

// mul(A_q, B_q, kk_q) for terms q in [0, nq), where term q's operand tiles
// are (M_a rows ra_q, cols ca_q) and (M_b rows rb_q, cols cb_q), both with
// kk_q valid columns, ready once both of its flags are published. The next
// term's tiles are copied while the current term is multiplied when its flags
// are already set. Returns false when the launch was aborted.
template <typename Term, typename Mul>
__device__ bool accumulate_with(const Dag& d, int nq, Term term, Smem& sm, Mul mul) {
    if (nq <= 0) return true;
    struct Op {
        const float* ma;
        int ra, ca;
        const float* mb;
        int rb, cb, kk;
        const int* fa;
        const int* fb;
    };
    auto issue = [&](const Op& o, int buf) {
        load_block(o.ma, d.n, d.ld, o.ra, o.ca, o.kk, sm.a[buf]);
        if (o.mb != o.ma || o.rb != o.ra || o.cb != o.ca) load_block(o.mb, d.n, d.ld, o.rb, o.cb, o.kk, sm.b[buf]);
        cp_async_commit();
    };
    Op cur;
    term(0, cur.ma, cur.ra, cur.ca, cur.mb, cur.rb, cur.cb, cur.kk, cur.fa, cur.fb);
    if (!wait_flag(d, cur.fa) || !wait_flag(d, cur.fb)) return false;
    issue(cur, 0);
    for (int q = 0; q < nq; ++q) {
        const int buf = q & 1;
        Op nxt;
        bool pre = false;
        if (q + 1 < nq) {
            term(q + 1, nxt.ma, nxt.ra, nxt.ca, nxt.mb, nxt.rb, nxt.cb, nxt.kk, nxt.fa, nxt.fb);
            if (is_ready(d, nxt.fa) && is_ready(d, nxt.fb)) {
                issue(nxt, buf ^ 1);
                pre = true;
            }
        }
        if (pre) cp_async_wait_one();
        else cp_async_wait_none();
        __syncthreads();
        const bool same = cur.mb == cur.ma && cur.rb == cur.ra && cur.cb == cur.ca;
        mul(sm.a[buf], same ? sm.a[buf] : sm.b[buf], cur.kk);
        __syncthreads();
        if (q + 1 < nq && !pre) {
            if (!wait_flag(d, nxt.fa) || !wait_flag(d, nxt.fb)) return false;
            issue(nxt, buf ^ 1);
        }
        cur = nxt;
    }
    return true;
}

// acc += sum over the terms of A_q B_q^T (accumulate_with).
template <typename Term>
__device__ bool accumulate(const Dag& d, int nq, Term term, Smem& sm, float acc[4][4]) {
    return accumulate_with(d, nq, term, sm,
                           [&](const float* A, const float* B, int kk) { tile_nt_acc(A, B, kk, acc); });
}

// Factors the diagonal tile C (64 x kPL in shared memory, kb valid rows) by
// elimination on the augmented block [C | I]: at step c the raw row c is
// published with the reciprocal of its pivot d_c, and every row r > c takes
// m_rc = a_rc / d_c times it away from itself in both halves. After the 64
// steps the right half is E = L'^-1 for C = L' D L'^T (L' unit lower), so
// L^-1 = D^-1/2 E and L_rc = a_rc d_c^-1/2 (a_rc: row r's value in column c
// when step c ran). The square roots and the final scaling stay off the
// step-to-step path, which is one barrier, the pivot's reciprocal and one
// fused multiply-add per step.
//
// Thread t owns row r = t / 4 and the columns j = 4 m + (t % 4), m < 16, of
// both halves in registers (so a column's owner and register are fixed when
// the step loop is unrolled); a published row is laid out by owner (q-major,
// stride kRowQ) for 16-byte broadcast reads. Pivot test at the real rows:
// d_c > eps (the reference's test, source/matrix_decomposition_cholesky.hpp:40,53).
// L_jj^-1 goes into X's tile (zeros above the diagonal) and its transpose
// into XT's; L_jj stays in sm.a[0] for store_diag_factor. Returns 0 when a
// pivot fails its test (uniform).
// (One out-of-line copy for both callers: the unrolled steps are long.)
__device__ __noinline__ int eliminate_diag(float* X, float* XT, int ld, int k0, int kb, const float* C, float eps,
                                           Smem& sm) {
    const int t = threadIdx.x, r = t >> 2, q = t & 3, lane = t & 31;
    const int grp = lane & ~3;
    float a[16], v[16];
#pragma unroll
    for (int m = 0; m < 16; ++m) {
        const int j = 4 * m + q;
        // from C's lower triangle only (the blocked form updates no more of a
        // diagonal block): row r right of the diagonal is column r below it
        a[m] = (r < kb && j < kb) ? (j <= r ? C[r * kPL + j] : C[j * kPL + r]) : (r == j ? 1.f : 0.f);
        v[m] = r == j ? 1.f : 0.f;
    }
    int fail = 0;
    float arc = __shfl_sync(0xffffffffu, a[0], grp);  // row r's column-0 value
#pragma unroll
    for (int c = 0; c < kP; ++c) {
        constexpr int kHalf = 4 * kRowQ;
        float* rowA = sm.rowbuf[c & 1];
        float* rowE = rowA + kHalf;
        const int mc = c >> 2;  // register of column c (owner q == c % 4)
        if (r == c) {
            float4* pa = reinterpret_cast<float4*>(rowA + q * kRowQ);
#pragma unroll
            for (int g = mc >> 2; g < 4; ++g) pa[g] = make_float4(a[4 * g], a[4 * g + 1], a[4 * g + 2], a[4 * g + 3]);
            float4* pe = reinterpret_cast<float4*>(rowE + q * kRowQ);
#pragma unroll
            for (int g = 0; g <= (mc >> 2); ++g) pe[g] = make_float4(v[4 * g], v[4 * g + 1], v[4 * g + 2], v[4 * g + 3]);
            if (q == (c & 3)) {
                const float dc = a[mc];
                if (c < kb && !(dc > eps)) fail = 1;
                sm.pinv[c & 1] = __fdividef(1.f, dc);
            }
        }
        __syncthreads();
        if (r > c) {
            const float coef = arc * sm.pinv[c & 1];
            const float4* pa = reinterpret_cast<const float4*>(rowA + q * kRowQ);
#pragma unroll
            for (int g = mc >> 2; g < 4; ++g) {
                const float4 u = pa[g];
                const float uu[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const int m = 4 * g + k;
                    if (m > mc || (m == mc && q > (c & 3))) a[m] = fmaf(-coef, uu[k], a[m]);
                }
            }
            const float4* pe = reinterpret_cast<const float4*>(rowE + q * kRowQ);
#pragma unroll
            for (int g = 0; g <= (mc >> 2); ++g) {
                const float4 u = pe[g];
                const float uu[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const int m = 4 * g + k;
                    if (m < mc || (m == mc && q <= (c & 3))) v[m] = fmaf(-coef, uu[k], v[m]);
                }
            }
        }
        if (c + 1 < kP) arc = __shfl_sync(0xffffffffu, a[(c + 1) >> 2], grp | ((c + 1) & 3));
    }
    // d_r^-1/2 from each row's pivot, still in its owner's register
#pragma unroll
    for (int m = 0; m < 16; ++m)
        if (4 * m + q == r) sm.rs[r] = rsqrtf(a[m]);
    if (__syncthreads_or(fail)) return 0;
    const float rr = sm.rs[r];
    float* Lout = sm.a[0];  // C is no longer read
#pragma unroll
    for (int m = 0; m < 16; ++m) {
        const int j = 4 * m + q;
        v[m] *= rr;  // (L^-1)_rj, zero above the diagonal
        Lout[r * kPL + j] = j <= r ? a[m] * sm.rs[j] : 0.f;
        if (r < kb && j < kb) {
            X[(int64_t)(k0 + r) * ld + k0 + j] = v[m];
            XT[(int64_t)(k0 + j) * ld + k0 + r] = v[m];
        }
    }
    return 1;
}

__device__ __forceinline__ int factor_diag(const Dag& d, int jb, int kb, const float* C, float eps, Smem& sm) {
    return eliminate_diag(d.X, d.XT, d.ld, kP * jb, kb, C, eps, sm);
}

// L_jj (row-major, zeros above the diagonal) into F from sm.a[0]. No task
// reads F's diagonal tiles; the solve test after the launch does.
__device__ void store_diag_factor(const Dag& d, int jb, int kb, const Smem& sm) {
    const int ld = d.ld, k0 = kP * jb;
    for (int e = threadIdx.x; e < kP * kP; e += blockDim.x) {
        const int i = e >> 6, j = e & 63;
        if (i < kb && j < kb) d.F[(int64_t)(k0 + i) * ld + k0 + j] = sm.a[0][i * kPL + j];
    }
}

// acc (the owner's 4 x 4 block of a 64 x 64 tile) into a shared-memory tile,
// as is or transposed.
__device__ __forceinline__ void acc_to_smem(const float acc[4][4], float* S, bool transposed) {
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            const int r = ty + 16 * a, c = tx + 16 * b;
            if (transposed) S[c * kPL + r] = acc[a][b];
            else S[r * kPL + c] = acc[a][b];
        }
}

// L tile (i, j), i >= j.
__device__ bool task_L(const Dag& d, int i, int j, int task, Smem& sm) {
    const int n = d.n, ld = d.ld, N = d.N;
    const int ri = tile_len(d, i), cj = tile_len(d, j);
    // the tile's S values, copied while the sums run (sm.inv is free until
    // the diagonal factor)
    load_block(d.F, n, ld, kP * i, kP * j, cj, sm.inv);
    cp_async_commit();
    float acc[4][4];
    zero_acc(acc);
    const bool ok = accumulate(d, j, [&](int k, const float*& ma, int& ra, int& ca, const float*& mb, int& rb,
                                          int& cb, int& kk, const int*& fa, const int*& fb) {
        ma = d.F; ra = kP * i; ca = kP * k;
        mb = d.F; rb = kP * j; cb = kP * k;
        kk = tile_len(d, k);
        fa = d.flagL + i * N + k;
        fb = d.flagL + j * N + k;
    }, sm, acc);
    if (!ok) return false;
    cp_async_wait_none();
    __syncthreads();
    // C = S_ij - acc into a[0]
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            const int r = ty + 16 * a, c = tx + 16 * b;
            acc[a][b] = sm.inv[r * kPL + c] - acc[a][b];
        }
    __syncthreads();
    acc_to_smem(acc, sm.a[0], false);
    __syncthreads();
    if (i == j) {
        if (!factor_diag(d, j, cj, sm.a[0], (float)__ldcg(&d.st->eps_factor), sm)) {
            abort_launch(d);
            return false;
        }
    } else {
        // L_ij = C L_jj^-T: out[r][c] = sum_m C[r][m] (L_jj^-1)[c][m]
        if (!wait_flag(d, d.flagL + j * N + j)) return false;
        load_block(d.X, n, ld, kP * j, kP * j, cj, sm.b[0]);
        cp_async_wait_all();
        __syncthreads();
        float out[4][4];
        tile_nt(sm.a[0], sm.b[0], cj, out);
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int b = 0; b < 4; ++b) {
                const int r = ty + 16 * a, c = tx + 16 * b;
                if (r < ri && c < cj) d.F[(int64_t)(kP * i + r) * ld + kP * j + c] = out[a][b];
            }
    }
    publish(d, d.flagL + i * N + j, task);
    if (i == j) store_diag_factor(d, j, cj, sm);
    __syncthreads();
    return true;
}

// L tile (j + 1, j) and then the diagonal tile j + 1, in one task: the
// diagonal chain's step from L_jj to L_{j+1,j+1} stays inside one CTA (one
// flag wait and one tile load instead of two of each). The sums of both
// tiles share their L_{j+1,k} operand tiles:
//   C_L = S_{j+1,j} - sum_{k<j} L_{j+1,k} L_jk^T,   L_{j+1,j} = C_L L_jj^-T
//   C_D = S_{j+1,j+1} - sum_{k<j} L_{j+1,k} L_{j+1,k}^T - L_{j+1,j} L_{j+1,j}^T
// and C_D is factored as task_L factors a diagonal tile.
__device__ bool task_LD(const Dag& d, int j, int task, Smem& sm) {
    const int n = d.n, ld = d.ld, N = d.N, i = j + 1;
    const int ri = tile_len(d, i), cj = tile_len(d, j);
    load_block(d.F, n, ld, kP * i, kP * j, cj, sm.inv);  // S_ij, copied while the sums run
    cp_async_commit();
    float accL[4][4], accD[4][4];
    zero_acc(accL);
    zero_acc(accD);
    const bool ok = accumulate_with(
        d, j,
        [&](int k, const float*& ma, int& ra, int& ca, const float*& mb, int& rb, int& cb, int& kk, const int*& fa,
            const int*& fb) {
            ma = d.F; ra = kP * i; ca = kP * k;
            mb = d.F; rb = kP * j; cb = kP * k;
            kk = tile_len(d, k);
            fa = d.flagL + i * N + k;
            fb = d.flagL + j * N + k;
        },
        sm,
        [&](const float* A, const float* B, int kk) {
            tile_nt_acc(A, B, kk, accL);
            tile_nt_acc(A, A, kk, accD);
        });
    if (!ok) return false;
    cp_async_wait_none();
    __syncthreads();
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    // C_L into a[0]
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            const int r = ty + 16 * a, c = tx + 16 * b;
            accL[a][b] = sm.inv[r * kPL + c] - accL[a][b];
        }
    __syncthreads();
    acc_to_smem(accL, sm.a[0], false);
    // S_ii into sm.inv while L_jj is awaited
    load_block(d.F, n, ld, kP * i, kP * i, ri, sm.inv);
    cp_async_commit();
    if (!wait_flag(d, d.flagL + j * N + j)) return false;
    load_block(d.X, n, ld, kP * j, kP * j, cj, sm.b[0]);
    cp_async_wait_all();
    __syncthreads();
    // L_ij = C_L L_jj^-T, out to F, kept in a[1]
    float out[4][4];
    tile_nt(sm.a[0], sm.b[0], cj, out);
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            const int r = ty + 16 * a, c = tx + 16 * b;
            if (r < ri && c < cj) d.F[(int64_t)(kP * i + r) * ld + kP * j + c] = out[a][b];
        }
    acc_to_smem(out, sm.a[1], false);
    publish(d, d.flagL + i * N + j, task);  // (its barrier also orders a[1])
    // C_D = S_ii - accD - L_ij L_ij^T into a[0]
    tile_nt(sm.a[1], sm.a[1], cj, out);
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            const int r = ty + 16 * a, c = tx + 16 * b;
            accD[a][b] = sm.inv[r * kPL + c] - accD[a][b] - out[a][b];
        }
    __syncthreads();
    acc_to_smem(accD, sm.a[0], false);
    __syncthreads();
    if (!factor_diag(d, i, ri, sm.a[0], (float)__ldcg(&d.st->eps_factor), sm)) {
        abort_launch(d);
        return false;
    }
    publish(d, d.flagL + i * N + i, task);
    store_diag_factor(d, i, ri, sm);
    __syncthreads();
    return true;
}

// X tile (i, j), i > j, and its transpose.
__device__ bool task_X(const Dag& d, int i, int j, int task, Smem& sm) {
    const int n = d.n, ld = d.ld, N = d.N;
    float acc[4][4];
    zero_acc(acc);
    // acc = sum_{m=j}^{i-1} L_im X_mj with X_mj^T = XT tile (j, m)
    const bool ok = accumulate(d, i - j, [&](int q, const float*& ma, int& ra, int& ca, const float*& mb, int& rb,
                                              int& cb, int& kk, const int*& fa, const int*& fb) {
        const int m = j + q;
        ma = d.F; ra = kP * i; ca = kP * m;
        mb = d.XT; rb = kP * j; cb = kP * m;
        kk = tile_len(d, m);
        fa = d.flagL + i * N + m;
        fb = (m == j) ? d.flagL + j * N + j : d.flagX + m * N + j;
    }, sm, acc);
    if (!ok) return false;
    if (!wait_flag(d, d.flagL + i * N + i)) return false;
    // X_ij = -L_ii^-1 acc: out[r][c] = sum_t (L_ii^-1)[r][t] acc^T[c][t]
    const int ri = tile_len(d, i), cj = tile_len(d, j);
    acc_to_smem(acc, sm.b[0], true);
    load_block(d.X, n, ld, kP * i, kP * i, ri, sm.a[0]);
    cp_async_wait_all();
    __syncthreads();
    float out[4][4];
    tile_nt(sm.a[0], sm.b[0], ri, out);
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            const int r = ty + 16 * a, c = tx + 16 * b;
            out[a][b] = -out[a][b];
            if (r < ri && c < cj) d.X[(int64_t)(kP * i + r) * ld + kP * j + c] = out[a][b];
        }
    // XT tile (j, i) = X_ij^T, staged so that its rows are written contiguously
    __syncthreads();
    acc_to_smem(out, sm.a[1], true);
    __syncthreads();
    for (int e = threadIdx.x; e < kP * kP; e += blockDim.x) {
        const int c = e >> 6, r = e & 63;
        if (r < ri && c < cj) d.XT[(int64_t)(kP * j + c) * ld + kP * i + r] = sm.a[1][c * kPL + r];
    }
    publish(d, d.flagX + i * N + j, task);
    return true;
}

__global__ void __launch_bounds__(t64::kThreads, 1) k_chol_inverse_dag(Dag d) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Smem& sm = *reinterpret_cast<Smem*>(smem_raw);
    if (__ldcg(&d.st->skip_factor) || !__ldcg(&d.st->solve_ok)) return;  // written by earlier launches: uniform
    const int N = d.N;
    const int tasks = N * N;
    for (int t = blockIdx.x; t < tasks; t += gridDim.x) {
        const int c = t / N, r = t % N;
        bool ok = true;
        if (r >= N - c) ok = task_X(d, c, r - (N - c), t, sm);
        else if (!d.fuse) ok = task_L(d, c + r, c, t, sm);
        else if (r == 1) ok = task_LD(d, c, t, sm);     // L_{c+1,c} and L_{c+1,c+1}
        else if (r > 1 || c == 0) ok = task_L(d, c + r, c, t, sm);
        // (fused, r == 0, c > 0: the diagonal tile c came with task (c - 1, 1))
        if (!ok) return;
    }
}

int stall_task_from_env() {
    const char* v = std::getenv("ZS_TEST_STALL_TILE_TASK");
    return v && *v ? std::atoi(v) : -1;
}

}  // namespace

int dag_flag_ints(int n) {
    const int N = (n + kP - 1) / kP;
    return 2 * N * N + 1;
}

cudaError_t launch_chol_inverse_dag(int n, float* F, float* X, float* XT, LmState* st, int* flags, int* epoch,
                                    cudaStream_t s) {
    return launch_chol_inverse_dag_ld(n, n, F, X, XT, st, flags, epoch, s);
}

cudaError_t launch_chol_inverse_dag_ld(int n, int ld, float* F, float* X, float* XT, LmState* st, int* flags,
                                       int* epoch, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    static const int stall = stall_task_from_env();
    static std::atomic<int> resident[kMaxDevices];
    const size_t smem = sizeof(Smem);
    // co-resident CTAs of the launch on this device (the attribute set and the
    // occupancy query once per device)
    const int co = per_device(resident, [&] {
        int dev = 0, sms = 0, per_sm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (cudaFuncSetAttribute(k_chol_inverse_dag, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
                cudaSuccess ||
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_chol_inverse_dag, t64::kThreads, smem) !=
                cudaSuccess)
            return 0;
        return sms * per_sm;
    });
    if (co < 1) {
        const cudaError_t e = cudaGetLastError();
        return e != cudaSuccess ? e : cudaErrorInvalidConfiguration;
    }
    cudaError_t e;
    const int N = (n + kP - 1) / kP;
    int blocks = co;
    if (blocks > N * N) blocks = N * N;
    Dag d;
    d.n = n;
    d.ld = ld;
    d.N = N;
    d.F = F;
    d.X = X;
    d.XT = XT;
    d.st = st;
    d.flagL = flags;
    d.flagX = flags + N * N;
    d.abort = flags + 2 * N * N;
    d.epoch = ++*epoch;
    d.stall = stall;
    d.fuse = N <= kFuseMaxN;
    void* args[] = {(void*)&d};
    e = cudaLaunchCooperativeKernel((const void*)k_chol_inverse_dag, dim3(blocks), dim3(t64::kThreads), args, smem,
                                    s);
    if (e != cudaSuccess) return e;
    note_launch();
    return cudaSuccess;
}

}  // namespace zs
