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
// takes its tasks in increasing order. Every dependency of a task has a
// smaller number, and all CTAs are co-resident (cooperative launch), so the
// lowest unfinished task can always proceed.
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
    float* F;
    float* X;
    float* XT;
    LmState* st;
    int* flagL;  // [N * N]: epoch once L tile (i, j) is final
    int* flagX;  // [N * N]: epoch once X tile (i, j) (i > j) is final
    int* abort;  // epoch once the launch has given up
    int epoch;
    int stall;   // a task whose flag is never published (failure-path tests), else -1
};

__device__ __forceinline__ int ld_acquire(const int* p) {
    int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release(int* p, int v) {
    asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Shared memory of one CTA.
struct Smem {
    float a[2][kTileFloats];
    float b[2][kTileFloats];
    float inv[kTileFloats];
    float dinv[kP];
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

// acc += sum over terms q in [0, nq) of A_q B_q^T, where term q's operand
// tiles are (M_a rows ra_q, cols ca_q) and (M_b rows rb_q, cols cb_q), both
// with kk_q valid columns, ready once both of its flags are published. The
// next term's tiles are copied while the current term is multiplied when its
// flags are already set. Returns false when the launch was aborted.
template <typename Term>
__device__ bool accumulate(const Dag& d, int nq, Term term, Smem& sm, float acc[4][4]) {
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
        load_block(o.ma, d.n, o.ra, o.ca, o.kk, sm.a[buf]);
        if (o.mb != o.ma || o.rb != o.ra || o.cb != o.ca) load_block(o.mb, d.n, o.rb, o.cb, o.kk, sm.b[buf]);
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
        tile_nt_acc(sm.a[buf], same ? sm.a[buf] : sm.b[buf], cur.kk, acc);
        __syncthreads();
        if (q + 1 < nq && !pre) {
            if (!wait_flag(d, nxt.fa) || !wait_flag(d, nxt.fb)) return false;
            issue(nxt, buf ^ 1);
        }
        cur = nxt;
    }
    return true;
}

// The lower triangle of a 64 x 64 tile (diagonal included, 2080 entries,
// packed row by row) shared out over the CTA: thread t owns entries
// t + 256 q, q < kOwn.
constexpr int kTri = kP * (kP + 1) / 2;
constexpr int kOwn = (kTri + t64::kThreads - 1) / t64::kThreads;

__device__ __forceinline__ void tri_entry(int e, int& i, int& j) {
    i = (int)((sqrtf(8.f * (float)e + 1.f) - 1.f) * 0.5f);
    while ((i + 1) * (i + 2) / 2 <= e) ++i;
    while (i * (i + 1) / 2 > e) --i;
    j = e - i * (i + 1) / 2;
}

// Factors the diagonal tile C (64 x kPL in shared memory, kb valid rows;
// rows and columns from kb on are an identity block) and inverts the factor,
// the whole CTA working with the tile's entries in registers (kOwn per
// thread) and one barrier per column:
// * factor, right-looking and unscaled: at column c every entry (i, j) with
//   j > c takes A_ij -= A_ic A_jc / A_cc, the column-c entries (final by
//   then) read from a shared column that their owners filled at the step
//   before; afterwards L_ij = A_ij / sqrt(A_jj). The pivot test is the
//   reference's d > eps on A_cc;
// * inverse, right-looking over the rows of X = L^-1: with row k of X final,
//   every entry (i, j), i > k >= j, takes x_ij -= L_ik X_kj, and the entries
//   of row k + 1 are final after it (X_ii = 1 / L_ii).
// L stays in sm.a[1] (row-major; store_diag_factor writes it out), X goes
// into X's tile (zeros above the diagonal) and its transpose into XT's.
// Returns 0 when a pivot fails its test (uniform).
__device__ int factor_diag(const Dag& d, int jb, int kb, const float* C, float eps, Smem& sm) {
    const int n = d.n, k0 = kP * jb;
    float* Lm = sm.a[1];
    float* col = sm.b[0];  // two 64-float columns, alternating
    float* Xs = sm.inv;
    int ei[kOwn], ej[kOwn];
    float a[kOwn];
#pragma unroll
    for (int q = 0; q < kOwn; ++q) {
        const int e = threadIdx.x + t64::kThreads * q;
        ei[q] = -1;
        ej[q] = 0;
        a[q] = 0.f;
        if (e < kTri) {
            tri_entry(e, ei[q], ej[q]);
            const int i = ei[q], j = ej[q];
            a[q] = (i < kb && j < kb) ? C[i * kPL + j] : (i == j ? 1.f : 0.f);
            if (j == 0) col[i] = a[q];
        }
    }
    for (int c = 0; c < kP; ++c) {
        __syncthreads();
        const float* cc = col + (c & 1) * kP;
        float* nc = col + ((c + 1) & 1) * kP;
        const float dc = cc[c];
        if (c < kb && !(dc > eps)) return 0;  // every thread reads the same pivot: uniform
        const float inv = __frcp_rn(dc);
        if (threadIdx.x == 0) sm.dinv[c] = rsqrtf(dc);
#pragma unroll
        for (int q = 0; q < kOwn; ++q) {
            const int i = ei[q], j = ej[q];
            if (j > c) {
                a[q] = fmaf(-(cc[i] * inv), cc[j], a[q]);
                if (j == c + 1) nc[i] = a[q];
            }
        }
    }
    __syncthreads();
    // L = A diag(A_jj)^-1/2 (lower), and the inverse's first row
    float x[kOwn];
#pragma unroll
    for (int q = 0; q < kOwn; ++q) {
        const int i = ei[q], j = ej[q];
        x[q] = i == j ? 1.f : 0.f;
        if (i >= 0) {
            Lm[i * kPL + j] = a[q] * sm.dinv[j];
            if (i == 0) Xs[0] = sm.dinv[0];
        }
    }
    for (int k = 0; k < kP - 1; ++k) {
        __syncthreads();
#pragma unroll
        for (int q = 0; q < kOwn; ++q) {
            const int i = ei[q], j = ej[q];
            if (i > k && j <= k) x[q] = fmaf(-Lm[i * kPL + k], Xs[k * kPL + j], x[q]);
            if (i == k + 1) Xs[i * kPL + j] = x[q] * sm.dinv[i];  // 1 / L_ii = A_ii^-1/2
        }
    }
    __syncthreads();
    // the inverse out (row-major, zeros above the diagonal) and its transpose
    // into XT: what the other tiles wait for (L_jj itself follows the flag)
    for (int e = threadIdx.x; e < kP * kP; e += blockDim.x) {
        const int i = e >> 6, j = e & 63;
        if (i >= kb || j >= kb) continue;
        d.X[(int64_t)(k0 + i) * n + k0 + j] = j <= i ? Xs[i * kPL + j] : 0.f;
        d.XT[(int64_t)(k0 + i) * n + k0 + j] = i <= j ? Xs[j * kPL + i] : 0.f;
    }
    return 1;
}

// L_jj (row-major, zeros above the diagonal) into F from sm.a[1].
// No task reads F's diagonal tiles; the solve test after the launch does.
__device__ void store_diag_factor(const Dag& d, int jb, int kb, const Smem& sm) {
    const int n = d.n, k0 = kP * jb;
    for (int e = threadIdx.x; e < kP * kP; e += blockDim.x) {
        const int i = e >> 6, j = e & 63;
        if (i >= kb || j >= kb) continue;
        d.F[(int64_t)(k0 + i) * n + k0 + j] = j <= i ? sm.a[1][i * kPL + j] : 0.f;
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
    const int n = d.n, N = d.N;
    const int ri = tile_len(d, i), cj = tile_len(d, j);
    // the tile's S values, copied while the sums run (sm.inv is free until
    // the diagonal factor)
    load_block(d.F, n, kP * i, kP * j, cj, sm.inv);
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
        load_block(d.X, n, kP * j, kP * j, cj, sm.b[0]);
        cp_async_wait_all();
        __syncthreads();
        float out[4][4];
        tile_nt(sm.a[0], sm.b[0], cj, out);
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int b = 0; b < 4; ++b) {
                const int r = ty + 16 * a, c = tx + 16 * b;
                if (r < ri && c < cj) d.F[(int64_t)(kP * i + r) * n + kP * j + c] = out[a][b];
            }
    }
    publish(d, d.flagL + i * N + j, task);
    if (i == j) store_diag_factor(d, j, cj, sm);
    __syncthreads();
    return true;
}

// X tile (i, j), i > j, and its transpose.
__device__ bool task_X(const Dag& d, int i, int j, int task, Smem& sm) {
    const int n = d.n, N = d.N;
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
    load_block(d.X, n, kP * i, kP * i, ri, sm.a[0]);
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
            if (r < ri && c < cj) d.X[(int64_t)(kP * i + r) * n + kP * j + c] = out[a][b];
        }
    // XT tile (j, i) = X_ij^T, staged so that its rows are written contiguously
    __syncthreads();
    acc_to_smem(out, sm.a[1], true);
    __syncthreads();
    for (int e = threadIdx.x; e < kP * kP; e += blockDim.x) {
        const int c = e >> 6, r = e & 63;
        if (r < ri && c < cj) d.XT[(int64_t)(kP * j + c) * n + kP * i + r] = sm.a[1][c * kPL + r];
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
        const bool ok = (r < N - c) ? task_L(d, c + r, c, t, sm) : task_X(d, c, r - (N - c), t, sm);
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
    if (n <= 0) return cudaSuccess;
    static const int stall = stall_task_from_env();
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const size_t smem = sizeof(Smem);
    cudaError_t e = cudaFuncSetAttribute(k_chol_inverse_dag, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_chol_inverse_dag, t64::kThreads, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    const int N = (n + kP - 1) / kP;
    int blocks = sms * per_sm;
    if (blocks > N * N) blocks = N * N;
    Dag d;
    d.n = n;
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
    void* args[] = {(void*)&d};
    e = cudaLaunchCooperativeKernel((const void*)k_chol_inverse_dag, dim3(blocks), dim3(t64::kThreads), args, smem,
                                    s);
    if (e != cudaSuccess) return e;
    note_launch();
    return cudaSuccess;
}

}  // namespace zs
