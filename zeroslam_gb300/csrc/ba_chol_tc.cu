// Factor S = L L^T and inverse X = L^-1 of the mixed form's FP32
// preconditioner at large n, in panels of kPanel columns: each panel's
// diagonal block by the dataflow kernel (k_chol_inverse_dag on a block of the
// matrix), everything else as tensor-core products (k_tc_gemm_nt, 3xTF32 at
// FP32 accuracy). Panel k holds columns [o, o + b) with m = n - o - b rows
// below it:
//   L_kk, X_kk = L_kk^-1          dataflow kernel, in place in F, X, XT
//   P = S_21 X_kk^T      (m x b)  L_21 (S_21 is F's block below L_kk), into
//                                 a scratch panel, then copied into F
//   S_22 -= P P^T                 trailing update, lower tiles only
//   Q = Y^T[0:o, k] X_kk^T        block row k of X, X_k = X_kk Y_k, kept
//                                 transposed: into scratch, then XT[0:o, k]
//   Y^T[0:o+b, o+b:n] -= XT[0:o+b, k] P^T    every later block row r of Y
//                                 loses L_rk X_k
// This is forward substitution L X = I in right-looking form: Y starts as
// the identity; once the panels before k have updated block row k of Y, that
// row times X_kk is block row k of X, and it updates the rows below. X lives
// transposed in XT's upper triangle (zeroed first: the updates accumulate
// into it) and k_lower_from_upper writes X's lower triangle at the end.
// Every kernel here returns at once when st says the factorisation is not
// wanted (skip_factor) or has already failed (solve_ok = 0), so that the
// preconditioner's armed-only-on-failure retry costs launches, not work.
// Per panel the products are (m x b x b), (m x m x b, half of it), (o x b x b)
// and ((o + b) x m x b): 2n^3/3 flops over all panels plus ~2 n^2 kPanel.
//
// Three streams with look-ahead. The chain of the factorisation runs on a
// high-priority stream: the diagonal block, the rows of P that belong to the
// next panel, and the next diagonal block's update, so the next dataflow
// launch can start at once. A second high-priority stream forms the rest of
// P and the next panel's columns below its diagonal block beside that launch;
// a low-priority stream takes the rest of each panel's products and fills
// the SMs the dataflow kernel leaves idle. Per-panel events order the three
// wherever they write the same blocks (a later panel's updates wait for the
// earlier rest-of-panel update of that region), and P's two buffers
// alternate, each reused only after the low-priority work of the panel
// before last is done.
//
// F, X and XT are n x n row-major with n % 4 == 0 (16-byte rows, as the
// tensor maps of the products need); the solves take this path only then,
// and only from kTcMinN on, where it is faster than the dataflow kernel
// alone (measured: equal near n = 3000, 2x at n = 6000).
#include <algorithm>

#include "ba_internal.h"
#include "ba_tile64.cuh"

namespace zs {

namespace {

constexpr int kTile = 32;

// X[i][j] = XT[j][i] for j <= i: 32 x 32 tiles through shared memory, one
// CTA per tile on or below the diagonal (tile index t -> (ti, tj), tj <= ti).
__global__ void __launch_bounds__(kTile * 8) k_lower_from_upper(int n, const float* __restrict__ XT,
                                                                float* __restrict__ X, const LmState* st) {
    __shared__ float t[kTile][kTile + 1];
    if (__ldcg(&st->skip_factor) || !__ldcg(&st->solve_ok)) return;
    const int64_t b = blockIdx.x;
    int ti = (int)((sqrt(8.0 * (double)b + 1.0) - 1.0) * 0.5);
    while ((int64_t)ti * (ti + 1) / 2 > b) --ti;
    while ((int64_t)(ti + 1) * (ti + 2) / 2 <= b) ++ti;
    const int tj = (int)(b - (int64_t)ti * (ti + 1) / 2);
    const int r0 = kTile * ti, c0 = kTile * tj;
    const int x = threadIdx.x & (kTile - 1), y = threadIdx.x / kTile;
    // read XT rows c0.. (X's columns), columns r0.. (X's rows)
    for (int k = y; k < kTile; k += 8) {
        const int row = c0 + k, col = r0 + x;
        t[k][x] = (row < n && col < n) ? XT[(int64_t)row * n + col] : 0.f;
    }
    __syncthreads();
    for (int k = y; k < kTile; k += 8) {
        const int row = r0 + k, col = c0 + x;
        if (row < n && col <= row) X[(int64_t)row * n + col] = t[x][k];
    }
}

// XT = 0 (every product below accumulates into XT's upper triangle).
__global__ void __launch_bounds__(256) k_zero(int64_t count, float4* __restrict__ p, const LmState* st) {
    if (__ldcg(&st->skip_factor) || !__ldcg(&st->solve_ok)) return;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x)
        p[i] = make_float4(0.f, 0.f, 0.f, 0.f);
}

// dst[r][c] = src[r][c] for r < rows, c < cols (row strides lds, ldd; cols,
// lds, ldd multiples of 4 and both bases 16-byte aligned).
__global__ void __launch_bounds__(256) k_copy_block(int rows, int cols, const float* __restrict__ src, int lds,
                                                    float* __restrict__ dst, int ldd, const LmState* st) {
    if (__ldcg(&st->skip_factor) || !__ldcg(&st->solve_ok)) return;
    const int c4 = cols / 4;
    const int64_t total = (int64_t)rows * c4;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int r = (int)(i / c4), c = 4 * (int)(i % c4);
        *reinterpret_cast<float4*>(dst + (int64_t)r * ldd + c) =
            __ldcg(reinterpret_cast<const float4*>(src + (int64_t)r * lds + c));
    }
}

// C (M x N) = alpha A B^T + beta C on the FP32 pipe, a CTA per 64 x 64 tile
// of C (lower: tiles above the diagonal skipped, entries above it kept), K in
// chunks of 64 double-buffered through shared memory by 16-byte
// asynchronous copies: the small products on the blocked form's chain
// (256 x 256 x 256), where a tensor-core tile's fixed costs (tensor-memory
// allocation, the pipeline's fill, the promotion of its partial sums) exceed
// the arithmetic. A, B 16-byte aligned with lda, ldb multiples of 4.
constexpr size_t kGemm64Smem = 4 * sizeof(float) * t64::kTileFloats;

__global__ void __launch_bounds__(t64::kThreads) k_gemm_nt64(int M, int N, int K, const float* __restrict__ A, int lda,
                                                             const float* __restrict__ B, int ldb, float* C, int ldc,
                                                             float alpha, float beta, int lower, const LmState* st) {
    extern __shared__ __align__(16) float g64[];
    if (__ldcg(&st->skip_factor) || !__ldcg(&st->solve_ok)) return;
    const int row0 = blockIdx.y * t64::kP, col0 = blockIdx.x * t64::kP;
    if (lower && col0 > row0 + t64::kP - 1) return;
    float* sa[2] = {g64, g64 + t64::kTileFloats};
    float* sb[2] = {g64 + 2 * t64::kTileFloats, g64 + 3 * t64::kTileFloats};
    float acc[4][4];
    t64::zero_acc(acc);
    const int nk = (K + t64::kP - 1) / t64::kP;
    auto issue = [&](int q, int buf) {
        const int kk = min(t64::kP, K - q * t64::kP);
        t64::load_block(A, M, lda, row0, q * t64::kP, kk, sa[buf]);
        t64::load_block(B, N, ldb, col0, q * t64::kP, kk, sb[buf]);
        t64::cp_async_commit();
    };
    issue(0, 0);
    for (int q = 0; q < nk; ++q) {
        const int buf = q & 1;
        if (q + 1 < nk) {
            issue(q + 1, buf ^ 1);
            t64::cp_async_wait_one();
        } else {
            t64::cp_async_wait_none();
        }
        __syncthreads();
        t64::tile_nt_acc(sa[buf], sb[buf], min(t64::kP, K - q * t64::kP), acc);
        __syncthreads();
    }
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            const int r = row0 + ty + 16 * a, c = col0 + tx + 16 * b;
            if (r < M && c < N && (!lower || c <= r)) {
                float* cp = C + (int64_t)r * ldc + c;
                *cp = alpha * acc[a][b] + (beta != 0.f ? beta * *cp : 0.f);
            }
        }
}

unsigned grid_of(int64_t items) { return (unsigned)std::max<int64_t>(1, std::min<int64_t>((items + 255) / 256, 4096)); }

}  // namespace

cudaError_t launch_gemm_nt64(int M, int N, int K, const float* A, int lda, const float* B, int ldb, float* C, int ldc,
                             float alpha, float beta, bool lower, const LmState* st, cudaStream_t s) {
    if (M <= 0 || N <= 0) return cudaSuccess;
    static std::atomic<int> attr_set[kMaxDevices];
    if (per_device(attr_set, [] {
            return cudaFuncSetAttribute(k_gemm_nt64, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)kGemm64Smem) == cudaSuccess
                       ? 1
                       : 0;
        }) < 1)
        return cudaErrorInvalidConfiguration;
    const dim3 grid((N + t64::kP - 1) / t64::kP, (M + t64::kP - 1) / t64::kP);
    k_gemm_nt64<<<grid, t64::kThreads, kGemm64Smem, s>>>(M, N, K, A, lda, B, ldb, C, ldc, alpha, beta, lower ? 1 : 0,
                                                          st);
    note_launch();
    return cudaGetLastError();
}

int chol_tc_scratch_floats(int n) { return 3 * n * kPanel; }

bool chol_tc_applies(int n) { return n >= kTcMinN && n % 4 == 0; }

TcStreams::~TcStreams() { release(); }

void TcStreams::release() {
    for (cudaEvent_t e : ev) cudaEventDestroy(e);
    ev.clear();
    for (cudaStream_t* p : {&hi, &mid, &lo})
        if (*p) cudaStreamDestroy(*p);
    hi = mid = lo = nullptr;
}

cudaError_t TcStreams::init(int n) {
    release();
    int least = 0, greatest = 0;
    cudaError_t e = cudaDeviceGetStreamPriorityRange(&least, &greatest);
    if (e != cudaSuccess) return e;
    if ((e = cudaStreamCreateWithPriority(&hi, cudaStreamNonBlocking, greatest)) != cudaSuccess) return e;
    if ((e = cudaStreamCreateWithPriority(&mid, cudaStreamNonBlocking, greatest)) != cudaSuccess) return e;
    if ((e = cudaStreamCreateWithPriority(&lo, cudaStreamNonBlocking, least)) != cudaSuccess) return e;
    ev.resize(4 * (size_t)panels_of(n) + 2, nullptr);
    for (cudaEvent_t& x : ev)
        if ((e = cudaEventCreateWithFlags(&x, cudaEventDisableTiming)) != cudaSuccess) return e;
    return cudaSuccess;
}

int TcStreams::panels_of(int n) { return (n + kPanel - 1) / kPanel; }

cudaError_t launch_chol_inverse_tc(int n, float* F, float* X, float* XT, float* scratch, LmState* st, int* flags,
                                   int* epoch, TcStreams& ts, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    const int panels = TcStreams::panels_of(n);
    if (n % 4 != 0 || !ts.hi || ts.ev.size() < 4 * (size_t)panels + 2) return cudaErrorInvalidValue;
    // two panel buffers (panel k uses P[k & 1]) and the block row of X
    float* Pb[2] = {scratch, scratch + (size_t)n * kPanel};
    float* Q = scratch + 2 * (size_t)n * kPanel;
    cudaEvent_t* E = ts.ev.data();  // [panels] hi: panel k's diagonal block, the top of P, the next diagonal block
    cudaEvent_t* M = E + panels;    // [panels] mid: the rest of P and the next panel's columns below it
    cudaEvent_t* R = M + panels;    // [panels] lo: the rest of panel k's trailing update
    cudaEvent_t* G = R + panels;    // [panels] lo: all of panel k's work
    cudaEvent_t fork = G[panels], join = G[panels + 1];
    cudaStream_t hi = ts.hi, mid = ts.mid, lo = ts.lo;
    int* err = &st->timeout;
    // the bulk stream's products leave 16 SMs to the dataflow launches of the
    // chain (measured at n = 6000: 4.46 ms against 4.80 with no cap)
    static std::atomic<int> sm_cache[kMaxDevices];
    const int sms = per_device(sm_cache, [] {
        int dev = 0, n = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        return n;
    });
    const int lo_cap = sms > 32 ? sms - 16 : 0;
    cudaError_t e;
#define ZS_TRY(x)                               \
    do {                                        \
        if ((e = (x)) != cudaSuccess) return e; \
    } while (0)
    ZS_TRY(cudaEventRecord(fork, s));
    for (cudaStream_t x : {hi, mid, lo}) ZS_TRY(cudaStreamWaitEvent(x, fork, 0));
    const int64_t nn4 = (int64_t)n * n / 4;
    k_zero<<<grid_of(nn4), 256, 0, hi>>>(nn4, reinterpret_cast<float4*>(XT), st);
    note_launch();
    // Panel k's trailing update S_22 -= P P^T is cut by column blocks: the
    // next panel's diagonal block (hi), the rest of the next panel's columns
    // (mid), the panel after it (mid) and everything beyond (lo). A block is
    // written by one panel after another, so each write waits for the
    // previous panel's write of the same block: R[k - 1] (lo's region of
    // panel k - 1 starts at the columns of panel k + 2).
    for (int k = 0; k < panels; ++k) {
        const int o = k * kPanel, b = std::min(kPanel, n - o), m = n - o - b;
        const int bn = std::min(kPanel, m);       // the next panel's width
        const int bn2 = std::min(kPanel, m - bn);  // the width of the panel after it
        const int r2 = m - bn - bn2;               // the columns beyond those
        float* Fkk = F + (size_t)o * n + o;
        float* Xkk = X + (size_t)o * n + o;
        float* S21 = F + (size_t)(o + b) * n + o;
        float* P = Pb[k & 1];
        float* F22 = F + (size_t)(o + b) * n + o + b;  // the trailing block
        // hi, the chain: the diagonal block, the top rows of P = S_21 X_kk^T
        // (L_21's rows of the next panel) and the next diagonal block's
        // update, the last two as FP32-pipe tiles (k_gemm_nt64)
        ZS_TRY(launch_chol_inverse_dag_ld(b, n, Fkk, Xkk, XT + (size_t)o * n + o, st, flags, epoch, hi));
        if (m > 0) {
            if (k >= 2) ZS_TRY(cudaStreamWaitEvent(hi, G[k - 2], 0));  // P[k & 1] is free
            if (k >= 1) ZS_TRY(cudaStreamWaitEvent(hi, M[k - 1], 0));  // S_21 is final
            ZS_TRY(launch_gemm_nt64(bn, b, b, S21, n, Xkk, n, P, kPanel, 1.f, 0.f, false, st, hi));
            k_copy_block<<<grid_of((int64_t)bn * b / 4), 256, 0, hi>>>(bn, b, P, kPanel, S21, n, st);
            note_launch();
            if (k >= 2) ZS_TRY(cudaStreamWaitEvent(hi, R[k - 2], 0));
            ZS_TRY(launch_gemm_nt64(bn, bn, b, P, kPanel, P, kPanel, F22, n, -1.f, 1.f, true, st, hi));
        }
        ZS_TRY(cudaEventRecord(E[k], hi));
        // mid, beside the next dataflow launch: the rest of P, the next
        // panel's columns below its diagonal block, and the panel after it
        ZS_TRY(cudaStreamWaitEvent(mid, E[k], 0));
        if (m > bn) {
            const int r = m - bn;
            float* Pr = P + (size_t)bn * kPanel;
            float* S21r = S21 + (size_t)bn * n;
            ZS_TRY(launch_tc_gemm_nt(r, b, b, S21r, n, Xkk, n, Pr, kPanel, 1.f, 0.f, false, err, mid, st));
            k_copy_block<<<grid_of((int64_t)r * b / 4), 256, 0, mid>>>(r, b, Pr, kPanel, S21r, n, st);
            note_launch();
            if (k >= 2) ZS_TRY(cudaStreamWaitEvent(mid, R[k - 2], 0));
            ZS_TRY(launch_tc_gemm_nt(r, bn, b, Pr, kPanel, P, kPanel, F22 + (size_t)bn * n, n, -1.f, 1.f, false, err,
                                     mid, st));
            if (k >= 1) ZS_TRY(cudaStreamWaitEvent(mid, R[k - 1], 0));
            ZS_TRY(launch_tc_gemm_nt(r, bn2, b, Pr, kPanel, Pr, kPanel, F22 + (size_t)bn * n + bn, n, -1.f, 1.f, true,
                                     err, mid, st));
        }
        ZS_TRY(cudaEventRecord(M[k], mid));
        // lo, the bulk: the trailing update beyond those columns, X's block
        // row k and the block rows below
        ZS_TRY(cudaStreamWaitEvent(lo, M[k], 0));
        if (r2 > 0) {
            float* Pz = P + (size_t)(bn + bn2) * kPanel;
            ZS_TRY(launch_tc_gemm_nt(r2, r2, b, Pz, kPanel, Pz, kPanel, F22 + (size_t)(bn + bn2) * (n + 1), n, -1.f,
                                     1.f, true, err, lo, st, lo_cap));
        }
        ZS_TRY(cudaEventRecord(R[k], lo));
        if (o > 0) {
            // Q = Y^T[0:o, k] X_kk^T, then into XT
            ZS_TRY(launch_tc_gemm_nt(o, b, b, XT + o, n, Xkk, n, Q, kPanel, 1.f, 0.f, false, err, lo, st, lo_cap));
            k_copy_block<<<grid_of((int64_t)o * b / 4), 256, 0, lo>>>(o, b, Q, kPanel, XT + o, n, st);
            note_launch();
        }
        if (m > 0)  // Y^T[0:o+b, o+b:n] -= XT[0:o+b, k] P^T
            ZS_TRY(launch_tc_gemm_nt(o + b, m, b, XT + o, n, P, kPanel, XT + o + b, n, -1.f, 1.f, false, err, lo, st,
                                     lo_cap));
        ZS_TRY(cudaEventRecord(G[k], lo));
    }
    ZS_TRY(cudaStreamWaitEvent(hi, G[panels - 1], 0));
    const int nt = (n + kTile - 1) / kTile;
    k_lower_from_upper<<<(unsigned)((int64_t)nt * (nt + 1) / 2), kTile * 8, 0, hi>>>(n, XT, X, st);
    note_launch();
    ZS_TRY(cudaGetLastError());
    ZS_TRY(cudaEventRecord(join, hi));
    ZS_TRY(cudaStreamWaitEvent(s, join, 0));
#undef ZS_TRY
    return cudaSuccess;
}

}  // namespace zs

// ---- C ABI: the preconditioner's factor and inverse on host arrays (tests and measurements) ----
#include <vector>

#include "../../include/zeroslam_ba.h"

extern "C" int zs_dense_chol_inverse_f32(const float* S, int n, float* L, float* X, int form, double* ms) {
    using namespace zs;
    if (!S || n <= 0 || form < 0 || form > 2) return ZS_ERR_INVALID;
    const bool blocked = form == 2 || (form == 0 && chol_tc_applies(n));
    if (blocked && n % 4 != 0) return ZS_ERR_INVALID;
    const size_t nn = (size_t)n * n;
    float *dF = nullptr, *dX = nullptr, *dXT = nullptr, *dscr = nullptr;
    int* flags = nullptr;
    LmState* st = nullptr;
    cudaStream_t s = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int status = ZS_OK;
    cudaError_t e;
    auto fail = [&](cudaError_t err) { status = record_cuda_error(err); };
    LmState init{};
    init.solve_ok = 1;
    int epoch = 0;
    TcStreams ts;
    if ((e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking)) != cudaSuccess) {
        fail(e);
        return status;
    }
    if ((e = cudaMalloc(&dF, 4 * nn)) != cudaSuccess || (e = cudaMalloc(&dX, 4 * nn)) != cudaSuccess ||
        (e = cudaMalloc(&dXT, 4 * nn)) != cudaSuccess ||
        (e = cudaMalloc(&flags, sizeof(int) * (size_t)dag_flag_ints(n))) != cudaSuccess ||
        (e = cudaMalloc(&st, sizeof(LmState))) != cudaSuccess ||
        (blocked && (e = cudaMalloc(&dscr, sizeof(float) * (size_t)chol_tc_scratch_floats(n))) != cudaSuccess) ||
        (e = cudaEventCreate(&e0)) != cudaSuccess || (e = cudaEventCreate(&e1)) != cudaSuccess) {
        fail(e);
    } else if ((e = cudaMemcpyAsync(dF, S, 4 * nn, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
               (e = cudaMemsetAsync(dX, 0, 4 * nn, s)) != cudaSuccess ||
               (e = cudaMemsetAsync(dXT, 0, 4 * nn, s)) != cudaSuccess ||
               (e = cudaMemsetAsync(flags, 0, sizeof(int) * (size_t)dag_flag_ints(n), s)) != cudaSuccess ||
               (e = cudaMemcpyAsync(st, &init, sizeof(init), cudaMemcpyHostToDevice, s)) != cudaSuccess ||
               (e = cudaEventRecord(e0, s)) != cudaSuccess ||
               (blocked && (e = ts.init(n)) != cudaSuccess) ||
               (e = blocked ? launch_chol_inverse_tc(n, dF, dX, dXT, dscr, st, flags, &epoch, ts, s)
                            : launch_chol_inverse_dag(n, dF, dX, dXT, st, flags, &epoch, s)) != cudaSuccess ||
               (e = cudaEventRecord(e1, s)) != cudaSuccess ||
               (L && (e = cudaMemcpyAsync(L, dF, 4 * nn, cudaMemcpyDeviceToHost, s)) != cudaSuccess) ||
               (X && (e = cudaMemcpyAsync(X, dX, 4 * nn, cudaMemcpyDeviceToHost, s)) != cudaSuccess) ||
               (e = cudaMemcpyAsync(&init, st, sizeof(init), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
               (e = cudaStreamSynchronize(s)) != cudaSuccess) {
        fail(e);
    } else {
        float t = 0.f;
        if ((e = cudaEventElapsedTime(&t, e0, e1)) != cudaSuccess) fail(e);
        if (ms) *ms = t;
        if (status == ZS_OK) status = init.timeout ? ZS_ERR_TIMEOUT : (init.solve_ok ? ZS_OK : ZS_ERR_CHOLESKY);
        for (int i = 0; i < n; ++i)
            for (int j = i + 1; j < n; ++j) {
                if (L) L[(size_t)i * n + j] = 0.f;
                if (X) X[(size_t)i * n + j] = 0.f;
            }
    }
    cudaFree(dF);
    cudaFree(dX);
    cudaFree(dXT);
    cudaFree(dscr);
    cudaFree(flags);
    cudaFree(st);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaStreamDestroy(s);
    return status;
}
