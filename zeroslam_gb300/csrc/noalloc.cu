// zs_dense_cholesky_solve_noalloc: the FP64 dense SPD solve of
// zs_dense_cholesky_solve without any device allocation.
//
// Who needs it: callers that must not allocate device memory once they are
// running, e.g. a real-time tracking thread that cannot afford to block in
// the allocator or to meet an out-of-memory error mid-sequence, or a host
// application whose device memory is owned by another allocator (a
// framework's memory pool) so that a private cudaMalloc is not allowed.
//
// How: every device buffer the solve needs (device copies of A and b, the
// factor, the diagonal-block inverses, the solve vectors and the status
// word) is carved out of one file-scope __device__ array of fixed size,
// sized for n <= ZS_NOALLOC_MAX_N. The array exists once per device that
// loads this library and stays allocated until the process exits.
#include <cstdio>
#include <cstring>

#include "../../include/zeroslam_ba.h"
#include "ba_internal.h"

namespace {

constexpr int kMaxN = ZS_NOALLOC_MAX_N;
constexpr size_t kBlocks = (kMaxN + 31) / 32;
constexpr size_t kStateDoubles = (sizeof(zs::LmState) + sizeof(double) - 1) / sizeof(double);
// A and F (n x n each), D (32 x 32 per diagonal block), b, x, the solve
// vectors (4n + 256) and the status word, all in doubles.
constexpr size_t kScratchDoubles =
    2 * (size_t)kMaxN * kMaxN + kBlocks * 1024 + 2 * (size_t)kMaxN + (4 * (size_t)kMaxN + 256) + kStateDoubles;

__device__ __align__(256) double g_scratch[kScratchDoubles];

// Device address of g_scratch per device ordinal. In host code the symbol
// g_scratch is only a host-side stand-in, so the address is looked up with
// cudaGetSymbolAddress, once per device, with that device current. The
// cached address belongs to the device's current context: a caller that
// resets a device (cudaDeviceReset) must not call this entry point on that
// device again in the same process.
constexpr int kMaxDevices = 64;
double* g_scratch_ptr[kMaxDevices] = {nullptr};

// A CUDA failure: recorded as zs_last_error() like every other entry point's.
int fail(cudaError_t e) { return zs::record_cuda_error(e); }

}  // namespace

extern "C" int zs_dense_cholesky_solve_noalloc(const double* A, int n, const double* b, double* L, double* x) {
    if (!A || !b || n <= 0) return ZS_ERR_INVALID;
    if (n > kMaxN) return ZS_ERR_INVALID;  // beyond the fixed workspace
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(e);
    if (dev < 0 || dev >= kMaxDevices) return fail(cudaErrorInvalidDevice);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_scratch);
        if (e != cudaSuccess) return fail(e);
        if (!p) return fail(cudaErrorInvalidSymbol);
        g_scratch_ptr[dev] = static_cast<double*>(p);
    }
    double* base = g_scratch_ptr[dev];
    const size_t nn = (size_t)n * n;
    double* dA = base;
    double* dF = dA + nn;
    double* dD = dF + nn;
    double* db = dD + 1024 * (size_t)((n + 31) / 32);
    double* dx = db + n;
    double* dwork = dx + n;
    zs::LmState* st = reinterpret_cast<zs::LmState*>(base + (kScratchDoubles - kStateDoubles));

    // The status word keeps the previous call's contents: reset it.
    zs::LmState init;
    std::memset(&init, 0, sizeof(init));
    init.solve_ok = 1;
    cudaStream_t s = 0;
    if ((e = cudaMemcpyAsync(st, &init, sizeof(init), cudaMemcpyHostToDevice, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(dA, A, nn * sizeof(double), cudaMemcpyHostToDevice, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(db, b, n * sizeof(double), cudaMemcpyHostToDevice, s)) != cudaSuccess)
        return fail(e);
    if ((e = zs::launch_reduced_solve<double, double>(n, dA, dF, dD, db, dx, dwork, st, 0, 0.0, s)) != cudaSuccess)
        return fail(e);
    zs::LmState out;
    if ((e = cudaMemcpyAsync(&out, st, sizeof(out), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (x && (e = cudaMemcpyAsync(x, dx, n * sizeof(double), cudaMemcpyDeviceToHost, s)) != cudaSuccess) ||
        (L && (e = cudaMemcpyAsync(L, dF, nn * sizeof(double), cudaMemcpyDeviceToHost, s)) != cudaSuccess) ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess)
        return fail(e);
    if (L)
        for (int i = 0; i < n; ++i)
            for (int j = i + 1; j < n; ++j) L[(size_t)i * n + j] = 0.0;
    return out.solve_ok ? ZS_OK : ZS_ERR_CHOLESKY;
}
