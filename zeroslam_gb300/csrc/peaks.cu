// FP64 / FP32 fused multiply-add pipe peaks (zs_pipe_peaks in
// include/zeroslam_ba.h): every thread runs eight independent FMA chains in
// registers on a grid that fills every SM, timed with CUDA events. The
// roofline denominators of the FP64-pipe-bound kernels come from here.
#include <cuda_runtime.h>

#include "../../include/zeroslam_ba.h"

namespace {

template <typename T>
__global__ void __launch_bounds__(256) k_fma_chain(T* out, int iters, T a, T b) {
    T x0 = (T)threadIdx.x * (T)1e-3, x1 = x0 + (T)0.1, x2 = x0 + (T)0.2, x3 = x0 + (T)0.3;
    T x4 = x0 + (T)0.4, x5 = x0 + (T)0.5, x6 = x0 + (T)0.6, x7 = x0 + (T)0.7;
    for (int i = 0; i < iters; ++i) {
        x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
        x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
    }
    const T s = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
    if (s == (T)-12345.0) out[blockIdx.x] = s;  // never true; keeps the chains alive
}

template <typename T>
double measure(int sms, int iters) {
    T* out = nullptr;
    if (cudaMalloc(&out, sizeof(T) * 4096) != cudaSuccess) return -1.0;
    const int blocks = sms * 8;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    k_fma_chain<T><<<blocks, 256>>>(out, iters / 10 + 1, (T)0.999999, (T)1e-6);  // warm-up
    cudaEventRecord(e0);
    k_fma_chain<T><<<blocks, 256>>>(out, iters, (T)0.999999, (T)1e-6);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (cudaGetLastError() != cudaSuccess || ms <= 0.f) return -1.0;
    const double fmas = (double)blocks * 256.0 * 8.0 * (double)iters;
    return 2.0 * fmas / (ms * 1e-3) / 1e12;
}

}  // namespace

extern "C" int zs_pipe_peaks(int device, double* fp64_tflops, double* fp32_tflops) {
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || device < 0 || device >= count) {
        cudaGetLastError();
        return ZS_ERR_CUDA;
    }
    if (cudaSetDevice(device) != cudaSuccess) return ZS_ERR_CUDA;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const double f64 = measure<double>(sms, 20000);
    const double f32 = measure<float>(sms, 400000);
    if (f64 <= 0.0 || f32 <= 0.0) return ZS_ERR_CUDA;
    if (fp64_tflops) *fp64_tflops = f64;
    if (fp32_tflops) *fp32_tflops = f32;
    return ZS_OK;
}
