// scir_probe_fma_peak: measured FMA throughput of the current device's CUDA
// cores, the roofline denominator for the kernels that are bound by the FP32
// pipe (long-tap FIR on the CUDA cores, ragged FIR) or by the FP64 pipe (the
// FP64-state SOS recursion).  Every thread runs kChains independent FMA
// chains (enough to cover the FMA latency at full occupancy), so the loop is
// bound only by the FMA pipe; the kernel is timed with CUDA events on a
// private stream after a warm-up launch.
#include "common.cuh"

namespace scir {
namespace {

constexpr int kChains = 16;

template <typename T>
__global__ void __launch_bounds__(256) fma_peak_kernel(T* out, int iters, T b, T c) {
    T v[kChains];
#pragma unroll
    for (int i = 0; i < kChains; ++i) v[i] = (T)(threadIdx.x + i) * (T)1e-3;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int i = 0; i < kChains; ++i) v[i] = fma(v[i], b, c);
    }
    T s = 0;
#pragma unroll
    for (int i = 0; i < kChains; ++i) s += v[i];
    if (s == (T)-1.2345) out[0] = s;  // keeps the chains live; never true for these inputs
}

template <typename T>
int probe(int iters, double* tflops) {
    const DeviceInfo* info = nullptr;
    int rc = current_device(&info);
    if (rc) return rc;
    cudaStream_t st = nullptr;
    SCIR_CUDA_TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    T* out = nullptr;
    cudaError_t e = cudaMallocAsync(&out, sizeof(T), st);
    const int blocks = info->sm_count * 8;  // 8 x 256 threads = 64 warps per SM
    float ms = 0.0f;
    if (e == cudaSuccess) {
        // b just below 1 and a small c keep every chain finite and non-denormal
        fma_peak_kernel<T><<<blocks, 256, 0, st>>>(out, iters / 4, (T)0.999999, (T)1e-4);
        cudaEventRecord(e0, st);
        fma_peak_kernel<T><<<blocks, 256, 0, st>>>(out, iters, (T)0.999999, (T)1e-4);
        cudaEventRecord(e1, st);
        e = cudaStreamSynchronize(st);
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
        cudaFreeAsync(out, st);
        cudaStreamSynchronize(st);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaStreamDestroy(st);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_error(SCIR_ERR_CUDA, "FMA probe failed: %s", cudaGetErrorString(e));
    }
    const double flops = 2.0 * kChains * (double)iters * blocks * 256.0;
    *tflops = flops / (ms * 1e-3) / 1e12;
    return SCIR_OK;
}

}  // namespace
}  // namespace scir

using namespace scir;

extern "C" SCIR_API int scir_probe_fma_peak(int fp64, double* tflops) {
    clear_error();
    SCIR_REQUIRE(tflops != nullptr, SCIR_ERR_INVALID_ARG, "tflops is NULL");
    *tflops = 0.0;
    // about 0.3 s of work each at the expected rates (~70 TFLOP/s FP32,
    // ~1.2 TFLOP/s FP64 on a GB300)
    return fp64 ? probe<double>(1 << 5, tflops) : probe<float>(1 << 11, tflops);
}
