// Arithmetic-pipe peak probes used as roofline denominators by bench.py.
//
// The PR76 flash is bound by the FP64 (plain form) or FP32 (mixed form)
// arithmetic pipes, not by HBM or tensor cores.  These kernels run long
// chains of independent fused multiply-adds (8 chains per thread, every SM
// fully occupied) and report the sustained FMA rate in FLOP/s (2 flops per
// FMA).  Exported through a tiny C ABI of its own; not part of the flash ABI.
#include <cuda_runtime.h>
#include <stdint.h>

namespace {

template <typename T>
__global__ void fma_chains(T* out, int iters, T a, T b) {
    T x0 = threadIdx.x * T(1e-3), x1 = x0 + T(1), x2 = x0 + T(2), x3 = x0 + T(3);
    T x4 = x0 + T(4), x5 = x0 + T(5), x6 = x0 + T(6), x7 = x0 + T(7);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 16; ++k) {
            x0 = fma(x0, a, b);
            x1 = fma(x1, a, b);
            x2 = fma(x2, a, b);
            x3 = fma(x3, a, b);
            x4 = fma(x4, a, b);
            x5 = fma(x5, a, b);
            x6 = fma(x6, a, b);
            x7 = fma(x7, a, b);
        }
    }
    const T s = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
    if (s == T(-12345)) out[0] = s;  // keeps the chains live; never true
}

template <typename T>
double run(int iters) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    T* out = nullptr;
    if (cudaMalloc(&out, sizeof(T)) != cudaSuccess) return -1.0;
    const int block = 256, blocks = sms * 8;
    fma_chains<T><<<blocks, block>>>(out, 2, T(0.999999), T(1e-7));  // warm-up
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0);
    fma_chains<T><<<blocks, block>>>(out, iters, T(0.999999), T(1e-7));
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (cudaGetLastError() != cudaSuccess || ms <= 0) return -1.0;
    const double fmas = double(blocks) * block * iters * 16.0 * 8.0;
    return 2.0 * fmas / (ms * 1e-3);
}

}  // namespace

extern "C" {
// Sustained FP64 FMA rate in FLOP/s on the current device (negative on error).
double mpmc_probe_fp64_flops(int iters) { return run<double>(iters); }
// Sustained FP32 FMA rate in FLOP/s on the current device (negative on error).
double mpmc_probe_fp32_flops(int iters) { return run<float>(iters); }
}
