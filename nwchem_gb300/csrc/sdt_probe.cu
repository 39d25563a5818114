// sdt_probe.cu -- FP64 tensor-core peak probe (the FP64 roofline denominator).
//
// Each warp issues independent mma.sync m8n8k4.f64 into 8 accumulator pairs
// from register operands, so neither memory nor dependencies limit it.
#include "sdt_common.cuh"

namespace sdt {
namespace {
__global__ void __launch_bounds__(256) fp64_mma_probe(double *out, int iters, double s) {
    double a = threadIdx.x * 1e-3 + s, b = 1.0 - threadIdx.x * 1e-4;
    double c[8][2];
#pragma unroll
    for (int q = 0; q < 8; ++q) c[q][0] = c[q][1] = 0.0;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int q = 0; q < 8; ++q) dmma_8x8x4(c[q][0], c[q][1], a, b);
    }
    double r = 0.0;
#pragma unroll
    for (int q = 0; q < 8; ++q) r += c[q][0] + c[q][1];
    out[blockIdx.x * blockDim.x + threadIdx.x] = r;
}
}  // namespace
}  // namespace sdt

using namespace sdt;

extern "C" double sdt_probe_fp64_tflops(int ms) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int blocks = sms * 4, threads = 256;
    double *out = (double *)gpu_get((size_t)blocks * threads * sizeof(double));
    if (!out) return -1.0;
    cudaStream_t st = lib_stream();
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    fp64_mma_probe<<<blocks, threads, 0, st>>>(out, 16, 0.0);
    count_launch();
    // Calibrate the iteration count to about `ms` milliseconds.
    int iters = 512;
    float t = 0.0f;
    for (int pass = 0; pass < 6; ++pass) {
        cudaEventRecord(e0, st);
        fp64_mma_probe<<<blocks, threads, 0, st>>>(out, iters, 0.0);
        count_launch();
        cudaEventRecord(e1, st);
        cudaEventSynchronize(e1);
        cudaEventElapsedTime(&t, e0, e1);
        if (t >= 0.5f * ms || iters > (1 << 24)) break;
        iters *= 4;
    }
    const double flops = 512.0 * 8.0 * (double)iters * blocks * (threads / 32);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    gpu_put(out);
    if (cudaGetLastError() != cudaSuccess || t <= 0.0f) return -1.0;
    return flops / (t * 1e-3) / 1e12;
}
