// sdt_common.cuh -- device helpers shared by the CUDA translation units.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <string>
#include "sdt_internal.h"

namespace sdt {

// FP64 tensor-core MMA: D(8x8) += A(8x4, row) * B(4x8, col).  Fragment
// ownership per lane l: A[l>>2][l&3], B[l&3][l>>2], C[l>>2][2*(l&3)+{0,1}].
__device__ __forceinline__ void dmma_8x8x4(double &c0, double &c1, double a, double b) {
    asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};\n"
                 : "+d"(c0), "+d"(c1)
                 : "d"(a), "d"(b));
}

// Neumaier-compensated accumulation of one double pair.
struct Comp {
    double s = 0.0, c = 0.0;
    __host__ __device__ void add(double x) {
        const double t = s + x;
        if (fabs(s) >= fabs(x)) c += (s - t) + x;
        else c += (x - t) + s;
        s = t;
    }
    __host__ __device__ double value() const { return s + c; }
};

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Library stream on the current device (created on first use).
cudaStream_t lib_stream();
// Returns SDT_OK or records a CUDA error with context.
int cuda_check(cudaError_t e, const char *what);

// Caching allocator (device and pinned host), memory.cu semantics.  Blocks
// taken with tile = true belong to the reference tile ABI and are the ones
// finalizememmodule_ requires to be released.
void *gpu_get(size_t bytes, bool tile = false);
void gpu_put(void *p);
void *host_get(size_t bytes, bool tile = false);
void host_put(void *p);

// Reduction of per-block (E[T], E(T)) partials: out[2] on the device.
// partials holds 2*n doubles laid out [e1_0, e2_0, e1_1, e2_1, ...].
int reduce_pairs(const double *partials, int64_t n, double *out_dev, cudaStream_t st);

}  // namespace sdt
