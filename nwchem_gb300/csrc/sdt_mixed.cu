// sdt_mixed.cu -- building blocks of the mixed-precision form on
// 5th-generation tensor cores, and their self-tests.
//
// Split products: an FP64 operand x is stored as two narrower values
// hi = round(x), lo = round(x - hi) and a product is taken as
// hi*hi + hi*lo + lo*hi with FP32 accumulation in tensor memory:
//   TF32x3  (kind::tf32, fp32 containers)      ~2^-22 of |x*y|
//   FP16x3  (kind::f16, power-of-two scaled)   ~2^-22 of |x*y|
//   BF16x3  (kind::f16 with bf16)              ~2^-16 of |x*y|
//
// This file holds the tensor-map encoder, a one-CTA split GEMM that checks
// the TMA / descriptor / TMEM / MMA path for each operand type (every
// mbarrier wait is bounded in time: on a timeout an error flag is set and
// the kernel drains and returns instead of spinning), and a check of the
// FP64 division used by the energy epilogue.
#include "sdt_common.cuh"
#include "sdt_job.h"
#include "sdt_tc.cuh"

#include <algorithm>
#include <cstring>
#include <vector>

#include <cuda.h>
#include <mutex>

namespace sdt {

// cuTensorMapEncodeTiled through the runtime's driver entry point (the
// library does not link libcuda directly).
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                  const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                  const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_tiled() {
    static std::once_flag once;
    static EncodeTiledFn fn = nullptr;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (EncodeTiledFn)p;
        else
            cudaGetLastError();
    });
    return fn;
}

// Tensor map of fp32 (TM_F32), bf16 (TM_BF16) or fp16 (TM_F16) elements
// with 32- or 64-byte swizzle; dims innermost first, strides in bytes for
// dims 1..rank-1.
int make_tmap(CUtensorMap *map, const void *base, int type, int rank, const uint64_t *dims,
              const uint64_t *strides_bytes, const uint32_t *box, int swizzle_bytes) {
    EncodeTiledFn fn = encode_tiled();
    if (!fn) return fail(SDT_ERR_CUDA, "cuTensorMapEncodeTiled is unavailable");
    if ((reinterpret_cast<uintptr_t>(base) & 15) != 0) return fail(SDT_ERR_ARG, "tensor map base not 16-byte aligned");
    const int es = type == TM_F32 ? 4 : 2;
    cuuint64_t gd[5], gs[4];
    cuuint32_t bx[5], el[5];
    for (int i = 0; i < rank; ++i) {
        gd[i] = dims[i];
        bx[i] = box[i];
        el[i] = 1;
        if (i > 0) {
            if (strides_bytes[i - 1] % 16) return fail(SDT_ERR_ARG, "tensor map stride not a multiple of 16 bytes");
            gs[i - 1] = strides_bytes[i - 1];
        }
    }
    if (swizzle_bytes != 32 && swizzle_bytes != 64) return fail(SDT_ERR_ARG, "swizzle must be 32 or 64 bytes");
    if ((int)box[0] * es != swizzle_bytes) return fail(SDT_ERR_ARG, "tensor map inner box must span its swizzle");
    const CUtensorMapDataType dt = type == TM_F32    ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32
                                   : type == TM_BF16 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16
                                                     : CU_TENSOR_MAP_DATA_TYPE_FLOAT16;
    CUresult r = fn(map, dt, rank, const_cast<void *>(base), gd, gs, bx, el, CU_TENSOR_MAP_INTERLEAVE_NONE,
                    swizzle_bytes == 32 ? CU_TENSOR_MAP_SWIZZLE_32B : CU_TENSOR_MAP_SWIZZLE_64B,
                    CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(SDT_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
    return SDT_OK;
}

namespace {

constexpr uint64_t kWaitNs = 2000000000ull;  // 2 s per wait
constexpr int ST_ROW = 64;                   // bytes of one K row of a stage (64-byte swizzle)
constexpr int ST_M = 128, ST_N = 256;
constexpr int A_BYTES = ST_M * ST_ROW;       // 8 KB
constexpr int B_BYTES = ST_N * ST_ROW;       // 16 KB
constexpr int STAGE_BYTES = 2 * A_BYTES + 2 * B_BYTES;

struct SelfTestArgs {
    CUtensorMap a_hi, a_lo, b_hi, b_lo;  // [M=128][K], [N=256][K]
    int K;
    float *D;   // [128][256]
    int *err;
};

// One CTA, 6 warps: 0 TMA producer, 1 MMA issuer + TMEM owner, 2-5 epilogue.
// TYPE: TM_F32 (TF32 operands, kind::tf32) or TM_BF16 / TM_F16 (kind::f16).
template <int TYPE>
__global__ void __launch_bounds__(192, 1) tc_selftest_kernel(const __grid_constant__ SelfTestArgs g) {
    constexpr int ES = TYPE == TM_F32 ? 4 : 2;
    constexpr int KC = ST_ROW / ES;  // K elements per stage
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint64_t *full = (uint64_t *)(smem + 2 * STAGE_BYTES);
    uint64_t *empty = full + 2;
    uint64_t *tfull = empty + 2;
    uint32_t *tslot = (uint32_t *)(tfull + 1);
    volatile int *abort = (volatile int *)(tslot + 1);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nk = (g.K + KC - 1) / KC;

    if (threadIdx.x == 0) {
        for (int s = 0; s < 2; ++s) {
            tc::mbar_init(&full[s], 1);
            tc::mbar_init(&empty[s], 1);
        }
        tc::mbar_init(tfull, 1);
        *abort = 0;
        tc::fence_mbar_init();
    }
    if (warp == 1) tc::tmem_alloc(tslot, 256);
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    const uint32_t tmem = *tslot;

    if (warp == 0 && lane == 0) {
        tc::prefetch_tmap(&g.a_hi);
        tc::prefetch_tmap(&g.b_hi);
        for (int kc = 0; kc < nk && !*abort; ++kc) {
            const int s = kc & 1;
            if (kc >= 2 && !tc::mbar_wait(&empty[s], ((kc >> 1) & 1) ^ 1, kWaitNs, abort)) {
                *abort = 1;
                atomicExch(g.err, 1);
                break;
            }
            uint8_t *st = smem + s * STAGE_BYTES;
            tc::mbar_arrive_expect_tx(&full[s], STAGE_BYTES);
            tc::tma_load_2d(st, &g.a_hi, &full[s], kc * KC, 0);
            tc::tma_load_2d(st + A_BYTES, &g.a_lo, &full[s], kc * KC, 0);
            tc::tma_load_2d(st + 2 * A_BYTES, &g.b_hi, &full[s], kc * KC, 0);
            tc::tma_load_2d(st + 2 * A_BYTES + B_BYTES, &g.b_lo, &full[s], kc * KC, 0);
        }
    } else if (warp == 1 && lane == 0) {
        const uint32_t idesc = TYPE == TM_F32 ? tc::idesc_tf32(ST_M, ST_N) : tc::idesc_f16(ST_M, ST_N, TYPE == TM_BF16);
        for (int kc = 0; kc < nk; ++kc) {
            const int s = kc & 1;
            if (!tc::mbar_wait(&full[s], (kc >> 1) & 1, kWaitNs, abort)) {
                *abort = 1;
                atomicExch(g.err, 2);
                break;
            }
            tc::tc_fence_after();
            const uint32_t st = tc::smem_u32(smem + s * STAGE_BYTES);
            for (int kk = 0; kk < 2; ++kk) {  // two 32-byte K steps per 64-byte row
                const uint32_t ah = st + kk * 32, al = st + A_BYTES + kk * 32;
                const uint32_t bh = st + 2 * A_BYTES + kk * 32, bl = st + 2 * A_BYTES + B_BYTES + kk * 32;
                const uint32_t first = (kc == 0 && kk == 0) ? 0u : 1u;
                if (TYPE == TM_F32) {
                    tc::mma_tf32(tmem, tc::sdesc_sw64(ah), tc::sdesc_sw64(bh), idesc, first);
                    tc::mma_tf32(tmem, tc::sdesc_sw64(ah), tc::sdesc_sw64(bl), idesc, 1u);
                    tc::mma_tf32(tmem, tc::sdesc_sw64(al), tc::sdesc_sw64(bh), idesc, 1u);
                } else {
                    tc::mma_f16(tmem, tc::sdesc_sw64(ah), tc::sdesc_sw64(bh), idesc, first);
                    tc::mma_f16(tmem, tc::sdesc_sw64(ah), tc::sdesc_sw64(bl), idesc, 1u);
                    tc::mma_f16(tmem, tc::sdesc_sw64(al), tc::sdesc_sw64(bh), idesc, 1u);
                }
            }
            tc::mma_commit(&empty[s]);
        }
        tc::mma_commit(tfull);
    } else if (warp >= 2) {
        const int quad = warp & 3;  // TMEM lanes 32*quad .. 32*quad+31
        if (tc::mbar_wait(tfull, 0, kWaitNs, abort)) {
            tc::tc_fence_after();
            const int row = quad * 32 + lane;
            for (int c = 0; c < ST_N / 32; ++c) {
                float v[32];
                tc::tmem_ld32(tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)(c * 32), v);
#pragma unroll
                for (int q = 0; q < 32; ++q) g.D[row * ST_N + c * 32 + q] = v[q];
            }
        } else {
            *abort = 1;
            atomicExch(g.err, 3);
        }
    }
    tc::tc_fence_before();
    __syncthreads();
    // Drain after an abort (bounded): copies in flight must land and issued
    // MMAs must finish before the CTA frees TMEM and exits.
    if (*abort && lane == 0 && warp <= 1) {
        volatile int never = 0;
        if (warp == 0)
            for (int s = 0; s < 2; ++s)
                for (uint32_t ph = 0; ph < 2; ++ph) tc::mbar_wait(&full[s], ph, kWaitNs / 8, &never);
        else
            tc::mbar_wait(tfull, 0, kWaitNs, &never);
    }
    __syncthreads();
    if (warp == 1) {
        tc::tc_fence_after();
        tc::tmem_dealloc(tmem, 256);
    }
}

template <int TYPE>
int run_selftest(const void *a_hi, const void *a_lo, const void *b_hi, const void *b_lo, int K, float *D,
                 const char *who) {
    constexpr int ES = TYPE == TM_F32 ? 4 : 2;
    SelfTestArgs g;
    const uint64_t da[2] = {(uint64_t)K, 128}, db[2] = {(uint64_t)K, 256};
    const uint64_t sa[1] = {(uint64_t)K * ES};
    const uint32_t ba[2] = {ST_ROW / ES, 128}, bb[2] = {ST_ROW / ES, 256};
    int rc = make_tmap(&g.a_hi, a_hi, TYPE, 2, da, sa, ba, 64);
    if (!rc) rc = make_tmap(&g.a_lo, a_lo, TYPE, 2, da, sa, ba, 64);
    if (!rc) rc = make_tmap(&g.b_hi, b_hi, TYPE, 2, db, sa, bb, 64);
    if (!rc) rc = make_tmap(&g.b_lo, b_lo, TYPE, 2, db, sa, bb, 64);
    if (rc) return rc;
    g.K = K;
    g.D = D;
    int *err = (int *)gpu_get(sizeof(int));
    if (!err) return fail(SDT_ERR_NOMEM, std::string(who) + ": flag");
    g.err = err;
    cudaStream_t st = lib_stream();
    const int smem = 2 * STAGE_BYTES + 1024 + 256;
    rc = cuda_check(cudaFuncSetAttribute(tc_selftest_kernel<TYPE>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem),
                    who);
    if (!rc) rc = cuda_check(cudaMemsetAsync(err, 0, sizeof(int), st), who);
    if (rc) {
        gpu_put(err);
        return rc;
    }
    tc_selftest_kernel<TYPE><<<1, 192, smem, st>>>(g);
    count_launch();
    int h = 0;
    rc = cuda_check(cudaGetLastError(), who);
    if (!rc) rc = cuda_check(cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, st), who);
    if (!rc) rc = cuda_check(cudaStreamSynchronize(st), who);
    gpu_put(err);
    if (rc) return rc;
    if (h) return fail(SDT_ERR_TIMEOUT, std::string(who) + ": a bounded wait ran out (stage " + std::to_string(h) + ")");
    return SDT_OK;
}

// Maximum relative error of the mixed form's FP32 energy quotient X/D
// against FP64 over n seeded samples, computed the way the energy warps
// compute it: orbital energies rounded to FP32 after the shift by the gap
// midpoint mu, D = ((e_i + e_j) + e_k) - ((e_a + e_b) + e_c) in FP32, and
// q = __fdividef(x, D).  Occupied levels in [-20, -0.25] (one sample in four
// with every hole in the valence range [-1.5, -0.25]), virtual levels in
// [0.05, 8], so mu = -0.1; x ~ U(-1,1) * 2^e (e in [-40, 40)), an FP32
// value.  The reference is x / D with D summed in FP64 from the unshifted
// levels.
__global__ void division_check_kernel(int64_t n, uint64_t seed, unsigned long long *worst_bits) {
    constexpr double kMu = -0.1;
    double worst = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        uint64_t z = seed + 0x9E3779B97F4A7C15ull * (uint64_t)(i + 1);
        double u[8];
#pragma unroll
        for (int r = 0; r < 8; ++r) {
            z += 0x9E3779B97F4A7C15ull;
            uint64_t y = z;
            y = (y ^ (y >> 30)) * 0xBF58476D1CE4E5B9ull;
            y = (y ^ (y >> 27)) * 0x94D049BB133111EBull;
            y ^= y >> 31;
            u[r] = (double)(y >> 11) * 0x1.0p-53;
        }
        const bool valence = (i & 3) == 0;
        double eo[3], ev[3];
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            eo[r] = valence ? -(0.25 + 1.25 * u[r]) : -(0.25 + 19.75 * u[r]);
            ev[r] = 0.05 + 7.95 * u[3 + r];
        }
        const int e = (int)(u[6] * 80.0) - 40;
        const float x = (float)ldexp(2.0 * u[7] - 1.0, e);
        float fo[3], fv[3];
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            fo[r] = (float)(eo[r] - kMu);
            fv[r] = (float)(ev[r] - kMu);
        }
        const float D32 = ((fo[0] + fo[1]) + fo[2]) - ((fv[0] + fv[1]) + fv[2]);
        const double D64 = (eo[0] + eo[1] + eo[2]) - (ev[0] + ev[1] + ev[2]);
        const double q = (double)__fdividef(x, D32), ref = (double)x / D64;
        if (ref != 0.0) worst = fmax(worst, fabs(q - ref) / fabs(ref));
    }
    atomicMax(worst_bits, (unsigned long long)__double_as_longlong(worst));
}

// The bounded mbarrier wait every kernel of the library uses, on a barrier
// nothing arrives on: it must give up after timeout_ns and report it.
// out[0] = SDT_ERR_TIMEOUT when it gave up (0 if the barrier completed),
// out[1] = microseconds waited.
__global__ void wait_timeout_kernel(uint64_t timeout_ns, int *out) {
    __shared__ uint64_t bar;
    __shared__ int abort_flag;
    if (threadIdx.x == 0) {
        tc::mbar_init(&bar, 1);
        abort_flag = 0;
        tc::fence_mbar_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const uint64_t t0 = tc::global_ns();
        const bool ok = tc::mbar_wait(&bar, 0, timeout_ns, &abort_flag);  // phase 0 never completes
        out[0] = ok ? 0 : SDT_ERR_TIMEOUT;
        out[1] = (int)((tc::global_ns() - t0) / 1000);
    }
}

}  // namespace
}  // namespace sdt

using namespace sdt;

// D[128][256] = A*B^T with A = a_hi + a_lo ([128][K]) and B = b_hi + b_lo
// ([256][K]) given as TF32 values in fp32 arrays; the three split products
// are accumulated in FP32 in tensor memory.  Returns SDT_ERR_TIMEOUT when a
// bounded wait inside the kernel ran out.
extern "C" int sdt_tc_selftest(const float *a_hi, const float *a_lo, const float *b_hi, const float *b_lo,
                               int K, float *D) {
    if (K < 4 || K % 4) return fail(SDT_ERR_ARG, "sdt_tc_selftest: K must be a positive multiple of 4");
    return run_selftest<TM_F32>(a_hi, a_lo, b_hi, b_lo, K, D, "sdt_tc_selftest");
}

// The same with 16-bit operands (bf16 != 0: BF16, else FP16; kind::f16).
extern "C" int sdt_tc_selftest16(const void *a_hi, const void *a_lo, const void *b_hi, const void *b_lo, int K,
                                 int bf16, float *D) {
    if (K < 8 || K % 8) return fail(SDT_ERR_ARG, "sdt_tc_selftest16: K must be a positive multiple of 8");
    if (bf16) return run_selftest<TM_BF16>(a_hi, a_lo, b_hi, b_lo, K, D, "sdt_tc_selftest16");
    return run_selftest<TM_F16>(a_hi, a_lo, b_hi, b_lo, K, D, "sdt_tc_selftest16");
}

extern "C" int sdt_check_division(int64_t n, uint64_t seed, double *max_rel_err) {
    if (n < 1 || !max_rel_err) return fail(SDT_ERR_ARG, "sdt_check_division: bad argument");
    unsigned long long *w = (unsigned long long *)gpu_get(sizeof(unsigned long long));
    if (!w) return fail(SDT_ERR_NOMEM, "sdt_check_division");
    cudaStream_t st = lib_stream();
    unsigned long long h = 0;
    int rc = cuda_check(cudaMemsetAsync(w, 0, sizeof(*w), st), "sdt_check_division");
    if (!rc) {
        division_check_kernel<<<152, 256, 0, st>>>(n, seed, w);
        count_launch();
        rc = cuda_check(cudaGetLastError(), "sdt_check_division");
    }
    if (!rc) rc = cuda_check(cudaMemcpyAsync(&h, w, sizeof(h), cudaMemcpyDeviceToHost, st), "sdt_check_division");
    if (!rc) rc = cuda_check(cudaStreamSynchronize(st), "sdt_check_division");
    gpu_put(w);
    if (rc) return rc;
    std::memcpy(max_rel_err, &h, sizeof(double));
    return SDT_OK;
}

// Failure-path check (no reference counterpart): one bounded wait on an
// mbarrier nothing arrives on, limited to timeout_s (at most 1 s).  Returns
// SDT_ERR_TIMEOUT with *waited_s the time it waited, as a kernel whose wait
// ran out would; the context stays usable.
extern "C" int sdt_check_wait_timeout(double timeout_s, double *waited_s) {
    if (!(timeout_s > 0.0 && timeout_s <= 1.0) || !waited_s)
        return fail(SDT_ERR_ARG, "sdt_check_wait_timeout: timeout must be in (0, 1] s");
    int *d = (int *)gpu_get(2 * sizeof(int));
    if (!d) return fail(SDT_ERR_NOMEM, "sdt_check_wait_timeout");
    cudaStream_t st = lib_stream();
    int h[2] = {0, 0};
    int rc = cuda_check(cudaMemsetAsync(d, 0, 2 * sizeof(int), st), "sdt_check_wait_timeout");
    if (!rc) {
        wait_timeout_kernel<<<1, 32, 0, st>>>((uint64_t)(timeout_s * 1e9), d);
        count_launch();
        rc = cuda_check(cudaGetLastError(), "sdt_check_wait_timeout");
    }
    if (!rc) rc = cuda_check(cudaMemcpyAsync(h, d, sizeof(h), cudaMemcpyDeviceToHost, st), "sdt_check_wait_timeout");
    if (!rc) rc = cuda_check(cudaStreamSynchronize(st), "sdt_check_wait_timeout");
    gpu_put(d);
    if (rc) return rc;
    *waited_s = h[1] * 1e-6;
    if (h[0] == SDT_ERR_TIMEOUT) return fail(SDT_ERR_TIMEOUT, "sdt_check_wait_timeout: the bounded wait ran out");
    return h[0];
}
