// sdt_mixed.cu -- the mixed-precision form on 5th-generation tensor cores.
//
// Split products: every FP64 operand x is stored as two TF32 values
// hi = tf32(x), lo = tf32(x - hi) (fp32 containers), and a product is taken
// as hi*hi + hi*lo + lo*hi with FP32 accumulation in tensor memory
// (tcgen05.mma kind::tf32).  The residual lo*lo and the split error are
// ~2^-22 of |x*y|.
//
// This file holds the building blocks and a self-test GEMM that checks
// them: TMA loads of 64-byte-swizzled K-major tiles, the shared-memory and
// instruction descriptors, TMEM allocation, MMA issue/commit and TMEM
// loads, with every mbarrier wait bounded in time (an error flag is set and
// the kernel drains and returns instead of spinning forever).
#include "sdt_common.cuh"
#include "sdt_job.h"
#include "sdt_tc.cuh"

#include <algorithm>
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

// fp32 tensor map with 64-byte swizzle; dims innermost first, strides in
// bytes for dims 1..rank-1.
int make_tmap_f32(CUtensorMap *map, const void *base, int rank, const uint64_t *dims,
                  const uint64_t *strides_bytes, const uint32_t *box, int swizzle_bytes) {
    EncodeTiledFn fn = encode_tiled();
    if (!fn) return fail(SDT_ERR_CUDA, "cuTensorMapEncodeTiled is unavailable");
    if ((reinterpret_cast<uintptr_t>(base) & 15) != 0) return fail(SDT_ERR_ARG, "tensor map base not 16-byte aligned");
    cuuint64_t gd[5], gs[4];
    cuuint32_t bx[5], es[5];
    for (int i = 0; i < rank; ++i) {
        gd[i] = dims[i];
        bx[i] = box[i];
        es[i] = 1;
        if (i > 0) {
            if (strides_bytes[i - 1] % 16) return fail(SDT_ERR_ARG, "tensor map stride not a multiple of 16 bytes");
            gs[i - 1] = strides_bytes[i - 1];
        }
    }
    if (swizzle_bytes != 32 && swizzle_bytes != 64) return fail(SDT_ERR_ARG, "swizzle must be 32 or 64 bytes");
    if ((int)box[0] * 4 > swizzle_bytes) return fail(SDT_ERR_ARG, "tensor map inner box wider than its swizzle");
    CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, rank, const_cast<void *>(base), gd, gs, bx, es,
                    CU_TENSOR_MAP_INTERLEAVE_NONE,
                    swizzle_bytes == 32 ? CU_TENSOR_MAP_SWIZZLE_32B : CU_TENSOR_MAP_SWIZZLE_64B,
                    CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(SDT_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
    return SDT_OK;
}

namespace {

constexpr uint64_t kWaitNs = 2000000000ull;  // 2 s per wait
constexpr int KC = 16;                       // fp32 K elements per stage (64 B rows)
constexpr int ST_M = 128, ST_N = 256;
constexpr int A_BYTES = ST_M * KC * 4;       // 8 KB
constexpr int B_BYTES = ST_N * KC * 4;       // 16 KB
constexpr int STAGE_BYTES = 2 * A_BYTES + 2 * B_BYTES;

struct SelfTestArgs {
    CUtensorMap a_hi, a_lo, b_hi, b_lo;  // [M=128][K], [N=256][K]
    int K;
    float *D;   // [128][256]
    int *err;
};

// One CTA, 6 warps: 0 TMA producer, 1 MMA issuer + TMEM owner, 2-5 epilogue.
__global__ void __launch_bounds__(192, 1) tc_selftest_kernel(const __grid_constant__ SelfTestArgs g) {
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
        const uint32_t idesc = tc::idesc_tf32(ST_M, ST_N);
        for (int kc = 0; kc < nk; ++kc) {
            const int s = kc & 1;
            if (!tc::mbar_wait(&full[s], (kc >> 1) & 1, kWaitNs, abort)) {
                *abort = 1;
                atomicExch(g.err, 2);
                break;
            }
            tc::tc_fence_after();
            const uint32_t st = tc::smem_u32(smem + s * STAGE_BYTES);
            for (int kk = 0; kk < KC / 8; ++kk) {
                const uint32_t ah = st + kk * 32, al = st + A_BYTES + kk * 32;
                const uint32_t bh = st + 2 * A_BYTES + kk * 32, bl = st + 2 * A_BYTES + B_BYTES + kk * 32;
                const uint32_t first = (kc == 0 && kk == 0) ? 0u : 1u;
                tc::mma_tf32(tmem, tc::sdesc_sw64(ah), tc::sdesc_sw64(bh), idesc, first);
                tc::mma_tf32(tmem, tc::sdesc_sw64(ah), tc::sdesc_sw64(bl), idesc, 1u);
                tc::mma_tf32(tmem, tc::sdesc_sw64(al), tc::sdesc_sw64(bh), idesc, 1u);
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
    SelfTestArgs g;
    const uint64_t da[2] = {(uint64_t)K, 128}, db[2] = {(uint64_t)K, 256};
    const uint64_t sa[1] = {(uint64_t)K * 4};
    const uint32_t ba[2] = {KC, 128}, bb[2] = {KC, 256};
    int rc = make_tmap_f32(&g.a_hi, a_hi, 2, da, sa, ba, 64);
    if (!rc) rc = make_tmap_f32(&g.a_lo, a_lo, 2, da, sa, ba, 64);
    if (!rc) rc = make_tmap_f32(&g.b_hi, b_hi, 2, db, sa, bb, 64);
    if (!rc) rc = make_tmap_f32(&g.b_lo, b_lo, 2, db, sa, bb, 64);
    if (rc) return rc;
    g.K = K;
    g.D = D;
    int *err = (int *)gpu_get(sizeof(int));
    if (!err) return fail(SDT_ERR_NOMEM, "sdt_tc_selftest: flag");
    g.err = err;
    cudaStream_t st = lib_stream();
    const int smem = 2 * STAGE_BYTES + 1024 + 256;
    rc = cuda_check(cudaFuncSetAttribute(tc_selftest_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem),
                    "sdt_tc_selftest");
    if (!rc) rc = cuda_check(cudaMemsetAsync(err, 0, sizeof(int), st), "sdt_tc_selftest");
    if (rc) {
        gpu_put(err);
        return rc;
    }
    tc_selftest_kernel<<<1, 192, smem, st>>>(g);
    count_launch();
    int h = 0;
    rc = cuda_check(cudaGetLastError(), "sdt_tc_selftest");
    if (!rc) rc = cuda_check(cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, st), "sdt_tc_selftest");
    if (!rc) rc = cuda_check(cudaStreamSynchronize(st), "sdt_tc_selftest");
    gpu_put(err);
    if (rc) return rc;
    if (h) return fail(SDT_ERR_TIMEOUT, "sdt_tc_selftest: a bounded wait ran out (stage " + std::to_string(h) + ")");
    return SDT_OK;
}

// ===========================================================================
// Fused mixed-precision tuple kernel.
//
// One CTA (192 threads, one per SM) owns an 8x8x8 (a,b,c) x 4x4x4 (i,j,k)
// sub-box of one tuple's triples tile: 32768 FP32 values in shared memory.
//
// Each d1 term has exactly the row/column index layout and the sign of one
// d2 term (d1_1/d2_8, d1_2/d2_9, d1_3/d2_7, d1_4/d2_2, d1_5/d2_3, d1_6/d2_1,
// d1_7/d2_5, d1_8/d2_6, d1_9/d2_4), so the 18 contractions become 9 merged
// 128x256 GEMMs with K = o + v into one TMEM accumulator each:
//   rows (R0;R1,R2) = one particle and two hole indices,
//   cols (C0,C1;C2) = two particle and one hole index,
//   D  = sum_m w(m,R0,R1,R2) t(C0,C1;C2,m)     A: Wd1, B: T2a   (K = m)
//      + sum_e t(R0,e;R1,R2) v(C0,C1,C2,e)     A: T2b, B: Vd2   (K = e)
// Operand tiles (8 K each) are staged by TMA with 32-byte swizzle in four
// stages; one thread issues the three split products (hi*hi, hi*lo, lo*hi)
// into one of two TMEM accumulators of 256 columns.  Four epilogue warps
// drain the other accumulator into the sub-box with the term's sign.  A term
// may be drained in K segments of `kseg` chunks, which shortens the tensor
// cores' FP32 accumulation chains (their rounding error grows with length).
// The sub-box uses a swizzled hole index so that the 32 rows a warp drains
// fall in 32 different shared-memory banks for every term layout.  The final
// epilogue promotes to FP64, adds the s1 products and the denominator and
// writes the CTA's (E[T], E(T)) pair.
// Warp roles: 0 TMA producer, 1 MMA issuer + TMEM owner, 2-5 epilogue.
// ===========================================================================
namespace sdt {
namespace {

constexpr int MX_THREADS = 192;
constexpr int MX_BV = 8, MX_BO = 4, MX_NX = 32768;
constexpr int MKC = 8;                                    // fp32 K elements per stage (32-byte rows)
constexpr int MNS = 4;                                    // stages
constexpr int MA_BYTES = 128 * MKC * 4, MB_BYTES = 256 * MKC * 4;
constexpr int MX_STAGE = 2 * MA_BYTES + 2 * MB_BYTES;     // 24 KB
constexpr int MX_SMEM = MX_NX * 4 + MNS * MX_STAGE + 256;
constexpr int MX_SMEM_ALLOC = MX_SMEM + 1024;

// Merged terms: rows (R0;R1,R2), cols (C0,C1;C2), sign.  Dims a=0 b=1 c=2 i=3 j=4 k=5.
struct MergedTerm {
    int8_t r[3], c[3];
    int8_t sign;
};
__constant__ MergedTerm kMerged[9] = {
    {{2, 4, 5}, {0, 1, 3}, -1},  // d1_1 + d2_8
    {{2, 3, 5}, {0, 1, 4}, +1},  // d1_2 + d2_9
    {{2, 3, 4}, {0, 1, 5}, -1},  // d1_3 + d2_7
    {{0, 4, 5}, {1, 2, 3}, -1},  // d1_4 + d2_2
    {{0, 3, 5}, {1, 2, 4}, +1},  // d1_5 + d2_3
    {{0, 3, 4}, {1, 2, 5}, -1},  // d1_6 + d2_1
    {{1, 4, 5}, {0, 2, 3}, +1},  // d1_7 + d2_5
    {{1, 3, 5}, {0, 2, 4}, -1},  // d1_8 + d2_6
    {{1, 3, 4}, {0, 2, 5}, +1}}; // d1_9 + d2_4

// Sub-box address of local (a,b,c,i,j,k): 64 floats per (a,b,c); inside,
// bit5 = k>>1, bit4 = (k&1)^parity(a+b+c), bits3-2 = (i+k)&3, bits1-0 = (j+k)&3.
__device__ __forceinline__ int xaddr(int a, int b, int c, int i, int j, int k) {
    const int par = (a + b + c) & 1;
    return ((((a << 3) | b) << 3 | c) << 6) | ((k >> 1) << 5) | ((((k & 1) ^ par)) << 4) |
           (((i + k) & 3) << 2) | ((j + k) & 3);
}

struct MixedParams {
    CUtensorMap t2b_hi, t2b_lo, t2a_hi, t2a_lo, wd1_hi, wd1_lo;
    const CUtensorMap *vd2_maps;  // [2*pair]: hi, lo
    const int32_t *pair_id;       // [nvab*nvab]
    const double *T1d, *Ud, *evl;
    const int32_t *tiles;         // [ntiles][4] start, range, spin, sym
    int32_t noab, nvab, nk_o, nk_v, kseg;
    int64_t nocc, nvir;
    const int64_t *klist, *item_pref;
    const double *factor;
    int64_t n_tasks, item_base;
    double *part;
    int *err;
};

__device__ __forceinline__ void named_bar(int id, int n) {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory");
}

// Drains 256 columns of TMEM row m for merged term T into the sub-box.
template <int T>
__device__ __forceinline__ void drain_term(float *X, uint32_t taddr, int m, float sign) {
    constexpr int R0 = T < 3 ? 2 : T < 6 ? 0 : 1;
    constexpr int R1 = (T % 3 == 0) ? 4 : 3;
    constexpr int R2 = (T % 3 == 2) ? 4 : 5;
    constexpr int C0 = T < 3 ? 0 : T < 6 ? 1 : 0;
    constexpr int C1 = T < 3 ? 1 : 2;
    constexpr int C2 = (T % 3 == 0) ? 3 : (T % 3 == 1) ? 4 : 5;
    int l[6];
    l[R0] = m >> 4;
    l[R1] = (m >> 2) & 3;
    l[R2] = m & 3;
#pragma unroll 1
    for (int cc = 0; cc < 8; ++cc) {
        float v[32];
        tc::tmem_ld32(taddr + (uint32_t)(cc * 32), v);
        l[C0] = cc;
#pragma unroll
        for (int q = 0; q < 32; ++q) {
            l[C1] = q >> 2;
            l[C2] = q & 3;
            const int x = xaddr(l[0], l[1], l[2], l[3], l[4], l[5]);
            X[x] += sign * v[q];
        }
    }
}

__device__ __forceinline__ void drain_any(int t, float *X, uint32_t taddr, int m, float sign) {
    switch (t) {
        case 0: drain_term<0>(X, taddr, m, sign); break;
        case 1: drain_term<1>(X, taddr, m, sign); break;
        case 2: drain_term<2>(X, taddr, m, sign); break;
        case 3: drain_term<3>(X, taddr, m, sign); break;
        case 4: drain_term<4>(X, taddr, m, sign); break;
        case 5: drain_term<5>(X, taddr, m, sign); break;
        case 6: drain_term<6>(X, taddr, m, sign); break;
        case 7: drain_term<7>(X, taddr, m, sign); break;
        default: drain_term<8>(X, taddr, m, sign); break;
    }
}

__global__ void __launch_bounds__(MX_THREADS, 1) fused_mixed_kernel(const __grid_constant__ MixedParams p) {
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    float *X = (float *)smem;
    uint8_t *stages = smem + MX_NX * 4;
    uint64_t *bars = (uint64_t *)(stages + MNS * MX_STAGE);
    uint64_t *full = bars, *empty = bars + MNS, *tfull = bars + 2 * MNS, *tempty = tfull + 2, *drain = tempty + 2;
    uint32_t *tslot = (uint32_t *)(drain + 1);
    volatile int *abort = (volatile int *)(tslot + 1);
    volatile int *epi_ok = (volatile int *)(tslot + 2);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    // ---- tuple and sub-box of this CTA ----
    const int64_t item = p.item_base + blockIdx.x;
    int64_t lo_ = 0, hi_ = p.n_tasks - 1;
    while (lo_ < hi_) {
        const int64_t mid = (lo_ + hi_ + 1) >> 1;
        if (p.item_pref[mid] <= item) lo_ = mid;
        else hi_ = mid - 1;
    }
    const int64_t tq = lo_;
    int64_t local = item - p.item_pref[tq];
    int tile[6], ext[6], start[6], boff[6];
#pragma unroll
    for (int d = 0; d < 6; ++d) {
        tile[d] = (int)p.klist[7 * tq + d];
        start[d] = __ldg(p.tiles + 4 * (tile[d] - 1));
        ext[d] = __ldg(p.tiles + 4 * (tile[d] - 1) + 1);
    }
#pragma unroll
    for (int d = 5; d >= 0; --d) {
        const int bx = d < 3 ? MX_BV : MX_BO;
        const int nb = (ext[d] + bx - 1) / bx;
        boff[d] = (int)(local % nb) * bx;
        local /= nb;
    }
    const int nk = p.nk_o + p.nk_v;                    // K chunks of a merged term
    const int kseg = p.kseg > 0 && p.kseg < nk ? p.kseg : nk;
    const int nseg = (nk + kseg - 1) / kseg;           // TMEM drains per term

    if (threadIdx.x == 0) {
        for (int s = 0; s < MNS; ++s) {
            tc::mbar_init(&full[s], 1);
            tc::mbar_init(&empty[s], 1);
        }
        for (int s = 0; s < 2; ++s) {
            tc::mbar_init(&tfull[s], 1);
            tc::mbar_init(&tempty[s], 1);
        }
        tc::mbar_init(drain, 1);
        *abort = 0;
        *epi_ok = 1;
        tc::fence_mbar_init();
    }
    if (warp == 1) tc::tmem_alloc(tslot, 512);
    for (int e = threadIdx.x; e < MX_NX; e += MX_THREADS) X[e] = 0.0f;
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    const uint32_t tmem = *tslot;

    if (warp == 0 && lane == 0) {
        // ---------------- TMA producer ----------------
        uint32_t g = 0;
        bool stop = false;
        for (int t = 0; t < 9 && !stop; ++t) {
            const MergedTerm td = kMerged[t];
            const int gr0 = start[td.r[0]] + boff[td.r[0]], gr1 = start[td.r[1]] + boff[td.r[1]],
                      gr2 = start[td.r[2]] + boff[td.r[2]];
            const int gc0 = start[td.c[0]] + boff[td.c[0]], gc1 = start[td.c[1]] + boff[td.c[1]],
                      gc2 = start[td.c[2]] + boff[td.c[2]];
            const int pr = p.pair_id[(tile[td.c[0]] - p.noab - 1) * p.nvab + (tile[td.c[1]] - p.noab - 1)];
            const CUtensorMap *vh = p.vd2_maps + 2 * pr, *vl = vh + 1;
            for (int kc = 0; kc < nk; ++kc, ++g) {
                const int s = g % MNS;
                if (g >= MNS && !tc::mbar_wait(&empty[s], ((g / MNS) & 1) ^ 1, kWaitNs, abort)) {
                    stop = true;
                    break;
                }
                uint8_t *st = stages + s * MX_STAGE;
                tc::mbar_arrive_expect_tx(&full[s], MX_STAGE);
                if (kc < p.nk_o) {  // d1 part: A = w(m,R0,R1,R2), B = t(C0,C1;C2,m)
                    const int k0 = kc * MKC;
                    tc::tma_load_4d(st, &p.wd1_hi, &full[s], k0, gr2, gr1, gr0);
                    tc::tma_load_4d(st + MA_BYTES, &p.wd1_lo, &full[s], k0, gr2, gr1, gr0);
                    tc::tma_load_4d(st + 2 * MA_BYTES, &p.t2a_hi, &full[s], k0, gc2, gc1, gc0);
                    tc::tma_load_4d(st + 2 * MA_BYTES + MB_BYTES, &p.t2a_lo, &full[s], k0, gc2, gc1, gc0);
                } else {  // d2 part: A = t(R0,e;R1,R2), B = v(C0,C1,C2,e)
                    const int k0 = (kc - p.nk_o) * MKC;
                    tc::tma_load_4d(st, &p.t2b_hi, &full[s], k0, gr2, gr1, gr0);
                    tc::tma_load_4d(st + MA_BYTES, &p.t2b_lo, &full[s], k0, gr2, gr1, gr0);
                    tc::tma_load_4d(st + 2 * MA_BYTES, vh, &full[s], k0, gc2, boff[td.c[1]], boff[td.c[0]]);
                    tc::tma_load_4d(st + 2 * MA_BYTES + MB_BYTES, vl, &full[s], k0, gc2, boff[td.c[1]],
                                    boff[td.c[0]]);
                }
            }
        }
        if (stop) {
            *abort = 1;
            atomicCAS(p.err, 0, 1);
            // copies already issued must land before the CTA exits
            volatile int never = 0;
            for (uint32_t x = g >= MNS ? g - MNS : 0; x < g; ++x)
                tc::mbar_wait(&full[x % MNS], (x / MNS) & 1, kWaitNs, &never);
        }
    } else if (warp == 1 && lane == 0) {
        // ---------------- MMA issuer ----------------
        const uint32_t idesc = tc::idesc_tf32(128, 256);
        uint32_t g = 0, sg = 0;  // chunk and segment counters
        bool stop = false;
        for (int t = 0; t < 9 && !stop; ++t) {
            for (int sgi = 0; sgi < nseg && !stop; ++sgi, ++sg) {
                const int buf = sg & 1;
                if (sg >= 2 && !tc::mbar_wait(&tempty[buf], ((sg >> 1) - 1) & 1, kWaitNs, abort)) {
                    stop = true;
                    break;
                }
                tc::tc_fence_after();
                const uint32_t d_tmem = tmem + (uint32_t)(buf * 256);
                const int kc_end = min(nk, (sgi + 1) * kseg);
                for (int kc = sgi * kseg; kc < kc_end; ++kc, ++g) {
                    const int s = g % MNS;
                    if (!tc::mbar_wait(&full[s], (g / MNS) & 1, kWaitNs, abort)) {
                        stop = true;
                        break;
                    }
                    tc::tc_fence_after();
                    const uint32_t st = tc::smem_u32(stages + s * MX_STAGE);
                    const uint32_t a_h = st, a_l = st + MA_BYTES;
                    const uint32_t b_h = st + 2 * MA_BYTES, b_l = st + 2 * MA_BYTES + MB_BYTES;
                    tc::mma_tf32(d_tmem, tc::sdesc_sw32(a_h), tc::sdesc_sw32(b_h), idesc,
                                 kc == sgi * kseg ? 0u : 1u);
                    tc::mma_tf32(d_tmem, tc::sdesc_sw32(a_h), tc::sdesc_sw32(b_l), idesc, 1u);
                    tc::mma_tf32(d_tmem, tc::sdesc_sw32(a_l), tc::sdesc_sw32(b_h), idesc, 1u);
                    tc::mma_commit(&empty[s]);
                }
                if (!stop) tc::mma_commit(&tfull[buf]);
            }
        }
        if (stop) {
            *abort = 1;
            atomicCAS(p.err, 0, 2);
        }
        // every issued MMA completes before TMEM is released
        tc::mma_commit(drain);
        volatile int never = 0;
        tc::mbar_wait(drain, 0, kWaitNs, &never);
    } else if (warp >= 2) {
        // ---------------- epilogue: drain TMEM into the sub-box ----------------
        const int quad = warp & 3;
        const int m = quad * 32 + lane;  // TMEM lane = GEMM row
        const bool leader = (warp == 2 && lane == 0);
        uint32_t sg = 0;
        bool ok = true;
        for (int t = 0; t < 9 && ok; ++t) {
            const float sign = (float)kMerged[t].sign;
            for (int sgi = 0; sgi < nseg; ++sgi, ++sg) {
                const int buf = sg & 1;
                if (leader) *epi_ok = tc::mbar_wait(&tfull[buf], (sg >> 1) & 1, kWaitNs, abort) ? 1 : 0;
                named_bar(1, 128);
                if (!*epi_ok) {
                    ok = false;
                    break;
                }
                tc::tc_fence_after();
                drain_any(t, X, tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)(buf * 256), m, sign);
                tc::tc_fence_before();
                named_bar(1, 128);
                if (leader) tc::mbar_arrive(&tempty[buf]);
            }
        }
        if (leader && !ok) {
            *abort = 1;
            atomicCAS(p.err, 0, 3);
        }
    }
    tc::tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc::tc_fence_after();
        tc::tmem_dealloc(tmem, 512);
    }
    if (*abort) {
        if (threadIdx.x == 0) {
            p.part[2 * item] = 0.0;
            p.part[2 * item + 1] = 0.0;
        }
        return;
    }

    // ---------------- FP64 epilogue: s1 terms, denominator, energies ----------------
    const double factor = p.factor[tq];
    const double *__restrict__ eo = p.evl;
    const double *__restrict__ ev = p.evl + p.nocc;
    const int64_t v = p.nvir, o = p.nocc;
    double e1 = 0.0, e2 = 0.0;
    for (int e = threadIdx.x; e < MX_NX; e += MX_THREADS) {
        const int l0 = e >> 12, l1 = (e >> 9) & 7, l2 = (e >> 6) & 7, l3 = (e >> 4) & 3, l4 = (e >> 2) & 3,
                  l5 = e & 3;
        if (boff[0] + l0 >= ext[0] || boff[1] + l1 >= ext[1] || boff[2] + l2 >= ext[2] ||
            boff[3] + l3 >= ext[3] || boff[4] + l4 >= ext[4] || boff[5] + l5 >= ext[5])
            continue;
        const int64_t a = start[0] + boff[0] + l0, b = start[1] + boff[1] + l1, c = start[2] + boff[2] + l2;
        const int64_t i = start[3] + boff[3] + l3, j = start[4] + boff[4] + l4, k = start[5] + boff[5] + l5;
        auto u = [&](int64_t x, int64_t y, int64_t h, int64_t gg) {
            return __ldg(p.Ud + ((x * v + y) * o + h) * o + gg);
        };
        auto t1 = [&](int64_t x, int64_t h) { return __ldg(p.T1d + x * o + h); };
        double sing = t1(a, i) * u(b, c, j, k);
        sing -= t1(a, j) * u(b, c, i, k);
        sing += t1(a, k) * u(b, c, i, j);
        sing -= t1(b, i) * u(a, c, j, k);
        sing += t1(b, j) * u(a, c, i, k);
        sing -= t1(b, k) * u(a, c, i, j);
        sing += t1(c, i) * u(a, b, j, k);
        sing -= t1(c, j) * u(a, b, i, k);
        sing += t1(c, k) * u(a, b, i, j);
        const double doub = (double)X[xaddr(l0, l1, l2, l3, l4, l5)];
        const double denom_0 = -(ev[a] + ev[b] + ev[c]);
        const double denom = doub * factor / (eo[i] + eo[j] + eo[k] + denom_0);
        e1 += denom * doub;
        e2 += denom * (doub + sing);
    }
    double *red = (double *)stages;  // stages are idle now
    e1 = warp_sum(e1);
    e2 = warp_sum(e2);
    if (lane == 0) {
        red[2 * warp] = e1;
        red[2 * warp + 1] = e2;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double x = 0.0, y = 0.0;
        for (int w = 0; w < MX_THREADS / 32; ++w) {
            x += red[2 * w];
            y += red[2 * w + 1];
        }
        p.part[2 * item] = x;
        p.part[2 * item + 1] = y;
    }
}

// FP64 rows [rows][n] -> TF32 hi/lo rows [rows][n_pad] (zero padding).
__global__ void __launch_bounds__(256) split_rows_kernel(const double *__restrict__ src, float *__restrict__ hi,
                                                         float *__restrict__ lo, int64_t rows, int64_t n,
                                                         int64_t n_pad) {
    const int64_t total = rows * n_pad;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = i / n_pad, c = i % n_pad;
        float h = 0.0f, l = 0.0f;
        if (c < n) {
            const double x = src[r * n + c];
            h = tc::to_tf32(__double2float_rn(x));
            l = tc::to_tf32(__double2float_rn(x - (double)h));
        }
        hi[i] = h;
        lo[i] = l;
    }
}

}  // namespace

void mixed_release(sdt_job *j) {
    for (int k = 0; k < 2 * SP_N; ++k) {
        gpu_put(j->sp[k]);
        j->sp[k] = nullptr;
        j->sp_n[k] = 0;
    }
    gpu_put(j->vd2_maps);
    gpu_put(j->pair_id);
    gpu_put(j->err_d);
    host_put(j->err_h);
    j->vd2_maps = nullptr;
    j->pair_id = nullptr;
    j->err_d = nullptr;
    j->err_h = nullptr;
    j->mixed_ready = false;
}

int mixed_prepare(sdt_job *j, cudaStream_t st) {
    mixed_release(j);
    const Tiling &t = j->t;
    const int64_t o = t.nocc, v = t.nvir, noab = t.noab, nvab = t.nvab;
    const int64_t op = (o + 3) / 4 * 4, vp = (v + 3) / 4 * 4;
    j->o_pad = op;
    j->v_pad = vp;
    struct Src { int idx; int64_t rows, n, npad; };
    const int64_t vd2_elems = (int64_t)j->arr_n[DST_VD2];
    const Src src[SP_N] = {{DST_T2A, v * v * o, o, op}, {DST_T2B, v * o * o, v, vp},
                           {DST_WD1, v * o * o, o, op}, {DST_VD2, vd2_elems / v, v, vp}};
    for (int k = 0; k < SP_N; ++k) {
        const size_t n = (size_t)(src[k].rows * src[k].npad);
        for (int h = 0; h < 2; ++h) {
            j->sp[2 * k + h] = (float *)gpu_get(std::max<size_t>(n, 1) * sizeof(float));
            if (!j->sp[2 * k + h]) {
                mixed_release(j);
                return fail(SDT_ERR_NOMEM, "mixed form: split operand allocation");
            }
            j->sp_n[2 * k + h] = n;
        }
        int64_t blocks = std::min<int64_t>((int64_t)(n + 255) / 256, 152 * 16);
        if (blocks < 1) blocks = 1;
        split_rows_kernel<<<(unsigned)blocks, 256, 0, st>>>(j->arr[src[k].idx], j->sp[2 * k], j->sp[2 * k + 1],
                                                            src[k].rows, src[k].n, src[k].npad);
        count_launch();
    }
    int rc = cuda_check(cudaGetLastError(), "mixed form: split");
    if (rc) return rc;
    // Tensor maps (fp32, 64-byte swizzle, 16 K elements per box row).
    const uint64_t B4 = 4;
    {
        const uint64_t d[4] = {(uint64_t)vp, (uint64_t)o, (uint64_t)o, (uint64_t)v};
        const uint64_t sb[3] = {vp * B4, o * vp * B4, o * o * vp * B4};
        const uint32_t box[4] = {MKC, 4, 4, 8};
        rc = make_tmap_f32(&j->maps[0], j->sp[2 * SP_T2B], 4, d, sb, box, 32);
        if (!rc) rc = make_tmap_f32(&j->maps[1], j->sp[2 * SP_T2B + 1], 4, d, sb, box, 32);
    }
    if (!rc) {
        const uint64_t d[4] = {(uint64_t)op, (uint64_t)o, (uint64_t)v, (uint64_t)v};
        const uint64_t sb[3] = {op * B4, o * op * B4, v * o * op * B4};
        const uint32_t box[4] = {MKC, 4, 8, 8};
        rc = make_tmap_f32(&j->maps[2], j->sp[2 * SP_T2A], 4, d, sb, box, 32);
        if (!rc) rc = make_tmap_f32(&j->maps[3], j->sp[2 * SP_T2A + 1], 4, d, sb, box, 32);
    }
    if (!rc) {
        const uint64_t d[4] = {(uint64_t)op, (uint64_t)o, (uint64_t)o, (uint64_t)v};
        const uint64_t sb[3] = {op * B4, o * op * B4, o * o * op * B4};
        const uint32_t box[4] = {MKC, 4, 4, 8};
        rc = make_tmap_f32(&j->maps[4], j->sp[2 * SP_WD1], 4, d, sb, box, 32);
        if (!rc) rc = make_tmap_f32(&j->maps[5], j->sp[2 * SP_WD1 + 1], 4, d, sb, box, 32);
    }
    std::vector<CUtensorMap> vmaps;
    std::vector<int32_t> pid(nvab * nvab, -1);
    for (int64_t B = noab + 1; B <= noab + nvab && !rc; ++B)
        for (int64_t C = B; C <= noab + nvab && !rc; ++C) {
            const int64_t off = j->pair_host[(B - noab - 1) * nvab + (C - noab - 1)];
            const int64_t nB = t.r(B), nC = t.r(C);
            const int64_t soff = off / v * vp;
            const uint64_t d[4] = {(uint64_t)vp, (uint64_t)o, (uint64_t)nC, (uint64_t)nB};
            const uint64_t sb[3] = {vp * B4, o * vp * B4, nC * o * vp * B4};
            const uint32_t box[4] = {MKC, 4, 8, 8};
            CUtensorMap mh, ml;
            rc = make_tmap_f32(&mh, j->sp[2 * SP_VD2] + soff, 4, d, sb, box, 32);
            if (!rc) rc = make_tmap_f32(&ml, j->sp[2 * SP_VD2 + 1] + soff, 4, d, sb, box, 32);
            pid[(B - noab - 1) * nvab + (C - noab - 1)] = (int32_t)(vmaps.size() / 2);
            vmaps.push_back(mh);
            vmaps.push_back(ml);
        }
    if (rc) {
        mixed_release(j);
        return rc;
    }
    j->vd2_maps = (CUtensorMap *)gpu_get(vmaps.size() * sizeof(CUtensorMap));
    j->pair_id = (int32_t *)gpu_get(pid.size() * sizeof(int32_t));
    j->err_d = (int *)gpu_get(sizeof(int));
    j->err_h = (int *)host_get(sizeof(int));
    if (!j->vd2_maps || !j->pair_id || !j->err_d || !j->err_h) {
        mixed_release(j);
        return fail(SDT_ERR_NOMEM, "mixed form: tables");
    }
    rc = cuda_check(cudaMemcpyAsync(j->vd2_maps, vmaps.data(), vmaps.size() * sizeof(CUtensorMap),
                                    cudaMemcpyHostToDevice, st), "mixed form: maps");
    if (!rc) rc = cuda_check(cudaMemcpyAsync(j->pair_id, pid.data(), pid.size() * sizeof(int32_t),
                                             cudaMemcpyHostToDevice, st), "mixed form: maps");
    if (!rc) rc = cuda_check(cudaStreamSynchronize(st), "mixed form: prepare");
    if (rc) {
        mixed_release(j);
        return rc;
    }
    j->mixed_ready = true;
    return SDT_OK;
}

int mixed_launch(sdt_job *j, int64_t items, int64_t n, cudaStream_t st) {
    const Tiling &t = j->t;
    MixedParams p;
    p.t2b_hi = j->maps[0]; p.t2b_lo = j->maps[1];
    p.t2a_hi = j->maps[2]; p.t2a_lo = j->maps[3];
    p.wd1_hi = j->maps[4]; p.wd1_lo = j->maps[5];
    p.vd2_maps = j->vd2_maps;
    p.pair_id = j->pair_id;
    p.T1d = j->arr[DST_T1];
    p.Ud = j->arr[DST_UD];
    p.evl = j->evl_d;
    p.tiles = j->tiles;
    p.noab = (int32_t)t.noab;
    p.nvab = (int32_t)t.nvab;
    p.nocc = t.nocc;
    p.nvir = t.nvir;
    p.nk_o = (int32_t)((t.nocc + MKC - 1) / MKC);
    p.nk_v = (int32_t)((t.nvir + MKC - 1) / MKC);
    p.kseg = j->mixed_kseg;
    p.klist = j->klist_d;
    p.item_pref = j->pref_d;
    p.factor = j->factor_d;
    p.n_tasks = n;
    p.part = j->part_d;
    p.err = j->err_d;
    int rc = cuda_check(cudaFuncSetAttribute(fused_mixed_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             MX_SMEM_ALLOC),
                        "mixed form: smem attribute");
    if (!rc) rc = cuda_check(cudaMemsetAsync(j->err_d, 0, sizeof(int), st), "mixed form");
    if (rc) return rc;
    const int64_t chunk = 1ll << 30;
    for (int64_t b0 = 0; b0 < items; b0 += chunk) {
        p.item_base = b0;
        const unsigned nb = (unsigned)std::min<int64_t>(chunk, items - b0);
        fused_mixed_kernel<<<nb, MX_THREADS, MX_SMEM_ALLOC, st>>>(p);
        count_launch();
    }
    rc = cuda_check(cudaGetLastError(), "mixed form: fused kernel");
    if (!rc) rc = cuda_check(cudaMemcpyAsync(j->err_h, j->err_d, sizeof(int), cudaMemcpyDeviceToHost, st),
                             "mixed form");
    return rc;
}

}  // namespace sdt
