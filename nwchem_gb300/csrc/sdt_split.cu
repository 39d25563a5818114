// sdt_split.cu -- the mixed-precision form: one persistent kernel that runs
// the d1/d2 contractions of every sub-box as split-operand tensor-core GEMMs
// (tcgen05) and the s1 terms, denominator and energy sums on the CUDA cores,
// the latter overlapped with the next sub-box's contractions.
//
// Work unit (item): an 8x8x8 (a,b,c) x 4x4x4 (i,j,k) sub-box of one tuple's
// triples tile, 32768 values.  Items are dealt to the CTAs round-robin (one
// CTA per SM; item = blockIdx.x + n * gridDim.x), so results do not depend on
// timing.
//
// Contractions.  Every d1 term has exactly the row/column index layout and the
// sign of one d2 term (d1_1/d2_8, d1_2/d2_9, d1_3/d2_7, d1_4/d2_2, d1_5/d2_3,
// d1_6/d2_1, d1_7/d2_5, d1_8/d2_6, d1_9/d2_4), so the 18 contractions are 9
// merged 128x256 GEMMs with K = o + v:
//   rows (R0;R1,R2) = one particle and two hole indices,
//   cols (C0,C1;C2) = two particle and one hole index,
//   D  = sum_m w(m,R0,R1,R2) t(C0,C1;C2,m)     A: Wd1, B: T2a   (K = m)
//      + sum_e t(R0,e;R1,R2) v(C0,C1,C2,e)     A: T2b, B: Vd2   (K = e)
// Operand tiles of 32-byte K rows (8 TF32 or 16 BF16/FP16 values) are staged
// by TMA with 32-byte swizzle in four stages; one thread issues the three
// split products of a stage (hi*hi, hi*lo, lo*hi) into one of two 256-column
// TMEM accumulators while the epilogue warps drain the other into the FP32
// sub-box in shared memory with the term's sign.  A term may be drained in K
// segments of `kseg` stages (shorter FP32 accumulation chains).  The sub-box
// uses a swizzled hole index so that the rows a warp drains fall in distinct
// shared-memory banks for all 9 layouts.
//
// Energies.  When an item's last term is drained, the energy warps copy the
// finished sub-box from shared memory into registers (128 values per thread)
// and release it; the drain warps then store the next item's first term into
// it while the energy warps evaluate the copy: the s1 products in FP32 from
// FP32 copies of T1 and the vvoo block, then, in FP64, the denominator, the
// division and the two energy sums.  So the energy work of one item overlaps
// the contractions of the next.
//
// Warp roles: 0 TMA producer, 1 MMA issuer + TMEM owner, 2-3 idle, 4-7 drain
// (TMEM lane quadrant warp % 4), 8-15 energy.  Every mbarrier wait is bounded
// (2 s); on a timeout the kernel sets an error flag, lets issued copies and
// MMAs land, frees TMEM and returns.
#include "sdt_common.cuh"
#include "sdt_job.h"
#include "sdt_tc.cuh"

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

namespace sdt {
namespace {

constexpr uint64_t kWaitNs = 2000000000ull;  // 2 s per wait
constexpr int SX_THREADS = 512;
constexpr int SX_DRAIN = 128;                 // drain threads (warps 4-7)
constexpr int SX_EPI = 256;                   // energy threads (warps 8-15)
// Register split (setmaxnreg): the launch gives 128 per thread (4 warps per
// SM sub-partition); warps 0-3 drop to 40, the drain warps to 88 and the
// energy warps rise to 192: 128*40 + 128*88 + 256*192 = 65536 = 512*128, and each
// sub-partition holds one warp of each group: (40+88+2*192)*32 = 16384.
constexpr int SX_REG_LAUNCH = 128, SX_REG_LOW = 40, SX_REG_DRAIN = 88, SX_REG_HIGH = 192;
static_assert(128 * SX_REG_LOW + 128 * SX_REG_DRAIN + 256 * SX_REG_HIGH <= SX_THREADS * SX_REG_LAUNCH,
              "register split");
// setmaxnreg.dec may only lower and setmaxnreg.inc only raise a warp's count.
static_assert(SX_REG_LOW <= SX_REG_LAUNCH && SX_REG_DRAIN <= SX_REG_LAUNCH && SX_REG_HIGH >= SX_REG_LAUNCH,
              "setmaxnreg direction");
constexpr int SX_BV = 8, SX_BO = 4, SX_NX = 32768;
constexpr int SX_NS = 4;                      // operand stages
constexpr int SX_A = 128 * 32, SX_B = 256 * 32;
constexpr int SX_STAGE = 2 * SX_A + 2 * SX_B;  // 24 KB
constexpr int SX_MISC = 1024;
constexpr int SX_SMEM = SX_NX * 4 + SX_NS * SX_STAGE + SX_MISC;
constexpr int SX_SMEM_ALLOC = SX_SMEM + 1024;  // room to align the base to 1024 bytes
static_assert(SX_SMEM_ALLOC <= 232448, "shared memory per block");

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

// What the energy chunks of an item need after its last drain.
struct EDesc {
    int g[6];       // global orbital index of the sub-box origin, per dimension
    int nv[6];      // valid extent of the sub-box, per dimension
    double factor;  // the tuple's multiplicity factor
    long long item;
};

struct SplitParams {
    CUtensorMap t2b_hi, t2b_lo, t2a_hi, t2a_lo, wd1_hi, wd1_lo;
    const CUtensorMap *vd2_maps;  // [2*pair]: hi, lo
    const int32_t *pair_id;       // [nvab*nvab]
    const float *T1f, *Uf;        // FP32 copies: [v][o], [v][v][o][o]
    const double *evl;
    const int32_t *tiles;         // [ntiles][4] start, range, spin, sym
    int32_t noab, nvab, nk_o, nk_v, kseg;
    int64_t nocc, nvir;
    const int64_t *klist, *item_pref;
    const double *factor;
    int64_t n_tasks, items;
    double inv_s, inv_s2;         // undo the operand scaling (FP16): X_true = X * inv_s
    double *part;
    int *err;
};

struct ItemBox {
    int tile[6], start[6], ext[6], boff[6];
    int64_t tq;
};

__device__ __forceinline__ void decode_item(const SplitParams &p, int64_t item, ItemBox &b) {
    int64_t lo = 0, hi = p.n_tasks - 1;
    while (lo < hi) {
        const int64_t mid = (lo + hi + 1) >> 1;
        if (p.item_pref[mid] <= item) lo = mid;
        else hi = mid - 1;
    }
    b.tq = lo;
    int64_t local = item - p.item_pref[lo];
#pragma unroll
    for (int d = 0; d < 6; ++d) {
        b.tile[d] = (int)p.klist[7 * lo + d];
        b.start[d] = __ldg(p.tiles + 4 * (b.tile[d] - 1));
        b.ext[d] = __ldg(p.tiles + 4 * (b.tile[d] - 1) + 1);
    }
#pragma unroll
    for (int d = 5; d >= 0; --d) {
        const int bx = d < 3 ? SX_BV : SX_BO;
        const int nb = (b.ext[d] + bx - 1) / bx;
        b.boff[d] = (int)(local % nb) * bx;
        local /= nb;
    }
}

__device__ __forceinline__ void named_bar(int id, int n) {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory");
}

template <int TYPE>
__device__ __forceinline__ void mma_split(uint32_t d, uint64_t a, uint64_t b, uint32_t acc) {
    if (TYPE == TM_F32) tc::mma_tf32(d, a, b, tc::idesc_tf32(128, 256), acc);
    else tc::mma_f16(d, a, b, tc::idesc_f16(128, 256, TYPE == TM_BF16), acc);
}

// ---------------------------------------------------------------------------
// TMA producer (one thread).
template <int TYPE>
__device__ __forceinline__ void run_producer(const SplitParams &p, uint8_t *stages, uint64_t *full,
                                             uint64_t *empty, volatile int *abort) {
    constexpr int KE = TYPE == TM_F32 ? 8 : 16;  // K elements per 32-byte row
    const int nk = p.nk_o + p.nk_v;
    tc::prefetch_tmap(&p.t2b_hi);
    tc::prefetch_tmap(&p.t2a_hi);
    tc::prefetch_tmap(&p.wd1_hi);
    uint32_t g = 0;
    bool stop = false;
    for (int64_t it = blockIdx.x; it < p.items && !stop; it += gridDim.x) {
        ItemBox bx;
        decode_item(p, it, bx);
        int gs[6];
#pragma unroll
        for (int d = 0; d < 6; ++d) gs[d] = bx.start[d] + bx.boff[d];
        for (int t = 0; t < 9 && !stop; ++t) {
            const MergedTerm td = kMerged[t];
            const int gr0 = gs[td.r[0]], gr1 = gs[td.r[1]], gr2 = gs[td.r[2]];
            const int gc0 = gs[td.c[0]], gc1 = gs[td.c[1]], gc2 = gs[td.c[2]];
            const int pr = p.pair_id[(bx.tile[td.c[0]] - p.noab - 1) * p.nvab + (bx.tile[td.c[1]] - p.noab - 1)];
            const CUtensorMap *vh = p.vd2_maps + 2 * pr, *vl = vh + 1;
            const int vb1 = bx.boff[td.c[1]], vb0 = bx.boff[td.c[0]];
            for (int kc = 0; kc < nk; ++kc, ++g) {
                const int s = g % SX_NS;
                if (g >= SX_NS && !tc::mbar_wait(&empty[s], ((g / SX_NS) & 1) ^ 1, kWaitNs, abort)) {
                    stop = true;
                    break;
                }
                uint8_t *st = stages + s * SX_STAGE;
                tc::mbar_arrive_expect_tx(&full[s], SX_STAGE);
                if (kc < p.nk_o) {  // d1 part: A = w(m,R0,R1,R2), B = t(C0,C1;C2,m)
                    const int k0 = kc * KE;
                    tc::tma_load_4d(st, &p.wd1_hi, &full[s], k0, gr2, gr1, gr0);
                    tc::tma_load_4d(st + SX_A, &p.wd1_lo, &full[s], k0, gr2, gr1, gr0);
                    tc::tma_load_4d(st + 2 * SX_A, &p.t2a_hi, &full[s], k0, gc2, gc1, gc0);
                    tc::tma_load_4d(st + 2 * SX_A + SX_B, &p.t2a_lo, &full[s], k0, gc2, gc1, gc0);
                } else {  // d2 part: A = t(R0,e;R1,R2), B = v(C0,C1,C2,e)
                    const int k0 = (kc - p.nk_o) * KE;
                    tc::tma_load_4d(st, &p.t2b_hi, &full[s], k0, gr2, gr1, gr0);
                    tc::tma_load_4d(st + SX_A, &p.t2b_lo, &full[s], k0, gr2, gr1, gr0);
                    tc::tma_load_4d(st + 2 * SX_A, vh, &full[s], k0, gc2, vb1, vb0);
                    tc::tma_load_4d(st + 2 * SX_A + SX_B, vl, &full[s], k0, gc2, vb1, vb0);
                }
            }
        }
    }
    if (stop) {
        *abort = 1;
        atomicCAS(p.err, 0, 1);
        // copies already issued must land before the CTA exits
        volatile int never = 0;
        for (uint32_t x = g >= SX_NS ? g - SX_NS : 0; x < g; ++x)
            tc::mbar_wait(&full[x % SX_NS], (x / SX_NS) & 1, kWaitNs, &never);
    }
}

// ---------------------------------------------------------------------------
// MMA issuer (one thread).
template <int TYPE>
__device__ __forceinline__ void run_mma(const SplitParams &p, uint8_t *stages, uint64_t *full, uint64_t *empty,
                                        uint64_t *tfull, uint64_t *tempty, uint64_t *drain, uint32_t tmem,
                                        volatile int *abort) {
    const int nk = p.nk_o + p.nk_v;
    const int kseg = p.kseg > 0 && p.kseg < nk ? p.kseg : nk;
    const int nseg = (nk + kseg - 1) / kseg;
    uint32_t g = 0, sg = 0;  // stage and segment counters
    bool stop = false;
    for (int64_t it = blockIdx.x; it < p.items && !stop; it += gridDim.x) {
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
                    const int s = g % SX_NS;
                    if (!tc::mbar_wait(&full[s], (g / SX_NS) & 1, kWaitNs, abort)) {
                        stop = true;
                        break;
                    }
                    tc::tc_fence_after();
                    const uint32_t st = tc::smem_u32(stages + s * SX_STAGE);
                    const uint64_t ah = tc::sdesc_sw32(st), al = tc::sdesc_sw32(st + SX_A);
                    const uint64_t bh = tc::sdesc_sw32(st + 2 * SX_A), bl = tc::sdesc_sw32(st + 2 * SX_A + SX_B);
                    mma_split<TYPE>(d_tmem, ah, bh, kc == sgi * kseg ? 0u : 1u);
                    mma_split<TYPE>(d_tmem, ah, bl, 1u);
                    mma_split<TYPE>(d_tmem, al, bh, 1u);
                    tc::mma_commit(&empty[s]);
                }
                if (!stop) tc::mma_commit(&tfull[buf]);
            }
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
}

// ---------------------------------------------------------------------------
// Drains: TMEM row m (all 256 columns) of merged term T into the sub-box with
// the term's sign, stored (STORE) or added.
template <int T, bool STORE>
__device__ __forceinline__ void drain_term(float *X, uint32_t taddr, int m) {
    constexpr int R0 = T < 3 ? 2 : T < 6 ? 0 : 1;
    constexpr int R1 = (T % 3 == 0) ? 4 : 3;
    constexpr int R2 = (T % 3 == 2) ? 4 : 5;
    constexpr int C0 = T < 3 ? 0 : T < 6 ? 1 : 0;
    constexpr int C1 = T < 3 ? 1 : 2;
    constexpr int C2 = (T % 3 == 0) ? 3 : (T % 3 == 1) ? 4 : 5;
    constexpr float sign = (T == 1 || T == 4 || T == 6 || T == 8) ? 1.0f : -1.0f;
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
            if (STORE) X[x] = sign * v[q];
            else X[x] += sign * v[q];
        }
    }
}

__device__ __forceinline__ void drain_any(int t, bool store, float *X, uint32_t taddr, int m) {
    switch (t) {
        case 0:
            if (store) drain_term<0, true>(X, taddr, m);
            else drain_term<0, false>(X, taddr, m);
            break;
        case 1: drain_term<1, false>(X, taddr, m); break;
        case 2: drain_term<2, false>(X, taddr, m); break;
        case 3: drain_term<3, false>(X, taddr, m); break;
        case 4: drain_term<4, false>(X, taddr, m); break;
        case 5: drain_term<5, false>(X, taddr, m); break;
        case 6: drain_term<6, false>(X, taddr, m); break;
        case 7: drain_term<7, false>(X, taddr, m); break;
        default: drain_term<8, false>(X, taddr, m); break;
    }
}

// ---------------------------------------------------------------------------
// Energies of one item from its values R in registers: thread (b;i,j) with
// R[32*A + 4*c + k] = X(a = 4*half + A, b, c, i, j, k).
//   X_s = t1(a,i)u(b,c,j,k) - t1(a,j)u(b,c,i,k) + t1(a,k)u(b,c,i,j)
//       - t1(b,i)u(a,c,j,k) + t1(b,j)u(a,c,i,k) - t1(b,k)u(a,c,i,j)
//       + t1(c,i)u(a,b,j,k) - t1(c,j)u(a,b,i,k) + t1(c,k)u(a,b,i,j)   (FP32)
//   D = (e_i + e_j + e_k) - (e_a + e_b + e_c)                          (FP64)
//   e1 += X^2 / D,  est += X X_s / D                                    (FP64)
template <int A>
__device__ __forceinline__ void energy_chunk(const float (&R)[128], const EDesc &d, const SplitParams &p, int half,
                                             int b, int i, int j, double &e1, double &est) {
    const int a = 4 * half + A;
    if (a >= d.nv[0] || b >= d.nv[1] || i >= d.nv[3] || j >= d.nv[4]) return;
    const int o = (int)p.nocc;
    const int64_t v = p.nvir, oo = (int64_t)o * o;
    const int ga = d.g[0] + a, gb = d.g[1] + b, gi = d.g[3] + i, gj = d.g[4] + j;
    const int nc = d.nv[2], nk = d.nv[5], gc0 = d.g[2], gk0 = d.g[5];
    const double *__restrict__ eo = p.evl;
    const double *__restrict__ ev = p.evl + p.nocc;
    const double eij = __ldg(eo + gi) + __ldg(eo + gj);
    const double eab = __ldg(ev + ga) + __ldg(ev + gb);
    const float *__restrict__ t1a = p.T1f + (int64_t)ga * o;
    const float *__restrict__ t1b = p.T1f + (int64_t)gb * o;
    const float t1ai = __ldg(t1a + gi), t1aj = __ldg(t1a + gj), t1bi = __ldg(t1b + gi), t1bj = __ldg(t1b + gj);
    const float *__restrict__ uab = p.Uf + ((int64_t)ga * v + gb) * oo;
    const float uabij = __ldg(uab + gi * o + gj);
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        if (c < nc) {
            const int gc = gc0 + c;
            const float *__restrict__ t1c = p.T1f + (int64_t)gc * o;
            const float *__restrict__ ubc = p.Uf + ((int64_t)gb * v + gc) * oo;
            const float *__restrict__ uac = p.Uf + ((int64_t)ga * v + gc) * oo;
            const float t1ci = __ldg(t1c + gi), t1cj = __ldg(t1c + gj);
            const float ubcij = __ldg(ubc + gi * o + gj), uacij = __ldg(uac + gi * o + gj);
            const double Q = eab + __ldg(ev + gc);
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                if (k < nk) {
                    const int gk = gk0 + k;
                    float s = t1ai * __ldg(ubc + gj * o + gk);
                    s = fmaf(-t1aj, __ldg(ubc + gi * o + gk), s);
                    s = fmaf(__ldg(t1a + gk), ubcij, s);
                    s = fmaf(-t1bi, __ldg(uac + gj * o + gk), s);
                    s = fmaf(t1bj, __ldg(uac + gi * o + gk), s);
                    s = fmaf(-__ldg(t1b + gk), uacij, s);
                    s = fmaf(t1ci, __ldg(uab + gj * o + gk), s);
                    s = fmaf(-t1cj, __ldg(uab + gi * o + gk), s);
                    s = fmaf(__ldg(t1c + gk), uabij, s);
                    const double x = (double)R[A * 32 + c * 4 + k];
                    const double D = (eij + __ldg(eo + gk)) - Q;
                    const double q = div_nr(x, D);
                    e1 = fma(q, x, e1);
                    est = fma(q, (double)s, est);
                }
            }
        }
    }
}

// Per-item pair: E[T] part f/S^2 sum X^2/D, E(T) part that + f/S sum X X_s/D.
__device__ __forceinline__ void write_partial(double &e1, double &est, double *red, const EDesc &d,
                                              const SplitParams &p, int ew, int lane, bool leader) {
    const double x = warp_sum(e1), y = warp_sum(est);
    if (lane == 0) {
        red[2 * ew] = x;
        red[2 * ew + 1] = y;
    }
    named_bar(2, SX_EPI);
    if (leader) {
        double s1 = 0.0, s2 = 0.0;
        for (int w = 0; w < SX_EPI / 32; ++w) {
            s1 += red[2 * w];
            s2 += red[2 * w + 1];
        }
        const double et = d.factor * s1 * p.inv_s2;
        p.part[2 * d.item] = et;
        p.part[2 * d.item + 1] = et + d.factor * s2 * p.inv_s;
    }
    e1 = 0.0;
    est = 0.0;
}

template <int TYPE>
__global__ void __launch_bounds__(SX_THREADS, 1) split_fused_kernel(const __grid_constant__ SplitParams p) {
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    float *X = (float *)smem;
    uint8_t *stages = smem + SX_NX * 4;
    uint8_t *misc = stages + SX_NS * SX_STAGE;
    uint64_t *bars = (uint64_t *)misc;
    uint64_t *full = bars, *empty = bars + SX_NS, *tfull = bars + 2 * SX_NS, *tempty = tfull + 2,
             *drain = tempty + 2, *xready = drain + 1, *xfree = xready + 1;
    uint32_t *tslot = (uint32_t *)(misc + 128);
    volatile int *abort = (volatile int *)(misc + 132);
    volatile int *dr_ok = (volatile int *)(misc + 136);
    volatile int *en_ok = (volatile int *)(misc + 140);
    EDesc *desc = (EDesc *)(misc + 256);
    double *red = (double *)(misc + 512);          // [8 energy warps][2]
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    if (threadIdx.x == 0) {
        for (int s = 0; s < SX_NS; ++s) {
            tc::mbar_init(&full[s], 1);
            tc::mbar_init(&empty[s], 1);
        }
        for (int s = 0; s < 2; ++s) {
            tc::mbar_init(&tfull[s], 1);
            tc::mbar_init(&tempty[s], 1);
        }
        tc::mbar_init(drain, 1);
        tc::mbar_init(xready, 1);
        tc::mbar_init(xfree, 1);
        *abort = 0;
        *dr_ok = 1;
        *en_ok = 1;
        tc::fence_mbar_init();
    }
    if (warp == 1) tc::tmem_alloc(tslot, 512);
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    const uint32_t tmem = *tslot;

    const int nk = p.nk_o + p.nk_v;
    const int kseg = p.kseg > 0 && p.kseg < nk ? p.kseg : nk;
    const int nseg = (nk + kseg - 1) / kseg;
    if (warp < 4) {
        asm volatile("setmaxnreg.dec.sync.aligned.u32 %0;" ::"n"(SX_REG_LOW));
        if (warp == 0 && lane == 0) run_producer<TYPE>(p, stages, full, empty, abort);
        else if (warp == 1 && lane == 0) run_mma<TYPE>(p, stages, full, empty, tfull, tempty, drain, tmem, abort);
    } else if (warp < 8) {
        // ---------------- drain warps ----------------
        asm volatile("setmaxnreg.dec.sync.aligned.u32 %0;" ::"n"(SX_REG_DRAIN));
        const int quad = warp & 3;
        const int m = quad * 32 + lane;  // TMEM lane = GEMM row
        const bool leader = (warp == 4 && lane == 0);
        const uint32_t tq = tmem + ((uint32_t)(quad * 32) << 16);
        uint32_t sg = 0;
        int n = 0;  // items started by this CTA
        bool ok = true;
        for (int64_t it = blockIdx.x; it < p.items && ok; it += gridDim.x, ++n) {
            for (int t = 0; t < 9 && ok; ++t) {
                for (int sgi = 0; sgi < nseg; ++sgi, ++sg) {
                    const int buf = sg & 1;
                    const bool first = (t == 0 && sgi == 0);
                    if (leader) {
                        bool w = tc::mbar_wait(&tfull[buf], (sg >> 1) & 1, kWaitNs, abort);
                        // the previous item's values must have left the sub-box
                        if (w && first && n > 0) w = tc::mbar_wait(xfree, (n - 1) & 1, kWaitNs, abort);
                        *dr_ok = w ? 1 : 0;
                    }
                    named_bar(1, SX_DRAIN);
                    if (!*dr_ok) {
                        ok = false;
                        break;
                    }
                    tc::tc_fence_after();
                    drain_any(t, first, X, tq + (uint32_t)(buf * 256), m);
                    tc::tc_fence_before();
                    named_bar(1, SX_DRAIN);
                    if (leader) {
                        tc::mbar_arrive(&tempty[buf]);
                        if (t == 8 && sgi == nseg - 1) tc::mbar_arrive(xready);
                    }
                }
            }
        }
        if (leader && !ok) {
            *abort = 1;
            atomicCAS(p.err, 0, 3);
        }
    } else {
        // ---------------- energy warps ----------------
        asm volatile("setmaxnreg.inc.sync.aligned.u32 %0;" ::"n"(SX_REG_HIGH));
        const int et = threadIdx.x - 256;
        const int mm = et & 127, half = et >> 7;
        const int rb = mm >> 4, ri = (mm >> 2) & 3, rj = mm & 3;  // thread row (b;i,j)
        const int ew = et >> 5;
        const bool leader = (et == 0);
        float R[128];
        double e1 = 0.0, est = 0.0;
        int n = 0;
        for (int64_t it = blockIdx.x; it < p.items; it += gridDim.x, ++n) {
            if (leader) {
                const bool w = tc::mbar_wait(xready, n & 1, kWaitNs, abort);
                *en_ok = w ? 1 : 0;
                if (w) {
                    ItemBox bx;
                    decode_item(p, it, bx);
#pragma unroll
                    for (int dd = 0; dd < 6; ++dd) {
                        desc->g[dd] = bx.start[dd] + bx.boff[dd];
                        desc->nv[dd] = min(dd < 3 ? SX_BV : SX_BO, bx.ext[dd] - bx.boff[dd]);
                    }
                    desc->factor = p.factor[bx.tq];
                    desc->item = it;
                } else {
                    *abort = 1;
                    atomicCAS(p.err, 0, 4);
                }
            }
            named_bar(2, SX_EPI);
            if (!*en_ok) break;
#pragma unroll
            for (int A = 0; A < 4; ++A)
#pragma unroll
                for (int c = 0; c < 8; ++c)
#pragma unroll
                    for (int k = 0; k < 4; ++k) R[A * 32 + c * 4 + k] = X[xaddr(4 * half + A, rb, c, ri, rj, k)];
            named_bar(2, SX_EPI);
            if (leader) tc::mbar_arrive(xfree);
            const EDesc &d = *desc;
            energy_chunk<0>(R, d, p, half, rb, ri, rj, e1, est);
            energy_chunk<1>(R, d, p, half, rb, ri, rj, e1, est);
            energy_chunk<2>(R, d, p, half, rb, ri, rj, e1, est);
            energy_chunk<3>(R, d, p, half, rb, ri, rj, e1, est);
            write_partial(e1, est, red, d, p, ew, lane, leader);
        }
    }
    tc::tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc::tc_fence_after();
        tc::tmem_dealloc(tmem, 512);
    }
}

// ---------------------------------------------------------------------------
// Operand preparation.

// FP64 rows [rows][n] -> split rows hi/lo [rows][n_pad] of element type TYPE
// (zero padding), each value first multiplied by the power of two `scale`.
template <int TYPE>
__global__ void __launch_bounds__(256) split_rows_kernel(const double *__restrict__ src, void *hi_, void *lo_,
                                                         int64_t rows, int64_t n, int64_t n_pad, double scale) {
    const int64_t total = rows * n_pad;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = i / n_pad, c = i % n_pad;
        const double x = c < n ? src[r * n + c] * scale : 0.0;
        if (TYPE == TM_F32) {
            const float h = tc::to_tf32(__double2float_rn(x));
            ((float *)hi_)[i] = h;
            ((float *)lo_)[i] = tc::to_tf32(__double2float_rn(x - (double)h));
        } else if (TYPE == TM_BF16) {
            const __nv_bfloat16 h = __float2bfloat16_rn(__double2float_rn(x));
            ((__nv_bfloat16 *)hi_)[i] = h;
            ((__nv_bfloat16 *)lo_)[i] = __float2bfloat16_rn(__double2float_rn(x - (double)__bfloat162float(h)));
        } else {
            const __half h = __float2half_rn(__double2float_rn(x));
            ((__half *)hi_)[i] = h;
            ((__half *)lo_)[i] = __float2half_rn(__double2float_rn(x - (double)__half2float(h)));
        }
    }
}

__global__ void __launch_bounds__(256) to_f32_kernel(const double *__restrict__ src, float *__restrict__ dst,
                                                     int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        dst[i] = __double2float_rn(src[i]);
}

// max |src| as the bit pattern of a non-negative double (orders like the value).
__global__ void __launch_bounds__(256) maxabs_kernel(const double *__restrict__ src, int64_t n,
                                                     unsigned long long *out) {
    double m = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        m = fmax(m, fabs(src[i]));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, (unsigned long long)__double_as_longlong(m));
}

unsigned grid_for(int64_t n) {
    int64_t b = (n + 255) / 256;
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>(b, 152 * 16));
}

// 2^(14 - e) with max|x| < 2^e: the scaled values stay below 2^14 (FP16 max 65504).
double fp16_scale(double maxabs) {
    if (!(maxabs > 0.0) || !std::isfinite(maxabs)) return 1.0;
    int e = 0;
    std::frexp(maxabs, &e);
    e = std::max(-200, std::min(200, 14 - e));
    return std::ldexp(1.0, e);
}

}  // namespace

void mixed_release(sdt_job *j) {
    for (int k = 0; k < 2 * SP_N; ++k) {
        gpu_put(j->sp[k]);
        j->sp[k] = nullptr;
        j->sp_n[k] = 0;
    }
    gpu_put(j->t1f);
    gpu_put(j->uf);
    gpu_put(j->vd2_maps);
    gpu_put(j->pair_id);
    gpu_put(j->err_d);
    host_put(j->err_h);
    j->t1f = j->uf = nullptr;
    j->vd2_maps = nullptr;
    j->pair_id = nullptr;
    j->err_d = nullptr;
    j->err_h = nullptr;
    j->mixed_type = -1;
}

int mixed_prepare(sdt_job *j, int type, cudaStream_t st) {
    mixed_release(j);
    const Tiling &t = j->t;
    const int64_t o = t.nocc, v = t.nvir, noab = t.noab, nvab = t.nvab;
    const int es = type == TM_F32 ? 4 : 2;
    const int ke = 32 / es;                      // K elements per 32-byte row
    const int64_t pad = 16 / es;                 // rows padded to 16-byte multiples
    const int64_t op = (o + pad - 1) / pad * pad, vp = (v + pad - 1) / pad * pad;
    j->o_pad = op;
    j->v_pad = vp;
    const int64_t vd2_elems = (int64_t)j->arr_n[DST_VD2];
    int rc = SDT_OK;
    // Power-of-two operand scales (FP16 only): s_T for T2, s_I for W and V,
    // so that every merged term accumulates s_T*s_I*X.
    double sT = 1.0, sI = 1.0;
    if (type == TM_F16) {
        unsigned long long *mx = (unsigned long long *)gpu_get(3 * sizeof(unsigned long long));
        if (!mx) return fail(SDT_ERR_NOMEM, "mixed form: scale buffer");
        unsigned long long hm[3] = {0, 0, 0};
        rc = cuda_check(cudaMemsetAsync(mx, 0, 3 * sizeof(unsigned long long), st), "mixed form: scales");
        const int idx[3] = {DST_T2A, DST_WD1, DST_VD2};
        for (int q = 0; q < 3 && !rc; ++q) {
            const int64_t n = (int64_t)j->arr_n[idx[q]];
            if (n > 0) {
                maxabs_kernel<<<grid_for(n), 256, 0, st>>>(j->arr[idx[q]], n, mx + q);
                count_launch();
            }
        }
        if (!rc) rc = cuda_check(cudaGetLastError(), "mixed form: scales");
        if (!rc) rc = cuda_check(cudaMemcpyAsync(hm, mx, sizeof(hm), cudaMemcpyDeviceToHost, st), "mixed form: scales");
        if (!rc) rc = cuda_check(cudaStreamSynchronize(st), "mixed form: scales");
        gpu_put(mx);
        if (rc) return rc;
        double m[3];
        for (int q = 0; q < 3; ++q) std::memcpy(&m[q], &hm[q], sizeof(double));
        sT = fp16_scale(m[0]);
        sI = fp16_scale(std::max(m[1], m[2]));
    }
    j->inv_s = 1.0 / (sT * sI);
    j->inv_s2 = j->inv_s * j->inv_s;
    struct Src { int idx; int64_t rows, n, npad; double scale; };
    const Src src[SP_N] = {{DST_T2A, v * v * o, o, op, sT}, {DST_T2B, v * o * o, v, vp, sT},
                           {DST_WD1, v * o * o, o, op, sI}, {DST_VD2, vd2_elems / std::max<int64_t>(v, 1), v, vp, sI}};
    for (int k = 0; k < SP_N && !rc; ++k) {
        const size_t n = (size_t)(src[k].rows * src[k].npad);
        for (int h = 0; h < 2; ++h) {
            j->sp[2 * k + h] = gpu_get(std::max<size_t>(n, 1) * es);
            if (!j->sp[2 * k + h]) {
                mixed_release(j);
                return fail(SDT_ERR_NOMEM, "mixed form: split operand allocation");
            }
            j->sp_n[2 * k + h] = n;
        }
        void *hi = j->sp[2 * k], *lo = j->sp[2 * k + 1];
        const double *s = j->arr[src[k].idx];
        const unsigned gb = grid_for((int64_t)n);
        if (type == TM_F32)
            split_rows_kernel<TM_F32><<<gb, 256, 0, st>>>(s, hi, lo, src[k].rows, src[k].n, src[k].npad, src[k].scale);
        else if (type == TM_BF16)
            split_rows_kernel<TM_BF16><<<gb, 256, 0, st>>>(s, hi, lo, src[k].rows, src[k].n, src[k].npad, src[k].scale);
        else
            split_rows_kernel<TM_F16><<<gb, 256, 0, st>>>(s, hi, lo, src[k].rows, src[k].n, src[k].npad, src[k].scale);
        count_launch();
    }
    // FP32 copies of T1 [v][o] and the vvoo block [v][v][o][o] for the s1 terms.
    const int64_t n_t1 = v * o, n_u = (int64_t)j->arr_n[DST_UD];
    j->t1f = (float *)gpu_get(std::max<int64_t>(n_t1, 1) * sizeof(float));
    j->uf = (float *)gpu_get(std::max<int64_t>(n_u, 1) * sizeof(float));
    if (!j->t1f || !j->uf) {
        mixed_release(j);
        return fail(SDT_ERR_NOMEM, "mixed form: FP32 copies");
    }
    to_f32_kernel<<<grid_for(n_t1), 256, 0, st>>>(j->arr[DST_T1], j->t1f, n_t1);
    count_launch();
    to_f32_kernel<<<grid_for(n_u), 256, 0, st>>>(j->arr[DST_UD], j->uf, n_u);
    count_launch();
    if (!rc) rc = cuda_check(cudaGetLastError(), "mixed form: split");
    if (rc) {
        mixed_release(j);
        return rc;
    }
    // Tensor maps (32-byte swizzle, 32-byte K rows).
    const uint64_t E = (uint64_t)es;
    const uint32_t KE = (uint32_t)ke;
    {
        const uint64_t d[4] = {(uint64_t)vp, (uint64_t)o, (uint64_t)o, (uint64_t)v};
        const uint64_t sb[3] = {vp * E, o * vp * E, o * o * vp * E};
        const uint32_t box[4] = {KE, 4, 4, 8};
        rc = make_tmap(&j->maps[0], j->sp[2 * SP_T2B], type, 4, d, sb, box, 32);
        if (!rc) rc = make_tmap(&j->maps[1], j->sp[2 * SP_T2B + 1], type, 4, d, sb, box, 32);
    }
    if (!rc) {
        const uint64_t d[4] = {(uint64_t)op, (uint64_t)o, (uint64_t)v, (uint64_t)v};
        const uint64_t sb[3] = {op * E, o * op * E, v * o * op * E};
        const uint32_t box[4] = {KE, 4, 8, 8};
        rc = make_tmap(&j->maps[2], j->sp[2 * SP_T2A], type, 4, d, sb, box, 32);
        if (!rc) rc = make_tmap(&j->maps[3], j->sp[2 * SP_T2A + 1], type, 4, d, sb, box, 32);
    }
    if (!rc) {
        const uint64_t d[4] = {(uint64_t)op, (uint64_t)o, (uint64_t)o, (uint64_t)v};
        const uint64_t sb[3] = {op * E, o * op * E, o * o * op * E};
        const uint32_t box[4] = {KE, 4, 4, 8};
        rc = make_tmap(&j->maps[4], j->sp[2 * SP_WD1], type, 4, d, sb, box, 32);
        if (!rc) rc = make_tmap(&j->maps[5], j->sp[2 * SP_WD1 + 1], type, 4, d, sb, box, 32);
    }
    std::vector<CUtensorMap> vmaps;
    std::vector<int32_t> pid(nvab * nvab, -1);
    for (int64_t B = noab + 1; B <= noab + nvab && !rc; ++B)
        for (int64_t C = B; C <= noab + nvab && !rc; ++C) {
            const int64_t off = j->pair_host[(B - noab - 1) * nvab + (C - noab - 1)];
            if (off < 0) continue;
            const int64_t nB = t.r(B), nC = t.r(C);
            const int64_t soff = off / v * vp;  // elements; a multiple of 16 bytes
            const uint64_t d[4] = {(uint64_t)vp, (uint64_t)o, (uint64_t)nC, (uint64_t)nB};
            const uint64_t sb[3] = {vp * E, o * vp * E, nC * o * vp * E};
            const uint32_t box[4] = {KE, 4, 8, 8};
            CUtensorMap mh, ml;
            rc = make_tmap(&mh, (const uint8_t *)j->sp[2 * SP_VD2] + soff * es, type, 4, d, sb, box, 32);
            if (!rc) rc = make_tmap(&ml, (const uint8_t *)j->sp[2 * SP_VD2 + 1] + soff * es, type, 4, d, sb, box, 32);
            pid[(B - noab - 1) * nvab + (C - noab - 1)] = (int32_t)(vmaps.size() / 2);
            vmaps.push_back(mh);
            vmaps.push_back(ml);
        }
    if (rc) {
        mixed_release(j);
        return rc;
    }
    j->vd2_maps = (CUtensorMap *)gpu_get(std::max<size_t>(vmaps.size(), 1) * sizeof(CUtensorMap));
    j->pair_id = (int32_t *)gpu_get(std::max<size_t>(pid.size(), 1) * sizeof(int32_t));
    j->err_d = (int *)gpu_get(sizeof(int));
    j->err_h = (int *)host_get(sizeof(int));
    if (!j->vd2_maps || !j->pair_id || !j->err_d || !j->err_h) {
        mixed_release(j);
        return fail(SDT_ERR_NOMEM, "mixed form: tables");
    }
    if (!vmaps.empty())
        rc = cuda_check(cudaMemcpyAsync(j->vd2_maps, vmaps.data(), vmaps.size() * sizeof(CUtensorMap),
                                        cudaMemcpyHostToDevice, st), "mixed form: maps");
    if (!rc && !pid.empty())
        rc = cuda_check(cudaMemcpyAsync(j->pair_id, pid.data(), pid.size() * sizeof(int32_t), cudaMemcpyHostToDevice,
                                        st), "mixed form: maps");
    if (!rc) rc = cuda_check(cudaStreamSynchronize(st), "mixed form: prepare");
    if (rc) {
        mixed_release(j);
        return rc;
    }
    j->mixed_type = type;
    return SDT_OK;
}

int mixed_launch(sdt_job *j, int64_t items, int64_t n, cudaStream_t st) {
    const Tiling &t = j->t;
    const int type = j->mixed_type;
    const int ke = type == TM_F32 ? 8 : 16;
    SplitParams p;
    p.t2b_hi = j->maps[0]; p.t2b_lo = j->maps[1];
    p.t2a_hi = j->maps[2]; p.t2a_lo = j->maps[3];
    p.wd1_hi = j->maps[4]; p.wd1_lo = j->maps[5];
    p.vd2_maps = j->vd2_maps;
    p.pair_id = j->pair_id;
    p.T1f = j->t1f;
    p.Uf = j->uf;
    p.evl = j->evl_d;
    p.tiles = j->tiles;
    p.noab = (int32_t)t.noab;
    p.nvab = (int32_t)t.nvab;
    p.nocc = t.nocc;
    p.nvir = t.nvir;
    p.nk_o = (int32_t)((t.nocc + ke - 1) / ke);
    p.nk_v = (int32_t)((t.nvir + ke - 1) / ke);
    p.kseg = j->mixed_kseg;
    p.klist = j->klist_d;
    p.item_pref = j->pref_d;
    p.factor = j->factor_d;
    p.n_tasks = n;
    p.items = items;
    p.inv_s = j->inv_s;
    p.inv_s2 = j->inv_s2;
    p.part = j->part_d;
    p.err = j->err_d;
    int nsm = 0;
    int rc = cuda_check(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, j->dev), "mixed form");
    if (rc) return rc;
    const unsigned grid = (unsigned)std::max<int64_t>(1, std::min<int64_t>(items, nsm));
    auto launch = [&](auto kern) {
        int r = cuda_check(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, SX_SMEM_ALLOC),
                           "mixed form: smem attribute");
        if (r) return r;
        kern<<<grid, SX_THREADS, SX_SMEM_ALLOC, st>>>(p);
        count_launch();
        return cuda_check(cudaGetLastError(), "mixed form: fused kernel");
    };
    rc = cuda_check(cudaMemsetAsync(j->err_d, 0, sizeof(int), st), "mixed form");
    if (rc) return rc;
    if (type == TM_F32) rc = launch(split_fused_kernel<TM_F32>);
    else if (type == TM_BF16) rc = launch(split_fused_kernel<TM_BF16>);
    else rc = launch(split_fused_kernel<TM_F16>);
    if (!rc) rc = cuda_check(cudaMemcpyAsync(j->err_h, j->err_d, sizeof(int), cudaMemcpyDeviceToHost, st),
                             "mixed form");
    return rc;
}

}  // namespace sdt
