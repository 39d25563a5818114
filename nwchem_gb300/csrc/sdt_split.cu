// sdt_split.cu -- the mixed-precision form: one persistent kernel that runs
// the d1/d2 contractions of every sub-box as split-operand tensor-core GEMMs
// (tcgen05) and the s1 terms, denominator and energy sums on the CUDA cores,
// the latter overlapped with the next sub-box's contractions.
//
// Work unit (item): an 8x8x8 (a,b,c) x 4x4x4 (i,j,k) sub-box of one tuple's
// triples tile, 32768 values.  One CTA per SM; CTAs draw items from a device
// queue (one atomic counter) until it is empty.  Each item's result depends
// only on its index, so results do not depend on timing.
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
// Energies.  When an item's eighth term is drained, the energy warps copy
// the sub-box from shared memory into registers (128 values per thread), add
// the ninth term's accumulator from TMEM to it themselves (its rows (b;i,j)
// and columns (a,c;k) are the layout of their copy), and release both; the
// drain warps then store the next item's first term into the sub-box while
// the energy warps evaluate the copy: the s1 products in FP32 from
// FP32 copies of T1 and the vvoo block, the denominator and the quotient in
// FP32 (orbital energies shifted by the midpoint of the occupied-virtual
// gap, so that no sum in a denominator cancels), and the two energy sums in
// FP64, one FP64 add per four elements.  So the energy work of one item overlaps
// the contractions of the next.  In the tensor-memory hold variant (HOLD = 1)
// the last drain writes the finished sub-box into the upper 256 TMEM columns
// instead, one accumulator remains, and 16 energy warps read the sub-box
// from TMEM.
//
// Warp roles: 0 TMA producer, 1 MMA issuer + TMEM owner, 2-3 idle, 4-7 drain
// (TMEM lane quadrant warp % 4), 8-15 energy (8-23 with HOLD = 1).  Every mbarrier wait is bounded
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
// Tensor-memory hold (the finished sub-box in TMEM, not in the energy warps'
// registers): 768 threads, 16 energy warps (warps 8-23, four per SM
// sub-partition, each a lane quadrant and a quarter of the hold columns).
// The launch gives 80 registers per thread (65536 / 768, rounded down to 8);
// warps 0-3 drop to 56, the drains to 72, the energy warps rise to 88:
// 128*56 + 128*72 + 512*88 = 61440 = 768*80, and per sub-partition
// (56 + 72 + 4*88)*32 = 15360 <= 16384.
constexpr int SX_THREADS_H = 768, SX_EPI_H = 512;
constexpr int SX_REG_LAUNCH_H = 80, SX_REG_HIGH_H = 88, SX_REG_DRAIN_H = 72;
// Register split (setmaxnreg): the launch gives 128 per thread (4 warps per
// SM sub-partition); warps 0-3 drop to 56, the drain warps to 88 and the
// energy warps rise to 184: 128*56 + 128*88 + 256*184 = 65536 = 512*128,
// and each sub-partition holds one warp of warps 0-3, one drain warp and two
// energy warps: (56+88+2*184)*32 = 16384.  (Measured against 72 / 192: the
// drains are the short-K bottleneck, and the FP32 energy pass fits in 184.)
constexpr int SX_REG_LAUNCH = 128, SX_REG_LOW = 56, SX_REG_DRAIN = 88, SX_REG_HIGH = 184;
static_assert(128 * SX_REG_LOW + 128 * SX_REG_DRAIN + 256 * SX_REG_HIGH <= SX_THREADS * SX_REG_LAUNCH,
              "register split");
static_assert((SX_REG_LOW + SX_REG_DRAIN + 2 * SX_REG_HIGH) * 32 <= 16384, "register split: sub-partition registers");
// setmaxnreg.dec may only lower and setmaxnreg.inc only raise a warp's count.
static_assert(SX_REG_LOW <= SX_REG_LAUNCH && SX_REG_DRAIN <= SX_REG_LAUNCH && SX_REG_HIGH >= SX_REG_LAUNCH,
              "setmaxnreg direction");
static_assert(SX_REG_LAUNCH_H * SX_THREADS_H <= 65536 && SX_REG_LAUNCH_H % 8 == 0 &&
                  (SX_REG_LAUNCH_H + 8) * SX_THREADS_H > 65536,
              "hold variant: launch registers = the most 768 threads can have");
static_assert(128 * SX_REG_LOW + 128 * SX_REG_DRAIN_H + SX_EPI_H * SX_REG_HIGH_H <= SX_THREADS_H * SX_REG_LAUNCH_H,
              "hold variant: register split");
static_assert(SX_REG_LOW <= SX_REG_LAUNCH_H && SX_REG_DRAIN_H <= SX_REG_LAUNCH_H && SX_REG_HIGH_H >= SX_REG_LAUNCH_H,
              "hold variant: setmaxnreg direction");
static_assert((SX_REG_LOW + SX_REG_DRAIN_H + 4 * SX_REG_HIGH_H) * 32 <= 16384, "hold variant: sub-partition registers");
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

// What the energy chunks of an item need after its last drain: the sub-box
// and the job data it reads and writes (several jobs may share a launch).
struct EDesc {
    int g[6];       // global orbital index of the sub-box origin, per dimension
    int nv[6];      // valid extent of the sub-box, per dimension
    int gp[6];      // holes (3..5): padded hole index of the origin (FP32 s1 copies)
    int op;         // padded hole count of the job's FP32 copies
    double factor;  // the tuple's multiplicity factor
    long long item; // the item's index within its job
    const float *T1f, *Uf;      // the job's FP32 copies of T1 and the vvoo block
    const float *eo, *ev;       // its occupied and virtual orbital energies, shifted, FP32
    double *part;               // its per-item energy pairs
    double inv_s, inv_s2;       // its operand scaling
    long long nvir;
};
static_assert(sizeof(EDesc) <= 192, "EDesc fits its shared-memory slot");

// Split operands live in HBM "block-major": one block per (row boxes, K chunk)
// holds a whole stage tile, its hi half then its lo half -- 128 rows (A) or
// 256 rows (B) of 32 bytes each, in the row order the MMA reads and already
// 32-byte swizzled -- so a stage is two contiguous bulk copies (A 8 KB, B
// 16 KB).  The single producer thread's issue rate bounds the long-K
// contractions: two copies per stage instead of four (hi and lo apart) ran
// 12 % faster.  Rows are the box products of the tiles' boxes (8 particle
// or 4 hole indices, zero padded at tile ends); box ids are global over all
// tiles of a space.
//   Wd1 (d1 A)  [X][H1][H2][kc_o]   rows (R0 8, R1 4, R2 4), K = m
//   T2b (d2 A)  [X][H1][H2][kc_v]   rows (R0 8, R1 4, R2 4), K = e
//   T2a (d1 B)  [X0][X1][H][kc_o]   rows (C0 8, C1 8, C2 4), K = m
//   Vd2 (d2 B)  per tile pair (B<=C): [lb0][lb1][H][kc_v], lb local boxes
enum { L_WD1 = 0, L_T2B, L_T2A, L_VD2, L_N };

struct alignas(16) SplitParams {
    const uint8_t *blk[2 * L_N];  // [2*layout + (0 hi, 1 lo)]
    const int32_t *tile_box;      // [ntiles]: global box id of the tile's first box (its space)
    const int64_t *pair_blk;      // [nvab*nvab]: first Vd2 block of tile pair (B<=C), -1 none
    const float *T1f, *Uf;        // FP32 copies: [v][OP], [v][v][OP][OP], holes padded per tile to 4
    int32_t op;                   // OP, the padded hole count (4 x hole boxes)
    const double *evl;
    const float *evf;             // orbital energies minus the gap midpoint, FP32 (occupied, then virtual)
    const int32_t *tiles;         // [ntiles][4] start, range, spin, sym
    int32_t noab, nvab, nk_o, nk_v, kseg, nob, nvb;
    int64_t nocc, nvir;
    const int64_t *klist, *item_pref;
    const double *factor;
    int64_t n_tasks, n_items;
    double inv_s, inv_s2;         // undo the operand scaling (FP16): X_true = X * inv_s
    double *part;
    int *err;
    unsigned long long *queue;    // item counter, zero at launch
    int32_t all_k;                // every K tile allowed for every term (one spin, no irreps)
};

static_assert(sizeof(SplitParams) % 16 == 0, "job parameters copy in 16-byte pieces");

// The shared item queue of the serving path: several jobs' items, drawn by
// one resident launch.  The host appends a job by writing its parameters to
// table[slot] and its first queue position to base[slot], then raising
// tail by the job's item count (queue positions base .. base + items - 1).
// CTAs take positions one at a time (never past tail), leave when nothing
// is left to take for idle_ns or when close is set, and count each job's
// finished items; the CTA that finishes a job's last item stores the launch
// number in last_gen[slot] (host-mapped memory), which is how the host
// learns that the job's per-item energies are complete.
struct QueueCtl {
    const SplitParams *table;        // [max_jobs]
    const long long *base;           // [max_jobs]; LLONG_MAX for slots not yet used
    unsigned long long *head;        // next position to take
    const unsigned long long *tail;  // positions published
    unsigned long long *done;        // [max_jobs] finished items per job
    int *first_gen, *last_gen;       // [max_jobs] host-mapped: launch that took the job's first / finished its last item
    const int *close;
    int *err;
    unsigned long long idle_ns;
    int max_jobs, gen;
};
constexpr int kSlotShift = 40;       // queue-mode ring entries: slot << 40 | item within the job
constexpr long long kItemMask = (1ll << kSlotShift) - 1;

__device__ __forceinline__ unsigned long long ld_volatile(const unsigned long long *p) {
    return *(const volatile unsigned long long *)p;
}

// Takes the next queue position (-1: nothing to take for idle_ns, or close).
__device__ __forceinline__ long long claim_position(const QueueCtl &q, volatile int *abort) {
    const uint64_t t0 = tc::global_ns();
    unsigned pause = 64;
    while (true) {
        const unsigned long long h = ld_volatile(q.head), t = ld_volatile(q.tail);
        if (h < t) {
            if (atomicCAS(q.head, h, h + 1) == h) {
                __threadfence();  // the job's table entry was written before tail grew
                return (long long)h;
            }
            continue;
        }
        if (*abort || *(const volatile int *)q.close) return -1;
        if (tc::global_ns() - t0 > q.idle_ns) return -1;
        __nanosleep(pause);
        if (pause < 8192) pause *= 2;
    }
}

// Slot of queue position pos: the last slot whose base is <= pos (unused
// slots hold LLONG_MAX).  Read through L2 only: the host rewrites entries
// while the launch runs.
__device__ __forceinline__ int find_slot(const QueueCtl &q, long long pos) {
    int lo = 0, hi = q.max_jobs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldcg(q.base + mid) <= pos) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ void load_job(const QueueCtl &q, int slot, SplitParams &out) {
    const uint4 *src = reinterpret_cast<const uint4 *>(q.table + slot);
    uint4 *dst = reinterpret_cast<uint4 *>(&out);
#pragma unroll
    for (int k = 0; k < (int)(sizeof(SplitParams) / 16); ++k) dst[k] = __ldcg(src + k);
}

struct ItemBox {
    int tile[6], start[6], ext[6], boff[6], lbox[6];  // lbox: local box, clamped into the tile
    int64_t tq, item;
};

// Decodes item si: its tuple (binary search of the item prefix) and its
// sub-box, k box fastest.
__device__ __forceinline__ void decode_item(const SplitParams &p, int64_t si, ItemBox &b) {
    int64_t lo = 0, hi = p.n_tasks - 1;
    while (lo < hi) {
        const int64_t mid = (lo + hi + 1) >> 1;
        if (p.item_pref[mid] <= si) lo = mid;
        else hi = mid - 1;
    }
    b.tq = lo;
    b.item = si;
    int64_t local = si - p.item_pref[lo];
    int nb[6];
#pragma unroll
    for (int d = 0; d < 6; ++d) {
        b.tile[d] = (int)p.klist[7 * lo + d];
        b.start[d] = __ldg(p.tiles + 4 * (b.tile[d] - 1));
        b.ext[d] = __ldg(p.tiles + 4 * (b.tile[d] - 1) + 1);
        const int bx = d < 3 ? SX_BV : SX_BO;
        nb[d] = (b.ext[d] + bx - 1) / bx;
    }
    int box[6];
#pragma unroll
    for (int d = 5; d >= 0; --d) {
        box[d] = (int)(local % nb[d]);
        local /= nb[d];
    }
#pragma unroll
    for (int d = 0; d < 6; ++d) {
        b.boff[d] = box[d] * (d < 3 ? SX_BV : SX_BO);
        b.lbox[d] = box[d];
    }
}

// K chunks of merged term td for one part (0: d1, K over occupied tiles;
// 1: d2, K over virtual tiles).  A chunk (KE consecutive orbitals of the
// space) is kept when it meets a K tile that spin and irrep allow for the
// term -- the T2 read t(C0,C1;C2,m) for d1 and t(R0,e;R1,R2) for d2
// (tce_hashnsort.F:31-36, :107-111); forbidden blocks are zero in the
// operands, so a kept chunk that straddles one adds nothing.  f(c) is called
// in increasing c; returns the count.
template <int KE, class F>
__device__ __forceinline__ int term_chunks(const SplitParams &p, const ItemBox &bx, const MergedTerm &td, int part,
                                           F &&f) {
    const int nk = part == 0 ? p.nk_o : p.nk_v;
    if (p.all_k) {
        for (int c = 0; c < nk; ++c) f(c);
        return nk;
    }
    const int32_t *tl = p.tiles;
    auto sp = [&](int d) { return __ldg(tl + 4 * (bx.tile[d] - 1) + 2); };
    auto sy = [&](int d) { return __ldg(tl + 4 * (bx.tile[d] - 1) + 3); };
    int need_s, need_y;  // spin and irrep the summed tile must have
    if (part == 0) {
        need_s = sp(td.c[0]) + sp(td.c[1]) - sp(td.c[2]);
        need_y = sy(td.c[0]) ^ sy(td.c[1]) ^ sy(td.c[2]);
    } else {
        need_s = sp(td.r[1]) + sp(td.r[2]) - sp(td.r[0]);
        need_y = sy(td.r[0]) ^ sy(td.r[1]) ^ sy(td.r[2]);
    }
    const int t0 = part == 0 ? 1 : p.noab + 1, t1 = part == 0 ? p.noab : p.noab + p.nvab;
    int last = -1, n = 0;
    for (int T = t0; T <= t1; ++T) {
        if (__ldg(tl + 4 * (T - 1) + 2) != need_s || __ldg(tl + 4 * (T - 1) + 3) != need_y) continue;
        const int st = __ldg(tl + 4 * (T - 1)), r = __ldg(tl + 4 * (T - 1) + 1);
        const int c1 = (st + r - 1) / KE;
        for (int c = max(st / KE, last + 1); c <= c1; ++c, ++n) f(c);
        last = max(last, c1);
    }
    return n;
}

template <int KE>
__device__ __forceinline__ int term_chunk_count(const SplitParams &p, const ItemBox &bx, int t) {
    const MergedTerm td = kMerged[t];
    return term_chunks<KE>(p, bx, td, 0, [](int) {}) + term_chunks<KE>(p, bx, td, 1, [](int) {});
}

// Drains (accumulator segments) of a term of nk kept chunks.
__device__ __forceinline__ int term_segments(int nk, int kseg_req, int &kseg) {
    kseg = (kseg_req > 0 && kseg_req < nk) ? kseg_req : (nk > 0 ? nk : 1);
    return nk > 0 ? (nk + kseg - 1) / kseg : 1;
}

// Items of a CTA: the producer thread takes the next item from the device
// queue and publishes it in a 4-slot ring (id, or -1 at the end), which the
// MMA thread, the drain leader and the energy leader each read and release.
constexpr int SX_RING = 4;
struct UnitRing {
    int64_t *id;
    uint64_t *full, *empty;
};
__device__ __forceinline__ bool ring_publish(const UnitRing &r, int n, int64_t u, volatile int *abort) {
    const int s = n % SX_RING;
    if (n >= SX_RING && !tc::mbar_wait(&r.empty[s], ((n / SX_RING) - 1) & 1, kWaitNs, abort)) return false;
    r.id[s] = u;
    tc::mbar_arrive(&r.full[s]);
    return true;
}
// Returns the unit, -1 at the end, -2 when the wait ran out.
__device__ __forceinline__ int64_t ring_take(const UnitRing &r, int n, volatile int *abort) {
    const int s = n % SX_RING;
    if (!tc::mbar_wait(&r.full[s], (n / SX_RING) & 1, kWaitNs, abort)) return -2;
    const int64_t u = r.id[s];
    tc::mbar_arrive(&r.empty[s]);
    return u;
}

__device__ __forceinline__ void named_bar(int id, int n) {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory");
}

template <int TYPE>
__device__ __forceinline__ void mma_split(uint32_t d, uint64_t a, uint64_t b, uint32_t acc) {
    if (TYPE == TM_F32) tc::mma_tf32(d, a, b, tc::idesc_tf32(128, 256), acc);
    else tc::mma_f16(d, a, b, tc::idesc_f16(128, 256, TYPE == TM_BF16), acc);
}

__device__ __forceinline__ void bulk_load(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 ::"r"(tc::smem_u32(dst)), "l"(src), "r"(bytes), "r"(tc::smem_u32(bar))
                 : "memory");
}

// ---------------------------------------------------------------------------
// Operand producer (one thread): takes the next item (from the launch's own
// counter, or in queue mode the next queue position and its job's table
// entry), publishes it to the other roles, and per stage issues the A and B
// blocks (hi, lo) of the term's K chunk, four contiguous bulk copies.
template <int TYPE, int QUEUE>
__device__ __forceinline__ void run_producer(const SplitParams &gp, const QueueCtl &q, uint8_t *stages,
                                             uint64_t *full, uint64_t *empty, volatile int *abort,
                                             const UnitRing &ring) {
    constexpr int KE = TYPE == TM_F32 ? 8 : 16;  // K values per 32-byte row
    SplitParams lp;                              // queue mode: the current item's job
    uint32_t g = 0;
    bool stop = false;
    for (int n = 0; !stop; ++n) {
        int64_t unit, item = 0;
        if (QUEUE) {
            const long long pos = claim_position(q, abort);
            unit = -1;
            if (pos >= 0) {
                const int slot = find_slot(q, pos);
                item = pos - __ldcg(q.base + slot);
                unit = ((int64_t)slot << kSlotShift) | item;
                load_job(q, slot, lp);
                if (item == 0) {
                    *(volatile int *)(q.first_gen + slot) = q.gen;
                    __threadfence_system();
                }
            }
        } else {
            const unsigned long long u = atomicAdd(gp.queue, 1ull);
            unit = item = u < (unsigned long long)gp.n_items ? (int64_t)u : -1;
        }
        if (!ring_publish(ring, n, unit, abort)) {
            stop = true;
            break;
        }
        if (unit < 0) break;
        const SplitParams &p = QUEUE ? lp : gp;
        const int64_t NOB = p.nob, NVB = p.nvb;
        ItemBox bx;
        decode_item(p, item, bx);
        int gb[6];  // global box ids
#pragma unroll
        for (int d = 0; d < 6; ++d) gb[d] = __ldg(p.tile_box + bx.tile[d] - 1) + bx.lbox[d];
        for (int t = 0; t < 9 && !stop; ++t) {
            const MergedTerm td = kMerged[t];
            // first blocks (K chunk 0) of the term's d1 and d2 operands
            const int64_t arow = ((int64_t)gb[td.r[0]] * NOB + gb[td.r[1]]) * NOB + gb[td.r[2]];
            const int64_t a1 = arow * p.nk_o, a2 = arow * p.nk_v;
            const int64_t b1 = (((int64_t)gb[td.c[0]] * NVB + gb[td.c[1]]) * NOB + gb[td.c[2]]) * p.nk_o;
            const int tc1 = bx.tile[td.c[1]];
            const int nbc1 = (__ldg(p.tiles + 4 * (tc1 - 1) + 1) + SX_BV - 1) / SX_BV;
            const int64_t b2 = __ldg(p.pair_blk + (bx.tile[td.c[0]] - p.noab - 1) * p.nvab + (tc1 - p.noab - 1)) +
                               (((int64_t)bx.lbox[td.c[0]] * nbc1 + bx.lbox[td.c[1]]) * NOB + gb[td.c[2]]) * p.nk_v;
            for (int part = 0; part < 2 && !stop; ++part) {
                const int la = part == 0 ? L_WD1 : L_T2B, lb = part == 0 ? L_T2A : L_VD2;
                const int64_t abase = part == 0 ? a1 : a2, bbase = part == 0 ? b1 : b2;
                term_chunks<KE>(p, bx, td, part, [&](int c) {
                    if (stop) return;
                    const int s = g % SX_NS;
                    if (g >= SX_NS && !tc::mbar_wait(&empty[s], ((g / SX_NS) & 1) ^ 1, kWaitNs, abort)) {
                        stop = true;
                        return;
                    }
                    ++g;
                    uint8_t *st = stages + s * SX_STAGE;
                    tc::mbar_arrive_expect_tx(&full[s], SX_STAGE);
                    // both source addresses first, then the two copies back to back (the
                    // single producer thread's issue rate bounds the long-K contractions)
                    const int64_t ab = abase + c, bb = bbase + c;
                    const uint8_t *a = p.blk[2 * la] + ab * (2 * SX_A), *b = p.blk[2 * lb] + bb * (2 * SX_B);
                    bulk_load(st, a, 2 * SX_A, &full[s]);
                    bulk_load(st + 2 * SX_A, b, 2 * SX_B, &full[s]);
                });
            }
        }
    }
    if (stop) {
        *abort = 1;
        atomicCAS(QUEUE ? q.err : gp.err, 0, 1);
        // copies already issued must land before the CTA exits
        volatile int never = 0;
        for (uint32_t x = g >= SX_NS ? g - SX_NS : 0; x < g; ++x)
            tc::mbar_wait(&full[x % SX_NS], (x / SX_NS) & 1, kWaitNs, &never);
    }
}

// ---------------------------------------------------------------------------
// MMA issuer (one thread).
template <int TYPE, int NB, int QUEUE>
__device__ __forceinline__ void run_mma(const SplitParams &gp, const QueueCtl &q, uint8_t *stages, uint64_t *full,
                                        uint64_t *empty, uint64_t *tfull, uint64_t *tempty, uint64_t *drain,
                                        uint32_t tmem, volatile int *abort, const UnitRing &ring) {
    constexpr int KE = TYPE == TM_F32 ? 8 : 16;
    SplitParams lp;
    uint32_t g = 0, sg = 0;  // stage and segment counters
    bool stop = false;
    for (int n = 0; !stop; ++n) {
        const int64_t unit = ring_take(ring, n, abort);
        if (unit == -2) stop = true;
        if (unit < 0) break;
        if (QUEUE) load_job(q, (int)(unit >> kSlotShift), lp);
        const SplitParams &p = QUEUE ? lp : gp;
        ItemBox bx;
        decode_item(p, QUEUE ? (unit & kItemMask) : unit, bx);
        for (int t = 0; t < 9 && !stop; ++t) {
            const int nk = term_chunk_count<KE>(p, bx, t);
            int kseg;
            const int nseg = term_segments(nk, p.kseg, kseg);
            for (int sgi = 0; sgi < nseg && !stop; ++sgi, ++sg) {
                const int buf = sg % NB;  // NB accumulators of 256 columns
                if (sg >= NB && !tc::mbar_wait(&tempty[buf], ((sg / NB) - 1) & 1, kWaitNs, abort)) {
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
                if (!stop) tc::mma_commit(&tfull[buf]);  // an empty term commits nothing new
            }
        }
    }
    if (stop) {
        *abort = 1;
        atomicCAS(QUEUE ? q.err : gp.err, 0, 2);
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

// The last term's drain when the sub-box is kept in tensor memory: the sum
// of the sub-box value and the accumulator goes to the hold region (row m =
// (b;i,j), column 32a + 4c + k), not back to shared memory.
__device__ __forceinline__ void drain_hold(const float *X, uint32_t tacc, uint32_t thold, int m) {
    const int b = m >> 4, i = (m >> 2) & 3, j = m & 3;
#pragma unroll 1
    for (int cc = 0; cc < 8; ++cc) {
        float v[32], w[32];
        tc::tmem_ld32(tacc + (uint32_t)(cc * 32), v);
#pragma unroll
        for (int q = 0; q < 32; ++q) w[q] = X[xaddr(cc, b, q >> 2, i, j, q & 3)] + v[q];  // term 8: sign +1
        tc::tmem_st32(thold + (uint32_t)(cc * 32), w);
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

// Exact FP32 -> FP64 widening by assembling the IEEE-754 fields on the
// integer pipes (the conversion instruction runs on the narrow FP64 pipe):
// sign kept, exponent rebiased by 1023 - 127,
// mantissa shifted into the top 23 of 52 bits; zero and FP32 subnormals
// (|x| < 2^-126) give signed zero, infinities and NaNs keep their class.
__device__ __forceinline__ double widen(float f) {
    const uint32_t u = __float_as_uint(f);
    const uint32_t e = (u >> 23) & 0xffu;
    const uint32_t m = u & 0x7fffffu;
    const uint32_t e64 = e == 0xffu ? 0x7ffu : e + 896u;
    const uint32_t hi = (u & 0x80000000u) | (e ? (e64 << 20) | (m >> 3) : 0u);
    const uint32_t lo = e ? (m << 29) : 0u;
    return __hiloint2double((int)hi, (int)lo);
}

// ---------------------------------------------------------------------------
// Energies of one item from its values R in registers: thread (b;i,j) with
// R[32*A + 4*c + k] = X(a = 4*half + A, b, c, i, j, k).
//   X_s = t1(a,i)u(b,c,j,k) - t1(a,j)u(b,c,i,k) + t1(a,k)u(b,c,i,j)
//       - t1(b,i)u(a,c,j,k) + t1(b,j)u(a,c,i,k) - t1(b,k)u(a,c,i,j)
//       + t1(c,i)u(a,b,j,k) - t1(c,j)u(a,b,i,k) + t1(c,k)u(a,b,i,j)   (FP32)
//   D = (e_i + e_j + e_k) - (e_a + e_b + e_c)                          (FP32)
//   q = X / D; per c, the four k terms q X and q X_s summed in FP32,
//   then added to e1 and est                                            (FP64)
// The orbital energies are FP32 copies of e - mu, mu the midpoint of the
// gap between the highest occupied and the lowest virtual level: every
// hole term of D is then negative and every particle term positive, so
// |D| is the sum of the terms' magnitudes and the FP32 sums round to a few
// units in the last place of |D| (relative ~1e-7), far below the error of
// the split products.
__device__ __forceinline__ float4 ld4(const float *p) { return __ldg(reinterpret_cast<const float4 *>(p)); }
__device__ __forceinline__ float el(const float4 &x, int k) { return k == 0 ? x.x : k == 1 ? x.y : k == 2 ? x.z : x.w; }

// The s1 operands are FP32 copies with every occupied tile padded to a
// multiple of 4 holes, so the 4 k values of a sub-box are one aligned float4.
// R[OFF + 4*c + k] holds local (a = 4*half + A, b, c, i, j, k).
template <int A, int OFF, int N>
__device__ __forceinline__ void energy_chunk(const float (&R)[N], const EDesc &d, int half, int b, int i, int j,
                                             double &e1, double &est) {
    const int a = 4 * half + A;
    if (a >= d.nv[0] || b >= d.nv[1] || i >= d.nv[3] || j >= d.nv[4]) return;
    const int op = d.op;
    const int64_t v = d.nvir, oo = (int64_t)op * op;
    const int ga = d.g[0] + a, gb = d.g[1] + b, gi = d.g[3] + i, gj = d.g[4] + j;
    const int pi = d.gp[3] + i, pj = d.gp[4] + j, pk0 = d.gp[5];  // padded holes
    const int nc = d.nv[2], nk = d.nv[5], gc0 = d.g[2], gk0 = d.g[5];
    const float *__restrict__ eo = d.eo;
    const float *__restrict__ ev = d.ev;
    const float eij = __ldg(eo + gi) + __ldg(eo + gj);
    const float eab = __ldg(ev + ga) + __ldg(ev + gb);
    float P[4];  // e_i + e_j + e_k
#pragma unroll
    for (int k = 0; k < 4; ++k) P[k] = k < nk ? eij + __ldg(eo + gk0 + k) : -1.0f;
    const float *__restrict__ t1a = d.T1f + (int64_t)ga * op;
    const float *__restrict__ t1b = d.T1f + (int64_t)gb * op;
    const float t1ai = __ldg(t1a + pi), t1aj = __ldg(t1a + pj), t1bi = __ldg(t1b + pi), t1bj = __ldg(t1b + pj);
    const float4 t1ak = ld4(t1a + pk0), t1bk = ld4(t1b + pk0);
    const float *__restrict__ uab = d.Uf + ((int64_t)ga * v + gb) * oo;
    const float uabij = __ldg(uab + pi * op + pj);
    const float4 uabj = ld4(uab + pj * op + pk0), uabi = ld4(uab + pi * op + pk0);
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        if (c < nc) {
            const int gc = gc0 + c;
            const float *__restrict__ t1c = d.T1f + (int64_t)gc * op;
            const float *__restrict__ ubc = d.Uf + ((int64_t)gb * v + gc) * oo;
            const float *__restrict__ uac = d.Uf + ((int64_t)ga * v + gc) * oo;
            const float t1ci = __ldg(t1c + pi), t1cj = __ldg(t1c + pj);
            const float ubcij = __ldg(ubc + pi * op + pj), uacij = __ldg(uac + pi * op + pj);
            const float4 ubcj = ld4(ubc + pj * op + pk0), ubci = ld4(ubc + pi * op + pk0);
            const float4 uacj = ld4(uac + pj * op + pk0), uaci = ld4(uac + pi * op + pk0);
            const float4 t1ck = ld4(t1c + pk0);
            const float Q = eab + __ldg(ev + gc);
            float e1c = 0.0f, estc = 0.0f;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                if (k < nk) {
                    float s = t1ai * el(ubcj, k);
                    s = fmaf(-t1aj, el(ubci, k), s);
                    s = fmaf(el(t1ak, k), ubcij, s);
                    s = fmaf(-t1bi, el(uacj, k), s);
                    s = fmaf(t1bj, el(uaci, k), s);
                    s = fmaf(-el(t1bk, k), uacij, s);
                    s = fmaf(t1ci, el(uabj, k), s);
                    s = fmaf(-t1cj, el(uabi, k), s);
                    s = fmaf(el(t1ck, k), uabij, s);
                    const float x = R[OFF + c * 4 + k];
                    const float q = __fdividef(x, P[k] - Q);
                    e1c = fmaf(q, x, e1c);
                    estc = fmaf(q, s, estc);
                }
            }
            e1 += widen(e1c);
            est += widen(estc);
        }
    }
}

// The same energies reading the finished sub-box from the tensor-memory hold
// columns (th: this warp's lane quadrant, column 128*half), 4 columns (the
// k values of one c) at a time in rolled loops: a small loop body, and
// registers free for the FP64 work.  All lanes take part in every TMEM load.
template <int NA>
__device__ __forceinline__ void energy_tmem(uint32_t th, const EDesc &d, int part, int b, int i, int j, double &e1,
                                            double &est) {
    const bool row_ok = b < d.nv[1] && i < d.nv[3] && j < d.nv[4];
    const int op = d.op;
    const int64_t v = d.nvir, oo = (int64_t)op * op;
    const int gb = d.g[1] + b, gi = d.g[3] + i, gj = d.g[4] + j;
    const int pi = d.gp[3] + i, pj = d.gp[4] + j, pk0 = d.gp[5];
    const int nc = d.nv[2], nk = d.nv[5], gc0 = d.g[2], gk0 = d.g[5];
    const float *__restrict__ eo = d.eo;
    const float *__restrict__ ev = d.ev;
    float P[4];
    const float eij = row_ok ? __ldg(eo + gi) + __ldg(eo + gj) : 0.0f;
#pragma unroll
    for (int k = 0; k < 4; ++k) P[k] = (row_ok && k < nk) ? eij + __ldg(eo + gk0 + k) : -1.0f;
    const float *__restrict__ t1b = d.T1f + (int64_t)(row_ok ? gb : 0) * op;
    const float t1bi = row_ok ? __ldg(t1b + pi) : 0.f, t1bj = row_ok ? __ldg(t1b + pj) : 0.f;
    const float4 t1bk = row_ok ? ld4(t1b + pk0) : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll 1
    for (int A = 0; A < NA; ++A) {
        const int a = NA * part + A;
        const bool ok_a = row_ok && a < d.nv[0];
        const int ga = d.g[0] + a;
        const float *__restrict__ t1a = d.T1f + (int64_t)(ok_a ? ga : 0) * op;
        const float *__restrict__ uab = d.Uf + ((int64_t)(ok_a ? ga : 0) * v + (ok_a ? gb : 0)) * oo;
        float t1ai = 0.f, t1aj = 0.f, uabij = 0.f;
        float4 t1ak = make_float4(0.f, 0.f, 0.f, 0.f), uabj = t1ak, uabi = t1ak;
        float eab = 0.0f;
        if (ok_a) {
            t1ai = __ldg(t1a + pi);
            t1aj = __ldg(t1a + pj);
            t1ak = ld4(t1a + pk0);
            uabij = __ldg(uab + pi * op + pj);
            uabj = ld4(uab + pj * op + pk0);
            uabi = ld4(uab + pi * op + pk0);
            eab = __ldg(ev + ga) + __ldg(ev + gb);
        }
#pragma unroll 1
        for (int c = 0; c < 8; ++c) {
            const float4 x4 = tc::tmem_ld4(th + (uint32_t)(32 * A + 4 * c));  // every lane
            if (!ok_a || c >= nc) continue;
            const int gc = gc0 + c;
            const float *__restrict__ t1c = d.T1f + (int64_t)gc * op;
            const float *__restrict__ ubc = d.Uf + ((int64_t)gb * v + gc) * oo;
            const float *__restrict__ uac = d.Uf + ((int64_t)ga * v + gc) * oo;
            const float t1ci = __ldg(t1c + pi), t1cj = __ldg(t1c + pj);
            const float ubcij = __ldg(ubc + pi * op + pj), uacij = __ldg(uac + pi * op + pj);
            const float4 ubcj = ld4(ubc + pj * op + pk0), ubci = ld4(ubc + pi * op + pk0);
            const float4 uacj = ld4(uac + pj * op + pk0), uaci = ld4(uac + pi * op + pk0);
            const float4 t1ck = ld4(t1c + pk0);
            const float Q = eab + __ldg(ev + gc);
            float e1c = 0.0f, estc = 0.0f;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                if (k < nk) {
                    float s = t1ai * el(ubcj, k);
                    s = fmaf(-t1aj, el(ubci, k), s);
                    s = fmaf(el(t1ak, k), ubcij, s);
                    s = fmaf(-t1bi, el(uacj, k), s);
                    s = fmaf(t1bj, el(uaci, k), s);
                    s = fmaf(-el(t1bk, k), uacij, s);
                    s = fmaf(t1ci, el(uabj, k), s);
                    s = fmaf(-t1cj, el(uabi, k), s);
                    s = fmaf(el(t1ck, k), uabij, s);
                    const float x = el(x4, k);
                    const float q = __fdividef(x, P[k] - Q);
                    e1c = fmaf(q, x, e1c);
                    estc = fmaf(q, s, estc);
                }
            }
            e1 += widen(e1c);
            est += widen(estc);
        }
    }
}

// Per-item pair: E[T] part f/S^2 sum X^2/D, E(T) part that + f/S sum X X_s/D.
// The sums run over 16 slots in a fixed order, slot = 4*quarter + quadrant
// (quarter: a pair of a values, quadrant: the TMEM lane quadrant), whatever
// the warp layout: NQ quarter partials per thread, the first quarter0 --
// so both work-unit shapes give the same bits.
template <int EPI, int NQ>
__device__ __forceinline__ void write_partial(double (&e1)[NQ], double (&est)[NQ], double *red, const EDesc &d,
                                              int quarter0, int quadrant, int lane, bool leader) {
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
        const double x = warp_sum(e1[q]), y = warp_sum(est[q]);
        if (lane == 0) {
            const int slot = 4 * (quarter0 + q) + quadrant;
            red[2 * slot] = x;
            red[2 * slot + 1] = y;
        }
        e1[q] = 0.0;
        est[q] = 0.0;
    }
    named_bar(2, EPI);
    if (leader) {
        double s1 = 0.0, s2 = 0.0;
        for (int w = 0; w < 16; ++w) {
            s1 += red[2 * w];
            s2 += red[2 * w + 1];
        }
        const double et = d.factor * s1 * d.inv_s2;
        d.part[2 * d.item] = et;
        d.part[2 * d.item + 1] = et + d.factor * s2 * d.inv_s;
    }
}

// Queue mode, energy leader, after the item's pair is written: counts the
// job's finished items; the one that finishes the job publishes the launch
// number to the host (its earlier pair writes are visible first).
__device__ __forceinline__ void job_item_done(const QueueCtl &q, int slot, int64_t items) {
    __threadfence();
    if (atomicAdd(q.done + slot, 1ull) + 1 == (unsigned long long)items) {
        __threadfence_system();
        *(volatile int *)(q.last_gen + slot) = q.gen;
    }
}

// HOLD = 0: the energy warps keep the finished sub-box in registers, two
// TMEM accumulators; HOLD = 1: the last drain writes it to the upper 256
// TMEM columns, which the energy warps read 32 columns at a time (their
// registers stay free for the FP64 work), one accumulator.
template <int TYPE, int HOLD, int QUEUE>
__device__ __forceinline__ void split_body(const SplitParams &gp, const QueueCtl &q) {
    constexpr int EPI = HOLD ? SX_EPI_H : SX_EPI;   // energy threads
    constexpr int NA = HOLD ? 2 : 4;                // a values per energy thread
    constexpr int NB = HOLD ? 1 : 2;
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    float *X = (float *)smem;
    uint8_t *stages = smem + SX_NX * 4;
    uint8_t *misc = stages + SX_NS * SX_STAGE;
    uint64_t *bars = (uint64_t *)misc;
    uint64_t *full = bars, *empty = bars + SX_NS, *tfull = bars + 2 * SX_NS, *tempty = tfull + 2,
             *drain = tempty + 2, *xready = drain + 1, *xfree = xready + 1, *ufull = xfree + 1,
             *uempty = ufull + SX_RING;  // 23 barriers: 184 bytes
    uint32_t *tslot = (uint32_t *)(misc + 192);
    volatile int *abort = (volatile int *)(misc + 196);
    volatile int *dr_ok = (volatile int *)(misc + 200);
    volatile int64_t *dr_unit = (volatile int64_t *)(misc + 208);
    volatile int64_t *en_unit = (volatile int64_t *)(misc + 216);
    int *dr_nk = (int *)(misc + 224);              // [9] kept K chunks per term of the drained item
    volatile int *dr_kseg = (volatile int *)(misc + 264);  // K chunks per drain of the drained item's job
    volatile int *en_buf = (volatile int *)(misc + 268);   // register hold: accumulator of the last term's
    volatile int *en_add = (volatile int *)(misc + 272);   // last segment, and whether it holds a product
    int *errp = QUEUE ? q.err : gp.err;
    EDesc *desc = (EDesc *)(misc + 320);
    double *red = (double *)(misc + 512);          // [16 energy warps at most][2]
    const UnitRing ring{(int64_t *)(misc + 768), ufull, uempty};
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    constexpr int KE = TYPE == TM_F32 ? 8 : 16;

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
        for (int s = 0; s < SX_RING; ++s) {
            tc::mbar_init(&ufull[s], 1);
            tc::mbar_init(&uempty[s], 3);  // MMA thread, drain leader, energy leader
        }
        *abort = 0;
        *dr_ok = 1;
        tc::fence_mbar_init();
    }
    if (warp == 1) tc::tmem_alloc(tslot, 512);
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    const uint32_t tmem = *tslot;

    if (warp < 4) {
        asm volatile("setmaxnreg.dec.sync.aligned.u32 %0;" ::"n"(SX_REG_LOW));
        if (warp == 0 && lane == 0)
            run_producer<TYPE, QUEUE>(gp, q, stages, full, empty, abort, ring);
        else if (warp == 1 && lane == 0)
            run_mma<TYPE, NB, QUEUE>(gp, q, stages, full, empty, tfull, tempty, drain, tmem, abort, ring);
    } else if (warp < 8) {
        // ---------------- drain warps ----------------
        asm volatile("setmaxnreg.dec.sync.aligned.u32 %0;" ::"n"(HOLD ? SX_REG_DRAIN_H : SX_REG_DRAIN));
        const int quad = warp & 3;
        const int m = quad * 32 + lane;  // TMEM lane = GEMM row
        const bool leader = (warp == 4 && lane == 0);
        const uint32_t tq = tmem + ((uint32_t)(quad * 32) << 16);
        uint32_t sg = 0;
        bool ok = true;
        for (int n = 0; ok; ++n) {
            if (leader) {
                const int64_t unit = ring_take(ring, n, abort);
                if (unit >= 0) {
                    SplitParams lp;
                    if (QUEUE) load_job(q, (int)(unit >> kSlotShift), lp);
                    const SplitParams &p = QUEUE ? lp : gp;
                    ItemBox bx;
                    decode_item(p, QUEUE ? (unit & kItemMask) : unit, bx);
                    for (int t = 0; t < 9; ++t) dr_nk[t] = term_chunk_count<KE>(p, bx, t);
                    *dr_kseg = p.kseg;
                }
                *dr_unit = unit;
            }
            named_bar(1, SX_DRAIN);
            const int64_t si = *dr_unit;
            if (si < 0) {
                ok = si == -1;
                break;
            }
            for (int t = 0; t < 9 && ok; ++t) {
                const int nk = dr_nk[t];
                int kseg;
                const int nseg = term_segments(nk, *dr_kseg, kseg);
                for (int sgi = 0; sgi < nseg; ++sgi, ++sg) {
                    const int buf = sg % NB;
                    const bool first = (t == 0 && sgi == 0);
                    const bool last = (t == 8 && sgi == nseg - 1);
                    if (!HOLD && last) {
                        // register hold: the energy warps add the last segment to their copy
                        // of the sub-box themselves (its rows and columns are theirs), so
                        // the sub-box is ready once the segments before it are drained
                        if (leader) tc::mbar_arrive(xready);
                        continue;
                    }
                    if (leader) {
                        bool w = tc::mbar_wait(&tfull[buf], (sg / NB) & 1, kWaitNs, abort);
                        // registers hold: the previous item's values must have left the sub-box;
                        // tensor-memory hold: they must have left the hold columns
                        if (w && n > 0 && (HOLD ? last : first)) w = tc::mbar_wait(xfree, (n - 1) & 1, kWaitNs, abort);
                        *dr_ok = w ? 1 : 0;
                    }
                    named_bar(1, SX_DRAIN);
                    if (!*dr_ok) {
                        ok = false;
                        break;
                    }
                    tc::tc_fence_after();
                    if (HOLD && last) {
                        if (nk > 0) {
                            drain_hold(X, tq + (uint32_t)(buf * 256), tq + 256u, m);
                        } else {  // no kept K chunk in the last term: the sub-box as it is
                            float z[32];
#pragma unroll
                            for (int q = 0; q < 32; ++q) z[q] = 0.0f;
                            const int bb = m >> 4, ii = (m >> 2) & 3, jj = m & 3;
                            for (int cc = 0; cc < 8; ++cc) {
#pragma unroll
                                for (int q = 0; q < 32; ++q) z[q] = X[xaddr(cc, bb, q >> 2, ii, jj, q & 3)];
                                tc::tmem_st32(tq + 256u + (uint32_t)(cc * 32), z);
                            }
                        }
                    } else if (nk > 0) {
                        drain_any(t, first, X, tq + (uint32_t)(buf * 256), m);
                    } else if (first) {  // no kept K chunk in the first term: start from zero
                        for (int e = m * 256; e < m * 256 + 256; ++e) X[e] = 0.0f;
                    }
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
            atomicCAS(errp, 0, 3);
        }
    } else {
        // ---------------- energy warps ----------------
        asm volatile("setmaxnreg.inc.sync.aligned.u32 %0;" ::"n"(HOLD ? SX_REG_HIGH_H : SX_REG_HIGH));
        const int et = threadIdx.x - 256;
        const int mm = et & 127, half = et >> 7;  // half: the part of the a range (a = NA*half + A)
        const int rb = mm >> 4, ri = (mm >> 2) & 3, rj_ = mm & 3;  // thread row (b;i,j)
        const bool leader = (et == 0);
        float R[HOLD ? 1 : 128];
        constexpr int NQ = HOLD ? 1 : 2;  // quarter partials per thread
        double e1[NQ], est[NQ];
#pragma unroll
        for (int x = 0; x < NQ; ++x) e1[x] = est[x] = 0.0;
        const int quarter0 = HOLD ? half : 2 * half;
        int slot = 0;            // queue mode, leader: the current item's job slot and item count
        int64_t job_items = 0;
        uint32_t en_sg = 0;      // register hold, leader: accumulator segments of the items so far
        for (int n = 0;; ++n) {
            if (leader) {
                int64_t si = ring_take(ring, n, abort);
                bool w = si != -2;
                if (si >= 0) {
                    w = tc::mbar_wait(xready, n & 1, kWaitNs, abort);
                    if (w) {
                        SplitParams lp;
                        if (QUEUE) {
                            slot = (int)(si >> kSlotShift);
                            load_job(q, slot, lp);
                        }
                        const SplitParams &p = QUEUE ? lp : gp;
                        job_items = p.n_items;
                        ItemBox bx;
                        decode_item(p, QUEUE ? (si & kItemMask) : si, bx);
#pragma unroll
                        for (int dd = 0; dd < 6; ++dd) {
                            desc->g[dd] = bx.start[dd] + bx.boff[dd];
                            desc->nv[dd] = min(dd < 3 ? SX_BV : SX_BO, bx.ext[dd] - bx.boff[dd]);
                            desc->gp[dd] = dd < 3 ? 0 : 4 * __ldg(p.tile_box + bx.tile[dd] - 1) + bx.boff[dd];
                        }
                        desc->factor = p.factor[bx.tq];
                        desc->item = bx.item;
                        desc->op = p.op;
                        desc->T1f = p.T1f;
                        desc->Uf = p.Uf;
                        desc->eo = p.evf;
                        desc->ev = p.evf + p.nocc;
                        desc->part = p.part;
                        desc->inv_s = p.inv_s;
                        desc->inv_s2 = p.inv_s2;
                        desc->nvir = p.nvir;
                        if constexpr (!HOLD) {
                            // the item's segments in the MMA's order; the last one (term 8)
                            // is added here, not by the drains
                            uint32_t nsg = 0;
                            int nk8 = 0;
                            for (int t = 0; t < 9; ++t) {
                                const int nk = term_chunk_count<KE>(p, bx, t);
                                int kseg;
                                nsg += (uint32_t)term_segments(nk, p.kseg, kseg);
                                if (t == 8) nk8 = nk;
                            }
                            const uint32_t sgl = en_sg + nsg - 1;
                            en_sg += nsg;
                            w = tc::mbar_wait(&tfull[sgl % NB], (sgl / NB) & 1, kWaitNs, abort);
                            *en_buf = (int)(sgl % NB);
                            *en_add = nk8 > 0 ? 1 : 0;
                        }
                    }
                }
                if (!w) {
                    *abort = 1;
                    atomicCAS(errp, 0, 4);
                    si = -2;
                }
                *en_unit = si;
            }
            named_bar(2, EPI);
            if (*en_unit < 0) break;
            const EDesc &d = *desc;
            if constexpr (HOLD) {
                // the sub-box is in the hold columns: this warp's lane quadrant, columns 32*(NA*half + A)
                tc::tc_fence_after();
                const uint32_t th = tmem + ((uint32_t)((warp & 3) * 32) << 16) + 256u + (uint32_t)(32 * NA * half);
                if (d.item >= 0) energy_tmem<NA>(th, d, half, rb, ri, rj_, e1[0], est[0]);
                tc::tc_fence_before();
                named_bar(2, EPI);
                if (leader) tc::mbar_arrive(xfree);  // the hold columns are free
                if (d.item >= 0) write_partial<EPI, NQ>(e1, est, red, d, quarter0, warp & 3, lane, leader);
                if (QUEUE && leader) job_item_done(q, slot, job_items);
            } else {
#pragma unroll
                for (int A = 0; A < 4; ++A)
#pragma unroll
                    for (int c = 0; c < 8; ++c)
#pragma unroll
                        for (int k = 0; k < 4; ++k) R[A * 32 + c * 4 + k] = X[xaddr(4 * half + A, rb, c, ri, rj_, k)];
                // the last term (rows (b;i,j), columns (a,c;k), sign +1): this thread's row,
                // columns 128*half .. +127 of the accumulator
                tc::tc_fence_after();
                if (*en_add) {
                    const uint32_t ta = tmem + ((uint32_t)((warp & 3) * 32) << 16) + (uint32_t)(*en_buf * 256 + 128 * half);
#pragma unroll
                    for (int h = 0; h < 8; ++h) {
                        float v[16];
                        tc::tmem_ld16(ta + (uint32_t)(16 * h), v);
#pragma unroll
                        for (int q = 0; q < 16; ++q) R[16 * h + q] += v[q];
                    }
                }
                tc::tc_fence_before();
                named_bar(2, EPI);
                if (leader) {
                    tc::mbar_arrive(&tempty[*en_buf]);
                    tc::mbar_arrive(xfree);
                }
                if (d.item >= 0) {  // a box outside the tuple has no item
                    energy_chunk<0, 0, 128>(R, d, half, rb, ri, rj_, e1[0], est[0]);
                    energy_chunk<1, 32, 128>(R, d, half, rb, ri, rj_, e1[0], est[0]);
                    energy_chunk<2, 64, 128>(R, d, half, rb, ri, rj_, e1[NQ - 1], est[NQ - 1]);
                    energy_chunk<3, 96, 128>(R, d, half, rb, ri, rj_, e1[NQ - 1], est[NQ - 1]);
                    write_partial<EPI, NQ>(e1, est, red, d, quarter0, warp & 3, lane, leader);
                    if (QUEUE && leader) job_item_done(q, slot, job_items);
                }
            }
        }
    }
    tc::tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc::tc_fence_after();
        tc::tmem_dealloc(tmem, 512);
    }
}

// One job's items (a plan group).
template <int TYPE, int HOLD>
__global__ void __launch_bounds__(HOLD ? SX_THREADS_H : SX_THREADS, 1)
    split_fused_kernel(const __grid_constant__ SplitParams p) {
    const QueueCtl none{};
    split_body<TYPE, HOLD, 0>(p, none);
}

// The shared queue of several jobs' items (serving): resident until the
// queue stays empty for idle_ns or close is set.
template <int TYPE, int HOLD>
__global__ void __launch_bounds__(HOLD ? SX_THREADS_H : SX_THREADS, 1)
    split_queue_kernel(const __grid_constant__ QueueCtl q) {
    split_body<TYPE, HOLD, 1>(q.table[0], q);
}

// ---------------------------------------------------------------------------
// Operand preparation.

struct PackArgs {
    const double *src;
    uint8_t *hi, *lo;
    int64_t nblocks;
    int layout, nk, ke, es;       // L_*, K chunks, K values per 32-byte row, bytes per value
    int64_t o, v;
    int nob, nvb;
    const int32_t *vrow0, *vn;    // [nvb] first particle index and valid rows of each box
    const int32_t *orow0, *on;    // [nob] the same for hole boxes
    const int64_t *pblk0;         // Vd2: [npairs+1] first block of each tile pair, then the total
    const int64_t *poff;          // Vd2: [npairs] FP64 offset of the pair's region
    const int32_t *pdim;          // Vd2: [npairs][3] rB, rC, boxes of C
    int npairs;
    double scale;
};

// One thread per value of the block-major layout: gathers the FP64 source
// (zero outside the tiles and past K), scales, splits into hi/lo of TYPE and
// stores both at the 32-byte-swizzled position of its row (16-byte halves
// swapped in rows with bit 2 set, the pattern of a 32-byte swizzled K-major
// shared-memory tile), hi in the block's first half and lo in its second
// (g.lo = g.hi + one half).
template <int TYPE>
__global__ void __launch_bounds__(256) pack_blocks_kernel(const PackArgs g) {
    const int rows = (g.layout == L_WD1 || g.layout == L_T2B) ? 128 : 256;
    const int64_t per_block = (int64_t)rows * g.ke;
    const int64_t total = g.nblocks * per_block;
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t blk = idx / per_block;
        const int rem = (int)(idx - blk * per_block);
        const int row = rem / g.ke, e = rem % g.ke;
        int64_t q = blk;
        const int kc = (int)(q % g.nk);
        q /= g.nk;
        const int kidx = kc * g.ke + e;
        double x = 0.0;
        if (g.layout == L_WD1 || g.layout == L_T2B) {
            const int h2 = (int)(q % g.nob);
            q /= g.nob;
            const int h1 = (int)(q % g.nob);
            const int xb = (int)(q / g.nob);
            const int r0 = row >> 4, r1 = (row >> 2) & 3, r2 = row & 3;
            const int64_t kext = g.layout == L_WD1 ? g.o : g.v;
            if (r0 < g.vn[xb] && r1 < g.on[h1] && r2 < g.on[h2] && kidx < kext) {
                const int64_t P = g.vrow0[xb] + r0, H = g.orow0[h1] + r1, L = g.orow0[h2] + r2;
                x = g.src[((P * g.o + H) * g.o + L) * kext + kidx];  // Wd1[c][j][k][m], T2b[p][h][l][e]
            }
        } else if (g.layout == L_T2A) {
            const int hb = (int)(q % g.nob);
            q /= g.nob;
            const int x1 = (int)(q % g.nvb);
            const int x0 = (int)(q / g.nvb);
            const int c0 = row >> 5, c1 = (row >> 2) & 7, c2 = row & 3;
            if (c0 < g.vn[x0] && c1 < g.vn[x1] && c2 < g.on[hb] && kidx < g.o) {
                const int64_t P = g.vrow0[x0] + c0, Q = g.vrow0[x1] + c1, H = g.orow0[hb] + c2;
                x = g.src[((P * g.v + Q) * g.o + H) * g.o + kidx];  // T2a[p][q][h][m]
            }
        } else {
            int lo = 0, hi = g.npairs - 1;
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (g.pblk0[mid] <= blk) lo = mid;
                else hi = mid - 1;
            }
            int64_t lq = blk - g.pblk0[lo];
            lq /= g.nk;
            const int hb = (int)(lq % g.nob);
            lq /= g.nob;
            const int rB = g.pdim[3 * lo], rC = g.pdim[3 * lo + 1], nbC = g.pdim[3 * lo + 2];
            const int l1 = (int)(lq % nbC), l0 = (int)(lq / nbC);
            const int c0 = row >> 5, c1 = (row >> 2) & 7, c2 = row & 3;
            const int bl = 8 * l0 + c0, cl = 8 * l1 + c1;
            if (bl < rB && cl < rC && c2 < g.on[hb] && kidx < g.v) {
                const int64_t K = g.orow0[hb] + c2;
                x = g.src[g.poff[lo] + (((int64_t)bl * rC + cl) * g.o + K) * g.v + kidx];  // region [b][c][k][e]
            }
        }
        x *= g.scale;
        const int eb = e * g.es;
        const int off = row * 32 + ((((eb >> 4) ^ (row >> 2)) & 1) << 4) + (eb & 15);
        const int64_t at = blk * (int64_t)rows * 64 + off;
        if (TYPE == TM_F32) {
            const float h = tc::to_tf32(__double2float_rn(x));
            *(float *)(g.hi + at) = h;
            *(float *)(g.lo + at) = tc::to_tf32(__double2float_rn(x - (double)h));
        } else if (TYPE == TM_BF16) {
            const __nv_bfloat16 h = __float2bfloat16_rn(__double2float_rn(x));
            *(__nv_bfloat16 *)(g.hi + at) = h;
            *(__nv_bfloat16 *)(g.lo + at) = __float2bfloat16_rn(__double2float_rn(x - (double)__bfloat162float(h)));
        } else {
            const __half h = __float2half_rn(__double2float_rn(x));
            *(__half *)(g.hi + at) = h;
            *(__half *)(g.lo + at) = __float2half_rn(__double2float_rn(x - (double)__half2float(h)));
        }
    }
}

// FP32 copy of rows of hole-indexed FP64 data with the trailing `nh` hole
// indices padded per tile (padded index = 4 x box id + local; padding 0):
// T1 [v][o] -> [v][OP] (nh = 1), the vvoo block [v][v][o][o] -> [v][v][OP][OP] (nh = 2).
__global__ void __launch_bounds__(256) pad_f32_kernel(const double *__restrict__ src, float *__restrict__ dst,
                                                      int64_t rows, int64_t o, int64_t op, int nh,
                                                      const int32_t *__restrict__ orow0,
                                                      const int32_t *__restrict__ on) {
    const int64_t per = nh == 1 ? op : op * op;
    const int64_t total = rows * per;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = i / per, rem = i % per;
        const int64_t hk = nh == 1 ? rem : rem % op, hj = nh == 1 ? 0 : rem / op;
        const int bk = (int)(hk >> 2), bj = (int)(hj >> 2);
        float x = 0.0f;
        if ((hk & 3) < on[bk] && (nh == 1 || (hj & 3) < on[bj])) {
            const int64_t k = orow0[bk] + (hk & 3);
            if (nh == 1) {
                x = __double2float_rn(src[r * o + k]);
            } else {
                const int64_t jj = orow0[bj] + (hj & 3);
                x = __double2float_rn(src[(r * o + jj) * o + k]);
            }
        }
        dst[i] = x;
    }
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
    gpu_put(j->tile_box_d);
    j->t1f = j->uf = nullptr;
    j->tile_box_d = nullptr;
    j->mixed_aux_n = 0;
    j->mixed_type = -1;
}

int mixed_prepare(sdt_job *j, int type, cudaStream_t st) {
    mixed_release(j);
    PhaseTrace tr("mixed_prepare");
    const Tiling &t = j->t;
    const int64_t o = t.nocc, v = t.nvir, noab = t.noab, nvab = t.nvab, nt = noab + nvab;
    const int es = type == TM_F32 ? 4 : 2;
    const int ke = 32 / es;  // K values per 32-byte row
    const int64_t nko = (o + ke - 1) / ke, nkv = (v + ke - 1) / ke;
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
    tr.mark("scales", st);
    j->inv_s = 1.0 / (sT * sI);
    j->inv_s2 = j->inv_s * j->inv_s;
    // Every K tile is allowed for every term when all tiles share one spin and one irrep.
    j->all_k = 1;
    for (int64_t b = 2; b <= nt; ++b)
        if (t.s(b) != t.s(1) || t.y(b) != t.y(1)) j->all_k = 0;
    // Box tables: global box ids per space, first index and valid rows.
    std::vector<int32_t> tile_box(nt), vrow0, vn, orow0, on;
    for (int64_t b = 1; b <= nt; ++b) {
        const bool virt = b > noab;
        const int bx = virt ? SX_BV : SX_BO;
        std::vector<int32_t> &row0 = virt ? vrow0 : orow0, &nvalid = virt ? vn : on;
        tile_box[b - 1] = (int32_t)row0.size();
        for (int64_t s0 = 0; s0 < t.r(b); s0 += bx) {
            row0.push_back((int32_t)(t.start(b) + s0));
            nvalid.push_back((int32_t)std::min<int64_t>(bx, t.r(b) - s0));
        }
    }
    const int64_t NOB = (int64_t)orow0.size(), NVB = (int64_t)vrow0.size();
    j->nob = (int32_t)NOB;
    j->nvb = (int32_t)NVB;
    // Vd2 tile pairs (B <= C): first block, FP64 region offset, dims.
    std::vector<int64_t> pblk0, poff, pair_blk(nvab * nvab, -1);
    std::vector<int32_t> pdim;
    int64_t nvd2 = 0;
    for (int64_t B = noab + 1; B <= nt; ++B)
        for (int64_t C = B; C <= nt; ++C) {
            const int64_t off = j->pair_host[(B - noab - 1) * nvab + (C - noab - 1)];
            if (off < 0) continue;
            const int64_t nbB = (t.r(B) + SX_BV - 1) / SX_BV, nbC = (t.r(C) + SX_BV - 1) / SX_BV;
            pair_blk[(B - noab - 1) * nvab + (C - noab - 1)] = nvd2;
            pblk0.push_back(nvd2);
            poff.push_back(off);
            pdim.push_back((int32_t)t.r(B));
            pdim.push_back((int32_t)t.r(C));
            pdim.push_back((int32_t)nbC);
            nvd2 += nbB * nbC * NOB * nkv;
        }
    const int npairs = (int)poff.size();
    pblk0.push_back(nvd2);
    // Tables on the device (one buffer, 8-byte aligned parts).
    std::vector<int64_t> tab;
    auto put32 = [&](const std::vector<int32_t> &x) {
        const size_t at = tab.size();
        tab.resize(at + (x.size() + 1) / 2, 0);
        if (!x.empty()) std::memcpy(tab.data() + at, x.data(), x.size() * sizeof(int32_t));
        return at;
    };
    auto put64 = [&](const std::vector<int64_t> &x) {
        const size_t at = tab.size();
        tab.insert(tab.end(), x.begin(), x.end());
        return at;
    };
    const size_t o_vrow0 = put32(vrow0), o_vn = put32(vn), o_orow0 = put32(orow0), o_on = put32(on);
    const size_t o_pblk0 = put64(pblk0), o_poff = put64(poff), o_pdim = put32(pdim);
    const size_t o_tbox = put32(tile_box), o_pairblk = put64(pair_blk);
    int64_t *tab_d = (int64_t *)gpu_get(std::max<size_t>(tab.size(), 1) * sizeof(int64_t));
    if (!tab_d) {
        gpu_put(tab_d);
        mixed_release(j);
        return fail(SDT_ERR_NOMEM, "mixed form: tables");
    }
    j->tile_box_d = tab_d;  // owns the whole table buffer
    j->mixed_aux_n = std::max<size_t>(tab.size(), 1) * sizeof(int64_t);
    rc = cuda_check(cudaMemcpyAsync(tab_d, tab.data(), tab.size() * sizeof(int64_t), cudaMemcpyHostToDevice, st),
                    "mixed form: tables");
    j->tile_box_off = (int64_t)o_tbox;
    j->pair_blk_off = (int64_t)o_pairblk;
    tr.mark("tables", st);
    // Block-major split operands.
    const int64_t nblk[L_N] = {NVB * NOB * NOB * nko, NVB * NOB * NOB * nkv, NVB * NVB * NOB * nko, nvd2};
    const int srcidx[L_N] = {DST_WD1, DST_T2B, DST_T2A, DST_VD2};
    const double scale[L_N] = {sI, sT, sT, sI};
    for (int l = 0; l < L_N && !rc; ++l) {
        const int rows = l < L_T2A ? 128 : 256;
        const size_t bytes = (size_t)nblk[l] * rows * 32;
        j->sp[2 * l] = gpu_get(std::max<size_t>(2 * bytes, 16));
        if (!j->sp[2 * l]) {
            mixed_release(j);
            return fail(SDT_ERR_NOMEM, "mixed form: split operand allocation");
        }
        j->sp_n[2 * l] = 2 * bytes;
        if (nblk[l] == 0) continue;
        PackArgs g;
        g.src = j->arr[srcidx[l]];
        g.hi = (uint8_t *)j->sp[2 * l];
        g.lo = (uint8_t *)j->sp[2 * l] + rows * 32;
        g.nblocks = nblk[l];
        g.layout = l;
        g.nk = (l == L_WD1 || l == L_T2A) ? (int)nko : (int)nkv;
        g.ke = ke;
        g.es = es;
        g.o = o;
        g.v = v;
        g.nob = (int)NOB;
        g.nvb = (int)NVB;
        const int32_t *t32 = (const int32_t *)tab_d;
        g.vrow0 = t32 + 2 * o_vrow0;
        g.vn = t32 + 2 * o_vn;
        g.orow0 = t32 + 2 * o_orow0;
        g.on = t32 + 2 * o_on;
        g.pblk0 = tab_d + o_pblk0;
        g.poff = tab_d + o_poff;
        g.pdim = t32 + 2 * o_pdim;
        g.npairs = npairs;
        g.scale = scale[l];
        const unsigned gb = grid_for(nblk[l] * rows * ke);
        if (type == TM_F32) pack_blocks_kernel<TM_F32><<<gb, 256, 0, st>>>(g);
        else if (type == TM_BF16) pack_blocks_kernel<TM_BF16><<<gb, 256, 0, st>>>(g);
        else pack_blocks_kernel<TM_F16><<<gb, 256, 0, st>>>(g);
        count_launch();
    }
    tr.mark("pack", st);
    // FP32 copies of T1 [v][OP] and the vvoo block [v][v][OP][OP] for the s1
    // terms, holes padded per tile to multiples of 4; the T1 buffer also holds
    // the shifted FP32 orbital energies after the T1 copy (o + v values).
    const int64_t OP = 4 * NOB;
    const int64_t n_t1 = v * OP, n_u = v * v * OP * OP;
    if (!rc) {
        j->t1f = (float *)gpu_get((n_t1 + o + v) * sizeof(float));
        j->uf = (float *)gpu_get(std::max<int64_t>(n_u, 1) * sizeof(float));
        j->mixed_aux_n += (size_t)(n_t1 + o + v + std::max<int64_t>(n_u, 1)) * sizeof(float);
        if (!j->t1f || !j->uf) {
            mixed_release(j);
            return fail(SDT_ERR_NOMEM, "mixed form: FP32 copies");
        }
        const int32_t *t32 = (const int32_t *)tab_d;
        pad_f32_kernel<<<grid_for(n_t1), 256, 0, st>>>(j->arr[DST_T1], j->t1f, v, o, OP, 1, t32 + 2 * o_orow0,
                                                       t32 + 2 * o_on);
        count_launch();
        pad_f32_kernel<<<grid_for(n_u), 256, 0, st>>>(j->arr[DST_UD], j->uf, v * v, o, OP, 2, t32 + 2 * o_orow0,
                                                      t32 + 2 * o_on);
        count_launch();
        rc = cuda_check(cudaGetLastError(), "mixed form: split");
    }
    std::vector<float> evf(o + v);
    if (!rc) {
        // orbital energies minus the midpoint of the occupied-virtual gap: every
        // hole term of a denominator is then negative and every particle term
        // positive, so its FP32 sums do not cancel
        double emax = -1e300, emin = 1e300;
        for (int64_t x = 0; x < o; ++x) emax = std::max(emax, j->evl[x]);
        for (int64_t x = o; x < o + v; ++x) emin = std::min(emin, j->evl[x]);
        const double mu = (o > 0 && v > 0) ? 0.5 * (emax + emin) : 0.0;
        for (int64_t x = 0; x < o + v; ++x) evf[x] = (float)(j->evl[x] - mu);
        rc = cuda_check(cudaMemcpyAsync(j->t1f + n_t1, evf.data(), (o + v) * sizeof(float), cudaMemcpyHostToDevice, st),
                        "mixed form: orbital energies");
    }
    if (!rc) rc = cuda_check(cudaStreamSynchronize(st), "mixed form: prepare");
    tr.mark("fp32 copies", nullptr);
    if (rc) {
        mixed_release(j);
        return rc;
    }
    j->mixed_type = type;
    return SDT_OK;
}

int mixed_grid(sdt_job *j, int shape, int64_t n_items, int *grid) {
    auto setup = [&](auto kern) -> int {
        int r = cuda_check(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, SX_SMEM_ALLOC),
                           "mixed form: smem attribute");
        if (r) return r;
        int nsm = 0;
        r = cuda_check(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, j->dev), "mixed form");
        if (r) return r;
        if (j->max_ctas > 0) nsm = std::min(nsm, j->max_ctas);
        *grid = (int)std::max<int64_t>(1, std::min<int64_t>(nsm, n_items));
        return SDT_OK;
    };
    const int type = j->mixed_type;
    if (shape == 2) {
        if (type == TM_F32) return setup(split_fused_kernel<TM_F32, 1>);
        if (type == TM_BF16) return setup(split_fused_kernel<TM_BF16, 1>);
        return setup(split_fused_kernel<TM_F16, 1>);
    }
    if (type == TM_F32) return setup(split_fused_kernel<TM_F32, 0>);
    if (type == TM_BF16) return setup(split_fused_kernel<TM_BF16, 0>);
    return setup(split_fused_kernel<TM_F16, 0>);
}

namespace {
SplitParams job_params(sdt_job *j, const LaunchArgs &a) {
    const Tiling &t = j->t;
    const int ke = j->mixed_type == TM_F32 ? 8 : 16;
    SplitParams p{};
    for (int k = 0; k < 2 * L_N; ++k) p.blk[k] = (const uint8_t *)j->sp[k];
    p.tile_box = (const int32_t *)(j->tile_box_d + j->tile_box_off);
    p.pair_blk = j->tile_box_d + j->pair_blk_off;
    p.T1f = j->t1f;
    p.Uf = j->uf;
    p.op = 4 * j->nob;
    p.evl = j->evl_d;
    p.evf = j->t1f + (int64_t)t.nvir * 4 * j->nob;
    p.tiles = j->tiles;
    p.noab = (int32_t)t.noab;
    p.nvab = (int32_t)t.nvab;
    p.nocc = t.nocc;
    p.nvir = t.nvir;
    p.nk_o = (int32_t)((t.nocc + ke - 1) / ke);
    p.nk_v = (int32_t)((t.nvir + ke - 1) / ke);
    p.nob = j->nob;
    p.nvb = j->nvb;
    p.kseg = j->mixed_kseg;
    p.klist = a.klist;
    p.item_pref = a.item_pref;
    p.factor = a.factor;
    p.n_tasks = a.n;
    p.n_items = a.items;
    p.inv_s = j->inv_s;
    p.inv_s2 = j->inv_s2;
    p.part = a.part;
    p.err = a.err;
    p.queue = a.queue;
    p.all_k = j->all_k;
    return p;
}
}  // namespace

int mixed_launch(sdt_job *j, const LaunchArgs &a, cudaStream_t st) {
    const int type = j->mixed_type;
    const SplitParams p = job_params(j, a);
    const int threads = a.shape == 2 ? SX_THREADS_H : SX_THREADS;
    auto launch = [&](auto kern) -> int {
        kern<<<(unsigned)a.grid, threads, SX_SMEM_ALLOC, st>>>(p);
        count_launch();
        return cuda_check(cudaGetLastError(), "mixed form: fused kernel");
    };
    int rc = cuda_check(cudaMemsetAsync(a.queue, 0, sizeof(unsigned long long), st), "mixed form");
    if (rc) return rc;
    if (a.shape == 2) {
        if (type == TM_F32) rc = launch(split_fused_kernel<TM_F32, 1>);
        else if (type == TM_BF16) rc = launch(split_fused_kernel<TM_BF16, 1>);
        else rc = launch(split_fused_kernel<TM_F16, 1>);
    } else {
        if (type == TM_F32) rc = launch(split_fused_kernel<TM_F32, 0>);
        else if (type == TM_BF16) rc = launch(split_fused_kernel<TM_BF16, 0>);
        else rc = launch(split_fused_kernel<TM_F16, 0>);
    }
    return rc;
}

size_t mixed_job_entry_bytes() { return sizeof(SplitParams); }

int mixed_job_entry(sdt_job *j, const LaunchArgs &a, void *entry) {
    if (j->mixed_type < 0) return fail(SDT_ERR_STATE, "mixed form: the job's split operands are not prepared");
    const SplitParams p = job_params(j, a);
    std::memcpy(entry, &p, sizeof(p));
    return SDT_OK;
}

int mixed_queue_prepare(int type, int shape) {
    auto setup = [](auto kern) {
        return cuda_check(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, SX_SMEM_ALLOC),
                          "mixed form: queue kernel smem attribute");
    };
    if (shape == 2) {
        if (type == TM_F32) return setup(split_queue_kernel<TM_F32, 1>);
        if (type == TM_BF16) return setup(split_queue_kernel<TM_BF16, 1>);
        return setup(split_queue_kernel<TM_F16, 1>);
    }
    if (type == TM_F32) return setup(split_queue_kernel<TM_F32, 0>);
    if (type == TM_BF16) return setup(split_queue_kernel<TM_BF16, 0>);
    return setup(split_queue_kernel<TM_F16, 0>);
}

int mixed_queue_launch(int type, int shape, const QueueArgs &a, int grid, cudaStream_t st) {
    QueueCtl q;
    q.table = (const SplitParams *)a.table;
    q.base = a.base;
    q.head = a.head;
    q.tail = a.tail;
    q.done = a.done;
    q.first_gen = a.first_gen;
    q.last_gen = a.last_gen;
    q.close = a.close;
    q.err = a.err;
    q.idle_ns = std::min<unsigned long long>(a.idle_ns, kWaitNs / 2);  // below the roles' own wait limit
    q.max_jobs = a.max_jobs;
    q.gen = a.gen;
    const int threads = shape == 2 ? SX_THREADS_H : SX_THREADS;
    auto launch = [&](auto kern) -> int {
        kern<<<(unsigned)grid, threads, SX_SMEM_ALLOC, st>>>(q);
        count_launch();
        return cuda_check(cudaGetLastError(), "mixed form: queue kernel");
    };
    if (shape == 2) {
        if (type == TM_F32) return launch(split_queue_kernel<TM_F32, 1>);
        if (type == TM_BF16) return launch(split_queue_kernel<TM_BF16, 1>);
        return launch(split_queue_kernel<TM_F16, 1>);
    }
    if (type == TM_F32) return launch(split_queue_kernel<TM_F32, 0>);
    if (type == TM_BF16) return launch(split_queue_kernel<TM_BF16, 0>);
    return launch(split_queue_kernel<TM_F16, 0>);
}

}  // namespace sdt
