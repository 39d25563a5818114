// sdt_fused.cu -- batched (T): device ingest of the TCE files and the fused
// FP64 tuple kernel.
//
// The reference evaluates one tuple (p4b<=p5b<=p6b, h1b<=h2b<=h3b) as 9 s1,
// 9 d1 (per h7b) and 9 d2 (per p7b) kernel calls into two Nt-sized device
// tiles, then a separate energy kernel (src/tce/ccsd_t/ccsd_t_gpu.F:87-241,
// sd_t_total.cu).  Here one CTA owns a 4x4x4x4x4x4 sub-box of one tuple's
// triples tile.  It accumulates all 18 d1/d2 contractions into that sub-box
// in shared memory with FP64 tensor-core MMAs (mma.sync m8n8k4.f64), adds
// the 9 s1 products and the orbital-energy denominator in the epilogue and
// writes one (E[T], E(T)) pair.  The triples tile never reaches HBM.
//
// In tuple coordinates (a,b,c in tiles p4b,p5b,p6b; i,j,k in h1b,h2b,h3b;
// t = T2, w = <h7 p6||h2 h3>, v = <p5 p6||h3 p7>, u = <p5 p6||h2 h3>, and
// t(p,q;h,l) read with the antisymmetry signs of tce_hashnsort.F) the
// 27 reference kernels (ccsd_t_kernels_omp.F) add up to:
//   d1:  -t(ab;im)w(mcjk) +t(ab;jm)w(mcik) -t(ab;km)w(mcij)
//        -t(bc;im)w(majk) +t(bc;jm)w(maik) -t(bc;km)w(maij)
//        +t(ac;im)w(mbjk) -t(ac;jm)w(mbik) +t(ac;km)w(mbij)     (sum over m)
//   d2:  -t(ae;ij)v(bcke) -t(ae;jk)v(bcie) +t(ae;ik)v(bcje)
//        +t(be;ij)v(acke) +t(be;jk)v(acie) -t(be;ik)v(acje)
//        -t(ce;ij)v(abke) -t(ce;jk)v(abie) +t(ce;ik)v(abje)     (sum over e)
//   s1:  +t1(ai)u(bcjk) -t1(aj)u(bcik) +t1(ak)u(bcij)
//        -t1(bi)u(acjk) +t1(bj)u(acik) -t1(bk)u(acij)
//        +t1(ci)u(abjk) -t1(cj)u(abik) +t1(ck)u(abij)
// (row k of each block is kernel k of its family, in order).
#include "sdt_common.cuh"
#include "sdt_job.h"

#include <algorithm>
#include <cstring>
#include <vector>

#include <unistd.h>

namespace sdt {
namespace {

// ---------------------------------------------------------------------------
// Dense device layouts (global orbital indices within each space):
//   T1d[a][i]                      v x o
//   T2a[p][q][h][l]                v x v x o x o   (d1 operand, l = summed m)
//   T2b[p][h][l][q]                v x o x o x v   (d2 operand, q = summed e)
//   Wd1[c][j][k][m]                v x o x o x o   (<m c||j k>, m fastest)
//   Vd2 per virtual tile pair B<=C: [b][c][k][e] with b,c tile-local
//   Ud[b][c][j][k]                 v x v x o x o   (<b c||j k>)
// Entries the path never reads (non-canonical orders of V2) stay zero, as
// do blocks that spin or irrep forbid.
// ---------------------------------------------------------------------------
struct CopyJob {
    int64_t src;          // offset of the 3-D slab in the raw file
    int64_t dst;          // element offset in the destination array
    int64_t n1, n2, n3;   // slab dims (key order, last fastest)
    int64_t s1, s2, s3;   // destination strides of those dims
    double sign;
    int32_t src_file;     // 0 T1, 1 T2, 2 V2
    int32_t dst_array;    // index into the destination table
};

struct IngestArgs {
    const double *src[3];
    double *dst[DST_N];
    const CopyJob *jobs;
};

__global__ void __launch_bounds__(256) ingest_kernel(const IngestArgs g) {
    const CopyJob j = g.jobs[blockIdx.x];
    const double *__restrict__ s = g.src[j.src_file] + j.src;
    double *__restrict__ d = g.dst[j.dst_array] + j.dst;
    const int64_t n = j.n1 * j.n2 * j.n3;
    for (int64_t e = threadIdx.x; e < n; e += blockDim.x) {
        const int64_t x3 = e % j.n3, t = e / j.n3;
        const int64_t x2 = t % j.n2, x1 = t / j.n2;
        d[x1 * j.s1 + x2 * j.s2 + x3 * j.s3] = j.sign * s[e];
    }
}

// ---------------------------------------------------------------------------
// Fused tuple kernel.
// ---------------------------------------------------------------------------
constexpr int BOX = 4;          // sub-box edge in every index
constexpr int NX = 4096;        // BOX^6
constexpr int kThreads = 128;   // 4 warps, 2x2 over the 64x64 term GEMM
constexpr int kMaxTiles = 256;

// Term table: row dims (r) and column dims (c) of the 64x64 GEMM, sign.
// Dims: 0=a 1=b 2=c 3=i 4=j 5=k.
struct TermDef {
    int8_t r[3], c[3];
    int8_t sign;
};
// d1: rows (P,P',H) of t(P,P';H,m); cols (Q,H',H'') of w(m,Q,H',H'').
__constant__ TermDef kD1[9] = {
    {{0, 1, 3}, {2, 4, 5}, -1}, {{0, 1, 4}, {2, 3, 5}, +1}, {{0, 1, 5}, {2, 3, 4}, -1},
    {{1, 2, 3}, {0, 4, 5}, -1}, {{1, 2, 4}, {0, 3, 5}, +1}, {{1, 2, 5}, {0, 3, 4}, -1},
    {{0, 2, 3}, {1, 4, 5}, +1}, {{0, 2, 4}, {1, 3, 5}, -1}, {{0, 2, 5}, {1, 3, 4}, +1}};
// d2: rows (P,H,H') of t(P,e;H,H'); cols (Q,Q',H'') of v(Q,Q',H'',e).
__constant__ TermDef kD2[9] = {
    {{0, 3, 4}, {1, 2, 5}, -1}, {{0, 4, 5}, {1, 2, 3}, -1}, {{0, 3, 5}, {1, 2, 4}, +1},
    {{1, 3, 4}, {0, 2, 5}, +1}, {{1, 4, 5}, {0, 2, 3}, +1}, {{1, 3, 5}, {0, 2, 4}, -1},
    {{2, 3, 4}, {0, 1, 5}, -1}, {{2, 4, 5}, {0, 1, 3}, -1}, {{2, 3, 5}, {0, 1, 4}, +1}};

struct FusedParams {
    const double *T1d, *T2a, *T2b, *Vd2, *Wd1, *Ud;
    const int64_t *pair_off;  // [nvab*nvab], virtual tile pair -> Vd2 region
    const double *evl;        // occupied then virtual
    const int32_t *tiles;     // [ntiles][4] = start in space, range, spin, sym
    int32_t noab, nvab;
    int64_t nocc, nvir;
    const int64_t *klist;     // [n][7]
    const int64_t *item_pref; // [n+1]
    const double *factor;     // [n]
    int64_t n_tasks, n_items;
    double *part;             // [items][2]
    unsigned long long *queue;  // work-item counter, zero at launch
};

struct TupleCtx {
    int32_t tile[6];
    int32_t ext[6];
    int32_t start[6];
    int32_t boff[6];
};

__device__ __forceinline__ int stride6(int d) { return 1 << (2 * (5 - d)); }

// One d1 (kind 1) or d2 (kind 2) term accumulated into X.
__device__ __forceinline__ void run_term(const FusedParams &p, const TupleCtx &t,
                                      const int32_t (*__restrict__ st)[4],
                                      double *__restrict__ X, int kind, int term) {
    const TermDef td = kind == 1 ? kD1[term] : kD2[term];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int r = lane >> 2, q = lane & 3;
    const int wm = warp >> 1, wn = warp & 1;

    // Order of the three row (column) indices inside the 64 GEMM rows: the
    // one with the fewest valid values in this sub-box is outermost, so the
    // rows past its extent are whole 16-row groups -- whole fragments, which
    // are skipped (a ragged tile's last sub-box costs what it holds).
    // lev_r[p]: level (0 outermost) of row index p of the term.
    const int nr0 = min(BOX, t.ext[td.r[0]] - t.boff[td.r[0]]), nr1 = min(BOX, t.ext[td.r[1]] - t.boff[td.r[1]]),
              nr2 = min(BOX, t.ext[td.r[2]] - t.boff[td.r[2]]);
    const int nc0 = min(BOX, t.ext[td.c[0]] - t.boff[td.c[0]]), nc1 = min(BOX, t.ext[td.c[1]] - t.boff[td.c[1]]),
              nc2 = min(BOX, t.ext[td.c[2]] - t.boff[td.c[2]]);
    const int orow = nr1 < nr0 ? (nr2 < nr1 ? 2 : 1) : (nr2 < nr0 ? 2 : 0);
    const int ocol = nc1 < nc0 ? (nc2 < nc1 ? 2 : 1) : (nc2 < nc0 ? 2 : 0);
    const int rlive = orow == 0 ? nr0 : orow == 1 ? nr1 : nr2;
    const int clive = ocol == 0 ? nc0 : ocol == 1 ? nc1 : nc2;
    int lev_r[3], lev_c[3];
#pragma unroll
    for (int e = 0; e < 3; ++e) {
        lev_r[e] = e == orow ? 0 : (e < orow ? e + 1 : e);
        lev_c[e] = e == ocol ? 0 : (e < ocol ? e + 1 : e);
    }
    auto lat = [](int lev, int m) { return lev == 0 ? (m >> 4) : lev == 1 ? ((m >> 2) & 3) : (m & 3); };
    // live fragments: row fragment i of this warp holds level-0 value 2*wm + i/2
    unsigned rfrag = 0, cfrag = 0;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        rfrag |= (2 * wm + (i >> 1) < rlive) ? (1u << i) : 0u;
        cfrag |= (2 * wn + (i >> 1) < clive) ? (1u << i) : 0u;
    }

    int64_t abase[4], bbase[4];
    unsigned aok = 0, bok = 0;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int m = wm * 32 + i * 8 + r;
        const int x0 = t.boff[td.r[0]] + lat(lev_r[0], m), x1 = t.boff[td.r[1]] + lat(lev_r[1], m),
                  x2 = t.boff[td.r[2]] + lat(lev_r[2], m);
        const bool ok = x0 < t.ext[td.r[0]] && x1 < t.ext[td.r[1]] && x2 < t.ext[td.r[2]];
        aok |= ok ? (1u << i) : 0u;
        const int64_t g0 = t.start[td.r[0]] + x0, g1 = t.start[td.r[1]] + x1,
                      g2 = t.start[td.r[2]] + x2;
        abase[i] = ok ? (kind == 1 ? ((g0 * p.nvir + g1) * p.nocc + g2) * p.nocc
                                   : ((g0 * p.nocc + g1) * p.nocc + g2) * p.nvir)
                      : 0;
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int n = wn * 32 + j * 8 + r;
        const int x0 = t.boff[td.c[0]] + lat(lev_c[0], n), x1 = t.boff[td.c[1]] + lat(lev_c[1], n),
                  x2 = t.boff[td.c[2]] + lat(lev_c[2], n);
        const bool ok = x0 < t.ext[td.c[0]] && x1 < t.ext[td.c[1]] && x2 < t.ext[td.c[2]];
        bok |= ok ? (1u << j) : 0u;
        const int64_t g0 = t.start[td.c[0]] + x0, g2 = t.start[td.c[2]] + x2;
        int64_t b;
        if (kind == 1) {
            const int64_t g1 = t.start[td.c[1]] + x1;
            b = ((g0 * p.nocc + g1) * p.nocc + g2) * p.nocc;
        } else {
            const int64_t pr = (int64_t)(t.tile[td.c[0]] - p.noab - 1) * p.nvab +
                               (t.tile[td.c[1]] - p.noab - 1);
            b = p.pair_off[pr] + (((int64_t)x0 * t.ext[td.c[1]] + x1) * p.nocc + g2) * p.nvir;
        }
        bbase[j] = ok ? b : 0;
    }

    double acc[4][4][2];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j][0] = acc[i][j][1] = 0.0;

    const double *__restrict__ A = kind == 1 ? p.T2a : p.T2b;
    const double *__restrict__ B = kind == 1 ? p.Wd1 : p.Vd2;
    // Allowed summed tiles: the T2 quad read must balance spin and irrep
    // (tce_hashnsort.F:31-36 for d1, :107-111 for d2).
    const int tP = t.tile[td.r[0]], tX = t.tile[td.r[1]], tY = t.tile[td.r[2]];
    const int sP = st[tP - 1][2], sX = st[tX - 1][2], sY = st[tY - 1][2];
    const int yP = st[tP - 1][3], yX = st[tX - 1][3], yY = st[tY - 1][3];
    const int first = kind == 1 ? 1 : p.noab + 1;
    const int last = kind == 1 ? p.noab : p.noab + p.nvab;
    int kt = first;
    while (kt <= last) {
        // Merge a run of consecutive allowed tiles into one K range.
        auto allowed = [&](int e) {
            const int se = st[e - 1][2], ye = st[e - 1][3];
            return kind == 1 ? (sP + sX == sY + se && (yP ^ yX ^ yY ^ ye) == 0)
                             : (sP + se == sX + sY && (yP ^ ye ^ yX ^ yY) == 0);
        };
        if (!allowed(kt)) {
            ++kt;
            continue;
        }
        const int64_t k_begin = st[kt - 1][0];
        int64_t k_end = k_begin + st[kt - 1][1];
        ++kt;
        while (kt <= last && allowed(kt)) {
            k_end += st[kt - 1][1];
            ++kt;
        }
        for (int64_t k0 = k_begin; k0 < k_end; k0 += 4) {
            const int64_t k = k0 + q;
            const bool kok = k < k_end;
            double a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                a[i] = (kok && (aok >> i & 1u)) ? __ldg(A + abase[i] + k) : 0.0;
                b[i] = (kok && (bok >> i & 1u)) ? __ldg(B + bbase[i] + k) : 0.0;
            }
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j)
                    if ((rfrag >> i & 1u) && (cfrag >> j & 1u))  // warp-uniform
                        dmma_8x8x4(acc[i][j][0], acc[i][j][1], a[i], b[j]);
        }
    }

    // Scatter the 64x64 result into the sub-box (a bijection, no conflicts).
    const double sign = (double)td.sign;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        if (!(aok >> i & 1u)) continue;
        const int m = wm * 32 + i * 8 + r;
        const int roff = lat(lev_r[0], m) * stride6(td.r[0]) + lat(lev_r[1], m) * stride6(td.r[1]) +
                         lat(lev_r[2], m) * stride6(td.r[2]);
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int n = wn * 32 + j * 8 + 2 * q + h;
                const int l0 = lat(lev_c[0], n), l1 = lat(lev_c[1], n), l2 = lat(lev_c[2], n);
                if (t.boff[td.c[0]] + l0 >= t.ext[td.c[0]] || t.boff[td.c[1]] + l1 >= t.ext[td.c[1]] ||
                    t.boff[td.c[2]] + l2 >= t.ext[td.c[2]])
                    continue;
                const int off = roff + l0 * stride6(td.c[0]) + l1 * stride6(td.c[1]) +
                                l2 * stride6(td.c[2]);
                X[off] += sign * acc[i][j][h];
            }
    }
    __syncthreads();
}

// Persistent: each CTA draws sub-boxes from the device queue until it is
// empty.  A sub-box's pair depends only on its index, not on the CTA.
__global__ void __launch_bounds__(kThreads, 4) fused_fp64_kernel(const FusedParams p) {
    __shared__ double X[NX];
    __shared__ int32_t st[kMaxTiles][4];
    __shared__ double red[2][kThreads / 32];
    __shared__ long long s_item;

    const int ntiles = p.noab + p.nvab;
    for (int e = threadIdx.x; e < ntiles * 4; e += kThreads) st[e >> 2][e & 3] = p.tiles[e];
    for (;;) {
    if (threadIdx.x == 0) s_item = (long long)atomicAdd(p.queue, 1ull);
    for (int e = threadIdx.x; e < NX; e += kThreads) X[e] = 0.0;
    __syncthreads();
    const int64_t item = s_item;
    if (item >= p.n_items) break;
    // Tuple owning this item: last q with item_pref[q] <= item.
    int64_t lo = 0, hi = p.n_tasks - 1;
    while (lo < hi) {
        const int64_t mid = (lo + hi + 1) >> 1;
        if (p.item_pref[mid] <= item) lo = mid;
        else hi = mid - 1;
    }
    const int64_t tq = lo;
    int64_t local = item - p.item_pref[tq];

    TupleCtx t;
#pragma unroll
    for (int d = 0; d < 6; ++d) {
        t.tile[d] = (int32_t)p.klist[7 * tq + d];
        t.ext[d] = st[t.tile[d] - 1][1];
        t.start[d] = st[t.tile[d] - 1][0];
    }
#pragma unroll
    for (int d = 5; d >= 0; --d) {
        const int nb = (t.ext[d] + BOX - 1) / BOX;
        t.boff[d] = (int32_t)(local % nb) * BOX;
        local /= nb;
    }

#pragma unroll 1
    for (int term = 0; term < 18; ++term) run_term(p, t, st, X, term < 9 ? 1 : 2, term % 9);

    // Epilogue: s1 terms, denominator and the (E[T], E(T)) sums in FP64
    // (ccsd_t_dot.F:101-124).
    const double factor = p.factor[tq];
    const double *__restrict__ eo = p.evl;
    const double *__restrict__ ev = p.evl + p.nocc;
    const int64_t v = p.nvir, o = p.nocc;
    double s1 = 0.0, s2 = 0.0;
    for (int e = threadIdx.x; e < NX; e += kThreads) {
        int l[6];
#pragma unroll
        for (int d = 0; d < 6; ++d) l[d] = (e >> (2 * (5 - d))) & 3;
        bool ok = true;
#pragma unroll
        for (int d = 0; d < 6; ++d) ok = ok && (t.boff[d] + l[d] < t.ext[d]);
        if (!ok) continue;
        const int64_t a = t.start[0] + t.boff[0] + l[0], b = t.start[1] + t.boff[1] + l[1],
                      c = t.start[2] + t.boff[2] + l[2], i = t.start[3] + t.boff[3] + l[3],
                      j = t.start[4] + t.boff[4] + l[4], k = t.start[5] + t.boff[5] + l[5];
        const double *T1 = p.T1d, *U = p.Ud;
        auto u = [&](int64_t x, int64_t y, int64_t h, int64_t g) {
            return __ldg(U + ((x * v + y) * o + h) * o + g);
        };
        auto t1 = [&](int64_t x, int64_t h) { return __ldg(T1 + x * o + h); };
        double sing = t1(a, i) * u(b, c, j, k);
        sing -= t1(a, j) * u(b, c, i, k);
        sing += t1(a, k) * u(b, c, i, j);
        sing -= t1(b, i) * u(a, c, j, k);
        sing += t1(b, j) * u(a, c, i, k);
        sing -= t1(b, k) * u(a, c, i, j);
        sing += t1(c, i) * u(a, b, j, k);
        sing -= t1(c, j) * u(a, b, i, k);
        sing += t1(c, k) * u(a, b, i, j);
        const double doub = X[e];
        const double denom_0 = -(ev[a] + ev[b] + ev[c]);
        const double denom = doub * factor / (eo[i] + eo[j] + eo[k] + denom_0);
        s1 += denom * doub;
        s2 += denom * (doub + sing);
    }
    s1 = warp_sum(s1);
    s2 = warp_sum(s2);
    if ((threadIdx.x & 31) == 0) {
        red[0][threadIdx.x >> 5] = s1;
        red[1][threadIdx.x >> 5] = s2;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double x = 0.0, y = 0.0;
        for (int w = 0; w < kThreads / 32; ++w) {
            x += red[0][w];
            y += red[1][w];
        }
        p.part[2 * item] = x;
        p.part[2 * item + 1] = y;
    }
    __syncthreads();  // red, X and s_item are reused by the next item
    }
}

// Per-tuple sums of item partials (fixed order, compensated).
__global__ void __launch_bounds__(256) tuple_sum_kernel(const double *__restrict__ part,
                                                        const int64_t *__restrict__ pref,
                                                        int64_t n, double *__restrict__ out) {
    const int64_t q = blockIdx.x;
    if (q >= n) return;
    __shared__ double sa[256], ca[256], sb[256], cb[256];
    Comp x, y;
    for (int64_t it = pref[q] + threadIdx.x; it < pref[q + 1]; it += 256) {
        x.add(part[2 * it]);
        y.add(part[2 * it + 1]);
    }
    sa[threadIdx.x] = x.s;
    ca[threadIdx.x] = x.c;
    sb[threadIdx.x] = y.s;
    cb[threadIdx.x] = y.c;
    __syncthreads();
    if (threadIdx.x == 0) {
        Comp u, w;
        for (int k = 0; k < 256; ++k) {
            u.add(sa[k]);
            u.add(ca[k]);
            w.add(sb[k]);
            w.add(cb[k]);
        }
        out[2 * q] = u.value();
        out[2 * q + 1] = w.value();
    }
}

}  // namespace

int tuple_sums(const double *part, const int64_t *gpref, int64_t n, double *task, double *out, cudaStream_t st) {
    for (int64_t q0 = 0; q0 < n; q0 += 65535) {
        const unsigned nb = (unsigned)std::min<int64_t>(65535, n - q0);
        tuple_sum_kernel<<<nb, 256, 0, st>>>(part, gpref + q0, nb, task + 2 * q0);
        count_launch();
    }
    return reduce_pairs(task, n, out, st);
}

// Dynamic shared memory (unused by the kernel) that a launch requests to
// keep one CTA per SM: with the 36.9 KB static part, two no longer fit.
constexpr int kExclusiveSmem = 96 * 1024;

int fp64_grid(sdt_job *j, int64_t items, int *grid) {
    int nsm = 0, per_sm = 0;
    int rc = cuda_check(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, j->dev), "FP64 form");
    if (!rc && j->sm_exclusive)
        rc = cuda_check(cudaFuncSetAttribute(fused_fp64_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             kExclusiveSmem), "FP64 form");
    if (!rc) rc = cuda_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fused_fp64_kernel, kThreads,
                                                                           j->sm_exclusive ? kExclusiveSmem : 0),
                             "FP64 form");
    if (rc) return rc;
    int64_t cap = (int64_t)nsm * std::max(per_sm, 1);
    if (j->max_ctas > 0) cap = std::min<int64_t>(cap, (int64_t)j->max_ctas * std::max(per_sm, 1));
    *grid = (int)std::max<int64_t>(1, std::min<int64_t>(items, cap));
    return SDT_OK;
}

int fp64_launch(sdt_job *j, const LaunchArgs &a, cudaStream_t st) {
    const Tiling &t = j->t;
    FusedParams p;
    p.T1d = j->arr[DST_T1]; p.T2a = j->arr[DST_T2A]; p.T2b = j->arr[DST_T2B];
    p.Vd2 = j->arr[DST_VD2]; p.Wd1 = j->arr[DST_WD1]; p.Ud = j->arr[DST_UD];
    p.pair_off = j->pair_off;
    p.evl = j->evl_d;
    p.tiles = j->tiles;
    p.noab = (int32_t)t.noab; p.nvab = (int32_t)t.nvab;
    p.nocc = t.nocc; p.nvir = t.nvir;
    p.klist = a.klist; p.item_pref = a.item_pref; p.factor = a.factor;
    p.n_tasks = a.n;
    p.n_items = a.items;
    p.part = a.part;
    p.queue = a.queue;
    int rc = cuda_check(cudaMemsetAsync(a.queue, 0, sizeof(unsigned long long), st), "FP64 form");
    if (rc) return rc;
    fused_fp64_kernel<<<(unsigned)a.grid, kThreads, j->sm_exclusive ? kExclusiveSmem : 0, st>>>(p);
    count_launch();
    return cuda_check(cudaGetLastError(), "FP64 form: fused kernel");
}

}  // namespace sdt

using namespace sdt;

namespace {

void job_free_arrays(sdt_job *j) {
    for (int a = 0; a < DST_N; ++a) {
        gpu_put(j->arr[a]);
        j->arr[a] = nullptr;
        j->arr_n[a] = 0;
    }
}

int tiles_upload(sdt_job *j, cudaStream_t st) {
    const int64_t nt = j->t.noab + j->t.nvab;
    std::vector<int32_t> tab(4 * nt);
    for (int64_t b = 1; b <= nt; ++b) {
        tab[4 * (b - 1) + 0] = (int32_t)j->t.start(b);
        tab[4 * (b - 1) + 1] = (int32_t)j->t.r(b);
        tab[4 * (b - 1) + 2] = (int32_t)j->t.s(b);
        tab[4 * (b - 1) + 3] = (int32_t)j->t.y(b);
    }
    j->tiles = (int32_t *)gpu_get(tab.size() * sizeof(int32_t));
    j->evl_d = (double *)gpu_get(j->evl.size() * sizeof(double));
    j->pair_off = (int64_t *)gpu_get((size_t)(j->t.nvab * j->t.nvab) * sizeof(int64_t));
    if (!j->tiles || !j->evl_d || !j->pair_off) return fail(SDT_ERR_NOMEM, "sdt_job_create: device tables");
    int rc = cuda_check(cudaMemcpyAsync(j->tiles, tab.data(), tab.size() * sizeof(int32_t),
                                        cudaMemcpyHostToDevice, st), "sdt_job_create");
    if (rc) return rc;
    rc = cuda_check(cudaMemcpyAsync(j->evl_d, j->evl.data(), j->evl.size() * sizeof(double),
                                    cudaMemcpyHostToDevice, st), "sdt_job_create");
    if (rc) return rc;
    return cuda_check(cudaStreamSynchronize(st), "sdt_job_create");
}

// restricted beta->alpha mapping of a tile quad (tce_restricted.F:28-71).
void restrict4(const Tiling &t, int64_t *b, int n) {
    int64_t s = 0;
    for (int q = 0; q < n; ++q) s += t.s(b[q]);
    if (t.restricted && s == 2 * n)
        for (int q = 0; q < n; ++q) b[q] = t.alpha[b[q] - 1];
}

}  // namespace

extern "C" int sdt_job_create(const sdt_tiling *ti, sdt_job **out) {
    if (!out) return fail(SDT_ERR_ARG, "sdt_job_create: null output");
    *out = nullptr;
    Tiling tt;
    if (!make_tiling(ti, &tt)) return fail(SDT_ERR_ARG, "sdt_job_create: bad tiling");
    if (tt.noab + tt.nvab > kMaxTiles) return fail(SDT_ERR_ARG, "sdt_job_create: more than 256 tiles");
    sdt_job *j = new sdt_job();
    const int64_t nt = tt.noab + tt.nvab;
    j->range.assign(ti->range, ti->range + nt);
    j->spin.assign(ti->spin, ti->spin + nt);
    j->sym.assign(ti->sym, ti->sym + nt);
    j->offset.assign(ti->offset, ti->offset + nt);
    if (ti->alpha) j->alpha.assign(ti->alpha, ti->alpha + nt);
    j->t = tt;
    j->evl.assign(ti->evl_sorted, ti->evl_sorted + (tt.nocc + tt.nvir));
    j->t.range = j->range.data();
    j->t.spin = j->spin.data();
    j->t.sym = j->sym.data();
    j->t.offset = j->offset.data();
    j->t.alpha = j->alpha.empty() ? nullptr : j->alpha.data();
    j->t.evl = j->evl.data();
    cudaGetDevice(&j->dev);
    if (cudaStreamCreateWithFlags(&j->stream, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        delete j;
        return fail(SDT_ERR_CUDA, "sdt_job_create: no stream");
    }
    cudaStream_t st = j->stream;
    int rc = tiles_upload(j, st);
    if (rc) {
        sdt_job_destroy(j);
        return rc;
    }
    *out = j;
    return SDT_OK;
}

extern "C" int64_t sdt_job_device_bytes(const sdt_job *j) {
    if (!j) return 0;
    int64_t b = 0;
    for (int a = 0; a < DST_N; ++a) b += (int64_t)j->arr_n[a] * 8;
    for (int k = 0; k < 2 * SP_N; ++k) b += (int64_t)j->sp_n[k];
    return b + (int64_t)j->mixed_aux_n;
}

// One read per host page of a buffer, just before the copy engines read it.
// Measured on GB300 (Grace host): copies of pinned pages the CPU had not
// touched for 8-40 s ran at 6-70 GB/s, and at ~200 GB/s right after one CPU
// read per page (the copy path depends on per-page state the CPU refreshes);
// the pass costs about a millisecond per 5 GB.
static void touch_host_pages(const void *p, size_t bytes) {
    static const size_t pg = [] {
        const long v = sysconf(_SC_PAGESIZE);
        return v > 0 ? (size_t)v : (size_t)4096;
    }();
    if (!bytes) return;
    const volatile unsigned char *c = (const volatile unsigned char *)p;
    // the buffer's first byte, then the first byte of every later page it spans
    const size_t first = (size_t)((((uintptr_t)p + pg) & ~(uintptr_t)(pg - 1)) - (uintptr_t)p);
    const int64_t n = bytes > first ? (int64_t)((bytes - first + pg - 1) / pg) : 0;
    unsigned sum = c[0];
#pragma omp parallel for reduction(+ : sum) num_threads(8) schedule(static) if (n > 4096)
    for (int64_t i = 0; i < n; ++i) sum += c[first + (size_t)i * pg];
    (void)sum;
}

extern "C" int sdt_job_load(sdt_job *j, const sdt_file *f1, const sdt_file *f2,
                            const sdt_file *fv, void *stream) {
    if (!j || !f1 || !f2 || !fv || !f1->hash || !f2->hash || !fv->hash)
        return fail(SDT_ERR_ARG, "sdt_job_load: null argument");
    cudaStream_t st = stream ? (cudaStream_t)stream : j->stream;
    const Tiling &t = j->t;
    const int64_t o = t.nocc, v = t.nvir, noab = t.noab, nvab = t.nvab, N = noab + nvab;
    PhaseTrace tr("sdt_job_load");

    // Virtual tile-pair regions of Vd2.
    std::vector<int64_t> pair(nvab * nvab, -1);
    int64_t vd2 = 0;
    for (int64_t B = noab + 1; B <= N; ++B)
        for (int64_t C = B; C <= N; ++C) {
            pair[(B - noab - 1) * nvab + (C - noab - 1)] = vd2;
            vd2 += t.r(B) * t.r(C) * o * v;
        }
    const size_t want[DST_N] = {(size_t)(v * o), (size_t)(v * v * o * o), (size_t)(v * v * o * o),
                                (size_t)vd2, (size_t)(v * o * o * o), (size_t)(v * v * o * o)};
    job_free_arrays(j);
    mixed_release(j);
    j->loaded = false;
    j->pair_host = pair;

    // Copy jobs, destination-driven: every canonical block the path can
    // read is looked up by its (restricted-mapped) key.
    std::vector<CopyJob> jobs;
    std::string missing;
    // Offset of a block; -1 (and an error) when absent or when the block
    // would reach past the end of the file's data.
    auto lookup = [&](const sdt_file *f, int64_t key, int64_t size) {
        const int64_t off = hash_lookup(f->hash, key);
        if ((off < 0 || off + size > f->ndata) && missing.empty())
            missing = (off < 0 ? "key " : "out-of-range block for key ") + std::to_string(key);
        return (off < 0 || off + size > f->ndata) ? (int64_t)-1 : off;
    };
    auto add = [&](int file, int dst, int64_t src_block, int64_t n0, int64_t n1, int64_t n2,
                   int64_t n3, int64_t d0, int64_t s0, int64_t s1, int64_t s2, int64_t s3, double sign) {
        // one job per leading index x0 (keeps each CTA's slab moderate)
        for (int64_t x0 = 0; x0 < n0; ++x0) {
            CopyJob c;
            c.src = src_block + x0 * n1 * n2 * n3;
            c.dst = d0 + x0 * s0;
            c.n1 = n1; c.n2 = n2; c.n3 = n3;
            c.s1 = s1; c.s2 = s2; c.s3 = s3;
            c.sign = sign;
            c.src_file = file;
            c.dst_array = dst;
            jobs.push_back(c);
        }
    };
    auto spin_ok = [&](int64_t a, int64_t b, int64_t c, int64_t d) {
        return t.s(a) + t.s(b) == t.s(c) + t.s(d) && (t.y(a) ^ t.y(b) ^ t.y(c) ^ t.y(d)) == 0;
    };
    // T1 (p,h): ccsd_t_singles_l.F:341-350 (sorted to t1sub(p4,h1)).
    for (int64_t p = noab + 1; p <= N; ++p)
        for (int64_t h = 1; h <= noab; ++h) {
            if (t.s(p) != t.s(h) || (t.y(p) ^ t.y(h)) != 0) continue;
            int64_t b[2] = {p, h};
            restrict4(t, b, 2);
            const int64_t off = lookup(f1, b[1] - 1 + noab * (b[0] - noab - 1), t.r(p) * t.r(h));
            if (off < 0) continue;
            add(0, DST_T1, off, 1, 1, t.r(p), t.r(h), t.start(p) * o + t.start(h), 0, 0, o, 1, 1.0);
        }
    // T2 (p1<=p2, h3<=h4): direct blocks plus the mirrors tce_hashnsort.F
    // reads with factor -1 (h7b<h1b for d1, p7b<p4b for d2).
    for (int64_t p1 = noab + 1; p1 <= N; ++p1)
        for (int64_t p2 = p1; p2 <= N; ++p2)
            for (int64_t h3 = 1; h3 <= noab; ++h3)
                for (int64_t h4 = h3; h4 <= noab; ++h4) {
                    if (!spin_ok(p1, p2, h3, h4)) continue;
                    int64_t b[4] = {p1, p2, h3, h4};
                    restrict4(t, b, 4);
                    const int64_t key = b[3] - 1 + noab * (b[2] - 1 + noab * (b[1] - noab - 1 + nvab * (b[0] - noab - 1)));
                    const int64_t off = lookup(f2, key, t.r(p1) * t.r(p2) * t.r(h3) * t.r(h4));
                    if (off < 0) continue;
                    const int64_t n0 = t.r(p1), n1 = t.r(p2), n2 = t.r(h3), n3 = t.r(h4);
                    const int64_t P1 = t.start(p1), P2 = t.start(p2), H3 = t.start(h3), H4 = t.start(h4);
                    // T2a[p][q][h][l]: strides v*o*o, o*o, o, 1
                    const int64_t ap = v * o * o, aq = o * o, ah = o, al = 1;
                    add(1, DST_T2A, off, n0, n1, n2, n3, P1 * ap + P2 * aq + H3 * ah + H4 * al, ap, aq, ah, al, 1.0);
                    if (h3 != h4)
                        add(1, DST_T2A, off, n0, n1, n2, n3, P1 * ap + P2 * aq + H4 * ah + H3 * al, ap, aq, al, ah, -1.0);
                    // T2b[p][h][l][q]: strides o*o*v, o*v, v, 1
                    const int64_t bp = o * o * v, bh = o * v, bl = v, bq = 1;
                    add(1, DST_T2B, off, n0, n1, n2, n3, P1 * bp + H3 * bh + H4 * bl + P2 * bq, bp, bq, bh, bl, 1.0);
                    if (p1 != p2)
                        add(1, DST_T2B, off, n0, n1, n2, n3, P2 * bp + H3 * bh + H4 * bl + P1 * bq, bq, bp, bh, bl, -1.0);
                }
    // V2 <p5 p6||h3 p7> (p5<=p6): Vd2 region of the pair, [b][c][k][e].
    for (int64_t p5 = noab + 1; p5 <= N; ++p5)
        for (int64_t p6 = p5; p6 <= N; ++p6)
            for (int64_t h3 = 1; h3 <= noab; ++h3)
                for (int64_t p7 = noab + 1; p7 <= N; ++p7) {
                    if (!spin_ok(p5, p6, h3, p7)) continue;
                    int64_t b[4] = {p5, p6, h3, p7};
                    restrict4(t, b, 4);
                    const int64_t off = lookup(fv, b[3] - 1 + N * (b[2] - 1 + N * (b[1] - 1 + N * (b[0] - 1))),
                                               t.r(p5) * t.r(p6) * t.r(h3) * t.r(p7));
                    if (off < 0) continue;
                    const int64_t n1 = t.r(p6);
                    const int64_t base = pair[(p5 - noab - 1) * nvab + (p6 - noab - 1)] + t.start(h3) * v + t.start(p7);
                    add(2, DST_VD2, off, t.r(p5), n1, t.r(h3), t.r(p7), base, n1 * o * v, o * v, v, 1, 1.0);
                }
    // V2 <h7 p6||h2 h3> (h2<=h3): Wd1[c][j][k][m].
    for (int64_t h7 = 1; h7 <= noab; ++h7)
        for (int64_t p6 = noab + 1; p6 <= N; ++p6)
            for (int64_t h2 = 1; h2 <= noab; ++h2)
                for (int64_t h3 = h2; h3 <= noab; ++h3) {
                    if (!spin_ok(h7, p6, h2, h3)) continue;
                    int64_t b[4] = {h7, p6, h2, h3};
                    restrict4(t, b, 4);
                    const int64_t off = lookup(fv, b[3] - 1 + N * (b[2] - 1 + N * (b[1] - 1 + N * (b[0] - 1))),
                                               t.r(h7) * t.r(p6) * t.r(h2) * t.r(h3));
                    if (off < 0) continue;
                    const int64_t base = ((t.start(p6) * o + t.start(h2)) * o + t.start(h3)) * o + t.start(h7);
                    // key order (m, c, j, k): strides 1, o^3, o^2, o
                    add(2, DST_WD1, off, t.r(h7), t.r(p6), t.r(h2), t.r(h3), base, 1, o * o * o, o * o, o, 1.0);
                }
    // V2 <p5 p6||h2 h3> (p5<=p6, h2<=h3): Ud[b][c][j][k].
    for (int64_t p5 = noab + 1; p5 <= N; ++p5)
        for (int64_t p6 = p5; p6 <= N; ++p6)
            for (int64_t h2 = 1; h2 <= noab; ++h2)
                for (int64_t h3 = h2; h3 <= noab; ++h3) {
                    if (!spin_ok(p5, p6, h2, h3)) continue;
                    int64_t b[4] = {p5, p6, h2, h3};
                    restrict4(t, b, 4);
                    const int64_t off = lookup(fv, b[3] - 1 + N * (b[2] - 1 + N * (b[1] - 1 + N * (b[0] - 1))),
                                               t.r(p5) * t.r(p6) * t.r(h2) * t.r(h3));
                    if (off < 0) continue;
                    const int64_t base = ((t.start(p5) * v + t.start(p6)) * o + t.start(h2)) * o + t.start(h3);
                    add(2, DST_UD, off, t.r(p5), t.r(p6), t.r(h2), t.r(h3), base, v * o * o, o * o, o, 1, 1.0);
                }
    if (!missing.empty()) {
        job_free_arrays(j);
        return fail(SDT_ERR_MISSING, "sdt_job_load: a block the path reads is absent (" + missing + ")");
    }

    tr.mark("copy lists", nullptr);
    // Raw files to the device first (copy engines only: they overlap kernels
    // of other streams), then the clears of the dense arrays and the ingest
    // (one launch per 65535 copy jobs), which need SMs.
    const sdt_file *files[3] = {f1, f2, fv};
    double *raw[3] = {nullptr, nullptr, nullptr};
    CopyJob *jobs_d = nullptr;
    // On an error: let issued work finish, return every buffer, leave the
    // job unloaded.
    auto bail = [&](int code) {
        cudaStreamSynchronize(st);
        for (int f = 0; f < 3; ++f) gpu_put(raw[f]);
        gpu_put(jobs_d);
        job_free_arrays(j);
        return code;
    };
    int rc = SDT_OK;
    for (int f = 0; f < 3; ++f) {
        raw[f] = (double *)gpu_get((size_t)std::max<int64_t>(files[f]->ndata, 1) * sizeof(double));
        if (!raw[f]) return bail(fail(SDT_ERR_NOMEM, "sdt_job_load: raw file allocation"));
        if (files[f]->ndata > 0) {
            touch_host_pages(files[f]->data, (size_t)files[f]->ndata * sizeof(double));
            rc = cuda_check(cudaMemcpyAsync(raw[f], files[f]->data, (size_t)files[f]->ndata * sizeof(double),
                                            cudaMemcpyHostToDevice, st), "sdt_job_load");
            if (rc) return bail(rc);
        }
        tr.mark(f == 0 ? "file T1" : f == 1 ? "file T2" : "file V2", st);
    }
    for (int a = 0; a < DST_N; ++a) {
        j->arr[a] = (double *)gpu_get(want[a] * sizeof(double));
        if (!j->arr[a]) return bail(fail(SDT_ERR_NOMEM, "sdt_job_load: dense operand allocation"));
        j->arr_n[a] = want[a];
        rc = cuda_check(cudaMemsetAsync(j->arr[a], 0, want[a] * sizeof(double), st), "sdt_job_load");
        if (rc) return bail(rc);
    }
    rc = cuda_check(cudaMemcpyAsync(j->pair_off, pair.data(), pair.size() * sizeof(int64_t),
                                    cudaMemcpyHostToDevice, st), "sdt_job_load");
    if (rc) return bail(rc);
    tr.mark("allocate+clear", st);
    jobs_d = (CopyJob *)gpu_get(std::max<size_t>(jobs.size(), 1) * sizeof(CopyJob));
    if (!jobs_d) return bail(fail(SDT_ERR_NOMEM, "sdt_job_load: job list"));
    rc = cuda_check(cudaMemcpyAsync(jobs_d, jobs.data(), jobs.size() * sizeof(CopyJob),
                                    cudaMemcpyHostToDevice, st), "sdt_job_load");
    if (rc) return bail(rc);
    IngestArgs g;
    for (int f = 0; f < 3; ++f) g.src[f] = raw[f];
    for (int a = 0; a < DST_N; ++a) g.dst[a] = j->arr[a];
    for (size_t b0 = 0; b0 < jobs.size(); b0 += 65535) {
        g.jobs = jobs_d + b0;
        const unsigned nb = (unsigned)std::min<size_t>(65535, jobs.size() - b0);
        ingest_kernel<<<nb, 256, 0, st>>>(g);
        count_launch();
    }
    rc = cuda_check(cudaGetLastError(), "sdt_job_load: ingest");
    if (rc) return bail(rc);
    // The raw copies and the job list are released once the stream is done.
    rc = cuda_check(cudaStreamSynchronize(st), "sdt_job_load: ingest");
    tr.mark("ingest", nullptr);
    if (rc) return bail(rc);
    for (int f = 0; f < 3; ++f) gpu_put(raw[f]);
    gpu_put(jobs_d);
    j->loaded = true;
    return SDT_OK;
}

// Multiplicity factor of a tuple (ccsd_t_dot.F:52-66).
namespace sdt {
double tuple_factor(const int64_t *k, bool restricted) {
    double f = restricted ? 2.0 : 1.0;
    if (k[0] == k[1] && k[1] == k[2]) f /= 6.0;
    else if (k[0] == k[1] || k[1] == k[2]) f /= 2.0;
    if (k[3] == k[4] && k[4] == k[5]) f /= 6.0;
    else if (k[3] == k[4] || k[4] == k[5]) f /= 2.0;
    return f;
}
}  // namespace sdt

extern "C" int sdt_job_destroy(sdt_job *j) {
    if (!j) return SDT_OK;
    cudaStreamSynchronize(j->stream);
    job_free_arrays(j);
    mixed_release(j);
    gpu_put(j->tiles);
    gpu_put(j->evl_d);
    gpu_put(j->pair_off);

    if (j->ev0) cudaEventDestroy(j->ev0);
    if (j->ev1) cudaEventDestroy(j->ev1);
    if (j->stream) cudaStreamDestroy(j->stream);
    delete j;
    return SDT_OK;
}

extern "C" int sdt_ccsd_t(const sdt_tiling *t, const sdt_file *t1, const sdt_file *t2,
                          const sdt_file *v2, double *energy1, double *energy2) {
    if (!energy1 || !energy2) return fail(SDT_ERR_ARG, "sdt_ccsd_t: null output");
    const int64_t n = sdt_tasks_count(t);
    if (n < 0) return SDT_ERR_ARG;
    std::vector<int64_t> klist(7 * std::max<int64_t>(n, 1));
    int rc = sdt_tasks_list(t, n, klist.data());
    if (rc) return rc;
    sdt_job *j = nullptr;
    rc = sdt_job_create(t, &j);
    if (rc) return rc;
    rc = sdt_job_load(j, t1, t2, v2, nullptr);
    double e[2] = {0.0, 0.0};
    if (!rc) rc = sdt_job_run(j, klist.data(), n, SDT_PREC_FP64, e, nullptr, nullptr);
    sdt_job_destroy(j);
    if (rc) return rc;
    *energy1 = e[0];
    *energy2 = e[1];
    return SDT_OK;
}

extern "C" int sdt_job_set_timing(sdt_job *j, int on) {
    if (!j) return fail(SDT_ERR_ARG, "sdt_job_set_timing: null job");
    j->timing = on != 0;
    return SDT_OK;
}

extern "C" double sdt_job_last_kernel_ms(const sdt_job *j) { return j ? (double)j->last_ms : -1.0; }

// FP64 persistent launches with one CTA per SM (on): a launch capped by
// sdt_job_set_max_ctas then occupies exactly that many SMs and leaves the
// others whole for kernels of other streams.
extern "C" int sdt_job_set_sm_exclusive(sdt_job *j, int on) {
    if (!j) return fail(SDT_ERR_ARG, "sdt_job_set_sm_exclusive: null job");
    j->sm_exclusive = on ? 1 : 0;
    return SDT_OK;
}

extern "C" int sdt_job_set_max_ctas(sdt_job *j, int sms) {
    if (!j || sms < 0) return fail(SDT_ERR_ARG, "sdt_job_set_max_ctas: bad argument");
    j->max_ctas = sms;
    return SDT_OK;
}

extern "C" void *sdt_job_stream(const sdt_job *j) { return j ? (void *)j->stream : nullptr; }

extern "C" int sdt_job_set_mixed_shape(sdt_job *j, int shape) {
    if (!j || (shape != 1 && shape != 2))
        return fail(SDT_ERR_ARG, "sdt_job_set_mixed_shape: shape 1 or 2");
    j->mixed_shape = shape;
    return SDT_OK;
}

extern "C" int sdt_job_set_mixed_segment(sdt_job *j, int chunks) {
    if (!j || chunks < 0) return fail(SDT_ERR_ARG, "sdt_job_set_mixed_segment: bad argument");
    j->mixed_kseg = chunks;
    return SDT_OK;
}
