/*
 * orc_synth.c -- the seeded synthetic inputs of the benchmark workloads,
 * produced on the checker side (TEST INFRASTRUCTURE ONLY).
 *
 * bench.py's reference arm times the oracle without loading the product
 * library, so it needs the workloads' inputs, tuple list and FLOP count from
 * here.  The definitions are those of the workloads, not of NWChem:
 *
 *   element    a pure function of (seed, tensor id, global orbital indices):
 *              S = an Irwin-Hall(12) sum of 32-bit halves of splitmix64
 *              outputs, centred (S * 2^-32 ~ N(0,1)), kept as an integer so
 *              that antisymmetrised combinations are exact before scaling;
 *   T1(a,i)        0.01         * 2^-32 * S(a,i)
 *   T2(a,b,i,j)    0.02/2       * 2^-32 * (S(abij) - S(baij) - S(abji) + S(baji))
 *   <ab||ie>       0.05/sqrt(2) * 2^-32 * (S(abie) - S(baie))
 *   <ma||ij>       0.05/sqrt(2) * 2^-32 * (S(maij) - S(maji))
 *   <ab||ij>       0.05/2       * 2^-32 * (four terms as T2)
 *   orbital energies   occupied -1.5 + 1.1 u, virtual 0.2 + 2.3 u, u in [0,1)
 *
 * The files follow NWChem's TCE layout: T1 blocks (p,h) keyed
 * h-1 + noab*(p-noab-1) (tce_t1_offset.F); T2 blocks p1<=p2, h3<=h4 keyed
 * h4-1 + noab*(h3-1 + noab*(p2-noab-1 + nvab*(p1-noab-1))) (tce_t2_offset.F);
 * V2 blocks g3<=g4, g1<=g2 keyed g2-1 + N*(g1-1 + N*(g4-1 + N*(g3-1)))
 * (tce_mo2e_offset.F), of the three kinds the triples path reads.  Blocks
 * that spin, irrep or (restricted) the all-beta rule exclude are absent.
 * tests/test_oracle.py checks that these bytes equal the library's.
 */
#include "sdt_oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>

typedef int64_t I;

static uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

enum { T_T1 = 1, T_T2 = 2, T_VVOV = 3, T_OVOO = 4, T_VVOO = 5, T_EVL = 6 };

/* The centred integer draw of element `idx` of tensor `tid`. */
static I draw_s(uint64_t seed, uint64_t tid, uint64_t idx) {
    const uint64_t key = mix64(seed ^ mix64((tid << 56) ^ mix64(idx)));
    I s = 0;
    for (uint64_t r = 0; r < 6; ++r) {
        const uint64_t z = mix64(key + r * 0xD1B54A32D192ED03ull);
        s += (I)(z & 0xffffffffull) + (I)(z >> 32);
    }
    return s - (I)6 * (I)4294967296LL;
}

typedef struct {
    uint64_t seed;
    I o, v;
    double c1, c2, ca, c4;
} gen_t;

static I s_oovv(const gen_t *g, uint64_t tid, I a, I b, I i, I j) {
    return draw_s(g->seed, tid, (uint64_t)(((a * g->v + b) * g->o + i) * g->o + j));
}
static double e_t2(const gen_t *g, I a, I b, I i, I j) {
    return g->c2 * (double)(s_oovv(g, T_T2, a, b, i, j) - s_oovv(g, T_T2, b, a, i, j) -
                            s_oovv(g, T_T2, a, b, j, i) + s_oovv(g, T_T2, b, a, j, i));
}
static double e_vvoo(const gen_t *g, I a, I b, I i, I j) {
    return g->c4 * (double)(s_oovv(g, T_VVOO, a, b, i, j) - s_oovv(g, T_VVOO, b, a, i, j) -
                            s_oovv(g, T_VVOO, a, b, j, i) + s_oovv(g, T_VVOO, b, a, j, i));
}
static double e_vvov(const gen_t *g, I a, I b, I i, I e) {
    const I x = draw_s(g->seed, T_VVOV, (uint64_t)(((a * g->v + b) * g->o + i) * g->v + e));
    const I y = draw_s(g->seed, T_VVOV, (uint64_t)(((b * g->v + a) * g->o + i) * g->v + e));
    return g->ca * (double)(x - y);
}
static double e_ovoo(const gen_t *g, I m, I a, I i, I j) {
    const I x = draw_s(g->seed, T_OVOO, (uint64_t)(((m * g->v + a) * g->o + i) * g->o + j));
    const I y = draw_s(g->seed, T_OVOO, (uint64_t)(((m * g->v + a) * g->o + j) * g->o + i));
    return g->ca * (double)(x - y);
}

void orc_synth_evl(I nocc, I nvir, uint64_t seed, double *evl) {
    for (I q = 0; q < nocc + nvir; ++q) {
        const uint64_t z = mix64(seed ^ mix64(((uint64_t)T_EVL << 56) ^ mix64((uint64_t)q)));
        const double u = (double)(z >> 11) * (1.0 / 9007199254740992.0);
        evl[q] = q < nocc ? -1.5 + 1.1 * u : 0.2 + 2.3 * u;
    }
}

/* Tile helpers on orc_tiling (1-based tiles). */
#define R(b) (t->range[(b)-1])
#define SP(b) (t->spin[(b)-1])
#define SY(b) (t->sym[(b)-1])

static I nocc_of(const orc_tiling *t) {
    I n = 0;
    for (I b = 1; b <= t->noab; ++b) n += R(b);
    return n;
}
static I nvir_of(const orc_tiling *t) {
    I n = 0;
    for (I b = t->noab + 1; b <= t->noab + t->nvab; ++b) n += R(b);
    return n;
}
/* First orbital of tile b inside its own space. */
static I start_of(const orc_tiling *t, I b) {
    return b <= t->noab ? t->offset[b - 1] : t->offset[b - 1] - nocc_of(t);
}

typedef struct {
    I key, tl[4], size;
    int kind; /* 0 T1, 1 T2, 2 <vv||ov>, 3 <ov||oo>, 4 <vv||oo> */
} blk_t;

/* Lists the blocks of file `kind` in key order; returns the count (out may
 * be NULL to count only). */
static I list_blocks(const orc_tiling *t, int kind, blk_t *out) {
    const I o = t->noab, nt = t->noab + t->nvab;
    I n = 0;
#define PUT(K, A, B, C, D, SZ, KIND)                              \
    do {                                                          \
        if (out) {                                                \
            blk_t bb = {(K), {(A), (B), (C), (D)}, (SZ), (KIND)}; \
            out[n] = bb;                                          \
        }                                                         \
        ++n;                                                      \
    } while (0)
    if (kind == 0) {
        for (I p = o + 1; p <= nt; ++p)
            for (I h = 1; h <= o; ++h) {
                if (SP(p) != SP(h) || (SY(p) ^ SY(h)) != 0) continue;
                if (t->restricted && SP(p) + SP(h) == 4) continue;
                PUT(h - 1 + o * (p - o - 1), p, h, 0, 0, R(p) * R(h), 0);
            }
    } else if (kind == 1) {
        for (I p1 = o + 1; p1 <= nt; ++p1)
            for (I p2 = p1; p2 <= nt; ++p2)
                for (I h3 = 1; h3 <= o; ++h3)
                    for (I h4 = h3; h4 <= o; ++h4) {
                        if (SP(p1) + SP(p2) != SP(h3) + SP(h4)) continue;
                        if ((SY(p1) ^ SY(p2) ^ SY(h3) ^ SY(h4)) != 0) continue;
                        if (t->restricted && SP(p1) + SP(p2) + SP(h3) + SP(h4) == 8) continue;
                        PUT(h4 - 1 + o * (h3 - 1 + o * (p2 - o - 1 + t->nvab * (p1 - o - 1))), p1, p2, h3, h4,
                            R(p1) * R(p2) * R(h3) * R(h4), 1);
                    }
    } else {
        for (I g3 = 1; g3 <= nt; ++g3)
            for (I g4 = g3; g4 <= nt; ++g4)
                for (I g1 = 1; g1 <= nt; ++g1)
                    for (I g2 = g1; g2 <= nt; ++g2) {
                        const int v3 = g3 > o, v4 = g4 > o, v1 = g1 > o, v2 = g2 > o;
                        int k;
                        if (v3 && v4 && !v1 && v2) k = 2;
                        else if (!v3 && v4 && !v1 && !v2) k = 3;
                        else if (v3 && v4 && !v1 && !v2) k = 4;
                        else continue;
                        if (SP(g3) + SP(g4) != SP(g1) + SP(g2)) continue;
                        if ((SY(g3) ^ SY(g4) ^ SY(g1) ^ SY(g2)) != 0) continue;
                        if (t->restricted && SP(g3) + SP(g4) + SP(g1) + SP(g2) == 8) continue;
                        PUT(g2 - 1 + nt * (g1 - 1 + nt * (g4 - 1 + nt * (g3 - 1))), g3, g4, g1, g2,
                            R(g3) * R(g4) * R(g1) * R(g2), k);
                    }
    }
#undef PUT
    return n;
}

static void fill(const orc_tiling *t, const gen_t *g, const blk_t *b, double *dst) {
    if (b->kind == 0) {
        const I P = start_of(t, b->tl[0]), H = start_of(t, b->tl[1]), np = R(b->tl[0]), nh = R(b->tl[1]);
        for (I a = 0; a < np; ++a)
            for (I i = 0; i < nh; ++i)
                dst[a * nh + i] = g->c1 * (double)draw_s(g->seed, T_T1, (uint64_t)((P + a) * g->o + H + i));
        return;
    }
    const I n0 = R(b->tl[0]), n1 = R(b->tl[1]), n2 = R(b->tl[2]), n3 = R(b->tl[3]);
    const I s0 = start_of(t, b->tl[0]), s1 = start_of(t, b->tl[1]);
    const I s2 = start_of(t, b->tl[2]), s3 = start_of(t, b->tl[3]);
    for (I x0 = 0; x0 < n0; ++x0)
        for (I x1 = 0; x1 < n1; ++x1)
            for (I x2 = 0; x2 < n2; ++x2)
                for (I x3 = 0; x3 < n3; ++x3) {
                    const I a = s0 + x0, c = s1 + x1, d = s2 + x2, e = s3 + x3;
                    double val;
                    if (b->kind == 1) val = e_t2(g, a, c, d, e);
                    else if (b->kind == 2) val = e_vvov(g, a, c, d, e);
                    else if (b->kind == 3) val = e_ovoo(g, a, c, d, e);
                    else val = e_vvoo(g, a, c, d, e);
                    dst[((x0 * n1 + x1) * n2 + x2) * n3 + x3] = val;
                }
}

int64_t orc_synth_file(const orc_tiling *t, int kind, uint64_t seed, int64_t *nblocks, int64_t *ndata,
                       int64_t *hash, double *data) {
    if (kind < 0 || kind > 2) return -1;
    const I n = list_blocks(t, kind, NULL);
    blk_t *bl = (blk_t *)malloc((size_t)(n > 0 ? n : 1) * sizeof(blk_t));
    I *off = (I *)malloc((size_t)(n > 0 ? n : 1) * sizeof(I));
    if (!bl || !off) {
        free(bl);
        free(off);
        return -2;
    }
    list_blocks(t, kind, bl);
    I total = 0;
    for (I q = 0; q < n; ++q) {
        off[q] = total;
        total += bl[q].size;
    }
    *nblocks = n;
    *ndata = total;
    if (hash && data) {
        hash[0] = n;
        for (I q = 0; q < n; ++q) {
            hash[1 + q] = bl[q].key;
            hash[1 + n + q] = off[q];
        }
        gen_t g = {seed, nocc_of(t), nvir_of(t), 0.0, 0.0, 0.0, 0.0};
        const double two_m32 = 1.0 / 4294967296.0;
        g.c1 = 0.01 * two_m32;
        g.c2 = 0.02 / 2.0 * two_m32;
        g.ca = 0.05 / sqrt(2.0) * two_m32;
        g.c4 = 0.05 / 2.0 * two_m32;
#pragma omp parallel for schedule(dynamic, 1)
        for (I q = 0; q < n; ++q) fill(t, &g, &bl[q], data + off[q]);
    }
    free(bl);
    free(off);
    return 0;
}

/* Algorithmic FLOPs of a tuple list: per tuple Nt * 2 * (sum over the 18
 * d1/d2 terms of the contraction lengths that spin and irrep allow, + 9 for
 * the s1 terms); without spin or irrep restrictions Nt * 18 * (o + v + 1). */
double orc_tasks_flops(const orc_tiling *t, const int64_t *klist, int64_t n) {
    static const int d1p[9][2] = {{0, 1}, {0, 1}, {0, 1}, {1, 2}, {1, 2}, {1, 2}, {0, 2}, {0, 2}, {0, 2}};
    static const int d1h[9] = {0, 1, 2, 0, 1, 2, 0, 1, 2};
    static const int d2p[9] = {0, 0, 0, 1, 1, 1, 2, 2, 2};
    static const int d2h[9][2] = {{0, 1}, {1, 2}, {0, 2}, {0, 1}, {1, 2}, {0, 2}, {0, 1}, {1, 2}, {0, 2}};
    double total = 0.0;
    for (I q = 0; q < n; ++q) {
        const I *k = klist + 7 * q;
        const I P[3] = {k[0], k[1], k[2]}, H[3] = {k[3], k[4], k[5]};
        const double nt = (double)(R(P[0]) * R(P[1]) * R(P[2]) * R(H[0]) * R(H[1]) * R(H[2]));
        double kd = 0.0;
        for (int x = 0; x < 9; ++x) {
            const I pa = P[d1p[x][0]], pb = P[d1p[x][1]], hc = H[d1h[x]];
            for (I m = 1; m <= t->noab; ++m)
                if (SP(pa) + SP(pb) == SP(hc) + SP(m) && (SY(pa) ^ SY(pb) ^ SY(hc) ^ SY(m)) == 0) kd += (double)R(m);
            const I pe = P[d2p[x]], h1 = H[d2h[x][0]], h2 = H[d2h[x][1]];
            for (I e = t->noab + 1; e <= t->noab + t->nvab; ++e)
                if (SP(pe) + SP(e) == SP(h1) + SP(h2) && (SY(pe) ^ SY(e) ^ SY(h1) ^ SY(h2)) == 0) kd += (double)R(e);
        }
        total += nt * 2.0 * (kd + 9.0);
    }
    return total;
}
