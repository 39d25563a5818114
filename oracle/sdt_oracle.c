/*
 * sdt_oracle.c -- CPU oracle (TEST INFRASTRUCTURE ONLY) for NWChem's TCE
 * CCSD(T) perturbative-triples tile path.
 *
 * This file is the checker.  It is loaded only by tests/, by
 * __graft_entry__.smoke() and by bench.py's CPU-baseline leg; the product
 * library never links or calls it.  It restates the reference's Fortran in
 * plain C with OpenMP, function by function (paths relative to the NWChem
 * source tree):
 *
 *   orc_sd_t_s1/_d1/_d2   src/tce/ccsd_t/ccsd_t_kernels_omp.F:5-1198
 *                         (same loop nests, same OpenMP collapse; the
 *                         CRAYFTN / __ppc64__ branches are not taken)
 *   orc_tce_sort_2        src/tce/sort/tce_sort2.F:1-31
 *   orc_tce_sort_4        src/tce/sort/tce_sort4.F:24-72
 *   orc_tce_hash          src/tce/tce_hash.F:271-316
 *   orc_get_hash_block    src/tce/get_hash_block.F:1-44 (in-memory file)
 *   restricted_2/_4       src/tce/tce_restricted.F:1-71
 *   orc_singles_l_1       src/tce/ccsd_t/ccsd_t_singles_l.F:30-464
 *   orc_doubles_l_12      src/tce/ccsd_t/offl_ccsd_t_doubles_l.F:72-1020
 *   hashnsort/_2          src/tce/ccsd_t/tce_hashnsort.F:1-173
 *   orc_ccsd_t_dot        src/tce/ccsd_t/ccsd_t_dot.F:20-138 (compensated sums)
 *   orc_6tasks/neword     src/tce/ccsd_t/ccsd_t_neword.F:1-244
 *   orc_ccsd_t            src/tce/ccsd_t/ccsd_t.F:150-297, 358-456
 *
 * Arithmetic: built with -ffp-contract=off so that "x = x - a*b" rounds the
 * product and the difference separately, as the Fortran statement reads.
 * The d1 h7 loop and d2 p7 loop accumulate in ascending order (the
 * reference's innermost loop); the plain CPU driver rotates the starting
 * h7b/p7b tile by rank (offl_ccsd_t_doubles_l.F:322-327,736-741), which is
 * the identity for rank 0 and only changes rounding otherwise.
 */
#include "sdt_oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>

/* Fortran column-major addressing with 0-based indices. */
#define F2(i1, i2, d1) ((i1) + (d1) * (i2))
#define F4(i1, i2, i3, i4, d1, d2, d3) \
    ((i1) + (d1) * ((i2) + (d2) * ((i3) + (d3) * (i4))))
#define F6(i1, i2, i3, i4, i5, i6, d1, d2, d3, d4, d5) \
    ((i1) + (d1) * ((i2) + (d2) * ((i3) + (d3) * ((i4) + (d4) * ((i5) + (d5) * (i6))))))

typedef int64_t I;

/* ======================================================================
 * s1 kernels: triplesx(perm) +/-= t1sub(p4,h1) * v2sub(h3,h2,p6,p5)
 * ccsd_t_kernels_omp.F:5-360
 * ==================================================================== */
#define T1S(p4, h1) t1sub[F2(p4, h1, p4d)]
#define V2S(h3, h2, p6, p5) v2sub[F4(h3, h2, p6, p5, h3d, h2d, p6d)]

static void s1_1(I h3d, I h2d, I h1d, I p6d, I p5d, I p4d, double *X,
                 const double *t1sub, const double *v2sub) {
#pragma omp parallel for collapse(3) schedule(static)
    for (I p4 = 0; p4 < p4d; p4++)
    for (I p5 = 0; p5 < p5d; p5++)
    for (I p6 = 0; p6 < p6d; p6++)
    for (I h1 = 0; h1 < h1d; h1++)
    for (I h2 = 0; h2 < h2d; h2++)
    for (I h3 = 0; h3 < h3d; h3++) {
        I x = F6(h3, h2, h1, p6, p5, p4, h3d, h2d, h1d, p6d, p5d);
        X[x] = X[x] + T1S(p4, h1) * V2S(h3, h2, p6, p5);
    }
}
static void s1_2(I h3d, I h2d, I h1d, I p6d, I p5d, I p4d, double *X,
                 const double *t1sub, const double *v2sub) {
#pragma omp parallel for collapse(3) schedule(static)
    for (I p4 = 0; p4 < p4d; p4++)
    for (I p5 = 0; p5 < p5d; p5++)
    for (I p6 = 0; p6 < p6d; p6++)
    for (I h1 = 0; h1 < h1d; h1++)
    for (I h2 = 0; h2 < h2d; h2++)
    for (I h3 = 0; h3 < h3d; h3++) {
        I x = F6(h3, h1, h2, p6, p5, p4, h3d, h1d, h2d, p6d, p5d);
        X[x] = X[x] - T1S(p4, h1) * V2S(h3, h2, p6, p5);
    }
}
static void s1_3(I h3d, I h2d, I h1d, I p6d, I p5d, I p4d, double *X,
                 const double *t1sub, const double *v2sub) {
#pragma omp parallel for collapse(3) schedule(static)
    for (I p4 = 0; p4 < p4d; p4++)
    for (I p5 = 0; p5 < p5d; p5++)
    for (I p6 = 0; p6 < p6d; p6++)
    for (I h2 = 0; h2 < h2d; h2++)
    for (I h3 = 0; h3 < h3d; h3++)
    for (I h1 = 0; h1 < h1d; h1++) {
        I x = F6(h1, h3, h2, p6, p5, p4, h1d, h3d, h2d, p6d, p5d);
        X[x] = X[x] + T1S(p4, h1) * V2S(h3, h2, p6, p5);
    }
}
static void s1_4(I h3d, I h2d, I h1d, I p6d, I p5d, I p4d, double *X,
                 const double *t1sub, const double *v2sub) {
#pragma omp parallel for collapse(3) schedule(static)
    for (I p5 = 0; p5 < p5d; p5++)
    for (I p4 = 0; p4 < p4d; p4++)
    for (I p6 = 0; p6 < p6d; p6++)
    for (I h1 = 0; h1 < h1d; h1++)
    for (I h2 = 0; h2 < h2d; h2++)
    for (I h3 = 0; h3 < h3d; h3++) {
        I x = F6(h3, h2, h1, p6, p4, p5, h3d, h2d, h1d, p6d, p4d);
        X[x] = X[x] - T1S(p4, h1) * V2S(h3, h2, p6, p5);
    }
}
static void s1_5(I h3d, I h2d, I h1d, I p6d, I p5d, I p4d, double *X,
                 const double *t1sub, const double *v2sub) {
#pragma omp parallel for collapse(3) schedule(static)
    for (I p5 = 0; p5 < p5d; p5++)
    for (I p4 = 0; p4 < p4d; p4++)
    for (I p6 = 0; p6 < p6d; p6++)
    for (I h1 = 0; h1 < h1d; h1++)
    for (I h2 = 0; h2 < h2d; h2++)
    for (I h3 = 0; h3 < h3d; h3++) {
        I x = F6(h3, h1, h2, p6, p4, p5, h3d, h1d, h2d, p6d, p4d);
        X[x] = X[x] + T1S(p4, h1) * V2S(h3, h2, p6, p5);
    }
}
static void s1_6(I h3d, I h2d, I h1d, I p6d, I p5d, I p4d, double *X,
                 const double *t1sub, const double *v2sub) {
#pragma omp parallel for collapse(3) schedule(static)
    for (I p5 = 0; p5 < p5d; p5++)
    for (I p4 = 0; p4 < p4d; p4++)
    for (I p6 = 0; p6 < p6d; p6++)
    for (I h2 = 0; h2 < h2d; h2++)
    for (I h3 = 0; h3 < h3d; h3++)
    for (I h1 = 0; h1 < h1d; h1++) {
        I x = F6(h1, h3, h2, p6, p4, p5, h1d, h3d, h2d, p6d, p4d);
        X[x] = X[x] - T1S(p4, h1) * V2S(h3, h2, p6, p5);
    }
}
static void s1_7(I h3d, I h2d, I h1d, I p6d, I p5d, I p4d, double *X,
                 const double *t1sub, const double *v2sub) {
#pragma omp parallel for collapse(3) schedule(static)
    for (I p5 = 0; p5 < p5d; p5++)
    for (I p6 = 0; p6 < p6d; p6++)
    for (I p4 = 0; p4 < p4d; p4++)
    for (I h1 = 0; h1 < h1d; h1++)
    for (I h2 = 0; h2 < h2d; h2++)
    for (I h3 = 0; h3 < h3d; h3++) {
        I x = F6(h3, h2, h1, p4, p6, p5, h3d, h2d, h1d, p4d, p6d);
        X[x] = X[x] + T1S(p4, h1) * V2S(h3, h2, p6, p5);
    }
}
static void s1_8(I h3d, I h2d, I h1d, I p6d, I p5d, I p4d, double *X,
                 const double *t1sub, const double *v2sub) {
#pragma omp parallel for collapse(3) schedule(static)
    for (I p5 = 0; p5 < p5d; p5++)
    for (I p6 = 0; p6 < p6d; p6++)
    for (I p4 = 0; p4 < p4d; p4++)
    for (I h2 = 0; h2 < h2d; h2++)
    for (I h1 = 0; h1 < h1d; h1++)
    for (I h3 = 0; h3 < h3d; h3++) {
        I x = F6(h3, h1, h2, p4, p6, p5, h3d, h1d, h2d, p4d, p6d);
        X[x] = X[x] - T1S(p4, h1) * V2S(h3, h2, p6, p5);
    }
}
static void s1_9(I h3d, I h2d, I h1d, I p6d, I p5d, I p4d, double *X,
                 const double *t1sub, const double *v2sub) {
#pragma omp parallel for collapse(3) schedule(static)
    for (I p5 = 0; p5 < p5d; p5++)
    for (I p6 = 0; p6 < p6d; p6++)
    for (I p4 = 0; p4 < p4d; p4++)
    for (I h2 = 0; h2 < h2d; h2++)
    for (I h3 = 0; h3 < h3d; h3++)
    for (I h1 = 0; h1 < h1d; h1++) {
        I x = F6(h1, h3, h2, p4, p6, p5, h1d, h3d, h2d, p4d, p6d);
        X[x] = X[x] + T1S(p4, h1) * V2S(h3, h2, p6, p5);
    }
}
#undef T1S
#undef V2S

void orc_sd_t_s1(I k, I h3d, I h2d, I h1d, I p6d, I p5d, I p4d,
                 double *triplesx, const double *t1sub, const double *v2sub) {
    typedef void (*fn)(I, I, I, I, I, I, double *, const double *,
                       const double *);
    static const fn tab[9] = {s1_1, s1_2, s1_3, s1_4, s1_5,
                              s1_6, s1_7, s1_8, s1_9};
    if (k < 1 || k > 9) return;
    tab[k - 1](h3d, h2d, h1d, p6d, p5d, p4d, triplesx, t1sub, v2sub);
}

/* ======================================================================
 * d1 kernels: triplesx(perm) -/+= sum_h7 t2sub(h7,p4,p5,h1)*v2sub(h3,h2,p6,h7)
 * ccsd_t_kernels_omp.F:362-856.  Each first transposes v2sub into
 * v2tmp(h7,h3,h2,p6) exactly as the reference does.
 * ==================================================================== */
#define T2S(h7, p4, p5, h1) t2sub[F4(h7, p4, p5, h1, h7d, p4d, p5d)]
#define VT(h7, h3, h2, p6) v2tmp[F4(h7, h3, h2, p6, h7d, h3d, h2d)]

static double *d1_v2tmp(I h3d, I h2d, I p6d, I h7d, const double *v2sub) {
    double *v2tmp = (double *)malloc(sizeof(double) * (size_t)(h7d * h3d * h2d * p6d + 1));
    if (!v2tmp) return NULL;
#pragma omp parallel for collapse(3) schedule(static)
    for (I p6 = 0; p6 < p6d; p6++)
    for (I h7 = 0; h7 < h7d; h7++)
    for (I h2 = 0; h2 < h2d; h2++)
    for (I h3 = 0; h3 < h3d; h3++)
        VT(h7, h3, h2, p6) = v2sub[F4(h3, h2, p6, h7, h3d, h2d, p6d)];
    return v2tmp;
}

/* The nine second loop nests.  SIGN is the statement's sign, XIDX the
 * permuted triplesx address, and the loop order is written out per kernel. */
#define D1_BODY(XIDX, OP)                                            \
    {                                                                \
        I x = XIDX;                                                  \
        for (I h7 = 0; h7 < h7d; h7++)                               \
            X[x] = X[x] OP T2S(h7, p4, p5, h1) * VT(h7, h3, h2, p6); \
    }

static void d1_1(I h3d, I h2d, I h1d, I p6d, I p5d, I p4d, I h7d, double *X,
                 const double *t2sub, const double *v2tmp) {
#pragma omp parallel for collapse(3) schedule(static)
    for (I p5 = 0; p5 < p5d; p5++)
    for (I p6 = 0; p6 < p6d; p6++)
    for (I p4 = 0; p4 < p4d; p4++)
    for (I h1 = 0; h1 < h1d; h1++)
    for (I h2 = 0; h2 < h2d; h2++)
    for (I h3 = 0; h3 < h3d; h3++)
        D1_BODY(F6(h3, h2, h1, p6, p5, p4, h3d, h2d, h1d, p6d, p5d), -)
}
static void d1_2(I h3d, I h2d, I h1d, I p6d, I p5d, I p4d, I h7d, double *X,
                 const double *t2sub, const double *v2tmp) {
#pragma omp parallel for collapse(3) schedule(static)
    for (I p4 = 0; p4 < p4d; p4++)
    for (I p5 = 0; p5 < p5d; p5++)
    for (I p6 = 0; p6 < p6d; p6++)
    for (I h2 = 0; h2 < h2d; h2++)
    for (I h1 = 0; h1 < h1d; h1++)
    for (I h3 = 0; h3 < h3d; h3++)
        D1_BODY(F6(h3, h1, h2, p6, p5, p4, h3d, h1d, h2d, p6d, p5d), +)
}
static void d1_3(I h3d, I h2d, I h1d, I p6d, I p5d, I p4d, I h7d, double *X,
                 const double *t2sub, const double *v2tmp) {
#pragma omp parallel for collapse(3) schedule(static)
    for (I p4 = 0; p4 < p4d; p4++)
    for (I p5 = 0; p5 < p5d; p5++)
    for (I p6 = 0; p6 < p6d; p6++)
    for (I h2 = 0; h2 < h2d; h2++)
    for (I h3 = 0; h3 < h3d; h3++)
    for (I h1 = 0; h1 < h1d; h1++)
        D1_BODY(F6(h1, h3, h2, p6, p5, p4, h1d, h3d, h2d, p6d, p5d), -)
}
static void d1_4(I h3d, I h2d, I h1d, I p6d, I p5d, I p4d, I h7d, double *X,
                 const double *t2sub, const double *v2tmp) {
#pragma omp parallel for collapse(3) schedule(static)
    for (I p6 = 0; p6 < p6d; p6++)
    for (I p5 = 0; p5 < p5d; p5++)
    for (I h1 = 0; h1 < h1d; h1++)
    for (I h2 = 0; h2 < h2d; h2++)
    for (I p4 = 0; p4 < p4d; p4++)
    for (I h3 = 0; h3 < h3d; h3++)
        D1_BODY(F6(h3, h2, h1, p5, p4, p6, h3d, h2d, h1d, p5d, p4d), -)
}
static void d1_5(I h3d, I h2d, I h1d, I p6d, I p5d, I p4d, I h7d, double *X,
                 const double *t2sub, const double *v2tmp) {
#pragma omp parallel for collapse(3) schedule(static)
    for (I p6 = 0; p6 < p6d; p6++)
    for (I p4 = 0; p4 < p4d; p4++)
    for (I p5 = 0; p5 < p5d; p5++)
    for (I h2 = 0; h2 < h2d; h2++)
    for (I h1 = 0; h1 < h1d; h1++)
    for (I h3 = 0; h3 < h3d; h3++)
        D1_BODY(F6(h3, h1, h2, p5, p4, p6, h3d, h1d, h2d, p5d, p4d), +)
}
static void d1_6(I h3d, I h2d, I h1d, I p6d, I p5d, I p4d, I h7d, double *X,
                 const double *t2sub, const double *v2tmp) {
#pragma omp parallel for collapse(3) schedule(static)
    for (I p6 = 0; p6 < p6d; p6++)
    for (I p4 = 0; p4 < p4d; p4++)
    for (I p5 = 0; p5 < p5d; p5++)
    for (I h2 = 0; h2 < h2d; h2++)
    for (I h3 = 0; h3 < h3d; h3++)
    for (I h1 = 0; h1 < h1d; h1++)
        D1_BODY(F6(h1, h3, h2, p5, p4, p6, h1d, h3d, h2d, p5d, p4d), -)
}
static void d1_7(I h3d, I h2d, I h1d, I p6d, I p5d, I p4d, I h7d, double *X,
                 const double *t2sub, const double *v2tmp) {
#pragma omp parallel for collapse(3) schedule(static)
    for (I p4 = 0; p4 < p4d; p4++)
    for (I p6 = 0; p6 < p6d; p6++)
    for (I p5 = 0; p5 < p5d; p5++)
    for (I h1 = 0; h1 < h1d; h1++)
    for (I h2 = 0; h2 < h2d; h2++)
    for (I h3 = 0; h3 < h3d; h3++)
        D1_BODY(F6(h3, h2, h1, p5, p6, p4, h3d, h2d, h1d, p5d, p6d), +)
}
static void d1_8(I h3d, I h2d, I h1d, I p6d, I p5d, I p4d, I h7d, double *X,
                 const double *t2sub, const double *v2tmp) {
#pragma omp parallel for collapse(3) schedule(static)
    for (I p4 = 0; p4 < p4d; p4++)
    for (I p6 = 0; p6 < p6d; p6++)
    for (I p5 = 0; p5 < p5d; p5++)
    for (I h2 = 0; h2 < h2d; h2++)
    for (I h1 = 0; h1 < h1d; h1++)
    for (I h3 = 0; h3 < h3d; h3++)
        D1_BODY(F6(h3, h1, h2, p5, p6, p4, h3d, h1d, h2d, p5d, p6d), -)
}
static void d1_9(I h3d, I h2d, I h1d, I p6d, I p5d, I p4d, I h7d, double *X,
                 const double *t2sub, const double *v2tmp) {
#pragma omp parallel for collapse(3) schedule(static)
    for (I p4 = 0; p4 < p4d; p4++)
    for (I p6 = 0; p6 < p6d; p6++)
    for (I p5 = 0; p5 < p5d; p5++)
    for (I h2 = 0; h2 < h2d; h2++)
    for (I h1 = 0; h1 < h1d; h1++)
    for (I h3 = 0; h3 < h3d; h3++)
        D1_BODY(F6(h1, h3, h2, p5, p6, p4, h1d, h3d, h2d, p5d, p6d), +)
}
#undef D1_BODY
#undef T2S
#undef VT

void orc_sd_t_d1(I k, I h3d, I h2d, I h1d, I p6d, I p5d, I p4d, I h7d,
                 double *triplesx, const double *t2sub, const double *v2sub) {
    typedef void (*fn)(I, I, I, I, I, I, I, double *, const double *,
                       const double *);
    static const fn tab[9] = {d1_1, d1_2, d1_3, d1_4, d1_5,
                              d1_6, d1_7, d1_8, d1_9};
    if (k < 1 || k > 9) return;
    double *v2tmp = d1_v2tmp(h3d, h2d, p6d, h7d, v2sub);
    if (!v2tmp) return;
    tab[k - 1](h3d, h2d, h1d, p6d, p5d, p4d, h7d, triplesx, t2sub, v2tmp);
    free(v2tmp);
}

/* ======================================================================
 * d2 kernels: triplesx(perm) -/+= sum_p7 t2sub(p7,p4,h1,h2)*v2sub(p7,h3,p6,p5)
 * ccsd_t_kernels_omp.F:857-1198
 * ==================================================================== */
#define T2S(p7, p4, h1, h2) t2sub[F4(p7, p4, h1, h2, p7d, p4d, h1d)]
#define V2S(p7, h3, p6, p5) v2sub[F4(p7, h3, p6, p5, p7d, h3d, p6d)]
#define D2_BODY(XIDX, OP)                                             \
    {                                                                 \
        I x = XIDX;                                                   \
        for (I p7 = 0; p7 < p7d; p7++)                                \
            X[x] = X[x] OP T2S(p7, p4, h1, h2) * V2S(p7, h3, p6, p5); \
    }

static void d2_1(I h3d, I h2d, I h1d, I p6d, I p5d, I p4d, I p7d, double *X,
                 const double *t2sub, const double *v2sub) {
#pragma omp parallel for collapse(3) schedule(static)
    for (I p4 = 0; p4 < p4d; p4++)
    for (I p5 = 0; p5 < p5d; p5++)
    for (I p6 = 0; p6 < p6d; p6++)
    for (I h1 = 0; h1 < h1d; h1++)
    for (I h2 = 0; h2 < h2d; h2++)
    for (I h3 = 0; h3 < h3d; h3++)
        D2_BODY(F6(h3, h2, h1, p6, p5, p4, h3d, h2d, h1d, p6d, p5d), -)
}
static void d2_2(I h3d, I h2d, I h1d, I p6d, I p5d, I p4d, I p7d, double *X,
                 const double *t2sub, const double *v2sub) {
#pragma omp parallel for collapse(3) schedule(static)
    for (I p5 = 0; p5 < p5d; p5++)
    for (I p6 = 0; p6 < p6d; p6++)
    for (I h1 = 0; h1 < h1d; h1++)
    for (I p4 = 0; p4 < p4d; p4++)
    for (I h3 = 0; h3 < h3d; h3++)
    for (I h2 = 0; h2 < h2d; h2++)
        D2_BODY(F6(h2, h1, h3, p6, p5, p4, h2d, h1d, h3d, p6d, p5d), -)
}
static void d2_3(I h3d, I h2d, I h1d, I p6d, I p5d, I p4d, I p7d, double *X,
                 const double *t2sub, const double *v2sub) {
#pragma omp parallel for collapse(3) schedule(static)
    for (I p5 = 0; p5 < p5d; p5++)
    for (I p6 = 0; p6 < p6d; p6++)
    for (I h1 = 0; h1 < h1d; h1++)
    for (I p4 = 0; p4 < p4d; p4++)
    for (I h3 = 0; h3 < h3d; h3++)
    for (I h2 = 0; h2 < h2d; h2++)
        D2_BODY(F6(h2, h3, h1, p6, p5, p4, h2d, h3d, h1d, p6d, p5d), +)
}
static void d2_4(I h3d, I h2d, I h1d, I p6d, I p5d, I p4d, I p7d, double *X,
                 const double *t2sub, const double *v2sub) {
#pragma omp parallel for collapse(3) schedule(static)
    for (I p5 = 0; p5 < p5d; p5++)
    for (I p4 = 0; p4 < p4d; p4++)
    for (I p6 = 0; p6 < p6d; p6++)
    for (I h1 = 0; h1 < h1d; h1++)
    for (I h2 = 0; h2 < h2d; h2++)
    for (I h3 = 0; h3 < h3d; h3++)
        D2_BODY(F6(h3, h2, h1, p6, p4, p5, h3d, h2d, h1d, p6d, p4d), +)
}
static void d2_5(I h3d, I h2d, I h1d, I p6d, I p5d, I p4d, I p7d, double *X,
                 const double *t2sub, const double *v2sub) {
#pragma omp parallel for collapse(3) schedule(static)
    for (I p5 = 0; p5 < p5d; p5++)
    for (I p4 = 0; p4 < p4d; p4++)
    for (I p6 = 0; p6 < p6d; p6++)
    for (I h1 = 0; h1 < h1d; h1++)
    for (I h2 = 0; h2 < h2d; h2++)
    for (I h3 = 0; h3 < h3d; h3++)
        D2_BODY(F6(h2, h1, h3, p6, p4, p5, h2d, h1d, h3d, p6d, p4d), +)
}
static void d2_6(I h3d, I h2d, I h1d, I p6d, I p5d, I p4d, I p7d, double *X,
                 const double *t2sub, const double *v2sub) {
#pragma omp parallel for collapse(3) schedule(static)
    for (I p5 = 0; p5 < p5d; p5++)
    for (I p4 = 0; p4 < p4d; p4++)
    for (I p6 = 0; p6 < p6d; p6++)
    for (I h1 = 0; h1 < h1d; h1++)
    for (I h3 = 0; h3 < h3d; h3++)
    for (I h2 = 0; h2 < h2d; h2++)
        D2_BODY(F6(h2, h3, h1, p6, p4, p5, h2d, h3d, h1d, p6d, p4d), -)
}
static void d2_7(I h3d, I h2d, I h1d, I p6d, I p5d, I p4d, I p7d, double *X,
                 const double *t2sub, const double *v2sub) {
#pragma omp parallel for collapse(3) schedule(static)
    for (I p5 = 0; p5 < p5d; p5++)
    for (I p6 = 0; p6 < p6d; p6++)
    for (I p4 = 0; p4 < p4d; p4++)
    for (I h1 = 0; h1 < h1d; h1++)
    for (I h2 = 0; h2 < h2d; h2++)
    for (I h3 = 0; h3 < h3d; h3++)
        D2_BODY(F6(h3, h2, h1, p4, p6, p5, h3d, h2d, h1d, p4d, p6d), -)
}
static void d2_8(I h3d, I h2d, I h1d, I p6d, I p5d, I p4d, I p7d, double *X,
                 const double *t2sub, const double *v2sub) {
#pragma omp parallel for collapse(3) schedule(static)
    for (I p5 = 0; p5 < p5d; p5++)
    for (I p6 = 0; p6 < p6d; p6++)
    for (I p4 = 0; p4 < p4d; p4++)
    for (I h1 = 0; h1 < h1d; h1++)
    for (I h3 = 0; h3 < h3d; h3++)
    for (I h2 = 0; h2 < h2d; h2++)
        D2_BODY(F6(h2, h1, h3, p4, p6, p5, h2d, h1d, h3d, p4d, p6d), -)
}
static void d2_9(I h3d, I h2d, I h1d, I p6d, I p5d, I p4d, I p7d, double *X,
                 const double *t2sub, const double *v2sub) {
#pragma omp parallel for collapse(3) schedule(static)
    for (I p5 = 0; p5 < p5d; p5++)
    for (I p6 = 0; p6 < p6d; p6++)
    for (I h1 = 0; h1 < h1d; h1++)
    for (I h2 = 0; h2 < h2d; h2++)
    for (I p4 = 0; p4 < p4d; p4++)
    for (I h3 = 0; h3 < h3d; h3++)
        D2_BODY(F6(h2, h3, h1, p4, p6, p5, h2d, h3d, h1d, p4d, p6d), +)
}
#undef D2_BODY
#undef T2S
#undef V2S

void orc_sd_t_d2(I k, I h3d, I h2d, I h1d, I p6d, I p5d, I p4d, I p7d,
                 double *triplesx, const double *t2sub, const double *v2sub) {
    typedef void (*fn)(I, I, I, I, I, I, I, double *, const double *,
                       const double *);
    static const fn tab[9] = {d2_1, d2_2, d2_3, d2_4, d2_5,
                              d2_6, d2_7, d2_8, d2_9};
    if (k < 1 || k > 9) return;
    tab[k - 1](h3d, h2d, h1d, p6d, p5d, p4d, p7d, triplesx, t2sub, v2sub);
}

/* ======================================================================
 * Sorts.  tce_sort2.F:1-31 and tce_sort4.F:24-72: the unsorted block is
 * row-major over (a,b[,c,d]); the sorted block is row-major over the
 * dimension order (i,j[,k,l]), each element scaled by factor.
 * ==================================================================== */
void orc_tce_sort_2(const double *unsorted, double *sorted, I a, I b, I i,
                    I j, double factor) {
    I id[2], jd[2] = {a, b};
    I ia = 0;
    for (I j1 = 0; j1 < a; j1++) {
        id[0] = j1;
        for (I j2 = 0; j2 < b; j2++) {
            id[1] = j2;
            I ib = id[j - 1] + jd[j - 1] * id[i - 1];
            sorted[ib] = unsorted[ia] * factor;
            ia++;
        }
    }
}

void orc_tce_sort_4(const double *unsorted, double *sorted, I a, I b, I c,
                    I d, I i, I j, I k, I l, double factor) {
    I id[4], jd[4] = {a, b, c, d};
    for (I j1 = 0; j1 < a; j1++) {
        id[0] = j1;
        for (I j2 = 0; j2 < b; j2++) {
            id[1] = j2;
            for (I j3 = 0; j3 < c; j3++) {
                id[2] = j3;
                for (I j4 = 0; j4 < d; j4++) {
                    id[3] = j4;
                    I ia = id[3] + jd[3] * (id[2] + jd[2] * (id[1] + jd[1] * id[0]));
                    I ib = id[l - 1] + jd[l - 1] * (id[k - 1] + jd[k - 1] *
                           (id[j - 1] + jd[j - 1] * id[i - 1]));
                    sorted[ib] = unsorted[ia] * factor;
                }
            }
        }
    }
}

/* ======================================================================
 * Hash lookup, tce_hash.F:271-316 (binary search narrowing to a linear
 * scan of <= 5 entries).  hash[0] = length.
 * ==================================================================== */
I orc_tce_hash(const I *hash, I key) {
    I length = hash[0];
    if (length <= 0) return -1;
    I less = 1, more = length, middle;
    for (;;) {
        if (more - less <= 4) {
            middle = -1;
            for (I i = less; i <= more; i++)
                if (hash[i] == key) middle = i;
            if (middle == -1) return -1;
            break;
        }
        middle = (less + more) / 2;
        if (hash[middle] == key) break;
        else if (hash[middle] > key) more = middle;
        else less = middle;
    }
    return hash[length + middle];
}

int orc_get_hash_block(const orc_file *f, double *array, I size, I key) {
    I off = orc_tce_hash(f->hash, key);
    if (off < 0) return -1;
    memcpy(array, f->data + off, sizeof(double) * (size_t)size);
    return 0;
}

/* tce_restricted.F:1-71 */
static void restricted_2(const orc_tiling *t, I a1, I a2, I *b1, I *b2) {
    if (t->restricted && t->spin[a1 - 1] + t->spin[a2 - 1] == 4) {
        *b1 = t->alpha[a1 - 1];
        *b2 = t->alpha[a2 - 1];
    } else {
        *b1 = a1;
        *b2 = a2;
    }
}
static void restricted_4(const orc_tiling *t, I a1, I a2, I a3, I a4, I *b1,
                         I *b2, I *b3, I *b4) {
    if (t->restricted && t->spin[a1 - 1] + t->spin[a2 - 1] +
                                 t->spin[a3 - 1] + t->spin[a4 - 1] == 8) {
        *b1 = t->alpha[a1 - 1];
        *b2 = t->alpha[a2 - 1];
        *b3 = t->alpha[a3 - 1];
        *b4 = t->alpha[a4 - 1];
    } else {
        *b1 = a1;
        *b2 = a2;
        *b3 = a3;
        *b4 = a4;
    }
}

#define RNG(b) (t->range[(b) - 1])
#define SPN(b) (t->spin[(b) - 1])
#define SYM(b) (t->sym[(b) - 1])

/* Remove duplicate rows of the 9x6 permutation table
 * (ccsd_t_singles_l.F:161-177; identical in offl_ccsd_t_doubles_l.F). */
static void dedup(I a3[9][6]) {
    for (int ia = 0; ia < 8; ia++) {
        if (a3[ia][0] == 0) continue;
        for (int ja = ia + 1; ja < 9; ja++) {
            int same = 1;
            for (int q = 0; q < 6; q++) same &= (a3[ia][q] == a3[ja][q]);
            if (same)
                for (int q = 0; q < 6; q++) a3[ja][q] = 0;
        }
    }
}

static void fill_row(I a3[9][6], int r, I p4, I p5, I p6, I h1, I h2, I h3) {
    a3[r][0] = p4; a3[r][1] = p5; a3[r][2] = p6;
    a3[r][3] = h1; a3[r][4] = h2; a3[r][5] = h3;
}

static int tuple_ok(const orc_tiling *t, I p4b, I p5b, I p6b, I h1b, I h2b,
                    I h3b) {
    I s = SPN(p4b) + SPN(p5b) + SPN(p6b) + SPN(h1b) + SPN(h2b) + SPN(h3b);
    if (!(!t->restricted || s != 12)) return 0;
    if (SPN(p4b) + SPN(p5b) + SPN(p6b) != SPN(h1b) + SPN(h2b) + SPN(h3b))
        return 0;
    if ((SYM(p4b) ^ SYM(p5b) ^ SYM(p6b) ^ SYM(h1b) ^ SYM(h2b) ^ SYM(h3b)) !=
        (t->irrep_v ^ t->irrep_t))
        return 0;
    return 1;
}

/* ======================================================================
 * ccsd_t_singles_l_1 (ccsd_t_singles_l.F:30-464), plain (non-ACC) branch.
 * ==================================================================== */
static I singles_impl(const orc_tiling *t, const orc_file *t1f,
                      const orc_file *v2f, double *a_c, I t_p4b, I t_p5b,
                      I t_p6b, I t_h1b, I t_h2b, I t_h3b, const orc_hooks *hk) {
    I a3[9][6];
    const I noab = t->noab, nvab = t->nvab, N = noab + nvab;
    fill_row(a3, 0, t_p4b, t_p5b, t_p6b, t_h1b, t_h2b, t_h3b);
    fill_row(a3, 1, t_p4b, t_p5b, t_p6b, t_h2b, t_h1b, t_h3b);
    fill_row(a3, 2, t_p4b, t_p5b, t_p6b, t_h3b, t_h1b, t_h2b);
    fill_row(a3, 3, t_p5b, t_p4b, t_p6b, t_h1b, t_h2b, t_h3b);
    fill_row(a3, 4, t_p5b, t_p4b, t_p6b, t_h2b, t_h1b, t_h3b);
    fill_row(a3, 5, t_p5b, t_p4b, t_p6b, t_h3b, t_h1b, t_h2b);
    fill_row(a3, 6, t_p6b, t_p4b, t_p5b, t_h1b, t_h2b, t_h3b);
    fill_row(a3, 7, t_p6b, t_p4b, t_p5b, t_h2b, t_h1b, t_h3b);
    fill_row(a3, 8, t_p6b, t_p4b, t_p5b, t_h3b, t_h1b, t_h2b);
    dedup(a3);
    I ncalls = 0;
    for (int ia6 = 0; ia6 < 9; ia6++) {
        I p4b = a3[ia6][0], p5b = a3[ia6][1], p6b = a3[ia6][2];
        I h1b = a3[ia6][3], h2b = a3[ia6][4], h3b = a3[ia6][5];
        if (!((p5b <= p6b) && (h2b <= h3b) && (p4b != 0))) continue;
        if (!tuple_ok(t, p4b, p5b, p6b, h1b, h2b, h3b)) continue;
        if (SPN(p4b) != SPN(h1b)) continue;
        if ((SYM(p4b) ^ SYM(h1b)) != t->irrep_t) continue;
        I p4b_1, h1b_1, p5b_2, p6b_2, h2b_2, h3b_2;
        restricted_2(t, p4b, h1b, &p4b_1, &h1b_1);
        restricted_4(t, p5b, p6b, h2b, h3b, &p5b_2, &p6b_2, &h2b_2, &h3b_2);
        I dima = RNG(p4b) * RNG(h1b);
        I dimb = RNG(p5b) * RNG(p6b) * RNG(h2b) * RNG(h3b);
        if (!(dima > 0 && dimb > 0)) continue;
        double *a = (double *)malloc(sizeof(double) * (size_t)dima);
        double *a_sort = (double *)malloc(sizeof(double) * (size_t)dima);
        double *b_sort = (double *)malloc(sizeof(double) * (size_t)dimb);
        if (!a || !a_sort || !b_sort) { free(a); free(a_sort); free(b_sort); return -1; }
        int rc = orc_get_hash_block(t1f, a, dima, h1b_1 - 1 + noab * (p4b_1 - noab - 1));
        if (rc == 0) {
            orc_tce_sort_2(a, a_sort, RNG(p4b), RNG(h1b), 2, 1, 1.0);
            rc = orc_get_hash_block(v2f, b_sort, dimb,
                    h3b_2 - 1 + N * (h2b_2 - 1 + N * (p6b_2 - 1 + N * (p5b_2 - 1))));
        }
        free(a);
        if (rc != 0) { free(a_sort); free(b_sort); return -1; }
        const I h3d = RNG(h3b), h2d = RNG(h2b), h1d = RNG(h1b);
        const I p6d = RNG(p6b), p5d = RNG(p5b), p4d = RNG(p4b);
#define S1CALL(k) do { \
            if (hk) { const I dd[6] = {h1d, h2d, h3d, p4d, p5d, p6d}; hk->s1(hk->user, k, dd, a_sort, b_sort); } \
            else orc_sd_t_s1(k, h3d, h2d, h1d, p6d, p5d, p4d, a_c, a_sort, b_sort); \
            ncalls++; } while (0)
        if (t_p4b == p4b && t_p5b == p5b && t_p6b == p6b && t_h1b == h1b && t_h2b == h2b && t_h3b == h3b) S1CALL(1);
        if (t_p4b == p4b && t_p5b == p5b && t_p6b == p6b && t_h1b == h2b && t_h2b == h1b && t_h3b == h3b) S1CALL(2);
        if (t_p4b == p4b && t_p5b == p5b && t_p6b == p6b && t_h1b == h2b && t_h2b == h3b && t_h3b == h1b) S1CALL(3);
        if (t_p4b == p5b && t_p5b == p4b && t_p6b == p6b && t_h1b == h1b && t_h2b == h2b && t_h3b == h3b) S1CALL(4);
        if (t_p4b == p5b && t_p5b == p4b && t_p6b == p6b && t_h1b == h2b && t_h2b == h1b && t_h3b == h3b) S1CALL(5);
        if (t_p4b == p5b && t_p5b == p4b && t_p6b == p6b && t_h1b == h2b && t_h2b == h3b && t_h3b == h1b) S1CALL(6);
        if (t_p4b == p5b && t_p5b == p6b && t_p6b == p4b && t_h1b == h1b && t_h2b == h2b && t_h3b == h3b) S1CALL(7);
        if (t_p4b == p5b && t_p5b == p6b && t_p6b == p4b && t_h1b == h2b && t_h2b == h1b && t_h3b == h3b) S1CALL(8);
        if (t_p4b == p5b && t_p5b == p6b && t_p6b == p4b && t_h1b == h2b && t_h2b == h3b && t_h3b == h1b) S1CALL(9);
#undef S1CALL
        free(a_sort);
        free(b_sort);
    }
    return ncalls;
}

I orc_singles_l_1(const orc_tiling *t, const orc_file *t1f,
                  const orc_file *v2f, double *a_c, I t_p4b, I t_p5b,
                  I t_p6b, I t_h1b, I t_h2b, I t_h3b) {
    return singles_impl(t, t1f, v2f, a_c, t_p4b, t_p5b, t_p6b, t_h1b, t_h2b, t_h3b, NULL);
}

/* ======================================================================
 * tce_hashnsort (tce_hashnsort.F:1-87): d1 block test, T2 fetch+sort to
 * t2sub(h7,p4,p5,h1) and V2 (h7,p6,h2,h3) fetch.  Returns 1 when the block
 * pair exists (spin/sym allowed), 0 when not, -1 on a missing block.
 * ==================================================================== */
static int hashnsort(const orc_tiling *t, int dryrun, const orc_file *d_a,
                     const orc_file *d_b, I p4b, I p5b, I h1b, I h7b, I p6b,
                     I h2b, I h3b, double *t2sub, double *v2sub) {
    const I noab = t->noab, nvab = t->nvab, N = noab + nvab;
    if (!((SPN(p4b) + SPN(p5b) == SPN(h1b) + SPN(h7b)) &&
          ((SYM(p4b) ^ SYM(p5b) ^ SYM(h1b) ^ SYM(h7b)) == t->irrep_t)))
        return 0;
    I dima = RNG(h7b) * RNG(p4b) * RNG(p5b) * RNG(h1b);
    I dimb = RNG(h7b) * RNG(p6b) * RNG(h2b) * RNG(h3b);
    if (!dryrun && dima > 0 && dimb > 0) {
        I p4b_1, p5b_1, h1b_1, h7b_1, p6b_2, h7b_2, h2b_2, h3b_2;
        restricted_4(t, p4b, p5b, h1b, h7b, &p4b_1, &p5b_1, &h1b_1, &h7b_1);
        restricted_4(t, p6b, h7b, h2b, h3b, &p6b_2, &h7b_2, &h2b_2, &h3b_2);
        double *a = (double *)malloc(sizeof(double) * (size_t)dima);
        if (!a) return -1;
        int rc = 0;
        if (h7b < h1b) {
            rc = orc_get_hash_block(d_a, a, dima,
                    h1b_1 - 1 + noab * (h7b_1 - 1 + noab * (p5b_1 - noab - 1 + nvab * (p4b_1 - noab - 1))));
            if (rc == 0)
                orc_tce_sort_4(a, t2sub, RNG(p4b), RNG(p5b), RNG(h7b), RNG(h1b), 4, 2, 1, 3, -1.0);
        }
        if (rc == 0 && h1b <= h7b) {
            rc = orc_get_hash_block(d_a, a, dima,
                    h7b_1 - 1 + noab * (h1b_1 - 1 + noab * (p5b_1 - noab - 1 + nvab * (p4b_1 - noab - 1))));
            if (rc == 0)
                orc_tce_sort_4(a, t2sub, RNG(p4b), RNG(p5b), RNG(h1b), RNG(h7b), 3, 2, 1, 4, 1.0);
        }
        free(a);
        if (rc != 0) return -1;
        if (h7b <= p6b) {
            rc = orc_get_hash_block(d_b, v2sub, dimb,
                    h3b_2 - 1 + N * (h2b_2 - 1 + N * (p6b_2 - 1 + N * (h7b_2 - 1))));
            if (rc != 0) return -1;
        }
    }
    return 1;
}

/* tce_hashnsort_2 (tce_hashnsort.F:88-173): d2 block test, T2 fetch+sort
 * to t2sub(p7,p4,h1,h2) and V2 (p5,p6,h3,p7) fetch. */
static int hashnsort_2(const orc_tiling *t, int dryrun, const orc_file *d_a,
                       const orc_file *d_b, I p4b, I p7b, I h1b, I h2b,
                       I p5b, I p6b, I h3b, double *t2sub, double *v2sub) {
    const I noab = t->noab, nvab = t->nvab, N = noab + nvab;
    if (!((SPN(p4b) + SPN(p7b) == SPN(h1b) + SPN(h2b)) &&
          ((SYM(p4b) ^ SYM(p7b) ^ SYM(h1b) ^ SYM(h2b)) == t->irrep_t)))
        return 0;
    I dima = RNG(p7b) * RNG(p4b) * RNG(h1b) * RNG(h2b);
    I dimb = RNG(p7b) * RNG(p5b) * RNG(p6b) * RNG(h3b);
    if (!dryrun && dima > 0 && dimb > 0) {
        I p4b_1, p7b_1, h1b_1, h2b_1, p5b_2, p6b_2, h3b_2, p7b_2;
        restricted_4(t, p4b, p7b, h1b, h2b, &p4b_1, &p7b_1, &h1b_1, &h2b_1);
        restricted_4(t, p5b, p6b, h3b, p7b, &p5b_2, &p6b_2, &h3b_2, &p7b_2);
        double *a = (double *)malloc(sizeof(double) * (size_t)dima);
        if (!a) return -1;
        int rc = 0;
        if (p7b < p4b) {
            rc = orc_get_hash_block(d_a, a, dima,
                    h2b_1 - 1 + noab * (h1b_1 - 1 + noab * (p4b_1 - noab - 1 + nvab * (p7b_1 - noab - 1))));
            if (rc == 0)
                orc_tce_sort_4(a, t2sub, RNG(p7b), RNG(p4b), RNG(h1b), RNG(h2b), 4, 3, 2, 1, -1.0);
        }
        if (rc == 0 && p4b <= p7b) {
            rc = orc_get_hash_block(d_a, a, dima,
                    h2b_1 - 1 + noab * (h1b_1 - 1 + noab * (p7b_1 - noab - 1 + nvab * (p4b_1 - noab - 1))));
            if (rc == 0)
                orc_tce_sort_4(a, t2sub, RNG(p4b), RNG(p7b), RNG(h1b), RNG(h2b), 4, 3, 1, 2, 1.0);
        }
        free(a);
        if (rc != 0) return -1;
        if (h3b <= p7b) {
            rc = orc_get_hash_block(d_b, v2sub, dimb,
                    p7b_2 - 1 + N * (h3b_2 - 1 + N * (p6b_2 - 1 + N * (p5b_2 - 1))));
            if (rc != 0) return -1;
        }
    }
    return 1;
}

/* ======================================================================
 * ccsd_t_doubles_l_12 (offl_ccsd_t_doubles_l.F:72-1020), non-offload,
 * non-ACC branch.  The reference dispatches to sdtransp_t_d*_k there; those
 * compute the same sums as ccsd_t_kernels_omp.F's sd_t_d*_k with other
 * loop orders, and the oracle calls the sd_t_* restatements.
 * ==================================================================== */
static I doubles_impl(const orc_tiling *t, const orc_file *t2f,
                      const orc_file *v2f, double *triplesx, I t_p4b, I t_p5b,
                      I t_p6b, I t_h1b, I t_h2b, I t_h3b, I *calls,
                      const orc_hooks *hk) {
    const I noab = t->noab, nvab = t->nvab;
    I maxo = 0, maxv = 0;
    for (I b = 1; b <= noab; b++) if (RNG(b) > maxo) maxo = RNG(b);
    for (I b = noab + 1; b <= noab + nvab; b++) if (RNG(b) > maxv) maxv = RNG(b);
    /* ccsd_t_v2t2lgth (ccsd_t_doubles_l.F:118-141): the largest sub-block */
    size_t l_t2 = (size_t)maxv * maxv * maxo * maxo;
    size_t l_v2 = (size_t)maxv * maxv * maxv * maxo;
    if ((size_t)maxo * maxo * maxo * maxv > l_v2) l_v2 = (size_t)maxo * maxo * maxo * maxv;
    double *t2sub = (double *)malloc(sizeof(double) * (l_t2 + 1));
    double *v2sub = (double *)malloc(sizeof(double) * (l_v2 + 1));
    if (!t2sub || !v2sub) { free(t2sub); free(v2sub); return -1; }
    I a3[9][6];

    /* ---- d1 part: table at offl_ccsd_t_doubles_l.F:176-229 ---- */
    fill_row(a3, 0, t_p4b, t_p5b, t_p6b, t_h1b, t_h2b, t_h3b);
    fill_row(a3, 1, t_p4b, t_p5b, t_p6b, t_h2b, t_h1b, t_h3b);
    fill_row(a3, 2, t_p4b, t_p5b, t_p6b, t_h3b, t_h1b, t_h2b);
    fill_row(a3, 3, t_p5b, t_p6b, t_p4b, t_h1b, t_h2b, t_h3b);
    fill_row(a3, 4, t_p5b, t_p6b, t_p4b, t_h2b, t_h1b, t_h3b);
    fill_row(a3, 5, t_p5b, t_p6b, t_p4b, t_h3b, t_h1b, t_h2b);
    fill_row(a3, 6, t_p4b, t_p6b, t_p5b, t_h1b, t_h2b, t_h3b);
    fill_row(a3, 7, t_p4b, t_p6b, t_p5b, t_h2b, t_h1b, t_h3b);
    fill_row(a3, 8, t_p4b, t_p6b, t_p5b, t_h3b, t_h1b, t_h2b);
    dedup(a3);
    for (int ia6 = 0; ia6 < 9; ia6++) {
        I p4b = a3[ia6][0], p5b = a3[ia6][1], p6b = a3[ia6][2];
        I h1b = a3[ia6][3], h2b = a3[ia6][4], h3b = a3[ia6][5];
        if (!((p4b <= p5b) && (h2b <= h3b) && (p4b != 0))) continue;
        if (!tuple_ok(t, p4b, p5b, p6b, h1b, h2b, h3b)) continue;
        const I h3d = RNG(h3b), h2d = RNG(h2b), h1d = RNG(h1b);
        const I p6d = RNG(p6b), p5d = RNG(p5b), p4d = RNG(p4b);
        I n_h7b = 0;
        for (I h7b = 1; h7b <= noab; h7b++)
            if (hashnsort(t, 1, t2f, v2f, p4b, p5b, h1b, h7b, p6b, h2b, h3b, t2sub, v2sub) == 1)
                n_h7b++;
        if (n_h7b == 0) continue;
        for (I h7b = 1; h7b <= noab; h7b++) {
            int rc = hashnsort(t, 0, t2f, v2f, p4b, p5b, h1b, h7b, p6b, h2b, h3b, t2sub, v2sub);
            if (rc < 0) { free(t2sub); free(v2sub); return -1; }
            if (rc == 0) continue;
            const I h7d = RNG(h7b);
#define D1CALL(k) do { \
                if (hk) { const I dd[7] = {h1d, h2d, h3d, h7d, p4d, p5d, p6d}; hk->d1(hk->user, k, dd, t2sub, v2sub); } \
                else orc_sd_t_d1(k, h3d, h2d, h1d, p6d, p5d, p4d, h7d, triplesx, t2sub, v2sub); \
                calls[0]++; } while (0)
            if (t_p4b == p4b && t_p5b == p5b && t_p6b == p6b && t_h1b == h1b && t_h2b == h2b && t_h3b == h3b) D1CALL(1);
            if (t_p4b == p4b && t_p5b == p5b && t_p6b == p6b && t_h1b == h2b && t_h2b == h1b && t_h3b == h3b) D1CALL(2);
            if (t_p4b == p4b && t_p5b == p5b && t_p6b == p6b && t_h1b == h2b && t_h2b == h3b && t_h3b == h1b) D1CALL(3);
            if (t_p4b == p6b && t_p5b == p4b && t_p6b == p5b && t_h1b == h1b && t_h2b == h2b && t_h3b == h3b) D1CALL(4);
            if (t_p4b == p6b && t_p5b == p4b && t_p6b == p5b && t_h1b == h2b && t_h2b == h1b && t_h3b == h3b) D1CALL(5);
            if (t_p4b == p6b && t_p5b == p4b && t_p6b == p5b && t_h1b == h2b && t_h2b == h3b && t_h3b == h1b) D1CALL(6);
            if (t_p4b == p4b && t_p5b == p6b && t_p6b == p5b && t_h1b == h1b && t_h2b == h2b && t_h3b == h3b) D1CALL(7);
            if (t_p4b == p4b && t_p5b == p6b && t_p6b == p5b && t_h1b == h2b && t_h2b == h1b && t_h3b == h3b) D1CALL(8);
            if (t_p4b == p4b && t_p5b == p6b && t_p6b == p5b && t_h1b == h2b && t_h2b == h3b && t_h3b == h1b) D1CALL(9);
#undef D1CALL
        }
    }

    /* ---- d2 part: table at offl_ccsd_t_doubles_l.F:611-664 ---- */
    fill_row(a3, 0, t_p4b, t_p5b, t_p6b, t_h1b, t_h2b, t_h3b);
    fill_row(a3, 1, t_p4b, t_p5b, t_p6b, t_h2b, t_h3b, t_h1b);
    fill_row(a3, 2, t_p4b, t_p5b, t_p6b, t_h1b, t_h3b, t_h2b);
    fill_row(a3, 3, t_p5b, t_p4b, t_p6b, t_h1b, t_h2b, t_h3b);
    fill_row(a3, 4, t_p5b, t_p4b, t_p6b, t_h2b, t_h3b, t_h1b);
    fill_row(a3, 5, t_p5b, t_p4b, t_p6b, t_h1b, t_h3b, t_h2b);
    fill_row(a3, 6, t_p6b, t_p4b, t_p5b, t_h1b, t_h2b, t_h3b);
    fill_row(a3, 7, t_p6b, t_p4b, t_p5b, t_h2b, t_h3b, t_h1b);
    fill_row(a3, 8, t_p6b, t_p4b, t_p5b, t_h1b, t_h3b, t_h2b);
    dedup(a3);
    for (int ia6 = 0; ia6 < 9; ia6++) {
        I p4b = a3[ia6][0], p5b = a3[ia6][1], p6b = a3[ia6][2];
        I h1b = a3[ia6][3], h2b = a3[ia6][4], h3b = a3[ia6][5];
        if (!((p5b <= p6b) && (h1b <= h2b) && (p4b != 0))) continue;
        if (!tuple_ok(t, p4b, p5b, p6b, h1b, h2b, h3b)) continue;
        const I h3d = RNG(h3b), h2d = RNG(h2b), h1d = RNG(h1b);
        const I p6d = RNG(p6b), p5d = RNG(p5b), p4d = RNG(p4b);
        I n_p7b = 0;
        for (I p7b = noab + 1; p7b <= noab + nvab; p7b++)
            if (hashnsort_2(t, 1, t2f, v2f, p4b, p7b, h1b, h2b, p5b, p6b, h3b, t2sub, v2sub) == 1)
                n_p7b++;
        if (n_p7b == 0) continue;
        for (I p7b = noab + 1; p7b <= noab + nvab; p7b++) {
            int rc = hashnsort_2(t, 0, t2f, v2f, p4b, p7b, h1b, h2b, p5b, p6b, h3b, t2sub, v2sub);
            if (rc < 0) { free(t2sub); free(v2sub); return -1; }
            if (rc == 0) continue;
            const I p7d = RNG(p7b);
#define D2CALL(k) do { \
                if (hk) { const I dd[7] = {h1d, h2d, h3d, p4d, p5d, p6d, p7d}; hk->d2(hk->user, k, dd, t2sub, v2sub); } \
                else orc_sd_t_d2(k, h3d, h2d, h1d, p6d, p5d, p4d, p7d, triplesx, t2sub, v2sub); \
                calls[1]++; } while (0)
            if (t_p4b == p4b && t_p5b == p5b && t_p6b == p6b && t_h1b == h1b && t_h2b == h2b && t_h3b == h3b) D2CALL(1);
            if (t_p4b == p4b && t_p5b == p5b && t_p6b == p6b && t_h1b == h3b && t_h2b == h1b && t_h3b == h2b) D2CALL(2);
            if (t_p4b == p4b && t_p5b == p5b && t_p6b == p6b && t_h1b == h1b && t_h2b == h3b && t_h3b == h2b) D2CALL(3);
            if (t_p4b == p5b && t_p5b == p4b && t_p6b == p6b && t_h1b == h1b && t_h2b == h2b && t_h3b == h3b) D2CALL(4);
            if (t_p4b == p5b && t_p5b == p4b && t_p6b == p6b && t_h1b == h3b && t_h2b == h1b && t_h3b == h2b) D2CALL(5);
            if (t_p4b == p5b && t_p5b == p4b && t_p6b == p6b && t_h1b == h1b && t_h2b == h3b && t_h3b == h2b) D2CALL(6);
            if (t_p4b == p5b && t_p5b == p6b && t_p6b == p4b && t_h1b == h1b && t_h2b == h2b && t_h3b == h3b) D2CALL(7);
            if (t_p4b == p5b && t_p5b == p6b && t_p6b == p4b && t_h1b == h3b && t_h2b == h1b && t_h3b == h2b) D2CALL(8);
            if (t_p4b == p5b && t_p5b == p6b && t_p6b == p4b && t_h1b == h1b && t_h2b == h3b && t_h3b == h2b) D2CALL(9);
#undef D2CALL
        }
    }
    free(t2sub);
    free(v2sub);
    return 0;
}

I orc_doubles_l_12(const orc_tiling *t, const orc_file *t2f,
                   const orc_file *v2f, double *triplesx, I t_p4b, I t_p5b,
                   I t_p6b, I t_h1b, I t_h2b, I t_h3b, I *calls) {
    return doubles_impl(t, t2f, v2f, triplesx, t_p4b, t_p5b, t_p6b, t_h1b,
                        t_h2b, t_h3b, calls, NULL);
}

I orc_tuple_drive(const orc_tiling *t, const orc_file *t1f,
                  const orc_file *t2f, const orc_file *v2f, const I *tp,
                  const orc_hooks *hooks, I *calls3) {
    I ns = singles_impl(t, t1f, v2f, NULL, tp[0], tp[1], tp[2], tp[3], tp[4], tp[5], hooks);
    if (ns < 0) return -1;
    I cd[2] = {0, 0};
    if (doubles_impl(t, t2f, v2f, NULL, tp[0], tp[1], tp[2], tp[3], tp[4], tp[5], cd, hooks) < 0)
        return -1;
    if (calls3) { calls3[0] = ns; calls3[1] = cd[0]; calls3[2] = cd[1]; }
    return 0;
}

/* ======================================================================
 * ccsd_t_dot (ccsd_t_dot.F:20-138).  Same loop order and per-element
 * arithmetic; the two sums are Neumaier-compensated.  The reference sums
 * with an OpenMP reduction, whose order is unspecified, so the oracle removes
 * the order-dependent rounding instead of picking one order.
 * ==================================================================== */
typedef struct { double s, c; } comp_t;
static void comp_add(comp_t *a, double x) {
    double t = a->s + x;
    if (fabs(a->s) >= fabs(x)) a->c += (a->s - t) + x;
    else a->c += (x - t) + a->s;
    a->s = t;
}

void orc_ccsd_t_dot(const double *a_singles, const double *a_doubles,
                    I restricted, I h1b, I h2b, I h3b, I p4b, I p5b, I p6b,
                    const double *o_h1, const double *o_h2, const double *o_h3,
                    const double *o_p4, const double *o_p5, const double *o_p6,
                    I r_h1, I r_h2, I r_h3, I r_p4, I r_p5, I r_p6,
                    double *energy1, double *energy2) {
    double factor = restricted ? 2.0 : 1.0;
    if (p4b == p5b && p5b == p6b) factor = factor / 6.0;
    else if (p4b == p5b || p5b == p6b) factor = factor / 2.0;
    if (h1b == h2b && h2b == h3b) factor = factor / 6.0;
    else if (h1b == h2b || h2b == h3b) factor = factor / 2.0;
    comp_t e1 = {*energy1, 0.0}, e2 = {*energy2, 0.0};
    for (I p4 = 0; p4 < r_p4; p4++)
    for (I p5 = 0; p5 < r_p5; p5++)
    for (I p6 = 0; p6 < r_p6; p6++) {
        double d_p4 = o_p4[p4], d_p5 = o_p5[p5], d_p6 = o_p6[p6];
        double denom_0 = -(d_p4 + d_p5 + d_p6);
        for (I h1 = 0; h1 < r_h1; h1++) {
            double d_h1 = o_h1[h1];
            for (I h2 = 0; h2 < r_h2; h2++) {
                double d_h2 = o_h2[h2];
                for (I h3 = 0; h3 < r_h3; h3++) {
                    double d_h3 = o_h3[h3];
                    I x = F6(h3, h2, h1, p6, p5, p4, r_h3, r_h2, r_h1, r_p6, r_p5);
                    double sing = a_singles[x];
                    double doub = a_doubles[x];
                    double denom = doub * factor / (d_h1 + d_h2 + d_h3 + denom_0);
                    comp_add(&e1, denom * doub);
                    comp_add(&e2, denom * (doub + sing));
                }
            }
        }
    }
    *energy1 = e1.s + e1.c;
    *energy2 = e2.s + e2.c;
}

/* ======================================================================
 * Tuple enumeration (ccsd_t_neword.F:1-217).
 * ==================================================================== */
static int task_ok(const orc_tiling *t, I p4, I p5, I p6, I h1, I h2, I h3) {
    if (SPN(p4) + SPN(p5) + SPN(p6) != SPN(h1) + SPN(h2) + SPN(h3)) return 0;
    if (!(!t->restricted ||
          SPN(p4) + SPN(p5) + SPN(p6) + SPN(h1) + SPN(h2) + SPN(h3) <= 8))
        return 0;
    if ((SYM(p4) ^ SYM(p5) ^ SYM(p6) ^ SYM(h1) ^ SYM(h2) ^ SYM(h3)) != 0) return 0;
    return 1;
}

I orc_6tasks(const orc_tiling *t) {
    const I noab = t->noab, nvab = t->nvab;
    I n = 0;
    for (I p4 = noab + 1; p4 <= noab + nvab; p4++)
    for (I p5 = p4; p5 <= noab + nvab; p5++)
    for (I p6 = p5; p6 <= noab + nvab; p6++)
    for (I h1 = 1; h1 <= noab; h1++)
    for (I h2 = h1; h2 <= noab; h2++)
    for (I h3 = h2; h3 <= noab; h3++)
        n += task_ok(t, p4, p5, p6, h1, h2, h3);
    return n;
}

/* ccsd_sillysort (ccsd_t_neword.F:218-244) */
static void sillysort(I value, I *kaux, I *klist, I n, I *found) {
    for (I m = 0; m < n; m++) {
        if (kaux[7 * m + 6] > value) {
            for (int j = 0; j < 7; j++) klist[7 * (*found) + j] = kaux[7 * m + j];
            (*found)++;
            kaux[7 * m + 6] = -99;
        }
    }
}

I orc_neword(const orc_tiling *t, I tot, I *klist) {
    const I noab = t->noab, nvab = t->nvab;
    I *kaux = (I *)malloc(sizeof(I) * (size_t)(7 * tot + 7));
    if (!kaux) return -2;
    I m = 0;
    for (I p4 = noab + 1; p4 <= noab + nvab; p4++)
    for (I p5 = p4; p5 <= noab + nvab; p5++)
    for (I p6 = p5; p6 <= noab + nvab; p6++)
    for (I h1 = 1; h1 <= noab; h1++)
    for (I h2 = h1; h2 <= noab; h2++)
    for (I h3 = h2; h3 <= noab; h3++) {
        if (!task_ok(t, p4, p5, p6, h1, h2, h3)) continue;
        if (m >= tot) { free(kaux); return -1; }
        I *r = kaux + 7 * m;
        r[0] = p4; r[1] = p5; r[2] = p6; r[3] = h1; r[4] = h2; r[5] = h3;
        r[6] = RNG(p4) * RNG(p5) * RNG(p6) * RNG(h1) * RNG(h2) * RNG(h3);
        m++;
    }
    if (m != tot) { free(kaux); return -1; }
    I wl_max = 0, wl_min;
    for (I q = 0; q < tot; q++) if (kaux[7 * q + 6] > wl_max) wl_max = kaux[7 * q + 6];
    wl_min = wl_max;
    for (I q = 0; q < tot; q++) if (kaux[7 * q + 6] < wl_min) wl_min = kaux[7 * q + 6];
    /* all tiles (nearly) the same: keep enumeration order (:134-142) */
    if (tot == 0 || ((double)(wl_max - wl_min) * 100.0) / (double)wl_max < 1.0) {
        memcpy(klist, kaux, sizeof(I) * (size_t)(7 * tot));
        free(kaux);
        return 0;
    }
    for (I q = 0; q < 7 * tot; q++) klist[q] = -1;
    I found = 0;
    const I nsplits = 16;
    for (I ii = nsplits; ii >= 1; ii--) {
        I w_in = wl_min + ((wl_max - wl_min) * (ii - 1)) / nsplits;
        sillysort(w_in, kaux, klist, tot, &found);
    }
    sillysort(0, kaux, klist, tot, &found);
    free(kaux);
    return found == tot ? 0 : -1;
}

/* ======================================================================
 * ccsd_t_loop (ccsd_t.F:358-456) over a task list, energies summed in task
 * order (the reference sums per rank, then ga_dgop, ccsd_t.F:297).
 * ==================================================================== */
static I tuple_tiles(const orc_tiling *t, const orc_file *t1f,
                     const orc_file *t2f, const orc_file *v2f, const I *tp,
                     double *singles, double *doubles, I *calls3) {
    const I t_p4b = tp[0], t_p5b = tp[1], t_p6b = tp[2];
    const I t_h1b = tp[3], t_h2b = tp[4], t_h3b = tp[5];
    const size_t size = (size_t)(RNG(t_p4b) * RNG(t_p5b) * RNG(t_p6b) *
                                 RNG(t_h1b) * RNG(t_h2b) * RNG(t_h3b));
    memset(singles, 0, sizeof(double) * size);
    memset(doubles, 0, sizeof(double) * size);
    I ns = orc_singles_l_1(t, t1f, v2f, singles, t_p4b, t_p5b, t_p6b, t_h1b, t_h2b, t_h3b);
    if (ns < 0) return -1;
    I cd[2] = {0, 0};
    if (orc_doubles_l_12(t, t2f, v2f, doubles, t_p4b, t_p5b, t_p6b, t_h1b, t_h2b, t_h3b, cd) < 0)
        return -1;
    if (calls3) { calls3[0] = ns; calls3[1] = cd[0]; calls3[2] = cd[1]; }
    return 0;
}

I orc_tuple_tiles(const orc_tiling *t, const orc_file *t1f,
                  const orc_file *t2f, const orc_file *v2f, const I *tuple6,
                  double *singles, double *doubles) {
    return tuple_tiles(t, t1f, t2f, v2f, tuple6, singles, doubles, NULL);
}

I orc_ccsd_t(const orc_tiling *t, const orc_file *t1f, const orc_file *t2f,
             const orc_file *v2f, const I *klist, I tot, const I *task_ids,
             I n, double *energy, double *per_task, I *kernel_calls) {
    if (!task_ids) n = tot;
    size_t maxsize = 1;
    for (I q = 0; q < n; q++) {
        I id = task_ids ? task_ids[q] : q;
        if (id < 0 || id >= tot) return -1;
        size_t w = (size_t)klist[7 * id + 6];
        if (w > maxsize) maxsize = w;
    }
    double *singles = (double *)malloc(sizeof(double) * maxsize);
    double *doubles = (double *)malloc(sizeof(double) * maxsize);
    if (!singles || !doubles) { free(singles); free(doubles); return -2; }
    comp_t e1 = {0.0, 0.0}, e2 = {0.0, 0.0};
    for (I q = 0; q < n; q++) {
        I id = task_ids ? task_ids[q] : q;
        const I *tp = klist + 7 * id;
        I c3[3];
        if (tuple_tiles(t, t1f, t2f, v2f, tp, singles, doubles, c3) < 0) {
            free(singles); free(doubles);
            return -1;
        }
        const I t_p4b = tp[0], t_p5b = tp[1], t_p6b = tp[2];
        const I t_h1b = tp[3], t_h2b = tp[4], t_h3b = tp[5];
        double te1 = 0.0, te2 = 0.0;
        const double *ev = t->evl_sorted;
        orc_ccsd_t_dot(singles, doubles, t->restricted, t_h1b, t_h2b, t_h3b,
                       t_p4b, t_p5b, t_p6b,
                       ev + t->offset[t_h1b - 1], ev + t->offset[t_h2b - 1],
                       ev + t->offset[t_h3b - 1], ev + t->offset[t_p4b - 1],
                       ev + t->offset[t_p5b - 1], ev + t->offset[t_p6b - 1],
                       RNG(t_h1b), RNG(t_h2b), RNG(t_h3b), RNG(t_p4b),
                       RNG(t_p5b), RNG(t_p6b), &te1, &te2);
        comp_add(&e1, te1);
        comp_add(&e2, te2);
        if (per_task) { per_task[2 * q] = te1; per_task[2 * q + 1] = te2; }
        if (kernel_calls) {
            kernel_calls[3 * q] = c3[0];
            kernel_calls[3 * q + 1] = c3[1];
            kernel_calls[3 * q + 2] = c3[2];
        }
    }
    free(singles);
    free(doubles);
    energy[0] = e1.s + e1.c;
    energy[1] = e2.s + e2.c;
    return 0;
}
