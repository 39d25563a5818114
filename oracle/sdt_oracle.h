/*
 * sdt_oracle.h -- CPU oracle for the CCSD(T) perturbative-triples tile path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of NWChem's TCE
 * (T) Fortran code, used as the checker for the CUDA path.  Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg load it; the
 * product library (nwchem_gb300) never links or calls it.
 *
 * Parity status: the reference's Fortran kernels cannot be compiled here (no
 * Fortran compiler) and the reference ships no kernel-level golden vectors;
 * the oracle is pinned by the self-consistency known answers in
 * tests/golden/ (re-tiling invariance, antisymmetry, hand-derived tiny
 * cases) -- see the header of sdt_oracle.c for what each function follows.
 *
 * Conventions: every integer is 64-bit (the reference is built -i8, header.h:51).
 * Tiles are numbered 1..noab (occupied) then noab+1..noab+nvab (virtual)
 * exactly as src/tce/include/tce.fh:14-21.
 */
#ifndef SDT_ORACLE_H
#define SDT_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Tile description (src/tce/tce_tile.F:1238-1335).  Arrays are indexed by
 * tile-1.  alpha[] is k_alpha (restricted beta->alpha tile map). */
typedef struct {
    int64_t noab, nvab;
    const int64_t *range;
    const int64_t *spin;
    const int64_t *sym;
    const int64_t *offset;      /* offset of the tile into evl_sorted */
    const int64_t *alpha;       /* may be NULL when restricted == 0 */
    const double  *evl_sorted;
    int64_t restricted;
    int64_t irrep_t, irrep_v;   /* both 0 for ground-state (T) */
} orc_tiling;

/* A TCE "file": hash table in the tce_hash layout (hash[0] = n, keys in
 * hash[1..n] ascending, offsets in hash[n+1..2n]) plus the block data. */
typedef struct {
    const int64_t *hash;
    const double  *data;
} orc_file;

/* ---- the 27 tile kernels (ccsd_t_kernels_omp.F) ----------------------
 * Arguments follow the Fortran CPU dialect: dims of the permuted block in
 * the order (h3d,h2d,h1d,p6d,p5d,p4d[,h7d|p7d]).  k = 1..9. */
void orc_sd_t_s1(int64_t k, int64_t h3d, int64_t h2d, int64_t h1d,
                 int64_t p6d, int64_t p5d, int64_t p4d,
                 double *triplesx, const double *t1sub, const double *v2sub);
void orc_sd_t_d1(int64_t k, int64_t h3d, int64_t h2d, int64_t h1d,
                 int64_t p6d, int64_t p5d, int64_t p4d, int64_t h7d,
                 double *triplesx, const double *t2sub, const double *v2sub);
void orc_sd_t_d2(int64_t k, int64_t h3d, int64_t h2d, int64_t h1d,
                 int64_t p6d, int64_t p5d, int64_t p4d, int64_t p7d,
                 double *triplesx, const double *t2sub, const double *v2sub);

/* ---- sorts and block fetch -------------------------------------------- */
void orc_tce_sort_2(const double *unsorted, double *sorted, int64_t a,
                    int64_t b, int64_t i, int64_t j, double factor);
void orc_tce_sort_4(const double *unsorted, double *sorted, int64_t a,
                    int64_t b, int64_t c, int64_t d, int64_t i, int64_t j,
                    int64_t k, int64_t l, double factor);
/* Returns the block offset for key, or -1 when the key is absent (the
 * reference calls errquit there). */
int64_t orc_tce_hash(const int64_t *hash, int64_t key);
int orc_get_hash_block(const orc_file *f, double *array, int64_t size,
                       int64_t key);

/* ---- drivers ------------------------------------------------------------ */
/* ccsd_t_singles_l_1: accumulates all s1 terms of one tuple into a_c
 * (tuple layout (h3,h2,h1,p6,p5,p4) column-major).  Returns the number of
 * s1 kernel calls made (27/3 = 9 for any sorted tuple), or -1 on a
 * missing block. */
int64_t orc_singles_l_1(const orc_tiling *t, const orc_file *t1,
                        const orc_file *v2, double *a_c, int64_t t_p4b,
                        int64_t t_p5b, int64_t t_p6b, int64_t t_h1b,
                        int64_t t_h2b, int64_t t_h3b);
/* ccsd_t_doubles_l_12: all d1 (over h7b) and d2 (over p7b) terms.
 * calls[0] += number of d1 kernel calls, calls[1] += number of d2 calls.
 * Returns 0, or -1 on a missing block. */
int64_t orc_doubles_l_12(const orc_tiling *t, const orc_file *t2,
                         const orc_file *v2, double *triplesx,
                         int64_t t_p4b, int64_t t_p5b, int64_t t_p6b,
                         int64_t t_h1b, int64_t t_h2b, int64_t t_h3b,
                         int64_t *calls);
/* ccsd_t_dot: adds the tuple's E[T] and E(T) contributions. */
void orc_ccsd_t_dot(const double *a_singles, const double *a_doubles,
                    int64_t restricted, int64_t h1b, int64_t h2b,
                    int64_t h3b, int64_t p4b, int64_t p5b, int64_t p6b,
                    const double *o_h1, const double *o_h2,
                    const double *o_h3, const double *o_p4,
                    const double *o_p5, const double *o_p6, int64_t r_h1,
                    int64_t r_h2, int64_t r_h3, int64_t r_p4, int64_t r_p5,
                    int64_t r_p6, double *energy1, double *energy2);

/* ---- tuple list ---------------------------------------------------------- */
int64_t orc_6tasks(const orc_tiling *t);
/* klist: 7*tot entries (p4b,p5b,p6b,h1b,h2b,h3b,weight), w_thresh = 0. */
int64_t orc_neword(const orc_tiling *t, int64_t tot, int64_t *klist);

/* ---- whole (T) ----------------------------------------------------------
 * Runs ccsd_t_loop for the tasks klist[task_ids[0..n-1]] (all tasks when
 * task_ids == NULL, n = tot) and sums energies in task order.
 * per_task (optional, 2*n doubles) receives each task's (E[T], E(T)).
 * kernel_calls (optional, 3*n) receives each task's s1/d1/d2 call counts.
 * Returns 0 on success, -1 on a missing block, -2 on allocation failure. */
int64_t orc_ccsd_t(const orc_tiling *t, const orc_file *t1,
                   const orc_file *t2, const orc_file *v2,
                   const int64_t *klist, int64_t tot,
                   const int64_t *task_ids, int64_t n, double *energy,
                   double *per_task, int64_t *kernel_calls);

/* The drivers with the tile kernels replaced by callbacks: the reference
 * driver logic (permutation tables, dedup, filters, fetch + sort) feeds the
 * sub-blocks to hooks instead of the oracle kernels.  Dims arrive in the
 * CUDA-ABI order of sd_t_total.cu: s1 (h1d,h2d,h3d,p4d,p5d,p6d), d1
 * (h1d,h2d,h3d,h7d,p4d,p5d,p6d), d2 (h1d,h2d,h3d,p4d,p5d,p6d,p7d). */
typedef struct {
    void *user;
    void (*s1)(void *user, int64_t k, const int64_t *dims,
               const double *t1sub, const double *v2sub);
    void (*d1)(void *user, int64_t k, const int64_t *dims,
               const double *t2sub, const double *v2sub);
    void (*d2)(void *user, int64_t k, const int64_t *dims,
               const double *t2sub, const double *v2sub);
} orc_hooks;
int64_t orc_tuple_drive(const orc_tiling *t, const orc_file *t1,
                        const orc_file *t2, const orc_file *v2,
                        const int64_t *tuple6, const orc_hooks *hooks,
                        int64_t *calls3);

/* Full triples tiles of one tuple (for small-tile parity tests): singles
 * and doubles buffers of Nt doubles each, tuple layout. */
int64_t orc_tuple_tiles(const orc_tiling *t, const orc_file *t1,
                        const orc_file *t2, const orc_file *v2,
                        const int64_t *tuple6, double *singles,
                        double *doubles);

/* ---- synthetic workload inputs (orc_synth.c) ----------------------------
 * The benchmark workloads' seeded inputs on the checker side, byte for byte
 * the library's sdt_synth_file / sdt_synth_evl, so that the CPU baseline
 * runs without the product library.  kind: 0 T1, 1 T2, 2 V2.  With hash or
 * data NULL only the counts are returned.  0 on success. */
void orc_synth_evl(int64_t nocc, int64_t nvir, uint64_t seed, double *evl);
int64_t orc_synth_file(const orc_tiling *t, int kind, uint64_t seed, int64_t *nblocks, int64_t *ndata,
                       int64_t *hash, double *data);
/* Algorithmic FLOPs of a tuple list (7 entries per tuple). */
double orc_tasks_flops(const orc_tiling *t, const int64_t *klist, int64_t n);

#ifdef __cplusplus
}
#endif
#endif
