/*
 * sdt_gb300.h -- C ABI of libsdt_gb300.so, a GB300 (sm_103a) implementation
 * of NWChem's TCE CCSD(T) perturbative-triples tile path.
 *
 * Two surfaces are exported.
 *
 *  1. The tile-level surface the reference's CUDA (T) driver binds
 *     (src/tce/ccsd_t/ccsd_t_gpu.F, ccsd_t_singles_gpu.F,
 *     ccsd_t_doubles_gpu.F).  Same Fortran-mangled names, same argument
 *     order, 64-bit Integer passed by reference (the reference is built -i8,
 *     src/tce/ccsd_t/header.h:51), same accumulate-into-device-tile
 *     semantics.  Sub-blocks come from host memory and are copied per call.
 *
 *  2. A batched surface (sdt_*) that replaces the whole ccsd_t(...) call
 *     (src/tce/ccsd_t/ccsd_t.F:19-20): the T1/T2/V2 TCE files (hash table +
 *     block data) go to the device once, and one fused kernel evaluates all
 *     27 tile kernels and the energy sum for every tuple.
 *
 * No torch types appear here.  Streams are passed as void* (cudaStream_t);
 * NULL means the library's own stream.
 */
#ifndef SDT_GB300_H
#define SDT_GB300_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int64_t sdt_int; /* Fortran Integer (-i8) */

/* ------------------------------------------------------------------------
 * 1. Reference tile-level ABI (sd_t_total.cu, memory.cu, hybrid.c)
 * --------------------------------------------------------------------- */

/* s1: t3_s[perm_k] +/-= t1sub(p4,h1) * v2sub(h3,h2,p6,p5).
 * Replaces sd_t_s1_k_cuda_ (sd_t_total.cu:5522-5526 for k=1; the other k
 * follow it in that file).  The t3 argument is ignored, as in the reference:
 * the singles tile lives on the device (dev_mem_s_). */
#define SDT_S1_DECL(k)                                                       \
    void sd_t_s1_##k##_cuda_(sdt_int *h1d, sdt_int *h2d, sdt_int *h3d,       \
                             sdt_int *p4d, sdt_int *p5d, sdt_int *p6d,       \
                             double *t3, double *t1sub, double *v2sub);
SDT_S1_DECL(1) SDT_S1_DECL(2) SDT_S1_DECL(3) SDT_S1_DECL(4) SDT_S1_DECL(5)
SDT_S1_DECL(6) SDT_S1_DECL(7) SDT_S1_DECL(8) SDT_S1_DECL(9)

/* d1: t3[perm_k] -/+= sum_h7 t2sub(h7,p4,p5,h1) * v2sub(h3,h2,p6,h7).
 * Replaces sd_t_d1_k_cuda_ (sd_t_total.cu:312-316 for k=1). */
#define SDT_D1_DECL(k)                                                       \
    void sd_t_d1_##k##_cuda_(sdt_int *h1d, sdt_int *h2d, sdt_int *h3d,       \
                             sdt_int *h7d, sdt_int *p4d, sdt_int *p5d,       \
                             sdt_int *p6d, double *t3, double *t2sub,        \
                             double *v2sub);
SDT_D1_DECL(1) SDT_D1_DECL(2) SDT_D1_DECL(3) SDT_D1_DECL(4) SDT_D1_DECL(5)
SDT_D1_DECL(6) SDT_D1_DECL(7) SDT_D1_DECL(8) SDT_D1_DECL(9)

/* d2: t3[perm_k] -/+= sum_p7 t2sub(p7,p4,h1,h2) * v2sub(p7,h3,p6,p5).
 * Replaces sd_t_d2_k_cuda_ (sd_t_total.cu:2885-2888 for k=1). */
#define SDT_D2_DECL(k)                                                       \
    void sd_t_d2_##k##_cuda_(sdt_int *h1d, sdt_int *h2d, sdt_int *h3d,       \
                             sdt_int *p4d, sdt_int *p5d, sdt_int *p6d,       \
                             sdt_int *p7d, double *t3, double *t2sub,        \
                             double *v2sub);
SDT_D2_DECL(1) SDT_D2_DECL(2) SDT_D2_DECL(3) SDT_D2_DECL(4) SDT_D2_DECL(5)
SDT_D2_DECL(6) SDT_D2_DECL(7) SDT_D2_DECL(8) SDT_D2_DECL(9)

/* Energy of the current device tiles: energy[0] is set (not added) to
 * E[T] = factor*sum t3^2/D and energy[1] to
 * E(T) = factor*sum t3*(t3+t3_s)/D, D = e_h1+e_h2+e_h3-e_p4-e_p5-e_p6.
 * host1/host2 are ignored, as in the reference.
 * Replaces compute_en_ (sd_t_total.cu:5373-5379). */
void compute_en_(double *factor, double *energy, double *eval1,
                 double *eval2, double *eval3, double *eval4, double *eval5,
                 double *eval6, sdt_int *h1d, sdt_int *h2d, sdt_int *h3d,
                 sdt_int *p4d, sdt_int *p5d, sdt_int *p6d, double *host1,
                 double *host2);

/* Allocate and zero the doubles / singles triples tiles of one tuple
 * (tuple dims).  Replace dev_mem_d_ (sd_t_total.cu:12-16) and dev_mem_s_
 * (sd_t_total.cu:5392-5396). */
void dev_mem_d_(sdt_int *h1d, sdt_int *h2d, sdt_int *h3d, sdt_int *p4d,
                sdt_int *p5d, sdt_int *p6d);
void dev_mem_s_(sdt_int *h1d, sdt_int *h2d, sdt_int *h3d, sdt_int *p4d,
                sdt_int *p5d, sdt_int *p6d);
/* Energy of triples tiles that the CALLER owns in device memory, without any
 * device allocation.  No counterpart in the reference.  It is for callers
 * that keep t3 (and t3_s) in device memory they manage themselves -- their
 * own pool, or arrays owned by a Fortran offload runtime -- and cannot or
 * must not call cudaMalloc/cudaFree (their pool holds the memory budget, or
 * an allocation would synchronise the device under their running work).
 * Arguments and results are compute_en_'s: host orbital energies
 * eval1..eval6 (h1,h2,h3,p4,p5,p6), tile lengths, factor, and energy[0] =
 * E[T], energy[1] = E(T) on the host; t3_d / t3s_d are the tuple-layout
 * (h3,h2,h1,p6,p5,p4) device tiles (t3s_d may be NULL: no singles).
 * Its scratch is one fixed __device__ array (about 82 KB on every GPU that
 * loads the library, held until exit): h1d+h2d+h3d+p4d+p5d+p6d may not
 * exceed 8192, larger requests fail with SDT_ERR_ARG.  The first call on a
 * device looks up that array's device address (cudaGetSymbolAddress) with
 * the device current; make that first call before any stream capture.
 * All calls share the array, so calls that overlap on the GPU race; every
 * scratch element a call reads is written earlier in the same call.
 * Work is queued on `stream` (NULL: the legacy default stream) and the
 * call returns after synchronising it. */
int sdt_compute_en_noalloc(double factor, double *energy, const double *eval1,
                           const double *eval2, const double *eval3,
                           const double *eval4, const double *eval5,
                           const double *eval6, int64_t h1d, int64_t h2d,
                           int64_t h3d, int64_t p4d, int64_t p5d,
                           int64_t p6d, const double *t3_d,
                           const double *t3s_d, void *stream);
/* Copies the current device tiles to host buffers of the tuple size (either
 * may be NULL).  No reference counterpart: the reference only exposes the
 * tiles through compute_en_; this read-back exists for parity tests. */
int sdt_tile_download(double *doubles, double *singles);
/* Release both tiles (sd_t_total.cu:17-28). */
void dev_release_(void);
/* Caching device / pinned-host allocator (memory.cu:69,164-178).  Blocks
 * freed between init and finalize are reused by size; finalize checks that
 * nothing is live. */
void initmemmodule_(void);
void finalizememmodule_(void);
/* Device binding (hybrid.c:25,32): check_device_ returns 1 when this
 * process's device index (SDT_LOCAL_RANK / LOCAL_RANK, default 0) is below
 * *icuda; device_init_ selects that device, or sets *cuda_device_number =
 * 30 when fewer than *icuda devices exist (the reference's warning path). */
int check_device_(long *icuda);
int device_init_(long *icuda, long *cuda_device_number);

/* ------------------------------------------------------------------------
 * Error handling.  The reference prints and exit(1)s on any CUDA error
 * (header.h:28-36).  The Fortran-facing symbols above keep that behaviour
 * by default (SDT_ERRMODE_EXIT); SDT_ERRMODE_RECORD makes them record the
 * error instead, readable with sdt_last_error().  The sdt_* functions
 * always return a status and never exit.
 * --------------------------------------------------------------------- */
enum {
    SDT_OK = 0,
    SDT_ERR_ARG = 1,      /* bad argument or size                        */
    SDT_ERR_CUDA = 2,     /* CUDA runtime error                          */
    SDT_ERR_NOMEM = 3,    /* allocation failed                           */
    SDT_ERR_STATE = 4,    /* call out of order (e.g. no dev_mem_d_)      */
    SDT_ERR_MISSING = 5,  /* a block the path needs is absent            */
    SDT_ERR_TIMEOUT = 6   /* a bounded device wait ran out               */
};
enum { SDT_ERRMODE_EXIT = 0, SDT_ERRMODE_RECORD = 1 };
void sdt_set_error_mode(int mode);
int sdt_last_error(char *msg, size_t len); /* returns code, clears it */

/* ------------------------------------------------------------------------
 * 2. Batched surface
 * --------------------------------------------------------------------- */

/* Tile description; arrays indexed by tile-1, tiles 1..noab occupied and
 * noab+1..noab+nvab virtual (src/tce/include/tce.fh:14-21). */
typedef struct {
    int64_t noab, nvab;
    const int64_t *range;
    const int64_t *spin;
    const int64_t *sym;
    const int64_t *offset;     /* into evl_sorted */
    const int64_t *alpha;      /* beta->alpha tile map; NULL if unrestricted */
    const double *evl_sorted;  /* orbital energies, occupied then virtual */
    int64_t restricted;
} sdt_tiling;

/* A TCE file: hash in the tce_hash layout (hash[0] = n, keys ascending in
 * hash[1..n], block offsets in hash[n+1..2n]) and ndata doubles of blocks. */
typedef struct {
    const int64_t *hash;
    const double *data;
    int64_t ndata;
} sdt_file;

/* Tuple list of the (T) driver (ccsd_t_6tasks / ccsd_t_neword,
 * src/tce/ccsd_t/ccsd_t_neword.F:1-217).  klist gets 7*n entries
 * (p4b,p5b,p6b,h1b,h2b,h3b,weight), weight-ordered like the reference. */
int64_t sdt_tasks_count(const sdt_tiling *t);
int sdt_tasks_list(const sdt_tiling *t, int64_t n, int64_t *klist);
/* Algorithmic FLOPs of the listed tuples: sum Nt*18*(O_allowed+V_allowed+1). */
double sdt_tasks_flops(const sdt_tiling *t, const int64_t *klist, int64_t n);

/* Synthetic seeded TCE files (the inputs the path reads).  kind: 0 = T1,
 * 1 = T2, 2 = V2 (vvov, ovoo and vvoo blocks in one hash).  Query sizes
 * with hash == data == NULL, then fill. */
enum { SDT_FILE_T1 = 0, SDT_FILE_T2 = 1, SDT_FILE_V2 = 2 };
int sdt_synth_file(const sdt_tiling *t, int kind, uint64_t seed,
                   int64_t *nblocks, int64_t *ndata, int64_t *hash,
                   double *data);
/* Hash table of a TCE file as NWChem lays it out on disk or in a global
 * array (tce_t1_offset.F, tce_t2_offset.F, tce_mo2e_offset.F): for V2 it
 * lists every spin/irrep-allowed block, including the kinds the triples
 * path never reads.  Query sizes with hash == NULL (2*nblocks+1 entries). */
int sdt_tce_layout(const sdt_tiling *t, int kind, int64_t *nblocks,
                   int64_t *ndata, int64_t *hash);
/* Orbital energies: occupied ~ U[-1.5,-0.4], virtual ~ U[0.2,2.5]. */
int sdt_synth_evl(int64_t nocc, int64_t nvir, uint64_t seed, double *evl);

/* A job holds one (T) problem resident on the device. */
typedef struct sdt_job sdt_job;
/* Precision of sdt_job_run: FP64 throughout, or a mixed form: the d1/d2
 * contractions as split products hi*hi + hi*lo + lo*hi with FP32
 * accumulation on the tensor cores (TF32x3; BF16x3; FP16x3 with
 * power-of-two operand scaling), the s1 products in FP32, and the
 * triples promoted to FP64 for the denominator, the division and the
 * energy sums. */
enum { SDT_PREC_FP64 = 0, SDT_PREC_MIXED_TF32 = 1, SDT_PREC_MIXED_BF16 = 2,
       SDT_PREC_MIXED_FP16 = 3 };
int sdt_job_create(const sdt_tiling *t, sdt_job **job);
/* Copy the host TCE files to the device and re-lay them out for the fused
 * kernel (antisymmetric mirrors, signs of tce_hashnsort.F).  Device-side
 * copies are enqueued on stream; the call returns after the host buffers
 * may be reused. */
int sdt_job_load(sdt_job *job, const sdt_file *t1, const sdt_file *t2,
                 const sdt_file *v2, void *stream);
/* Evaluate the tuples klist[0..n-1] (7 entries each).  energy[0] = E[T],
 * energy[1] = E(T).  per_task (optional, 2*n doubles, host) receives each
 * tuple's pair.  Synchronises the stream. */
int sdt_job_run(sdt_job *job, const int64_t *klist, int64_t n,
                int precision, double *energy, double *per_task,
                void *stream);
int sdt_job_destroy(sdt_job *job);
/* Device bytes held by a job: its dense FP64 operands and, once a mixed
 * precision has run, that form's split operands, FP32 copies and tables. */
int64_t sdt_job_device_bytes(const sdt_job *job);
/* Mixed form: drain the tensor-core accumulator every `chunks` K chunks
 * (8 TF32 or 16 BF16/FP16 values each; 0, the default: once per
 * contraction term).  Shorter accumulation
 * chains reduce the FP32 rounding of the split products at the cost of more
 * drains. */
int sdt_job_set_mixed_segment(sdt_job *job, int chunks);
/* Mixed form: the kernel's work-unit shape.  1 (the default): one CTA per
 * sub-box, the finished sub-box kept in registers while the next one is
 * contracted; 2: the same with the finished sub-box kept in tensor memory
 * (one accumulator instead of two, the energy work gets the registers --
 * for tuples whose spin/irrep-kept K is short). */
int sdt_job_set_mixed_shape(sdt_job *job, int shape);
/* When on, sdt_job_run brackets its fused-kernel launches with CUDA events
 * on the run's stream; sdt_job_last_kernel_ms returns that interval. */
int sdt_job_set_timing(sdt_job *job, int on);
double sdt_job_last_kernel_ms(const sdt_job *job);

/* Plans (no reference counterpart): a prepared evaluation of a tuple
 * list.  sdt_plan_create checks the list, builds the work indexes, sizes
 * the persistent launches (and, for a mixed precision, encodes the job's
 * split operands if needed) and uploads them; shapes (optional, one per
 * tuple: 1 or 2 as in sdt_job_set_mixed_shape) picks the mixed
 * kernel's work-unit shape per tuple.
 * sdt_plan_launch only enqueues device work -- per group a queue reset and
 * one persistent kernel, the compensated sums and the copy of the results
 * to pinned host memory -- and can be recorded by stream capture;
 * sdt_plan_capture records one launch into a CUDA graph, which
 * sdt_plan_run then replays (else it launches), synchronises the stream and
 * returns E[T], E(T) and, optionally, the per-tuple pairs in the caller's
 * order.  A plan is bound to its job; destroy it after its last run. */
typedef struct sdt_plan sdt_plan;
int sdt_plan_create(sdt_job *job, const int64_t *klist, int64_t n,
                    int precision, const int32_t *shapes, sdt_plan **plan);
int sdt_plan_launch(sdt_plan *plan, void *stream);
int sdt_plan_capture(sdt_plan *plan, void *stream);
int sdt_plan_run(sdt_plan *plan, void *stream, double *energy,
                 double *per_task);
int sdt_plan_destroy(sdt_plan *plan);
/* The per-item (E[T], E(T)) pairs of the plan's last run (factor
 * included), n = sdt_plan_items: items in tuple order (the plan's order for
 * a single work-unit shape), each tuple's sub-boxes with the h3 box fastest
 * and the p4 box slowest (4-wide boxes in the FP64 form; 8-wide particle
 * boxes in the mixed forms).  For checks of parts of a tuple. */
int sdt_plan_item_energies(sdt_plan *plan, double *pairs, int64_t n);
/* Sub-box work items of a plan. */
int64_t sdt_plan_items(const sdt_plan *plan);

/* Serving (no reference counterpart): a loop of independent (T) jobs on
 * one GPU.  Jobs wait in one FIFO queue and are admitted when fewer than
 * `slots` jobs are in flight and sdt_job_bytes of the job fits in the byte
 * budget minus the admitted jobs' bytes (a job larger than the budget
 * fails with SDT_ERR_NOMEM); `slots` workers load admitted jobs, each on
 * its own stream.  Continuous batching: jobs of the server's mixed form
 * (FP16x3 unless sdt_server_set_queue says otherwise) have their sub-box
 * items appended to one device work queue that a resident persistent
 * kernel drains while they arrive; it keeps `reserve` SMs free for loading
 * and finishing other jobs, and each job's energies are delivered when its
 * last item is done.  Jobs of other precisions run their own launches
 * (max_ctas, 0: all SMs, caps those).  A job submitted with check_fp64
 * keeps its device memory after its energies are delivered (state 3) and
 * runs the FP64 form as a check when no admissible job is waiting.
 * The caller keeps a job's files alive until its state is 2 (done) or -1
 * (failed).  Times are seconds since sdt_server_create. */
typedef struct sdt_server sdt_server;
int sdt_server_create(int64_t budget_bytes, int slots, int max_ctas,
                      sdt_server **server);
int sdt_server_submit(sdt_server *server, const sdt_tiling *t,
                      const sdt_file *t1, const sdt_file *t2,
                      const sdt_file *v2, int precision, int check_fp64,
                      int64_t *ticket);
/* state 0 queued, 1 running, 3 energies ready with the FP64 check pending,
 * 2 done, -1 failed (the job's error code is
 * returned and its message copied to msg); energy[2], fp64[2] (check) and
 * times[5] (submitted, admitted, inputs on the device, energies ready,
 * finished) may be NULL. */
int sdt_server_status(sdt_server *server, int64_t ticket, int *state,
                      double *energy, double *fp64, double *times,
                      char *msg, size_t len);
/* SMs (one CTA each) of each deferred FP64 check: default half the SMs the
 * shared queue leaves free (with the queue: 1 to reserve_sms, one check at
 * a time, so the resident kernel never waits for a check's SMs), or a
 * quarter of the SMs without the queue. */
int sdt_server_set_check_ctas(sdt_server *server, int ctas);
/* The shared queue: its precision (SDT_PREC_FP64 turns it off), work-unit
 * shape (1 or 2, as sdt_job_set_mixed_shape; default 1), SMs kept free of
 * the resident kernel (default 16) and the seconds (at most 1) the kernel
 * waits for new work before it leaves (default 0.2).  Before the first
 * submit. */
int sdt_server_set_queue(sdt_server *server, int precision, int shape,
                         int reserve_sms, double idle_s);
/* stats[4]: resident-kernel launches, jobs that went through the queue,
 * most jobs in the queue at once, jobs in it now. */
int sdt_server_queue_stats(sdt_server *server, int64_t *stats);
/* The resident-kernel launches (numbered from 1) that took the job's first
 * item and finished its last item; 0 when the job did not go through the
 * queue or has not finished. */
int sdt_server_job_launches(sdt_server *server, int64_t ticket, int *first,
                            int *last);
/* Cancels a queued job (state -1, SDT_ERR_STATE); an admitted job is not
 * stopped (SDT_ERR_STATE is returned). */
int sdt_server_cancel(sdt_server *server, int64_t ticket);
/* Waits for every submitted job (SDT_ERR_TIMEOUT after timeout_s). */
int sdt_server_drain(sdt_server *server, double timeout_s);
int64_t sdt_server_peak_bytes(sdt_server *server);
int sdt_server_destroy(sdt_server *server);
/* Device bytes a job of this tiling needs at its peak (admission bound). */
int64_t sdt_job_bytes(const sdt_tiling *t, int precision);
/* The admission policy alone, simulated on the host: jobs arriving at
 * arrival[q] (ascending) with bytes[q] and run times service[q]; start[q]
 * and end[q] receive admission and completion times (-1: larger than the
 * budget). */
int sdt_admission_simulate(int64_t n, const double *arrival,
                           const int64_t *bytes, const double *service,
                           int64_t budget, int slots, double *start,
                           double *end);
/* The serving policy with deferred FP64 checks, simulated on the host: as
 * sdt_admission_simulate, plus check_service[q] (< 0: no check); a pending
 * check takes a free slot only when no queue head can be admitted, and the
 * job's bytes stay admitted until its check ends.  start, ready (energies)
 * and done (check finished) receive the times (-1: refused). */
int sdt_serving_simulate(int64_t n, const double *arrival, const int64_t *bytes,
                         const double *service, const double *check_service,
                         int64_t budget, int slots, double *start,
                         double *ready, double *done);
/* Caps a job's persistent launches at `ctas` SMs' worth of CTAs (0: all
 * SMs; a mixed launch runs one CTA per SM, an FP64 launch up to four). */
int sdt_job_set_max_ctas(sdt_job *job, int ctas);
/* FP64 persistent launches with one CTA per SM (on != 0): a launch capped
 * by sdt_job_set_max_ctas then occupies exactly that many SMs. */
int sdt_job_set_sm_exclusive(sdt_job *job, int on);
/* The job's own stream (the default stream of its calls). */
void *sdt_job_stream(const sdt_job *job);

/* One-shot replacement for ccsd_t(d_t1,k_t1_offset,d_t2,k_t2_offset,
 * d_v2,k_v2_offset,energy1,energy2,size_t1) (ccsd_t.F:19-20): builds the
 * tuple list, loads the files, runs every tuple and returns E[T] in
 * *energy1 and E(T) in *energy2. */
int sdt_ccsd_t(const sdt_tiling *t, const sdt_file *t1, const sdt_file *t2,
               const sdt_file *v2, double *energy1, double *energy2);

/* Kernel launches made by this library since load (all entry points). */
int64_t sdt_launch_count(void);

/* Measured FP64 tensor-core (mma.sync m8n8k4.f64) throughput of the current
 * device in TFLOP/s: a register-resident loop of independent MMAs over all
 * SMs for about `ms` milliseconds.  The roofline denominator of the FP64
 * form. */
double sdt_probe_fp64_tflops(int ms);

/* Self-test of the tensor-core path of the mixed form (no reference
 * counterpart): D[128][256] = A*B^T on one SM with A = a_hi + a_lo
 * ([128][K]) and B = b_hi + b_lo ([256][K]) given as TF32 values in fp32
 * device arrays, K a multiple of 4, the three split products accumulated in
 * FP32 by tcgen05.mma from TMA-staged shared memory.  D is a device array.
 * SDT_ERR_TIMEOUT if a bounded wait in the kernel ran out. */
int sdt_tc_selftest(const float *a_hi, const float *a_lo, const float *b_hi,
                    const float *b_lo, int K, float *D);
/* The same with 16-bit operands (bf16 != 0: BF16, else FP16; raw 16-bit
 * values in device arrays, K a multiple of 8), kind::f16 MMAs. */
int sdt_tc_selftest16(const void *a_hi, const void *a_lo, const void *b_hi,
                      const void *b_lo, int K, int bf16, float *D);
/* Check of the mixed form's FP32 energy quotient (no reference
 * counterpart): largest relative difference of X/D, with D summed in FP32
 * from gap-shifted orbital energies the way the energy epilogue sums it,
 * from the FP64 quotient, over n seeded samples. */
int sdt_check_division(int64_t n, uint64_t seed, double *max_rel_err);
/* Failure-path check (no reference counterpart): one bounded device wait on
 * an mbarrier nothing arrives on, limited to timeout_s (0 < timeout_s <= 1).
 * Returns SDT_ERR_TIMEOUT with *waited_s the time waited; the CUDA context
 * stays usable. */
int sdt_check_wait_timeout(double timeout_s, double *waited_s);

#ifdef __cplusplus
}
#endif
#endif
