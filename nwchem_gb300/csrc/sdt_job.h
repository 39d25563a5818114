// sdt_job.h -- the batched job object shared by the FP64 and mixed paths.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <vector>
#include "sdt_internal.h"

namespace sdt {
enum { DST_T1 = 0, DST_T2A, DST_T2B, DST_VD2, DST_WD1, DST_UD, DST_N };
// Split (hi/lo) copies of the contraction operands (mixed form).
enum { SP_T2A = 0, SP_T2B, SP_WD1, SP_VD2, SP_N };
// Operand element types of the mixed form (tensor maps, split copies).
enum { TM_F32 = 0, TM_BF16 = 1, TM_F16 = 2 };
}  // namespace sdt

struct sdt_job {
    using Tiling = sdt::Tiling;
    Tiling t;
    std::vector<int64_t> range, spin, sym, offset, alpha;
    std::vector<double> evl;
    int dev = 0;
    cudaStream_t stream = nullptr;       // the job's own stream (default for its work)
    int max_ctas = 0;                    // cap on the CTAs of its persistent launches (0: all SMs)
    int sm_exclusive = 0;                // FP64 persistent launches: one CTA per SM
    // device
    int32_t *tiles = nullptr;
    double *evl_d = nullptr;
    int64_t *pair_off = nullptr;
    double *arr[sdt::DST_N] = {nullptr};
    size_t arr_n[sdt::DST_N] = {0};
    std::vector<int64_t> pair_host;     // Vd2 region offsets (fp64 elements), -1 if none
    // mixed form: split operands in block-major layouts (one buffer per
    // layout at [2*k], each block its hi half then its lo half; [2*k+1]
    // unused; fp32 holding TF32 values, or bf16 / fp16), FP32 copies of T1d
    // and Ud for the s1 terms (the T1 buffer followed by the orbital energies
    // minus the gap midpoint, FP32), and the box tables
    void *sp[2 * sdt::SP_N] = {nullptr};
    size_t sp_n[2 * sdt::SP_N] = {0};    // bytes
    int mixed_type = -1;                 // TM_* of the prepared copies, -1: none
    float *t1f = nullptr, *uf = nullptr;
    size_t mixed_aux_n = 0;              // bytes of the FP32 copies and the box tables
    double inv_s = 1.0, inv_s2 = 1.0;    // FP16: 1/(s_T s_I), its square
    int64_t *tile_box_d = nullptr;       // device table buffer (box tables, pair blocks)
    int64_t tile_box_off = 0, pair_blk_off = 0;
    int32_t nob = 0, nvb = 0;            // hole and particle boxes over all tiles
    int mixed_kseg = 0;                  // K chunks per TMEM drain (0: whole term)
    int mixed_shape = 1;                 // work-unit shape of the mixed kernel: 1 register hold, 2 tensor-memory hold
    int all_k = 1;                       // every K tile allowed for every term
    bool loaded = false;
    // optional CUDA-event timing of the fused launches of the last run
    bool timing = false;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    float last_ms = 0.0f;
};


namespace sdt {
// Returns SDT_OK or records a CUDA error with context.
int cuda_check(cudaError_t e, const char *what);
// Multiplicity factor of a tuple (ccsd_t_dot.F:52-66).
double tuple_factor(const int64_t *k, bool restricted);

// One persistent launch over a contiguous group of tuples.  The item prefix
// is relative to the group (item_pref[0] = 0); part receives the group's
// item pairs.
struct LaunchArgs {
    const int64_t *klist = nullptr, *item_pref = nullptr;
    const double *factor = nullptr;
    double *part = nullptr;
    int64_t n = 0, items = 0;
    unsigned long long *queue = nullptr;  // work counter, reset by the launch
    int *err = nullptr;                   // mixed form: wait-timeout code, reset by the launch
    int shape = 1, grid = 1;              // mixed form: work-unit shape 1 or 2
};

// Per-tuple compensated sums of item pairs (gpref: global item prefix, n+1)
// into task (2n) and the compensated total into out (2).
int tuple_sums(const double *part, const int64_t *gpref, int64_t n, double *task, double *out, cudaStream_t st);
int fp64_grid(sdt_job *j, int64_t items, int *grid);
int fp64_launch(sdt_job *j, const LaunchArgs &a, cudaStream_t st);
// Frees the mixed-form operands of a job.
void mixed_release(sdt_job *j);
// Builds the split operands of element type `type` (TM_*) and the box
// tables (after a successful load).
int mixed_prepare(sdt_job *j, int type, cudaStream_t st);
// Grid of the mixed kernel for a group of work-unit shape 1 or 2 (sets the
// kernel's shared-memory attribute; call outside stream capture).
int mixed_grid(sdt_job *j, int shape, int64_t n_items, int *grid);
int mixed_launch(sdt_job *j, const LaunchArgs &a, cudaStream_t st);

// The shared item queue of the serving path (device buffers owned by the
// caller; see QueueCtl in sdt_split.cu for the protocol).  table holds
// max_jobs entries of mixed_job_entry_bytes() each.
struct QueueArgs {
    const void *table = nullptr;
    const long long *base = nullptr;
    unsigned long long *head = nullptr;
    const unsigned long long *tail = nullptr;
    unsigned long long *done = nullptr;
    int *first_gen = nullptr, *last_gen = nullptr;  // host-mapped
    const int *close = nullptr;
    int *err = nullptr;
    unsigned long long idle_ns = 0;
    int max_jobs = 0, gen = 0;
};
size_t mixed_job_entry_bytes();
// Writes the queue-table entry of a plan group of job j (prepared split operands).
int mixed_job_entry(sdt_job *j, const LaunchArgs &a, void *entry);
// Sets the queue kernel's shared-memory attribute (outside stream capture).
int mixed_queue_prepare(int type, int shape);
int mixed_queue_launch(int type, int shape, const QueueArgs &a, int grid, cudaStream_t st);

// Plans, for the serving queue: create; the queue-table entry of a mixed
// plan of one work-unit shape (and its item count); the sums and read-back
// of its energies once every item pair is written; free.
int plan_make(sdt_job *j, const int64_t *klist, int64_t n, int precision, const int32_t *shapes, sdt_plan **out);
int plan_queue_entry(sdt_plan *p, void *entry, int64_t *items);
int plan_finish(sdt_plan *p, cudaStream_t st, double *energy);
void plan_release(sdt_plan *p);
}  // namespace sdt
