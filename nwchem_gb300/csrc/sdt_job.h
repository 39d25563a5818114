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
    // device
    int32_t *tiles = nullptr;
    double *evl_d = nullptr;
    int64_t *pair_off = nullptr;
    double *arr[sdt::DST_N] = {nullptr};
    size_t arr_n[sdt::DST_N] = {0};
    std::vector<int64_t> pair_host;     // Vd2 region offsets (fp64 elements), -1 if none
    // mixed form: split operands in block-major layouts (hi at [2*k], lo at
    // [2*k+1]; fp32 holding TF32 values, or bf16 / fp16), FP32 copies of T1d
    // and Ud for the s1 terms, and the box tables
    void *sp[2 * sdt::SP_N] = {nullptr};
    size_t sp_n[2 * sdt::SP_N] = {0};    // bytes
    int mixed_type = -1;                 // TM_* of the prepared copies, -1: none
    float *t1f = nullptr, *uf = nullptr;
    double inv_s = 1.0, inv_s2 = 1.0;    // FP16: 1/(s_T s_I), its square
    int64_t *tile_box_d = nullptr;       // device table buffer (box tables, pair blocks)
    int64_t tile_box_off = 0, pair_blk_off = 0;
    int32_t nob = 0, nvb = 0;            // hole and particle boxes over all tiles
    int mixed_kseg = 0;                  // K chunks per TMEM drain (0: whole term)
    int mixed_cluster = 1;               // CTAs per cluster of the mixed kernel: 1 or 4
    int *err_d = nullptr;
    int *err_h = nullptr;                // pinned copy of err_d
    bool loaded = false;
    // run workspace
    int64_t *klist_d = nullptr, *pref_d = nullptr, *spref_d = nullptr;
    double *factor_d = nullptr, *part_d = nullptr, *task_d = nullptr, *out_d = nullptr;
    size_t cap_tasks = 0, cap_items = 0;
    double *host_out = nullptr;
    size_t cap_host = 0;
    // optional CUDA-event timing of the fused launches of the last run
    bool timing = false;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    float last_ms = 0.0f;
};


namespace sdt {
// Per-tuple compensated sums of the item partials, the total, into out_d.
int finish_run(sdt_job *j, int64_t n, cudaStream_t st);
// Frees the mixed-form operands and maps of a job.
void mixed_release(sdt_job *j);
// Builds the split operands of element type `type` (TM_*) and the tensor
// maps (after a successful load).
int mixed_prepare(sdt_job *j, int type, cudaStream_t st);
// Launches the persistent mixed kernel over the n_super cluster work units
// (super-item prefix in spref_d) of the n tuples.
int mixed_launch(sdt_job *j, int64_t n_super, int64_t n, cudaStream_t st);
int make_tmap(CUtensorMap *map, const void *base, int type, int rank, const uint64_t *dims,
              const uint64_t *strides_bytes, const uint32_t *box, int swizzle_bytes);
}  // namespace sdt
