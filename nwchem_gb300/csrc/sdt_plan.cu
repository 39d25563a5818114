// sdt_plan.cu -- prepared evaluations of tuple lists (plans) and the job run.
//
// A plan does the host work of a run once: it checks the tuple list, builds
// the item prefixes and the multiplicity factors, groups the tuples by the
// mixed kernel's work-unit shape (the finished sub-box kept in registers or
// in tensor memory), uploads everything and sizes every launch.
// sdt_plan_launch then only enqueues device work -- per group a queue reset
// and one persistent launch, the per-tuple and total compensated sums, and
// the copy of the results to pinned host memory -- so a launch can be
// captured once into a CUDA graph and replayed.  sdt_job_run is a one-shot
// plan.
#include "sdt_common.cuh"
#include "sdt_job.h"

#include <algorithm>
#include <cstring>
#include <numeric>
#include <vector>

struct sdt_plan {
    sdt_job *job = nullptr;
    int precision = SDT_PREC_FP64, mtype = -1;
    int64_t n = 0, items = 0;
    std::vector<int64_t> order;  // plan position -> caller's tuple index
    struct Group {
        int shape = 1, grid = 1;
        int64_t t0 = 0, t1 = 0, i0 = 0, items = 0;
    };
    std::vector<Group> groups;
    // device
    int64_t *klist_d = nullptr, *rpref_d = nullptr, *gpref_d = nullptr;
    double *factor_d = nullptr, *part_d = nullptr, *task_d = nullptr, *out_d = nullptr;
    unsigned long long *queue_d = nullptr;  // one counter per group
    int *err_d = nullptr;
    // host (pinned): [2 totals][2n per-tuple], error flag
    double *host_out = nullptr;
    int *err_h = nullptr;
    // graph
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int64_t kernels = 0;  // kernel launches per plan launch
};

namespace sdt {
namespace {

void plan_free(sdt_plan *p) {
    if (p->exec) cudaGraphExecDestroy(p->exec);
    if (p->graph) cudaGraphDestroy(p->graph);
    gpu_put(p->klist_d);
    gpu_put(p->rpref_d);
    gpu_put(p->gpref_d);
    gpu_put(p->factor_d);
    gpu_put(p->part_d);
    gpu_put(p->task_d);
    gpu_put(p->out_d);
    gpu_put(p->queue_d);
    gpu_put(p->err_d);
    host_put(p->host_out);
    host_put(p->err_h);
    delete p;
}

int mixed_type_of(int precision) {
    return precision == SDT_PREC_MIXED_TF32 ? TM_F32 : precision == SDT_PREC_MIXED_BF16 ? TM_BF16 : TM_F16;
}

// Builds a plan; shapes[q] (optional, caller order) is the work-unit shape of
// tuple q in the mixed form: 1 the finished sub-box in the energy warps'
// registers, 2 the finished sub-box kept in tensor memory.
int plan_create(sdt_job *j, const int64_t *klist, int64_t n, int precision, const int32_t *shapes,
                sdt_plan **out, const char *who) {
    *out = nullptr;
    if (!j || (n > 0 && !klist)) return fail(SDT_ERR_ARG, std::string(who) + ": null argument");
    if (!j->loaded) return fail(SDT_ERR_STATE, std::string(who) + ": sdt_job_load has not succeeded");
    if (precision < SDT_PREC_FP64 || precision > SDT_PREC_MIXED_FP16)
        return fail(SDT_ERR_ARG, std::string(who) + ": unknown precision");
    const bool mixed = precision != SDT_PREC_FP64;
    const Tiling &t = j->t;
    const int64_t nt = t.noab + t.nvab;
    for (int64_t q = 0; q < n; ++q) {
        const int64_t *k = klist + 7 * q;
        for (int d = 0; d < 6; ++d) {
            const bool virt = d < 3;
            if (k[d] < 1 || k[d] > nt || (virt ? k[d] <= t.noab : k[d] > t.noab))
                return fail(SDT_ERR_ARG, std::string(who) + ": tuple tile out of range");
        }
        if (!(k[0] <= k[1] && k[1] <= k[2] && k[3] <= k[4] && k[4] <= k[5]))
            return fail(SDT_ERR_ARG, std::string(who) + ": tuple tiles not sorted");
        if (shapes && shapes[q] != 1 && shapes[q] != 2)
            return fail(SDT_ERR_ARG, std::string(who) + ": work-unit shape must be 1 or 2");
    }
    sdt_plan *p = new sdt_plan();
    p->job = j;
    p->precision = precision;
    p->n = n;
    // Group by work-unit shape (FP64: one group), keeping the caller's order inside a group.
    auto cl = [&](int64_t q) { return mixed ? (shapes ? (int)shapes[q] : j->mixed_shape) : 1; };
    for (int c : {1, 2})
        for (int64_t q = 0; q < n; ++q)
            if (cl(q) == c) p->order.push_back(q);
    const int box_v = mixed ? 8 : 4, box_o = 4;
    std::vector<int64_t> kl(7 * std::max<int64_t>(n, 1)), rpref, gpref(n + 1, 0);
    std::vector<double> fac(std::max<int64_t>(n, 1));
    for (int64_t pos = 0; pos < n;) {
        sdt_plan::Group g;
        g.shape = cl(p->order[pos]);
        g.t0 = pos;
        g.i0 = gpref[pos];
        rpref.push_back(0);
        while (pos < n && cl(p->order[pos]) == g.shape) {
            const int64_t *k = klist + 7 * p->order[pos];
            std::memcpy(kl.data() + 7 * pos, k, 7 * sizeof(int64_t));
            int64_t boxes = 1;
            for (int d = 0; d < 6; ++d) {
                const int bx = d < 3 ? box_v : box_o;
                const int64_t nb = (t.r(k[d]) + bx - 1) / bx;
                boxes *= nb;
            }
            fac[pos] = tuple_factor(k, t.restricted != 0);
            gpref[pos + 1] = gpref[pos] + boxes;
            rpref.push_back(rpref.back() + boxes);
            ++pos;
        }
        g.t1 = pos;
        g.items = rpref.back();
        p->groups.push_back(g);
    }
    p->items = gpref[n];
    const size_t ng = std::max<size_t>(p->groups.size(), 1);
    p->klist_d = (int64_t *)gpu_get(kl.size() * sizeof(int64_t));
    p->rpref_d = (int64_t *)gpu_get(std::max<size_t>(rpref.size(), 1) * sizeof(int64_t));
    p->gpref_d = (int64_t *)gpu_get(gpref.size() * sizeof(int64_t));
    p->factor_d = (double *)gpu_get(fac.size() * sizeof(double));
    p->part_d = (double *)gpu_get(std::max<int64_t>(2 * p->items, 2) * sizeof(double));
    p->task_d = (double *)gpu_get(std::max<int64_t>(2 * n, 2) * sizeof(double));
    p->out_d = (double *)gpu_get(2 * sizeof(double));
    p->queue_d = (unsigned long long *)gpu_get(ng * sizeof(unsigned long long));
    p->err_d = (int *)gpu_get(sizeof(int));
    p->host_out = (double *)host_get((2 + 2 * std::max<int64_t>(n, 1)) * sizeof(double));
    p->err_h = (int *)host_get(sizeof(int));
    if (!p->klist_d || !p->rpref_d || !p->gpref_d || !p->factor_d || !p->part_d || !p->task_d ||
        !p->out_d || !p->queue_d || !p->err_d || !p->host_out || !p->err_h) {
        plan_free(p);
        return fail(SDT_ERR_NOMEM, std::string(who) + ": plan buffers");
    }
    *p->err_h = 0;
    if (j->timing) {
        if (!j->ev0 && cudaEventCreate(&j->ev0) != cudaSuccess) j->ev0 = nullptr;
        if (!j->ev1 && cudaEventCreate(&j->ev1) != cudaSuccess) j->ev1 = nullptr;
        cudaGetLastError();
    }
    cudaStream_t st = j->stream;
    int rc = SDT_OK;
    if (mixed) {
        p->mtype = mixed_type_of(precision);
        if (j->mixed_type != p->mtype) rc = mixed_prepare(j, p->mtype, st);
    }
    auto up = [&](void *dst, const void *src, size_t bytes) {
        if (!rc && bytes) rc = cuda_check(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st), who);
    };
    up(p->klist_d, kl.data(), 7 * n * sizeof(int64_t));
    up(p->rpref_d, rpref.data(), rpref.size() * sizeof(int64_t));
    up(p->gpref_d, gpref.data(), gpref.size() * sizeof(int64_t));
    up(p->factor_d, fac.data(), n * sizeof(double));
    for (auto &g : p->groups) {
        if (rc) break;
        rc = mixed ? mixed_grid(j, g.shape, g.items, &g.grid) : fp64_grid(j, g.items, &g.grid);
        p->kernels += 1;
    }
    p->kernels += (n + 65534) / 65535 + 1;  // tuple sums and the total
    if (!rc) rc = cuda_check(cudaStreamSynchronize(st), who);
    if (rc) {
        plan_free(p);
        return rc;
    }
    *out = p;
    return SDT_OK;
}

LaunchArgs group_args(sdt_plan *p, size_t gi) {
    const auto &g = p->groups[gi];
    LaunchArgs a;
    a.klist = p->klist_d + 7 * g.t0;
    a.item_pref = p->rpref_d + g.t0 + gi;
    a.factor = p->factor_d + g.t0;
    a.part = p->part_d + 2 * g.i0;
    a.n = g.t1 - g.t0;
    a.items = g.items;
    a.queue = p->queue_d + gi;
    a.err = p->err_d;
    a.shape = g.shape;
    a.grid = g.grid;
    return a;
}

// The per-tuple and total sums of the plan's item pairs and their copy to
// pinned host memory.
int plan_sums(sdt_plan *p, cudaStream_t st) {
    int rc = tuple_sums(p->part_d, p->gpref_d, p->n, p->task_d, p->out_d, st);
    if (!rc) rc = cuda_check(cudaMemcpyAsync(p->host_out, p->out_d, 2 * sizeof(double), cudaMemcpyDeviceToHost, st),
                             "sdt_plan_launch");
    if (!rc) rc = cuda_check(cudaMemcpyAsync(p->host_out + 2, p->task_d, 2 * p->n * sizeof(double),
                                             cudaMemcpyDeviceToHost, st), "sdt_plan_launch");
    if (!rc) rc = cuda_check(cudaMemcpyAsync(p->err_h, p->err_d, sizeof(int), cudaMemcpyDeviceToHost, st),
                             "sdt_plan_launch");
    return rc;
}

// Enqueues one evaluation (device work only).
int plan_enqueue(sdt_plan *p, cudaStream_t st) {
    sdt_job *j = p->job;
    if (p->mtype >= 0 && j->mixed_type != p->mtype)
        return fail(SDT_ERR_STATE, "sdt_plan_launch: the job's split operands are of another precision "
                                   "(a later plan or run re-encoded them); create the plan again");
    if (p->n == 0) return SDT_OK;
    int rc = cuda_check(cudaMemsetAsync(p->err_d, 0, sizeof(int), st), "sdt_plan_launch");
    if (rc) return rc;
    // Under stream capture the timing events are recorded as external events,
    // which become event-record nodes of the graph, so replays time the
    // kernels too (outside capture that flag is not accepted).
    const bool timed = j->timing && j->ev0 && j->ev1;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (timed) rc = cuda_check(cudaStreamIsCapturing(st, &cap), "sdt_plan_launch");
    const unsigned evflag = cap == cudaStreamCaptureStatusActive ? cudaEventRecordExternal : cudaEventRecordDefault;
    if (timed && !rc) rc = cuda_check(cudaEventRecordWithFlags(j->ev0, st, evflag), "sdt_plan_launch");
    if (rc) return rc;
    for (size_t gi = 0; gi < p->groups.size() && !rc; ++gi) {
        const LaunchArgs a = group_args(p, gi);
        rc = p->mtype >= 0 ? mixed_launch(j, a, st) : fp64_launch(j, a, st);
    }
    if (timed && !rc) rc = cuda_check(cudaEventRecordWithFlags(j->ev1, st, evflag), "sdt_plan_launch");
    if (!rc) rc = plan_sums(p, st);
    return rc;
}

int plan_read(sdt_plan *p, cudaStream_t st, double *energy, double *per_task, const char *who) {
    int rc = cuda_check(cudaStreamSynchronize(st), who);
    if (rc) return rc;
    sdt_job *j = p->job;
    if (j->timing && j->ev0 && j->ev1 && cudaEventElapsedTime(&j->last_ms, j->ev0, j->ev1) != cudaSuccess) {
        cudaGetLastError();  // no timing for this run; leave no stale error behind
        j->last_ms = -1.0f;
    }
    if (*p->err_h)
        return fail(SDT_ERR_TIMEOUT, std::string(who) + ": a bounded wait in the mixed kernel ran out (code " +
                                         std::to_string(*p->err_h) + ")");
    energy[0] = p->n ? p->host_out[0] : 0.0;
    energy[1] = p->n ? p->host_out[1] : 0.0;
    if (per_task)
        for (int64_t pos = 0; pos < p->n; ++pos) {
            per_task[2 * p->order[pos]] = p->host_out[2 + 2 * pos];
            per_task[2 * p->order[pos] + 1] = p->host_out[3 + 2 * pos];
        }
    return SDT_OK;
}

}  // namespace

int plan_make(sdt_job *j, const int64_t *klist, int64_t n, int precision, const int32_t *shapes, sdt_plan **out) {
    return plan_create(j, klist, n, precision, shapes, out, "sdt_plan_create");
}

int plan_queue_entry(sdt_plan *p, void *entry, int64_t *items) {
    if (p->mtype < 0 || p->groups.size() != 1)
        return fail(SDT_ERR_ARG, "queue entry: a mixed-form plan of one work-unit shape is needed");
    *items = p->items;
    return mixed_job_entry(p->job, group_args(p, 0), entry);
}

int plan_finish(sdt_plan *p, cudaStream_t st, double *energy) {
    if (p->n == 0) {
        energy[0] = energy[1] = 0.0;
        return SDT_OK;
    }
    int rc = cuda_check(cudaMemsetAsync(p->err_d, 0, sizeof(int), st), "plan finish");
    if (!rc) rc = plan_sums(p, st);
    if (!rc) rc = plan_read(p, st, energy, nullptr, "plan finish");
    return rc;
}

void plan_release(sdt_plan *p) { plan_free(p); }
}  // namespace sdt

using namespace sdt;

extern "C" int sdt_plan_create(sdt_job *job, const int64_t *klist, int64_t n, int precision, const int32_t *shapes,
                               sdt_plan **plan) {
    if (!plan) return fail(SDT_ERR_ARG, "sdt_plan_create: null output");
    return plan_create(job, klist, n, precision, shapes, plan, "sdt_plan_create");
}

extern "C" int sdt_plan_launch(sdt_plan *plan, void *stream) {
    if (!plan) return fail(SDT_ERR_ARG, "sdt_plan_launch: null plan");
    return plan_enqueue(plan, stream ? (cudaStream_t)stream : plan->job->stream);
}

extern "C" int sdt_plan_capture(sdt_plan *plan, void *stream) {
    if (!plan) return fail(SDT_ERR_ARG, "sdt_plan_capture: null plan");
    cudaStream_t st = stream ? (cudaStream_t)stream : plan->job->stream;
    if (plan->exec) {
        cudaGraphExecDestroy(plan->exec);
        plan->exec = nullptr;
    }
    if (plan->graph) {
        cudaGraphDestroy(plan->graph);
        plan->graph = nullptr;
    }
    int rc = cuda_check(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal), "sdt_plan_capture");
    if (rc) return rc;
    const int64_t before = g_launches.load();
    const int rc_launch = plan_enqueue(plan, st);
    g_launches.store(before);  // a capture launches nothing
    cudaGraph_t g = nullptr;
    rc = cuda_check(cudaStreamEndCapture(st, &g), "sdt_plan_capture");
    if (rc_launch || rc) {
        if (g) cudaGraphDestroy(g);
        return rc_launch ? rc_launch : rc;
    }
    plan->graph = g;
    return cuda_check(cudaGraphInstantiate(&plan->exec, g, 0), "sdt_plan_capture: instantiate");
}

extern "C" int sdt_plan_run(sdt_plan *plan, void *stream, double *energy, double *per_task) {
    if (!plan || !energy) return fail(SDT_ERR_ARG, "sdt_plan_run: null argument");
    cudaStream_t st = stream ? (cudaStream_t)stream : plan->job->stream;
    int rc;
    if (plan->exec) {
        if (plan->mtype >= 0 && plan->job->mixed_type != plan->mtype)
            return fail(SDT_ERR_STATE, "sdt_plan_run: the job's split operands are of another precision");
        rc = cuda_check(cudaGraphLaunch(plan->exec, st), "sdt_plan_run");
        if (!rc && plan->n) count_launch(plan->kernels);
    } else {
        rc = plan_enqueue(plan, st);
    }
    if (rc) return rc;
    return plan_read(plan, st, energy, per_task, "sdt_plan_run");
}

extern "C" int sdt_plan_destroy(sdt_plan *plan) {
    if (!plan) return SDT_OK;
    cudaStreamSynchronize(plan->job->stream);
    plan_free(plan);
    return SDT_OK;
}

extern "C" int64_t sdt_plan_items(const sdt_plan *plan) { return plan ? plan->items : -1; }

extern "C" int sdt_plan_item_energies(sdt_plan *plan, double *pairs, int64_t n) {
    if (!plan || !pairs || n != plan->items) return fail(SDT_ERR_ARG, "sdt_plan_item_energies: bad argument");
    cudaStream_t st = plan->job->stream;
    int rc = cuda_check(cudaMemcpyAsync(pairs, plan->part_d, 2 * n * sizeof(double), cudaMemcpyDeviceToHost, st),
                        "sdt_plan_item_energies");
    if (!rc) rc = cuda_check(cudaStreamSynchronize(st), "sdt_plan_item_energies");
    return rc;
}

extern "C" int sdt_job_run(sdt_job *j, const int64_t *klist, int64_t n, int precision, double *energy,
                           double *per_task, void *stream) {
    if (!j || !energy || (n > 0 && !klist)) return fail(SDT_ERR_ARG, "sdt_job_run: null argument");
    energy[0] = energy[1] = 0.0;
    PhaseTrace tr("sdt_job_run");
    cudaStream_t st = stream ? (cudaStream_t)stream : j->stream;
    sdt_plan *p = nullptr;
    int rc = plan_create(j, klist, n, precision, nullptr, &p, "sdt_job_run");
    if (rc) return rc;
    tr.mark("plan", st);
    rc = plan_enqueue(p, st);
    if (!rc) rc = plan_read(p, st, energy, per_task, "sdt_job_run");
    else cudaStreamSynchronize(st);
    tr.mark("kernels+sums", nullptr);
    plan_free(p);
    return rc;
}
