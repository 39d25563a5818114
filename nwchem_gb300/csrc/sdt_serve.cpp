// sdt_serve.cpp -- a serving loop for independent (T) jobs on one GPU (no
// reference counterpart: NWChem evaluates one (T) problem per run).
//
// Clients submit jobs (a tiling and its T1/T2/V2 files) at any time.  Jobs
// wait in one FIFO queue; a job is admitted when fewer than `slots` jobs are
// in flight and its device bytes fit in the HBM budget minus the bytes of
// the jobs already admitted (a job larger than the whole budget is
// rejected).  `slots` worker threads admit and load jobs: device tables, H2D
// copy and ingest of the files, the mixed form's operand encoding and the
// job's work index, each job on its own CUDA stream.
//
// Continuous batching (the default, for jobs of the server's mixed form):
// a loaded job's sub-box items are appended to one shared device queue that
// a resident persistent kernel drains -- the job's parameters go into a
// device job table and the queue's tail grows by its item count, while the
// kernel runs.  The kernel holds all SMs but `reserve` of them, which stay
// free for the loading, encoding and final sums of other jobs and for FP64
// checks, so jobs arriving while others compute are loaded and enter the
// same queue.  The kernel counts each job's finished items and the last one
// sets a host-visible flag; a monitor thread then runs the job's per-tuple
// and total sums, delivers its energies and returns its memory.  The kernel
// leaves after a quiet period with nothing to take; the monitor launches it
// again when work is appended.  Other precisions run one launch per job.
//
// A job with an FP64 check keeps its device memory (and its admitted bytes)
// after its energies are delivered; the check runs when no admissible job is
// waiting, on `check_ctas` SMs, so checks do not hold back the stream.  A
// job's result depends only on its inputs, never on what ran beside it.
#include "sdt_internal.h"
#include "sdt_job.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

namespace sdt {
namespace {

// FIFO admission against slots and a byte budget (the server and
// sdt_admission_simulate share it).
struct Admission {
    int64_t budget = 0, in_use = 0, peak = 0;
    int slots = 1, busy = 0;
    bool fits_ever(int64_t bytes) const { return bytes <= budget; }
    bool can_admit(int64_t bytes) const { return busy < slots && in_use + bytes <= budget; }
    void admit(int64_t bytes) {
        ++busy;
        in_use += bytes;
        peak = std::max(peak, in_use);
    }
    void release(int64_t bytes) {
        --busy;
        in_use -= bytes;
    }
    // A job held for its deferred FP64 check keeps its bytes but no slot.
    void free_slot() { --busy; }
    void take_slot() { ++busy; }
};

int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

}  // namespace

// Device bytes a job needs at its peak (an upper bound of the allocations of
// sdt_job_create/load/run): the dense FP64 operands, the raw files during
// ingest, for a mixed precision the split block layouts and FP32 copies, and
// the run's partial sums.
int64_t job_bytes(const sdt_tiling *ti, int precision) {
    Tiling t;
    if (!make_tiling(ti, &t)) return -1;
    const int64_t o = t.nocc, v = t.nvir, N = t.noab + t.nvab;
    int64_t vd2 = 0, vd2_blocks_pairs = 0, nob = 0, nvb = 0;
    for (int64_t b = 1; b <= t.noab; ++b) nob += ceil_div(t.r(b), 4);
    for (int64_t b = t.noab + 1; b <= N; ++b) nvb += ceil_div(t.r(b), 8);
    for (int64_t B = t.noab + 1; B <= N; ++B)
        for (int64_t C = B; C <= N; ++C) {
            vd2 += t.r(B) * t.r(C) * o * v;
            vd2_blocks_pairs += ceil_div(t.r(B), 8) * ceil_div(t.r(C), 8);
        }
    int64_t bytes = 8 * (v * o + 3 * v * v * o * o + vd2 + v * o * o * o);
    // raw TCE files (canonical blocks: at most the dense sizes) during ingest
    bytes += 8 * (v * o + v * v * o * o + vd2 + v * o * o * o + v * v * o * o);
    int64_t items = 0;
    const int64_t n = sdt_tasks_count(ti);
    if (n > 0) {
        std::vector<int64_t> kl(7 * n);
        if (sdt_tasks_list(ti, n, kl.data()) == SDT_OK) {
            const int bv = precision == SDT_PREC_FP64 ? 4 : 8;
            for (int64_t q = 0; q < n; ++q) {
                int64_t boxes = 1;
                for (int d = 0; d < 6; ++d) boxes *= ceil_div(t.r(kl[7 * q + d]), d < 3 ? bv : 4);
                items += boxes;
            }
        }
        bytes += 16 * items + 64 * n;
    }
    if (precision != SDT_PREC_FP64) {
        const int64_t es = precision == SDT_PREC_MIXED_TF32 ? 4 : 2, ke = 32 / es;
        const int64_t nko = ceil_div(o, ke), nkv = ceil_div(v, ke);
        const int64_t blocks_a = nvb * nob * nob * (nko + nkv);
        const int64_t blocks_b = nvb * nvb * nob * nko + vd2_blocks_pairs * nob * nkv;
        bytes += 2 * (blocks_a * 4096 + blocks_b * 8192);
        // FP32 copies of T1 and the vvoo block with holes padded per tile to
        // multiples of 4, then the orbital energies
        const int64_t op = 4 * nob;
        bytes += 4 * (v * op + v * v * op * op + o + v);
    }
    return bytes + bytes / 20 + (64ll << 20);
}

}  // namespace sdt

using namespace sdt;

struct sdt_server {
    struct Job {
        int64_t id = 0;
        std::vector<int64_t> range, spin, sym, offset, alpha;
        std::vector<double> evl;
        sdt_tiling t{};
        sdt_file f1{}, f2{}, fv{};
        int precision = SDT_PREC_MIXED_FP16, check = 0;
        int64_t bytes = 0;
        int state = 0;  // 0 queued, 1 running, 3 energies ready (FP64 check pending), 2 done, -1 failed
        double e[2] = {0, 0}, f[2] = {0, 0};
        double t_submit = 0, t_start = 0, t_loaded = 0, t_ran = 0, t_end = 0;
        int err = 0;
        std::string msg;
        sdt_job *held = nullptr;  // kept on the device for the deferred FP64 check
        std::vector<int64_t> kl;
        // shared-queue jobs: device data and plan while queued, queue slot,
        // launch numbers that took the first and finished the last item
        sdt_job *dj = nullptr;
        sdt_plan *plan = nullptr;
        int slot = -1, first_gen = 0, last_gen = 0;
    };
    // The shared item queue (continuous batching), set up at its first use.
    struct Queue {
        int precision = SDT_PREC_MIXED_FP16, type = TM_F16, shape = 1, reserve = 16, max_jobs = 4096;
        double idle_s = 0.2;
        bool ready = false;
        size_t entry = 0;
        void *table_d = nullptr;
        long long *base_d = nullptr;
        unsigned long long *head_d = nullptr, *tail_d = nullptr, *done_d = nullptr;
        int *close_d = nullptr, *err_d = nullptr;
        int *gen_h = nullptr, *gen_dp = nullptr;  // host-mapped [2][max_jobs]: first / last launch per slot
        uint8_t *stage_h = nullptr;               // pinned: table entries, bases, tails, read-back
        cudaStream_t kst = nullptr, pst = nullptr;
        cudaEvent_t kev = nullptr;
        bool running = false;
        int gen = 0, next_slot = 0, grid = 0;
        unsigned long long tail = 0;
        int64_t launches = 0, jobs = 0, in_flight = 0, max_in_flight = 0;
        std::vector<Job *> by_slot;
        std::mutex mu;
    } q;
    std::thread monitor;
    bool use_queue = true, mon_stop = false;
    int64_t budget = 0;
    int slots = 1, max_ctas = 0;
    int sms = 0, check_ctas = 0, checks_running = 0;
    std::mutex mu;
    std::condition_variable cv;
    std::deque<Job *> queue;
    std::deque<Job *> checks;  // energies delivered, FP64 check pending (FIFO)
    std::vector<std::unique_ptr<Job>> jobs;
    Admission adm;
    std::vector<std::thread> workers;
    bool stop = false;
    int device = 0;
    std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
    double now() const {
        return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
};

namespace {

void run_one(sdt_server *s, sdt_server::Job *job) {
    cudaSetDevice(s->device);
    sdt_job *j = nullptr;
    auto failed = [&](int rc) {
        char buf[512] = {0};
        sdt_last_error(buf, sizeof(buf));
        job->err = rc;
        job->msg = buf;
        return rc;
    };
    int rc = sdt_job_create(&job->t, &j);
    if (rc) {
        failed(rc);
        return;
    }
    rc = sdt_job_load(j, &job->f1, &job->f2, &job->fv, nullptr);
    job->t_loaded = s->now();
    int64_t n = 0;
    if (!rc) {
        n = sdt_tasks_count(&job->t);
        job->kl.resize(7 * std::max<int64_t>(n, 1));
        rc = n < 0 ? SDT_ERR_ARG : sdt_tasks_list(&job->t, n, job->kl.data());
        if (!rc) job->kl.resize(7 * n);
    }
    if (!rc) {
        // While an FP64 check holds check_ctas SMs, launch on the others (a
        // persistent launch wider than the free SMs would end only after
        // the check).
        int cap = s->max_ctas;
        {
            std::lock_guard<std::mutex> lk(s->mu);
            if (s->checks_running > 0 && s->check_ctas > 0) {
                const int free_sms = std::max(s->sms - s->check_ctas * s->checks_running, 1);
                cap = cap > 0 ? std::min(cap, free_sms) : free_sms;
            }
        }
        sdt_job_set_max_ctas(j, cap);
        rc = sdt_job_run(j, job->kl.data(), n, job->precision, job->e, nullptr, nullptr);
    }
    job->t_ran = s->now();
    if (!rc && job->check) {
        job->held = j;  // the FP64 check runs later, when no admissible job waits
        return;
    }
    if (rc) failed(rc);
    sdt_job_destroy(j);
}

// ---------------------------------------------------------------------------
// The shared item queue.

constexpr long long kUnusedBase = 0x7fffffffffffffffll;

// Device and pinned buffers of the queue and its two streams (q.mu held).
int queue_setup(sdt_server *s) {
    auto &Q = s->q;
    if (Q.ready) return SDT_OK;
    Q.entry = mixed_job_entry_bytes();
    Q.by_slot.assign(Q.max_jobs, nullptr);
    Q.grid = std::max(1, s->sms - Q.reserve);
    int rc = mixed_queue_prepare(Q.type, Q.shape);
    auto dev = [&](void **p, size_t bytes) {
        if (!rc) rc = cuda_check(cudaMalloc(p, bytes), "sdt_server: queue buffers");
    };
    dev(&Q.table_d, Q.entry * Q.max_jobs);
    dev((void **)&Q.base_d, sizeof(long long) * Q.max_jobs);
    dev((void **)&Q.done_d, sizeof(unsigned long long) * Q.max_jobs);
    dev((void **)&Q.head_d, 2 * sizeof(unsigned long long));
    dev((void **)&Q.close_d, 2 * sizeof(int));
    if (Q.head_d) Q.tail_d = Q.head_d + 1;
    if (Q.close_d) Q.err_d = Q.close_d + 1;
    if (!rc) rc = cuda_check(cudaHostAlloc((void **)&Q.gen_h, 2 * sizeof(int) * Q.max_jobs, cudaHostAllocMapped),
                             "sdt_server: queue flags");
    if (!rc) rc = cuda_check(cudaHostGetDevicePointer((void **)&Q.gen_dp, Q.gen_h, 0), "sdt_server: queue flags");
    if (!rc) rc = cuda_check(cudaHostAlloc((void **)&Q.stage_h, (Q.entry + 16) * Q.max_jobs + 64, cudaHostAllocDefault),
                             "sdt_server: queue staging");
    if (!rc) rc = cuda_check(cudaStreamCreateWithFlags(&Q.kst, cudaStreamNonBlocking), "sdt_server: queue stream");
    if (!rc) rc = cuda_check(cudaStreamCreateWithFlags(&Q.pst, cudaStreamNonBlocking), "sdt_server: queue stream");
    if (!rc) rc = cuda_check(cudaEventCreateWithFlags(&Q.kev, cudaEventDisableTiming), "sdt_server: queue event");
    if (rc) return rc;
    Q.ready = true;
    Q.next_slot = Q.max_jobs;  // the first publish resets the queue
    return SDT_OK;
}

long long *stage_base(sdt_server::Queue &Q) { return (long long *)(Q.stage_h + Q.entry * Q.max_jobs); }
unsigned long long *stage_tail(sdt_server::Queue &Q) {
    return (unsigned long long *)(Q.stage_h + (Q.entry + 8) * Q.max_jobs);
}
int *stage_word(sdt_server::Queue &Q) { return (int *)(Q.stage_h + (Q.entry + 16) * Q.max_jobs); }

// Empties the queue for a new round of slots (no kernel running, no job in
// flight; q.mu held).
int queue_reset(sdt_server *s) {
    auto &Q = s->q;
    int rc = cuda_check(cudaMemsetAsync(Q.base_d, 0x7f, sizeof(long long) * Q.max_jobs, Q.pst), "sdt_server: queue");
    if (!rc) rc = cuda_check(cudaMemsetAsync(Q.done_d, 0, sizeof(unsigned long long) * Q.max_jobs, Q.pst), "sdt_server");
    if (!rc) rc = cuda_check(cudaMemsetAsync(Q.head_d, 0, 2 * sizeof(unsigned long long), Q.pst), "sdt_server");
    if (!rc) rc = cuda_check(cudaMemsetAsync(Q.close_d, 0, 2 * sizeof(int), Q.pst), "sdt_server");
    if (!rc) rc = cuda_check(cudaStreamSynchronize(Q.pst), "sdt_server: queue reset");
    std::memset(Q.gen_h, 0, 2 * sizeof(int) * Q.max_jobs);
    std::fill(Q.by_slot.begin(), Q.by_slot.end(), nullptr);
    Q.next_slot = 0;
    Q.tail = 0;
    return rc;
}

// Notes a finished kernel (q.mu held): returns its error code, 0 if none.
int queue_reap(sdt_server *s) {
    auto &Q = s->q;
    if (!Q.running) return SDT_OK;
    const cudaError_t e = cudaEventQuery(Q.kev);
    if (e == cudaErrorNotReady) return SDT_OK;
    Q.running = false;
    if (trace_on()) std::fprintf(stderr, "[sdt trace] t=%.4f queue launch %d ended\n", s->now(), Q.gen);
    int rc = cuda_check(e, "sdt_server: queue kernel");
    int *w = stage_word(Q);
    if (!rc) rc = cuda_check(cudaMemcpyAsync(w, Q.err_d, sizeof(int), cudaMemcpyDeviceToHost, Q.pst), "sdt_server");
    if (!rc) rc = cuda_check(cudaStreamSynchronize(Q.pst), "sdt_server");
    if (!rc && *w)
        rc = fail(SDT_ERR_TIMEOUT, "sdt_server: a bounded wait in the queue kernel ran out (code " +
                                       std::to_string(*w) + ")");
    return rc;
}

// Launches the resident kernel when it is not running and queue positions
// are left to take (q.mu held).
int queue_ensure(sdt_server *s) {
    auto &Q = s->q;
    int rc = queue_reap(s);
    if (rc || Q.running || Q.in_flight == 0) return rc;
    unsigned long long head = 0;
    rc = cuda_check(cudaMemcpyAsync(stage_word(Q) + 2, Q.head_d, sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                                    Q.pst), "sdt_server");
    if (!rc) rc = cuda_check(cudaStreamSynchronize(Q.pst), "sdt_server");
    if (rc) return rc;
    std::memcpy(&head, stage_word(Q) + 2, sizeof(head));
    if (head >= Q.tail) return SDT_OK;  // every published item is taken (and, with no kernel, finished)
    QueueArgs a;
    a.table = Q.table_d;
    a.base = Q.base_d;
    a.head = Q.head_d;
    a.tail = Q.tail_d;
    a.done = Q.done_d;
    a.first_gen = Q.gen_dp;
    a.last_gen = Q.gen_dp + Q.max_jobs;
    a.close = Q.close_d;
    a.err = Q.err_d;
    a.idle_ns = (unsigned long long)(Q.idle_s * 1e9);
    a.max_jobs = Q.max_jobs;
    a.gen = ++Q.gen;
    rc = cuda_check(cudaMemsetAsync(Q.close_d, 0, 2 * sizeof(int), Q.pst), "sdt_server");
    cudaEvent_t ev = nullptr;
    if (!rc) rc = cuda_check(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "sdt_server");
    if (!rc) rc = cuda_check(cudaEventRecord(ev, Q.pst), "sdt_server");
    if (!rc) rc = cuda_check(cudaStreamWaitEvent(Q.kst, ev, 0), "sdt_server");
    if (ev) cudaEventDestroy(ev);
    if (!rc) rc = mixed_queue_launch(Q.type, Q.shape, a, Q.grid, Q.kst);
    if (!rc) rc = cuda_check(cudaEventRecord(Q.kev, Q.kst), "sdt_server");
    if (!rc) {
        Q.running = true;
        ++Q.launches;
    }
    if (trace_on())
        std::fprintf(stderr, "[sdt trace] t=%.4f queue launch %d (head %llu, tail %llu, jobs in queue %lld)\n",
                     s->now(), Q.gen, head, Q.tail, (long long)Q.in_flight);
    return rc;
}

constexpr int kRetry = -1;

// Appends a loaded job's items to the queue (q.mu held).  kRetry: the slot
// table is used up and in use; call again once the queue has emptied.
int queue_publish(sdt_server *s, sdt_server::Job *job) {
    auto &Q = s->q;
    int rc = queue_setup(s);
    if (rc) return rc;
    if (Q.next_slot >= Q.max_jobs) {
        // a new round of slots: only once the queue is idle and empty
        if (Q.in_flight > 0) return kRetry;
        rc = queue_reap(s);
        if (rc) return rc;
        if (Q.running) return kRetry;
        rc = queue_reset(s);
        if (rc) return rc;
    }
    const int slot = Q.next_slot++;
    uint8_t *ent = Q.stage_h + Q.entry * slot;
    int64_t items = 0;
    rc = plan_queue_entry(job->plan, ent, &items);
    if (rc) return rc;
    stage_base(Q)[slot] = (long long)Q.tail;
    Q.tail += (unsigned long long)items;
    stage_tail(Q)[slot] = Q.tail;
    if (!rc) rc = cuda_check(cudaMemcpyAsync((uint8_t *)Q.table_d + Q.entry * slot, ent, Q.entry,
                                             cudaMemcpyHostToDevice, Q.pst), "sdt_server: publish");
    if (!rc) rc = cuda_check(cudaMemcpyAsync(Q.base_d + slot, stage_base(Q) + slot, sizeof(long long),
                                             cudaMemcpyHostToDevice, Q.pst), "sdt_server: publish");
    // the tail last: the kernel reads an entry only below the tail
    if (!rc) rc = cuda_check(cudaMemcpyAsync(Q.tail_d, stage_tail(Q) + slot, sizeof(unsigned long long),
                                             cudaMemcpyHostToDevice, Q.pst), "sdt_server: publish");
    if (rc) return rc;
    job->slot = slot;
    if (trace_on())
        std::fprintf(stderr, "[sdt trace] t=%.4f job %lld appended: slot %d, positions %lld..%llu\n", s->now(),
                     (long long)job->id, slot, stage_base(Q)[slot], Q.tail);
    Q.by_slot[slot] = job;
    ++Q.in_flight;
    ++Q.jobs;
    Q.max_in_flight = std::max(Q.max_in_flight, Q.in_flight);
    return queue_ensure(s);
}

std::string take_error() {
    char buf[512] = {0};
    sdt_last_error(buf, sizeof(buf));
    return buf;
}

// Loads a job and appends its items to the shared queue.  true: the job is
// in the queue (the monitor completes it); false: it finished here (an
// error, or no tuples).
bool run_queued(sdt_server *s, sdt_server::Job *job) {
    cudaSetDevice(s->device);
    sdt_job *j = nullptr;
    int rc = sdt_job_create(&job->t, &j);
    if (!rc) rc = sdt_job_load(j, &job->f1, &job->f2, &job->fv, nullptr);
    int64_t n = 0;
    if (!rc) {
        n = sdt_tasks_count(&job->t);
        job->kl.resize(7 * std::max<int64_t>(n, 1));
        rc = n < 0 ? SDT_ERR_ARG : sdt_tasks_list(&job->t, n, job->kl.data());
        if (!rc) job->kl.resize(7 * n);
    }
    if (!rc && n > 0) {
        std::vector<int32_t> shapes(n, s->q.shape);
        rc = plan_make(j, job->kl.data(), n, s->q.precision, shapes.data(), &job->plan);
    }
    job->t_loaded = s->now();
    if (!rc && n > 0) {
        job->dj = j;
        while (true) {
            {
                std::lock_guard<std::mutex> lk(s->q.mu);
                rc = queue_publish(s, job);
            }
            if (rc != kRetry) break;
            std::this_thread::sleep_for(std::chrono::milliseconds(1));
        }
        if (!rc) return true;
        job->dj = nullptr;
    }
    if (rc) {
        job->err = rc;
        job->msg = take_error();
    }
    job->t_ran = s->now();
    if (job->plan) plan_release(job->plan);
    job->plan = nullptr;
    if (!rc && job->check) {
        job->held = j;
        return false;
    }
    sdt_job_destroy(j);
    return false;
}

// A queued job whose items are all finished: its sums and energies, then
// its memory is returned (or kept for its FP64 check).
void queue_finish(sdt_server *s, sdt_server::Job *job, int rc_in) {
    int rc = rc_in;
    if (trace_on())
        std::fprintf(stderr, "[sdt trace] t=%.4f job %lld items done (launches %d..%d)\n", s->now(),
                     (long long)job->id, job->first_gen, job->last_gen);
    if (!rc) rc = plan_finish(job->plan, (cudaStream_t)sdt_job_stream(job->dj), job->e);
    if (rc) {
        job->err = rc;
        job->msg = rc_in ? "sdt_server: the queue kernel failed: " + take_error() : take_error();
    }
    job->t_ran = s->now();
    plan_release(job->plan);
    job->plan = nullptr;
    if (!rc && job->check) {
        job->held = job->dj;
    } else {
        sdt_job_destroy(job->dj);
    }
    job->dj = nullptr;
    std::lock_guard<std::mutex> lk(s->mu);
    if (job->held) {
        s->adm.free_slot();
        job->state = 3;
        s->checks.push_back(job);
    } else {
        s->adm.release(job->bytes);
        job->t_end = s->now();
        job->state = job->err ? -1 : 2;
    }
    s->cv.notify_all();
}

// Completes queued jobs as their last items finish and keeps the resident
// kernel running while queue positions are left to take.
void monitor(sdt_server *s) {
    cudaSetDevice(s->device);
    auto &Q = s->q;
    while (true) {
        std::vector<sdt_server::Job *> done;
        int rc = SDT_OK;
        bool stop = false;
        {
            std::lock_guard<std::mutex> lk(Q.mu);
            if (Q.ready) {
                const volatile int *last = Q.gen_h + Q.max_jobs;
                for (int slot = 0; slot < Q.next_slot && slot < Q.max_jobs; ++slot) {
                    sdt_server::Job *job = Q.by_slot[slot];
                    if (!job || last[slot] == 0) continue;
                    job->first_gen = ((const volatile int *)Q.gen_h)[slot];
                    job->last_gen = last[slot];
                    Q.by_slot[slot] = nullptr;
                    --Q.in_flight;
                    done.push_back(job);
                }
                rc = queue_ensure(s);
                if (rc) {  // the kernel failed: every job still in the queue fails with it
                    for (int slot = 0; slot < Q.max_jobs; ++slot)
                        if (Q.by_slot[slot]) {
                            done.push_back(Q.by_slot[slot]);
                            Q.by_slot[slot] = nullptr;
                        }
                    Q.in_flight = 0;
                    Q.next_slot = Q.max_jobs;  // the next publish starts a fresh queue
                }
            }
            stop = s->mon_stop && Q.in_flight == 0;
        }
        for (auto *job : done) queue_finish(s, job, (rc && job->last_gen == 0) ? rc : SDT_OK);
        if (stop) break;
        if (done.empty()) std::this_thread::sleep_for(std::chrono::microseconds(100));
    }
    // close the resident kernel and wait for it (its wait for work is bounded)
    std::lock_guard<std::mutex> lk(Q.mu);
    if (Q.ready && Q.running) {
        int one = 1;
        std::memcpy(stage_word(Q), &one, sizeof(int));
        cudaMemcpyAsync(Q.close_d, stage_word(Q), sizeof(int), cudaMemcpyHostToDevice, Q.pst);
        cudaStreamSynchronize(Q.pst);
        cudaEventSynchronize(Q.kev);
        Q.running = false;
    }
}

// The deferred FP64 check of a held job, then its device memory is returned.
void run_check(sdt_server *s, sdt_server::Job *job) {
    cudaSetDevice(s->device);
    const int64_t n = (int64_t)job->kl.size() / 7;
    // A check takes exactly check_ctas SMs (one CTA each).  With the shared queue those are part
    // of the SMs the resident kernel leaves free, so the kernel never waits for SMs a check holds
    // (a check runs for seconds) -- one check at a time, check_ctas <= reserve.
    sdt_job_set_sm_exclusive(job->held, s->check_ctas > 0);
    sdt_job_set_max_ctas(job->held, s->check_ctas);
    if (trace_on()) std::fprintf(stderr, "[sdt trace] t=%.4f FP64 check of job %lld starts\n", s->now(), (long long)job->id);
    const int rc = sdt_job_run(job->held, job->kl.data(), n, SDT_PREC_FP64, job->f, nullptr, nullptr);
    if (trace_on()) std::fprintf(stderr, "[sdt trace] t=%.4f FP64 check of job %lld ends\n", s->now(), (long long)job->id);
    if (rc) {
        char buf[512] = {0};
        sdt_last_error(buf, sizeof(buf));
        job->err = rc;
        job->msg = buf;
    }
    sdt_job_destroy(job->held);
    job->held = nullptr;
}

// Workers take the queue head when it can be admitted (or must be refused);
// otherwise, and only then, a pending FP64 check -- so checks fill the gaps
// instead of holding the GPU while admissible jobs wait.
void worker(sdt_server *s) {
    std::unique_lock<std::mutex> lk(s->mu);
    auto head_ready = [&] {
        return !s->queue.empty() &&
               (!s->adm.fits_ever(s->queue.front()->bytes) || s->adm.can_admit(s->queue.front()->bytes));
    };
    auto check_ready = [&] {
        return !s->checks.empty() && s->adm.busy < s->adm.slots && !head_ready() &&
               (!s->use_queue || s->checks_running == 0);
    };
    while (true) {
        s->cv.wait(lk, [&] { return s->stop || head_ready() || check_ready(); });
        if (s->stop) return;
        if (!head_ready()) {
            sdt_server::Job *job = s->checks.front();
            s->checks.pop_front();
            s->adm.take_slot();
            ++s->checks_running;
            lk.unlock();
            run_check(s, job);
            lk.lock();
            --s->checks_running;
            s->adm.release(job->bytes);
            job->t_end = s->now();
            job->state = job->err ? -1 : 2;
            s->cv.notify_all();
            continue;
        }
        sdt_server::Job *job = s->queue.front();
        s->queue.pop_front();
        if (!s->adm.fits_ever(job->bytes)) {
            job->state = -1;
            job->err = SDT_ERR_NOMEM;
            job->msg = "sdt_server: the job needs more device memory than the whole budget";
            job->t_start = job->t_end = s->now();
            s->cv.notify_all();
            continue;
        }
        s->adm.admit(job->bytes);
        job->state = 1;
        job->t_start = s->now();
        const bool queued = s->use_queue && job->precision == s->q.precision;
        lk.unlock();
        bool in_queue = false;
        if (queued) in_queue = run_queued(s, job);
        else run_one(s, job);
        lk.lock();
        if (in_queue) {  // the monitor completes it
            s->cv.notify_all();
            continue;
        }
        if (job->held) {  // energies delivered; memory kept for the check
            s->adm.free_slot();
            job->state = 3;
            s->checks.push_back(job);
        } else {
            s->adm.release(job->bytes);
            job->t_end = s->now();
            job->state = job->err ? -1 : 2;
        }
        s->cv.notify_all();
    }
}

}  // namespace

extern "C" int64_t sdt_job_bytes(const sdt_tiling *t, int precision) {
    if (!t || precision < SDT_PREC_FP64 || precision > SDT_PREC_MIXED_FP16) return -1;
    return job_bytes(t, precision);
}

extern "C" int sdt_server_create(int64_t budget_bytes, int slots, int max_ctas, sdt_server **out) {
    if (!out || budget_bytes <= 0 || slots < 1 || slots > 64 || max_ctas < 0)
        return fail(SDT_ERR_ARG, "sdt_server_create: bad argument");
    sdt_server *s = new sdt_server();
    s->budget = budget_bytes;
    s->slots = slots;
    s->max_ctas = max_ctas;
    s->adm.budget = budget_bytes;
    s->adm.slots = slots;
    cudaGetDevice(&s->device);
    if (cudaDeviceGetAttribute(&s->sms, cudaDevAttrMultiProcessorCount, s->device) != cudaSuccess) {
        cudaGetLastError();
        s->sms = 0;
    }
    s->check_ctas = std::max(1, s->q.reserve / 2);  // checks leave half the kernel-free SMs to job loads
    for (int k = 0; k < slots; ++k) s->workers.emplace_back(worker, s);
    s->monitor = std::thread(monitor, s);
    *out = s;
    return SDT_OK;
}

// The shared queue's form (precision; 0 turns the queue off: every job gets
// its own launches), work-unit shape (1 or 2), the SMs kept free of the
// resident kernel, and how long the kernel waits for work before it leaves.
// Before the first submit.
extern "C" int sdt_server_set_queue(sdt_server *s, int precision, int shape, int reserve_sms, double idle_s) {
    if (!s || precision < SDT_PREC_FP64 || precision > SDT_PREC_MIXED_FP16 || (shape != 1 && shape != 2) ||
        reserve_sms < 1 || !(idle_s > 0.0) || idle_s > 1.0)
        return fail(SDT_ERR_ARG, "sdt_server_set_queue: bad argument");
    std::lock_guard<std::mutex> lk(s->mu);
    std::lock_guard<std::mutex> lq(s->q.mu);
    if (!s->jobs.empty() || s->q.ready) return fail(SDT_ERR_STATE, "sdt_server_set_queue: jobs were submitted");
    if (s->sms > 0 && reserve_sms >= s->sms) return fail(SDT_ERR_ARG, "sdt_server_set_queue: no SM left for the queue");
    s->use_queue = precision != SDT_PREC_FP64;
    s->q.precision = precision;
    s->q.type = precision == SDT_PREC_MIXED_TF32 ? TM_F32 : precision == SDT_PREC_MIXED_BF16 ? TM_BF16 : TM_F16;
    s->q.shape = shape;
    s->q.reserve = reserve_sms;
    s->q.idle_s = idle_s;
    s->check_ctas = s->use_queue ? std::max(1, reserve_sms / 2) : s->sms / 4;
    return SDT_OK;
}

// stats[0] resident-kernel launches, [1] jobs that went through the queue,
// [2] most jobs in the queue at once, [3] jobs in it now.
extern "C" int sdt_server_queue_stats(sdt_server *s, int64_t *stats) {
    if (!s || !stats) return fail(SDT_ERR_ARG, "sdt_server_queue_stats: null argument");
    std::lock_guard<std::mutex> lk(s->q.mu);
    stats[0] = s->q.launches;
    stats[1] = s->q.jobs;
    stats[2] = s->q.max_in_flight;
    stats[3] = s->q.in_flight;
    return SDT_OK;
}

// The resident-kernel launches (numbered from 1) that took a queued job's
// first item and finished its last one; 0 for a job that did not go through
// the queue (or has not finished).
extern "C" int sdt_server_job_launches(sdt_server *s, int64_t ticket, int *first, int *last) {
    if (!s || !first || !last) return fail(SDT_ERR_ARG, "sdt_server_job_launches: null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    if (ticket < 0 || ticket >= (int64_t)s->jobs.size()) return fail(SDT_ERR_ARG, "sdt_server_job_launches: bad ticket");
    *first = s->jobs[ticket]->first_gen;
    *last = s->jobs[ticket]->last_gen;
    return SDT_OK;
}

// SMs of each deferred FP64 check's persistent launch (default: a quarter
// of them, one CTA per SM); while checks run, mixed jobs launch on the
// remaining SMs.  0: checks use the whole GPU and do not cap other jobs.
extern "C" int sdt_server_set_check_ctas(sdt_server *s, int ctas) {
    if (!s || ctas < 0) return fail(SDT_ERR_ARG, "sdt_server_set_check_ctas: bad argument");
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->use_queue && (ctas < 1 || ctas > s->q.reserve))
        return fail(SDT_ERR_ARG, "sdt_server_set_check_ctas: with the shared queue, 1 to reserve SMs");
    s->check_ctas = s->sms > 0 ? std::min(ctas, s->sms - 1) : ctas;
    return SDT_OK;
}

extern "C" int sdt_server_submit(sdt_server *s, const sdt_tiling *t, const sdt_file *t1, const sdt_file *t2,
                                 const sdt_file *v2, int precision, int check_fp64, int64_t *ticket) {
    if (!s || !t || !t1 || !t2 || !v2 || !ticket) return fail(SDT_ERR_ARG, "sdt_server_submit: null argument");
    if (precision < SDT_PREC_FP64 || precision > SDT_PREC_MIXED_FP16)
        return fail(SDT_ERR_ARG, "sdt_server_submit: unknown precision");
    Tiling tt;
    if (!make_tiling(t, &tt)) return fail(SDT_ERR_ARG, "sdt_server_submit: bad tiling");
    auto job = std::make_unique<sdt_server::Job>();
    const int64_t nt = t->noab + t->nvab;
    job->range.assign(t->range, t->range + nt);
    job->spin.assign(t->spin, t->spin + nt);
    job->sym.assign(t->sym, t->sym + nt);
    job->offset.assign(t->offset, t->offset + nt);
    if (t->alpha) job->alpha.assign(t->alpha, t->alpha + nt);
    job->evl.assign(t->evl_sorted, t->evl_sorted + (tt.nocc + tt.nvir));
    job->t = *t;
    job->t.range = job->range.data();
    job->t.spin = job->spin.data();
    job->t.sym = job->sym.data();
    job->t.offset = job->offset.data();
    job->t.alpha = job->alpha.empty() ? nullptr : job->alpha.data();
    job->t.evl_sorted = job->evl.data();
    job->f1 = *t1;
    job->f2 = *t2;
    job->fv = *v2;
    job->precision = precision;
    job->check = check_fp64 ? 1 : 0;
    job->bytes = job_bytes(&job->t, precision);
    if (job->bytes < 0) return fail(SDT_ERR_ARG, "sdt_server_submit: bad tiling");
    std::lock_guard<std::mutex> lk(s->mu);
    job->id = (int64_t)s->jobs.size();
    job->t_submit = s->now();
    *ticket = job->id;
    s->queue.push_back(job.get());
    s->jobs.push_back(std::move(job));
    s->cv.notify_all();
    return SDT_OK;
}

// state: 0 queued, 1 running, 3 energies ready with the FP64 check pending,
// 2 done, -1 failed (sdt_last_error-style message in msg when given).  energy: the job's (E[T], E(T)); fp64: the FP64 check
// (when requested); times (5 values, seconds since the server was created):
// submission, admission, inputs on the device (job tables built, files
// copied and ingested), energies of the requested precision ready (operand
// encoding, plan and kernels done), and completion (after the FP64 check
// when one was requested, and the job's memory returned).
extern "C" int sdt_server_status(sdt_server *s, int64_t ticket, int *state, double *energy, double *fp64,
                                 double *times, char *msg, size_t len) {
    if (!s || !state) return fail(SDT_ERR_ARG, "sdt_server_status: null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    if (ticket < 0 || ticket >= (int64_t)s->jobs.size()) return fail(SDT_ERR_ARG, "sdt_server_status: bad ticket");
    const auto &j = *s->jobs[ticket];
    *state = j.state;
    if (energy) energy[0] = j.e[0], energy[1] = j.e[1];
    if (fp64) fp64[0] = j.f[0], fp64[1] = j.f[1];
    if (times) {
        times[0] = j.t_submit, times[1] = j.t_start, times[2] = j.t_loaded;
        times[3] = j.t_ran, times[4] = j.t_end;
    }
    if (msg && len) std::snprintf(msg, len, "%s", j.msg.c_str());
    return j.state < 0 ? j.err : SDT_OK;
}

// Cancels a job that is still queued: it leaves the queue with state -1 and
// SDT_ERR_STATE ("cancelled").  A job already admitted runs to the end
// (SDT_ERR_STATE is returned and nothing changes).
extern "C" int sdt_server_cancel(sdt_server *s, int64_t ticket) {
    if (!s) return fail(SDT_ERR_ARG, "sdt_server_cancel: null server");
    std::lock_guard<std::mutex> lk(s->mu);
    if (ticket < 0 || ticket >= (int64_t)s->jobs.size()) return fail(SDT_ERR_ARG, "sdt_server_cancel: bad ticket");
    sdt_server::Job *job = s->jobs[ticket].get();
    auto it = std::find(s->queue.begin(), s->queue.end(), job);
    if (it == s->queue.end()) return fail(SDT_ERR_STATE, "sdt_server_cancel: the job is no longer queued");
    s->queue.erase(it);
    job->state = -1;
    job->err = SDT_ERR_STATE;
    job->msg = "sdt_server: cancelled while queued";
    job->t_start = job->t_end = s->now();
    s->cv.notify_all();
    return SDT_OK;
}

// Waits until every submitted job has finished (or timeout_s passed:
// SDT_ERR_TIMEOUT).
extern "C" int sdt_server_drain(sdt_server *s, double timeout_s) {
    if (!s) return fail(SDT_ERR_ARG, "sdt_server_drain: null server");
    std::unique_lock<std::mutex> lk(s->mu);
    auto done = [&] { return s->queue.empty() && s->checks.empty() && !s->adm.busy; };
    if (!s->cv.wait_for(lk, std::chrono::duration<double>(timeout_s), done))
        return fail(SDT_ERR_TIMEOUT, "sdt_server_drain: jobs still running");
    return SDT_OK;
}

extern "C" int64_t sdt_server_peak_bytes(sdt_server *s) {
    if (!s) return -1;
    std::lock_guard<std::mutex> lk(s->mu);
    return s->adm.peak;
}

// Stops the workers after their running jobs; queued jobs and pending FP64
// checks are dropped (the held jobs' memory is returned).
extern "C" int sdt_server_destroy(sdt_server *s) {
    if (!s) return SDT_OK;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
        s->cv.notify_all();
    }
    for (auto &w : s->workers) w.join();
    {
        std::lock_guard<std::mutex> lq(s->q.mu);
        s->mon_stop = true;  // the monitor finishes the queued jobs, then closes the kernel
    }
    if (s->monitor.joinable()) s->monitor.join();
    for (auto &job : s->jobs)
        if (job->held) {
            sdt_job_destroy(job->held);
            job->held = nullptr;
        }
    auto &Q = s->q;
    if (Q.ready) {
        cudaFree(Q.table_d);
        cudaFree(Q.base_d);
        cudaFree(Q.done_d);
        cudaFree(Q.head_d);
        cudaFree(Q.close_d);
        cudaFreeHost(Q.gen_h);
        cudaFreeHost(Q.stage_h);
        cudaStreamDestroy(Q.kst);
        cudaStreamDestroy(Q.pst);
        cudaEventDestroy(Q.kev);
    }
    delete s;
    return SDT_OK;
}

// The admission policy alone, as an event simulation: n jobs arriving at
// arrival[q] (ascending) with device bytes bytes[q] and run times
// service[q]; start[q] and end[q] receive admission and completion times
// (-1 for a job larger than the budget).  No GPU is used.
extern "C" int sdt_admission_simulate(int64_t n, const double *arrival, const int64_t *bytes, const double *service,
                                      int64_t budget, int slots, double *start, double *end) {
    if (n < 0 || (n > 0 && (!arrival || !bytes || !service || !start || !end)) || budget <= 0 || slots < 1)
        return fail(SDT_ERR_ARG, "sdt_admission_simulate: bad argument");
    Admission adm;
    adm.budget = budget;
    adm.slots = slots;
    std::vector<std::pair<double, int64_t>> running;  // (end time, job)
    int64_t head = 0;
    double clock = 0.0;
    while (head < n || !running.empty()) {
        // admit in FIFO order everything that has arrived and fits now
        bool progress = true;
        while (progress && head < n && arrival[head] <= clock) {
            progress = false;
            if (!adm.fits_ever(bytes[head])) {
                start[head] = end[head] = -1.0;
                ++head;
                progress = true;
            } else if (adm.can_admit(bytes[head])) {
                adm.admit(bytes[head]);
                start[head] = clock;
                end[head] = clock + service[head];
                running.emplace_back(end[head], head);
                ++head;
                progress = true;
            }
        }
        // next event: the earliest completion or the next arrival
        double next = 1e300;
        for (auto &r : running) next = std::min(next, r.first);
        if (head < n && (adm.can_admit(bytes[head]) || !adm.fits_ever(bytes[head])))
            next = std::min(next, std::max(clock, arrival[head]));
        if (next >= 1e300) break;
        clock = next;
        for (size_t q = 0; q < running.size();) {
            if (running[q].first <= clock) {
                adm.release(bytes[running[q].second]);
                running[q] = running.back();
                running.pop_back();
            } else {
                ++q;
            }
        }
    }
    return SDT_OK;
}

// The serving policy with deferred FP64 checks, as an event simulation on the
// host (the same rules as the workers above): jobs arrive at arrival[q]
// (ascending) with device bytes bytes[q], mixed run time service[q] and FP64
// check time check_service[q] (< 0: no check).  A queue head is refused if it
// can never fit and admitted (FIFO) when a slot is free and its bytes fit;
// only when no head can be admitted does a free slot take the oldest pending
// check.  A checked job keeps its bytes, but not its slot, between its
// energies and its check.  start[q], ready[q] (energies) and done[q] (check
// finished, memory returned) receive the times; -1 for a refused job.
extern "C" int sdt_serving_simulate(int64_t n, const double *arrival, const int64_t *bytes, const double *service,
                                    const double *check_service, int64_t budget, int slots, double *start,
                                    double *ready, double *done) {
    if (n < 0 || (n > 0 && (!arrival || !bytes || !service || !check_service || !start || !ready || !done)) ||
        budget <= 0 || slots < 1)
        return fail(SDT_ERR_ARG, "sdt_serving_simulate: bad argument");
    struct Run {
        double end;
        int64_t job;
        bool check;
    };
    Admission adm;
    adm.budget = budget;
    adm.slots = slots;
    std::vector<Run> running;
    std::deque<int64_t> checks;
    int64_t head = 0;
    double clock = 0.0;
    while (true) {
        bool progress = true;
        while (progress) {
            progress = false;
            const bool has_head = head < n && arrival[head] <= clock;
            if (has_head && !adm.fits_ever(bytes[head])) {
                start[head] = ready[head] = done[head] = -1.0;
                ++head;
                progress = true;
            } else if (has_head && adm.can_admit(bytes[head])) {
                adm.admit(bytes[head]);
                start[head] = clock;
                running.push_back({clock + service[head], head, false});
                ++head;
                progress = true;
            } else if (!checks.empty() && adm.busy < adm.slots) {
                adm.take_slot();
                const int64_t q = checks.front();
                checks.pop_front();
                running.push_back({clock + check_service[q], q, true});
                progress = true;
            }
        }
        double next = 1e300;
        for (const Run &r : running) next = std::min(next, r.end);
        if (head < n && arrival[head] > clock) next = std::min(next, arrival[head]);
        if (next >= 1e300) break;
        clock = next;
        for (size_t k = 0; k < running.size();) {
            const Run r = running[k];
            if (r.end > clock) {
                ++k;
                continue;
            }
            running[k] = running.back();
            running.pop_back();
            if (r.check) {
                adm.release(bytes[r.job]);
                done[r.job] = r.end;
            } else if (check_service[r.job] >= 0.0) {
                ready[r.job] = r.end;
                adm.free_slot();  // the bytes stay admitted until the check
                checks.push_back(r.job);
            } else {
                ready[r.job] = done[r.job] = r.end;
                adm.release(bytes[r.job]);
            }
        }
    }
    return SDT_OK;
}
