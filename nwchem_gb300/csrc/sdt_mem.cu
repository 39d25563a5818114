// sdt_mem.cu -- caching allocator, library stream, device binding and the
// deterministic pair reduction shared by both surfaces.
//
// Replaces src/tce/ccsd_t/memory.cu (initmemmodule_, getGpuMem, getHostMem,
// freeGpuMem, freeHostMem, finalizememmodule_) and src/tce/ccsd_t/hybrid.c
// (check_device_, device_init_).
#include "sdt_common.cuh"

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>

namespace sdt {

namespace {
struct Pool {
    std::multimap<size_t, void *> free_dev, free_host;
    std::map<void *, size_t> live_dev, live_host;
    std::map<void *, bool> tile_owned;  // live blocks of the tile ABI
    bool init = false;
};
Pool &pool() {
    static Pool p;
    return p;
}
std::mutex &pool_mu() {
    static std::mutex m;
    return m;
}
cudaStream_t g_stream = nullptr;
int g_stream_dev = -1;
cudaStream_t g_alloc_stream = nullptr;
int g_alloc_dev = -1;

// Device blocks come from the stream-ordered allocator on a stream of their
// own (then that stream is synchronised, which waits for nothing else).  A
// plain cudaMalloc is an implicit synchronisation point: work issued after
// it waits for all work issued before it, so a job loaded while a long
// kernel runs (a resident serving kernel, an FP64 check) would wait for it.
cudaError_t dev_alloc(void **p, size_t bytes) {
    int dev = 0;
    cudaGetDevice(&dev);
    if (!g_alloc_stream || g_alloc_dev != dev) {
        cudaStream_t s = nullptr;
        if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) {
            cudaGetLastError();
            return cudaMalloc(p, bytes);
        }
        g_alloc_stream = s;
        g_alloc_dev = dev;
    }
    cudaError_t e = cudaMallocAsync(p, bytes, g_alloc_stream);
    if (e == cudaErrorNotSupported) {
        cudaGetLastError();
        return cudaMalloc(p, bytes);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(g_alloc_stream);
    return e;
}
void dev_free(void *p) {
    if (g_alloc_stream && cudaFreeAsync(p, g_alloc_stream) == cudaSuccess) {
        cudaStreamSynchronize(g_alloc_stream);
        return;
    }
    cudaGetLastError();
    cudaFree(p);
}
}  // namespace

int cuda_check(cudaError_t e, const char *what) {
    if (e == cudaSuccess) return SDT_OK;
    return fail(SDT_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

cudaStream_t lib_stream() {
    int dev = 0;
    cudaGetDevice(&dev);
    if (!g_stream || g_stream_dev != dev) {
        cudaStream_t s = nullptr;
        if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) return nullptr;
        g_stream = s;
        g_stream_dev = dev;
    }
    return g_stream;
}

// Reuse the smallest cached block of at least `bytes`; otherwise allocate.
static void *take(std::multimap<size_t, void *> &fl, std::map<void *, size_t> &live,
                  size_t bytes, bool dev) {
    auto it = fl.lower_bound(bytes);
    if (it != fl.end() && it->first <= bytes * 2 + (1u << 20)) {
        void *p = it->second;
        live[p] = it->first;
        fl.erase(it);
        return p;
    }
    void *p = nullptr;
    PhaseTrace tr(dev ? "pool: cudaMalloc" : "pool: cudaMallocHost");
    cudaError_t e = dev ? dev_alloc(&p, bytes) : cudaMallocHost(&p, bytes);
    tr.mark(std::to_string(bytes).c_str(), nullptr);
    if (e != cudaSuccess) {
        cudaGetLastError();
        // Drop the cache and retry once.
        for (auto &kv : fl) dev ? dev_free(kv.second) : (void)cudaFreeHost(kv.second);
        fl.clear();
        tr.mark("cache dropped", nullptr);
        e = dev ? dev_alloc(&p, bytes) : cudaMallocHost(&p, bytes);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
    }
    live[p] = bytes;
    return p;
}

void *gpu_get(size_t bytes, bool tile) {
    std::lock_guard<std::mutex> lk(pool_mu());
    if (bytes == 0) bytes = 8;
    void *p = take(pool().free_dev, pool().live_dev, bytes, true);
    if (p && tile) pool().tile_owned[p] = true;
    return p;
}
void gpu_put(void *p) {
    if (!p) return;
    std::lock_guard<std::mutex> lk(pool_mu());
    pool().tile_owned.erase(p);
    auto it = pool().live_dev.find(p);
    if (it == pool().live_dev.end()) return;
    pool().free_dev.emplace(it->second, p);
    pool().live_dev.erase(it);
}
void *host_get(size_t bytes, bool tile) {
    std::lock_guard<std::mutex> lk(pool_mu());
    if (bytes == 0) bytes = 8;
    void *p = take(pool().free_host, pool().live_host, bytes, false);
    if (p && tile) pool().tile_owned[p] = true;
    return p;
}
void host_put(void *p) {
    if (!p) return;
    std::lock_guard<std::mutex> lk(pool_mu());
    pool().tile_owned.erase(p);
    auto it = pool().live_host.find(p);
    if (it == pool().live_host.end()) return;
    pool().free_host.emplace(it->second, p);
    pool().live_host.erase(it);
}

// ---------------------------------------------------------------------------
// Deterministic sum of n (E[T], E(T)) pairs: one block, fixed thread count,
// each thread a Neumaier sum over a fixed stride, then a fixed-order tree.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) reduce_pairs_kernel(const double *__restrict__ part,
                                                           int64_t n, double *__restrict__ out) {
    __shared__ double s1[256], c1[256], s2[256], c2[256];
    Comp a, b;
    for (int64_t i = threadIdx.x; i < n; i += 256) {
        a.add(part[2 * i]);
        b.add(part[2 * i + 1]);
    }
    s1[threadIdx.x] = a.s;
    c1[threadIdx.x] = a.c;
    s2[threadIdx.x] = b.s;
    c2[threadIdx.x] = b.c;
    __syncthreads();
    if (threadIdx.x == 0) {
        Comp x, y;
        for (int q = 0; q < 256; ++q) {
            x.add(s1[q]);
            x.add(c1[q]);
            y.add(s2[q]);
            y.add(c2[q]);
        }
        out[0] = x.value();
        out[1] = y.value();
    }
}

int reduce_pairs(const double *partials, int64_t n, double *out_dev, cudaStream_t st) {
    reduce_pairs_kernel<<<1, 256, 0, st>>>(partials, n, out_dev);
    count_launch();
    return cuda_check(cudaGetLastError(), "reduce_pairs");
}

bool trace_on() {
    static const bool on = [] {
        const char *v = std::getenv("SDT_TRACE");
        return v && *v && std::strcmp(v, "0") != 0;
    }();
    return on;
}

static double wall_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

PhaseTrace::PhaseTrace(const char *w) : who(w) {
    if (trace_on()) t0 = last = wall_s();
}

void PhaseTrace::mark(const char *phase, void *stream) {
    if (!trace_on()) return;
    if (stream) cudaStreamSynchronize((cudaStream_t)stream);
    const double t = wall_s();
    char buf[96];
    std::snprintf(buf, sizeof(buf), " %s %.3f ms", phase, 1e3 * (t - last));
    line += buf;
    last = t;
}

PhaseTrace::~PhaseTrace() {
    if (trace_on()) std::fprintf(stderr, "[sdt trace] %s:%s; total %.3f ms\n", who, line.c_str(), 1e3 * (wall_s() - t0));
}

static int local_index() {
    const char *names[] = {"SDT_LOCAL_RANK", "LOCAL_RANK", "OMPI_COMM_WORLD_LOCAL_RANK",
                           "MPI_LOCALRANKID", "SLURM_LOCALID"};
    for (const char *n : names) {
        const char *v = std::getenv(n);
        if (v && *v) return std::atoi(v);
    }
    return 0;
}

}  // namespace sdt

using namespace sdt;

extern "C" void initmemmodule_(void) {
    std::lock_guard<std::mutex> lk(pool_mu());
    pool().init = true;
}

extern "C" void finalizememmodule_(void) {
    bool leaked;
    {
        std::lock_guard<std::mutex> lk(pool_mu());
        leaked = !pool().tile_owned.empty();
        pool().init = false;
        // Freed blocks stay cached for the next tuple; memory.cu returns them
        // to the driver here, which costs a cudaFree/cudaMalloc per tuple.
    }
    if (leaked) {
        fail(SDT_ERR_STATE, "finalizememmodule_: live device or host blocks remain");
        fortran_abort_if_exit_mode();
    }
}

extern "C" int check_device_(long *icuda) {
    if (!icuda) return 0;
    return local_index() < *icuda ? 1 : 0;
}

extern "C" int device_init_(long *icuda, long *cuda_device_number) {
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess) {
        cudaGetLastError();
        count = 0;
    }
    if (!icuda || count < *icuda) {
        std::printf("Warning: Please check whether you have %ld cuda devices per node\n",
                    icuda ? *icuda : 0L);
        std::fflush(stdout);
        if (cuda_device_number) *cuda_device_number = 30;
    } else {
        cudaSetDevice(local_index());
    }
    return 1;
}
