// sdt_noalloc.cu -- energy reduction of caller-owned triples tiles that
// allocates nothing.
//
// Who needs it: a caller that keeps the doubles/singles triples tiles in
// device memory it manages itself (its own memory pool, or device data
// owned by a Fortran offload runtime) and that cannot, or must not, call
// cudaMalloc/cudaFree -- because its pool already holds the memory budget,
// or because cudaMalloc/cudaFree would synchronise the device under its
// running work.  compute_en_ cannot serve it: compute_en_ works on the
// library's own tiles (dev_mem_d_/dev_mem_s_) and takes per-call buffers
// from the library's allocator.
//
// The scratch this reduction needs -- the six orbital-energy vectors copied
// from the host, one (E[T], E(T)) partial per thread block and the two
// results -- lives in one file-scope __device__ array of fixed size.  Every
// GPU that loads the library holds it (about 82 KB) until the process exits.
#include "sdt_common.cuh"

#include <mutex>

namespace sdt {
namespace {

constexpr int kNaMaxEvals = 8192;    // h1d+h2d+h3d+p4d+p5d+p6d at most
constexpr int kNaMaxBlocks = 1024;   // partial sums, one pair per block
constexpr int kNaThreads = 256;
constexpr int kNaEvalOff = 0;
constexpr int kNaPartOff = kNaMaxEvals;
constexpr int kNaOutOff = kNaMaxEvals + 2 * kNaMaxBlocks;
constexpr int kNaTotal = kNaOutOff + 2;

// The scratch.  In host code this name is only a host-side stand-in: kernels
// receive the device address obtained with cudaGetSymbolAddress below.
static __device__ __align__(256) double g_noalloc_scratch[kNaTotal];

constexpr int kNaMaxDevices = 64;
std::mutex g_na_mu;
double *g_na_ptr[kNaMaxDevices] = {nullptr};

// (E[T], E(T)) partial of each block over the tuple layout (h3,h2,h1,p6,p5,p4),
// the arithmetic of ccsd_t_dot.F:101-124.
__global__ void __launch_bounds__(kNaThreads) noalloc_energy_partials(
    const double *__restrict__ t3, const double *__restrict__ t3s, double *__restrict__ scratch,
    int64_t h1d, int64_t h2d, int64_t h3d, int64_t p4d, int64_t p5d, int64_t p6d, double factor) {
    const double *ev = scratch + kNaEvalOff;
    const double *e1 = ev, *e2 = e1 + h1d, *e3 = e2 + h2d;
    const double *e4 = e3 + h3d, *e5 = e4 + p4d, *e6 = e5 + p5d;
    const int64_t total = h1d * h2d * h3d * p4d * p5d * p6d;
    double s1 = 0.0, s2 = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (int64_t)gridDim.x * blockDim.x) {
        int64_t x = i;
        const int64_t h3 = x % h3d; x /= h3d;
        const int64_t h2 = x % h2d; x /= h2d;
        const int64_t h1 = x % h1d; x /= h1d;
        const int64_t p6 = x % p6d; x /= p6d;
        const int64_t p5 = x % p5d; const int64_t p4 = x / p5d;
        const double denom_0 = -(e4[p4] + e5[p5] + e6[p6]);
        const double doub = t3[i], sing = t3s ? t3s[i] : 0.0;
        const double denom = doub * factor / (e1[h1] + e2[h2] + e3[h3] + denom_0);
        s1 += denom * doub;
        s2 += denom * (doub + sing);
    }
    __shared__ double w1[kNaThreads / 32], w2[kNaThreads / 32];
    s1 = warp_sum(s1);
    s2 = warp_sum(s2);
    if ((threadIdx.x & 31) == 0) {
        w1[threadIdx.x >> 5] = s1;
        w2[threadIdx.x >> 5] = s2;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, b = 0.0;
        for (int w = 0; w < kNaThreads / 32; ++w) {
            a += w1[w];
            b += w2[w];
        }
        scratch[kNaPartOff + 2 * blockIdx.x] = a;
        scratch[kNaPartOff + 2 * blockIdx.x + 1] = b;
    }
}

// Compensated sum of the nblk partials into scratch[kNaOutOff..+1].
__global__ void __launch_bounds__(kNaThreads) noalloc_energy_total(double *__restrict__ scratch,
                                                                   int nblk) {
    __shared__ double sa[kNaThreads], ca[kNaThreads], sb[kNaThreads], cb[kNaThreads];
    Comp x, y;
    for (int i = threadIdx.x; i < nblk; i += kNaThreads) {
        x.add(scratch[kNaPartOff + 2 * i]);
        y.add(scratch[kNaPartOff + 2 * i + 1]);
    }
    sa[threadIdx.x] = x.s;
    ca[threadIdx.x] = x.c;
    sb[threadIdx.x] = y.s;
    cb[threadIdx.x] = y.c;
    __syncthreads();
    if (threadIdx.x == 0) {
        Comp u, w;
        for (int k = 0; k < kNaThreads; ++k) {
            u.add(sa[k]);
            u.add(ca[k]);
            w.add(sb[k]);
            w.add(cb[k]);
        }
        scratch[kNaOutOff] = u.value();
        scratch[kNaOutOff + 1] = w.value();
    }
}

// Device address of the scratch on the current device, looked up once per
// device (with that device current) and cached.
int scratch_address(double **out) {
    int dev = 0;
    int rc = cuda_check(cudaGetDevice(&dev), "sdt_compute_en_noalloc");
    if (rc) return rc;
    if (dev < 0 || dev >= kNaMaxDevices)
        return fail(SDT_ERR_ARG, "sdt_compute_en_noalloc: device index above 63");
    std::lock_guard<std::mutex> lk(g_na_mu);
    if (!g_na_ptr[dev]) {
        void *p = nullptr;
        rc = cuda_check(cudaGetSymbolAddress(&p, g_noalloc_scratch),
                        "sdt_compute_en_noalloc: cudaGetSymbolAddress");
        if (rc) return rc;
        g_na_ptr[dev] = (double *)p;
    }
    *out = g_na_ptr[dev];
    return SDT_OK;
}

}  // namespace
}  // namespace sdt

using namespace sdt;

extern "C" int sdt_compute_en_noalloc(double factor, double *energy, const double *eval1,
                                      const double *eval2, const double *eval3,
                                      const double *eval4, const double *eval5,
                                      const double *eval6, int64_t h1d, int64_t h2d,
                                      int64_t h3d, int64_t p4d, int64_t p5d, int64_t p6d,
                                      const double *t3_d, const double *t3s_d, void *stream) {
    const int64_t d[6] = {h1d, h2d, h3d, p4d, p5d, p6d};
    const double *ev[6] = {eval1, eval2, eval3, eval4, eval5, eval6};
    int64_t nev = 0;
    for (int q = 0; q < 6; ++q) {
        if (d[q] < 1 || !ev[q])
            return fail(SDT_ERR_ARG, "sdt_compute_en_noalloc: every tile length must be >= 1 "
                                     "and every orbital-energy pointer non-null");
        nev += d[q];
    }
    if (nev > kNaMaxEvals)
        return fail(SDT_ERR_ARG, "sdt_compute_en_noalloc: h1d+h2d+h3d+p4d+p5d+p6d exceeds the "
                                 "8192 orbital energies its fixed scratch holds");
    if (!energy || !t3_d) return fail(SDT_ERR_ARG, "sdt_compute_en_noalloc: null energy or t3_d");
    double *scratch = nullptr;
    int rc = scratch_address(&scratch);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    int64_t at = 0;
    for (int q = 0; q < 6; ++q) {
        rc = cuda_check(cudaMemcpyAsync(scratch + kNaEvalOff + at, ev[q], d[q] * sizeof(double),
                                        cudaMemcpyHostToDevice, st),
                        "sdt_compute_en_noalloc");
        if (rc) return rc;
        at += d[q];
    }
    const int64_t total = h1d * h2d * h3d * p4d * p5d * p6d;
    int64_t nblk = (total + kNaThreads - 1) / kNaThreads;
    if (nblk > kNaMaxBlocks) nblk = kNaMaxBlocks;
    noalloc_energy_partials<<<(unsigned)nblk, kNaThreads, 0, st>>>(t3_d, t3s_d, scratch, h1d, h2d,
                                                                   h3d, p4d, p5d, p6d, factor);
    noalloc_energy_total<<<1, kNaThreads, 0, st>>>(scratch, (int)nblk);
    count_launch(2);
    rc = cuda_check(cudaGetLastError(), "sdt_compute_en_noalloc");
    if (rc) return rc;
    rc = cuda_check(cudaMemcpyAsync(energy, scratch + kNaOutOff, 2 * sizeof(double),
                                    cudaMemcpyDeviceToHost, st),
                    "sdt_compute_en_noalloc");
    if (rc) return rc;
    return cuda_check(cudaStreamSynchronize(st), "sdt_compute_en_noalloc");
}
