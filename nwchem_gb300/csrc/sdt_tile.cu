// sdt_tile.cu -- the reference's tile-level CUDA surface on sm_103a.
//
// Replaces, symbol for symbol, the host wrappers and kernels of
// src/tce/ccsd_t/sd_t_total.cu: sd_t_s1_k_cuda_, sd_t_d1_k_cuda_,
// sd_t_d2_k_cuda_ (k = 1..9), compute_en_, dev_mem_d_, dev_mem_s_ and
// dev_release_.  The semantics are the reference's: dev_mem_* allocate and
// zero the tuple's doubles/singles tiles on the device, every s1/d1/d2 call
// copies its host sub-blocks to the device and accumulates its permuted
// term into the matching tile, and compute_en_ reduces both tiles with the
// orbital-energy denominator into (E[T], E(T)).
//
// Differences in how, not what:
//  * all 18 d1/d2 variants run one FP64 tensor-core kernel (mma.sync
//    m8n8k4.f64); a variant is only a set of scatter strides and a sign;
//  * copies and kernels are queued on one stream without a device-wide
//    synchronisation per call (the reference syncs after every kernel);
//    the host sub-blocks may be reused as soon as a call returns;
//  * compute_en_ reduces with a full thread block per partial and a
//    compensated final sum (the reference uses one thread per block).
#include "sdt_common.cuh"

#include <cstdio>
#include <cstring>

namespace sdt {
namespace {

// Index names used in the declared triplesx orders below.
enum { H1 = 0, H2 = 1, H3 = 2, P4 = 3, P5 = 4, P6 = 5, K7 = 6 };

// Declared triplesx dimension order (first = fastest) and sign of each
// kernel, from src/tce/ccsd_t/ccsd_t_kernels_omp.F (s1 :5-360, d1
// :362-856, d2 :857-1198).  The same signs appear in sd_t_total.cu.
const int kS1Order[9][6] = {
    {H3, H2, H1, P6, P5, P4}, {H3, H1, H2, P6, P5, P4}, {H1, H3, H2, P6, P5, P4},
    {H3, H2, H1, P6, P4, P5}, {H3, H1, H2, P6, P4, P5}, {H1, H3, H2, P6, P4, P5},
    {H3, H2, H1, P4, P6, P5}, {H3, H1, H2, P4, P6, P5}, {H1, H3, H2, P4, P6, P5}};
const double kS1Sign[9] = {+1, -1, +1, -1, +1, -1, +1, -1, +1};
const int kD1Order[9][6] = {
    {H3, H2, H1, P6, P5, P4}, {H3, H1, H2, P6, P5, P4}, {H1, H3, H2, P6, P5, P4},
    {H3, H2, H1, P5, P4, P6}, {H3, H1, H2, P5, P4, P6}, {H1, H3, H2, P5, P4, P6},
    {H3, H2, H1, P5, P6, P4}, {H3, H1, H2, P5, P6, P4}, {H1, H3, H2, P5, P6, P4}};
const double kD1Sign[9] = {-1, +1, -1, -1, +1, -1, +1, -1, +1};
const int kD2Order[9][6] = {
    {H3, H2, H1, P6, P5, P4}, {H2, H1, H3, P6, P5, P4}, {H2, H3, H1, P6, P5, P4},
    {H3, H2, H1, P6, P4, P5}, {H2, H1, H3, P6, P4, P5}, {H2, H3, H1, P6, P4, P5},
    {H3, H2, H1, P4, P6, P5}, {H2, H1, H3, P4, P6, P5}, {H2, H3, H1, P4, P6, P5}};
const double kD2Sign[9] = {-1, -1, +1, +1, +1, -1, -1, -1, +1};

// Strides of each named index in a triplesx declared with `order`.
void strides_for(const int order[6], const int64_t dims[7], int64_t st[7]) {
    int64_t acc = 1;
    for (int q = 0; q < 7; ++q) st[q] = 0;
    for (int q = 0; q < 6; ++q) {
        st[order[q]] = acc;
        acc *= dims[order[q]];
    }
}

// ---------------------------------------------------------------------------
// C[m,n] scattered into t3: t3[moff(m) + noff(n)] += sign * sum_k A[m,k] B[k,n]
// with m = (m0,m1,m2), n = (n0,n1,n2) mixed-radix and per-digit strides.
// ---------------------------------------------------------------------------
struct TileGemm {
    const double *A, *B;
    double *C;
    int64_t M, N, K;
    int64_t a_m, a_k;          // A[m*a_m + k*a_k]
    int64_t b_n, b_k;          // B[n*b_n + k*b_k]
    int64_t md0, md1, ms0, ms1, ms2;
    int64_t nd0, nd1, ns0, ns1, ns2;
    double sign;
};

constexpr int TG_WM = 32, TG_WN = 32;     // warp tile
constexpr int TG_BM = 64, TG_BN = 64;     // block tile (2x2 warps)

__global__ void __launch_bounds__(128) tile_gemm_kernel(const TileGemm g) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t m_base = (int64_t)blockIdx.y * TG_BM + (warp >> 1) * TG_WM;
    const int64_t n_base = (int64_t)blockIdx.x * TG_BN + (warp & 1) * TG_WN;
    const int r = lane >> 2, q = lane & 3;

    // Rows this lane loads for A (one per 8-row fragment) and columns for B.
    const double *arow[4];
    const double *bcol[4];
    bool aok[4], bok[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int64_t m = m_base + i * 8 + r;
        aok[i] = m < g.M;
        arow[i] = g.A + (aok[i] ? m : 0) * g.a_m;
        const int64_t n = n_base + i * 8 + r;
        bok[i] = n < g.N;
        bcol[i] = g.B + (bok[i] ? n : 0) * g.b_n;
    }
    double acc[4][4][2];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j][0] = acc[i][j][1] = 0.0;

    for (int64_t k0 = 0; k0 < g.K; k0 += 4) {
        const int64_t k = k0 + q;
        const bool kok = k < g.K;
        double a[4], b[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            a[i] = (aok[i] && kok) ? __ldg(arow[i] + k * g.a_k) : 0.0;
            b[i] = (bok[i] && kok) ? __ldg(bcol[i] + k * g.b_k) : 0.0;
        }
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) dmma_8x8x4(acc[i][j][0], acc[i][j][1], a[i], b[j]);
    }

#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int64_t m = m_base + i * 8 + r;
        if (m >= g.M) continue;
        const int64_t m0 = m % g.md0, mt = m / g.md0;
        const int64_t moff = m0 * g.ms0 + (mt % g.md1) * g.ms1 + (mt / g.md1) * g.ms2;
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int64_t n = n_base + j * 8 + 2 * q + h;
                if (n >= g.N) continue;
                const int64_t n0 = n % g.nd0, nt = n / g.nd0;
                const int64_t noff = n0 * g.ns0 + (nt % g.nd1) * g.ns1 + (nt / g.nd1) * g.ns2;
                g.C[moff + noff] += g.sign * acc[i][j][h];
            }
    }
}

// s1: t3s[perm] += sign * t1(p4,h1) * v2(h3,h2,p6,p5); one thread per
// (v2 element, t1 element) pair, each t3 element written once.
struct TileS1 {
    const double *t1, *v2;
    double *C;
    int64_t nv, nt;                  // v2 elements, t1 elements
    int64_t h3d, h2d, p6d, p4d;      // mixed-radix digits
    int64_t s_h3, s_h2, s_p6, s_p5, s_p4, s_h1;
    double sign;
};

__global__ void __launch_bounds__(256) tile_s1_kernel(const TileS1 g) {
    const int64_t total = g.nv * g.nt;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t vi = i % g.nv, ti = i / g.nv;
        int64_t x = vi;
        const int64_t h3 = x % g.h3d; x /= g.h3d;
        const int64_t h2 = x % g.h2d; x /= g.h2d;
        const int64_t p6 = x % g.p6d; const int64_t p5 = x / g.p6d;
        const int64_t p4 = ti % g.p4d, h1 = ti / g.p4d;
        const int64_t o = h3 * g.s_h3 + h2 * g.s_h2 + p6 * g.s_p6 + p5 * g.s_p5 +
                          p4 * g.s_p4 + h1 * g.s_h1;
        g.C[o] += g.sign * (g.t1[ti] * g.v2[vi]);
    }
}

// Energy of the tuple tiles (layout (h3,h2,h1,p6,p5,p4)), ccsd_t_dot.F:101-124.
__global__ void __launch_bounds__(256) tile_energy_kernel(
    const double *__restrict__ t3, const double *__restrict__ t3s,
    const double *__restrict__ ev, int64_t h1d, int64_t h2d, int64_t h3d,
    int64_t p4d, int64_t p5d, int64_t p6d, double factor, double *__restrict__ part) {
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
    __shared__ double w1[8], w2[8];
    s1 = warp_sum(s1);
    s2 = warp_sum(s2);
    if ((threadIdx.x & 31) == 0) {
        w1[threadIdx.x >> 5] = s1;
        w2[threadIdx.x >> 5] = s2;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, b = 0.0;
        for (int w = 0; w < 8; ++w) {
            a += w1[w];
            b += w2[w];
        }
        part[2 * blockIdx.x] = a;
        part[2 * blockIdx.x + 1] = b;
    }
}

// ---------------------------------------------------------------------------
// Per-process tile state (the reference keeps t3_d / t3_s_d as globals).
// ---------------------------------------------------------------------------
struct TileState {
    double *t3 = nullptr, *t3s = nullptr;
    int64_t n3 = 0, n3s = 0;
    double *scratch_a = nullptr, *scratch_b = nullptr;
    size_t cap_a = 0, cap_b = 0;
    double *ebuf = nullptr;   // evals (device)
    double *epart = nullptr;  // partial sums (device)
    double *eout = nullptr;   // 2 doubles (device)
    double *ehost = nullptr;  // pinned
} g_tile;

constexpr int kEnergyBlocks = 2 * 152;

// Entry points record the error and, in EXIT mode, terminate like CUDA_SAFE.
bool ok_or_abort(int rc) {
    if (rc == SDT_OK) return true;
    fortran_abort_if_exit_mode();
    return false;
}

bool ensure(double **buf, size_t *cap, size_t n) {
    if (*cap >= n && *buf) return true;
    cudaStream_t st = lib_stream();
    if (*buf) {
        cudaStreamSynchronize(st);
        gpu_put(*buf);
    }
    size_t want = n < 4096 ? 4096 : n + n / 4;
    *buf = (double *)gpu_get(want * sizeof(double), true);
    *cap = *buf ? want : 0;
    return *buf != nullptr;
}

int upload(double **buf, size_t *cap, const double *host, size_t n, const char *what) {
    if (!host && n) return fail(SDT_ERR_ARG, std::string(what) + ": null sub-block");
    if (!ensure(buf, cap, n)) return fail(SDT_ERR_NOMEM, std::string(what) + ": device allocation");
    return cuda_check(cudaMemcpyAsync(*buf, host, n * sizeof(double), cudaMemcpyHostToDevice,
                                      lib_stream()),
                      what);
}

int alloc_tile(double **t, int64_t *n, int64_t size, const char *what) {
    if (size <= 0) return fail(SDT_ERR_ARG, std::string(what) + ": empty tile");
    cudaStream_t st = lib_stream();
    if (*t) {
        cudaStreamSynchronize(st);
        gpu_put(*t);
        *t = nullptr;
    }
    *t = (double *)gpu_get((size_t)size * sizeof(double), true);
    if (!*t) return fail(SDT_ERR_NOMEM, std::string(what) + ": device allocation");
    *n = size;
    return cuda_check(cudaMemsetAsync(*t, 0, (size_t)size * sizeof(double), st), what);
}

void run_d(int kind, int k, const int64_t dims[7], const double *t2sub, const double *v2sub) {
    const char *what = kind == 1 ? "sd_t_d1_cuda" : "sd_t_d2_cuda";
    const int64_t size = dims[H1] * dims[H2] * dims[H3] * dims[P4] * dims[P5] * dims[P6];
    if (!g_tile.t3) {
        ok_or_abort(fail(SDT_ERR_STATE, std::string(what) + ": dev_mem_d_ was not called"));
        return;
    }
    if (size != g_tile.n3 || dims[K7] < 1) {
        ok_or_abort(fail(SDT_ERR_ARG, std::string(what) + ": block dims do not match the tuple tile"));
        return;
    }
    TileGemm g;
    int64_t st[7];
    strides_for(kind == 1 ? kD1Order[k - 1] : kD2Order[k - 1], dims, st);
    g.sign = kind == 1 ? kD1Sign[k - 1] : kD2Sign[k - 1];
    g.K = dims[K7];
    if (kind == 1) {
        // A = t2sub(h7,p4,p5,h1): m = (p4,p5,h1); B = v2sub(h3,h2,p6,h7): n = (h3,h2,p6)
        g.M = dims[P4] * dims[P5] * dims[H1];
        g.N = dims[H3] * dims[H2] * dims[P6];
        g.a_m = g.K; g.a_k = 1;
        g.b_n = 1; g.b_k = g.N;
        g.md0 = dims[P4]; g.md1 = dims[P5];
        g.ms0 = st[P4]; g.ms1 = st[P5]; g.ms2 = st[H1];
        g.nd0 = dims[H3]; g.nd1 = dims[H2];
        g.ns0 = st[H3]; g.ns1 = st[H2]; g.ns2 = st[P6];
    } else {
        // A = t2sub(p7,p4,h1,h2): m = (p4,h1,h2); B = v2sub(p7,h3,p6,p5): n = (h3,p6,p5)
        g.M = dims[P4] * dims[H1] * dims[H2];
        g.N = dims[H3] * dims[P6] * dims[P5];
        g.a_m = g.K; g.a_k = 1;
        g.b_n = g.K; g.b_k = 1;
        g.md0 = dims[P4]; g.md1 = dims[H1];
        g.ms0 = st[P4]; g.ms1 = st[H1]; g.ms2 = st[H2];
        g.nd0 = dims[H3]; g.nd1 = dims[P6];
        g.ns0 = st[H3]; g.ns1 = st[P6]; g.ns2 = st[P5];
    }
    if (!ok_or_abort(upload(&g_tile.scratch_a, &g_tile.cap_a, t2sub, (size_t)(g.M * g.K), what))) return;
    if (!ok_or_abort(upload(&g_tile.scratch_b, &g_tile.cap_b, v2sub, (size_t)(g.N * g.K), what))) return;
    g.A = g_tile.scratch_a;
    g.B = g_tile.scratch_b;
    g.C = g_tile.t3;
    dim3 grid((unsigned)((g.N + TG_BN - 1) / TG_BN), (unsigned)((g.M + TG_BM - 1) / TG_BM));
    if (grid.y > 65535u) {
        ok_or_abort(fail(SDT_ERR_ARG, std::string(what) + ": block too large"));
        return;
    }
    tile_gemm_kernel<<<grid, 128, 0, lib_stream()>>>(g);
    count_launch();
    ok_or_abort(cuda_check(cudaGetLastError(), what));
}

void run_s1(int k, const int64_t dims[7], const double *t1sub, const double *v2sub) {
    const char *what = "sd_t_s1_cuda";
    const int64_t size = dims[H1] * dims[H2] * dims[H3] * dims[P4] * dims[P5] * dims[P6];
    if (!g_tile.t3s) {
        ok_or_abort(fail(SDT_ERR_STATE, "sd_t_s1_cuda: dev_mem_s_ was not called"));
        return;
    }
    if (size != g_tile.n3s) {
        ok_or_abort(fail(SDT_ERR_ARG, "sd_t_s1_cuda: block dims do not match the tuple tile"));
        return;
    }
    TileS1 g;
    int64_t st[7];
    strides_for(kS1Order[k - 1], dims, st);
    g.sign = kS1Sign[k - 1];
    g.nt = dims[P4] * dims[H1];
    g.nv = dims[H3] * dims[H2] * dims[P6] * dims[P5];
    g.h3d = dims[H3]; g.h2d = dims[H2]; g.p6d = dims[P6]; g.p4d = dims[P4];
    g.s_h3 = st[H3]; g.s_h2 = st[H2]; g.s_p6 = st[P6]; g.s_p5 = st[P5];
    g.s_p4 = st[P4]; g.s_h1 = st[H1];
    if (!ok_or_abort(upload(&g_tile.scratch_a, &g_tile.cap_a, t1sub, (size_t)g.nt, what))) return;
    if (!ok_or_abort(upload(&g_tile.scratch_b, &g_tile.cap_b, v2sub, (size_t)g.nv, what))) return;
    g.t1 = g_tile.scratch_a;
    g.v2 = g_tile.scratch_b;
    g.C = g_tile.t3s;
    const int64_t total = g.nt * g.nv;
    int64_t blocks = (total + 255) / 256;
    if (blocks > 8 * 152) blocks = 8 * 152;
    tile_s1_kernel<<<(unsigned)blocks, 256, 0, lib_stream()>>>(g);
    count_launch();
    ok_or_abort(cuda_check(cudaGetLastError(), what));
}

}  // namespace
}  // namespace sdt

using namespace sdt;

#define SDT_S1_DEF(k)                                                                   \
    extern "C" void sd_t_s1_##k##_cuda_(sdt_int *h1d, sdt_int *h2d, sdt_int *h3d,       \
                                        sdt_int *p4d, sdt_int *p5d, sdt_int *p6d,       \
                                        double *t3, double *t1sub, double *v2sub) {     \
        (void)t3;                                                                       \
        const int64_t dims[7] = {*h1d, *h2d, *h3d, *p4d, *p5d, *p6d, 1};                \
        run_s1(k, dims, t1sub, v2sub);                                                  \
    }
SDT_S1_DEF(1) SDT_S1_DEF(2) SDT_S1_DEF(3) SDT_S1_DEF(4) SDT_S1_DEF(5)
SDT_S1_DEF(6) SDT_S1_DEF(7) SDT_S1_DEF(8) SDT_S1_DEF(9)

#define SDT_D1_DEF(k)                                                                   \
    extern "C" void sd_t_d1_##k##_cuda_(sdt_int *h1d, sdt_int *h2d, sdt_int *h3d,       \
                                        sdt_int *h7d, sdt_int *p4d, sdt_int *p5d,       \
                                        sdt_int *p6d, double *t3, double *t2sub,        \
                                        double *v2sub) {                                \
        (void)t3;                                                                       \
        const int64_t dims[7] = {*h1d, *h2d, *h3d, *p4d, *p5d, *p6d, *h7d};             \
        run_d(1, k, dims, t2sub, v2sub);                                                \
    }
SDT_D1_DEF(1) SDT_D1_DEF(2) SDT_D1_DEF(3) SDT_D1_DEF(4) SDT_D1_DEF(5)
SDT_D1_DEF(6) SDT_D1_DEF(7) SDT_D1_DEF(8) SDT_D1_DEF(9)

#define SDT_D2_DEF(k)                                                                   \
    extern "C" void sd_t_d2_##k##_cuda_(sdt_int *h1d, sdt_int *h2d, sdt_int *h3d,       \
                                        sdt_int *p4d, sdt_int *p5d, sdt_int *p6d,       \
                                        sdt_int *p7d, double *t3, double *t2sub,        \
                                        double *v2sub) {                                \
        (void)t3;                                                                       \
        const int64_t dims[7] = {*h1d, *h2d, *h3d, *p4d, *p5d, *p6d, *p7d};             \
        run_d(2, k, dims, t2sub, v2sub);                                                \
    }
SDT_D2_DEF(1) SDT_D2_DEF(2) SDT_D2_DEF(3) SDT_D2_DEF(4) SDT_D2_DEF(5)
SDT_D2_DEF(6) SDT_D2_DEF(7) SDT_D2_DEF(8) SDT_D2_DEF(9)

extern "C" void dev_mem_d_(sdt_int *h1d, sdt_int *h2d, sdt_int *h3d, sdt_int *p4d,
                           sdt_int *p5d, sdt_int *p6d) {
    ok_or_abort(alloc_tile(&g_tile.t3, &g_tile.n3, *h1d * *h2d * *h3d * *p4d * *p5d * *p6d,
                           "dev_mem_d_"));
}

extern "C" void dev_mem_s_(sdt_int *h1d, sdt_int *h2d, sdt_int *h3d, sdt_int *p4d,
                           sdt_int *p5d, sdt_int *p6d) {
    ok_or_abort(alloc_tile(&g_tile.t3s, &g_tile.n3s, *h1d * *h2d * *h3d * *p4d * *p5d * *p6d,
                           "dev_mem_s_"));
}

extern "C" void dev_release_(void) {
    cudaStream_t st = lib_stream();
    cudaStreamSynchronize(st);
    gpu_put(g_tile.t3);
    gpu_put(g_tile.t3s);
    gpu_put(g_tile.scratch_a);
    gpu_put(g_tile.scratch_b);
    g_tile.t3 = g_tile.t3s = g_tile.scratch_a = g_tile.scratch_b = nullptr;
    g_tile.n3 = g_tile.n3s = 0;
    g_tile.cap_a = g_tile.cap_b = 0;
}

extern "C" void compute_en_(double *factor, double *energy, double *eval1, double *eval2,
                            double *eval3, double *eval4, double *eval5, double *eval6,
                            sdt_int *h1d, sdt_int *h2d, sdt_int *h3d, sdt_int *p4d,
                            sdt_int *p5d, sdt_int *p6d, double *host1, double *host2) {
    (void)host1;
    (void)host2;
    const int64_t d[6] = {*h1d, *h2d, *h3d, *p4d, *p5d, *p6d};
    const int64_t size = d[0] * d[1] * d[2] * d[3] * d[4] * d[5];
    if (!g_tile.t3 || size != g_tile.n3 || (g_tile.t3s && size != g_tile.n3s)) {
        ok_or_abort(fail(SDT_ERR_STATE, "compute_en_: tuple tiles missing or of another size"));
        return;
    }
    cudaStream_t st = lib_stream();
    // Per-call buffers (memory.cu-style: taken and given back every call;
    // the cache makes the second call allocation-free).
    g_tile.ebuf = (double *)gpu_get(6 * 4096 * sizeof(double), true);
    g_tile.epart = (double *)gpu_get(2 * kEnergyBlocks * sizeof(double), true);
    g_tile.eout = (double *)gpu_get(2 * sizeof(double), true);
    g_tile.ehost = (double *)host_get(8 * 4096 * sizeof(double), true);
    struct Release {
        ~Release() {
            gpu_put(g_tile.ebuf);
            gpu_put(g_tile.epart);
            gpu_put(g_tile.eout);
            host_put(g_tile.ehost);
            g_tile.ebuf = g_tile.epart = g_tile.eout = g_tile.ehost = nullptr;
        }
    } release;
    if (!g_tile.ebuf || !g_tile.epart || !g_tile.eout || !g_tile.ehost) {
        ok_or_abort(fail(SDT_ERR_NOMEM, "compute_en_: allocation"));
        return;
    }
    double *ev[6] = {eval1, eval2, eval3, eval4, eval5, eval6};
    int64_t at = 0;
    for (int q = 0; q < 6; ++q) {
        if (d[q] > 4096) {
            ok_or_abort(fail(SDT_ERR_ARG, "compute_en_: tile longer than 4096"));
            return;
        }
        std::memcpy(g_tile.ehost + at, ev[q], d[q] * sizeof(double));
        at += d[q];
    }
    if (!ok_or_abort(cuda_check(cudaMemcpyAsync(g_tile.ebuf, g_tile.ehost, at * sizeof(double),
                                                cudaMemcpyHostToDevice, st),
                                "compute_en_")))
        return;
    tile_energy_kernel<<<kEnergyBlocks, 256, 0, st>>>(g_tile.t3, g_tile.t3s, g_tile.ebuf, d[0],
                                                      d[1], d[2], d[3], d[4], d[5], *factor,
                                                      g_tile.epart);
    count_launch();
    if (!ok_or_abort(cuda_check(cudaGetLastError(), "compute_en_"))) return;
    if (!ok_or_abort(reduce_pairs(g_tile.epart, kEnergyBlocks, g_tile.eout, st))) return;
    double *out = g_tile.ehost + 6 * 4096;
    if (!ok_or_abort(cuda_check(cudaMemcpyAsync(out, g_tile.eout, 2 * sizeof(double),
                                                cudaMemcpyDeviceToHost, st),
                                "compute_en_")))
        return;
    if (!ok_or_abort(cuda_check(cudaStreamSynchronize(st), "compute_en_"))) return;
    energy[0] = out[0];
    energy[1] = out[1];
}

extern "C" int sdt_tile_download(double *doubles, double *singles) {
    cudaStream_t st = lib_stream();
    int rc = SDT_OK;
    if (doubles) {
        if (!g_tile.t3) return fail(SDT_ERR_STATE, "sdt_tile_download: no doubles tile");
        rc = cuda_check(cudaMemcpyAsync(doubles, g_tile.t3, (size_t)g_tile.n3 * sizeof(double),
                                        cudaMemcpyDeviceToHost, st), "sdt_tile_download");
    }
    if (!rc && singles) {
        if (!g_tile.t3s) return fail(SDT_ERR_STATE, "sdt_tile_download: no singles tile");
        rc = cuda_check(cudaMemcpyAsync(singles, g_tile.t3s, (size_t)g_tile.n3s * sizeof(double),
                                        cudaMemcpyDeviceToHost, st), "sdt_tile_download");
    }
    if (rc) return rc;
    return cuda_check(cudaStreamSynchronize(st), "sdt_tile_download");
}
