// sdt_host.cpp -- host side of libsdt_gb300: error state, tiling checks, the
// (T) tuple list, algorithmic FLOP count and the seeded synthetic TCE files.
//
// Reference behaviour followed (NWChem source tree paths):
//   tuple filters and weight order  src/tce/ccsd_t/ccsd_t_neword.F:1-244
//   hash layout and lookup          src/tce/tce_hash.F:271-316
//   T1/T2 block keys                src/tce/tce_t1_offset.F, tce_t2_offset.F
//   V2 block keys                   src/tce/tce_mo2e_offset.F
//                                   (key forms used at ccsd_t_singles_l.F:355-364,
//                                    tce_hashnsort.F:47-80,129-165)
#include "sdt_internal.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>

namespace sdt {

std::atomic<int64_t> g_launches{0};

static std::mutex g_err_mu;
static int g_err_code = SDT_OK;
static std::string g_err_msg;
static std::atomic<int> g_err_mode{SDT_ERRMODE_EXIT};

int fail(int code, const std::string &msg) {
    std::lock_guard<std::mutex> lk(g_err_mu);
    if (g_err_code == SDT_OK) {
        g_err_code = code;
        g_err_msg = msg;
    }
    return code;
}

int error_mode() { return g_err_mode.load(); }

void fortran_abort_if_exit_mode() {
    if (g_err_mode.load() != SDT_ERRMODE_EXIT) return;
    std::string m;
    {
        std::lock_guard<std::mutex> lk(g_err_mu);
        m = g_err_msg;
    }
    std::fprintf(stderr, "libsdt_gb300: %s\n", m.c_str());
    std::fflush(stderr);
    std::exit(1);
}

bool make_tiling(const sdt_tiling *in, Tiling *out) {
    if (!in || in->noab < 1 || in->nvab < 1 || !in->range || !in->spin ||
        !in->sym || !in->offset || !in->evl_sorted)
        return false;
    if (in->restricted && !in->alpha) return false;
    Tiling t;
    t.noab = in->noab;
    t.nvab = in->nvab;
    t.range = in->range;
    t.spin = in->spin;
    t.sym = in->sym;
    t.offset = in->offset;
    t.alpha = in->alpha;
    t.evl = in->evl_sorted;
    t.restricted = in->restricted;
    int64_t acc = 0;
    for (int64_t b = 1; b <= t.noab + t.nvab; ++b) {
        if (t.r(b) < 1 || t.r(b) > 4096) return false;
        if (t.offset[b - 1] != acc) return false;  // tiles contiguous, in order
        if (t.y(b) < 0 || t.y(b) > 7) return false;
        acc += t.r(b);
        if (b == t.noab) t.nocc = acc;
    }
    t.nvir = acc - t.nocc;
    *out = t;
    return true;
}

int64_t hash_lookup(const int64_t *hash, int64_t key) {
    const int64_t n = hash[0];
    int64_t lo = 1, hi = n;
    while (lo <= hi) {
        int64_t mid = lo + (hi - lo) / 2;
        if (hash[mid] == key) return hash[n + mid];
        if (hash[mid] < key) lo = mid + 1;
        else hi = mid - 1;
    }
    return -1;
}

// ---------------------------------------------------------------------------
// Tuple list: ccsd_t_6tasks / ccsd_t_neword with w_thresh = 0.
// ---------------------------------------------------------------------------
static bool tuple_allowed(const Tiling &t, int64_t p4, int64_t p5, int64_t p6,
                          int64_t h1, int64_t h2, int64_t h3) {
    const int64_t sp = t.s(p4) + t.s(p5) + t.s(p6);
    const int64_t sh = t.s(h1) + t.s(h2) + t.s(h3);
    if (sp != sh) return false;
    if (t.restricted && sp + sh > 8) return false;
    return (t.y(p4) ^ t.y(p5) ^ t.y(p6) ^ t.y(h1) ^ t.y(h2) ^ t.y(h3)) == 0;
}

static std::vector<int64_t> enumerate(const Tiling &t) {
    std::vector<int64_t> rows;
    const int64_t o = t.noab, nt = t.noab + t.nvab;
    for (int64_t p4 = o + 1; p4 <= nt; ++p4)
        for (int64_t p5 = p4; p5 <= nt; ++p5)
            for (int64_t p6 = p5; p6 <= nt; ++p6)
                for (int64_t h1 = 1; h1 <= o; ++h1)
                    for (int64_t h2 = h1; h2 <= o; ++h2)
                        for (int64_t h3 = h2; h3 <= o; ++h3) {
                            if (!tuple_allowed(t, p4, p5, p6, h1, h2, h3)) continue;
                            const int64_t w = t.r(p4) * t.r(p5) * t.r(p6) *
                                              t.r(h1) * t.r(h2) * t.r(h3);
                            const int64_t row[7] = {p4, p5, p6, h1, h2, h3, w};
                            rows.insert(rows.end(), row, row + 7);
                        }
    return rows;
}

}  // namespace sdt

using namespace sdt;

extern "C" int64_t sdt_tasks_count(const sdt_tiling *ti) {
    Tiling t;
    if (!make_tiling(ti, &t)) return -fail(SDT_ERR_ARG, "sdt_tasks_count: bad tiling");
    return (int64_t)(enumerate(t).size() / 7);
}

extern "C" int sdt_tasks_list(const sdt_tiling *ti, int64_t n, int64_t *klist) {
    Tiling t;
    if (!make_tiling(ti, &t) || !klist) return fail(SDT_ERR_ARG, "sdt_tasks_list: bad argument");
    std::vector<int64_t> aux = enumerate(t);
    const int64_t tot = (int64_t)(aux.size() / 7);
    if (tot != n) return fail(SDT_ERR_ARG, "sdt_tasks_list: n differs from the task count");
    if (tot == 0) return SDT_OK;
    int64_t wmax = 0, wmin;
    for (int64_t m = 0; m < tot; ++m) wmax = std::max(wmax, aux[7 * m + 6]);
    wmin = wmax;
    for (int64_t m = 0; m < tot; ++m) wmin = std::min(wmin, aux[7 * m + 6]);
    // Weights within 1%: keep enumeration order (ccsd_t_neword.F:134-142).
    if ((double)(wmax - wmin) * 100.0 / (double)wmax < 1.0) {
        std::memcpy(klist, aux.data(), sizeof(int64_t) * aux.size());
        return SDT_OK;
    }
    // Descending buckets: 16 thresholds then 0; within a bucket the
    // enumeration order is kept (ccsd_sillysort, ccsd_t_neword.F:218-244).
    std::vector<char> taken(tot, 0);
    int64_t found = 0;
    auto pass = [&](int64_t value) {
        for (int64_t m = 0; m < tot; ++m) {
            if (taken[m] || aux[7 * m + 6] <= value) continue;
            std::memcpy(klist + 7 * found, &aux[7 * m], 7 * sizeof(int64_t));
            taken[m] = 1;
            ++found;
        }
    };
    for (int64_t ii = 16; ii >= 1; --ii) pass(wmin + ((wmax - wmin) * (ii - 1)) / 16);
    pass(0);
    return found == tot ? SDT_OK : fail(SDT_ERR_STATE, "sdt_tasks_list: ordering incomplete");
}

// Allowed h7b / p7b tiles for one permuted block row, as tce_hashnsort /
// tce_hashnsort_2 test them: the T2 quad's spin and irrep must balance.
extern "C" double sdt_tasks_flops(const sdt_tiling *ti, const int64_t *klist, int64_t n) {
    Tiling t;
    if (!make_tiling(ti, &t) || (!klist && n > 0)) return -1.0;
    double total = 0.0;
    for (int64_t q = 0; q < n; ++q) {
        const int64_t *k = klist + 7 * q;
        const int64_t P[3] = {k[0], k[1], k[2]}, H[3] = {k[3], k[4], k[5]};
        const double nt = (double)(t.r(P[0]) * t.r(P[1]) * t.r(P[2]) *
                                   t.r(H[0]) * t.r(H[1]) * t.r(H[2]));
        // Nine d1 terms read t(Pa,Pb;Hc,m); nine d2 terms read t(Pa,e;Hb,Hc).
        static const int d1p[9][2] = {{0, 1}, {0, 1}, {0, 1}, {1, 2}, {1, 2},
                                      {1, 2}, {0, 2}, {0, 2}, {0, 2}};
        static const int d1h[9] = {0, 1, 2, 0, 1, 2, 0, 1, 2};
        static const int d2p[9] = {0, 0, 0, 1, 1, 1, 2, 2, 2};
        static const int d2h[9][2] = {{0, 1}, {1, 2}, {0, 2}, {0, 1}, {1, 2},
                                      {0, 2}, {0, 1}, {1, 2}, {0, 2}};
        double kd = 0.0;
        for (int x = 0; x < 9; ++x) {
            const int64_t pa = P[d1p[x][0]], pb = P[d1p[x][1]], hc = H[d1h[x]];
            for (int64_t m = 1; m <= t.noab; ++m)
                if (t.s(pa) + t.s(pb) == t.s(hc) + t.s(m) &&
                    (t.y(pa) ^ t.y(pb) ^ t.y(hc) ^ t.y(m)) == 0)
                    kd += (double)t.r(m);
            const int64_t pe = P[d2p[x]], h1 = H[d2h[x][0]], h2 = H[d2h[x][1]];
            for (int64_t e = t.noab + 1; e <= t.noab + t.nvab; ++e)
                if (t.s(pe) + t.s(e) == t.s(h1) + t.s(h2) &&
                    (t.y(pe) ^ t.y(e) ^ t.y(h1) ^ t.y(h2)) == 0)
                    kd += (double)t.r(e);
        }
        total += nt * 2.0 * (kd + 9.0);
    }
    return total;
}

// ---------------------------------------------------------------------------
// Seeded synthetic inputs.
//
// Each tensor element is a pure function of (seed, tensor id, global
// orbital indices), so any block can be produced independently and the same
// bytes come out on every machine.  A raw draw is an Irwin-Hall(12) sum of
// 32-bit uniforms from a splitmix64 counter hash, kept as an exact integer
// S in [-6*2^32, 6*2^32) (mean 0, variance 2^64: S*2^-32 ~ N(0,1)).
// Antisymmetrisation combines integer draws exactly before one scaling:
//   T2(p,q,i,j)  = 0.02/2       * 2^-32 * (S(pqij) - S(qpij) - S(pqji) + S(qpji))
//   vvov(a,b,i,e)= 0.05/sqrt(2) * 2^-32 * (S(abie) - S(baie))
//   ovoo(m,a,i,j)= 0.05/sqrt(2) * 2^-32 * (S(maij) - S(maji))
//   vvoo(a,b,i,j)= 0.05/2       * 2^-32 * (four terms as T2)
//   T1(a,i)      = 0.01         * 2^-32 * S(ai)
// The 1/2 and 1/sqrt(2) factors keep the stated standard deviation for
// off-diagonal elements.  Orbital energies: occupied -1.5 + 1.1*u,
// virtual 0.2 + 2.3*u, u = uniform in [0,1).
// ---------------------------------------------------------------------------
namespace {

inline uint64_t splitmix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

enum : uint64_t { TID_T1 = 1, TID_T2 = 2, TID_VVOV = 3, TID_OVOO = 4, TID_VVOO = 5, TID_EVL = 6 };

inline int64_t draw(uint64_t seed, uint64_t tid, uint64_t idx) {
    const uint64_t key = splitmix64(seed ^ splitmix64((tid << 56) ^ splitmix64(idx)));
    int64_t s = 0;
    for (uint64_t r = 0; r < 6; ++r) {
        const uint64_t z = splitmix64(key + r * 0xD1B54A32D192ED03ull);
        s += (int64_t)(z & 0xffffffffull) + (int64_t)(z >> 32);
    }
    return s - (int64_t)6 * (int64_t)4294967296ll;
}

const double TWO_M32 = 1.0 / 4294967296.0;

struct Gen {
    uint64_t seed;
    int64_t o, v;
    double c_t1, c_t2, c_v2a, c_v4;
    explicit Gen(uint64_t s, int64_t o_, int64_t v_) : seed(s), o(o_), v(v_) {
        c_t1 = 0.01 * TWO_M32;
        c_t2 = 0.02 / 2.0 * TWO_M32;
        c_v2a = 0.05 / std::sqrt(2.0) * TWO_M32;
        c_v4 = 0.05 / 2.0 * TWO_M32;
    }
    double t1(int64_t a, int64_t i) const { return c_t1 * (double)draw(seed, TID_T1, (uint64_t)(a * o + i)); }
    int64_t s_vvoo(uint64_t tid, int64_t a, int64_t b, int64_t i, int64_t j) const {
        return draw(seed, tid, (uint64_t)(((a * v + b) * o + i) * o + j));
    }
    double t2(int64_t a, int64_t b, int64_t i, int64_t j) const {
        const int64_t s = s_vvoo(TID_T2, a, b, i, j) - s_vvoo(TID_T2, b, a, i, j) -
                          s_vvoo(TID_T2, a, b, j, i) + s_vvoo(TID_T2, b, a, j, i);
        return c_t2 * (double)s;
    }
    double vvoo(int64_t a, int64_t b, int64_t i, int64_t j) const {
        const int64_t s = s_vvoo(TID_VVOO, a, b, i, j) - s_vvoo(TID_VVOO, b, a, i, j) -
                          s_vvoo(TID_VVOO, a, b, j, i) + s_vvoo(TID_VVOO, b, a, j, i);
        return c_v4 * (double)s;
    }
    double vvov(int64_t a, int64_t b, int64_t i, int64_t e) const {
        auto S = [&](int64_t x, int64_t y) {
            return draw(seed, TID_VVOV, (uint64_t)(((x * v + y) * o + i) * v + e));
        };
        return c_v2a * (double)(S(a, b) - S(b, a));
    }
    double ovoo(int64_t m, int64_t a, int64_t i, int64_t j) const {
        auto S = [&](int64_t x, int64_t y) {
            return draw(seed, TID_OVOO, (uint64_t)(((m * v + a) * o + x) * o + y));
        };
        return c_v2a * (double)(S(i, j) - S(j, i));
    }
};

struct Block {
    int64_t key;
    int64_t t[4];   // tiles in key order (g3,g4,g1,g2) / (p1,p2,h3,h4) / (p,h)
    int64_t size;
    int kind;       // 0 T1, 1 T2, 2 vvov, 3 ovoo, 4 vvoo
};

std::vector<Block> file_blocks(const Tiling &t, int kind, bool full_v2 = false) {
    std::vector<Block> out;
    const int64_t o = t.noab, nt = t.noab + t.nvab, N = nt;
    auto skip_restricted = [&](int64_t ssum, int64_t all_beta) {
        return t.restricted && ssum == all_beta;
    };
    if (kind == SDT_FILE_T1) {
        for (int64_t p = o + 1; p <= nt; ++p)
            for (int64_t h = 1; h <= o; ++h) {
                if (t.s(p) != t.s(h) || (t.y(p) ^ t.y(h)) != 0) continue;
                if (skip_restricted(t.s(p) + t.s(h), 4)) continue;
                out.push_back({h - 1 + o * (p - o - 1), {p, h, 0, 0}, t.r(p) * t.r(h), 0});
            }
    } else if (kind == SDT_FILE_T2) {
        for (int64_t p1 = o + 1; p1 <= nt; ++p1)
            for (int64_t p2 = p1; p2 <= nt; ++p2)
                for (int64_t h3 = 1; h3 <= o; ++h3)
                    for (int64_t h4 = h3; h4 <= o; ++h4) {
                        if (t.s(p1) + t.s(p2) != t.s(h3) + t.s(h4)) continue;
                        if ((t.y(p1) ^ t.y(p2) ^ t.y(h3) ^ t.y(h4)) != 0) continue;
                        if (skip_restricted(t.s(p1) + t.s(p2) + t.s(h3) + t.s(h4), 8)) continue;
                        const int64_t key = h4 - 1 + o * (h3 - 1 + o * (p2 - o - 1 + t.nvab * (p1 - o - 1)));
                        out.push_back({key, {p1, p2, h3, h4}, t.r(p1) * t.r(p2) * t.r(h3) * t.r(h4), 1});
                    }
    } else {
        // V2 blocks (g3b<=g4b, g1b<=g2b), key g2-1+N*(g1-1+N*(g4-1+N*(g3-1))),
        // restricted to the three kinds the triples path reads.
        for (int64_t g3 = 1; g3 <= nt; ++g3)
            for (int64_t g4 = g3; g4 <= nt; ++g4)
                for (int64_t g1 = 1; g1 <= nt; ++g1)
                    for (int64_t g2 = g1; g2 <= nt; ++g2) {
                        const bool v3 = g3 > o, v4 = g4 > o, v1 = g1 > o, v2 = g2 > o;
                        int k;
                        if (v3 && v4 && !v1 && v2) k = 2;        // <p5 p6 || h3 p7>
                        else if (!v3 && v4 && !v1 && !v2) k = 3; // <h7 p6 || h2 h3>
                        else if (v3 && v4 && !v1 && !v2) k = 4;  // <p5 p6 || h2 h3>
                        else if (full_v2) k = 5;                 // a block the path never reads
                        else continue;
                        if (t.s(g3) + t.s(g4) != t.s(g1) + t.s(g2)) continue;
                        if ((t.y(g3) ^ t.y(g4) ^ t.y(g1) ^ t.y(g2)) != 0) continue;
                        if (skip_restricted(t.s(g3) + t.s(g4) + t.s(g1) + t.s(g2), 8)) continue;
                        const int64_t key = g2 - 1 + N * (g1 - 1 + N * (g4 - 1 + N * (g3 - 1)));
                        out.push_back({key, {g3, g4, g1, g2},
                                       t.r(g3) * t.r(g4) * t.r(g1) * t.r(g2), k});
                    }
    }
    return out;
}

void fill_block(const Tiling &t, const Gen &g, const Block &b, double *dst) {
    auto st = [&](int64_t tile) { return t.start(tile); };
    if (b.kind == 0) {
        const int64_t P = st(b.t[0]), H = st(b.t[1]), np = t.r(b.t[0]), nh = t.r(b.t[1]);
        for (int64_t a = 0; a < np; ++a)
            for (int64_t i = 0; i < nh; ++i) dst[a * nh + i] = g.t1(P + a, H + i);
        return;
    }
    const int64_t n0 = t.r(b.t[0]), n1 = t.r(b.t[1]), n2 = t.r(b.t[2]), n3 = t.r(b.t[3]);
    const int64_t s0 = st(b.t[0]), s1 = st(b.t[1]), s2 = st(b.t[2]), s3 = st(b.t[3]);
    for (int64_t x0 = 0; x0 < n0; ++x0)
        for (int64_t x1 = 0; x1 < n1; ++x1)
            for (int64_t x2 = 0; x2 < n2; ++x2)
                for (int64_t x3 = 0; x3 < n3; ++x3) {
                    double val;
                    switch (b.kind) {
                        case 1: val = g.t2(s0 + x0, s1 + x1, s2 + x2, s3 + x3); break;
                        case 2: val = g.vvov(s0 + x0, s1 + x1, s2 + x2, s3 + x3); break;
                        case 3: val = g.ovoo(s0 + x0, s1 + x1, s2 + x2, s3 + x3); break;
                        default: val = g.vvoo(s0 + x0, s1 + x1, s2 + x2, s3 + x3); break;
                    }
                    dst[((x0 * n1 + x1) * n2 + x2) * n3 + x3] = val;
                }
}

}  // namespace

extern "C" int sdt_synth_file(const sdt_tiling *ti, int kind, uint64_t seed,
                              int64_t *nblocks, int64_t *ndata, int64_t *hash,
                              double *data) {
    Tiling t;
    if (!make_tiling(ti, &t) || kind < 0 || kind > 2 || !nblocks || !ndata)
        return fail(SDT_ERR_ARG, "sdt_synth_file: bad argument");
    std::vector<Block> blocks = file_blocks(t, kind);
    std::vector<int64_t> offs(blocks.size());
    int64_t total = 0;
    for (size_t q = 0; q < blocks.size(); ++q) {
        offs[q] = total;
        total += blocks[q].size;
    }
    *nblocks = (int64_t)blocks.size();
    *ndata = total;
    if (!hash && !data) return SDT_OK;
    if (!hash || !data) return fail(SDT_ERR_ARG, "sdt_synth_file: hash and data must both be given");
    const int64_t n = (int64_t)blocks.size();
    hash[0] = n;
    for (int64_t q = 0; q < n; ++q) {
        hash[1 + q] = blocks[q].key;
        hash[1 + n + q] = offs[q];
        if (q > 0 && blocks[q].key <= blocks[q - 1].key)
            return fail(SDT_ERR_STATE, "sdt_synth_file: keys not ascending");
    }
    Gen g(seed, t.nocc, t.nvir);
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t q = 0; q < n; ++q) fill_block(t, g, blocks[q], data + offs[q]);
    return SDT_OK;
}

// Hash table of a file laid out exactly as NWChem's TCE lays it out
// (tce_t1_offset.F, tce_t2_offset.F, tce_mo2e_offset.F): blocks in loop
// order, keys ascending, offsets the running sum of block sizes.  For V2 it
// covers every (g3b<=g4b, g1b<=g2b) block the spin/irrep rules allow, so an
// integral file written by NWChem can be read as it is.
extern "C" int sdt_tce_layout(const sdt_tiling *ti, int kind, int64_t *nblocks, int64_t *ndata,
                              int64_t *hash) {
    Tiling t;
    if (!make_tiling(ti, &t) || kind < 0 || kind > 2 || !nblocks || !ndata)
        return fail(SDT_ERR_ARG, "sdt_tce_layout: bad argument");
    std::vector<Block> blocks = file_blocks(t, kind, true);
    const int64_t n = (int64_t)blocks.size();
    int64_t total = 0;
    if (hash) hash[0] = n;
    for (int64_t q = 0; q < n; ++q) {
        if (hash) {
            hash[1 + q] = blocks[q].key;
            hash[1 + n + q] = total;
        }
        total += blocks[q].size;
    }
    *nblocks = n;
    *ndata = total;
    return SDT_OK;
}

extern "C" int sdt_synth_evl(int64_t nocc, int64_t nvir, uint64_t seed, double *evl) {
    if (nocc < 1 || nvir < 1 || !evl) return fail(SDT_ERR_ARG, "sdt_synth_evl: bad argument");
    for (int64_t q = 0; q < nocc + nvir; ++q) {
        const uint64_t z = splitmix64(seed ^ splitmix64((TID_EVL << 56) ^ splitmix64((uint64_t)q)));
        const double u = (double)(z >> 11) * (1.0 / 9007199254740992.0);
        evl[q] = q < nocc ? -1.5 + 1.1 * u : 0.2 + 2.3 * u;
    }
    return SDT_OK;
}

extern "C" void sdt_set_error_mode(int mode) {
    sdt::g_err_mode.store(mode == SDT_ERRMODE_RECORD ? SDT_ERRMODE_RECORD : SDT_ERRMODE_EXIT);
}

extern "C" int sdt_last_error(char *msg, size_t len) {
    std::lock_guard<std::mutex> lk(sdt::g_err_mu);
    const int code = sdt::g_err_code;
    if (msg && len > 0) {
        std::snprintf(msg, len, "%s", sdt::g_err_msg.c_str());
    }
    sdt::g_err_code = SDT_OK;
    sdt::g_err_msg.clear();
    return code;
}

extern "C" int64_t sdt_launch_count(void) { return sdt::g_launches.load(); }
