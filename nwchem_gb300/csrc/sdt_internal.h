// sdt_internal.h -- shared declarations of libsdt_gb300 (not installed).
#pragma once
#include "../../include/sdt_gb300.h"
#include <atomic>
#include <cstdint>
#include <string>

namespace sdt {

// Records an error (code + message).  In SDT_ERRMODE_EXIT the Fortran-facing
// entry points print and exit(1) like the reference's CUDA_SAFE macro
// (src/tce/ccsd_t/header.h:28-36); fail() returns the code for sdt_* calls.
int fail(int code, const std::string &msg);
// Fortran-facing entry points call this after fail(): exits in EXIT mode.
void fortran_abort_if_exit_mode();
int error_mode();

extern std::atomic<int64_t> g_launches;
inline void count_launch(int64_t n = 1) { g_launches.fetch_add(n, std::memory_order_relaxed); }

// Phase tracing: with SDT_TRACE set (not "0") the job surface prints the
// wall time of its phases to stderr, synchronising its stream between
// phases so that device work is attributed to the phase that issued it.
bool trace_on();
struct PhaseTrace {
    const char *who;
    double t0 = 0, last = 0;
    std::string line;
    explicit PhaseTrace(const char *w);
    void mark(const char *phase, void *stream);  // stream: cudaStream_t to synchronise, or null
    ~PhaseTrace();
};

// Tiling helpers (tiles are 1-based as in tce.fh).
struct Tiling {
    int64_t noab = 0, nvab = 0, nocc = 0, nvir = 0;
    const int64_t *range = nullptr, *spin = nullptr, *sym = nullptr;
    const int64_t *offset = nullptr, *alpha = nullptr;
    const double *evl = nullptr;
    int64_t restricted = 0;
    int64_t r(int64_t b) const { return range[b - 1]; }
    int64_t s(int64_t b) const { return spin[b - 1]; }
    int64_t y(int64_t b) const { return sym[b - 1]; }
    // Start of tile b inside its own space (occupied or virtual).
    int64_t start(int64_t b) const {
        return b <= noab ? offset[b - 1] : offset[b - 1] - nocc;
    }
};
bool make_tiling(const sdt_tiling *in, Tiling *out);

// Binary search of tce_hash (src/tce/tce_hash.F:271-316); -1 when absent.
int64_t hash_lookup(const int64_t *hash, int64_t key);

}  // namespace sdt
