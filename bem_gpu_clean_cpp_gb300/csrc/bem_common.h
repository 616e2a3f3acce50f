// Internal definitions shared by the GB300 BEM library sources.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <cstdio>
#include <stdexcept>
#include <string>

#include "../../include/bem_gb300.h"

namespace bem {

// Error carried from the library internals to the C ABI boundary, where it is
// turned into a status code plus a thread-local message (bem_last_error()).
struct Error : std::runtime_error {
    int status;
    Error(int st, const std::string &msg) : std::runtime_error(msg), status(st) {}
};

[[noreturn]] void fail(int status, const char *file, int line, const std::string &msg);

#define BEM_FAIL(st, msg) ::bem::fail((st), __FILE__, __LINE__, (msg))
#define BEM_CHECK_ARG(cond, msg) \
    do { if (!(cond)) BEM_FAIL(BEM_ERR_INVALID_ARG, (msg)); } while (0)
#define CUDA_TRY(x)                                                                  \
    do {                                                                             \
        cudaError_t e_ = (x);                                                        \
        if (e_ != cudaSuccess)                                                       \
            ::bem::fail(e_ == cudaErrorMemoryAllocation ? BEM_ERR_NOMEM : BEM_ERR_CUDA, \
                        __FILE__, __LINE__,                                          \
                        std::string(#x) + ": " + cudaGetErrorString(e_));           \
    } while (0)
// Message of the last failed call on this thread (bem_last_error()).
extern thread_local std::string g_last_error;
// Body of an extern "C" entry point: exceptions become status codes.
#define BEM_API_BEGIN try {
#define BEM_API_END                                   \
    return BEM_SUCCESS;                               \
    }                                                 \
    catch (const ::bem::Error &e) {                   \
        ::bem::g_last_error = e.what();               \
        return e.status;                              \
    }                                                 \
    catch (const std::bad_alloc &) {                  \
        ::bem::g_last_error = "host out of memory";   \
        return BEM_ERR_NOMEM;                         \
    }                                                 \
    catch (const std::exception &e) {                 \
        ::bem::g_last_error = e.what();               \
        return BEM_FAILURE;                           \
    }

// After a kernel launch: configuration errors surface here.
#define KERNEL_CHECK() CUDA_TRY(cudaGetLastError())

// Counts kernels launched by this library (reported by bench.py).
extern std::atomic<long long> g_launches;
inline void count_launch(long long n = 1) { g_launches.fetch_add(n, std::memory_order_relaxed); }

// Optional kernel timing: while enabled (bem_profile_enable), a ProfScope
// brackets a launch with CUDA events on its stream; bem_profile_report sums
// the elapsed times per name.
extern std::atomic<bool> g_profiling;
struct ProfScope {
    ProfScope(const char *name, cudaStream_t st);
    ~ProfScope();
    int slot = -1;
    cudaStream_t stream = nullptr;
};
#define BEM_PROF(name, st) ::bem::ProfScope bem_prof_scope_((name), (st))
// Host-side counterpart: wall time of a host code section (table builds,
// host-device round trips), reported as "host:<name>" while profiling.
struct HostProfScope {
    explicit HostProfScope(const char *name);
    ~HostProfScope();
    const char *name = nullptr;
    long long t0_ns = 0;
};
#define BEM_HOST_PROF(name) ::bem::HostProfScope bem_host_prof_scope_(name)

// Streaming multiprocessors of the current device (queried once per device).
int device_sm_count();

constexpr double kPi = 3.14159265358979323846;
constexpr int kMaxOrder = 12;              // Gauss points per direction
constexpr int kMaxQ = kMaxOrder * kMaxOrder;

// Per-element boundary condition ratios used by the assembly:
// bcA = ca/cb, bcC = cc/cb for the element's ca*p + cb*v = cc.
struct BcRatios {
    double a_re, a_im, c_re, c_im;
};

// A record in a column tile's element list (far-field kernel input).
struct TileRec {
    int eid;        // element index
    int node[3];    // the element's node indices
    int slot[3];    // tile-local column of node j, -1 when node j is outside the tile
    int owner;      // 1 when this tile counts the element's c and beta terms
};

}  // namespace bem
