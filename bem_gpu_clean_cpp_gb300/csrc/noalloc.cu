// GMRES on caller-owned device buffers without any allocation.
//
// Some callers cannot allocate GPU memory when they solve: a serving process
// whose device memory is owned by its own pool allocator and capped, an
// application that must not add allocations while another component's CUDA
// stream capture is in progress, or a real-time loop where cudaMalloc's
// latency and implicit synchronisation are not acceptable.  They own A, b and x
// on the device already and only need the solve.
//
// bem_gmres_c64_noalloc runs the same unrestarted GMRES as bem_gmres_c64
// (the reference's GMRES.cu:145-279 stopping rule; FP32 operator products,
// FP64 Arnoldi with Gram-Schmidt applied twice, FP64 Givens rotations and back
// substitution), with every piece of scratch (Krylov basis, Hessenberg matrix,
// rotations, the split partial sums of the operator product, FP64 copies of b
// and x) carved out of one file-scope __device__ array of fixed size.
// It calls no cudaMalloc, cudaFree, cudaMallocHost or allocating library
// routine, and creates no handles: kernels go on the caller's stream, and the
// per-iteration residual estimate is copied into a local host variable.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <string>

#include "../../include/bem_gb300.h"
#include "bem_common.h"
#include "kernels.h"

namespace bem {
extern thread_local std::string g_last_error;
}

using namespace bem;

namespace {

// Scratch layout for m <= BEM_NOALLOC_MAX_M unknowns and at most
// BEM_NOALLOC_MAX_ITER iterations (sizes in bytes):
//   V     m x (kmax+1) c128        basis
//   H     (kmax+1) x kmax c128     Hessenberg / R
//   cs, sn, y            kmax c128 each
//   g, h1, h2         (kmax+1) c128 each
//   w, r, xd, bd            m c128 each
//   part    splits(m) x m c64      operator-product partial sums
//   scal    8 doubles
constexpr size_t kM = BEM_NOALLOC_MAX_M;
constexpr size_t kK = BEM_NOALLOC_MAX_ITER;
constexpr size_t kSplitsMax = kM / 32;   // gemv_h_splits(R, N) <= max(1, R/32)
constexpr size_t kBytes =
    16 * kM * (kK + 1) + 16 * (kK + 1) * kK + 3 * 16 * kK + 3 * 16 * (kK + 1) + 4 * 16 * kM +
    8 * kSplitsMax * kM + 8 * 8 + 16 * 256;   // + slack for the 256-byte carving (about 5.4 MiB)

__device__ __align__(256) unsigned char g_noalloc_scratch[kBytes];

std::mutex g_setup_mu;
struct ScratchAddr {
    CUcontext ctx;   // the context the address was looked up in
    void *addr;      // device address of g_noalloc_scratch there
};
ScratchAddr g_scratch_addr[64];

// The calling thread's current CUDA context (driver entry point through the
// runtime, no link against the driver library).
CUcontext current_context() {
    using Fn = CUresult (*)(CUcontext *);
    static Fn fn = [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        return cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) ==
                           cudaSuccess &&
                       q == cudaDriverEntryPointSuccess
                   ? reinterpret_cast<Fn>(p)
                   : nullptr;
    }();
    CUcontext c = nullptr;
    if (!fn || fn(&c) != CUDA_SUCCESS) BEM_FAIL(BEM_ERR_CUDA, "cuCtxGetCurrent is not available");
    return c;
}

// Once per device and context, with that device current: the array's device
// address (looked up again when the device's primary context was re-created,
// e.g. after cudaDeviceReset, where the module may load at another address).
// In host code g_noalloc_scratch names a host-side shadow, not device memory.
unsigned char *scratch_for_current_device() {
    int dev = 0;
    CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) BEM_FAIL(BEM_ERR_CUDA, "device index out of range");
    CUcontext ctx = current_context();   // null until the runtime made one current on this thread
    std::lock_guard<std::mutex> lk(g_setup_mu);
    if (!g_scratch_addr[dev].addr || !ctx || g_scratch_addr[dev].ctx != ctx) {
        void *p = nullptr;
        CUDA_TRY(cudaGetSymbolAddress(&p, g_noalloc_scratch));   // makes the device's context current
        ctx = current_context();
        g_scratch_addr[dev] = {ctx, p};
    }
    return static_cast<unsigned char *>(g_scratch_addr[dev].addr);
}

struct Carver {
    unsigned char *p;
    template <class T> T *take(size_t count) {
        T *out = reinterpret_cast<T *>(p);
        size_t bytes = (count * sizeof(T) + 255) / 256 * 256;
        p += bytes;
        return out;
    }
};

__global__ void c64_to_c128_kernel(int n, const float2 *__restrict__ s, double2 *__restrict__ d) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) d[i] = make_double2(s[i].x, s[i].y);
}

__global__ void c128_to_c64_kernel(int n, const double2 *__restrict__ s, float2 *__restrict__ d) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) d[i] = make_float2((float)s[i].x, (float)s[i].y);
}

void gmres_noalloc(const float *A_dev, int lda, const float *b_dev, int m, int max_iter, float thr,
                   float *x_dev, cudaStream_t st, int *iters) {
    BEM_CHECK_ARG(A_dev && b_dev && x_dev, "null device pointer");
    BEM_CHECK_ARG(m >= 1 && max_iter >= 1 && thr >= 0.0f, "bad GMRES arguments");
    if (m > (int)kM || std::min(max_iter, m) > (int)kK)
        BEM_FAIL(BEM_ERR_TOO_LARGE, "bem_gmres_c64_noalloc supports m <= " + std::to_string(kM) +
                                        " and min(max_iter, m) <= " + std::to_string(kK) + " (got m = " +
                                        std::to_string(m) + ", max_iter = " + std::to_string(max_iter) + ")");
    BEM_CHECK_ARG(lda >= m && lda % 2 == 0, "lda must be >= m and even (16-byte rows)");
    BEM_CHECK_ARG(((uintptr_t)A_dev & 15) == 0, "A must be 16-byte aligned");
    const int kmax = std::min(max_iter, m);
    Carver cv{scratch_for_current_device()};
    double2 *V = cv.take<double2>(kM * (kK + 1));
    double2 *H = cv.take<double2>((kK + 1) * kK);
    double2 *cs = cv.take<double2>(kK), *sn = cv.take<double2>(kK), *y = cv.take<double2>(kK);
    double2 *g = cv.take<double2>(kK + 1), *h1 = cv.take<double2>(kK + 1), *h2 = cv.take<double2>(kK + 1);
    double2 *w = cv.take<double2>(kM), *r = cv.take<double2>(kM);
    double2 *xd = cv.take<double2>(kM), *bd = cv.take<double2>(kM);
    float2 *part = cv.take<float2>(kSplitsMax * kM);
    double *scal = cv.take<double>(8);
    static_assert(kSplitsMax >= 1, "scratch layout");   // gemv_h_splits(m, m) <= max(1, m/32) <= kSplitsMax
    const float2 *A = reinterpret_cast<const float2 *>(A_dev);
    const int ldh = kmax + 1;
    const int nb = (m + 255) / 256;
    auto read = [&](int i) {
        double v = 0.0;   // pageable host scalar: no pinned allocation
        CUDA_TRY(cudaMemcpyAsync(&v, scal + i, sizeof(double), cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaStreamSynchronize(st));
        return v;
    };
    c64_to_c128_kernel<<<nb, 256, 0, st>>>(m, reinterpret_cast<const float2 *>(x_dev), xd);
    c64_to_c128_kernel<<<nb, 256, 0, st>>>(m, reinterpret_cast<const float2 *>(b_dev), bd);
    count_launch(2);
    KERNEL_CHECK();
    // r = b - A x0: w = A x0 (column-major A read as the row-major transpose),
    // then r = b - w via the one-vector update with h = 1 (kept in scal[7]).
    launch_gemv_h_c64(m, m, A, lda, xd, 1, w, 1, part, st, false);
    launch_copy_f64(m, bd, r, st);
    const double one[2] = {1.0, 0.0};
    CUDA_TRY(cudaMemcpyAsync(h1, one, sizeof(double2), cudaMemcpyHostToDevice, st));
    launch_update(m, 1, w, m, h1, r, st);
    launch_nrm2(m, bd, scal + 0, nullptr, st);
    launch_nrm2(m, r, scal + 1, nullptr, st);
    const double nbn = read(0), nr = read(1);
    int it = 0;
    if (nbn > 0.0 && !(nr / nbn < thr)) {
        launch_scale_copy(m, r, scal + 1, V, st);
        launch_zero_f64(kmax + 1, g, st);      // the scratch keeps the last call's contents
        launch_set_scalar_c(g, scal + 1, st);
        for (int j = 0; j < kmax; j++) {
            launch_gemv_h_c64(m, m, A, lda, V + (size_t)j * m, 1, w, 1, part, st, false);
            launch_dots(m, j + 1, V, m, w, h1, nullptr, st);
            launch_update(m, j + 1, V, m, h1, w, st);
            launch_dots(m, j + 1, V, m, w, h2, nullptr, st);
            launch_update(m, j + 1, V, m, h2, w, st);
            launch_nrm2(m, w, scal + 2, nullptr, st);
            launch_hcol_finish(j, h1, h2, scal + 2, H, ldh, st);
            launch_scale_copy(m, w, scal + 2, V + (size_t)(j + 1) * m, st);
            launch_givens(j, H, ldh, cs, sn, g, scal + 3, st);
            it = j + 1;
            if (read(3) / nbn < thr) break;
        }
        launch_trisolve(it, H, ldh, g, y, st);
        launch_axpy_combo(m, it, V, m, y, xd, st);
        c128_to_c64_kernel<<<nb, 256, 0, st>>>(m, xd, reinterpret_cast<float2 *>(x_dev));
        count_launch();
        KERNEL_CHECK();
    }
    CUDA_TRY(cudaStreamSynchronize(st));
    if (iters) *iters = it;
}

}  // namespace

extern "C" int bem_gmres_c64_noalloc(const float *A_dev, int lda, const float *b_dev, int m, int max_iter,
                                     float thr, float *x_dev, void *stream, int *iters) {
    try {
        gmres_noalloc(A_dev, lda, b_dev, m, max_iter, thr, x_dev, static_cast<cudaStream_t>(stream), iters);
        return BEM_SUCCESS;
    } catch (const bem::Error &e) {
        bem::g_last_error = e.what();
        return e.status;
    } catch (const std::exception &e) {
        bem::g_last_error = e.what();
        return BEM_FAILURE;
    }
}
