// extern "C" boundary: status codes, thread-local error messages, and the
// drop-in calls that keep the reference's host-buffer call surface
// (bemSystem, qrSolver, GMRES, genExtPressure, wrtCplxMat, mesh methods).
#include <cublas_v2.h>
#include <cusolverDn.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "../../include/bem_gb300.h"
#include "bem_common.h"
#include "kernels.h"
#include "mesh.h"
#include "solver.h"

namespace bem {

std::atomic<long long> g_launches{0};
std::atomic<bool> g_profiling{false};
thread_local std::string g_last_error;

int device_sm_count() {
    constexpr int kMaxDev = 64;
    static std::atomic<int> cache[kMaxDev];
    int dev = 0;
    CUDA_TRY(cudaGetDevice(&dev));
    if (dev >= 0 && dev < kMaxDev) {
        const int c = cache[dev].load(std::memory_order_relaxed);
        if (c > 0) return c;
    }
    int v = 0;
    CUDA_TRY(cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev));
    if (v < 1) BEM_FAIL(BEM_ERR_CUDA, "device reports no multiprocessors");
    if (dev >= 0 && dev < kMaxDev) cache[dev].store(v, std::memory_order_relaxed);
    return v;
}

namespace {
struct ProfRec {
    const char *name;
    cudaEvent_t ev[2];
};
std::mutex g_prof_mu;
std::vector<ProfRec> g_prof;           // records of the current profiling window
std::vector<std::pair<const char *, double>> g_host_prof;   // host sections: name, ms
long long now_ns() {
    return std::chrono::duration_cast<std::chrono::nanoseconds>(
               std::chrono::steady_clock::now().time_since_epoch())
        .count();
}
std::vector<cudaEvent_t> g_ev_pool;    // events for reuse

cudaEvent_t pool_event() {
    if (!g_ev_pool.empty()) {
        cudaEvent_t e = g_ev_pool.back();
        g_ev_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}
}  // namespace

ProfScope::ProfScope(const char *name, cudaStream_t st) : stream(st) {
    if (!g_profiling.load(std::memory_order_relaxed)) return;
    std::lock_guard<std::mutex> lk(g_prof_mu);
    ProfRec r{name, {pool_event(), pool_event()}};
    cudaEventRecord(r.ev[0], st);
    slot = (int)g_prof.size();
    g_prof.push_back(r);
}

ProfScope::~ProfScope() {
    if (slot < 0) return;
    std::lock_guard<std::mutex> lk(g_prof_mu);
    if (slot < (int)g_prof.size()) cudaEventRecord(g_prof[slot].ev[1], stream);
}

HostProfScope::HostProfScope(const char *n) {
    if (!g_profiling.load(std::memory_order_relaxed)) return;
    name = n;
    t0_ns = now_ns();
}

HostProfScope::~HostProfScope() {
    if (!name) return;
    const double ms = 1e-6 * (double)(now_ns() - t0_ns);
    std::lock_guard<std::mutex> lk(g_prof_mu);
    g_host_prof.emplace_back(name, ms);
}

[[noreturn]] void fail(int status, const char *file, int line, const std::string &msg) {
    const char *base = std::strrchr(file, '/');
    throw Error(status, msg + " (" + (base ? base + 1 : file) + ":" + std::to_string(line) + ")");
}

// Gauss-Legendre nodes/weights (ascending) by Newton's method on the
// three-term Legendre recurrence; the reference gets the same rule from the
// Golub-Welsch eigenproblem (numerical.cu:186-225).
void gauss_legendre_host(int n, double *x, double *w) {
    for (int i = 0; i < n; i++) {
        double z = std::cos(kPi * (i + 0.75) / (n + 0.5));
        double p0 = 1.0, p1 = z, dp = 1.0;
        for (int it = 0; it < 100; it++) {
            p0 = 1.0;
            p1 = z;
            for (int l = 2; l <= n; l++) {
                double p2 = ((2.0 * l - 1.0) * z * p1 - (l - 1.0) * p0) / l;
                p0 = p1;
                p1 = p2;
            }
            if (n == 1) { p1 = z; p0 = 1.0; }
            dp = n * (z * p1 - p0) / (z * z - 1.0);
            double dz = p1 / dp;
            z -= dz;
            if (std::fabs(dz) < 1e-16) break;
        }
        p0 = 1.0;
        p1 = z;
        for (int l = 2; l <= n; l++) {
            double p2 = ((2.0 * l - 1.0) * z * p1 - (l - 1.0) * p0) / l;
            p0 = p1;
            p1 = p2;
        }
        if (n == 1) { p1 = z; p0 = 1.0; }
        dp = n * (z * p1 - p0) / (z * z - 1.0);
        x[n - 1 - i] = z;
        w[n - 1 - i] = 2.0 / ((1.0 - z * z) * dp * dp);
    }
}

// Unrestarted GMRES on a square system with the reference's stopping rule
// (GMRES.cu:145-279): stop at once when ||b - A x0||/||b|| < thr, otherwise
// iterate until |residual estimate|/||b|| < thr or maxIter steps.  A is the
// caller's column-major c64 matrix; the operator product runs in FP32 on the
// device (a column-major matrix read as the row-major transpose), the
// Arnoldi basis, Givens rotations and the back substitution in FP64.
void gmres_square_c64(const float *A_h, const float *b_h, int m, int max_iter, float thr, float *x_h) {
    BEM_CHECK_ARG(A_h && b_h && x_h && m >= 1 && max_iter >= 1, "bad GMRES arguments");
    bem_solver_s ctx;   // stream + handles
    cudaStream_t st = ctx.stream;
    const int kmax = std::min(max_iter, m);
    const size_t ldm = (m + 7) / 8 * 8;
    DevMem A, V, H, cs, sn, g, y, h1, h2, w, t, part, scal, x, b, r;
    A.ensure(sizeof(float2) * ldm * m);
    CUDA_TRY(cudaMemcpy2DAsync(A.p, sizeof(float2) * ldm, A_h, sizeof(float2) * m, sizeof(float2) * m, m,
                               cudaMemcpyHostToDevice, st));
    V.ensure(sizeof(double2) * (size_t)m * (kmax + 1));
    H.ensure(sizeof(double2) * (size_t)(kmax + 1) * kmax);
    cs.ensure(sizeof(double2) * kmax);
    sn.ensure(sizeof(double2) * kmax);
    g.ensure(sizeof(double2) * (kmax + 1));
    y.ensure(sizeof(double2) * kmax);
    h1.ensure(sizeof(double2) * (kmax + 1));
    h2.ensure(sizeof(double2) * (kmax + 1));
    w.ensure(sizeof(double2) * m);
    t.ensure(sizeof(float2) * m);
    part.ensure(sizeof(float2) * (size_t)gemv_h_splits(m, m) * m);
    scal.ensure(sizeof(double) * 8);
    x.ensure(sizeof(double2) * m);
    b.ensure(sizeof(double2) * m);
    r.ensure(sizeof(double2) * m);
    std::vector<double2> hx(m), hb(m);
    for (int i = 0; i < m; i++) {
        hx[i] = make_double2(x_h[2 * i], x_h[2 * i + 1]);
        hb[i] = make_double2(b_h[2 * i], b_h[2 * i + 1]);
    }
    CUDA_TRY(cudaMemcpyAsync(x.p, hx.data(), sizeof(double2) * m, cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(b.p, hb.data(), sizeof(double2) * m, cudaMemcpyHostToDevice, st));
    double *sc = scal.as<double>();
    auto read = [&](int i) {
        CUDA_TRY(cudaMemcpyAsync(ctx.h_pinned + i, sc + i, sizeof(double), cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaStreamSynchronize(st));
        return ctx.h_pinned[i];
    };
    // r = b - A x0  (A x via the transposed view)
    launch_gemv_h_c64(m, m, A.as<float2>(), ldm, x.p, 1, w.p, 1, part.p, st, false);
    launch_copy_f64(m, b.as<double2>(), r.as<double2>(), st);
    // r -= w : reuse update with one basis vector and h = 1
    double2 one = make_double2(1.0, 0.0);
    CUDA_TRY(cudaMemcpyAsync(h1.p, &one, sizeof(double2), cudaMemcpyHostToDevice, st));
    launch_update(m, 1, w.as<double2>(), m, h1.as<double2>(), r.as<double2>(), st);
    launch_nrm2(m, b.as<double2>(), sc + 0, nullptr, st);
    launch_nrm2(m, r.as<double2>(), sc + 1, nullptr, st);
    const double nb = read(0), nr = read(1);
    if (!(nb > 0.0) || nr / nb < thr) return;   // initial guess accurate enough
    launch_scale_copy(m, r.as<double2>(), sc + 1, V.as<double2>(), st);
    launch_zero_f64(kmax + 1, g.as<double2>(), st);
    launch_set_scalar_c(g.as<double2>(), sc + 1, st);
    const int ldh = kmax + 1;
    int it = 0;
    for (int j = 0; j < kmax; j++) {
        double2 *vj = V.as<double2>() + (size_t)j * m;
        launch_gemv_h_c64(m, m, A.as<float2>(), ldm, vj, 1, w.p, 1, part.p, st, false);
        launch_dots(m, j + 1, V.as<double2>(), m, w.as<double2>(), h1.as<double2>(), nullptr, st);
        launch_update(m, j + 1, V.as<double2>(), m, h1.as<double2>(), w.as<double2>(), st);
        launch_dots(m, j + 1, V.as<double2>(), m, w.as<double2>(), h2.as<double2>(), nullptr, st);
        launch_update(m, j + 1, V.as<double2>(), m, h2.as<double2>(), w.as<double2>(), st);
        launch_nrm2(m, w.as<double2>(), sc + 2, nullptr, st);
        launch_hcol_finish(j, h1.as<double2>(), h2.as<double2>(), sc + 2, H.as<double2>(), ldh, st);
        launch_scale_copy(m, w.as<double2>(), sc + 2, V.as<double2>() + (size_t)(j + 1) * m, st);
        launch_givens(j, H.as<double2>(), ldh, cs.as<double2>(), sn.as<double2>(), g.as<double2>(), sc + 3, st);
        it = j + 1;
        const double res = read(3);
        if (res / nb < thr) break;
    }
    launch_trisolve(it, H.as<double2>(), ldh, g.as<double2>(), y.as<double2>(), st);
    launch_axpy_combo(m, it, V.as<double2>(), m, y.as<double2>(), x.as<double2>(), st);
    CUDA_TRY(cudaMemcpyAsync(hx.data(), x.p, sizeof(double2) * m, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    for (int i = 0; i < m; i++) {
        x_h[2 * i] = (float)hx[i].x;
        x_h[2 * i + 1] = (float)hx[i].y;
    }
}

// qrSolver (numerical.cu:580-644): cuSOLVER Cgeqrf + Cunmqr + cuBLAS Ctrsm on
// device copies of the caller's host buffers; B is overwritten (ldB x nB).
void qr_solve_c64(const float *A_h, int mA, int nA, int ldA, float *B_h, int nB, int ldB) {
    BEM_CHECK_ARG(A_h && B_h && mA >= nA && nA >= 1 && nB >= 1 && ldA >= mA && ldB >= mA, "bad qrSolver arguments");
    bem_solver_s ctx;
    cudaStream_t st = ctx.stream;
    DevMem A, B, tau, work, info;
    A.ensure(sizeof(cuComplex) * (size_t)ldA * nA);
    B.ensure(sizeof(cuComplex) * (size_t)ldB * nB);
    CUDA_TRY(cudaMemcpyAsync(A.p, A_h, sizeof(cuComplex) * (size_t)ldA * nA, cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(B.p, B_h, sizeof(cuComplex) * (size_t)ldB * nB, cudaMemcpyHostToDevice, st));
    int lw1 = 0, lw2 = 0;
    tau.ensure(sizeof(cuComplex) * nA);
    info.ensure(sizeof(int));
    if (cusolverDnCgeqrf_bufferSize(ctx.cusolver, mA, nA, A.as<cuComplex>(), ldA, &lw1) != CUSOLVER_STATUS_SUCCESS ||
        cusolverDnCunmqr_bufferSize(ctx.cusolver, CUBLAS_SIDE_LEFT, CUBLAS_OP_C, mA, nB, nA, A.as<cuComplex>(), ldA,
                                    tau.as<cuComplex>(), B.as<cuComplex>(), ldB, &lw2) != CUSOLVER_STATUS_SUCCESS)
        BEM_FAIL(BEM_ERR_CUDA, "cusolver buffer query failed");
    int lw = std::max(1, std::max(lw1, lw2));
    work.ensure(sizeof(cuComplex) * lw);
    if (cusolverDnCgeqrf(ctx.cusolver, mA, nA, A.as<cuComplex>(), ldA, tau.as<cuComplex>(), work.as<cuComplex>(), lw,
                         info.as<int>()) != CUSOLVER_STATUS_SUCCESS ||
        cusolverDnCunmqr(ctx.cusolver, CUBLAS_SIDE_LEFT, CUBLAS_OP_C, mA, nB, nA, A.as<cuComplex>(), ldA,
                         tau.as<cuComplex>(), B.as<cuComplex>(), ldB, work.as<cuComplex>(), lw,
                         info.as<int>()) != CUSOLVER_STATUS_SUCCESS)
        BEM_FAIL(BEM_ERR_CUDA, "cusolver QR failed");
    cuComplex one = make_cuComplex(1.f, 0.f);
    if (cublasCtrsm(ctx.cublas, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_UPPER, CUBLAS_OP_N, CUBLAS_DIAG_NON_UNIT, nA, nB,
                    &one, A.as<cuComplex>(), ldA, B.as<cuComplex>(), ldB) != CUBLAS_STATUS_SUCCESS)
        BEM_FAIL(BEM_ERR_CUDA, "cublasCtrsm failed");
    int hinfo = 0;
    CUDA_TRY(cudaMemcpyAsync(B_h, B.p, sizeof(cuComplex) * (size_t)ldB * nB, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaMemcpyAsync(&hinfo, info.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    if (hinfo != 0) BEM_FAIL(BEM_ERR_NUMERIC, "QR reported info = " + std::to_string(hinfo));
}

void validate_options(const bem_options_t &o) {
    BEM_CHECK_ARG(o.order >= 1 && o.order <= kMaxOrder, "order must be in [1, 12]");
    BEM_CHECK_ARG(o.density > 0 && o.speed > 0, "density and speed must be positive");
    BEM_CHECK_ARG(o.near_eta >= 0 && o.near_depth >= 0 && o.near_depth <= 4, "near_eta >= 0, near_depth in [0, 4]");
    BEM_CHECK_ARG(o.tol > 0 && o.max_iter >= 1 && o.inner_tol > 0 && o.max_refine >= 0, "bad solver tolerances");
    BEM_CHECK_ARG(o.tile_cols >= 0, "tile_cols must be >= 0");
    BEM_CHECK_ARG(o.far_variant >= -1 && o.far_variant < far_variants(BEM_PREC_C64), "bad far_variant");
    BEM_CHECK_ARG(o.gemm_mode >= BEM_GEMM_AUTO && o.gemm_mode <= BEM_GEMM_TC, "bad gemm_mode");
    BEM_CHECK_ARG(o.block_tol > 0, "block_tol must be positive");
}

void apply_global_options(bem_options_t *o) {
    Globals &g = globals();
    std::lock_guard<std::mutex> lk(g.mu);
    o->order = g.order;
    o->density = g.density;
    o->speed = g.speed;
}

}  // namespace bem

using namespace bem;

extern "C" {

const char *bem_status_string(int s) {
    switch (s) {
        case BEM_SUCCESS: return "success";
        case BEM_FAILURE: return "failure";
        case BEM_ERR_INVALID_ARG: return "invalid argument";
        case BEM_ERR_CUDA: return "CUDA error";
        case BEM_ERR_NOMEM: return "out of memory";
        case BEM_ERR_NOT_CONVERGED: return "not converged";
        case BEM_ERR_IO: return "I/O error";
        case BEM_ERR_STATE: return "invalid state";
        case BEM_ERR_TOO_LARGE: return "size above the supported maximum";
        case BEM_ERR_NUMERIC: return "numerical failure";
        case BEM_ERR_TIMEOUT: return "timed out";
        default: return "unknown status";
    }
}

const char *bem_last_error(void) { return g_last_error.c_str(); }
int bem_version(void) { return 10000; }
long long bem_launch_count(void) { return g_launches.load(); }

int bem_profile_enable(int on) {
    BEM_API_BEGIN
    std::lock_guard<std::mutex> lk(g_prof_mu);
    for (ProfRec &r : g_prof) {
        cudaEventSynchronize(r.ev[1]);
        g_ev_pool.push_back(r.ev[0]);
        g_ev_pool.push_back(r.ev[1]);
    }
    g_prof.clear();
    g_host_prof.clear();
    g_profiling.store(on != 0);
    BEM_API_END
}

int bem_profile_report(char *buf, int buflen) {
    try {
        std::lock_guard<std::mutex> lk(g_prof_mu);
        std::vector<std::string> names;
        std::vector<long long> cnt;
        std::vector<double> tot;
        for (ProfRec &r : g_prof) {
            CUDA_TRY(cudaEventSynchronize(r.ev[1]));
            float ms = 0.f;
            CUDA_TRY(cudaEventElapsedTime(&ms, r.ev[0], r.ev[1]));
            size_t i = 0;
            while (i < names.size() && names[i] != r.name) i++;
            if (i == names.size()) {
                names.push_back(r.name);
                cnt.push_back(0);
                tot.push_back(0.0);
            }
            cnt[i]++;
            tot[i] += ms;
        }
        for (const auto &h : g_host_prof) {
            const std::string nm = std::string("host:") + h.first;
            size_t i = 0;
            while (i < names.size() && names[i] != nm) i++;
            if (i == names.size()) {
                names.push_back(nm);
                cnt.push_back(0);
                tot.push_back(0.0);
            }
            cnt[i]++;
            tot[i] += h.second;
        }
        std::string out;
        for (size_t i = 0; i < names.size(); i++)
            out += names[i] + " " + std::to_string(cnt[i]) + " " + std::to_string(tot[i]) + "\n";
        if (!buf || buflen <= (int)out.size()) {
            g_last_error = "report buffer too small";
            return -BEM_ERR_INVALID_ARG;
        }
        std::memcpy(buf, out.c_str(), out.size() + 1);
        return (int)names.size();
    } catch (const bem::Error &e) {
        g_last_error = e.what();
        return -e.status;
    }
}

int bem_gauss_legendre(int order, double *nodes, double *weights) {
    BEM_API_BEGIN
    BEM_CHECK_ARG(order >= 1 && order <= kMaxOrder && nodes && weights, "order must be in [1, 12]");
    gauss_legendre_host(order, nodes, weights);
    BEM_API_END
}

int bem_set_quadrature(int order) {
    BEM_API_BEGIN
    BEM_CHECK_ARG(order >= 1 && order <= kMaxOrder, "order must be in [1, 12]");
    std::lock_guard<std::mutex> lk(globals().mu);
    globals().order = order;
    BEM_API_END
}

int bem_get_quadrature(void) {
    std::lock_guard<std::mutex> lk(globals().mu);
    return globals().order;
}

int bem_set_medium(double density, double speed) {
    BEM_API_BEGIN
    BEM_CHECK_ARG(density > 0 && speed > 0, "density and speed must be positive");
    std::lock_guard<std::mutex> lk(globals().mu);
    globals().density = density;
    globals().speed = speed;
    BEM_API_END
}

int bem_set_point_source_strength(double q) {
    BEM_API_BEGIN
    BEM_CHECK_ARG(std::isfinite(q), "strength must be finite");
    std::lock_guard<std::mutex> lk(globals().mu);
    globals().strength = q;
    BEM_API_END
}

// ---- mesh ----
int bem_mesh_create(bem_mesh_t *out) {
    BEM_API_BEGIN
    BEM_CHECK_ARG(out, "null handle pointer");
    *out = new bem_mesh_s();
    BEM_API_END
}

int bem_mesh_destroy(bem_mesh_t m) {
    delete m;
    return BEM_SUCCESS;
}

int bem_mesh_read_obj(bem_mesh_t m, const char *path) {
    BEM_API_BEGIN
    BEM_CHECK_ARG(m && path, "null argument");
    read_obj_reference(*m, path);
    BEM_API_END
}

int bem_mesh_read_obj_robust(bem_mesh_t m, const char *path) {
    BEM_API_BEGIN
    BEM_CHECK_ARG(m && path, "null argument");
    read_obj_robust(*m, path);
    BEM_API_END
}

int bem_mesh_read_ply(bem_mesh_t m, const char *path) {
    BEM_API_BEGIN
    BEM_CHECK_ARG(m && path, "null argument");
    read_ply(*m, path);
    BEM_API_END
}

int bem_mesh_orient(bem_mesh_t m, int *flipped, int *components, int *open_edges, int *nonmanifold,
                    double *volume) {
    BEM_API_BEGIN
    BEM_CHECK_ARG(m, "null mesh");
    m->validate();
    const MeshOrientReport r = orient_mesh(*m);
    if (flipped) *flipped = r.flipped;
    if (components) *components = r.components;
    if (open_edges) *open_edges = r.open_edges;
    if (nonmanifold) *nonmanifold = r.nonmanifold;
    if (volume) *volume = r.volume;
    BEM_API_END
}

int bem_mesh_set(bem_mesh_t m, const double *pnts, int num_pnts, const int *elems, int num_elems) {
    BEM_API_BEGIN
    BEM_CHECK_ARG(m && pnts && elems && num_pnts > 0 && num_elems > 0, "bad mesh arrays");
    for (long long i = 0; i < 3LL * num_elems; i++)
        BEM_CHECK_ARG(elems[i] >= 0 && elems[i] < num_pnts, "element node index out of range");
    m->pnts.assign(pnts, pnts + 3 * (size_t)num_pnts);
    m->elems.assign(elems, elems + 3 * (size_t)num_elems);
    m->chief.clear();
    m->has_bb = false;
    m->default_bc();
    BEM_API_END
}

int bem_mesh_set_bc(bem_mesh_t m, const double *bc) {
    BEM_API_BEGIN
    BEM_CHECK_ARG(m && bc, "null argument");
    for (int e = 0; e < m->num_elems(); e++)
        BEM_CHECK_ARG(bc[6 * e + 2] != 0.0 || bc[6 * e + 3] != 0.0, "cb must be nonzero");
    m->bc.assign(bc, bc + 6 * (size_t)m->num_elems());
    BEM_API_END
}

int bem_mesh_set_uniform_bc(bem_mesh_t m, double ca_re, double ca_im, double cb_re, double cb_im,
                            double cc_re, double cc_im) {
    BEM_API_BEGIN
    BEM_CHECK_ARG(m, "null mesh");
    BEM_CHECK_ARG(cb_re != 0.0 || cb_im != 0.0, "cb must be nonzero");
    double b[6] = {ca_re, ca_im, cb_re, cb_im, cc_re, cc_im};
    m->bc.resize(6 * (size_t)m->num_elems());
    for (int e = 0; e < m->num_elems(); e++) std::memcpy(&m->bc[6 * (size_t)e], b, sizeof(b));
    BEM_API_END
}

int bem_mesh_find_bb(bem_mesh_t m, float threshold) {
    BEM_API_BEGIN
    BEM_CHECK_ARG(m, "null mesh");
    find_bb(*m, threshold);
    BEM_API_END
}

int bem_mesh_get_bb(bem_mesh_t m, float *bb6) {
    BEM_API_BEGIN
    BEM_CHECK_ARG(m && bb6, "null argument");
    if (!m->has_bb) BEM_FAIL(BEM_ERR_STATE, "findBB not called");
    std::memcpy(bb6, m->bb, sizeof(m->bb));
    BEM_API_END
}

int bem_mesh_gen_chief(bem_mesh_t m, int num, float threshold) {
    BEM_API_BEGIN
    BEM_CHECK_ARG(m, "null mesh");
    gen_chief(*m, num, threshold);
    BEM_API_END
}

int bem_mesh_set_chief(bem_mesh_t m, const double *pnts, int num) {
    BEM_API_BEGIN
    BEM_CHECK_ARG(m && num >= 0 && (num == 0 || pnts), "bad CHIEF arguments");
    m->chief.assign(pnts, pnts + 3 * (size_t)num);
    BEM_API_END
}

int bem_mesh_get_counts(bem_mesh_t m, int *num_pnts, int *num_elems, int *num_chief) {
    BEM_API_BEGIN
    BEM_CHECK_ARG(m, "null mesh");
    if (num_pnts) *num_pnts = m->num_pnts();
    if (num_elems) *num_elems = m->num_elems();
    if (num_chief) *num_chief = m->num_chief();
    BEM_API_END
}

int bem_mesh_get_points(bem_mesh_t m, double *pnts) {
    BEM_API_BEGIN
    BEM_CHECK_ARG(m && pnts, "null argument");
    std::copy(m->pnts.begin(), m->pnts.end(), pnts);
    BEM_API_END
}

int bem_mesh_get_elems(bem_mesh_t m, int *elems) {
    BEM_API_BEGIN
    BEM_CHECK_ARG(m && elems, "null argument");
    std::copy(m->elems.begin(), m->elems.end(), elems);
    BEM_API_END
}

int bem_mesh_get_chief(bem_mesh_t m, double *pnts) {
    BEM_API_BEGIN
    BEM_CHECK_ARG(m && (pnts || m->chief.empty()), "null argument");
    std::copy(m->chief.begin(), m->chief.end(), pnts);
    BEM_API_END
}

int bem_mesh_icosphere(bem_mesh_t m, int subdiv, double radius) {
    BEM_API_BEGIN
    BEM_CHECK_ARG(m, "null mesh");
    make_icosphere(*m, subdiv, radius);
    BEM_API_END
}

int bem_mesh_surface_area(bem_mesh_t m, double *area) {
    BEM_API_BEGIN
    BEM_CHECK_ARG(m && area, "null argument");
    double a = 0;
    for (int e = 0; e < m->num_elems(); e++) {
        const double *p1 = &m->pnts[3 * (size_t)m->elems[3 * e]], *p2 = &m->pnts[3 * (size_t)m->elems[3 * e + 1]],
                     *p3 = &m->pnts[3 * (size_t)m->elems[3 * e + 2]];
        double u[3] = {p1[0] - p3[0], p1[1] - p3[1], p1[2] - p3[2]};
        double v[3] = {p2[0] - p3[0], p2[1] - p3[1], p2[2] - p3[2]};
        double c[3] = {u[1] * v[2] - u[2] * v[1], u[2] * v[0] - u[0] * v[2], u[0] * v[1] - u[1] * v[0]};
        a += 0.5 * std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
    }
    *area = a;
    BEM_API_END
}

int bem_mesh_geodesic(bem_mesh_t m, int nu, double radius) {
    BEM_API_BEGIN
    BEM_CHECK_ARG(m, "null mesh");
    make_geodesic(*m, nu, radius);
    BEM_API_END
}

int bem_mesh_perturbed_ellipsoid(bem_mesh_t m, double a, double b, double c, int lmax, double amp,
                                 unsigned long long seed) {
    BEM_API_BEGIN
    BEM_CHECK_ARG(m, "null mesh");
    map_perturbed_ellipsoid(*m, a, b, c, lmax, amp, seed);
    BEM_API_END
}

int bem_fibonacci_sphere(int n, double radius, double *pts) {
    BEM_API_BEGIN
    fibonacci_sphere(n, radius, pts);
    BEM_API_END
}

// ---- drop-in calls ----
static void reference_options(bem_options_t *o) {
    bem_options_default(o);
    o->near_eta = 0.0;   // the reference integrates every non-vertex pair with the plain rule
}

int bem_system_c64(bem_mesh_t m, float k, const float *srcs, int num_srcs, float *A, int lda, float *B, int ldb) {
    BEM_API_BEGIN
    BEM_CHECK_ARG(m && srcs && A && B && num_srcs >= 1, "bad bemSystem arguments");
    m->validate();
    bem_solver_s s;
    reference_options(&s.opt);
    s.set_geometry(m->pnts.data(), m->num_pnts(), m->elems.data(), m->num_elems(), m->bc.data(),
                   m->chief.data(), m->num_chief());
    double q;
    {
        std::lock_guard<std::mutex> lk(globals().mu);
        q = globals().strength;
    }
    std::vector<bem_source_t> src(num_srcs);
    for (int i = 0; i < num_srcs; i++) {
        src[i].kind = BEM_SRC_POINT;
        for (int d = 0; d < 3; d++) src[i].vec[d] = srcs[3 * i + d];
        src[i].amp_re = q;
        src[i].amp_im = 0.0;
    }
    s.set_sources(src.data(), num_srcs);
    s.assemble((double)k, BEM_PREC_C64);
    s.get_system(A, lda, B, ldb, BEM_PREC_C64);
    BEM_API_END
}

int bem_qr_solve_c64(const float *A, int mA, int nA, int ldA, float *B, int nB, int ldB) {
    BEM_API_BEGIN
    qr_solve_c64(A, mA, nA, ldA, B, nB, ldB);
    BEM_API_END
}

int bem_gmres_c64(const float *A, const float *b, int m, int max_iter, float thr, float *x) {
    BEM_API_BEGIN
    gmres_square_c64(A, b, m, max_iter, thr, x);
    BEM_API_END
}

int bem_ext_pressure_c64(float k, bem_mesh_t m, const float *src, const float *x, const float *surf_p, float *p_out) {
    BEM_API_BEGIN
    BEM_CHECK_ARG(m && src && x && surf_p && p_out, "bad genExtPressure arguments");
    m->validate();
    bem_solver_s s;
    reference_options(&s.opt);
    s.set_geometry(m->pnts.data(), m->num_pnts(), m->elems.data(), m->num_elems(), m->bc.data(), nullptr, 0);
    bem_source_t sr;
    sr.kind = BEM_SRC_POINT;
    for (int d = 0; d < 3; d++) sr.vec[d] = src[d];
    {
        std::lock_guard<std::mutex> lk(globals().mu);
        sr.amp_re = globals().strength;
    }
    sr.amp_im = 0.0;
    s.set_sources(&sr, 1);
    s.k = (double)k;
    DevMem u;
    u.ensure(sizeof(float2) * s.N);
    CUDA_TRY(cudaMemcpyAsync(u.p, surf_p, sizeof(float2) * s.N, cudaMemcpyHostToDevice, s.stream));
    double xd[3] = {x[0], x[1], x[2]};
    s.eval_field(xd, 1, p_out, 1, BEM_PREC_C64, u.p, BEM_PREC_C64);
    BEM_API_END
}

int bem_write_cplx_mat_c64(const float *mat, int rows, int cols, int ldm, const char *path) {
    BEM_API_BEGIN
    BEM_CHECK_ARG(mat && path && rows >= 0 && cols >= 0 && ldm >= rows, "bad wrtCplxMat arguments");
    FILE *f = std::fopen(path, "w");
    if (!f) BEM_FAIL(BEM_ERR_IO, std::string("Failed to open file ") + path);
    for (int i = 0; i < rows; i++) {
        for (int j = 0; j < cols; j++) {
            size_t idx = (size_t)ldm * j + i;
            if (std::fprintf(f, "(%f,%f) ", mat[2 * idx], mat[2 * idx + 1]) < 0) {
                std::fclose(f);
                BEM_FAIL(BEM_ERR_IO, "Failed to write!");
            }
        }
        std::fprintf(f, "\n");
    }
    std::fclose(f);
    BEM_API_END
}

// ---- solver handle ----
int bem_options_default(bem_options_t *o) {
    if (!o) return BEM_ERR_INVALID_ARG;
    o->density = 1.2041;
    o->speed = 343.21;
    o->order = 6;
    o->near_eta = 0.0;
    o->near_depth = 3;
    o->tol = 1e-8;
    o->max_iter = 300;
    o->inner_tol = 1e-4;
    o->max_refine = 10;
    o->tile_cols = 0;
    o->far_variant = -1;
    o->gemm_mode = BEM_GEMM_AUTO;
    o->block_tol = 1e-6;
    apply_global_options(o);
    return BEM_SUCCESS;
}

int bem_solver_create(bem_solver_t *out) {
    BEM_API_BEGIN
    BEM_CHECK_ARG(out, "null handle pointer");
    *out = new bem_solver_s();
    BEM_API_END
}

int bem_solver_destroy(bem_solver_t s) {
    delete s;
    return BEM_SUCCESS;
}

int bem_solver_set_options(bem_solver_t s, const bem_options_t *o) {
    BEM_API_BEGIN
    BEM_CHECK_ARG(s && o, "null argument");
    validate_options(*o);
    if (o->tile_cols != s->opt.tile_cols) s->tiles[0].valid = s->tiles[1].valid = false;
    s->opt = *o;
    s->assembled = s->solved = false;
    BEM_API_END
}

int bem_solver_get_options(bem_solver_t s, bem_options_t *o) {
    BEM_API_BEGIN
    BEM_CHECK_ARG(s && o, "null argument");
    *o = s->opt;
    BEM_API_END
}

int bem_solver_set_mesh(bem_solver_t s, bem_mesh_t m) {
    BEM_API_BEGIN
    BEM_CHECK_ARG(s && m, "null argument");
    m->validate();
    s->set_geometry(m->pnts.data(), m->num_pnts(), m->elems.data(), m->num_elems(), m->bc.data(),
                    m->chief.data(), m->num_chief());
    BEM_API_END
}

int bem_solver_set_geometry(bem_solver_t s, const double *pnts, int num_pnts, const int *elems, int num_elems,
                            const double *bc, const double *chief, int num_chief) {
    BEM_API_BEGIN
    BEM_CHECK_ARG(s, "null solver");
    s->set_geometry(pnts, num_pnts, elems, num_elems, bc, chief, num_chief);
    BEM_API_END
}

int bem_solver_set_sources(bem_solver_t s, const bem_source_t *srcs, int num_srcs) {
    BEM_API_BEGIN
    BEM_CHECK_ARG(s, "null solver");
    s->set_sources(srcs, num_srcs);
    BEM_API_END
}

int bem_solver_assemble(bem_solver_t s, double k, int precision) {
    BEM_API_BEGIN
    BEM_CHECK_ARG(s, "null solver");
    s->assemble(k, precision);
    BEM_API_END
}

int bem_solver_solve(bem_solver_t s, int method, bem_solve_info_t *info) {
    BEM_API_BEGIN
    BEM_CHECK_ARG(s, "null solver");
    bem_solve_info_t local{};
    s->solve(method, &local);
    if (info) *info = local;
    if (method == BEM_SOLVE_GMRES_REFINED && !local.converged) {
        g_last_error = "refinement did not reach the tolerance";
        return BEM_ERR_NOT_CONVERGED;
    }
    BEM_API_END
}

int bem_solver_get_solution(bem_solver_t s, void *x, int ldx, int precision) {
    BEM_API_BEGIN
    BEM_CHECK_ARG(s, "null solver");
    s->get_solution(x, ldx, precision);
    BEM_API_END
}

int bem_solver_get_system(bem_solver_t s, void *A, int lda, void *B, int ldb, int precision) {
    BEM_API_BEGIN
    BEM_CHECK_ARG(s, "null solver");
    s->get_system(A, lda, B, ldb, precision);
    BEM_API_END
}

int bem_solver_eval_field(bem_solver_t s, const double *pts, int num_pts, void *p, int ldp, int precision) {
    BEM_API_BEGIN
    BEM_CHECK_ARG(s, "null solver");
    s->eval_field(pts, num_pts, p, ldp, precision);
    BEM_API_END
}

int bem_solver_sync(bem_solver_t s) {
    BEM_API_BEGIN
    BEM_CHECK_ARG(s, "null solver");
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    BEM_API_END
}

void *bem_solver_stream(bem_solver_t s) { return s ? (void *)s->stream : nullptr; }

int bem_solver_sizes(bem_solver_t s, int *n, int *m, int *num_elems, int *num_srcs) {
    BEM_API_BEGIN
    BEM_CHECK_ARG(s, "null solver");
    if (n) *n = s->N;
    if (m) *m = s->M;
    if (num_elems) *num_elems = s->E;
    if (num_srcs) *num_srcs = s->S;
    BEM_API_END
}

int bem_solver_block_gemm_mode(bem_solver_t s, int *mode) {
    BEM_API_BEGIN
    BEM_CHECK_ARG(s && mode, "null argument");
    *mode = s->last_block_gemm_mode;
    BEM_API_END
}

int bem_solver_far_variant(bem_solver_t s, int *variant) {
    BEM_API_BEGIN
    BEM_CHECK_ARG(s && variant, "null argument");
    *variant = s->far_variant_used;
    BEM_API_END
}

}  // extern "C"
