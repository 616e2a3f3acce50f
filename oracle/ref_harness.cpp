// Reference-kernel harness -- TEST AND BENCHMARK INFRASTRUCTURE ONLY.
//
// Runs the reference's own GPU code on this machine's GPU so that its results
// and timings can be compared with the oracle and the engine:
//   refh_assemble  loads the reference's assembly kernels from the cubin that
//                  oracle/ref_build.py compiles from the reference sources
//                  (atomicPntsElems_g_h_c_nsgl, atomicFuncs.cu:69-117, and
//                  atomicPntsElems_sgl, atomicFuncs.cu:119-216) and launches
//                  them exactly as atomicGenSystem does (atomicFuncs.cu:218-298):
//                  A = [I; 0] and B = p_inc on the host, 16x16 blocks over
//                  (points, elements), then 16-thread blocks over elements.
//   refh_qr        the library sequence of qrSolver (numerical.cu:580-644):
//                  cusolverDnCgeqrf, cusolverDnCunmqr (Q^H B), cublasCtrsm.
// Nothing here is product code; the engine never loads it.
#include <cublas_v2.h>
#include <cuda.h>
#include <cuda_runtime.h>
#include <cusolverDn.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace {

// triElem (mesh.h:140-209): int nodes[3]; cuFloatComplex bc[3] (8-byte aligned).
struct RefTri {
    int nodes[3];
    int pad;
    float bc[6];
};
static_assert(sizeof(RefTri) == 40, "triElem layout");

std::string g_err;

#define CU(x)                                                                       \
    do {                                                                            \
        CUresult r_ = (x);                                                          \
        if (r_ != CUDA_SUCCESS) {                                                   \
            const char *s_ = nullptr;                                               \
            cuGetErrorString(r_, &s_);                                              \
            g_err = std::string(#x) + ": " + (s_ ? s_ : "?");                       \
            return 3;                                                               \
        }                                                                           \
    } while (0)
#define CR(x)                                                                       \
    do {                                                                            \
        cudaError_t r_ = (x);                                                       \
        if (r_ != cudaSuccess) {                                                    \
            g_err = std::string(#x) + ": " + cudaGetErrorString(r_);                \
            return 3;                                                               \
        }                                                                           \
    } while (0)

struct Module {
    CUmodule mod = nullptr;
    CUfunction nsgl = nullptr, sgl = nullptr;
};

// Kernel handles by Itanium-mangled name prefix (<length><name>), which
// separates atomicPntsElems_sgl from atomicPntsElems_sgl_test.
int load_module(const char *cubin, Module &m) {
    CR(cudaFree(nullptr));   // runtime + primary context
    CU(cuModuleLoad(&m.mod, cubin));
    unsigned int n = 0;
    CU(cuModuleGetFunctionCount(&n, m.mod));
    std::vector<CUfunction> fs(n);
    CU(cuModuleEnumerateFunctions(fs.data(), n, m.mod));
    for (CUfunction f : fs) {
        const char *name = nullptr;
        CU(cuFuncGetName(&name, f));
        if (!name) continue;
        if (std::strncmp(name, "_Z26atomicPntsElems_g_h_c_nsgl", 30) == 0) m.nsgl = f;
        if (std::strncmp(name, "_Z19atomicPntsElems_sgl", 23) == 0) m.sgl = f;
    }
    if (!m.nsgl || !m.sgl) {
        g_err = "reference kernels not found in the cubin";
        return 3;
    }
    return 0;
}

}  // namespace

extern "C" {

const char *refh_last_error(void) { return g_err.c_str(); }

// pts: 3*(N+M) floats (nodes then CHIEF points); elems 3*E ints; bc 6*E
// floats (ca, cb, cc as re, im); gl_x/gl_w: the INTORDER = 6 rule as the
// reference's gaussQuad::sendToDevice uploads it; srcs 3*S floats of point
// sources with amplitude `strength` (STRENGTH).  A ((N+M) x N) and B
// ((N+M) x S) are column-major c64 with ld = N+M.  ms: the reference's own
// timer span (both kernels).
int refh_assemble(const char *cubin, int N, int M, const float *pts, int E, const int *elems, const float *bc,
                  float k, const float *gl_x, const float *gl_w, int S, const float *srcs, float strength,
                  float *A, float *B, float *ms) {
    Module mod;
    if (int st = load_module(cubin, mod)) return st;
    const int R = N + M;
    CUdeviceptr dp;
    size_t bytes = 0;
    CU(cuModuleGetGlobal(&dp, &bytes, mod.mod, "INTPNTS"));
    CU(cuMemcpyHtoD(dp, gl_x, 6 * sizeof(float)));
    CU(cuModuleGetGlobal(&dp, &bytes, mod.mod, "INTWGTS"));
    CU(cuMemcpyHtoD(dp, gl_w, 6 * sizeof(float)));
    // host initialisation (atomicFuncs.cu:227-242); p_inc = STRENGTH * G(k, |x - src|)
    std::vector<float> hA(2 * (size_t)R * N, 0.0f), hB(2 * (size_t)R * S, 0.0f);
    for (int i = 0; i < N; i++) hA[2 * ((size_t)i * R + i)] = 1.0f;
    for (int s = 0; s < S; s++)
        for (int i = 0; i < R; i++) {
            float dx = pts[3 * i] - srcs[3 * s], dy = pts[3 * i + 1] - srcs[3 * s + 1], dz = pts[3 * i + 2] - srcs[3 * s + 2];
            float r = std::sqrt(dx * dx + dy * dy + dz * dz);
            float y = 4.0f * 3.1415926535897932f * r;
            hB[2 * ((size_t)s * R + i)] = strength * std::cos(-k * r) / y;
            hB[2 * ((size_t)s * R + i) + 1] = strength * std::sin(-k * r) / y;
        }
    std::vector<RefTri> te(E);
    for (int e = 0; e < E; e++) {
        for (int j = 0; j < 3; j++) te[e].nodes[j] = elems[3 * e + j];
        te[e].pad = 0;
        for (int j = 0; j < 6; j++) te[e].bc[j] = bc[6 * e + j];
    }
    float *d_p = nullptr, *d_A = nullptr, *d_B = nullptr;
    RefTri *d_e = nullptr;
    CR(cudaMalloc(&d_p, sizeof(float) * 3 * R));
    CR(cudaMalloc(&d_e, sizeof(RefTri) * E));
    CR(cudaMalloc(&d_A, sizeof(float) * hA.size()));
    CR(cudaMalloc(&d_B, sizeof(float) * hB.size()));
    CR(cudaMemcpy(d_p, pts, sizeof(float) * 3 * R, cudaMemcpyHostToDevice));
    CR(cudaMemcpy(d_e, te.data(), sizeof(RefTri) * E, cudaMemcpyHostToDevice));
    CR(cudaMemcpy(d_A, hA.data(), sizeof(float) * hA.size(), cudaMemcpyHostToDevice));
    CR(cudaMemcpy(d_B, hB.data(), sizeof(float) * hB.size(), cudaMemcpyHostToDevice));
    cudaEvent_t e0, e1;
    CR(cudaEventCreate(&e0));
    CR(cudaEventCreate(&e1));
    int numNods = N, i0 = 0, i1 = R - 1, lda = R, ldb = R, nS = S, nE = E;
    void *a1[] = {&k, &d_p, &numNods, &i0, &i1, &d_e, &nE, &d_A, &lda, &d_B, &nS, &ldb};
    void *a2[] = {&k, &d_p, &d_e, &nE, &d_A, &lda, &d_B, &nS, &ldb};
    CR(cudaEventRecord(e0));
    CU(cuLaunchKernel(mod.nsgl, (R + 15) / 16, (E + 15) / 16, 1, 16, 16, 1, 0, nullptr, a1, nullptr));
    CU(cuLaunchKernel(mod.sgl, (E + 15) / 16, 1, 1, 16, 1, 1, 0, nullptr, a2, nullptr));
    CR(cudaEventRecord(e1));
    CR(cudaEventSynchronize(e1));
    CR(cudaGetLastError());
    float t = 0.f;
    CR(cudaEventElapsedTime(&t, e0, e1));
    if (ms) *ms = t;
    CR(cudaMemcpy(A, d_A, sizeof(float) * hA.size(), cudaMemcpyDeviceToHost));
    CR(cudaMemcpy(B, d_B, sizeof(float) * hB.size(), cudaMemcpyDeviceToHost));
    cudaFree(d_p);
    cudaFree(d_e);
    cudaFree(d_A);
    cudaFree(d_B);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cuModuleUnload(mod.mod);
    return 0;
}

// qrSolver's library sequence on (m x n) A and (m x S) B, column-major c64
// with ld = m; B is overwritten (solution in rows 0..n-1).  ms: the span of
// the three library calls, as the reference times it.
int refh_qr(int m, int n, const float *A, float *B, int S, float *ms) {
    cusolverDnHandle_t h = nullptr;
    cublasHandle_t hb = nullptr;
    if (cusolverDnCreate(&h) != CUSOLVER_STATUS_SUCCESS || cublasCreate(&hb) != CUBLAS_STATUS_SUCCESS) {
        g_err = "handle creation failed";
        return 3;
    }
    cuComplex *dA = nullptr, *dB = nullptr, *work = nullptr, *tau = nullptr;
    int *info = nullptr;
    CR(cudaMalloc(&dA, sizeof(cuComplex) * (size_t)m * n));
    CR(cudaMalloc(&dB, sizeof(cuComplex) * (size_t)m * S));
    CR(cudaMalloc(&tau, sizeof(cuComplex) * n));
    CR(cudaMalloc(&info, sizeof(int)));
    CR(cudaMemcpy(dA, A, sizeof(cuComplex) * (size_t)m * n, cudaMemcpyHostToDevice));
    CR(cudaMemcpy(dB, B, sizeof(cuComplex) * (size_t)m * S, cudaMemcpyHostToDevice));
    int lw = 0, lw2 = 0;
    cusolverDnCgeqrf_bufferSize(h, m, n, dA, m, &lw);
    cusolverDnCunmqr_bufferSize(h, CUBLAS_SIDE_LEFT, CUBLAS_OP_C, m, S, n, dA, m, tau, dB, m, &lw2);
    lw = lw > lw2 ? lw : lw2;
    CR(cudaMalloc(&work, sizeof(cuComplex) * (lw > 0 ? lw : 1)));
    cudaEvent_t e0, e1;
    CR(cudaEventCreate(&e0));
    CR(cudaEventCreate(&e1));
    CR(cudaEventRecord(e0));
    cusolverStatus_t s1 = cusolverDnCgeqrf(h, m, n, dA, m, tau, work, lw, info);
    cusolverStatus_t s2 = cusolverDnCunmqr(h, CUBLAS_SIDE_LEFT, CUBLAS_OP_C, m, S, n, dA, m, tau, dB, m, work, lw, info);
    cuComplex one = make_cuComplex(1.f, 0.f);
    cublasStatus_t s3 = cublasCtrsm(hb, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_UPPER, CUBLAS_OP_N, CUBLAS_DIAG_NON_UNIT,
                                    n, S, &one, dA, m, dB, m);
    CR(cudaEventRecord(e1));
    CR(cudaEventSynchronize(e1));
    float t = 0.f;
    CR(cudaEventElapsedTime(&t, e0, e1));
    if (ms) *ms = t;
    CR(cudaMemcpy(B, dB, sizeof(cuComplex) * (size_t)m * S, cudaMemcpyDeviceToHost));
    cudaFree(dA);
    cudaFree(dB);
    cudaFree(tau);
    cudaFree(info);
    cudaFree(work);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cublasDestroy(hb);
    cusolverDnDestroy(h);
    if (s1 != CUSOLVER_STATUS_SUCCESS || s2 != CUSOLVER_STATUS_SUCCESS || s3 != CUBLAS_STATUS_SUCCESS) {
        g_err = "qr library call failed";
        return 3;
    }
    return 0;
}

}  // extern "C"
