// Multi-right-hand-side least-squares solve (BEM_SOLVE_BLOCK_GMRES).
//
// All S right-hand sides (source positions) iterate together.  The normal
// operator A^H A is applied to all S vectors at once as two real GEMMs on the
// interleaved-real view of the c64 matrix:
//   A is row-major R x N complex = row-major R x 2N real  =: At^T, At column-major (2N x R);
//   T  = A V    : Tt (R x 2S)  = At^T Vt, Vt (2N x 2S) rows 2j = [Re v_j, Im v_j],
//                                          rows 2j+1 = [-Im v_j, Re v_j];
//   W  = A^H T  : Wt (2N x 2S) = At Tt,  W_j = (Wt[2j,s] + Wt[2j+1,S+s]) + i (Wt[2j,S+s] - Wt[2j+1,s]).
// The GEMMs run on the tensor cores with FP32-accurate split-BF16 emulation
// (cuBLAS CUBLAS_COMPUTE_32F_EMULATED_16BFX9) or, by option, plain FP32 or
// TF32.  Each right-hand side keeps its own Krylov space with FP64 Arnoldi
// (classical Gram-Schmidt twice), Givens rotations and back substitution;
// iteration stops per right-hand side at its tolerance.  Outer refinement
// recomputes R = B - A X and G = A^H R with the same GEMMs.
#include <cublas_v2.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "solver.h"

namespace bem {
namespace {

__global__ void build_vt_kernel(int N, int S, const double2 *__restrict__ V, float *__restrict__ Vt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, s = blockIdx.y;
    if (i >= N) return;
    const double2 v = V[(size_t)s * N + i];
    const size_t ld = 2 * (size_t)N;
    Vt[(size_t)s * ld + 2 * i] = (float)v.x;
    Vt[(size_t)(S + s) * ld + 2 * i] = (float)v.y;
    Vt[(size_t)s * ld + 2 * i + 1] = -(float)v.y;
    Vt[(size_t)(S + s) * ld + 2 * i + 1] = (float)v.x;
}

// From Tt = A X (R x 2S, real and imaginary column blocks): the residual
// r = b - t in FP64 (Rv) and packed as floats into Rt for the next GEMM.  Rt
// may be Tt itself (each element is read and written by the same thread).
__global__ void resid_from_t_kernel(int R, int S, const float *Tt, const double2 *__restrict__ B,
                                    double2 *__restrict__ Rv, float *Rt) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x, s = blockIdx.y;
    if (r >= R) return;
    const double tr = Tt[(size_t)s * R + r], ti = Tt[(size_t)(S + s) * R + r];
    const double2 b = B[(size_t)s * R + r];
    const double2 v = make_double2(b.x - tr, b.y - ti);
    Rv[(size_t)s * R + r] = v;
    Rt[(size_t)s * R + r] = (float)v.x;
    Rt[(size_t)(S + s) * R + r] = (float)v.y;
}

__global__ void combine_w_kernel(int N, int S, const float *__restrict__ Wt, double2 *__restrict__ W) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x, s = blockIdx.y;
    if (j >= N) return;
    const size_t ld = 2 * (size_t)N;
    const double a = Wt[(size_t)s * ld + 2 * j], b = Wt[(size_t)(S + s) * ld + 2 * j + 1];
    const double c = Wt[(size_t)(S + s) * ld + 2 * j], d = Wt[(size_t)s * ld + 2 * j + 1];
    W[(size_t)s * N + j] = make_double2(a + b, c - d);
}

// h[s*ldv + l] = V_l(:,s)^H W(:,s), l < k.  V_l block l: N x S column-major.
__global__ void bdots_kernel(int N, int S, const double2 *__restrict__ V, const double2 *__restrict__ W,
                             double2 *__restrict__ h, int ldv) {
    const int l = blockIdx.x, s = blockIdx.y;
    const double2 *v = V + ((size_t)l * S + s) * N;
    const double2 *w = W + (size_t)s * N;
    double sr = 0, si = 0;
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
        const double2 a = v[i], b = w[i];
        sr += a.x * b.x + a.y * b.y;
        si += a.x * b.y - a.y * b.x;
    }
    __shared__ double rr[32], ri[32];
    for (int o = 16; o > 0; o >>= 1) {
        sr += __shfl_xor_sync(0xffffffffu, sr, o);
        si += __shfl_xor_sync(0xffffffffu, si, o);
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) { rr[warp] = sr; ri[warp] = si; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0, b = 0;
        for (int t = 0; t < (int)(blockDim.x >> 5); t++) { a += rr[t]; b += ri[t]; }
        h[(size_t)s * ldv + l] = make_double2(a, b);
    }
}

// W(:,s) -= sum_{l<k} V_l(:,s) h[s][l]   (sign = -1), or X(:,s) += ... (sign = +1)
__global__ void bcombo_kernel(int N, int S, int k, const int *__restrict__ kk, const double2 *__restrict__ V,
                              const double2 *__restrict__ h, int ldv, double2 *__restrict__ W, double sign) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, s = blockIdx.y;
    if (i >= N) return;
    const int ks = kk ? min(k, kk[s]) : k;
    double sr = 0, si = 0;
    for (int l = 0; l < ks; l++) {
        const double2 a = V[((size_t)l * S + s) * N + i], c = h[(size_t)s * ldv + l];
        sr += a.x * c.x - a.y * c.y;
        si += a.x * c.y + a.y * c.x;
    }
    const double2 w = W[(size_t)s * N + i];
    W[(size_t)s * N + i] = make_double2(w.x + sign * sr, w.y + sign * si);
}

__global__ void bnrm2_kernel(int N, const double2 *__restrict__ W, double *__restrict__ out) {
    const int s = blockIdx.x;
    const double2 *w = W + (size_t)s * N;
    double a = 0;
    for (int i = threadIdx.x; i < N; i += blockDim.x) a += w[i].x * w[i].x + w[i].y * w[i].y;
    __shared__ double red[32];
    for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = a;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0;
        for (int q = 0; q < (int)(blockDim.x >> 5); q++) t += red[q];
        out[s] = sqrt(t);
    }
}

__global__ void bscale_kernel(int N, const double2 *__restrict__ W, const double *__restrict__ nrm,
                              double2 *__restrict__ Vn) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, s = blockIdx.y;
    if (i >= N) return;
    const double n = nrm[s];
    const double inv = n > 0 ? 1.0 / n : 0.0;
    const double2 w = W[(size_t)s * N + i];
    Vn[(size_t)s * N + i] = make_double2(w.x * inv, w.y * inv);
}

// Per right-hand side: H_s[:, j] = h1 + h2, H_s[j+1, j] = nrm, then the Givens
// update of GMRES.cu:44-88 and the residual estimate |g_{j+1}|.  H_s is
// (m+1) x m column-major at H + s*(m+1)*m.
__global__ void bhess_givens_kernel(int j, int S, int m, const double2 *__restrict__ h1,
                                    const double2 *__restrict__ h2, int ldv, const double *__restrict__ nrm,
                                    double2 *__restrict__ H, double2 *__restrict__ cs, double2 *__restrict__ sn,
                                    double2 *__restrict__ g, double *__restrict__ res) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= S) return;
    const int ldh = m + 1;
    double2 *h = H + ((size_t)s * m + j) * ldh;
    for (int t = 0; t <= j; t++) {
        const double2 a = h1[(size_t)s * ldv + t], b = h2[(size_t)s * ldv + t];
        h[t] = make_double2(a.x + b.x, a.y + b.y);
    }
    h[j + 1] = make_double2(nrm[s], 0.0);
    double2 *c_ = cs + (size_t)s * m, *s_ = sn + (size_t)s * m, *gg = g + (size_t)s * (m + 1);
    for (int l = 0; l < j; l++) {
        const double2 c = c_[l], sv = s_[l], a = h[l], b = h[l + 1];
        const double2 t0 = make_double2(c.x * a.x - c.y * a.y + sv.x * b.x - sv.y * b.y,
                                        c.x * a.y + c.y * a.x + sv.x * b.y + sv.y * b.x);
        const double2 t1 = make_double2(-(sv.x * a.x + sv.y * a.y) + (c.x * b.x + c.y * b.y),
                                        -(sv.x * a.y - sv.y * a.x) + (c.x * b.y - c.y * b.x));
        h[l] = t0;
        h[l + 1] = t1;
    }
    const double2 rho = h[j], sig = h[j + 1];
    const double mag = sqrt(rho.x * rho.x + rho.y * rho.y + sig.x * sig.x + sig.y * sig.y);
    double2 c, sv;
    if (mag > 0) {
        c = make_double2(rho.x / mag, -rho.y / mag);
        sv = make_double2(sig.x / mag, -sig.y / mag);
    } else {
        c = make_double2(1.0, 0.0);
        sv = make_double2(0.0, 0.0);
    }
    c_[j] = c;
    s_[j] = sv;
    h[j] = make_double2(mag, 0.0);
    h[j + 1] = make_double2(0.0, 0.0);
    const double2 gj = gg[j];
    gg[j + 1] = make_double2(-(sv.x * gj.x + sv.y * gj.y), -(sv.x * gj.y - sv.y * gj.x));
    gg[j] = make_double2(c.x * gj.x - c.y * gj.y, c.x * gj.y + c.y * gj.x);
    res[s] = sqrt(gg[j + 1].x * gg[j + 1].x + gg[j + 1].y * gg[j + 1].y);
}

__global__ void btrisolve_kernel(int S, int m, const int *__restrict__ kk, const double2 *__restrict__ H,
                                 const double2 *__restrict__ g, double2 *__restrict__ y, int ldv) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= S) return;
    const int k = kk[s], ldh = m + 1;
    const double2 *Hs = H + (size_t)s * m * ldh;
    const double2 *gs = g + (size_t)s * (m + 1);
    double2 *ys = y + (size_t)s * ldv;
    for (int i = k - 1; i >= 0; i--) {
        double sr = gs[i].x, si = gs[i].y;
        for (int l = i + 1; l < k; l++) {
            const double2 a = Hs[(size_t)l * ldh + i], b = ys[l];
            sr -= a.x * b.x - a.y * b.y;
            si -= a.x * b.y + a.y * b.x;
        }
        const double2 d = Hs[(size_t)i * ldh + i];
        const double den = d.x * d.x + d.y * d.y;
        ys[i] = den > 0 ? make_double2((sr * d.x + si * d.y) / den, (si * d.x - sr * d.y) / den)
                        : make_double2(0.0, 0.0);
    }
}

__global__ void binit_g_kernel(int S, int m, const double *__restrict__ nrm, double2 *__restrict__ g) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= S) return;
    for (int t = 0; t <= m; t++) g[(size_t)s * (m + 1) + t] = make_double2(t == 0 ? nrm[s] : 0.0, 0.0);
}

inline dim3 grid2(int n, int S) { return dim3((n + 255) / 256, S); }

}  // namespace
}  // namespace bem

using namespace bem;

namespace {
void cublas_ok(cublasStatus_t s, const char *what) {
    if (s != CUBLAS_STATUS_SUCCESS)
        BEM_FAIL(BEM_ERR_CUDA, std::string(what) + " failed (cublas status " + std::to_string((int)s) + ")");
}
}  // namespace

// Tt (R x 2S) = At^T Vt (first) and/or Wt (2N x 2S) = At Tt (second).
static void normal_gemms(bem_solver_s &sv, const float *Vt, float *Tt, float *Wt, int S, bool first, bool second) {
    const float one = 1.f, zero = 0.f;
    const int N = sv.N, R = sv.R;
    const float *At = reinterpret_cast<const float *>(sv.d_A.p);
    const int ldat = (int)(2 * sv.lda);
    const cublasComputeType_t ct = sv.opt.gemm_mode == 0   ? CUBLAS_COMPUTE_32F
                                   : sv.opt.gemm_mode == 2 ? CUBLAS_COMPUTE_32F_FAST_TF32
                                                           : CUBLAS_COMPUTE_32F_EMULATED_16BFX9;
    if (first) {
        BEM_PROF("gemm_AV", sv.stream);
        cublas_ok(cublasGemmEx(sv.cublas, CUBLAS_OP_T, CUBLAS_OP_N, R, 2 * S, 2 * N, &one, At, CUDA_R_32F, ldat, Vt,
                               CUDA_R_32F, 2 * N, &zero, Tt, CUDA_R_32F, R, ct, CUBLAS_GEMM_DEFAULT),
                  "GEMM A V");
    }
    if (second) {
        BEM_PROF("gemm_AhT", sv.stream);
        cublas_ok(cublasGemmEx(sv.cublas, CUBLAS_OP_N, CUBLAS_OP_N, 2 * N, 2 * S, R, &one, At, CUDA_R_32F, ldat, Tt,
                               CUDA_R_32F, R, &zero, Wt, CUDA_R_32F, 2 * N, ct, CUBLAS_GEMM_DEFAULT),
                  "GEMM A^H T");
    }
}

void bem_solver_s::solve_block(bem_solve_info_t *info) {
    const int n = N, m = std::max(1, std::min(opt.max_iter, 200));
    const int ldv = m + 1;
    const size_t NS = (size_t)n * S;
    w_V.ensure(sizeof(double2) * NS * (m + 1));
    w_H.ensure(sizeof(double2) * (size_t)S * m * (m + 1));
    w_cs.ensure(sizeof(double2) * (size_t)S * m);
    w_sn.ensure(sizeof(double2) * (size_t)S * m);
    w_g.ensure(sizeof(double2) * (size_t)S * (m + 1));
    w_y.ensure(sizeof(double2) * (size_t)S * ldv);
    w_h1.ensure(sizeof(double2) * (size_t)S * ldv);
    w_h2.ensure(sizeof(double2) * (size_t)S * ldv);
    w_w.ensure(sizeof(double2) * NS);                    // W and the gradient G
    w_r.ensure(sizeof(double2) * (size_t)R * S);         // residual R
    w_gv.ensure(sizeof(double2) * NS);                   // A^H B (norms)
    w_vf.ensure(sizeof(float) * 4 * NS);                 // Vt (2N x 2S)
    w_t.ensure(sizeof(float) * 2 * (size_t)R * S);       // Tt (R x 2S)
    w_part.ensure(sizeof(float) * 4 * NS);               // Wt (2N x 2S)
    w_scal.ensure(sizeof(double) * 4 * (size_t)S + sizeof(int) * S);
    double *nrm_b = w_scal.as<double>(), *nrm_g = nrm_b + S, *nrm_w = nrm_b + 2 * S, *res = nrm_b + 3 * S;
    int *kk = reinterpret_cast<int *>(nrm_b + 4 * S);
    double2 *V = w_V.as<double2>(), *W = w_w.as<double2>(), *X = d_x.as<double2>();
    float *Vt = w_vf.as<float>(), *Tt = w_t.as<float>(), *Wt = w_part.as<float>();
    std::vector<double> h_bn(S), h_gn(S), h_res(S);
    std::vector<int> h_kk(S);
    auto rd = [&](const double *d, std::vector<double> &h) {
        CUDA_TRY(cudaMemcpyAsync(h.data(), d, sizeof(double) * S, cudaMemcpyDeviceToHost, stream));
        CUDA_TRY(cudaStreamSynchronize(stream));
    };
    const int nb = (n + 255) / 256, sb = (S + 127) / 128;
    // ||A^H b_s||: X = 0 so the residual is B
    launch_zero_f64(NS, X, stream);
    int total_it = 0, refs = 0;
    double worst = 0.0;
    bool conv = false;
    for (;; refs++) {
        // R = B - A X ; G = A^H R
        build_vt_kernel<<<grid2(n, S), 256, 0, stream>>>(n, S, X, Vt);
        normal_gemms(*this, Vt, Tt, Wt, S, true, false);
        resid_from_t_kernel<<<grid2(R, S), 256, 0, stream>>>(R, S, Tt, d_B.as<double2>(), w_r.as<double2>(), Tt);
        normal_gemms(*this, Vt, Tt, Wt, S, false, true);
        combine_w_kernel<<<grid2(n, S), 256, 0, stream>>>(n, S, Wt, W);
        bnrm2_kernel<<<S, 256, 0, stream>>>(n, W, nrm_g);
        count_launch(5);
        KERNEL_CHECK();
        rd(nrm_g, h_gn);
        if (refs == 0) h_bn = h_gn;
        worst = 0.0;
        for (int s = 0; s < S; s++) worst = std::max(worst, h_bn[s] > 0 ? h_gn[s] / h_bn[s] : 0.0);
        if (worst <= opt.block_tol) { conv = true; break; }
        if (refs >= opt.max_refine) break;
        // inner batched GMRES on A^H A D = G, D accumulated into X
        bscale_kernel<<<grid2(n, S), 256, 0, stream>>>(n, W, nrm_g, V);
        binit_g_kernel<<<sb, 128, 0, stream>>>(S, m, nrm_g, w_g.as<double2>());
        count_launch(2);
        std::fill(h_kk.begin(), h_kk.end(), 0);
        int j = 0;
        for (; j < m; j++) {
            double2 *Vj = V + (size_t)j * NS;
            build_vt_kernel<<<grid2(n, S), 256, 0, stream>>>(n, S, Vj, Vt);
            count_launch();
            normal_gemms(*this, Vt, Tt, Wt, S, true, true);
            combine_w_kernel<<<grid2(n, S), 256, 0, stream>>>(n, S, Wt, W);
            bdots_kernel<<<dim3(j + 1, S), 256, 0, stream>>>(n, S, V, W, w_h1.as<double2>(), ldv);
            bcombo_kernel<<<grid2(n, S), 256, 0, stream>>>(n, S, j + 1, nullptr, V, w_h1.as<double2>(), ldv, W, -1.0);
            bdots_kernel<<<dim3(j + 1, S), 256, 0, stream>>>(n, S, V, W, w_h2.as<double2>(), ldv);
            bcombo_kernel<<<grid2(n, S), 256, 0, stream>>>(n, S, j + 1, nullptr, V, w_h2.as<double2>(), ldv, W, -1.0);
            bnrm2_kernel<<<S, 256, 0, stream>>>(n, W, nrm_w);
            bscale_kernel<<<grid2(n, S), 256, 0, stream>>>(n, W, nrm_w, V + (size_t)(j + 1) * NS);
            bhess_givens_kernel<<<sb, 128, 0, stream>>>(j, S, m, w_h1.as<double2>(), w_h2.as<double2>(), ldv, nrm_w,
                                                        w_H.as<double2>(), w_cs.as<double2>(), w_sn.as<double2>(),
                                                        w_g.as<double2>(), res);
            count_launch(9);
            KERNEL_CHECK();
            rd(res, h_res);
            bool all = true;
            for (int s = 0; s < S; s++) {
                if (h_kk[s] == 0 && !(h_gn[s] > 0 && h_res[s] / h_gn[s] > opt.inner_tol)) h_kk[s] = j + 1;
                all &= h_kk[s] > 0;
            }
            if (all) { j++; break; }
        }
        for (int s = 0; s < S; s++)
            if (h_kk[s] == 0) h_kk[s] = j;
        total_it += j;
        CUDA_TRY(cudaMemcpyAsync(kk, h_kk.data(), sizeof(int) * S, cudaMemcpyHostToDevice, stream));
        btrisolve_kernel<<<sb, 128, 0, stream>>>(S, m, kk, w_H.as<double2>(), w_g.as<double2>(), w_y.as<double2>(), ldv);
        bcombo_kernel<<<grid2(n, S), 256, 0, stream>>>(n, S, j, kk, V, w_y.as<double2>(), ldv, X, 1.0);
        count_launch(2);
        KERNEL_CHECK();
    }
    CUDA_TRY(cudaStreamSynchronize(stream));
    (void)nb;
    if (info) {
        info->iterations = total_it;
        info->refinements = refs;
        info->rel_residual = worst;
        info->converged = conv ? 1 : 0;
    }
}
