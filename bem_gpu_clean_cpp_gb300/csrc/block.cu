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
// TF32.  The TF32x3 products run either on that interleaved form or, by
// option, in the 3M form: separate real planes of Re A, Im A and Re A + Im A,
// three real products per complex product instead of four.
//
// Precision.  Each right-hand side keeps its own Krylov space.  The inner
// solve only has to reduce the correction equation's residual by inner_tol,
// so its basis is stored and orthogonalised in FP32 (classical Gram-Schmidt
// twice); the Hessenberg matrix, Givens rotations, back substitution and the
// solution X are FP64.  Accuracy comes from the outer refinement: the
// residual R = B - A X, where all the cancellation happens, is kept in FP64.
// After the first inner cycle it is computed FP64-accurately from X with
// double-float arithmetic on the FP32 pipe (8 sources per pass over A); after
// every later cycle it is updated with that cycle's correction D, R -= A D,
// by the first GEMM (|A D| has already shrunk by inner_tol, so the GEMM's
// FP32-level error stays below the FP64 level of R).  G = A^H R cancels
// strongly (R, the least-squares residual, does not vanish), so it runs
// FP32-accurate (split-BF16 or FP32) in every mode.  On GB300 the FP64 pipe runs at
// about 1/64 of FP32, so FP64 Arnoldi over 256 Krylov spaces would cost more
// than the GEMMs themselves.
#include <cublas_v2.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "dfloat.h"
#include "solver.h"
#include "tc_gemm.h"

namespace bem {
namespace {

constexpr int kResSB = 8;        // right-hand sides per pass of the residual kernel
constexpr int kResRPW = 2;       // rows per warp of the residual kernel
constexpr int kResWarps = 8;     // warps per CTA of the residual kernel
constexpr int kDotLB = 8;        // basis vectors per CTA of the dot kernel

template <typename T>
__device__ __forceinline__ double2 ld_c(const T *p, size_t i);
template <>
__device__ __forceinline__ double2 ld_c<double2>(const double2 *p, size_t i) { return p[i]; }
template <>
__device__ __forceinline__ double2 ld_c<float2>(const float2 *p, size_t i) {
    const float2 v = p[i];
    return make_double2(v.x, v.y);
}

// TF32 head of a float: round to the nearest value with 10 stored mantissa
// bits (ties away from zero); v - head(v) is exact in FP32.
__device__ __forceinline__ float tf32_head(float v) {
    return __uint_as_float((__float_as_uint(v) + 0x1000u) & 0xFFFFE000u);
}

// Vt (2N x 2S) from the N x S complex block V (column-major, ld = N); with
// Vlo, Vt gets the TF32 heads and Vlo the tails.
template <typename T>
__global__ void build_vt_kernel(int N, int S, const T *__restrict__ V, float *__restrict__ Vt,
                                float *__restrict__ Vlo) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, s = blockIdx.y;
    if (i >= N) return;
    const double2 v = ld_c(V, (size_t)s * N + i);
    const size_t ld = 2 * (size_t)N;
    const size_t o[4] = {(size_t)s * ld + 2 * i, (size_t)(S + s) * ld + 2 * i, (size_t)s * ld + 2 * i + 1,
                         (size_t)(S + s) * ld + 2 * i + 1};
    const float val[4] = {(float)v.x, (float)v.y, -(float)v.y, (float)v.x};
#pragma unroll
    for (int q = 0; q < 4; q++) {
        if (Vlo) {
            const float h = tf32_head(val[q]);
            Vt[o[q]] = h;
            Vlo[o[q]] = val[q] - h;
        } else {
            Vt[o[q]] = val[q];
        }
    }
}

// hi/lo TF32 planes of the interleaved-real view of A (R rows of N2 = 2N
// floats, row stride ld floats).
__global__ void split_a_tf32_kernel(int R, int N2, size_t ld, const float *__restrict__ A, float *__restrict__ hi,
                                    float *__restrict__ lo) {
    const size_t total = (size_t)R * N2;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
        const size_t i = (t / N2) * ld + t % N2;
        const float v = A[i], h = tf32_head(v);
        hi[i] = h;
        lo[i] = v - h;
    }
}

// Rv = B (the residual of X = 0) and its float packing Tt (R x 2S, real and
// imaginary column blocks).
__global__ void pack_b_kernel(int R, int S, const double2 *__restrict__ B, double2 *__restrict__ Rv,
                              float *__restrict__ Tt) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x, s = blockIdx.y;
    if (r >= R) return;
    const double2 b = B[(size_t)s * R + r];
    Rv[(size_t)s * R + r] = b;
    Tt[(size_t)s * R + r] = (float)b.x;
    Tt[(size_t)(S + s) * R + r] = (float)b.y;
}

// Residual update Rv -= A D with A D given packed in Tt (from the first
// GEMM), then Tt = float(Rv) for the A^H R GEMM.  Each thread reads and
// writes only its own elements of Tt.
__global__ void resid_update_kernel(int R, int S, double2 *__restrict__ Rv, float *Tt) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x, s = blockIdx.y;
    if (r >= R) return;
    const size_t ir = (size_t)s * R + r, ii = (size_t)(S + s) * R + r;
    const double2 v = Rv[ir];
    const double2 u = make_double2(v.x - (double)Tt[ir], v.y - (double)Tt[ii]);
    Rv[ir] = u;
    Tt[ir] = (float)u.x;
    Tt[ii] = (float)u.y;
}

// Head/tail float split of X (N x S, ld N) into xh/xl (ld ldx, even).
__global__ void split_x_kernel(int N, int ldx, const double2 *__restrict__ X, float2 *__restrict__ xh,
                               float2 *__restrict__ xl) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, s = blockIdx.y;
    if (i >= N) return;
    const double2 v = X[(size_t)s * N + i];
    const float hr = (float)v.x, hi = (float)v.y;
    xh[(size_t)s * ldx + i] = make_float2(hr, hi);
    xl[(size_t)s * ldx + i] = make_float2((float)(v.x - (double)hr), (float)(v.y - (double)hi));
}

// R(:, s) = B(:, s) - A X(:, s) for kResSB consecutive sources, FP64-accurate
// (double-float on the FP32 pipe), written packed as floats into Tt for the
// A^H R GEMM.  A warp owns kResRPW rows; lanes stride over column pairs
// (float4 of A).  Each head/tail load of X serves kResRPW rows, and the
// sources' blocks (N x kResSB) are shared by the CTA's warps through L1; A is
// read once per kResSB sources.
__global__ void __launch_bounds__(32 * kResWarps)
resid_df_multi_kernel(int R, int N, int S, const float2 *__restrict__ A, size_t lda,
                      const float2 *__restrict__ xh, const float2 *__restrict__ xl, int ldx,
                      const double2 *__restrict__ B, double2 *__restrict__ Rv, float *__restrict__ Tt) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int row0 = (blockIdx.x * kResWarps + warp) * kResRPW;
    const int s0 = blockIdx.y * kResSB;
    if (row0 >= R) return;
    const int ns = min(kResSB, S - s0), nr = min(kResRPW, R - row0);
    float rh[kResRPW][kResSB], rl[kResRPW][kResSB], ih[kResRPW][kResSB], il[kResRPW][kResSB];
#pragma unroll
    for (int p = 0; p < kResRPW; p++)
#pragma unroll
        for (int q = 0; q < kResSB; q++) rh[p][q] = rl[p][q] = ih[p][q] = il[p][q] = 0.f;
    const float4 *a4[kResRPW];
#pragma unroll
    for (int p = 0; p < kResRPW; p++)
        a4[p] = reinterpret_cast<const float4 *>(A + (size_t)(row0 + min(p, nr - 1)) * lda);
    const float4 *xh4 = reinterpret_cast<const float4 *>(xh), *xl4 = reinterpret_cast<const float4 *>(xl);
    const int N2 = N >> 1;
    for (int j2 = lane; j2 < N2; j2 += 32) {
        float4 v[kResRPW];
#pragma unroll
        for (int p = 0; p < kResRPW; p++) v[p] = __ldcs(a4[p] + j2);
#pragma unroll
        for (int q = 0; q < kResSB; q++) {
            if (q < ns) {
                const size_t o = (size_t)(s0 + q) * (ldx / 2) + j2;
                const float4 h = xh4[o], l = xl4[o];
#pragma unroll
                for (int p = 0; p < kResRPW; p++) {
                    df_mac(rh[p][q], rl[p][q], v[p].x, h.x, l.x);
                    df_mac(rh[p][q], rl[p][q], -v[p].y, h.y, l.y);
                    df_mac(ih[p][q], il[p][q], v[p].x, h.y, l.y);
                    df_mac(ih[p][q], il[p][q], v[p].y, h.x, l.x);
                    df_mac(rh[p][q], rl[p][q], v[p].z, h.z, l.z);
                    df_mac(rh[p][q], rl[p][q], -v[p].w, h.w, l.w);
                    df_mac(ih[p][q], il[p][q], v[p].z, h.w, l.w);
                    df_mac(ih[p][q], il[p][q], v[p].w, h.z, l.z);
                }
            }
        }
    }
    if ((N & 1) && lane == 0) {
#pragma unroll
        for (int p = 0; p < kResRPW; p++) {
            const float2 v = reinterpret_cast<const float2 *>(a4[p])[N - 1];
#pragma unroll
            for (int q = 0; q < kResSB; q++) {
                if (q < ns) {
                    const float2 h = xh[(size_t)(s0 + q) * ldx + N - 1], l = xl[(size_t)(s0 + q) * ldx + N - 1];
                    df_mac(rh[p][q], rl[p][q], v.x, h.x, l.x);
                    df_mac(rh[p][q], rl[p][q], -v.y, h.y, l.y);
                    df_mac(ih[p][q], il[p][q], v.x, h.y, l.y);
                    df_mac(ih[p][q], il[p][q], v.y, h.x, l.x);
                }
            }
        }
    }
#pragma unroll
    for (int p = 0; p < kResRPW; p++) {
#pragma unroll
        for (int q = 0; q < kResSB; q++) {
            double sr = (double)rh[p][q] + (double)rl[p][q], si = (double)ih[p][q] + (double)il[p][q];
            for (int o = 16; o > 0; o >>= 1) {
                sr += __shfl_xor_sync(0xffffffffu, sr, o);
                si += __shfl_xor_sync(0xffffffffu, si, o);
            }
            if (lane == 0 && q < ns && p < nr) {
                const int s = s0 + q, row = row0 + p;
                const double2 b = B[(size_t)s * R + row];
                const double2 r = make_double2(b.x - sr, b.y - si);
                Rv[(size_t)s * R + row] = r;
                Tt[(size_t)s * R + row] = (float)r.x;
                Tt[(size_t)(S + s) * R + row] = (float)r.y;
            }
        }
    }
}

// W (N x S complex, float) from Wt (2N x 2S), or from Wt + Wb (TF32x3: the
// head product and the two tail products, each 2N x 2S).
__global__ void combine_w_kernel(int N, int S, const float *__restrict__ Wt, const float *__restrict__ Wb,
                                 float2 *__restrict__ W) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x, s = blockIdx.y;
    if (j >= N) return;
    const size_t ld = 2 * (size_t)N;
    const size_t oa = (size_t)s * ld + 2 * j, ob = (size_t)(S + s) * ld + 2 * j + 1;
    const size_t oc = (size_t)(S + s) * ld + 2 * j, od = (size_t)s * ld + 2 * j + 1;
    float a = Wt[oa], b = Wt[ob], c = Wt[oc], d = Wt[od];
    if (Wb) {
        a += Wb[oa];
        b += Wb[ob];
        c += Wb[oc];
        d += Wb[od];
    }
    W[(size_t)s * N + j] = make_float2(a + b, c - d);
}

// out[i] = pair[i] + pair[n + i] (the two halves of a TF32x3 product pair).
__global__ void add_halves_kernel(size_t n, const float *__restrict__ pair, float *__restrict__ out) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        out[i] = pair[i] + pair[n + i];
}

// pair = [head(x) | tail(x)] (TF32 head, exact tail), n floats each.
__global__ void split_pair_kernel(size_t n, const float *__restrict__ x, float *__restrict__ pair) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float v = x[i], h = tf32_head(v);
        pair[i] = h;
        pair[n + i] = v - h;
    }
}

// h[s*ldv + l] = V_l(:,s)^H W(:,s) for l in [l0, l0 + kDotLB) ∩ [0, nl).
// Basis block l is N x S, column-major, at V + l*N*S.  Per-thread FP32
// partial sums (N/256 terms), FP64 across threads.
__global__ void __launch_bounds__(256)
bdots_kernel(int N, int S, int nl, const float2 *__restrict__ V, const float2 *__restrict__ W,
             double2 *__restrict__ h, int ldv) {
    const int s = blockIdx.x, l0 = blockIdx.y * kDotLB;
    const int nb = min(kDotLB, nl - l0);
    const size_t NS = (size_t)N * S;
    const float2 *w = W + (size_t)s * N;
    const float2 *v = V + (size_t)l0 * NS + (size_t)s * N;
    float ar[kDotLB], ai[kDotLB];
#pragma unroll
    for (int q = 0; q < kDotLB; q++) ar[q] = ai[q] = 0.f;
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
        const float2 b = w[i];
#pragma unroll
        for (int q = 0; q < kDotLB; q++) {
            if (q < nb) {
                const float2 a = v[(size_t)q * NS + i];
                ar[q] = fmaf(a.x, b.x, fmaf(a.y, b.y, ar[q]));
                ai[q] = fmaf(a.x, b.y, fmaf(-a.y, b.x, ai[q]));
            }
        }
    }
    __shared__ double red[kDotLB][2][8];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < kDotLB; q++) {
        double xr = ar[q], xi = ai[q];
        for (int o = 16; o > 0; o >>= 1) {
            xr += __shfl_xor_sync(0xffffffffu, xr, o);
            xi += __shfl_xor_sync(0xffffffffu, xi, o);
        }
        if (lane == 0) { red[q][0][warp] = xr; red[q][1][warp] = xi; }
    }
    __syncthreads();
    if (threadIdx.x < nb) {
        const int q = threadIdx.x;
        double xr = 0, xi = 0;
        for (int t = 0; t < (int)(blockDim.x >> 5); t++) { xr += red[q][0][t]; xi += red[q][1][t]; }
        h[(size_t)s * ldv + l0 + q] = make_double2(xr, xi);
    }
}

// W(:,s) -= sum_{l<k} V_l(:,s) h[s][l]   (FP32 basis and W).
__global__ void __launch_bounds__(256)
bcombo_kernel(int N, int S, int k, const float2 *__restrict__ V, const double2 *__restrict__ h, int ldv,
              float2 *__restrict__ W) {
    __shared__ float2 hs[256];
    const int i = blockIdx.x * blockDim.x + threadIdx.x, s = blockIdx.y;
    for (int t = threadIdx.x; t < k && t < 256; t += blockDim.x) {
        const double2 c = h[(size_t)s * ldv + t];
        hs[t] = make_float2((float)c.x, (float)c.y);
    }
    __syncthreads();
    if (i >= N) return;
    const size_t NS = (size_t)N * S;
    float sr = 0, si = 0;
    for (int l = 0; l < k; l++) {
        const float2 a = V[(size_t)l * NS + (size_t)s * N + i], c = hs[l];
        sr = fmaf(a.x, c.x, fmaf(-a.y, c.y, sr));
        si = fmaf(a.x, c.y, fmaf(a.y, c.x, si));
    }
    const float2 w = W[(size_t)s * N + i];
    W[(size_t)s * N + i] = make_float2(w.x - sr, w.y - si);
}

// D(:,s) = sum_{l<kk[s]} V_l(:,s) y[s][l] (FP64 accumulation); X += D.
__global__ void __launch_bounds__(256)
bupdate_x_kernel(int N, int S, const int *__restrict__ kk, const float2 *__restrict__ V,
                 const double2 *__restrict__ y, int ldv, double2 *__restrict__ X, double2 *__restrict__ D) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, s = blockIdx.y;
    if (i >= N) return;
    const int k = kk[s];
    const size_t NS = (size_t)N * S;
    double sr = 0, si = 0;
    for (int l = 0; l < k; l++) {
        const float2 a = V[(size_t)l * NS + (size_t)s * N + i];
        const double2 c = y[(size_t)s * ldv + l];
        sr += (double)a.x * c.x - (double)a.y * c.y;
        si += (double)a.x * c.y + (double)a.y * c.x;
    }
    const double2 x = X[(size_t)s * N + i];
    X[(size_t)s * N + i] = make_double2(x.x + sr, x.y + si);
    D[(size_t)s * N + i] = make_double2(sr, si);
}

__global__ void __launch_bounds__(256) bnrm2_kernel(int N, const float2 *__restrict__ W, double *__restrict__ out) {
    const int s = blockIdx.x;
    const float2 *w = W + (size_t)s * N;
    float a = 0.f;
    for (int i = threadIdx.x; i < N; i += blockDim.x) a = fmaf(w[i].x, w[i].x, fmaf(w[i].y, w[i].y, a));
    double d = a;
    __shared__ double red[8];
    for (int o = 16; o > 0; o >>= 1) d += __shfl_xor_sync(0xffffffffu, d, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = d;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0;
        for (int q = 0; q < (int)(blockDim.x >> 5); q++) t += red[q];
        out[s] = sqrt(t);
    }
}

__global__ void bscale_kernel(int N, const float2 *__restrict__ W, const double *__restrict__ nrm,
                              float2 *__restrict__ Vn) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, s = blockIdx.y;
    if (i >= N) return;
    const double n = nrm[s];
    const float inv = n > 0 ? (float)(1.0 / n) : 0.f;
    const float2 w = W[(size_t)s * N + i];
    Vn[(size_t)s * N + i] = make_float2(w.x * inv, w.y * inv);
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

// ---- 3M form of the TF32x3 products (BEM_GEMM_TF32X3_3M) ----
// A = Ar + i Ai, As = Ar + Ai.  T = A V:  P1 = Ar Vr, P2 = Ai Vi,
// P3 = As (Vr + Vi);  Tr = P1 - P2, Ti = P3 - P1 - P2.  W = A^H T:
// Q1 = Ar^T Tr, Q2 = Ai^T Ti, Q3 = As^T (Tr - Ti);  Wr = Q1 + Q2,
// Wi = Q1 - Q2 - Q3.  Every real operand is kept as TF32 head and tail
// planes; a real product is two GEMMs, head(A) [head(B) | tail(B)] (one pass
// over the head plane of A for both terms) and tail(A) head(B), whose output
// lands on the second block.

// A's planes, each R x N real (row-major, ld = lda): [r_hi, r_lo, i_hi, i_lo, s_hi, s_lo]
__global__ void split_a3_kernel(int R, int N, size_t lda, const float2 *__restrict__ A, float *__restrict__ P) {
    const size_t plane = (size_t)R * lda, total = (size_t)R * N;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
        const size_t i = (t / N) * lda + t % N;
        const float2 a = A[i];
        const float v[3] = {a.x, a.y, a.x + a.y};
#pragma unroll
        for (int q = 0; q < 3; q++) {
            const float h = tf32_head(v[q]);
            P[(2 * q) * plane + i] = h;
            P[(2 * q + 1) * plane + i] = v[q] - h;
        }
    }
}

// Planes of a complex block (n x S): for q = r, i, s the head then the tail
// (each n x S, ld n), so [head | tail] of q is one n x 2S matrix (plane =
// 2 n S floats apart).  The complex
// value is X[s n + i] (ld_c) or, from the packed float form Tt (n x 2S: real
// block, imaginary block), (Tt[s n + i], Tt[(S + s) n + i]).  s = r + i, or
// r - i with sub.
__device__ __forceinline__ void put_planes3(float *__restrict__ P, size_t plane, size_t o, float r, float im,
                                           bool sub) {
    const float v[3] = {r, im, sub ? r - im : r + im};
#pragma unroll
    for (int q = 0; q < 3; q++) {
        const float h = tf32_head(v[q]);
        P[(size_t)q * plane + o] = h;
        P[(size_t)q * plane + plane / 2 + o] = v[q] - h;
    }
}

template <typename T>
__global__ void split_x3_kernel(int n, int S, const T *__restrict__ X, float *__restrict__ P) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, s = blockIdx.y;
    if (i >= n) return;
    const size_t o = (size_t)s * n + i;
    const double2 x = ld_c(X, o);
    put_planes3(P, 2 * (size_t)n * S, o, (float)x.x, (float)x.y, false);
}

__global__ void split_t3_kernel(int n, int S, const float *__restrict__ Tt, float *__restrict__ P) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, s = blockIdx.y;
    if (i >= n) return;
    const size_t o = (size_t)s * n + i;
    put_planes3(P, 2 * (size_t)n * S, o, Tt[o], Tt[(size_t)(S + s) * n + i], true);
}

// C holds the three real products, product q as m x 2S (ld m) at C + 2 q m S,
// its value the sum of the two blocks.
__device__ __forceinline__ float prod3(const float *__restrict__ C, size_t mS, int q, size_t o) {
    const float *c = C + 2 * (size_t)q * mS;
    return c[o] + c[mS + o];
}

// Tt (R x 2S) = (P1 - P2 | P3 - P1 - P2).
__global__ void combine_t3_kernel(int R, int S, const float *__restrict__ C, float *__restrict__ Tt) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x, s = blockIdx.y;
    if (r >= R) return;
    const size_t o = (size_t)s * R + r, mS = (size_t)R * S;
    const float p1 = prod3(C, mS, 0, o), p2 = prod3(C, mS, 1, o), p3 = prod3(C, mS, 2, o);
    Tt[o] = p1 - p2;
    Tt[mS + o] = p3 - p1 - p2;
}

// W (n x S complex) = (Q1 + Q2, Q1 - Q2 - Q3).
__global__ void combine_w3_kernel(int n, int S, const float *__restrict__ C, float2 *__restrict__ W) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x, s = blockIdx.y;
    if (j >= n) return;
    const size_t o = (size_t)s * n + j, mS = (size_t)n * S;
    const float q1 = prod3(C, mS, 0, o), q2 = prod3(C, mS, 1, o), q3 = prod3(C, mS, 2, o);
    W[o] = make_float2(q1 + q2, q1 - q2 - q3);
}

}  // namespace

namespace {
std::mutex g_block_mode_mu;
std::map<std::tuple<int, int, int, int>, int> g_block_mode;   // (device, R, N, S) -> BEM_GEMM_*
}  // namespace

int block_mode_cached(int device, int R, int N, int S) {
    std::lock_guard<std::mutex> lk(g_block_mode_mu);
    const auto it = g_block_mode.find(std::make_tuple(device, R, N, S));
    return it == g_block_mode.end() ? -1 : it->second;
}

void block_mode_store(int device, int R, int N, int S, int mode) {
    std::lock_guard<std::mutex> lk(g_block_mode_mu);
    g_block_mode[std::make_tuple(device, R, N, S)] = mode;
}

}  // namespace bem

using namespace bem;

namespace {
void cublas_ok(cublasStatus_t s, const char *what) {
    if (s != CUBLAS_STATUS_SUCCESS)
        BEM_FAIL(BEM_ERR_CUDA, std::string(what) + " failed (cublas status " + std::to_string((int)s) + ")");
}
}  // namespace

// Tt (R x 2S) = At^T Vt (first) and/or Wt (2N x 2S) = At Tt (second).  In
// TF32x3 mode Vt holds the heads and Vlo = Vt + 4NS the tails of the
// right-hand block, Tlo is scratch for the product pair (R x 4S), Wt holds
// the pair [Wa | Wb] (2N x 4S) that combine_w adds; each product is
// head(A) [head(B) | tail(B)] (one pass over the head plane of A for two of
// the three terms) plus tail(A) head(B) onto the second half.
static void normal_gemms(bem_solver_s &sv, int mode, const float *Vt, const float *Vlo, float *Tt, float *Tlo,
                         float *Wt, int S, bool first, bool second) {
    const float one = 1.f, zero = 0.f;
    const int N = sv.N, R = sv.R;
    const float *At = reinterpret_cast<const float *>(sv.d_A.p);
    const int ldat = (int)(2 * sv.lda);
    const bool x3 = mode == BEM_GEMM_TF32X3;
    const cublasComputeType_t ct = mode == BEM_GEMM_FP32         ? CUBLAS_COMPUTE_32F
                                   : mode == BEM_GEMM_SPLIT_BF16 ? CUBLAS_COMPUTE_32F_EMULATED_16BFX9
                                                                 : CUBLAS_COMPUTE_32F_FAST_TF32;
    const float *Ahi = x3 ? sv.x_Ahi.as<float>() : At, *Alo = x3 ? sv.x_Alo.as<float>() : nullptr;
    auto gemm1 = [&](const float *a, const float *b, const float *beta) {
        cublas_ok(cublasGemmEx(sv.cublas, CUBLAS_OP_T, CUBLAS_OP_N, R, 2 * S, 2 * N, &one, a, CUDA_R_32F, ldat, b,
                               CUDA_R_32F, 2 * N, beta, Tt, CUDA_R_32F, R, ct, CUBLAS_GEMM_DEFAULT),
                  "GEMM A V");
    };
    auto gemm2 = [&](const float *a, const float *b, const float *beta) {
        cublas_ok(cublasGemmEx(sv.cublas, CUBLAS_OP_N, CUBLAS_OP_N, 2 * N, 2 * S, R, &one, a, CUDA_R_32F, ldat, b,
                               CUDA_R_32F, R, beta, Wt, CUDA_R_32F, 2 * N, ct, CUBLAS_GEMM_DEFAULT),
                  "GEMM A^H T");
    };
    // C = [Ahi B | Ahi Blo + Alo B] for B = [B | Blo] (k x 4S, ld ldb; each
    // half k x 2S): one pass over the head plane for both terms, then the
    // tail plane's product added onto the second half
    auto gemm_pair = [&](cublasOperation_t op, int m, int k, const float *Ahi, const float *Alo, int lda_,
                         const float *B, int ldb, float *C, int ldc) {
        cublas_ok(cublasGemmEx(sv.cublas, op, CUBLAS_OP_N, m, 4 * S, k, &one, Ahi, CUDA_R_32F, lda_, B, CUDA_R_32F,
                               ldb, &zero, C, CUDA_R_32F, ldc, ct, CUBLAS_GEMM_DEFAULT),
                  "GEMM (TF32x3, head)");
        cublas_ok(cublasGemmEx(sv.cublas, op, CUBLAS_OP_N, m, 2 * S, k, &one, Alo, CUDA_R_32F, lda_, B, CUDA_R_32F,
                               ldb, &one, C + (size_t)ldc * 2 * S, CUDA_R_32F, ldc, ct, CUBLAS_GEMM_DEFAULT),
                  "GEMM (TF32x3, tail)");
    };
    if (first) {
        BEM_PROF("gemm_AV", sv.stream);
        if (x3) {
            // Vlo = Vt + 4NS (the block [Vt | Vlo] is 2N x 4S), Tlo = the pair
            // [Ta | Tb] (R x 4S): Ta = Ahi Vt, Tb = Ahi Vlo + Alo Vt, Tt = Ta + Tb
            gemm_pair(CUBLAS_OP_T, R, 2 * N, Ahi, Alo, ldat, Vt, 2 * N, Tlo, R);
            add_halves_kernel<<<(unsigned)std::min<size_t>((2 * (size_t)R * S + 255) / 256, 4096), 256, 0,
                                sv.stream>>>(2 * (size_t)R * S, Tlo, Tt);
            count_launch();
        } else {
            gemm1(At, Vt, &zero);
        }
    }
    if (second) {
        BEM_PROF("gemm_AhT", sv.stream);
        if (x3) {
            // Tlo = [head(Tt) | tail(Tt)] (R x 4S); Wt = [Wa | Wb] (2N x 4S):
            // Wa = Ahi head, Wb = Ahi tail + Alo head (combine_w adds them)
            const size_t n = 2 * (size_t)R * S;
            split_pair_kernel<<<(unsigned)std::min<size_t>((n + 255) / 256, 4096), 256, 0, sv.stream>>>(n, Tt, Tlo);
            count_launch();
            gemm_pair(CUBLAS_OP_N, 2 * N, R, Ahi, Alo, ldat, Tlo, R, Wt, 2 * N);
        } else {
            gemm2(At, Tt, &zero);
        }
    }
}

// C (m x 2S, ld m) for one real product of the 3M form: [Ahi Bhi | Ahi Blo +
// Alo Bhi], op(A) m x k from the planes Ahi, Alo (ld lda), B = [Bhi | Blo]
// (k x 2S, ld k).
static void tf32x3_real(bem_solver_s &sv, cublasOperation_t opA, int m, int k, const float *Ahi, const float *Alo,
                        const float *B, float *C) {
    const float one = 1.f, zero = 0.f;
    const int S = sv.S, lda = (int)sv.lda;
    cublas_ok(cublasGemmEx(sv.cublas, opA, CUBLAS_OP_N, m, 2 * S, k, &one, Ahi, CUDA_R_32F, lda, B, CUDA_R_32F, k,
                           &zero, C, CUDA_R_32F, m, CUBLAS_COMPUTE_32F_FAST_TF32, CUBLAS_GEMM_DEFAULT),
              "GEMM (3M, head)");
    cublas_ok(cublasGemmEx(sv.cublas, opA, CUBLAS_OP_N, m, S, k, &one, Alo, CUDA_R_32F, lda, B, CUDA_R_32F, k, &one,
                           C + (size_t)m * S, CUDA_R_32F, m, CUBLAS_COMPUTE_32F_FAST_TF32, CUBLAS_GEMM_DEFAULT),
              "GEMM (3M, tail)");
}

// Tt (R x 2S) = A X for the complex block X (N x S) in the 3M form.  Ap: A's
// six planes; Bp: scratch for six N x S planes; C: scratch 6 R x S.
template <typename T>
static void apply_a_3m(bem_solver_s &sv, const T *X, const float *Ap, float *Bp, float *C, float *Tt) {
    const int N = sv.N, R = sv.R, S = sv.S;
    const size_t ap = (size_t)R * sv.lda, bp = 2 * (size_t)N * S, cp = 2 * (size_t)R * S;
    BEM_PROF("gemm_AV", sv.stream);
    split_x3_kernel<T><<<grid2(N, S), 256, 0, sv.stream>>>(N, S, X, Bp);
    count_launch();
    for (int q = 0; q < 3; q++)
        tf32x3_real(sv, CUBLAS_OP_T, R, N, Ap + 2 * q * ap, Ap + (2 * q + 1) * ap, Bp + q * bp, C + q * cp);
    combine_t3_kernel<<<grid2(R, S), 256, 0, sv.stream>>>(R, S, C, Tt);
    count_launch();
}

// W (N x S complex) = A^H T for T given as Tt (R x 2S), in the 3M form.  Bp:
// scratch for six R x S planes; C: scratch 6 N x S.
static void apply_ah_3m(bem_solver_s &sv, const float *Tt, const float *Ap, float *Bp, float *C, float2 *W) {
    const int N = sv.N, R = sv.R, S = sv.S;
    const size_t ap = (size_t)R * sv.lda, bp = 2 * (size_t)R * S, cp = 2 * (size_t)N * S;
    BEM_PROF("gemm_AhT", sv.stream);
    split_t3_kernel<<<grid2(R, S), 256, 0, sv.stream>>>(R, S, Tt, Bp);
    count_launch();
    for (int q = 0; q < 3; q++)
        tf32x3_real(sv, CUBLAS_OP_N, N, R, Ap + 2 * q * ap, Ap + (2 * q + 1) * ap, Bp + q * bp, C + q * cp);
    combine_w3_kernel<<<grid2(N, S), 256, 0, sv.stream>>>(N, S, C, W);
    count_launch();
}

void bem_solver_s::solve_block(bem_solve_info_t *info) {
    const int n = N, m = std::max(1, std::min(opt.max_iter, 200));
    const int ldv = m + 1;
    const int ldx = (int)lda;   // even: float4 access to the head/tail split of X
    const size_t NS = (size_t)n * S;
    w_V.ensure(sizeof(float2) * NS * (m + 1));             // FP32 Krylov bases, block l = N x S
    w_H.ensure(sizeof(double2) * (size_t)S * m * (m + 1));
    w_cs.ensure(sizeof(double2) * (size_t)S * m);
    w_sn.ensure(sizeof(double2) * (size_t)S * m);
    w_g.ensure(sizeof(double2) * (size_t)S * (m + 1));
    w_y.ensure(sizeof(double2) * (size_t)S * ldv);
    w_h1.ensure(sizeof(double2) * (size_t)S * ldv);
    w_h2.ensure(sizeof(double2) * (size_t)S * ldv);
    w_w.ensure(sizeof(float2) * NS);                       // W and the gradient G
    w_gv.ensure(sizeof(float2) * 2 * (size_t)ldx * S);     // head/tail split of X
    w_r.ensure(sizeof(double2) * (size_t)R * S);           // residual R (FP64)
    w_d.ensure(sizeof(double2) * NS);                      // correction D of the last cycle
    w_vf.ensure(sizeof(float) * 4 * NS);                   // Vt (2N x 2S)
    w_t.ensure(sizeof(float) * 2 * (size_t)R * S);         // Tt (R x 2S)
    w_part.ensure(sizeof(float) * 4 * NS);                 // Wt (2N x 2S)
    w_scal.ensure(sizeof(double) * 4 * (size_t)S + sizeof(int) * S);
    double *nrm_b = w_scal.as<double>(), *nrm_g = nrm_b + S, *res = nrm_b + 2 * S, *nrm_w = nrm_b + 3 * S;
    int *kk = reinterpret_cast<int *>(nrm_b + 4 * S);
    float2 *V = w_V.as<float2>(), *W = w_w.as<float2>();
    double2 *X = d_x.as<double2>(), *Rv = w_r.as<double2>(), *Dc = w_d.as<double2>();
    float2 *xh = w_gv.as<float2>(), *xl = xh + (size_t)ldx * S;
    float *Vt = w_vf.as<float>(), *Tt = w_t.as<float>(), *Wt = w_part.as<float>();
    const float2 *A = d_A.as<float2>();
    // Product mode and its buffers; setup() may run more than once while the
    // candidates of AUTO are timed (block_gemm_candidates).
    int gmode = -1;
    bool x3 = false, x3m = false, simt = false, tc = false;
    d_status.ensure(4 * sizeof(int));
    int *tc_status = d_status.as<int>() + 1;
    CUDA_TRY(cudaMemsetAsync(tc_status, 0, sizeof(int), stream));
    const float *Af = reinterpret_cast<const float *>(A);
    float *Vlo = nullptr, *Tlo = nullptr, *A3 = nullptr, *B3 = nullptr, *C3 = nullptr, *simt_scratch = nullptr;
    auto setup = [&](int mode) {
        gmode = mode;
        x3 = mode == BEM_GEMM_TF32X3;
        x3m = mode == BEM_GEMM_TF32X3_3M;
        simt = mode == BEM_GEMM_SIMT;
        tc = mode == BEM_GEMM_TC;
        Vt = w_vf.as<float>();
        Wt = w_part.as<float>();
        Vlo = Tlo = A3 = B3 = C3 = simt_scratch = nullptr;
        if (simt) {
            // packed operands and partial sums of the split products
            x_tlo.ensure(sizeof(float) * block_simt_scratch_floats(R, n, S));
            simt_scratch = x_tlo.as<float>();
        } else if (tc) {
            // the packed right-hand operand (up to three fp16 parts of the
            // larger of V's and T's interleaved blocks), split-K partial sums,
            // A's power-of-two scale (once per assembly)
            x_vlo.ensure(tc_operand_bytes(std::max(2 * n, R), 2 * S, 3));
            const size_t pf = std::max({tc_gemm_part_floats(R, 2 * n, 2 * S, 2), tc_gemm_part_floats(R, 2 * n, 2 * S, 3),
                                        tc_gemm_part_floats(2 * n, R, 2 * S, 2), tc_gemm_part_floats(2 * n, R, 2 * S, 3)});
            if (pf) x_tlo.ensure(sizeof(float) * pf);
            if (!tc_scale_valid) {
                tc_scale.ensure(4 * sizeof(float));
                tc_a_scale(Af, 2 * lda, R, 2 * n, tc_scale.as<float>(), stream);
                tc_scale_valid = true;
            }
        } else if (x3) {
            // [Vt | Vlo] (2N x 4S), the product pair [Ta | Tb] or [head | tail]
            // of Tt (R x 4S), and [Wa | Wb] (2N x 4S)
            x_vlo.ensure(sizeof(float) * 8 * NS);
            x_tlo.ensure(sizeof(float) * 4 * (size_t)R * S);
            w_part.ensure(sizeof(float) * 8 * NS);
            Vt = x_vlo.as<float>();
            Vlo = Vt + 4 * NS;
            Tlo = x_tlo.as<float>();
            Wt = w_part.as<float>();
            if (tf32_split_mode != mode) {
                x_Ahi.ensure(sizeof(float) * 2 * lda * (size_t)R);
                x_Alo.ensure(sizeof(float) * 2 * lda * (size_t)R);
                split_a_tf32_kernel<<<device_sm_count() * 16, 256, 0, stream>>>(R, 2 * n, 2 * lda,
                                                                  reinterpret_cast<const float *>(A),
                                                                  x_Ahi.as<float>(), x_Alo.as<float>());
                count_launch();
                KERNEL_CHECK();
                tf32_split_mode = mode;
            }
        } else if (x3m) {
            // A's six planes (built once per assembly), six planes of the
            // right-hand block, the three products (two blocks each)
            x_vlo.ensure(sizeof(float) * 6 * (size_t)std::max(n, R) * S);
            x_tlo.ensure(sizeof(float) * 6 * (size_t)std::max(n, R) * S);
            B3 = x_vlo.as<float>();
            C3 = x_tlo.as<float>();
            if (tf32_split_mode != mode) {
                x_Ahi.ensure(sizeof(float) * 6 * lda * (size_t)R);
                split_a3_kernel<<<device_sm_count() * 16, 256, 0, stream>>>(R, n, lda, A, x_Ahi.as<float>());
                count_launch();
                KERNEL_CHECK();
                tf32_split_mode = mode;
            }
            A3 = x_Ahi.as<float>();
        }
    };
    const std::vector<int> cands = block_gemm_candidates(opt, S, R, n);
    const int tuned = cands.size() > 1 ? bem::block_mode_cached(device, R, n, S) : cands[0];
    setup(tuned >= 0 ? tuned : cands[0]);
    // T = A X into Tt (X: the FP64 correction or an FP32 basis block), and
    // W = A^H T from Tt, in the mode's form
    // R -= A D once per refinement cycle (D: the cycle's FP64 correction):
    // FP32-accurate like the gradient, whatever the inner products use
    // Tensor-core products: Tt = A X (X: N x S complex, packed as the
    // interleaved real block), and W = A^H T from Tt; parts = 2 for the
    // inner products, 3 (FP32-accurate) for the once-per-cycle ones.
    auto tc_av = [&](const void *Xs, bool f64, int parts) {
        BEM_PROF("gemm_AV", stream);
        TcOperand op = tc_operand_view(x_vlo.p, 2 * n, 2 * S, parts);
        if (f64) tc_pack_cplx_f64(static_cast<const double2 *>(Xs), n, S, op, stream);
        else tc_pack_cplx_f32(static_cast<const float2 *>(Xs), n, S, op, stream);
        tc_gemm(Af, 2 * lda, false, R, 2 * n, tc_scale.as<float>(), op, Tt, R, x_tlo.as<float>(),
                x_tlo.bytes / sizeof(float), tc_status, stream);
    };
    auto tc_aht = [&](int parts) {
        BEM_PROF("gemm_AhT", stream);
        TcOperand op = tc_operand_view(x_vlo.p, R, 2 * S, parts);
        tc_pack_real(Tt, R, op, stream);
        tc_gemm(Af, 2 * lda, true, 2 * n, R, tc_scale.as<float>(), op, Wt, 2 * n, x_tlo.as<float>(),
                x_tlo.bytes / sizeof(float), tc_status,
                stream);
        combine_w_kernel<<<grid2(n, S), 256, 0, stream>>>(n, S, Wt, nullptr, W);
        count_launch();
    };
    auto apply_a_d = [&](const double2 *Xs) {
        if (tc) {
            tc_av(Xs, true, 3);
            return;
        }
        if (simt) {
            BEM_PROF("gemm_AV", stream);
            launch_block_av_c128(A, lda, R, n, S, Xs, Tt, simt_scratch, stream);
            return;
        }
        const int gm = gmode == BEM_GEMM_FP32 ? BEM_GEMM_FP32 : BEM_GEMM_SPLIT_BF16;
        build_vt_kernel<double2><<<grid2(n, S), 256, 0, stream>>>(n, S, Xs, Vt, nullptr);
        count_launch();
        normal_gemms(*this, gm, Vt, nullptr, Tt, nullptr, Wt, S, true, false);
    };
    auto apply_a_f = [&](const float2 *Xs) {
        if (tc) {
            tc_av(Xs, false, 2);
            return;
        }
        if (simt) {
            BEM_PROF("gemm_AV", stream);
            launch_block_av(A, lda, R, n, S, Xs, Tt, simt_scratch, stream);
            return;
        }
        if (x3m) {
            apply_a_3m<float2>(*this, Xs, A3, B3, C3, Tt);
            return;
        }
        build_vt_kernel<float2><<<grid2(n, S), 256, 0, stream>>>(n, S, Xs, Vt, Vlo);
        count_launch();
        normal_gemms(*this, gmode, Vt, Vlo, Tt, Tlo, Wt, S, true, false);
    };
    auto apply_ah = [&]() {
        if (tc) {
            tc_aht(2);
            return;
        }
        if (simt) {
            BEM_PROF("gemm_AhT", stream);
            launch_block_aht(A, lda, R, n, S, Tt, W, simt_scratch, stream);
            return;
        }
        if (x3m) {
            apply_ah_3m(*this, Tt, A3, B3, C3, W);
            return;
        }
        normal_gemms(*this, gmode, Vt, Vlo, Tt, Tlo, Wt, S, false, true);
        combine_w_kernel<<<grid2(n, S), 256, 0, stream>>>(n, S, Wt, x3 ? Wt + 4 * NS : nullptr, W);
        count_launch();
    };
    // G = A^H R once per refinement cycle.  R is the least-squares residual,
    // which the CHIEF rows keep from vanishing, so the product cancels
    // strongly and its rounding bounds what the refinement can reach: it runs
    // FP32-accurate (split-BF16 emulation, or plain FP32 in FP32 mode) whatever
    // the inner products use.
    auto apply_ah_grad = [&]() {
        if (tc) {
            tc_aht(3);
            return;
        }
        if (simt) {
            BEM_PROF("gemm_AhT", stream);
            launch_block_aht(A, lda, R, n, S, Tt, W, simt_scratch, stream);
            return;
        }
        const int gm = gmode == BEM_GEMM_FP32 ? BEM_GEMM_FP32 : BEM_GEMM_SPLIT_BF16;
        normal_gemms(*this, gm, Vt, nullptr, Tt, nullptr, Wt, S, false, true);
        combine_w_kernel<<<grid2(n, S), 256, 0, stream>>>(n, S, Wt, nullptr, W);
        count_launch();
    };
    std::vector<double> h_bn(S), h_gn(S), h_res(S);
    std::vector<int> h_kk(S);
    auto rd = [&](const double *d, std::vector<double> &h) {
        CUDA_TRY(cudaMemcpyAsync(h.data(), d, sizeof(double) * S, cudaMemcpyDeviceToHost, stream));
        CUDA_TRY(cudaStreamSynchronize(stream));
    };
    const int sb = (S + 127) / 128;
    launch_zero_f64(NS, X, stream);
    int total_it = 0, refs = 0;
    double worst = 0.0;
    bool conv = false;
    for (;; refs++) {
        // The residual R = B - A X, then G = A^H R.  After the first inner
        // cycle R is formed FP64-accurately (double float) from X; after each
        // later cycle it is updated, R -= A D, with the correction D of that
        // cycle: |A D| is already down by inner_tol per cycle, so the GEMM's
        // FP32-level error in A D stays below the FP64 level of R.
        if (refs == 0) {
            pack_b_kernel<<<grid2(R, S), 256, 0, stream>>>(R, S, d_B.as<double2>(), Rv, Tt);
            count_launch();
        } else if (refs == 1) {
            BEM_PROF("resid_df_multi", stream);
            split_x_kernel<<<grid2(n, S), 256, 0, stream>>>(n, ldx, X, xh, xl);
            resid_df_multi_kernel<<<dim3((R + kResWarps * kResRPW - 1) / (kResWarps * kResRPW),
                                         (S + kResSB - 1) / kResSB),
                                    32 * kResWarps, 0, stream>>>(R, n, S, A, lda, xh, xl, ldx,
                                                                 d_B.as<double2>(), Rv, Tt);
            count_launch(2);
        } else {
            apply_a_d(Dc);
            resid_update_kernel<<<grid2(R, S), 256, 0, stream>>>(R, S, Rv, Tt);
            count_launch();
        }
        apply_ah_grad();
        bnrm2_kernel<<<S, 256, 0, stream>>>(n, W, nrm_g);
        count_launch();
        KERNEL_CHECK();
        rd(nrm_g, h_gn);
        if (refs == 0) h_bn = h_gn;
        worst = 0.0;
        for (int s = 0; s < S; s++) worst = std::max(worst, h_bn[s] > 0 ? h_gn[s] / h_bn[s] : 0.0);
        if (worst <= opt.block_tol) { conv = true; break; }
        if (refs >= opt.max_refine) break;
        // inner GMRES on A^H A D = G for every source, D accumulated into X
        bscale_kernel<<<grid2(n, S), 256, 0, stream>>>(n, W, nrm_g, V);
        binit_g_kernel<<<sb, 128, 0, stream>>>(S, m, nrm_g, w_g.as<double2>());
        count_launch(2);
        if (refs == 0 && tuned < 0) {
            // First solve of this shape with several AUTO candidates: time one
            // product pair A^H (A V) per candidate on the first basis block
            // (after one untimed pair) and keep the fastest for the shape.
            // W and Tt are free here; the products' results are discarded.
            cudaEvent_t e0, e1;
            CUDA_TRY(cudaEventCreate(&e0));
            CUDA_TRY(cudaEventCreate(&e1));
            int best = cands[0];
            float best_ms = 0.f;
            for (const int c : cands) {
                setup(c);
                apply_a_f(V);
                apply_ah();
                CUDA_TRY(cudaEventRecord(e0, stream));
                for (int rep = 0; rep < 2; rep++) {
                    apply_a_f(V);
                    apply_ah();
                }
                CUDA_TRY(cudaEventRecord(e1, stream));
                CUDA_TRY(cudaEventSynchronize(e1));
                float ms = 0.f;
                CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
                if (c == cands[0] || ms < best_ms) {
                    best_ms = ms;
                    best = c;
                }
            }
            CUDA_TRY(cudaEventDestroy(e0));
            CUDA_TRY(cudaEventDestroy(e1));
            bem::block_mode_store(device, R, n, S, best);
            if (best != BEM_GEMM_TF32X3 && best != BEM_GEMM_TF32X3_3M) {
                x_Ahi.release();   // planes built only for the timing
                x_Alo.release();
                tf32_split_mode = -1;
            }
            setup(best);
        }
        std::fill(h_kk.begin(), h_kk.end(), 0);
        int j = 0;
        for (; j < m; j++) {
            const float2 *Vj = V + (size_t)j * NS;
            apply_a_f(Vj);
            apply_ah();
            const dim3 gd(S, (j + 1 + kDotLB - 1) / kDotLB);
            {
                BEM_PROF("block_arnoldi", stream);
                bdots_kernel<<<gd, 256, 0, stream>>>(n, S, j + 1, V, W, w_h1.as<double2>(), ldv);
                bcombo_kernel<<<grid2(n, S), 256, 0, stream>>>(n, S, j + 1, V, w_h1.as<double2>(), ldv, W);
                bdots_kernel<<<gd, 256, 0, stream>>>(n, S, j + 1, V, W, w_h2.as<double2>(), ldv);
                bcombo_kernel<<<grid2(n, S), 256, 0, stream>>>(n, S, j + 1, V, w_h2.as<double2>(), ldv, W);
                bnrm2_kernel<<<S, 256, 0, stream>>>(n, W, nrm_w);
                bscale_kernel<<<grid2(n, S), 256, 0, stream>>>(n, W, nrm_w, V + (size_t)(j + 1) * NS);
                bhess_givens_kernel<<<sb, 128, 0, stream>>>(j, S, m, w_h1.as<double2>(), w_h2.as<double2>(), ldv,
                                                            nrm_w, w_H.as<double2>(), w_cs.as<double2>(),
                                                            w_sn.as<double2>(), w_g.as<double2>(), res);
                count_launch(7);
            }
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
        bupdate_x_kernel<<<grid2(n, S), 256, 0, stream>>>(n, S, kk, V, w_y.as<double2>(), ldv, X, Dc);
        count_launch(2);
        KERNEL_CHECK();
    }
    CUDA_TRY(cudaStreamSynchronize(stream));
    last_block_gemm_mode = gmode;
    int h_status = 0;
    CUDA_TRY(cudaMemcpy(&h_status, tc_status, sizeof(int), cudaMemcpyDeviceToHost));
    if (h_status) BEM_FAIL(BEM_ERR_TIMEOUT, "block solve: a bounded wait of the tensor-core GEMM timed out");
    if (info) {
        info->iterations = total_it;
        info->refinements = refs;
        info->rel_residual = worst;
        info->converged = conv ? 1 : 0;
    }
}
