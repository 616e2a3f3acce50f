// Quadrature kernels of the GB300 BEM engine: element tables, far-field
// assembly (FP32 or FP64), singular / near-singular assembly (FP64) and
// field-point evaluation.  The formulas restate the reference's element
// integrals (mesh.cu:253-672) and assembly (atomicFuncs.cu:69-298); the
// parallel structure is new:
//   * far-field: a CTA owns TR collocation rows x one column tile and loops
//     over the tile's element list; each element's three nodal
//     contributions are summed in a shared-memory row accumulator, and the
//     finished row segment is written to HBM once (no global atomics);
//   * near-field: one warp per row scans the elements, integrates the
//     singular and near pairs in FP64 with the whole warp (points spread over
//     lanes, shuffle reduction), then finalises the diagonal and the RHS.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <mutex>
#include <type_traits>
#include <vector>

#include "bem_common.h"
#include "kernels.h"
#include "tma.h"

namespace bem {

// ---------------------------------------------------------------------------
// Gauss tables in constant memory.
//   c_qf[q]       = (xi1, xi2, w, 0) of the regular Duffy rule in float,
//                   w = 0.25*w_n*w_m*rho (mesh.cu:623-636)
//   c_qd[v][q][.] = (xi1, xi2, w) in double for the map collapsed at vertex
//                   v+1 (v = 2 is the regular rule; rhoThetaToXi_1/2/3,
//                   mesh.cu:1710-1729)
// ---------------------------------------------------------------------------
__constant__ float4 c_qf[kMaxQ];
__constant__ double c_qd[3][kMaxQ][3];
// c_qs[v][q] = (xi1 - v1, xi2 - v2, w) in float for the map collapsed at
// vertex v (reference coordinates (v1, v2)): the offsets from the collapse
// vertex, formed in double (1 - rho minus 1 would cancel in float)
__constant__ float4 c_qs[3][kMaxQ];
__constant__ int c_nq;

namespace {
std::mutex g_quad_mu;
int g_quad_order[64];   // per device, 0 = none
int g_nq_host = 36;
}  // namespace

void gauss_legendre_host(int n, double *x, double *w);

void ensure_quadrature(int order) {
    BEM_CHECK_ARG(order >= 1 && order <= kMaxOrder, "quadrature order must be in [1, 12]");
    int dev = 0;
    CUDA_TRY(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(g_quad_mu);
    if (dev < 64 && g_quad_order[dev] == order) {
        g_nq_host = order * order;
        return;
    }
    double gx[kMaxOrder], gw[kMaxOrder];
    gauss_legendre_host(order, gx, gw);
    int nq = order * order;
    std::vector<float4> qf(nq);
    std::vector<double> qd(3 * kMaxQ * 3, 0.0);
    std::vector<float4> qs(3 * kMaxQ, make_float4(0.f, 0.f, 0.f, 0.f));
    int q = 0;
    for (int n = 0; n < order; n++) {
        double theta = 0.5 + 0.5 * gx[n];
        for (int m = 0; m < order; m++, q++) {
            double rho = 0.5 + 0.5 * gx[m];
            double w = 0.25 * gw[n] * gw[m] * rho;
            double x3a = rho * (1.0 - theta), x3b = rho * theta;        // collapse at vertex 3
            double x1a = 1.0 - rho, x1b = rho * (1.0 - theta);          // at vertex 1
            double x2a = rho * theta, x2b = 1.0 - rho;                  // at vertex 2
            qf[q] = make_float4((float)x3a, (float)x3b, (float)w, 0.0f);
            double v[3][2] = {{x1a, x1b}, {x2a, x2b}, {x3a, x3b}};
            const double off[3][2] = {{-rho, x1b}, {x2a, -rho}, {x3a, x3b}};   // minus (1, 0), (0, 1), (0, 0)
            for (int c = 0; c < 3; c++) {
                qd[(c * kMaxQ + q) * 3 + 0] = v[c][0];
                qd[(c * kMaxQ + q) * 3 + 1] = v[c][1];
                qd[(c * kMaxQ + q) * 3 + 2] = w;
                qs[c * kMaxQ + q] = make_float4((float)off[c][0], (float)off[c][1], (float)w, 0.0f);
            }
        }
    }
    CUDA_TRY(cudaMemcpyToSymbol(c_qf, qf.data(), sizeof(float4) * nq));
    CUDA_TRY(cudaMemcpyToSymbol(c_qd, qd.data(), sizeof(double) * qd.size()));
    CUDA_TRY(cudaMemcpyToSymbol(c_qs, qs.data(), sizeof(float4) * qs.size()));
    CUDA_TRY(cudaMemcpyToSymbol(c_nq, &nq, sizeof(int)));
    if (dev < 64) g_quad_order[dev] = order;
    g_nq_host = nq;
}

int quadrature_points() { return g_nq_host; }

// ---------------------------------------------------------------------------
// Element tables.
// Float table, 9 float4 per element:
//   [0] (p3hi.xyz, J)   [1] (p3lo.xyz, near_r2)   [2] (e1, coff.x)   [3] (e2, coff.y)
//   [4] (n, coff.z)     [5] (bcA.re, bcA.im, bcC.re, bcC.im)    [6] (centroid, n tail z)
//   [7] (e1 tail, n tail x)   [8] (e2 tail, n tail y)
//   with coff = centroid - p3 = (e1 + e2) / 3; the tails are the remainders
//   of e1, e2 and n after rounding to float (heads in [2]-[4])
// p3 is split into hi + lo floats so that p3 - x keeps full float precision
// for nearby pairs.  e1 = p1-p3, e2 = p2-p3, n = e1 x e2 / J, J = |e1 x e2|
// (mesh.cu:612-617), near_r2 = (eta * longest edge)^2.
// Double table, 18 doubles: p3[3] e1[3] e2[3] n[3] J bcA[2] bcC[2] diam.
// ---------------------------------------------------------------------------
constexpr int kGeoF = 9;
constexpr int kFarRecG = 7;   // the leading float4 of an element's entry that a far record carries
constexpr int kGeoD = 18;

__global__ void elem_setup_kernel(const double *__restrict__ nodes, const int4 *__restrict__ elems,
                                  const double *__restrict__ bc, int E, double eta,
                                  float4 *__restrict__ gf, double *__restrict__ gd) {
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    int4 nd = elems[e];
    const double *p1 = nodes + 3 * (size_t)nd.x, *p2 = nodes + 3 * (size_t)nd.y,
                 *p3 = nodes + 3 * (size_t)nd.z;
    double e1[3], e2[3], c[3], cen[3];
    for (int d = 0; d < 3; d++) {
        e1[d] = p1[d] - p3[d];
        e2[d] = p2[d] - p3[d];
        cen[d] = (p1[d] + p2[d] + p3[d]) / 3.0;
    }
    c[0] = e1[1] * e2[2] - e1[2] * e2[1];
    c[1] = e1[2] * e2[0] - e1[0] * e2[2];
    c[2] = e1[0] * e2[1] - e1[1] * e2[0];
    double J = sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
    double n[3] = {c[0] / J, c[1] / J, c[2] / J};
    double l12 = 0, l23 = 0, l31 = 0;
    for (int d = 0; d < 3; d++) {
        l12 += (p1[d] - p2[d]) * (p1[d] - p2[d]);
        l23 += (p2[d] - p3[d]) * (p2[d] - p3[d]);
        l31 += (p3[d] - p1[d]) * (p3[d] - p1[d]);
    }
    double diam = sqrt(fmax(l12, fmax(l23, l31)));
    // bcA = ca/cb, bcC = cc/cb (cuCdivf(bc[0], bc[1]) etc., atomicFuncs.cu:87,105)
    const double *b = bc + 6 * (size_t)e;
    double den = b[2] * b[2] + b[3] * b[3];
    double aR = (b[0] * b[2] + b[1] * b[3]) / den, aI = (b[1] * b[2] - b[0] * b[3]) / den;
    double cR = (b[4] * b[2] + b[5] * b[3]) / den, cI = (b[5] * b[2] - b[4] * b[3]) / den;
    float r2 = (float)((eta * diam) * (eta * diam));
    float4 *g = gf + (size_t)kGeoF * e;
    float hx = (float)p3[0], hy = (float)p3[1], hz = (float)p3[2];
    g[0] = make_float4(hx, hy, hz, (float)J);
    g[1] = make_float4((float)(p3[0] - (double)hx), (float)(p3[1] - (double)hy),
                       (float)(p3[2] - (double)hz), eta > 0 ? r2 : 0.0f);
    g[2] = make_float4((float)e1[0], (float)e1[1], (float)e1[2], (float)((e1[0] + e2[0]) / 3.0));
    g[3] = make_float4((float)e2[0], (float)e2[1], (float)e2[2], (float)((e1[1] + e2[1]) / 3.0));
    g[4] = make_float4((float)n[0], (float)n[1], (float)n[2], (float)((e1[2] + e2[2]) / 3.0));
    g[5] = make_float4((float)aR, (float)aI, (float)cR, (float)cI);
    // tails of e1, e2 and n (the FP32 near path forms its pair geometry in
    // double float from heads and tails): g[7] = (e1 tail, n tail x),
    // g[8] = (e2 tail, n tail y), g[6].w = n tail z
    float lo[9];
    for (int d = 0; d < 3; d++) {
        lo[d] = (float)(e1[d] - (double)(float)e1[d]);
        lo[3 + d] = (float)(e2[d] - (double)(float)e2[d]);
        lo[6 + d] = (float)(n[d] - (double)(float)n[d]);
    }
    g[6] = make_float4((float)cen[0], (float)cen[1], (float)cen[2], lo[8]);
    g[7] = make_float4(lo[0], lo[1], lo[2], lo[6]);
    g[8] = make_float4(lo[3], lo[4], lo[5], lo[7]);
    double *h = gd + (size_t)kGeoD * e;
    for (int d = 0; d < 3; d++) {
        h[d] = p3[d];
        h[3 + d] = e1[d];
        h[6 + d] = e2[d];
        h[9 + d] = n[d];
    }
    h[12] = J;
    h[13] = aR; h[14] = aI; h[15] = cR; h[16] = cI;
    h[17] = diam;
}

void launch_elem_setup(const double *d_nodes, const int4 *d_elems, const double *d_bc, int E,
                       double near_eta, float4 *geo_f, double *geo_d, cudaStream_t st) {
    BEM_PROF("elem_setup", st);
    if (E <= 0) return;
    elem_setup_kernel<<<(E + 127) / 128, 128, 0, st>>>(d_nodes, d_elems, d_bc, E, near_eta, geo_f, geo_d);
    count_launch();
    KERNEL_CHECK();
}

// ---------------------------------------------------------------------------
// Pair classification shared by the far and near kernels.  It must give the
// same answer in both, so it uses only float inputs and _rn intrinsics (no
// FMA contraction).  A pair is "near" when x is a node of the element (the
// singular pairs of atomicFuncs.cu:119-216) or, with eta > 0, when
// |x - centroid|^2 < (eta*diam)^2.
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool pair_is_near_v(int row, int N, int4 nd, float4 xh, float r2, float4 c) {
    if (row < N && (row == nd.x || row == nd.y || row == nd.z)) return true;
    if (r2 > 0.0f) {
        float dx = __fsub_rn(xh.x, c.x), dy = __fsub_rn(xh.y, c.y), dz = __fsub_rn(xh.z, c.z);
        float d2 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
        return d2 < r2;
    }
    return false;
}
__device__ __forceinline__ bool pair_is_near(int row, int N, int4 nd, float4 xh, const float4 *g) {
    return pair_is_near_v(row, N, nd, xh, g[1].w, g[6]);
}

// ---------------------------------------------------------------------------
// Regular (far) pair integral, FP32.  With d = y - x = d3 + xi1*e1 + xi2*e2
// (d3 = p3 - x) and the constant height hgt = d3.n ((y-x).n is the same for
// every y of a flat element):
//   G = exp(-ikr)/(4 pi r), dG/dn = G (-1/r - ik) hgt/r, dG0/dn = -hgt/(4 pi r^3)
// (green, pGpn2, pPsiLpn2: numerical.cu:70-74, mesh.cu:120-136), and the
// weighted sums  S0 = sum w f, S1 = sum w xi1 f, S2 = sum w xi2 f  give the
// three nodal integrals (N1 = xi1, N2 = xi2, N3 = 1 - xi1 - xi2).  The 1/(4 pi)
// and |J| factors are applied once per pair by the caller.
// ---------------------------------------------------------------------------
// Phase of the FP32 quadrature.  The hardware sin/cos approximation
// (sin.approx, as in __sincosf) is documented with a bounded error on
// [-pi, pi] only and its error grows with |x| outside (kr
// reaches ~30 at 8 kHz on a 0.11 m body).  Three modes, chosen per launch on
// the host from the problem's size in wavelengths:
//
// kPhaseShift: over one element kr varies by at most k * diam, so one multiple
//   of 2 pi per pair, n = round(k r_c / 2 pi) (r_c = distance to the centroid),
//   brings every point's phase into [-pi - k diam, pi + k diam]:
//   y = fma(k, r, -n C1) + (-n C2), the two-constant Cody-Waite scheme (Cody &
//   Waite, "Software Manual for the Elementary Functions", 1980) with C1 = 2 pi
//   cut to 16 significant bits (n C1 is exact for n < 256), C2 = fl(2 pi - C1).
// kPhaseWrap: the same, and the point's own multiple of 2 pi is removed too
//   (elements spanning a large phase: k * longest edge above kWrapKh).
// kPhaseAcc: FP32 r carries a relative error of ~1e-7, a phase error of
//   ~1e-7 kr that dominates when kr is large.  The phase is split as
//   k r = k r_c + k (r - r_c): k r_c in double float once per pair (centroid
//   offset from the row point in head/tail floats, k as head/tail), reduced by
//   2 pi; r - r_c = (r^2 - r_c^2) / (r + r_c) where r^2 - r_c^2 =
//   (d - d_c).(d + d_c) is a quadratic in the Duffy radius with coefficients
//   free of cancellation, so the per-point term is accurate to ~1e-7 of
//   k (r - r_c) <= k * diam.  sin and cos then come from sincos_acc instead
//   of the fast intrinsic.  Used when k * extent > kAccKd or k * longest edge
//   > kAccKh (coarse meshes at high frequency, whose oscillating sums cancel).
constexpr double kWrapKh = 0.75;    // k * longest edge above which the point phase is wrapped
constexpr double kAccKd = 40.0;     // k * extent above which kPhaseAcc is used
constexpr double kAccKh = 1.2;      // k * longest edge above which kPhaseAcc is used
enum { kPhaseShift = 0, kPhaseWrap = 1, kPhaseAcc = 2 };

struct PairPhase {
    float c1, c2;    // shift modes: -n C1, -n C2
    float yc, rc;    // kPhaseAcc: k r_c reduced by 2 pi, r_c
    float c0;        // kPhaseAcc: |d3|^2 - |d_c|^2 = -coff.(2 d3 + coff)
};

constexpr float kInv2PiF = 0.15915493667125702f;
constexpr float kC1F = 6.2830810546875f;
constexpr float kC2F = 0.00010425248910905793f;

__device__ __forceinline__ PairPhase pair_phase_shift(float k, float3 d3, float3 coff) {
    const float cx = d3.x + coff.x, cy = d3.y + coff.y, cz = d3.z + coff.z;
    const float rc = sqrtf(fmaf(cz, cz, fmaf(cy, cy, cx * cx)));
    const float n = fminf(rintf(k * rc * kInv2PiF), 255.0f);
    PairPhase p;
    p.c1 = -n * kC1F;
    p.c2 = -n * kC2F;
    p.yc = p.rc = p.c0 = 0.f;
    return p;
}

// x + y = s + e exactly (Knuth's TwoSum)
__device__ __forceinline__ float two_sum(float a, float b, float &e) {
    const float s = __fadd_rn(a, b), bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return s;
}

// kPhaseAcc per-pair terms: p3 = p3h + p3l and the row point x = xh + xl as
// head/tail floats, coff = centroid - p3, k = kh + kl.
__device__ __forceinline__ PairPhase pair_phase_acc(float kh, float kl, float3 p3h, float3 p3l, float4 xh,
                                                    float4 xl, float3 d3, float3 coff) {
    // centroid - x = (p3h - xh) + coff + (p3l - xl): head hx (two rounded sums), tail lx
    float a0, a1, a2, b0, b1, b2;
    const float hx = two_sum(two_sum(p3h.x, -xh.x, a0), coff.x, b0);
    const float hy = two_sum(two_sum(p3h.y, -xh.y, a1), coff.y, b1);
    const float hz = two_sum(two_sum(p3h.z, -xh.z, a2), coff.z, b2);
    const float lx = (a0 + b0) + (p3l.x - xl.x), ly = (a1 + b1) + (p3l.y - xl.y), lz = (a2 + b2) + (p3l.z - xl.z);
    // r_c^2 = |(hx, hy, hz) + (lx, ly, lz)|^2 in double float
    const float px = __fmul_rn(hx, hx), py = __fmul_rn(hy, hy), pz = __fmul_rn(hz, hz);
    const float ex = __fmaf_rn(hx, hx, -px), ey = __fmaf_rn(hy, hy, -py), ez = __fmaf_rn(hz, hz, -pz);
    float t0, t1;
    const float s01 = two_sum(px, py, t0);
    const float shi = two_sum(s01, pz, t1);
    const float slo = (t0 + t1) + (ex + ey + ez) + 2.0f * (hx * lx + hy * ly + hz * lz);
    const float r0 = __fsqrt_rn(shi);
    const float rlo = (__fmaf_rn(-r0, r0, shi) + slo) * (0.5f / r0);
    // k r_c = (kh + kl)(r0 + rlo), reduced by 2 pi
    const float ph = __fmul_rn(kh, r0);
    const float plo = __fmaf_rn(kh, r0, -ph) + kh * rlo + kl * r0;
    const float n = fminf(rintf(ph * kInv2PiF), 255.0f);
    PairPhase p;
    p.c1 = p.c2 = 0.f;
    p.yc = __fmaf_rn(-n, kC2F, __fmaf_rn(-n, kC1F, ph)) + plo;
    p.rc = r0;
    p.c0 = -(coff.x * (2.0f * d3.x + coff.x) + coff.y * (2.0f * d3.y + coff.y) + coff.z * (2.0f * d3.z + coff.z));
    return p;
}

__device__ __forceinline__ float wrap_phase(float y) {
    constexpr float kRound = 12582912.0f;   // 1.5 * 2^23: rounds to an integer (|y| < 2^22)
    const float n = __fsub_rn(__fmaf_rn(y, kInv2PiF, kRound), kRound);
    return __fmaf_rn(-n, kC2F, __fmaf_rn(-n, kC1F, y));
}

// sin and cos to ~1e-7 absolute for |y| < 400 (kPhaseAcc): quadrant
// j = round(2y/pi), z = y - j pi/2 by a two-constant Cody-Waite FMA (P1 = pi/2
// cut to 16 significant bits, P2 = fl(pi/2 - P1)), then the Taylor series of
// sin (to z^9) and cos (to z^8) on |z| <= pi/4, whose truncation errors are
// 2e-9 and 3e-8, and the quadrant's swap and signs.  The fast __sincosf is
// documented at 2^-21.41 absolute on [-pi, pi]; on coarse meshes at high
// frequency the quadrature sums cancel and that error shows in the matrix.
__device__ __forceinline__ void sincos_acc(float y, float *sn, float *cs) {
    constexpr float k2OverPi = 0.6366197723675814f, kRound = 12582912.0f;
    constexpr float kP1 = 1.570770263671875f, kP2 = 2.6063122277264483e-05f;
    const float t = __fmaf_rn(y, k2OverPi, kRound);
    const float j = __fsub_rn(t, kRound);
    const unsigned qd = __float_as_uint(t) & 3u;      // j mod 4 (t's last mantissa bits)
    const float z = __fmaf_rn(-j, kP2, __fmaf_rn(-j, kP1, y));
    const float z2 = z * z;
    const float ps = fmaf(z2, fmaf(z2, fmaf(z2, fmaf(z2, 2.7557319223985893e-06f, -1.984126984126984e-04f),
                                             8.333333333333333e-03f), -0.16666666666666666f), 1.0f) * z;
    const float pc = fmaf(z2, fmaf(z2, fmaf(z2, fmaf(z2, 2.48015873015873e-05f, -1.388888888888889e-03f),
                                             4.1666666666666664e-02f), -0.5f), 1.0f);
    const float s0 = (qd & 1u) ? pc : ps, c0 = (qd & 1u) ? ps : pc;
    *sn = (qd & 2u) ? -s0 : s0;
    *cs = ((qd + 1u) & 2u) ? -c0 : c0;
}

// The hardware approximations (PTX rsqrt/sin/cos.approx) with subnormal
// inputs and results flushed to zero.  The quadrature's r^2 and phases are
// far from the subnormal range, so the flush changes nothing there; it drops
// the subnormal handling that the default (non-flushing) forms carry.
__device__ __forceinline__ float rsqrt_ftz(float x) {
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ void sincos_ftz(float x, float *sn, float *cs) {
    asm("sin.approx.ftz.f32 %0, %1;" : "=f"(*sn) : "f"(x));
    asm("cos.approx.ftz.f32 %0, %1;" : "=f"(*cs) : "f"(x));
}

// sin and cos of the phase of a point at distance r; q = r^2 - r_c^2
// (kPhaseAcc only).
template <int PH>
__device__ __forceinline__ void phase_sincos(float k, float r, float q, const PairPhase &pp, float *sn, float *cs) {
    if (PH == kPhaseAcc) {
        sincos_acc(fmaf(k, __fdividef(q, r + pp.rc), pp.yc), sn, cs);
    } else {
        const float y = fmaf(k, r, pp.c1) + pp.c2;
        sincos_ftz(PH == kPhaseWrap ? wrap_phase(y) : y, sn, cs);
    }
}

struct SumsF {
    float g0r, g0i, g1r, g1i, g2r, g2i;   // G sums
    float h0r, h0i, h1r, h1i, h2r, h2i;   // dG/dn sums
    float c;                              // dG0/dn sum
};

template <int PH>
__device__ __forceinline__ void far_sums_f32(float3 d3, float3 e1, float3 e2, float3 coff, float hgt, float k,
                                             const PairPhase &pp, int nq, SumsF &S) {
    S.g0r = S.g0i = S.g1r = S.g1i = S.g2r = S.g2i = 0.0f;
    S.h0r = S.h0i = S.h1r = S.h1i = S.h2r = S.h2i = 0.0f;
    S.c = 0.0f;
#pragma unroll 4
    for (int q = 0; q < nq; q++) {
        const float4 t = c_qf[q];
        float dx = fmaf(t.y, e2.x, fmaf(t.x, e1.x, d3.x));
        float dy = fmaf(t.y, e2.y, fmaf(t.x, e1.y, d3.y));
        float dz = fmaf(t.y, e2.z, fmaf(t.x, e1.z, d3.z));
        float r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
        float ri = rsqrt_ftz(r2);
        float r = r2 * ri;
        float sn, cs;
        float dq = 0.f;
        if (PH == kPhaseAcc) {
            // (d - d_c).(d + d_c) with d - d_c = t.x e1 + t.y e2 - coff
            const float ux = fmaf(t.y, e2.x, fmaf(t.x, e1.x, -coff.x));
            const float uy = fmaf(t.y, e2.y, fmaf(t.x, e1.y, -coff.y));
            const float uz = fmaf(t.y, e2.z, fmaf(t.x, e1.z, -coff.z));
            dq = fmaf(uz, dz + d3.z + coff.z, fmaf(uy, dy + d3.y + coff.y, ux * (dx + d3.x + coff.x)));
        }
        phase_sincos<PH>(k, r, dq, pp, &sn, &cs);
        float gr = cs * ri, gi = -sn * ri;            // 4 pi G
        float hq = hgt * ri;                          // dr/dn
        float tr = fmaf(gi, k, -gr * ri);             // 4 pi G (-1/r - ik)
        float ti = -fmaf(gr, k, gi * ri);
        float dgr = tr * hq, dgi = ti * hq;           // 4 pi dG/dn
        float c0 = -hq * ri * ri;                     // 4 pi dG0/dn
        float w = t.z, w1 = w * t.x, w2 = w * t.y;
        S.g0r = fmaf(w, gr, S.g0r);  S.g0i = fmaf(w, gi, S.g0i);
        S.g1r = fmaf(w1, gr, S.g1r); S.g1i = fmaf(w1, gi, S.g1i);
        S.g2r = fmaf(w2, gr, S.g2r); S.g2i = fmaf(w2, gi, S.g2i);
        S.h0r = fmaf(w, dgr, S.h0r);  S.h0i = fmaf(w, dgi, S.h0i);
        S.h1r = fmaf(w1, dgr, S.h1r); S.h1i = fmaf(w1, dgi, S.h1i);
        S.h2r = fmaf(w2, dgr, S.h2r); S.h2i = fmaf(w2, dgi, S.h2i);
        S.c = fmaf(w, c0, S.c);
    }
}

// The same sums for the 6 x 6 rule (the reference's INTORDER = 6), arranged
// for the FP32 issue rate:
//   * the Duffy points lie on lines of constant theta_n: d = d3 + rho_m v_n
//     with v_n = e1 + theta_n (e2 - e1), so r^2 is a quadratic in rho_m
//     with per-line coefficients: 2 FMAs per point;
//   * along a line, S0 needs sum w_m rho_m f and S1, S2 both need
//     sum w_m rho_m^2 f (xi1 = rho (1-theta), xi2 = rho theta): two inner sums
//     per quantity instead of three;
//   * with E = exp(-ikr) = c - i s:  4 pi G = E/r  and
//     4 pi dG/dn = -(hgt/r^3) [(c + kr s) + i (kr c - s)],
//     4 pi dG0/dn = -hgt/r^3, so the height leaves the sums.
// The Gauss abscissae/weights are the published 6-point values as
// compile-time constants; the loops unroll completely.
__device__ __forceinline__ float gl6_x(int i) {
    return i == 0 ? -0.9324695142031521f : i == 1 ? -0.6612093864662645f : i == 2 ? -0.2386191860831969f
         : i == 3 ? 0.2386191860831969f : i == 4 ? 0.6612093864662645f : 0.9324695142031521f;
}
__device__ __forceinline__ float gl6_w(int i) {
    return (i == 0 || i == 5) ? 0.1713244923791704f : (i == 1 || i == 4) ? 0.3607615730481386f
                                                                           : 0.4679139345726910f;
}

template <int PH>
__device__ __forceinline__ void far_sums_f32_o6(float3 d3, float3 e1, float3 e2, float3 coff, float hgt, float k,
                                                const PairPhase &pp, SumsF &S) {
    S.g0r = S.g0i = S.g1r = S.g1i = S.g2r = S.g2i = 0.0f;
    S.h0r = S.h0i = S.h1r = S.h1i = S.h2r = S.h2i = 0.0f;
    S.c = 0.0f;
    // Along line n, v = e1 + th e21: qa = |v|^2 and qb = 2 v.d3 from five dot
    // products per pair, qa = a0 + th a1 + th^2 a2.  The expansion cancels
    // where |v| is well below |e1| (an obtuse angle at the shared vertex, e1.e21
    // < 0): qa then carries about (|e1| / h)^2 ulps of |v|^2, h the element's
    // height over that vertex's opposite edge; for far pairs r^2 = qa rho^2 +
    // qb rho + |d3|^2 is dominated by |d3|^2 and the effect on r is below
    // FP32 rounding unless the element is a sliver.
    const float3 e21 = make_float3(e2.x - e1.x, e2.y - e1.y, e2.z - e1.z);
    const float a0 = fmaf(e1.z, e1.z, fmaf(e1.y, e1.y, e1.x * e1.x));
    const float a1 = 2.0f * fmaf(e1.z, e21.z, fmaf(e1.y, e21.y, e1.x * e21.x));
    const float a2 = fmaf(e21.z, e21.z, fmaf(e21.y, e21.y, e21.x * e21.x));
    const float b0 = 2.0f * fmaf(e1.z, d3.z, fmaf(e1.y, d3.y, e1.x * d3.x));
    const float b1 = 2.0f * fmaf(e21.z, d3.z, fmaf(e21.y, d3.y, e21.x * d3.x));
    const float dd = fmaf(d3.z, d3.z, fmaf(d3.y, d3.y, d3.x * d3.x));   // |d3|^2
#pragma unroll
    for (int n = 0; n < 6; n++) {
        const float th = 0.5f + 0.5f * gl6_x(n);
        // along the line r^2 = qa rho^2 + qb rho + |d3|^2 (and, kPhaseAcc,
        // r^2 - r_c^2 = qa rho^2 + qb rho + c0).  The terms are within a few
        // ulps of r^2 for a far pair (|d3| and rho |v| are bounded by r plus
        // the element's size), as accurate as summing the squared components.
        const float qa = fmaf(th * th, a2, fmaf(th, a1, a0));
        const float qb = fmaf(th, b1, b0);
        float u0gr = 0.f, u1gr = 0.f, u0gs = 0.f, u1gs = 0.f;
        float u0ha = 0.f, u1ha = 0.f, u0hb = 0.f, u1hb = 0.f, u0c = 0.f;
#pragma unroll
        for (int m = 0; m < 6; m++) {
            const float rho = 0.5f + 0.5f * gl6_x(m);
            const float wr1 = gl6_w(m) * rho, wr2 = gl6_w(m) * rho * rho;
            const float r2 = fmaf(qa, rho * rho, fmaf(qb, rho, dd));
            const float ri = rsqrt_ftz(r2);
            const float r = r2 * ri;
            float sn, cs;
            const float q = PH == kPhaseAcc ? fmaf(fmaf(qa, rho, qb), rho, pp.c0) : 0.f;
            phase_sincos<PH>(k, r, q, pp, &sn, &cs);
            // (c + kr s)/r^3 = (gr + k s)/r^2 and (kr c - s)/r^3 = (k c - gs)/r^2
            const float ri2 = ri * ri;
            const float gr = cs * ri, gs = sn * ri;
            const float ha = ri2 * fmaf(k, sn, gr), hb = ri2 * fmaf(k, cs, -gs);
            const float ri3 = ri2 * ri;
            u0gr = fmaf(wr1, gr, u0gr); u1gr = fmaf(wr2, gr, u1gr);
            u0gs = fmaf(wr1, gs, u0gs); u1gs = fmaf(wr2, gs, u1gs);
            u0ha = fmaf(wr1, ha, u0ha); u1ha = fmaf(wr2, ha, u1ha);
            u0hb = fmaf(wr1, hb, u0hb); u1hb = fmaf(wr2, hb, u1hb);
            u0c = fmaf(wr1, ri3, u0c);
        }
        const float a = 0.25f * gl6_w(n), b = a * (1.0f - th), c = a * th;
        S.g0r = fmaf(a, u0gr, S.g0r); S.g1r = fmaf(b, u1gr, S.g1r); S.g2r = fmaf(c, u1gr, S.g2r);
        S.g0i = fmaf(a, u0gs, S.g0i); S.g1i = fmaf(b, u1gs, S.g1i); S.g2i = fmaf(c, u1gs, S.g2i);
        S.h0r = fmaf(a, u0ha, S.h0r); S.h1r = fmaf(b, u1ha, S.h1r); S.h2r = fmaf(c, u1ha, S.h2r);
        S.h0i = fmaf(a, u0hb, S.h0i); S.h1i = fmaf(b, u1hb, S.h1i); S.h2i = fmaf(c, u1hb, S.h2i);
        S.c = fmaf(a, u0c, S.c);
    }
    // signs and the height: G = (gr, -gs); dG/dn = -hgt (ha, hb); dG0/dn = -hgt c
    const float mh = -hgt;
    S.g0i = -S.g0i; S.g1i = -S.g1i; S.g2i = -S.g2i;
    S.h0r *= mh; S.h1r *= mh; S.h2r *= mh;
    S.h0i *= mh; S.h1i *= mh; S.h2i *= mh;
    S.c *= mh;
}

// Two-lane FP32 arithmetic: a 64-bit register pair holds two floats and one
// f32x2 instruction does both lanes' operations, each lane rounded exactly
// like the scalar instruction (fma.rn / mul.rn / add.rn).
__device__ __forceinline__ uint64_t f2(float lo, float hi) {
    uint64_t r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ void f2_split(uint64_t v, float &lo, float &hi) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ float f2_sum(uint64_t v) {
    float lo, hi;
    f2_split(v, lo, hi);
    return lo + hi;
}
__device__ __forceinline__ uint64_t fma2(uint64_t a, uint64_t b, uint64_t c) {
    uint64_t d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
__device__ __forceinline__ uint64_t mul2(uint64_t a, uint64_t b) {
    uint64_t d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ uint64_t add2(uint64_t a, uint64_t b) {
    uint64_t d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}

// far_sums_f32_o6 for the shift and wrap phase modes with the two lanes of
// f32x2 arithmetic carrying the mirror lines n and 5 - n at the same point m
// (theta_{5-n} = 1 - theta_n and equal weights, the Gauss rule being
// symmetric): the same operations per point with the point's constants
// shared by both lanes, half the instructions for all but rsqrt, sin and cos.
// The line-pair tail needs no lane reduction but S0's: the lanes' xi1 and
// xi2 weights are each other's (a (1 - theta) for one line is a theta' for
// the other), so S1 += b U1_n + c U1_{5-n} and S2 += c U1_n + b U1_{5-n}.
// The dG/dn imaginary sums collect -hb (fma(-k, c, gs) = -fma(k, c, -gs)
// exactly) and take the sign with the height at the end.
// The phase shift's second constant is folded into r: y = k (r + c2 / k) + c1
// with r + c2 / k formed by one FMA from r^2 and 1/r (one operation less per
// point than k r + c1 + c2; r + c2 / k is rounded once, as r was).
// GM (which sums of G the BCs need): 2 = all (some element has bcA != 0, so
// G enters A); 1 = S0 only (bcA = 0 everywhere, e.g. the BC (0, 1, gamma):
// beta needs sum_j g_j = S0); 0 = none (bcA = bcC = 0 everywhere, the rigid
// BC (0, 1, 0)).  The sums not formed are left zero.
template <int PH, int GM>
__device__ __forceinline__ void far_sums_f32_o6x2(float3 d3, float3 e1, float3 e2, float hgt, float k, float kinv,
                                                  const PairPhase &pp, SumsF &S) {
    static_assert(PH != kPhaseAcc, "the accurate phase mode has its own per-point arithmetic");
    S.g0r = S.g0i = S.g1r = S.g1i = S.g2r = S.g2i = 0.0f;
    S.h0r = S.h0i = S.h1r = S.h1i = S.h2r = S.h2i = 0.0f;
    S.c = 0.0f;
    // Along line n, v = e1 + th e21: qa = |v|^2 and qb = 2 v.d3 from five dot
    // products per pair, qa = a0 + th a1 + th^2 a2.  The expansion cancels
    // where |v| is well below |e1| (an obtuse angle at the shared vertex, e1.e21
    // < 0): qa then carries about (|e1| / h)^2 ulps of |v|^2, h the element's
    // height over that vertex's opposite edge; for far pairs r^2 = qa rho^2 +
    // qb rho + |d3|^2 is dominated by |d3|^2 and the effect on r is below
    // FP32 rounding unless the element is a sliver.
    const float3 e21 = make_float3(e2.x - e1.x, e2.y - e1.y, e2.z - e1.z);
    const float a0 = fmaf(e1.z, e1.z, fmaf(e1.y, e1.y, e1.x * e1.x));
    const float a1 = 2.0f * fmaf(e1.z, e21.z, fmaf(e1.y, e21.y, e1.x * e21.x));
    const float a2 = fmaf(e21.z, e21.z, fmaf(e21.y, e21.y, e21.x * e21.x));
    const float b0 = 2.0f * fmaf(e1.z, d3.z, fmaf(e1.y, d3.y, e1.x * d3.x));
    const float b1 = 2.0f * fmaf(e21.z, d3.z, fmaf(e21.y, d3.y, e21.x * d3.x));
    const float dd = fmaf(d3.z, d3.z, fmaf(d3.y, d3.y, d3.x * d3.x));
    const uint64_t dd2 = f2(dd, dd), k2 = f2(k, k), nk2 = f2(-k, -k);
    const float dr = pp.c2 * kinv;
    const uint64_t c1 = f2(pp.c1, pp.c1), dr2 = f2(dr, dr);
#pragma unroll
    for (int n = 0; n < 3; n++) {
        const float th = 0.5f + 0.5f * gl6_x(n), tm = 0.5f + 0.5f * gl6_x(5 - n);   // tm = 1 - th
        const uint64_t qa2 = f2(fmaf(th * th, a2, fmaf(th, a1, a0)), fmaf(tm * tm, a2, fmaf(tm, a1, a0)));
        const uint64_t qb2 = f2(fmaf(th, b1, b0), fmaf(tm, b1, b0));
        uint64_t u0gr = 0, u1gr = 0, u0gs = 0, u1gs = 0, u0ha = 0, u1ha = 0, u0hb = 0, u1hb = 0, u0c = 0;
#pragma unroll
        for (int m = 0; m < 6; m++) {
            const float rho_m = 0.5f + 0.5f * gl6_x(m);
            const uint64_t rho = f2(rho_m, rho_m);
            const uint64_t wr1 = f2(gl6_w(m) * rho_m, gl6_w(m) * rho_m);
            const uint64_t wr2 = f2(gl6_w(m) * rho_m * rho_m, gl6_w(m) * rho_m * rho_m);
            const uint64_t r2 = fma2(fma2(qa2, rho, qb2), rho, dd2);   // (qa rho + qb) rho + |d3|^2
            float ra, rb;
            f2_split(r2, ra, rb);
            const uint64_t ri = f2(rsqrt_ftz(ra), rsqrt_ftz(rb));
            const uint64_t r = fma2(r2, ri, dr2);   // r + c2 / k
            uint64_t y = fma2(k2, r, c1);
            if (PH == kPhaseWrap) {
                // wrap_phase on both lanes
                const uint64_t kr = f2(12582912.0f, 12582912.0f);
                const uint64_t nn = add2(fma2(y, f2(kInv2PiF, kInv2PiF), kr), f2(-12582912.0f, -12582912.0f));
                y = fma2(nn, f2(-kC2F, -kC2F), fma2(nn, f2(-kC1F, -kC1F), y));
            }
            float ya, yb, sa, ca, sb, cb;
            f2_split(y, ya, yb);
            sincos_ftz(ya, &sa, &ca);
            sincos_ftz(yb, &sb, &cb);
            const uint64_t sn = f2(sa, sb), cs = f2(ca, cb);
            const uint64_t ri2 = mul2(ri, ri);
            const uint64_t gr = mul2(cs, ri), gs = mul2(sn, ri);
            const uint64_t ha = mul2(ri2, fma2(k2, sn, gr));
            const uint64_t hbn = mul2(ri2, fma2(nk2, cs, gs));
            const uint64_t ri3 = mul2(ri2, ri);
            if constexpr (GM >= 1) {
                u0gr = fma2(wr1, gr, u0gr);
                u0gs = fma2(wr1, gs, u0gs);
            }
            if constexpr (GM == 2) {
                u1gr = fma2(wr2, gr, u1gr);
                u1gs = fma2(wr2, gs, u1gs);
            }
            u0ha = fma2(wr1, ha, u0ha); u1ha = fma2(wr2, ha, u1ha);
            u0hb = fma2(wr1, hbn, u0hb); u1hb = fma2(wr2, hbn, u1hb);
            u0c = fma2(wr1, ri3, u0c);
        }
        // lane 0 = line n (weights a, b = a (1 - th), c = a th), lane 1 = line
        // 5 - n (a, c, b)
        const float a = 0.25f * gl6_w(n), b = a * (1.0f - th), c = a * th;
        float p0, p1;
        if constexpr (GM >= 1) {
            f2_split(u0gr, p0, p1); S.g0r = fmaf(a, p0 + p1, S.g0r);
            f2_split(u0gs, p0, p1); S.g0i = fmaf(a, p0 + p1, S.g0i);
        }
        if constexpr (GM == 2) {
            f2_split(u1gr, p0, p1); S.g1r = fmaf(b, p0, fmaf(c, p1, S.g1r)); S.g2r = fmaf(c, p0, fmaf(b, p1, S.g2r));
            f2_split(u1gs, p0, p1); S.g1i = fmaf(b, p0, fmaf(c, p1, S.g1i)); S.g2i = fmaf(c, p0, fmaf(b, p1, S.g2i));
        }
        f2_split(u0ha, p0, p1); S.h0r = fmaf(a, p0 + p1, S.h0r);
        f2_split(u1ha, p0, p1); S.h1r = fmaf(b, p0, fmaf(c, p1, S.h1r)); S.h2r = fmaf(c, p0, fmaf(b, p1, S.h2r));
        f2_split(u0hb, p0, p1); S.h0i = fmaf(a, p0 + p1, S.h0i);
        f2_split(u1hb, p0, p1); S.h1i = fmaf(b, p0, fmaf(c, p1, S.h1i)); S.h2i = fmaf(c, p0, fmaf(b, p1, S.h2i));
        f2_split(u0c, p0, p1); S.c = fmaf(a, p0 + p1, S.c);
    }
    // G = (gr, -gs); dG/dn = -hgt (ha, hb) = (-hgt ha, hgt (-hb)); dG0/dn = -hgt c
    const float mh = -hgt;
    S.g0i = -S.g0i; S.g1i = -S.g1i; S.g2i = -S.g2i;
    S.h0r *= mh; S.h1r *= mh; S.h2r *= mh;
    S.h0i *= hgt; S.h1i *= hgt; S.h2i *= hgt;
    S.c *= mh;
}

// Same in FP64 (used by the c128 far path and by the field kernel in c128).
struct SumsD {
    double g0r, g0i, g1r, g1i, g2r, g2i;
    double h0r, h0i, h1r, h1i, h2r, h2i;
    double c;
};

__device__ __forceinline__ void far_sums_f64(const double *d3, const double *e1, const double *e2,
                                             double hgt, double k, int nq, SumsD &S) {
    S.g0r = S.g0i = S.g1r = S.g1i = S.g2r = S.g2i = 0.0;
    S.h0r = S.h0i = S.h1r = S.h1i = S.h2r = S.h2i = 0.0;
    S.c = 0.0;
    for (int q = 0; q < nq; q++) {
        const double x1 = c_qd[2][q][0], x2 = c_qd[2][q][1], w = c_qd[2][q][2];
        double dx = d3[0] + x1 * e1[0] + x2 * e2[0];
        double dy = d3[1] + x1 * e1[1] + x2 * e2[1];
        double dz = d3[2] + x1 * e1[2] + x2 * e2[2];
        double r = sqrt(dx * dx + dy * dy + dz * dz);
        double ri = 1.0 / r;
        double sn, cs;
        sincos(k * r, &sn, &cs);
        double gr = cs * ri, gi = -sn * ri;
        double hq = hgt * ri;
        double tr = gi * k - gr * ri;
        double ti = -(gr * k + gi * ri);
        double dgr = tr * hq, dgi = ti * hq;
        double c0 = -hq * ri * ri;
        double w1 = w * x1, w2 = w * x2;
        S.g0r += w * gr;  S.g0i += w * gi;
        S.g1r += w1 * gr; S.g1i += w1 * gi;
        S.g2r += w2 * gr; S.g2i += w2 * gi;
        S.h0r += w * dgr;  S.h0i += w * dgi;
        S.h1r += w1 * dgr; S.h1i += w1 * dgi;
        S.h2r += w2 * dgr; S.h2i += w2 * dgi;
        S.c += w * c0;
    }
}

// Nodal coefficients from the sums (g_h_c_l_nsgl's tail, mesh.cu:655-671):
// node j's integral = scale * S_j with S_3 = S0 - S1 - S2, g *= i*rho*omega,
// a_j = h_j - bcA*g_j, beta = bcC * sum_j g_j, c = scale * Sc.
template <typename T, typename S>
struct Coeffs {
    T ar[3], ai[3];
    T br, bi;
    T c;
};

// GM < 2 (bcA = 0 for the element): a_j = h_j, and beta takes
// sum_j g_j = i rw scale G0 from the S0 sums alone (GM = 0: bcC = 0 too,
// beta = 0).
template <typename T, typename SUMS, int GM = 2>
__device__ __forceinline__ void finish_coeffs(const SUMS &S, T scale, T rw, T bAr, T bAi, T bCr,
                                              T bCi, Coeffs<T, SUMS> &o) {
    if constexpr (GM < 2) {
#pragma unroll
        for (int j = 0; j < 3; j++) {
            o.ar[j] = scale * (j == 0 ? S.h1r : j == 1 ? S.h2r : S.h0r - S.h1r - S.h2r);
            o.ai[j] = scale * (j == 0 ? S.h1i : j == 1 ? S.h2i : S.h0i - S.h1i - S.h2i);
        }
        if constexpr (GM == 1) {
            const T sgr = -rw * scale * S.g0i, sgi = rw * scale * S.g0r;
            o.br = bCr * sgr - bCi * sgi;
            o.bi = bCr * sgi + bCi * sgr;
        } else {
            o.br = o.bi = T(0);
        }
        o.c = scale * S.c;
        return;
    }
    T gr[3] = {S.g1r, S.g2r, S.g0r - S.g1r - S.g2r};
    T gi[3] = {S.g1i, S.g2i, S.g0i - S.g1i - S.g2i};
    T hr[3] = {S.h1r, S.h2r, S.h0r - S.h1r - S.h2r};
    T hi[3] = {S.h1i, S.h2i, S.h0i - S.h1i - S.h2i};
    T sgr = 0, sgi = 0;
#pragma unroll
    for (int j = 0; j < 3; j++) {
        // g = i*rw*scale*G  ->  (-rw*scale*Gi, rw*scale*Gr)
        T g_r = -rw * scale * gi[j], g_i = rw * scale * gr[j];
        T h_r = scale * hr[j], h_i = scale * hi[j];
        o.ar[j] = h_r - (bAr * g_r - bAi * g_i);
        o.ai[j] = h_i - (bAr * g_i + bAi * g_r);
        sgr += g_r;
        sgi += g_i;
    }
    o.br = bCr * sgr - bCi * sgi;
    o.bi = bCr * sgi + bCi * sgr;
    o.c = scale * S.c;
}

// ---------------------------------------------------------------------------
// Far-field assembly kernel.
// grid = (ceil(R/TR), ntiles), block = NT threads, dynamic smem = acc[TR][tc].
// ---------------------------------------------------------------------------
// GM < 2: the G sums that no BC needs are not formed (far_sums_f32_o6x2);
// only the O6 shift/wrap path is instantiated that way.
template <int TR, int NT, int MINB, bool O6, int PH, int GM>
__global__ void __launch_bounds__(NT, MINB)
far_assembly_f32(RowPoints rows, int N, GeoTables geo, TileSet tiles, float k, float k_lo, float rw,
                 float2 *__restrict__ A, size_t lda, float *__restrict__ c_part,
                 float2 *__restrict__ beta_part) {
    static_assert(GM == 2 || (O6 && PH != kPhaseAcc), "the reduced G sums exist for the order-6 shift/wrap path");
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2 *acc = reinterpret_cast<float2 *>(smem_raw);
    __shared__ float red[NT / 32][3];
    const int tc_s = tiles.col_cnt[blockIdx.y];
    // this thread's c and beta sums of row t: cb[(q TR + t) NT + tid], q = c, Re beta, Im beta
    // (in shared memory rather than registers: they are touched once per owned record)
    float *cb = reinterpret_cast<float *>(acc + (size_t)TR * tc_s);
    __shared__ __align__(8) uint64_t batch_done;   // phase i completes when every thread added batch i
    __shared__ int wait_abort;
    const int tile = blockIdx.y;
    const int tc = tiles.col_cnt[tile];
    const int r0 = blockIdx.x * TR;
    const int R = rows.R;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) {
        mbar_init(&batch_done, NT);
        wait_abort = 0;
    }
    for (int i = threadIdx.x; i < TR * tc; i += NT) acc[i] = make_float2(0.f, 0.f);
    __syncthreads();

    const int nq = c_nq;
    const float inv4pi = (float)(1.0 / (4.0 * kPi));
    const float kinv = 1.0f / k;
    const int b0 = tiles.tile_batch[tile], b1 = tiles.tile_batch[tile + 1];
    const int nr = min(TR, R - r0);                       // rows of this CTA
    // Records come in node-disjoint batches.  Per batch the CTA's threads
    // share the (row, record) items of all its rows (item w: row w / bs,
    // record w % bs) and add into the rows' shared-memory accumulators with
    // plain adds (no two items of a batch and row meet on a column).  A
    // split-phase barrier orders the batches: a thread integrates its item of
    // batch i first, then waits (on the mbarrier batch_done) until every
    // thread has added batch i - 1, adds, and arrives; so every column of a
    // row receives its terms in batch order while the wait overlaps the
    // integration.  The c and beta sums are per thread and row.
#pragma unroll
    for (int q = 0; q < 3 * TR; q++) cb[q * NT + threadIdx.x] = 0.f;
    auto wait_batch = [&](int i) {   // batch i (counted from the tile's first) added by every thread
        if (!mbar_wait_bounded(&batch_done, (uint32_t)(i & 1), kFarWaitCycles, &wait_abort)) {
            wait_abort = 1;
            atomicExch(tiles.status, 1);
        }
    };
#pragma unroll 1
    for (int b = b0; b < b1; b++) {
        const int rb = tiles.batch_ptr[b], bs = tiles.batch_ptr[b + 1] - rb;
        const int items = nr * bs;
        bool waited = b == b0;
        for (int w = threadIdx.x; w < items; w += NT) {
            const int t = w / bs;
            const int i = rb + (w - t * bs);
            const int row = r0 + t;
            const float4 xh = rows.f[2 * (size_t)row], xl = rows.f[2 * (size_t)row + 1];
            float2 *arow = acc + (size_t)t * tc;
            const FarRec *fr = tiles.frecs + i;
            const int4 nd = fr->nodes;
            const float4 g1 = fr->g[1];
            if (pair_is_near_v(row, N, nd, xh, g1.w, fr->g[6])) continue;
            const float4 g0 = fr->g[0], g2 = fr->g[2], g3 = fr->g[3], g4 = fr->g[4], g5 = fr->g[5];
            const int4 sl = fr->slots;
            const float3 e1 = make_float3(g2.x, g2.y, g2.z), e2 = make_float3(g3.x, g3.y, g3.z);
            const float3 d3 = make_float3((g0.x - xh.x) + (g1.x - xl.x), (g0.y - xh.y) + (g1.y - xl.y),
                                          (g0.z - xh.z) + (g1.z - xl.z));
            const float hgt = d3.x * g4.x + d3.y * g4.y + d3.z * g4.z;
            SumsF S;
            const float3 coff = make_float3(g2.w, g3.w, g4.w);
            const PairPhase pp = PH == kPhaseAcc
                                     ? pair_phase_acc(k, k_lo, make_float3(g0.x, g0.y, g0.z),
                                                      make_float3(g1.x, g1.y, g1.z), xh, xl, d3, coff)
                                     : pair_phase_shift(k, d3, coff);
            if constexpr (O6 && PH != kPhaseAcc) far_sums_f32_o6x2<PH, GM>(d3, e1, e2, hgt, k, kinv, pp, S);
            else if (O6) far_sums_f32_o6<PH>(d3, e1, e2, coff, hgt, k, pp, S);
            else far_sums_f32<PH>(d3, e1, e2, coff, hgt, k, pp, nq, S);
            Coeffs<float, SumsF> o;
            finish_coeffs<float, SumsF, GM>(S, g0.w * inv4pi, rw, g5.x, g5.y, g5.z, g5.w, o);
            if (!waited) {
                wait_batch(b - b0 - 1);
                waited = true;
            }
            const int slot[3] = {sl.x, sl.y, sl.z};
#pragma unroll
            for (int j = 0; j < 3; j++) {
                const int s = slot[j];
                if (s >= 0) {
                    arow[s].x += o.ar[j];
                    arow[s].y += o.ai[j];
                }
            }
            if (nd.w) {   // this tile counts the element's c and beta terms
                cb[(0 * TR + t) * NT + threadIdx.x] += o.c;
                if constexpr (GM > 0) {
                    cb[(1 * TR + t) * NT + threadIdx.x] += o.br;
                    cb[(2 * TR + t) * NT + threadIdx.x] += o.bi;
                }
            }
        }
        if (!waited) wait_batch(b - b0 - 1);   // arrivals for batch i only after batch i - 1 completed
        mbar_arrive(&batch_done);
    }
    __syncthreads();   // every thread's adds of the last batch are done
    // Row reductions of the c and beta partial sums (fixed order).
#pragma unroll
    for (int t = 0; t < TR; t++) {
        if (t >= nr) break;                               // uniform over the CTA
        float cs = cb[(0 * TR + t) * NT + threadIdx.x], br = cb[(1 * TR + t) * NT + threadIdx.x],
              bi = cb[(2 * TR + t) * NT + threadIdx.x];
        for (int off = 16; off > 0; off >>= 1) {
            cs += __shfl_xor_sync(0xffffffffu, cs, off);
            br += __shfl_xor_sync(0xffffffffu, br, off);
            bi += __shfl_xor_sync(0xffffffffu, bi, off);
        }
        if (lane == 0) { red[warp][0] = cs; red[warp][1] = br; red[warp][2] = bi; }
        __syncthreads();
        if (threadIdx.x == 0) {
            float a = 0, b = 0, c = 0;
            for (int w = 0; w < NT / 32; w++) { a += red[w][0]; b += red[w][1]; c += red[w][2]; }
            c_part[(size_t)tile * R + r0 + t] = a;
            beta_part[(size_t)tile * R + r0 + t] = make_float2(b, c);
        }
        __syncthreads();
    }
    // Write the finished row segments (coalesced when the tile is contiguous).
    const int *cols = tiles.cols + (size_t)tile * tiles.tc_max;
    for (int t = 0; t < TR; t++) {
        const int row = r0 + t;
        if (row >= R) break;
        float2 *dst = A + (size_t)row * lda;
        const float2 *src = acc + (size_t)t * tc;
        for (int i = threadIdx.x; i < tc; i += NT) dst[cols[i]] = src[i];
    }
}

template <int NT>
__global__ void __launch_bounds__(NT, 1)
far_assembly_f64(RowPoints rows, int N, GeoTables geo, TileSet tiles, double k, double rw,
                 double2 *__restrict__ A, size_t lda, double *__restrict__ c_part,
                 double2 *__restrict__ beta_part) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double2 *acc = reinterpret_cast<double2 *>(smem_raw);
    const int tile = blockIdx.y;
    const int tc = tiles.col_cnt[tile];
    const int row = blockIdx.x;
    const int R = rows.R;
    for (int i = threadIdx.x; i < tc; i += NT) acc[i] = make_double2(0.0, 0.0);
    const float4 xh = rows.f[2 * (size_t)row];
    const double x[3] = {rows.d[3 * (size_t)row], rows.d[3 * (size_t)row + 1], rows.d[3 * (size_t)row + 2]};
    __syncthreads();
    const int nq = c_nq;
    const double inv4pi = 1.0 / (4.0 * kPi);
    double csum = 0, bsr = 0, bsi = 0;
    const int b0 = tiles.tile_batch[tile], b1 = tiles.tile_batch[tile + 1];
    for (int b = b0; b < b1; b++) {
    const int rb = tiles.batch_ptr[b], re = tiles.batch_ptr[b + 1];
    for (int i = rb + threadIdx.x; i < re; i += NT) {
        const TileRec rec = tiles.recs[i];
        const float4 *g = geo.geo_f + (size_t)kGeoF * rec.eid;
        const int4 nd = make_int4(rec.node[0], rec.node[1], rec.node[2], 0);
        if (pair_is_near(row, N, nd, xh, g)) continue;
        const double *h = geo.geo_d + (size_t)kGeoD * rec.eid;
        double d3[3] = {h[0] - x[0], h[1] - x[1], h[2] - x[2]};
        double hgt = d3[0] * h[9] + d3[1] * h[10] + d3[2] * h[11];
        SumsD S;
        far_sums_f64(d3, h + 3, h + 6, hgt, k, nq, S);
        Coeffs<double, SumsD> o;
        finish_coeffs<double, SumsD>(S, h[12] * inv4pi, rw, h[13], h[14], h[15], h[16], o);
#pragma unroll
        for (int j = 0; j < 3; j++) {
            int s = rec.slot[j];
            if (s >= 0) {
                acc[s].x += o.ar[j];
                acc[s].y += o.ai[j];
            }
        }
        if (rec.owner) { csum += o.c; bsr += o.br; bsi += o.bi; }
    }
    __syncthreads();
    }
    __shared__ double red[NT / 32][3];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int o = 16; o > 0; o >>= 1) {
        csum += __shfl_xor_sync(0xffffffffu, csum, o);
        bsr += __shfl_xor_sync(0xffffffffu, bsr, o);
        bsi += __shfl_xor_sync(0xffffffffu, bsi, o);
    }
    if (lane == 0) { red[warp][0] = csum; red[warp][1] = bsr; red[warp][2] = bsi; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0, b = 0, c = 0;
        for (int w = 0; w < NT / 32; w++) { a += red[w][0]; b += red[w][1]; c += red[w][2]; }
        c_part[(size_t)tile * R + row] = a;
        beta_part[(size_t)tile * R + row] = make_double2(b, c);
    }
    const int *cols = tiles.cols + (size_t)tile * tiles.tc_max;
    double2 *dst = A + (size_t)row * lda;
    for (int i = threadIdx.x; i < tc; i += NT) dst[cols[i]] = acc[i];
}

constexpr int kFarNT64 = 256;

// Launch shapes of the FP32 far kernel (the autotuner times each once per
// problem shape and keeps the fastest):
//   0: 2 rows x 512 threads, 1 CTA/SM     1: 2 rows x 1024 threads, 1 CTA/SM
//   2: 1 row  x 512 threads, 2 CTAs/SM    3: 4 rows x 1024 threads, 1 CTA/SM
//   4: 1 row  x 384 threads, 2 CTAs/SM    5: 1 row  x 256 threads, 3 CTAs/SM
//   6: 1 row  x 256 threads, 2 CTAs/SM
// (4 and 5 trade occupancy for up to 80 registers per thread, 6 for up to 128:
// no spills).
struct FarShape {
    int tr, nt;
};
constexpr FarShape kFarShapes[] = {{2, 512}, {2, 1024}, {1, 512}, {4, 1024}, {1, 384}, {1, 256}, {1, 256}};
constexpr int kNumFarShapes = 7;

int far_variants(int prec) { return prec == BEM_PREC_C64 ? kNumFarShapes : 1; }

int far_rows_per_cta(int prec, int variant) {
    return prec == BEM_PREC_C64 ? kFarShapes[variant].tr : 1;
}

// c64: the rows' accumulators (tr x tc) and each thread's c and beta sums of
// its rows (3 x tr x nt floats); c128: one row's accumulators.
size_t far_smem_bytes(int prec, int tc, int variant) {
    return prec == BEM_PREC_C64 ? (size_t)kFarShapes[variant].tr * tc * sizeof(float2) +
                                      (size_t)3 * kFarShapes[variant].tr * kFarShapes[variant].nt * sizeof(float)
                                : (size_t)tc * sizeof(double2);
}

// The dynamic shared-memory limit is an attribute of the kernel function,
// shared by every thread and stream of the process: it is raised once to the
// device's opt-in maximum less the kernel's static shared memory (a launch
// still gets only the bytes it asks for),
// never set per launch, so that concurrent solvers cannot lower it under one
// another's launches.
template <auto Kern>
static void allow_max_smem() {
    static std::once_flag once;   // one per kernel (the kernel is the template argument)
    static cudaError_t err = cudaSuccess;
    std::call_once(once, [&] {
        int dev = 0, maxs = 0;
        err = cudaGetDevice(&dev);
        if (err == cudaSuccess) err = cudaDeviceGetAttribute(&maxs, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        cudaFuncAttributes fa{};
        if (err == cudaSuccess) err = cudaFuncGetAttributes(&fa, Kern);   // static shared memory counts too
        if (err == cudaSuccess)
            err = cudaFuncSetAttribute(Kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       maxs - (int)fa.sharedSizeBytes);
    });
    CUDA_TRY(err);
}

bool far_variant_fits(int prec, int tc, int variant) {
    int dev = 0, maxs = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&maxs, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    return far_smem_bytes(prec, tc, variant) + 1024 <= (size_t)maxs;
}

int far_phase_mode(const Physics &ph) {
    if (ph.k * ph.extent > kAccKd || ph.k * ph.max_edge > kAccKh) return kPhaseAcc;
    if (ph.k * ph.max_edge > kWrapKh) return kPhaseWrap;
    return kPhaseShift;
}

template <int TR, int NT, int MINB>
static void launch_far_f32(const RowPoints &rows, int N, const GeoTables &geo, const TileSet &tiles,
                           const Physics &ph, void *A, size_t lda, void *c_part, void *beta_part,
                           size_t smem, cudaStream_t st) {
    const bool o6 = quadrature_points() == 36;
    const int mode = far_phase_mode(ph);
    decltype(&far_assembly_f32<TR, NT, MINB, true, kPhaseShift, 2>) kern;
#define BEM_FAR_PICK(O6_, PH_, GM_)                                   \
    do {                                                              \
        kern = far_assembly_f32<TR, NT, MINB, O6_, PH_, GM_>;          \
        allow_max_smem<far_assembly_f32<TR, NT, MINB, O6_, PH_, GM_>>(); \
    } while (0)
    const int gm = ph.g_sums;
    if (!o6)   // other Gauss orders: always the accurate phase (not the tuned path)
        BEM_FAR_PICK(false, kPhaseAcc, 2);
    else if (mode == kPhaseAcc)
        BEM_FAR_PICK(true, kPhaseAcc, 2);
    else if (mode == kPhaseWrap) {
        if (gm == 2) BEM_FAR_PICK(true, kPhaseWrap, 2);
        else if (gm == 1) BEM_FAR_PICK(true, kPhaseWrap, 1);
        else BEM_FAR_PICK(true, kPhaseWrap, 0);
    } else {
        if (gm == 2) BEM_FAR_PICK(true, kPhaseShift, 2);
        else if (gm == 1) BEM_FAR_PICK(true, kPhaseShift, 1);
        else BEM_FAR_PICK(true, kPhaseShift, 0);
    }
#undef BEM_FAR_PICK
    const float kh = (float)ph.k, kl = (float)(ph.k - (double)kh);
    dim3 grid((rows.R + TR - 1) / TR, tiles.ntiles);
    kern<<<grid, NT, smem, st>>>(rows, N, geo, tiles, kh, kl, (float)ph.rw, (float2 *)A, lda,
                                 (float *)c_part, (float2 *)beta_part);
}

__global__ void far_recs_kernel(const TileRec *__restrict__ recs, int nrec, const float4 *__restrict__ geo_f,
                                FarRec *__restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nrec) return;
    const TileRec r = recs[i];
    FarRec f;
#pragma unroll
    for (int k = 0; k < kFarRecG; k++) f.g[k] = geo_f[(size_t)kGeoF * r.eid + k];
    f.nodes = make_int4(r.node[0], r.node[1], r.node[2], r.owner);
    f.slots = make_int4(r.slot[0], r.slot[1], r.slot[2], 0);
    out[i] = f;
}

void launch_far_recs(const TileRec *recs, int nrec, const float4 *geo_f, FarRec *frecs, cudaStream_t st) {
    static_assert(sizeof(FarRec) == 16 * (kFarRecG + 2) && kGeoF >= kFarRecG, "far record layout");
    if (nrec <= 0) return;
    far_recs_kernel<<<(nrec + 255) / 256, 256, 0, st>>>(recs, nrec, geo_f, frecs);
    count_launch();
    KERNEL_CHECK();
}

void launch_far_assembly(int prec, const RowPoints &rows, int N, const GeoTables &geo,
                         const TileSet &tiles, const Physics &ph, void *A, size_t lda,
                         void *c_part, void *beta_part, cudaStream_t st, int variant) {
    BEM_PROF((prec == BEM_PREC_C64 ? "far_assembly_f32" : "far_assembly_f64"), st);
    if (rows.R <= 0 || tiles.ntiles <= 0) return;
    BEM_CHECK_ARG(variant >= 0 && variant < far_variants(prec), "bad far-kernel variant");
    if (!far_variant_fits(prec, tiles.tc_max, variant))
        BEM_FAIL(BEM_ERR_TOO_LARGE, "column tile does not fit in shared memory");
    const size_t smem = far_smem_bytes(prec, tiles.tc_max, variant);
    if (prec == BEM_PREC_C64) {
        BEM_CHECK_ARG(tiles.frecs != nullptr, "far kernel: records with geometry not formed");
        switch (variant) {
            case 0: launch_far_f32<2, 512, 1>(rows, N, geo, tiles, ph, A, lda, c_part, beta_part, smem, st); break;
            case 1: launch_far_f32<2, 1024, 1>(rows, N, geo, tiles, ph, A, lda, c_part, beta_part, smem, st); break;
            case 2: launch_far_f32<1, 512, 2>(rows, N, geo, tiles, ph, A, lda, c_part, beta_part, smem, st); break;
            case 3: launch_far_f32<4, 1024, 1>(rows, N, geo, tiles, ph, A, lda, c_part, beta_part, smem, st); break;
            case 4: launch_far_f32<1, 384, 2>(rows, N, geo, tiles, ph, A, lda, c_part, beta_part, smem, st); break;
            case 5: launch_far_f32<1, 256, 3>(rows, N, geo, tiles, ph, A, lda, c_part, beta_part, smem, st); break;
            default: launch_far_f32<1, 256, 2>(rows, N, geo, tiles, ph, A, lda, c_part, beta_part, smem, st); break;
        }
    } else {
        auto kern = far_assembly_f64<kFarNT64>;
        allow_max_smem<far_assembly_f64<kFarNT64>>();
        dim3 grid(rows.R, tiles.ntiles);
        kern<<<grid, kFarNT64, smem, st>>>(rows, N, geo, tiles, ph.k, ph.rw, (double2 *)A, lda,
                                           (double *)c_part, (double2 *)beta_part);
    }
    count_launch();
    KERNEL_CHECK();
}

// ---------------------------------------------------------------------------
// FP64 near-pair integration by one warp.
// Leaves: sub-triangles (parent local vertices va, vb, vc) with a Duffy map
// collapsed at vertex `collapse` (1, 2, 3).  Singular pairs use one leaf, the
// whole element with the map collapsed at x's vertex (g/h/c_l_sgl1..3,
// mesh.cu:253-595).  Near-singular pairs subdivide the element into four at
// edge midpoints while dist(x, sub-centroid) < eta * sub-diameter, up to
// near_depth levels, and use the regular map on every leaf.
// ---------------------------------------------------------------------------
constexpr int kMaxDepth = 4;
constexpr int kMaxLeaves = 256;        // 4^kMaxDepth
constexpr int kNearWarps = 4;

// A leaf triangle in the element's (xi1, xi2) coordinates; its corners are
// multiples of 2^-depth (depth <= 4), exact in float.
// A leaf triangle in the element's reference coordinates (corners a, b, c;
// dyadic fractions from midpoint subdivision, exact in float).
// near_integrate turns a and b into the edges a - c, b - c in place and
// fills area = |det(a - c, b - c)|, all exact in float.
struct Leaf {
    float a[2], b[2], c[2];
    float area;
};

struct NearOut {
    double gr[3], gi[3], hr[3], hi[3], c;
};

__device__ __forceinline__ void xi_point(const double *h, double x1, double x2, double *y) {
    for (int d = 0; d < 3; d++) y[d] = h[d] + x1 * h[3 + d] + x2 * h[6 + d];
}

// Corners of the sub-triangle reached from the element by the child indices
// in code (two bits per level, level i in bits 2i..2i+1); children of (a, b, c)
// are (a,ab,ca), (ab,b,bc), (ca,bc,c), (ab,bc,ca).
__device__ __forceinline__ Leaf leaf_from_code(int code, int depth) {
    float ax = 1.f, ay = 0.f, bx = 0.f, by = 1.f, cx = 0.f, cy = 0.f;
    for (int i = 0; i < depth; i++) {
        const int k = (code >> (2 * i)) & 3;
        const float abx = 0.5f * (ax + bx), aby = 0.5f * (ay + by);
        const float bcx = 0.5f * (bx + cx), bcy = 0.5f * (by + cy);
        const float cax = 0.5f * (cx + ax), cay = 0.5f * (cy + ay);
        if (k == 0) { bx = abx; by = aby; cx = cax; cy = cay; }
        else if (k == 1) { ax = abx; ay = aby; cx = bcx; cy = bcy; }
        else if (k == 2) { ax = cax; ay = cay; bx = bcx; by = bcy; }
        else { ax = abx; ay = aby; bx = bcx; by = bcy; cx = cax; cy = cay; }
    }
    return Leaf{{ax, ay}, {bx, by}, {cx, cy}};
}

// The leaf list of a near-singular pair, built by the whole warp breadth
// first: at each level the lanes test the frontier's triangles in parallel
// (split while |centroid - x| < eta * diameter and depth < depth_max, as the
// reference-style recursion does), leaves and children are compacted with
// ballots.  cur/nxt: per-warp scratch of kMaxLeaves codes each.  Returns the
// number of leaves in every lane.
// With fast32 (the c64 assembly) the split test is first evaluated in FP32
// as |c - x|^2 against (eta d)^2 from the pair's offset p3 - x (rounded from
// FP64) and the element's edges; outside a relative band of 1e-4 around the
// threshold (FP32's error here is a few 1e-6) that decides, inside it the
// FP64 test below does, so the leaves are the FP64 rule's.
// A near pair's geometry for the FP32 path, in double float on the FP32 pipe
// from the element table's heads and tails and the row point's head and tail
// (no FP64 operation): d3 = p3 - x, e1, e2 as head + tail, the height of x
// over the element (d3 . n) and |J| / (4 pi).
struct PairGeoF {
    float dh[3], dl[3], e1h[3], e1l[3], e2h[3], e2l[3];
    float hgt, scale;
};
__device__ __forceinline__ PairGeoF pair_geo_f(const float4 *__restrict__ gf, float4 xh, float4 xl) {
    const float4 g0 = gf[0], g1 = gf[1], g2 = gf[2], g3 = gf[3], g4 = gf[4], g6 = gf[6], g7 = gf[7], g8 = gf[8];
    PairGeoF p;
    const float ph[3] = {g0.x, g0.y, g0.z}, pl[3] = {g1.x, g1.y, g1.z};
    const float xhh[3] = {xh.x, xh.y, xh.z}, xll[3] = {xl.x, xl.y, xl.z};
    const float nh[3] = {g4.x, g4.y, g4.z}, nt[3] = {g7.w, g8.w, g6.w};
    p.e1h[0] = g2.x; p.e1h[1] = g2.y; p.e1h[2] = g2.z;
    p.e2h[0] = g3.x; p.e2h[1] = g3.y; p.e2h[2] = g3.z;
    p.e1l[0] = g7.x; p.e1l[1] = g7.y; p.e1l[2] = g7.z;
    p.e2l[0] = g8.x; p.e2l[1] = g8.y; p.e2l[2] = g8.z;
    float hh = 0.f, hl = 0.f;
#pragma unroll
    for (int a = 0; a < 3; a++) {
        float e;
        p.dh[a] = two_sum(ph[a], -xhh[a], e);
        p.dl[a] = __fadd_rn(e, __fsub_rn(pl[a], xll[a]));
        const float pr = __fmul_rn(p.dh[a], nh[a]), pe = __fmaf_rn(p.dh[a], nh[a], -pr);
        float t;
        hh = two_sum(hh, pr, t);
        hl += t + pe + p.dh[a] * nt[a] + p.dl[a] * nh[a];
    }
    p.hgt = hh + hl;
    p.scale = g0.w * (float)(1.0 / (4.0 * kPi));
    return p;
}

// The warp's leaves of a near-singular pair.  fast32: the split tests in FP32
// from the pair's double-float geometry (pg), with the FP64 test on h and x
// inside a relative guard band of the threshold.
template <bool fast32>
__device__ int build_leaves_warp(const double *h, const double *x, double eta, int depth_max, Leaf *leaves,
                                 int *cur, int *nxt, const PairGeoF *pg = nullptr) {
    const int lane = threadIdx.x & 31;
    const unsigned below = (1u << lane) - 1u;
    if (lane == 0) cur[0] = 0;
    __syncwarp();
    int ncur = 1, nl = 0;
    float3 d3f = make_float3(0.f, 0.f, 0.f), e1f = d3f, e2f = d3f;
    if (fast32) {
        d3f = make_float3(pg->dh[0] + pg->dl[0], pg->dh[1] + pg->dl[1], pg->dh[2] + pg->dl[2]);
        e1f = make_float3(pg->e1h[0], pg->e1h[1], pg->e1h[2]);
        e2f = make_float3(pg->e2h[0], pg->e2h[1], pg->e2h[2]);
    }
    const float eta2f = fast32 ? (float)eta * (float)eta : 0.f;
    for (int depth = 0; depth <= depth_max && ncur > 0; depth++) {
        int nnext = 0;
        for (int base = 0; base < ncur; base += 32) {
            const int i = base + lane;
            const bool valid = i < ncur;
            const int code = valid ? cur[i] : 0;
            const Leaf t = leaf_from_code(code, depth);
            bool split = false;
            bool decided = false;
            if (fast32 && valid && depth < depth_max) {
                auto sq = [&](float u1, float u2) {   // |u1 e1 + u2 e2|^2
                    const float vx = fmaf(u2, e2f.x, u1 * e1f.x), vy = fmaf(u2, e2f.y, u1 * e1f.y),
                                vz = fmaf(u2, e2f.z, u1 * e1f.z);
                    return fmaf(vz, vz, fmaf(vy, vy, vx * vx));
                };
                const float lab = sq(t.a[0] - t.b[0], t.a[1] - t.b[1]);
                const float lbc = sq(t.b[0] - t.c[0], t.b[1] - t.c[1]);
                const float lca = sq(t.c[0] - t.a[0], t.c[1] - t.a[1]);
                const float c1 = (t.a[0] + t.b[0] + t.c[0]) * (1.0f / 3.0f), c2 = (t.a[1] + t.b[1] + t.c[1]) * (1.0f / 3.0f);
                const float qx = fmaf(c2, e2f.x, fmaf(c1, e1f.x, d3f.x)), qy = fmaf(c2, e2f.y, fmaf(c1, e1f.y, d3f.y)),
                            qz = fmaf(c2, e2f.z, fmaf(c1, e1f.z, d3f.z));
                const float dc = fmaf(qz, qz, fmaf(qy, qy, qx * qx));
                const float rhs = eta2f * fmaxf(lab, fmaxf(lbc, lca));
                if (fabsf(dc - rhs) > 1e-4f * (dc + rhs)) {
                    split = dc < rhs;
                    decided = true;
                }
            }
            if (!decided && valid && depth < depth_max) {
                double ya[3], yb[3], yc[3], cen[3];
                xi_point(h, t.a[0], t.a[1], ya);
                xi_point(h, t.b[0], t.b[1], yb);
                xi_point(h, t.c[0], t.c[1], yc);
                xi_point(h, ((double)t.a[0] + t.b[0] + t.c[0]) / 3.0, ((double)t.a[1] + t.b[1] + t.c[1]) / 3.0, cen);
                double lab = 0, lbc = 0, lca = 0, dc = 0;
                for (int d = 0; d < 3; d++) {
                    lab += (ya[d] - yb[d]) * (ya[d] - yb[d]);
                    lbc += (yb[d] - yc[d]) * (yb[d] - yc[d]);
                    lca += (yc[d] - ya[d]) * (yc[d] - ya[d]);
                    dc += (cen[d] - x[d]) * (cen[d] - x[d]);
                }
                split = sqrt(dc) < eta * sqrt(fmax(lab, fmax(lbc, lca)));
            }
            const unsigned mleaf = __ballot_sync(0xffffffffu, valid && !split);
            const unsigned msplit = __ballot_sync(0xffffffffu, split);
            if (valid && !split) {
                const int pos = nl + __popc(mleaf & below);
                if (pos < kMaxLeaves) leaves[pos] = t;
            }
            if (split) {
                const int pos = nnext + 4 * __popc(msplit & below);
                for (int c = 0; c < 4; c++) nxt[pos + c] = code | (c << (2 * depth));
            }
            nl += __popc(mleaf);
            nnext += 4 * __popc(msplit);
        }
        __syncwarp();
        int *tmp = cur;
        cur = nxt;
        nxt = tmp;
        ncur = nnext;
    }
    return min(nl, kMaxLeaves);
}

// Warp-cooperative FP64 integration over the leaves; the result is valid in
// every lane.  Returns g (before the i*rho*omega factor), h, c, scaled by
// |J|/(4 pi) as in the far path.
// sin and cos in FP64 for the near-field quadrature: quadrant j = round(2y/pi),
// z = y - j pi/2 by a three-constant Cody-Waite reduction with FMAs (P1 =
// fl(pi/2), P2 = fl(pi/2 - P1), P3 = fl(pi/2 - P1 - P2)), then on |z| <= pi/4,
// with u = z^2,  sin z = z + z^3 P(u)  and  cos z = 1 - u/2 + u^2 Q(u)  with
// P, Q of degree 5: Chebyshev interpolants of the exact functions on
// [0, (pi/4)^2] (P(u) = (sin sqrt(u) - sqrt(u)) / u^1.5, Q(u) = (cos sqrt(u)
// - 1 + u/2) / u^2), interpolated at the 6 Chebyshev nodes of that interval
// in 60-digit arithmetic, converted to monomial coefficients and rounded to
// double (maximum error of the double-evaluated Horner schemes on a dense
// grid: 7e-17 for sin, 1.2e-16 for cos), and the
// quadrant's swap and signs.  Near pairs have kr of order one, so the
// reduction is short and exact; this replaces the general-argument library
// call on the FP64 pipe, which GB300 runs at ~1/64 of FP32.
__device__ __forceinline__ void sincos_near(double y, double *sn, double *cs) {
    const double j = rint(y * 0.6366197723675814);
    double z = fma(-j, 1.5707963267948966, y);
    z = fma(-j, 6.123233995736766e-17, z);
    z = fma(-j, -1.4973849048591698e-33, z);
    const double u = z * z;
    double ps = 1.5918129294866608e-10;
    ps = fma(ps, u, -2.5051131845003624e-08);
    ps = fma(ps, u, 2.755731610255244e-06);
    ps = fma(ps, u, -0.00019841269836758574);
    ps = fma(ps, u, 0.008333333333330948);
    ps = fma(ps, u, -0.16666666666666666);
    ps = fma(ps * u, z, z);
    double pc = -1.1382632425521717e-11;
    pc = fma(pc, u, 2.08761462684032e-09);
    pc = fma(pc, u, -2.7557317271729793e-07);
    pc = fma(pc, u, 2.480158729876569e-05);
    pc = fma(pc, u, -0.0013888888888887398);
    pc = fma(pc, u, 0.041666666666666664);
    pc = fma(pc, u * u, fma(-0.5, u, 1.0));
    const unsigned q = (unsigned)((long long)j & 3);
    const double s0 = (q & 1u) ? pc : ps, c0 = (q & 1u) ? ps : pc;
    *sn = (q & 2u) ? -s0 : s0;
    *cs = ((q + 1u) & 2u) ? -c0 : c0;
}

__device__ void near_integrate(const double *h, const double *x, double k, int collapse,
                               const Leaf *leaves, int nl, int nq, NearOut &o) {
    const int lane = threadIdx.x & 31;
    double acc[13];
#pragma unroll
    for (int i = 0; i < 13; i++) acc[i] = 0.0;
    const double *n = h + 9;
    const int cv = collapse - 1;
    // per leaf once: edges and area (exact in float; the leaves are rebuilt
    // for every pair, so they are changed in place)
    for (int l = lane; l < nl; l += 32) {
        Leaf &t = const_cast<Leaf &>(leaves[l]);
        const float ea0 = t.a[0] - t.c[0], ea1 = t.a[1] - t.c[1];
        const float eb0 = t.b[0] - t.c[0], eb1 = t.b[1] - t.c[1];
        t.a[0] = ea0;
        t.a[1] = ea1;
        t.b[0] = eb0;
        t.b[1] = eb1;
        t.area = fabsf(ea0 * eb1 - ea1 * eb0);
    }
    __syncwarp();
    const double d3[3] = {h[0] - x[0], h[1] - x[1], h[2] - x[2]};
    // dr/dn = (d . n)/r with d . n = d3 . n for every point of the flat
    // element (its edges are orthogonal to n): the height leaves the sums,
    //   4 pi dG/dn = -hgt (gr + k s + i (k c - gs)) / r^2,  4 pi dG0/dn = -hgt / r^3
    // (gr = c/r, gs = s/r), as in the far-field sums.
    const double hgt = d3[0] * n[0] + d3[1] * n[1] + d3[2] * n[2];
    for (int idx = lane; idx < nl * nq; idx += 32) {
        const int l = idx / nq, q = idx - l * nq;
        const Leaf &t = leaves[l];
        const double ea0 = t.a[0], ea1 = t.a[1], eb0 = t.b[0], eb1 = t.b[1];
        double s1 = c_qd[cv][q][0], s2 = c_qd[cv][q][1], w = c_qd[cv][q][2] * (double)t.area;
        double x1 = t.c[0] + s1 * ea0 + s2 * eb0;
        double x2 = t.c[1] + s1 * ea1 + s2 * eb1;
        double d[3];
        for (int dd = 0; dd < 3; dd++) d[dd] = d3[dd] + x1 * h[3 + dd] + x2 * h[6 + dd];
        const double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
        const double ri = rsqrt(r2);
        const double r = r2 * ri;
        double sn, cs;
        sincos_near(k * r, &sn, &cs);
        const double ri2 = ri * ri;
        const double gr = cs * ri, gs = sn * ri;
        const double ha = ri2 * fma(k, sn, gr), hb = ri2 * fma(k, cs, -gs);
        const double ri3 = ri2 * ri;
        const double wn[3] = {w * x1, w * x2, w * (1.0 - x1 - x2)};
#pragma unroll
        for (int j = 0; j < 3; j++) {
            acc[j] += wn[j] * gr;
            acc[3 + j] += wn[j] * gs;
            acc[6 + j] += wn[j] * ha;
            acc[9 + j] += wn[j] * hb;
        }
        acc[12] += w * ri3;
    }
#pragma unroll
    for (int i = 0; i < 13; i++)
        for (int off = 16; off > 0; off >>= 1) acc[i] += __shfl_xor_sync(0xffffffffu, acc[i], off);
    // signs and the height: G = (gr, -gs), dG/dn = -hgt (ha, hb), dG0/dn = -hgt ri3
#pragma unroll
    for (int j = 0; j < 3; j++) acc[3 + j] = -acc[3 + j];
#pragma unroll
    for (int i = 6; i < 13; i++) acc[i] *= -hgt;
    const double scale = h[12] / (4.0 * kPi);
    for (int j = 0; j < 3; j++) {
        o.gr[j] = scale * acc[j];
        o.gi[j] = scale * acc[3 + j];
        o.hr[j] = scale * acc[6 + j];
        o.hi[j] = scale * acc[9 + j];
    }
    o.c = scale * acc[12];
}

// The same integrals for the c64 assembly with FP32 point arithmetic (the
// FP64 pipe runs at ~1/64 of FP32 on this part).  The pair's geometry is
// prepared in FP64 so that no FP32 difference cancels:
//   * singular pair (x is vertex v of the element, one leaf): d = dxi1 e1 +
//     dxi2 e2 with the point's offsets from v (c_qs, formed in double), and
//     the FP64 remainder p_v - x (zero up to the rounding of the edges);
//   * near-singular leaf: d = d_l + s1 E1 + s2 E2 with d_l = (leaf corner -
//     x) and the leaf's edge vectors E1, E2 formed in FP64 per leaf, so d's
//     rounding is relative to the leaf's size, which the subdivision keeps
//     comparable to r.
// sin and cos are CUDA's full-accuracy sincosf (k r is of order one here),
// the 13 sums are compensated (TwoSum with round-to-nearest intrinsics, so
// nothing is contracted), also across the warp's lanes.  At most
// kNearF32Leaves leaves (their FP32 data go into the warp's leaf-code
// scratch, free once the leaves are built); the caller takes the FP64
// routine beyond that.
constexpr int kNearF32Leaves = 48;
constexpr int kNearLeafF = 10;   // floats per leaf: d_l (3), E1 (3), E2 (3), area
static_assert(kNearF32Leaves * kNearLeafF <= 2 * kMaxLeaves, "leaf data fit the leaf-code scratch");

__device__ __forceinline__ void ksum(float &s, float &c, float t) {
    const float u = __fadd_rn(s, t), bb = __fsub_rn(u, s);
    c = __fadd_rn(c, __fadd_rn(__fsub_rn(s, __fsub_rn(u, bb)), __fsub_rn(t, bb)));
    s = u;
}

// Outputs of the FP32 near integration: the dG/dn parts of the three A
// coefficients in FP32 (the c64 entries they are added to are FP32), the G
// sums (for beta and bcA terms) in FP64, and the pair's free-term
// contribution (formed in FP32, added to the row's FP64 sum).
struct NearOutF {
    float hr[3], hi[3];
    double gr[3], gi[3], c;
};

// GM as in far_sums_f32_o6x2: the G sums are formed only when some BC needs
// them (GM > 0).  The pair geometry comes in double float (PairGeoF); no FP64
// operation is left per pair but those of the G sums.
template <int GM>
__device__ void near_integrate_f32(const double *h, const PairGeoF &pg, float kf, int collapse, bool sing,
                                   const Leaf *leaves, int nl, int nq, float *lg, NearOutF &o) {
    const int lane = threadIdx.x & 31;
    const float3 e1 = make_float3(pg.e1h[0], pg.e1h[1], pg.e1h[2]);
    const float3 e2 = make_float3(pg.e2h[0], pg.e2h[1], pg.e2h[2]);
    const int cv = collapse - 1;
    // u e1 + v e2 + w (head, tail) as a float, in double float: u and v are
    // exact floats with few bits (0, 1 or dyadic leaf coordinates), so the
    // heads' products are split exactly (TwoProduct) and summed by TwoSum
    auto comb = [&](float u, float v, float wh, float wl, int a) {
        const float p1 = __fmul_rn(u, pg.e1h[a]), q1 = __fmaf_rn(u, pg.e1h[a], -p1);
        const float p2 = __fmul_rn(v, pg.e2h[a]), q2 = __fmaf_rn(v, pg.e2h[a], -p2);
        float t1, t2;
        const float s1 = two_sum(wh, p1, t1);
        const float s2 = two_sum(s1, p2, t2);
        return s2 + (wl + q1 + q2 + t1 + t2 + u * pg.e1l[a] + v * pg.e2l[a]);
    };
    float3 dv = make_float3(0.f, 0.f, 0.f);   // singular: p_v - x
    if (sing) {
        const float v1 = cv == 0 ? 1.f : 0.f, v2 = cv == 1 ? 1.f : 0.f;
        dv = make_float3(comb(v1, v2, pg.dh[0], pg.dl[0], 0), comb(v1, v2, pg.dh[1], pg.dl[1], 1),
                         comb(v1, v2, pg.dh[2], pg.dl[2], 2));
    } else {
        // per leaf (lanes over leaves): the corner's offset d_l and the edges
        // E1, E2 in double float, then float; the corners are dyadic, so the
        // edge coordinates and the area are exact in float
        for (int l = lane; l < nl; l += 32) {
            const Leaf t = leaves[l];
            const float ea0 = t.a[0] - t.c[0], ea1 = t.a[1] - t.c[1];
            const float eb0 = t.b[0] - t.c[0], eb1 = t.b[1] - t.c[1];
            float *g = lg + (size_t)l * kNearLeafF;
#pragma unroll
            for (int dd = 0; dd < 3; dd++) {
                g[dd] = comb(t.c[0], t.c[1], pg.dh[dd], pg.dl[dd], dd);
                g[3 + dd] = comb(ea0, ea1, 0.f, 0.f, dd);
                g[6 + dd] = comb(eb0, eb1, 0.f, 0.f, dd);
            }
            g[9] = fabsf(__fsub_rn(__fmul_rn(ea0, eb1), __fmul_rn(ea1, eb0)));
        }
        __syncwarp();
    }
    float s[13], c[13];
#pragma unroll
    for (int i = 0; i < 13; i++) s[i] = c[i] = 0.f;
    for (int idx = lane; idx < nl * nq; idx += 32) {
        const int l = idx / nq, q = idx - l * nq;
        float3 d;
        float x1, x2, w;
        if (sing) {
            const float4 t = c_qs[cv][q];
            d = make_float3(fmaf(t.y, e2.x, fmaf(t.x, e1.x, dv.x)), fmaf(t.y, e2.y, fmaf(t.x, e1.y, dv.y)),
                            fmaf(t.y, e2.z, fmaf(t.x, e1.z, dv.z)));
            x1 = (cv == 0 ? 1.f : 0.f) + t.x;
            x2 = (cv == 1 ? 1.f : 0.f) + t.y;
            w = t.z;
        } else {
            const float4 t = c_qf[q];
            const float *g = lg + (size_t)l * kNearLeafF;
            d = make_float3(fmaf(t.y, g[6], fmaf(t.x, g[3], g[0])), fmaf(t.y, g[7], fmaf(t.x, g[4], g[1])),
                            fmaf(t.y, g[8], fmaf(t.x, g[5], g[2])));
            const Leaf &lf = leaves[l];
            x1 = fmaf(t.y, lf.b[0] - lf.c[0], fmaf(t.x, lf.a[0] - lf.c[0], lf.c[0]));
            x2 = fmaf(t.y, lf.b[1] - lf.c[1], fmaf(t.x, lf.a[1] - lf.c[1], lf.c[1]));
            w = t.z * g[9];
        }
        const float r2 = fmaf(d.z, d.z, fmaf(d.y, d.y, d.x * d.x));
        const float r = sqrtf(r2), ri = 1.0f / r;
        float sn, cs;
        sincosf(kf * r, &sn, &cs);
        const float ri2 = ri * ri;
        const float gr = cs * ri, gs = sn * ri;
        const float ha = ri2 * fmaf(kf, sn, gr), hb = ri2 * fmaf(kf, cs, -gs);
        const float ri3 = ri2 * ri;
        const float wn[3] = {w * x1, w * x2, w * (1.0f - x1 - x2)};
#pragma unroll
        for (int j = 0; j < 3; j++) {
            if constexpr (GM == 2) {
                ksum(s[j], c[j], wn[j] * gr);
                ksum(s[3 + j], c[3 + j], wn[j] * gs);
            }
            ksum(s[6 + j], c[6 + j], wn[j] * ha);
            ksum(s[9 + j], c[9 + j], wn[j] * hb);
        }
        if constexpr (GM == 1) {   // beta needs sum_j g_j only: the weights' sum is w
            ksum(s[0], c[0], w * gr);
            ksum(s[3], c[3], w * gs);
        }
        ksum(s[12], c[12], w * ri3);
    }
    // lanes' (sum, compensation) pairs added by TwoSum across the warp, in FP32
#pragma unroll
    for (int i = GM > 0 ? 0 : 6; i < 13; i++) {
        if (GM == 1 && (i == 1 || i == 2 || i == 4 || i == 5)) continue;
        float hi = s[i], lo = c[i];
        for (int off = 16; off > 0; off >>= 1) {
            const float h2 = __shfl_xor_sync(0xffffffffu, hi, off), l2 = __shfl_xor_sync(0xffffffffu, lo, off);
            ksum(hi, lo, h2);
            lo = __fadd_rn(lo, l2);
        }
        s[i] = hi;
        c[i] = lo;
    }
    // signs, height and scale: G = (gr, -gs), dG/dn = -hgt (ha, hb), dG0/dn =
    // -hgt ri3; the dG/dn coefficients and the free-term contribution in FP32
    // from the heads and tails (the entries they go into are FP32)
    const float fsh = -pg.hgt * pg.scale;
#pragma unroll
    for (int j = 0; j < 3; j++) {
        o.hr[j] = fmaf(fsh, s[6 + j], fsh * c[6 + j]);
        o.hi[j] = fmaf(fsh, s[9 + j], fsh * c[9 + j]);
        if (GM == 2 || (GM == 1 && j == 0)) {   // GM = 1: the sum over j in entry 0
            const double scale = h[12] * (1.0 / (4.0 * kPi));   // beta's terms stay FP64
            o.gr[j] = scale * ((double)s[j] + (double)c[j]);
            o.gi[j] = -scale * ((double)s[3 + j] + (double)c[3 + j]);
        } else {
            o.gr[j] = o.gi[j] = 0.0;
        }
    }
    o.c = fmaf(fsh, s[12], fsh * c[12]);
}

__device__ __forceinline__ double2 incident_field(const DevSource &s, double k, const double *x) {
    double ph, amp_scale = 1.0;
    if (s.kind == BEM_SRC_PLANE) {
        ph = -k * (s.vec[0] * x[0] + s.vec[1] * x[1] + s.vec[2] * x[2]);
    } else {
        double dx = x[0] - s.vec[0], dy = x[1] - s.vec[1], dz = x[2] - s.vec[2];
        double r = sqrt(dx * dx + dy * dy + dz * dz);
        ph = -k * r;
        amp_scale = 1.0 / (4.0 * kPi * r);
    }
    double sn, cs;
    sincos(ph, &sn, &cs);
    cs *= amp_scale;
    sn *= amp_scale;
    return make_double2(s.amp_re * cs - s.amp_im * sn, s.amp_re * sn + s.amp_im * cs);
}

template <typename TA> __device__ __forceinline__ void add_entry(TA *p, double re, double im);
template <> __device__ __forceinline__ void add_entry<float2>(float2 *p, double re, double im) {
    float2 v = *p;
    *p = make_float2((float)((double)v.x + re), (float)((double)v.y + im));
}
template <> __device__ __forceinline__ void add_entry<double2>(double2 *p, double re, double im) {
    double2 v = *p;
    *p = make_double2(v.x + re, v.y + im);
}

// GM: which G sums the BCs need (as in far_sums_f32_o6x2), used by the c64
// (TA = float2) FP32 path; the c128 kernel is instantiated with GM = 2.
template <typename TA, typename TP, typename TP2, int GM>
__global__ void __launch_bounds__(32 * kNearWarps, 4)
near_assembly_kernel(RowPoints rows, int N, GeoTables geo, Physics ph, int nq, TA *__restrict__ A,
                     size_t lda, const TP *__restrict__ c_part, const TP2 *__restrict__ beta_part,
                     int ntiles, const DevSource *__restrict__ srcs, int S, double2 *__restrict__ B,
                     double2 *__restrict__ beta_out, const int *__restrict__ near_ptr,
                     const int *__restrict__ near_ids) {
    __shared__ Leaf leaves_all[kNearWarps][kMaxLeaves];
    __shared__ int codes_all[kNearWarps][2][kMaxLeaves];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int row = blockIdx.x * kNearWarps + warp;
    if (row >= rows.R) return;
    Leaf *leaves = leaves_all[warp];
    const double x[3] = {rows.d[3 * (size_t)row], rows.d[3 * (size_t)row + 1], rows.d[3 * (size_t)row + 2]};
    constexpr bool f32 = std::is_same<TA, float2>::value;
    float4 xh = make_float4(0.f, 0.f, 0.f, 0.f), xl = xh;   // the row point's head and tail (FP32 path)
    if (f32) {
        xh = rows.f[2 * (size_t)row];
        xl = rows.f[2 * (size_t)row + 1];
    }
    const float kf = (float)ph.k;
    double cn = 0.0, bnr = 0.0, bni = 0.0;
    // The row's near elements, in increasing element order (near_list_kernel).
    const int pe = near_ptr[row + 1];
    for (int p0 = near_ptr[row]; p0 < pe; p0 += 32) {
        const int cnt = min(32, pe - p0);
        int ebl = 0;
        int4 nd = make_int4(-1, -1, -1, 0);
        if (lane < cnt) {
            ebl = near_ids[p0 + lane];
            nd = geo.elems[ebl];
        }
        for (int b = 0; b < cnt; b++) {
            const int eb = __shfl_sync(0xffffffffu, ebl, b);
            const int4 ndb = make_int4(__shfl_sync(0xffffffffu, nd.x, b), __shfl_sync(0xffffffffu, nd.y, b),
                                       __shfl_sync(0xffffffffu, nd.z, b), 0);
            const double *h = geo.geo_d + (size_t)kGeoD * eb;
            int collapse = 3, nl = 1;
            const int vtx = (row < N) ? (row == ndb.x ? 1 : row == ndb.y ? 2 : row == ndb.z ? 3 : 0) : 0;
            const float4 *gfe = geo.geo_f + (size_t)kGeoF * eb;
            if (vtx) {
                collapse = vtx;
                if (lane == 0) leaves[0] = {{1.f, 0.f}, {0.f, 1.f}, {0.f, 0.f}};
            } else {
                PairGeoF pg0;   // (formed again below rather than kept live through the leaf builder)
                if (f32) pg0 = pair_geo_f(gfe, xh, xl);
                nl = build_leaves_warp<f32>(h, x, ph.near_eta, ph.near_depth, leaves, codes_all[warp][0],
                                            codes_all[warp][1], &pg0);
            }
            __syncwarp();
            NearOut o;
            const int node[3] = {ndb.x, ndb.y, ndb.z};
            if (f32 && nl <= kNearF32Leaves) {
                NearOutF of;
                const PairGeoF pg = pair_geo_f(gfe, xh, xl);
                near_integrate_f32<GM>(h, pg, kf, collapse, vtx != 0, leaves, nl, nq,
                                       reinterpret_cast<float *>(&codes_all[warp][0][0]), of);
                __syncwarp();
                if constexpr (GM < 2 && std::is_same<TA, float2>::value) {
                    // bcA = 0: the coefficients are the dG/dn parts, added in
                    // FP32 to the FP32 entries (one rounding, as the FP64 add
                    // and conversion gave)
                    if (lane == 0) {
                        double sgr = 0, sgi = 0;
                        for (int j = 0; j < 3; j++) {
                            float2 *p = A + (size_t)row * lda + node[j];
                            const float2 v = *p;
                            *p = make_float2(__fadd_rn(v.x, of.hr[j]), __fadd_rn(v.y, of.hi[j]));
                            if constexpr (GM == 1) {
                                sgr -= ph.rw * of.gi[j];
                                sgi += ph.rw * of.gr[j];
                            }
                        }
                        if (row < N) cn += of.c;
                        if constexpr (GM == 1) {
                            const double bCr = h[15], bCi = h[16];
                            bnr += bCr * sgr - bCi * sgi;
                            bni += bCr * sgi + bCi * sgr;
                        }
                    }
                    continue;
                }
                for (int j = 0; j < 3; j++) {
                    o.hr[j] = of.hr[j];
                    o.hi[j] = of.hi[j];
                    o.gr[j] = of.gr[j];
                    o.gi[j] = of.gi[j];
                }
                o.c = of.c;
            } else {
                near_integrate(h, x, ph.k, collapse, leaves, nl, nq, o);
                __syncwarp();
            }
            if (lane == 0) {
                const double bAr = h[13], bAi = h[14], bCr = h[15], bCi = h[16];
                double sgr = 0, sgi = 0;
                for (int j = 0; j < 3; j++) {
                    double g_r = -ph.rw * o.gi[j], g_i = ph.rw * o.gr[j];
                    double a_r = o.hr[j] - (bAr * g_r - bAi * g_i);
                    double a_i = o.hi[j] - (bAr * g_i + bAi * g_r);
                    add_entry<TA>(A + (size_t)row * lda + node[j], a_r, a_i);
                    sgr += g_r;
                    sgi += g_i;
                }
                if (row < N) cn += o.c;
                bnr += bCr * sgr - bCi * sgi;
                bni += bCr * sgi + bCi * sgr;
            }
        }
    }
    // Finalise the row: diagonal 1 - sum c (surface rows only,
    // atomicFuncs.cu:99-102 and :227-235) and B = p_inc - beta.
    double cf = 0.0, bfr = 0.0, bfi = 0.0;
    if (lane == 0) {
        for (int t = 0; t < ntiles; t++) {
            cf += (double)c_part[(size_t)t * rows.R + row];
            bfr += (double)beta_part[(size_t)t * rows.R + row].x;
            bfi += (double)beta_part[(size_t)t * rows.R + row].y;
        }
        if (row < N) add_entry<TA>(A + (size_t)row * lda + row, 1.0 - (cf + cn), 0.0);
    }
    const double br = __shfl_sync(0xffffffffu, bfr + bnr, 0);
    const double bi = __shfl_sync(0xffffffffu, bfi + bni, 0);
    if (beta_out && lane == 0) beta_out[row] = make_double2(br, bi);
    for (int s = lane; s < S; s += 32) {
        double2 p = incident_field(srcs[s], ph.k, x);
        B[(size_t)s * rows.R + row] = make_double2(p.x - br, p.y - bi);
    }
}

// One thread per (row, source): the same incident field and subtraction as
// the end of near_assembly_kernel.
__global__ void rhs_from_beta_kernel(RowPoints rows, double k, const DevSource *__restrict__ srcs, int S,
                                     const double2 *__restrict__ beta, double2 *__restrict__ B) {
    const int row = blockIdx.x * blockDim.x + threadIdx.x, s = blockIdx.y;
    if (row >= rows.R || s >= S) return;
    const double x[3] = {rows.d[3 * (size_t)row], rows.d[3 * (size_t)row + 1], rows.d[3 * (size_t)row + 2]};
    const double2 b = beta[row];
    const double2 p = incident_field(srcs[s], k, x);
    B[(size_t)s * rows.R + row] = make_double2(p.x - b.x, p.y - b.y);
}

void launch_rhs_from_beta(const RowPoints &rows, double k, const DevSource *srcs, int S, const double2 *beta,
                          double2 *B, cudaStream_t st) {
    BEM_PROF("rhs_from_beta", st);
    if (rows.R <= 0 || S <= 0) return;
    BEM_CHECK_ARG(S <= 65535, "too many sources for one launch");
    rhs_from_beta_kernel<<<dim3((rows.R + 127) / 128, S), 128, 0, st>>>(rows, k, srcs, S, beta, B);
    count_launch();
    KERNEL_CHECK();
}

// Near pairs of every row (the pairs pair_is_near flags, which the far kernel
// skips).  Candidates come from a uniform grid over the element centroids
// whose cell edge is at least the largest near radius and the longest element
// (NearGrid, built on the host): every element that can be near a row point
// has its centroid in the 27 cells around the point's cell, and pair_is_near
// decides exactly as in the far kernel.  Count pass (ids == nullptr:
// cnt[row]) and fill pass (ids[ptr[row]..], cells in fixed order, elements
// in increasing order within a cell).  One warp per row, ballot over 32
// candidates.
__global__ void near_list_kernel(RowPoints rows, int N, GeoTables geo, NearGrid grid, const int *__restrict__ ptr,
                                 int *__restrict__ cnt, int *__restrict__ ids) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int row = blockIdx.x * kNearWarps + warp;
    if (row >= rows.R) return;
    const float4 xh = rows.f[2 * (size_t)row];
    const double *xd = rows.d + 3 * (size_t)row;
    int c[3];
    for (int a = 0; a < 3; a++) {
        const int v = (int)floor((xd[a] - grid.lo[a]) * grid.inv_cell);
        c[a] = min(max(v, 0), grid.dim[a] - 1);
    }
    int n = 0;
    for (int dz = -1; dz <= 1; dz++) {
        const int z = c[2] + dz;
        if (z < 0 || z >= grid.dim[2]) continue;
        for (int dy = -1; dy <= 1; dy++) {
            const int y = c[1] + dy;
            if (y < 0 || y >= grid.dim[1]) continue;
            for (int dx = -1; dx <= 1; dx++) {
                const int x = c[0] + dx;
                if (x < 0 || x >= grid.dim[0]) continue;
                const size_t cell = ((size_t)z * grid.dim[1] + y) * grid.dim[0] + x;
                const int cb = grid.cell_start[cell], ce = grid.cell_start[cell + 1];
                for (int e0 = cb; e0 < ce; e0 += 32) {
                    bool flag = false;
                    int e = 0;
                    if (e0 + lane < ce) {
                        e = grid.cell_elems[e0 + lane];
                        flag = pair_is_near(row, N, geo.elems[e], xh, geo.geo_f + (size_t)kGeoF * e);
                    }
                    const unsigned mask = __ballot_sync(0xffffffffu, flag);
                    if (ids && flag) ids[ptr[row] + n + __popc(mask & ((1u << lane) - 1u))] = e;
                    n += __popc(mask);
                }
            }
        }
    }
    if (!ids && lane == 0) cnt[row] = n;
}

void launch_near_list(const RowPoints &rows, int N, const GeoTables &geo, const NearGrid &grid, const int *d_ptr,
                      int *d_cnt, int *d_ids, cudaStream_t st) {
    if (rows.R <= 0) return;
    const dim3 g((rows.R + kNearWarps - 1) / kNearWarps);
    near_list_kernel<<<g, 32 * kNearWarps, 0, st>>>(rows, N, geo, grid, d_ptr, d_cnt, d_ids);
    count_launch();
    KERNEL_CHECK();
}

void launch_near_assembly(int prec, const RowPoints &rows, int N, const GeoTables &geo,
                          const Physics &ph, void *A, size_t lda, const void *c_part,
                          const void *beta_part, int ntiles, const DevSource *srcs, int S,
                          double2 *B, double2 *beta_out, const int *near_ptr, const int *near_ids,
                          cudaStream_t st) {
    BEM_PROF("near_assembly", st);   // both precisions
    if (rows.R <= 0) return;
    BEM_CHECK_ARG(ph.near_depth >= 0 && ph.near_depth <= kMaxDepth, "near_depth must be in [0, 4]");
    int nq = quadrature_points();
    dim3 grid((rows.R + kNearWarps - 1) / kNearWarps);
    if (prec == BEM_PREC_C64) {
        auto kern = ph.g_sums == 0   ? near_assembly_kernel<float2, float, float2, 0>
                    : ph.g_sums == 1 ? near_assembly_kernel<float2, float, float2, 1>
                                     : near_assembly_kernel<float2, float, float2, 2>;
        kern<<<grid, 32 * kNearWarps, 0, st>>>(rows, N, geo, ph, nq, (float2 *)A, lda, (const float *)c_part,
                                                (const float2 *)beta_part, ntiles, srcs, S, B, beta_out, near_ptr,
                                                near_ids);
    } else {
        near_assembly_kernel<double2, double, double2, 2><<<grid, 32 * kNearWarps, 0, st>>>(
            rows, N, geo, ph, nq, (double2 *)A, lda, (const double *)c_part,
            (const double2 *)beta_part, ntiles, srcs, S, B, beta_out, near_ptr, near_ids);
    }
    count_launch();
    KERNEL_CHECK();
}

// ---------------------------------------------------------------------------
// Field evaluation (genExtPressure / pntElemsOffset, mesh.cu:1008-1073),
// batched: grid (points, element splits), threads over elements, per-thread
// sums for up to kFieldSB sources, block reduction to part[split][p][s].
// ---------------------------------------------------------------------------
constexpr int kFieldNT = 256;
constexpr int kFieldSB = 8;

template <typename T> struct CplxT;
template <> struct CplxT<float> { using t = float2; };
template <> struct CplxT<double> { using t = double2; };

template <typename T>
__global__ void __launch_bounds__(kFieldNT)
field_far_kernel(RowPoints pts, GeoTables geo, T k, T rw, int nq,
                 const typename CplxT<T>::t *__restrict__ u, size_t ldu, int S, int s0, int nsplit,
                 double2 *__restrict__ part) {
    const int p = blockIdx.x, split = blockIdx.y;
    const int per = (geo.E + nsplit - 1) / nsplit;
    const int eb = split * per, ee = min(geo.E, eb + per);
    const float4 xh = pts.f[2 * (size_t)p], xl = pts.f[2 * (size_t)p + 1];
    const double xd[3] = {pts.d[3 * (size_t)p], pts.d[3 * (size_t)p + 1], pts.d[3 * (size_t)p + 2]};
    const int sb = min(kFieldSB, S - s0);
    T accr[kFieldSB], acci[kFieldSB];
#pragma unroll
    for (int s = 0; s < kFieldSB; s++) accr[s] = acci[s] = 0;
    for (int e = eb + threadIdx.x; e < ee; e += kFieldNT) {
        const float4 *g = geo.geo_f + (size_t)kGeoF * e;
        const int4 nd = geo.elems[e];
        if (pair_is_near(-1, 0, nd, xh, g)) continue;
        Coeffs<T, int> o;
        if constexpr (sizeof(T) == 4) {
            const float4 g0 = g[0], g1 = g[1], g2 = g[2], g3 = g[3], g4 = g[4], g5 = g[5];
            float3 d3 = make_float3((g0.x - xh.x) + (g1.x - xl.x), (g0.y - xh.y) + (g1.y - xl.y),
                                    (g0.z - xh.z) + (g1.z - xl.z));
            float hgt = d3.x * g4.x + d3.y * g4.y + d3.z * g4.z;
            SumsF Sm;
            const float3 coff = make_float3(g2.w, g3.w, g4.w);
            const PairPhase pp = pair_phase_shift((float)k, d3, coff);
            far_sums_f32<kPhaseWrap>(d3, make_float3(g2.x, g2.y, g2.z), make_float3(g3.x, g3.y, g3.z), coff, hgt,
                                     (float)k, pp, nq, Sm);
            Coeffs<float, SumsF> oo;
            finish_coeffs<float, SumsF>(Sm, g0.w * (float)(1.0 / (4.0 * kPi)), (float)rw, g5.x, g5.y,
                                        g5.z, g5.w, oo);
            for (int j = 0; j < 3; j++) { o.ar[j] = oo.ar[j]; o.ai[j] = oo.ai[j]; }
            o.br = oo.br; o.bi = oo.bi;
        } else {
            const double *h = geo.geo_d + (size_t)kGeoD * e;
            double d3[3] = {h[0] - xd[0], h[1] - xd[1], h[2] - xd[2]};
            double hgt = d3[0] * h[9] + d3[1] * h[10] + d3[2] * h[11];
            SumsD Sm;
            far_sums_f64(d3, h + 3, h + 6, hgt, (double)k, nq, Sm);
            Coeffs<double, SumsD> oo;
            finish_coeffs<double, SumsD>(Sm, h[12] / (4.0 * kPi), (double)rw, h[13], h[14], h[15],
                                         h[16], oo);
            for (int j = 0; j < 3; j++) { o.ar[j] = oo.ar[j]; o.ai[j] = oo.ai[j]; }
            o.br = oo.br; o.bi = oo.bi;
        }
        const int node[3] = {nd.x, nd.y, nd.z};
#pragma unroll
        for (int s = 0; s < kFieldSB; s++) {
            if (s >= sb) break;
            T vr = o.br, vi = o.bi;
#pragma unroll
            for (int j = 0; j < 3; j++) {
                const typename CplxT<T>::t uu = u[(size_t)(s0 + s) * ldu + node[j]];
                vr += o.ar[j] * uu.x - o.ai[j] * uu.y;
                vi += o.ar[j] * uu.y + o.ai[j] * uu.x;
            }
            accr[s] += vr;
            acci[s] += vi;
        }
    }
    __shared__ double red[kFieldNT / 32][kFieldSB][2];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int s = 0; s < kFieldSB; s++) {
        double a = accr[s], b = acci[s];
        for (int o = 16; o > 0; o >>= 1) {
            a += __shfl_xor_sync(0xffffffffu, a, o);
            b += __shfl_xor_sync(0xffffffffu, b, o);
        }
        if (lane == 0) { red[warp][s][0] = a; red[warp][s][1] = b; }
    }
    __syncthreads();
    if (threadIdx.x < sb) {
        const int s = threadIdx.x;
        double a = 0, b = 0;
        for (int w = 0; w < kFieldNT / 32; w++) { a += red[w][s][0]; b += red[w][s][1]; }
        part[((size_t)split * pts.R + p) * S + s0 + s] = make_double2(a, b);
    }
}

// Near-singular field pairs (eta > 0): one warp per point, FP64.
template <typename TU>
__global__ void __launch_bounds__(32 * kNearWarps)
field_near_kernel(RowPoints pts, GeoTables geo, Physics ph, int nq, const TU *__restrict__ u, size_t ldu,
                  int S, double2 *__restrict__ near_part) {
    __shared__ Leaf leaves_all[kNearWarps][kMaxLeaves];
    __shared__ int codes_all[kNearWarps][2][kMaxLeaves];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int p = blockIdx.x * kNearWarps + warp;
    if (p >= pts.R) return;
    Leaf *leaves = leaves_all[warp];
    const float4 xh = pts.f[2 * (size_t)p];
    const double x[3] = {pts.d[3 * (size_t)p], pts.d[3 * (size_t)p + 1], pts.d[3 * (size_t)p + 2]};
    for (int s = lane; s < S; s += 32) near_part[(size_t)p * S + s] = make_double2(0.0, 0.0);
    __syncwarp();
    for (int e0 = 0; e0 < geo.E; e0 += 32) {
        const int e = e0 + lane;
        bool flag = false;
        int4 nd = make_int4(-1, -1, -1, 0);
        if (e < geo.E) {
            nd = geo.elems[e];
            flag = pair_is_near(-1, 0, nd, xh, geo.geo_f + (size_t)kGeoF * e);
        }
        unsigned mask = __ballot_sync(0xffffffffu, flag);
        while (mask) {
            const int b = __ffs(mask) - 1;
            mask &= mask - 1;
            const int eb = e0 + b;
            const int node[3] = {__shfl_sync(0xffffffffu, nd.x, b), __shfl_sync(0xffffffffu, nd.y, b),
                                 __shfl_sync(0xffffffffu, nd.z, b)};
            const double *h = geo.geo_d + (size_t)kGeoD * eb;
            int nl = 0;
            nl = build_leaves_warp<false>(h, x, ph.near_eta, ph.near_depth, leaves, codes_all[warp][0], codes_all[warp][1]);
            __syncwarp();
            NearOut o;
            near_integrate(h, x, ph.k, 3, leaves, nl, nq, o);
            __syncwarp();
            const double bAr = h[13], bAi = h[14], bCr = h[15], bCi = h[16];
            double ar[3], ai[3], sgr = 0, sgi = 0;
            for (int j = 0; j < 3; j++) {
                double g_r = -ph.rw * o.gi[j], g_i = ph.rw * o.gr[j];
                ar[j] = o.hr[j] - (bAr * g_r - bAi * g_i);
                ai[j] = o.hi[j] - (bAr * g_i + bAi * g_r);
                sgr += g_r;
                sgi += g_i;
            }
            double br = bCr * sgr - bCi * sgi, bi = bCr * sgi + bCi * sgr;
            for (int s = lane; s < S; s += 32) {
                double vr = br, vi = bi;
                for (int j = 0; j < 3; j++) {
                    TU uu = u[(size_t)s * ldu + node[j]];
                    vr += ar[j] * (double)uu.x - ai[j] * (double)uu.y;
                    vi += ar[j] * (double)uu.y + ai[j] * (double)uu.x;
                }
                double2 cur = near_part[(size_t)p * S + s];
                near_part[(size_t)p * S + s] = make_double2(cur.x + vr, cur.y + vi);
            }
        }
    }
}

__global__ void field_finalize_kernel(RowPoints pts, int S, int nsplit, double k,
                                      const DevSource *__restrict__ srcs,
                                      const double2 *__restrict__ part,
                                      const double2 *__restrict__ near_part, double2 *__restrict__ out) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= pts.R * S) return;
    const int p = idx / S, s = idx - p * S;
    const double x[3] = {pts.d[3 * (size_t)p], pts.d[3 * (size_t)p + 1], pts.d[3 * (size_t)p + 2]};
    double sr = 0, si = 0;
    for (int t = 0; t < nsplit; t++) {
        double2 v = part[((size_t)t * pts.R + p) * S + s];
        sr += v.x;
        si += v.y;
    }
    if (near_part) {
        sr += near_part[(size_t)p * S + s].x;
        si += near_part[(size_t)p * S + s].y;
    }
    double2 inc = incident_field(srcs[s], k, x);
    out[(size_t)s * pts.R + p] = make_double2(inc.x - sr, inc.y - si);
}

void launch_field(int prec, const RowPoints &pts, const GeoTables &geo, const Physics &ph,
                  const void *u, size_t ldu, int S, const DevSource *srcs, double2 *part, int nsplit,
                  double2 *near_part, double2 *out, cudaStream_t st) {
    BEM_PROF("field_eval", st);
    if (pts.R <= 0 || S <= 0) return;
    int nq = quadrature_points();
    dim3 grid(pts.R, nsplit);
    for (int s0 = 0; s0 < S; s0 += kFieldSB) {
        if (prec == BEM_PREC_C64)
            field_far_kernel<float><<<grid, kFieldNT, 0, st>>>(pts, geo, (float)ph.k, (float)ph.rw, nq,
                                                               (const float2 *)u, ldu, S, s0, nsplit, part);
        else
            field_far_kernel<double><<<grid, kFieldNT, 0, st>>>(pts, geo, ph.k, ph.rw, nq,
                                                                (const double2 *)u, ldu, S, s0, nsplit, part);
        count_launch();
        KERNEL_CHECK();
    }
    double2 *np = nullptr;
    if (ph.near_eta > 0.0 && near_part) {
        dim3 g2((pts.R + kNearWarps - 1) / kNearWarps);
        if (prec == BEM_PREC_C64)
            field_near_kernel<float2><<<g2, 32 * kNearWarps, 0, st>>>(pts, geo, ph, nq, (const float2 *)u, ldu, S, near_part);
        else
            field_near_kernel<double2><<<g2, 32 * kNearWarps, 0, st>>>(pts, geo, ph, nq, (const double2 *)u, ldu, S, near_part);
        count_launch();
        KERNEL_CHECK();
        np = near_part;
    }
    int tot = pts.R * S;
    field_finalize_kernel<<<(tot + 255) / 256, 256, 0, st>>>(pts, S, nsplit, ph.k, srcs, part, np, out);
    count_launch();
    KERNEL_CHECK();
}

}  // namespace bem
