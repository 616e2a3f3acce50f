// Least squares by blocked Householder QR with the trailing updates on the
// tcgen05 tensor cores (BEM_SOLVE_QR_TC).  Replaces the blocked WY Householder
// QR of the reference (QR_thin / lsqSolver, numerical.cu:246-554, whose
// trailing updates are Cgemm calls, :375-396) and its cuSOLVER qrSolver
// sequence (numerical.cu:580-644) for the device-resident solver.
//
// Method (m x n complex A, m >= n, S right-hand sides B).
// * A and B are copied (c64, column-major, leading dimension ldq) into one
//   workspace [A | B]: B rides along as extra trailing columns, so Q^H B is
//   formed by the same updates and Q is never formed.
// * Panels of kQrNB = 128 columns.  A panel is factored by one thread-block
//   cluster (up to 16 CTAs, qr_panel_kernel): the CTAs split the panel's rows
//   and keep a leaf of W = 16 columns in shared memory; per column the
//   Householder vector (LAPACK's zlarfg convention: beta real, H = I - tau v
//   v^H, v_1 = 1) needs two cluster-wide sums exchanged through distributed
//   shared memory (the norm, then v^H times the leaf's other columns).  A
//   finished leaf is applied to the panel's remaining columns as a block
//   reflector (I - V T V^H)^H in the same kernel.
// * The trailing matrix C (the columns right of the panel, B included) is
//   updated as C -= V T^H (V^H C) with two tensor-core GEMMs (tc_gemm, fp16
//   split products, TF32x3-level accuracy) on the interleaved-real form of
//   the complex products, T from V^H V (a third, small GEMM) and the taus.
// * X = R^{-1} (Q^H B)[0:n] by blocked back substitution.
// * Refinement to the FP64 least-squares solution (semi-normal equations,
//   corrected): r = b - A x and g = A^H r with FP64-accurate products (c128
//   A, or c64 A with double-float sums), R^H R dx = g by two FP32 triangular
//   solves with the FP32 factor (g scaled to order one), x += dx, until
//   ||g|| <= tol ||A^H b||.  It converges by a factor of about
//   kappa(A)^2 x 6e-8 per step; FP32 arithmetic in the solves adds errors of
//   the factor's own order.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <mutex>
#include <string>
#include <vector>

#include "bem_common.h"
#include "kernels.h"
#include "solver.h"
#include "tc_gemm.h"
#include "tc_split.cuh"
#include "tma.h"

namespace bem {
namespace {

namespace cg = cooperative_groups;

constexpr int kQrNT = 512;      // threads per CTA of the panel kernel
constexpr int kQrNB = 128;      // panel width (the trailing updates' K)
constexpr int kQrW = 16;        // leaf width held in shared memory
constexpr int kQrCL = 16;       // CTAs per cluster (non-portable size)
constexpr int kQrTB = 64;       // block of the triangular solves
// Refinement target: relative normal-equation residual ||A^H (b - A x)|| /
// ||A^H b|| (stagnation at the precision of the FP64-accurate products ends
// it earlier).
constexpr long long kQrWaitCycles = 2000000000LL;   // ~1 s at 2 GHz: the panel's bounded waits
constexpr double kQrRefineTol = 1e-14;
constexpr double kQrStagnationOk = 1e-11;
static_assert(kQrW == 16, "the panel kernel pairs lanes c and c + 16 of a warp on one leaf column");

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// conj(a) b
__device__ __forceinline__ float2 cjmul(float2 a, float2 b) {
    return make_float2(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
}

// Shared-memory layout of the panel kernel (float2 units): the leaf L[W][lds]
// (column-major, lds = 1 mod 16: the W columns of one row fall in distinct
// banks), then the reduction slots.
struct PanelLayout {
    int lds;
    size_t leaf, tin, sums, prev, gpart, gram, wpart, gsum, tmat, ysum, scratch, taus, total;
    __host__ __device__ PanelLayout(int rb) {
        lds = ((rb + 15) / 16) * 16 + 1;
        size_t o = 0;
        leaf = o;    o += (size_t)kQrW * lds;
        tin = o;     o += 2 * kQrCL * 2 * kQrW;          // [slot][source CTA][d_c | pivot-row x_c]: column sums received
        sums = o;    o += 2 * kQrW;                      // the cluster's sums of red
        prev = o;    o += 2;                             // (scal, beta) of the column whose scaling is pending
        gpart = o;   o += 2 * kQrW * kQrW;               // two row halves of this CTA's V^H V
        gram = o;    o += kQrW * kQrW;                   // this CTA's V^H V
        wpart = o;   o += (size_t)kQrW * kQrNB;          // this CTA's V^H P (leaf x rest of the panel)
        gsum = o;    o += kQrW * kQrW;
        tmat = o;    o += kQrW * kQrW;
        ysum = o;    o += (size_t)kQrW * kQrNB;
        scratch = o; o += (kQrNT / 32) * kQrW;
        taus = o;    o += kQrW;                          // this leaf's taus (every CTA forms them)
        total = o;
    }
};

// Sum over the cluster's CTAs of the float2 at shared offset `off` + idx:
// the loads of all peers are issued before any is added (kQrCL independent
// remote loads in flight instead of one latency per peer).
template <class Peer>
__device__ __forceinline__ float2 cluster_sum(const Peer &peer, size_t off, size_t idx, int CL) {
    float2 u[kQrCL];
#pragma unroll
    for (int p = 0; p < kQrCL; p++) u[p] = p < CL ? peer(off, p)[idx] : make_float2(0.f, 0.f);
    float2 t = make_float2(0.f, 0.f);
#pragma unroll
    for (int p = 0; p < kQrCL; p++) {
        t.x += u[p].x;
        t.y += u[p].y;
    }
    return t;
}

// The reflector of a column from the cluster's sums (zlarfg's convention):
// t = |x|^2 below the pivot, a = the pivot value; beta = -sign(Re a) |x|,
// tau = (beta - a) / beta, scal = 1 / (a - beta) (v = x scal below the
// pivot, 1 on it).  A column that is already reduced (t = 0, Im a = 0)
// reflects nothing: tau = scal = 0, beta = a.
__device__ __forceinline__ void qr_reflector(float t, float2 a, float2 &tau, float2 &scal, float &beta) {
    if (t == 0.f && a.y == 0.f) {
        tau = make_float2(0.f, 0.f);
        scal = make_float2(0.f, 0.f);
        beta = a.x;
    } else {
        beta = -copysignf(sqrtf(a.x * a.x + a.y * a.y + t), a.x);
        tau = make_float2((beta - a.x) / beta, -a.y / beta);
        const float2 d = make_float2(a.x - beta, a.y);
        const float dd = d.x * d.x + d.y * d.y;
        scal = make_float2(d.x / dd, -d.y / dd);
    }
}

// Factors the panel Q[j0:m, j0:j0+pc] in place (Householder vectors below the
// diagonal, R on and above it); tau_out[0..pc) receives the taus.  One
// cluster of gridDim.x CTAs; CTA q owns the rows j0 + q rb .. + rb - 1.
//
// Per column one cluster-wide reduction (pushed by st.async into every CTA's
// mbarrier-tracked receive slot, no cluster barrier): from the column x as it stands
// (before scaling), every CTA sums over its rows below the pivot g the
// products conj(x_i) x_c[i] for the column itself (|x|^2) and the leaf's
// later columns (d_c), and the owner of row g adds the pivot-row values
// x_c[g].  Then every CTA forms the reflector and, with
// v^H x_c = x_c[g] + conj(scal) d_c, updates the later columns; the column's
// own scaling (x_i scal below the pivot, beta on it) is done while the next
// column is being summed (those sums do not read it).  A finished leaf is
// written back, its shared copy turned into V itself (zeros above the unit
// diagonal), and applied to the panel's remaining columns as a block
// reflector (I - V T V^H)^H.
__global__ void __launch_bounds__(kQrNT, 1)
qr_panel_kernel(float2 *__restrict__ Q, size_t ldq, int m, int j0, int pc, int rb, float2 *__restrict__ tau_out,
                int *status) {
    cg::cluster_group cluster = cg::this_cluster();
    const int CL = (int)cluster.num_blocks();
    const int q = (int)cluster.block_rank();
    extern __shared__ __align__(16) float2 ps[];
    // the per-column exchange: every CTA pushes its 2 kQrW partial sums into
    // every CTA's receive slot (column k into slot k % 2) with st.async,
    // completing bytes on that slot's mbarrier
    __shared__ __align__(8) uint64_t col_bar[2];
    __shared__ int col_abort;
    const uint32_t col_bytes = (uint32_t)(CL * 2 * kQrW * sizeof(float2));
    if (threadIdx.x == 0) {
        mbar_init(&col_bar[0], 1);
        mbar_init(&col_bar[1], 1);
        col_abort = 0;
        mbar_fence_init();
        mbar_arrive_expect_tx(&col_bar[0], col_bytes);
        mbar_arrive_expect_tx(&col_bar[1], col_bytes);
    }
    cluster.sync();   // every CTA's barriers are armed before any column sum is sent
    const PanelLayout lay(rb);
    const int lds = lay.lds;
    float2 *L = ps + lay.leaf;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int r0 = j0 + q * rb;
    const int nrows = max(0, min(rb, m - r0));
    float2 *scratch = ps + lay.scratch;
    auto peer = [&](size_t off, int p) -> const float2 * {
        return cluster.map_shared_rank(ps + off, p);
    };
    // thread (column c of the leaf, row slice il) in the column loop
    const int c = tid % kQrW, il = tid / kQrW;
    constexpr int NIL = kQrNT / kQrW;

    for (int l0 = 0; l0 < pc; l0 += kQrW) {
        const int lw = min(kQrW, pc - l0), G0 = j0 + l0;
        for (int cc = 0; cc < lw; cc++)
            for (int i = tid; i < nrows; i += kQrNT) L[(size_t)cc * lds + i] = Q[(size_t)(G0 + cc) * ldq + r0 + i];
        __syncthreads();
        for (int jj = 0; jj < lw; jj++) {
            const int g = G0 + jj;                        // pivot row
            const int ib = max(0, g + 1 - r0);            // first local row below the pivot
            const bool own = g >= r0 && g < r0 + nrows;   // this CTA holds the pivot row
            const float2 *xj = L + (size_t)jj * lds;
            // (1) sums over this CTA's rows below the pivot; the previous
            // column's pending scaling meanwhile
            float2 acc = make_float2(0.f, 0.f);
            if (c >= jj && c < lw) {
                const float2 *xc = L + (size_t)c * lds;
                for (int i = ib + il; i < nrows; i += NIL) {
                    const float2 u = cjmul(xj[i], xc[i]);
                    acc.x += u.x;
                    acc.y += u.y;
                }
            } else if (jj > 0 && c == jj - 1) {
                const float2 sc = ps[lay.prev];
                float2 *xp = L + (size_t)(jj - 1) * lds;
                for (int i = max(0, g - r0) + il; i < nrows; i += NIL) xp[i] = cmul(xp[i], sc);
                if (il == 0 && g - 1 >= r0 && g - 1 < r0 + nrows) xp[g - 1 - r0] = make_float2(ps[lay.prev + 1].x, 0.f);
            }
            acc.x += __shfl_xor_sync(0xffffffffu, acc.x, 16);   // lanes c and c + 16 share a column
            acc.y += __shfl_xor_sync(0xffffffffu, acc.y, 16);
            if (lane < kQrW) scratch[warp * kQrW + lane] = acc;
            __syncthreads();
            // (2) exchange: warp 0 pushes this CTA's 2 kQrW values (the d_c
            // sums, then the pivot row's x_c) to every CTA, waits for the
            // cluster's and adds them in rank order (the same order everywhere)
            if (tid < 2 * kQrW) {
                const int cc = tid % kQrW, kx = l0 + jj, slot = kx & 1;
                float2 t = make_float2(0.f, 0.f);
                if (tid < kQrW) {
                    for (int w = 0; w < kQrNT / 32; w++) {
                        t.x += scratch[w * kQrW + tid].x;
                        t.y += scratch[w * kQrW + tid].y;
                    }
                } else if (own && cc >= jj && cc < lw) {
                    t = L[(size_t)cc * lds + (g - r0)];
                }
                const float2 *mine = ps + lay.tin + ((size_t)slot * kQrCL + q) * 2 * kQrW + tid;
                for (int p = 0; p < CL; p++)
                    st_async_f2(cluster_addr(mine, (uint32_t)p), t, cluster_addr(&col_bar[slot], (uint32_t)p));
                if (!mbar_wait_cluster_bounded(&col_bar[slot], (uint32_t)((kx >> 1) & 1), kQrWaitCycles, &col_abort)) {
                    col_abort = 1;
                    atomicExch(status, 1);
                }
                float2 u = make_float2(0.f, 0.f);
                for (int p = 0; p < CL; p++) {
                    const float2 v = ps[lay.tin + ((size_t)slot * kQrCL + p) * 2 * kQrW + tid];
                    u.x += v.x;
                    u.y += v.y;
                }
                ps[lay.sums + tid] = (cc >= jj && cc < lw) ? u : make_float2(0.f, 0.f);
                // re-arm the slot for column kx + 2: its bytes can come only
                // after this CTA's column kx + 1 push, which follows
                if (tid == 0 && !col_abort) mbar_arrive_expect_tx(&col_bar[slot], col_bytes);
            }
            __syncthreads();
            // (3) the reflector (every thread), then x_c -= v y_c with
            // y_c = conj(tau) v^H x_c for the leaf's later columns
            float2 tau, scal;
            float beta;
            qr_reflector(ps[lay.sums + jj].x, ps[lay.sums + kQrW + jj], tau, scal, beta);
            if (tid == 0) {
                ps[lay.taus + jj] = tau;
                if (q == 0) tau_out[l0 + jj] = tau;
                ps[lay.prev] = scal;
                ps[lay.prev + 1] = make_float2(beta, 0.f);
            }
            if (c > jj && c < lw) {
                const float2 d = ps[lay.sums + c], xg = ps[lay.sums + kQrW + c];
                const float2 sd = cjmul(scal, d);
                const float2 y = cjmul(tau, make_float2(xg.x + sd.x, xg.y + sd.y));
                const float2 sy = cmul(scal, y);   // v_i y = x_i (scal y) below the pivot
                float2 *xc = L + (size_t)c * lds;
                if (il == 0 && own) {
                    xc[g - r0].x -= y.x;
                    xc[g - r0].y -= y.y;
                }
                for (int i = ib + il; i < nrows; i += NIL) {
                    const float2 u = cmul(xj[i], sy);
                    xc[i].x -= u.x;
                    xc[i].y -= u.y;
                }
            }
            __syncthreads();
        }
        {
            // the leaf's last column: its pending scaling
            const int jl = lw - 1, gl = G0 + jl;
            const float2 sc = ps[lay.prev];
            float2 *xp = L + (size_t)jl * lds;
            for (int i = max(0, gl + 1 - r0) + tid; i < nrows; i += kQrNT) xp[i] = cmul(xp[i], sc);
            if (tid == 0 && gl >= r0 && gl < r0 + nrows) xp[gl - r0] = make_float2(ps[lay.prev + 1].x, 0.f);
        }
        __syncthreads();
        // the factored leaf back to Q
        for (int cc = 0; cc < lw; cc++)
            for (int i = tid; i < nrows; i += kQrNT) Q[(size_t)(G0 + cc) * ldq + r0 + i] = L[(size_t)cc * lds + i];
        const int c1 = l0 + lw, nrest = pc - c1;
        if (nrest <= 0) continue;
        __syncthreads();
        // ---- the leaf's block reflector applied to the panel's later columns:
        // P -= V T^H (V^H P), P = Q[j0:m, j0+c1 : j0+pc] ----
        // L becomes V: zero above the unit diagonal in the leaf's pivot rows
        // (rows above G0 are zero in every column and skipped below)
        for (int e = tid; e < lw * lw; e += kQrNT) {
            const int k = e / lw, d = e % lw, grow = G0 + d;
            if (grow >= r0 && grow < r0 + nrows && d <= k)
                L[(size_t)k * lds + (grow - r0)] = d == k ? make_float2(1.f, 0.f) : make_float2(0.f, 0.f);
        }
        __syncthreads();
        const int i0 = max(0, G0 - r0);
        // (a) this CTA's V^H V (lw x lw; thread = entry and row half) and V^H P (lw x nrest)
        {
            const int pr = tid % (kQrW * kQrW), h = tid / (kQrW * kQrW);
            const int a = pr / kQrW, b = pr % kQrW;
            float2 t = make_float2(0.f, 0.f);
            if (a < lw && b < lw) {
                const float2 *va = L + (size_t)a * lds, *vb = L + (size_t)b * lds;
                for (int i = i0 + h; i < nrows; i += kQrNT / (kQrW * kQrW)) {
                    const float2 u = cjmul(va[i], vb[i]);
                    t.x += u.x;
                    t.y += u.y;
                }
            }
            ps[lay.gpart + tid] = t;
        }
        for (int cc = warp; cc < nrest; cc += kQrNT / 32) {
            const float2 *pcol = Q + (size_t)(j0 + c1 + cc) * ldq + r0;
            float2 acc[kQrW];
#pragma unroll
            for (int k = 0; k < kQrW; k++) acc[k] = make_float2(0.f, 0.f);
            for (int i = i0 + lane; i < nrows; i += 32) {
                const float2 x = pcol[i];
#pragma unroll
                for (int k = 0; k < kQrW; k++)
                    if (k < lw) {
                        const float2 u = cjmul(L[(size_t)k * lds + i], x);
                        acc[k].x += u.x;
                        acc[k].y += u.y;
                    }
            }
#pragma unroll
            for (int k = 0; k < kQrW; k++)
                for (int o = 16; o > 0; o >>= 1) {
                    acc[k].x += __shfl_xor_sync(0xffffffffu, acc[k].x, o);
                    acc[k].y += __shfl_xor_sync(0xffffffffu, acc[k].y, o);
                }
            if (lane == 0)
#pragma unroll
                for (int k = 0; k < kQrW; k++)
                    if (k < lw) ps[lay.wpart + (size_t)k * kQrNB + cc] = acc[k];
        }
        __syncthreads();
        if (tid < kQrW * kQrW) {
            float2 t = ps[lay.gpart + tid];
            for (int h = 1; h < kQrNT / (kQrW * kQrW); h++) {
                t.x += ps[lay.gpart + h * kQrW * kQrW + tid].x;
                t.y += ps[lay.gpart + h * kQrW * kQrW + tid].y;
            }
            ps[lay.gram + tid] = t;   // entry (a, b) at a kQrW + b
        }
        cluster.sync();
        // (b) the cluster sums
        for (int e = tid; e < lw * lw; e += kQrNT) {
            const int a = e / lw, b = e % lw;
            ps[lay.gsum + a * kQrW + b] = cluster_sum(peer, lay.gram, a * kQrW + b, CL);
        }
        for (int e = tid; e < lw * nrest; e += kQrNT) {
            const int k = e / nrest, cc = e % nrest;
            ps[lay.ysum + (size_t)k * kQrNB + cc] = cluster_sum(peer, lay.wpart, (size_t)k * kQrNB + cc, CL);   // W = V^H P for now
        }
        __syncthreads();
        // (c) T (upper triangular, lw x lw): T_kk = tau_k, T[0:k, k] = -tau_k T[0:k, 0:k] G[0:k, k]
        float2 *T = ps + lay.tmat;
        if (warp == 0) {
            for (int k = 0; k < lw; k++) {
                const float2 tk = ps[lay.taus + k];
                float2 t = make_float2(0.f, 0.f);
                if (lane < k) {
                    for (int l = lane; l < k; l++) {
                        const float2 u = cmul(T[lane * kQrW + l], ps[lay.gsum + l * kQrW + k]);
                        t.x += u.x;
                        t.y += u.y;
                    }
                }
                __syncwarp();
                if (lane < k) T[lane * kQrW + k] = cmul(make_float2(-tk.x, -tk.y), t);
                if (lane == k) T[k * kQrW + k] = tk;
                if (lane > k && lane < kQrW) T[lane * kQrW + k] = make_float2(0.f, 0.f);
                __syncwarp();
            }
        }
        __syncthreads();
        // (d) Y = T^H W (in place, column by column: each column's lw values
        // are read before any is written)
        for (int cc = tid; cc < nrest; cc += kQrNT) {
            float2 w[kQrW];
#pragma unroll
            for (int k = 0; k < kQrW; k++) w[k] = k < lw ? ps[lay.ysum + (size_t)k * kQrNB + cc] : make_float2(0.f, 0.f);
#pragma unroll
            for (int k = 0; k < kQrW; k++) {
                if (k >= lw) break;
                float2 y = make_float2(0.f, 0.f);
                for (int l = 0; l <= k; l++) {
                    const float2 u = cjmul(T[l * kQrW + k], w[l]);
                    y.x += u.x;
                    y.y += u.y;
                }
                ps[lay.ysum + (size_t)k * kQrNB + cc] = y;
            }
        }
        __syncthreads();
        // (e) P -= V Y (this CTA's rows from the leaf's first pivot row down)
        for (int cc = warp; cc < nrest; cc += kQrNT / 32) {
            float2 *pcol = Q + (size_t)(j0 + c1 + cc) * ldq + r0;
            float2 yk[kQrW];
#pragma unroll
            for (int k = 0; k < kQrW; k++) yk[k] = k < lw ? ps[lay.ysum + (size_t)k * kQrNB + cc] : make_float2(0.f, 0.f);
            for (int i = i0 + lane; i < nrows; i += 32) {
                float2 x = pcol[i];
#pragma unroll
                for (int k = 0; k < kQrW; k++)
                    if (k < lw) {
                        const float2 u = cmul(L[(size_t)k * lds + i], yk[k]);
                        x.x -= u.x;
                        x.y -= u.y;
                    }
                pcol[i] = x;
            }
        }
        __syncthreads();
    }
    cluster.sync();   // peers' shared memory is read until here
}


// Q[r + c ldq] = A[r lda + c] (row-major c64 or c128 system) for c < n, and
// Q[r + (n + j) ldq] = B[r + j R] (c128, column-major): 32 x 32 tiles
// through shared memory (coalesced on both sides).  grid (ceil(n/32),
// ceil(R/32)) for A; B by a separate plain kernel.
template <typename T>
__global__ void qr_copy_a_kernel(int R, int n, const T *__restrict__ A, size_t lda, float2 *__restrict__ Q,
                                 size_t ldq) {
    __shared__ float2 tile[32][33];
    const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;   // 32 x 8 threads
    for (int k = ty; k < 32; k += 8) {
        const int r = r0 + k, c = c0 + tx;
        if (r < R && c < n) {
            const T v = A[(size_t)r * lda + c];
            tile[k][tx] = make_float2((float)v.x, (float)v.y);
        }
    }
    __syncthreads();
    for (int k = ty; k < 32; k += 8) {
        const int c = c0 + k, r = r0 + tx;
        if (r < R && c < n) Q[(size_t)c * ldq + r] = tile[tx][k];
    }
}

__global__ void qr_copy_b_kernel(int R, int S, const double2 *__restrict__ B, float2 *__restrict__ Qb, size_t ldq) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
    if (r < R) {
        const double2 v = B[(size_t)j * R + r];
        Qb[(size_t)j * ldq + r] = make_float2((float)v.x, (float)v.y);
    }
}

// Largest column 2-norm of Q's ncols columns (m rows) into out (as the bits of
// a non-negative float); one CTA per column.
__global__ void qr_colnorm_kernel(int m, const float2 *__restrict__ Q, size_t ldq, unsigned *__restrict__ out) {
    __shared__ float red[32];
    const float2 *q = Q + (size_t)blockIdx.x * ldq;
    float s = 0.f;
    for (int r = threadIdx.x; r < m; r += blockDim.x) s = fmaf(q[r].x, q[r].x, fmaf(q[r].y, q[r].y, s));
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        float t = 0.f;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += red[w];
        atomicMax(out, __float_as_uint(sqrtf(t)));
    }
}

// Scale pairs (scale, 1 / scale) of the GEMMs' left operands: sc[0..1] for the
// trailing matrix, from the largest column norm (orthogonal updates keep
// column norms, so it bounds every entry through the factorisation; 2% slack
// for rounding), sc[2..3] for V (|entries| <= 1: the unit diagonal, and
// |v_i| = |x_i| / |alpha - beta| <= 1 below it).
__global__ void qr_scales_kernel(float *sc) {
    const float bound = __uint_as_float(*reinterpret_cast<const unsigned *>(sc + 4)) * 1.02f;
    const float s = pow2_scale(bound);
    sc[0] = s;
    sc[1] = 1.f / s;
    sc[2] = 16384.f;
    sc[3] = 1.f / 16384.f;
}

// Vf (mr x pc, column-major, ldv): the panel's Householder vectors with the
// unit diagonal and zeros above it.
__global__ void qr_vfull_kernel(int mr, int pc, const float2 *__restrict__ P, size_t ldq, float2 *__restrict__ Vf,
                                size_t ldv) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, k = blockIdx.y;
    if (i >= mr) return;
    float2 v = make_float2(0.f, 0.f);
    if (i == k) v = make_float2(1.f, 0.f);
    else if (i > k) v = P[(size_t)k * ldq + i];
    Vf[(size_t)k * ldv + i] = v;
}

// Vrr (2 mr x ldk floats, row-major): row 2i = (Re v_ik, -Im v_ik)_k, row 2i+1
// = (Im v_ik, Re v_ik)_k, so that Vrr times the block with rows 2k, 2k+1 =
// (Re w_k, Im w_k) gives (Re, Im) of V w in rows 2i, 2i+1.
__global__ void qr_vrr_kernel(int mr, int pc, const float2 *__restrict__ Vf, size_t ldv, float *__restrict__ Vrr,
                              int ldk) {
    const int i = blockIdx.x, k = threadIdx.x;
    if (k >= pc) return;
    const float2 v = Vf[(size_t)k * ldv + i];
    float *r0 = Vrr + (size_t)(2 * i) * ldk, *r1 = r0 + ldk;
    r0[2 * k] = v.x;
    r0[2 * k + 1] = -v.y;
    r1[2 * k] = v.y;
    r1[2 * k + 1] = v.x;
}

// T (pc x pc, row-major, ld kQrNB, upper triangular) of the panel's block
// reflector H_1 ... H_pc = I - V T V^H from the Gram matrix G = V^H V
// (Greal: pc x 2pc column-major, [Re G | Im G]) and the taus, by doubling:
// the T of 16-column leaves by the column recurrence (T_kk = tau_k,
// T[0:k, k] = -tau_k T[0:k, 0:k] G[0:k, k]), one warp per leaf, then
// adjacent blocks merged at widths 32, 64 and 128 through
// (I - V1 T1 V1^H)(I - V2 T2 V2^H) = I - [V1 V2] [[T1, -T1 G12 T2], [0, T2]] [V1 V2]^H,
// all pairs of a level at once (two triangular products).  Columns past pc
// act as tau = 0, G = 0 (their T columns come out zero).  FP32 throughout,
// like the factor it serves; one CTA, T in shared memory as [col][row].
constexpr int kQrLeafT = 16;
constexpr int kQrLarftNT = 512;
constexpr size_t kQrLarftSmem = sizeof(float2) * ((size_t)kQrNB * kQrNB + (size_t)kQrNB * kQrNB / 4);
__global__ void __launch_bounds__(kQrLarftNT)
qr_larft_kernel(int pc, const float *__restrict__ Greal, const float2 *__restrict__ tau, float2 *__restrict__ T) {
    extern __shared__ float2 lt_smem[];
    float2 *Ts = lt_smem;                        // T[row][col] at Ts[col * kQrNB + row]
    float2 *Ys = lt_smem + kQrNB * kQrNB;        // G12 T2 per pair of the current level
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    auto G = [&](int r, int c) {
        return (r < pc && c < pc) ? make_float2(Greal[(size_t)c * pc + r], Greal[(size_t)(pc + c) * pc + r])
                                  : make_float2(0.f, 0.f);
    };
    for (int e = tid; e < kQrNB * kQrNB; e += kQrLarftNT) Ts[e] = make_float2(0.f, 0.f);
    __syncthreads();
    // leaves: warp w < kQrNB / kQrLeafT forms leaf w (lane r = row)
    if (warp < kQrNB / kQrLeafT) {
        const int o = warp * kQrLeafT, r = lane;
        for (int k = 0; k < kQrLeafT; k++) {
            const float2 tk = o + k < pc ? tau[o + k] : make_float2(0.f, 0.f);
            float2 t = make_float2(0.f, 0.f);
            if (r < k)
                for (int l = r; l < k; l++) {
                    const float2 trl = Ts[(size_t)(o + l) * kQrNB + o + r], g = G(o + l, o + k);
                    t.x = fmaf(trl.x, g.x, fmaf(-trl.y, g.y, t.x));
                    t.y = fmaf(trl.x, g.y, fmaf(trl.y, g.x, t.y));
                }
            __syncwarp();
            if (r < k) Ts[(size_t)(o + k) * kQrNB + o + r] = make_float2(-(tk.x * t.x - tk.y * t.y), -(tk.x * t.y + tk.y * t.x));
            else if (r == k) Ts[(size_t)(o + k) * kQrNB + o + k] = tk;
            __syncwarp();
        }
    }
    __syncthreads();
    for (int h = kQrLeafT; h < kQrNB; h *= 2) {
        const int pairs = kQrNB / (2 * h), hh = h * h;
        // Y = G12 T2 (T2 upper triangular): Y[r][c] = sum_{l <= c} G(o1 + r, o2 + l) T[o2 + l][o2 + c]
        for (int e = tid; e < pairs * hh; e += kQrLarftNT) {
            const int pr = e / hh, rem = e % hh, r = rem % h, c = rem / h;
            const int o1 = 2 * pr * h, o2 = o1 + h;
            float2 y = make_float2(0.f, 0.f);
            for (int l = 0; l <= c; l++) {
                const float2 g = G(o1 + r, o2 + l), t = Ts[(size_t)(o2 + c) * kQrNB + o2 + l];
                y.x = fmaf(g.x, t.x, fmaf(-g.y, t.y, y.x));
                y.y = fmaf(g.x, t.y, fmaf(g.y, t.x, y.y));
            }
            Ys[(size_t)pr * hh + (size_t)c * h + r] = y;
        }
        __syncthreads();
        // T12 = -T1 Y (T1 upper triangular): T12[r][c] = -sum_{l >= r} T[o1 + r][o1 + l] Y[l][c]
        for (int e = tid; e < pairs * hh; e += kQrLarftNT) {
            const int pr = e / hh, rem = e % hh, r = rem % h, c = rem / h;
            const int o1 = 2 * pr * h, o2 = o1 + h;
            float2 t = make_float2(0.f, 0.f);
            for (int l = r; l < h; l++) {
                const float2 a = Ts[(size_t)(o1 + l) * kQrNB + o1 + r], y = Ys[(size_t)pr * hh + (size_t)c * h + l];
                t.x = fmaf(a.x, y.x, fmaf(-a.y, y.y, t.x));
                t.y = fmaf(a.x, y.y, fmaf(a.y, y.x, t.y));
            }
            Ts[(size_t)(o2 + c) * kQrNB + o1 + r] = make_float2(-t.x, -t.y);
        }
        __syncthreads();
    }
    for (int e = tid; e < pc * pc; e += kQrLarftNT) {
        const int r = e / pc, k = e % pc;
        T[(size_t)r * kQrNB + k] = Ts[(size_t)k * kQrNB + r];
    }
}

// The right-hand operand of the rank-pc update: for trailing column c, W'[:, c]
// = T^H W[:, c] with W = V^H C = Z^H (Z = C^H V: Zreal nct x 2pc column-major,
// [Re Z | Im Z]), i.e. W'[k, c] = conj(sum_{l <= k} T[l, k] Z[c, l]), packed
// as rows 2k, 2k+1 = (Re, Im) of column c, scaled per column.  kQrTwCols
// columns per CTA with T and the CTA's rows of Z in shared memory; thread
// (k = tid % kQrNB, group g = tid / kQrNB) forms row k of the group's
// kQrTwPer columns (independent sums, Z values broadcast).
constexpr int kQrTwPer = 16;
constexpr int kQrTwGroups = 4;
constexpr int kQrTwCols = kQrTwPer * kQrTwGroups;
constexpr int kQrTwLdz = kQrNB + 1;
constexpr size_t kQrTwSmem = sizeof(float2) * ((size_t)kQrNB * kQrNB + (size_t)kQrTwCols * kQrTwLdz);
template <int P>
__global__ void __launch_bounds__(kQrNB * kQrTwGroups)
qr_pack_tw_kernel(int nct, int pc, const float *__restrict__ Zreal, const float2 *__restrict__ T, int Kp,
                  int ncols_pad, __half *__restrict__ planes, float *__restrict__ col_inv) {
    extern __shared__ float2 tw_smem[];
    float2 *Ts = tw_smem;                         // T[l][k] (row-major, ld kQrNB)
    float2 *zs = tw_smem + kQrNB * kQrNB;         // Z[c0 + c][l] as zs[c * kQrTwLdz + l]
    __shared__ float red[kQrTwGroups][kQrNB / 32][kQrTwPer];
    const int tid = threadIdx.x, k = tid % kQrNB, g = tid / kQrNB, lane = tid & 31, wg = k >> 5;
    const int c0 = blockIdx.x * kQrTwCols;
    for (int e = tid; e < pc * kQrNB; e += blockDim.x) Ts[e] = T[e];
    for (int e = tid; e < pc * kQrTwCols; e += blockDim.x) {
        const int c = e % kQrTwCols, l = e / kQrTwCols;
        float2 z = make_float2(0.f, 0.f);
        if (c0 + c < nct) z = make_float2(Zreal[(size_t)l * nct + c0 + c], Zreal[(size_t)(pc + l) * nct + c0 + c]);
        zs[c * kQrTwLdz + l] = z;
    }
    __syncthreads();
    float2 y[kQrTwPer];
#pragma unroll
    for (int j = 0; j < kQrTwPer; j++) y[j] = make_float2(0.f, 0.f);
    const float2 *zg = zs + (size_t)(g * kQrTwPer) * kQrTwLdz;
    if (k < pc)
        for (int l = 0; l <= k; l++) {
            const float2 t = Ts[l * kQrNB + k];
#pragma unroll
            for (int j = 0; j < kQrTwPer; j++) {
                const float2 z = zg[j * kQrTwLdz + l];
                y[j].x = fmaf(t.x, z.x, fmaf(-t.y, z.y, y[j].x));
                y[j].y = fmaf(t.x, z.y, fmaf(t.y, z.x, y[j].y));
            }
        }
    // per column, the largest |part| over the kQrNB rows (warp, then the
    // group's warps)
#pragma unroll
    for (int j = 0; j < kQrTwPer; j++) {
        float v = fmaxf(fabsf(y[j].x), fabsf(y[j].y));
        for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
        if (lane == 0) red[g][wg][j] = v;
    }
    __syncthreads();
    const size_t ps = (size_t)ncols_pad * Kp;
#pragma unroll
    for (int j = 0; j < kQrTwPer; j++) {
        const int c = c0 + g * kQrTwPer + j;
        if (c >= nct) break;
        float mx = 0.f;
#pragma unroll
        for (int w = 0; w < kQrNB / 32; w++) mx = fmaxf(mx, red[g][w][j]);
        const float sc = pow2_scale(mx);
        if (k == 0) col_inv[c] = 1.f / sc;
        if (k < pc) put_parts<P>(planes, ps, (size_t)c * Kp + 2 * k, y[j].x * sc, -y[j].y * sc);   // the conjugate
        else if (2 * k < Kp) put_parts<P>(planes, ps, (size_t)c * Kp + 2 * k, 0.f, 0.f);
    }
}

// ---- triangular solves with the FP32 factor R (upper triangle of Q[0:n,
// 0:n]) in FP32, blocks of kQrTB rows, one launch per block ----
//
// The inverses of R's diagonal blocks are formed once per factorisation
// (qr_diag_inv_kernel), so that solving a block is a matrix-vector product
// rather than a chain of kQrTB dependent steps.
//
// Back substitution R x = y, block b = rows [b0, b1), the block solved
// before it [b1, b2) (empty for the last block).  CTA 0 subtracts
// R[b0:b1, b1:b2] x[b1:b2] from its rows and multiplies by the block's
// inverse; the other CTAs subtract R[0:b0, b1:b2] x[b1:b2] from rows
// [0, b0).  So when block b is solved, every block after it has been
// subtracted from its rows: block b + 1 in this launch, the others in
// theirs.  Forward substitution R^H x = y mirrors it (previous block
// [bp, b0), the other CTAs updating rows [b1, n), the inverse's conjugate
// transpose).  In place on X (float2, column s at X + s ldx; grid.y =
// columns).  R's diagonal is nonzero (a Householder beta, real, of the
// magnitude of the column it came from).
constexpr int kQrTsNT = 256;
constexpr int kQrTsP = kQrTsNT / kQrTB;   // partial sums per row in CTA 0
static_assert(kQrTsNT % kQrTB == 0, "CTA 0 splits the block's columns evenly");

// 1 / r with the division scaled by the larger part of r.
__device__ __forceinline__ float2 qr_crecip(float2 r) {
    const float s = fmaxf(fabsf(r.x), fabsf(r.y));
    const float rx = r.x / s, ry = r.y / s;
    const float inv = 1.f / (s * (rx * rx + ry * ry));
    return make_float2(rx * inv, -ry * inv);
}

// Dinv + b kQrTB^2 (column-major: element (row, col) at col kQrTB + row) =
// the inverse of R's diagonal block b, zero outside the block's nbk x nbk
// upper triangle; one CTA of kQrTB threads per block, thread j forming
// column j by back substitution (R_bb X = I).  R is read through the cache
// (every thread reads the same entry at each step); the columns sit in
// shared memory as Xs[row][col] (consecutive threads, consecutive words).
__global__ void __launch_bounds__(kQrTB)
qr_diag_inv_kernel(int n, const float2 *__restrict__ Q, size_t ldq, float2 *__restrict__ Dinv) {
    __shared__ float2 Xs[kQrTB][kQrTB];
    __shared__ float2 rinv[kQrTB];
    const int b0 = blockIdx.x * kQrTB, nbk = min(kQrTB, n - b0), j = threadIdx.x;
    const float2 *Rb = Q + (size_t)b0 * ldq + b0;   // R[b0 + i][b0 + l] at Rb[l ldq + i]
    for (int i = 0; i < kQrTB; i++) Xs[i][j] = make_float2(0.f, 0.f);
    if (j < nbk) rinv[j] = qr_crecip(Rb[(size_t)j * ldq + j]);
    __syncthreads();
    if (j < nbk) {
        Xs[j][j] = rinv[j];
        for (int i = j - 1; i >= 0; i--) {
            float2 t = make_float2(0.f, 0.f);
            for (int l = i + 1; l <= j; l++) {
                const float2 r = __ldg(Rb + (size_t)l * ldq + i), x = Xs[l][j];
                t.x = fmaf(r.x, x.x, fmaf(-r.y, x.y, t.x));
                t.y = fmaf(r.x, x.y, fmaf(r.y, x.x, t.y));
            }
            const float2 ri = rinv[i];
            Xs[i][j] = make_float2(-(ri.x * t.x - ri.y * t.y), -(ri.x * t.y + ri.y * t.x));
        }
    }
    __syncthreads();
    float2 *D = Dinv + (size_t)blockIdx.x * kQrTB * kQrTB;
    for (int c = 0; c < kQrTB; c++) D[(size_t)c * kQrTB + j] = Xs[j][c];
}

// Each launch issues its loads that do not depend on the vector (R's blocks,
// the inverse) before it reads the vector, so CTA 0 -- the chain from one
// block to the next -- waits about one memory round trip.
constexpr int kQrTsK = kQrTB / kQrTsP;   // columns per thread of a 64-row group

__global__ void __launch_bounds__(kQrTsNT)
qr_trsv_back_kernel(int b0, int b1, int b2, const float2 *__restrict__ Q, size_t ldq,
                    const float2 *__restrict__ Dinv, float2 *X, size_t ldx) {
    float2 *x = X + (size_t)blockIdx.y * ldx;
    const int tid = threadIdx.x, row = tid % kQrTB, p = tid / kQrTB;
    const int np = b2 - b1;
    __shared__ float2 xs[kQrTB], ys[kQrTB];
    __shared__ float2 part[kQrTsP][kQrTB];
    if (blockIdx.x > 0) {
        // rows [0, b0) in groups of kQrTB: y_i -= R[i, b1:b2] x[b1:b2],
        // thread (row, column group p)
        const int i = (blockIdx.x - 1) * kQrTB + row;
        float2 rv[kQrTsK];
#pragma unroll
        for (int t = 0; t < kQrTsK; t++) {
            const int k = p + kQrTsP * t;
            rv[t] = (i < b0 && k < np) ? Q[(size_t)(b1 + k) * ldq + i] : make_float2(0.f, 0.f);
        }
        if (tid < kQrTB) xs[tid] = tid < np ? x[b1 + tid] : make_float2(0.f, 0.f);
        __syncthreads();
        float2 acc = make_float2(0.f, 0.f);
#pragma unroll
        for (int t = 0; t < kQrTsK; t++) {
            const float2 xk = xs[p + kQrTsP * t];
            acc.x += rv[t].x * xk.x - rv[t].y * xk.y;
            acc.y += rv[t].x * xk.y + rv[t].y * xk.x;
        }
        part[p][row] = acc;
        __syncthreads();
        if (p == 0 && i < b0) {
            float2 y = x[i];
#pragma unroll
            for (int q = 0; q < kQrTsP; q++) {
                y.x -= part[q][row].x;
                y.y -= part[q][row].y;
            }
            x[i] = y;
        }
        return;
    }
    const int nbk = b1 - b0;
    const float2 *D = Dinv + (size_t)(b0 / kQrTB) * kQrTB * kQrTB;
    float2 rv[kQrTsK], dv[kQrTsK];
#pragma unroll
    for (int t = 0; t < kQrTsK; t++) {
        const int k = p + kQrTsP * t;
        rv[t] = (row < nbk && k < np) ? Q[(size_t)(b1 + k) * ldq + b0 + row] : make_float2(0.f, 0.f);
        dv[t] = k < nbk ? D[(size_t)k * kQrTB + row] : make_float2(0.f, 0.f);   // Dinv(row, k)
    }
    const float2 y0 = (tid < nbk) ? x[b0 + tid] : make_float2(0.f, 0.f);
    if (tid < kQrTB) xs[tid] = tid < np ? x[b1 + tid] : make_float2(0.f, 0.f);
    __syncthreads();
    {
        float2 acc = make_float2(0.f, 0.f);
#pragma unroll
        for (int t = 0; t < kQrTsK; t++) {
            const float2 xk = xs[p + kQrTsP * t];
            acc.x += rv[t].x * xk.x - rv[t].y * xk.y;
            acc.y += rv[t].x * xk.y + rv[t].y * xk.x;
        }
        part[p][row] = acc;
    }
    __syncthreads();
    if (tid < kQrTB) {
        float2 y = y0;
#pragma unroll
        for (int q = 0; q < kQrTsP; q++) {
            y.x -= part[q][tid].x;
            y.y -= part[q][tid].y;
        }
        ys[tid] = tid < nbk ? y : make_float2(0.f, 0.f);
    }
    __syncthreads();
    float2 acc = make_float2(0.f, 0.f);
#pragma unroll
    for (int t = 0; t < kQrTsK; t++) {
        const float2 yc = ys[p + kQrTsP * t];
        acc.x += dv[t].x * yc.x - dv[t].y * yc.y;
        acc.y += dv[t].x * yc.y + dv[t].y * yc.x;
    }
    part[p][row] = acc;
    __syncthreads();
    if (tid < nbk) {
        float2 t = part[0][tid];
#pragma unroll
        for (int q = 1; q < kQrTsP; q++) {
            t.x += part[q][tid].x;
            t.y += part[q][tid].y;
        }
        x[b0 + tid] = t;
    }
}

__global__ void __launch_bounds__(kQrTsNT)
qr_trsv_fwd_kernel(int bp, int b0, int b1, int n, const float2 *__restrict__ Q, size_t ldq,
                   const float2 *__restrict__ Dinv, float2 *X, size_t ldx) {
    float2 *x = X + (size_t)blockIdx.y * ldx;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int np = b0 - bp;
    if (blockIdx.x > 0) {
        // one warp per row i >= b1: y_i -= sum_k conj(R[k, i]) x_k over the
        // previous block (R's column i is contiguous in k)
        const int i = b1 + (blockIdx.x - 1) * (kQrTsNT / 32) + warp;
        if (i >= n || np <= 0) return;
        float2 acc = make_float2(0.f, 0.f);
        for (int k = lane; k < np; k += 32) {
            const float2 r = Q[(size_t)i * ldq + bp + k], xk = x[bp + k];
            acc.x += r.x * xk.x + r.y * xk.y;
            acc.y += r.x * xk.y - r.y * xk.x;
        }
        for (int o = 16; o > 0; o >>= 1) {
            acc.x += __shfl_xor_sync(0xffffffffu, acc.x, o);
            acc.y += __shfl_xor_sync(0xffffffffu, acc.y, o);
        }
        if (lane == 0) {
            x[i].x -= acc.x;
            x[i].y -= acc.y;
        }
        return;
    }
    // CTA 0: warp w owns rows w R8 .. + R8 - 1 of the block, lanes over k
    constexpr int R8 = kQrTB / (kQrTsNT / 32);
    static_assert(kQrTB == 64, "two columns per lane");
    __shared__ float2 xs[kQrTB], ys[kQrTB];
    __shared__ float2 part[kQrTB];
    const int nbk = b1 - b0;
    const float2 *D = Dinv + (size_t)(b0 / kQrTB) * kQrTB * kQrTB;
    float2 rv[R8][2], dv[R8][2];
#pragma unroll
    for (int r = 0; r < R8; r++) {
        const int row = warp * R8 + r;
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const int k = lane + 32 * h;
            rv[r][h] = (row < nbk && k < np) ? Q[(size_t)(b0 + row) * ldq + bp + k] : make_float2(0.f, 0.f);
            dv[r][h] = (row < nbk && k < nbk) ? D[(size_t)row * kQrTB + k] : make_float2(0.f, 0.f);   // Dinv(k, row)
        }
    }
    const float2 y0 = (tid < nbk) ? x[b0 + tid] : make_float2(0.f, 0.f);
    if (tid < kQrTB) xs[tid] = tid < np ? x[bp + tid] : make_float2(0.f, 0.f);
    __syncthreads();
#pragma unroll
    for (int r = 0; r < R8; r++) {
        float2 acc = make_float2(0.f, 0.f);
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const float2 xk = xs[lane + 32 * h];
            acc.x += rv[r][h].x * xk.x + rv[r][h].y * xk.y;   // conj(R[k, row]) x_k
            acc.y += rv[r][h].x * xk.y - rv[r][h].y * xk.x;
        }
        for (int o = 16; o > 0; o >>= 1) {
            acc.x += __shfl_xor_sync(0xffffffffu, acc.x, o);
            acc.y += __shfl_xor_sync(0xffffffffu, acc.y, o);
        }
        if (lane == 0) part[warp * R8 + r] = acc;
    }
    __syncthreads();
    if (tid < kQrTB) ys[tid] = tid < nbk ? make_float2(y0.x - part[tid].x, y0.y - part[tid].y) : make_float2(0.f, 0.f);
    __syncthreads();
    // x_b = Dinv_b^H y: (Dinv^H)(row, k) = conj(Dinv(k, row))
#pragma unroll
    for (int r = 0; r < R8; r++) {
        float2 acc = make_float2(0.f, 0.f);
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const float2 yc = ys[lane + 32 * h];
            acc.x += dv[r][h].x * yc.x + dv[r][h].y * yc.y;
            acc.y += dv[r][h].x * yc.y - dv[r][h].y * yc.x;
        }
        for (int o = 16; o > 0; o >>= 1) {
            acc.x += __shfl_xor_sync(0xffffffffu, acc.x, o);
            acc.y += __shfl_xor_sync(0xffffffffu, acc.y, o);
        }
        const int row = warp * R8 + r;
        if (lane == 0 && row < nbk) x[b0 + row] = acc;
    }
}

// X (FP64, n x S) from the solved FP32 columns (ld ldq).
__global__ void qr_take_rhs_kernel(int n, int S, const float2 *__restrict__ Qb, size_t ldq, double2 *__restrict__ X) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
    if (i < n) {
        const float2 v = Qb[(size_t)j * ldq + i];
        X[(size_t)j * n + i] = make_double2(v.x, v.y);
    }
}

// gf = g 2^-e (FP32) with 2^e the power of two at or below *nrm (> 0), so the
// FP32 solves run on entries of order one whatever the residual's size.
__global__ void qr_g_to_f32_kernel(int n, const double2 *__restrict__ g, const double *__restrict__ nrm,
                                   float2 *__restrict__ gf) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        const double s = scalbn(1.0, -ilogb(*nrm));
        gf[i] = make_float2((float)(g[i].x * s), (float)(g[i].y * s));
    }
}

// x += d 2^e (the scale qr_g_to_f32_kernel took off).
__global__ void qr_axpy_scaled_kernel(int n, const float2 *__restrict__ d, const double *__restrict__ nrm,
                                      double2 *__restrict__ x) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        const double s = scalbn(1.0, ilogb(*nrm));
        x[i].x += (double)d[i].x * s;
        x[i].y += (double)d[i].y * s;
    }
}

// R X = Y (back) or R^H X = Y (forward) for the S columns of X (ld ldx);
// Dinv from qr_diag_inv_kernel.
void qr_trsv(bool forward, int n, int S, const float2 *Q, size_t ldq, const float2 *Dinv, float2 *X, size_t ldx,
             cudaStream_t st) {
    const int nb = (n + kQrTB - 1) / kQrTB;
    if (!forward) {
        for (int b = nb - 1; b >= 0; b--) {
            const int b0 = b * kQrTB, b1 = std::min(n, b0 + kQrTB), b2 = b == nb - 1 ? b1 : std::min(n, b1 + kQrTB);
            const int others = b2 > b1 ? (b0 + kQrTB - 1) / kQrTB : 0;
            qr_trsv_back_kernel<<<dim3(1 + others, S), kQrTsNT, 0, st>>>(b0, b1, b2, Q, ldq, Dinv, X, ldx);
        }
    } else {
        constexpr int rows_per_cta = kQrTsNT / 32;
        for (int b = 0; b < nb; b++) {
            const int b0 = b * kQrTB, b1 = std::min(n, b0 + kQrTB), bp = b == 0 ? b0 : b0 - kQrTB;
            const int others = b0 > bp ? (n - b1 + rows_per_cta - 1) / rows_per_cta : 0;
            qr_trsv_fwd_kernel<<<dim3(1 + others, S), kQrTsNT, 0, st>>>(bp, b0, b1, n, Q, ldq, Dinv, X, ldx);
        }
    }
    count_launch(nb);
    KERNEL_CHECK();
}

// Cluster size of the panel kernel for `smem16` bytes of shared memory per
// CTA at 16 CTAs: 16 when the device schedules that non-portable size, else
// 8.  The kernel's attributes (shared-memory limit raised to the device's
// opt-in maximum, non-portable cluster sizes allowed) are set once.
int qr_cluster_size(size_t smem16) {
    static std::once_flag once;
    static bool nonportable = false;
    static cudaError_t err = cudaSuccess;
    std::call_once(once, [&] {
        int maxs = 0, dev = 0;
        err = cudaGetDevice(&dev);
        if (err == cudaSuccess) err = cudaDeviceGetAttribute(&maxs, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        cudaFuncAttributes fa{};
        if (err == cudaSuccess) err = cudaFuncGetAttributes(&fa, qr_panel_kernel);   // its static shared memory
        if (err == cudaSuccess)
            err = cudaFuncSetAttribute(qr_panel_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       maxs - (int)fa.sharedSizeBytes);
        if (err == cudaSuccess)
            err = cudaFuncSetAttribute(qr_larft_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)kQrLarftSmem);
        if (err == cudaSuccess)
            err = cudaFuncSetAttribute(qr_pack_tw_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)kQrTwSmem);
        nonportable = cudaFuncSetAttribute(qr_panel_kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) ==
                      cudaSuccess;
        cudaGetLastError();
    });
    CUDA_TRY(err);
    if (!nonportable) return 8;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(16);
    cfg.blockDim = dim3(kQrNT);
    cfg.dynamicSmemBytes = smem16;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = 16;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int nclusters = 0;
    const bool ok = cudaOccupancyMaxActiveClusters(&nclusters, qr_panel_kernel, &cfg) == cudaSuccess && nclusters >= 1;
    cudaGetLastError();
    return ok ? 16 : 8;
}

}  // namespace
}  // namespace bem

using namespace bem;

void bem_solver_s::solve_qr_tc(bem_solve_info_t *info) {
    const int m = R, n = N;
    BEM_CHECK_ARG(m >= n && n >= 1, "QR: fewer rows than unknowns");
    const size_t ldq = (size_t)((m + 1) & ~1);   // even: every column start is 16-byte aligned
    const size_t ncq = (size_t)n + S;
    // workspace: [A | B] (c64) with slack for the GEMM converter's last
    // 16-byte read past the final column, taus, V, its interleaved form, T,
    // G, Z, the packed operands, split-K partial sums, scales, status
    const size_t ldv = (size_t)((m + 1) & ~1);
    const int ldk = ((2 * kQrNB + 3) / 4) * 4;
    q_A.ensure(sizeof(float2) * (ldq * ncq + 8));
    q_tau.ensure(sizeof(float2) * (size_t)n);
    // Look-ahead: panel j + 1 is factored (on a high-priority stream) while
    // the trailing update of panel j runs on the solver's stream, so the
    // panel's buffers (V, its interleaved form, T and G, the packed V) come
    // twice, by panel parity, and the update's (Z, the packed W', split-K
    // partial sums) twice, one set per stream.
    auto r256 = [](size_t b) { return (b + 255) & ~size_t(255); };
    const size_t v_b = r256(sizeof(float2) * ldv * kQrNB), vrr_b = r256(sizeof(float) * 2 * (size_t)m * ldk),
                 t_b = r256(sizeof(float2) * kQrNB * kQrNB + sizeof(float) * 2 * kQrNB * kQrNB),
                 opv_b = r256(tc_operand_bytes(2 * m, 2 * kQrNB, 2)), z_b = r256(sizeof(float) * 2 * kQrNB * ncq),
                 opw_b = r256(tc_operand_bytes(2 * kQrNB, (int)ncq, 2));
    qt_v.ensure(2 * v_b);
    qt_vrr.ensure(2 * vrr_b);
    qt_t.ensure(2 * t_b);
    qt_opv.ensure(2 * opv_b);
    qt_z.ensure(2 * z_b);
    qt_opw.ensure(2 * opw_b);
    auto at = [](DevMem &d, size_t b, int i) { return static_cast<void *>(static_cast<char *>(d.p) + b * i); };
    // split-K partial sums: the largest any panel's products plan, per set (a
    // later panel with fewer tiles may split more than the first)
    size_t pf_n = 1, pf_w = 1;
    for (int j0 = 0; j0 < n; j0 += kQrNB) {
        const int pc = std::min(kQrNB, n - j0), mr = m - j0, c1 = j0 + pc;
        const int pc2 = c1 < n ? std::min(kQrNB, n - c1) : 0, nw = (int)ncq - c1 - pc2;
        pf_n = std::max(pf_n, tc_gemm_part_floats(pc, 2 * mr, 2 * pc, 2));
        if (pc2 > 0)
            pf_n = std::max({pf_n, tc_gemm_part_floats(pc2, 2 * mr, 2 * pc, 2), tc_gemm_part_floats(2 * mr, 2 * pc, pc2, 2)});
        if (nw > 0)
            pf_w = std::max({pf_w, tc_gemm_part_floats(nw, 2 * mr, 2 * pc, 2), tc_gemm_part_floats(2 * mr, 2 * pc, nw, 2)});
    }
    const size_t pn_b = r256(sizeof(float) * pf_n), pw_b = r256(sizeof(float) * pf_w);
    qt_part.ensure(pn_b + pw_b);
    float *const part_set[2] = {qt_part.as<float>(), reinterpret_cast<float *>(static_cast<char *>(qt_part.p) + pn_b)};
    const size_t part_cap[2] = {pn_b / sizeof(float), pw_b / sizeof(float)};
    ensure_aux();
    cudaEvent_t ev_in = qr_ev[0], ev_out = qr_ev[1], ev_ready[2] = {qr_ev[2], qr_ev[3]},
                ev_wide[2] = {qr_ev[4], qr_ev[5]};
    qt_scal.ensure(sizeof(float) * 8);
    qt_dinv.ensure(sizeof(float2) * (size_t)((n + kQrTB - 1) / kQrTB) * kQrTB * kQrTB);
    d_status.ensure(4 * sizeof(int));
    int *status = d_status.as<int>() + 1;
    CUDA_TRY(cudaMemsetAsync(status, 0, sizeof(int), stream));
    float2 *Q = q_A.as<float2>();
    float *sc = qt_scal.as<float>();
    {
        BEM_PROF("qr_copy", stream);
        const dim3 g((n + 31) / 32, (m + 31) / 32);
        if (prec == BEM_PREC_C64)
            qr_copy_a_kernel<float2><<<g, 256, 0, stream>>>(m, n, d_A.as<float2>(), lda, Q, ldq);
        else
            qr_copy_a_kernel<double2><<<g, 256, 0, stream>>>(m, n, d_A.as<double2>(), lda, Q, ldq);
        qr_copy_b_kernel<<<dim3((m + 255) / 256, S), 256, 0, stream>>>(m, S, d_B.as<double2>(), Q + (size_t)n * ldq,
                                                                      ldq);
        CUDA_TRY(cudaMemsetAsync(sc + 4, 0, sizeof(float), stream));
        qr_colnorm_kernel<<<(unsigned)ncq, 256, 0, stream>>>(m, Q, ldq, reinterpret_cast<unsigned *>(sc + 4));
        qr_scales_kernel<<<1, 1, 0, stream>>>(sc);
        count_launch(4);
        KERNEL_CHECK();
    }
    // panel cluster: 16 CTAs when schedulable and the rows fit
    const size_t smax = [] {   // the panel kernel's dynamic shared memory at most
        int dev = 0, v = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        cudaFuncAttributes fa{};
        cudaFuncGetAttributes(&fa, qr_panel_kernel);
        return (size_t)v - fa.sharedSizeBytes;
    }();
    auto smem_for = [](int rows, int cl) { return sizeof(float2) * PanelLayout((rows + cl - 1) / cl).total; };
    const int CL16 = qr_cluster_size(smem_for(m, 16));   // also sets the kernels' shared-memory limits
    const int CL = smem_for(m, 16) <= smax ? CL16 : 8;
    if (smem_for(m, CL) > smax)
        BEM_FAIL(BEM_ERR_TOO_LARGE, "QR_TC: " + std::to_string(m) + " rows do not fit the panel cluster's shared memory");
    // C -= V T^H (V^H C) for the trailing columns C (ncols of them, interleaved
    // real, leading dimension 2 ldq) with update set u on stream st
    auto update = [&](cudaStream_t st, int u, float *C, int ncols, int mr, int pc, const TcOperand &opv,
                      const float2 *Tp, const float *Vrr) {
        BEM_PROF("qr_update", st);
        float *Z = static_cast<float *>(at(qt_z, z_b, u));
        tc_gemm(C, 2 * ldq, false, ncols, 2 * mr, sc, opv, Z, ncols, part_set[u], part_cap[u], status, st);
        TcOperand opw = tc_operand_view(at(qt_opw, opw_b, u), 2 * pc, ncols, 2);
        qr_pack_tw_kernel<2><<<(ncols + kQrTwCols - 1) / kQrTwCols, kQrNB * kQrTwGroups, kQrTwSmem, st>>>(
            ncols, pc, Z, Tp, opw.Kp, opw.ncols_pad, opw.planes, opw.col_inv);
        count_launch();
        tc_gemm(Vrr, ldk, false, 2 * mr, 2 * pc, sc + 2, opw, C, 2 * ldq, part_set[u], part_cap[u], status, st, true);
    };
    // Panel j on qr_aux, its T and the update of panel j + 1's columns
    // (narrow) there too, the update of the rest (wide, B included) on the
    // solver's stream.  The narrow update of panel j waits for the wide
    // update of panel j - 1 (it also updated those columns); so does
    // everything after it on qr_aux, including panel j + 1, whose columns the
    // wide update of panel j - 1 touched too, and the reuse of panel j - 1's
    // buffers by panel j + 1.
    cudaStream_t sa = qr_aux;
    CUDA_TRY(cudaEventRecord(ev_in, stream));
    CUDA_TRY(cudaStreamWaitEvent(sa, ev_in, 0));
    bool wide_prev = false;
    for (int j0 = 0, step = 0; j0 < n; j0 += kQrNB, step++) {
        const int pc = std::min(kQrNB, n - j0), mr = m - j0, par = step & 1;
        const int c1 = j0 + pc;
        const int pc2 = c1 < n ? std::min(kQrNB, n - c1) : 0;   // the next panel's columns
        const int nw = (int)ncq - c1 - pc2;                      // the rest, B included
        {
            BEM_PROF("qr_panel", sa);
            const int rb = (mr + CL - 1) / CL;
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3(CL);
            cfg.blockDim = dim3(kQrNT);
            cfg.dynamicSmemBytes = smem_for(mr, CL);
            cfg.stream = sa;
            cudaLaunchAttribute at_[1];
            at_[0].id = cudaLaunchAttributeClusterDimension;
            at_[0].val.clusterDim.x = CL;
            at_[0].val.clusterDim.y = 1;
            at_[0].val.clusterDim.z = 1;
            cfg.attrs = at_;
            cfg.numAttrs = 1;
            CUDA_TRY(cudaLaunchKernelEx(&cfg, qr_panel_kernel, Q, ldq, m, j0, pc, rb, q_tau.as<float2>() + j0,
                                        status));
            count_launch();
        }
        if (pc2 + nw <= 0) continue;
        float2 *P = Q + (size_t)j0 * ldq + j0;   // the panel
        float2 *Vp = static_cast<float2 *>(at(qt_v, v_b, par));
        float *Vrr = static_cast<float *>(at(qt_vrr, vrr_b, par));
        float2 *Tp = static_cast<float2 *>(at(qt_t, t_b, par));
        float *Gp = reinterpret_cast<float *>(Tp + kQrNB * kQrNB);
        const TcOperand opv = tc_operand_view(at(qt_opv, opv_b, par), 2 * mr, 2 * pc, 2);
        {
            BEM_PROF("qr_t", sa);
            qr_vfull_kernel<<<dim3((mr + 255) / 256, pc), 256, 0, sa>>>(mr, pc, P, ldq, Vp, ldv);
            TcOperand opvw = opv;
            tc_pack_cplx_f32(Vp, mr, pc, opvw, sa, ldv, true);
            // G = V^H V (pc x pc): conj(V^T) V with V^T's rows the columns of Vf
            tc_gemm(reinterpret_cast<const float *>(Vp), 2 * ldv, false, pc, 2 * mr, sc + 2, opv, Gp, pc,
                    part_set[0], part_cap[0], status, sa);
            qr_larft_kernel<<<1, kQrLarftNT, kQrLarftSmem, sa>>>(pc, Gp, q_tau.as<float2>() + j0, Tp);
            qr_vrr_kernel<<<mr, kQrNB, 0, sa>>>(mr, pc, Vp, ldv, Vrr, ldk);
            count_launch(3);
        }
        if (wide_prev) CUDA_TRY(cudaStreamWaitEvent(sa, ev_wide[par ^ 1], 0));
        if (pc2 > 0) update(sa, 0, reinterpret_cast<float *>(P + (size_t)pc * ldq), pc2, mr, pc, opv, Tp, Vrr);
        CUDA_TRY(cudaEventRecord(ev_ready[par], sa));
        wide_prev = nw > 0;
        if (nw > 0) {
            CUDA_TRY(cudaStreamWaitEvent(stream, ev_ready[par], 0));
            update(stream, 1, reinterpret_cast<float *>(P + (size_t)(pc + pc2) * ldq), nw, mr, pc, opv, Tp, Vrr);
            CUDA_TRY(cudaEventRecord(ev_wide[par], stream));
        }
        KERNEL_CHECK();
    }
    CUDA_TRY(cudaEventRecord(ev_out, sa));
    CUDA_TRY(cudaStreamWaitEvent(stream, ev_out, 0));
    // X = R^{-1} (Q^H B)[0:n]
    double2 *X = d_x.as<double2>();
    {
        BEM_PROF("qr_trsv", stream);
        qr_diag_inv_kernel<<<(n + kQrTB - 1) / kQrTB, kQrTB, 0, stream>>>(n, Q, ldq, qt_dinv.as<float2>());
        count_launch();
        qr_trsv(false, n, S, Q, ldq, qt_dinv.as<float2>(), Q + (size_t)n * ldq, ldq, stream);   // in place on (Q^H B)[0:n]
        qr_take_rhs_kernel<<<dim3((n + 255) / 256, S), 256, 0, stream>>>(n, S, Q + (size_t)n * ldq, ldq, X);
        count_launch();
    }
    // FP64 refinement through the semi-normal equations with the FP32 factor
    w_r.ensure(sizeof(double2) * (size_t)m);
    w_gv.ensure(sizeof(double2) * (size_t)n);
    w_vf.ensure(sizeof(float2) * (2 * (size_t)std::max(n, m) + 2));
    w_part.ensure(std::max(sizeof(float2) * (size_t)gemv_h_splits(m, n), sizeof(double2) * (size_t)gemv_h_f64_splits(m, n)) *
                  (size_t)n);
    w_scal.ensure(sizeof(double) * 8);
    double *scal = w_scal.as<double>();
    auto read_scalar = [&](int i) {
        CUDA_TRY(cudaMemcpyAsync(h_pinned + i, scal + i, sizeof(double), cudaMemcpyDeviceToHost, stream));
        CUDA_TRY(cudaStreamSynchronize(stream));
        return h_pinned[i];
    };
    int steps_max = 0;
    double worst = 0.0;
    bool all_conv = true;
    const double tol = kQrRefineTol;
    for (int s = 0; s < S; s++) {
        const double2 *b = d_B.as<double2>() + (size_t)s * m;
        double2 *x = X + (size_t)s * n;
        launch_gemv_h_f64(prec, m, n, d_A.p, lda, b, w_gv.as<double2>(), w_part.as<double2>(), w_vf.as<float2>(),
                          stream);
        launch_nrm2(n, w_gv.as<double2>(), scal + 0, w_part.as<double>(), stream);
        const double bn = read_scalar(0);
        double rel = 0.0, prev = 1e300;
        int it = 0;
        bool conv = !(bn > 0.0);
        for (; !conv && it <= opt.max_refine; it++) {
            BEM_PROF("qr_refine", stream);
            launch_resid(prec, m, n, d_A.p, lda, x, b, w_r.as<double2>(), w_vf.as<float2>(), stream);
            launch_gemv_h_f64(prec, m, n, d_A.p, lda, w_r.as<double2>(), w_gv.as<double2>(), w_part.as<double2>(),
                              w_vf.as<float2>(), stream);
            launch_nrm2(n, w_gv.as<double2>(), scal + 1, w_part.as<double>(), stream);
            rel = read_scalar(1) / bn;
            if (!std::isfinite(rel)) {
                int h_st = 0;   // a tensor-core GEMM that gave up on a wait explains it
                CUDA_TRY(cudaMemcpy(&h_st, status, sizeof(int), cudaMemcpyDeviceToHost));
                if (h_st) BEM_FAIL(BEM_ERR_TIMEOUT, "QR_TC: a bounded wait of the tensor-core GEMM timed out");
                BEM_FAIL(BEM_ERR_NUMERIC, "QR refinement residual is not finite");
            }
            if (rel <= tol) { conv = true; break; }
            if (rel > 0.5 * prev || it == opt.max_refine) {
                // stagnated at the precision of the FP64-accurate products:
                // converged when that level is FP64's
                conv = rel <= kQrStagnationOk;
                break;
            }
            prev = rel;
            // R^H y = g, R d = y in FP32 on g scaled to order one (the free
            // Z buffer), then x += d
            float2 *gf = qt_z.as<float2>();
            qr_g_to_f32_kernel<<<(n + 255) / 256, 256, 0, stream>>>(n, w_gv.as<double2>(), scal + 1, gf);
            qr_trsv(true, n, 1, Q, ldq, qt_dinv.as<float2>(), gf, n, stream);
            qr_trsv(false, n, 1, Q, ldq, qt_dinv.as<float2>(), gf, n, stream);
            qr_axpy_scaled_kernel<<<(n + 255) / 256, 256, 0, stream>>>(n, gf, scal + 1, x);
            count_launch(2);
        }
        steps_max = std::max(steps_max, it);
        worst = std::max(worst, rel);
        all_conv &= conv;
    }
    CUDA_TRY(cudaStreamSynchronize(stream));
    int h_status = 0;
    CUDA_TRY(cudaMemcpy(&h_status, status, sizeof(int), cudaMemcpyDeviceToHost));
    if (h_status) BEM_FAIL(BEM_ERR_TIMEOUT, "QR_TC: a bounded wait of the tensor-core GEMM timed out");
    if (info) {
        info->iterations = 0;
        info->refinements = steps_max;
        info->rel_residual = worst;
        info->converged = all_conv ? 1 : 0;
    }
}
