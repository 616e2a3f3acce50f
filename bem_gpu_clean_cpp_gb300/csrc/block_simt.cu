// FP32 products of the block solve on the CUDA cores (BEM_GEMM_SIMT):
//   T = A X   (block_av_kernel)    and    W = A^H T   (block_aht_kernel)
// with A the row-major R x N c64 system matrix (rows = collocation points,
// leading dimension lda, a multiple of 8), X and W N x S column-major c64,
// and T planar: R x 2S floats, Re T in columns 0..S-1 and Im T in columns
// S..2S-1 (the layout the residual and gradient kernels of block.cu use).
//
// At 2S <= 64 real columns the interleaved-real GEMMs are too skinny for the
// library GEMMs: on a 40962-node system cuBLAS SGEMM took 4.3-6.1 ms per
// product for 4..16 sources where one pass over A (13.4 GB) takes about
// 2.1 ms, and its FP32 emulation on the tensor cores is not used at these
// shapes.  Here each product streams A once through shared memory (cp.async,
// kStages-deep pipeline) for up to 32 sources (more take further passes);
// every element of A feeds 4 x SB FMAs, every thread keeps 128 accumulators.
//
// The complex multiply-adds run as packed two-lane FP32 FMAs
// (fma.rn.f32x2: (re, im) += (p, q) * (u, v)), two per complex product, which
// halves the instructions issued per FMA.  The operand pairs are prepared so
// that the inner loops hold no shuffles:
//   T += a x:       (re, im) += (ar, ai) * (xr, xr) + (-ai, ar) * (xi, xi)
//                   X packed beforehand as (xr, xr, xi, xi) per element;
//   W += conj(a) t: (re, im) += (ar, ar) * (tr, ti) + (ai, ai) * (ti, -tr)
//                   T packed beforehand as (tr, ti, ti, -tr) per element.
// The FMAs are the same as in scalar FP32 code (each output component is a
// chain of single-rounded FMAs), so the results are FP32-accurate.
//
// T = A X: lane l of every warp owns the rows l, l+32, .. (TM rows; a CTA
// 32 TM rows) and the 8 warps split each stage's 32 columns, two column pairs
// each, so the X values a warp reads are the same in every lane
// (shared-memory broadcasts) and each A value is read by one lane.  A rows
// are padded to 272 bytes in shared memory so that the lanes' 16-byte reads
// of 32 different rows fall in distinct banks.
// W = A^H T: lane l owns the column pairs (2l, 2l+1), (64+2l, 65+2l), ..
// (TK columns; a CTA 32 TK columns) and each warp takes 4 of a stage's 32
// rows, reading their T values as broadcasts.
// In both the 8 warps' partial sums are added in fixed order through shared
// memory at the end, and the reduction dimension is split over grid.y when
// that evens out the waves of one CTA per SM; the splits' partial results are
// summed in fixed order by sum_parts_kernel.  No atomics: results are bitwise
// reproducible.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <mutex>

#include "bem_common.h"
#include "kernels.h"
#include "tma.h"

namespace bem {
namespace {

constexpr int kThreads = 256;    // 8 warps
constexpr int kWarps = kThreads / 32;
constexpr int kStages = 4;       // cp.async pipeline depth
constexpr int kAvBK = 32;        // block_av_kernel: columns per stage (2 column pairs per warp)
constexpr int kAvLd = kAvBK + 2; // block_av_kernel: shared-memory row stride (float2), 272 bytes
constexpr int kAhBR = 32;        // block_aht_kernel: rows per stage (4 per warp)
constexpr int kMaxSplits = 16;

// 16-byte asynchronous copy global -> shared; `bytes` < 16 zero-fills the
// rest (0: nothing is read, the destination is zeroed).
__device__ __forceinline__ void cp16(uint32_t dst, const void *src, int bytes) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst), "l"(src), "r"(bytes) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// Two floats in one 64-bit register pair (lo = first lane) and back.
__device__ __forceinline__ uint64_t pk2(float lo, float hi) {
    uint64_t r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ void up2(uint64_t v, float &lo, float &hi) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
// d = a * b + d lane by lane, each lane one single-rounded FP32 FMA.
__device__ __forceinline__ void fma2(uint64_t &d, uint64_t a, uint64_t b) {
    asm("fma.rn.f32x2 %0, %1, %2, %0;" : "+l"(d) : "l"(a), "l"(b));
}

template <int TM, int SB>
constexpr size_t av_smem() {
    return std::max(sizeof(float2) * (size_t)kStages * 32 * TM * kAvLd + sizeof(float4) * (size_t)kStages * SB * kAvBK,
                    sizeof(float) * (size_t)kWarps * 2 * TM * SB * 32);
}

template <int TK, int SB>
constexpr size_t aht_smem() {
    return std::max(sizeof(float2) * (size_t)kStages * kAhBR * 32 * TK + sizeof(float4) * (size_t)kStages * kAhBR * SB,
                    sizeof(float) * (size_t)kWarps * 2 * TK * SB * 32);
}

// Adds the 8 warps' accumulators (each lane NV floats) in warp order through
// shared memory; calls emit(j, l, sum) for the sum of value j of lane l.
template <int NV, typename Emit>
__device__ __forceinline__ void cta_sum(const uint64_t (&acc)[NV / 2], unsigned char *smem, Emit emit) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    float *red = reinterpret_cast<float *>(smem);   // [warp][NV][lane]
#pragma unroll
    for (int j = 0; j < NV / 2; j++) {
        float lo, hi;
        up2(acc[j], lo, hi);
        red[(warp * NV + 2 * j) * 32 + lane] = lo;
        red[(warp * NV + 2 * j + 1) * 32 + lane] = hi;
    }
    __syncthreads();
    for (int e = tid; e < NV * 32; e += kThreads) {
        const int j = e >> 5, l = e & 31;
        float sum = 0.f;
#pragma unroll
        for (int w = 0; w < kWarps; w++) sum += red[(w * NV + j) * 32 + l];
        emit(j, l, sum);
    }
}

// T (or split y's partial T at out + y * split_stride) = A X for the rows
// blockIdx.x * 32 TM ..+32 TM, the column chunks [y cps, min((y+1) cps, nch))
// of 32 columns, the sources blockIdx.z * SB ..+SB.  Xd: X packed as
// (xr, xr, xi, xi) per element, N x S column-major float4.
template <int TM, int SB>
__global__ void __launch_bounds__(kThreads, 1)
block_av_kernel(int R, int N, int S, const float2 *__restrict__ A, size_t lda, const float4 *__restrict__ Xd,
                int cps, int nch, float *__restrict__ out, size_t split_stride) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr int RB = 32 * TM;                 // rows per CTA
    constexpr int kAStage = RB * kAvLd;         // float2 per stage
    constexpr int kXStage = SB * kAvBK;         // float4 per stage
    constexpr int NV = 2 * TM * SB;             // accumulators: [row r][source s][re, im]
    float2 *As = reinterpret_cast<float2 *>(smem_raw);
    float4 *Xs = reinterpret_cast<float4 *>(As + kStages * kAStage);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int r0 = blockIdx.x * RB, s0 = blockIdx.z * SB;
    const int c_beg = blockIdx.y * cps, nloc = min(c_beg + cps, nch) - c_beg;

    // Copy geometry of this thread, fixed for the whole kernel.  A: rows
    // a_row + 16 q (q < 2 TM) of the block, column pair a_pc of each stage;
    // Xd: sources x_s + 8 q (q < SB / 8; SB = 4: x_s < 4), column x_k.
    constexpr int kAq = RB * 16 / kThreads, kXq = SB * kAvBK / kThreads;
    const int a_row = tid >> 4, a_pc = tid & 15, x_s = tid >> 5, x_k = tid & 31;
    uint32_t a_rows_ok = 0, x_srcs_ok = 0;
#pragma unroll
    for (int q = 0; q < kAq; q++) a_rows_ok |= (r0 + a_row + 16 * q < R ? 1u : 0u) << q;
#pragma unroll
    for (int q = 0; q < (kXq > 0 ? kXq : 1); q++)
        x_srcs_ok |= (x_s + 8 * q < SB && s0 + x_s + 8 * q < S ? 1u : 0u) << q;
    const float2 *a_base = A + (size_t)(r0 + a_row) * lda + 2 * a_pc;   // read only for valid rows
    const float4 *x_base = Xd + (size_t)(s0 + x_s) * N + x_k;            // read only for valid sources
    const size_t a_step = 16 * lda, x_step = 8 * (size_t)N;
    const uint32_t a_dst = smem_u32(As) + sizeof(float2) * (a_row * kAvLd + 2 * a_pc);
    const uint32_t x_dst = smem_u32(Xs) + sizeof(float4) * (x_s * kAvBK + x_k);

    auto load = [&](int c, int b) {
        const int k0 = c * kAvBK;
        const int ka = k0 + 2 * a_pc, kx = k0 + x_k;
        const int a_bytes = ka < N ? 8 * min(N - ka, 2) : 0, x_bytes = kx < N ? 16 : 0;
        const float2 *src = a_base + k0;
        const uint32_t dst = a_dst + b * (uint32_t)(sizeof(float2) * kAStage);
#pragma unroll
        for (int q = 0; q < kAq; q++) {
            const bool ok = (a_rows_ok >> q) & 1u;
            cp16(dst + q * (uint32_t)(sizeof(float2) * 16 * kAvLd), ok ? (const void *)src : (const void *)A,
                 ok ? a_bytes : 0);
            src += a_step;
        }
        const float4 *xsrc = x_base + k0;
        const uint32_t xd = x_dst + b * (uint32_t)(sizeof(float4) * kXStage);
#pragma unroll
        for (int q = 0; q < (kXq > 0 ? kXq : 1); q++) {
            if (kXq == 0 && x_s >= SB) break;
            const bool ok = (x_srcs_ok >> q) & 1u;
            cp16(xd + q * (uint32_t)(sizeof(float4) * 8 * kAvBK), ok ? (const void *)xsrc : (const void *)Xd,
                 ok ? x_bytes : 0);
            xsrc += x_step;
        }
    };

    uint64_t acc[NV / 2];
#pragma unroll
    for (int j = 0; j < NV / 2; j++) acc[j] = 0;

#pragma unroll
    for (int q = 0; q < kStages - 1; q++) {
        if (q < nloc) load(c_beg + q, q);
        cp_commit();
    }
    for (int it = 0; it < nloc; it++) {
        cp_wait<kStages - 2>();
        __syncthreads();   // stage `it` visible to all; stage it-1 free for the refill
        if (it + kStages - 1 < nloc) load(c_beg + it + kStages - 1, (it + kStages - 1) % kStages);
        cp_commit();
        const int b = it % kStages;
        const float2 *as = As + b * kAStage + lane * kAvLd;
        const ulonglong2 *xs = reinterpret_cast<const ulonglong2 *>(Xs + b * kXStage);
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const int kp = 2 * warp + h;   // column pair of the stage: columns 2 kp, 2 kp + 1
            float4 a[TM];
#pragma unroll
            for (int r = 0; r < TM; r++) a[r] = *reinterpret_cast<const float4 *>(as + 32 * r * kAvLd + 2 * kp);
#pragma unroll
            for (int j = 0; j < 2; j++) {   // column 2 kp + j
                uint64_t an[TM], ar[TM];     // (ar, ai) and (-ai, ar)
#pragma unroll
                for (int r = 0; r < TM; r++) {
                    const float re = j ? a[r].z : a[r].x, im = j ? a[r].w : a[r].y;
                    an[r] = pk2(re, im);
                    ar[r] = pk2(-im, re);
                }
#pragma unroll
                for (int s = 0; s < SB; s++) {
                    const ulonglong2 x = xs[s * kAvBK + 2 * kp + j];   // same address in every lane: broadcast
#pragma unroll
                    for (int r = 0; r < TM; r++) fma2(acc[r * SB + s], an[r], x.x);
#pragma unroll
                    for (int r = 0; r < TM; r++) fma2(acc[r * SB + s], ar[r], x.y);
                }
            }
        }
    }
    cp_wait<0>();
    __syncthreads();   // every warp is done with the stages: reuse them for the warp sums

    float *o = out + (size_t)blockIdx.y * split_stride;
    cta_sum<NV>(acc, smem_raw, [&](int j, int l, float sum) {
        const int c = j & 1, s = (j >> 1) % SB, r = (j >> 1) / SB;
        const int i = r0 + l + 32 * r;
        if (i < R && s0 + s < S) o[(size_t)(c ? S + s0 + s : s0 + s) * R + i] = sum;
    });
}

// W (or split y's partial W at out + y * split_stride) = A^H T for the
// columns blockIdx.x * 32 TK ..+32 TK, the row chunks [y cps, min((y+1) cps,
// nch)) of 32 rows, the sources blockIdx.z * SB ..+SB.  Tq: T packed as
// (tr, ti, ti, -tr) per element, R x S row-major float4.
template <int TK, int SB>
__global__ void __launch_bounds__(kThreads, 1)
block_aht_kernel(int R, int N, int S, const float2 *__restrict__ A, size_t lda, const float4 *__restrict__ Tq,
                 int cps, int nch, float2 *__restrict__ out, size_t split_stride) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr int CB = 32 * TK;                 // columns per CTA
    constexpr int kAStage = kAhBR * CB;         // float2 per stage
    constexpr int kTStage = kAhBR * SB;         // float4 per stage
    constexpr int NV = 2 * TK * SB;             // accumulators: [column q][source s][re, im]
    float2 *As = reinterpret_cast<float2 *>(smem_raw);
    float4 *Ts = reinterpret_cast<float4 *>(As + kStages * kAStage);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int c0 = blockIdx.x * CB, s0 = blockIdx.z * SB;
    const int ch_beg = blockIdx.y * cps, nloc = min(ch_beg + cps, nch) - ch_beg;

    // Copy geometry of this thread, fixed for the whole kernel.  A: rows
    // a_row + RQ q (q < kAq) of each stage, column pair a_pc of the block;
    // Tq: rows t_row + TQ q (q < SB / 8; SB = 4: t_row < 32), source t_s.
    constexpr int kAq = kAhBR * CB / 2 / kThreads, RQ = kThreads / (CB / 2);
    constexpr int kTq = kAhBR * SB / kThreads, TQ = kThreads / SB;
    const int a_row = tid / (CB / 2), a_pc = tid % (CB / 2);
    const int t_row = tid / SB, t_s = tid % SB;
    const int ka = c0 + 2 * a_pc;
    const int a_bytes = ka < N ? 8 * min(N - ka, 2) : 0;
    const int t_bytes = s0 + t_s < S ? 16 : 0;
    const float2 *a_base = A + (size_t)a_row * lda + (a_bytes ? ka : 0);
    const float4 *t_base = Tq + (size_t)t_row * S + (t_bytes ? s0 + t_s : 0);
    const size_t a_step = (size_t)RQ * lda, t_step = (size_t)TQ * S;
    const uint32_t a_dst = smem_u32(As) + 16 * tid;
    const uint32_t t_dst = smem_u32(Ts) + 16 * tid;

    auto load = [&](int c, int b) {
        const int i0 = c * kAhBR;
        const bool full = i0 + kAhBR <= R;
        const float2 *src = a_base + (size_t)i0 * lda;
        const uint32_t dst = a_dst + b * (uint32_t)(sizeof(float2) * kAStage);
#pragma unroll
        for (int q = 0; q < kAq; q++) {
            const bool ok = a_bytes && (full || i0 + a_row + RQ * q < R);
            cp16(dst + q * (uint32_t)(16 * kThreads), ok ? (const void *)src : (const void *)A, ok ? a_bytes : 0);
            src += a_step;
        }
        const float4 *tsrc = t_base + (size_t)i0 * S;
        const uint32_t td = t_dst + b * (uint32_t)(sizeof(float4) * kTStage);
#pragma unroll
        for (int q = 0; q < (kTq > 0 ? kTq : 1); q++) {
            if (kTq == 0 && t_row >= kAhBR) break;
            const bool ok = t_bytes && (full || i0 + t_row + TQ * q < R);
            cp16(td + q * (uint32_t)(16 * kThreads), ok ? (const void *)tsrc : (const void *)Tq, ok ? 16 : 0);
            tsrc += t_step;
        }
    };

    uint64_t acc[NV / 2];
#pragma unroll
    for (int j = 0; j < NV / 2; j++) acc[j] = 0;

#pragma unroll
    for (int q = 0; q < kStages - 1; q++) {
        if (q < nloc) load(ch_beg + q, q);
        cp_commit();
    }
    for (int it = 0; it < nloc; it++) {
        cp_wait<kStages - 2>();
        __syncthreads();
        if (it + kStages - 1 < nloc) load(ch_beg + it + kStages - 1, (it + kStages - 1) % kStages);
        cp_commit();
        const int b = it % kStages;
        const float4 *as = reinterpret_cast<const float4 *>(As + b * kAStage);
        const ulonglong2 *ts = reinterpret_cast<const ulonglong2 *>(Ts + b * kTStage);
#pragma unroll
        for (int rr = 0; rr < 4; rr++) {
            const int row = warp * 4 + rr;
            uint64_t dr[TK], di[TK];   // (ar, ar) and (ai, ai)
#pragma unroll
            for (int h = 0; h < TK / 2; h++) {
                const float4 a = as[row * (CB / 2) + 32 * h + lane];   // columns 64 h + 2 lane, +1
                dr[2 * h] = pk2(a.x, a.x);
                di[2 * h] = pk2(a.y, a.y);
                dr[2 * h + 1] = pk2(a.z, a.z);
                di[2 * h + 1] = pk2(a.w, a.w);
            }
#pragma unroll
            for (int s = 0; s < SB; s++) {
                const ulonglong2 t = ts[row * SB + s];   // same address in every lane: broadcast
#pragma unroll
                for (int q = 0; q < TK; q++) fma2(acc[q * SB + s], dr[q], t.x);
#pragma unroll
                for (int q = 0; q < TK; q++) fma2(acc[q * SB + s], di[q], t.y);
            }
        }
    }
    cp_wait<0>();
    __syncthreads();   // every warp is done with the stages: reuse them for the warp sums

    float *o = reinterpret_cast<float *>(out + (size_t)blockIdx.y * split_stride);
    cta_sum<NV>(acc, smem_raw, [&](int j, int l, float sum) {
        const int c = j & 1, s = (j >> 1) % SB, q = (j >> 1) / SB;
        const int col = c0 + (q >> 1) * 64 + 2 * l + (q & 1);
        if (col < N && s0 + s < S) o[((size_t)(s0 + s) * N + col) * 2 + c] = sum;
    });
}

// Xd[s N + k] = (xr, xr, xi, xi) for x = X[s N + k] (c64 or c128).
template <typename TX>
__global__ void pack_x_kernel(size_t n, const TX *__restrict__ X, float4 *__restrict__ Xd) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const TX v = X[i];
        const float re = (float)v.x, im = (float)v.y;
        Xd[i] = make_float4(re, re, im, im);
    }
}

// Tq[i S + s] = (tr, ti, ti, -tr) for the planar T (R x 2S floats).
__global__ void pack_t_kernel(int R, int S, const float *__restrict__ T, float4 *__restrict__ Tq) {
    const size_t n = (size_t)R * S;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
        const int s = (int)(e / R), i = (int)(e % R);   // coalesced reads of the planar columns
        const float tr = T[(size_t)s * R + i], ti = T[(size_t)(S + s) * R + i];
        Tq[(size_t)i * S + s] = make_float4(tr, ti, ti, -tr);
    }
}

// out[i] = sum over y < ns of part[y * stride + i], y in increasing order.
__global__ void sum_parts_kernel(size_t n, const float *__restrict__ part, size_t stride, int ns,
                                 float *__restrict__ out) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        float s = part[i];
        for (int y = 1; y < ns; y++) s += part[y * stride + i];
        out[i] = s;
    }
}

int num_sms() { return device_sm_count(); }

// Splits of the reduction dimension (nred chunks) for `units` CTAs per split:
// the count (<= kMaxSplits, >= 4 chunks per split) whose waves of one CTA per
// SM are best filled, fewer splits on near ties.
int pick_splits(long long units, int nred) {
    const int sms = num_sms();
    const int kmax = std::max(1, std::min(kMaxSplits, nred / 4));
    int best = 1;
    double best_score = -1.0;
    for (int k = 1; k <= kmax; k++) {
        const long long ctas = units * k;
        const long long waves = (ctas + sms - 1) / sms;
        const double score = (double)ctas / (double)(waves * sms) - 0.004 * k;
        if (score > best_score + 1e-12) {
            best_score = score;
            best = k;
        }
    }
    return best;
}

// Sources per pass SB and rows (columns) per lane TM: 4 x 4, 4 x 8, 4 x 16 up
// to 16 sources, 2 x 32 above (passes of 32).
struct Plan {
    int sb, tm, passes, nch, cps, splits;
};

Plan plan(int S, int nout, int nred_chunks) {
    Plan p;
    p.sb = S <= 4 ? 4 : S <= 8 ? 8 : S <= 16 ? 16 : 32;
    p.tm = p.sb == 32 ? 2 : 4;
    p.passes = (S + p.sb - 1) / p.sb;
    p.nch = nred_chunks;
    const int per_cta = 32 * p.tm;   // rows (T = A X) or columns (W = A^H T) per CTA
    const long long units = (long long)((nout + per_cta - 1) / per_cta) * p.passes;
    p.splits = pick_splits(units, p.nch);
    p.cps = (p.nch + p.splits - 1) / p.splits;
    p.splits = (p.nch + p.cps - 1) / p.cps;
    return p;
}

Plan plan_av(int R, int N, int S) { return plan(S, R, (N + kAvBK - 1) / kAvBK); }
Plan plan_aht(int R, int N, int S) { return plan(S, N, (R + kAhBR - 1) / kAhBR); }

cudaError_t set_smem_attributes() {
    static std::once_flag once;
    static cudaError_t err = cudaSuccess;
    std::call_once(once, [] {
        auto set = [](const void *f, size_t bytes) {
            if (err == cudaSuccess)
                err = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
        };
        set((const void *)block_av_kernel<4, 4>, av_smem<4, 4>());
        set((const void *)block_av_kernel<4, 8>, av_smem<4, 8>());
        set((const void *)block_av_kernel<4, 16>, av_smem<4, 16>());
        set((const void *)block_av_kernel<2, 32>, av_smem<2, 32>());
        set((const void *)block_aht_kernel<4, 4>, aht_smem<4, 4>());
        set((const void *)block_aht_kernel<4, 8>, aht_smem<4, 8>());
        set((const void *)block_aht_kernel<4, 16>, aht_smem<4, 16>());
        set((const void *)block_aht_kernel<2, 32>, aht_smem<2, 32>());
    });
    return err;
}

unsigned ew_grid(size_t n) { return (unsigned)std::min<size_t>((n + 255) / 256, (size_t)num_sms() * 8); }

// floats of the packed operand (Xd or Tq) at the head of the scratch
size_t pack_floats(int R, int N, int S) { return 4 * (size_t)S * std::max(R, N); }

template <typename TX>
void launch_av(const float2 *A, size_t lda, int R, int N, int S, const TX *X, float *T, float *scratch,
               cudaStream_t st) {
    CUDA_TRY(set_smem_attributes());
    const Plan p = plan_av(R, N, S);
    float4 *Xd = reinterpret_cast<float4 *>(scratch);
    pack_x_kernel<TX><<<ew_grid((size_t)N * S), 256, 0, st>>>((size_t)N * S, X, Xd);
    count_launch();
    float *part = scratch + pack_floats(R, N, S);
    const size_t stride = 2 * (size_t)S * R;
    float *out = p.splits > 1 ? part : T;
    const dim3 grid((R + 32 * p.tm - 1) / (32 * p.tm), p.splits, p.passes);
#define BEM_AV(TM, SB) \
    block_av_kernel<TM, SB><<<grid, kThreads, av_smem<TM, SB>(), st>>>(R, N, S, A, lda, Xd, p.cps, p.nch, out, stride)
    if (p.sb == 4)
        BEM_AV(4, 4);
    else if (p.sb == 8)
        BEM_AV(4, 8);
    else if (p.sb == 16)
        BEM_AV(4, 16);
    else
        BEM_AV(2, 32);
#undef BEM_AV
    count_launch();
    if (p.splits > 1) {
        sum_parts_kernel<<<ew_grid(stride), 256, 0, st>>>(stride, part, stride, p.splits, T);
        count_launch();
    }
    KERNEL_CHECK();
}

}  // namespace

size_t block_simt_scratch_floats(int R, int N, int S) {
    const Plan a = plan_av(R, N, S), h = plan_aht(R, N, S);
    const size_t fa = a.splits > 1 ? (size_t)a.splits * 2 * S * (size_t)R : 0;
    const size_t fh = h.splits > 1 ? (size_t)h.splits * 2 * S * (size_t)N : 0;
    return pack_floats(R, N, S) + std::max(fa, fh);
}

void launch_block_av(const float2 *A, size_t lda, int R, int N, int S, const float2 *X, float *T, float *scratch,
                     cudaStream_t st) {
    launch_av<float2>(A, lda, R, N, S, X, T, scratch, st);
}

void launch_block_av_c128(const float2 *A, size_t lda, int R, int N, int S, const double2 *X, float *T,
                          float *scratch, cudaStream_t st) {
    launch_av<double2>(A, lda, R, N, S, X, T, scratch, st);
}

void launch_block_aht(const float2 *A, size_t lda, int R, int N, int S, const float *T, float2 *W, float *scratch,
                      cudaStream_t st) {
    CUDA_TRY(set_smem_attributes());
    const Plan p = plan_aht(R, N, S);
    float4 *Tq = reinterpret_cast<float4 *>(scratch);
    pack_t_kernel<<<ew_grid((size_t)R * S), 256, 0, st>>>(R, S, T, Tq);
    count_launch();
    float *part = scratch + pack_floats(R, N, S);
    const size_t stride = (size_t)S * N;   // float2
    float2 *out = p.splits > 1 ? reinterpret_cast<float2 *>(part) : W;
    const dim3 grid((N + 32 * p.tm - 1) / (32 * p.tm), p.splits, p.passes);
#define BEM_AHT(TK, SB) \
    block_aht_kernel<TK, SB><<<grid, kThreads, aht_smem<TK, SB>(), st>>>(R, N, S, A, lda, Tq, p.cps, p.nch, out, stride)
    if (p.sb == 4)
        BEM_AHT(4, 4);
    else if (p.sb == 8)
        BEM_AHT(4, 8);
    else if (p.sb == 16)
        BEM_AHT(4, 16);
    else
        BEM_AHT(2, 32);
#undef BEM_AHT
    count_launch();
    if (p.splits > 1) {
        sum_parts_kernel<<<ew_grid(2 * stride), 256, 0, st>>>(2 * stride, part, 2 * stride, p.splits,
                                                              reinterpret_cast<float *>(W));
        count_launch();
    }
    KERNEL_CHECK();
}

}  // namespace bem
