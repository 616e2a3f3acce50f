// Real GEMM C = op(A) B on the tcgen05 tensor cores, FP32-accurate through
// fp16 split products.
//
// Method.  Every operand value x is scaled by a power of two s (one for A,
// one per column of B) that brings the largest |x s| into [2^14, 2^15), then
// split into fp16 parts: h = fp16(x s), l = fp16(x s - h) (and m between
// them for three parts).  x s - h is exact in FP32 and |l| <= 2^-11 |h|, so
// two parts carry 22 bits and three 33; values far below the largest of
// their operand lose relative precision only below 2^-24 of that largest
// value, which is the scale the products are accurate to anyway.  The
// product keeps the terms of order up to 2^-11 (two parts: hh + hl + lh) or
// 2^-22 (three parts: hh + hm + mh + hl + lh + mm); each fp16 x fp16 product
// is exact, and the tensor core adds them into its FP32 accumulator (not with
// IEEE round-to-nearest: measured errors grow like sqrt(K) 2^-24 relative to
// sum |a||b|, a few times those of a blocked FP32 sum).  Two parts give about
// 2^-22 per product on top (what TF32x3 gives, at twice the tensor rate of
// TF32); three parts leave the accumulation as the only error.  The scales
// are undone in the epilogue (exact: powers of two).
//
// Data path.  A is read by the CTA's converter warps straight from global
// memory as FP32 (row-major, or transposed: op(A) = A^T), scaled, split and
// written into shared memory as K-major fp16 tiles in the 128-byte swizzle
// layout (so no split copy of A ever sits in HBM).  B is packed beforehand
// (tc_pack_*: it is the small operand, N x S or R x S) and staged by tiled
// TMA loads.  One elected thread issues tcgen05.mma (M = 128, N = NT, K = 16
// per instruction) into an FP32 accumulator in tensor memory; a commit to an
// mbarrier frees each stage.  The epilogue warps read the accumulator with
// tcgen05.ld (lane = output row, so each column's 128 rows are written as
// coalesced 128-byte segments).
//
// Warp roles (320 threads): warp 0 issues the TMA loads of B and owns the
// tensor-memory allocation; warp 1 issues the MMAs; warps 2-9 convert A and,
// at the end, run the epilogue (warp w reads tensor-memory lanes 32 (w % 4)).
//
// Split-K: with few output tiles, grid.z splits the K blocks; each split
// writes its partial product, and tc_sum_splits adds them in fixed order.
//
// Every mbarrier wait is bounded (about 0.5 s of SM clock).  On a timeout the
// CTA raises a shared abort flag that every other wait also watches, sets
// *status, stops issuing work, waits (bounded) for its copies and MMAs in
// flight, frees its tensor memory and returns.
#include <cuda.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <string>

#include "bem_common.h"
#include "solver.h"
#include "tc_gemm.h"
#include "tc_split.cuh"
#include "tcgen05.h"

namespace bem {
namespace {

constexpr int kTcM = 128;                  // rows of op(A) per CTA (tensor-memory lanes)
constexpr int kTcKB = 64;                  // K per stage: one 128-byte fp16 row
constexpr int kTcConvWarps = 8;            // converter / epilogue warps
constexpr int kTcThreads = 32 * (2 + kTcConvWarps);
constexpr long long kTcWaitCycles = 1000000000LL;   // ~0.5 s at 2 GHz
constexpr int kTcMaxSplits = 16;

template <int NT, int P>
struct TcCfg {
    static constexpr int A_PLANE = kTcM * 128;   // bytes
    static constexpr int B_PLANE = NT * 128;
    static constexpr int STAGE = P * (A_PLANE + B_PLANE);
    static constexpr int STAGES_RAW = (200 * 1024) / STAGE;
    static constexpr int STAGES = STAGES_RAW < 2 ? 2 : (STAGES_RAW > 4 ? 4 : STAGES_RAW);
    static constexpr int SMEM = STAGES * STAGE + 1024;   // + alignment slack
    static_assert(SMEM <= 227 * 1024, "stage buffers exceed shared memory");
    static_assert(NT % 32 == 0 && NT >= 32 && NT <= 256, "N tile");
};

// Bounded wait on an mbarrier phase; false on timeout or abort.
__device__ __forceinline__ bool tc_wait(uint64_t *bar, uint32_t parity, volatile int *abort) {
    return mbar_wait_bounded(bar, parity, kTcWaitCycles, abort);
}


// Byte offset of the 16-byte chunk c (K values 8c..8c+7) of row r in a
// K-major 128-byte-swizzled tile.
__device__ __forceinline__ uint32_t sw128_chunk(int r, int c) {
    return (uint32_t)((r >> 3) * 1024 + (r & 7) * 128 + ((c ^ (r & 7)) << 4));
}

template <int NT, int P, bool TA>
__global__ void __launch_bounds__(kTcThreads, 1)
tc_gemm_kernel(const float *__restrict__ A, size_t lda, int M, int K, const float *__restrict__ a_scale,
               const __grid_constant__ CUtensorMap tmB, int ncols_pad, const float *__restrict__ col_inv, int ncols,
               float *__restrict__ C, size_t ldc, size_t split_stride, int kb_per_split, int accum,
               int *status) {
    using Cfg = TcCfg<NT, P>;
    constexpr int STAGES = Cfg::STAGES;
    extern __shared__ uint8_t tc_smem_raw[];
    uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(tc_smem_raw) + 1023) & ~uintptr_t(1023));
    __shared__ __align__(8) uint64_t full_a[STAGES], full_b[STAGES], empty[STAGES], accum_full;
    __shared__ uint32_t tmem_base;
    __shared__ int abort_flag;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int n0 = blockIdx.x * NT, m0 = blockIdx.y * kTcM;
    const int nkb_total = (K + kTcKB - 1) / kTcKB;
    const int kb0 = blockIdx.z * kb_per_split;
    const int nkb = max(0, min(nkb_total, kb0 + kb_per_split) - kb0);
    float *Cz = C + blockIdx.z * split_stride;
    volatile int *abort_v = &abort_flag;

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; s++) {
            mbar_init(&full_a[s], 32 * kTcConvWarps);
            mbar_init(&full_b[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(&accum_full, 1);
        abort_flag = 0;
        mbar_fence_init();
    }
    if (warp == 0) {
        tmem_alloc(&tmem_base, NT);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_base;
    auto a_plane = [&](int s, int p) { return smem + (size_t)s * Cfg::STAGE + (size_t)p * Cfg::A_PLANE; };
    auto b_plane = [&](int s, int p) {
        return smem + (size_t)s * Cfg::STAGE + (size_t)P * Cfg::A_PLANE + (size_t)p * Cfg::B_PLANE;
    };
    auto fail = [&]() {
        *abort_v = 1;
        atomicExch(status, 1);
    };

    if (warp == 0) {
        if (lane == 0) {
            // TMA producer for B
            int issued = 0;
            for (int i = 0; i < nkb; i++) {
                const int s = i % STAGES;
                if (i >= STAGES && !tc_wait(&empty[s], (uint32_t)((i / STAGES - 1) & 1), abort_v)) {
                    fail();
                    break;
                }
                if (*abort_v) break;
                mbar_arrive_expect_tx(&full_b[s], (uint32_t)(P * Cfg::B_PLANE));
                for (int p = 0; p < P; p++)
                    tma_load_2d(b_plane(s, p), &tmB, (kb0 + i) * kTcKB, p * ncols_pad + n0, &full_b[s]);
                issued = i + 1;
            }
            if (*abort_v) {
                // let the copies in flight land before the CTA exits
                for (int j = max(0, issued - STAGES); j < issued; j++) {
                    volatile int never = 0;
                    mbar_wait_bounded(&full_b[j % STAGES], (uint32_t)((j / STAGES) & 1), kTcWaitCycles, &never);
                }
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            // MMA issuer
            constexpr uint32_t idesc = umma_idesc_f16_f32(kTcM, NT);
            constexpr int NPROD = P == 2 ? 3 : 6;
            constexpr int pa_of[6] = {0, 0, 1, 0, 2, 1};
            constexpr int pb_of[6] = {0, 1, 0, 2, 0, 1};
            for (int i = 0; i < nkb; i++) {
                const int s = i % STAGES;
                const uint32_t par = (uint32_t)((i / STAGES) & 1);
                if (!tc_wait(&full_b[s], par, abort_v) || !tc_wait(&full_a[s], par, abort_v)) {
                    fail();
                    break;
                }
                tc_fence_after();
                uint64_t ad[P], bd[P];
#pragma unroll
                for (int p = 0; p < P; p++) {
                    ad[p] = umma_desc_k128(smem_u32(a_plane(s, p)));
                    bd[p] = umma_desc_k128(smem_u32(b_plane(s, p)));
                }
#pragma unroll
                for (int kk = 0; kk < kTcKB / 16; kk++) {
#pragma unroll
                    for (int q = 0; q < NPROD; q++) {
                        // K step kk: 16 halfs = 32 bytes further along the swizzled row
                        umma_f16(tmem, ad[pa_of[q]] + (uint64_t)(2 * kk), bd[pb_of[q]] + (uint64_t)(2 * kk), idesc,
                                 (i > 0 || kk > 0 || q > 0) ? 1u : 0u);
                    }
                }
                umma_commit(&empty[s]);
            }
            // completes when every MMA issued above has (also after an abort)
            umma_commit(&accum_full);
        }
    } else {
        // converters: A tile (128 rows of op(A) x 64 K) -> P fp16 planes
        const int ct = threadIdx.x - 64;   // 0..255
        const float sa = a_scale[0];
        float cur[32], nxt[32];
        auto load = [&](int kb, float (&r)[32]) {
            const int k0 = kb * kTcKB;
            if (!TA) {
                // thread: rows (ct >> 4) + 16 e, K values 4 (ct & 15) .. + 3
                const int c4 = ct & 15, kq = k0 + 4 * c4;
#pragma unroll
                for (int e = 0; e < 8; e++) {
                    const int row = m0 + (ct >> 4) + 16 * e;
                    float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
                    if (row < M && kq < K) {
                        v = __ldg(reinterpret_cast<const float4 *>(A + (size_t)row * lda + kq));
                        if (kq + 1 >= K) v.y = 0.f;
                        if (kq + 2 >= K) v.z = 0.f;
                        if (kq + 3 >= K) v.w = 0.f;
                    }
                    r[4 * e] = v.x;
                    r[4 * e + 1] = v.y;
                    r[4 * e + 2] = v.z;
                    r[4 * e + 3] = v.w;
                }
            } else {
                // thread: K rows 8 (ct >> 5) + e, op(A) rows lane + 32 j
                const int wc = ct >> 5;
#pragma unroll
                for (int e = 0; e < 8; e++) {
                    const int k = k0 + 8 * wc + e;
#pragma unroll
                    for (int j = 0; j < 4; j++) {
                        const int m = m0 + lane + 32 * j;
                        r[8 * j + e] = (k < K && m < M) ? __ldg(A + (size_t)k * lda + m) : 0.f;
                    }
                }
            }
        };
        auto store = [&](int s, const float (&r)[32]) {
            uint8_t *pl[P];
#pragma unroll
            for (int p = 0; p < P; p++) pl[p] = a_plane(s, p);
            if (!TA) {
                const int c4 = ct & 15;
#pragma unroll
                for (int e = 0; e < 8; e++) {
                    const int row = (ct >> 4) + 16 * e;
                    uint32_t h01[3], h23[3];
                    split_pair<P>(r[4 * e] * sa, r[4 * e + 1] * sa, h01);
                    split_pair<P>(r[4 * e + 2] * sa, r[4 * e + 3] * sa, h23);
                    const uint32_t off = sw128_chunk(row, c4 >> 1) + ((c4 & 1) << 3);
#pragma unroll
                    for (int p = 0; p < P; p++)
                        *reinterpret_cast<uint2 *>(pl[p] + off) = make_uint2(h01[p], h23[p]);
                }
            } else {
                const int wc = ct >> 5;
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const int row = lane + 32 * j;
                    uint32_t h[4][3];
#pragma unroll
                    for (int e = 0; e < 4; e++) split_pair<P>(r[8 * j + 2 * e] * sa, r[8 * j + 2 * e + 1] * sa, h[e]);
                    const uint32_t off = sw128_chunk(row, wc);
#pragma unroll
                    for (int p = 0; p < P; p++)
                        *reinterpret_cast<uint4 *>(pl[p] + off) = make_uint4(h[0][p], h[1][p], h[2][p], h[3][p]);
                }
            }
        };
        // L2 prefetch of a K block's lines (distance 3), register loads two
        // K blocks ahead (a ring of three), so that about 64 KB of A per SM
        // is in flight while the tensor cores work
        auto prefetch = [&](int kb) {
            const int k0 = kb * kTcKB;
            if (!TA) {
                const int kq = k0 + 4 * (ct & 15);
                if ((ct & 7) == 0 && kq < K)
#pragma unroll
                    for (int e = 0; e < 8; e++) {
                        const int row = m0 + (ct >> 4) + 16 * e;
                        if (row < M) asm volatile("prefetch.global.L2 [%0];" ::"l"(A + (size_t)row * lda + kq));
                    }
            } else {
                const int k = k0 + (ct >> 5) * 8 + (lane >> 2);
                const int m = m0 + 32 * (lane & 3);
                if (k < K && m < M) asm volatile("prefetch.global.L2 [%0];" ::"l"(A + (size_t)k * lda + m));
            }
        };
        float nx2[32];
        if (nkb > 0) load(kb0, cur);
        if (nkb > 1) load(kb0 + 1, nxt);
        if (nkb > 2) prefetch(kb0 + 2);
        for (int i = 0; i < nkb; i++) {
            if (i + 2 < nkb) load(kb0 + i + 2, nx2);
            if (i + 3 < nkb) prefetch(kb0 + i + 3);
            const int s = i % STAGES;
            if (i >= STAGES && !tc_wait(&empty[s], (uint32_t)((i / STAGES - 1) & 1), abort_v)) {
                fail();
                break;
            }
            if (*abort_v) break;
            store(s, cur);
            fence_proxy_async_smem();   // generic-proxy writes -> visible to the tensor core
            mbar_arrive(&full_a[s]);
#pragma unroll
            for (int q = 0; q < 32; q++) {
                cur[q] = nxt[q];
                nxt[q] = nx2[q];
            }
        }
        // epilogue
        const int quad = warp & 3, half = (warp - 2) >> 2;
        const int row = m0 + 32 * quad + lane;
        constexpr int HALF_N = NT / 2;
        if (accum && row < M && !*abort_v) {
            // C -= ...: bring this thread's C lines into L2 while the last
            // MMAs run (a warp's 32 rows of one column are one or two lines)
            for (int c = half * HALF_N; c < (half + 1) * HALF_N; c++)
                if (n0 + c < ncols) asm volatile("prefetch.global.L2 [%0];" ::"l"(Cz + (size_t)(n0 + c) * ldc + row));
        }
        bool ok = true;
        if (nkb > 0) {
            ok = tc_wait(&accum_full, 0u, abort_v);
            if (!ok) fail();
        }
        tc_fence_after();
        const float inv_a = a_scale[1];
        for (int c = half * HALF_N; c < (half + 1) * HALF_N; c += 16) {
            // the 16 old values are loaded together (in flight at once)
            // before any store, rather than one load-store round trip each
            float old[16];
#pragma unroll
            for (int j = 0; j < 16; j++) old[j] = 0.f;
            if (accum && ok && !*abort_v && row < M) {
#pragma unroll
                for (int j = 0; j < 16; j++)
                    if (n0 + c + j < ncols) old[j] = Cz[(size_t)(n0 + c + j) * ldc + row];
            }
            uint32_t v[16];
            if (nkb > 0) {
                tmem_ld16(tmem + ((uint32_t)(32 * quad) << 16) + (uint32_t)c, v);
                tmem_wait_ld();
            }
            if (ok && !*abort_v && row < M) {
#pragma unroll
                for (int j = 0; j < 16; j++) {
                    const int n = n0 + c + j;
                    if (n < ncols) {
                        const float r = nkb > 0 ? __uint_as_float(v[j]) * inv_a * col_inv[n] : 0.f;
                        Cz[(size_t)n * ldc + row] = accum ? old[j] - r : r;
                    }
                }
            }
        }
    }
    __syncwarp();
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tmem, NT);
    }
}

// C[n * ldc + m] = sum over z < nz of part[z * stride + n * M + m] (fixed
// order); grid (rows / 256, columns).
__global__ void tc_sum_splits_kernel(int M, const float *__restrict__ part, size_t stride, int nz,
                                     float *__restrict__ C, size_t ldc, int accum) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x, n = blockIdx.y;
    if (m >= M) return;
    const size_t t = (size_t)n * M + m;
    float s = part[t];
    for (int z = 1; z < nz; z++) s += part[z * stride + t];
    float *dst = C + (size_t)n * ldc + m;
    *dst = accum ? *dst - s : s;
}




// One CTA per column of a real K x ncols matrix (column-major, ld).
template <int P>
__global__ void tc_pack_real_kernel(const float *__restrict__ B, size_t ld, int K, int Kp, int ncols_pad,
                                    __half *__restrict__ planes, float *__restrict__ col_inv) {
    __shared__ float red[32];
    const int n = blockIdx.x;
    const float *b = B + (size_t)n * ld;
    float mx = 0.f;
    for (int k = threadIdx.x; k < K; k += blockDim.x) mx = fmaxf(mx, fabsf(b[k]));
    const float sc = pow2_scale(block_max(mx, red));
    if (threadIdx.x == 0) col_inv[n] = 1.f / sc;
    const size_t ps = (size_t)ncols_pad * Kp;
    for (int k2 = threadIdx.x; 2 * k2 < Kp; k2 += blockDim.x) {
        const int k = 2 * k2;
        const float x0 = k < K ? b[k] * sc : 0.f, x1 = k + 1 < K ? b[k + 1] * sc : 0.f;
        put_parts<P>(planes, ps, (size_t)n * Kp + k, x0, x1);
    }
}

// One CTA per column s of the complex block X (n x S, leading dimension ldx):
// columns s and S + s of the interleaved real block (2n x 2S), both with the
// column's scale.  conj_left: the block for conj(X_left) Y instead of X_left
// Y (rows 2j, 2j + 1 of column s: (Re y, Im y); of column S + s: (Im y, -Re y)).
template <int P, typename T>
__global__ void tc_pack_cplx_kernel(const T *__restrict__ X, int n, int S, size_t ldx, int conj_left, int Kp,
                                    int ncols_pad, __half *__restrict__ planes, float *__restrict__ col_inv) {
    __shared__ float red[32];
    const int s = blockIdx.x;
    const T *x = X + (size_t)s * ldx;
    float mx = 0.f;
    for (int j = threadIdx.x; j < n; j += blockDim.x) mx = fmaxf(mx, fmaxf(fabsf((float)x[j].x), fabsf((float)x[j].y)));
    const double sc = (double)pow2_scale(block_max(mx, red));
    if (threadIdx.x == 0) col_inv[s] = col_inv[S + s] = (float)(1.0 / sc);
    const size_t ps = (size_t)ncols_pad * Kp;
    for (int j = threadIdx.x; 2 * j < Kp; j += blockDim.x) {
        float re = 0.f, im = 0.f;
        if (j < n) {
            // scaled in the input precision, then rounded once to FP32
            re = (float)((double)x[j].x * sc);
            im = (float)((double)x[j].y * sc);
        }
        if (conj_left) {
            put_parts<P>(planes, ps, (size_t)s * Kp + 2 * j, re, im);
            put_parts<P>(planes, ps, (size_t)(S + s) * Kp + 2 * j, im, -re);
        } else {
            put_parts<P>(planes, ps, (size_t)s * Kp + 2 * j, re, -im);
            put_parts<P>(planes, ps, (size_t)(S + s) * Kp + 2 * j, im, re);
        }
    }
}

// Largest |A| over rows x cols (row stride ld): CTAs stride over rows.
__global__ void tc_amax_kernel(const float *__restrict__ A, size_t ld, int rows, int cols, unsigned *__restrict__ out) {
    __shared__ float red[32];
    float mx = 0.f;
    for (int r = blockIdx.x; r < rows; r += gridDim.x) {
        const float *a = A + (size_t)r * ld;
        for (int c = threadIdx.x; c < cols; c += blockDim.x) mx = fmaxf(mx, fabsf(a[c]));
    }
    mx = block_max(mx, red);
    if (threadIdx.x == 0) atomicMax(out, __float_as_uint(mx));   // non-negative floats order as integers
}

__global__ void tc_scale_finish_kernel(float *scale) {
    const float amax = __uint_as_float(*reinterpret_cast<const unsigned *>(scale + 2));
    const float sc = pow2_scale(amax);
    scale[0] = sc;
    scale[1] = 1.f / sc;
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// against the driver library).
using EncodeTiledFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                   const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiledFn encode_fn() {
    static std::once_flag once;
    static EncodeTiledFn fn = nullptr;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
    });
    if (!fn) BEM_FAIL(BEM_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the CUDA driver");
    return fn;
}

int sm_count_current() { return device_sm_count(); }

int tc_nt(int ncols, int P) {
    if (ncols <= 32) return 32;
    if (ncols <= 64) return 64;
    if (ncols <= 128 || P == 3) return 128;
    return 256;
}

// Splits of the K blocks: fill whole waves of one CTA per SM, at least 8 K
// blocks per split, at most 8 CTAs per SM in all (bounds the partial sums),
// fewer splits on near ties.  When even the most splits leave part of one
// wave idle (a few output tiles over a long K), the most are taken.
int tc_splits(long long tiles, int nkb, int sms) {
    const int kmax = std::max(1, std::min({kTcMaxSplits, nkb / 8, (int)std::max(1LL, 8LL * sms / tiles)}));
    if (tiles * kmax <= sms) return kmax;
    int best = 1;
    double best_score = -1.0;
    for (int k = 1; k <= kmax; k++) {
        const long long ctas = tiles * k;
        const long long waves = (ctas + sms - 1) / sms;
        const double score = (double)ctas / (double)(waves * sms) - 0.01 * k;
        if (score > best_score + 1e-12) {
            best_score = score;
            best = k;
        }
    }
    return best;
}

template <int NT, int P, bool TA>
void launch_tc(const float *A, size_t lda, int M, int K, const float *a_scale, const CUtensorMap &tm,
               const TcOperand &B, float *C, size_t ldc, size_t split_stride, int kbps, int splits, int accum,
               int *status, cudaStream_t st) {
    using Cfg = TcCfg<NT, P>;
    static std::once_flag once;
    std::call_once(once, [] {
        cudaFuncSetAttribute(tc_gemm_kernel<NT, P, TA>, cudaFuncAttributeMaxDynamicSharedMemorySize, Cfg::SMEM);
    });
    const dim3 grid((B.ncols + NT - 1) / NT, (M + kTcM - 1) / kTcM, splits);
    tc_gemm_kernel<NT, P, TA><<<grid, kTcThreads, Cfg::SMEM, st>>>(A, lda, M, K, a_scale, tm, B.ncols_pad, B.col_inv,
                                                                    B.ncols, C, ldc, split_stride, kbps, accum,
                                                                    status);
    count_launch();
    KERNEL_CHECK();
}

template <int P, bool TA>
void dispatch_nt(int NT, const float *A, size_t lda, int M, int K, const float *a_scale, const CUtensorMap &tm,
                 const TcOperand &B, float *C, size_t ldc, size_t ss, int kbps, int splits, int accum, int *status,
                 cudaStream_t st) {
    switch (NT) {
    case 32: launch_tc<32, P, TA>(A, lda, M, K, a_scale, tm, B, C, ldc, ss, kbps, splits, accum, status, st); break;
    case 64: launch_tc<64, P, TA>(A, lda, M, K, a_scale, tm, B, C, ldc, ss, kbps, splits, accum, status, st); break;
    case 128: launch_tc<128, P, TA>(A, lda, M, K, a_scale, tm, B, C, ldc, ss, kbps, splits, accum, status, st); break;
    default:
        if constexpr (P == 2)
            launch_tc<256, P, TA>(A, lda, M, K, a_scale, tm, B, C, ldc, ss, kbps, splits, accum, status, st);
        else BEM_FAIL(BEM_ERR_INVALID_ARG, "tc_gemm: N tile 256 with three parts");
    }
}

struct TcPlan {
    int NT, nkb, splits, kbps;
};

TcPlan tc_plan(int M, int K, int ncols, int P) {
    TcPlan p;
    p.NT = tc_nt(ncols, P);
    p.nkb = (K + kTcKB - 1) / kTcKB;
    const long long tiles = (long long)((ncols + p.NT - 1) / p.NT) * ((M + kTcM - 1) / kTcM);
    p.splits = tc_splits(tiles, p.nkb, sm_count_current());
    p.kbps = (p.nkb + p.splits - 1) / p.splits;
    p.splits = (p.nkb + p.kbps - 1) / p.kbps;   // no empty split
    return p;
}

}  // namespace

size_t tc_operand_bytes(int K, int ncols, int P) {
    const size_t Kp = (size_t)((K + kTcKP - 1) / kTcKP) * kTcKP;
    const size_t np = (size_t)((ncols + kTcColPad - 1) / kTcColPad) * kTcColPad;
    return sizeof(__half) * (size_t)P * np * Kp + 256 + sizeof(float) * np;
}

TcOperand tc_operand_view(void *mem, int K, int ncols, int P) {
    TcOperand op;
    op.K = K;
    op.Kp = ((K + kTcKP - 1) / kTcKP) * kTcKP;
    op.ncols = ncols;
    op.ncols_pad = ((ncols + kTcColPad - 1) / kTcColPad) * kTcColPad;
    op.P = P;
    op.planes = static_cast<__half *>(mem);
    const size_t hb = sizeof(__half) * (size_t)P * op.ncols_pad * op.Kp;
    op.col_inv = reinterpret_cast<float *>(static_cast<uint8_t *>(mem) + ((hb + 255) & ~size_t(255)));
    return op;
}

void tc_pack_real(const float *B, size_t ld, TcOperand &op, cudaStream_t st) {
    if (op.P == 2)
        tc_pack_real_kernel<2><<<op.ncols, 256, 0, st>>>(B, ld, op.K, op.Kp, op.ncols_pad, op.planes, op.col_inv);
    else
        tc_pack_real_kernel<3><<<op.ncols, 256, 0, st>>>(B, ld, op.K, op.Kp, op.ncols_pad, op.planes, op.col_inv);
    count_launch();
    KERNEL_CHECK();
}

template <typename T>
static void pack_cplx(const T *X, int n, int S, size_t ldx, bool conj_left, TcOperand &op, cudaStream_t st) {
    BEM_CHECK_ARG(op.K == 2 * n && op.ncols == 2 * S && ldx >= (size_t)n, "tc_pack_cplx: operand shape");
    const int cj = conj_left ? 1 : 0;
    if (op.P == 2)
        tc_pack_cplx_kernel<2, T><<<S, 256, 0, st>>>(X, n, S, ldx, cj, op.Kp, op.ncols_pad, op.planes, op.col_inv);
    else
        tc_pack_cplx_kernel<3, T><<<S, 256, 0, st>>>(X, n, S, ldx, cj, op.Kp, op.ncols_pad, op.planes, op.col_inv);
    count_launch();
    KERNEL_CHECK();
}
void tc_pack_cplx_f32(const float2 *X, int n, int S, TcOperand &op, cudaStream_t st, size_t ldx, bool conj_left) {
    pack_cplx(X, n, S, ldx ? ldx : (size_t)n, conj_left, op, st);
}
void tc_pack_cplx_f64(const double2 *X, int n, int S, TcOperand &op, cudaStream_t st, size_t ldx, bool conj_left) {
    pack_cplx(X, n, S, ldx ? ldx : (size_t)n, conj_left, op, st);
}

void tc_a_scale(const float *A, size_t ld, int rows, int cols, float *scale, cudaStream_t st) {
    CUDA_TRY(cudaMemsetAsync(scale + 2, 0, sizeof(float), st));
    const unsigned grid = (unsigned)std::min(rows, sm_count_current() * 8);
    tc_amax_kernel<<<std::max(1u, grid), 256, 0, st>>>(A, ld, rows, cols, reinterpret_cast<unsigned *>(scale + 2));
    tc_scale_finish_kernel<<<1, 1, 0, st>>>(scale);
    count_launch(2);
    KERNEL_CHECK();
}

size_t tc_gemm_part_floats(int M, int K, int ncols, int P) {
    const TcPlan p = tc_plan(M, K, ncols, P);
    return p.splits > 1 ? (size_t)p.splits * M * ncols : 0;
}

size_t tc_gemm_part_floats_bound(int M, int ncols) {
    // splits <= 16, and splits x tiles <= 8 CTAs per SM with tiles of at
    // most 128 x 256 outputs (SM count <= 256)
    return std::min((size_t)kTcMaxSplits * M * ncols, (size_t)8 * 256 * kTcM * 256);
}

void tc_gemm(const float *A, size_t lda, bool trans, int M, int K, const float *a_scale, const TcOperand &B, float *C,
             size_t ldc, float *part, size_t part_floats, int *status, cudaStream_t st, bool subtract) {
    BEM_CHECK_ARG(B.K == K && M > 0 && K > 0 && B.ncols > 0, "tc_gemm: shapes");
    BEM_CHECK_ARG(lda % 4 == 0 && (reinterpret_cast<uintptr_t>(A) & 15) == 0, "tc_gemm: A alignment");
    BEM_CHECK_ARG(trans ? lda >= (size_t)M : lda >= (size_t)((K + 3) & ~3), "tc_gemm: lda");
    BEM_CHECK_ARG(B.P == 2 || B.P == 3, "tc_gemm: parts");
    BEM_CHECK_ARG(status != nullptr && a_scale != nullptr, "tc_gemm: status and scale words");
    const TcPlan p = tc_plan(M, K, B.ncols, B.P);
    if (p.splits > 1)
        BEM_CHECK_ARG(part != nullptr && part_floats >= (size_t)p.splits * M * B.ncols,
                      "tc_gemm: split-K scratch missing or smaller than the plan's partial sums");
    CUtensorMap tm;
    const cuuint64_t gdim[2] = {(cuuint64_t)B.Kp, (cuuint64_t)B.P * B.ncols_pad};
    const cuuint64_t gstride[1] = {(cuuint64_t)B.Kp * sizeof(__half)};
    const cuuint32_t box[2] = {(cuuint32_t)kTcKB, (cuuint32_t)p.NT};
    const cuuint32_t estr[2] = {1, 1};
    const CUresult r = encode_fn()(&tm, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, B.planes, gdim, gstride, box, estr,
                                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                                   CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) BEM_FAIL(BEM_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
    float *out = p.splits > 1 ? part : C;
    const size_t out_ld = p.splits > 1 ? (size_t)M : ldc;
    const size_t ss = p.splits > 1 ? (size_t)M * B.ncols : 0;
    const int acc = (subtract && p.splits == 1) ? 1 : 0;   // with splits the sum kernel subtracts
    if (B.P == 2) {
        if (trans) dispatch_nt<2, true>(p.NT, A, lda, M, K, a_scale, tm, B, out, out_ld, ss, p.kbps, p.splits, acc, status, st);
        else dispatch_nt<2, false>(p.NT, A, lda, M, K, a_scale, tm, B, out, out_ld, ss, p.kbps, p.splits, acc, status, st);
    } else {
        if (trans) dispatch_nt<3, true>(p.NT, A, lda, M, K, a_scale, tm, B, out, out_ld, ss, p.kbps, p.splits, acc, status, st);
        else dispatch_nt<3, false>(p.NT, A, lda, M, K, a_scale, tm, B, out, out_ld, ss, p.kbps, p.splits, acc, status, st);
    }
    if (p.splits > 1) {
        tc_sum_splits_kernel<<<dim3((M + 255) / 256, B.ncols), 256, 0, st>>>(M, part, ss, p.splits, C, ldc,
                                                                             subtract ? 1 : 0);
        count_launch();
        KERNEL_CHECK();
    }
}

}  // namespace bem

using namespace bem;

extern "C" int bem_tc_gemm_f32(int trans, int m, int k, int n, const float *A, int lda, const float *B, int ldb,
                               float *C, int ldc, int parts) {
    BEM_API_BEGIN
    BEM_CHECK_ARG(A && B && C && m > 0 && k > 0 && n > 0, "bem_tc_gemm_f32: null buffer or empty shape");
    BEM_CHECK_ARG(parts == 2 || parts == 3, "bem_tc_gemm_f32: parts must be 2 or 3");
    BEM_CHECK_ARG(lda % 4 == 0 && lda >= (trans ? m : k), "bem_tc_gemm_f32: lda (a multiple of 4, >= row length)");
    BEM_CHECK_ARG(ldb >= k && ldc >= m, "bem_tc_gemm_f32: ldb/ldc");
    const size_t arows = (size_t)(trans ? k : m);
    DevMem dA, dB, dC, dOp, dPart, dScal;
    dA.ensure(sizeof(float) * arows * lda);
    dB.ensure(sizeof(float) * (size_t)ldb * n);
    dC.ensure(sizeof(float) * (size_t)ldc * n);
    dOp.ensure(tc_operand_bytes(k, n, parts));
    dScal.ensure(sizeof(float) * 4 + sizeof(int));
    const size_t pf = tc_gemm_part_floats(trans ? m : m, k, n, parts);
    if (pf) dPart.ensure(sizeof(float) * pf);
    CUDA_TRY(cudaMemcpy(dA.p, A, sizeof(float) * arows * lda, cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(dB.p, B, sizeof(float) * (size_t)ldb * n, cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(dC.p, C, sizeof(float) * (size_t)ldc * n, cudaMemcpyHostToDevice));
    float *scal = dScal.as<float>();
    int *status = reinterpret_cast<int *>(scal + 4);
    CUDA_TRY(cudaMemset(status, 0, sizeof(int)));
    cudaStream_t st = nullptr;
    tc_a_scale(dA.as<float>(), lda, (int)arows, trans ? m : k, scal, st);
    TcOperand op = tc_operand_view(dOp.p, k, n, parts);
    tc_pack_real(dB.as<float>(), ldb, op, st);
    tc_gemm(dA.as<float>(), lda, trans != 0, m, k, scal, op, dC.as<float>(), ldc, dPart.as<float>(), pf, status, st);
    CUDA_TRY(cudaStreamSynchronize(st));
    int h_status = 0;
    CUDA_TRY(cudaMemcpy(&h_status, status, sizeof(int), cudaMemcpyDeviceToHost));
    if (h_status) BEM_FAIL(BEM_ERR_TIMEOUT, "bem_tc_gemm_f32: a bounded wait of the tensor-core kernel timed out");
    CUDA_TRY(cudaMemcpy(C, dC.p, sizeof(float) * (size_t)ldc * n, cudaMemcpyDeviceToHost));
    BEM_API_END
}
