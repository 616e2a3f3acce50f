// Hierarchical (H-matrix) form of a c64 collocation matrix on the device:
// the blocks of bem_hmat_partition, admissible ones compressed by partially
// pivoted adaptive cross approximation (ACA), inadmissible ones (and blocks
// whose ACA does not reach the tolerance below the break-even rank) kept
// dense; then y = H x and y = H^H x without atomics.  No reference
// counterpart: the reference stores A dense (mesh.cu:985-1006).
//
// Storage (one pool of c64 entries owned by the handle):
//   dense block   rc x cc, row-major;
//   low-rank block of rank k: U (rc x k) then V (cc x k), both column-major,
//   block ~= U V^T (ACA's cross approximation, no conjugation).
// Products, three launches each:
//   project: per low-rank block t = V^T x_J (H x) or t = U^H x_I (H^H x),
//            one warp per rank column;
//   apply:   per output segment (the finest intervals cut by the block edges
//            on that side) the dense and low-rank terms of every block
//            covering it, split over a few CTAs and their warps in a fixed
//            assignment; combine: the CTAs' partials added in order.  No
//            atomics and fixed summation orders: the product is bitwise
//            repeatable.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <memory>
#include <vector>

#include "bem_common.h"
#include "solver.h"

namespace bem {
namespace {

constexpr int kHT = 256;              // threads per CTA
constexpr int kHW = kHT / 32;         // warps per CTA
constexpr int kHMaxRank = 128;        // largest kmax (shared staging of one row / column of coefficients)
constexpr int kAcaMisses = 8;         // vanishing residual rows tolerated before falling back to dense

struct AcaJob {
    int r0, rc, c0, cc, kcap, pad;
    long long off_u, off_v, off_used;
};

struct HBlock {
    int r0, rc, c0, cc;
    int kind;        // 0 dense, 1 low rank
    int k;           // rank (low rank)
    long long off;   // dense: D; low rank: U, V at off + k * rc
    int t_off;       // low rank: its projected values in the work vector
    int pad;
};

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// conj(a) * b
__device__ __forceinline__ float2 cmulc(float2 a, float2 b) {
    return make_float2(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }

__device__ __forceinline__ float2 warp_sum2(float2 v) {
    for (int o = 16; o; o >>= 1) {
        v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
        v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
    }
    return v;
}

// Largest v over the CTA, the smallest index among equal values; every
// thread gets the result.  Threads without a candidate pass v = -1.
__device__ void cta_argmax(float v, int idx, float *sv, int *si, float &bv, int &bi) {
    for (int o = 16; o; o >>= 1) {
        const float ov = __shfl_down_sync(0xffffffffu, v, o);
        const int oi = __shfl_down_sync(0xffffffffu, idx, o);
        if (ov > v || (ov == v && oi < idx)) { v = ov; idx = oi; }
    }
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) { sv[w] = v; si[w] = idx; }
    __syncthreads();
    if (w == 0) {
        v = l < kHW ? sv[l] : -1.f;
        idx = l < kHW ? si[l] : INT_MAX;
        for (int o = 16; o; o >>= 1) {
            const float ov = __shfl_down_sync(0xffffffffu, v, o);
            const int oi = __shfl_down_sync(0xffffffffu, idx, o);
            if (ov > v || (ov == v && oi < idx)) { v = ov; idx = oi; }
        }
        if (l == 0) { sv[0] = v; si[0] = idx; }
    }
    __syncthreads();
    bv = sv[0];
    bi = si[0];
    __syncthreads();
}

// One CTA per admissible block: partially pivoted ACA on the block of A
// (row-major, lda).  Step k: the residual of pivot row i gives v_k (scaled
// by its largest entry, at column j), the residual of column j gives u_k;
// the next pivot row is the unused row where |u_k| is largest.  Stops when
// |u_k| |v_k| <= tol ||S_k||_F (S_k = sum of the k terms, its norm updated
// from the cross products of the new terms with the old ones).  status:
// 0 converged, 1 not converged within kcap terms (or residual rows kept
// vanishing), 2 non-finite entries.
__global__ void __launch_bounds__(kHT) aca_kernel(const float2 *__restrict__ A, size_t lda, const AcaJob *__restrict__ jobs,
                                                  float2 *pool, unsigned char *used_pool, float tol, int *rank_out,
                                                  int *status_out) {
    const AcaJob b = jobs[blockIdx.x];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    __shared__ float sv[kHW];
    __shared__ int si[kHW];
    __shared__ float2 s_coef[kHMaxRank];
    __shared__ float2 s_du[kHMaxRank + 1], s_dv[kHMaxRank + 1];
    __shared__ int s_conv;
    float2 *U = pool + b.off_u;
    float2 *V = pool + b.off_v;
    unsigned char *used = used_pool + b.off_used;
    const float2 *Ab = A + (size_t)b.r0 * lda + b.c0;
    for (int r = tid; r < b.rc; r += kHT) used[r] = r == 0;
    __syncthreads();
    double frob2 = 0.0;   // thread 0 only
    int i = 0, k = 0, status = 1, misses = 0;
    while (k < b.kcap) {
        // residual of row i -> V[:, k]
        for (int q = tid; q < k; q += kHT) s_coef[q] = U[(size_t)q * b.rc + i];
        __syncthreads();
        float2 *Vk = V + (size_t)k * b.cc;
        const float2 *arow = Ab + (size_t)i * lda;
        float best = -1.f;
        int bidx = INT_MAX;
        int bad = 0;
        for (int c = tid; c < b.cc; c += kHT) {
            float2 a = arow[c];
            for (int q = 0; q < k; q++) a = csub(a, cmul(s_coef[q], V[(size_t)q * b.cc + c]));
            Vk[c] = a;
            const float m = a.x * a.x + a.y * a.y;
            if (!isfinite(m)) bad = 1;
            else if (m > best) { best = m; bidx = c; }
        }
        if (__syncthreads_or(bad)) { status = 2; break; }
        float bv;
        int j;
        cta_argmax(best, bidx, sv, si, bv, j);
        if (!(bv > 0.f)) {
            // the residual vanishes on row i: take the smallest unused row
            if (++misses > kAcaMisses) break;
            float uv = -1.f;
            int ui = INT_MAX;
            for (int r = tid; r < b.rc; r += kHT)
                if (!used[r]) { uv = 1.f; ui = r; break; }
            float gv;
            int gi;
            cta_argmax(uv, ui, sv, si, gv, gi);
            if (gv < 0.f) break;   // every row used
            i = gi;
            if (tid == 0) used[i] = 1;
            __syncthreads();
            continue;
        }
        const float2 d = Vk[j];
        __syncthreads();   // every thread has read the pivot before it is scaled
        const float dn = d.x * d.x + d.y * d.y;
        const float2 dinv = make_float2(d.x / dn, -d.y / dn);
        for (int c = tid; c < b.cc; c += kHT) Vk[c] = cmul(Vk[c], dinv);
        for (int q = tid; q < k; q += kHT) s_coef[q] = V[(size_t)q * b.cc + j];
        __syncthreads();
        // residual of column j -> U[:, k]
        float2 *Uk = U + (size_t)k * b.rc;
        for (int r = tid; r < b.rc; r += kHT) {
            float2 a = Ab[(size_t)r * lda + j];
            for (int q = 0; q < k; q++) a = csub(a, cmul(U[(size_t)q * b.rc + r], s_coef[q]));
            Uk[r] = a;
        }
        __syncthreads();
        // u_q^H u_k and v_q^H v_k for q <= k (q = k: the squared norms)
        for (int q = warp; q <= k; q += kHW) {
            const float2 *uq = U + (size_t)q * b.rc, *vq = V + (size_t)q * b.cc;
            float2 au = make_float2(0.f, 0.f), av = make_float2(0.f, 0.f);
            for (int r = lane; r < b.rc; r += 32) au = cadd(au, cmulc(uq[r], Uk[r]));
            for (int c = lane; c < b.cc; c += 32) av = cadd(av, cmulc(vq[c], Vk[c]));
            au = warp_sum2(au);
            av = warp_sum2(av);
            if (lane == 0) { s_du[q] = au; s_dv[q] = av; }
        }
        __syncthreads();
        if (tid == 0) {
            double cross = 0.0;
            for (int q = 0; q < k; q++)
                cross += (double)s_du[q].x * s_dv[q].x - (double)s_du[q].y * s_dv[q].y;
            const double nu2 = s_du[k].x, nv2 = s_dv[k].x;
            frob2 += 2.0 * cross + nu2 * nv2;
            s_conv = sqrt(nu2 * nv2) <= (double)tol * sqrt(fmax(frob2, 0.0));
        }
        __syncthreads();
        k++;
        if (s_conv) { status = 0; break; }
        // next pivot row: largest |u_k| among the unused rows
        float mu = -1.f;
        int mi = INT_MAX;
        for (int r = tid; r < b.rc; r += kHT) {
            if (used[r]) continue;
            const float m = Uk[r].x * Uk[r].x + Uk[r].y * Uk[r].y;
            if (m > mu) { mu = m; mi = r; }
        }
        float gv;
        int gi;
        cta_argmax(mu, mi, sv, si, gv, gi);
        if (gv < 0.f) break;   // every row used
        i = gi;
        if (tid == 0) used[i] = 1;
        __syncthreads();
    }
    if (tid == 0) {
        rank_out[blockIdx.x] = k;
        status_out[blockIdx.x] = status;
    }
}

// Dense blocks copied out of A (one CTA per block), and converged low-rank
// factors moved from the kcap-wide scratch into the tight pool.
__global__ void __launch_bounds__(kHT) hmat_fill_kernel(const float2 *__restrict__ A, size_t lda,
                                                        const HBlock *__restrict__ desc, const int *__restrict__ list,
                                                        const long long *__restrict__ src_off, const int *__restrict__ src_cap,
                                                        const float2 *__restrict__ scratch, float2 *pool) {
    const HBlock b = desc[list[blockIdx.x]];
    float2 *dst = pool + b.off;
    if (b.kind == 0) {
        for (int r = 0; r < b.rc; r++) {
            const float2 *src = A + (size_t)(b.r0 + r) * lda + b.c0;
            for (int c = threadIdx.x; c < b.cc; c += kHT) dst[(size_t)r * b.cc + c] = src[c];
        }
    } else {
        const float2 *su = scratch + src_off[blockIdx.x];
        const float2 *sv = su + (size_t)src_cap[blockIdx.x] * b.rc;
        const size_t nu = (size_t)b.k * b.rc, nv = (size_t)b.k * b.cc;
        for (size_t e = threadIdx.x; e < nu; e += kHT) dst[e] = su[e];
        for (size_t e = threadIdx.x; e < nv; e += kHT) dst[nu + e] = sv[e];
    }
}

// t = V^T x_J (trans 0) or U^H x_I (trans 1) for each low-rank block.
__global__ void __launch_bounds__(kHT) hmv_project_kernel(const HBlock *__restrict__ desc, const int *__restrict__ lr,
                                                          const float2 *__restrict__ pool, const float2 *__restrict__ x,
                                                          float2 *t, int trans) {
    const HBlock b = desc[lr[blockIdx.x]];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const float2 *U = pool + b.off, *V = U + (size_t)b.k * b.rc;
    for (int q = warp; q < b.k; q += kHW) {
        float2 s = make_float2(0.f, 0.f);
        if (trans == 0) {
            const float2 *vq = V + (size_t)q * b.cc, *xj = x + b.c0;
            for (int c = lane; c < b.cc; c += 32) s = cadd(s, cmul(vq[c], xj[c]));
        } else {
            const float2 *uq = U + (size_t)q * b.rc, *xi = x + b.r0;
            for (int r = lane; r < b.rc; r += 32) s = cadd(s, cmulc(uq[r], xi[r]));
        }
        s = warp_sum2(s);
        if (lane == 0) t[b.t_off + q] = s;
    }
}

// One output segment, split over P CTAs: warp w of CTA p takes the
// segment's blocks e0 + p * 8 + w, then every 8 P-th one, and accumulates
// its terms for every output entry of the segment (lanes over the entries,
// loads independent across the inner loop) into its own shared slice; the
// CTA adds the eight slices in warp order and writes its partial, and
// hmv_combine_kernel adds the P partials in order.  The assignment and every
// order are fixed, so the product is bitwise repeatable.
// trans 0: entries are rows, y_I += D x_J (D row-major: each lane walks its
// row) or U (V^T x_J) (U column-major: lanes read consecutive rows).
// trans 1: entries are columns, y_J += D^H x_I (lanes read consecutive
// columns of each row) or conj(V) (U^H x_I).
constexpr int kSegChunk = 128;

__global__ void __launch_bounds__(kHT) hmv_apply_kernel(const HBlock *__restrict__ desc, const int2 *__restrict__ seg,
                                                        const int *__restrict__ ptr, const int *__restrict__ idx,
                                                        const float2 *__restrict__ pool, const float2 *__restrict__ x,
                                                        const float2 *__restrict__ t, float2 *part, int n_out, int P,
                                                        int trans) {
    __shared__ float2 acc[kHW][kSegChunk];
    const int s = blockIdx.x / P, p = blockIdx.x - s * P;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int2 sg = seg[s];
    const int e0 = ptr[s], e1 = ptr[s + 1];
    for (int ch = 0; ch < sg.y; ch += kSegChunk) {
        const int nout = min(kSegChunk, sg.y - ch);
        for (int o = lane; o < kSegChunk; o += 32) acc[warp][o] = make_float2(0.f, 0.f);
        __syncwarp();
        for (int e = e0 + p * kHW + warp; e < e1; e += P * kHW) {
            const HBlock b = desc[idx[e]];
            const float2 *D = pool + b.off;
            if (trans == 0) {
                const int base = sg.x + ch - b.r0;   // block row of the chunk's first row
                if (b.kind == 0) {
                    const float2 *xj = x + b.c0;
                    for (int o = lane; o < nout; o += 32) {
                        const float2 *drow = D + (size_t)(base + o) * b.cc;
                        float2 a = make_float2(0.f, 0.f);
#pragma unroll 4
                        for (int c = 0; c < b.cc; c++) a = cadd(a, cmul(drow[c], xj[c]));
                        acc[warp][o] = cadd(acc[warp][o], a);
                    }
                } else {
                    const float2 *tb = t + b.t_off;
                    for (int o = lane; o < nout; o += 32) {
                        float2 a = make_float2(0.f, 0.f);
#pragma unroll 4
                        for (int q = 0; q < b.k; q++) a = cadd(a, cmul(D[(size_t)q * b.rc + base + o], tb[q]));
                        acc[warp][o] = cadd(acc[warp][o], a);
                    }
                }
            } else {
                const int base = sg.x + ch - b.c0;   // block column of the chunk's first column
                if (b.kind == 0) {
                    const float2 *xi = x + b.r0;
                    for (int o = lane; o < nout; o += 32) {
                        float2 a = make_float2(0.f, 0.f);
#pragma unroll 4
                        for (int r = 0; r < b.rc; r++) a = cadd(a, cmulc(D[(size_t)r * b.cc + base + o], xi[r]));
                        acc[warp][o] = cadd(acc[warp][o], a);
                    }
                } else {
                    const float2 *V = D + (size_t)b.k * b.rc;
                    const float2 *tb = t + b.t_off;
                    for (int o = lane; o < nout; o += 32) {
                        float2 a = make_float2(0.f, 0.f);
#pragma unroll 4
                        for (int q = 0; q < b.k; q++) a = cadd(a, cmulc(V[(size_t)q * b.cc + base + o], tb[q]));
                        acc[warp][o] = cadd(acc[warp][o], a);
                    }
                }
            }
        }
        __syncthreads();
        for (int o = tid; o < nout; o += kHT) {
            float2 a = acc[0][o];
            for (int w = 1; w < kHW; w++) a = cadd(a, acc[w][o]);
            part[(size_t)p * n_out + sg.x + ch + o] = a;
        }
        __syncthreads();
    }
}

__global__ void hmv_combine_kernel(const float2 *__restrict__ part, int n_out, int P, float2 *y) {
    for (int o = blockIdx.x * blockDim.x + threadIdx.x; o < n_out; o += gridDim.x * blockDim.x) {
        float2 a = part[o];
        for (int p = 1; p < P; p++) a = cadd(a, part[(size_t)p * n_out + o]);
        y[o] = a;
    }
}

// Output segments on one side: the intervals between consecutive block
// edges, each with the blocks covering it in block order (CSR).
void build_segments(const std::vector<HBlock> &desc, int n, bool rows, std::vector<int2> &seg, std::vector<int> &ptr,
                    std::vector<int> &idx) {
    std::vector<int> cut;
    cut.reserve(2 * desc.size() + 2);
    cut.push_back(0);
    cut.push_back(n);
    for (const HBlock &b : desc) {
        const int a = rows ? b.r0 : b.c0, len = rows ? b.rc : b.cc;
        cut.push_back(a);
        cut.push_back(a + len);
    }
    std::sort(cut.begin(), cut.end());
    cut.erase(std::unique(cut.begin(), cut.end()), cut.end());
    const int ns = (int)cut.size() - 1;
    seg.resize(ns);
    for (int s = 0; s < ns; s++) seg[s] = make_int2(cut[s], cut[s + 1] - cut[s]);
    std::vector<int> cnt(ns + 1, 0);
    auto first_seg = [&](int a) { return (int)(std::lower_bound(cut.begin(), cut.end(), a) - cut.begin()); };
    for (const HBlock &b : desc) {
        const int a = rows ? b.r0 : b.c0, len = rows ? b.rc : b.cc;
        for (int s = first_seg(a); s < ns && cut[s] < a + len; s++) cnt[s + 1]++;
    }
    ptr.assign(ns + 1, 0);
    for (int s = 0; s < ns; s++) ptr[s + 1] = ptr[s] + cnt[s + 1];
    idx.resize(ptr[ns]);
    std::vector<int> fill(ptr.begin(), ptr.end() - 1);
    for (int bi = 0; bi < (int)desc.size(); bi++) {
        const HBlock &b = desc[bi];
        const int a = rows ? b.r0 : b.c0, len = rows ? b.rc : b.cc;
        for (int s = first_seg(a); s < ns && cut[s] < a + len; s++) idx[fill[s]++] = bi;
    }
}

template <class T> void upload(DevMem &m, const std::vector<T> &v, cudaStream_t st) {
    m.ensure(std::max<size_t>(sizeof(T) * v.size(), sizeof(T)));
    if (!v.empty()) CUDA_TRY(cudaMemcpyAsync(m.p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice, st));
}

}  // namespace
}  // namespace bem

struct bem_hmat_s {
    int R = 0, N = 0;
    bem::DevMem pool, desc, lr, t;
    bem::DevMem rseg, rptr, ridx, cseg, cptr, cidx;
    bem::DevMem part;                       // P partial outputs of the apply kernel
    int n_lr = 0, n_rseg = 0, n_cseg = 0;
    int p_rows = 1, p_cols = 1;             // CTAs per output segment
    long long entries = 0;
    int max_rank = 0, n_lowrank = 0, n_dense = 0;
};

extern "C" int bem_hmat_compress_c64(const void *A_dev, int R, int N, int lda, const int *blocks, int num_blocks,
                                     double tol, int kmax, void *stream, bem_hmat_t *out) {
    using namespace bem;
    BEM_API_BEGIN
    BEM_CHECK_ARG(A_dev && blocks && out && num_blocks > 0, "null argument");
    BEM_CHECK_ARG(R > 0 && N > 0 && lda >= N, "bad matrix shape");
    BEM_CHECK_ARG(std::isfinite(tol) && tol > 0.0 && tol < 1.0, "tol must lie in (0, 1)");
    BEM_CHECK_ARG(kmax >= 1 && kmax <= kHMaxRank, "kmax must lie in [1, 128]");
    *out = nullptr;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // the blocks must tile R x N exactly once
    long long area = 0;
    for (int q = 0; q < num_blocks; q++) {
        const int *b = blocks + 5 * q;
        BEM_CHECK_ARG(b[1] > 0 && b[3] > 0 && b[0] >= 0 && b[2] >= 0 && b[0] + b[1] <= R && b[2] + b[3] <= N &&
                          (b[4] == 0 || b[4] == 1),
                      "block outside the matrix");
        area += (long long)b[1] * b[3];
    }
    BEM_CHECK_ARG(area == (long long)R * N, "blocks do not tile the matrix");
    std::unique_ptr<bem_hmat_s> h(new bem_hmat_s);
    h->R = R;
    h->N = N;
    const float2 *A = static_cast<const float2 *>(A_dev);

    // ACA over the admissible blocks whose break-even rank is at least 1
    std::vector<AcaJob> jobs;
    std::vector<int> job_block;
    long long scratch = 0, used = 0;
    for (int q = 0; q < num_blocks; q++) {
        const int *b = blocks + 5 * q;
        if (!b[4]) continue;
        const long long rc = b[1], cc = b[3];
        // below the break-even rank: k (rc + cc) < rc cc
        const int kcap = (int)std::min<long long>(kmax, (rc * cc - 1) / (rc + cc));
        if (kcap < 1) continue;
        AcaJob j{b[0], b[1], b[2], b[3], kcap, 0, scratch, scratch + (long long)kcap * rc, used};
        scratch += (long long)kcap * (rc + cc);
        used += rc;
        jobs.push_back(j);
        job_block.push_back(q);
    }
    const int nj = (int)jobs.size();
    DevMem d_scratch, d_used, d_jobs, d_rank, d_status;
    std::vector<int> rank(nj), status(nj);
    if (nj) {
        d_scratch.ensure(sizeof(float2) * (size_t)scratch);
        d_used.ensure((size_t)used);
        upload(d_jobs, jobs, st);
        d_rank.ensure(sizeof(int) * nj);
        d_status.ensure(sizeof(int) * nj);
        {
            BEM_PROF("hmat_aca", st);
            aca_kernel<<<nj, kHT, 0, st>>>(A, (size_t)lda, d_jobs.as<AcaJob>(), d_scratch.as<float2>(),
                                           d_used.as<unsigned char>(), (float)tol, d_rank.as<int>(),
                                           d_status.as<int>());
            count_launch();
            KERNEL_CHECK();
        }
        CUDA_TRY(cudaMemcpyAsync(rank.data(), d_rank.p, sizeof(int) * nj, cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaMemcpyAsync(status.data(), d_status.p, sizeof(int) * nj, cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaStreamSynchronize(st));
    }
    std::vector<int> job_of(num_blocks, -1);
    for (int q = 0; q < nj; q++)
        if (status[q] == 0 && rank[q] >= 1) job_of[job_block[q]] = q;

    // descriptors: dense blocks first in the pool, then the low-rank factors
    std::vector<HBlock> desc(num_blocks);
    std::vector<int> lr_list, fill_list;
    std::vector<long long> src_off;
    std::vector<int> src_cap;
    long long off = 0;
    int toff = 0;
    for (int pass = 0; pass < 2; pass++) {
        for (int q = 0; q < num_blocks; q++) {
            const int *b = blocks + 5 * q;
            const int jq = job_of[q];
            if ((pass == 0) != (jq < 0)) continue;
            HBlock d{b[0], b[1], b[2], b[3], jq >= 0 ? 1 : 0, 0, off, 0, 0};
            if (jq >= 0) {
                d.k = rank[jq];
                d.t_off = toff;
                toff += d.k;
                off += (long long)d.k * (b[1] + b[3]);
                lr_list.push_back(q);
                h->max_rank = std::max(h->max_rank, d.k);
                h->n_lowrank++;
                src_off.push_back(jobs[jq].off_u);
                src_cap.push_back(jobs[jq].kcap);
            } else {
                off += (long long)b[1] * b[3];
                h->n_dense++;
                src_off.push_back(0);
                src_cap.push_back(0);
            }
            desc[q] = d;
            fill_list.push_back(q);
        }
    }
    h->entries = off;
    h->pool.ensure(sizeof(float2) * (size_t)std::max<long long>(off, 1));
    upload(h->desc, desc, st);
    DevMem d_fill, d_soff, d_scap;
    upload(d_fill, fill_list, st);
    upload(d_soff, src_off, st);
    upload(d_scap, src_cap, st);
    {
        BEM_PROF("hmat_fill", st);
        hmat_fill_kernel<<<num_blocks, kHT, 0, st>>>(A, (size_t)lda, h->desc.as<HBlock>(), d_fill.as<int>(),
                                                     d_soff.as<long long>(), d_scap.as<int>(),
                                                     nj ? d_scratch.as<float2>() : nullptr, h->pool.as<float2>());
        count_launch();
        KERNEL_CHECK();
    }
    h->n_lr = (int)lr_list.size();
    upload(h->lr, lr_list, st);
    h->t.ensure(sizeof(float2) * (size_t)std::max(toff, 1));
    std::vector<int2> seg;
    std::vector<int> ptr, idx;
    build_segments(desc, R, true, seg, ptr, idx);
    h->n_rseg = (int)seg.size();
    upload(h->rseg, seg, st);
    upload(h->rptr, ptr, st);
    upload(h->ridx, idx, st);
    std::vector<int2> cseg;
    std::vector<int> cptr, cidx;
    build_segments(desc, N, false, cseg, cptr, cidx);
    h->n_cseg = (int)cseg.size();
    upload(h->cseg, cseg, st);
    upload(h->cptr, cptr, st);
    upload(h->cidx, cidx, st);
    // enough CTAs per segment to give every SM four
    const int want = 4 * device_sm_count();
    h->p_rows = std::min(8, std::max(1, (want + h->n_rseg - 1) / h->n_rseg));
    h->p_cols = std::min(8, std::max(1, (want + h->n_cseg - 1) / h->n_cseg));
    h->part.ensure(sizeof(float2) * (size_t)std::max(R * h->p_rows, N * h->p_cols));
    // the host vectors and the scratch are released on return
    CUDA_TRY(cudaStreamSynchronize(st));
    *out = h.release();
    BEM_API_END
}

extern "C" int bem_hmat_matvec_c64(bem_hmat_t h, int trans, const void *x_dev, void *y_dev, void *stream) {
    using namespace bem;
    BEM_API_BEGIN
    BEM_CHECK_ARG(h && x_dev && y_dev && (trans == 0 || trans == 1), "bad argument");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const float2 *x = static_cast<const float2 *>(x_dev);
    float2 *y = static_cast<float2 *>(y_dev);
    if (h->n_lr) {
        BEM_PROF("hmat_project", st);
        hmv_project_kernel<<<h->n_lr, kHT, 0, st>>>(h->desc.as<HBlock>(), h->lr.as<int>(), h->pool.as<float2>(), x,
                                                    h->t.as<float2>(), trans);
        count_launch();
        KERNEL_CHECK();
    }
    {
        BEM_PROF("hmat_apply", st);
        const int P = trans == 0 ? h->p_rows : h->p_cols;
        const int nseg = trans == 0 ? h->n_rseg : h->n_cseg;
        const int n_out = trans == 0 ? h->R : h->N;
        const DevMem &sg = trans == 0 ? h->rseg : h->cseg, &pt = trans == 0 ? h->rptr : h->cptr,
                     &ix = trans == 0 ? h->ridx : h->cidx;
        hmv_apply_kernel<<<nseg * P, kHT, 0, st>>>(h->desc.as<HBlock>(), sg.as<int2>(), pt.as<int>(), ix.as<int>(),
                                                   h->pool.as<float2>(), x, h->t.as<float2>(),
                                                   h->part.as<float2>(), n_out, P, trans);
        count_launch();
        KERNEL_CHECK();
        hmv_combine_kernel<<<(n_out + kHT - 1) / kHT, kHT, 0, st>>>(h->part.as<float2>(), n_out, P, y);
        count_launch();
        KERNEL_CHECK();
    }
    BEM_API_END
}

extern "C" int bem_hmat_info(bem_hmat_t h, long long *entries, int *max_rank, int *lowrank_blocks,
                             int *dense_blocks) {
    BEM_API_BEGIN
    BEM_CHECK_ARG(h, "null handle");
    if (entries) *entries = h->entries;
    if (max_rank) *max_rank = h->max_rank;
    if (lowrank_blocks) *lowrank_blocks = h->n_lowrank;
    if (dense_blocks) *dense_blocks = h->n_dense;
    BEM_API_END
}

extern "C" int bem_hmat_destroy(bem_hmat_t h) {
    BEM_API_BEGIN
    delete h;
    BEM_API_END
}
