// GPU test of CHIEF candidates: one CTA per candidate counts the ray/triangle
// crossings over all elements and the minimum distance to the nodes.
// Restates the reference's per-candidate kernels rayTrnglsInt and
// distPntPnts (mesh.cu:1411-1428) and the host tests inObj / arrayMin
// (numerical.cu:109-131), batched over many candidates per launch.
#include <cuda_runtime.h>

#include <cmath>
#include <vector>

#include "bem_common.h"
#include "mesh.h"

namespace {

struct V3 {
    float x, y, z;
};
__device__ __forceinline__ V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ V3 crs(V3 a, V3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ float dt(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

// cartCoord::nrmlzd (mesh.cu:1119-1126): NaN vector for a zero vector.
__device__ __forceinline__ V3 unit(V3 a) {
    float n = sqrtf(dt(a, a));
    if (n == 0.0f) return {nanf(""), nanf(""), nanf("")};
    return {a.x / n, a.y / n, a.z / n};
}
// cartCoord::isEqual with EPS = 5e-5 (numerical.h:124-126, mesh.cu:1156-1162).
__device__ __forceinline__ bool close(V3 a, V3 b) {
    const float eps = 0.00005f;
    return fabsf(a.x - b.x) < eps && fabsf(a.y - b.y) < eps && fabsf(a.z - b.z) < eps;
}

// rayTrnglInt = rayPlaneInt + isInsideTrngl (mesh.cu:1127-1189).
__device__ bool ray_hits(V3 sp, V3 dir, V3 p1, V3 p2, V3 p3) {
    V3 n = crs(sub(p2, p1), sub(p3, p1));
    V3 P;
    if (dt(n, sub(sp, p1)) == 0.0f) {
        P = sp;
    } else {
        float nd = dt(n, dir);
        if (nd == 0.0f) return false;
        float t = (dt(n, p1) - dt(n, sp)) / nd;
        if (!(t > 0.0f)) return false;
        P = {sp.x + t * dir.x, sp.y + t * dir.y, sp.z + t * dir.z};
    }
    if (P.x != P.x || P.y != P.y || P.z != P.z) return false;
    V3 t1 = unit(crs(sub(p2, p1), sub(P, p1)));
    V3 t2 = unit(crs(sub(p3, p2), sub(P, p2)));
    V3 t3 = unit(crs(sub(p1, p3), sub(P, p3)));
    return close(t1, t2) && close(t2, t3);
}

__global__ void __launch_bounds__(256) chief_candidates_kernel(
    const float *__restrict__ pnts, int num_pnts, const int *__restrict__ elems, int num_elems,
    const float *__restrict__ cand_pts, const float *__restrict__ cand_dirs, float threshold,
    int *__restrict__ accepted) {
    const int c = blockIdx.x;
    V3 sp = {cand_pts[3 * c], cand_pts[3 * c + 1], cand_pts[3 * c + 2]};
    V3 dir = {cand_dirs[3 * c], cand_dirs[3 * c + 1], cand_dirs[3 * c + 2]};
    int hits = 0;
    for (int e = threadIdx.x; e < num_elems; e += blockDim.x) {
        const int *nd = elems + 3 * (size_t)e;
        V3 p1 = {pnts[3 * nd[0]], pnts[3 * nd[0] + 1], pnts[3 * nd[0] + 2]};
        V3 p2 = {pnts[3 * nd[1]], pnts[3 * nd[1] + 1], pnts[3 * nd[1] + 2]};
        V3 p3 = {pnts[3 * nd[2]], pnts[3 * nd[2] + 1], pnts[3 * nd[2] + 2]};
        hits += ray_hits(sp, dir, p1, p2, p3) ? 1 : 0;
    }
    float mind = INFINITY;
    for (int i = threadIdx.x; i < num_pnts; i += blockDim.x) {
        V3 p = {pnts[3 * i], pnts[3 * i + 1], pnts[3 * i + 2]};
        V3 d = sub(p, sp);
        mind = fminf(mind, sqrtf(dt(d, d)));
    }
    // Warp then block reduction (fixed order).
    for (int o = 16; o > 0; o >>= 1) {
        hits += __shfl_xor_sync(0xffffffffu, hits, o);
        mind = fminf(mind, __shfl_xor_sync(0xffffffffu, mind, o));
    }
    __shared__ int sh[8];
    __shared__ float sm[8];
    int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) { sh[w] = hits; sm[w] = mind; }
    __syncthreads();
    if (threadIdx.x == 0) {
        int h = 0;
        float md = INFINITY;
        for (int i = 0; i < (int)(blockDim.x >> 5); i++) { h += sh[i]; md = fminf(md, sm[i]); }
        accepted[c] = ((h % 2) == 1 && !(md < threshold)) ? 1 : 0;
    }
}

}  // namespace

namespace bem {

void chief_test_candidates(const std::vector<float> &pnts_f, const std::vector<int> &elems,
                           const std::vector<float> &cand_pts, const std::vector<float> &cand_dirs,
                           float threshold, std::vector<int> &accepted) {
    int np = (int)(pnts_f.size() / 3), ne = (int)(elems.size() / 3), nc = (int)(cand_pts.size() / 3);
    float *d_p = nullptr, *d_cp = nullptr, *d_cd = nullptr;
    int *d_e = nullptr, *d_acc = nullptr;
    accepted.assign(nc, 0);
    auto cleanup = [&]() {
        cudaFree(d_p); cudaFree(d_cp); cudaFree(d_cd); cudaFree(d_e); cudaFree(d_acc);
    };
    try {
        CUDA_TRY(cudaMalloc(&d_p, sizeof(float) * pnts_f.size()));
        CUDA_TRY(cudaMalloc(&d_e, sizeof(int) * elems.size()));
        CUDA_TRY(cudaMalloc(&d_cp, sizeof(float) * cand_pts.size()));
        CUDA_TRY(cudaMalloc(&d_cd, sizeof(float) * cand_dirs.size()));
        CUDA_TRY(cudaMalloc(&d_acc, sizeof(int) * nc));
        CUDA_TRY(cudaMemcpy(d_p, pnts_f.data(), sizeof(float) * pnts_f.size(), cudaMemcpyHostToDevice));
        CUDA_TRY(cudaMemcpy(d_e, elems.data(), sizeof(int) * elems.size(), cudaMemcpyHostToDevice));
        CUDA_TRY(cudaMemcpy(d_cp, cand_pts.data(), sizeof(float) * cand_pts.size(), cudaMemcpyHostToDevice));
        CUDA_TRY(cudaMemcpy(d_cd, cand_dirs.data(), sizeof(float) * cand_dirs.size(), cudaMemcpyHostToDevice));
        chief_candidates_kernel<<<nc, 256>>>(d_p, np, d_e, ne, d_cp, d_cd, threshold, d_acc);
        count_launch();
        KERNEL_CHECK();
        CUDA_TRY(cudaMemcpy(accepted.data(), d_acc, sizeof(int) * nc, cudaMemcpyDeviceToHost));
    } catch (...) {
        cleanup();
        throw;
    }
    cleanup();
}

}  // namespace bem
