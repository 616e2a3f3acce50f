// Launch wrappers for the quadrature kernels (kernels.cu) and the linear
// algebra kernels (linalg.cu).  All launches go on the given stream.
#pragma once

#include <cuda_runtime.h>

#include "bem_common.h"

namespace bem {

// Incident field record on the device (same layout as bem_source_t).
struct DevSource {
    int kind;
    double vec[3];
    double amp_re, amp_im;
};

struct GeoTables {
    const float4 *geo_f;      // 9 float4 per element (layout in kernels.cu)
    const double *geo_d;      // 18 doubles per element
    const int4 *elems;        // (n0, n1, n2, 0)
    int E;
};

struct RowPoints {
    const float4 *f;          // 2 per point: hi = (x, y, z, 0) floats, lo = remainders
    const double *d;          // 3 doubles per point
    int R;                    // number of points (rows)
};

// A tile's records come in batches of at most kFarBatch records whose nodes
// inside the tile are all distinct (no two records of a batch add to the
// same column), so the far kernels add each batch's contributions without
// atomics and, with a CTA barrier between batches, in batch order: every
// column of A receives its far-field terms in one fixed order, whatever the
// launch shape (bitwise repeatable assembly).
constexpr int kFarBatch = 1024;
constexpr long long kFarWaitCycles = 2000000000LL;   // bound of the far kernel's batch waits (~1 s)

// A far-kernel record with its element's geometry gathered in record order
// (the seven float4 of GeoTables::geo_f), so that an item's data is one
// contiguous 144-byte read instead of a record read followed by a dependent
// read of the element's table.  nodes.w = owner; slots.w unused.
struct FarRec {
    float4 g[7];
    int4 nodes;
    int4 slots;
};

struct TileSet {
    const TileRec *recs;      // all tiles' records
    const int *rec_ptr;       // ntiles + 1 offsets into recs
    const int *batch_ptr;     // batch boundaries (offsets into recs), all tiles' batches in order
    const int *tile_batch;    // ntiles + 1: the batches of tile t are tile_batch[t] .. tile_batch[t+1]-1
    int *status;              // the solver's status word: set when a bounded wait of the far kernel timed out
    const int *cols;          // ntiles * tc_max tile-local column -> global column (node index)
    const int *col_cnt;       // ntiles: columns in each tile
    int ntiles;
    int tc_max;
    const FarRec *frecs;      // recs with their geometry (FP32 far kernel); filled by launch_far_recs
};

struct Physics {
    double k;
    double rw;                // density * omega = density * k * speed
    int near_depth;
    double near_eta;
    double max_edge = 0.0;    // longest element edge } select the phase mode of the
    double extent = 0.0;      // diagonal of the rows' and nodes' box } FP32 quadrature
    // which single-layer (G) sums the BCs need: 2 = all (some element has
    // bcA != 0), 1 = S0 only (bcA = 0 everywhere; beta needs sum_j g_j),
    // 0 = none (bcA = bcC = 0 everywhere)
    int g_sums = 2;
};
// Phase mode of the FP32 far kernel for this problem (kernels.cu).
int far_phase_mode(const Physics &ph);

// Upload the Gauss rule of the given order to this device's constant memory
// (no-op when already current on the device).
void ensure_quadrature(int order);
int quadrature_points();      // order^2 of the uploaded rule

// Element tables from nodes/elements/bc.  near_eta scales the near-pair
// radius stored in the float table.
void launch_elem_setup(const double *d_nodes, const int4 *d_elems, const double *d_bc, int E,
                       double near_eta, float4 *geo_f, double *geo_d, cudaStream_t st);

// Far-field assembly.  c64: FP32 quadrature, acc/partials in float.  c128: FP64.
constexpr int kGeoFloat4 = 9;     // float4 per element in GeoTables::geo_f
constexpr int kGeoDouble = 18;    // doubles per element in GeoTables::geo_d
// `variant` selects a launch shape (rows per CTA, threads, CTAs per SM);
// far_variants(prec) shapes exist, far_variant_fits says whether the
// shape's shared-memory row accumulator fits the device for tile width tc.
int far_variants(int prec);
int far_rows_per_cta(int prec, int variant);
size_t far_smem_bytes(int prec, int tc, int variant);
bool far_variant_fits(int prec, int tc, int variant);
// frecs[i] = recs[i] with the geometry of element recs[i].eid (nrec records).
void launch_far_recs(const TileRec *recs, int nrec, const float4 *geo_f, FarRec *frecs, cudaStream_t st);
void launch_far_assembly(int prec, const RowPoints &rows, int N, const GeoTables &geo,
                         const TileSet &tiles, const Physics &ph, void *A, size_t lda,
                         void *c_part, void *beta_part, cudaStream_t st, int variant);

// Near-field (singular + near-singular, FP64) assembly and row finalisation:
// adds the near contributions to A, the diagonal term 1 - sum c, and writes
// B[s*R + row] = p_inc_s(x) - beta (c128, column-major R x S).  beta, the
// source-independent row term sum_e (cc/cb) sum_j g_j, is also stored in
// beta_out[row] when beta_out is not null.
// The near elements of each row are listed in CSR form (near_ptr: R + 1
// offsets, near_ids: element ids in increasing order), built once per
// geometry and near_eta by launch_near_list.
void launch_near_assembly(int prec, const RowPoints &rows, int N, const GeoTables &geo,
                          const Physics &ph, void *A, size_t lda, const void *c_part,
                          const void *beta_part, int ntiles, const DevSource *srcs, int S,
                          double2 *B, double2 *beta_out, const int *near_ptr, const int *near_ids,
                          cudaStream_t st);
// Uniform grid over element centroids for the near-pair search: cell edge
// 1/inv_cell, dim[0] x dim[1] x dim[2] cells from corner lo, elements of cell
// c at cell_elems[cell_start[c] .. cell_start[c+1]).
struct NearGrid {
    double lo[3];
    double inv_cell;
    int dim[3];
    const int *cell_start;
    const int *cell_elems;
};
// The pairs the far kernel skips (pair_is_near): with d_ids null, d_cnt[row]
// = number of near elements of the row; else the ids are written at
// d_ids[d_ptr[row]..].
void launch_near_list(const RowPoints &rows, int N, const GeoTables &geo, const NearGrid &grid, const int *d_ptr,
                      int *d_cnt, int *d_ids, cudaStream_t st);
// B[s*R + row] = p_inc_s(x_row) - beta[row]: the right-hand sides of an
// assembled system for a new set of sources (no element integrals).
void launch_rhs_from_beta(const RowPoints &rows, double k, const DevSource *srcs, int S,
                          const double2 *beta, double2 *B, cudaStream_t st);

// Field evaluation.  u: surface solution, column-major N x S (u[s*ldu + node]),
// c64 or c128 per prec.  out[s*P + p] (c128) = p_inc_s(x_p) - sum_e(...);
// part holds nsplit*P*S partial sums, near_part P*S (used when eta > 0).
void launch_field(int prec, const RowPoints &pts, const GeoTables &geo, const Physics &ph,
                  const void *u, size_t ldu, int S, const DevSource *srcs, double2 *part, int nsplit,
                  double2 *near_part, double2 *out, cudaStream_t st);

// ---- linear algebra (linalg.cu) ----
// y = A x for row-major A (R x N, lda) in c64 with FP32 accumulation; x and y
// are c64 or c128 (xd/yd flags: 1 means c128).
void launch_gemv_c64(int R, int N, const float2 *A, size_t lda, const void *x, int xd, void *y,
                     int yd, cudaStream_t st);
// y = x rounded to c64 (n entries)
void launch_to_c64(int n, const double2 *x, float2 *y, cudaStream_t st);
// w = A^H u (N), two-pass column-block reduction through `part`
// (nsplit x N c64 or c128).
int gemv_h_splits(int R, int N);
// conj = false gives w = A^T u (used on a column-major matrix viewed as the
// row-major transpose).
void launch_gemv_h_c64(int R, int N, const float2 *A, size_t lda, const void *u, int ud,
                       void *w, int wd, void *part, cudaStream_t st, bool conj = true);
// One Arnoldi step (CGS2, norm, next basis vector and its c64 copy, the
// Hessenberg column and its Givens rotation, *res = |g_{j+1}|) in a single
// cooperative launch; part is scratch of 3 (j+1) x arnoldi_step_blocks()
// c128.  Returns false (nothing launched) when a cooperative launch is not
// available, then the caller runs the separate kernels.
int arnoldi_step_blocks();
// With wpart, w is first formed as the sum of nsplit partial products
// (wpart[t N + i], double float in split order), in the same launch; without
// it w holds A^H A v_j in FP64.  Vff: the basis in double float (float4 per
// entry: re head, im head, re tail, im tail; same stride as V), kept beside
// V by this step and by launch_scale_copy; w and part are used as double
// float in place.
bool launch_arnoldi_step(int n, int j, double2 *V, size_t ldv, float4 *Vff, double2 *w, float2 *vf, double2 *h1,
                         double2 *h2, double2 *H, int ldh, double2 *cs, double2 *sn, double2 *g, double *res,
                         double2 *part, cudaStream_t st, const float2 *wpart = nullptr, int nsplit = 0);
// w = A^H (A v) for c64 A with A read once (cluster kernel, A streamed by
// TMA bulk copies); v c64, w c128; part: scratch of normal_op_clusters(N) x N
// c64.  Returns false (nothing launched) when N is above what one cluster
// covers (45056).
int normal_op_clusters(int N);
// status: the calling solver's status word (device int), set to 1 when a
// bounded wait of the kernel times out.
// With nsplit_out, the clusters' partial products are left in part (nsplit_out
// of them, stride N) for the caller to sum (launch_normal_op_sum, or the
// Arnoldi step), and w is not written.
bool launch_normal_op(int R, int N, const float2 *A, size_t lda, const float2 *v, double2 *w, float2 *part,
                      int *status, cudaStream_t st, int *nsplit_out = nullptr);
void launch_normal_op_sum(int N, int nsplit, const float2 *part, double2 *w, cudaStream_t st);
// True (and the word cleared) when a normal-operator launch gave up waiting
// for one of its copies and recorded it in *status; synchronises the stream.
bool normal_op_timed_out(int *status, cudaStream_t st);
int gemv_h_f64_splits(int R, int N);
// Block products in FP32 on the CUDA cores (block_simt.cu), one pass over A
// per product for up to 32 sources: T = A X with X N x S column-major (c64,
// or c128 rounded to c64) and T planar (R x 2S floats: Re in columns 0..S-1,
// Im in S..2S-1); W = A^H T with W N x S column-major c64.  A row-major
// R x N c64, lda a multiple of 8.  scratch: block_simt_scratch_floats(R, N, S)
// floats (the packed operand and the split products' partial sums).
size_t block_simt_scratch_floats(int R, int N, int S);
void launch_block_av(const float2 *A, size_t lda, int R, int N, int S, const float2 *X, float *T, float *scratch,
                     cudaStream_t st);
void launch_block_av_c128(const float2 *A, size_t lda, int R, int N, int S, const double2 *X, float *T,
                          float *scratch, cudaStream_t st);
void launch_block_aht(const float2 *A, size_t lda, int R, int N, int S, const float *T, float2 *W, float *scratch,
                      cudaStream_t st);
// FP64 accumulation variants (the refinement residuals): A is c64 or c128.
// r = b - A x.  For c64 A the products are exact double-float FP32
// arithmetic; xsplit is scratch for x's float head and tail (2N + 1 c64:
// the tail starts at N rounded up to even).
void launch_resid(int prec, int R, int N, const void *A, size_t lda, const double2 *x,
                  const double2 *b, double2 *r, float2 *xsplit, cudaStream_t st);
// w = A^H u, FP64-accurate; for c64 A, usplit is scratch for u's float head
// and tail (2R c64).
void launch_gemv_h_f64(int prec, int R, int N, const void *A, size_t lda, const double2 *u,
                       double2 *w, double2 *part, float2 *usplit, cudaStream_t st);
// Row-major (R x N) -> column-major (R x N, ld_out) copy with conversion.
void launch_to_colmajor(int prec_in, const void *A, size_t lda, int R, int N, int prec_out,
                        void *out, size_t ld_out, cudaStream_t st);

// GMRES building blocks on FP64 vectors of length n.
void launch_dots(int n, int k, const double2 *V, size_t ldv, const double2 *w, double2 *h,
                 double2 *part, cudaStream_t st);            // h[j] = V_j^H w, j < k
void launch_update(int n, int k, const double2 *V, size_t ldv, const double2 *h, double2 *w,
                   cudaStream_t st);                          // w -= V h
// |w| into *out; part: nrm2_parts() doubles of scratch for the per-CTA
// partial sums (null: one CTA does it all)
void launch_nrm2(int n, const double2 *w, double *out, double *part, cudaStream_t st);
int nrm2_parts();
// v = w / *nrm; also writes a c64 copy to vf and a double-float copy to vff
// when they are not null, and with g0 the GMRES right-hand side g0 = *nrm e_1
// (gn entries).
void launch_scale_copy(int n, const double2 *w, const double *nrm, double2 *v, cudaStream_t st,
                       float2 *vf = nullptr, float4 *vff = nullptr, double2 *g0 = nullptr, int gn = 0);
void launch_axpy_combo(int n, int k, const double2 *V, size_t ldv, const double2 *y, double2 *x,
                       cudaStream_t st);                      // x += V y
void launch_copy_f64(int n, const double2 *src, double2 *dst, cudaStream_t st);
void launch_zero_f64(size_t n, double2 *dst, cudaStream_t st);
void launch_cast(int n, const double2 *src, float2 *dst, cudaStream_t st);
void launch_cast_up(int n, const float2 *src, double2 *dst, cudaStream_t st);
// H[0..j, j] = h1 + h2 (h2 may be null), H[j+1, j] = *nrm.
void launch_hcol_finish(int j, const double2 *h1, const double2 *h2, const double *nrm, double2 *H,
                        int ldh, cudaStream_t st);
// Apply rotations 0..j-1 to column j, form rotation j, update g; *res = |g[j+1]|.
void launch_givens(int j, double2 *H, int ldh, double2 *cs, double2 *sn, double2 *g, double *res,
                   cudaStream_t st);
void launch_trisolve(int k, const double2 *H, int ldh, const double2 *g, double2 *y, cudaStream_t st);
void launch_set_scalar_c(double2 *dst, const double *v, cudaStream_t st);   // *dst = (*v, 0)

}  // namespace bem
