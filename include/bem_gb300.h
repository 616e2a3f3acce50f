/*
 * bem_gb300.h -- C ABI of the GB300-native Helmholtz BEM engine.
 *
 * Plain pointers, sizes and opaque handles only.  Complex arrays are
 * interleaved (re, im) pairs of float (c64) or double (c128).  Matrices are
 * column-major with a leading dimension: entry (r, c) at ld*c + r, the
 * reference's IDXC0 (numerical.h:44-46).
 *
 * Every call returns a status code.  BEM_SUCCESS (0) and BEM_FAILURE (1) are
 * EXIT_SUCCESS and EXIT_FAILURE, the only values the reference returns
 * (numerical.h:59-122); the other codes refine the failure, and
 * bem_last_error() gives a message for the calling thread.
 *
 * Each declaration cites the reference function it replaces, as
 * file:line within ZiqiFrancisFan/BEM_GPU_Clean_CPP.
 */
#ifndef BEM_GB300_H
#define BEM_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#define BEM_SUCCESS 0
#define BEM_FAILURE 1
#define BEM_ERR_INVALID_ARG 2
#define BEM_ERR_CUDA 3
#define BEM_ERR_NOMEM 4
#define BEM_ERR_NOT_CONVERGED 5
#define BEM_ERR_IO 6
#define BEM_ERR_STATE 7
#define BEM_ERR_TOO_LARGE 8
#define BEM_ERR_NUMERIC 9
#define BEM_ERR_TIMEOUT 10

/* Library status and introspection (no reference counterpart). */
const char *bem_status_string(int status);
const char *bem_last_error(void);
int bem_version(void);
/* Number of CUDA kernels this library has launched in the process. */
long long bem_launch_count(void);
/* Kernel timing: while on, every kernel (and cuSOLVER call sequence) the
 * library launches is bracketed by CUDA events on its stream.  Turning it
 * on clears the previous records. */
int bem_profile_enable(int on);
/* Writes one "name launches total_ms\n" line per kernel name into buf
 * (after waiting for the recorded events); returns the number of lines or a
 * negative status. */
int bem_profile_report(char *buf, int buflen);

/* ------------------------------------------------------------------ */
/* Quadrature: gaussQuad (numerical.h:166-187)                          */
/* ------------------------------------------------------------------ */
/* Gauss-Legendre nodes/weights on [-1,1], ascending: gaussQuad::
 * genGaussParams (numerical.cu:186-225). */
int bem_gauss_legendre(int order, double *nodes, double *weights);
/* Default Gauss order for new solvers and the drop-in calls:
 * gaussQuad(order) + sendToDevice() (numerical.cu:152-156, 227-231). */
int bem_set_quadrature(int order);
int bem_get_quadrature(void);
/* Medium constants: __constant__ density/speed (numerical.cu:12-14). */
int bem_set_medium(double density, double speed);
/* Point-source strength q in p_inc = q*G: the STRENGTH macro
 * (numerical.h:128-130), 0 by default as in the reference. */
int bem_set_point_source_strength(double q);

/* ------------------------------------------------------------------ */
/* Mesh: class mesh (mesh.h:216-259)                                    */
/* ------------------------------------------------------------------ */
typedef struct bem_mesh_s *bem_mesh_t;

int bem_mesh_create(bem_mesh_t *out);                    /* mesh::mesh() */
int bem_mesh_destroy(bem_mesh_t m);                      /* mesh::~mesh (mesh.cu:1301-1311) */
/* mesh::readObj (mesh.cu:1215-1265), same parse rules: 48-char line
 * chunks, any line starting 'v' is a vertex, first integer of each face
 * field, bc = (0, 1, -1). */
int bem_mesh_read_obj(bem_mesh_t m, const char *path);
/* Robust OBJ reader (no reference counterpart): v/vt/vn, f a/b/c, negative
 * indices, polygons (fan-triangulated), any line length. */
int bem_mesh_read_obj_robust(bem_mesh_t m, const char *path);
/* PLY reader (no reference counterpart: the reference ships
 * Head_20kHz_iso.ply but reads OBJ only): ascii, binary_little_endian and
 * binary_big_endian; x, y, z of "vertex" (any numeric type), the
 * vertex_indices list of "face" (polygons fan-triangulated), other elements
 * and properties skipped; bc = (0, 1, -1). */
int bem_mesh_read_ply(bem_mesh_t m, const char *path);
/* Winding check and repair (no reference counterpart; the reference trusts
 * the file, mesh.cu:1215-1265): makes the winding consistent over each
 * edge-connected component and turns every closed component so that
 * (p1-p3) x (p2-p3) points into the body.  Any output pointer may be NULL:
 * elements flipped, components, edges with one element, edges with more than
 * two, enclosed volume of the closed components. */
int bem_mesh_orient(bem_mesh_t m, int *flipped, int *components, int *open_edges, int *nonmanifold,
                    double *volume);
/* Direct geometry (no reference counterpart); bc reset to (0, 1, -1). */
int bem_mesh_set(bem_mesh_t m, const double *pnts, int num_pnts, const int *elems, int num_elems);
/* Per-element bc (ca, cb, cc) as 6 doubles (re, im) each: the triElem::bc
 * field (mesh.h:202), which readObj hard-codes (mesh.cu:1240-1242). */
int bem_mesh_set_bc(bem_mesh_t m, const double *bc);
int bem_mesh_set_uniform_bc(bem_mesh_t m, double ca_re, double ca_im, double cb_re,
                            double cb_im, double cc_re, double cc_im);
/* mesh::findBB (mesh.cu:1369-1409): bounding box padded by threshold. */
int bem_mesh_find_bb(bem_mesh_t m, float threshold);
int bem_mesh_get_bb(bem_mesh_t m, float *bb6);
/* mesh::genCHIEF (mesh.cu:1430-1483): candidates from cuRAND's host XORWOW
 * generator with seeds 0, 1, 2, ...; a candidate is accepted when a ray from
 * it crosses the surface an odd number of times and it is at least
 * threshold from every node.  The ray tests run on the GPU in batches. */
int bem_mesh_gen_chief(bem_mesh_t m, int num, float threshold);
/* Explicit CHIEF points (no reference counterpart: chiefPnts is private,
 * mesh.h:233). */
int bem_mesh_set_chief(bem_mesh_t m, const double *pnts, int num);
/* getNumPnts / getNumElems / getNumChief (mesh.h:255-258). */
int bem_mesh_get_counts(bem_mesh_t m, int *num_pnts, int *num_elems, int *num_chief);
int bem_mesh_get_points(bem_mesh_t m, double *pnts);
int bem_mesh_get_elems(bem_mesh_t m, int *elems);
int bem_mesh_get_chief(bem_mesh_t m, double *pnts);
/* Icosphere generator (no reference counterpart) with the reference
 * spheres' inward winding: (p1-p3) x (p2-p3) points into the body. */
int bem_mesh_icosphere(bem_mesh_t m, int subdiv, double radius);
/* cmptSurfArea (mesh.cu:1082-1117). */
int bem_mesh_surface_area(bem_mesh_t m, double *area);
/* Synthetic geometry for the benchmark configurations (no reference
 * counterpart).  Class-I geodesic sphere of frequency nu (V = 10 nu^2 + 2,
 * F = 20 nu^2), inward winding. */
int bem_mesh_geodesic(bem_mesh_t m, int nu, double radius);
/* Maps a unit-sphere mesh onto the ellipsoid (a, b, c) radially perturbed by
 * a seeded real-spherical-harmonic field up to degree lmax whose largest
 * magnitude over the nodes is amp (relative). */
int bem_mesh_perturbed_ellipsoid(bem_mesh_t m, double a, double b, double c, int lmax, double amp,
                                 unsigned long long seed);
/* n points (3 doubles each) of a Fibonacci lattice on a sphere. */
int bem_fibonacci_sphere(int n, double radius, double *pts);
/* Block partition of the collocation matrix for a hierarchical (H-matrix)
 * representation (no reference counterpart: the reference stores A dense,
 * mesh.cu:985-1006).  Host only.  rows: num_rows points (3 doubles each:
 * the nodes, then the CHIEF points); cols: num_cols points (the nodes).  Each
 * set is clustered by median bisection along the longest axis of the
 * cluster's bounding box down to clusters of at most leaf points (clusters of
 * coincident points stay whole).  A block pairs a row cluster I with a
 * column cluster J: admissible (low rank, flag 1) when the boxes are apart
 * and min(diam I, diam J) <= eta * dist(I, J), dense (flag 0) when neither
 * can be split further.  row_perm[num_rows] and col_perm[num_cols] (may be
 * NULL) receive the clustered order (position -> original index); blocks
 * (may be NULL) receives 5 ints per block, (row_begin, row_count, col_begin,
 * col_count, admissible) in clustered positions.  The blocks tile the
 * num_rows x num_cols index space exactly once.  *num_blocks is always set;
 * BEM_ERR_TOO_LARGE when blocks is not NULL and max_blocks is smaller. */
int bem_hmat_partition(const double *rows, int num_rows, const double *cols, int num_cols, int leaf,
                       double eta, int *row_perm, int *col_perm, int *blocks, int max_blocks,
                       int *num_blocks);
/* The same partition for a collocation system whose rows are the nodes and
 * then the CHIEF points (no reference counterpart).  The node rows use the
 * column tree itself: row position p < num_pnts and column position p are the
 * same node, node_perm[p] (num_pnts entries); row position num_pnts + p is
 * CHIEF point chief_perm[p] (num_chief entries, its own cluster tree).
 * Renumbering the mesh nodes by node_perm and the CHIEF points by chief_perm
 * before assembly therefore gives A directly in the clustered order.  No
 * block mixes node rows and CHIEF rows.  Other arguments and results as for
 * bem_hmat_partition. */
int bem_hmat_partition_system(const double *pnts, int num_pnts, const double *chief, int num_chief, int leaf,
                              double eta, int *node_perm, int *chief_perm, int *blocks, int max_blocks,
                              int *num_blocks);
/* Hierarchical form of a c64 matrix already on the device (no reference
 * counterpart).  A_dev: R x N, row-major with row stride lda, rows and
 * columns in the clustered order of the partition (A[row_perm][:, col_perm]);
 * blocks: num_blocks x 5 ints from bem_hmat_partition.  Admissible blocks are
 * compressed by partially pivoted adaptive cross approximation to relative
 * tolerance tol (|u_k| |v_k| <= tol ||S_k||_F) with at most kmax <= 128 terms;
 * a block whose approximation needs more terms, or as many as the dense block
 * would hold, is stored dense, as are the inadmissible blocks.  The handle
 * owns its device memory (A may be freed afterwards).  Work is queued on
 * stream (a cudaStream_t, NULL for the legacy stream) and the call returns
 * once it is complete. */
typedef struct bem_hmat_s *bem_hmat_t;
int bem_hmat_compress_c64(const void *A_dev, int R, int N, int lda, const int *blocks, int num_blocks,
                          double tol, int kmax, void *stream, bem_hmat_t *out);
/* y = H x (trans 0: x has N entries, y R) or y = H^H x (trans 1: x has R
 * entries, y N); c64 device vectors in the clustered order, queued on stream.
 * One product at a time per handle (it keeps one work vector).  The result is
 * bitwise repeatable: every output entry has one writer and a fixed order. */
int bem_hmat_matvec_c64(bem_hmat_t h, int trans, const void *x_dev, void *y_dev, void *stream);
/* Stored complex entries, largest rank, low-rank and dense block counts. */
int bem_hmat_info(bem_hmat_t h, long long *entries, int *max_rank, int *lowrank_blocks, int *dense_blocks);
int bem_hmat_destroy(bem_hmat_t h);

/* ------------------------------------------------------------------ */
/* Drop-in calls with host buffers (the reference's call surface)       */
/* ------------------------------------------------------------------ */
/* bemSystem (mesh.h:222-223, mesh.cu:985-1006): A ((N+M) x N) and B
 * ((N+M) x numSrcs), c64, for point sources of strength STRENGTH at
 * srcs[3*i]; FP32 regular quadrature, FP64 singular integrals. */
int bem_system_c64(bem_mesh_t m, float k, const float *srcs, int num_srcs, float *A, int lda,
                   float *B, int ldb);
/* qrSolver (numerical.h:196-197, numerical.cu:580-644): least-squares
 * solve, B overwritten, solution in rows 0..nA-1. */
int bem_qr_solve_c64(const float *A, int mA, int nA, int ldA, float *B, int nB, int ldB);
/* GMRES (GMRES.h:104-105, GMRES.cu:145-279): unrestarted GMRES on a square
 * m x m system, x holds x0 on entry. */
int bem_gmres_c64(const float *A, const float *b, int m, int max_iter, float thr, float *x);
/* GMRES on device buffers that allocates nothing.  No counterpart in the
 * reference: it is for callers that cannot allocate GPU memory while they
 * solve (a serving process whose device memory is owned and capped by its
 * own pool allocator, code that must not add allocations while a CUDA stream
 * capture of another component is in progress, a real-time loop that cannot
 * afford cudaMalloc's latency and implicit synchronisation).  Same algorithm
 * and stopping rule as bem_gmres_c64.  A_dev is m x m column-major c64 with
 * an even lda >= m and a 16-byte aligned start; b_dev and x_dev hold m c64
 * values (x_dev: x0 on entry, the solution on return); stream is a
 * cudaStream_t or NULL; *iters (may be NULL) receives the iteration count.
 * All scratch lives in one static device array of about 5.4 MiB that every
 * GPU loading the library keeps until exit, which limits m to
 * BEM_NOALLOC_MAX_M and min(max_iter, m) to BEM_NOALLOC_MAX_ITER; larger
 * sizes return BEM_ERR_TOO_LARGE.  The first call on a device, and the first
 * after the device's context was re-created (cudaDeviceReset), looks up the
 * array's device address: make that call before any stream capture.  Each
 * iteration reads an 8-byte residual estimate and synchronises `stream`: a
 * caller that solves while another component's stream capture runs passes a
 * stream created with cudaStreamNonBlocking, not NULL (work on the legacy
 * NULL stream synchronises with blocking streams, which would break that
 * capture).  Calls share the array: calls that overlap on the GPU race. */
#define BEM_NOALLOC_MAX_M 2048
#define BEM_NOALLOC_MAX_ITER 128
int bem_gmres_c64_noalloc(const float *A_dev, int lda, const float *b_dev, int m, int max_iter,
                          float thr, float *x_dev, void *stream, int *iters);
/* Dense real product C = op(A) B on the tcgen05 tensor cores: the kernel
 * the block solve's multi-right-hand-side products (which replace the
 * Cgemm/Cgemv products of numerical.cu:375-396 and GMRES.cu:90-143) and the
 * QR trailing updates run on.  A is row-major with row stride lda (a
 * multiple of 4): trans = 0: op(A) = A (m x k); trans = 1: op(A) = A^T with A
 * stored k x m.  B is k x n and C m x n, column-major (ldb, ldc).  parts = 2:
 * fp16 head + tail split products, about 2^-22 relative to sum |a||b| (the
 * accuracy of TF32x3); parts = 3: head + middle + tail, only the tensor
 * core's FP32 accumulation left (errors of order sqrt(k) 2^-24 relative to
 * sum |a||b|).  Host buffers; device memory is allocated and freed inside
 * the call. */
int bem_tc_gemm_f32(int trans, int m, int k, int n, const float *A, int lda, const float *B, int ldb, float *C,
                    int ldc, int parts);
/* genExtPressure (mesh.h:425-426, mesh.cu:1038-1073): pressure at x from
 * the surface pressure surf_p (numPnts c64 values). */
int bem_ext_pressure_c64(float k, bem_mesh_t m, const float *src, const float *x,
                         const float *surf_p, float *p_out);
/* wrtCplxMat (numerical.cu:556-578): "(%f,%f) " rows. */
int bem_write_cplx_mat_c64(const float *mat, int rows, int cols, int ldm, const char *path);

/* ------------------------------------------------------------------ */
/* Device-resident solver handle (extends bemSystem/qrSolver/GMRES/     */
/* genExtPressure: matrices, sources and solutions stay in HBM)         */
/* ------------------------------------------------------------------ */
typedef struct bem_solver_s *bem_solver_t;

enum { BEM_SRC_POINT = 0, BEM_SRC_PLANE = 1 };
/* One incident field: point source a*G(k,|x-vec|) (pntSrc, mesh.cu:114-118)
 * or plane wave a*exp(-i k vec.x) (no reference counterpart). */
typedef struct {
    int kind;
    double vec[3];
    double amp_re, amp_im;
} bem_source_t;

enum { BEM_PREC_C64 = 0, BEM_PREC_C128 = 1 };
enum { BEM_SOLVE_QR = 0, BEM_SOLVE_GMRES_REFINED = 1, BEM_SOLVE_BLOCK_GMRES = 2, BEM_SOLVE_QR_TC = 3 };
/* Block-solve GEMMs (the products inside the inner GMRES).
 * BEM_GEMM_TC (the default's choice from 9 sources on): this library's own
 * tcgen05 tensor-core kernel (bem_tc_gemm_f32) on the interleaved-real form
 * of the complex products, reading the c64 matrix directly (no split copies
 * of A): fp16 head + tail split products (TF32x3-level accuracy) inside the
 * inner GMRES, head + middle + tail (FP32-accurate) for the once-per-cycle
 * refinement products (the residual update R -= A D and the gradient
 * A^H R).
 * BEM_GEMM_SIMT: FP32 products on the CUDA cores by this library's own
 * streaming kernels (one pass over A per product for up to 32 right-hand
 * sides, more in further passes; no extra copies of A; the refinement
 * products FP32 as well).
 * Library (cuBLAS) modes, kept for comparison: FP32, FP32-accurate
 * split-BF16 emulation, plain TF32, TF32x3 on the interleaved-real form (A
 * and the right-hand block split into TF32 head + tail planes), or TF32x3 in
 * the 3M form (planes of Re A, Im A, Re A + Im A); their refinement products
 * run split-BF16 (FP32 in FP32 mode).
 * AUTO: up to 8 right-hand sides the faster of SIMT and TC for the shape
 * (timed on the first solve of each shape, kept for the process), TC from
 * 9 on. */
enum { BEM_GEMM_AUTO = -1, BEM_GEMM_FP32 = 0, BEM_GEMM_SPLIT_BF16 = 1, BEM_GEMM_TF32 = 2, BEM_GEMM_TF32X3 = 3,
       BEM_GEMM_TF32X3_3M = 4, BEM_GEMM_SIMT = 5, BEM_GEMM_TC = 6 };

typedef struct {
    double density;     /* 1.2041 (numerical.cu:12) */
    double speed;       /* 343.21 (numerical.cu:14) */
    int order;          /* Gauss points per direction, INTORDER = 6 */
    double near_eta;    /* 0: plain rule for every x not a vertex of e (reference) */
    int near_depth;     /* maximum subdivision depth of near-singular pairs */
    double tol;         /* refinement: relative normal-equation residual */
    int max_iter;       /* inner GMRES iterations per refinement step */
    double inner_tol;   /* inner GMRES relative tolerance */
    int max_refine;     /* refinement steps */
    int tile_cols;      /* far-field column tile width, 0 = automatic (<= 12288) */
    int far_variant;    /* far-field launch shape, -1 = autotuned per problem shape */
    int gemm_mode;      /* block solve products: BEM_GEMM_* */
    double block_tol;   /* block solve: relative normal-equation residual per right-hand side */
} bem_options_t;

typedef struct {
    int iterations;      /* total inner iterations */
    int refinements;     /* outer refinement steps */
    double rel_residual; /* final ||A^H (b - A x)|| / ||A^H b|| (max over sources) */
    int converged;
} bem_solve_info_t;

int bem_options_default(bem_options_t *o);
int bem_solver_create(bem_solver_t *out);   /* binds the current CUDA device */
int bem_solver_destroy(bem_solver_t s);
int bem_solver_set_options(bem_solver_t s, const bem_options_t *o);
int bem_solver_get_options(bem_solver_t s, bem_options_t *o);
/* Upload nodes, elements, bc and CHIEF points of a mesh. */
int bem_solver_set_mesh(bem_solver_t s, bem_mesh_t m);
/* Same from raw host arrays; bc (6 doubles per element) may be NULL for
 * (0, 1, -1), chief may be NULL when num_chief is 0. */
int bem_solver_set_geometry(bem_solver_t s, const double *pnts, int num_pnts, const int *elems,
                            int num_elems, const double *bc, const double *chief, int num_chief);
int bem_solver_set_sources(bem_solver_t s, const bem_source_t *srcs, int num_srcs);
/* Assemble A and B on the device for wavenumber k.  BEM_PREC_C64: FP32
 * regular quadrature, FP64 singular and near-singular integrals, c64
 * storage.  BEM_PREC_C128: FP64 throughout, c128 storage. */
int bem_solver_assemble(bem_solver_t s, double k, int precision);
/* BEM_SOLVE_QR: dense least squares (Householder QR) in the assembly
 * precision.  BEM_SOLVE_GMRES_REFINED: GMRES on the normal equations with
 * FP32 matrix products and FP64 Arnoldi/Givens, inside FP64 iterative
 * refinement (requires a c64 assembly).  BEM_SOLVE_BLOCK_GMRES: all sources
 * together; the normal-operator products for every source are GEMMs on the
 * tensor cores (gemm_mode), each source keeps its own FP32 Krylov space
 * with FP64 Hessenberg/Givens, outer refinement to block_tol (requires a c64
 * assembly).
 * BEM_SOLVE_QR_TC (either assembly precision): least squares by this
 * library's blocked Householder QR (the WY blocked QR_thin / lsqSolver of
 * numerical.cu:246-554 and the qrSolver sequence of numerical.cu:580-644):
 * panels of 128 columns factored in FP32 by one thread-block cluster each,
 * trailing updates (I - V T V^H)^H C as tensor-core GEMMs (the kernel of
 * bem_tc_gemm_f32), Q applied to B on the way and never formed, then FP64
 * refinement through the semi-normal equations with the FP32 factor (FP64-
 * accurate residuals of the assembled matrix) to a relative normal-equation
 * residual of 1e-14 or until it stagnates; info->refinements = refinement
 * steps, info->rel_residual = the residual reached. */
int bem_solver_solve(bem_solver_t s, int method, bem_solve_info_t *info);
/* Copy results to host buffers in the given precision (BEM_PREC_*). */
int bem_solver_get_solution(bem_solver_t s, void *x, int ldx, int precision);
int bem_solver_get_system(bem_solver_t s, void *A, int lda, void *B, int ldb, int precision);
/* Field pressure at num_pts points (3 doubles each) for every source:
 * p (num_pts x S, column-major, ldp) in the given precision. */
int bem_solver_eval_field(bem_solver_t s, const double *pts, int num_pts, void *p, int ldp,
                          int precision);
int bem_solver_sync(bem_solver_t s);
/* The cudaStream_t all work of the handle is queued on. */
void *bem_solver_stream(bem_solver_t s);
int bem_solver_sizes(bem_solver_t s, int *n, int *m, int *num_elems, int *num_srcs);
/* The BEM_GEMM_* mode the handle's last BEM_SOLVE_BLOCK_GMRES ran its
 * products in (AUTO's choice), or BEM_GEMM_AUTO before any block solve (no
 * reference counterpart). */
int bem_solver_block_gemm_mode(bem_solver_t s, int *mode);
/* The far-field kernel's launch shape the handle's last c64 assembly ran
 * (the autotuner's choice unless options fix it; 0 .. 6), or -1 before any
 * (no reference counterpart). */
int bem_solver_far_variant(bem_solver_t s, int *variant);

/* ------------------------------------------------------------------ */
/* Request server (no reference counterpart: the reference solves one   */
/* problem per process, main.cpp:27-73).  Independent surface solves of  */
/* different meshes, wavenumbers and source counts run concurrently:    */
/* each of `slots` workers drives its own solver handle on its own CUDA  */
/* stream, and a request is admitted as soon as a worker is free and its */
/* device footprint fits the HBM budget, while other requests are on the */
/* GPU (continuous batching).  Assembled systems stay resident after     */
/* their request (LRU, `cache_systems`): a later request with the same   */
/* geometry, boundary condition, CHIEF points and wavenumber reuses A    */
/* and rebuilds only B for its sources.                                  */
/* ------------------------------------------------------------------ */
typedef struct bem_server_s *bem_server_t;

typedef struct {
    int slots;                 /* requests in flight at once (worker threads) */
    double hbm_budget_bytes;   /* admission limit; 0 = 85% of the free device memory at creation */
    int cache_systems;         /* idle assembled systems kept for reuse */
    int block_min_sources;     /* BEM_SOLVE_BLOCK_GMRES from this many sources on, else GMRES_REFINED */
    bem_options_t solver;      /* options of every solve */
} bem_server_options_t;

/* One request.  All arrays are copied by bem_server_submit.  bc: 6 doubles
 * per element or NULL for (0, 1, -1); chief: NULL when num_chief is 0. */
typedef struct {
    const double *pnts;
    int num_pnts;
    const int *elems;
    int num_elems;
    const double *bc;
    const double *chief;
    int num_chief;
    double k;
    const bem_source_t *srcs;
    int num_srcs;
} bem_request_t;

typedef struct {
    int status;                /* BEM_SUCCESS or the status of the failed step */
    int method;                /* BEM_SOLVE_* used */
    int iterations, refinements, converged;
    double rel_residual;
    double queue_ms;           /* submit -> admitted */
    double service_ms;         /* admitted -> solution on the host */
    double latency_ms;         /* submit -> solution on the host */
    int cache_hit;             /* 1: the assembled system was reused */
    double device_bytes;       /* footprint the request was admitted with */
    int num_pnts, num_srcs;    /* shape of the solution (N x S) */
} bem_request_result_t;

typedef struct {
    long long submitted, completed, failed, solves, cache_hits, evictions;
    double p50_ms, p99_ms, mean_ms, max_ms;   /* request latency of completed requests */
    double resident_bytes, peak_bytes;        /* admitted footprints (in flight + cached) */
    int max_in_flight;
} bem_server_stats_t;

int bem_server_options_default(bem_server_options_t *o);
/* Binds the current CUDA device.  Fails with BEM_ERR_CUDA without one. */
int bem_server_create(const bem_server_options_t *o, bem_server_t *out);
/* Finishes every admitted and queued request, then frees all device memory. */
int bem_server_destroy(bem_server_t s);
int bem_server_submit(bem_server_t s, const bem_request_t *r, long long *ticket);
/* Waits up to timeout_s seconds (< 0: no limit) for the request.  On
 * completion copies the surface pressure (N x S c128, column-major, ldx >= N)
 * to x when x is not NULL, fills res when not NULL, releases the ticket and
 * returns the request's status; BEM_ERR_TIMEOUT leaves the ticket valid. */
int bem_server_wait(bem_server_t s, long long ticket, double timeout_s, void *x, int ldx,
                    bem_request_result_t *res);
int bem_server_stats(bem_server_t s, bem_server_stats_t *st);
int bem_server_reset_stats(bem_server_t s);

#ifdef __cplusplus
}
#endif

#endif /* BEM_GB300_H */
