// Device-resident solver state behind bem_solver_t.
#pragma once

#include <cublas_v2.h>
#include <cusolverDn.h>

#include <future>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "bem_common.h"
#include "kernels.h"
#include "mesh.h"

namespace bem {

// Process-wide defaults set by the reference-style global calls
// (gaussQuad::sendToDevice, the STRENGTH macro, the density/speed constants).
struct Globals {
    std::mutex mu;
    int order = 6;
    double density = 1.2041;
    double speed = 343.21;
    double strength = 0.0;
};
Globals &globals();
// Throws BEM_ERR_INVALID_ARG for options a solver cannot run with.
void validate_options(const bem_options_t &o);

// Owning device allocation that only grows.
struct DevMem {
    void *p = nullptr;
    size_t bytes = 0;
    void ensure(size_t b);
    void release();
    ~DevMem() { release(); }
    template <class T> T *as() const { return static_cast<T *>(p); }
};

// Host side of the far kernel's column tiles: per tile its element records
// (ordered by element colour), the tile-local column map and counts; cap =
// the column cap they were built for.
struct HostTiles {
    int cap = -1, ntiles = 0, per = 0;
    std::vector<TileRec> recs;
    std::vector<int> ptr, cols, cnt;
    std::vector<int> bptr, tbatch;   // node-disjoint batches of records (TileSet::batch_ptr, tile_batch)
};
// The near-pair search grid's host part: element centroids binned into cells
// of edge >= max(1, eta) x the longest edge x 1.01 (and >= the box's span /
// 160) over the row points' box, elements in increasing order within a cell.
struct NearGridHost {
    double eta = -1.0, cell = 0.0, lo[3] = {0.0, 0.0, 0.0};
    int dim[3] = {0, 0, 0};
    std::vector<int> start, order;   // ncell + 1 cell offsets, E element ids
};
// Host scratch of the table builders, kept by the solver across geometries:
// the vectors keep their capacity, so a new geometry of the same size writes
// into pages already mapped instead of faulting in fresh allocations (which
// cost more than the builders' arithmetic at 20480 elements).
struct HostScratch {
    std::vector<int> order, tile_of, slot_of, size, batch_of, start, cid, fill;
    std::vector<uint32_t> key;
    std::vector<uint64_t> used, level, busy;
    std::vector<std::vector<TileRec>> lists;
};
// Both fill `out`, reusing its vectors' storage.
void build_near_grid(int E, const std::vector<double> &h_nodes, const std::vector<int> &h_elems, const double *lo,
                     const double *hi, double max_edge, double eta, NearGridHost &out, HostScratch &scr);
void build_host_tiles(int N, int E, const std::vector<double> &h_nodes, const std::vector<int> &h_elems, int cap,
                      HostTiles &out, HostScratch &scr);
// Block-solve GEMM mode chosen by timing for (device, R, N, S), shared by
// every handle of the process: -1 while none is stored.
int block_mode_cached(int device, int R, int N, int S);
void block_mode_store(int device, int R, int N, int S, int mode);

}  // namespace bem

struct bem_solver_s {
    int device = 0;
    cudaStream_t stream = nullptr;
    cusolverDnHandle_t cusolver = nullptr;
    cublasHandle_t cublas = nullptr;
    bem_options_t opt{};

    int N = 0, M = 0, E = 0, S = 0, R = 0;
    std::vector<double> h_nodes, h_rows, h_bc;
    std::vector<int> h_elems;
    std::vector<bem_source_t> h_srcs;

    bem::DevMem d_nodes, d_rows_f, d_rows_d, d_elems, d_bc, d_geo_f, d_geo_d, d_srcs;
    double geo_eta = -1.0;   // near_eta the element tables were built with
    // near pairs per row (CSR), valid for the current geometry and geo_eta
    bool near_valid = false;
    bem::DevMem d_near_ptr, d_near_ids, d_grid_start, d_grid_elems;
    double max_edge = 0.0;   // longest element edge (written by set_geometry's grid task: read through physics())
    double extent = 0.0;     // diagonal of the box around nodes and CHIEF points
    double row_lo[3] = {0.0, 0.0, 0.0}, row_hi[3] = {0.0, 0.0, 0.0};   // that box
    int g_sums = 2;   // Physics::g_sums of the BCs: 2 some alpha != 0, 1 alpha = 0 everywhere, 0 gamma = 0 too

    struct Tiles {
        bool valid = false;
        int ntiles = 0, tc_max = 0;
        bem::DevMem recs, rec_ptr, cols, col_cnt, batch_ptr, tile_batch;
        bem::DevMem frecs;   // recs with their geometry (FP32 far kernel), re-formed by every c64 assembly
        int nrec = 0;
    } tiles[2];

    int far_variant_used = -1;

    int prec = -1;
    double k = 0.0;
    size_t lda = 0;
    bool assembled = false, solved = false;
    bem::DevMem d_A, d_B, d_cpart, d_bpart, d_x, d_beta;   // d_beta: source-independent row term (R c128)

    // GMRES / refinement workspace
    bem::DevMem w_V, w_H, w_cs, w_sn, w_g, w_y, w_h1, w_h2, w_w, w_t, w_r, w_gv, w_vf, w_part, w_scal;
    // TF32x3 block products: head/tail planes of A (interleaved form: x_Ahi
    // and x_Alo; 3M form: six planes in x_Ahi) and scratch for the right-hand
    // blocks and products (x_vlo, x_tlo; in the CUDA-core mode x_tlo holds the
    // packed operand and the split products' partial sums)
    bem::DevMem x_Ahi, x_Alo, x_vlo, x_tlo, w_d;
    bem::DevMem w_ap;   // partial sums of the cooperative Arnoldi step
    bem::DevMem w_Vff;  // the refined GMRES basis in double float (float4 an entry), beside w_V
    int tf32_split_mode = -1;   // BEM_GEMM_* the planes of A were built for (this assembly), -1 none
    // tensor-core products (BEM_GEMM_TC): the power-of-two scale of A ([0]
    // scale, [1] inverse, [2] scratch), valid for this assembly
    bem::DevMem tc_scale;
    bool tc_scale_valid = false;
    int last_block_gemm_mode = -1;   // BEM_GEMM_* the last block solve ran its products in
    // device status words of this handle's kernels (each zeroed by its user
    // before its kernels run): [0] a bounded wait of the normal operator timed
    // out, [1] one of the tensor-core GEMM's did, [2] one of the far-field
    // assembly kernel's did
    bem::DevMem d_status;
    double *h_pinned = nullptr;
    cudaEvent_t ev_res[2] = {nullptr, nullptr};   // refined GMRES: residual estimate of step j in h_pinned[4 + (j & 1)]
    cudaEvent_t ev_up = nullptr;                  // set_geometry: its host-to-device copies have landed
    void *h_stage = nullptr;     // pinned staging for geometry uploads
    size_t h_stage_bytes = 0;
    // QR workspace
    bem::DevMem q_A, q_B, q_tau, q_work, q_info;
    // tensor-core QR (solve_qr_tc): the panel's V and its interleaved form, T
    // and V^H V, Z = C^H V, the packed right-hand operands, split-K partial
    // sums, scales
    bem::DevMem qt_v, qt_vrr, qt_t, qt_z, qt_opv, qt_opw, qt_part, qt_scal, qt_dinv;
    // A high-priority second stream of the handle (created on first use by
    // ensure_aux): the QR_TC look-ahead's panel chain, and the near-pair list
    // built beside the far kernel; the QR's events and the assembly's two
    // (element tables ready, near list ready)
    cudaStream_t qr_aux = nullptr;
    cudaEvent_t qr_ev[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    cudaEvent_t asm_ev[2] = {nullptr, nullptr};
    void ensure_aux();
    // field workspace
    bem::DevMem f_rows_f, f_rows_d, f_part, f_near, f_out, f_u;

    // column-tile host tables: the ones in use (host_tiles) and the ones being
    // built beside set_geometry (tiles_next, by tile_future's task), swapped
    // when ensure_tiles takes them; likewise the near-pair grid's host part.
    // The futures are declared after everything their tasks touch, so they
    // are destroyed (their destructors wait for the tasks) first.
    bem::HostTiles host_tiles, tiles_next;
    bem::NearGridHost near_grid_h, grid_next;
    bem::HostScratch tile_scratch, grid_scratch;
    std::vector<int> near_ptr_h, near_cnt_h;
    std::future<void> tile_future, grid_future;

    bem_solver_s();
    ~bem_solver_s();

    void set_geometry(const double *pnts, int num_pnts, const int *elems, int num_elems,
                      const double *bc, const double *chief, int num_chief);
    void set_sources(const bem_source_t *srcs, int num);
    void assemble(double k, int precision);
    void solve(int method, bem_solve_info_t *info);
    void get_solution(void *x, int ldx, int precision);
    void get_system(void *A, int lda_out, void *B, int ldb_out, int precision);
    // Field at host points; u_dev: surface solution on the device in
    // precision u_prec (column-major N x S, ld = N), or null for the solver's
    // own solution.
    void eval_field(const double *pts, int num_pts, void *out, int ldo, int precision,
                    const void *u_dev = nullptr, int u_prec = BEM_PREC_C128);

    // Device bytes currently held by the handle.
    size_t device_bytes() const;
    // Upper estimate of the device bytes an assembly (c64) plus solve with the
    // given method needs, before any allocation.
    static size_t estimate_bytes(int N, int E, int M, int S, int method, const bem_options_t &o);

    void ensure_geo();
    void ensure_near_list(cudaStream_t st);   // its uploads, kernels and read-back on st
    void ensure_tiles(int precision);
    bem::GeoTables geo_tables() const;
    bem::RowPoints row_points() const;
    bem::Physics physics() const;
    void solve_qr();
    void solve_qr_tc(bem_solve_info_t *info);
    void solve_refined(bem_solve_info_t *info);
    void solve_block(bem_solve_info_t *info);
    // GEMM modes of the block solve worth running for S right-hand sides and
    // an R x N system: the fixed mode, or AUTO's candidates; with two, the
    // first solve of each shape times both and the process keeps the faster
    // (block_mode_cached / block_mode_store).  Measured per A V + A^H T pair:
    // * up to 8 sources the streaming CUDA-core kernels (one pass over A per
    //   product) beat the library GEMMs, whose skinny-shape kernels run far
    //   below the bandwidth bound (40962 nodes, 4 / 8 sources: 4.2 / 6.3 ms
    //   against cuBLAS SGEMM 10.2 / 10.3 ms; 15212 nodes, 8 sources: 0.88 ms
    //   against 1.19 TF32x3 and 1.82 SGEMM);
    // * from 9 to 32 sources, while A is at most 4 GB, the order of the
    //   CUDA-core kernels and TF32x3 depends on the shape (16 sources: 10242
    //   nodes 0.70 against 1.30 ms, 15212 nodes 1.41 against 1.18 ms): both
    //   are candidates;
    // * the TF32x3 modes keep head/tail planes of A (2x or 3x the c64
    //   matrix), so they are taken only while A is at most 4 GB: for larger
    //   systems the planes' memory costs the request server more concurrency
    //   than the faster products gain (64 frequencies up to 40962 nodes: 17.9
    //   against 33.0 solves/s).  There SGEMM (split-BF16 emulation from 32
    //   sources) stays from 9 sources on: at 16 sources on 40962 nodes the
    //   CUDA-core kernels are 6% faster alone, but seven such solves side by
    //   side in the request server finished later with them (one 172 KB CTA
    //   per SM) than with SGEMM.
    static std::vector<int> block_gemm_candidates(const bem_options_t &o, int S, int R, int N) {
        if (o.gemm_mode >= 0) return {o.gemm_mode};
        if (S <= 8) return {BEM_GEMM_SIMT, BEM_GEMM_TC};
        return {BEM_GEMM_TC};
    }
};
