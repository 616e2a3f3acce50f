// Host orchestration of the device-resident solver: geometry upload, column
// tiles, assembly launches, the dense QR least-squares solve and the
// mixed-precision refined GMRES solve.
#include "solver.h"
#include "tc_gemm.h"

#include <algorithm>
#include <future>
#include <cmath>
#include <cstring>
#include <numeric>
#include <string>

namespace bem {

Globals &globals() {
    static Globals g;
    return g;
}

void DevMem::ensure(size_t b) {
    if (b <= bytes && p) return;
    release();
    if (b == 0) return;
    CUDA_TRY(cudaMalloc(&p, b));
    bytes = b;
}

void DevMem::release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
}

namespace {

constexpr int kTileColsMax = 12288;   // columns per tile: 2 rows x 12288 x 8 B = 192 KB smem (c64)

size_t round_up(size_t v, size_t m) { return (v + m - 1) / m * m; }

// Morton (Z-order) key of a point inside the bounding box, 10 bits per axis.
uint32_t morton_key(const double *p, const double *lo, const double *inv) {
    uint32_t k = 0;
    uint32_t q[3];
    for (int d = 0; d < 3; d++) {
        double t = (p[d] - lo[d]) * inv[d];
        t = std::min(std::max(t, 0.0), 1023.0);
        q[d] = (uint32_t)t;
    }
    for (int b = 9; b >= 0; b--)
        for (int d = 0; d < 3; d++) k = (k << 1) | ((q[d] >> b) & 1u);
    return k;
}

// Balanced packing of one tile's records (in element order) into batches of
// at most kFarBatch records whose in-tile columns are all distinct: a record
// goes to the least-filled batch that has room and none of its columns (a new
// batch when none qualifies), starting from ceil(records / kFarBatch)
// batches.  An element shares a node with about a dozen others, so the
// batches come out equal (icosphere subdivision 5: 20 batches of 1024; small
// meshes: at least 13).  Appends the records batch by batch to `out` and the
// batch boundaries (offsets into `out`) to `bptr`.
// The assignment loop of pack_batches with every batch in one word (up to
// 64 batches: the bit sets are single words, no inner loops over words); the
// same choices as the general loop.  False when a 65th batch would be needed.
bool assign_batches_1w(const std::vector<TileRec> &list, int tile_cols, int nb0, HostScratch &scr) {
    if (nb0 > 64) return false;
    std::vector<uint64_t> &used = scr.used, &level = scr.level;
    std::vector<int> &size = scr.size, &batch_of = scr.batch_of;
    used.assign(tile_cols, 0);
    level.assign(kFarBatch + 1, 0);
    size.assign(nb0, 0);
    batch_of.resize(list.size());
    uint64_t *U = used.data(), *L = level.data();
    L[0] = nb0 == 64 ? ~0ull : (1ull << nb0) - 1;
    int low = 0, high = 0, nb = nb0;
    for (size_t r = 0; r < list.size(); r++) {
        const TileRec &rec = list[r];
        uint64_t busy = 0;
        for (int j = 0; j < 3; j++)
            if (rec.slot[j] >= 0) busy |= U[rec.slot[j]];
        int best = -1;
        const int top = std::min(high, kFarBatch - 1);
        for (int s = low; s <= top; s++) {
            const uint64_t m = L[s] & ~busy;
            if (m) {
                best = __builtin_ctzll(m);
                break;
            }
        }
        if (best < 0) {
            best = nb++;
            if (best >= 64) return false;
            size.push_back(0);
            L[0] |= 1ull << best;
            low = 0;
        }
        const int s = size[best]++;
        high = std::max(high, s + 1);
        const uint64_t bit = 1ull << best;
        L[s] &= ~bit;
        L[s + 1] |= bit;
        while (low < kFarBatch && L[low] == 0) low++;
        batch_of[r] = best;
        for (int j = 0; j < 3; j++)
            if (rec.slot[j] >= 0) U[rec.slot[j]] |= bit;
    }
    return true;
}

// The general assignment loop (any number of batches; the bit sets widen
// as batches are added).
void general_assign(const std::vector<TileRec> &list, int tile_cols, int nb0, HostScratch &scr) {
    std::vector<uint64_t> &used = scr.used, &level = scr.level, &busy = scr.busy;
    std::vector<int> &size = scr.size, &batch_of = scr.batch_of;
    int words = std::max(1, (nb0 + 8 + 63) / 64);
    used.assign((size_t)tile_cols * words, 0);
    level.assign((size_t)(kFarBatch + 1) * words, 0);
    size.assign(nb0, 0);
    batch_of.resize(list.size());
    for (int b = 0; b < nb0; b++) level[b / 64] |= 1ull << (b % 64);
    int low = 0, high = 0;   // lowest and highest fill levels holding a batch
    busy.assign(words, 0);
    for (size_t r = 0; r < list.size(); r++) {
        const TileRec &rec = list[r];
        for (int w = 0; w < words; w++) {
            uint64_t u = 0;
            for (int j = 0; j < 3; j++)
                if (rec.slot[j] >= 0) u |= used[(size_t)rec.slot[j] * words + w];
            busy[w] = u;
        }
        int best = -1;
        for (int s = low; s <= std::min(high, kFarBatch - 1) && best < 0; s++)
            for (int w = 0; w < words; w++) {
                const uint64_t m = level[(size_t)s * words + w] & ~busy[w];
                if (m) {
                    best = w * 64 + __builtin_ctzll(m);
                    break;
                }
            }
        if (best < 0) {
            best = (int)size.size();
            size.push_back(0);
            if ((best + 64) / 64 > words) {   // widen the bit sets
                const int nw = words * 2;
                auto widen = [](std::vector<uint64_t> &v, size_t rows, int w0, int w1) {
                    std::vector<uint64_t> v2(rows * w1, 0);
                    for (size_t c = 0; c < rows; c++)
                        for (int w = 0; w < w0; w++) v2[c * w1 + w] = v[c * w0 + w];
                    v.swap(v2);
                };
                widen(used, (size_t)tile_cols, words, nw);
                widen(level, (size_t)kFarBatch + 1, words, nw);
                busy.resize(nw, 0);
                words = nw;
            }
            level[best / 64] |= 1ull << (best % 64);
            low = 0;
        }
        const int s = size[best]++;
        high = std::max(high, s + 1);
        const uint64_t bit = 1ull << (best % 64);
        level[(size_t)s * words + best / 64] &= ~bit;
        level[(size_t)(s + 1) * words + best / 64] |= bit;
        while (low < kFarBatch) {   // advance past emptied levels
            bool any = false;
            for (int w = 0; w < words && !any; w++) any = level[(size_t)low * words + w] != 0;
            if (any) break;
            low++;
        }
        batch_of[r] = best;
        for (int j = 0; j < 3; j++)
            if (rec.slot[j] >= 0) used[(size_t)rec.slot[j] * words + best / 64] |= bit;
    }
}

void pack_batches(const std::vector<TileRec> &list, int tile_cols, std::vector<TileRec> &out,
                  std::vector<int> &bptr, HostScratch &scr) {
    // Bit sets, 64 batches per word: per slot, the batches already holding a
    // record on it (`used`); per fill level s, the batches holding s records
    // (`level`).  A record's allowed batches are the complement of its slots'
    // union; the occupied levels are scanned upward from the lowest, so
    // the first allowed batch found is the least-filled (lowest index among
    // equals) with room, and the fills stay within a few levels of each
    // other: a handful of word operations per record.
    const int nb0 = (int)((list.size() + kFarBatch - 1) / kFarBatch);
    if (!assign_batches_1w(list, tile_cols, nb0, scr)) general_assign(list, tile_cols, nb0, scr);
    const std::vector<int> &size = scr.size, &batch_of = scr.batch_of;
    // stable counting sort of the records by batch
    std::vector<int> &start = scr.start;
    start.assign(size.size() + 1, 0);
    for (size_t b = 0; b < size.size(); b++) start[b + 1] = start[b] + size[b];
    const size_t base = out.size();
    out.resize(base + list.size());
    for (size_t b = 0; b < size.size(); b++) bptr.push_back((int)(base + start[b + 1]));
    for (size_t r = 0; r < list.size(); r++) out[base + start[batch_of[r]]++] = list[r];
}

// Far-kernel launch shapes chosen by the autotuner, per device and problem
// shape (precision, N, R, tile width, tiles, Gauss points), for the process.
using FarTuneKey = std::tuple<int, int, int, int, int, int, int>;
std::mutex g_far_tune_mu;
std::map<FarTuneKey, int> g_far_tuned;

}  // namespace
}  // namespace bem

using namespace bem;

bem_solver_s::bem_solver_s() {
    CUDA_TRY(cudaGetDevice(&device));
    CUDA_TRY(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    if (cusolverDnCreate(&cusolver) != CUSOLVER_STATUS_SUCCESS) BEM_FAIL(BEM_ERR_CUDA, "cusolverDnCreate failed");
    cusolverDnSetStream(cusolver, stream);
    if (cublasCreate(&cublas) != CUBLAS_STATUS_SUCCESS) BEM_FAIL(BEM_ERR_CUDA, "cublasCreate failed");
    cublasSetStream(cublas, stream);
    CUDA_TRY(cudaMallocHost(&h_pinned, 64 * sizeof(double)));
    for (auto &e : ev_res) CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    CUDA_TRY(cudaEventCreateWithFlags(&ev_up, cudaEventDisableTiming));
    bem_options_default(&opt);
}

bem_solver_s::~bem_solver_s() {
    int cur = -1;
    cudaGetDevice(&cur);
    if (cur != device) cudaSetDevice(device);
    if (stream) cudaStreamSynchronize(stream);
    if (cusolver) cusolverDnDestroy(cusolver);
    if (cublas) cublasDestroy(cublas);
    if (h_pinned) cudaFreeHost(h_pinned);
    for (auto &e : ev_res)
        if (e) cudaEventDestroy(e);
    if (ev_up) cudaEventDestroy(ev_up);
    if (h_stage) cudaFreeHost(h_stage);
    if (qr_aux) cudaStreamSynchronize(qr_aux);
    for (auto &e : qr_ev)
        if (e) cudaEventDestroy(e);
    for (auto &e : asm_ev)
        if (e) cudaEventDestroy(e);
    if (qr_aux) cudaStreamDestroy(qr_aux);
    if (stream) cudaStreamDestroy(stream);
    if (cur >= 0 && cur != device) cudaSetDevice(cur);
}

namespace {
// The longest element edge: the largest squared length, one square root.
double longest_edge(int E, const std::vector<double> &h_nodes, const std::vector<int> &h_elems) {
    double m2 = 0.0;
    for (int e = 0; e < E; e++) {
        const double *v[3] = {&h_nodes[3 * (size_t)h_elems[3 * e]], &h_nodes[3 * (size_t)h_elems[3 * e + 1]],
                              &h_nodes[3 * (size_t)h_elems[3 * e + 2]]};
        for (int a = 0; a < 3; a++) {
            const double *p = v[a], *q = v[a == 2 ? 0 : a + 1];
            m2 = std::max(m2, (p[0] - q[0]) * (p[0] - q[0]) + (p[1] - q[1]) * (p[1] - q[1]) +
                                  (p[2] - q[2]) * (p[2] - q[2]));
        }
    }
    return std::sqrt(m2);
}
}  // namespace

void bem_solver_s::set_geometry(const double *pnts, int num_pnts, const int *elems, int num_elems,
                                const double *bc, const double *chief, int num_chief) {
    BEM_HOST_PROF("set_geometry");
    if (tile_future.valid()) tile_future.wait();   // they read h_nodes and h_elems
    if (grid_future.valid()) grid_future.wait();
    BEM_CHECK_ARG(pnts && elems && num_pnts > 0 && num_elems > 0, "empty geometry");
    BEM_CHECK_ARG(num_chief >= 0 && (num_chief == 0 || chief), "bad CHIEF points");
    for (long long i = 0; i < 3LL * num_elems; i++)
        BEM_CHECK_ARG(elems[i] >= 0 && elems[i] < num_pnts, "element node index out of range");
    if (bc)   // checked before any state changes (the default BC has cb = 1)
        for (int e = 0; e < num_elems; e++)
            BEM_CHECK_ARG(bc[6 * (size_t)e + 2] != 0.0 || bc[6 * (size_t)e + 3] != 0.0, "element with cb = 0");
    N = num_pnts;
    E = num_elems;
    M = num_chief;
    R = N + M;
    h_nodes.assign(pnts, pnts + 3 * (size_t)N);
    h_elems.assign(elems, elems + 3 * (size_t)E);
    // The column-tile tables (host work of ~1 ms at 20480 elements) are
    // built on another host thread while this call and the assembly's first
    // steps go on; ensure_tiles takes them.
    host_tiles.cap = -1;   // (its storage is kept for reuse)
    {
        const int cap = opt.tile_cols > 0 ? std::min(opt.tile_cols, kTileColsMax) : kTileColsMax;
        tile_future = std::async(std::launch::async, [this, cap] {
            build_host_tiles(N, E, h_nodes, h_elems, cap, tiles_next, tile_scratch);
        });
    }
    // Nodes, CHIEF points and BCs go up straight from the caller's arrays (no
    // host copy; a pinned caller buffer is a direct DMA) while the host work
    // below goes on; the float head/tail rows and the int4 element table
    // follow from a pinned staging buffer.  The caller's arrays are only read
    // until this call returns.
    if (!bc) {   // the default BC (0, 1, -1) per element, uploaded from here
        h_bc.resize(6 * (size_t)E);
        for (int e = 0; e < E; e++) {
            double d[6] = {0, 0, 1, 0, -1, 0};
            std::memcpy(&h_bc[6 * (size_t)e], d, sizeof(d));
        }
    }
    d_nodes.ensure(sizeof(double) * 3 * N);
    d_rows_d.ensure(sizeof(double) * 3 * (size_t)R);
    d_rows_f.ensure(sizeof(float4) * 2 * (size_t)R);
    d_elems.ensure(sizeof(int4) * E);
    d_bc.ensure(sizeof(double) * 6 * (size_t)E);
    d_geo_f.ensure(sizeof(float4) * kGeoFloat4 * (size_t)E);
    d_geo_d.ensure(sizeof(double) * kGeoDouble * (size_t)E);
    CUDA_TRY(cudaMemcpyAsync(d_nodes.p, pnts, sizeof(double) * 3 * N, cudaMemcpyHostToDevice, stream));
    CUDA_TRY(cudaMemcpyAsync(d_rows_d.p, pnts, sizeof(double) * 3 * N, cudaMemcpyHostToDevice, stream));
    if (M)
        CUDA_TRY(cudaMemcpyAsync(d_rows_d.as<double>() + 3 * (size_t)N, chief, sizeof(double) * 3 * (size_t)M,
                                 cudaMemcpyHostToDevice, stream));
    CUDA_TRY(cudaMemcpyAsync(d_bc.p, bc ? bc : h_bc.data(), sizeof(double) * 6 * (size_t)E, cudaMemcpyHostToDevice,
                             stream));
    // alpha = 0 on every element (bcA = 0: the far kernel forms no G sums
    // for A), and gamma = 0 too (bcC = 0: none for beta either)
    {
        bool a_nz = false, c_nz = !bc;   // the default BC: alpha = 0, gamma = -1
        for (int e = 0; bc && e < E && !a_nz; e++) {
            const double *b = bc + 6 * (size_t)e;
            a_nz = b[0] != 0.0 || b[1] != 0.0;
            c_nz = c_nz || b[4] != 0.0 || b[5] != 0.0;
        }
        g_sums = a_nz ? 2 : c_nz ? 1 : 0;
    }
    h_rows.assign(h_nodes.begin(), h_nodes.end());
    if (M) h_rows.insert(h_rows.end(), chief, chief + 3 * (size_t)M);
    {
        double *lo = row_lo, *hi = row_hi;   // the box of the row points (nodes and CHIEF points)
        for (int d = 0; d < 3; d++) {
            lo[d] = 1e300;
            hi[d] = -1e300;
        }
        for (size_t i = 0; i + 2 < h_rows.size(); i += 3)
            for (int d = 0; d < 3; d++) {
                lo[d] = std::min(lo[d], h_rows[i + d]);
                hi[d] = std::max(hi[d], h_rows[i + d]);
            }
        extent = std::sqrt((hi[0] - lo[0]) * (hi[0] - lo[0]) + (hi[1] - lo[1]) * (hi[1] - lo[1]) +
                           (hi[2] - lo[2]) * (hi[2] - lo[2]));
    }
    // the longest edge and the near-pair grid's host part on another host
    // thread (physics() waits for the edge; ensure_near_list takes the grid
    // when near_eta is still the one it was built for)
    grid_next.eta = -1.0;
    grid_future = std::async(std::launch::async, [this, eta = opt.near_eta] {
        max_edge = longest_edge(E, h_nodes, h_elems);
        build_near_grid(E, h_nodes, h_elems, row_lo, row_hi, max_edge, eta, grid_next, grid_scratch);
    });

    // the float head/tail rows and the int4 element table, staged
    const size_t rf_bytes = sizeof(float4) * 2 * (size_t)R, el_bytes = sizeof(int4) * (size_t)E;
    if (h_stage_bytes < rf_bytes + el_bytes) {
        if (h_stage) CUDA_TRY(cudaFreeHost(h_stage));
        h_stage = nullptr;
        h_stage_bytes = 0;
        CUDA_TRY(cudaMallocHost(&h_stage, rf_bytes + el_bytes));
        h_stage_bytes = rf_bytes + el_bytes;
    }
    float4 *rf = static_cast<float4 *>(h_stage);
    int4 *el = reinterpret_cast<int4 *>(static_cast<unsigned char *>(h_stage) + rf_bytes);
    for (int i = 0; i < R; i++) {
        float hx = (float)h_rows[3 * i], hy = (float)h_rows[3 * i + 1], hz = (float)h_rows[3 * i + 2];
        rf[2 * i] = make_float4(hx, hy, hz, 0.f);
        rf[2 * i + 1] = make_float4((float)(h_rows[3 * i] - hx), (float)(h_rows[3 * i + 1] - hy),
                                    (float)(h_rows[3 * i + 2] - hz), 0.f);
    }
    for (int e = 0; e < E; e++) el[e] = make_int4(h_elems[3 * e], h_elems[3 * e + 1], h_elems[3 * e + 2], 0);
    CUDA_TRY(cudaMemcpyAsync(d_rows_f.p, rf, rf_bytes, cudaMemcpyHostToDevice, stream));
    CUDA_TRY(cudaMemcpyAsync(d_elems.p, el, el_bytes, cudaMemcpyHostToDevice, stream));
    // the element tables for the current near_eta, queued behind the uploads;
    // the call returns once the copies (not the kernel) are done: the
    // caller's arrays and the staging buffer are free again then
    CUDA_TRY(cudaEventRecord(ev_up, stream));
    geo_eta = -1.0;
    ensure_geo();
    CUDA_TRY(cudaEventSynchronize(ev_up));
    tiles[0].valid = tiles[1].valid = false;
    assembled = solved = false;
}

void bem_solver_s::set_sources(const bem_source_t *srcs, int num) {
    BEM_CHECK_ARG(num >= 1 && srcs, "need at least one source");
    for (int i = 0; i < num; i++)
        BEM_CHECK_ARG(srcs[i].kind == BEM_SRC_POINT || srcs[i].kind == BEM_SRC_PLANE, "bad source kind");
    h_srcs.assign(srcs, srcs + num);
    S = num;
    static_assert(sizeof(DevSource) == sizeof(bem_source_t), "source layout");
    d_srcs.ensure(sizeof(bem_source_t) * num);
    CUDA_TRY(cudaMemcpyAsync(d_srcs.p, h_srcs.data(), sizeof(bem_source_t) * num, cudaMemcpyHostToDevice, stream));
    if (assembled) {
        // A does not depend on the sources: only B = p_inc - beta is rebuilt.
        d_B.ensure(sizeof(double2) * (size_t)R * S);
        launch_rhs_from_beta(row_points(), k, d_srcs.as<DevSource>(), S, d_beta.as<double2>(), d_B.as<double2>(),
                             stream);
    }
    CUDA_TRY(cudaStreamSynchronize(stream));
    solved = false;
}

void bem_solver_s::ensure_aux() {
    if (qr_aux) return;
    int least = 0, greatest = 0;
    CUDA_TRY(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    CUDA_TRY(cudaStreamCreateWithPriority(&qr_aux, cudaStreamNonBlocking, greatest));
    for (auto &e : qr_ev) CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    for (auto &e : asm_ev) CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
}

void bem_solver_s::ensure_geo() {
    if (E == 0) BEM_FAIL(BEM_ERR_STATE, "no geometry set");
    if (geo_eta == opt.near_eta) return;
    launch_elem_setup(d_nodes.as<double>(), d_elems.as<int4>(), d_bc.as<double>(), E, opt.near_eta,
                      d_geo_f.as<float4>(), d_geo_d.as<double>(), stream);
    geo_eta = opt.near_eta;
    near_valid = false;
}

// The near-pair list depends on the geometry and near_eta only, so every
// assembly of one geometry (any wavenumber, any sources) reuses it.
void bem_solver_s::ensure_near_list(cudaStream_t st) {
    if (near_valid) return;
    BEM_HOST_PROF("near_list");
    // (the uploads below are from pageable host memory, which the copy
    // stages before it returns: the arrays may be reused right after)
    NearGridHost &gh = near_grid_h;
    if (grid_future.valid()) {
        grid_future.get();
        std::swap(gh, grid_next);
    }
    if (gh.eta != opt.near_eta || gh.start.empty())
        build_near_grid(E, h_nodes, h_elems, row_lo, row_hi, max_edge, opt.near_eta, gh, grid_scratch);
    const double *lo = gh.lo, cell = gh.cell;
    const int *dim = gh.dim;
    const size_t ncell = gh.start.size() - 1;
    const std::vector<int> &start = gh.start, &order = gh.order;
    d_grid_start.ensure(sizeof(int) * (ncell + 1));
    d_grid_elems.ensure(sizeof(int) * std::max(1, E));
    CUDA_TRY(cudaMemcpyAsync(d_grid_start.p, start.data(), sizeof(int) * (ncell + 1), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(d_grid_elems.p, order.data(), sizeof(int) * E, cudaMemcpyHostToDevice, st));
    NearGrid grid{{lo[0], lo[1], lo[2]}, 1.0 / cell, {dim[0], dim[1], dim[2]}, d_grid_start.as<int>(),
                  d_grid_elems.as<int>()};
    d_near_ptr.ensure(sizeof(int) * ((size_t)R + 1));
    launch_near_list(row_points(), N, geo_tables(), grid, nullptr, d_near_ptr.as<int>(), nullptr, st);
    std::vector<int> &cnt = near_cnt_h;
    cnt.resize(R);
    CUDA_TRY(cudaMemcpyAsync(cnt.data(), d_near_ptr.p, sizeof(int) * R, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    std::vector<int> &ptr = near_ptr_h;
    ptr.assign(R + 1, 0);
    for (int r = 0; r < R; r++) {
        if (ptr[r] > 0x7fffffff - cnt[r]) BEM_FAIL(BEM_ERR_TOO_LARGE, "too many near pairs");
        ptr[r + 1] = ptr[r] + cnt[r];
    }
    CUDA_TRY(cudaMemcpyAsync(d_near_ptr.p, ptr.data(), sizeof(int) * (R + 1), cudaMemcpyHostToDevice, st));
    d_near_ids.ensure(sizeof(int) * std::max(1, ptr[R]));
    launch_near_list(row_points(), N, geo_tables(), grid, d_near_ptr.as<int>(), nullptr, d_near_ids.as<int>(), st);
    near_valid = true;
}

// Column tiles of the far-field kernel.  When N fits one tile the columns
// are the nodes in their own order (every row segment is written
// contiguously).  Otherwise the nodes are ordered along a Morton curve and
// cut into equal tiles, and each tile lists every element with a node in it;
// an element straddling tiles is integrated once per tile it touches and
// counted for the c and beta sums only in the tile of its first node.
// Grid of element centroids: cell edge >= the largest near radius (near_eta
// x element diameter) and >= the longest element (vertex pairs), over the box
// of all row points; at most ~4M cells.
void bem::build_near_grid(int E, const std::vector<double> &h_nodes, const std::vector<int> &h_elems, const double *lo,
                          const double *hi, double max_edge, double eta, NearGridHost &g, HostScratch &scr) {
    g.eta = eta;
    double cell = std::max(1.0, eta) * max_edge * 1.01 + 1e-12;
    const double span = std::max({hi[0] - lo[0], hi[1] - lo[1], hi[2] - lo[2], 1e-12});
    cell = std::max(cell, span / 160.0);
    g.cell = cell;
    for (int a = 0; a < 3; a++) {
        g.lo[a] = lo[a];
        g.dim[a] = std::max(1, (int)std::floor((hi[a] - lo[a]) / cell) + 1);
    }
    const size_t ncell = (size_t)g.dim[0] * g.dim[1] * g.dim[2];
    std::vector<int> &cid = scr.cid, &fill = scr.fill;
    cid.resize(E);
    g.start.assign(ncell + 1, 0);
    g.order.resize(E);
    // (the cell size has a 1% margin over the near radius, so binning by a
    // reciprocal instead of a division moves nothing out of a row's 27 cells)
    const double inv = 1.0 / cell, third = 1.0 / 3.0;
    for (int e = 0; e < E; e++) {
        int c[3];
        const double *p0 = &h_nodes[3 * (size_t)h_elems[3 * e]], *p1 = &h_nodes[3 * (size_t)h_elems[3 * e + 1]],
                     *p2 = &h_nodes[3 * (size_t)h_elems[3 * e + 2]];
        for (int a = 0; a < 3; a++) {
            const double m = (p0[a] + p1[a] + p2[a]) * third;
            c[a] = std::min(std::max((int)std::floor((m - lo[a]) * inv), 0), g.dim[a] - 1);
        }
        cid[e] = (int)(((size_t)c[2] * g.dim[1] + c[1]) * g.dim[0] + c[0]);
        g.start[cid[e] + 1]++;
    }
    for (size_t c = 0; c < ncell; c++) g.start[c + 1] += g.start[c];
    fill.assign(g.start.begin(), g.start.end() - 1);
    for (int e = 0; e < E; e++) g.order[fill[cid[e]]++] = e;   // increasing e within a cell
}

void bem::build_host_tiles(int N, int E, const std::vector<double> &h_nodes, const std::vector<int> &h_elems,
                           int cap, HostTiles &out, HostScratch &scr) {
    out.cap = cap;
    int ntiles = (N + cap - 1) / cap;
    int per = (N + ntiles - 1) / ntiles;
    std::vector<int> &order = scr.order;
    order.resize(N);
    std::iota(order.begin(), order.end(), 0);
    if (ntiles > 1) {
        double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300}, inv[3];
        for (int i = 0; i < N; i++)
            for (int d = 0; d < 3; d++) {
                lo[d] = std::min(lo[d], h_nodes[3 * i + d]);
                hi[d] = std::max(hi[d], h_nodes[3 * i + d]);
            }
        for (int d = 0; d < 3; d++) inv[d] = hi[d] > lo[d] ? 1023.0 / (hi[d] - lo[d]) : 0.0;
        std::vector<uint32_t> &key = scr.key;
        key.resize(N);
        for (int i = 0; i < N; i++) key[i] = morton_key(&h_nodes[3 * i], lo, inv);
        std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return key[a] < key[b]; });
    }
    std::vector<int> &tile_of = scr.tile_of, &slot_of = scr.slot_of;
    tile_of.resize(N);
    slot_of.resize(N);
    std::vector<int> &cols = out.cols, &cnt = out.cnt;
    cols.assign((size_t)ntiles * per, 0);
    cnt.assign(ntiles, 0);
    for (int i = 0; i < N; i++) {
        int t = i / per, s = i - t * per;
        tile_of[order[i]] = t;
        slot_of[order[i]] = s;
        cols[(size_t)t * per + s] = order[i];
        cnt[t]++;
    }
    std::vector<std::vector<TileRec>> &lists = scr.lists;
    if ((int)lists.size() < ntiles) lists.resize(ntiles);
    for (int t = 0; t < ntiles; t++) lists[t].clear();
    if (ntiles == 1) lists[0].reserve(E);
    for (int e = 0; e < E; e++) {
        const int *nd = &h_elems[3 * (size_t)e];
        int seen[3] = {-1, -1, -1}, ns = 0;
        for (int j = 0; j < 3; j++) {
            int t = tile_of[nd[j]];
            bool dup = false;
            for (int q = 0; q < ns; q++) dup |= seen[q] == t;
            if (dup) continue;
            seen[ns++] = t;
            TileRec r;
            r.eid = e;
            for (int q = 0; q < 3; q++) {
                r.node[q] = nd[q];
                r.slot[q] = tile_of[nd[q]] == t ? slot_of[nd[q]] : -1;
            }
            r.owner = (t == tile_of[nd[0]]) ? 1 : 0;
            lists[t].push_back(r);
        }
    }
    std::vector<TileRec> &recs = out.recs;
    std::vector<int> &ptr = out.ptr;
    recs.clear();
    ptr.assign(ntiles + 1, 0);
    out.bptr.assign(1, 0);
    out.tbatch.assign(ntiles + 1, 0);
    recs.reserve(lists[0].size() * ntiles);
    for (int t = 0; t < ntiles; t++) {
        pack_batches(lists[t], per, recs, out.bptr, scr);
        ptr[t + 1] = (int)recs.size();
        out.tbatch[t + 1] = (int)out.bptr.size() - 1;
    }
    out.ntiles = ntiles;
    out.per = per;
}

void bem_solver_s::ensure_tiles(int precision) {
    Tiles &T = tiles[precision];
    if (T.valid) return;
    BEM_HOST_PROF("tiles");
    const int cap = opt.tile_cols > 0 ? std::min(opt.tile_cols, kTileColsMax) : kTileColsMax;
    // the host tables, built beside set_geometry when the column cap matches
    if (tile_future.valid()) {
        tile_future.get();
        std::swap(host_tiles, tiles_next);
    }
    if (host_tiles.cap != cap || host_tiles.ptr.empty())
        build_host_tiles(N, E, h_nodes, h_elems, cap, host_tiles, tile_scratch);
    const HostTiles &ht = host_tiles;
    const std::vector<TileRec> &recs = ht.recs;
    const std::vector<int> &ptr = ht.ptr, &cols = ht.cols, &cnt = ht.cnt;
    const int ntiles = ht.ntiles, per = ht.per;
    T.recs.ensure(sizeof(TileRec) * recs.size());
    T.rec_ptr.ensure(sizeof(int) * ptr.size());
    T.cols.ensure(sizeof(int) * cols.size());
    T.col_cnt.ensure(sizeof(int) * cnt.size());
    T.batch_ptr.ensure(sizeof(int) * ht.bptr.size());
    T.tile_batch.ensure(sizeof(int) * ht.tbatch.size());
    CUDA_TRY(cudaMemcpyAsync(T.batch_ptr.p, ht.bptr.data(), sizeof(int) * ht.bptr.size(), cudaMemcpyHostToDevice,
                             stream));
    CUDA_TRY(cudaMemcpyAsync(T.tile_batch.p, ht.tbatch.data(), sizeof(int) * ht.tbatch.size(),
                             cudaMemcpyHostToDevice, stream));
    CUDA_TRY(cudaMemcpyAsync(T.recs.p, recs.data(), sizeof(TileRec) * recs.size(), cudaMemcpyHostToDevice, stream));
    CUDA_TRY(cudaMemcpyAsync(T.rec_ptr.p, ptr.data(), sizeof(int) * ptr.size(), cudaMemcpyHostToDevice, stream));
    CUDA_TRY(cudaMemcpyAsync(T.cols.p, cols.data(), sizeof(int) * cols.size(), cudaMemcpyHostToDevice, stream));
    CUDA_TRY(cudaMemcpyAsync(T.col_cnt.p, cnt.data(), sizeof(int) * cnt.size(), cudaMemcpyHostToDevice, stream));
    CUDA_TRY(cudaStreamSynchronize(stream));
    T.ntiles = ntiles;
    T.tc_max = per;
    T.nrec = (int)recs.size();
    T.valid = true;
}

GeoTables bem_solver_s::geo_tables() const {
    return GeoTables{d_geo_f.as<float4>(), d_geo_d.as<double>(), d_elems.as<int4>(), E};
}

RowPoints bem_solver_s::row_points() const { return RowPoints{d_rows_f.as<float4>(), d_rows_d.as<double>(), R}; }

Physics bem_solver_s::physics() const {
    if (grid_future.valid()) grid_future.wait();   // max_edge is formed by set_geometry's grid task
    return Physics{k, opt.density * k * opt.speed, opt.near_depth, opt.near_eta, max_edge, extent, g_sums};
}

void bem_solver_s::assemble(double kk, int precision) {
    BEM_HOST_PROF("assemble");
    BEM_CHECK_ARG(precision == BEM_PREC_C64 || precision == BEM_PREC_C128, "bad precision");
    BEM_CHECK_ARG(std::isfinite(kk) && kk > 0, "wavenumber must be positive");
    if (E == 0) BEM_FAIL(BEM_ERR_STATE, "no geometry set");
    if (S == 0) BEM_FAIL(BEM_ERR_STATE, "no sources set");
    ensure_quadrature(opt.order);
    ensure_geo();
    // The near-pair list (two small kernels and a read-back of the per-row
    // counts) is built on the handle's second, high-priority stream while the
    // far kernel runs: that stream starts after the element tables, and the
    // near kernel waits for the list.
    const bool near_build = !near_valid;
    if (near_build) {
        ensure_aux();
        CUDA_TRY(cudaEventRecord(asm_ev[0], stream));
    }
    ensure_tiles(precision);
    k = kk;
    prec = precision;
    Tiles &T = tiles[precision];
    size_t esz = precision == BEM_PREC_C64 ? sizeof(float2) : sizeof(double2);
    size_t rsz = precision == BEM_PREC_C64 ? sizeof(float) : sizeof(double);
    lda = round_up(N, 8);
    d_A.ensure(esz * lda * (size_t)R);
    d_B.ensure(sizeof(double2) * (size_t)R * S);
    d_cpart.ensure(rsz * (size_t)T.ntiles * R);
    d_bpart.ensure(2 * rsz * (size_t)T.ntiles * R);
    d_status.ensure(4 * sizeof(int));
    CUDA_TRY(cudaMemsetAsync(d_status.as<int>() + 2, 0, sizeof(int), stream));
    const FarRec *frecs = nullptr;
    if (precision == BEM_PREC_C64) {
        // the records with their elements' geometry in record order (the
        // geometry depends on near_eta as well as the mesh: formed every time)
        T.frecs.ensure(sizeof(FarRec) * (size_t)std::max(1, T.nrec));
        launch_far_recs(T.recs.as<TileRec>(), T.nrec, d_geo_f.as<float4>(), T.frecs.as<FarRec>(), stream);
        frecs = T.frecs.as<FarRec>();
    }
    TileSet ts{T.recs.as<TileRec>(), T.rec_ptr.as<int>(), T.batch_ptr.as<int>(), T.tile_batch.as<int>(),
               d_status.as<int>() + 2, T.cols.as<int>(), T.col_cnt.as<int>(), T.ntiles, T.tc_max, frecs};
    Physics ph = physics();
    int variant = opt.far_variant;
    bool done = false;
    if (variant < 0) {
        variant = 0;
        const FarTuneKey key{device, precision, N, R, T.tc_max, T.ntiles, quadrature_points()};
        int cached = -1;
        {
            std::lock_guard<std::mutex> lk(g_far_tune_mu);
            auto it = g_far_tuned.find(key);
            if (it != g_far_tuned.end()) cached = it->second;
        }
        if (cached >= 0) {
            variant = cached;
        } else if (far_variants(precision) > 1) {
            // Autotune: time every launch shape that fits (twice, keep the
            // minimum; once when a launch takes over 20 ms) on this very
            // assembly; the last launch leaves a complete far-field A, so no
            // extra launch is needed afterwards when it is the chosen shape.
            // The result is shared by every solver of the process on this
            // device (the request server's slots tune a problem shape once).
            cudaEvent_t e0, e1;
            CUDA_TRY(cudaEventCreate(&e0));
            CUDA_TRY(cudaEventCreate(&e1));
            float best = 1e30f;
            int last = -1, reps = 2;
            for (int v = 0; v < far_variants(precision); v++) {
                if (!far_variant_fits(precision, T.tc_max, v)) continue;
                last = v;
                for (int rep = 0; rep < reps; rep++) {
                    CUDA_TRY(cudaEventRecord(e0, stream));
                    launch_far_assembly(precision, row_points(), N, geo_tables(), ts, ph, d_A.p, lda,
                                        d_cpart.p, d_bpart.p, stream, v);
                    CUDA_TRY(cudaEventRecord(e1, stream));
                    CUDA_TRY(cudaEventSynchronize(e1));
                    float ms = 0.f;
                    CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
                    if (ms < best) { best = ms; variant = v; }
                    if (ms > 20.f) reps = 1;
                }
            }
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            {
                std::lock_guard<std::mutex> lk(g_far_tune_mu);
                g_far_tuned.emplace(key, variant);   // a concurrent tuner's entry stays if it came first
                variant = g_far_tuned[key];
            }
            // The shapes split the c and beta row sums differently (FP32 order),
            // so the matrix is left by the chosen shape: every assembly of this
            // problem shape then gives the same bits.
            done = last == variant;
        }
    }
    if (!done)
        launch_far_assembly(precision, row_points(), N, geo_tables(), ts, ph, d_A.p, lda, d_cpart.p, d_bpart.p,
                            stream, variant);
    far_variant_used = variant;
    if (near_build) {
        CUDA_TRY(cudaStreamWaitEvent(qr_aux, asm_ev[0], 0));
        ensure_near_list(qr_aux);
        CUDA_TRY(cudaEventRecord(asm_ev[1], qr_aux));
        CUDA_TRY(cudaStreamWaitEvent(stream, asm_ev[1], 0));
    }
    d_beta.ensure(sizeof(double2) * (size_t)R);
    launch_near_assembly(precision, row_points(), N, geo_tables(), ph, d_A.p, lda, d_cpart.p, d_bpart.p,
                         T.ntiles, d_srcs.as<DevSource>(), S, d_B.as<double2>(), d_beta.as<double2>(),
                         d_near_ptr.as<int>(), d_near_ids.as<int>(), stream);
    assembled = true;
    solved = false;
    tf32_split_mode = -1;
    tc_scale_valid = false;
}

void bem_solver_s::solve(int method, bem_solve_info_t *info) {
    if (!assembled) BEM_FAIL(BEM_ERR_STATE, "solve before assemble");
    BEM_CHECK_ARG(R >= N, "fewer rows than unknowns");
    d_x.ensure(sizeof(double2) * (size_t)N * S);
    if (method == BEM_SOLVE_QR) {
        solve_qr();
        if (info) { info->iterations = 0; info->refinements = 0; info->rel_residual = 0; info->converged = 1; }
    } else if (method == BEM_SOLVE_GMRES_REFINED) {
        if (prec != BEM_PREC_C64) BEM_FAIL(BEM_ERR_STATE, "refined GMRES needs a c64 assembly");
        solve_refined(info);
    } else if (method == BEM_SOLVE_BLOCK_GMRES) {
        if (prec != BEM_PREC_C64) BEM_FAIL(BEM_ERR_STATE, "block GMRES needs a c64 assembly");
        solve_block(info);
    } else if (method == BEM_SOLVE_QR_TC) {
        solve_qr_tc(info);
    } else {
        BEM_FAIL(BEM_ERR_INVALID_ARG, "unknown solve method");
    }
    // a bounded wait of the assembly's far kernel that timed out (status word 2)
    int far_status = 0;
    CUDA_TRY(cudaMemcpyAsync(&far_status, d_status.as<int>() + 2, sizeof(int), cudaMemcpyDeviceToHost, stream));
    CUDA_TRY(cudaStreamSynchronize(stream));
    if (far_status) BEM_FAIL(BEM_ERR_TIMEOUT, "assembly: a bounded wait of the far-field kernel timed out");
    solved = true;
}

void bem_solver_s::get_solution(void *x, int ldx, int precision) {
    if (!solved) BEM_FAIL(BEM_ERR_STATE, "no solution");
    BEM_CHECK_ARG(x && ldx >= N, "bad solution buffer");
    std::vector<double2> h((size_t)N * S);
    CUDA_TRY(cudaMemcpyAsync(h.data(), d_x.p, sizeof(double2) * h.size(), cudaMemcpyDeviceToHost, stream));
    CUDA_TRY(cudaStreamSynchronize(stream));
    for (int s = 0; s < S; s++)
        for (int i = 0; i < N; i++) {
            double2 v = h[(size_t)s * N + i];
            if (precision == BEM_PREC_C64) {
                ((float *)x)[2 * ((size_t)s * ldx + i)] = (float)v.x;
                ((float *)x)[2 * ((size_t)s * ldx + i) + 1] = (float)v.y;
            } else {
                ((double *)x)[2 * ((size_t)s * ldx + i)] = v.x;
                ((double *)x)[2 * ((size_t)s * ldx + i) + 1] = v.y;
            }
        }
}

void bem_solver_s::get_system(void *A, int lda_out, void *B, int ldb_out, int precision) {
    if (!assembled) BEM_FAIL(BEM_ERR_STATE, "no system assembled");
    BEM_CHECK_ARG(precision == BEM_PREC_C64 || precision == BEM_PREC_C128, "bad precision");
    size_t esz = precision == BEM_PREC_C64 ? sizeof(float2) : sizeof(double2);
    if (A) {
        BEM_CHECK_ARG(lda_out >= R, "lda smaller than N+M");
        q_A.ensure(esz * (size_t)R * N);
        launch_to_colmajor(prec, d_A.p, lda, R, N, precision, q_A.p, R, stream);
        CUDA_TRY(cudaMemcpy2DAsync(A, esz * lda_out, q_A.p, esz * R, esz * R, N, cudaMemcpyDeviceToHost, stream));
    }
    if (B) {
        BEM_CHECK_ARG(ldb_out >= R, "ldb smaller than N+M");
        std::vector<double2> hb((size_t)R * S);
        CUDA_TRY(cudaMemcpyAsync(hb.data(), d_B.p, sizeof(double2) * hb.size(), cudaMemcpyDeviceToHost, stream));
        CUDA_TRY(cudaStreamSynchronize(stream));
        for (int s = 0; s < S; s++)
            for (int r = 0; r < R; r++) {
                double2 v = hb[(size_t)s * R + r];
                if (precision == BEM_PREC_C64) {
                    ((float *)B)[2 * ((size_t)s * ldb_out + r)] = (float)v.x;
                    ((float *)B)[2 * ((size_t)s * ldb_out + r) + 1] = (float)v.y;
                } else {
                    ((double *)B)[2 * ((size_t)s * ldb_out + r)] = v.x;
                    ((double *)B)[2 * ((size_t)s * ldb_out + r) + 1] = v.y;
                }
            }
    }
    CUDA_TRY(cudaStreamSynchronize(stream));
}

size_t bem_solver_s::device_bytes() const {
    const DevMem *all[] = {&d_nodes, &d_rows_f, &d_rows_d, &d_elems, &d_bc, &d_geo_f, &d_geo_d, &d_srcs,
                           &tiles[0].recs, &tiles[0].rec_ptr, &tiles[0].cols, &tiles[0].col_cnt,
                           &tiles[0].batch_ptr, &tiles[0].tile_batch,
                           &tiles[1].recs, &tiles[1].rec_ptr, &tiles[1].cols, &tiles[1].col_cnt,
                           &tiles[1].batch_ptr, &tiles[1].tile_batch,
                           &d_A, &d_B, &d_cpart, &d_bpart, &d_x, &d_beta, &d_near_ptr, &d_near_ids, &d_grid_start, &d_grid_elems,
                           &w_V, &w_H, &w_cs, &w_sn, &w_g, &w_y, &w_h1, &w_h2, &w_w, &w_t, &w_r, &w_gv, &w_vf,
                           &w_part, &w_scal, &x_Ahi, &x_Alo, &x_vlo, &x_tlo, &w_d, &w_ap, &tc_scale, &d_status, &q_A, &q_B, &q_tau, &q_work, &q_info,
                           &qt_v, &qt_vrr, &qt_t, &qt_z, &qt_opv, &qt_opw, &qt_part, &qt_scal,
                           &f_rows_f, &f_rows_d, &f_part, &f_near, &f_out, &f_u};
    size_t b = 0;
    for (const DevMem *d : all) b += d->bytes;
    return b;
}

size_t bem_solver_s::estimate_bytes(int N, int E, int M, int S, int method, const bem_options_t &o) {
    const size_t n = (size_t)N, e = (size_t)E, r = (size_t)N + (size_t)M, s = (size_t)S;
    const size_t lda = (n + 7) / 8 * 8;
    const size_t ntiles = N <= kTileColsMax ? 1 : (n + kTileColsMax - 1) / kTileColsMax;
    size_t b = 0;
    b += 24 * n + 24 * r + 32 * r + 16 * e + 48 * e;                  // nodes, rows, elements, bc
    b += sizeof(float4) * kGeoFloat4 * e + sizeof(double) * kGeoDouble * e;
    b += 3 * e * (sizeof(TileRec) + sizeof(FarRec)) + 4 * (ntiles + 1) + 4 * n + 4 * ntiles;   // <= 3 tiles per element
    b += 4 * (3 * e + 2 * ntiles + 2);                                     // record batches (>= 1 record each)
    b += 4 * (r + 1) + 256 * r + 4 * e + (16u << 20);                       // near-pair list and search grid
    b += 8 * lda * r + 16 * r * s + 12 * ntiles * r + 16 * n * s + 16 * r + 48 * s;
    if (method == BEM_SOLVE_BLOCK_GMRES) {
        const size_t m = (size_t)std::max(1, std::min(o.max_iter, 200));
        b += 16 * n * s * (m + 1) + 16 * s * m * (m + 1) + 16 * s * (4 * m + 4);
        b += 16 * n * s * 2 + 16 * r * s + 16 * n * s + 8 * r * s + 16 * n * s + 40 * s + 16 * n * s;
        size_t extra = 0;   // the largest of the candidate modes' buffers
        for (const int gm : block_gemm_candidates(o, S, (int)r, N)) {
            if (gm == BEM_GEMM_TF32X3) extra = std::max(extra, 16 * lda * r + 48 * n * s + 16 * r * s);
            if (gm == BEM_GEMM_TF32X3_3M) extra = std::max(extra, 24 * lda * r + 48 * std::max(n, r) * s);
            if (gm == BEM_GEMM_SIMT) extra = std::max(extra, 4 * block_simt_scratch_floats((int)r, N, S));
            if (gm == BEM_GEMM_TC) {
                // the packed right-hand operand and the split-K partial sums of
                // the four products as the launch plans them on this device
                size_t pf = 0;
                for (const int P : {2, 3})
                    pf = std::max({pf, tc_gemm_part_floats((int)r, 2 * N, 2 * S, P),
                                   tc_gemm_part_floats(2 * N, (int)r, 2 * S, P)});
                extra = std::max(extra, tc_operand_bytes((int)std::max(2 * n, r), 2 * S, 3) + 4 * pf + 64);
            }
        }
        b += extra;
    } else if (method == BEM_SOLVE_GMRES_REFINED) {
        const size_t m = (size_t)std::max(1, o.max_iter);
        b += 2 * 16 * n * (m + 1) + 16 * (m + 1) * m + 16 * 6 * (m + 1);   // the basis in FP64 and double float
        b += 16 * n * 2 + 8 * r + 16 * r + 16 * std::max(n, r);
        b += 16 * n * (size_t)std::max(gemv_h_splits((int)r, N), gemv_h_f64_splits((int)r, N)) + 64;
        b += 8 * n * (size_t)std::max(0, normal_op_clusters(N) - 2 * gemv_h_splits((int)r, N));
        b += 48 * (m + 1) * 160;                                                     // Arnoldi step partials
    } else if (method == BEM_SOLVE_QR_TC) {
        const size_t nb = 128, rp = r + 1;
        b += 8 * (rp * (n + s) + 8) + 8 * n;                                     // [A | B] c64, taus
        b += 2 * (8 * rp * nb + 4 * 2 * r * 256 + 8 * nb * nb + 8 * nb * nb);  // V, Vrr, T, G: per panel parity
        b += 2 * (4 * 2 * nb * (n + s) + tc_operand_bytes((int)(2 * r), (int)(2 * nb), 2) +
                  tc_operand_bytes((int)(2 * nb), (int)(n + s), 2) +
                  4 * tc_gemm_part_floats_bound((int)(2 * r), (int)(n + s))) + 4096;   // per update set
        b += 16 * r + 16 * n + 8 * (2 * std::max(n, r) + 2) +
             16 * n * (size_t)std::max(gemv_h_splits((int)r, N), gemv_h_f64_splits((int)r, N));
        b += 8 * (n + 64) * 64;                                              // diagonal-block inverses
    } else {
        b += 8 * r * n + 8 * r * s + 64 * n + (64u << 20);               // QR copy, tau, library workspace
    }
    return b + b / 16 + (8u << 20);
}
