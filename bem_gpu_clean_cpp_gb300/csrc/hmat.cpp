// Block partition of the collocation matrix for a hierarchical (H-matrix)
// representation: the first stage of a compressed operator for meshes whose
// dense A no longer fits in device memory.  No reference counterpart (the
// reference stores A dense, mesh.cu:985-1006 and atomicFuncs.cu:218-298).
//
// The row points (collocation nodes, then CHIEF points) and the column points
// (the nodes) are each clustered by bisection: a cluster's bounding box is
// split at the median along its longest axis until a cluster holds at most
// `leaf` points.  The block tree then pairs a row cluster I with a column
// cluster J and stops at
//   * an admissible block, min(diam I, diam J) <= eta * dist(I, J) with
//     dist > 0 (diameters and distance of the bounding boxes): the kernel is
//     smooth on I x J, so the block is stored in low rank;
//   * an inadmissible block of two leaves: stored dense;
// and otherwise splits every non-leaf cluster of the pair.  The clustered
// order makes every cluster a contiguous range of positions.
#include <algorithm>
#include <array>
#include <cmath>
#include <vector>

#include "bem_common.h"

namespace bem {
namespace {

struct Cluster {
    int begin, count;
    double lo[3], hi[3];
    int child[2];
};

struct ClusterTree {
    const double *p = nullptr;   // points, 3 doubles each
    std::vector<int> perm;       // position -> original index
    std::vector<Cluster> nodes;  // nodes[0] is the root
};

// Bisection of positions [begin, begin + count); returns the node's index.
int build_cluster(ClusterTree &t, int begin, int count, int leaf) {
    Cluster c{begin, count, {HUGE_VAL, HUGE_VAL, HUGE_VAL}, {-HUGE_VAL, -HUGE_VAL, -HUGE_VAL}, {-1, -1}};
    for (int q = begin; q < begin + count; q++) {
        const double *x = t.p + 3 * (size_t)t.perm[q];
        for (int d = 0; d < 3; d++) {
            c.lo[d] = std::min(c.lo[d], x[d]);
            c.hi[d] = std::max(c.hi[d], x[d]);
        }
    }
    const int id = (int)t.nodes.size();
    t.nodes.push_back(c);
    int ax = 0;
    for (int d = 1; d < 3; d++)
        if (c.hi[d] - c.lo[d] > c.hi[ax] - c.lo[ax]) ax = d;
    // A box of zero extent (coincident points) cannot be split: it stays a leaf.
    if (count > leaf && c.hi[ax] > c.lo[ax]) {
        const int half = count / 2;
        auto first = t.perm.begin() + begin;
        const double *p = t.p;
        // (coordinate, index) is a strict total order: the split is the same
        // on every platform.
        std::nth_element(first, first + half, first + count, [p, ax](int a, int b) {
            const double xa = p[3 * (size_t)a + ax], xb = p[3 * (size_t)b + ax];
            return xa < xb || (xa == xb && a < b);
        });
        const int l = build_cluster(t, begin, half, leaf);
        const int r = build_cluster(t, begin + half, count - half, leaf);
        t.nodes[id].child[0] = l;
        t.nodes[id].child[1] = r;
    } else {
        std::sort(t.perm.begin() + begin, t.perm.begin() + begin + count);
    }
    return id;
}

void build_tree(ClusterTree &t, const double *p, int n, int leaf) {
    t.p = p;
    t.perm.resize(n);
    for (int i = 0; i < n; i++) t.perm[i] = i;
    t.nodes.clear();
    t.nodes.reserve(4 * (size_t)(n / std::max(leaf, 1) + 1));
    build_cluster(t, 0, n, leaf);
}

double diameter(const Cluster &c) {
    double s = 0.0;
    for (int d = 0; d < 3; d++) s += (c.hi[d] - c.lo[d]) * (c.hi[d] - c.lo[d]);
    return std::sqrt(s);
}

double box_distance(const Cluster &a, const Cluster &b) {
    double s = 0.0;
    for (int d = 0; d < 3; d++) {
        const double g = std::max({0.0, b.lo[d] - a.hi[d], a.lo[d] - b.hi[d]});
        s += g * g;
    }
    return std::sqrt(s);
}

void build_blocks(const ClusterTree &rt, int i, const ClusterTree &ct, int j, double eta,
                  std::vector<std::array<int, 5>> &out) {
    const Cluster &a = rt.nodes[i], &b = ct.nodes[j];
    const double dist = box_distance(a, b);
    if (dist > 0.0 && std::min(diameter(a), diameter(b)) <= eta * dist) {
        out.push_back({a.begin, a.count, b.begin, b.count, 1});
        return;
    }
    const bool la = a.child[0] < 0, lb = b.child[0] < 0;
    if (la && lb) {
        out.push_back({a.begin, a.count, b.begin, b.count, 0});
        return;
    }
    const int *ca = a.child, *cb = b.child;
    if (!la && !lb) {
        for (int x = 0; x < 2; x++)
            for (int y = 0; y < 2; y++) build_blocks(rt, ca[x], ct, cb[y], eta, out);
    } else if (la) {
        for (int y = 0; y < 2; y++) build_blocks(rt, i, ct, cb[y], eta, out);
    } else {
        for (int x = 0; x < 2; x++) build_blocks(rt, ca[x], ct, j, eta, out);
    }
}

// Row tree of a collocation system: a root over the nodes' tree (the column
// tree itself, so row position p < N is column position p) and the CHIEF
// points' tree, whose positions follow at N.
void system_row_tree(const ClusterTree &nodes, const ClusterTree &chief, int N, ClusterTree &rt) {
    rt.p = nullptr;
    rt.perm = nodes.perm;
    for (int i : chief.perm) rt.perm.push_back(N + i);
    rt.nodes.clear();
    Cluster root = nodes.nodes[0];
    const Cluster &cr = chief.nodes[0];
    for (int d = 0; d < 3; d++) {
        root.lo[d] = std::min(root.lo[d], cr.lo[d]);
        root.hi[d] = std::max(root.hi[d], cr.hi[d]);
    }
    const int off_n = 1, off_c = 1 + (int)nodes.nodes.size();
    root.begin = 0;
    root.count = N + cr.count;
    root.child[0] = off_n;
    root.child[1] = off_c;
    rt.nodes.push_back(root);
    for (Cluster c : nodes.nodes) {
        for (int &ch : c.child)
            if (ch >= 0) ch += off_n;
        rt.nodes.push_back(c);
    }
    for (Cluster c : chief.nodes) {
        c.begin += N;
        for (int &ch : c.child)
            if (ch >= 0) ch += off_c;
        rt.nodes.push_back(c);
    }
}

}  // namespace
}  // namespace bem

extern "C" int bem_hmat_partition(const double *rows, int num_rows, const double *cols, int num_cols, int leaf,
                                  double eta, int *row_perm, int *col_perm, int *blocks, int max_blocks,
                                  int *num_blocks) {
    BEM_API_BEGIN
    BEM_CHECK_ARG(rows && cols && num_blocks, "null argument");
    BEM_CHECK_ARG(num_rows > 0 && num_cols > 0, "empty point set");
    BEM_CHECK_ARG(leaf >= 1, "leaf size must be at least 1");
    BEM_CHECK_ARG(std::isfinite(eta) && eta > 0.0, "eta must be positive and finite");
    for (long long q = 0; q < 3LL * num_rows; q++) BEM_CHECK_ARG(std::isfinite(rows[q]), "row point not finite");
    for (long long q = 0; q < 3LL * num_cols; q++) BEM_CHECK_ARG(std::isfinite(cols[q]), "column point not finite");
    bem::ClusterTree rt, ct;
    bem::build_tree(rt, rows, num_rows, leaf);
    bem::build_tree(ct, cols, num_cols, leaf);
    std::vector<std::array<int, 5>> out;
    bem::build_blocks(rt, 0, ct, 0, eta, out);
    *num_blocks = (int)out.size();
    if (row_perm) std::copy(rt.perm.begin(), rt.perm.end(), row_perm);
    if (col_perm) std::copy(ct.perm.begin(), ct.perm.end(), col_perm);
    if (blocks) {
        if (max_blocks < (int)out.size())
            BEM_FAIL(BEM_ERR_TOO_LARGE, "block array holds fewer entries than the partition has blocks");
        for (size_t q = 0; q < out.size(); q++)
            std::copy(out[q].begin(), out[q].end(), blocks + 5 * q);
    }
    BEM_API_END
}

extern "C" int bem_hmat_partition_system(const double *pnts, int num_pnts, const double *chief, int num_chief,
                                         int leaf, double eta, int *node_perm, int *chief_perm, int *blocks,
                                         int max_blocks, int *num_blocks) {
    BEM_API_BEGIN
    BEM_CHECK_ARG(pnts && num_blocks && (chief || num_chief == 0), "null argument");
    BEM_CHECK_ARG(num_pnts > 0 && num_chief >= 0, "empty point set");
    BEM_CHECK_ARG(leaf >= 1, "leaf size must be at least 1");
    BEM_CHECK_ARG(std::isfinite(eta) && eta > 0.0, "eta must be positive and finite");
    for (long long q = 0; q < 3LL * num_pnts; q++) BEM_CHECK_ARG(std::isfinite(pnts[q]), "node not finite");
    for (long long q = 0; q < 3LL * num_chief; q++) BEM_CHECK_ARG(std::isfinite(chief[q]), "CHIEF point not finite");
    bem::ClusterTree ct, cht, rt;
    bem::build_tree(ct, pnts, num_pnts, leaf);
    std::vector<std::array<int, 5>> out;
    if (num_chief > 0) {
        bem::build_tree(cht, chief, num_chief, leaf);
        bem::system_row_tree(ct, cht, num_pnts, rt);
        // node rows against the node tree level by level, then the CHIEF rows
        bem::build_blocks(rt, rt.nodes[0].child[0], ct, 0, eta, out);
        bem::build_blocks(rt, rt.nodes[0].child[1], ct, 0, eta, out);
    } else {
        bem::build_blocks(ct, 0, ct, 0, eta, out);
    }
    *num_blocks = (int)out.size();
    if (node_perm) std::copy(ct.perm.begin(), ct.perm.end(), node_perm);
    if (chief_perm && num_chief > 0) std::copy(cht.perm.begin(), cht.perm.end(), chief_perm);
    if (blocks) {
        if (max_blocks < (int)out.size())
            BEM_FAIL(BEM_ERR_TOO_LARGE, "block array holds fewer entries than the partition has blocks");
        for (size_t q = 0; q < out.size(); q++)
            std::copy(out[q].begin(), out[q].end(), blocks + 5 * q);
    }
    BEM_API_END
}
