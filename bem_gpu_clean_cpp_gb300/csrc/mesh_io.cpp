// Mesh ingestion beyond OBJ: PLY (ASCII and binary, either byte order) and a
// winding check and repair.  The reference reads OBJ only (mesh.cu:1215-1265)
// and trusts the file's winding; its meshes ship as PLY too (Head_20kHz_iso.ply)
// and a mesh with mixed winding silently gives a wrong system.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <deque>
#include <fstream>
#include <sstream>
#include <string>
#include <unordered_map>
#include <vector>

#include "mesh.h"

namespace bem {
namespace {

enum PlyType { kI8, kU8, kI16, kU16, kI32, kU32, kF32, kF64, kBad };

PlyType ply_type(const std::string &t) {
    if (t == "char" || t == "int8") return kI8;
    if (t == "uchar" || t == "uint8") return kU8;
    if (t == "short" || t == "int16") return kI16;
    if (t == "ushort" || t == "uint16") return kU16;
    if (t == "int" || t == "int32") return kI32;
    if (t == "uint" || t == "uint32") return kU32;
    if (t == "float" || t == "float32") return kF32;
    if (t == "double" || t == "float64") return kF64;
    return kBad;
}

int ply_size(PlyType t) {
    switch (t) {
        case kI8: case kU8: return 1;
        case kI16: case kU16: return 2;
        case kI32: case kU32: case kF32: return 4;
        case kF64: return 8;
        default: return 0;
    }
}

struct PlyProp {
    std::string name;
    PlyType type = kBad;
    bool list = false;
    PlyType count_type = kBad;
};

struct PlyElement {
    std::string name;
    long long count = 0;
    std::vector<PlyProp> props;
};

// Reads one binary scalar of type t (file byte order `big`) as a double.
double read_bin(std::istream &in, PlyType t, bool big) {
    unsigned char b[8];
    const int n = ply_size(t);
    if (!in.read(reinterpret_cast<char *>(b), n)) BEM_FAIL(BEM_ERR_IO, "PLY: unexpected end of data");
    // assemble the value from its bytes in file order: host byte order does not matter
    uint64_t u = 0;
    for (int i = 0; i < n; i++) u |= (uint64_t)b[big ? n - 1 - i : i] << (8 * i);
    switch (t) {
        case kI8: return (double)(int8_t)(uint8_t)u;
        case kU8: return (double)(uint8_t)u;
        case kI16: return (double)(int16_t)(uint16_t)u;
        case kU16: return (double)(uint16_t)u;
        case kI32: return (double)(int32_t)(uint32_t)u;
        case kU32: return (double)(uint32_t)u;
        case kF32: { uint32_t w = (uint32_t)u; float f; std::memcpy(&f, &w, 4); return f; }
        case kF64: { double d; std::memcpy(&d, &u, 8); return d; }
        default: BEM_FAIL(BEM_ERR_IO, "PLY: bad property type");
    }
}

}  // namespace

// PLY reader: "vertex" elements give x, y, z (any numeric type, other
// properties skipped); "face" elements give a vertex_indices (or
// vertex_index) list, polygons fan-triangulated from the first vertex; other
// elements are skipped.  Formats ascii, binary_little_endian and
// binary_big_endian.
void read_ply(bem_mesh_s &m, const char *path) {
    std::ifstream in(path, std::ios::binary);
    if (!in) BEM_FAIL(BEM_ERR_IO, std::string("cannot open ") + path);
    std::string line;
    std::getline(in, line);
    if (line.compare(0, 3, "ply") != 0) BEM_FAIL(BEM_ERR_IO, "PLY: missing magic line");
    int format = -1;   // 0 ascii, 1 little endian, 2 big endian
    std::vector<PlyElement> els;
    for (;;) {
        if (!std::getline(in, line)) BEM_FAIL(BEM_ERR_IO, "PLY: header without end_header");
        if (!line.empty() && line.back() == '\r') line.pop_back();
        std::istringstream is(line);
        std::string kw;
        is >> kw;
        if (kw == "format") {
            std::string f;
            is >> f;
            format = f == "ascii" ? 0 : f == "binary_little_endian" ? 1 : f == "binary_big_endian" ? 2 : -1;
            if (format < 0) BEM_FAIL(BEM_ERR_IO, "PLY: unknown format " + f);
        } else if (kw == "element") {
            PlyElement e;
            is >> e.name >> e.count;
            if (e.count < 0) BEM_FAIL(BEM_ERR_IO, "PLY: negative element count");
            els.push_back(e);
        } else if (kw == "property") {
            if (els.empty()) BEM_FAIL(BEM_ERR_IO, "PLY: property before element");
            PlyProp p;
            std::string t;
            is >> t;
            if (t == "list") {
                std::string ct, it;
                is >> ct >> it >> p.name;
                p.list = true;
                p.count_type = ply_type(ct);
                p.type = ply_type(it);
                if (p.count_type == kBad || p.count_type == kF32 || p.count_type == kF64 || p.type == kBad)
                    BEM_FAIL(BEM_ERR_IO, "PLY: bad list property " + p.name);
            } else {
                p.type = ply_type(t);
                is >> p.name;
                if (p.type == kBad) BEM_FAIL(BEM_ERR_IO, "PLY: bad property type " + t);
            }
            els.back().props.push_back(p);
        } else if (kw == "end_header") {
            break;
        }
    }
    if (format < 0) BEM_FAIL(BEM_ERR_IO, "PLY: no format line");
    std::vector<double> pnts;
    std::vector<int> elems;
    long long nvert = -1;
    const bool big = format == 2;
    for (const PlyElement &e : els) {
        int ix = -1, iy = -1, iz = -1, iface = -1;
        for (size_t k = 0; k < e.props.size(); k++) {
            const std::string &n = e.props[k].name;
            if (n == "x") ix = (int)k;
            if (n == "y") iy = (int)k;
            if (n == "z") iz = (int)k;
            if ((n == "vertex_indices" || n == "vertex_index") && e.props[k].list) iface = (int)k;
        }
        const bool is_vert = e.name == "vertex", is_face = e.name == "face";
        if (is_vert) {
            if (ix < 0 || iy < 0 || iz < 0) BEM_FAIL(BEM_ERR_IO, "PLY: vertex without x, y, z");
            nvert = e.count;
            pnts.reserve(3 * (size_t)e.count);
        }
        if (is_face && iface < 0) BEM_FAIL(BEM_ERR_IO, "PLY: face without vertex_indices");
        std::vector<long long> idx;
        for (long long r = 0; r < e.count; r++) {
            double xyz[3] = {0, 0, 0};
            idx.clear();
            std::istringstream row;
            if (format == 0) {
                if (!std::getline(in, line)) BEM_FAIL(BEM_ERR_IO, "PLY: unexpected end of data");
                row.str(line);
            }
            for (size_t k = 0; k < e.props.size(); k++) {
                const PlyProp &p = e.props[k];
                auto scalar = [&](PlyType t) {
                    if (format != 0) return read_bin(in, t, big);
                    double v;
                    if (!(row >> v)) BEM_FAIL(BEM_ERR_IO, "PLY: bad ASCII value in " + e.name);
                    return v;
                };
                if (p.list) {
                    const double c = scalar(p.count_type);
                    if (c < 0 || c > 1e6) BEM_FAIL(BEM_ERR_IO, "PLY: bad list length");
                    for (int q = 0; q < (int)c; q++) {
                        const double v = scalar(p.type);
                        if ((int)k == iface) idx.push_back((long long)v);
                    }
                } else {
                    const double v = scalar(p.type);
                    if ((int)k == ix) xyz[0] = v;
                    if ((int)k == iy) xyz[1] = v;
                    if ((int)k == iz) xyz[2] = v;
                }
            }
            if (is_vert) {
                pnts.push_back(xyz[0]);
                pnts.push_back(xyz[1]);
                pnts.push_back(xyz[2]);
            } else if (is_face) {
                if (idx.size() < 3) BEM_FAIL(BEM_ERR_IO, "PLY: face with fewer than 3 nodes");
                for (long long v : idx)
                    if (v < 0 || v > 0x7fffffffLL) BEM_FAIL(BEM_ERR_IO, "PLY: face index out of range");
                for (size_t t = 1; t + 1 < idx.size(); t++) {
                    elems.push_back((int)idx[0]);
                    elems.push_back((int)idx[t]);
                    elems.push_back((int)idx[t + 1]);
                }
            }
        }
    }
    if (nvert < 0) BEM_FAIL(BEM_ERR_IO, "PLY: no vertex element");
    for (int v : elems)
        if (v < 0 || v >= nvert) BEM_FAIL(BEM_ERR_IO, "PLY: face index out of range");
    m.pnts.swap(pnts);
    m.elems.swap(elems);
    m.chief.clear();
    m.has_bb = false;
    m.default_bc();
}

// Makes the winding consistent across every edge-connected component (a
// breadth-first walk flips a neighbour whose shared edge runs the same way)
// and then orients each closed component so that (p1-p3) x (p2-p3) points
// into the body, the reference's convention: the signed volume
// sum p1 . (p2 x p3) / 6 of such a component is negative.  An edge shared by
// more than two elements is counted in `nonmanifold` and not used for
// propagation; `open_edges` counts edges with a single element (such
// components keep the orientation of their first element).
MeshOrientReport orient_mesh(bem_mesh_s &m) {
    const int E = m.num_elems();
    MeshOrientReport rep{};
    auto key = [](int a, int b) { return ((uint64_t)(uint32_t)std::min(a, b) << 32) | (uint32_t)std::max(a, b); };
    std::unordered_map<uint64_t, std::vector<int>> edge_faces;
    edge_faces.reserve(3 * (size_t)E);
    for (int e = 0; e < E; e++)
        for (int k = 0; k < 3; k++)
            edge_faces[key(m.elems[3 * e + k], m.elems[3 * e + (k + 1) % 3])].push_back(e);
    for (auto &kv : edge_faces) {
        if (kv.second.size() == 1) rep.open_edges++;
        if (kv.second.size() > 2) rep.nonmanifold++;
    }
    // runs a->b in element e?
    auto has_dir = [&](int e, int a, int b) {
        for (int k = 0; k < 3; k++)
            if (m.elems[3 * e + k] == a && m.elems[3 * e + (k + 1) % 3] == b) return true;
        return false;
    };
    auto flip = [&](int e) { std::swap(m.elems[3 * e], m.elems[3 * e + 1]); };
    std::vector<int> comp(E, -1);
    std::vector<char> flipped(E, 0);
    for (int seed = 0; seed < E; seed++) {
        if (comp[seed] >= 0) continue;
        const int c = rep.components++;
        std::deque<int> q{seed};
        comp[seed] = c;
        std::vector<int> members;
        bool closed = true;
        while (!q.empty()) {
            const int e = q.front();
            q.pop_front();
            members.push_back(e);
            for (int k = 0; k < 3; k++) {
                const int a = m.elems[3 * e + k], b = m.elems[3 * e + (k + 1) % 3];
                const std::vector<int> &nb = edge_faces[key(a, b)];
                if (nb.size() == 1) closed = false;
                if (nb.size() != 2) continue;
                const int f = nb[0] == e ? nb[1] : nb[0];
                if (comp[f] >= 0) continue;
                comp[f] = c;
                if (has_dir(f, a, b)) {   // same direction as in e: inconsistent
                    flip(f);
                    flipped[f] ^= 1;
                }
                q.push_back(f);
            }
        }
        double vol = 0.0;
        for (int e : members) {
            const double *p1 = &m.pnts[3 * (size_t)m.elems[3 * e]];
            const double *p2 = &m.pnts[3 * (size_t)m.elems[3 * e + 1]];
            const double *p3 = &m.pnts[3 * (size_t)m.elems[3 * e + 2]];
            vol += p1[0] * (p2[1] * p3[2] - p2[2] * p3[1]) - p1[1] * (p2[0] * p3[2] - p2[2] * p3[0]) +
                   p1[2] * (p2[0] * p3[1] - p2[1] * p3[0]);
        }
        if (closed && vol > 0.0)
            for (int e : members) {
                flip(e);
                flipped[e] ^= 1;
            }
        if (closed) rep.volume += std::fabs(vol) / 6.0;
    }
    // (the per-element boundary condition belongs to the element, not to its winding)
    for (int e = 0; e < E; e++) rep.flipped += flipped[e];
    return rep;
}

}  // namespace bem
