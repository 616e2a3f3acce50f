// Mesh input and preprocessing on the host: OBJ readers, icosphere
// generator, bounding box and the CHIEF point search driver.
#include "mesh.h"

#include <curand.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <sstream>
#include <string>
#include <utility>

void bem_mesh_s::default_bc() {
    // readObj's per-face default (mesh.cu:1240-1242): ca = 0, cb = 1, cc = -1.
    bc.assign(6 * (size_t)num_elems(), 0.0);
    for (int e = 0; e < num_elems(); e++) {
        bc[6 * e + 2] = 1.0;
        bc[6 * e + 4] = -1.0;
    }
}

void bem_mesh_s::validate() const {
    int N = num_pnts();
    if (N == 0 || num_elems() == 0) BEM_FAIL(BEM_ERR_STATE, "mesh has no nodes or no elements");
    for (size_t i = 0; i < elems.size(); i++)
        if (elems[i] < 0 || elems[i] >= N)
            BEM_FAIL(BEM_ERR_INVALID_ARG, "element " + std::to_string(i / 3) +
                                              " references node " + std::to_string(elems[i]) +
                                              " outside [0," + std::to_string(N) + ")");
    for (int e = 0; e < num_elems(); e++) {
        const int *nd = &elems[3 * (size_t)e];
        if (nd[0] == nd[1] || nd[1] == nd[2] || nd[0] == nd[2])
            BEM_FAIL(BEM_ERR_INVALID_ARG, "element " + std::to_string(e) + " repeats a node");
        const double *b = &bc[6 * (size_t)e];
        if (b[2] == 0.0 && b[3] == 0.0)
            BEM_FAIL(BEM_ERR_INVALID_ARG, "element " + std::to_string(e) + " has cb = 0");
    }
}

namespace bem {

// mesh::readObj (mesh.cu:1215-1265).  The same parse rules: fgets with a
// 49-byte buffer (lines are read in chunks of at most 48 characters), a chunk
// starting with 'v' is parsed as "%s %f %f %f" (so vn/vt lines are read as
// vertices too), a chunk starting with 'f' as "%s %d %d %d" (1-based, the
// first integer of each field), and fields that fail to parse keep the values
// of the previous line, as the reference's reused locals do.
void read_obj_reference(bem_mesh_s &m, const char *path) {
    FILE *fp = std::fopen(path, "r");
    if (!fp) BEM_FAIL(BEM_ERR_IO, std::string("cannot open ") + path);
    std::vector<double> pnts;
    std::vector<int> elems;
    char line[50];
    char type[64];
    float pnt[3] = {0, 0, 0};
    int tmp[3] = {0, 0, 0};
    while (std::fgets(line, 49, fp) != nullptr) {
        if (line[0] == 'v') {
            std::sscanf(line, "%63s %f %f %f", type, &pnt[0], &pnt[1], &pnt[2]);
            for (int d = 0; d < 3; d++) pnts.push_back((double)pnt[d]);
        }
        if (line[0] == 'f') {
            std::sscanf(line, "%63s %d %d %d", type, &tmp[0], &tmp[1], &tmp[2]);
            for (int d = 0; d < 3; d++) elems.push_back(tmp[d] - 1);
        }
    }
    std::fclose(fp);
    m.pnts.swap(pnts);
    m.elems.swap(elems);
    m.chief.clear();
    m.has_bb = false;
    m.default_bc();
}

// Robust OBJ reader: whole lines of any length; "v" vertices only; faces with
// "a", "a/b", "a//c" or "a/b/c" fields, negative (relative) indices, and
// polygons triangulated as a fan from the first vertex.
void read_obj_robust(bem_mesh_s &m, const char *path) {
    FILE *fp = std::fopen(path, "r");
    if (!fp) BEM_FAIL(BEM_ERR_IO, std::string("cannot open ") + path);
    std::vector<double> pnts;
    std::vector<int> elems;
    std::string line;
    int ch;
    long lineno = 0;
    auto flush_line = [&](const std::string &ln) {
        lineno++;
        size_t p = ln.find_first_not_of(" \t\r");
        if (p == std::string::npos) return;
        std::istringstream is(ln.substr(p));
        std::string tag;
        is >> tag;
        if (tag == "v") {
            double x, y, z;
            if (!(is >> x >> y >> z)) {
                std::fclose(fp);
                BEM_FAIL(BEM_ERR_IO, "bad vertex at line " + std::to_string(lineno));
            }
            pnts.push_back(x); pnts.push_back(y); pnts.push_back(z);
        } else if (tag == "f") {
            std::vector<int> idx;
            std::string tok;
            int nv = (int)(pnts.size() / 3);
            while (is >> tok) {
                size_t slash = tok.find('/');
                std::string head = tok.substr(0, slash);
                char *end = nullptr;
                long v = std::strtol(head.c_str(), &end, 10);
                if (head.empty() || *end != '\0' || v == 0) {
                    std::fclose(fp);
                    BEM_FAIL(BEM_ERR_IO, "bad face index at line " + std::to_string(lineno));
                }
                idx.push_back(v > 0 ? (int)(v - 1) : nv + (int)v);
            }
            if (idx.size() < 3) {
                std::fclose(fp);
                BEM_FAIL(BEM_ERR_IO, "face with fewer than 3 nodes at line " + std::to_string(lineno));
            }
            for (size_t t = 1; t + 1 < idx.size(); t++) {
                elems.push_back(idx[0]);
                elems.push_back(idx[t]);
                elems.push_back(idx[t + 1]);
            }
        }
    };
    while ((ch = std::fgetc(fp)) != EOF) {
        if (ch == '\n') {
            flush_line(line);
            line.clear();
        } else {
            line.push_back((char)ch);
        }
    }
    if (!line.empty()) flush_line(line);
    std::fclose(fp);
    int nv = (int)(pnts.size() / 3);
    for (int v : elems)
        if (v < 0 || v >= nv) BEM_FAIL(BEM_ERR_IO, "face index out of range in " + std::string(path));
    m.pnts.swap(pnts);
    m.elems.swap(elems);
    m.chief.clear();
    m.has_bb = false;
    m.default_bc();
}

// Icosphere: an icosahedron subdivided `subdiv` times (each triangle split in
// four at edge midpoints, new nodes projected onto the sphere).  V = 10*4^s+2,
// F = 20*4^s.  Every face is wound so that (p1-p3) x (p2-p3) points towards the
// centre, the orientation of the reference's sphere meshes.
void make_icosphere(bem_mesh_s &m, int subdiv, double radius) {
    BEM_CHECK_ARG(subdiv >= 0 && subdiv <= 9, "icosphere subdivision must be in [0, 9]");
    BEM_CHECK_ARG(radius > 0, "icosphere radius must be positive");
    const double t = (1.0 + std::sqrt(5.0)) / 2.0;
    std::vector<double> v = {-1, t, 0, 1, t, 0, -1, -t, 0, 1, -t, 0, 0, -1, t, 0, 1, t,
                             0, -1, -t, 0, 1, -t, t, 0, -1, t, 0, 1, -t, 0, -1, -t, 0, 1};
    std::vector<int> f = {0, 11, 5, 0, 5, 1, 0, 1, 7, 0, 7, 10, 0, 10, 11, 1, 5, 9, 5, 11, 4,
                          11, 10, 2, 10, 7, 6, 7, 1, 8, 3, 9, 4, 3, 4, 2, 3, 2, 6, 3, 6, 8,
                          3, 8, 9, 4, 9, 5, 2, 4, 11, 6, 2, 10, 8, 6, 7, 9, 8, 1};
    auto normalize = [&](size_t i) {
        double n = std::sqrt(v[3 * i] * v[3 * i] + v[3 * i + 1] * v[3 * i + 1] + v[3 * i + 2] * v[3 * i + 2]);
        v[3 * i] /= n; v[3 * i + 1] /= n; v[3 * i + 2] /= n;
    };
    for (size_t i = 0; i < 12; i++) normalize(i);
    for (int s = 0; s < subdiv; s++) {
        std::map<std::pair<int, int>, int> mid;
        auto midpoint = [&](int a, int b) {
            std::pair<int, int> key(std::min(a, b), std::max(a, b));
            auto it = mid.find(key);
            if (it != mid.end()) return it->second;
            int id = (int)(v.size() / 3);
            for (int d = 0; d < 3; d++) v.push_back(0.5 * (v[3 * a + d] + v[3 * b + d]));
            normalize(id);
            mid.emplace(key, id);
            return id;
        };
        std::vector<int> nf;
        nf.reserve(f.size() * 4);
        for (size_t i = 0; i < f.size(); i += 3) {
            int a = f[i], b = f[i + 1], c = f[i + 2];
            int ab = midpoint(a, b), bc = midpoint(b, c), ca = midpoint(c, a);
            int tri[12] = {a, ab, ca, b, bc, ab, c, ca, bc, ab, bc, ca};
            nf.insert(nf.end(), tri, tri + 12);
        }
        f.swap(nf);
    }
    // Inward winding.
    for (size_t i = 0; i < f.size(); i += 3) {
        const double *p1 = &v[3 * f[i]], *p2 = &v[3 * f[i + 1]], *p3 = &v[3 * f[i + 2]];
        double a[3] = {p1[0] - p3[0], p1[1] - p3[1], p1[2] - p3[2]};
        double b[3] = {p2[0] - p3[0], p2[1] - p3[1], p2[2] - p3[2]};
        double n[3] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
        double c[3] = {p1[0] + p2[0] + p3[0], p1[1] + p2[1] + p3[1], p1[2] + p2[2] + p3[2]};
        if (n[0] * c[0] + n[1] * c[1] + n[2] * c[2] > 0) std::swap(f[i], f[i + 1]);
    }
    for (double &x : v) x *= radius;
    m.pnts.swap(v);
    m.elems.swap(f);
    m.chief.clear();
    m.has_bb = false;
    m.default_bc();
}

// mesh::findBB (mesh.cu:1369-1409), in float like the reference.
void find_bb(bem_mesh_s &m, float threshold) {
    if (m.num_pnts() == 0 || m.num_elems() == 0) BEM_FAIL(BEM_ERR_STATE, "Not enough mesh information!");
    float lo[3], hi[3];
    for (int d = 0; d < 3; d++) lo[d] = hi[d] = (float)m.pnts[d];
    for (int i = 1; i < m.num_pnts(); i++)
        for (int d = 0; d < 3; d++) {
            float x = (float)m.pnts[3 * (size_t)i + d];
            if (x < lo[d]) lo[d] = x;
            if (x > hi[d]) hi[d] = x;
        }
    for (int d = 0; d < 3; d++) {
        m.bb[2 * d] = lo[d] - threshold;
        m.bb[2 * d + 1] = hi[d] + threshold;
    }
    m.has_bb = true;
}

// mesh::genCHIEF (mesh.cu:1430-1483).  Candidate c uses cuRAND's default host
// generator (XORWOW) reseeded with seed c; its three uniforms u are both the
// ray direction and, through descale (numerical.cu:105-107), the point
// lb + (ub-lb)*u inside the bounding box.  Candidates are accepted in seed
// order, so the result equals the reference's one-candidate-at-a-time loop;
// here candidates are tested on the GPU in batches.  The search gives up
// after a bounded number of candidates instead of looping forever.
void gen_chief(bem_mesh_s &m, int num, float threshold) {
    BEM_CHECK_ARG(num >= 0, "CHIEF count must be >= 0");
    if (!m.has_bb) BEM_FAIL(BEM_ERR_STATE, "genCHIEF needs findBB first");
    m.validate();
    std::vector<double> out;
    if (num == 0) {
        m.chief.clear();
        return;
    }
    curandGenerator_t gen;
    if (curandCreateGeneratorHost(&gen, CURAND_RNG_PSEUDO_DEFAULT) != CURAND_STATUS_SUCCESS)
        BEM_FAIL(BEM_ERR_CUDA, "curandCreateGeneratorHost failed");
    std::vector<float> pf(m.pnts.size());
    for (size_t i = 0; i < pf.size(); i++) pf[i] = (float)m.pnts[i];
    const int batch = 256;
    const long long max_cand = 1 << 20;
    long long seed = 0;
    int got = 0;
    std::vector<float> cp(3 * batch), cd(3 * batch);
    std::vector<int> acc;
    try {
        while (got < num) {
            if (seed >= max_cand)
                BEM_FAIL(BEM_ERR_NUMERIC, "genCHIEF: no acceptable CHIEF point among " +
                                              std::to_string(max_cand) + " candidates");
            for (int c = 0; c < batch; c++) {
                float u[3];
                if (curandSetPseudoRandomGeneratorSeed(gen, (unsigned long long)(seed + c)) != CURAND_STATUS_SUCCESS ||
                    curandGenerateUniform(gen, u, 3) != CURAND_STATUS_SUCCESS)
                    BEM_FAIL(BEM_ERR_CUDA, "cuRAND host generation failed");
                for (int d = 0; d < 3; d++) {
                    cd[3 * c + d] = u[d];
                    float lo = m.bb[2 * d], hi = m.bb[2 * d + 1];
                    cp[3 * c + d] = lo + (hi - lo) * u[d];
                }
            }
            chief_test_candidates(pf, m.elems, cp, cd, threshold, acc);
            for (int c = 0; c < batch && got < num; c++)
                if (acc[c]) {
                    for (int d = 0; d < 3; d++) out.push_back((double)cp[3 * c + d]);
                    got++;
                }
            seed += batch;
        }
    } catch (...) {
        curandDestroyGenerator(gen);
        throw;
    }
    curandDestroyGenerator(gen);
    m.chief.swap(out);
}

}  // namespace bem
