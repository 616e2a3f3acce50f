// Synthetic-geometry generators for the benchmark configurations (no
// reference counterpart): class-I geodesic spheres, smooth radially perturbed
// ellipsoids, and Fibonacci-lattice source sets.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <map>
#include <tuple>
#include <vector>

#include "mesh.h"

namespace bem {

namespace {

void normalize3(double *p) {
    double n = std::sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]);
    p[0] /= n; p[1] /= n; p[2] /= n;
}

// Every face wound so that (p1-p3) x (p2-p3) points into the body (the
// orientation of the reference's meshes).  The body must be star-shaped
// around the origin.
void wind_inward(const std::vector<double> &v, std::vector<int> &f) {
    for (size_t i = 0; i < f.size(); i += 3) {
        const double *p1 = &v[3 * (size_t)f[i]], *p2 = &v[3 * (size_t)f[i + 1]], *p3 = &v[3 * (size_t)f[i + 2]];
        double a[3] = {p1[0] - p3[0], p1[1] - p3[1], p1[2] - p3[2]};
        double b[3] = {p2[0] - p3[0], p2[1] - p3[1], p2[2] - p3[2]};
        double n[3] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
        double c[3] = {p1[0] + p2[0] + p3[0], p1[1] + p2[1] + p3[1], p1[2] + p2[2] + p3[2]};
        if (n[0] * c[0] + n[1] * c[1] + n[2] * c[2] > 0) std::swap(f[i], f[i + 1]);
    }
}

// SplitMix64 + Box-Muller: a seeded normal stream that is identical on every
// platform.
struct Rng {
    uint64_t s;
    uint64_t next() {
        uint64_t z = (s += 0x9e3779b97f4a7c15ULL);
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
        return z ^ (z >> 31);
    }
    double uniform() { return ((next() >> 11) + 0.5) * (1.0 / 9007199254740992.0); }
    double normal() {
        double u1 = uniform(), u2 = uniform();
        return std::sqrt(-2.0 * std::log(u1)) * std::cos(2.0 * kPi * u2);
    }
};

// Real spherical harmonics up to degree lmax at direction (x, y, z), by the
// standard associated-Legendre recurrences (orthonormal up to a common
// factor per (l, m)); out holds (lmax+1)^2 values ordered (l, m = -l..l).
void real_sh(int lmax, double x, double y, double z, std::vector<double> &out) {
    out.assign((size_t)(lmax + 1) * (lmax + 1), 0.0);
    const double ct = z, st = std::sqrt(std::max(0.0, 1.0 - z * z));
    const double phi = std::atan2(y, x);
    std::vector<double> P((size_t)(lmax + 1) * (lmax + 1), 0.0);   // P[l*(lmax+1)+m]
    auto at = [&](int l, int m) -> double & { return P[(size_t)l * (lmax + 1) + m]; };
    at(0, 0) = 1.0;
    for (int m = 1; m <= lmax; m++) at(m, m) = -(2.0 * m - 1.0) * st * at(m - 1, m - 1);
    for (int m = 0; m < lmax; m++) at(m + 1, m) = (2.0 * m + 1.0) * ct * at(m, m);
    for (int m = 0; m <= lmax; m++)
        for (int l = m + 2; l <= lmax; l++)
            at(l, m) = ((2.0 * l - 1.0) * ct * at(l - 1, m) - (l + m - 1.0) * at(l - 2, m)) / (l - m);
    for (int l = 0; l <= lmax; l++) {
        for (int m = 0; m <= l; m++) {
            double lf = 1.0;   // sqrt((2l+1)/(4pi) (l-m)!/(l+m)!)
            for (int t = l - m + 1; t <= l + m; t++) lf /= t;
            double nrm = std::sqrt((2.0 * l + 1.0) / (4.0 * kPi) * lf);
            double v = nrm * at(l, m);
            size_t base = (size_t)l * l + l;
            if (m == 0) {
                out[base] = v;
            } else {
                out[base + m] = std::sqrt(2.0) * v * std::cos(m * phi);
                out[base - m] = std::sqrt(2.0) * v * std::sin(m * phi);
            }
        }
    }
}

}  // namespace

// Class-I geodesic sphere of frequency nu: every icosahedron face split into
// nu^2 triangles on its barycentric grid, nodes projected to the sphere.
// V = 10 nu^2 + 2, F = 20 nu^2 (nu = 39 gives 30420 triangles).
void make_geodesic(bem_mesh_s &m, int nu, double radius) {
    BEM_CHECK_ARG(nu >= 1 && nu <= 400, "geodesic frequency must be in [1, 400]");
    BEM_CHECK_ARG(radius > 0, "radius must be positive");
    const double t = (1.0 + std::sqrt(5.0)) / 2.0;
    const double ico[12][3] = {{-1, t, 0}, {1, t, 0}, {-1, -t, 0}, {1, -t, 0}, {0, -1, t}, {0, 1, t},
                               {0, -1, -t}, {0, 1, -t}, {t, 0, -1}, {t, 0, 1}, {-t, 0, -1}, {-t, 0, 1}};
    const int faces[20][3] = {{0, 11, 5}, {0, 5, 1}, {0, 1, 7}, {0, 7, 10}, {0, 10, 11}, {1, 5, 9}, {5, 11, 4},
                              {11, 10, 2}, {10, 7, 6}, {7, 1, 8}, {3, 9, 4}, {3, 4, 2}, {3, 2, 6}, {3, 6, 8},
                              {3, 8, 9}, {4, 9, 5}, {2, 4, 11}, {6, 2, 10}, {8, 6, 7}, {9, 8, 1}};
    // A grid node is identified by its integer barycentric weights on the
    // icosahedron vertices (shared edges and corners map to the same key).
    std::map<std::tuple<int, int, int, int, int, int>, int> index;
    std::vector<double> v;
    std::vector<int> f;
    f.reserve(60 * (size_t)nu * nu);
    auto node = [&](const int *fv, int i, int j) {
        int w[3] = {nu - i - j, i, j};
        int ids[3] = {fv[0], fv[1], fv[2]};
        // canonical key: (vertex, weight) pairs with weight > 0, sorted by vertex
        std::vector<std::pair<int, int>> kv;
        for (int q = 0; q < 3; q++)
            if (w[q] > 0) kv.emplace_back(ids[q], w[q]);
        std::sort(kv.begin(), kv.end());
        while (kv.size() < 3) kv.emplace_back(-1, 0);
        auto key = std::make_tuple(kv[0].first, kv[0].second, kv[1].first, kv[1].second, kv[2].first, kv[2].second);
        auto it = index.find(key);
        if (it != index.end()) return it->second;
        double p[3];
        for (int d = 0; d < 3; d++)
            p[d] = (w[0] * ico[ids[0]][d] + w[1] * ico[ids[1]][d] + w[2] * ico[ids[2]][d]) / nu;
        normalize3(p);
        int id = (int)(v.size() / 3);
        v.insert(v.end(), p, p + 3);
        index.emplace(key, id);
        return id;
    };
    for (const auto &fv : faces) {
        for (int i = 0; i < nu; i++)
            for (int j = 0; i + j < nu; j++) {
                int a = node(fv, i, j), b = node(fv, i + 1, j), c = node(fv, i, j + 1);
                f.insert(f.end(), {a, b, c});
                if (i + j + 2 <= nu) {
                    int d = node(fv, i + 1, j + 1);
                    f.insert(f.end(), {b, d, c});
                }
            }
    }
    wind_inward(v, f);
    for (double &x : v) x *= radius;
    m.pnts.swap(v);
    m.elems.swap(f);
    m.chief.clear();
    m.has_bb = false;
    m.default_bc();
}

// Maps the nodes of a unit sphere mesh onto a triaxial ellipsoid with semi-axes
// (a, b, c), radially perturbed by a seeded smooth field: node u (unit vector)
// goes to (a ux, b uy, c uz) (1 + f(u)), f = sum_{l <= lmax} c_lm Y_lm(u) with
// c_lm standard normal from `seed`, scaled so that max over the nodes of |f| is
// `amp`.  The mesh keeps its connectivity and inward winding.
void map_perturbed_ellipsoid(bem_mesh_s &m, double a, double b, double c, int lmax, double amp,
                             unsigned long long seed) {
    BEM_CHECK_ARG(a > 0 && b > 0 && c > 0, "semi-axes must be positive");
    BEM_CHECK_ARG(lmax >= 0 && lmax <= 32 && amp >= 0 && amp < 0.5, "lmax in [0, 32], amplitude in [0, 0.5)");
    const int N = m.num_pnts();
    BEM_CHECK_ARG(N > 0, "empty mesh");
    Rng rng{seed};
    std::vector<double> coef((size_t)(lmax + 1) * (lmax + 1));
    for (double &x : coef) x = rng.normal();
    std::vector<double> f(N), sh;
    double fmax = 0.0;
    for (int i = 0; i < N; i++) {
        double u[3] = {m.pnts[3 * (size_t)i], m.pnts[3 * (size_t)i + 1], m.pnts[3 * (size_t)i + 2]};
        normalize3(u);
        real_sh(lmax, u[0], u[1], u[2], sh);
        double s = 0.0;
        for (size_t q = 0; q < sh.size(); q++) s += coef[q] * sh[q];
        f[i] = s;
        fmax = std::max(fmax, std::fabs(s));
    }
    const double scale = fmax > 0 ? amp / fmax : 0.0;
    for (int i = 0; i < N; i++) {
        double u[3] = {m.pnts[3 * (size_t)i], m.pnts[3 * (size_t)i + 1], m.pnts[3 * (size_t)i + 2]};
        normalize3(u);
        double g = 1.0 + scale * f[i];
        m.pnts[3 * (size_t)i] = a * u[0] * g;
        m.pnts[3 * (size_t)i + 1] = b * u[1] * g;
        m.pnts[3 * (size_t)i + 2] = c * u[2] * g;
    }
    m.chief.clear();
    m.has_bb = false;
}

// n points of a Fibonacci lattice on a sphere of the given radius.
void fibonacci_sphere(int n, double radius, double *out) {
    BEM_CHECK_ARG(n >= 1 && out && radius > 0, "bad Fibonacci lattice arguments");
    const double ga = kPi * (3.0 - std::sqrt(5.0));
    for (int i = 0; i < n; i++) {
        double z = 1.0 - 2.0 * (i + 0.5) / n;
        double r = std::sqrt(std::max(0.0, 1.0 - z * z));
        double ph = ga * i;
        out[3 * i] = radius * r * std::cos(ph);
        out[3 * i + 1] = radius * r * std::sin(ph);
        out[3 * i + 2] = radius * z;
    }
}

}  // namespace bem
