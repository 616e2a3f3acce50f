// bem_gb300.hpp -- the reference's C++ call surface over the C ABI.
//
// A program written against ZiqiFrancisFan/BEM_GPU_Clean_CPP (mesh.h,
// numerical.h, GMRES.h) switches by including this header instead and
// linking libbem_gb300.so.  Names, argument order, meaning and the
// EXIT_SUCCESS / nonzero return convention follow the reference; every call
// forwards to the C ABI in bem_gb300.h, so the GPU work is the engine's own.
// Define BEM_GB300_GLOBAL_NAMES before including to get the names in the
// global namespace, as the reference declares them.
#ifndef BEM_GB300_HPP
#define BEM_GB300_HPP

#include <cuComplex.h>

#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "bem_gb300.h"

// The reference's status-check macro (numerical.h:59-64), which its callers use
// around every call.
#ifndef HOST_CALL
#define HOST_CALL(x)                                              \
    do {                                                          \
        if ((x) != EXIT_SUCCESS) {                                \
            std::printf("Error at %s:%d\n", __FILE__, __LINE__); \
            return EXIT_FAILURE;                                  \
        }                                                         \
    } while (0)
#endif

namespace bem_gb300 {

// Error report in the reference's style ("Error at file:line", numerical.h:59-122)
// plus the engine's message.
inline int report(int status, const char *what) {
    if (status != BEM_SUCCESS) std::fprintf(stderr, "Error in %s: %s\n", what, bem_last_error());
    return status;
}

// class cartCoord (mesh.h:26-99): the fields and constructors callers use.
class cartCoord {
   public:
    float coords[3];
    cartCoord() : coords{0.f, 0.f, 0.f} {}
    cartCoord(float x, float y, float z) : coords{x, y, z} {}
    void set(float x, float y, float z) {
        coords[0] = x;
        coords[1] = y;
        coords[2] = z;
    }
};

// class mesh (mesh.h:216-259).
class mesh {
   public:
    mesh() { report(bem_mesh_create(&h_), "mesh"); }
    ~mesh() { bem_mesh_destroy(h_); }
    mesh(const mesh &o) : mesh() { copy_from(o); }
    mesh &operator=(const mesh &o) {
        if (this != &o) copy_from(o);
        return *this;
    }
    int readObj(const char *file) { return report(bem_mesh_read_obj(h_, file), "readObj"); }
    int findBB(const float threshold) { return report(bem_mesh_find_bb(h_, threshold), "findBB"); }
    int genCHIEF(const int num, const float threshold) {
        return report(bem_mesh_gen_chief(h_, num, threshold), "genCHIEF");
    }
    int getNumChief() const { return counts()[2]; }
    int getNumPnts() const { return counts()[0]; }
    int getNumElems() const { return counts()[1]; }
    void printCHIEF() const {
        std::vector<double> c(3 * (size_t)getNumChief());
        if (!c.empty()) bem_mesh_get_chief(h_, c.data());
        for (size_t i = 0; i < c.size(); i += 3) std::printf("(%f,%f,%f)\n", c[i], c[i + 1], c[i + 2]);
    }
    // extensions (no reference counterpart)
    int readObjRobust(const char *file) { return report(bem_mesh_read_obj_robust(h_, file), "readObjRobust"); }
    int readPly(const char *file) { return report(bem_mesh_read_ply(h_, file), "readPly"); }
    // Consistent winding with (p1-p3) x (p2-p3) into the body; returns the
    // number of flipped elements, or -1 on failure.
    int orient() {
        int flipped = 0;
        return report(bem_mesh_orient(h_, &flipped, nullptr, nullptr, nullptr, nullptr), "orient") == EXIT_SUCCESS
                   ? flipped
                   : -1;
    }
    int setCHIEF(const std::vector<cartCoord> &pts) {
        std::vector<double> c;
        for (const cartCoord &p : pts) c.insert(c.end(), {p.coords[0], p.coords[1], p.coords[2]});
        return report(bem_mesh_set_chief(h_, c.data(), (int)pts.size()), "setCHIEF");
    }
    bem_mesh_t handle() const { return h_; }

   private:
    bem_mesh_t h_ = nullptr;
    std::vector<int> counts() const {
        std::vector<int> c(3, 0);
        bem_mesh_get_counts(h_, &c[0], &c[1], &c[2]);
        return c;
    }
    void copy_from(const mesh &o) {
        std::vector<int> c = o.counts();
        if (c[0] == 0 || c[1] == 0) return;
        std::vector<double> p(3 * (size_t)c[0]), ch(3 * (size_t)c[2]);
        std::vector<int> e(3 * (size_t)c[1]);
        bem_mesh_get_points(o.h_, p.data());
        bem_mesh_get_elems(o.h_, e.data());
        if (c[2]) bem_mesh_get_chief(o.h_, ch.data());
        bem_mesh_set(h_, p.data(), c[0], e.data(), c[1]);
        if (c[2]) bem_mesh_set_chief(h_, ch.data(), c[2]);
    }
};

// class gaussQuad (numerical.h:166-187): the order and sendToDevice().
class gaussQuad {
   public:
    explicit gaussQuad(int order = 6) : n(order), evalPnts(order), wgts(order) {
        report(bem_gauss_legendre(order, evalPnts.data(), wgts.data()), "gaussQuad");
    }
    int sendToDevice() { return report(bem_set_quadrature(n), "sendToDevice"); }

   private:
    int n;
    std::vector<double> evalPnts, wgts;
};

// bemSystem (mesh.h:222-223): A ((N+M) x N) and B ((N+M) x numSrcs).
inline int bemSystem(const mesh &m, const float k, const cartCoord *srcs, const int numSrcs,
                     cuFloatComplex *A, const int lda, cuFloatComplex *B, const int ldb) {
    std::vector<float> s;
    for (int i = 0; i < numSrcs; i++) s.insert(s.end(), {srcs[i].coords[0], srcs[i].coords[1], srcs[i].coords[2]});
    return report(bem_system_c64(m.handle(), k, s.data(), numSrcs, reinterpret_cast<float *>(A), lda,
                                 reinterpret_cast<float *>(B), ldb),
                  "bemSystem");
}

// qrSolver (numerical.h:196-197).
inline int qrSolver(const cuFloatComplex *A, const int mA, const int nA, const int ldA, cuFloatComplex *B,
                    const int nB, const int ldB) {
    return report(bem_qr_solve_c64(reinterpret_cast<const float *>(A), mA, nA, ldA,
                                   reinterpret_cast<float *>(B), nB, ldB),
                  "qrSolver");
}

// GMRES (GMRES.h:104-105).
inline int GMRES(const cuFloatComplex *A_h, const cuFloatComplex *b_h, const int m, const int maxIter,
                 const float threshold, cuFloatComplex *x_h) {
    return report(bem_gmres_c64(reinterpret_cast<const float *>(A_h), reinterpret_cast<const float *>(b_h), m,
                                maxIter, threshold, reinterpret_cast<float *>(x_h)),
                  "GMRES");
}

// genExtPressure (mesh.h:425-426).
inline cuFloatComplex genExtPressure(const float k, const mesh &m, const cartCoord src, const cartCoord x,
                                     const cuFloatComplex *surfPressure) {
    float out[2] = {0.f, 0.f};
    report(bem_ext_pressure_c64(k, m.handle(), src.coords, x.coords, reinterpret_cast<const float *>(surfPressure),
                                out),
           "genExtPressure");
    return make_cuFloatComplex(out[0], out[1]);
}

// wrtCplxMat (numerical.h:192-193).
inline int wrtCplxMat(const cuFloatComplex *mat, const int numRows, const int numCols, const int ldm,
                      const char *file) {
    return report(bem_write_cplx_mat_c64(reinterpret_cast<const float *>(mat), numRows, numCols, ldm, file),
                  "wrtCplxMat");
}

// printComplexMatrix (numerical.cu:81-93).
inline void printComplexMatrix(const cuFloatComplex *A, const int row, const int col, const int lda) {
    for (int i = 0; i < row; i++) {
        for (int j = 0; j < col; j++)
            std::printf("(%f,%f) ", cuCrealf(A[(size_t)lda * j + i]), cuCimagf(A[(size_t)lda * j + i]));
        std::printf("\n");
    }
}

}  // namespace bem_gb300

#ifdef BEM_GB300_GLOBAL_NAMES
using bem_gb300::bemSystem;
using bem_gb300::cartCoord;
using bem_gb300::gaussQuad;
using bem_gb300::genExtPressure;
using bem_gb300::GMRES;
using bem_gb300::mesh;
using bem_gb300::printComplexMatrix;
using bem_gb300::qrSolver;
using bem_gb300::wrtCplxMat;
#endif

#endif  // BEM_GB300_HPP
