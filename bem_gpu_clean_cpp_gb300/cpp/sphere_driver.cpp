// The reference driver's call sequence (main.cpp:24-107 with the field
// evaluation of main.cpp:74-97 enabled) written against bem_gb300.hpp:
// readObj -> findBB -> genCHIEF -> gaussQuad::sendToDevice -> bemSystem ->
// qrSolver -> genExtPressure at (-(1+0.2 i), 0, 0), i = 1..10 -> wrtCplxMat.
//
// usage: bem_sphere_driver <mesh.obj> <out file> [freq Hz] [CHIEF points] [CHIEF threshold]
#define BEM_GB300_GLOBAL_NAMES
#include "../../include/bem_gb300.hpp"

#include <cstdio>
#include <cstdlib>
#include <vector>

#ifndef PI
#define PI 3.1415926535897932
#endif

int main(int argc, char **argv) {
    if (argc < 3) {
        std::fprintf(stderr, "usage: %s mesh.obj out.txt [freq] [nchief] [threshold]\n", argv[0]);
        return EXIT_FAILURE;
    }
    float f = argc > 3 ? (float)std::atof(argv[3]) : 171.5f;
    int nchief = argc > 4 ? std::atoi(argv[4]) : 1;
    float thr = argc > 5 ? (float)std::atof(argv[5]) : 0.1f;
    float k = 2 * PI * f / 343.21;
    mesh m;
    HOST_CALL(m.readObj(argv[1]));
    HOST_CALL(m.findBB(0.0001));
    HOST_CALL(m.genCHIEF(nchief, thr));
    gaussQuad gss(6);
    HOST_CALL(gss.sendToDevice());
    cartCoord src(1000000, 1000000, 1000000);
    int numSrcs = 1;
    int rows = m.getNumPnts() + m.getNumChief();
    std::vector<cuFloatComplex> A((size_t)rows * m.getNumPnts()), B((size_t)rows * numSrcs);
    HOST_CALL(bemSystem(m, k, &src, numSrcs, A.data(), rows, B.data(), rows));
    HOST_CALL(qrSolver(A.data(), rows, m.getNumPnts(), rows, B.data(), numSrcs, rows));
    const float step = 0.2f;
    const int numLocs = 11;
    std::vector<cuFloatComplex> pressure(numLocs);
    pressure[0] = B[0];
    for (int i = 1; i < numLocs; i++) pressure[i] = genExtPressure(k, m, src, cartCoord(-(1 + step * i), 0, 0), B.data());
    printComplexMatrix(pressure.data(), 1, numLocs, 1);
    HOST_CALL(wrtCplxMat(pressure.data(), 1, numLocs, 1, argv[2]));
    return EXIT_SUCCESS;
}
