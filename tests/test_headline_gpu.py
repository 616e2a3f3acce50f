"""The benchmark's headline system against the FP64 oracle, on sampled rows.

Workload: rigid unit sphere as an icosphere at subdivision 5 (10242 nodes,
20480 triangles), ka = 10, a plane wave from the seeded direction, 32 seeded
CHIEF points in r < 0.5, near-singular rule eta = 1, depth 2 (the far kernel
runs its shift phase mode here: k x extent = 34.6).  The oracle assembles 24
node rows at each of three places in the matrix and all 32 CHIEF rows (104
rows; every node row holds its singular pairs and near-singular pairs).
Tolerances as in the assembly tests: c128 1e-10 (near-singular rule active),
c64 2e-6, relative to the largest entry of the sampled rows."""
import argparse

import numpy as np
import pytest

from helpers import rel_err

pytestmark = pytest.mark.gpu

ROW_RANGES = [(0, 24), (5109, 5133), (10218, 10242), (10242, 10274)]


def test_headline_system_sampled_rows_match_oracle(bemlib, orc):
    import bench
    pts, el, chief, d, k, bc = bench.workload(argparse.Namespace(subdiv=5, ka=10.0, chief=32, seed=0))
    srcs = [("plane", d, 1.0)]
    N = pts.shape[0]
    assert N == 10242 and chief.shape[0] == 32
    prm = orc.params(near_eta=1.0, near_depth=2)
    allp = np.vstack([pts, chief])
    ref = [orc.assemble(allp, el, k, N, srcs, bc=bc, prm=prm, rows=r) for r in ROW_RANGES]
    Ao = np.vstack([x[0] for x in ref])
    Bo = np.vstack([x[1] for x in ref])
    idx = np.concatenate([np.arange(*r) for r in ROW_RANGES])
    s = bemlib.Solver(near_eta=1.0, near_depth=2)
    s.set_geometry(pts, el, bc=bc, chief=chief)
    s.set_sources(srcs)
    for prec, tol in ((bemlib.PREC_C128, 1e-10), (bemlib.PREC_C64, 2e-6)):
        s.assemble(k, prec)
        A, B = s.system(bemlib.PREC_C128)
        assert rel_err(A[idx], Ao) < tol, prec
        assert rel_err(B[idx], Bo) < tol, prec
