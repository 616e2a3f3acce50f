"""Least squares by this library's blocked Householder QR (BEM_SOLVE_QR_TC):
FP32 panels factored by a thread-block cluster, trailing updates on the
tcgen05 tensor cores, then FP64 refinement (semi-normal equations).

Tolerances: c128 assembly, 1e-10 against the oracle's FP64 Householder least
squares (the bar of the FP64 QR path); c64 assembly, 1e-9 against the FP64
least-squares solution of the same c64 matrix (numpy), i.e. the refinement
reaches FP64 accuracy whatever the factor's precision.  Shapes: 162 nodes
(two panels, the second 34 columns wide), 642 nodes (config 1: ka = 1, 8
CHIEF points), 2562 nodes (21 panels, a ragged last one), several
right-hand sides."""
import numpy as np
import pytest

from helpers import icosphere, rel_err

pytestmark = pytest.mark.gpu


def _problem(subdiv, n_chief, seed=1):
    p, f = icosphere(subdiv)
    rng = np.random.default_rng(seed)
    u = rng.random((n_chief, 3))
    r = 0.5 * np.cbrt(u[:, 0])
    th = np.arccos(1 - 2 * u[:, 1])
    ph = 2 * np.pi * u[:, 2]
    chief = np.stack([r * np.sin(th) * np.cos(ph), r * np.sin(th) * np.sin(ph), r * np.cos(th)], axis=1)
    bc = np.tile(np.array([0, 1, 0], dtype=np.complex128), (f.shape[0], 1))
    return p, f, chief, bc


@pytest.mark.parametrize("subdiv,n_chief,k", [(2, 4, 1.3), (3, 8, 1.0), (4, 16, 5.0)])
def test_qr_tc_c128_matches_oracle(bemlib, orc, subdiv, n_chief, k):
    p, f, chief, bc = _problem(subdiv, n_chief)
    srcs = [("plane", (0, 0, 1), 1.0), ("point", (2, 1, 0), 1.0 - 0.5j)]
    s = bemlib.Solver()
    s.set_geometry(p, f, bc=bc, chief=chief)
    s.set_sources(srcs)
    s.assemble(k, bemlib.PREC_C128)
    info = s.solve(bemlib.SOLVE_QR_TC)
    assert info.converged, (info.refinements, info.rel_residual)
    x = s.solution()
    if subdiv <= 3:
        Ao, Bo = orc.assemble(np.vstack([p, chief]), f, k, p.shape[0], srcs, bc=bc)
        xo = orc.lsq_qr(Ao, Bo)
    else:
        A, B = s.system(bemlib.PREC_C128)
        xo = np.linalg.lstsq(A, B, rcond=None)[0]
    assert rel_err(x, xo) < 1e-10
    # the FP64 QR path (cuSOLVER, the reference's sequence) agrees too
    s.solve(bemlib.SOLVE_QR)
    assert rel_err(x, s.solution()) < 1e-10


@pytest.mark.parametrize("subdiv,n_chief", [(2, 3), (3, 8)])
def test_qr_tc_c64_reaches_fp64_solution_of_c64_system(bemlib, subdiv, n_chief):
    p, f, chief, bc = _problem(subdiv, n_chief, seed=5)
    srcs = [("plane", (0.6, 0, 0.8), 1.0), ("plane", (0, 1, 0), 2.0), ("point", (0, 0, 3), 1.0)]
    s = bemlib.Solver()
    s.set_geometry(p, f, bc=bc, chief=chief)
    s.set_sources(srcs)
    s.assemble(2.5, bemlib.PREC_C64)
    info = s.solve(bemlib.SOLVE_QR_TC)
    assert info.converged
    A, B = s.system(bemlib.PREC_C128)    # the c64 matrix, widened
    xo = np.linalg.lstsq(A, B, rcond=None)[0]
    assert rel_err(s.solution(), xo) < 1e-9


def test_qr_tc_repeatable(bemlib):
    p, f, chief, bc = _problem(3, 8)
    s = bemlib.Solver()
    s.set_geometry(p, f, bc=bc, chief=chief)
    s.set_sources([("plane", (0, 0, 1), 1.0)])
    s.assemble(1.0, bemlib.PREC_C128)
    s.solve(bemlib.SOLVE_QR_TC)
    x1 = s.solution()
    s.solve(bemlib.SOLVE_QR_TC)
    assert np.array_equal(x1, s.solution())
