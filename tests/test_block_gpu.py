"""Multi-right-hand-side solve (BEM_SOLVE_BLOCK_GMRES) and the geometry
generators of the batching configuration: a perturbed triaxial ellipsoid on a
geodesic mesh, point sources on a Fibonacci lattice, checked source by source
against the FP64 solve of the same system (1e-5 relative)."""
import numpy as np
import pytest

from helpers import rel_err

pytestmark = pytest.mark.gpu


def _ellipsoid_problem(bemlib, nu=8, nsrc=16, f_hz=4000.0, seed=3):
    m = bemlib.Mesh.geodesic(nu).perturbed_ellipsoid(0.075, 0.09, 0.11, lmax=8, amp=0.05, seed=seed)
    p, e = m.points(), m.elems()
    rng = np.random.default_rng(seed)
    u = rng.random((8, 3))
    r = 0.03 * np.cbrt(u[:, 0])
    th = np.arccos(1 - 2 * u[:, 1])
    ph = 2 * np.pi * u[:, 2]
    chief = np.stack([r * np.sin(th) * np.cos(ph), r * np.sin(th) * np.sin(ph), r * np.cos(th)], axis=1)
    src = bemlib.fibonacci_sphere(nsrc, 1.0)
    srcs = [("point", s, 1.0) for s in src]
    bc = np.tile(np.array([0, 1, 0], dtype=np.complex128), (e.shape[0], 1))
    k = 2 * np.pi * f_hz / 343.21
    return p, e, chief, srcs, bc, k


@pytest.mark.parametrize("gemm_mode", [-1, 0, 1, 3, 4])
def test_block_gmres_matches_fp64(bemlib, gemm_mode):
    p, e, chief, srcs, bc, k = _ellipsoid_problem(bemlib)
    s = bemlib.Solver(gemm_mode=gemm_mode, block_tol=1e-8)
    s.set_geometry(p, e, bc=bc, chief=chief)
    s.set_sources(srcs)
    s.assemble(k, bemlib.PREC_C128)
    s.solve(bemlib.SOLVE_QR)
    x64 = s.solution()
    s.assemble(k, bemlib.PREC_C64)
    info = s.solve(bemlib.SOLVE_BLOCK_GMRES)
    xb = s.solution()
    assert info.converged and info.rel_residual <= 1e-8
    for j in range(xb.shape[1]):
        assert rel_err(xb[:, j], x64[:, j]) < 1e-5, j
    # same answer as solving the sources one by one with the refined solver
    s.solve(bemlib.SOLVE_GMRES_REFINED)
    assert rel_err(s.solution(), xb) < 1e-5


def test_block_gmres_tf32_mode_runs(bemlib):
    """TF32 products are below FP32 accuracy; the solve still returns a
    usable answer (its residual floor is reported, not hidden)."""
    p, e, chief, srcs, bc, k = _ellipsoid_problem(bemlib, nsrc=4)
    s = bemlib.Solver(gemm_mode=2, block_tol=1e-6, max_refine=3)
    s.set_geometry(p, e, bc=bc, chief=chief)
    s.set_sources(srcs)
    s.assemble(k, bemlib.PREC_C128)
    s.solve(bemlib.SOLVE_QR)
    x64 = s.solution()
    s.assemble(k, bemlib.PREC_C64)
    info = s.solve(bemlib.SOLVE_BLOCK_GMRES, check=False)
    assert rel_err(s.solution(), x64) < 1e-2
    assert info.rel_residual < 1e-2
