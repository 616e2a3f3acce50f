"""Multi-right-hand-side solve (BEM_SOLVE_BLOCK_GMRES) and the geometry
generators of the batching configuration: a perturbed triaxial ellipsoid on a
geodesic mesh, point sources on a Fibonacci lattice, checked source by source
against the FP64 solve of the same system (1e-5 relative)."""
import numpy as np
import pytest

from helpers import rel_err, uv_sphere

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


@pytest.mark.parametrize("gemm_mode", [-1, 0, 1, 3, 4, 5, 6])
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


@pytest.mark.parametrize("gemm_mode", [-1, 4, 5, 6])
def test_block_gmres_odd_node_count(bemlib, gemm_mode):
    """3005 nodes (odd: the interleaved and 3M TF32x3 planes and right-hand
    blocks have odd leading dimensions), 5 point sources; AUTO takes the
    interleaved TF32x3 products here.  Against the FP64 solve."""
    p, e = uv_sphere(39, 77)
    assert p.shape[0] % 2 == 1
    m = bemlib.Mesh.from_arrays(p, e)
    m.orient()
    p, e = m.points(), m.elems()
    chief = np.random.default_rng(39).uniform(-0.3, 0.3, (6, 3))
    srcs = [("point", s, 1.0) for s in bemlib.fibonacci_sphere(5, 3.0)]
    s = bemlib.Solver(gemm_mode=gemm_mode, block_tol=1e-8)
    s.set_geometry(p, e, bc=np.tile(np.array([0, 1, 0], dtype=np.complex128), (e.shape[0], 1)), chief=chief)
    s.set_sources(srcs)
    s.assemble(6.0, bemlib.PREC_C128)
    s.solve(bemlib.SOLVE_QR)
    x64 = s.solution()
    s.assemble(6.0, bemlib.PREC_C64)
    info = s.solve(bemlib.SOLVE_BLOCK_GMRES)
    assert info.converged
    xb = s.solution()
    for j in range(xb.shape[1]):
        assert rel_err(xb[:, j], x64[:, j]) < 1e-5, j



@pytest.mark.parametrize("nsrc", [1, 3, 12, 20, 37])
def test_block_simt_source_counts(bemlib, nsrc):
    """The CUDA-core block products (gemm_mode 5) at source counts that leave
    passes partly empty (1, 3 of 4; 12 of 16), take two and three passes (20,
    37), on an odd node count (255) whose row count (263) is not a multiple
    of the kernels' 32-row blocks.  Against the FP64 solve, source by source."""
    p, e = uv_sphere(11, 23)
    assert p.shape[0] % 2 == 1
    m = bemlib.Mesh.from_arrays(p, e)
    m.orient()
    p, e = m.points(), m.elems()
    chief = np.random.default_rng(11).uniform(-0.3, 0.3, (8, 3))
    srcs = [("point", q, 1.0) for q in bemlib.fibonacci_sphere(nsrc, 3.0)]
    s = bemlib.Solver(gemm_mode=5, block_tol=1e-8)
    s.set_geometry(p, e, bc=np.tile(np.array([0, 1, 0], dtype=np.complex128), (e.shape[0], 1)), chief=chief)
    s.set_sources(srcs)
    s.assemble(4.0, bemlib.PREC_C128)
    s.solve(bemlib.SOLVE_QR)
    x64 = s.solution()
    s.assemble(4.0, bemlib.PREC_C64)
    info = s.solve(bemlib.SOLVE_BLOCK_GMRES)
    assert info.converged
    xb = s.solution()
    for j in range(nsrc):
        assert rel_err(xb[:, j], x64[:, j]) < 1e-5, j
    # bitwise reproducible (fixed-order sums, no atomics)
    s.solve(bemlib.SOLVE_BLOCK_GMRES)
    assert np.array_equal(s.solution(), xb)
