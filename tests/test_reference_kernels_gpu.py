"""The reference's own assembly kernels and QR sequence, run on this GPU
(oracle/_ref: compiled from the reference sources, launched as
atomicGenSystem and qrSolver do), against the FP64 oracle and the engine.

This pins the oracle to the reference itself: the reference computes in
FP32 with -use_fast_math, so agreement is at FP32 level (2e-5 relative to the
largest entry), and the engine's c64 assembly agrees with both."""
import numpy as np
import pytest

from helpers import FIELD_GOLDEN, GOLDEN, K_GOLDEN, chief_candidates, float_bb, golden, icosphere, rel_err

pytestmark = pytest.mark.gpu

TOL_REF = 2e-5


@pytest.fixture(scope="module")
def refk():
    from oracle import ref, ref_build
    ref_build.build_if_possible()
    if not ref.available():
        pytest.skip("reference kernel cubin not built (needs the reference sources where the tree was built)")
    return ref


def _case(orc, name):
    if name == "ico2":
        p, f = icosphere(2)
        p = p.astype(np.float32)
        chief = np.array([[0.1, 0.05, -0.2], [-0.15, 0.2, 0.1], [0.0, 0.0, 0.25]], dtype=np.float32)
        return p, f, chief, 2.2, [(2.0, 0.3, -0.5)], 1.0
    p, f = orc.read_obj_reference(f"{GOLDEN}/{name}")
    chief = np.zeros((0, 3), dtype=np.float32)
    if name == "sphere.obj":
        ch, _ = orc.chief_select(p.astype(np.float64), f, float_bb(p, 1e-4), 0.1, chief_candidates(), 1)
        chief = ch.astype(np.float32)
    return p, f, chief, K_GOLDEN if name == "sphere.obj" else 1.7, [(1e6, 1e6, 1e6)], 0.0


@pytest.mark.parametrize("name", ["test.obj", "cube.obj", "sphere.obj", "ico2"])
def test_reference_kernels_vs_oracle_and_engine(bemlib, orc, refk, name):
    p, f, chief, k, srcs, q = _case(orc, name)
    rows = np.vstack([p, chief]).astype(np.float32)
    A_ref, B_ref, _ = refk.assemble(rows, f, p.shape[0], k, srcs=srcs, strength=q)
    osrc = [("point", s, q) for s in srcs]
    A_o, B_o = orc.assemble(rows.astype(np.float64), f, k, p.shape[0], osrc)
    assert rel_err(A_ref, A_o) < TOL_REF
    assert rel_err(B_ref, B_o) < TOL_REF or np.abs(B_o).max() == 0
    s = bemlib.Solver()
    s.set_geometry(p.astype(np.float64), f, chief=chief.astype(np.float64) if chief.size else None)
    s.set_sources(osrc)
    s.assemble(k, bemlib.PREC_C64)
    A_e, B_e = s.system(bemlib.PREC_C128)
    assert rel_err(A_e, A_ref) < TOL_REF
    assert rel_err(B_e, B_ref) < TOL_REF or np.abs(B_ref).max() == 0


def test_reference_pipeline_on_golden_case(orc, refk):
    """main.cpp's configuration with the reference's kernels and QR on this
    GPU, against its committed golden output and the FP64 oracle."""
    p, f, chief, k, srcs, q = _case(orc, "sphere.obj")
    rows = np.vstack([p, chief]).astype(np.float32)
    A, B, _ = refk.assemble(rows, f, p.shape[0], k)
    x, _ = refk.qr(A, B)
    x = x[:, 0]
    A_o, B_o = orc.assemble(rows.astype(np.float64), f, k, p.shape[0], [("point", (1e6, 1e6, 1e6), 0.0)])
    x_o = orc.lsq_qr(A_o, B_o)[:, 0]
    assert rel_err(x, x_o) < 1e-4
    g = golden("sphere171Hz_CHIEF")
    assert abs(x[0] - g[0]) / abs(g[0]) < 5e-3
