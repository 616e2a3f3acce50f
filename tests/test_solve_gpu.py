"""GPU solves, field evaluation and the reference's drop-in calls, against
the FP64 oracle and the analytic sphere solutions (through the C ABI).

Tolerances: FP64 QR 1e-10; refined GMRES (FP32 matvecs inside FP64
refinement) 1e-5 relative surface-pressure error against the FP64 solve of
the same formulation; c64 field evaluation 1e-5."""
import numpy as np
import pytest

from helpers import FIELD_GOLDEN, GOLDEN, K_GOLDEN, chief_candidates, float_bb, golden, icosphere, rel_err, uv_sphere

pytestmark = pytest.mark.gpu


def _rigid_ico(subdiv, n_chief, seed=1):
    p, f = icosphere(subdiv)
    rng = np.random.default_rng(seed)
    u = rng.random((n_chief, 3))
    r = 0.5 * np.cbrt(u[:, 0])
    th = np.arccos(1 - 2 * u[:, 1])
    ph = 2 * np.pi * u[:, 2]
    chief = np.stack([r * np.sin(th) * np.cos(ph), r * np.sin(th) * np.sin(ph), r * np.cos(th)], axis=1)
    bc = np.tile(np.array([0, 1, 0], dtype=np.complex128), (f.shape[0], 1))
    return p, f, chief, bc


def test_refined_solve_zero_rhs(bemlib):
    """A source of zero strength next to a real one: its surface pressure
    is zero (|A^H b| = 0 is recognised with the first inner step's result),
    the other one converges as alone; with no refinement allowed the
    solution stays zero and is reported unconverged."""
    p, f, chief, bc = _rigid_ico(2, 4)
    srcs = [("point", (2.0, 1.0, 0.5), 0.0), ("plane", (0, 0, 1), 1.0)]
    s = bemlib.Solver()
    s.set_geometry(p, f, bc=bc, chief=chief)
    s.set_sources(srcs)
    s.assemble(1.3, bemlib.PREC_C64)
    info = s.solve(bemlib.SOLVE_GMRES_REFINED)
    x = s.solution()
    assert info.converged and np.all(x[:, 0] == 0) and np.all(np.isfinite(x))
    alone = bemlib.Solver()
    alone.set_geometry(p, f, bc=bc, chief=chief)
    alone.set_sources(srcs[1:])
    alone.assemble(1.3, bemlib.PREC_C64)
    alone.solve(bemlib.SOLVE_GMRES_REFINED)
    assert rel_err(x[:, 1], alone.solution()[:, 0]) < 1e-10
    none = bemlib.Solver(max_refine=0)
    none.set_geometry(p, f, bc=bc, chief=chief)
    none.set_sources(srcs[1:])
    none.assemble(1.3, bemlib.PREC_C64)
    info0 = none.solve(bemlib.SOLVE_GMRES_REFINED, check=False)   # BEM_ERR_NOT_CONVERGED, reported in info
    assert not info0.converged and np.all(none.solution() == 0)


def test_qr_c128_matches_oracle(bemlib, orc):
    p, f, chief, bc = _rigid_ico(2, 4)
    srcs = [("plane", (0, 0, 1), 1.0), ("point", (2, 1, 0), 1.0)]
    s = bemlib.Solver()
    s.set_geometry(p, f, bc=bc, chief=chief)
    s.set_sources(srcs)
    s.assemble(1.3, bemlib.PREC_C128)
    s.solve(bemlib.SOLVE_QR)
    x = s.solution()
    Ao, Bo = orc.assemble(np.vstack([p, chief]), f, 1.3, p.shape[0], srcs, bc=bc)
    xo = orc.lsq_qr(Ao, Bo)
    assert rel_err(x, xo) < 1e-10


def test_refined_gmres_icosphere_s3_ka1(bemlib, orc):
    """Rigid unit sphere, icosphere subdivision 3 (642 nodes, 1280
    triangles), plane wave along +z at ka = 1, 8 seeded CHIEF points in
    r < 0.5: mixed-precision solve within 1e-5 of the FP64 solve, and within
    discretisation error of the rigid-sphere series."""
    p, f, chief, bc = _rigid_ico(3, 8)
    srcs = [("plane", (0, 0, 1), 1.0)]
    s = bemlib.Solver()
    s.set_geometry(p, f, bc=bc, chief=chief)
    s.set_sources(srcs)
    s.assemble(1.0, bemlib.PREC_C128)
    s.solve(bemlib.SOLVE_QR)
    x64 = s.solution()[:, 0]
    s.assemble(1.0, bemlib.PREC_C64)
    info = s.solve(bemlib.SOLVE_GMRES_REFINED)
    x = s.solution()[:, 0]
    assert info.converged and info.rel_residual < 1e-8
    assert rel_err(x, x64) < 1e-5
    ref = orc.rigid_sphere_surface(p[:, 2], 1.0)
    assert rel_err(x64, ref) < 1e-2
    Ao, Bo = orc.assemble(np.vstack([p, chief]), f, 1.0, p.shape[0], srcs, bc=bc)
    assert rel_err(x64, orc.lsq_qr(Ao, Bo)[:, 0]) < 1e-10


def test_refined_gmres_multi_source_and_higher_k(bemlib):
    p, f, chief, bc = _rigid_ico(3, 8, seed=2)
    srcs = [("plane", (0, 0, 1), 1.0), ("plane", (0.6, 0, 0.8), 1.0), ("point", (0, 2, 0), 1.0)]
    s = bemlib.Solver()
    s.set_geometry(p, f, bc=bc, chief=chief)
    s.set_sources(srcs)
    s.assemble(4.0, bemlib.PREC_C128)
    s.solve(bemlib.SOLVE_QR)
    x64 = s.solution()
    s.assemble(4.0, bemlib.PREC_C64)
    info = s.solve(bemlib.SOLVE_GMRES_REFINED)
    assert info.converged
    assert rel_err(s.solution(), x64) < 1e-5


def test_qr_c64_close_to_fp64(bemlib):
    p, f, chief, bc = _rigid_ico(2, 4)
    s = bemlib.Solver()
    s.set_geometry(p, f, bc=bc, chief=chief)
    s.set_sources([("plane", (0, 0, 1), 1.0)])
    s.assemble(2.0, bemlib.PREC_C128)
    s.solve(bemlib.SOLVE_QR)
    x64 = s.solution()
    s.assemble(2.0, bemlib.PREC_C64)
    s.solve(bemlib.SOLVE_QR)
    assert rel_err(s.solution(), x64) < 1e-4


@pytest.mark.parametrize("prec,tol", [(0, 1e-5), (1, 1e-10)])
def test_field_matches_oracle(bemlib, orc, prec, tol):
    p, f, chief, bc = _rigid_ico(2, 4)
    srcs = [("plane", (0, 0, 1), 1.0), ("point", (0.0, 3.0, 0.0), 2.0)]
    s = bemlib.Solver()
    s.set_geometry(p, f, bc=bc, chief=chief)
    s.set_sources(srcs)
    s.assemble(1.5, bemlib.PREC_C128)
    s.solve(bemlib.SOLVE_QR)
    x = s.solution()
    rng = np.random.default_rng(5)
    d = rng.standard_normal((37, 3))
    fp = d / np.linalg.norm(d, axis=1)[:, None] * rng.uniform(1.5, 4.0, (37, 1))
    s.assemble(1.5, prec)
    s.solve(bemlib.SOLVE_QR)
    out = s.field(fp)
    ref = orc.field(p, f, 1.5, s.solution(), fp, srcs, bc=bc)
    assert rel_err(out, ref) < tol
    assert rel_err(orc.field(p, f, 1.5, x, fp, srcs, bc=bc), ref) < max(tol, 1e-4)


def test_field_near_surface_eta(bemlib, orc):
    p, f, chief, bc = _rigid_ico(2, 2)
    srcs = [("plane", (0, 0, 1), 1.0)]
    s = bemlib.Solver(near_eta=2.0, near_depth=3)
    s.set_geometry(p, f, bc=bc, chief=chief)
    s.set_sources(srcs)
    s.assemble(1.0, bemlib.PREC_C128)
    s.solve(bemlib.SOLVE_QR)
    fp = np.array([[0, 0, 1.02], [0.5, 0.5, 0.75], [0, -1.5, 0]])
    out = s.field(fp)
    ref = orc.field(p, f, 1.0, s.solution(), fp, srcs, bc=bc, prm=orc.params(near_eta=2.0, near_depth=3))
    assert rel_err(out, ref) < 1e-10


def test_dropin_golden_pipeline(bemlib, orc):
    """The reference's main.cpp sequence through the drop-in calls:
    readObj, findBB(1e-4), genCHIEF(1, 0.1), gaussQuad(6).sendToDevice(),
    bemSystem, qrSolver, genExtPressure at the golden field points; compared
    with the golden file and with the oracle running the same steps."""
    m = bemlib.Mesh()
    m.readObj(f"{GOLDEN}/sphere.obj")
    m.findBB(0.0001)
    m.genCHIEF(1, 0.1)
    pts = m.points()
    ch_o, _ = orc.chief_select(pts, m.elems(), float_bb(pts, 1e-4), 0.1, chief_candidates(), 1)
    np.testing.assert_array_equal(m.chief(), ch_o.astype(np.float32).astype(np.float64))
    bemlib.gaussQuad(6).sendToDevice()
    src = np.array([1e6, 1e6, 1e6])
    A, B = bemlib.bemSystem(m, K_GOLDEN, src)
    Ao, Bo = orc.assemble(np.vstack([pts, m.chief()]), m.elems(), K_GOLDEN, pts.shape[0],
                          [("point", src, 0.0)])
    assert rel_err(A, Ao) < 2e-6 and rel_err(B, Bo) < 2e-6
    bemlib.qrSolver(A, B)
    x = B[:pts.shape[0], 0]
    res = [x[0]] + [bemlib.genExtPressure(K_GOLDEN, m, src, fp, x) for fp in FIELD_GOLDEN]
    res = np.array(res)
    xo = orc.lsq_qr(Ao, Bo)[:, 0]
    reso = np.concatenate([[xo[0]], orc.field(pts, m.elems(), K_GOLDEN, xo, FIELD_GOLDEN,
                                               [("point", src, 0.0)])[:, 0]])
    assert rel_err(res, reso) < 2e-4
    g = golden("sphere171Hz_CHIEF")
    assert (np.abs(res - g) / np.abs(g)).max() < 5e-3


def test_dropin_gmres_square(bemlib, orc):
    """GMRES (GMRES.cu:145-279) on the square no-CHIEF system of test.obj."""
    m = bemlib.Mesh()
    m.readObj(f"{GOLDEN}/test.obj")
    bemlib.set_point_source_strength(1.0)
    try:
        A, B = bemlib.bemSystem(m, 1.1, [3.0, 0.0, 0.0])
    finally:
        bemlib.set_point_source_strength(0.0)
    x = bemlib.GMRES(A, B[:, 0], A.shape[0], 1e-6)
    xd = np.linalg.solve(A.astype(np.complex128), B[:, 0].astype(np.complex128))
    assert rel_err(x, xd) < 1e-5
    xo, it, _ = orc.gmres(A.astype(np.complex128), B[:, 0], A.shape[0], 1e-6)
    assert rel_err(x, xo) < 1e-5
    # a converged initial guess returns unchanged
    x0 = xd.astype(np.complex64)
    x2 = bemlib.GMRES(A, B[:, 0], A.shape[0], 1e-3, x=x0.copy())
    np.testing.assert_array_equal(x2, x0)


def test_dropin_qr_vs_numpy(bemlib):
    rng = np.random.default_rng(9)
    A = (rng.standard_normal((50, 40)) + 1j * rng.standard_normal((50, 40))).astype(np.complex64)
    B = np.asfortranarray((rng.standard_normal((50, 2)) + 1j * rng.standard_normal((50, 2))).astype(np.complex64))
    X = np.linalg.lstsq(A.astype(np.complex128), B.astype(np.complex128), rcond=None)[0]
    bemlib.qrSolver(A, B)
    assert rel_err(B[:40], X) < 1e-4


@pytest.mark.parametrize("nu", [24, 33, 36])
def test_refined_solve_cluster_sizes(bemlib, nu):
    """Refined GMRES on meshes whose node counts need two- and three-CTA
    clusters in the fused A^H A v kernel (5762, 10892 and 12962 nodes),
    against the FP64 solve."""
    m = bemlib.Mesh.geodesic(nu).perturbed_ellipsoid(1.0, 0.8, 0.9, lmax=4, amp=0.03, seed=nu)
    p, e = m.points(), m.elems()
    rng = np.random.default_rng(nu)
    chief = rng.uniform(-0.25, 0.25, (8, 3))
    d = np.array([0.3, -0.5, 0.81])
    src = [("plane", d / np.linalg.norm(d), 1.0)]
    s = bemlib.Solver(near_eta=1.0, near_depth=2)
    s.set_geometry(p, e, bc=np.tile(np.array([0, 1, 0], dtype=np.complex128), (e.shape[0], 1)), chief=chief)
    s.set_sources(src)
    s.assemble(5.0, bemlib.PREC_C128)
    s.solve(bemlib.SOLVE_QR)
    x64 = s.solution()
    s.assemble(5.0, bemlib.PREC_C64)
    info = s.solve(bemlib.SOLVE_GMRES_REFINED)
    assert info.converged
    assert rel_err(s.solution(), x64) < 1e-5


_VARIANT_SCRIPT = r"""
import sys
import numpy as np
sys.path.insert(0, sys.argv[1])
import bem_gpu_clean_cpp_gb300 as bem
m = bem.Mesh.geodesic(33).perturbed_ellipsoid(1.0, 0.8, 0.9, lmax=4, amp=0.03, seed=33)
p, e = m.points(), m.elems()
chief = np.random.default_rng(33).uniform(-0.25, 0.25, (8, 3))
d = np.array([0.3, -0.5, 0.81])
s = bem.Solver(near_eta=1.0, near_depth=2)
s.set_geometry(p, e, bc=np.tile(np.array([0, 1, 0], dtype=np.complex128), (e.shape[0], 1)), chief=chief)
s.set_sources([("plane", d / np.linalg.norm(d), 1.0)])
s.assemble(5.0, bem.PREC_C128)
s.solve(bem.SOLVE_QR)
x64 = s.solution()
s.assemble(5.0, bem.PREC_C64)
info = s.solve(bem.SOLVE_GMRES_REFINED)
err = np.linalg.norm(s.solution() - x64) / np.linalg.norm(x64)
print("RESULT", int(info.converged), err)
"""


@pytest.mark.parametrize("variant", ["regs", "tma"])
def test_normal_op_variants(bemlib, variant):
    """The other two normal-operator kernels, chosen per process by
    BEM_NORMAL_OP_KERNEL (register-loading, and the 512-thread TMA kernel
    with one CTA per SM and two-CTA clusters at 10892 nodes), give a
    refined solve within 1e-5 of the FP64 solve, like the default 256-thread
    one (two CTAs per SM, four-CTA clusters)."""
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ, BEM_NORMAL_OP_KERNEL=variant)
    out = subprocess.run([sys.executable, "-c", _VARIANT_SCRIPT, root], env=env, capture_output=True, text=True,
                         timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    line = [ln for ln in out.stdout.splitlines() if ln.startswith("RESULT")][-1].split()
    assert line[1] == "1" and float(line[2]) < 1e-5, line


def test_refined_solve_odd_node_count(bemlib):
    """7577 nodes (odd): the fused normal operator's second column segment
    has an odd length (1945 columns), so its bulk copy is rounded up into the
    row padding, which must stay masked.  Refined GMRES against the FP64 QR
    solve."""
    p, e = uv_sphere(75, 101)
    assert p.shape[0] == 7577
    m = bemlib.Mesh.from_arrays(p, e)
    m.orient()
    p, e = m.points(), m.elems()
    rng = np.random.default_rng(7577)
    chief = rng.uniform(-0.3, 0.3, (8, 3))
    s = bemlib.Solver(near_eta=1.0, near_depth=2)
    s.set_geometry(p, e, bc=np.tile(np.array([0, 1, 0], dtype=np.complex128), (e.shape[0], 1)), chief=chief)
    s.set_sources([("plane", np.array([0.0, 0.6, 0.8]), 1.0)])
    s.assemble(4.0, bemlib.PREC_C128)
    s.solve(bemlib.SOLVE_QR)
    x64 = s.solution()
    s.assemble(4.0, bemlib.PREC_C64)
    info = s.solve(bemlib.SOLVE_GMRES_REFINED)
    assert info.converged
    assert rel_err(s.solution(), x64) < 1e-5


_STALL_SCRIPT = r"""
import sys
import numpy as np
sys.path.insert(0, sys.argv[1])
import bem_gpu_clean_cpp_gb300 as bem
p, e = bem.Mesh.icosphere(3, 1.0).points(), bem.Mesh.icosphere(3, 1.0).elems()
bc = np.tile(np.array([0, 1, 0], dtype=np.complex128), (e.shape[0], 1))
chief = np.random.default_rng(3).uniform(-0.3, 0.3, (8, 3))
s = bem.Solver(near_eta=1.0, near_depth=2)
s.set_geometry(p, e, bc=bc, chief=chief)
s.set_sources([("plane", np.array([0.0, 0.0, 1.0]), 1.0)])
s.assemble(1.0, bem.PREC_C128)
s.solve(bem.SOLVE_QR)
x64 = s.solution()
s.assemble(1.0, bem.PREC_C64)
status = 0
try:
    s.solve(bem.SOLVE_GMRES_REFINED)
except bem.BemError as err:
    status = err.status
info = s.solve(bem.SOLVE_GMRES_REFINED)
err2 = np.linalg.norm(s.solution() - x64) / np.linalg.norm(x64)
print("RESULT", status, int(info.converged), err2)
"""


def test_normal_op_wait_timeout_reported(bemlib):
    """The TMA normal operator's waits are bounded.  With
    BEM_TEST_NORMAL_OP_STALL=1 the first launch of the process announces 16
    bytes per stage that no copy delivers: every copy completes, no barrier
    phase does, the waits run out after about a second (no fault, no hang),
    and the refined solve reports BEM_ERR_TIMEOUT.  The next solve in the same
    process converges to the FP64 answer: the device stays usable and the
    flag is cleared."""
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ, BEM_TEST_NORMAL_OP_STALL="1")
    out = subprocess.run([sys.executable, "-c", _STALL_SCRIPT, root], env=env, capture_output=True, text=True,
                         timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    line = [ln for ln in out.stdout.splitlines() if ln.startswith("RESULT")][-1].split()
    assert int(line[1]) == bemlib.ERR_TIMEOUT, line
    assert line[2] == "1" and float(line[3]) < 1e-5, line


_STALL_CONCURRENT_SCRIPT = r"""
import sys, threading, time
import numpy as np
sys.path.insert(0, sys.argv[1])
import bem_gpu_clean_cpp_gb300 as bem
def problem(seed, subdiv):
    m = bem.Mesh.icosphere(subdiv, 1.0)
    p, e = m.points(), m.elems()
    bc = np.tile(np.array([0, 1, 0], dtype=np.complex128), (e.shape[0], 1))
    chief = np.random.default_rng(seed).uniform(-0.3, 0.3, (8, 3))
    s = bem.Solver(near_eta=1.0, near_depth=2)
    s.set_geometry(p, e, bc=bc, chief=chief)
    s.set_sources([("plane", np.array([0.0, 0.6, 0.8]), 1.0)])
    s.assemble(1.5, bem.PREC_C128)
    s.solve(bem.SOLVE_QR)
    x64 = s.solution()
    s.assemble(1.5, bem.PREC_C64)
    s.sync()
    return s, x64
a, xa = problem(3, 3)
b, xb = problem(4, 4)
res = {}
def run_a():
    try:
        a.solve(bem.SOLVE_GMRES_REFINED)
        res["a"] = 0
    except bem.BemError as err:
        res["a"] = err.status
t = threading.Thread(target=run_a)
t.start()                # a's first normal-operator launch is the stalled one
time.sleep(0.3)
status_b = 0
try:
    info_b = b.solve(bem.SOLVE_GMRES_REFINED)   # runs while a's launch waits out
except bem.BemError as err:
    status_b = err.status
t.join()
err_b = np.linalg.norm(b.solution() - xb) / np.linalg.norm(xb) if status_b == 0 else 1.0
info_a = a.solve(bem.SOLVE_GMRES_REFINED)
err_a = np.linalg.norm(a.solution() - xa) / np.linalg.norm(xa)
print("RESULT", res["a"], status_b, err_b, int(info_a.converged), err_a)
"""


def test_normal_op_timeout_reported_to_its_own_solver(bemlib):
    """The timeout status is per solver: while one solver's stalled launch
    waits out (BEM_TEST_NORMAL_OP_STALL=1, as above), a second solver in
    another thread solves its own system.  Only the stalled solver reports
    BEM_ERR_TIMEOUT; the other converges to its FP64 answer, and the stalled
    one converges on its next solve."""
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ, BEM_TEST_NORMAL_OP_STALL="1")
    out = subprocess.run([sys.executable, "-c", _STALL_CONCURRENT_SCRIPT, root], env=env, capture_output=True,
                         text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    line = [ln for ln in out.stdout.splitlines() if ln.startswith("RESULT")][-1].split()
    assert int(line[1]) == bemlib.ERR_TIMEOUT, line
    assert int(line[2]) == 0 and float(line[3]) < 1e-5, line
    assert line[4] == "1" and float(line[5]) < 1e-5, line


@pytest.mark.parametrize("mesh", ["geodesic50", "icosphere6"])
def test_normal_op_large_clusters(bemlib, mesh):
    """The fused normal operator with five- and eight-CTA clusters (25002 and
    40962 nodes, where an FP64 QR reference would take minutes): the refined
    GMRES solution (normal-operator products) agrees with the block GMRES
    solution of the same c64 system for one source (cuBLAS products, no
    normal operator) to 1e-6."""
    if mesh == "geodesic50":
        m = bemlib.Mesh.geodesic(50).perturbed_ellipsoid(1.0, 0.85, 0.9, lmax=4, amp=0.03, seed=50)
    else:
        m = bemlib.Mesh.icosphere(6, 1.0)
    p, e = m.points(), m.elems()
    chief = np.random.default_rng(6).uniform(-0.3, 0.3, (8, 3))
    s = bemlib.Solver(near_eta=1.0, near_depth=2, block_tol=1e-8)
    s.set_geometry(p, e, bc=np.tile(np.array([0, 1, 0], dtype=np.complex128), (e.shape[0], 1)), chief=chief)
    s.set_sources([("plane", np.array([0.36, 0.48, 0.8]), 1.0)])
    s.assemble(3.0, bemlib.PREC_C64)
    info = s.solve(bemlib.SOLVE_GMRES_REFINED)
    assert info.converged
    xr = s.solution()
    info = s.solve(bemlib.SOLVE_BLOCK_GMRES)
    assert info.converged
    assert rel_err(xr, s.solution()) < 1e-6
