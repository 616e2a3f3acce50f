"""GPU assembly parity against the FP64 oracle, through the C ABI.

Tolerances: c128 (FP64 everywhere) 1e-11 relative to the largest entry;
c64 (FP32 regular quadrature, FP64 singular/near pairs, c64 storage) 2e-6.
"""
import numpy as np
import pytest

from helpers import GOLDEN, icosphere, rel_err

pytestmark = pytest.mark.gpu

TOL64 = 1e-11
TOL32 = 2e-6


def _problem(kind):
    if kind == "test.obj":
        import oracle
        p, f = oracle.read_obj_reference(f"{GOLDEN}/test.obj")
        p = p.astype(np.float64)
        chief = np.array([[0.1, 0.05, -0.2], [-0.15, 0.2, 0.1]])
    elif kind == "cube.obj":
        import oracle
        p, f = oracle.read_obj_reference(f"{GOLDEN}/cube.obj")
        p = p.astype(np.float64)
        chief = np.array([[0.2, -0.1, 0.3]])
    else:
        p, f = icosphere(2, 0.7)
        chief = np.array([[0.1, 0.05, -0.2], [-0.15, 0.2, 0.1], [0.0, 0.0, 0.25]])
    return p, f, chief


SRCS = [("plane", (0.0, 0.6, 0.8), 1.0), ("point", (3.0, -1.0, 0.5), 2.0 - 1.0j)]


def _bc(bckind, E):
    """default: None, the BC (0, 1, -1) (alpha = 0, gamma != 0: the FP32 far
    kernel forms the S0 sums of G only); rigid: (0, 1, 0) (no G sums at
    all); impedance: random alpha, beta, gamma per element (all G sums)."""
    if bckind == "default":
        return None
    if bckind == "rigid":
        return np.tile(np.array([0, 1, 0], dtype=np.complex128), (E, 1))
    rng = np.random.default_rng(7)
    return np.stack([0.3 + 0.1j * rng.random(E), 1.0 + 0.2j * rng.random(E), -1.0 + 0.5j * rng.random(E)], axis=1)


@pytest.mark.parametrize("kind", ["test.obj", "cube.obj", "ico2"])
@pytest.mark.parametrize("bckind", ["default", "rigid", "impedance"])
def test_c128_assembly_matches_oracle(bemlib, orc, kind, bckind):
    p, f, chief = _problem(kind)
    bc = _bc(bckind, f.shape[0])
    k = 2.3
    s = bemlib.Solver()
    s.set_geometry(p, f, bc=bc, chief=chief)
    s.set_sources(SRCS)
    s.assemble(k, bemlib.PREC_C128)
    A, B = s.system(bemlib.PREC_C128)
    Ao, Bo = orc.assemble(np.vstack([p, chief]), f, k, p.shape[0], SRCS, bc=bc)
    assert rel_err(A, Ao) < TOL64
    assert rel_err(B, Bo) < TOL64


@pytest.mark.parametrize("kind", ["test.obj", "ico2"])
@pytest.mark.parametrize("bckind", ["default", "rigid", "impedance"])
def test_c64_assembly_matches_oracle(bemlib, orc, kind, bckind):
    p, f, chief = _problem(kind)
    bc = _bc(bckind, f.shape[0])
    k = 4.0
    s = bemlib.Solver()
    s.set_geometry(p, f, bc=bc, chief=chief)
    s.set_sources(SRCS)
    s.assemble(k, bemlib.PREC_C64)
    A, B = s.system(bemlib.PREC_C128)
    Ao, Bo = orc.assemble(np.vstack([p, chief]), f, k, p.shape[0], SRCS, bc=bc)
    assert rel_err(A, Ao) < TOL32
    assert rel_err(B, Bo) < TOL32


@pytest.mark.parametrize("eta,depth", [(1.5, 2), (3.0, 3)])
def test_near_singular_assembly_matches_oracle(bemlib, orc, eta, depth):
    p, f, chief = _problem("ico2")
    chief = np.vstack([chief, [[0.0, 0.0, 0.66]]])    # a CHIEF point close to the surface
    k = 3.0
    s = bemlib.Solver(near_eta=eta, near_depth=depth)
    s.set_geometry(p, f, chief=chief)
    s.set_sources(SRCS)
    s.assemble(k, bemlib.PREC_C128)
    A, B = s.system(bemlib.PREC_C128)
    prm = orc.params(near_eta=eta, near_depth=depth)
    Ao, Bo = orc.assemble(np.vstack([p, chief]), f, k, p.shape[0], SRCS, prm=prm)
    assert rel_err(A, Ao) < 1e-10
    assert rel_err(B, Bo) < 1e-10
    s.assemble(k, bemlib.PREC_C64)
    A32, _ = s.system(bemlib.PREC_C128)
    assert rel_err(A32, Ao) < TOL32


@pytest.mark.parametrize("variant", [0, 1, 2, 3, 4, 5, 6])
@pytest.mark.parametrize("order", [6, 5])
def test_far_kernel_launch_shapes(bemlib, orc, variant, order):
    """Every far-kernel launch shape (and both the unrolled 6x6 path and the
    generic Gauss loop) gives the oracle's matrix."""
    p, f, chief = _problem("ico2")
    s = bemlib.Solver(far_variant=variant, order=order)
    s.set_geometry(p, f, chief=chief)
    s.set_sources(SRCS)
    s.assemble(5.0, bemlib.PREC_C64)
    A, B = s.system(bemlib.PREC_C128)
    Ao, Bo = orc.assemble(np.vstack([p, chief]), f, 5.0, p.shape[0], SRCS, prm=orc.params(order=order))
    assert rel_err(A, Ao) < TOL32 and rel_err(B, Bo) < TOL32


def test_quadrature_order(bemlib, orc):
    p, f, chief = _problem("test.obj")
    s = bemlib.Solver(order=4)
    s.set_geometry(p, f, chief=chief)
    s.set_sources(SRCS)
    s.assemble(1.5, bemlib.PREC_C128)
    A, B = s.system(bemlib.PREC_C128)
    Ao, Bo = orc.assemble(np.vstack([p, chief]), f, 1.5, p.shape[0], SRCS, prm=orc.params(order=4))
    assert rel_err(A, Ao) < TOL64 and rel_err(B, Bo) < TOL64


@pytest.mark.parametrize("prec", [0, 1])
def test_multi_tile_assembly(bemlib, orc, prec):
    """Column tiles narrower than N: Morton-ordered tiles, elements straddling
    tiles integrated once per tile, c/beta counted in the owner tile only."""
    p, f = icosphere(3, 1.0)                   # 642 nodes
    chief = np.array([[0.1, 0.2, -0.3]])
    s = bemlib.Solver(tile_cols=100)           # 7 tiles
    s.set_geometry(p, f, chief=chief)
    s.set_sources(SRCS)
    s.assemble(3.0, prec)
    A, B = s.system(bemlib.PREC_C128)
    Ao, Bo = orc.assemble(np.vstack([p, chief]), f, 3.0, p.shape[0], SRCS)
    tol = TOL32 if prec == 0 else TOL64
    assert rel_err(A, Ao) < tol and rel_err(B, Bo) < tol


@pytest.mark.parametrize("tile_cols", [0, 100])
def test_assembly_bitwise_repeatable(bemlib, tile_cols):
    """The far kernels add each column's terms in one fixed order (records in
    node-disjoint batches, plain shared-memory adds, a CTA barrier between
    batches; no atomics), so repeated assemblies give the same bits: c64 with
    every launch shape of the far kernel, and c128, with one column tile and
    with several (tile_cols = 100 on 162 nodes).  The off-diagonal entries
    are also bitwise the same across launch shapes; only the diagonal's c sum
    and B's beta sum follow the shape's reduction tree."""
    p, f, chief = _problem("ico2")
    n = p.shape[0]
    ref_off = None
    for v in range(7):
        s = bemlib.Solver(far_variant=v, tile_cols=tile_cols)
        s.set_geometry(p, f, chief=chief)
        s.set_sources(SRCS)
        s.assemble(2.0, bemlib.PREC_C64)
        A1, B1 = s.system(bemlib.PREC_C64)
        s.assemble(2.0, bemlib.PREC_C64)
        A2, B2 = s.system(bemlib.PREC_C64)
        assert np.array_equal(A1, A2) and np.array_equal(B1, B2), v
        off = A1.copy()
        off[np.arange(n), np.arange(n)] = 0
        if ref_off is None:
            ref_off = off
        else:
            assert np.array_equal(off, ref_off), v
    s = bemlib.Solver(tile_cols=tile_cols)
    s.set_geometry(p, f, chief=chief)
    s.set_sources(SRCS)
    s.assemble(2.0, bemlib.PREC_C128)
    A1, B1 = s.system(bemlib.PREC_C128)
    s.assemble(2.0, bemlib.PREC_C128)
    A2, B2 = s.system(bemlib.PREC_C128)
    assert np.array_equal(A1, A2) and np.array_equal(B1, B2)


def test_errors_are_status_codes(bemlib):
    s = bemlib.Solver()
    with pytest.raises(bemlib.BemError) as e:
        s.assemble(1.0)
    assert e.value.status == 7
    p, f, _ = _problem("test.obj")
    s.set_geometry(p, f)
    with pytest.raises(bemlib.BemError) as e:
        s.assemble(1.0)                       # no sources
    assert e.value.status == 7
    s.set_sources([("plane", (0, 0, 1), 1.0)])
    with pytest.raises(bemlib.BemError) as e:
        s.assemble(-1.0)
    assert e.value.status == 2
    with pytest.raises(bemlib.BemError):
        s.solve()                             # nothing assembled


@pytest.mark.parametrize("prec", [0, 1])
def test_new_sources_reuse_assembly(bemlib, prec):
    """set_sources on an assembled system rebuilds B = p_inc - beta only; it
    equals a full assembly with those sources, and A is unchanged."""
    p, e, chief = _problem("ico2")
    k = 2.0
    bc = np.tile(np.array([0.3 + 0.1j, 1.0, 0.7 - 0.2j]), (e.shape[0], 1))   # cc != 0: beta matters
    s1 = [("point", (2.0, 0.5, -1.0), 1.0)]
    s2 = [("plane", (0.0, 0.6, 0.8), 1.0), ("point", (-1.5, 2.0, 0.3), 0.5 - 0.2j)]
    a = bemlib.Solver()
    a.set_geometry(p, e, bc=bc, chief=chief)
    a.set_sources(s1)
    a.assemble(k, prec)
    A1, _ = a.system()
    a.set_sources(s2)
    A2, B2 = a.system()
    b = bemlib.Solver()
    b.set_geometry(p, e, bc=bc, chief=chief)
    b.set_sources(s2)
    b.assemble(k, prec)
    Ab, Bb = b.system()
    assert rel_err(B2, Bb) < 1e-14
    assert np.array_equal(A1, A2)
    assert rel_err(A2, Ab) < (1e-14 if prec == 1 else 1e-6)


@pytest.mark.parametrize("radius,k,mode", [(0.7, 4.0, "wrap"), (0.7, 7.0, "split"), (1.0, 25.0, "split"),
                                           (0.6, 30.0, "split")])
def test_c64_phase_modes_match_oracle(bemlib, orc, radius, k, mode):
    """The FP32 quadrature's phase modes: per-point wrap (k times the longest
    edge in (0.75, 1.2]) and the split accurate phase with the polynomial
    sin/cos (k times the extent above 40 or k times the longest edge above
    1.2), on coarse meshes where kr reaches ~90, against the FP64 oracle."""
    p, f = icosphere(2, radius)
    chief = np.array([[0.1, 0.05, -0.2], [-0.15, 0.2, 0.1]]) * radius
    edge = max(np.linalg.norm(p[f[:, a]] - p[f[:, b]], axis=1).max() for a, b in ((0, 1), (1, 2), (2, 0)))
    extent = np.linalg.norm(np.ptp(np.vstack([p, chief]), axis=0))
    assert k * edge > 0.75 and ((k * extent > 40 or k * edge > 1.2) == (mode == "split"))
    s = bemlib.Solver()
    s.set_geometry(p, f, chief=chief)
    s.set_sources(SRCS)
    s.assemble(k, bemlib.PREC_C64)
    A, B = s.system(bemlib.PREC_C128)
    Ao, Bo = orc.assemble(np.vstack([p, chief]), f, k, p.shape[0], SRCS)
    assert rel_err(A, Ao) < TOL32
    assert rel_err(B, Bo) < TOL32


def test_c64_assembly_high_aspect_elements(bemlib, orc):
    """Obtuse, high-aspect-ratio elements (an icosphere stretched 8:1, aspect
    ratios up to about 10): the far kernel's line coefficients of r^2 lose
    precision there (a cancellation of about (|e1| / h)^2 ulps in |v|^2), yet
    the c64 matrix stays within the c64 tolerance of the FP64 oracle."""
    p, f = icosphere(2, 1.0)
    p = p * np.array([0.25, 0.25, 2.0])
    chief = np.array([[0.05, 0.0, 0.9], [-0.05, 0.02, -1.1]])
    e = np.stack([np.linalg.norm(p[f[:, a]] - p[f[:, b]], axis=1) for a, b in ((0, 1), (1, 2), (2, 0))], axis=1)
    assert (e.max(axis=1) / e.min(axis=1)).max() > 6.0
    k = 2.0
    s = bemlib.Solver()
    s.set_geometry(p, f, chief=chief)
    s.set_sources(SRCS)
    s.assemble(k, bemlib.PREC_C64)
    A, B = s.system(bemlib.PREC_C128)
    Ao, Bo = orc.assemble(np.vstack([p, chief]), f, k, p.shape[0], SRCS)
    assert rel_err(A, Ao) < TOL32
    assert rel_err(B, Bo) < TOL32
