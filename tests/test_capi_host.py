"""C ABI library: loads, exports every declared symbol, and the host-only
logic (mesh readers, generators, bounding box, quadrature, output format)
agrees with the oracle.  No GPU compute is called here."""
import os
import re

import numpy as np
import pytest

from helpers import GOLDEN, ROOT, icosphere


def _declared_symbols():
    text = open(os.path.join(ROOT, "include", "bem_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(bem_[a-z0-9_]+)\s*\(", text)))


def test_every_declared_symbol_is_exported(bemlib):
    syms = _declared_symbols()
    assert len(syms) >= 40
    L = bemlib.lib()
    missing = [s for s in syms if not hasattr(L, s)]
    assert not missing, missing
    # the Python binding table covers the header exactly
    assert sorted(bemlib.SIGNATURES) == syms


def test_status_strings(bemlib):
    L = bemlib.lib()
    assert L.bem_status_string(0) == b"success"
    assert L.bem_status_string(1) == b"failure"
    assert L.bem_version() >= 10000


def test_gauss_legendre_matches_oracle(bemlib, orc):
    for n in (1, 4, 6, 12):
        x, w = bemlib.gauss_legendre(n)
        xo, wo = orc.gauss_legendre(n)
        np.testing.assert_allclose(x, xo, atol=1e-15)
        np.testing.assert_allclose(w, wo, atol=1e-15)
    with pytest.raises(bemlib.BemError) as e:
        bemlib.gauss_legendre(13)
    assert e.value.status == 2


@pytest.mark.parametrize("name", ["sphere.obj", "test.obj", "cube.obj"])
def test_read_obj_reference_semantics(bemlib, orc, name):
    m = bemlib.Mesh()
    assert m.readObj(f"{GOLDEN}/{name}") == 0
    p, f = orc.read_obj_reference(f"{GOLDEN}/{name}")
    assert m.counts() == (p.shape[0], f.shape[0], 0)
    np.testing.assert_array_equal(m.points(), p.astype(np.float64))
    np.testing.assert_array_equal(m.elems(), f)


def test_read_obj_quirks(bemlib, orc, tmp_path):
    """vn lines count as vertices and 'f a/b/c' keeps the first integer of
    the first field only, as the reference's sscanf parse does; the robust
    reader handles both."""
    path = tmp_path / "q.obj"
    path.write_text("v 0 0 0\nv 1 0 0\nv 0 1 0\nv 0 0 1\nvn 0 0 1\n"
                    "f 1 2 3\nf 1/1/1 2/2/2 4/4/4\nf -4 -3 -1\n" +
                    "v " + " ".join(["0.5"] * 3) + "   " + "#" * 60 + "\n")
    m = bemlib.Mesh()
    m.readObj(str(path))
    p, f = orc.read_obj_reference(str(path))
    assert m.counts()[:2] == (p.shape[0], f.shape[0])
    np.testing.assert_array_equal(m.elems(), f)
    r = bemlib.Mesh()
    r.read_obj_robust(str(path))
    assert r.counts()[:2] == (5, 3)
    np.testing.assert_array_equal(r.elems(), [[0, 1, 2], [0, 1, 3], [0, 1, 3]])   # -k counts v lines seen so far


def test_read_obj_errors(bemlib, tmp_path):
    m = bemlib.Mesh()
    with pytest.raises(bemlib.BemError) as e:
        m.readObj(str(tmp_path / "missing.obj"))
    assert e.value.status == 6
    bad = tmp_path / "bad.obj"
    bad.write_text("v 0 0 0\nv 1 0 0\nf 1 2 9\n")
    with pytest.raises(bemlib.BemError):
        m.read_obj_robust(str(bad))
    empty = bemlib.Mesh()
    with pytest.raises(bemlib.BemError) as e:
        empty.findBB(0.1)
    assert e.value.status == 7


@pytest.mark.parametrize("s", [0, 1, 2, 3])
def test_icosphere_generator(bemlib, s):
    m = bemlib.Mesh.icosphere(s, 2.0)
    n, e, _ = m.counts()
    assert (n, e) == (10 * 4 ** s + 2, 20 * 4 ** s)
    p, f = m.points(), m.elems()
    np.testing.assert_allclose(np.linalg.norm(p, axis=1), 2.0, rtol=1e-14)
    nrm = np.cross(p[f[:, 0]] - p[f[:, 2]], p[f[:, 1]] - p[f[:, 2]])
    assert np.all(np.einsum("ij,ij->i", nrm, p[f].mean(axis=1)) < 0)     # inward winding
    pt, ft = icosphere(s, 2.0)
    assert abs(m.surface_area() - 0.5 * np.linalg.norm(
        np.cross(pt[ft[:, 0]] - pt[ft[:, 2]], pt[ft[:, 1]] - pt[ft[:, 2]]), axis=1).sum()) < 1e-10


def test_find_bb_float(bemlib):
    from helpers import float_bb
    m = bemlib.Mesh()
    m.readObj(f"{GOLDEN}/sphere.obj")
    m.findBB(1e-4)
    np.testing.assert_array_equal(m.bb(), float_bb(m.points(), 1e-4).astype(np.float32))


def test_set_and_bc_validation(bemlib):
    m = bemlib.Mesh()
    with pytest.raises(bemlib.BemError) as e:
        m.set([[0, 0, 0], [1, 0, 0], [0, 1, 0]], [[0, 1, 5]])
    assert e.value.status == 2
    m.set([[0, 0, 0], [1, 0, 0], [0, 1, 0]], [[0, 1, 2]])
    with pytest.raises(bemlib.BemError):
        m.set_uniform_bc(0, 0, 1)          # cb = 0
    m.set_uniform_bc(0, 1, 0)
    m.set_chief([[0.1, 0.1, 0.1]])
    assert m.counts() == (3, 1, 1)


def test_wrtcplxmat_format(bemlib, tmp_path):
    a = np.array([[1 + 2j, -0.5j], [3.25 - 1j, 0]], dtype=np.complex64)
    out = tmp_path / "m.txt"
    bemlib.wrtCplxMat(a, str(out))
    assert out.read_text() == ("(1.000000,2.000000) (-0.000000,-0.500000) \n"
                               "(3.250000,-1.000000) (0.000000,0.000000) \n") or \
        out.read_text() == ("(1.000000,2.000000) (0.000000,-0.500000) \n"
                            "(3.250000,-1.000000) (0.000000,0.000000) \n")


def test_geodesic_and_ellipsoid_generators(bemlib):
    for nu in (1, 3, 8):
        m = bemlib.Mesh.geodesic(nu)
        assert m.counts()[:2] == (10 * nu * nu + 2, 20 * nu * nu)
    m = bemlib.Mesh.geodesic(12).perturbed_ellipsoid(0.075, 0.09, 0.11, 8, 0.05, 7)
    p, f = m.points(), m.elems()
    # radial perturbation at most 5% of the ellipsoid radius in that direction
    u = p / np.linalg.norm(p, axis=1)[:, None]
    base = 1.0 / np.sqrt((u[:, 0] / 0.075) ** 2 + (u[:, 1] / 0.09) ** 2 + (u[:, 2] / 0.11) ** 2)
    ratio = np.linalg.norm(p, axis=1) / base
    assert abs(np.abs(ratio - 1).max() - 0.05) < 1e-9
    n = np.cross(p[f[:, 0]] - p[f[:, 2]], p[f[:, 1]] - p[f[:, 2]])
    assert np.all(np.einsum("ij,ij->i", n, p[f].mean(axis=1)) < 0)
    pts = bemlib.fibonacci_sphere(256, 1.0)
    np.testing.assert_allclose(np.linalg.norm(pts, axis=1), 1.0, rtol=1e-14)
    assert abs(pts[:, 2].mean()) < 1e-12


def test_server_host_checks(bemlib):
    """Server options and argument checks that run before any device work."""
    import ctypes
    L = bemlib.lib()
    o = bemlib.ServerOptions()
    assert L.bem_server_options_default(ctypes.byref(o)) == 0
    assert (o.slots, o.cache_systems, o.block_min_sources) == (4, 8, 4)
    assert o.solver.max_iter == 300 and o.solver.order == 6
    h = ctypes.c_void_p()
    bad = bemlib.ServerOptions.from_buffer_copy(o)
    bad.slots = 0
    assert L.bem_server_create(ctypes.byref(bad), ctypes.byref(h)) == 2
    bad = bemlib.ServerOptions.from_buffer_copy(o)
    bad.solver.near_depth = 9
    assert L.bem_server_create(ctypes.byref(bad), ctypes.byref(h)) == 2
    t = ctypes.c_longlong()
    r = bemlib.Request()
    assert L.bem_server_submit(None, ctypes.byref(r), ctypes.byref(t)) == 2
    assert L.bem_server_wait(None, 1, 0.0, None, 0, None) == 2
    st = L.bem_server_create(ctypes.byref(o), ctypes.byref(h))
    if st == 0:           # a device is present: the empty server shuts down cleanly
        s = bemlib.ServerStats()
        assert L.bem_server_stats(h, ctypes.byref(s)) == 0 and s.submitted == 0
        assert L.bem_server_submit(h, ctypes.byref(r), ctypes.byref(t)) == 2   # empty geometry
        assert L.bem_server_destroy(h) == 0
    else:
        assert st == 3    # no CUDA device: a status, not a crash


def _write_ply(path, p, f, fmt, extra=False):
    """PLY writer for the tests (numpy): optional extra vertex property and an
    extra element, to check they are skipped."""
    import struct
    nv, nf = p.shape[0], f.shape[0]
    hdr = ["ply", f"format {fmt} 1.0", "comment test", f"element vertex {nv}", "property double x",
           "property double y", "property double z"]
    if extra:
        hdr.append("property uchar red")
    hdr += [f"element face {nf}", "property list uchar int vertex_indices"]
    if extra:
        hdr += ["element edge 1", "property int vertex1", "property int vertex2"]
    hdr.append("end_header")
    with open(path, "wb") as fh:
        fh.write(("\n".join(hdr) + "\n").encode())
        if fmt == "ascii":
            for v in p:
                fh.write((" ".join(repr(float(c)) for c in v) + (" 7" if extra else "") + "\n").encode())
            for t in f:
                fh.write(("3 " + " ".join(str(int(i)) for i in t) + "\n").encode())
            if extra:
                fh.write(b"0 1\n")
        else:
            e = "<" if fmt == "binary_little_endian" else ">"
            for v in p:
                fh.write(struct.pack(e + "ddd", *v) + (struct.pack("B", 7) if extra else b""))
            for t in f:
                fh.write(struct.pack(e + "Biii", 3, *[int(i) for i in t]))
            if extra:
                fh.write(struct.pack(e + "ii", 0, 1))


@pytest.mark.parametrize("fmt", ["ascii", "binary_little_endian", "binary_big_endian"])
def test_read_ply(bemlib, tmp_path, fmt):
    p, f = icosphere(2, 0.3)
    path = str(tmp_path / "m.ply")
    _write_ply(path, p, f, fmt, extra=True)
    m = bemlib.Mesh()
    m.read_ply(path)
    assert np.array_equal(m.elems(), f)
    assert np.allclose(m.points(), p, rtol=0, atol=1e-15 if fmt != "ascii" else 1e-15)
    # a quad face is fan-triangulated
    with open(tmp_path / "q.ply", "w") as fh:
        fh.write("ply\nformat ascii 1.0\nelement vertex 4\nproperty float x\nproperty float y\nproperty float z\n"
                 "element face 1\nproperty list uchar int vertex_indices\nend_header\n"
                 "0 0 0\n1 0 0\n1 1 0\n0 1 0\n4 0 1 2 3\n")
    m.read_ply(str(tmp_path / "q.ply"))
    assert m.elems().tolist() == [[0, 1, 2], [0, 2, 3]]
    with open(tmp_path / "bad.ply", "w") as fh:
        fh.write("ply\nformat ascii 1.0\nelement vertex 1\nproperty float x\nproperty float y\nproperty float z\n"
                 "element face 1\nproperty list uchar int vertex_indices\nend_header\n0 0 0\n3 0 1 2\n")
    with pytest.raises(bemlib.BemError):
        m.read_ply(str(tmp_path / "bad.ply"))


def test_orient_repairs_winding(bemlib):
    p, f = icosphere(3, 1.0)
    rng = np.random.default_rng(0)
    g = f.copy()
    flip = rng.random(len(g)) < 0.3
    g[flip, 0], g[flip, 1] = g[flip, 1].copy(), g[flip, 0].copy()
    m = bemlib.Mesh.from_arrays(p, g)
    rep = m.orient()
    e = m.elems()
    assert rep["components"] == 1 and rep["open_edges"] == 0 and rep["nonmanifold"] == 0
    assert rep["flipped"] == int(flip.sum())
    # same winding as the icosphere (inward normals): every face equals the original up to rotation
    canon = lambda t: tuple(np.roll(t, -int(np.argmin(t))))
    assert [canon(t) for t in e] == [canon(t) for t in f]
    assert abs(rep["volume"] - 4 / 3 * np.pi) < 0.05
    # a fully outward mesh is turned inward; a second call changes nothing
    m2 = bemlib.Mesh.from_arrays(p, f[:, [1, 0, 2]])
    assert m2.orient()["flipped"] == len(f)
    assert m2.orient()["flipped"] == 0


def test_python_constants_match_the_header(bemlib):
    """Every enum of bem_gb300.h that the Python binding mirrors (precisions,
    solve methods, block-solve GEMM modes, source kinds) has the header's
    value."""
    text = open(os.path.join(ROOT, "include", "bem_gb300.h")).read()
    enums = {}
    for body in re.findall(r"enum\s*\{([^}]*)\}", text):
        for name, val in re.findall(r"(BEM_[A-Z0-9_]+)\s*=\s*(-?\d+)", body):
            enums[name] = int(val)
    checked = 0
    for name, val in enums.items():
        py = name[len("BEM_"):]
        if hasattr(bemlib, py):
            assert getattr(bemlib, py) == val, name
            checked += 1
    assert enums["BEM_GEMM_SIMT"] == 5 and bemlib.GEMM_SIMT == 5
    assert checked >= 12
