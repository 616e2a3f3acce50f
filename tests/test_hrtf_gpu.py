"""HRTF-style workflow (the reference's head meshes at 12-20 kHz with many
sources, output in wrtCplxMat format), on a synthetic head-sized body: a
binary PLY with the opposite winding is read, its winding repaired, 64
sources solved together, the field evaluated at two ear points and a ring,
and the matrix written in the reference's text format.  Checked against the
FP64 path (c128 assembly, QR, FP64 field)."""
import struct

import numpy as np
import pytest

from helpers import read_cplx_file, rel_err

pytestmark = pytest.mark.gpu


def _write_binary_ply(path, p, f):
    with open(path, "wb") as fh:
        fh.write(("ply\nformat binary_little_endian 1.0\nelement vertex %d\nproperty float x\nproperty float y\n"
                  "property float z\nelement face %d\nproperty list uchar int vertex_indices\nend_header\n"
                  % (p.shape[0], f.shape[0])).encode())
        for v in p.astype(np.float32):
            fh.write(struct.pack("<fff", *v))
        for t in f:
            fh.write(struct.pack("<Biii", 3, *[int(i) for i in t]))


def test_head_like_pipeline(bemlib, tmp_path):
    body = bemlib.Mesh.icosphere(4).perturbed_ellipsoid(0.08, 0.1, 0.12, lmax=6, amp=0.04, seed=21)
    p0, f0 = body.points(), body.elems()
    path = str(tmp_path / "head.ply")
    _write_binary_ply(path, p0, f0[:, [1, 0, 2]])          # outward winding, as mesh tools often write
    m = bemlib.Mesh()
    m.read_ply(path)
    rep = m.orient()
    assert rep["flipped"] == f0.shape[0] and rep["components"] == 1 and rep["open_edges"] == 0
    rng = np.random.default_rng(4)
    u = rng.random((16, 3))
    r = 0.03 * np.cbrt(u[:, 0])
    th, ph = np.arccos(1 - 2 * u[:, 1]), 2 * np.pi * u[:, 2]
    chief = np.stack([r * np.sin(th) * np.cos(ph), r * np.sin(th) * np.sin(ph), r * np.cos(th)], axis=1)
    srcs = [("point", s, 1.0) for s in bemlib.fibonacci_sphere(64, 1.0)]
    k = 2 * np.pi * 6000.0 / 343.21
    ears = np.array([[0.0, 0.115, 0.0], [0.0, -0.115, 0.0]])
    ring = np.array([[0.5 * np.cos(a), 0.5 * np.sin(a), 0.0] for a in np.linspace(0, 2 * np.pi, 8, endpoint=False)])
    field_pts = np.vstack([ears, ring])

    m.set_uniform_bc(0, 1, 0)                               # rigid
    m.set_chief(chief)
    s = bemlib.Solver(near_eta=1.0, near_depth=2)
    s.set_mesh(m)
    s.set_sources(srcs)
    s.assemble(k, bemlib.PREC_C128)
    s.solve(bemlib.SOLVE_QR)
    x64, fld64 = s.solution(), s.field(field_pts, bemlib.PREC_C128)
    s.assemble(k, bemlib.PREC_C64)
    info = s.solve(bemlib.SOLVE_BLOCK_GMRES)
    assert info.converged
    assert rel_err(s.solution(), x64) < 1e-5
    fld = s.field(field_pts, bemlib.PREC_C128)
    assert rel_err(fld, fld64) < 1e-4
    out = str(tmp_path / "hrtf.txt")
    bemlib.wrtCplxMat(fld.astype(np.complex64), out)
    back = read_cplx_file(out).reshape(fld.shape)                      # one line per row
    assert np.abs(back - fld).max() < 1e-6 + 1e-6 * np.abs(fld).max()
