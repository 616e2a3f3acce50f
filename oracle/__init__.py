"""FP64 CPU oracle for the Helmholtz BEM hot path -- TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and the CPU legs of ``bench.py``
import this package, and only as the checker.  The product library
(``bem_gpu_clean_cpp_gb300``) never imports, links or calls anything here.

Contents
--------
* ctypes bindings to ``libbem_oracle.so`` (built from ``bem_oracle.c``): the C
  restatement of the reference's quadrature, assembly, QR least-squares,
  GMRES, field evaluation and CHIEF acceptance (file:line citations in
  ``bem_oracle.c``).
* ``read_obj_reference``: the reference's ``mesh::readObj`` parse rules
  (mesh.cu:1215-1265) restated in Python.
* analytic solutions used as physics checks: the pulsating sphere
  (sphere.m:3-11) and the rigid sphere under a plane wave (series solution).

Parity pin: tests/test_oracle_golden.py reproduces the reference's committed
golden outputs ``sphere171Hz_CHIEF`` / ``sphere171Hz_NoCHIEF`` (copied to
tests/golden/) with this oracle.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "libbem_oracle.so")
_lock = threading.Lock()
_lib = None

DENSITY = 1.2041   # numerical.cu:12
SPEED = 343.21     # numerical.cu:14


class Params(ctypes.Structure):
    _fields_ = [("density", ctypes.c_double), ("speed", ctypes.c_double),
                ("order", ctypes.c_int), ("near_eta", ctypes.c_double),
                ("near_depth", ctypes.c_int)]


class Source(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("vec", ctypes.c_double * 3),
                ("amp_re", ctypes.c_double), ("amp_im", ctypes.c_double)]


def build(force: bool = False) -> str:
    """Compile libbem_oracle.so with the Makefile beside this file."""
    src = os.path.join(_HERE, "bem_oracle.c")
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", _HERE, "-B", "libbem_oracle.so"], check=True)
    return _LIB_PATH


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = ctypes.CDLL(_LIB_PATH)
            dp = ctypes.POINTER(ctypes.c_double)
            ip = ctypes.POINTER(ctypes.c_int)
            L.orc_gauss_legendre.argtypes = [ctypes.c_int, dp, dp]
            L.orc_elem_coeffs.argtypes = [ctypes.c_double, dp, dp, dp, dp, ctypes.c_int,
                                          ctypes.POINTER(Params), dp, dp, dp]
            L.orc_assemble.argtypes = [ctypes.c_int, ctypes.c_int, dp, ctypes.c_int, ip, dp,
                                       ctypes.c_double, ctypes.POINTER(Params), ctypes.c_int,
                                       ctypes.POINTER(Source), dp, ctypes.c_int, dp, ctypes.c_int,
                                       ctypes.c_int, ctypes.c_int]
            L.orc_field.argtypes = [ctypes.c_int, dp, ctypes.c_int, ip, dp, ctypes.c_double,
                                    ctypes.POINTER(Params), ctypes.c_int, ctypes.POINTER(Source),
                                    dp, ctypes.c_int, ctypes.c_int, dp, dp, ctypes.c_int]
            L.orc_lsq_qr.argtypes = [ctypes.c_int, ctypes.c_int, dp, ctypes.c_int, dp,
                                     ctypes.c_int, ctypes.c_int]
            L.orc_matvec.argtypes = [ctypes.c_int, ctypes.c_int, dp, ctypes.c_int, dp, dp]
            L.orc_gmres.argtypes = [dp, dp, ctypes.c_int, ctypes.c_int, ctypes.c_double, dp,
                                    ip, dp]
            L.orc_chief_select.argtypes = [ctypes.c_int, dp, ctypes.c_int, ip, dp, ctypes.c_double,
                                           ctypes.c_int, dp, ctypes.c_int, dp, ip]
            L.orc_ray_tri.argtypes = [dp, dp, dp, dp, dp]
            L.orc_set_threads.argtypes = [ctypes.c_int]
            L.orc_num_threads.restype = ctypes.c_int
            _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


def set_threads(n: int) -> None:
    lib().orc_set_threads(int(n))


def num_threads() -> int:
    return int(lib().orc_num_threads())


def params(order=6, near_eta=0.0, near_depth=0, density=DENSITY, speed=SPEED) -> Params:
    return Params(density, speed, order, near_eta, near_depth)


def sources(srcs) -> ctypes.Array:
    """srcs: list of (kind, (x, y, z), amplitude) with kind 'point' or 'plane'."""
    arr = (Source * max(1, len(srcs)))()
    for i, (kind, vec, amp) in enumerate(srcs):
        arr[i].kind = 1 if kind == "plane" else 0
        for d in range(3):
            arr[i].vec[d] = float(vec[d])
        amp = complex(amp)
        arr[i].amp_re, arr[i].amp_im = amp.real, amp.imag
    return arr


def gauss_legendre(n: int):
    x = np.zeros(n)
    w = np.zeros(n)
    if lib().orc_gauss_legendre(n, _dp(x), _dp(w)) != 0:
        raise ValueError("bad order")
    return x, w


def elem_coeffs(k, x, p1, p2, p3, sing=0, prm=None):
    prm = prm or params()
    a = [np.ascontiguousarray(v, dtype=np.float64) for v in (x, p1, p2, p3)]
    g = np.zeros(6)
    h = np.zeros(6)
    c = np.zeros(1)
    lib().orc_elem_coeffs(float(k), _dp(a[0]), _dp(a[1]), _dp(a[2]), _dp(a[3]), int(sing),
                          ctypes.byref(prm), _dp(g), _dp(h), _dp(c))
    return g.view(np.complex128), h.view(np.complex128), float(c[0])


def assemble(pts, elems, k, n_nodes, srcs, bc=None, prm=None, rows=None, want_A=True):
    """A ((N+M) x N) and B ((N+M) x S) in FP64, column-major complex128 arrays.

    pts holds the N nodes followed by the M CHIEF points.  rows=(r0, r1)
    computes only that row range and returns its (r1-r0) rows."""
    prm = prm or params()
    pts = np.ascontiguousarray(pts, dtype=np.float64)
    elems = np.ascontiguousarray(elems, dtype=np.int32)
    R = pts.shape[0]
    N = int(n_nodes)
    M = R - N
    S = len(srcs)
    r0, r1 = (0, R) if rows is None else rows
    nr = r1 - r0
    A = np.zeros((nr, N), dtype=np.complex128, order="F") if want_A else None
    B = np.zeros((nr, max(S, 1)), dtype=np.complex128, order="F")
    bcp = None
    if bc is not None:
        bcarr = np.ascontiguousarray(np.asarray(bc, dtype=np.complex128).reshape(-1, 3))
        bcp = bcarr.view(np.float64)
    st = lib().orc_assemble(N, M, _dp(pts), elems.shape[0], _ip(elems),
                            _dp(bcp) if bcp is not None else None, float(k), ctypes.byref(prm),
                            S, sources(srcs), _dp(A.reshape(-1, order="F").view(np.float64))
                            if A is not None else None, nr,
                            _dp(B.reshape(-1, order="F").view(np.float64)), nr, int(r0), int(r1))
    if st != 0:
        raise ValueError(f"orc_assemble failed ({st})")
    return A, B


def field(pts_nodes, elems, k, surfP, fpts, srcs, bc=None, prm=None):
    prm = prm or params()
    pts_nodes = np.ascontiguousarray(pts_nodes, dtype=np.float64)
    elems = np.ascontiguousarray(elems, dtype=np.int32)
    surfP = np.asfortranarray(np.asarray(surfP, dtype=np.complex128).reshape(pts_nodes.shape[0], -1))
    S = surfP.shape[1]
    fpts = np.ascontiguousarray(fpts, dtype=np.float64).reshape(-1, 3)
    P = fpts.shape[0]
    out = np.zeros((P, S), dtype=np.complex128, order="F")
    bcp = None
    if bc is not None:
        bcarr = np.ascontiguousarray(np.asarray(bc, dtype=np.complex128).reshape(-1, 3))
        bcp = bcarr.view(np.float64)
    srcs = list(srcs) + [("point", (0, 0, 0), 0.0)] * (S - len(srcs))
    lib().orc_field(pts_nodes.shape[0], _dp(pts_nodes), elems.shape[0], _ip(elems),
                    _dp(bcp) if bcp is not None else None, float(k), ctypes.byref(prm), S,
                    sources(srcs), _dp(surfP.reshape(-1, order="F").view(np.float64)),
                    pts_nodes.shape[0], P, _dp(fpts),
                    _dp(out.reshape(-1, order="F").view(np.float64)), P)
    return out


def lsq_qr(A, B):
    """min ||A X - B|| by Householder QR; returns X (n x nrhs)."""
    A = np.array(A, dtype=np.complex128, order="F", copy=True)
    B = np.array(B, dtype=np.complex128, order="F", copy=True)
    if B.ndim == 1:
        B = B.reshape(-1, 1, order="F")
    m, n = A.shape
    st = lib().orc_lsq_qr(m, n, _dp(A.reshape(-1, order="F").view(np.float64)), m,
                          _dp(B.reshape(-1, order="F").view(np.float64)), B.shape[1], m)
    if st != 0:
        raise ValueError("orc_lsq_qr failed")
    return B[:n].copy()


def gmres(A, b, max_iter, thr, x0=None):
    A = np.array(A, dtype=np.complex128, order="F", copy=True)
    m = A.shape[0]
    b = np.ascontiguousarray(b, dtype=np.complex128).reshape(m)
    x = np.zeros(m, dtype=np.complex128) if x0 is None else np.array(x0, dtype=np.complex128)
    it = np.zeros(1, dtype=np.int32)
    rr = np.zeros(1)
    lib().orc_gmres(_dp(A.reshape(-1, order="F").view(np.float64)), _dp(b.view(np.float64)),
                    m, int(max_iter), float(thr), _dp(x.view(np.float64)), _ip(it), _dp(rr))
    return x, int(it[0]), float(rr[0])


def chief_select(pts, elems, bb, threshold, cand, num):
    pts = np.ascontiguousarray(pts, dtype=np.float64)
    elems = np.ascontiguousarray(elems, dtype=np.int32)
    bb = np.ascontiguousarray(bb, dtype=np.float64)
    cand = np.ascontiguousarray(cand, dtype=np.float64).reshape(-1, 3)
    out = np.zeros((num, 3))
    used = np.zeros(1, dtype=np.int32)
    got = lib().orc_chief_select(pts.shape[0], _dp(pts), elems.shape[0], _ip(elems), _dp(bb),
                                 float(threshold), cand.shape[0], _dp(cand), int(num), _dp(out),
                                 _ip(used))
    return out[:got], int(used[0])


# --------------------------------------------------------------------------
# mesh::readObj (mesh.cu:1215-1265) parse rules, restated:
#   * fgets(line, 49, fp): lines are consumed in chunks of at most 48 chars;
#   * a chunk whose first char is 'v' is a vertex ("%s %f %f %f", so vn/vt
#     lines count too); a chunk starting with 'f' is a face ("%s %d %d %d",
#     1-based, only the leading integer of each a/b/c field is read);
#   * every face gets bc = (0, 1, -1).
# --------------------------------------------------------------------------
def read_obj_reference(path):
    pts, faces = [], []
    with open(path, "r", errors="replace") as f:
        data = f.read()
    pos = 0
    n = len(data)
    last_face = [0, 0, 0]
    while pos < n:
        end = data.find("\n", pos)
        end = n if end < 0 else end + 1
        chunk_end = min(end, pos + 48)
        chunk = data[pos:chunk_end]
        pos = chunk_end
        if not chunk:
            break
        toks = chunk.split()
        if chunk[0] == "v":
            vals = []
            for t in toks[1:4]:
                try:
                    vals.append(float(t))
                except ValueError:
                    break
            v = list(pts[-1]) if pts else [0.0, 0.0, 0.0]
            for i, val in enumerate(vals):
                v[i] = val
            pts.append(tuple(np.float32(v)))
        if chunk[0] == "f":
            vals = list(last_face)
            for i, t in enumerate(toks[1:4]):
                head = t.split("/")[0]
                try:
                    vals[i] = int(head)
                except ValueError:
                    break
                if "/" in t:
                    break
            last_face = vals
            faces.append([vals[0] - 1, vals[1] - 1, vals[2] - 1])
    return np.array(pts, dtype=np.float32).reshape(-1, 3), np.array(faces, dtype=np.int32).reshape(-1, 3)


# --------------------------------------------------------------------------
# Analytic solutions (e^{+i w t} convention, G = exp(-ikr)/(4 pi r))
# --------------------------------------------------------------------------
def pulsating_sphere(r, a, k, density=DENSITY, speed=SPEED):
    """sphere.m:11: p(r) = a^2/r * i rho w/(1 + i k a) * exp(-i k (r - a)) for unit
    outward normal velocity."""
    w = k * speed
    r = np.asarray(r, dtype=np.float64)
    return a * a / r * 1j * density * w / (1 + 1j * k * a) * np.exp(-1j * k * (r - a))


def rigid_sphere_surface(cos_theta, ka, nmax=None):
    """Total surface pressure on a rigid sphere of radius a under the unit plane
    wave exp(-i k d.x), cos_theta = d . x/|x|.  With h_n = j_n - i y_n (outgoing
    for e^{+i w t}) and the Wronskian, p = sum_n (-i)^n (2n+1) P_n(cos) *
    (-i) / ((ka)^2 h_n'(ka))."""
    from scipy.special import eval_legendre, spherical_jn, spherical_yn
    ka = float(ka)
    if nmax is None:
        nmax = int(ka + 4 * ka ** (1 / 3) + 12)
    ct = np.asarray(cos_theta, dtype=np.float64)
    p = np.zeros(ct.shape, dtype=np.complex128)
    for n in range(nmax + 1):
        hp = spherical_jn(n, ka, derivative=True) - 1j * spherical_yn(n, ka, derivative=True)
        coef = (-1j) ** n * (2 * n + 1) * (-1j) / (ka * ka * hp)
        p += coef * eval_legendre(n, ct)
    return p
