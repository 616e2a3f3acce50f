"""ctypes access to the reference-kernel harness (oracle/_ref/) -- test and
benchmark infrastructure only (see ref_harness.cpp and ref_build.py)."""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import ref_build

_lib = None

# The 6-point Gauss-Legendre rule as the reference uploads it: float nodes and
# weights (gaussQuad::sendToDevice, numerical.cu:227-231).
_GL6_X = [-0.9324695142031521, -0.6612093864662645, -0.2386191860831969,
          0.2386191860831969, 0.6612093864662645, 0.9324695142031521]
_GL6_W = [0.1713244923791704, 0.3607615730481386, 0.4679139345726910,
          0.4679139345726910, 0.3607615730481386, 0.1713244923791704]


def available() -> bool:
    return os.path.exists(ref_build.CUBIN) and os.path.exists(ref_build.HARNESS)


def lib():
    global _lib
    if _lib is None:
        ref_build.build_harness()
        L = ctypes.CDLL(ref_build.HARNESS)
        vp = ctypes.c_void_p
        L.refh_assemble.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, vp, ctypes.c_int, vp, vp,
                                    ctypes.c_float, vp, vp, ctypes.c_int, vp, ctypes.c_float, vp, vp, vp]
        L.refh_qr.argtypes = [ctypes.c_int, ctypes.c_int, vp, vp, ctypes.c_int, vp]
        L.refh_last_error.restype = ctypes.c_char_p
        _lib = L
    return _lib


def _p(a):
    return ctypes.c_void_p(a.ctypes.data)


def assemble(pts, elems, n_nodes, k, srcs=((1e6, 1e6, 1e6),), strength=0.0, bc=None):
    """The reference's atomicGenSystem on this GPU: (A, B, ms), A (N+M) x N
    and B (N+M) x S complex64 column-major, ms the kernels' span."""
    pts = np.ascontiguousarray(pts, dtype=np.float32).reshape(-1, 3)
    elems = np.ascontiguousarray(elems, dtype=np.int32).reshape(-1, 3)
    R, N, E = pts.shape[0], int(n_nodes), elems.shape[0]
    if bc is None:
        bc = np.tile(np.array([0, 0, 1, 0, -1, 0], dtype=np.float32), (E, 1))
    else:
        b = np.asarray(bc, dtype=np.complex128).reshape(-1, 3)
        bc = np.stack([b.real, b.imag], axis=2).reshape(E, 6).astype(np.float32)
    bc = np.ascontiguousarray(bc, dtype=np.float32)
    srcs = np.ascontiguousarray(srcs, dtype=np.float32).reshape(-1, 3)
    S = srcs.shape[0]
    A = np.zeros((R, N), dtype=np.complex64, order="F")
    B = np.zeros((R, S), dtype=np.complex64, order="F")
    glx = np.array(_GL6_X, dtype=np.float32)
    glw = np.array(_GL6_W, dtype=np.float32)
    ms = np.zeros(1, dtype=np.float32)
    st = lib().refh_assemble(os.fsencode(ref_build.CUBIN), N, R - N, _p(pts), E, _p(elems), _p(bc),
                             float(k), _p(glx), _p(glw), S, _p(srcs), float(strength), _p(A), _p(B), _p(ms))
    if st != 0:
        raise RuntimeError(lib().refh_last_error().decode())
    return A, B, float(ms[0])


def qr(A, B):
    """qrSolver's library sequence: (X, ms)."""
    A = np.asfortranarray(A, dtype=np.complex64)
    B = np.array(B, dtype=np.complex64, order="F", copy=True)
    if B.ndim == 1:
        B = B.reshape(-1, 1, order="F")
    m, n = A.shape
    ms = np.zeros(1, dtype=np.float32)
    st = lib().refh_qr(m, n, _p(A), _p(B), B.shape[1], _p(ms))
    if st != 0:
        raise RuntimeError(lib().refh_last_error().decode())
    return B[:n].copy(), float(ms[0])
