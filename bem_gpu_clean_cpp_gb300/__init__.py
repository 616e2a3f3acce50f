"""GB300-native Helmholtz BEM engine -- Python host side over the C ABI.

Every call goes through ``libbem_gb300.so`` (``include/bem_gb300.h``) with
ctypes.  There is no Python or CPU fallback: if the library is missing the
import of any compute call raises.  Names mirror the reference's C++ call
surface (ZiqiFrancisFan/BEM_GPU_Clean_CPP):

==========================  ==============================================
reference                   here
==========================  ==============================================
mesh::readObj (mesh.cu:1215)         ``Mesh.readObj`` / ``Mesh.read_obj``
mesh::findBB (mesh.cu:1369)          ``Mesh.findBB``
mesh::genCHIEF (mesh.cu:1430)        ``Mesh.genCHIEF``
gaussQuad + sendToDevice             ``gaussQuad(order).sendToDevice()``
bemSystem (mesh.cu:985)              ``bemSystem``
qrSolver (numerical.cu:580)          ``qrSolver``
GMRES (GMRES.cu:145)                 ``GMRES``
genExtPressure (mesh.cu:1038)        ``genExtPressure``
wrtCplxMat (numerical.cu:556)        ``wrtCplxMat``
==========================  ==============================================

``Solver`` exposes the device-resident engine (assembly, QR and refined
GMRES solves, batched field evaluation) that the drop-in calls sit on.
"""
from __future__ import annotations

import ctypes
import os
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libbem_gb300.so")

SUCCESS = 0
PREC_C64, PREC_C128 = 0, 1
SOLVE_QR, SOLVE_GMRES_REFINED, SOLVE_BLOCK_GMRES, SOLVE_QR_TC = 0, 1, 2, 3
GEMM_AUTO, GEMM_FP32, GEMM_SPLIT_BF16, GEMM_TF32, GEMM_TF32X3, GEMM_TF32X3_3M, GEMM_SIMT, GEMM_TC = -1, 0, 1, 2, 3, 4, 5, 6
SRC_POINT, SRC_PLANE = 0, 1
ERR_INVALID_ARG = 2
ERR_NOT_CONVERGED = 5
ERR_TOO_LARGE = 8
ERR_TIMEOUT = 10

_lock = threading.Lock()
_lib = None


class BemError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"[{status}] {msg}")
        self.status = status


class Source(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("vec", ctypes.c_double * 3),
                ("amp_re", ctypes.c_double), ("amp_im", ctypes.c_double)]


class Options(ctypes.Structure):
    _fields_ = [("density", ctypes.c_double), ("speed", ctypes.c_double), ("order", ctypes.c_int),
                ("near_eta", ctypes.c_double), ("near_depth", ctypes.c_int), ("tol", ctypes.c_double),
                ("max_iter", ctypes.c_int), ("inner_tol", ctypes.c_double),
                ("max_refine", ctypes.c_int), ("tile_cols", ctypes.c_int), ("far_variant", ctypes.c_int),
                ("gemm_mode", ctypes.c_int), ("block_tol", ctypes.c_double)]


class SolveInfo(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int), ("refinements", ctypes.c_int),
                ("rel_residual", ctypes.c_double), ("converged", ctypes.c_int)]


class ServerOptions(ctypes.Structure):
    _fields_ = [("slots", ctypes.c_int), ("hbm_budget_bytes", ctypes.c_double),
                ("cache_systems", ctypes.c_int), ("block_min_sources", ctypes.c_int),
                ("solver", Options)]


class Request(ctypes.Structure):
    _fields_ = [("pnts", ctypes.c_void_p), ("num_pnts", ctypes.c_int), ("elems", ctypes.c_void_p),
                ("num_elems", ctypes.c_int), ("bc", ctypes.c_void_p), ("chief", ctypes.c_void_p),
                ("num_chief", ctypes.c_int), ("k", ctypes.c_double), ("srcs", ctypes.c_void_p),
                ("num_srcs", ctypes.c_int)]


class RequestResult(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int), ("method", ctypes.c_int), ("iterations", ctypes.c_int),
                ("refinements", ctypes.c_int), ("converged", ctypes.c_int), ("rel_residual", ctypes.c_double),
                ("queue_ms", ctypes.c_double), ("service_ms", ctypes.c_double), ("latency_ms", ctypes.c_double),
                ("cache_hit", ctypes.c_int), ("device_bytes", ctypes.c_double), ("num_pnts", ctypes.c_int),
                ("num_srcs", ctypes.c_int)]


class ServerStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_longlong), ("completed", ctypes.c_longlong), ("failed", ctypes.c_longlong),
                ("solves", ctypes.c_longlong), ("cache_hits", ctypes.c_longlong), ("evictions", ctypes.c_longlong),
                ("p50_ms", ctypes.c_double), ("p99_ms", ctypes.c_double), ("mean_ms", ctypes.c_double),
                ("max_ms", ctypes.c_double), ("resident_bytes", ctypes.c_double), ("peak_bytes", ctypes.c_double),
                ("max_in_flight", ctypes.c_int)]


# Exported symbols and their signatures (the C ABI of include/bem_gb300.h).
_VP = ctypes.c_void_p
_I = ctypes.c_int
_D = ctypes.c_double
_F = ctypes.c_float
_S = ctypes.c_char_p
SIGNATURES = {
    "bem_status_string": (_S, [_I]),
    "bem_last_error": (_S, []),
    "bem_version": (_I, []),
    "bem_launch_count": (ctypes.c_longlong, []),
    "bem_profile_enable": (_I, [_I]),
    "bem_profile_report": (_I, [ctypes.c_char_p, _I]),
    "bem_gauss_legendre": (_I, [_I, _VP, _VP]),
    "bem_set_quadrature": (_I, [_I]),
    "bem_get_quadrature": (_I, []),
    "bem_set_medium": (_I, [_D, _D]),
    "bem_set_point_source_strength": (_I, [_D]),
    "bem_mesh_create": (_I, [ctypes.POINTER(_VP)]),
    "bem_mesh_destroy": (_I, [_VP]),
    "bem_mesh_read_obj": (_I, [_VP, _S]),
    "bem_mesh_read_obj_robust": (_I, [_VP, _S]),
    "bem_mesh_read_ply": (_I, [_VP, _S]),
    "bem_mesh_orient": (_I, [_VP, _VP, _VP, _VP, _VP, _VP]),
    "bem_mesh_set": (_I, [_VP, _VP, _I, _VP, _I]),
    "bem_mesh_set_bc": (_I, [_VP, _VP]),
    "bem_mesh_set_uniform_bc": (_I, [_VP, _D, _D, _D, _D, _D, _D]),
    "bem_mesh_find_bb": (_I, [_VP, _F]),
    "bem_mesh_get_bb": (_I, [_VP, _VP]),
    "bem_mesh_gen_chief": (_I, [_VP, _I, _F]),
    "bem_mesh_set_chief": (_I, [_VP, _VP, _I]),
    "bem_mesh_get_counts": (_I, [_VP, _VP, _VP, _VP]),
    "bem_mesh_get_points": (_I, [_VP, _VP]),
    "bem_mesh_get_elems": (_I, [_VP, _VP]),
    "bem_mesh_get_chief": (_I, [_VP, _VP]),
    "bem_mesh_icosphere": (_I, [_VP, _I, _D]),
    "bem_mesh_surface_area": (_I, [_VP, _VP]),
    "bem_mesh_geodesic": (_I, [_VP, _I, _D]),
    "bem_mesh_perturbed_ellipsoid": (_I, [_VP, _D, _D, _D, _I, _D, ctypes.c_ulonglong]),
    "bem_fibonacci_sphere": (_I, [_I, _D, _VP]),
    "bem_hmat_partition": (_I, [_VP, _I, _VP, _I, _I, _D, _VP, _VP, _VP, _I, ctypes.POINTER(_I)]),
    "bem_hmat_partition_system": (_I, [_VP, _I, _VP, _I, _I, _D, _VP, _VP, _VP, _I, ctypes.POINTER(_I)]),
    "bem_hmat_compress_c64": (_I, [_VP, _I, _I, _I, _VP, _I, _D, _I, _VP, ctypes.POINTER(_VP)]),
    "bem_hmat_matvec_c64": (_I, [_VP, _I, _VP, _VP, _VP]),
    "bem_hmat_info": (_I, [_VP, ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(_I), ctypes.POINTER(_I),
                           ctypes.POINTER(_I)]),
    "bem_hmat_destroy": (_I, [_VP]),
    "bem_system_c64": (_I, [_VP, _F, _VP, _I, _VP, _I, _VP, _I]),
    "bem_qr_solve_c64": (_I, [_VP, _I, _I, _I, _VP, _I, _I]),
    "bem_gmres_c64": (_I, [_VP, _VP, _I, _I, _F, _VP]),
    "bem_gmres_c64_noalloc": (_I, [_VP, _I, _VP, _I, _I, _F, _VP, _VP, ctypes.POINTER(_I)]),
    "bem_tc_gemm_f32": (_I, [_I, _I, _I, _I, _VP, _I, _VP, _I, _VP, _I, _I]),
    "bem_ext_pressure_c64": (_I, [_F, _VP, _VP, _VP, _VP, _VP]),
    "bem_write_cplx_mat_c64": (_I, [_VP, _I, _I, _I, _S]),
    "bem_options_default": (_I, [_VP]),
    "bem_solver_create": (_I, [ctypes.POINTER(_VP)]),
    "bem_solver_destroy": (_I, [_VP]),
    "bem_solver_set_options": (_I, [_VP, _VP]),
    "bem_solver_get_options": (_I, [_VP, _VP]),
    "bem_solver_set_mesh": (_I, [_VP, _VP]),
    "bem_solver_set_geometry": (_I, [_VP, _VP, _I, _VP, _I, _VP, _VP, _I]),
    "bem_solver_set_sources": (_I, [_VP, _VP, _I]),
    "bem_solver_assemble": (_I, [_VP, _D, _I]),
    "bem_solver_solve": (_I, [_VP, _I, _VP]),
    "bem_solver_get_solution": (_I, [_VP, _VP, _I, _I]),
    "bem_solver_get_system": (_I, [_VP, _VP, _I, _VP, _I, _I]),
    "bem_solver_eval_field": (_I, [_VP, _VP, _I, _VP, _I, _I]),
    "bem_solver_sync": (_I, [_VP]),
    "bem_solver_stream": (_VP, [_VP]),
    "bem_solver_sizes": (_I, [_VP, _VP, _VP, _VP, _VP]),
    "bem_solver_block_gemm_mode": (_I, [_VP, ctypes.POINTER(_I)]),
    "bem_solver_far_variant": (_I, [_VP, ctypes.POINTER(_I)]),
    "bem_server_options_default": (_I, [_VP]),
    "bem_server_create": (_I, [_VP, ctypes.POINTER(_VP)]),
    "bem_server_destroy": (_I, [_VP]),
    "bem_server_submit": (_I, [_VP, _VP, ctypes.POINTER(ctypes.c_longlong)]),
    "bem_server_wait": (_I, [_VP, ctypes.c_longlong, _D, _VP, _I, _VP]),
    "bem_server_stats": (_I, [_VP, _VP]),
    "bem_server_reset_stats": (_I, [_VP]),
}


def lib():
    """Load libbem_gb300.so; raise when it has not been built."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise BemError(1, f"{LIB_PATH} is missing: build it with "
                                  "`python -c 'import __graft_entry__ as g; g.build()'`")
            L = ctypes.CDLL(LIB_PATH)
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            _lib = L
    return _lib


def _check(status: int) -> None:
    if status != SUCCESS:
        msg = lib().bem_last_error().decode(errors="replace")
        raise BemError(status, msg or lib().bem_status_string(status).decode())


def _ptr(a: np.ndarray):
    return ctypes.c_void_p(a.ctypes.data)


def launch_count() -> int:
    return int(lib().bem_launch_count())


def profile_enable(on: bool = True) -> None:
    """Bracket every library kernel launch with CUDA events (clears old records)."""
    _check(lib().bem_profile_enable(1 if on else 0))


def profile_report() -> dict:
    """{kernel name: (launches, total_ms)} for the current profiling window."""
    buf = ctypes.create_string_buffer(1 << 16)
    n = lib().bem_profile_report(buf, len(buf))
    if n < 0:
        _check(-n)
    out = {}
    for line in buf.value.decode().splitlines():
        name, cnt, ms = line.split()
        out[name] = (int(cnt), float(ms))
    return out


def sources(srcs) -> ctypes.Array:
    """srcs: iterable of (kind, (x, y, z), amplitude) with kind 'point' or 'plane'."""
    srcs = list(srcs)
    arr = (Source * len(srcs))()
    for i, (kind, vec, amp) in enumerate(srcs):
        arr[i].kind = SRC_PLANE if kind == "plane" else SRC_POINT
        for d in range(3):
            arr[i].vec[d] = float(vec[d])
        amp = complex(amp)
        arr[i].amp_re, arr[i].amp_im = amp.real, amp.imag
    return arr


# ---------------------------------------------------------------------------
# Quadrature (gaussQuad, numerical.h:166-187)
# ---------------------------------------------------------------------------
def gauss_legendre(order: int):
    x = np.zeros(order)
    w = np.zeros(order)
    _check(lib().bem_gauss_legendre(order, _ptr(x), _ptr(w)))
    return x, w


class gaussQuad:
    """gaussQuad(order).sendToDevice(): sets the Gauss order used by the
    drop-in calls and new solvers (numerical.cu:152-156, 227-231)."""

    def __init__(self, order: int = 6):
        self.n = int(order)
        self.evalPnts, self.wgts = gauss_legendre(self.n)

    def sendToDevice(self) -> int:
        _check(lib().bem_set_quadrature(self.n))
        return SUCCESS


def fibonacci_sphere(n: int, radius: float = 1.0) -> np.ndarray:
    """n points of a Fibonacci lattice on a sphere (source sets of the benchmarks)."""
    out = np.zeros((n, 3))
    _check(lib().bem_fibonacci_sphere(int(n), float(radius), _ptr(out)))
    return out


def hmat_partition(rows, cols, leaf: int = 128, eta: float = 1.0):
    """Block partition of the (rows x cols) collocation matrix for a
    hierarchical representation (bem_hmat_partition).  Returns (row_perm,
    col_perm, blocks): the clustered orders (position -> original index) and
    an int array of (row_begin, row_count, col_begin, col_count, admissible)
    per block, in clustered positions."""
    rows = np.ascontiguousarray(rows, dtype=np.float64).reshape(-1, 3)
    cols = np.ascontiguousarray(cols, dtype=np.float64).reshape(-1, 3)
    R, N = rows.shape[0], cols.shape[0]
    n = _I(0)
    L = lib()
    _check(L.bem_hmat_partition(_ptr(rows), R, _ptr(cols), N, int(leaf), float(eta), None, None, None, 0,
                                ctypes.byref(n)))
    row_perm = np.zeros(R, dtype=np.int32)
    col_perm = np.zeros(N, dtype=np.int32)
    blocks = np.zeros((max(n.value, 1), 5), dtype=np.int32)
    _check(L.bem_hmat_partition(_ptr(rows), R, _ptr(cols), N, int(leaf), float(eta), _ptr(row_perm),
                                _ptr(col_perm), _ptr(blocks), n.value, ctypes.byref(n)))
    return row_perm, col_perm, blocks[:n.value]


def hmat_partition_system(pnts, chief, leaf: int = 128, eta: float = 1.0):
    """Partition of a collocation system (bem_hmat_partition_system): rows
    are the nodes in the column tree's order, then the CHIEF points.  Returns
    (node_perm, chief_perm, blocks)."""
    pnts = np.ascontiguousarray(pnts, dtype=np.float64).reshape(-1, 3)
    chief = np.ascontiguousarray(chief if chief is not None else np.zeros((0, 3)), dtype=np.float64).reshape(-1, 3)
    N, M = pnts.shape[0], chief.shape[0]
    cptr = _ptr(chief) if M else None
    n = _I(0)
    L = lib()
    _check(L.bem_hmat_partition_system(_ptr(pnts), N, cptr, M, int(leaf), float(eta), None, None, None, 0,
                                       ctypes.byref(n)))
    node_perm = np.zeros(N, dtype=np.int32)
    chief_perm = np.zeros(M, dtype=np.int32)
    blocks = np.zeros((max(n.value, 1), 5), dtype=np.int32)
    _check(L.bem_hmat_partition_system(_ptr(pnts), N, cptr, M, int(leaf), float(eta), _ptr(node_perm),
                                       _ptr(chief_perm) if M else None, _ptr(blocks), n.value, ctypes.byref(n)))
    return node_perm, chief_perm, blocks[:n.value]


class HMatrix:
    """Hierarchical form of a c64 matrix on the device (``bem_hmat_*``).
    ``A_ptr``: device address of an R x N row-major matrix (row stride
    ``lda``) in the clustered order of ``blocks`` (from ``hmat_partition``);
    admissible blocks are compressed by adaptive cross approximation to
    relative tolerance ``tol`` with at most ``kmax`` terms.  ``stream`` is a
    cudaStream_t address (0: the legacy default stream)."""

    def __init__(self, A_ptr: int, R: int, N: int, lda: int, blocks, tol: float = 1e-5, kmax: int = 64,
                 stream: int = 0):
        b = np.ascontiguousarray(blocks, dtype=np.int32).reshape(-1, 5)
        h = ctypes.c_void_p()
        _check(lib().bem_hmat_compress_c64(A_ptr, int(R), int(N), int(lda), _ptr(b), b.shape[0], float(tol),
                                           int(kmax), stream or None, ctypes.byref(h)))
        self._h = h
        self.R, self.N = int(R), int(N)

    def matvec(self, x_ptr: int, y_ptr: int, trans: int = 0, stream: int = 0) -> None:
        """y = H x (trans 0) or H^H x (trans 1), device addresses, queued on stream."""
        _check(lib().bem_hmat_matvec_c64(self._h, int(trans), x_ptr, y_ptr, stream or None))

    def info(self) -> dict:
        e = ctypes.c_longlong()
        k, nl, nd = _I(), _I(), _I()
        _check(lib().bem_hmat_info(self._h, ctypes.byref(e), ctypes.byref(k), ctypes.byref(nl), ctypes.byref(nd)))
        return {"entries": e.value, "max_rank": k.value, "lowrank_blocks": nl.value, "dense_blocks": nd.value}

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().bem_hmat_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:   # interpreter shutdown: the library may already be gone
            pass


def set_medium(density: float, speed: float) -> None:
    _check(lib().bem_set_medium(float(density), float(speed)))


def set_point_source_strength(q: float) -> None:
    """The reference's STRENGTH macro (numerical.h:128-130), 0 by default."""
    _check(lib().bem_set_point_source_strength(float(q)))


# ---------------------------------------------------------------------------
# Mesh (class mesh, mesh.h:216-259)
# ---------------------------------------------------------------------------
class Mesh:
    def __init__(self):
        h = ctypes.c_void_p()
        _check(lib().bem_mesh_create(ctypes.byref(h)))
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _lib is not None:
            _lib.bem_mesh_destroy(h)
            self._h = None

    @property
    def handle(self):
        return self._h

    # reference names
    def readObj(self, path: str) -> int:
        _check(lib().bem_mesh_read_obj(self._h, os.fsencode(path)))
        return SUCCESS

    def findBB(self, threshold: float) -> int:
        _check(lib().bem_mesh_find_bb(self._h, float(threshold)))
        return SUCCESS

    def genCHIEF(self, num: int, threshold: float) -> int:
        _check(lib().bem_mesh_gen_chief(self._h, int(num), float(threshold)))
        return SUCCESS

    def getNumPnts(self) -> int:
        return self.counts()[0]

    def getNumElems(self) -> int:
        return self.counts()[1]

    def getNumChief(self) -> int:
        return self.counts()[2]

    # extensions
    read_obj = readObj

    def read_obj_robust(self, path: str) -> None:
        _check(lib().bem_mesh_read_obj_robust(self._h, os.fsencode(path)))

    def read_ply(self, path: str) -> None:
        _check(lib().bem_mesh_read_ply(self._h, os.fsencode(path)))

    def orient(self) -> dict:
        """Consistent winding with (p1-p3) x (p2-p3) into the body; returns
        flipped / components / open_edges / nonmanifold / volume."""
        v = [ctypes.c_int() for _ in range(4)]
        vol = ctypes.c_double()
        _check(lib().bem_mesh_orient(self._h, *[ctypes.byref(x) for x in v], ctypes.byref(vol)))
        return dict(zip(("flipped", "components", "open_edges", "nonmanifold"), (x.value for x in v)),
                    volume=vol.value)

    def set(self, pnts, elems) -> None:
        p = np.ascontiguousarray(pnts, dtype=np.float64).reshape(-1, 3)
        e = np.ascontiguousarray(elems, dtype=np.int32).reshape(-1, 3)
        _check(lib().bem_mesh_set(self._h, _ptr(p), p.shape[0], _ptr(e), e.shape[0]))

    def set_bc(self, bc) -> None:
        """bc: (E, 3) complex array of (ca, cb, cc)."""
        b = np.ascontiguousarray(np.asarray(bc, dtype=np.complex128).reshape(-1, 3))
        _check(lib().bem_mesh_set_bc(self._h, _ptr(b)))

    def set_uniform_bc(self, ca, cb, cc) -> None:
        ca, cb, cc = complex(ca), complex(cb), complex(cc)
        _check(lib().bem_mesh_set_uniform_bc(self._h, ca.real, ca.imag, cb.real, cb.imag, cc.real, cc.imag))

    def set_chief(self, pts) -> None:
        p = np.ascontiguousarray(pts, dtype=np.float64).reshape(-1, 3)
        _check(lib().bem_mesh_set_chief(self._h, _ptr(p) if p.size else None, p.shape[0]))

    def counts(self):
        n, e, m = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        _check(lib().bem_mesh_get_counts(self._h, ctypes.byref(n), ctypes.byref(e), ctypes.byref(m)))
        return n.value, e.value, m.value

    def points(self) -> np.ndarray:
        n = self.counts()[0]
        p = np.zeros((n, 3))
        _check(lib().bem_mesh_get_points(self._h, _ptr(p)))
        return p

    def elems(self) -> np.ndarray:
        e = np.zeros((self.counts()[1], 3), dtype=np.int32)
        _check(lib().bem_mesh_get_elems(self._h, _ptr(e)))
        return e

    def chief(self) -> np.ndarray:
        m = self.counts()[2]
        c = np.zeros((m, 3))
        if m:
            _check(lib().bem_mesh_get_chief(self._h, _ptr(c)))
        return c

    def bb(self) -> np.ndarray:
        b = np.zeros(6, dtype=np.float32)
        _check(lib().bem_mesh_get_bb(self._h, _ptr(b)))
        return b

    def surface_area(self) -> float:
        a = ctypes.c_double()
        _check(lib().bem_mesh_surface_area(self._h, ctypes.byref(a)))
        return a.value

    @classmethod
    def icosphere(cls, subdiv: int, radius: float = 1.0) -> "Mesh":
        m = cls()
        _check(lib().bem_mesh_icosphere(m._h, int(subdiv), float(radius)))
        return m

    @classmethod
    def geodesic(cls, nu: int, radius: float = 1.0) -> "Mesh":
        m = cls()
        _check(lib().bem_mesh_geodesic(m._h, int(nu), float(radius)))
        return m

    def perturbed_ellipsoid(self, a: float, b: float, c: float, lmax: int = 8, amp: float = 0.05,
                            seed: int = 0) -> "Mesh":
        """Map this unit-sphere mesh onto a seeded, radially perturbed ellipsoid."""
        _check(lib().bem_mesh_perturbed_ellipsoid(self._h, float(a), float(b), float(c), int(lmax),
                                                  float(amp), int(seed)))
        return self

    @classmethod
    def from_arrays(cls, pnts, elems) -> "Mesh":
        m = cls()
        m.set(pnts, elems)
        return m


# ---------------------------------------------------------------------------
# Drop-in calls with host buffers
# ---------------------------------------------------------------------------
def bemSystem(m: Mesh, k: float, srcs, A: np.ndarray | None = None, B: np.ndarray | None = None):
    """bemSystem (mesh.cu:985-1006): returns (A, B) as complex64 Fortran
    arrays of shapes (N+M, N) and (N+M, numSrcs); srcs are point-source
    positions (numSrcs x 3) of strength STRENGTH."""
    n, _, mc = m.counts()
    s = np.ascontiguousarray(srcs, dtype=np.float32).reshape(-1, 3)
    R = n + mc
    if A is None:
        A = np.zeros((R, n), dtype=np.complex64, order="F")
    if B is None:
        B = np.zeros((R, s.shape[0]), dtype=np.complex64, order="F")
    _check(lib().bem_system_c64(m.handle, float(k), _ptr(s), s.shape[0], _ptr(A), A.shape[0], _ptr(B), B.shape[0]))
    return A, B


def qrSolver(A: np.ndarray, B: np.ndarray) -> np.ndarray:
    """qrSolver (numerical.cu:580-644): least squares; B (complex64,
    Fortran) is overwritten and returned, solution in rows 0..n-1."""
    A = np.asfortranarray(A, dtype=np.complex64)
    if B.dtype != np.complex64 or not B.flags.f_contiguous:
        raise ValueError("B must be a complex64 Fortran-ordered array")
    m, n = A.shape
    nb = B.shape[1] if B.ndim == 2 else 1
    _check(lib().bem_qr_solve_c64(_ptr(A), m, n, m, _ptr(B), nb, B.shape[0]))
    return B


def GMRES(A: np.ndarray, b: np.ndarray, maxIter: int, thr: float, x: np.ndarray | None = None) -> np.ndarray:
    """GMRES (GMRES.cu:145-279) on a square complex64 system; x is the
    initial guess (zeros by default) and is overwritten."""
    A = np.asfortranarray(A, dtype=np.complex64)
    m = A.shape[0]
    b = np.ascontiguousarray(b, dtype=np.complex64).reshape(m)
    if x is None:
        x = np.zeros(m, dtype=np.complex64)
    _check(lib().bem_gmres_c64(_ptr(A), _ptr(b), m, int(maxIter), float(thr), _ptr(x)))
    return x


def tc_gemm(A: np.ndarray, B: np.ndarray, trans: bool = False, parts: int = 2) -> np.ndarray:
    """C = op(A) B on the tcgen05 tensor cores (bem_tc_gemm_f32): A float32
    (op(A) = A, or A^T when trans), B float32 (k x n); fp16 split products,
    parts = 2 (TF32x3-level accuracy) or 3 (FP32-level)."""
    A = np.asarray(A, dtype=np.float32)
    rows, cols = A.shape
    lda = (cols + 3) // 4 * 4
    Ap = np.zeros((rows, lda), dtype=np.float32)
    Ap[:, :cols] = A
    m, k = (cols, rows) if trans else (rows, cols)
    Bf = np.asfortranarray(B, dtype=np.float32)
    if Bf.shape[0] != k:
        raise ValueError("tc_gemm: inner dimensions differ")
    n = Bf.shape[1]
    C = np.zeros((m, n), dtype=np.float32, order="F")
    _check(lib().bem_tc_gemm_f32(1 if trans else 0, m, k, n, _ptr(Ap), lda, _ptr(Bf), k, _ptr(C), m, int(parts)))
    return C


def genExtPressure(k: float, m: Mesh, src, x, surfP) -> complex:
    """genExtPressure (mesh.cu:1038-1073): pressure at x from the surface
    pressure surfP (complex64, numPnts)."""
    s = np.ascontiguousarray(src, dtype=np.float32).reshape(3)
    xx = np.ascontiguousarray(x, dtype=np.float32).reshape(3)
    u = np.ascontiguousarray(surfP, dtype=np.complex64).reshape(-1)
    out = np.zeros(1, dtype=np.complex64)
    _check(lib().bem_ext_pressure_c64(float(k), m.handle, _ptr(s), _ptr(xx), _ptr(u), _ptr(out)))
    return complex(out[0])


def wrtCplxMat(mat: np.ndarray, path: str) -> int:
    """wrtCplxMat (numerical.cu:556-578): '(%f,%f) ' per entry, one line per row."""
    a = np.asfortranarray(np.atleast_2d(mat), dtype=np.complex64)
    _check(lib().bem_write_cplx_mat_c64(_ptr(a), a.shape[0], a.shape[1], a.shape[0], os.fsencode(path)))
    return SUCCESS


# ---------------------------------------------------------------------------
# Device-resident solver
# ---------------------------------------------------------------------------
class Solver:
    def __init__(self, **opts):
        h = ctypes.c_void_p()
        _check(lib().bem_solver_create(ctypes.byref(h)))
        self._h = h
        if opts:
            self.set_options(**opts)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _lib is not None:
            _lib.bem_solver_destroy(h)
            self._h = None

    @property
    def handle(self):
        return self._h

    def options(self) -> Options:
        o = Options()
        _check(lib().bem_solver_get_options(self._h, ctypes.byref(o)))
        return o

    def set_options(self, **kw) -> None:
        o = self.options()
        for key, v in kw.items():
            if not hasattr(o, key):
                raise KeyError(key)
            setattr(o, key, v)
        _check(lib().bem_solver_set_options(self._h, ctypes.byref(o)))

    def set_mesh(self, m: Mesh) -> None:
        _check(lib().bem_solver_set_mesh(self._h, m.handle))

    def set_geometry(self, pnts, elems, bc=None, chief=None) -> None:
        p = np.ascontiguousarray(pnts, dtype=np.float64).reshape(-1, 3)
        e = np.ascontiguousarray(elems, dtype=np.int32).reshape(-1, 3)
        b = None if bc is None else np.ascontiguousarray(np.asarray(bc, dtype=np.complex128).reshape(-1, 3))
        c = None if chief is None else np.ascontiguousarray(chief, dtype=np.float64).reshape(-1, 3)
        nc = 0 if c is None else c.shape[0]
        _check(lib().bem_solver_set_geometry(self._h, _ptr(p), p.shape[0], _ptr(e), e.shape[0],
                                             _ptr(b) if b is not None else None,
                                             _ptr(c) if (c is not None and nc) else None, nc))

    def set_sources(self, srcs) -> None:
        arr = sources(srcs)
        _check(lib().bem_solver_set_sources(self._h, arr, len(arr)))

    def sizes(self):
        v = [ctypes.c_int() for _ in range(4)]
        _check(lib().bem_solver_sizes(self._h, *[ctypes.byref(x) for x in v]))
        return tuple(x.value for x in v)

    def block_gemm_mode(self) -> int:
        """GEMM_* mode of the last block solve's products (AUTO's choice)."""
        v = ctypes.c_int()
        _check(lib().bem_solver_block_gemm_mode(self._h, ctypes.byref(v)))
        return v.value

    def far_variant(self) -> int:
        """Launch shape of the far kernel in the last c64 assembly (-1: none)."""
        v = ctypes.c_int()
        _check(lib().bem_solver_far_variant(self._h, ctypes.byref(v)))
        return v.value

    def assemble(self, k: float, precision: int = PREC_C64) -> None:
        _check(lib().bem_solver_assemble(self._h, float(k), int(precision)))

    def solve(self, method: int = SOLVE_GMRES_REFINED, check: bool = True) -> SolveInfo:
        info = SolveInfo()
        st = lib().bem_solver_solve(self._h, int(method), ctypes.byref(info))
        if check or st != ERR_NOT_CONVERGED:
            _check(st)
        return info

    def solution(self, precision: int = PREC_C128, out: np.ndarray | None = None) -> np.ndarray:
        """Surface pressure (N x S, Fortran order); `out` may be a
        caller-owned (e.g. pinned) array of the right dtype and shape."""
        n, _, _, s = self.sizes()
        dt = np.complex64 if precision == PREC_C64 else np.complex128
        x = np.zeros((n, s), dtype=dt, order="F") if out is None else out
        if x.dtype != dt or x.shape != (n, s) or not x.flags.f_contiguous:
            raise ValueError("solution buffer must be an (N, S) Fortran array of the requested precision")
        _check(lib().bem_solver_get_solution(self._h, _ptr(x), n, int(precision)))
        return x

    def system(self, precision: int = PREC_C128):
        n, m, _, s = self.sizes()
        dt = np.complex64 if precision == PREC_C64 else np.complex128
        A = np.zeros((n + m, n), dtype=dt, order="F")
        B = np.zeros((n + m, s), dtype=dt, order="F")
        _check(lib().bem_solver_get_system(self._h, _ptr(A), n + m, _ptr(B), n + m, int(precision)))
        return A, B

    def field(self, pts, precision: int = PREC_C128) -> np.ndarray:
        p = np.ascontiguousarray(pts, dtype=np.float64).reshape(-1, 3)
        s = self.sizes()[3]
        dt = np.complex64 if precision == PREC_C64 else np.complex128
        out = np.zeros((p.shape[0], s), dtype=dt, order="F")
        _check(lib().bem_solver_eval_field(self._h, _ptr(p), p.shape[0], _ptr(out), p.shape[0], int(precision)))
        return out

    def sync(self) -> None:
        _check(lib().bem_solver_sync(self._h))

    def stream(self) -> int:
        return int(lib().bem_solver_stream(self._h) or 0)


# ---------------------------------------------------------------------------
# Request server (continuous batching of independent solves)
# ---------------------------------------------------------------------------
class Server:
    """Concurrent surface solves on one GPU (``bem_server_*``): requests are
    admitted by device footprint while others run, assembled systems are
    cached by geometry and wavenumber.  ``slots``, ``hbm_budget_bytes``,
    ``cache_systems`` and ``block_min_sources`` are server options; any other
    keyword is a solver option (``Options``)."""

    def __init__(self, **kw):
        o = ServerOptions()
        _check(lib().bem_server_options_default(ctypes.byref(o)))
        for key, v in kw.items():
            if key in ("slots", "hbm_budget_bytes", "cache_systems", "block_min_sources"):
                setattr(o, key, v)
            elif hasattr(o.solver, key):
                setattr(o.solver, key, v)
            else:
                raise KeyError(key)
        h = ctypes.c_void_p()
        _check(lib().bem_server_create(ctypes.byref(o), ctypes.byref(h)))
        self._h = h
        self._shapes = {}

    def close(self) -> None:
        h = getattr(self, "_h", None)
        if h and _lib is not None:
            _lib.bem_server_destroy(h)
            self._h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def submit(self, pnts, elems, k: float, srcs, bc=None, chief=None) -> int:
        p = np.ascontiguousarray(pnts, dtype=np.float64).reshape(-1, 3)
        e = np.ascontiguousarray(elems, dtype=np.int32).reshape(-1, 3)
        b = None if bc is None else np.ascontiguousarray(np.asarray(bc, dtype=np.complex128).reshape(-1, 3))
        c = None if chief is None else np.ascontiguousarray(chief, dtype=np.float64).reshape(-1, 3)
        nc = 0 if c is None else c.shape[0]
        arr = sources(srcs)
        r = Request(p.ctypes.data, p.shape[0], e.ctypes.data, e.shape[0],
                    b.ctypes.data if b is not None else None, c.ctypes.data if nc else None, nc,
                    float(k), ctypes.cast(arr, ctypes.c_void_p), len(arr))
        t = ctypes.c_longlong()
        _check(lib().bem_server_submit(self._h, ctypes.byref(r), ctypes.byref(t)))
        self._shapes[t.value] = (p.shape[0], len(arr))
        return t.value

    def wait(self, ticket: int, timeout: float = -1.0, check: bool = True):
        """(x, result): x is the N x S c128 surface pressure (Fortran order)."""
        n, s = self._shapes[ticket]
        x = np.zeros((n, s), dtype=np.complex128, order="F")
        res = RequestResult()
        st = lib().bem_server_wait(self._h, int(ticket), float(timeout), _ptr(x), n, ctypes.byref(res))
        if st == ERR_TIMEOUT:
            _check(st)
        self._shapes.pop(ticket, None)
        if check or st != ERR_NOT_CONVERGED:
            _check(st)
        out = {f: getattr(res, f) for f, _ in RequestResult._fields_}
        return x, out

    def stats(self) -> dict:
        st = ServerStats()
        _check(lib().bem_server_stats(self._h, ctypes.byref(st)))
        return {f: getattr(st, f) for f, _ in ServerStats._fields_}

    def reset_stats(self) -> None:
        _check(lib().bem_server_reset_stats(self._h))
