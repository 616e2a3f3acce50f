"""Hierarchical form of the engine's own c64 system matrix
(`bem_hmat_compress_c64`, `bem_hmat_matvec_c64`) against plain torch
products with the dense matrix (complex128 accumulation of the same c64
entries).  Workload: unit icosphere, ka = 10, 8 seeded CHIEF rows, the
partition of `bem_hmat_partition` (eta = 1).  Bounds: the products' relative
error stays below 0.5 tol + 2e-6 (partially pivoted ACA lands near 0.1 tol
on these blocks; 2e-6 covers the FP32 sums of both sides); the products are
bitwise repeatable; at subdivision 5 the compressed form holds well under
half of the dense entries."""
import numpy as np
import pytest

from helpers import icosphere

pytestmark = pytest.mark.gpu


def _clustered_system(bemlib, subdiv, leaf):
    p, el = icosphere(subdiv)
    c = np.random.default_rng(1).uniform(-0.3, 0.3, (8, 3))
    s = bemlib.Solver(near_eta=1.0, near_depth=2)
    s.set_geometry(p, el, chief=c)
    s.set_sources([("plane", (0, 0, 1), 1.0)])
    s.assemble(10.0, bemlib.PREC_C64)
    A, _ = s.system(bemlib.PREC_C64)
    rp, cp, blocks = bemlib.hmat_partition(np.vstack([p, c]), p, leaf, 1.0)
    return np.ascontiguousarray(A[rp][:, cp]), blocks


@pytest.fixture(scope="module")
def s4(bemlib):
    return _clustered_system(bemlib, 4, 64)


def _vectors(torch, R, N):
    g = torch.Generator().manual_seed(0)
    x = torch.randn(N, dtype=torch.complex64, generator=g).cuda()
    y = torch.randn(R, dtype=torch.complex64, generator=g).cuda()
    return x, y


def _rel(a, b):
    return float((a.to(b.dtype) - b).norm() / b.norm())


@pytest.mark.parametrize("tol", [1e-4, 1e-6])
def test_hmat_products_match_dense(bemlib, s4, tol):
    import torch
    Ap, blocks = s4
    R, N = Ap.shape
    Ad = torch.from_numpy(Ap).cuda()
    H = bemlib.HMatrix(Ad.data_ptr(), R, N, N, blocks, tol=tol, kmax=64)
    x, y = _vectors(torch, R, N)
    hx = torch.empty(R, dtype=torch.complex64, device="cuda")
    hy = torch.empty(N, dtype=torch.complex64, device="cuda")
    H.matvec(x.data_ptr(), hx.data_ptr(), 0)
    H.matvec(y.data_ptr(), hy.data_ptr(), 1)
    torch.cuda.synchronize()
    A64 = Ad.to(torch.complex128)
    ref = A64 @ x.to(torch.complex128)
    refh = A64.conj().T @ y.to(torch.complex128)
    bound = 0.5 * tol + 2e-6
    assert _rel(hx, ref) < bound
    assert _rel(hy, refh) < bound
    info = H.info()
    assert info["lowrank_blocks"] > 0 and 1 <= info["max_rank"] <= 64
    assert info["entries"] < R * N
    # bitwise repeatable
    hx2 = torch.empty_like(hx)
    H.matvec(x.data_ptr(), hx2.data_ptr(), 0)
    torch.cuda.synchronize()
    assert torch.equal(hx, hx2)
    H.close()


def test_hmat_compression_at_subdivision_5(bemlib):
    import torch
    Ap, blocks = _clustered_system(bemlib, 5, 128)
    R, N = Ap.shape
    Ad = torch.from_numpy(Ap).cuda()
    H = bemlib.HMatrix(Ad.data_ptr(), R, N, N, blocks, tol=1e-4, kmax=64)
    info = H.info()
    x, _ = _vectors(torch, R, N)
    hx = torch.empty(R, dtype=torch.complex64, device="cuda")
    H.matvec(x.data_ptr(), hx.data_ptr(), 0)
    torch.cuda.synchronize()
    ref = Ad.to(torch.complex128) @ x.to(torch.complex128)
    assert _rel(hx, ref) < 0.5e-4 + 2e-6
    assert info["entries"] < 0.5 * R * N, info
    H.close()


def test_hmat_argument_errors(bemlib, s4):
    import torch
    Ap, blocks = s4
    R, N = Ap.shape
    Ad = torch.from_numpy(Ap[:64, :64].copy()).cuda()
    with pytest.raises(bemlib.BemError) as e:   # blocks that do not tile the matrix
        bemlib.HMatrix(Ad.data_ptr(), 64, 64, 64, blocks, tol=1e-4)
    assert e.value.status == bemlib.ERR_INVALID_ARG
    one = np.array([[0, 64, 0, 64, 0]], dtype=np.int32)
    for tol, kmax in ((0.0, 16), (1e-4, 0), (1e-4, 129)):
        with pytest.raises(bemlib.BemError) as e:
            bemlib.HMatrix(Ad.data_ptr(), 64, 64, 64, one, tol=tol, kmax=kmax)
        assert e.value.status == bemlib.ERR_INVALID_ARG
    # a single dense block reproduces the matrix product exactly
    H = bemlib.HMatrix(Ad.data_ptr(), 64, 64, 64, one, tol=1e-4)
    assert H.info() == {"entries": 64 * 64, "max_rank": 0, "lowrank_blocks": 0, "dense_blocks": 1}
    x, _ = _vectors(torch, 64, 64)
    hx = torch.empty(64, dtype=torch.complex64, device="cuda")
    H.matvec(x.data_ptr(), hx.data_ptr(), 0)
    torch.cuda.synchronize()
    assert _rel(hx, Ad.to(torch.complex128) @ x.to(torch.complex128)) < 1e-6
    H.close()
