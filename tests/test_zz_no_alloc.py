"""GMRES on caller-owned device buffers, with no allocation inside the call.

This entry point exists for callers that cannot allocate GPU memory while
they solve: a serving process whose device memory is owned and capped by its
own pool allocator, code that must not add allocations while another
component's CUDA stream capture is running, or a real-time loop that cannot
pay for cudaMalloc's latency and implicit synchronisation.  They already hold
A, b and x on the device and hand them over; the solver's scratch comes from a
fixed static device array.

The checks: on two calls in a row (different systems, the shared scratch
keeping the first call's contents), the allocation-free entry point agrees
with the host-buffer GMRES entry point within the tolerance of the other
GMRES tests; so it does for an odd order (the padded leading dimension), a
non-zero initial guess, an initial guess that already meets the threshold
(no iteration, x unchanged) and a run of the full min(max_iter, m)
iterations; sizes above the stated maximum are refused.
"""
import ctypes

import numpy as np
import pytest

from helpers import rel_err, uv_sphere

pytestmark = pytest.mark.gpu

TOL = 1e-5


def _system(bemlib, k, subdiv):
    m = bemlib.Mesh.icosphere(subdiv, 1.0)
    bemlib.set_point_source_strength(1.0)
    try:
        A, B = bemlib.bemSystem(m, k, [3.0, 0.5, 0.0])
    finally:
        bemlib.set_point_source_strength(0.0)
    return A, B[:, 0].copy()


def _device_colmajor(torch, A):
    """A (m x m) as a caller would hold it on the device: column-major c64
    with an even leading dimension."""
    m = A.shape[0]
    lda = m + (m % 2)
    dev = torch.zeros((m, lda), dtype=torch.complex64, device="cuda")
    dev[:, :m] = torch.from_numpy(np.ascontiguousarray(A.T))   # row j of dev = column j of A
    return dev, lda


def test_noalloc_gmres_matches_host_entry_point(bemlib):
    torch = pytest.importorskip("torch")
    L = bemlib.lib()
    for k, subdiv in [(1.1, 2), (2.7, 3)]:          # two calls in a row
        A, b = _system(bemlib, k, subdiv)
        m = A.shape[0]
        x_ref = bemlib.GMRES(A, b, min(m, 128), 1e-6)
        A_dev, lda = _device_colmajor(torch, A)
        b_dev = torch.from_numpy(b.astype(np.complex64)).cuda()
        x_dev = torch.zeros(m, dtype=torch.complex64, device="cuda")
        torch.cuda.synchronize()
        it = ctypes.c_int(-1)
        st = L.bem_gmres_c64_noalloc(A_dev.data_ptr(), lda, b_dev.data_ptr(), m, min(m, 128), 1e-6,
                                     x_dev.data_ptr(), None, ctypes.byref(it))
        assert st == 0, L.bem_last_error()
        x = x_dev.cpu().numpy()
        assert 0 < it.value <= 128
        assert rel_err(x, x_ref) < TOL
        xd = np.linalg.solve(A.astype(np.complex128), b.astype(np.complex128))
        assert rel_err(x, xd) < TOL


def _noalloc(L, A_dev, lda, b_dev, m, max_iter, thr, x_dev):
    it = ctypes.c_int(-1)
    st = L.bem_gmres_c64_noalloc(A_dev.data_ptr(), lda, b_dev.data_ptr(), m, max_iter, thr, x_dev.data_ptr(),
                                 None, ctypes.byref(it))
    assert st == 0, L.bem_last_error()
    return it.value


def test_noalloc_gmres_odd_order_initial_guess_and_full_run(bemlib):
    torch = pytest.importorskip("torch")
    L = bemlib.lib()
    p, e = uv_sphere(19, 39)                         # 743 nodes: odd order, lda = m + 1
    mesh = bemlib.Mesh.from_arrays(p, e)
    mesh.orient()
    bemlib.set_point_source_strength(1.0)
    try:
        A, B = bemlib.bemSystem(mesh, 1.7, [3.0, 0.5, 0.0])
    finally:
        bemlib.set_point_source_strength(0.0)
    b = B[:, 0].copy()
    m = A.shape[0]
    assert m % 2 == 1
    A_dev, lda = _device_colmajor(torch, A)
    assert lda == m + 1
    b_dev = torch.from_numpy(b.astype(np.complex64)).cuda()
    xd = np.linalg.solve(A.astype(np.complex128), b.astype(np.complex128))
    # zero initial guess
    x_dev = torch.zeros(m, dtype=torch.complex64, device="cuda")
    it0 = _noalloc(L, A_dev, lda, b_dev, m, 128, 1e-6, x_dev)
    x0 = x_dev.cpu().numpy()
    assert 0 < it0 <= 128 and rel_err(x0, xd) < TOL
    assert rel_err(x0, bemlib.GMRES(A, b, 128, 1e-6)) < TOL
    # non-zero initial guess (r = b - A x0 path)
    guess = (0.5 * xd).astype(np.complex64)
    x_dev = torch.from_numpy(guess.copy()).cuda()
    it1 = _noalloc(L, A_dev, lda, b_dev, m, 128, 1e-6, x_dev)
    assert 0 < it1 <= 128
    assert rel_err(x_dev.cpu().numpy(), bemlib.GMRES(A, b, 128, 1e-6, x=guess.copy())) < TOL
    assert rel_err(x_dev.cpu().numpy(), xd) < TOL
    # an initial guess that already meets the threshold: no iteration, unchanged
    x_dev = torch.from_numpy(x0.copy()).cuda()
    it2 = _noalloc(L, A_dev, lda, b_dev, m, 128, 1e-3, x_dev)
    assert it2 == 0
    np.testing.assert_array_equal(x_dev.cpu().numpy(), x0)
    # threshold 0: exactly min(max_iter, m) = 128 iterations
    x_dev = torch.zeros(m, dtype=torch.complex64, device="cuda")
    it3 = _noalloc(L, A_dev, lda, b_dev, m, 128, 0.0, x_dev)
    assert it3 == 128
    assert rel_err(x_dev.cpu().numpy(), xd) < TOL


def test_noalloc_gmres_refuses_oversized_problems(bemlib):
    torch = pytest.importorskip("torch")
    L = bemlib.lib()
    small = torch.zeros(8, dtype=torch.complex64, device="cuda")
    p = small.data_ptr()
    # Every case below is refused by the argument checks before any device
    # work, so the tiny buffer is never read.
    m = 2048 + 2                                     # above BEM_NOALLOC_MAX_M
    st = L.bem_gmres_c64_noalloc(p, m, p, m, 10, 1e-6, p, None, None)
    assert st == 8 and b"2048" in L.bem_last_error()
    st = L.bem_gmres_c64_noalloc(p, 200, p, 200, 200, 1e-6, p, None, None)   # 200 iterations > 128
    assert st == 8
    st = L.bem_gmres_c64_noalloc(p, 3, p, 3, 3, 1e-6, p, None, None)         # odd lda
    assert st == 2
