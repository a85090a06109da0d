"""GPU test of the allocation-free SVD entry point (qr_svd_noalloc).

Callers that own all device memory (a Julia CUDA.jl pool, a serving loop that only allocates at
start-up) pass their own device buffers; the entry point keeps its scratch in a static device
array.  Here its results are checked, on calls in a row with different shapes, against the
allocating SVD entry point of the same library and against LAPACK (numpy.linalg.svd), with the
tolerance of the other SVD tests (1e-10 relative on singular values and on U S Vh).  Cases cover
tall and wide blocks, the QR-preconditioned sweeps (more than 32 columns) and the plain ones, a
rank-deficient block (zero singular values, the re-orthonormalisation branch), an odd column count
(padding column), 12 decades of singular values, and entries near the ends of the FP64 range.
Device buffers come from torch, standing in for the caller's own pool.
"""
import ctypes as C

import numpy as np
import pytest

from qrochet import _lib
from qrochet import random as R

pytestmark = pytest.mark.gpu

TOL = 1e-10


def _reference_svd(A):
    m, n = A.shape
    k = min(m, n)
    A = np.asfortranarray(A)
    U = np.empty((m, k), dtype=np.complex128, order="F")
    Vh = np.empty((k, n), dtype=np.complex128, order="F")
    S = np.empty(k)
    ms = C.c_double()
    _lib.check(_lib.lib().qr_test_svd(0, m, n, _lib.dptr(A), _lib.dptr(U), _lib.dptr(S), _lib.dptr(Vh), C.byref(ms)))
    return U, S, Vh


def _noalloc_svd(torch, A):
    m, n = A.shape
    k = min(m, n)
    dev = torch.device("cuda:0")
    # column-major buffers: a (n, m) row-major tensor is the (m, n) column-major matrix
    a = torch.from_numpy(np.ascontiguousarray(A.T)).to(dev)
    u = torch.empty((k, m), dtype=torch.complex128, device=dev)
    s = torch.empty((k,), dtype=torch.float64, device=dev)
    vh = torch.empty((n, k), dtype=torch.complex128, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    torch.cuda.synchronize(dev)
    _lib.check(_lib.lib().qr_svd_noalloc(m, n, a.data_ptr(), m, u.data_ptr(), m, s.data_ptr(), vh.data_ptr(), k,
                                         stream))
    return u.cpu().numpy().T, s.cpu().numpy(), vh.cpu().numpy().T


def _check(A, got, ref):
    U, S, Vh = got
    Ur, Sr, Vhr = ref
    smax = Sr[0]
    s_lapack = np.linalg.svd(A, compute_uv=False)
    assert np.max(np.abs(S - s_lapack)) <= TOL * s_lapack[0]
    assert np.max(np.abs(S - Sr)) <= TOL * smax
    assert np.max(np.abs((U * S) @ Vh - (Ur * Sr) @ Vhr)) <= TOL * smax * np.sqrt(max(A.shape))
    assert np.max(np.abs((U * S) @ Vh - A)) <= TOL * smax * np.sqrt(max(A.shape))
    k = S.size
    assert np.max(np.abs(U.conj().T @ U - np.eye(k))) <= TOL
    assert np.max(np.abs(Vh @ Vh.conj().T - np.eye(k))) <= TOL


def test_noalloc_svd_matches_allocating_svd_twice():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    g = R.rng(4242)
    first = R.complex_gaussian(g, (300, 200))   # tall
    second = R.complex_gaussian(g, (150, 400))  # wide: the scratch holds the first call's data
    for A in (first, second):
        _check(A, _noalloc_svd(torch, A), _reference_svd(A))


def _graded(g, m, n, decades):
    u, _ = np.linalg.qr(R.complex_gaussian(g, (m, min(m, n))))
    v, _ = np.linalg.qr(R.complex_gaussian(g, (n, min(m, n))))
    return (u * np.logspace(0, -decades, min(m, n))) @ v.conj().T


def test_noalloc_svd_hard_cases():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    g = R.rng(77)
    cases = [
        R.complex_gaussian(g, (200, 60)) @ R.complex_gaussian(g, (60, 101)),  # 200 x 101, rank 60
        _graded(g, 240, 240, 12),                                             # 12 decades
        R.complex_gaussian(g, (90, 31)),                                      # odd k, no QR step
        R.complex_gaussian(g, (25, 300)),                                     # wide, no QR step
        _graded(g, 120, 333, 10),                                             # wide, odd rows
    ]
    for A in cases:
        _check(A, _noalloc_svd(torch, A), _reference_svd(A))


@pytest.mark.parametrize("scale", [1e-170, 1e170])
def test_noalloc_svd_extreme_scales(scale):
    """Entries near the ends of the FP64 range: the power-of-two prescale keeps the rotation test's
    squared norms finite, and S comes back in the caller's scale."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    g = R.rng(31)
    for shape in ((160, 90), (40, 20)):
        A0 = R.complex_gaussian(g, shape)
        U, S, Vh = _noalloc_svd(torch, A0 * scale)
        s0 = np.linalg.svd(A0, compute_uv=False)
        assert np.max(np.abs(S / scale - s0)) <= TOL * s0[0]
        assert np.max(np.abs((U * (S / scale)) @ Vh - A0)) <= TOL * s0[0] * np.sqrt(max(shape))
        k = S.size
        assert np.max(np.abs(U.conj().T @ U - np.eye(k))) <= TOL
        assert np.max(np.abs(Vh @ Vh.conj().T - np.eye(k))) <= TOL


def test_noalloc_svd_rejects_sizes_above_the_limit():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    with pytest.raises(_lib.ArgumentError, match="scratch limit"):
        _noalloc_svd(torch, np.ones((600, 10), dtype=np.complex128))
    with pytest.raises(_lib.ArgumentError, match="scratch limit"):
        _noalloc_svd(torch, np.ones((300, 300), dtype=np.complex128))
