"""Kernel-level GPU checks through the C ABI test hooks: the FP64 DMMA ZGEMM against NumPy, and
the thin SVD / Householder QR against LAPACK (through NumPy) on tall, wide, rank-deficient and
graded matrices.  FP64 tolerance 1e-12 relative (GEMM) and 1e-10 relative on gauge-invariant SVD
quantities (singular values, U S Vh); the mixed SVD is held to the same bar because its singular
values and vectors come out of the FP64 refinement."""
import ctypes as C

import numpy as np
import pytest

from qrochet import _lib
from qrochet import random as R

pytestmark = pytest.mark.gpu

OPS = {0: lambda x: x, 1: lambda x: x.T, 2: lambda x: x.conj().T, 3: lambda x: x.conj()}


def _p(a):
    return _lib.dptr(a)


def zgemm(opA, opB, A, B, Cm, alpha=1.0, beta=0.0, dk=None):
    M, N = Cm.shape
    K = OPS[opA](A).shape[1]
    A = np.asfortranarray(A, dtype=np.complex128)
    B = np.asfortranarray(B, dtype=np.complex128)
    out = np.asfortranarray(Cm, dtype=np.complex128).copy(order="F")
    al = np.array([complex(alpha).real, complex(alpha).imag])
    be = np.array([complex(beta).real, complex(beta).imag])
    ms = C.c_double()
    dkp = None if dk is None else _p(np.ascontiguousarray(dk, dtype=np.float64))
    _lib.check(_lib.lib().qr_test_zgemm(opA, opB, M, N, K, _p(al), _p(A), A.shape[0], _p(B), B.shape[0],
                                        _p(be), _p(out), M, dkp, 1, C.byref(ms)))
    return out


@pytest.mark.parametrize("opA", [0, 1, 2, 3])
@pytest.mark.parametrize("opB", [0, 1, 2, 3])
def test_zgemm_ops(opA, opB):
    g = R.rng(100 + 4 * opA + opB)
    M, N, K = 77, 45, 130
    A0 = R.complex_gaussian(g, (M, K))
    B0 = R.complex_gaussian(g, (K, N))
    A = OPS[opA](A0) if opA in (0, 3) else A0.T.copy() if opA == 1 else A0.conj().T.copy()
    B = OPS[opB](B0) if opB in (0, 3) else B0.T.copy() if opB == 1 else B0.conj().T.copy()
    A = A if opA != 3 else A0.conj()
    B = B if opB != 3 else B0.conj()
    Cm = R.complex_gaussian(g, (M, N))
    alpha, beta = 0.7 - 0.2j, -0.3 + 0.4j
    dk = g.random(K)
    got = zgemm(opA, opB, A, B, Cm, alpha, beta, dk)
    ref = alpha * (OPS[opA](A) * dk[None, :]) @ OPS[opB](B) + beta * Cm
    assert np.max(np.abs(got - ref)) <= 1e-12 * np.max(np.abs(ref))


def test_zgemm_large_exact_tiles():
    g = R.rng(7)
    A = R.complex_gaussian(g, (256, 512))
    B = R.complex_gaussian(g, (512, 192))
    got = zgemm(0, 0, A, B, np.zeros((256, 192)))
    assert np.max(np.abs(got - A @ B)) <= 1e-12 * np.max(np.abs(A @ B))


def svd(mode, A):
    A = np.asfortranarray(A, dtype=np.complex128)
    m, n = A.shape
    k = min(m, n)
    U = np.empty((m, k), dtype=np.complex128, order="F")
    Vh = np.empty((k, n), dtype=np.complex128, order="F")
    S = np.empty(k)
    ms = C.c_double()
    _lib.check(_lib.lib().qr_test_svd(mode, m, n, _p(A), _p(U), _p(S), _p(Vh), C.byref(ms)))
    return U, S, Vh


def _graded(g, m, n, decades):
    u, _ = np.linalg.qr(R.complex_gaussian(g, (m, min(m, n))))
    v, _ = np.linalg.qr(R.complex_gaussian(g, (n, min(m, n))))
    s = np.logspace(0, -decades, min(m, n))
    return (u * s) @ v.conj().T


CASES = {
    "square": lambda g: R.complex_gaussian(g, (96, 96)),
    "tall": lambda g: R.complex_gaussian(g, (200, 64)),
    "wide": lambda g: R.complex_gaussian(g, (48, 130)),
    "rank2": lambda g: R.complex_gaussian(g, (60, 2)) @ R.complex_gaussian(g, (2, 50)),
    "graded12": lambda g: _graded(g, 80, 80, 12),
    "zero_cols": lambda g: np.hstack([R.complex_gaussian(g, (40, 10)), np.zeros((40, 6))]),
    "tiny": lambda g: R.complex_gaussian(g, (2, 1)),
    # cluster kernels for <= 128 columns of <= 128 rows: an odd number of 4-column blocks with a
    # partial last block, and the largest size (16 block pairs, 10 decades of singular values)
    "blocks_odd": lambda g: R.complex_gaussian(g, (120, 33)),
    "graded128": lambda g: _graded(g, 128, 128, 10),
    # above 128 columns the mixed mode takes the FP32-preconditioned path with the polish sweeps
    "square300": lambda g: R.complex_gaussian(g, (300, 300)),
    "wide200x400": lambda g: R.complex_gaussian(g, (200, 400)),
    "graded300": lambda g: _graded(g, 300, 300, 10),
    # 12 decades with random singular vectors: plain Hestenes sweeps converge slowly here, so the
    # FP64 path runs on R^H of a QR and the mixed path falls back to it after its FP32 probe
    "graded600": lambda g: _graded(g, 600, 600, 12),
    "graded_wide": lambda g: _graded(g, 180, 400, 12),
}


@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("case", sorted(CASES))
def test_svd_against_lapack(mode, case):
    g = R.rng(hash(case) % 1000)
    A = CASES[case](g)
    U, S, Vh = svd(mode, A)
    s_ref = np.linalg.svd(A, compute_uv=False)
    smax = s_ref[0]
    assert np.all(np.diff(S) <= 1e-14 * smax)  # descending
    assert np.max(np.abs(S - s_ref)) <= 1e-10 * smax
    assert np.max(np.abs((U * S) @ Vh - A)) <= 1e-10 * smax * np.sqrt(max(A.shape))
    k = S.size
    assert np.max(np.abs(U.conj().T @ U - np.eye(k))) <= 1e-10
    assert np.max(np.abs(Vh @ Vh.conj().T - np.eye(k))) <= 1e-10


def test_qr_against_lapack():
    g = R.rng(5)
    # up to the canonize_site! factorisation of a chi = 1024 site (2048 x 1024), wide and odd shapes
    for m, n in [(64, 32), (32, 64), (50, 50), (2, 1), (1, 3), (257, 300), (2048, 1024)]:
        A = np.asfortranarray(R.complex_gaussian(g, (m, n)))
        k = min(m, n)
        Q = np.empty((m, k), dtype=np.complex128, order="F")
        Rm = np.empty((k, n), dtype=np.complex128, order="F")
        ms = C.c_double()
        _lib.check(_lib.lib().qr_test_qr(m, n, _p(A), _p(Q), _p(Rm), C.byref(ms)))
        assert np.allclose(Q @ Rm, A, atol=1e-12 * np.abs(A).max())
        assert np.allclose(Q.conj().T @ Q, np.eye(k), atol=1e-12)
        assert np.allclose(np.tril(Rm, -1), 0)
        assert np.allclose(np.abs(np.diag(Rm)), np.abs(np.diag(np.linalg.qr(A)[1])), rtol=1e-10)


def zgemm_df(mode, opA, A, B, M, N, D=None):
    K = OPS[opA](A).shape[1]
    A = np.asfortranarray(A, dtype=np.complex128)
    B = np.asfortranarray(B, dtype=np.complex128)
    out = np.zeros((M, N), dtype=np.complex128, order="F")
    Dp = None if D is None else _p(np.asfortranarray(D, dtype=np.complex128))
    ms = C.c_double()
    _lib.check(_lib.lib().qr_test_zgemm_df(mode, opA, M, N, K, _p(A), A.shape[0], _p(B), B.shape[0], Dp, _p(out), M,
                                           1, C.byref(ms)))
    return out


# double-float products: inputs rounded to ~2^-49, compensated sums ~2^-48 of sum |a||b|
DF_TOL = 1e-13


@pytest.mark.parametrize("opA", [0, 1, 2])
def test_zgemm_df_store(opA):
    g = R.rng(400 + opA)
    M, N, K = 90, 70, 300
    A0 = R.complex_gaussian(g, (M, K))
    B0 = R.complex_gaussian(g, (K, N))
    A = {0: A0, 1: A0.T.copy(), 2: A0.conj().T.copy()}[opA]
    got = zgemm_df(0, opA, A, B0, M, N)
    scale = (np.abs(A0) @ np.abs(B0)).max()
    assert np.max(np.abs(got - A0 @ B0)) <= DF_TOL * scale


def test_zgemm_df_large_k_ragged():
    g = R.rng(411)
    M, N, K = 131, 67, 2053  # partial tiles in every dimension
    A0 = R.complex_gaussian(g, (M, K))
    B0 = R.complex_gaussian(g, (K, N))
    got = zgemm_df(0, 0, A0, B0, M, N)
    scale = (np.abs(A0) @ np.abs(B0)).max()
    assert np.max(np.abs(got - A0 @ B0)) <= DF_TOL * scale


def test_zgemm_df_identity_minus_gram():
    """I - X^H X for a unitary X perturbed at 1e-6 (the Newton-Schulz residual): the result is
    ~1e-6 and must be accurate to the double-float level, not the FP32 level."""
    g = R.rng(412)
    k = 160
    q, _ = np.linalg.qr(R.complex_gaussian(g, (k, k)))
    X = q + 1e-6 * R.complex_gaussian(g, (k, k))
    got = zgemm_df(1, 2, X, X, k, k)
    ref = np.eye(k) - X.conj().T @ X
    assert np.max(np.abs(ref)) > 1e-7
    assert np.max(np.abs(got - ref)) <= 1e-13 + 1e-7 * np.max(np.abs(ref))


def test_zgemm_df_axpy_fp32_products():
    g = R.rng(413)
    M, N, K = 100, 80, 120
    A = R.complex_gaussian(g, (M, K))
    Bm = 1e-6 * R.complex_gaussian(g, (K, N))
    D = R.complex_gaussian(g, (M, N))
    got = zgemm_df(2, 0, A, Bm, M, N, D=D)
    ref = D + 0.5 * A @ Bm
    # FP32 products of FP32-rounded inputs: ~1e-7 relative to the correction term, double-float D
    assert np.max(np.abs(got - ref)) <= 1e-6 * 0.5 * (np.abs(A) @ np.abs(Bm)).max() + DF_TOL * np.abs(D).max()


@pytest.mark.parametrize("k", [160, 200])
def test_zgemm_df_gram_half(k):
    """I - X^H X from the tiles on or above the diagonal (mirrored): equal to the full product."""
    g = R.rng(414 + k)
    q, _ = np.linalg.qr(R.complex_gaussian(g, (k, k)))
    X = q + 1e-6 * R.complex_gaussian(g, (k, k))
    half = zgemm_df(3, 2, X, X, k, k)
    full = zgemm_df(1, 2, X, X, k, k)
    ref = np.eye(k) - X.conj().T @ X
    assert np.max(np.abs(half - ref)) <= 1e-13 + 1e-7 * np.max(np.abs(ref))
    # R is stored in FP32: mirrored and directly computed entries differ by ~1 ulp of |R|
    ulp = 2.0 ** -23 * np.max(np.abs(ref))
    assert np.max(np.abs(half - full)) <= 2 * ulp
    assert np.max(np.abs(half - half.conj().T)) <= 2 * ulp
