"""The tcgen05 split-precision complex GEMM (gemm_tc.cu: TMA-staged BF16x3 slices, TMEM
accumulators) against NumPy FP64 products, through the C-ABI test hook.

Tolerance: the 3-way BF16 split carries ~24 significant bits and the accumulation is FP32, so the
error bound is ~sqrt(K) 2^-24 relative to |A||B| (2e-6 scaled by sqrt(K) for random entries; 1e-6
relative in the Frobenius norm at K = 2048, where the six-product split alone leaves ~2e-7).  All 16 op pairs on ragged shapes (padding in M, N and
K), batched products with a shared and with a per-batch B, and a non-negative product whose sums
grow monotonically (where a truncating accumulation would show as a bias).
"""
import ctypes as C

import numpy as np
import pytest

from qrochet import _lib
from qrochet import random as R

pytestmark = pytest.mark.gpu

OPS = {0: lambda x: x, 1: lambda x: x.T, 2: lambda x: x.conj().T, 3: lambda x: x.conj()}
STORE = {0: lambda x: x, 1: lambda x: x.T.copy(), 2: lambda x: x.conj().T.copy(), 3: lambda x: x.conj()}
SPLIT_TOL = 2e-6


def zgemm_tc(opA, opB, As, Bs, M, N, shared_b=False):
    """As: list of stored A matrices (batch), Bs: list of stored B (length 1 when shared)."""
    batch = len(As)
    K = OPS[opA](As[0]).shape[1]
    lda, ldb = As[0].shape[0], Bs[0].shape[0]
    A = np.concatenate([np.asfortranarray(a).ravel(order="F") for a in As]).astype(np.complex128)
    B = np.concatenate([np.asfortranarray(b).ravel(order="F") for b in Bs]).astype(np.complex128)
    sA = As[0].size if batch > 1 else 0
    sB = 0 if shared_b else Bs[0].size
    out = np.zeros(M * N * batch, dtype=np.complex128)
    ms = C.c_double()
    _lib.check(_lib.lib().qr_test_zgemm_tc(opA, opB, M, N, K, batch, _lib.dptr(A), lda, sA, _lib.dptr(B), ldb, sB,
                                           _lib.dptr(out), M, 1, C.byref(ms)))
    return [out[b * M * N:(b + 1) * M * N].reshape((M, N), order="F") for b in range(batch)]


@pytest.mark.parametrize("opA", [0, 1, 2, 3])
@pytest.mark.parametrize("opB", [0, 1, 2, 3])
def test_tc_gemm_ops_ragged(opA, opB):
    g = R.rng(700 + 4 * opA + opB)
    M, N, K = 90, 150, 200
    A0 = R.complex_gaussian(g, (M, K))
    B0 = R.complex_gaussian(g, (K, N))
    got = zgemm_tc(opA, opB, [STORE[opA](A0)], [STORE[opB](B0)], M, N)[0]
    ref = A0 @ B0
    assert np.max(np.abs(got - ref)) <= SPLIT_TOL * np.sqrt(K) * 4


def test_tc_gemm_large_k():
    g = R.rng(9)
    A = R.complex_gaussian(g, (256, 2048))
    B = R.complex_gaussian(g, (2048, 256))
    got = zgemm_tc(0, 0, [A], [B], 256, 256)[0]
    ref = A @ B
    rel = np.linalg.norm(got - ref) / np.linalg.norm(ref)
    assert rel <= 1e-6, rel


def test_tc_gemm_nonnegative_sums():
    g = R.rng(11)
    K = 4096
    A = g.random((128, K)) + 0j
    B = g.random((K, 128)) + 0j
    got = zgemm_tc(0, 0, [A], [B], 128, 128)[0]
    ref = A @ B
    rel = np.max(np.abs(got - ref) / np.abs(ref))
    assert rel <= 1e-6, rel


@pytest.mark.parametrize("shared_b", [True, False])
def test_tc_gemm_batched(shared_b):
    # the shapes of the environment sweep's second contraction: E'_w = Y_w^T conj(B), 5 MPO columns
    g = R.rng(13 + shared_b)
    batch, M, N, K = 5, 96, 80, 160
    Ys = [R.complex_gaussian(g, (K, M)) for _ in range(batch)]
    Bs = [R.complex_gaussian(g, (K, N)) for _ in range(1 if shared_b else batch)]
    got = zgemm_tc(1, 3, Ys, Bs, M, N, shared_b=shared_b)
    for b in range(batch):
        ref = Ys[b].T @ Bs[0 if shared_b else b].conj()
        assert np.max(np.abs(got[b] - ref)) <= SPLIT_TOL * np.sqrt(K) * 4, b
