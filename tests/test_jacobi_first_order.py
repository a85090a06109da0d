"""CPU checks (NumPy) of the mathematics the mixed SVD's last polish step relies on: when every
remaining Jacobi pair of the one-sided (Hestenes) iteration has a first-order tangent t <= 1e-8,
the rotations are applied at once as B <- B (I + E), V <- V (I + E) with the anti-Hermitian

    E_pq = g_pq / (|b_q|^2 - |b_p|^2),    g_pq = b_p^H b_q,

which zeroes the couplings to first order (the terms left are products of two tangents), keeps
I + E unitary to |E|^2, and agrees with rotating the pairs one after another to the same order.
The device kernels that do this are tested against LAPACK on the GPU; this pins the algebra."""
import numpy as np


def _near_diagonal_columns(g, m, n, tan):
    """B = U diag(s) W with W a product of rotations by tangents ~tan: couplings ~tan * gaps."""
    u, _ = np.linalg.qr(g.standard_normal((m, n)) + 1j * g.standard_normal((m, n)))
    s = np.sort(g.uniform(0.5, 2.0, n))[::-1]
    x = tan * (g.standard_normal((n, n)) + 1j * g.standard_normal((n, n)))
    a = (x - x.conj().T) / 2  # anti-Hermitian: exp(a) is unitary
    w = np.eye(n) + a + a @ a / 2 + a @ a @ a / 6
    return (u * s) @ w


def _first_order_e(b):
    gram = b.conj().T @ b
    d = np.real(np.diag(gram))
    n = b.shape[1]
    e = np.zeros((n, n), dtype=complex)
    for p in range(n):
        for q in range(n):
            if p != q:
                e[p, q] = gram[p, q] / (d[q] - d[p])
    return e, gram


def _offdiag_rel(b):
    gram = b.conj().T @ b
    d = np.sqrt(np.real(np.diag(gram)))
    off = np.abs(gram - np.diag(np.diag(gram))) / np.outer(d, d)
    return float(off.max())


def test_first_order_step_leaves_second_order_couplings():
    g = np.random.default_rng(3)
    for tan in (1e-5, 1e-6, 1e-8):
        b = _near_diagonal_columns(g, 96, 40, tan)
        e, _ = _first_order_e(b)
        assert np.allclose(e, -e.conj().T, atol=1e-15 + 1e-9 * np.abs(e).max())  # anti-Hermitian
        before, after = _offdiag_rel(b), _offdiag_rel(b @ (np.eye(40) + e))
        t = float(np.abs(e).max())
        assert before > 0.1 * tan
        # what is left is second order in the tangents (plus rounding)
        assert after <= 50 * t * t + 1e-14, (tan, before, after, t)


def test_identity_plus_e_is_unitary_to_second_order():
    g = np.random.default_rng(5)
    b = _near_diagonal_columns(g, 64, 24, 1e-6)
    e, _ = _first_order_e(b)
    m = np.eye(24) + e
    t = float(np.abs(e).max())
    # (I + E)^H (I + E) = I - E^2 for anti-Hermitian E
    assert np.abs(m.conj().T @ m - np.eye(24)).max() <= 24 * t * t + 1e-15


def test_simultaneous_matches_sequential_rotations_to_second_order():
    """Rotating the pairs one after another (exact 2 x 2 Jacobi rotations in round-robin order)
    and applying I + E at once end within products of two tangents of each other."""
    g = np.random.default_rng(7)
    n = 16
    b = _near_diagonal_columns(g, 48, n, 1e-7)
    e, _ = _first_order_e(b)
    simultaneous = b @ (np.eye(n) + e)
    seq = b.copy()
    for p in range(n):
        for q in range(p + 1, n):
            bp, bq = seq[:, p], seq[:, q]
            a, c, gpq = np.vdot(bp, bp).real, np.vdot(bq, bq).real, np.vdot(bp, bq)
            # the Hermitian 2 x 2 eigenproblem of [[a, g], [conj(g), c]]: tangent of the rotation
            zeta = (c - a) / (2 * abs(gpq))
            t = np.sign(zeta) / (abs(zeta) + np.sqrt(1 + zeta * zeta))
            cs = 1 / np.sqrt(1 + t * t)
            sn = t * cs * gpq / abs(gpq)
            seq[:, p], seq[:, q] = cs * bp - np.conj(sn) * bq, sn * bp + cs * bq
    tmax = float(np.abs(e).max())
    # the same subspace rotation up to O(t^2) in every column (columns keep their order: no sort)
    diff = np.abs(seq - simultaneous).max() / np.abs(b).max()
    assert diff <= 20 * n * tmax * tmax + 1e-14, (diff, tmax)
    assert _offdiag_rel(seq) <= 1e-10 and _offdiag_rel(simultaneous) <= 1e-10
