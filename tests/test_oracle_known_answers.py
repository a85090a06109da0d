"""Pins the oracle's untested-by-the-reference paths (``evolve!``, ``expect``, ``overlap``,
MPO expectation; ``Chain_test.jl:396`` leaves ``evolve!`` untested) against exact dense
state-vector arithmetic and closed-form answers."""
import numpy as np
import pytest

from oracle import chain_oracle as O
from qrochet import random as R


def _dense_apply(v, n, site, m, k=1):
    """Apply a d^k x d^k matrix on sites site..site+k-1 (0-based) of a dense state."""
    d = 2
    t = v.reshape((d,) * n)
    t = np.moveaxis(t, list(range(site, site + k)), list(range(k)))
    sh = t.shape
    t = (m @ t.reshape(d ** k, -1)).reshape(sh)
    t = np.moveaxis(t, list(range(k)), list(range(site, site + k)))
    return t.reshape(-1)


def _gate(m, lanes):
    d = 2
    k = len(lanes)
    arr = np.asarray(m).reshape((d,) * (2 * k))
    sites = tuple(O.OSite(l) for l in lanes) + tuple(O.OSite(l, True) for l in lanes)
    return O.ODense(arr, sites)


def test_evolve_matches_dense_without_truncation():
    n = 6
    psi = O.from_reference_arrays(R.gaussian_mps_arrays(n, 4, seed=1, uniform=False))
    v = O.to_statevector(psi)
    g = R.rng(2)
    for layer in R.brickwall_layers(n, 4, seed=3):
        for s, u in layer:
            O.evolve_(psi, _gate(u, [s, s + 1]))
            v = _dense_apply(v, n, s - 1, u, 2)
    x = R.haar_unitary(g, 2)
    O.evolve_(psi, _gate(x, [3]))
    v = _dense_apply(v, n, 2, x, 1)
    assert np.allclose(O.to_statevector(psi), v, atol=1e-12)


def test_gate_site_order_is_respected():
    # Dense(Operator(), array; sites) maps array dims to sites in the order given
    n = 4
    psi = O.from_reference_arrays(R.gaussian_mps_arrays(n, 2, seed=5))
    u = R.haar_unitary(R.rng(6), 4)
    a = O.evolve_(psi.copy(), _gate(u, [2, 3]))
    # the same operator written with sites [3, 2, 3', 2']: swap both output and input dims
    t = u.reshape(2, 2, 2, 2).transpose(1, 0, 3, 2)
    b = O.evolve_(psi.copy(), O.ODense(t, (O.OSite(3), O.OSite(2), O.OSite(3, True),
                                           O.OSite(2, True))))
    assert np.allclose(O.to_statevector(a), O.to_statevector(b))


def test_evolve_errors():
    psi = O.from_reference_arrays(R.gaussian_mps_arrays(4, 2, seed=7))
    u = np.eye(4)
    with pytest.raises(O.ArgumentError):  # non-contiguous lanes
        O.evolve_(psi.copy(), _gate(np.eye(4), [1, 3]))
    with pytest.raises(O.ArgumentError):  # not an operator (no inputs)
        O.evolve_(psi.copy(), O.ODense(np.ones((2, 2)), (O.OSite(1), O.OSite(2))))
    with pytest.raises(O.ArgumentError):  # inputs != outputs
        O.evolve_(psi.copy(), O.ODense(u.reshape(2, 2, 2, 2),
                                       (O.OSite(1), O.OSite(2), O.OSite(2, True),
                                        O.OSite(3, True))))
    with pytest.raises(O.ArgumentError):  # outside the chain
        O.evolve_(psi.copy(), _gate(np.eye(2), [9]))
    with pytest.raises(O.ArgumentError):  # three lanes
        O.evolve_(psi.copy(), _gate(np.eye(8), [1, 2, 3]))


def test_expect_overlap_norm_dense():
    n = 7
    psi = O.from_reference_arrays(R.gaussian_mps_arrays(n, 8, seed=8))
    phi = O.from_reference_arrays(R.gaussian_mps_arrays(n, 8, seed=9))
    vp, vf = O.to_statevector(psi), O.to_statevector(phi)
    assert np.isclose(O.overlap(psi, phi), np.vdot(vf, vp))
    assert np.isclose(O.norm(psi), np.linalg.norm(vp))
    zz = np.kron(R.PAULI["Z"], R.PAULI["Z"])
    for i in range(1, n):
        e = O.expect(psi, [_gate(zz, [i, i + 1])])
        assert np.isclose(e, np.vdot(vp, _dense_apply(vp, n, i - 1, zz, 2)))
    # product of observables: expect applies them in sequence
    obs = [_gate(R.PAULI["X"], [2]), _gate(R.PAULI["Y"], [5]), _gate(zz, [3, 4])]
    w = vp
    w = _dense_apply(w, n, 1, R.PAULI["X"], 1)
    w = _dense_apply(w, n, 4, R.PAULI["Y"], 1)
    w = _dense_apply(w, n, 2, zz, 2)
    assert np.isclose(O.expect(psi, obs), np.vdot(vp, w))


def test_xxz_mpo_matches_pauli_sum():
    n = 5
    jz, jxy = 1.0, 0.7
    w = [np.asarray(a) for a in R.xxz_mpo_arrays(n, jz, jxy)]
    # to (wl, o, i, wr)
    ws = []
    for i, a in enumerate(w):
        if i == 0:
            a = a[:, :, None, :]
        elif i == n - 1:
            a = a[:, :, :, None]
        ws.append(np.transpose(a, (2, 0, 1, 3)))
    h = O.mpo_to_dense(ws)
    ref = np.zeros((2 ** n, 2 ** n), dtype=complex)
    P = R.PAULI
    for i in range(n - 1):
        for p, c in (("X", jxy), ("Y", jxy), ("Z", jz)):
            ops = [P["I"]] * n
            ops[i] = ops[i + 1] = P[p]
            t = ops[0]
            for o in ops[1:]:
                t = np.kron(t, o)
            ref += c * t
    assert np.allclose(h, ref)
    psi = O.from_reference_arrays(R.gaussian_mps_arrays(n, 4, seed=10))
    v = O.to_statevector(psi)
    assert np.isclose(O.mpo_expect(psi, ws), np.vdot(v, ref @ v))


def test_ghz_schmidt_values():
    # H on site 1 then CNOT chain from |0..0>: every bond has Schmidt values (1/sqrt2, 1/sqrt2)
    n = 6
    psi = O.from_reference_arrays(R.zero_product_arrays(n))
    h = np.array([[1, 1], [1, -1]]) / np.sqrt(2)
    cnot = np.array([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 0, 1], [0, 0, 1, 0]], dtype=complex)
    O.evolve_(psi, _gate(h, [1]))
    for i in range(1, n):
        O.evolve_(psi, _gate(cnot, [i, i + 1]), threshold=1e-10)
    assert psi.bond_dims() == [2] * (n - 1)
    # the default (non-Vidal) path does not absorb the neighbouring Lambda before the SVD, so
    # only the first bond carries the GHZ Schmidt values; the later bonds see isometries
    assert np.allclose(psi.lam[0], [1 / np.sqrt(2)] * 2)
    for i in range(1, n - 1):
        assert np.allclose(psi.lam[i], [1.0, 1.0])
    v = O.to_statevector(psi)
    ref = np.zeros(2 ** n)
    ref[0] = ref[-1] = 1 / np.sqrt(2)
    assert np.allclose(v, ref)


def test_tebd_truncation_keeps_exact_rank():
    n = 8
    psi = O.from_reference_arrays(R.zero_product_arrays(n))
    v = O.to_statevector(psi)
    for layer in R.brickwall_layers(n, 3, seed=21):
        for s, u in layer:
            O.evolve_(psi, _gate(u, [s, s + 1]), threshold=1e-10, maxdim=64)
            v = _dense_apply(v, n, s - 1, u, 2)
    assert np.allclose(O.to_statevector(psi), v, atol=1e-10)
    assert max(psi.bond_dims()) <= 8


def test_renormalize_paths():
    n = 6
    psi = O.from_reference_arrays(R.gaussian_mps_arrays(n, 4, seed=22, uniform=False))
    u = R.haar_unitary(R.rng(23), 4)
    a = O.evolve_(psi.copy(), _gate(u, [3, 4]), maxdim=2, renormalize=True)
    assert np.isclose(O.norm(a), 1.0)
    with pytest.raises(O.ArgumentError):  # normalize! at site 1 -> mixed_canonize! errors
        O.evolve_(psi.copy(), _gate(u, [1, 2]), maxdim=2, renormalize=True)
    # Vidal path: canonical form, renormalised Lambda
    c = O.canonize_(psi.copy())
    c2 = O.evolve_(c.copy(), _gate(u, [3, 4]), iscanonical=True)
    assert np.allclose(O.to_statevector(c2), _dense_apply(O.to_statevector(c), n, 2, u, 2))
    c3 = O.evolve_(c.copy(), _gate(u, [3, 4]), maxdim=2, iscanonical=True, renormalize=True)
    assert np.isclose(np.linalg.norm(c3.lam[2]), 1.0)
