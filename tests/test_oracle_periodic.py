"""Periodic-boundary chains in the oracle, pinned by the reference's Periodic testset
(test/Ansatz/Chain_test.jl:2-78, site sizes and the closing bond) and by brute-force ring traces."""
import numpy as np
import pytest

from oracle import chain_oracle as O
from qrochet import checkpoint
from qrochet import random as R


def _rand(g, shape):
    return g.standard_normal(shape) + 1j * g.standard_normal(shape)


def test_periodic_sizes_and_closing_bond():
    g = R.rng(1)
    arrays = [_rand(g, (2, 1, 4)), _rand(g, (2, 4, 3)), _rand(g, (2, 3, 1))]  # (:o, :l, :r)
    ch = O.from_reference_arrays_periodic(arrays)
    assert [a.shape for a in ch.sites] == [(1, 2, 4), (4, 2, 3), (3, 2, 1)]
    assert ch.bond_dims() == [4, 3, 1]  # bond 3 closes site 3 onto site 1
    perm = [np.transpose(a, (2, 0, 1)) for a in arrays]  # (:r, :o, :l)
    ch2 = O.from_reference_arrays_periodic(perm, order=("r", "o", "l"))
    assert all(np.array_equal(a, b) for a, b in zip(ch.sites, ch2.sites))


def test_periodic_statevector_is_the_ring_trace():
    g = R.rng(2)
    arrays = [_rand(g, (2, 3, 2)), _rand(g, (2, 2, 4)), _rand(g, (2, 4, 3))]
    ch = O.from_reference_arrays_periodic(arrays)
    sv = O.to_statevector(ch)
    ref = np.empty(8, dtype=complex)
    for x in range(8):
        o = [(x >> 2) & 1, (x >> 1) & 1, x & 1]
        m = arrays[0][o[0]] @ arrays[1][o[1]] @ arrays[2][o[2]]
        ref[x] = np.trace(m)
    assert np.allclose(sv, ref)
    assert np.isclose(O.overlap(ch, ch), np.vdot(ref, ref))


def test_periodic_gate_on_inner_bond_matches_dense():
    g = R.rng(3)
    n = 4
    arrays = [_rand(g, (2, 2, 2)) for _ in range(n)]
    ch = O.from_reference_arrays_periodic(arrays)
    u = R.haar_unitary(g, 4)
    sv = O.to_statevector(ch).reshape(2, 2, 2, 2)
    ref = np.einsum("ab,xbz->xaz", u, sv.reshape(2, 4, 2)).reshape(16)
    O.evolve_2site_(ch, 1, u)
    assert np.allclose(O.to_statevector(ch), ref)
    assert ch.lam[1] is not None  # the SVD leaves Lambda on the bond, as svd! does


def test_canonical_forms_are_open_only():
    g = R.rng(4)
    ch = O.from_reference_arrays_periodic([_rand(g, (2, 2, 2)) for _ in range(3)])
    with pytest.raises(O.ArgumentError):
        O.canonize_(ch)
    with pytest.raises(O.ArgumentError):
        O.canonize_site_(ch, 0, "right")


def test_periodic_checkpoint_layout(tmp_path):
    g = R.rng(5)
    arrays = [_rand(g, (2, 3, 2)), _rand(g, (2, 2, 3))]
    path = tmp_path / "p.qrchain"
    checkpoint.write(path, arrays, periodic=True)
    back, lams, prec, per = checkpoint.read(path, with_boundary=True)
    assert per and prec == 0 and lams == [None]
    assert all(np.array_equal(a, b) for a, b in zip(arrays, back))
