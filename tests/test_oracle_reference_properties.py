"""Pins the CPU oracle to every property that Qrochet.jl's own tests assert for the Chain path
(``test/Ansatz/Chain_test.jl``).  The reference tests run on unseeded ``rand`` data; here the
same checks run on seeded data of the same shapes."""
import numpy as np
import pytest

from oracle import chain_oracle as O
from qrochet import random as R


def _real_arrays(g, shapes):
    return [g.random(s) for s in shapes]


def _chain(g, shapes):
    return O.from_reference_arrays(_real_arrays(g, shapes))


def _sv(ch):
    return O.to_statevector(ch)


def test_truncate_properties():
    # Chain_test.jl:189-204
    g = R.rng(11)
    qtn = _chain(g, [(2, 2), (2, 2, 2), (2, 2)])
    O.canonize_site_(qtn, 1, "right", "svd")
    with pytest.raises(O.MissingSchmidtCoefficientsException):
        O.truncate_(qtn.copy(), (0, 1), maxdim=1)
    t = O.truncate_(qtn.copy(), (1, 2), maxdim=1)
    assert t.sites[1].shape[2] == 1 and t.sites[2].shape[0] == 1
    lam = qtn.lam[1]
    t = O.truncate_(qtn.copy(), (1, 2), threshold=lam[1] + 0.1)
    assert t.sites[1].shape[2] == 1 and t.sites[2].shape[0] == 1


def test_rand_state_properties():
    # Chain_test.jl:209-221
    n, chi = 8, 10
    arrays = R.rand_chain_state_arrays(R.rng(3), n, chi, p=2)
    qtn = O.from_reference_arrays(arrays)
    assert np.isclose(O.norm(qtn), 1.0)
    assert max(qtn.bond_dims()) <= chi


def test_canonize_contract_between():
    # Chain_test.jl:241-266
    qtn = O.from_reference_arrays(R.rand_chain_state_arrays(R.rng(5), 5, 20, p=2))
    can = O.canonize_(qtn.copy())
    with pytest.raises(O.ArgumentError):
        O.contract_between_(can.copy(), 0, 1, direction="dummy")
    for i in range(4):
        some = O.contract_between_(can.copy(), i, i + 1)
        assert np.allclose(_sv(some), _sv(qtn))
        assert some.lam[i] is None
        assert O.isrightcanonical(some, i)
        other = O.contract_between_(can.copy(), i, i + 1, direction="right")
        assert O.isleftcanonical(other, i + 1)
        b = some.sites[i]
        assert np.allclose(b, can.sites[i] * can.lam[i][None, None, :])


def test_contract_between_site_pairs():
    """tensors(tn; between) (Ansatz.jl:78-89) behind contract! (Chain.jl:309-333): the same site
    twice is an assertion, sites without a shared bond leave the chain as it is, and an adjacent
    pair in reverse order absorbs the same bond's Lambda into the named site."""
    can = O.canonize_(O.from_reference_arrays(R.rand_chain_state_arrays(R.rng(5), 5, 20, p=2)))
    with pytest.raises(AssertionError):
        O.contract_between_(can.copy(), 2, 2)
    with pytest.raises(AssertionError):
        O.contract_between_(can.copy(), 0, 7)
    far = O.contract_between_(can.copy(), 0, 2)
    assert all(np.array_equal(x, y) for x, y in zip(far.sites, can.sites))
    assert all(l is not None for l in far.lam)
    for i in range(4):
        fwd = O.contract_between_(can.copy(), i, i + 1, direction="right")
        rev = O.contract_between_(can.copy(), i + 1, i, direction="left")
        assert rev.lam[i] is None
        assert all(np.array_equal(x, y) for x, y in zip(fwd.sites, rev.sites))
        fwd = O.contract_between_(can.copy(), i, i + 1, direction="left")
        rev = O.contract_between_(can.copy(), i + 1, i, direction="right")
        assert all(np.array_equal(x, y) for x, y in zip(fwd.sites, rev.sites))


@pytest.mark.parametrize("method", ["qr", "svd"])
def test_canonize_site(method):
    # Chain_test.jl:268-306
    g = R.rng(7)
    qtn = _chain(g, [(4, 4), (4, 4, 4), (4, 4)])
    with pytest.raises(O.ArgumentError):
        O.canonize_site_(qtn.copy(), 0, "left")
    with pytest.raises(O.ArgumentError):
        O.canonize_site_(qtn.copy(), 2, "right")
    for site, direction, pred in [(0, "right", O.isleftcanonical), (1, "right", O.isleftcanonical),
                                  (1, "left", O.isrightcanonical), (2, "left", O.isrightcanonical)]:
        c = O.canonize_site_(qtn.copy(), site, direction, method)
        assert pred(c, site)
        assert np.allclose(_sv(c), _sv(qtn))
    assert O.canonize_site_(qtn.copy(), 1, "left", "svd").ntensors() == 4


def test_canonize():
    # Chain_test.jl:308-356
    g = R.rng(9)
    qtn = _chain(g, [(4, 4), (4, 4, 4), (4, 4, 4), (4, 4, 4), (4, 4)])
    can = O.canonize_(qtn.copy())
    assert can.ntensors() == 9
    assert np.allclose(_sv(can), _sv(qtn))
    assert np.isclose(O.norm(qtn), O.norm(can))
    sums = [np.sum(lm ** 2) for lm in can.lam]
    assert np.allclose(sums, np.ones(4) * O.norm(can) ** 2)
    for i in range(5):
        c = O.canonize_(qtn.copy())
        if i == 0:
            assert O.isleftcanonical(c, i)
        elif i == 4:
            O.contract_between_(c, i - 1, i, direction="right")
            c.sites[i] = c.sites[i] / O.norm(c)
            assert O.isleftcanonical(c, i)
        else:
            O.contract_between_(c, i - 1, i, direction="right")
            assert O.isleftcanonical(c, i)
    for i in range(5):
        c = O.canonize_(qtn.copy())
        if i == 0:
            O.contract_between_(c, i, i + 1, direction="left")
            c.sites[i] = c.sites[i] / O.norm(c)
            assert O.isrightcanonical(c, i)
        elif i == 4:
            assert O.isrightcanonical(c, i)
        else:
            O.contract_between_(c, i, i + 1, direction="left")
            assert O.isrightcanonical(c, i)


def test_mixed_canonize():
    # Chain_test.jl:358-374
    g = R.rng(13)
    qtn = _chain(g, [(4, 4), (4, 4, 4), (4, 4, 4), (4, 4, 4), (4, 4)])
    can = O.mixed_canonize_(qtn.copy(), 2)
    assert can.ntensors() == qtn.ntensors() + 1
    assert O.isleftcanonical(can, 0) and O.isleftcanonical(can, 1)
    assert O.isrightcanonical(can, 2) and O.isrightcanonical(can, 3) and O.isrightcanonical(can, 4)
    assert np.allclose(_sv(can), _sv(qtn))
    with pytest.raises(O.ArgumentError):
        O.mixed_canonize_(qtn.copy(), 0)


def test_normalize():
    # Chain_test.jl:377-381
    g = R.rng(17)
    qtn = _chain(g, [(4, 4), (4, 4, 4), (4, 4, 4), (4, 4, 4), (4, 4)])
    O.normalize_(qtn, 2)
    assert np.isclose(O.norm(qtn), 1.0)


@pytest.mark.parametrize("p", [1, np.inf, 3])
def test_normalize_p_norm(p):
    """normalize!(tn, root; p) divides the centre Lambda by its p-norm (Chain.jl:532-536)."""
    g = R.rng(17)
    qtn = _chain(g, [(4, 4), (4, 4, 4), (4, 4, 4), (4, 4, 4), (4, 4)])
    two = O.normalize_(qtn.copy(), 2)
    other = O.normalize_(qtn.copy(), 2, p=p)
    lam2, lamp = two.lam[1], other.lam[1]
    assert np.isclose(np.linalg.norm(lamp, p), 1.0)
    assert np.allclose(lamp / lamp[0], lam2 / lam2[0])


def test_order_permutation():
    # Chain_test.jl:92-116: custom order (:r, :o, :l) gives the same network
    g = R.rng(19)
    arrays = [g.random((2, 1)), g.random((2, 1, 3)), g.random((2, 3))]
    a = O.from_reference_arrays(arrays)
    perm = [np.transpose(arrays[0], (1, 0)), np.transpose(arrays[1], (2, 0, 1)), arrays[2]]
    b = O.from_reference_arrays(perm, order=("r", "o", "l"))
    assert np.allclose(_sv(a), _sv(b))
    assert a.bond_dims() == [1, 3]


def test_truncate_to_an_empty_extent_leaves_a_size_0_bond():
    """truncate! slices with whatever extent survives the filter (Chain.jl:404-419); an empty one
    leaves a bond of size 0 and a null state."""
    arrays = R.gaussian_mps_arrays(4, 3, seed=5, uniform=False)
    ch = O.from_reference_arrays(arrays)
    O.canonize_site_(ch, 1, "right", "svd")
    O.truncate_(ch, (1, 2), threshold=10 * ch.lam[1][0])
    assert ch.bond_dims()[1] == 0 and ch.lam[1].size == 0
    assert ch.sites[1].shape[2] == 0 and ch.sites[2].shape[0] == 0
    assert O.norm(ch) == 0.0
