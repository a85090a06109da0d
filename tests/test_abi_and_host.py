"""CPU checks of the boundary: the C-ABI library loads and exports every symbol its header
declares, and the host-side logic (sites, gates, validation) behaves like the reference."""
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    import __graft_entry__ as g

    g.build()
    from qrochet import _lib

    return _lib.lib()


def _declared():
    inc = os.path.join(ROOT, "include")
    text = "".join(open(os.path.join(inc, f)).read() for f in sorted(os.listdir(inc)) if f.endswith(".h"))
    return sorted(set(re.findall(r"\b(qr_[a-z0-9_]+)\s*\(", text)))


def test_header_symbols_exported(lib):
    names = _declared()
    assert len(names) >= 30
    for name in names:
        assert hasattr(lib, name), name


def test_python_binding_covers_header():
    from qrochet import _lib

    names = set(_declared())
    bound = set(_lib.SIGNATURES) | {"qr_last_error_string"}
    assert names <= bound, names - bound


def test_no_device_is_reported_not_faked(lib):
    import qrochet as Q

    if Q.device_count() > 0:
        pytest.skip("a GPU is present")
    with pytest.raises(Q.GPUError):
        Q.MPS([np.ones((2, 1)), np.ones((2, 1))])


def test_site_parsing_and_adjoint():
    from qrochet import Site, site

    assert site("3") == Site(3)
    assert site("3'") == Site(3, True)
    assert Site(2).adjoint() == Site(2, True)
    assert Site(1) < Site(2)
    with pytest.raises(ValueError):
        site("x1")


def test_dense_matrix_and_validation():
    import qrochet as Q
    from qrochet import random as R

    u = R.haar_unitary(R.rng(1), 4)
    g = Q.gate_from_matrix(u, [2, 3])
    assert np.allclose(g.matrix([2, 3]), u)
    t = u.reshape(2, 2, 2, 2).transpose(1, 0, 3, 2)
    g2 = Q.Dense(Q.Operator(), t, [Q.Site(3), Q.Site(2), Q.Site(3, True), Q.Site(2, True)])
    assert np.allclose(g2.matrix([2, 3]), u)
    assert Q.validate_gate(5, g) == [2, 3]
    with pytest.raises(Q.ArgumentError):
        Q.validate_gate(5, Q.gate_from_matrix(np.eye(4), [2, 4]))
    with pytest.raises(Q.ArgumentError):
        Q.validate_gate(3, Q.gate_from_matrix(np.eye(2), [4]))
    with pytest.raises(Q.ArgumentError):
        Q.validate_gate(5, Q.Dense(Q.Operator(), np.ones((2, 2)), [Q.Site(1), Q.Site(2)]))
    with pytest.raises(AssertionError):
        Q.Dense(Q.Operator(), np.ones((2, 1)), [Q.Site(1), Q.Site(1, True)])


def test_index_counter_and_random_generators():
    from qrochet import nextindex
    from qrochet import random as R

    a, b = nextindex(), nextindex()
    assert a != b
    u = R.haar_unitary(R.rng(3), 4)
    assert np.allclose(u.conj().T @ u, np.eye(4))
    arrs = R.gaussian_mps_arrays(5, 3, seed=4)
    assert arrs[0].shape == (2, 3) and arrs[2].shape == (2, 3, 3) and arrs[4].shape == (2, 3)
    assert all(a.flags.f_contiguous for a in arrs)


@pytest.mark.parametrize("kind,code,text", [(0, "QR_ENOMEM", "host memory allocation failed"),
                                            (1, "QR_EHOST", "planted by qr_test_host_exception"),
                                            (2, "QR_EHOST", "host-side failure")])
def test_abi_guard_turns_host_exceptions_into_status(lib, kind, code, text):
    """A C++ exception inside an exported function comes back as a status and a message (no
    unwinding into the caller); the hook throws on the host, no GPU involved."""
    from qrochet import _lib

    assert lib.qr_test_host_exception(kind) == getattr(_lib, code)
    assert text in _lib.last_error()
    assert lib.qr_test_host_exception(3) == _lib.QR_OK


def test_socket_and_lane_queries():
    """socket / inputs / outputs / ninputs / noutputs / isdual (src/Quantum.jl:25,118-143,228-239)
    on the host bookkeeping of a chain (no device buffers needed), its adjoint, an MPO's site
    list and a gate."""
    import qrochet as Q
    from qrochet.chain import MPO

    psi = Q.Chain(None, 5, 2)  # bookkeeping only: no handle
    assert Q.socket(psi) == Q.State() and Q.socket(psi) != Q.State(dual=True)
    assert Q.outputs(psi) == [Q.Site(i) for i in range(1, 6)] and Q.inputs(psi) == []
    assert (Q.noutputs(psi), Q.ninputs(psi), Q.nsites(psi)) == (5, 0, 5)
    adj = psi.adjoint()
    assert Q.socket(adj) == Q.State(dual=True) == adj.socket
    assert Q.inputs(adj) == [Q.Site(i, True) for i in range(1, 6)] and Q.noutputs(adj) == 0
    assert all(Q.isdual(s) for s in adj.sites()) and not Q.isdual(Q.Site(2))
    w = MPO.__new__(MPO)
    w.n, w.d = 4, 2
    assert Q.socket(w) == Q.Operator()
    assert (Q.ninputs(w), Q.noutputs(w)) == (4, 4)
    assert Q.inputs(w) == [Q.Site(i, True) for i in range(1, 5)]
    g = Q.gate_from_matrix(np.eye(4), [3, 2])
    assert Q.socket(g) == Q.Operator()
    assert Q.outputs(g) == [Q.Site(2), Q.Site(3)] and Q.inputs(g) == [Q.Site(2, True), Q.Site(3, True)]

    class Empty:
        sites = ()

    assert Q.socket(Empty()) == Q.Scalar()
    assert len({Q.State(), Q.State(), Q.State(dual=True), Q.Operator(), Q.Scalar()}) == 4


def test_product_arrays_and_lanes():
    """zeros / ones(Product, n) as MPS(arrays) takes them (Product.jl:44-54, Chain.jl:174-183),
    and lanes / nlanes (src/Quantum.jl:171-184)."""
    import qrochet as Q
    from qrochet import random as R
    from qrochet.chain import MPO

    for make, level in ((R.zero_product_arrays, 0), (R.one_product_arrays, 1)):
        arrs = make(5, 3)
        assert [a.shape for a in arrs] == [(3, 1), (3, 1, 1), (3, 1, 1), (3, 1, 1), (3, 1)]
        for a in arrs:
            v = a.reshape(3)
            assert v[level] == 1 and np.count_nonzero(v) == 1
    with pytest.raises(ValueError):
        R.basis_product_arrays(4, 2, 2)
    g = Q.gate_from_matrix(np.eye(4), [3, 2])
    assert Q.lanes(g) == [Q.Site(2), Q.Site(3)] and Q.nlanes(g) == 2 == g.nlanes()
    psi = Q.Chain(None, 4, 2)
    assert Q.lanes(psi) == [Q.Site(i) for i in range(1, 5)]
    assert Q.lanes(psi.adjoint()) == Q.lanes(psi)
    w = MPO.__new__(MPO)
    w.n, w.d = 3, 2
    assert Q.nlanes(w) == 3


def test_product_state_arrays():
    """Product(vectors) (Product.jl:17-31) and its conversion to a chain's arrays with bonds of
    size 1 (Chain.jl:174-183); bad inputs are rejected on the host."""
    import qrochet as Q
    from qrochet import random as R

    vs = [np.array([1, 0]), np.array([0.6, 0.8j]), np.array([0, 1]), np.array([0.5, 0.5])]
    p = Q.Product(vs)
    assert Q.socket(p) == Q.State() and Q.nsites(p) == 4
    arrs = R.product_arrays(vs)
    assert [a.shape for a in arrs] == [(2, 1), (2, 1, 1), (2, 1, 1), (2, 1)]
    for v, a in zip(vs, arrs):
        assert np.array_equal(a.reshape(-1), v.astype(complex))
    assert all(np.array_equal(a, b) for a, b in zip(R.product_arrays([np.eye(3)[0]] * 3), R.zero_product_arrays(3, 3)))
    with pytest.raises(ValueError):
        Q.Product([np.array([1, 0])])
    with pytest.raises(ValueError):
        Q.Product([np.array([1, 0]), np.array([1, 0, 0])])
