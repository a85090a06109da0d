"""GPU parity of every Chain operation against the CPU oracle, through the C ABI.

Tolerances: FP64 path -- gauge-invariant quantities (state vectors, norms, Lambda spectra,
expectation values) within 1e-10 relative; bond dimensions and Lambda placement bit-exact.
"""
import numpy as np
import pytest

import qrochet as Q
from oracle import chain_oracle as O
from qrochet import random as R

pytestmark = pytest.mark.gpu

RTOL = 1e-10


def _close(a, b, rtol=RTOL):
    a, b = np.asarray(a), np.asarray(b)
    scale = max(1e-300, float(np.max(np.abs(b))) if b.size else 1.0)
    return float(np.max(np.abs(a - b))) <= rtol * scale if a.size else True


def _sv(psi: Q.Chain):
    """State vector of a GPU chain (download + oracle contraction)."""
    ch = (O.from_reference_arrays_periodic if psi.periodic else O.from_reference_arrays)(psi.arrays())
    for b, f in enumerate(psi.lambda_flags()):
        if f:
            ch.lam[b] = psi.lambda_between(b + 1, b + 2)
    return O.to_statevector(ch)


def _pair(n, chi, seed, uniform=True, real=False):
    if real:
        g = R.rng(seed)
        shapes = [(2, chi)] + [(2, chi, chi)] * (n - 2) + [(2, chi)]
        arrays = [np.asfortranarray(g.random(s)) for s in shapes]
    else:
        arrays = R.gaussian_mps_arrays(n, chi, seed=seed, uniform=uniform)
    return Q.MPS(arrays), O.from_reference_arrays(arrays)


def _check_same(psi, ref, rtol=RTOL, statevector=True):
    assert psi.bond_dims() == ref.bond_dims()
    assert psi.lambda_flags() == ref.lambda_flags()
    assert psi.ntensors() == ref.ntensors()
    for b, lm in enumerate(ref.lam):
        if lm is not None:
            assert _close(psi.lambda_between(b + 1, b + 2), lm, rtol), b
    if statevector:
        assert _close(_sv(psi), O.to_statevector(ref), rtol)


@pytest.mark.parametrize("order", [("o", "l", "r"), ("r", "o", "l"), ("l", "r", "o")])
def test_upload_download_roundtrip(order):
    arrays = R.gaussian_mps_arrays(5, 3, seed=3, uniform=False)
    psi = Q.MPS(arrays)
    perm = []
    for i, a in enumerate(arrays):
        src = [x for x in ("o", "l", "r") if not ((i == 0 and x == "l") or (i == 4 and x == "r"))]
        dst = [x for x in order if not ((i == 0 and x == "l") or (i == 4 and x == "r"))]
        perm.append(np.transpose(a, [src.index(x) for x in dst]))
    psi2 = Q.MPS(perm, order=order)
    for i in range(5):
        assert np.array_equal(psi.site_array(i + 1), arrays[i])
        assert np.array_equal(psi2.site_array(i + 1), arrays[i])
        assert np.array_equal(psi2.site_array(i + 1, order), perm[i])


@pytest.mark.parametrize("order", [("o", "l", "r"), ("r", "o", "l"), ("l", "r", "o"), ("r", "l", "o")])
def test_upload_download_large_sites(order):
    """Site layouts large enough for the shared-memory tiled permute to take several tiles per
    dimension with ragged edges (bonds 600 and 45); bit-exact both ways."""
    g = R.rng(11)
    shapes = [(2, 600), (2, 600, 45), (2, 45)]
    arrays = [R.complex_gaussian(g, sh) for sh in shapes]
    perm = []
    for i, a in enumerate(arrays):
        src = [x for x in ("o", "l", "r") if not ((i == 0 and x == "l") or (i == 2 and x == "r"))]
        dst = [x for x in order if not ((i == 0 and x == "l") or (i == 2 and x == "r"))]
        perm.append(np.ascontiguousarray(np.transpose(a, [src.index(x) for x in dst])))
    psi = Q.MPS(perm, order=order)
    for i in range(3):
        assert np.array_equal(psi.site_array(i + 1), arrays[i])
        assert np.array_equal(psi.site_array(i + 1, order), perm[i])


@pytest.mark.parametrize("method", ["qr", "svd"])
@pytest.mark.parametrize("site,direction", [(1, "right"), (2, "right"), (2, "left"), (3, "left")])
def test_canonize_site(method, site, direction):
    psi, ref = _pair(3, 4, seed=7, real=True)
    Q.canonize_site_(psi, site, direction, method)
    O.canonize_site_(ref, site - 1, direction, method)
    _check_same(psi, ref)
    pred = Q.isleftcanonical if direction == "right" else Q.isrightcanonical
    assert pred(psi, site)


def test_canonize_site_errors():
    psi, _ = _pair(3, 4, seed=7, real=True)
    with pytest.raises(Q.ArgumentError):
        Q.canonize_site_(psi, 1, "left")
    with pytest.raises(Q.ArgumentError):
        Q.canonize_site_(psi, 3, "right")
    with pytest.raises(Q.ArgumentError):
        Q.canonize_site_(psi, 2, "up")
    assert Q.canonize_site(psi, 2, "left", "svd").ntensors() == 4


def test_canonize_reference_properties():
    # the checks of test/Ansatz/Chain_test.jl:308-356 on the GPU chain
    psi, ref = _pair(5, 4, seed=9, real=True)
    can = Q.canonize(psi)
    O.canonize_(ref)
    assert can.ntensors() == 9
    _check_same(can, ref)
    assert np.isclose(Q.norm(psi), Q.norm(can), rtol=RTOL)
    nrm2 = Q.norm(can) ** 2
    for b in range(4):
        assert np.isclose(np.sum(can.lambda_between(b + 1, b + 2) ** 2), nrm2, rtol=1e-10)
    for i in range(1, 6):
        c = Q.canonize(psi)
        if i == 1:
            assert Q.isleftcanonical(c, i)
        else:
            Q.contract_between_(c, i - 1, i, direction="right")
            if i == 5:  # the end tensor carries the norm: its 1x1 Gram is ||psi||^2
                assert abs(Q.canonicality_error(c, i, "left") - abs(nrm2 - 1)) <= 1e-10 * nrm2
            else:
                assert Q.isleftcanonical(c, i)
    for i in range(1, 6):
        c = Q.canonize(psi)
        if i == 5:
            assert Q.isrightcanonical(c, i)
        else:
            Q.contract_between_(c, i, i + 1, direction="left")
            if i == 1:
                assert abs(Q.canonicality_error(c, i, "right") - abs(nrm2 - 1)) <= 1e-10 * nrm2
            else:
                assert Q.isrightcanonical(c, i)


@pytest.mark.parametrize("n,chi,seed", [(16, 32, 1), (9, 7, 2), (6, 40, 3)])
def test_canonize_gaussian(n, chi, seed):
    psi, ref = _pair(n, chi, seed)
    Q.canonize_(psi)
    O.canonize_(ref)
    _check_same(psi, ref, statevector=n <= 12)


def test_mixed_canonize_and_normalize():
    psi, ref = _pair(5, 4, seed=13, real=True)
    can = Q.mixed_canonize(psi, 3)
    O.mixed_canonize_(ref, 2)
    _check_same(can, ref)
    assert Q.isleftcanonical(can, 1) and Q.isleftcanonical(can, 2)
    for s in (3, 4, 5):
        assert Q.isrightcanonical(can, s)
    with pytest.raises(Q.ArgumentError):
        Q.mixed_canonize(psi, 1)
    for p in (1, np.inf):  # normalize!(tn, root; p): the centre Lambda over its p-norm
        a = Q.normalize_(psi.copy(), 3, p=p)
        r = O.normalize_(ref.copy(), 2, p=p)
        _check_same(a, r)
        assert np.isclose(np.linalg.norm(a.lambda_between(2, 3), p), 1.0, rtol=1e-12)
    Q.normalize_(psi, 3)
    assert np.isclose(Q.norm(psi), 1.0, rtol=1e-12)


def test_truncate():
    psi, ref = _pair(3, 2, seed=11, real=True)
    Q.canonize_site_(psi, 2, "right", "svd")
    O.canonize_site_(ref, 1, "right", "svd")
    with pytest.raises(Q.MissingSchmidtCoefficientsException):
        Q.truncate_(psi.copy(), (1, 2), maxdim=1)
    with pytest.raises(Q.ArgumentError):
        Q.truncate_(psi.copy(), (1, 3), maxdim=1)
    t = Q.truncate(psi, (2, 3), maxdim=1)
    assert t.bond_dims()[1] == 1
    lam = psi.lambda_between(2, 3)
    t = Q.truncate(psi, (2, 3), threshold=lam[1] + 0.1)
    assert t.bond_dims()[1] == 1
    O.truncate_(ref, (1, 2), maxdim=1)
    Q.truncate_(psi, (2, 3), maxdim=1)
    _check_same(psi, ref)


def test_truncate_to_an_empty_bond():
    """A threshold above every singular value slices the bond to size 0 (slice! with an empty
    extent, Chain.jl:404-419), like the oracle: the chain is the null state, its contractions are
    0 and factorisations refuse it."""
    psi, ref = _pair(4, 3, seed=12)
    Q.canonize_site_(psi, 2, "right", "svd")
    O.canonize_site_(ref, 1, "right", "svd")
    lam = psi.lambda_between(2, 3)
    Q.truncate_(psi, (2, 3), threshold=2 * lam[0])
    O.truncate_(ref, (1, 2), threshold=2 * lam[0])
    assert psi.bond_dims() == ref.bond_dims() and psi.bond_dims()[1] == 0
    assert psi.lambda_between(2, 3).size == 0
    assert psi.site_array(2).size == 0 and psi.site_array(3).size == 0
    assert Q.norm(psi) == 0.0 and O.norm(ref) == 0.0
    assert Q.expect(psi, [Q.gate_from_matrix(R.PAULI["Z"], [1])]) == 0
    with pytest.raises(Q.ArgumentError, match="size 0"):
        Q.canonize_(psi)
    with pytest.raises(Q.ArgumentError, match="size 0"):
        Q.evolve_(psi, Q.gate_from_matrix(np.eye(4), [1, 2]), threshold=1e-10, maxdim=4)
    # a maxdim below 1 keeps nothing either: 1:min(dim, maxdim) is empty (Chain.jl:404-406)
    for md in (0, -3):
        psi2, ref2 = _pair(4, 3, seed=12)
        Q.canonize_site_(psi2, 2, "right", "svd")
        O.canonize_site_(ref2, 1, "right", "svd")
        Q.truncate_(psi2, (2, 3), maxdim=md)
        O.truncate_(ref2, (1, 2), maxdim=md)
        assert psi2.bond_dims() == ref2.bond_dims() and psi2.bond_dims()[1] == 0
    # and evolve! truncates its new bond the same way (Chain.jl:645-649 -> truncate!)
    u = R.haar_unitary(R.rng(4), 4)
    psi3, ref3 = _pair(4, 3, seed=12)
    Q.evolve_(psi3, Q.gate_from_matrix(u, [2, 3]), maxdim=-2)
    O.evolve_2site_(ref3, 1, u, maxdim=-2)
    assert psi3.bond_dims() == ref3.bond_dims() and psi3.bond_dims()[1] == 0
    assert Q.norm(psi3) == 0.0


def test_contract_between():
    # Chain_test.jl:241-266 runs on rand(Chain, Open, State; n=5, p=2, chi=20): a normalised state
    arrays = R.rand_chain_state_arrays(R.rng(21), 5, 20, p=2)
    psi, ref = Q.MPS(arrays), O.from_reference_arrays(arrays)
    Q.canonize_(psi)
    O.canonize_(ref)
    for i in range(1, 5):
        a = Q.contract_between(psi, i, i + 1)
        r = O.contract_between_(ref.copy(), i - 1, i)
        _check_same(a, r)
        assert Q.isrightcanonical(a, i)
        b = Q.contract_between(psi, i, i + 1, direction="right")
        assert Q.isleftcanonical(b, i + 1)
    with pytest.raises(Q.ArgumentError):
        Q.contract_between(psi, 1, 2, direction="dummy")
    # tensors(tn; between) (Ansatz.jl:78-89): the same site twice asserts, sites without a shared
    # bond leave the chain as it is, a reversed adjacent pair absorbs that bond's Lambda
    with pytest.raises(AssertionError):
        Q.contract_between(psi, 2, 2)
    far = Q.contract_between(psi, 1, 3)
    assert far.lambda_flags() == psi.lambda_flags()
    for i in range(1, 5):
        a = Q.contract_between(psi, i + 1, i, direction="left")
        r = O.contract_between_(ref.copy(), i, i - 1, direction="left")
        _check_same(a, r)
        assert a.lambda_between(i, i + 1) is None


def test_evolve_1site_and_2site_exact():
    n = 7
    psi, ref = _pair(n, 4, seed=31, uniform=False)
    for layer in R.brickwall_layers(n, 4, seed=32):
        for s, u in layer:
            Q.evolve_(psi, Q.gate_from_matrix(u, [s, s + 1]))
            O.evolve_2site_(ref, s - 1, u)
    x = R.haar_unitary(R.rng(33), 2)
    Q.evolve_(psi, Q.gate_from_matrix(x, [4]))
    O.evolve_1site_(ref, 3, x)
    _check_same(psi, ref)


def test_evolve_gate_site_order():
    psi, _ = _pair(4, 3, seed=41)
    u = R.haar_unitary(R.rng(42), 4)
    a = Q.evolve_(psi.copy(), Q.gate_from_matrix(u, [2, 3]))
    t = u.reshape(2, 2, 2, 2).transpose(1, 0, 3, 2)
    g = Q.Dense(Q.Operator(), t, [Q.Site(3), Q.Site(2), Q.Site(3, True), Q.Site(2, True)])
    b = Q.evolve_(psi.copy(), g)
    assert _close(_sv(a), _sv(b))


def test_evolve_errors():
    psi, _ = _pair(4, 2, seed=43)
    with pytest.raises(Q.ArgumentError):
        Q.evolve_(psi, Q.gate_from_matrix(np.eye(4), [1, 3]))
    with pytest.raises(Q.ArgumentError):
        Q.evolve_(psi, Q.gate_from_matrix(np.eye(2), [7]))
    with pytest.raises(Q.ArgumentError):
        Q.evolve_(psi, Q.gate_from_matrix(np.eye(8), [1, 2, 3]))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_tebd_with_truncation(precision):
    # TEBD of the n=64 / chi_max=256 workload shrunk to oracle size: |0..0>, Haar brick wall,
    # threshold 1e-10 and maxdim; bond dims must match after every gate.
    n, depth, maxdim = 12, 8, 12
    arrays = R.zero_product_arrays(n)
    psi, ref = Q.MPS(arrays), O.from_reference_arrays(arrays)
    psi.set_precision(precision)
    for layer in R.brickwall_layers(n, depth, seed=51):
        for s, u in layer:
            Q.evolve_(psi, Q.gate_from_matrix(u, [s, s + 1]), threshold=1e-10, maxdim=maxdim)
            O.evolve_2site_(ref, s - 1, u, threshold=1e-10, maxdim=maxdim)
            assert psi.bond_dims() == ref.bond_dims()
    tol = RTOL if precision == "fp64" else 1e-8
    _check_same(psi, ref, rtol=tol)
    for i in range(1, n + 1):
        xi = Q.gate_from_matrix(R.PAULI["X"], [i])
        e = Q.expect(psi, [xi])
        e_ref = O.expect(ref, [O.ODense(R.PAULI["X"], (O.OSite(i), O.OSite(i, True)))])
        assert abs(e - e_ref) <= tol * max(1.0, abs(e_ref))


@pytest.mark.parametrize("precision,lanes", [("fp64", 4), ("mixed", 4), ("mixed", 3)])
def test_layer_evolve_matches_gate_by_gate(precision, lanes):
    """evolve_layer_ runs a brick-wall layer's gates on several streams at once: the result is the
    gate-by-gate evolve! result (bond dims exact, Lambdas and sites to rounding), here through
    bonds up to 128 (theta 256 x 256: the multi-CTA FP32 / double-float sweeps run side by side),
    and the oracle's on the same gates."""
    n, depth, maxdim = 16, 10, 128
    arrays = R.zero_product_arrays(n)
    a, b = Q.MPS(arrays), Q.MPS(arrays)
    ref = O.from_reference_arrays(arrays)
    a.set_precision(precision)
    b.set_precision(precision)
    for layer in R.brickwall_layers(n, depth, seed=77):
        Q.evolve_layer_(a, [Q.gate_from_matrix(u, [s_, s_ + 1]) for s_, u in layer], threshold=1e-10, maxdim=maxdim,
                        lanes=lanes)
        for s_, u in layer:
            Q.evolve_(b, Q.gate_from_matrix(u, [s_, s_ + 1]), threshold=1e-10, maxdim=maxdim)
            O.evolve_2site_(ref, s_ - 1, u, threshold=1e-10, maxdim=maxdim)
        assert a.bond_dims() == b.bond_dims() == ref.bond_dims()
    assert max(a.bond_dims()) == maxdim
    for bnd in range(1, n):
        la, lb = a.lambda_between(bnd, bnd + 1), b.lambda_between(bnd, bnd + 1)
        assert np.max(np.abs(la - lb)) <= 1e-12 * lb[0]
    tol = RTOL if precision == "fp64" else 1e-8
    _check_same(a, ref, rtol=tol)
    assert abs(Q.overlap(a, b) - Q.norm(a) * Q.norm(b)) <= 1e-10 * Q.norm(a) * Q.norm(b)


def test_layer_evolve_rejects_overlapping_gates():
    psi = Q.MPS(R.zero_product_arrays(6))
    u = R.haar_unitary(R.rng(1), 4)
    with pytest.raises(Q.ArgumentError):
        Q.evolve_layer_(psi, [Q.gate_from_matrix(u, [2, 3]), Q.gate_from_matrix(u, [3, 4])], maxdim=4)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_truncated_gate_on_large_bond(precision):
    """A gate on a chi = 128 bond (theta 256 x 256: the mixed path's FP32-preconditioned SVD with
    double-float GEMMs and polish) truncated to maxdim = 100, so only the leading triplets are kept:
    bond dimension, the kept Lambda spectrum and local expectations against the oracle."""
    n, chi, maxdim = 16, 128, 100
    arrays = R.rand_chain_state_arrays(R.rng(61), n, chi, p=2)
    psi, ref = Q.MPS(arrays), O.from_reference_arrays(arrays)
    psi.set_precision(precision)
    u = R.haar_unitary(R.rng(62), 4)
    Q.evolve_(psi, Q.gate_from_matrix(u, [8, 9]), threshold=1e-12, maxdim=maxdim)
    O.evolve_2site_(ref, 7, u, threshold=1e-12, maxdim=maxdim)
    assert psi.bond_dims() == ref.bond_dims()
    assert psi.bond_dims()[7] == maxdim
    lam, lam_ref = psi.lambda_between(8, 9), ref.lam[7]
    assert _close(lam, lam_ref, 1e-10 if precision == "fp64" else 1e-9)
    tol = RTOL if precision == "fp64" else 1e-8
    for i in (7, 8, 9, 10):
        z = Q.gate_from_matrix(R.PAULI["Z"], [i])
        e = Q.expect(psi, [z])
        e_ref = O.expect(ref, [O.ODense(R.PAULI["Z"], (O.OSite(i), O.OSite(i, True)))])
        assert abs(e - e_ref) <= tol * max(1.0, abs(e_ref)), i


def test_checkpoint_roundtrip(tmp_path):
    """qr_chain_save / qr_chain_load: the file holds the reference-layout arrays and Lambdas
    (read back independently on the host) and restores the same chain."""
    from qrochet import checkpoint

    psi, ref = _pair(6, 4, seed=21, uniform=False)
    Q.canonize_(psi)
    O.canonize_(ref)
    psi.set_precision("mixed")
    path = tmp_path / "psi.qrchain"
    psi.save(path)
    arrays, lams, prec = checkpoint.read(path)
    assert prec == 1
    for a, b in zip(psi.arrays(), arrays):
        assert np.array_equal(np.asarray(a), b)
    assert [x is not None for x in lams] == psi.lambda_flags()
    back = Q.Chain.load(path)
    _check_same(back, ref)
    assert back.bond_dims() == psi.bond_dims()
    # a file from the host writer (e.g. exported from Julia) loads as well
    host = tmp_path / "host.qrchain"
    raw = R.gaussian_mps_arrays(5, 3, seed=22, uniform=True)
    checkpoint.write(host, raw)
    c2 = Q.Chain.load(host)
    assert _close(_sv(c2), O.to_statevector(O.from_reference_arrays(raw)))
    with pytest.raises(Q.ArgumentError):
        Q.Chain.load(tmp_path / "missing.qrchain")


@pytest.mark.parametrize("eltype", [np.float64, np.complex128])
def test_rand_state_on_device(eltype):
    """rand(Chain, Open, State; n, p, χ) on the device (Chain_test.jl:209-221): norm 1, bonds at
    most χ and equal to the sampler's pattern, sites 2..n right-canonical, seed-deterministic."""
    n, chi = 8, 10
    psi = Q.rand(Q.Chain, Q.Open, Q.State, n=n, chi=chi, p=2, eltype=eltype, seed=5)
    assert psi.bond_dims() == Q.sampler_bond_dims(n, chi, 2)
    assert max(psi.bond_dims()) <= chi
    assert abs(Q.norm(psi) - 1.0) <= 1e-12
    for i in range(2, n + 1):
        assert Q.isrightcanonical(psi, i)
    arrays = psi.arrays()
    if eltype is np.float64:
        assert all(np.max(np.abs(np.imag(a))) == 0 for a in arrays)
    else:
        assert any(np.max(np.abs(np.imag(a))) > 0.01 for a in arrays)
    again = Q.rand(Q.Chain, Q.Open, Q.State, n=n, chi=chi, p=2, eltype=eltype, seed=5)
    other = Q.rand(Q.Chain, Q.Open, Q.State, n=n, chi=chi, p=2, eltype=eltype, seed=6)
    assert all(np.array_equal(a, b) for a, b in zip(arrays, again.arrays()))
    assert not all(np.allclose(a, b) for a, b in zip(arrays, other.arrays()))
    # the oracle agrees on the state's norm from the same arrays
    assert abs(O.norm(O.from_reference_arrays(arrays)) - 1.0) <= 1e-12


def test_rand_operator_on_device():
    """rand(Chain, Open, Operator; n, p, χ) on the device (Chain_test.jl:223-235): Frobenius norm 1
    and bonds at most χ, checked on the downloaded arrays with the oracle."""
    n, chi = 6, 10
    w = Q.rand(Q.Chain, Q.Open, Q.Operator, n=n, chi=chi, p=2, seed=9)
    assert max(w._bonds) <= chi
    arrays = w.arrays()
    ws = [arrays[0][None, :, :, :]]
    ws += [np.transpose(a, (2, 0, 1, 3)) for a in arrays[1:-1]]
    ws += [np.transpose(arrays[-1], (2, 0, 1))[..., None]]
    dense = O.mpo_to_dense(ws)
    assert abs(np.linalg.norm(dense) - 1.0) <= 1e-12


def _ring(n, chi, seed, closing=2):
    g = R.rng(seed)
    bonds = [chi] * (n - 1) + [closing]
    arrays = [(g.standard_normal((2, bonds[i - 1], bonds[i])) + 1j * g.standard_normal((2, bonds[i - 1], bonds[i])))
              / np.sqrt(2 * bonds[i - 1]) for i in range(n)]
    arrays = [np.asfortranarray(a) for a in arrays]
    return Q.pMPS(arrays), O.from_reference_arrays_periodic(arrays), arrays


def test_periodic_construction_and_bookkeeping():
    """pMPS / Chain(State(), Periodic(), arrays) (Chain_test.jl:2-36, 165-176): site sizes,
    the closing bond, leftsite/rightsite/leftindex/rightindex wrapping around."""
    g = R.rng(30)
    arrays = [g.random((2, 1, 4)), g.random((2, 4, 3)), g.random((2, 3, 1))]
    psi = Q.pMPS(arrays)
    assert isinstance(psi.boundary, Q.Periodic)
    assert [psi.site_array(i + 1).shape for i in range(3)] == [(2, 1, 4), (2, 4, 3), (2, 3, 1)]
    assert psi.bond_dims() == [4, 3, 1]
    assert psi.leftindex(1) == psi.rightindex(3) is not None
    assert psi.leftindex(2) == psi.rightindex(1)
    assert psi.leftindex(3) == psi.rightindex(2)
    assert [psi.leftsite(i).id for i in (1, 2, 3)] == [3, 1, 2]
    assert [psi.rightsite(i).id for i in (1, 2, 3)] == [2, 3, 1]
    perm = Q.pMPS([np.transpose(a, (2, 0, 1)) for a in arrays], order=("r", "o", "l"))
    assert [perm.site_array(i + 1, ("r", "o", "l")).shape for i in range(3)] == [(4, 2, 1), (3, 2, 4), (1, 2, 3)]
    assert _close(_sv(perm), _sv(psi))
    with pytest.raises(Q.ArgumentError):
        Q.canonize_(psi)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_periodic_contractions_and_gates(precision):
    """Ring contraction (norm, overlap), evolve! on inner bonds with truncation, and expect of
    1- and 2-site observables on periodic chains, against the oracle."""
    psi, ref, _ = _ring(5, 3, seed=31, closing=2)
    phi, ref_phi, _ = _ring(5, 3, seed=32, closing=2)
    psi.set_precision(precision)
    assert abs(Q.norm(psi) - O.norm(ref)) <= RTOL * O.norm(ref)
    ov, ov_ref = Q.overlap(psi, phi), O.overlap(ref, ref_phi)
    assert abs(ov - ov_ref) <= RTOL * max(1.0, abs(ov_ref))
    u = R.haar_unitary(R.rng(33), 4)
    Q.evolve_(psi, Q.gate_from_matrix(u, [2, 3]), maxdim=4)
    O.evolve_2site_(ref, 1, u, maxdim=4)
    assert psi.bond_dims() == ref.bond_dims()
    assert _close(_sv(psi), O.to_statevector(ref), 1e-10)
    z = R.PAULI["Z"]
    zz = np.kron(z, z)
    e = Q.expect(psi, [Q.gate_from_matrix(z, [1]), Q.gate_from_matrix(zz, [4, 5])])
    e_ref = O.expect(ref, [O.ODense(z, (O.OSite(1), O.OSite(1, True))),
                           O.ODense(zz.reshape(2, 2, 2, 2), (O.OSite(4), O.OSite(5), O.OSite(4, True),
                                                            O.OSite(5, True)))])
    assert abs(e - e_ref) <= 1e-10 * max(1.0, abs(e_ref))


def test_periodic_checkpoint(tmp_path):
    psi, ref, arrays = _ring(4, 2, seed=34, closing=3)
    path = tmp_path / "ring.qrchain"
    psi.save(path)
    back = Q.Chain.load(path)
    assert back.periodic and back.bond_dims() == [2, 2, 2, 3]
    assert _close(_sv(back), O.to_statevector(ref))


def test_config1_pipeline():
    # plain workload: n=16, d=2, chi=32 Gaussian MPS; canonize!, norm, <Z_i Z_{i+1}> for all i
    psi, ref = _pair(16, 32, seed=1)
    Q.canonize_(psi)
    O.canonize_(ref)
    _check_same(psi, ref, statevector=False)
    assert np.isclose(Q.norm(psi), O.norm(ref), rtol=RTOL)
    zz = np.kron(R.PAULI["Z"], R.PAULI["Z"])
    for i in range(1, 16):
        e = Q.expect(psi, [Q.gate_from_matrix(zz, [i, i + 1])])
        e_ref = O.expect(ref, [O.ODense(zz.reshape(2, 2, 2, 2), (O.OSite(i), O.OSite(i + 1),
                                                              O.OSite(i, True), O.OSite(i + 1, True)))])
        assert abs(e - e_ref) <= RTOL * abs(O.norm(ref)) ** 2


def test_expect_products_and_overlap():
    n = 7
    psi, ref = _pair(n, 6, seed=61)
    phi, refp = _pair(n, 5, seed=62)
    assert np.isclose(Q.overlap(psi, phi), O.overlap(ref, refp), rtol=RTOL)
    zz = np.kron(R.PAULI["Z"], R.PAULI["Z"])
    obs_q = [Q.gate_from_matrix(R.PAULI["X"], [2]), Q.gate_from_matrix(R.PAULI["Y"], [5]),
             Q.gate_from_matrix(zz, [3, 4]), Q.gate_from_matrix(R.haar_unitary(R.rng(63), 4), [2, 3])]
    obs_o = [O.ODense(g.array, tuple(O.OSite(s.id, s.dual) for s in g.sites)) for g in obs_q]
    assert np.isclose(Q.expect(psi, obs_q), O.expect(ref, obs_o), rtol=RTOL)


def test_mpo_expect_xxz():
    n = 8
    psi, ref = _pair(n, 6, seed=71)
    arrs = R.xxz_mpo_arrays(n, 1.0, 0.7)
    H = Q.MPO(arrs)
    ws = []
    for i, a in enumerate(arrs):
        a = np.asarray(a)
        if i == 0:
            a = a[:, :, None, :]
        elif i == n - 1:
            a = a[:, :, :, None]
        ws.append(np.transpose(a, (2, 0, 1, 3)))
    assert np.isclose(Q.mpo_expect(psi, H), O.mpo_expect(ref, ws), rtol=RTOL)


def test_vidal_path_and_renormalize():
    n = 6
    psi, ref = _pair(n, 4, seed=81, uniform=False)
    Q.canonize_(psi)
    O.canonize_(ref)
    u = R.haar_unitary(R.rng(82), 4)
    a = Q.evolve_(psi.copy(), Q.gate_from_matrix(u, [3, 4]), iscanonical=True)
    ra = O.evolve_2site_(ref.copy(), 2, u, iscanonical=True)
    _check_same(a, ra)
    b = Q.evolve_(psi.copy(), Q.gate_from_matrix(u, [3, 4]), maxdim=2, iscanonical=True, renormalize=True)
    rb = O.evolve_2site_(ref.copy(), 2, u, maxdim=2, iscanonical=True, renormalize=True)
    _check_same(b, rb)
    c = Q.evolve_(psi.copy(), Q.gate_from_matrix(u, [3, 4]), maxdim=2, renormalize=True)
    rc = O.evolve_2site_(ref.copy(), 2, u, maxdim=2, renormalize=True)
    _check_same(c, rc)
    assert np.isclose(Q.norm(c), 1.0, rtol=1e-12)
    with pytest.raises(Q.ArgumentError):
        Q.evolve_(psi.copy(), Q.gate_from_matrix(u, [1, 2]), maxdim=2, renormalize=True)


def test_rank_deficient_and_zero_singular_values():
    # identity gate on |0..0> leaves theta rank 1: thin SVD keeps a zero singular value and
    # an orthonormal completion of U, like LAPACK
    n = 4
    psi, ref = Q.zeros_chain(n), O.from_reference_arrays(R.zero_product_arrays(n))
    Q.evolve_(psi, Q.gate_from_matrix(np.eye(4), [2, 3]))
    O.evolve_2site_(ref, 1, np.eye(4))
    _check_same(psi, ref)
    assert Q.isleftcanonical(psi, 2)


def test_ones_product_chain():
    """convert(Chain, ones(Product, n)) (Product.jl:48-54, Chain.jl:174-183): |1...1> with bonds
    of size 1, so <Z_i> = -1 on every site, norm 1 and no overlap with |0...0>."""
    n = 5
    psi = Q.ones_chain(n)
    assert list(psi.bond_dims()) == [1] * (n - 1)
    assert np.isclose(Q.norm(psi), 1.0, rtol=1e-14)
    for i in range(1, n + 1):
        assert abs(Q.expect(psi, [Q.gate_from_matrix(R.PAULI["Z"], [i])]) + 1.0) <= 1e-14
    assert abs(Q.overlap(psi, Q.zeros_chain(n))) <= 1e-15
    # overlap(::Product, ::Chain) (Chain.jl:751): the product converted to bonds of size 1
    vs = [np.array([1, 0]), np.array([0.6, 0.8j]), np.array([0, 1]), np.array([1, 1]) / np.sqrt(2), np.array([1, 0])]
    prod = Q.Product(vs)
    chain, ref = _pair(5, 3, seed=14)
    e, e_ref = Q.overlap(prod, chain), O.overlap(O.from_reference_arrays(R.product_arrays(vs)), ref)
    assert abs(e - e_ref) <= RTOL * max(1.0, abs(e_ref))
    assert abs(Q.overlap(chain, prod) - np.conj(e_ref)) <= RTOL * max(1.0, abs(e_ref))


# Split-precision environment contractions (QR_SPLIT_CONTRACT): ~FP32 accuracy per site step.
SPLIT_RTOL = 1e-5


def test_mpo_energy_config3_sites_reduced_chi_against_oracle():
    """The MPS-MPO workload's shape at 128 sites (XXZ, Jz = 1, Jxy = 0.7, w = 5) with chi = 16 in
    place of 1024, so the oracle's contraction finishes in seconds: the FP64 path within 1e-10
    and the split (tcgen05 BF16x3) path within the split tolerance of the oracle's energy."""
    n, chi = 128, 16
    g = R.rng(3)
    arrays = []
    for i in range(n):
        cl = 1 if i == 0 else min(chi, 2 ** i, 2 ** (n - i))
        cr = 1 if i == n - 1 else min(chi, 2 ** (i + 1), 2 ** (n - i - 1))
        a = R.complex_gaussian(g, (2, cl, cr)) / np.sqrt(2.0 * cl)
        arrays.append(np.asfortranarray(a[:, 0, :] if i == 0 else a[:, :, 0] if i == n - 1 else a))
    ref = O.from_reference_arrays(arrays)
    arrs = R.xxz_mpo_arrays(n, 1.0, 0.7)
    ws = []
    for i, a in enumerate(arrs):
        a = np.asarray(a)
        if i == 0:
            a = a[:, :, None, :]
        elif i == n - 1:
            a = a[:, :, :, None]
        ws.append(np.transpose(a, (2, 0, 1, 3)))
    e_ref = O.mpo_expect(ref, ws)
    scale = abs(O.norm(ref)) ** 2 * n
    H = Q.MPO(arrs)
    psi = Q.MPS(arrays)
    e64 = Q.mpo_expect(psi, H)
    assert abs(e64 - e_ref) <= 1e-10 * scale
    psi.set_precision("mixed+split")
    es = Q.mpo_expect(psi, H)
    assert abs(es - e_ref) <= SPLIT_RTOL * scale
    assert abs(es - e64) <= SPLIT_RTOL * scale


def test_split_contractions_match_fp64():
    n = 10
    psi, ref = _pair(n, 24, seed=91)
    phi, refp = _pair(n, 16, seed=92)
    for p in (psi, phi):
        p.set_precision("mixed+split")
    arrs = R.xxz_mpo_arrays(n, 1.0, 0.7)
    H = Q.MPO(arrs)
    ws = []
    for i, a in enumerate(arrs):
        a = np.asarray(a)
        if i == 0:
            a = a[:, :, None, :]
        elif i == n - 1:
            a = a[:, :, :, None]
        ws.append(np.transpose(a, (2, 0, 1, 3)))
    e_ref = O.mpo_expect(ref, ws)
    assert abs(Q.mpo_expect(psi, H) - e_ref) <= SPLIT_RTOL * abs(O.norm(ref)) ** 2 * 10
    assert abs(Q.overlap(psi, phi) - O.overlap(ref, refp)) <= SPLIT_RTOL * O.norm(ref) * O.norm(refp)
    assert abs(Q.norm(psi) - O.norm(ref)) <= SPLIT_RTOL * O.norm(ref)
    zz = np.kron(R.PAULI["Z"], R.PAULI["Z"])
    e = Q.expect(psi, [Q.gate_from_matrix(zz, [4, 5])])
    e_o = O.expect(ref, [O.ODense(zz.reshape(2, 2, 2, 2), (O.OSite(4), O.OSite(5), O.OSite(4, True),
                                                           O.OSite(5, True)))])
    assert abs(e - e_o) <= SPLIT_RTOL * abs(O.norm(ref)) ** 2
