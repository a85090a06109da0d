"""GPU tests of the batched engine (batch.cu) through the C ABI: every request's bond dimensions,
Lambda spectra and Pauli-string expectation values against the oracle (FP64: 1e-10 relative for
spectra, 1e-10 relative to <psi|psi> for expectation values; the FP32-preconditioned mode 1e-9),
the same requests through the request server, the graph and the autotuner's bookkeeping."""
import numpy as np
import pytest

from oracle import chain_oracle as O
from qrochet import random as R
from qrochet import serve as S
from qrochet.batch import Batch

pytestmark = pytest.mark.gpu

PAULI = {"X": R.PAULI["X"], "Y": R.PAULI["Y"], "Z": R.PAULI["Z"]}


def _oracle(req):
    psi = O.from_reference_arrays(R.zero_product_arrays(req.n))
    for s, u in req.gates:
        O.evolve_2site_(psi, s - 1, u, threshold=req.threshold, maxdim=req.chi_max)
    vals = []
    for o in req.observables:
        obs = [O.ODense(PAULI[p], (O.OSite(s), O.OSite(s, True))) for s, p in o if p != "I"]
        vals.append(O.expect(psi, obs))
    return psi, np.array(vals)


def _requests(count, seed, chi=(4, 8, 16, 32), n_range=(6, 14), depth_range=(2, 8)):
    g = R.rng(seed)
    return [S.random_request(g, n_range=n_range, depth_range=depth_range, chi_choices=chi, nobs=4)
            for _ in range(count)]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batch_matches_oracle(precision):
    tol = 1e-10 if precision == "fp64" else 1e-9
    reqs = _requests(12, 41)
    with Batch(precision=precision) as b:
        ids = [b.add(r) for r in reqs]
        b.run()
        info = b.info()
        assert info["graph_nodes"] >= info["launches"] >= info["layers"] >= 8
        assert info["warps_per_cta"] in (4, 8, 16)
        for rid, r in zip(ids, reqs):
            ref, vals = _oracle(r)
            assert b.bond_dims(rid) == ref.bond_dims()
            for bond, lm in enumerate(ref.lam):
                got = b.lambda_on(rid, bond)
                if lm is None:
                    assert got is None
                else:
                    assert np.max(np.abs(got - lm)) <= tol * lm[0], (rid, bond)
            nrm2 = abs(O.overlap(ref, ref))
            assert np.max(np.abs(b.values(rid) - vals)) <= tol * max(nrm2, 1e-300), rid


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batch_full_bond_class_matches_server(precision):
    """chi_max = 64 requests deep enough to saturate (theta of 128 x 128, re-orthonormalised
    vectors), against the same requests through the request server in FP64."""
    reqs = _requests(4, 43, chi=(64,), n_range=(14, 16), depth_range=(9, 10))
    with Batch(precision=precision) as b:
        ids = [b.add(r) for r in reqs]
        b.run()
        with S.Server(workers=4, precision="fp64") as sv:
            tickets = [sv.submit(r) for r in reqs]
            for rid, t, r in zip(ids, tickets, reqs):
                ref = sv.wait(t)["values"]
                assert max(b.bond_dims(rid)) == 64
                scale = max(1e-300, float(np.max(np.abs(ref))))
                assert np.max(np.abs(b.values(rid) - ref)) <= 1e-9 * scale, rid


def test_batch_edge_cases():
    """Two-site chains, a chain with no gates, an identity string (<psi|psi>), and a threshold
    that keeps no singular value (the engine flags that request with QR_EINVAL instead of leaving
    a size-0 bond in its fixed-capacity layout; the others are unaffected)."""
    g = R.rng(47)
    two = S.random_request(g, n_range=(2, 2), depth_range=(3, 3), chi_choices=(2,), nobs=2, weight_range=(1, 2))
    none = S.Request(n=5, chi_max=4, gates=[], observables=[[(1, "Z")], [(3, "X")]])
    ident = S.random_request(g, n_range=(6, 6), depth_range=(4, 4), chi_choices=(8,), nobs=1)
    ident.observables = [[]]
    empty = S.random_request(g, n_range=(4, 4), depth_range=(1, 1), chi_choices=(4,), nobs=1, threshold=10.0)
    with Batch() as b:
        ids = [b.add(r) for r in (two, none, ident, empty)]
        b.run()
        for rid, r in zip(ids[:3], (two, none, ident)):
            ref, vals = _oracle(r)
            assert b.bond_dims(rid) == ref.bond_dims()
            nrm2 = abs(O.overlap(ref, ref))
            assert np.max(np.abs(b.values(rid) - vals)) <= 1e-10 * max(nrm2, 1e-300), rid
        assert np.allclose(b.values(ids[1]), [1.0, 0.0])
        assert b.result(ids[3])["status"] == 1  # QR_EINVAL
