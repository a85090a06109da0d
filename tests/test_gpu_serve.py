"""GPU tests of the request server: results against the oracle, and each request's result the
same alone and in a concurrent mix (continuous batching), within 1e-12."""
import numpy as np
import pytest

from oracle import chain_oracle as O
from qrochet import random as R
from qrochet import serve as S

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
    return np.array(vals)


def _requests(count, seed):
    g = R.rng(seed)
    return [S.random_request(g, n_range=(6, 12), depth_range=(2, 6), chi_choices=(4, 8, 16), nobs=4)
            for _ in range(count)]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_server_matches_oracle(precision):
    reqs = _requests(4, 7)
    with S.Server(workers=2, precision=precision) as sv:
        tickets = [sv.submit(r) for r in reqs]
        for r, t in zip(reqs, tickets):
            out = sv.wait(t)
            ref = _oracle(r)
            tol = 1e-10 if precision == "fp64" else 1e-8
            assert np.max(np.abs(out["values"] - ref)) <= tol, (out["values"], ref)
            assert out["latency_ms"] >= out["queue_ms"] >= 0


def test_results_same_alone_and_in_the_mix():
    reqs = _requests(10, 11)
    alone = []
    with S.Server(workers=1) as sv:
        for r in reqs:
            alone.append(sv.wait(sv.submit(r))["values"])
    with S.Server(workers=6) as sv:
        tickets = [sv.submit(r) for r in reqs]
        mixed = [sv.wait(t)["values"] for t in tickets]
        st = sv.stats()
    assert st["completed"] == len(reqs) and st["in_flight"] == 0
    for a, b in zip(alone, mixed):
        assert np.max(np.abs(a - b)) <= 1e-12


def test_large_mixed_requests_same_alone_and_in_the_mix():
    """Mixed-precision requests whose bonds reach chi = 128-256 (theta of 256-512 columns: the
    FP32-preconditioned SVD with the double-float polish, beyond the single-cluster kernels), run
    alone and then four at a time on one GPU; every expectation value must agree within 1e-12."""
    g = R.rng(23)
    reqs = [S.random_request(g, n_range=(16, 18), depth_range=(8, 10), chi_choices=(128, 256), nobs=4)
            for _ in range(4)]
    with S.Server(workers=1, precision="mixed") as sv:
        alone = [sv.wait(sv.submit(r))["values"] for r in reqs]
    with S.Server(workers=4, precision="mixed") as sv:
        tickets = [sv.submit(r) for r in reqs]
        mixed = [sv.wait(t)["values"] for t in tickets]
    for a, b in zip(alone, mixed):
        assert np.max(np.abs(a - b)) <= 1e-12
