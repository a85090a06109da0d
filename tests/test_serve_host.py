"""Host-side behaviour of the request server (no GPU needed): validation, admission control by
device-memory footprint, and failures reported per request instead of hanging the server."""
import numpy as np
import pytest

import qrochet as Q
from qrochet import serve as S
from qrochet import random as R


@pytest.fixture(scope="module", autouse=True)
def _built():
    import __graft_entry__ as g

    g.build()


def _req(n=6, chi=8, ngates=3):
    g = R.rng(1)
    gates = [(1 + (k % (n - 1)), R.haar_unitary(g, 4)) for k in range(ngates)]
    return S.Request(n=n, chi_max=chi, gates=gates, observables=[[(2, "Z")], [(1, "X"), (3, "Y")]])


def test_footprint_model_grows_with_chi():
    assert S.footprint(32, 1024) > S.footprint(32, 128) > S.footprint(32, 16)
    # n=128 at chi=1024: 4 GiB of sites plus about 0.8 GiB of SVD/theta workspace
    assert 4 << 30 < S.footprint(128, 1024) < 5 << 30


def test_malformed_requests_are_rejected():
    with S.Server(workers=1, hbm_budget_bytes=1 << 30) as sv:
        with pytest.raises(Q.ArgumentError):
            sv.submit(S.Request(n=1, chi_max=4, gates=[], observables=[]))
        bad_gate = _req()
        bad_gate.gates = [(6, np.eye(4))]  # lanes 6,7 outside a 6-site chain
        with pytest.raises(Q.ArgumentError):
            sv.submit(bad_gate)
        bad_obs = _req()
        bad_obs.observables = [[(9, "Z")]]
        with pytest.raises(Q.ArgumentError):
            sv.submit(bad_obs)


def test_requests_larger_than_the_budget_are_refused():
    big = _req(n=64, chi=1024)
    with S.Server(workers=1, hbm_budget_bytes=S.footprint(64, 1024) - 1) as sv:
        with pytest.raises(Q.GPUError, match="HBM budget"):
            sv.submit(big)


def test_failed_request_is_reported_not_hung():
    if Q.device_count() > 0:
        pytest.skip("needs a host without a GPU to make the request fail")
    with S.Server(workers=2, hbm_budget_bytes=1 << 30) as sv:
        t = sv.submit(_req())
        with pytest.raises(Q.GPUError):
            sv.wait(t, timeout=60)
        st = sv.stats()
        assert st["completed"] == 1 and st["in_flight"] == 0 and st["hbm_in_use"] == 0
