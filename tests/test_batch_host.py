"""Host-side logic of the batched engine, no GPU needed: request validation and the layer
schedule (a gate opens a new layer when it shares a site with the current layer, so a depth-d
brick wall is d layers)."""
import numpy as np
import pytest

from qrochet import _lib
from qrochet import random as R
from qrochet import serve as S


@pytest.fixture(scope="module")
def built():
    import __graft_entry__ as g

    g.build()


def test_layers_of_a_brick_wall(built):
    from qrochet.batch import Batch

    g = R.rng(3)
    with Batch() as b:
        for n, depth in [(7, 5), (12, 9), (3, 3)]:
            req = S.random_request(g, n_range=(n, n), depth_range=(depth, depth), chi_choices=(16,), nobs=1,
                                   weight_range=(1, 2))
            rid = b.add(req)
            layer, nl = b.plan(rid)
            assert nl == depth
            # every layer's gates sit on disjoint site pairs, in circuit order
            for L in range(nl):
                sites = [s for (s, _), ly in zip(req.gates, layer) if ly == L]
                used = [x for s in sites for x in (s, s + 1)]
                assert len(used) == len(set(used))
            assert list(layer) == sorted(layer)


def test_rejects_what_it_cannot_run(built):
    from qrochet.batch import Batch

    g = R.rng(4)
    with Batch() as b:
        big = S.random_request(g, n_range=(10, 10), depth_range=(4, 4), chi_choices=(128,), nobs=1)
        with pytest.raises(_lib.ArgumentError, match="chi_max <= 64"):
            b.add(big)
        bad = S.Request(n=4, chi_max=8, gates=[(4, np.eye(4))], observables=[])
        with pytest.raises(_lib.ArgumentError, match="gate site"):
            b.add(bad)
        ok = b.add(S.random_request(g, n_range=(6, 6), depth_range=(2, 2), chi_choices=(8,), nobs=1))
        with pytest.raises(_lib.ArgumentError, match="not run"):
            b.result(ok)


def test_validation_and_empty_cases(built):
    """Each rejection qr_batch_add / qr_batch_plan / qr_batch_run make before any device work, and
    the plan of a request without gates (no layers)."""
    from qrochet.batch import Batch

    with Batch() as b:
        with pytest.raises(_lib.ArgumentError, match="empty batch"):
            b.run()
        with pytest.raises(_lib.ArgumentError, match="n >= 2"):
            b.add(S.Request(n=1, chi_max=8, gates=[], observables=[]))
        with pytest.raises(_lib.ArgumentError, match="Pauli string entry"):
            b.add(S.Request(n=4, chi_max=8, gates=[], observables=[[(5, "Z")]]))
        with pytest.raises(_lib.ArgumentError, match="Pauli letter"):
            b.add(S.Request(n=4, chi_max=8, gates=[], observables=[[(1, "W")]]))
        with pytest.raises(_lib.ArgumentError, match="gate site"):
            b.add(S.Request(n=4, chi_max=8, gates=[(0, np.eye(4))], observables=[]))
        rid = b.add(S.Request(n=4, chi_max=8, gates=[], observables=[[(1, "Z")]]))
        layers, nl = b.plan(rid)
        assert nl == 0 and len(layers) == 0
        with pytest.raises(_lib.ArgumentError, match="request id"):
            b.plan(rid + 1)


def test_layers_follow_circuit_order(built):
    """A gate opens a new layer exactly when it shares a site with a gate of the current layer,
    so gates on disjoint sites stay together and the order of the circuit is kept."""
    from qrochet.batch import Batch

    u = np.eye(4)
    gates = [(1, u), (3, u), (5, u), (2, u), (4, u), (1, u), (6, u), (3, u)]
    with Batch() as b:
        rid = b.add(S.Request(n=8, chi_max=8, gates=gates, observables=[]))
        layers, nl = b.plan(rid)
    assert list(layers) == [0, 0, 0, 1, 1, 2, 2, 2] and nl == 3


def test_unknown_precision_names(built):
    from qrochet.batch import Batch

    with pytest.raises(_lib.ArgumentError, match="fp64"):
        Batch(precision="fp32")
    with pytest.raises(_lib.ArgumentError, match="precision"):
        S.Server(precision="half")
