"""CPU checks of the committed TEBD golden file (tests/golden/tebd_n64_chi256_d40.npz) against the
generator that made it (tests/golden/make_tebd_golden.py): the same Haar gate stream, and
results that have the structure evolve! with maxdim 256 and cutoff 1e-10 gives (Chain.jl:543-661,
390-422) -- bond dimensions within min(256, 2^i, 2^(n-i)), descending Lambda spectra above the
cutoff, a norm that truncation only lowers, and <X_i> bounded by <psi|psi>."""
import importlib.util
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden", "tebd_n64_chi256_d40.npz")


@pytest.fixture(scope="module")
def gen():
    spec = importlib.util.spec_from_file_location("make_tebd_golden", os.path.join(HERE, "golden", "make_tebd_golden.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLDEN)


def test_gate_stream_matches_generator(gen, gold):
    from qrochet import random as R

    layers = R.brickwall_layers(gen.N, gen.DEPTH, seed=gen.SEED)
    assert len(layers) == 40
    cs = gen.gate_checksum(layers)
    assert abs(cs - float(gold["gate_checksum"])) <= 1e-12 * abs(cs)
    for L, layer in enumerate(layers):
        first = 1 if L % 2 == 0 else 2  # odd layers (1-based) on bonds (1,2),(3,4)...; even on (2,3)...
        assert [s for s, _ in layer] == list(range(first, gen.N, 2))
        for _, u in layer:
            assert u.shape == (4, 4)
            np.testing.assert_allclose(u.conj().T @ u, np.eye(4), atol=1e-13)


@pytest.mark.parametrize("prefix", ["d20_", ""])
def test_golden_structure(gen, gold, prefix):
    n = gen.N
    bonds = gold[prefix + "bond_dims"]
    lam = gold[prefix + "lambdas"]
    x = gold[prefix + "x"]
    nrm = float(gold[prefix + "norm"])
    assert bonds.shape == (n - 1,) and x.shape == (n,)
    for b in range(n - 1):
        assert 1 <= bonds[b] <= min(gen.MAXDIM, 2 ** (b + 1), 2 ** (n - b - 1))
    assert int(bonds.sum()) == lam.size
    for s in np.split(lam, np.cumsum(bonds)[:-1]):
        assert np.all(np.diff(s) <= 0), "Lambda spectra are descending"
        assert np.all(s > gen.CUTOFF), "truncate! keeps only values above the cutoff"
    assert 0.0 < nrm <= 1.0 + 1e-12, "unitary gates and truncation never raise the norm"
    assert np.all(np.abs(x) <= nrm ** 2 * (1 + 1e-9)), "|<X_i>| <= <psi|psi>"
    if prefix == "":
        assert int(bonds.max()) == gen.MAXDIM, "depth 40 saturates the bond cap"


def test_golden_records_oracle_spread(gold):
    """The generator's --sensitivity run (gesvd against gesdd) is stored, so the GPU tolerance has
    a measured floor."""
    for k in ("sens_lambda_rel", "sens_x_over_norm2", "sens_norm_rel"):
        v = float(gold[k])
        assert 0.0 < v < 1e-1, k
