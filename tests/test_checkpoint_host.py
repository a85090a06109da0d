"""Chain checkpoint layout on the host (no GPU): the pure-Python writer and reader agree, and the
arrays come back in the reference's (:o, :l, :r) layout that MPS(arrays) / the oracle accept."""
import numpy as np
import pytest

from oracle import chain_oracle as O
from qrochet import checkpoint
from qrochet import random as R


def test_roundtrip_arrays_and_lambdas(tmp_path):
    arrays = R.gaussian_mps_arrays(5, 3, seed=11, uniform=False)
    lams = [None, np.array([0.9, 0.3, 0.1]), None, None]
    lams[1] = lams[1][: arrays[1].shape[2]]
    path = tmp_path / "c.qrchain"
    checkpoint.write(path, arrays, lams, precision=1)
    back, lb, prec = checkpoint.read(path)
    assert prec == 1
    assert [a.shape for a in back] == [a.shape for a in arrays]
    for a, b in zip(arrays, back):
        assert np.array_equal(np.asarray(a, dtype=complex), b)
    assert lb[0] is None and np.array_equal(lb[1], lams[1])
    # the arrays feed MPS(arrays) directly
    sv1 = O.to_statevector(O.from_reference_arrays(arrays))
    sv2 = O.to_statevector(O.from_reference_arrays(back))
    assert np.allclose(sv1, sv2)


def test_rejects_foreign_and_truncated_files(tmp_path):
    bad = tmp_path / "x.bin"
    bad.write_bytes(b"NOTACHAIN" + bytes(32))
    with pytest.raises(ValueError):
        checkpoint.read(bad)
    arrays = R.gaussian_mps_arrays(4, 2, seed=3, uniform=True)
    good = tmp_path / "g.qrchain"
    checkpoint.write(good, arrays)
    data = good.read_bytes()
    cut = tmp_path / "cut.qrchain"
    cut.write_bytes(data[:-8])
    with pytest.raises(ValueError):
        checkpoint.read(cut)


def test_roundtrip_with_an_empty_bond(tmp_path):
    """A chain whose bond was sliced to size 0 by truncate! (the null state) keeps its shapes and
    its empty Lambda through a checkpoint."""
    arrays = R.gaussian_mps_arrays(4, 3, seed=5, uniform=True)
    arrays[1] = np.zeros((2, arrays[1].shape[1], 0), dtype=complex)
    arrays[2] = np.zeros((2, 0, arrays[2].shape[2]), dtype=complex)
    lams = [None, np.zeros(0), None]
    path = tmp_path / "e.qrchain"
    checkpoint.write(path, arrays, lams)
    back, lb, _ = checkpoint.read(path)
    assert [a.shape for a in back] == [a.shape for a in arrays]
    assert lb[1] is not None and lb[1].size == 0 and lb[0] is None and lb[2] is None
