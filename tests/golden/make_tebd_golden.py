"""Generates tests/golden/tebd_n64_chi256_d40.npz: the oracle's results for the TEBD workload of
n = 64 qubits from |0...0>, a depth-40 brick wall of Haar-random 4 x 4 unitaries (seed 2), maxdim
256 and singular-value cutoff 1e-10, with evolve!'s defaults (iscanonical = false, renormalize =
false; Chain.jl:543-661).  Stored, after layer 20 (prefix d20_) and after layer 40: the bond
dimensions, every bond's Lambda spectrum (the last SVD on that bond), <X_i> for every site
(unnormalised, as expect does, Chain.jl:724-735) and the norm; plus a checksum of the gates so a
change in the gate stream is caught.

The workload amplifies rounding differences: every gate truncates theta to 256 of up to 512
singular values without the neighbouring Lambda weights, and an O(eps) change of theta moves the
kept subspace.  Measured here, two correct FP64 runs drift apart by a factor ~1.8 per layer.  With
--sensitivity the script also reruns the circuit with LAPACK's gesvd in place of gesdd (both
backward stable) and stores how far the two oracles end apart (sens_*): the spread that any FP64
implementation can be expected to show against this golden file after 40 layers.

Run from the repository root:  python tests/golden/make_tebd_golden.py [--sensitivity]
(about three minutes of LAPACK work on 8 cores; --sensitivity adds ~20 minutes).
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "qrochet.jl_gb300"))

from oracle import chain_oracle as O  # noqa: E402
from qrochet import random as R  # noqa: E402

N, DEPTH, MID, MAXDIM, CUTOFF, SEED = 64, 40, 20, 256, 1e-10, 2
OUT = os.path.join(HERE, "tebd_n64_chi256_d40.npz")


def gate_checksum(layers):
    return float(sum(np.abs(u).sum() + 0.5 * u.real.sum() for layer in layers for _, u in layer))


def summary(ch):
    bonds = np.array(ch.bond_dims(), dtype=np.int32)
    lam = np.concatenate([ch.lam[b] for b in range(N - 1)])
    x = np.array([O.expect(ch, [O.ODense(R.PAULI["X"], (O.OSite(i), O.OSite(i, True)))]) for i in range(1, N + 1)])
    return bonds, lam, x, O.norm(ch)


def run(layers):
    ch = O.from_reference_arrays(R.zero_product_arrays(N))
    out = {}
    for L, layer in enumerate(layers):
        for s, u in layer:
            O.evolve_2site_(ch, s - 1, u, threshold=CUTOFF, maxdim=MAXDIM)
        if L + 1 == MID:
            out["mid"] = summary(ch)
    out["end"] = summary(ch)
    return out


def main():
    t0 = time.time()
    layers = R.brickwall_layers(N, DEPTH, seed=SEED)
    res = run(layers)
    data = {"gate_checksum": gate_checksum(layers)}
    for tag, key in (("mid", "d20_"), ("end", "")):
        bonds, lam, x, nrm = res[tag]
        data.update({key + "bond_dims": bonds, key + "lambdas": lam, key + "x": x, key + "norm": nrm})
    if "--sensitivity" in sys.argv:
        import scipy.linalg as sl

        def svd_gesvd(m):
            return sl.svd(m, full_matrices=False, lapack_driver="gesvd")

        O._thin_svd = svd_gesvd
        bonds, lam, x, nrm = run(layers)["end"]
        lg = np.split(data["lambdas"], np.cumsum(data["bond_dims"])[:-1])
        la = np.split(lam, np.cumsum(bonds)[:-1])
        data["sens_lambda_rel"] = max(float(np.max(np.abs(la[b] - lg[b])) / lg[b][0]) for b in range(N - 1))
        data["sens_x_over_norm2"] = float(np.max(np.abs(x - data["x"]))) / float(data["norm"]) ** 2
        data["sens_norm_rel"] = abs(nrm - float(data["norm"])) / float(data["norm"])
    np.savez_compressed(OUT, **data)
    print(f"wrote {OUT}: {time.time() - t0:.0f} s; " +
          ", ".join(f"{k}={float(v):.3g}" for k, v in data.items() if k.startswith("sens_")))


if __name__ == "__main__":
    main()
