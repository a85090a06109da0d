"""Generates tests/golden/tebd_n64_chi256_d40.npz: the oracle's results for the TEBD workload of
n = 64 qubits from |0...0>, a depth-40 brick wall of Haar-random 4 x 4 unitaries (seed 2), maxdim
256 and singular-value cutoff 1e-10, with evolve!'s defaults (iscanonical = false, renormalize =
false; Chain.jl:543-661).  Stored: the bond dimensions, every bond's Lambda spectrum (the last SVD
on that bond), <X_i> for every site (unnormalised, as expect does, Chain.jl:724-735), the norm,
and a checksum of the gates so a change in the gate stream is caught.

Run from the repository root:  python tests/golden/make_tebd_golden.py
(about two minutes of LAPACK work on a few cores).
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

N, DEPTH, MAXDIM, CUTOFF, SEED = 64, 40, 256, 1e-10, 2
OUT = os.path.join(HERE, "tebd_n64_chi256_d40.npz")


def gate_checksum(layers):
    return float(sum(np.abs(u).sum() + 0.5 * u.real.sum() for layer in layers for _, u in layer))


def main():
    t0 = time.time()
    layers = R.brickwall_layers(N, DEPTH, seed=SEED)
    ch = O.from_reference_arrays(R.zero_product_arrays(N))
    for layer in layers:
        for s, u in layer:
            O.evolve_2site_(ch, s - 1, u, threshold=CUTOFF, maxdim=MAXDIM)
    bonds = np.array(ch.bond_dims(), dtype=np.int32)
    lam = np.concatenate([ch.lam[b] for b in range(N - 1)])
    x = np.array([O.expect(ch, [O.ODense(R.PAULI["X"], (O.OSite(i), O.OSite(i, True)))]) for i in range(1, N + 1)])
    np.savez_compressed(OUT, bond_dims=bonds, lambdas=lam, x=x, norm=O.norm(ch), gate_checksum=gate_checksum(layers))
    print(f"wrote {OUT}: max bond {bonds.max()}, {time.time() - t0:.0f} s")


if __name__ == "__main__":
    main()
