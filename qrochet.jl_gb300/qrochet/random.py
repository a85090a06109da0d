"""Seeded host-side generators for chains, gates and operators (NumPy ``PCG64``).

All complex Gaussians are (N(0,1) + i N(0,1)) / sqrt(2).  Arrays are returned in the
reference's own layout: Julia column-major with dims in the default ``order``
``(:o, :l, :r)`` for states and ``(:o, :i, :l, :r)`` for operators (``src/Ansatz/Chain.jl:33-34``),
i.e. NumPy arrays whose *shape* lists the Julia dims; callers pass them to ``MPS``/``MPO``
exactly as a Julia user passes ``Array``s.
"""
from __future__ import annotations

import numpy as np


def rng(seed):
    return np.random.Generator(np.random.PCG64(seed))


def complex_gaussian(g, shape):
    return (g.standard_normal(shape) + 1j * g.standard_normal(shape)) / np.sqrt(2.0)


def gaussian_mps_arrays(n, chi, d=2, seed=0, uniform=True):
    """Open-boundary MPS with i.i.d. complex Gaussian entries.

    ``uniform=True``: every bond has size ``chi`` (ends are (d, chi)), as in the plain n=16, chi=32
    workload.  ``uniform=False``: bonds are ``min(chi, d^i, d^(n-i))`` (no rank-deficient bonds).
    Returns reference-layout arrays: site 1 is (o, r), site n is (o, l), the rest (o, l, r).
    """
    g = rng(seed)
    dims = bond_dims(n, chi, d, uniform)
    arrays = []
    for i in range(n):
        cl = 1 if i == 0 else dims[i - 1]
        cr = 1 if i == n - 1 else dims[i]
        a = complex_gaussian(g, (d, cl, cr))
        if i == 0:
            a = a[:, 0, :]
        elif i == n - 1:
            a = a[:, :, 0]
        arrays.append(np.asfortranarray(a))
    return arrays


def bond_dims(n, chi, d=2, uniform=True):
    if uniform:
        return [chi] * (n - 1)
    return [min(chi, d ** (i + 1), d ** (n - i - 1)) for i in range(n - 1)]


def haar_unitary(g, dim):
    """Haar-random unitary: QR of a complex Gaussian with the phases of diag(R) divided out
    (Mezzadri, 'How to generate random matrices from the classical compact groups', 2007)."""
    z = complex_gaussian(g, (dim, dim))
    q, r = np.linalg.qr(z)
    ph = np.diag(r) / np.abs(np.diag(r))
    return q * ph[None, :]


def gate_array_from_matrix(m, d=2):
    """4x4 matrix M[(o1,o2),(i1,i2)] (o1 slowest) -> Julia-layout array with dims
    (o1, o2, i1, i2) for ``Dense(Operator(), array; sites=[l, r, l', r'])``."""
    t = np.asarray(m, dtype=np.complex128).reshape(d, d, d, d)
    return np.asfortranarray(t)


def brickwall_layers(n, depth, seed):
    """Depth-``depth`` brick wall of Haar 4x4 unitaries on n qubits.

    Odd layers (1st, 3rd, ...) act on bonds (1,2), (3,4), ...; even layers on (2,3), (4,5), ...
    (1-based sites).  Returns a list of layers, each a list of (left_site_1based, 4x4 matrix).
    """
    g = rng(seed)
    layers = []
    for layer in range(depth):
        start = 1 if layer % 2 == 0 else 2
        layers.append([(s, haar_unitary(g, 4)) for s in range(start, n, 2)])
    return layers


PAULI = {
    "I": np.eye(2, dtype=np.complex128),
    "X": np.array([[0, 1], [1, 0]], dtype=np.complex128),
    "Y": np.array([[0, -1j], [1j, 0]], dtype=np.complex128),
    "Z": np.array([[1, 0], [0, -1]], dtype=np.complex128),
}


def xxz_mpo_arrays(n, jz=1.0, jxy=0.7):
    """Heisenberg XXZ MPO with bond dimension 5, Pauli convention (sigma, not sigma/2):

        H = sum_i  jxy (X_i X_{i+1} + Y_i Y_{i+1}) + jz Z_i Z_{i+1}

    Bulk tensor (lower-triangular automaton), as a 5x5 block matrix of 2x2 operators:
        row 0: I  .  .  .  .
        row 1: X  .  .  .  .
        row 2: Y  .  .  .  .
        row 3: Z  .  .  .  .
        row 4: .  jxy X  jxy Y  jz Z  I
    Site 1 takes row 4, site n takes column 0.  Returned in the reference's operator layout:
    interior (o, i, l, r), site 1 (o, i, r), site n (o, i, l).
    """
    P = PAULI
    w = np.zeros((5, 5, 2, 2), dtype=np.complex128)  # [left, right, o, i]
    w[0, 0] = P["I"]
    w[1, 0] = P["X"]
    w[2, 0] = P["Y"]
    w[3, 0] = P["Z"]
    w[4, 1] = jxy * P["X"]
    w[4, 2] = jxy * P["Y"]
    w[4, 3] = jz * P["Z"]
    w[4, 4] = P["I"]
    arrays = []
    for i in range(n):
        t = np.transpose(w, (2, 3, 0, 1))  # (o, i, l, r)
        if i == 0:
            t = t[:, :, 4, :]
        elif i == n - 1:
            t = t[:, :, :, 0]
        arrays.append(np.asfortranarray(t))
    return arrays


def rand_chain_state_arrays(g, n, chi, p=2):
    """Sampler of ``rand(Chain, Open, State; n, chi, p)`` (``Chain.jl:223-256``): bond dims
    ``min(chi, p^i)`` mirrored about the midpoint, every site an isometry, state normalised.

    The reference orthogonalises a uniform random matrix with Muscle's Gram-Schmidt; here the
    isometry is the thin Q of a complex Gaussian (a different, seeded draw of the same family).
    """
    arrays = []
    for i in range(1, n + 1):
        after_mid = i > n // 2
        ii = (n + 1 - abs(2 * i - n - 1)) // 2
        cl, cr = min(chi, p ** (ii - 1)), min(chi, p ** ii)
        if n % 2 == 1 and i == n // 2 + 1:
            cl, cr = cl, cl
        elif after_mid:
            cl, cr = cr, cl
        if i == 1:
            cl, cr = cr, 1
        z = complex_gaussian(g, (cr * p, cl))
        q, _ = np.linalg.qr(z)  # (cr*p, cl) with orthonormal columns
        a = q.T.reshape(cl, cr, p)  # rows orthonormal: A A^dagger = I over (cr, p)
        a = np.transpose(a, (2, 0, 1))  # (p, cl, cr)
        arrays.append(a)
    arrays[0] = arrays[0].reshape(p, p)
    arrays[-1] = arrays[-1].reshape(p, p)
    arrays[0] = arrays[0] / np.sqrt(p)
    return [np.asfortranarray(a) for a in arrays]


def zero_product_arrays(n, d=2):
    """``convert(Chain, zeros(Product, n))``: |0...0> with bonds of size 1 (``Chain.jl:174-183``,
    ``Product.jl:44-46``)."""
    return basis_product_arrays(n, d, 0)


def one_product_arrays(n, d=2):
    """``convert(Chain, ones(Product, n))``: |1...1> with bonds of size 1 (``Chain.jl:174-183``,
    ``Product.jl:48-54``)."""
    return basis_product_arrays(n, d, 1)


def product_arrays(vectors):
    """``convert(Chain, Product(vectors))`` (Chain.jl:174-183): every site vector becomes a site
    with bonds of size 1, (o, r) at site 1, (o, l, r) inside, (o, l) at site n."""
    vs = [np.asarray(v) for v in vectors]
    if len(vs) < 2 or any(v.ndim != 1 for v in vs) or len({v.shape[0] for v in vs}) != 1:
        raise ValueError("a product state needs n >= 2 site vectors of one length")
    n = len(vs)
    out = []
    for i, v in enumerate(vs):
        v = v.astype(np.complex128)
        out.append(np.asfortranarray(v.reshape(-1, 1) if i in (0, n - 1) else v.reshape(-1, 1, 1)))
    return out


def basis_product_arrays(n, d, level):
    """Every lane in basis state ``level``: arrays as ``MPS(arrays)`` takes them, (o, r) at site 1,
    (o, l, r) inside, (o, l) at site n, all bonds of size 1."""
    if n < 2 or not 0 <= level < d:
        raise ValueError("a product chain needs n >= 2 sites and 0 <= level < d")
    arrays = []
    for i in range(n):
        v = np.zeros(d, dtype=np.complex128)
        v[level] = 1.0
        if i == 0 or i == n - 1:
            arrays.append(np.asfortranarray(v.reshape(d, 1)))
        else:
            arrays.append(np.asfortranarray(v.reshape(d, 1, 1)))
    return arrays
