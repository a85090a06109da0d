"""Chain checkpoint files (``qr_chain_save`` / ``qr_chain_load``), readable without a GPU.

Layout (little-endian):
    b"QRCHAIN1" | int32 n, d, precision, periodic | int32 bond_dims[n-1, or n when periodic: the
    last joins site n and site 1] | uint8 has_lambda[n-1]
    | site 1..n: ComplexF64 data, column-major in the reference's (:o, :l, :r) order, the open
      ends without :l (site 1) and :r (site n) -- exactly the arrays ``MPS(arrays)`` (or, all 3-d,
      ``pMPS(arrays)``) takes
    | for every bond with has_lambda: Float64 Lambda[bond_dim]
"""
from __future__ import annotations

import numpy as np

MAGIC = b"QRCHAIN1"


def site_shapes(n, d, bonds, periodic=False):
    """Reference-layout shapes of the n site arrays for bond dimensions ``bonds``."""
    if periodic:
        return [(d, bonds[(i - 1) % n], bonds[i]) for i in range(n)]
    shapes = []
    for i in range(n):
        if i == 0:
            shapes.append((d, bonds[0]))
        elif i == n - 1:
            shapes.append((d, bonds[-1]))
        else:
            shapes.append((d, bonds[i - 1], bonds[i]))
    return shapes


def read(path, with_boundary=False):
    """Returns (arrays, lambdas, precision) -- and the periodic flag when ``with_boundary`` --
    arrays in the reference layout (Fortran order), lambdas[b] the Lambda vector of bond b
    (between sites b+1 and b+2) or None."""
    with open(path, "rb") as f:
        if f.read(8) != MAGIC:
            raise ValueError("not a chain checkpoint")
        n, d, prec, per = (int(x) for x in np.frombuffer(f.read(16), dtype="<i4"))
        nb = n if per else n - 1
        bonds = [int(x) for x in np.frombuffer(f.read(4 * nb), dtype="<i4")]
        flags = np.frombuffer(f.read(n - 1), dtype=np.uint8)
        arrays = []
        for shp in site_shapes(int(n), int(d), bonds, bool(per)):
            cnt = int(np.prod(shp))
            data = np.frombuffer(f.read(16 * cnt), dtype="<c16")
            if data.size != cnt:
                raise ValueError("truncated chain checkpoint")
            arrays.append(np.asfortranarray(data.reshape(shp, order="F")))
        lams = []
        for b in range(int(n) - 1):
            if flags[b]:
                lam = np.frombuffer(f.read(8 * bonds[b]), dtype="<f8").copy()
                if lam.size != bonds[b]:
                    raise ValueError("truncated chain checkpoint")
                lams.append(lam)
            else:
                lams.append(None)
    if with_boundary:
        return arrays, lams, int(prec), bool(per)
    return arrays, lams, int(prec)


def write(path, arrays, lambdas=None, precision=0, periodic=False):
    """Writes reference-layout arrays (and optional Lambda vectors) in the checkpoint layout."""
    n = len(arrays)
    d = int(np.asarray(arrays[0]).shape[0])
    if periodic:
        bonds = [int(np.asarray(a).shape[2]) for a in arrays]
    else:
        bonds = [int(np.asarray(arrays[0]).shape[1])] + [int(np.asarray(a).shape[2]) for a in arrays[1:-1]]
    lambdas = lambdas or [None] * (n - 1)
    with open(path, "wb") as f:
        f.write(MAGIC)
        f.write(np.array([n, d, precision, 1 if periodic else 0], dtype="<i4").tobytes())
        f.write(np.array(bonds, dtype="<i4").tobytes())
        f.write(np.array([lam is not None for lam in lambdas], dtype=np.uint8).tobytes())
        for a in arrays:
            f.write(np.asarray(a, dtype="<c16").tobytes(order="F"))
        for lam in lambdas:
            if lam is not None:
                f.write(np.asarray(lam, dtype="<f8").tobytes())
