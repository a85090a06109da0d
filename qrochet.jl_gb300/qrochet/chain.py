"""Host mirror of Qrochet.jl's ``Chain`` API (src/Ansatz/Chain.jl) over the CUDA library.

A ``Chain`` owns one open-boundary MPS resident in GPU memory.  Julia's in-place methods
(``canonize!``) are the trailing-underscore functions here (``canonize_``); the copying forms
keep the Julia name.  Sites are 1-based ``Site`` objects as in the reference; errors are the
reference's exception types.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from ._lib import ArgumentError, check, dptr, lib
from .dense import Dense, Operator, State, validate_gate
from .site import Site, nextindex


class Open:
    """Open boundary."""


class Periodic:
    """Periodic boundary: the last site's right bond is the first site's left bond."""


_DIR = {"left": L.QR_DIR_LEFT, "right": L.QR_DIR_RIGHT}
_METHOD = {"qr": L.QR_METHOD_QR, "svd": L.QR_METHOD_SVD}
# "mixed": FP32-preconditioned SVD with FP64 refinement; "split": environment contractions on the
# BF16 tensor cores (3-way split, FP32 accumulation); "mixed+split": both
_PREC = {"fp64": 0, "mixed": 1, "split": 2, "mixed+split": 3}


def _choice(table, key, what):
    """table[key], or the ArgumentError the reference raises for an unknown symbol."""
    key = str(key).lstrip(":")
    if key not in table:
        raise ArgumentError(f"Unknown {what}=:{key}")
    return table[key]


def _norm_order(order, letters):
    order = tuple(str(x).lstrip(":") for x in order)
    if len(order) != len(letters) or set(order) != set(letters):
        raise ArgumentError(f"order must be a permutation of {tuple(letters)}")
    return order


def _site_id(s):
    if isinstance(s, Site):
        return s.id
    return int(s)


class Chain:
    """MPS in device memory (``Chain{Quantum, Open}`` or ``Chain{Quantum, Periodic}`` with a
    ``State`` socket)."""

    def __init__(self, handle, n, d, phys=None, bonds=None, periodic=False):
        self._h = handle
        self.n = n
        self.d = d
        self.periodic = bool(periodic)
        self._phys = phys or [nextindex() for _ in range(n)]
        self._bonds = bonds or [nextindex() for _ in range(n if self.periodic else n - 1)]

    # ---- construction ------------------------------------------------------------------------
    @classmethod
    def from_arrays(cls, arrays, order=("o", "l", "r")):
        """``Chain(State(), Open(), arrays; order)`` (Chain.jl:64-100)."""
        order = _norm_order(order, "olr")
        n = len(arrays)
        if n < 2:
            raise ArgumentError("a Chain needs at least 2 sites")
        arrays = [np.asarray(a) for a in arrays]
        if arrays[0].ndim != 2:
            raise AssertionError("First array must have 2 dimensions")
        if arrays[-1].ndim != 2:
            raise AssertionError("Last array must have 2 dimensions")
        if any(a.ndim != 3 for a in arrays[1:-1]):
            raise AssertionError("All arrays must have 3 dimensions")
        dims = []
        for i, a in enumerate(arrays):
            sub = [x for x in order if not ((i == 0 and x == "l") or (i == n - 1 and x == "r"))]
            dims.append(dict(zip(sub, a.shape)))
        d = dims[0]["o"]
        bond = []
        for i in range(n - 1):
            r, l = dims[i]["r"], dims[i + 1]["l"]
            if r != l:
                raise L.DimensionMismatch(f"bond {i + 1}: {r} != {l}")
            bond.append(r)
        if any(x["o"] != d for x in dims):
            raise L.DimensionMismatch("all sites must share the physical dimension")
        h = C.c_void_p()
        b = (C.c_int * (n - 1))(*bond)
        check(lib().qr_chain_create(n, d, b, C.byref(h)))
        ch = cls(h, n, d)
        ordstr = "".join(order).encode()
        for i, a in enumerate(arrays):
            buf = np.asfortranarray(a, dtype=np.complex128)
            check(lib().qr_chain_upload_site(h, i, dptr(buf), ordstr))
        return ch

    @classmethod
    def from_arrays_periodic(cls, arrays, order=("o", "l", "r")):
        """``Chain(State(), Periodic(), arrays; order)`` (Chain.jl:36-62): every site is 3-d and
        site n's right bond closes onto site 1's left bond."""
        order = _norm_order(order, "olr")
        n = len(arrays)
        if n < 2:
            raise ArgumentError("a Chain needs at least 2 sites")
        arrays = [np.asarray(a) for a in arrays]
        if any(a.ndim != 3 for a in arrays):
            raise AssertionError("All arrays must have 3 dimensions")
        dims = [dict(zip(order, a.shape)) for a in arrays]
        d = dims[0]["o"]
        bond = []
        for i in range(n):
            r, l = dims[i]["r"], dims[(i + 1) % n]["l"]
            if r != l:
                raise L.DimensionMismatch(f"bond {i + 1}: {r} != {l}")
            bond.append(r)
        if any(x["o"] != d for x in dims):
            raise L.DimensionMismatch("all sites must share the physical dimension")
        h = C.c_void_p()
        check(lib().qr_chain_create_periodic(n, d, (C.c_int * n)(*bond), C.byref(h)))
        ch = cls(h, n, d, periodic=True)
        ordstr = "".join(order).encode()
        for i, a in enumerate(arrays):
            buf = np.asfortranarray(a, dtype=np.complex128)
            check(lib().qr_chain_upload_site(h, i, dptr(buf), ordstr))
        return ch

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and L._lib is not None:
            try:
                L._lib.qr_chain_free(h)
            except Exception:
                pass
            self._h = None

    def copy(self):
        h = C.c_void_p()
        check(lib().qr_chain_copy(self._h, C.byref(h)))
        return Chain(h, self.n, self.d, list(self._phys), list(self._bonds), self.periodic)

    def save(self, path):
        """Checkpoint: the sites in the reference's ``(:o, :l, :r)`` layout, bond dimensions,
        Lambda vectors and precision (``qr_chain_save``; layout in ``qrochet.checkpoint``)."""
        check(lib().qr_chain_save(self._h, str(path).encode()))

    @classmethod
    def load(cls, path):
        """Restore a checkpoint written by ``save`` (or by any writer of the same layout)."""
        h = C.c_void_p()
        check(lib().qr_chain_load(str(path).encode(), C.byref(h)))
        n = C.c_int()
        check(lib().qr_chain_nsites(h, C.byref(n)))
        a, d, b = C.c_int(), C.c_int(), C.c_int()
        check(lib().qr_chain_site_dims(h, 0, C.byref(a), C.byref(d), C.byref(b)))
        per = C.c_int()
        check(lib().qr_chain_boundary(h, C.byref(per)))
        return cls(h, n.value, d.value, periodic=bool(per.value))

    __copy__ = copy
    __deepcopy__ = lambda self, memo: self.copy()  # noqa: E731

    # ---- bookkeeping -------------------------------------------------------------------------
    socket = State()

    @property
    def boundary(self):
        return Periodic() if self.periodic else Open()

    def nsites(self):
        return self.n

    def sites(self):
        return [Site(i + 1) for i in range(self.n)]

    def bond_dims(self):
        """Bond sizes: bond b joins sites b+1 and b+2; a periodic chain has an n-th bond
        between site n and site 1."""
        nb = self.n if self.periodic else self.n - 1
        out = (C.c_int * nb)()
        check(lib().qr_chain_bond_dims(self._h, out))
        return list(out)

    def lambda_flags(self):
        f = C.c_int()
        res = []
        for b in range(self.n - 1):
            check(lib().qr_chain_has_lambda(self._h, b, C.byref(f)))
            res.append(bool(f.value))
        return res

    def ntensors(self):
        """``length(tensors(tn))``: sites plus Lambda vectors."""
        c = C.c_int()
        check(lib().qr_chain_ntensors(self._h, C.byref(c)))
        return c.value

    def site_dims(self, site):
        i = _site_id(site) - 1
        a, d, b = C.c_int(), C.c_int(), C.c_int()
        check(lib().qr_chain_site_dims(self._h, i, C.byref(a), C.byref(d), C.byref(b)))
        return a.value, d.value, b.value

    def leftsite(self, site):
        """``leftsite`` (Chain.jl:185-188): wraps around on a periodic chain."""
        i = _site_id(site)
        if self.periodic:
            return Site((i - 2) % self.n + 1)
        return Site(i - 1) if 2 <= i <= self.n else None

    def rightsite(self, site):
        i = _site_id(site)
        if self.periodic:
            return Site(i % self.n + 1)
        return Site(i + 1) if 1 <= i <= self.n - 1 else None

    def leftindex(self, site):
        """``leftindex`` (Chain.jl:195-197)."""
        i = _site_id(site)
        if self.periodic:
            return self._bonds[(i - 2) % self.n]
        return None if i == 1 else self._bonds[i - 2]

    def rightindex(self, site):
        i = _site_id(site)
        if self.periodic:
            return self._bonds[i - 1]
        return None if i == self.n else self._bonds[i - 1]

    def physindex(self, site):
        return self._phys[_site_id(site) - 1]

    def bond_index(self, s1, s2):
        """``inds(tn; bond=(s1, s2))``: the shared index, or None when not adjacent."""
        a, b = sorted((_site_id(s1), _site_id(s2)))
        if self.periodic and (a, b) == (1, self.n) and self.n > 2:
            return self._bonds[self.n - 1]
        return self._bonds[a - 1] if b == a + 1 else None

    def index_size(self, name):
        if name in self._phys:
            return self.d
        b = self._bonds.index(name)
        return self.bond_dims()[b]

    def lambda_between(self, s1, s2):
        """``tensors(tn; between=(s1, s2))`` if it is a Lambda vector, else None."""
        a, b = sorted((_site_id(s1), _site_id(s2)))
        if b != a + 1:
            return None
        n = C.c_int()
        f = C.c_int()
        check(lib().qr_chain_has_lambda(self._h, a - 1, C.byref(f)))
        if not f.value:
            return None
        check(lib().qr_chain_get_lambda(self._h, a - 1, None, C.byref(n)))
        out = np.empty(n.value, dtype=np.float64)
        check(lib().qr_chain_get_lambda(self._h, a - 1, dptr(out), C.byref(n)))
        return out

    def set_lambda(self, bond, lam):
        lam = np.ascontiguousarray(lam, dtype=np.float64)
        check(lib().qr_chain_set_lambda(self._h, bond, dptr(lam), lam.size))

    def upload_site(self, site, array, order=("o", "l", "r")):
        """Overwrite a site tensor from host memory (same dims as the current site)."""
        order = _norm_order(order, "olr")
        buf = array if (isinstance(array, np.ndarray) and array.flags.f_contiguous
                        and array.dtype == np.complex128) else np.asfortranarray(array, dtype=np.complex128)
        check(lib().qr_chain_upload_site(self._h, _site_id(site) - 1, dptr(buf), "".join(order).encode()))

    def download_site(self, site, out, order=("o", "l", "r")):
        """Copy a site tensor into the preallocated Fortran-ordered complex128 array ``out``."""
        order = _norm_order(order, "olr")
        check(lib().qr_chain_download_site(self._h, _site_id(site) - 1, dptr(out), "".join(order).encode()))
        return out

    def site_array(self, site, order=("o", "l", "r")):
        """Site tensor in the reference layout (column-major, dims by ``order``)."""
        order = _norm_order(order, "olr")
        i = _site_id(site) - 1
        cl, d, cr = self.site_dims(site)
        dims = {"l": cl, "o": d, "r": cr}
        ends = not self.periodic
        sub = [x for x in order if not ends or not ((i == 0 and x == "l") or (i == self.n - 1 and x == "r"))]
        out = np.empty([dims[x] for x in sub], dtype=np.complex128, order="F")
        check(lib().qr_chain_download_site(self._h, i, dptr(out), "".join(order).encode()))
        return out

    def arrays(self, order=("o", "l", "r")):
        return [self.site_array(i + 1, order) for i in range(self.n)]

    def set_precision(self, mode):
        check(lib().qr_chain_set_precision(self._h, _choice(_PREC, mode, "precision")))

    def stream(self):
        p = C.c_void_p()
        check(lib().qr_chain_stream(self._h, C.byref(p)))
        return p.value

    def sync(self):
        check(lib().qr_chain_sync(self._h))

    def adjoint(self):
        """Bookkeeping of ``adjoint(::Chain)``: dual sites and virtual indices renamed with a
        trailing ' (src/Quantum.jl:100-115).  The tensors are not materialised: overlaps
        conjugate on the fly."""
        return AdjointChain(self)


class AdjointChain:
    def __init__(self, parent):
        self.parent = parent

    socket = State(dual=True)

    def sites(self):
        return [Site(i + 1, True) for i in range(self.parent.n)]

    def nsites(self):
        return self.parent.n

    def boundary(self):
        return self.parent.boundary()

    def leftindex(self, site):
        ix = self.parent.leftindex(_site_id(site))
        return None if ix is None else ix + "'"

    def rightindex(self, site):
        ix = self.parent.rightindex(_site_id(site))
        return None if ix is None else ix + "'"


# ---- constructors ---------------------------------------------------------------------------------
def MPS(arrays, order=("o", "l", "r")):
    """``MPS(arrays)`` (Chain.jl:18)."""
    return Chain.from_arrays(arrays, order)


def pMPS(arrays, order=("o", "l", "r")):
    """``pMPS(arrays)`` (Chain.jl:19): a periodic MPS."""
    return Chain.from_arrays_periodic(arrays, order)


class MPO:
    """Open-boundary MPO in device memory (``MPO(arrays)``, Chain.jl:20,133-172), dims in the
    reference's operator order ``(:o, :i, :l, :r)``; ends drop ``:l`` / ``:r``."""

    def __init__(self, arrays, order=("o", "i", "l", "r")):
        order = _norm_order(order, "oilr")
        n = len(arrays)
        arrays = [np.asarray(a) for a in arrays]
        if arrays[0].ndim != 3 or arrays[-1].ndim != 3 or any(a.ndim != 4 for a in arrays[1:-1]):
            raise AssertionError("MPO ends must have 3 dimensions and the rest 4")
        dims = []
        for i, a in enumerate(arrays):
            sub = [x for x in order if not ((i == 0 and x == "l") or (i == n - 1 and x == "r"))]
            dims.append(dict(zip(sub, a.shape)))
        d = dims[0]["o"]
        bond = [dims[i]["r"] for i in range(n - 1)]
        for i in range(n - 1):
            if dims[i + 1]["l"] != bond[i]:
                raise L.DimensionMismatch(f"MPO bond {i + 1} mismatch")
        h = C.c_void_p()
        check(lib().qr_mpo_create(n, d, (C.c_int * (n - 1))(*bond), C.byref(h)))
        self._h = h
        self.n, self.d = n, d
        self._bonds = list(bond)
        for i, a in enumerate(arrays):
            buf = np.asfortranarray(a, dtype=np.complex128)
            check(lib().qr_mpo_upload_site(h, i, dptr(buf), "".join(order).encode()))

    @classmethod
    def _from_handle(cls, h, n, d):
        w = cls.__new__(cls)
        w._h, w.n, w.d = h, n, d
        return w

    def sites(self):
        """Outputs ``Site(i)`` and inputs ``Site(i; dual=true)`` of every lane (Chain.jl:168-169)."""
        return [Site(i + 1) for i in range(self.n)] + [Site(i + 1, True) for i in range(self.n)]

    def nsites(self):
        return self.n

    def boundary(self):
        return Open()

    def site_array(self, i, order=("o", "i", "l", "r")):
        """Site ``i`` (0-based) in the reference layout (ends without ``:l`` / ``:r``)."""
        order = _norm_order(order, "oilr")
        shp = self._shape(i)
        sub = [x for x in order if not ((i == 0 and x == "l") or (i == self.n - 1 and x == "r"))]
        out = np.empty(tuple(shp[x] for x in sub), dtype=np.complex128, order="F")
        check(lib().qr_mpo_download_site(self._h, i, dptr(out), "".join(order).encode()))
        return out

    def arrays(self, order=("o", "i", "l", "r")):
        return [self.site_array(i, order) for i in range(self.n)]

    def _shape(self, i):
        if not hasattr(self, "_bonds"):
            # bond sizes from the sites' element counts would need the C ABI; the sampler and the
            # array constructor record them
            raise ArgumentError("MPO bond sizes unknown")
        b = self._bonds
        return {"o": self.d, "i": self.d, "l": 1 if i == 0 else b[i - 1], "r": 1 if i == self.n - 1 else b[i]}

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and L._lib is not None:
            try:
                L._lib.qr_mpo_free(h)
            except Exception:
                pass
            self._h = None


def sampler_bond_dims(n, chi, p=2, socket=State):
    """Bond dimensions of ``rand(Chain, Open, socket; n, p, χ)`` (Chain.jl:223-297)."""
    q = p if socket is State else p * p
    L_, R_ = [], []
    for i in range(1, n + 1):
        after_mid = i > n // 2
        m = (n + 1 - abs(2 * i - n - 1)) // 2
        l, r = min(chi, q ** (m - 1)), min(chi, q ** m)
        if n % 2 == 1 and i == n // 2 + 1:
            r = l
        elif after_mid:
            l, r = r, l
        L_.append(l)
        R_.append(r)
    return R_[: n - 1]


def rand(A, B, S, *, n, chi, p=2, eltype=np.float64, seed=0):
    """``rand(Chain, Open, State; n, p, χ, eltype)`` / ``rand(Chain, Open, Operator; ...)``
    (Chain.jl:223-297), generated on the device: the reference's bond pattern, uniform [0,1)
    entries with Gram-Schmidt orthonormalised rows, the first site normalised.  The stream of
    random numbers is the library's own (Philox-4x32-10 keyed by ``seed``), not Julia's."""
    if A is not Chain:
        raise ArgumentError("rand(A, B, S) builds a Chain")
    if B is not Open:
        raise ArgumentError("only Open chains have a sampler (as in the reference)")
    cplx = int(np.issubdtype(np.dtype(eltype), np.complexfloating))
    h = C.c_void_p()
    if S is State:
        check(lib().qr_chain_random(int(n), int(p), int(chi), int(seed) & (2 ** 64 - 1), cplx, C.byref(h)))
        return Chain(h, int(n), int(p))
    if S is Operator:
        check(lib().qr_mpo_random(int(n), int(p), int(chi), int(seed) & (2 ** 64 - 1), cplx, C.byref(h)))
        w = MPO._from_handle(h, int(n), int(p))
        w._bonds = sampler_bond_dims(int(n), int(chi), int(p), Operator)
        return w
    raise ArgumentError("socket must be State or Operator")


# ---- canonical forms --------------------------------------------------------------------------------
def canonize_site_(psi: Chain, site, direction, method="qr"):
    """``canonize_site!`` (Chain.jl:339-376)."""
    direction = str(direction).lstrip(":")
    method = str(method).lstrip(":")
    if direction not in _DIR:
        raise ArgumentError(f"Unknown direction=:{direction}")
    if method not in _METHOD:
        raise ArgumentError(f"Unknown factorization method=:{method}")
    check(lib().qr_canonize_site(psi._h, _site_id(site) - 1, _DIR[direction], _METHOD[method]))
    return psi


def canonize_site(psi, site, direction, method="qr"):
    return canonize_site_(psi.copy(), site, direction, method)


def canonize_(psi: Chain):
    """``canonize!`` to the Vidal form (Chain.jl:469-497)."""
    check(lib().qr_canonize(psi._h))
    return psi


def canonize(psi):
    return canonize_(psi.copy())


def mixed_canonize_(psi: Chain, center):
    """``mixed_canonize!`` (Chain.jl:509-524)."""
    check(lib().qr_mixed_canonize(psi._h, _site_id(center) - 1))
    return psi


def mixed_canonize(psi, center):
    return mixed_canonize_(psi.copy(), center)


def normalize_(psi: Chain, root, p=2):
    """``normalize!(::Chain, ::Site; p)`` (Chain.jl:532-536): mixed-canonical around ``root``, then
    the Lambda between sites root - 1 and root divided by its p-norm (p = 2 on the device; other
    p re-scale that Lambda on the host)."""
    if p == 2:
        check(lib().qr_normalize(psi._h, _site_id(root) - 1))
        return psi
    mixed_canonize_(psi, root)
    r = _site_id(root)
    lam = psi.lambda_between(r - 1, r)
    psi.set_lambda(r - 2, lam / np.linalg.norm(lam, p))
    return psi


def contract_between_(psi: Chain, site1, site2, direction="left", delete_lambda=True):
    """``contract!(::Chain, Val(:between), site1, site2; direction, delete_Λ)`` (Chain.jl:309-333)."""
    direction = str(direction).lstrip(":")
    if direction not in _DIR:
        raise ArgumentError(f"Unknown direction=:{direction}")
    check(lib().qr_contract_between(psi._h, _site_id(site1) - 1, _site_id(site2) - 1, _DIR[direction],
                                    int(bool(delete_lambda))))
    return psi


def contract_between(psi, site1, site2, direction="left", delete_lambda=True):
    return contract_between_(psi.copy(), site1, site2, direction, delete_lambda)


def canonicality_error(psi: Chain, site, side):
    e = C.c_double()
    check(lib().qr_canonicality_error(psi._h, _site_id(site) - 1, _choice(_DIR, side, "direction"), C.byref(e)))
    return e.value


def isleftcanonical(psi: Chain, site, atol=1e-12):
    """``isleftcanonical`` (Chain.jl:424-440): ||A^H A - I||_F <= atol."""
    return canonicality_error(psi, site, "left") <= atol


def isrightcanonical(psi: Chain, site, atol=1e-12):
    """``isrightcanonical`` (Chain.jl:442-458)."""
    return canonicality_error(psi, site, "right") <= atol


def truncate_(psi: Chain, bond, threshold=None, maxdim=None):
    """``truncate!`` (Chain.jl:390-422).  A maxdim below 1 keeps nothing, as ``1:min(dim,
    maxdim)`` is empty there: the bond is sliced to size 0."""
    s1, s2 = (_site_id(s) for s in bond)
    th = float("nan") if threshold is None else float(threshold)
    md = -1 if maxdim is None else max(0, int(maxdim))  # -1 tells the C ABI "no maxdim"
    check(lib().qr_truncate(psi._h, s1 - 1, s2 - 1, th, md), bond=tuple(bond))
    return psi


def truncate(psi, bond, threshold=None, maxdim=None):
    return truncate_(psi.copy(), bond, threshold, maxdim)


# ---- gates ----------------------------------------------------------------------------------------------
def evolve_(psi: Chain, gate: Dense, threshold=None, maxdim=None, iscanonical=False, renormalize=False):
    """``evolve!`` (Chain.jl:543-661)."""
    lanes = validate_gate(psi.n, gate)
    m = np.ascontiguousarray(gate.matrix(lanes))
    if len(lanes) == 1:
        check(lib().qr_evolve_1site(psi._h, lanes[0] - 1, dptr(m)))
    else:
        th = float("nan") if threshold is None else float(threshold)
        md = -1 if maxdim is None else max(0, int(maxdim))  # below 1: the bond is sliced to size 0
        check(lib().qr_evolve_2site(psi._h, lanes[0] - 1, dptr(m), th, md, int(bool(iscanonical)),
                                    int(bool(renormalize))))
    return psi


def evolve_layer_(psi: Chain, gates, threshold=None, maxdim=None, iscanonical=False, renormalize=False, lanes=0):
    """A layer of two-site gates on disjoint site pairs: the same result as ``evolve!`` of each
    gate in turn (Chain.jl:543-661), with `lanes` gates at a time on their own streams (0: the
    library's default)."""
    sites, mats = [], []
    for g in gates:
        ls = validate_gate(psi.n, g)
        if len(ls) != 2:
            raise ArgumentError("evolve_layer_ takes two-site gates")
        sites.append(ls[0] - 1)
        mats.append(np.ascontiguousarray(g.matrix(ls)).ravel())
    k = len(sites)
    packed = np.ascontiguousarray(np.concatenate(mats) if mats else np.zeros(1, dtype=np.complex128))
    th = float("nan") if threshold is None else float(threshold)
    md = -1 if maxdim is None else max(0, int(maxdim))
    check(lib().qr_evolve_layer(psi._h, k, (C.c_int * max(k, 1))(*sites), dptr(packed), th, md,
                                int(bool(iscanonical)), int(bool(renormalize)), int(lanes)))
    return psi


# ---- contractions ---------------------------------------------------------------------------------------
def overlap(a, b):
    """``overlap(a, b)`` = <b|a> (Chain.jl:740-748); one side may be a ``Product``, converted to a
    chain with bonds of size 1 (``overlap(::Product, ::Chain)``, Chain.jl:751-752)."""
    if isinstance(a, Product) and isinstance(b, Chain):
        a = a.to_chain()
    elif isinstance(b, Product) and isinstance(a, Chain):
        b = b.to_chain()
    if not isinstance(a, Chain) or not isinstance(b, Chain):
        raise ArgumentError("overlap needs two Chains, or a Chain and a Product")
    out = np.zeros(2)
    check(lib().qr_overlap(a._h, b._h, dptr(out)))
    return complex(out[0], out[1])


def norm(psi: Chain, p=2):
    """``LinearAlgebra.norm(::Ansatz)`` (Ansatz.jl:101-109)."""
    if p != 2:
        raise ArgumentError("only L2-norm is implemented yet")
    out = C.c_double()
    check(lib().qr_norm(psi._h, C.byref(out)))
    return out.value


def expect(psi: Chain, observables):
    """``expect(psi, observables)`` (Chain.jl:724-735): the unnormalised
    <psi| O_k ... O_1 |psi>, observables applied in list order."""
    firsts, nls, mats = [], [], []
    for g in observables:
        lanes = validate_gate(psi.n, g)
        firsts.append(lanes[0] - 1)
        nls.append(len(lanes))
        mats.append(np.ascontiguousarray(g.matrix(lanes)).ravel())
    k = len(firsts)
    packed = np.ascontiguousarray(np.concatenate(mats) if mats else np.zeros(1, dtype=np.complex128))
    out = np.zeros(2)
    check(lib().qr_expect(psi._h, k, (C.c_int * max(k, 1))(*firsts), (C.c_int * max(k, 1))(*nls),
                          dptr(packed), dptr(out)))
    return complex(out[0], out[1])


def mpo_expect(psi: Chain, h: MPO):
    """<psi|H|psi> = contract(merge(Quantum(psi), Quantum(H), Quantum(psi)')) (src/Quantum.jl:330-348)."""
    out = np.zeros(2)
    check(lib().qr_mpo_expect(psi._h, h._h, dptr(out)))
    return complex(out[0], out[1])


class PinnedArray:
    """Page-locked host array (cudaHostAlloc), Fortran-ordered complex128 by default."""

    def __init__(self, shape, dtype=np.complex128):
        nbytes = int(np.prod(shape)) * np.dtype(dtype).itemsize
        self._p = C.c_void_p()
        check(lib().qr_host_alloc(nbytes, C.byref(self._p)))
        raw = (C.c_char * nbytes).from_address(self._p.value)
        self.array = np.frombuffer(raw, dtype=dtype).reshape(shape, order="F")

    def __del__(self):
        p = getattr(self, "_p", None)
        if p is not None and p.value and L._lib is not None:
            L._lib.qr_host_free(p)
            self._p = None


def probe_peak(kind):
    """Peak TFLOP/s of one pipe measured now: 'dmma' (FP64 tensor), 'ffma' (FP32), 'dfma' (FP64)."""
    k = {"dmma": 0, "ffma": 1, "dfma": 2}[kind]
    out = C.c_double()
    check(lib().qr_probe_peak(k, C.byref(out)))
    return out.value


PROF_KINDS = {"zgemm_dmma": 0, "jacobi_fp64": 1, "jacobi_fp32": 2, "householder_qr": 3, "env_mix": 4,
              "zgemm_tc_bf16x3": 5, "jacobi_df": 6,
              "zgemm_df": 7}


def prof_enable(on=True):
    check(lib().qr_prof_enable(int(bool(on))))


def prof_read(kind):
    ms, fl, by = C.c_double(), C.c_double(), C.c_double()
    n = C.c_uint64()
    check(lib().qr_prof_read(PROF_KINDS[kind], C.byref(ms), C.byref(n), C.byref(fl), C.byref(by)))
    return {"ms": ms.value, "launches": int(n.value), "flops": fl.value, "bytes": by.value}


def set_device(i):
    check(lib().qr_set_device(int(i)))


def zeros_chain(n, d=2):
    """``convert(Chain, zeros(Product, n))``: |0...0> with bonds of size 1."""
    from .random import zero_product_arrays

    return MPS(zero_product_arrays(n, d))


class Product:
    """``Product(arrays)`` of site vectors, a product state (src/Ansatz/Product.jl:17-31), on the
    host; ``to_chain()`` is ``convert(Chain, ::Product)`` (Chain.jl:174-183)."""

    def __init__(self, vectors):
        self.vectors = [np.asarray(v) for v in vectors]
        from .random import product_arrays

        self._arrays = product_arrays(self.vectors)  # validates

    def sites(self):
        return [Site(i + 1) for i in range(len(self.vectors))]

    def nsites(self):
        return len(self.vectors)

    def to_chain(self):
        return MPS(self._arrays)


def ones_chain(n, d=2):
    """``convert(Chain, ones(Product, n))``: |1...1> with bonds of size 1."""
    from .random import one_product_arrays

    return MPS(one_product_arrays(n, d))


def device_count():
    c = C.c_int()
    rc = lib().qr_device_count(C.byref(c))
    return c.value if rc == 0 else 0

