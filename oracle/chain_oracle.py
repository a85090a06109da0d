"""CPU oracle for the Chain (MPS/MPO) hot path -- TEST INFRASTRUCTURE ONLY.

This module checks the library and is never part of it: only ``tests/``, ``__graft_entry__.smoke()``
and the ``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` may import it.

It restates, in NumPy on LAPACK, the semantics of Qrochet.jl's ``src/Ansatz/Chain.jl`` (v0.1.2)
for open-boundary chains, and for periodic ones the operations the reference does not restrict to
``::Open`` (construction, evolve!, truncate!, overlap, expect).  Qrochet itself is Julia, and its arithmetic lives in the un-vendored
packages Tenet.jl (compat 0.6) and Muscle.jl (compat 0.2) on top of Julia ``LinearAlgebra``:
``qr`` = LAPACK geqrf + ungqr (thin Q) and ``svd`` = LAPACK gesdd (thin, descending singular
values).  NumPy's ``linalg.qr(mode="reduced")`` and ``linalg.svd(full_matrices=False)`` call the
same LAPACK routines, so the factorisations here are those the reference gets.

Representation (same index grouping as the reference, different stride order):
  * ``sites[i]`` is a complex128 array of shape ``(chi_l, d, chi_r)``; the open ends carry a
    bond of size 1 (the reference drops the ``:l`` index of site 1 and ``:r`` of site n,
    ``Chain.jl:74-93``).
  * ``lam[i]`` is ``None`` or the real vector Lambda held as a separate hyperindex tensor on the
    bond between sites i and i+1 (0-based), exactly the tensors that ``canonize_site!`` with
    ``method=:svd`` and ``svd!`` in ``evolve_2site!`` leave on a bond (``Chain.jl:338,645``).
  * ``contract!(tn, bond)`` contracts every tensor carrying the bond index, so merging across a
    bond always absorbs that bond's Lambda (``Chain.jl:372,616``).

Parity pinning: the reference cannot be run here (no Julia, Tenet/Muscle absent) and its tests
hold no golden vectors.  This oracle is pinned against every property the reference's own
tests assert (``test/Ansatz/Chain_test.jl``) and against exact state-vector known answers; see
``tests/test_oracle_reference_properties.py`` and ``tests/test_oracle_known_answers.py``.
"""
from __future__ import annotations

import copy as _copy
from dataclasses import dataclass, field

import numpy as np


class ArgumentError(ValueError):
    """Julia ``ArgumentError``."""


class MissingSchmidtCoefficientsException(RuntimeError):
    """Qrochet ``MissingSchmidtCoefficientsException`` (``src/Ansatz.jl:91-99``)."""

    def __init__(self, bond):
        super().__init__(f"Can't access the spectrum on bond {bond}")
        self.bond = bond


# ---------------------------------------------------------------------------------------------
# Chain container
# ---------------------------------------------------------------------------------------------
@dataclass
class OChain:
    """MPS: ``sites[i]`` shaped (chi_l, d, chi_r), ``lam[i]`` on bond (i, i+1).  Open boundary by
    default (end bonds of size 1); ``periodic=True`` closes site n's right bond onto site 1's
    left bond (``Chain(State(), Periodic(), arrays)``, ``Chain.jl:36-62``)."""

    sites: list
    lam: list = field(default=None)
    periodic: bool = False

    def __post_init__(self):
        n = len(self.sites)
        if self.lam is None:
            self.lam = [None] * (n - 1)
        assert len(self.lam) == n - 1
        for i, a in enumerate(self.sites):
            assert a.ndim == 3, "site tensors are (chi_l, d, chi_r)"
            if i > 0:
                assert self.sites[i - 1].shape[2] == a.shape[0], f"bond {i - 1} mismatch"
        if self.periodic:
            assert self.sites[-1].shape[2] == self.sites[0].shape[0], "closing bond mismatch"
        else:
            assert self.sites[0].shape[0] == 1 and self.sites[-1].shape[2] == 1

    @property
    def n(self):
        return len(self.sites)

    def bond_dims(self):
        """Sizes of the n-1 virtual bonds (n for a periodic chain: the last closes the ring)."""
        return [a.shape[2] for a in (self.sites if self.periodic else self.sites[:-1])]

    def lambda_flags(self):
        """Which bonds hold a Lambda hyperindex tensor."""
        return [lm is not None for lm in self.lam]

    def ntensors(self):
        """``length(tensors(tn))``: sites plus the Lambda vectors."""
        return self.n + sum(self.lambda_flags())

    def copy(self):
        return _copy.deepcopy(self)


def from_reference_arrays_periodic(arrays, order=("o", "l", "r")):
    """``pMPS(arrays)`` / ``Chain(State(), Periodic(), arrays; order)`` (``Chain.jl:36-62``):
    every array is 3-d."""
    order = tuple(order)
    if set(order) != {"o", "l", "r"} or len(order) != 3:
        raise ArgumentError("order must be a permutation of (o, l, r)")
    sites = []
    for a in arrays:
        a = np.asarray(a, dtype=np.complex128)
        assert a.ndim == 3, "All arrays must have 3 dimensions"
        sites.append(np.ascontiguousarray(np.transpose(a, (order.index("l"), order.index("o"), order.index("r")))))
    return OChain(sites, periodic=True)


def from_reference_arrays(arrays, order=("o", "l", "r")):
    """``MPS(arrays)`` / ``Chain(State(), Open(), arrays; order)`` (``Chain.jl:64-100``).

    ``arrays`` follow the reference's dims: ends are 2-d (the ``:l`` of site 1 and ``:r`` of
    site n are absent), interior sites are 3-d, dims named by ``order``.
    """
    order = tuple(order)
    if set(order) != {"o", "l", "r"} or len(order) != 3:
        raise ArgumentError("order must be a permutation of (o, l, r)")
    n = len(arrays)
    sites = []
    for i, a in enumerate(arrays):
        a = np.asarray(a, dtype=np.complex128)
        if i == 0:
            sub = tuple(x for x in order if x != "l")
            assert a.ndim == 2, "First array must have 2 dimensions"
            a = np.transpose(a, (sub.index("o"), sub.index("r")))[None, :, :]
        elif i == n - 1:
            sub = tuple(x for x in order if x != "r")
            assert a.ndim == 2, "Last array must have 2 dimensions"
            a = np.transpose(a, (sub.index("l"), sub.index("o")))[:, :, None]
        else:
            assert a.ndim == 3, "All arrays must have 3 dimensions"
            a = np.transpose(a, (order.index("l"), order.index("o"), order.index("r")))
        sites.append(np.ascontiguousarray(a))
    return OChain(sites)


# ---------------------------------------------------------------------------------------------
# Small helpers restating Julia / LAPACK behaviour
# ---------------------------------------------------------------------------------------------
def _pinv_diag(lam, atol):
    """``diag(pinv(Diagonal(lam), atol=atol))`` of Julia LinearAlgebra (atol>0 => rtol=0):
    entries with |x| > atol are inverted, the rest become 0."""
    out = np.zeros_like(lam, dtype=np.float64)
    mask = np.abs(lam) > atol
    out[mask] = 1.0 / lam[mask]
    return out


def _require_open(ch):
    """Canonical forms dispatch on ``::Open`` only (``Chain.jl:339,469,509``)."""
    if ch.periodic:
        raise ArgumentError("canonical forms are defined for Open chains only")


def _thin_qr(m):
    q, r = np.linalg.qr(m, mode="reduced")
    return q, r


def _thin_svd(m):
    u, s, vh = np.linalg.svd(m, full_matrices=False)
    return u, s, vh


def _scale_left(a, v):
    """Multiply a site tensor along its left bond (``contract(A, Lambda; dims=())``)."""
    return a * v[:, None, None]


def _scale_right(a, v):
    return a * v[None, None, :]


# ---------------------------------------------------------------------------------------------
# contract!(::Chain, Val(:between)) -- Chain.jl:309-333
# ---------------------------------------------------------------------------------------------
def contract_between_(ch: OChain, site1: int, site2: int, direction="left", delete_lambda=True):
    """Absorb the Lambda of the bond site1 and site2 share into site2 (``:right``) or site1
    (``:left``) (Chain.jl:309-333).  ``tensors(tn; between)`` (Ansatz.jl:78-89) asserts two
    different sites of the chain and finds nothing when they share no bond, which leaves the chain
    as it is; the two sites may come in either order."""
    if not (0 <= site1 < ch.n and 0 <= site2 < ch.n):
        raise AssertionError("Site not found")
    if site1 == site2:
        raise AssertionError("Sites must be different")
    if abs(site2 - site1) != 1:
        return ch
    b = min(site1, site2)
    lm = ch.lam[b]
    if lm is None:
        return ch
    # the bond is site1's right index when site1 is the left site of the pair, else its left index
    if direction == "right":
        ch.sites[site2] = (_scale_left if site2 > site1 else _scale_right)(ch.sites[site2], lm)
    elif direction == "left":
        ch.sites[site1] = (_scale_right if site2 > site1 else _scale_left)(ch.sites[site1], lm)
    else:
        raise ArgumentError(f"Unknown direction=:{direction}")
    if delete_lambda:
        ch.lam[b] = None
    return ch


# ---------------------------------------------------------------------------------------------
# canonize_site! -- Chain.jl:339-376
# ---------------------------------------------------------------------------------------------
def canonize_site_(ch: OChain, site: int, direction: str, method: str = "qr"):
    """One QR/SVD step across a bond.

    ``:right``: A[(l,o) x r] = Q R (or U S Vh); Q/U stays, R (Vh) is contracted into site+1
    together with any Lambda already on that bond, S becomes that bond's Lambda.
    ``:left`` mirrors it with A[(o,r) x l] and site-1.
    """
    _require_open(ch)
    n = ch.n
    if direction == "left":
        if site == 0:
            raise ArgumentError("Cannot right-canonize left-most tensor")
    elif direction == "right":
        if site == n - 1:
            raise ArgumentError("Cannot left-canonize right-most tensor")
    else:
        raise ArgumentError(f"Unknown direction=:{direction}")
    if method not in ("qr", "svd"):
        raise ArgumentError(f"Unknown factorization method=:{method}")

    a = ch.sites[site]
    cl, d, cr = a.shape
    if direction == "right":
        m = a.reshape(cl * d, cr)
        if method == "qr":
            q, r = _thin_qr(m)
            s = None
        else:
            q, s, r = _thin_svd(m)
        k = q.shape[1]
        ch.sites[site] = q.reshape(cl, d, k)
        nxt = ch.sites[site + 1]
        if ch.lam[site] is not None:  # contract!(tn, virtualind) also eats the old Lambda
            nxt = _scale_left(nxt, ch.lam[site])
        ch.sites[site + 1] = np.einsum("kb,bor->kor", r, nxt, optimize=True)
        ch.lam[site] = None if s is None else s.astype(np.float64)
    else:
        m = np.transpose(a, (1, 2, 0)).reshape(d * cr, cl)
        if method == "qr":
            q, r = _thin_qr(m)
            s = None
        else:
            q, s, r = _thin_svd(m)
        k = q.shape[1]
        ch.sites[site] = np.ascontiguousarray(np.transpose(q.reshape(d, cr, k), (2, 0, 1)))
        prv = ch.sites[site - 1]
        if ch.lam[site - 1] is not None:
            prv = _scale_right(prv, ch.lam[site - 1])
        ch.sites[site - 1] = np.einsum("lob,kb->lok", prv, r, optimize=True)
        ch.lam[site - 1] = None if s is None else s.astype(np.float64)
    return ch


# ---------------------------------------------------------------------------------------------
# truncate! -- Chain.jl:390-422
# ---------------------------------------------------------------------------------------------
def truncate_(ch: OChain, bond, threshold=None, maxdim=None):
    """Keep ``1:min(dim, maxdim)`` filtered by ``|lambda| > threshold`` (default 1e-16)."""
    s1, s2 = bond
    if s2 != s1 + 1 or not (0 <= s1 < ch.n - 1):
        raise ArgumentError(f"Invalid bond {bond}")
    lm = ch.lam[s1]
    if lm is None:
        raise MissingSchmidtCoefficientsException(bond)
    dim = lm.shape[0]
    extent = np.arange(min(dim, maxdim) if maxdim is not None else dim)
    if threshold is None:
        threshold = 1e-16
    extent = extent[np.abs(lm[extent]) > threshold]
    # an empty extent leaves a bond of size 0 (slice! with an empty range, Chain.jl:404-419)
    ch.sites[s1] = ch.sites[s1][:, :, extent]
    ch.sites[s2] = ch.sites[s2][extent, :, :]
    ch.lam[s1] = lm[extent]
    return ch


# ---------------------------------------------------------------------------------------------
# canonicality predicates -- Chain.jl:424-458
# ---------------------------------------------------------------------------------------------
def isleftcanonical(ch: OChain, site: int, atol=1e-12):
    a = ch.sites[site]
    m = a.reshape(-1, a.shape[2])
    g = m.conj().T @ m
    return np.linalg.norm(g - np.eye(g.shape[0])) <= atol


def isrightcanonical(ch: OChain, site: int, atol=1e-12):
    a = ch.sites[site]
    m = a.reshape(a.shape[0], -1)
    g = m @ m.conj().T
    return np.linalg.norm(g - np.eye(g.shape[0])) <= atol


# ---------------------------------------------------------------------------------------------
# canonize! (Vidal form) -- Chain.jl:469-497
# ---------------------------------------------------------------------------------------------
def canonize_(ch: OChain):
    _require_open(ch)
    n = ch.n
    for i in range(n - 1, 0, -1):  # right-to-left QR sweep
        canonize_site_(ch, i, "left", "qr")
    lams = []
    for i in range(n - 1):  # left-to-right SVD sweep, Lambda pushed right
        canonize_site_(ch, i, "right", "svd")
        lm = ch.lam[i]
        ch.lam[i] = None
        ch.sites[i + 1] = _scale_left(ch.sites[i + 1], lm)
        lams.append(lm)
    for i in range(1, n):  # Gamma_i = Lambda_{i-1}^+ A_i
        lm = lams[i - 1]
        ch.sites[i] = _scale_left(ch.sites[i], _pinv_diag(lm, 1e-64))
        ch.lam[i - 1] = lm
    return ch


# ---------------------------------------------------------------------------------------------
# mixed_canonize! / normalize! -- Chain.jl:509-536
# ---------------------------------------------------------------------------------------------
def mixed_canonize_(ch: OChain, center: int):
    _require_open(ch)
    n = ch.n
    for i in range(0, center):
        canonize_site_(ch, i, "right", "qr")
    for i in range(n - 1, center, -1):
        canonize_site_(ch, i, "left", "qr")
    canonize_site_(ch, center, "left", "svd")
    return ch


def normalize_(ch: OChain, root: int, p=2):
    """``normalize!(tn, root; p)`` (Chain.jl:532-536): mixed-canonical around ``root``, then the
    Lambda between sites root - 1 and root divided by its p-norm."""
    _require_open(ch)
    mixed_canonize_(ch, root)
    lm = ch.lam[root - 1]
    ch.lam[root - 1] = lm / np.linalg.norm(lm, p)
    return ch


# ---------------------------------------------------------------------------------------------
# Gates: Dense(Operator(), array; sites) -- src/Ansatz/Dense.jl:21-34
# ---------------------------------------------------------------------------------------------
@dataclass(frozen=True)
class OSite:
    """``Site(id; dual)`` with a 1-based id (``src/Quantum.jl:10-43``)."""

    id: int
    dual: bool = False

    def adjoint(self):
        return OSite(self.id, not self.dual)


@dataclass
class ODense:
    """A gate: array dims map to ``sites`` in order (dual sites are inputs)."""

    array: np.ndarray
    sites: tuple

    def inputs(self):
        return [s for s in self.sites if s.dual]

    def outputs(self):
        return [s for s in self.sites if not s.dual]


def gate_matrix(g: ODense, lanes):
    """Matrix M[(o_1..o_k), (i_1..i_k)] of a gate for the ordered lanes (1-based ids), with
    the first lane's index slowest (row-major over lanes)."""
    k = len(lanes)
    axes_out = [g.sites.index(OSite(l, False)) for l in lanes]
    axes_in = [g.sites.index(OSite(l, True)) for l in lanes]
    t = np.transpose(np.asarray(g.array, dtype=np.complex128), axes_out + axes_in)
    d = t.shape[0]
    return t.reshape(d ** k, d ** k)


def _validate_gate(ch: OChain, g: ODense):
    """Checks of ``evolve!`` (``Chain.jl:552-581``)."""
    ins, outs = g.inputs(), g.outputs()
    if not ins or not outs:
        raise ArgumentError("Gate must be an operator")
    if set(s.adjoint() for s in ins) != set(outs):
        raise ArgumentError("Gate inputs and outputs must be the same")
    chain_sites = {OSite(i + 1) for i in range(ch.n)}
    if not set(s.adjoint() for s in ins) <= chain_sites:
        raise ArgumentError("Gate inputs must be a subset of the TN sites")
    lanes = sorted(s.id for s in outs)
    if len(lanes) == 2 and lanes[1] != lanes[0] + 1:
        raise ArgumentError("Gate lanes must be contiguous")
    if len(lanes) > 2:
        raise ArgumentError(f"Invalid number of lanes {len(lanes)}, maximum is 2")
    return lanes


# ---------------------------------------------------------------------------------------------
# evolve! -- Chain.jl:543-661 (+ Vidal helpers 669-722)
# ---------------------------------------------------------------------------------------------
def evolve_(ch: OChain, g: ODense, threshold=None, maxdim=None, iscanonical=False,
            renormalize=False):
    lanes = _validate_gate(ch, g)
    if len(lanes) == 1:
        evolve_1site_(ch, lanes[0] - 1, gate_matrix(g, lanes))
    else:
        evolve_2site_(ch, lanes[0] - 1, gate_matrix(g, lanes), threshold, maxdim, iscanonical,
                      renormalize)
    return ch


def evolve_1site_(ch: OChain, site: int, g2):
    """``evolve_1site!`` (``Chain.jl:586-603``): A[l,o',r] = sum_o G[o',o] A[l,o,r]."""
    ch.sites[site] = np.einsum("po,lor->lpr", g2, ch.sites[site], optimize=True)
    return ch


def evolve_2site_(ch: OChain, sl: int, g4, threshold=None, maxdim=None, iscanonical=False,
                  renormalize=False):
    """``evolve_2site!`` on bond (sl, sl+1) with the 4x4 gate G[(o1',o2'),(o1,o2)]."""
    n = ch.n
    sr = sl + 1
    lam_prev = lam_next = None
    if iscanonical:  # contract_2sitewf! (Chain.jl:669-685)
        lam_prev = None if sl == 0 else ch.lam[sl - 1]
        lam_next = None if sl == n - 2 else ch.lam[sr]
        if lam_prev is not None:
            ch.sites[sl] = _scale_left(ch.sites[sl], lam_prev)
        if lam_next is not None:
            ch.sites[sr] = _scale_right(ch.sites[sr], lam_next)
    al, ar = ch.sites[sl], ch.sites[sr]
    if ch.lam[sl] is not None:
        al = _scale_right(al, ch.lam[sl])
    theta = np.einsum("lab,bcr->lacr", al, ar, optimize=True)
    d = theta.shape[1]
    g = g4.reshape(d, d, d, d)
    theta = np.einsum("pqac,lacr->lpqr", g, theta, optimize=True)
    cl, cr = theta.shape[0], theta.shape[3]
    u, s, vh = _thin_svd(theta.reshape(cl * d, d * cr))
    k = s.shape[0]
    ul = u.reshape(cl, d, k)
    vr = vh.reshape(k, d, cr)
    if iscanonical:  # unpack_2sitewf! (Chain.jl:693-722)
        if lam_prev is not None:
            ul = _scale_left(ul, _pinv_diag(lam_prev, 1e-32))
        if lam_next is not None:
            vr = _scale_right(vr, _pinv_diag(lam_next, 1e-32))
    ch.sites[sl], ch.sites[sr] = ul, vr
    ch.lam[sl] = s.astype(np.float64)
    if threshold is not None or maxdim is not None:
        truncate_(ch, (sl, sr), threshold=threshold, maxdim=maxdim)
        if renormalize and iscanonical:
            ch.lam[sl] = ch.lam[sl] / np.linalg.norm(ch.lam[sl])
        elif renormalize:
            normalize_(ch, sl)
    return ch


# ---------------------------------------------------------------------------------------------
# Contractions: overlap / norm / expect / MPO expectation -- Chain.jl:724-748, Ansatz.jl:101-109
# ---------------------------------------------------------------------------------------------
def _with_lambdas(ch: OChain):
    """Site tensors with every bond Lambda absorbed to the right (same contracted network)."""
    out = [a for a in ch.sites]
    for i, lm in enumerate(ch.lam):
        if lm is not None:
            out[i] = _scale_right(out[i], lm)
    return out


def overlap(a: OChain, b: OChain):
    """``overlap(a, b)`` = contract(a with b'), i.e. <b|a> (b conjugated)."""
    if a.n != b.n:
        raise ArgumentError("Ansatzes must have the same sites")
    if a.periodic or b.periodic:  # ring: contract the state vectors (oracle sizes are small)
        return np.vdot(to_statevector(b), to_statevector(a))
    sa, sb = _with_lambdas(a), _with_lambdas(b)
    if any(x.size == 0 for x in sa + sb):  # a size-0 bond: the contraction is an empty sum
        return 0j
    env = np.ones((1, 1), dtype=np.complex128)  # env[ket, bra]
    for x, y in zip(sa, sb):
        env = np.einsum("ab,aor,bos->rs", env, x, y.conj(), optimize=True)
    return env[0, 0]


def norm(ch: OChain):
    """``LinearAlgebra.norm(::Ansatz)`` = |sqrt(<psi|psi>)| (``Ansatz.jl:101-109``)."""
    return abs(np.sqrt(overlap(ch, ch)))


def expect(psi: OChain, observables):
    """``expect`` (``Chain.jl:724-735``): phi = copy(psi); evolve! every observable (no
    truncation); then contract phi with psi' -> the unnormalised <psi|O_k...O_1|psi>."""
    phi = psi.copy()
    for g in observables:
        evolve_(phi, g)
    return overlap(phi, psi)


def mpo_expect(psi: OChain, w_sites):
    """<psi|H|psi> for an MPO given as tensors W[wl, o, i, wr] (contract of
    merge(Quantum(psi), Quantum(H), Quantum(psi)'), ``src/Quantum.jl:330-348``)."""
    s = _with_lambdas(psi)
    env = np.ones((1, 1, 1), dtype=np.complex128)  # env[ket, w, bra]
    for a, w in zip(s, w_sites):
        env = np.einsum("awb,aic,woix,bod->cxd", env, a, w, a.conj(), optimize=True)
    return env[0, 0, 0]


def to_statevector(ch: OChain):
    """Full contraction to a dense vector indexed (o_1, ..., o_n), o_1 slowest; a periodic
    chain is traced over its closing bond."""
    s = _with_lambdas(ch)
    if ch.periodic:
        v = s[0]  # (a0, d, chi_r): the closing index a0 rides along
        for a in s[1:]:
            v = np.einsum("kxb,bor->kxor", v, a, optimize=True).reshape(v.shape[0], -1, a.shape[2])
        return np.einsum("kxk->x", v, optimize=True)
    v = s[0][0]  # (d, chi_r)
    for a in s[1:]:
        v = np.einsum("xb,bor->xor", v, a, optimize=True).reshape(-1, a.shape[2])
    return v[:, 0]


def mpo_to_dense(w_sites):
    """Dense operator H[(o_1..o_n), (i_1..i_n)] of an MPO W[wl, o, i, wr]."""
    h = w_sites[0][0]  # (o, i, wr)
    h = h.reshape(h.shape[0], h.shape[1], h.shape[2])
    for w in w_sites[1:]:
        h = np.einsum("OIw,woix->OoIix", h, w, optimize=True)
        h = h.reshape(h.shape[0] * h.shape[1], h.shape[2] * h.shape[3], h.shape[4])
    return h[:, :, 0]
