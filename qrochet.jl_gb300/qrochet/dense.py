"""``Dense`` gates (src/Ansatz/Dense.jl:21-34) and the checks ``evolve!`` runs on them
(src/Ansatz/Chain.jl:552-581).  Pure host logic: it turns a gate into the row-major matrix
M[(o_1..o_k), (i_1..i_k)] (left lane slowest) that the C ABI takes."""
from __future__ import annotations

import numpy as np

from ._lib import ArgumentError
from .site import Site


class Scalar:
    """Socket of a network with no open sites (src/Quantum.jl:203-208)."""

    def __eq__(self, other):
        return isinstance(other, Scalar)

    def __hash__(self):
        return hash("Scalar")

    def __repr__(self):
        return "Scalar()"


class State:
    """Socket of a state; ``dual=True``: a state on dual sites only, such as an adjoint
    (src/Quantum.jl:210-217)."""

    def __init__(self, dual=False):
        self.dual = bool(dual)

    def __eq__(self, other):
        return isinstance(other, State) and other.dual == self.dual

    def __hash__(self):
        return hash(("State", self.dual))

    def __repr__(self):
        return "State(dual=true)" if self.dual else "State()"


class Operator:
    """Socket of an operator (src/Quantum.jl:219-224)."""

    def __eq__(self, other):
        return isinstance(other, Operator)

    def __hash__(self):
        return hash("Operator")

    def __repr__(self):
        return "Operator()"


class Dense:
    """``Dense(Operator(), array; sites)``: array dims map to ``sites`` in order."""

    def __init__(self, socket, array, sites):
        array = np.asarray(array)
        if array.ndim == 0 or any(s <= 1 for s in array.shape):
            raise AssertionError("Dense arrays need every dim > 1")
        sites = tuple(sites)
        if len(sites) != array.ndim:
            raise AssertionError("length(sites) must equal ndims(array)")
        self.socket = socket
        self.array = array.astype(np.complex128)
        self.sites = sites

    def inputs(self):
        return [s for s in self.sites if s.dual]

    def outputs(self):
        return [s for s in self.sites if not s.dual]

    def nlanes(self):
        return len({s.id for s in self.sites})

    def matrix(self, lanes):
        """M[(o_1..o_k), (i_1..i_k)] for the ordered lanes (1-based ids)."""
        k = len(lanes)
        ax_o = [self.sites.index(Site(l, False)) for l in lanes]
        ax_i = [self.sites.index(Site(l, True)) for l in lanes]
        t = np.transpose(self.array, ax_o + ax_i)
        d = t.shape[0]
        return np.ascontiguousarray(t.reshape(d ** k, d ** k))


def gate_from_matrix(m, lanes):
    """Dense operator from a d^k x d^k matrix with the first lane slowest (helper)."""
    m = np.asarray(m, dtype=np.complex128)
    k = len(lanes)
    d = int(round(m.shape[0] ** (1.0 / k)))
    arr = m.reshape((d,) * (2 * k))
    sites = [Site(l) for l in lanes] + [Site(l, True) for l in lanes]
    return Dense(Operator(), arr, sites)


def validate_gate(nsites, gate):
    """The checks of ``evolve!`` (Chain.jl:552-581); returns the sorted lanes (1-based)."""
    if not isinstance(gate, Dense):
        raise ArgumentError("gate must be a Dense operator")
    ins, outs = gate.inputs(), gate.outputs()
    if not ins or not outs:
        raise ArgumentError("Gate must be an operator")
    if {s.adjoint() for s in ins} != set(outs):
        raise ArgumentError(f"Gate inputs ({ins}) and outputs ({outs}) must be the same")
    chain = {Site(i + 1) for i in range(nsites)}
    if not {s.adjoint() for s in ins} <= chain:
        raise ArgumentError(f"Gate inputs ({ins}) must be a subset of the TN sites")
    lanes = sorted(s.id for s in outs)
    if len(lanes) > 2:
        raise ArgumentError(f"Invalid number of lanes {len(lanes)}, maximum is 2")
    if len(lanes) == 2 and lanes[1] != lanes[0] + 1:
        raise ArgumentError("Gate lanes must be contiguous")
    return lanes
