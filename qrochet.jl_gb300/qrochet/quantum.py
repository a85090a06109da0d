"""The lane queries every ``Quantum`` network answers, forwarded to every ``Ansatz``
(src/Quantum.jl:25,118-143,228-239; src/Ansatz.jl:19-33): which sites are inputs (dual) and which
are outputs, and whether the network is a scalar, a state or an operator.  Host bookkeeping on
anything with a ``sites`` list or method (``Chain``, its adjoint, ``MPO``, ``Dense``)."""
from __future__ import annotations

from .dense import Operator, Scalar, State


def isdual(site):
    """``isdual(::Site)`` (src/Quantum.jl:25)."""
    return site.dual


def sites(q):
    """The network's sites, outputs and inputs (``sites(::Quantum)``)."""
    s = q.sites
    return list(s() if callable(s) else s)


def nsites(q):
    return len(sites(q))


def inputs(q):
    """Dual sites, sorted by lane (src/Quantum.jl:136)."""
    return sorted(s for s in sites(q) if isdual(s))


def outputs(q):
    """Non-dual sites, sorted by lane (src/Quantum.jl:143)."""
    return sorted(s for s in sites(q) if not isdual(s))


def ninputs(q):
    return len(inputs(q))


def noutputs(q):
    return len(outputs(q))


def lanes(q):
    """The lanes as non-dual sites, each once, in the order first seen over the inputs and then
    the outputs (src/Quantum.jl:175)."""
    out = []
    for s in inputs(q) + outputs(q):
        lane = s.adjoint() if isdual(s) else s
        if lane not in out:
            out.append(lane)
    return out


def nlanes(q):
    return len(lanes(q))


def socket(q):
    """``Scalar()`` without sites, ``State()`` with outputs only, ``State(dual=true)`` with inputs
    only, else ``Operator()`` (src/Quantum.jl:228-239)."""
    s = sites(q)
    if not s:
        return Scalar()
    if not any(isdual(x) for x in s):
        return State()
    if all(isdual(x) for x in s):
        return State(dual=True)
    return Operator()
