"""``Site`` and the ``site"..."`` string form (src/Quantum.jl:10-43), and the global index-name
counter (src/Utils.jl:3-7)."""
from __future__ import annotations

import itertools
import re
import threading
from dataclasses import dataclass


@dataclass(frozen=True, order=False)
class Site:
    """A physical lane; ``dual=True`` marks an input (``Site(id; dual)``).  1-based id."""

    id: int
    dual: bool = False

    def adjoint(self):
        return Site(self.id, not self.dual)

    def __lt__(self, other):  # Base.isless(a::Site, b::Site) = id(a) < id(b)
        return self.id < other.id

    def __repr__(self):
        return f"{self.id}{chr(39) if self.dual else ''}"


_SITE_RE = re.compile(r"^(\d+,)*\d+('?)$")


def site(text: str) -> Site:
    """``site"3"`` / ``site"3'"``."""
    m = _SITE_RE.match(text)
    if m is None:
        raise ValueError(f"Invalid site string: {text}")
    ids = [int(x) for x in re.findall(r"\d+", text)]
    if len(ids) != 1:
        raise ValueError("only one-dimensional sites are supported on a Chain")
    return Site(ids[0], text.endswith("'"))


_counter = itertools.count(1)
_counter_lock = threading.Lock()
_RESET_AT = 135000


def nextindex() -> str:
    """Fresh index name from a global counter that wraps at 135000 like the reference's."""
    global _counter
    with _counter_lock:
        k = next(_counter)
        if k >= _RESET_AT:
            _counter = itertools.count(2)
            k = 1
    return f"i{k}"
