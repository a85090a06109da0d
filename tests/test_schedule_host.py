"""Host-side schedule of the masked Jacobi sweeps (greedy colouring of the marked pairs), on CPU.

A masked sweep rotates only the pairs a Gram test marked; the host lists them colour class by
colour class and gives each listed pair its ordinal on its two columns (blocks), which the sweep
kernels wait on.  These checks hold for any mask: every marked pair is listed once, the ordinals
are the pair's position among the listed pairs of each column in list order (so a pair only ever
waits on pairs listed before it), the number of classes is at most 2 d - 1 for the largest degree
d, and with flags every flagged vertex is met by a `full` item.
"""
import ctypes as C

import numpy as np
import pytest

from qrochet import _lib


def schedule(mask_pairs, nv, flags=None):
    mw = (nv + 31) // 32
    mask = np.zeros(nv * mw, dtype=np.uint32)
    for p, q in mask_pairs:
        mask[p * mw + q // 32] |= np.uint32(1 << (q % 32))
    flag = None if flags is None else np.asarray(flags, dtype=np.uint32)
    cap = nv * (nv - 1) // 2
    items = np.zeros(max(cap, 1), dtype=np.uint32)
    ord_ = np.zeros(max(2 * cap, 2), dtype=np.uint32)
    listed = C.c_long()
    classes = C.c_int()
    _lib.check(_lib.lib().qr_test_schedule_pairs(
        mask.ctypes.data, None if flag is None else flag.ctypes.data, nv, 0 if flag is None else 1,
        items.ctypes.data, ord_.ctypes.data, C.byref(listed), C.byref(classes)))
    n = listed.value
    it = [(int(v & 0x7fff), int((v >> 15) & 0x7fff), bool((v >> 30) & 1)) for v in items[:n]]
    return it, ord_[:2 * n].reshape(-1, 2), classes.value


@pytest.mark.parametrize("nv,density,seed", [(2, 1.0, 0), (8, 0.5, 1), (64, 0.05, 2), (64, 0.6, 3),
                                             (258, 0.02, 4), (512, 0.004, 5)])
def test_every_marked_pair_once_with_consistent_ordinals(nv, density, seed):
    g = np.random.default_rng(seed)
    pairs = {(p, q) for p in range(nv) for q in range(p + 1, nv) if g.random() < density}
    items, ords, classes = schedule(sorted(pairs), nv)
    assert sorted((p, q) for p, q, _ in items) == sorted(pairs)
    seen = [0] * nv
    for (p, q, full), (op, oq) in zip(items, ords):
        assert p < q and not full
        assert (op, oq) == (seen[p], seen[q])
        seen[p] += 1
        seen[q] += 1
    deg = np.zeros(nv, dtype=int)
    for p, q in pairs:
        deg[p] += 1
        deg[q] += 1
    if pairs:
        assert deg.max() <= classes <= 2 * deg.max() - 1
    else:
        assert classes == 0


def test_classes_are_disjoint_in_list_order():
    """Listing class by class: a pair's class is the number of class boundaries before it, and two
    pairs of one class never share a vertex.  Recovered here from the ordinals: within one class
    each vertex occurs at most once, so a greedy split of the list at the first repeated vertex
    must need no more pieces than the reported number of classes."""
    nv = 128
    g = np.random.default_rng(7)
    pairs = sorted({(p, q) for p in range(nv) for q in range(p + 1, nv) if g.random() < 0.1})
    items, _, classes = schedule(pairs, nv)
    pieces, used = 1, set()
    for p, q, _ in items:
        if p in used or q in used:
            pieces += 1
            used = set()
        used |= {p, q}
    assert pieces <= classes


def test_flagged_vertices_are_met_by_full_items():
    nv = 16
    flags = [0] * nv
    for v in (0, 5, 6, 11):
        flags[v] = 1
    pairs = [(5, 9), (9, 12), (2, 3)]  # vertex 5 has a marked pair; 0, 6, 11 have none
    items, ords, _ = schedule(pairs, nv, flags)
    listed = {(p, q) for p, q, _ in items}
    assert set(pairs) <= listed
    for v in (0, 6, 11):  # listed with their neighbour v ^ 1
        assert (min(v, v ^ 1), max(v, v ^ 1)) in listed
    for v in (0, 5, 6, 11):
        assert any(full and v in (p, q) for p, q, full in items), v
    seen = [0] * nv
    for (p, q, _), (op, oq) in zip(items, ords):
        assert (op, oq) == (seen[p], seen[q])
        seen[p] += 1
        seen[q] += 1


def test_bad_arguments_are_refused():
    with pytest.raises(Exception):
        schedule([(0, 1)], 3)
