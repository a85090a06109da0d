"""Continuous-batching request server (C++ in the library) and request generators.

A request is a brick-wall circuit on |0...0> plus Pauli-string observables; results are the
unnormalised <psi|P|psi> of each string, the value ``expect(psi, [P_1, ..., P_k])`` gives for a
string of single-site observables (src/Ansatz/Chain.jl:724-735).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from ._lib import ArgumentError, check, dptr, lib
from . import random as R

PAULI_CODE = {"I": 0, "X": 1, "Y": 2, "Z": 3}


def pauli_codes(observables):
    """The library's codes (0 I, 1 X, 2 Y, 3 Z) of every string's letters, in order."""
    out = []
    for o in observables:
        for _, p in o:
            if p not in PAULI_CODE:
                raise ArgumentError(f"Pauli letter must be one of I, X, Y, Z, got {p!r}")
            out.append(PAULI_CODE[p])
    return out


@dataclass
class Request:
    n: int
    chi_max: int
    gates: list  # [(left_site_1based, 4x4 matrix)]
    observables: list  # [[(site_1based, 'X'|'Y'|'Z'|'I'), ...], ...]
    threshold: float = 1e-10
    meta: dict = field(default_factory=dict)


class Server:
    def __init__(self, workers=8, hbm_budget_bytes=64 << 30, precision="mixed", device=0):
        self._h = None
        modes = {"fp64": 0, "mixed": 1, "split": 2, "mixed+split": 3}
        if precision not in modes:
            raise ArgumentError(f"precision must be one of {sorted(modes)}, not {precision!r}")
        prec = modes[precision]
        self._h = C.c_void_p()
        check(lib().qr_server_create(device, workers, int(hbm_budget_bytes), prec, C.byref(self._h)))

    def close(self):
        if self._h is not None and self._h.value:
            lib().qr_server_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def submit(self, req: Request) -> int:
        gs = np.array([s - 1 for s, _ in req.gates], dtype=np.int32)
        gm = np.ascontiguousarray(np.array([np.asarray(m, dtype=np.complex128) for _, m in req.gates]).reshape(-1)
                                  if req.gates else np.zeros(1, dtype=np.complex128))
        w = np.array([len(o) for o in req.observables], dtype=np.int32)
        sites = np.array([s - 1 for o in req.observables for s, _ in o] or [0], dtype=np.int32)
        codes = np.array(pauli_codes(req.observables) or [0], dtype=np.int32)
        t = C.c_uint64()
        ip = lambda a: a.ctypes.data_as(C.POINTER(C.c_int))  # noqa: E731
        check(lib().qr_server_submit(self._h, req.n, req.chi_max, float(req.threshold), len(req.gates), ip(gs),
                                     dptr(gm), len(req.observables), ip(w), ip(sites), ip(codes), C.byref(t)))
        return int(t.value), len(req.observables)

    def wait(self, ticket, timeout=-1.0):
        t, nobs = ticket
        done, status = C.c_int(), C.c_int()
        res = np.zeros(2 * max(nobs, 1))
        lat, que = C.c_double(), C.c_double()
        check(lib().qr_server_wait(self._h, t, float(timeout), C.byref(done), C.byref(status), dptr(res),
                                   C.byref(lat), C.byref(que)))
        if not done.value:
            return None
        check(status.value)
        vals = res[0:2 * nobs:2] + 1j * res[1:2 * nobs:2]
        return {"values": vals, "latency_ms": lat.value, "queue_ms": que.value}

    def stats(self):
        a, b, d = C.c_uint64(), C.c_uint64(), C.c_uint64()
        c, q = C.c_int(), C.c_int()
        check(lib().qr_server_stats(self._h, C.byref(a), C.byref(b), C.byref(c), C.byref(d), C.byref(q)))
        return {"submitted": a.value, "completed": b.value, "in_flight": c.value, "hbm_in_use": d.value,
                "queued": q.value}


def footprint(n, chi_max):
    b = C.c_uint64()
    check(lib().qr_server_footprint(n, chi_max, C.byref(b)))
    return b.value


def random_request(g, n_range=(16, 128), depth_range=(4, 32), chi_choices=(32, 128, 512, 1024), nobs=8,
                   weight_range=(1, 4), threshold=1e-10):
    """One serving request: random brick-wall circuit (Haar 4x4 gates) and ``nobs`` random Pauli
    strings of weight 1-4 on random sites."""
    n = int(g.integers(n_range[0], n_range[1] + 1))
    depth = int(g.integers(depth_range[0], depth_range[1] + 1))
    chi = int(chi_choices[int(g.integers(0, len(chi_choices)))])
    gates = []
    for layer in range(depth):
        start = 1 if layer % 2 == 0 else 2
        gates += [(s, R.haar_unitary(g, 4)) for s in range(start, n, 2)]
    obs = []
    for _ in range(nobs):
        w = int(g.integers(weight_range[0], weight_range[1] + 1))
        sites = sorted(g.choice(n, size=w, replace=False) + 1)
        obs.append([(int(s), "XYZ"[int(g.integers(0, 3))]) for s in sites])
    return Request(n=n, chi_max=chi, gates=gates, observables=obs, threshold=threshold,
                   meta={"depth": depth})


def batched_requests(count, seed, n_range=(8, 96), depth_range=(4, 32), chi_log2=(4, 9), nobs=1):
    """The batched workload: n ~ U[8, 96], chi_max log-uniform in {16 .. 512}, depth ~ U[4, 32]."""
    g = R.rng(seed)
    out = []
    for _ in range(count):
        chi = 2 ** int(g.integers(chi_log2[0], chi_log2[1] + 1))
        out.append(random_request(g, n_range=n_range, depth_range=depth_range, chi_choices=(chi,), nobs=nobs))
    return out
