"""Batched engine (C++/CUDA in the library): many independent simulate-and-measure requests of
uneven length and bond dimension, every brick-wall layer of all of them in one fused launch, the
whole circuit in one CUDA graph.  Requests are ``serve.Request`` objects with chi_max <= 64.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import ArgumentError, check, dptr, lib
from .serve import Request, pauli_codes


class Batch:
    def __init__(self, device=0, precision="fp64"):
        self._h = None
        if precision not in ("fp64", "mixed"):
            raise ArgumentError(f"the batched engine runs in \"fp64\" or \"mixed\", not {precision!r}")
        self._h = C.c_void_p()
        check(lib().qr_batch_create(device, C.byref(self._h)))
        check(lib().qr_batch_set_precision(self._h, {"fp64": 0, "mixed": 1}[precision]))
        self._reqs = []

    def close(self):
        if self._h is not None and self._h.value:
            lib().qr_batch_free(self._h)
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

    def add(self, req: Request) -> int:
        gs = np.array([s - 1 for s, _ in req.gates] or [0], dtype=np.int32)
        gm = np.ascontiguousarray(np.array([np.asarray(m, dtype=np.complex128) for _, m in req.gates]).reshape(-1)
                                  if req.gates else np.zeros(1, dtype=np.complex128))
        w = np.array([len(o) for o in req.observables] or [0], dtype=np.int32)
        sites = np.array([s - 1 for o in req.observables for s, _ in o] or [0], dtype=np.int32)
        codes = np.array(pauli_codes(req.observables) or [0], dtype=np.int32)
        ip = lambda a: a.ctypes.data_as(C.POINTER(C.c_int))  # noqa: E731
        rid = C.c_int()
        check(lib().qr_batch_add(self._h, req.n, req.chi_max, float(req.threshold), len(req.gates), ip(gs), dptr(gm),
                                 len(req.observables), ip(w), ip(sites), ip(codes), C.byref(rid)))
        self._reqs.append(req)
        return rid.value

    def _req(self, rid):
        if not isinstance(rid, (int, np.integer)) or not 0 <= rid < len(self._reqs):
            raise ArgumentError("bad batch request id")
        return self._reqs[rid]

    def plan(self, rid):
        req = self._req(rid)
        out = np.zeros(max(1, len(req.gates)), dtype=np.int32)
        nl = C.c_int()
        check(lib().qr_batch_plan(self._h, rid, out.ctypes.data_as(C.POINTER(C.c_int)), C.byref(nl)))
        return out[:len(req.gates)], nl.value

    def run(self):
        ms = C.c_double()
        check(lib().qr_batch_run(self._h, C.byref(ms)))
        return ms.value

    def result(self, rid):
        """{'values': <psi|P|psi> per string, 'status': 0 or the failing status code}"""
        n = len(self._req(rid).observables)
        vals = np.zeros(2 * max(1, n))
        st = C.c_int()
        check(lib().qr_batch_result(self._h, rid, C.byref(st), dptr(vals)))
        return {"values": vals[0:2 * n:2] + 1j * vals[1:2 * n:2], "status": st.value}

    def values(self, rid):
        r = self.result(rid)
        check(r["status"])
        return r["values"]

    def bond_dims(self, rid):
        out = np.zeros(self._req(rid).n - 1, dtype=np.int32)
        check(lib().qr_batch_bond_dims(self._h, rid, out.ctypes.data_as(C.POINTER(C.c_int))))
        return [int(x) for x in out]

    def lambda_on(self, rid, bond):
        """Lambda on bond ``bond`` (0-based, between sites bond and bond + 1), or None."""
        ln = C.c_int()
        check(lib().qr_batch_lambda(self._h, rid, bond, None, C.byref(ln)))
        if ln.value == 0:
            return None
        out = np.zeros(ln.value)
        check(lib().qr_batch_lambda(self._h, rid, bond, dptr(out), C.byref(ln)))
        return out

    def info(self):
        a, b, c, d, e = (C.c_int() for _ in range(5))
        f, g = C.c_double(), C.c_double()
        check(lib().qr_batch_info(self._h, C.byref(a), C.byref(b), C.byref(c), C.byref(d), C.byref(e), C.byref(f),
                                  C.byref(g)))
        return {"layers": a.value, "launches": b.value, "graph_nodes": c.value, "warps_per_cta": d.value,
                "tuned_from_cache": bool(e.value), "graph_ms": f.value, "tune_ms": g.value}
