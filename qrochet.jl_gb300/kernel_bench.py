"""Kernel-level benchmark of the library's hot kernels through the C ABI test hooks.

    python qrochet.jl_gb300/kernel_bench.py zgemm M N K [iters]
    python qrochet.jl_gb300/kernel_bench.py svd fp64|mixed N [M]
    python qrochet.jl_gb300/kernel_bench.py qr M N
    python qrochet.jl_gb300/kernel_bench.py zgemm_tc M N K [iters] [batch]
    python qrochet.jl_gb300/kernel_bench.py batch CHI_MAX REQUESTS fp64|mixed
    python qrochet.jl_gb300/kernel_bench.py mpo_env N CHI split|fp64 [reps]
    python qrochet.jl_gb300/kernel_bench.py upload CHI

Inputs are seeded complex Gaussians; prints one JSON line with the event-timed duration, the
algorithmic flop count and the achieved rate.  Used for ncu captures of single kernels.
"""
import ctypes as C
import json
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
from qrochet import _lib  # noqa: E402
from qrochet import random as R  # noqa: E402

p = _lib.dptr


def main(argv):
    L = _lib.lib()
    g = R.rng(1)
    what = argv[0]
    if what == "zgemm":
        M, N, K = (int(x) for x in argv[1:4])
        iters = int(argv[4]) if len(argv) > 4 else 3
        A = np.asfortranarray(R.complex_gaussian(g, (M, K)))
        B = np.asfortranarray(R.complex_gaussian(g, (K, N)))
        Cm = np.zeros((M, N), dtype=np.complex128, order="F")
        ms = C.c_double()
        _lib.check(L.qr_test_zgemm(0, 0, M, N, K, p(np.array([1.0, 0.0])), p(A), M, p(B), K, p(np.zeros(2)), p(Cm),
                                   M, None, iters, C.byref(ms)))
        fl = 8.0 * M * N * K
        out = {"op": "zgemm", "M": M, "N": N, "K": K, "ms": ms.value, "tflops": fl / ms.value / 1e9}
    elif what == "svd":
        mode = {"fp64": 0, "mixed": 1}[argv[1]]
        n = int(argv[2])
        m = int(argv[3]) if len(argv) > 3 else n
        A = np.asfortranarray(R.complex_gaussian(g, (m, n)))
        k = min(m, n)
        U = np.empty((m, k), dtype=np.complex128, order="F")
        Vh = np.empty((k, n), dtype=np.complex128, order="F")
        S = np.empty(k)
        ms = C.c_double()
        _lib.check(L.qr_test_svd(mode, m, n, p(A), p(U), p(S), p(Vh), C.byref(ms)))
        out = {"op": "svd", "mode": argv[1], "m": m, "n": n, "ms": ms.value,
               "recon": float(np.max(np.abs((U * S) @ Vh - A)) / S[0])}
    elif what == "qr":
        m, n = int(argv[1]), int(argv[2])
        A = np.asfortranarray(R.complex_gaussian(g, (m, n)))
        k = min(m, n)
        Q = np.empty((m, k), dtype=np.complex128, order="F")
        Rm = np.empty((k, n), dtype=np.complex128, order="F")
        ms = C.c_double()
        _lib.check(L.qr_test_qr(m, n, p(A), p(Q), p(Rm), C.byref(ms)))
        out = {"op": "qr", "m": m, "n": n, "ms": ms.value}
    elif what == "zgemm_tc":
        # the tcgen05 split kernel with the environment sweep's operand shapes: op(A) = A^T with K
        # contiguous, B shared by the batch
        M, N, K = (int(x) for x in argv[1:4])
        iters = int(argv[4]) if len(argv) > 4 else 3
        batch = int(argv[5]) if len(argv) > 5 else 1
        A = np.asfortranarray(R.complex_gaussian(g, (K, M * batch)))
        B = np.asfortranarray(R.complex_gaussian(g, (K, N)))
        Cm = np.zeros(M * N * batch, dtype=np.complex128)
        ms = C.c_double()
        _lib.check(L.qr_test_zgemm_tc(1, 0, M, N, K, batch, p(A), K, K * M if batch > 1 else 0, p(B), K, 0, p(Cm), M,
                                      iters, C.byref(ms)))
        ref = A[:, :M].T @ B
        got = Cm[:M * N].reshape((M, N), order="F")
        fl = 8.0 * M * N * K * batch
        out = {"op": "zgemm_tc", "M": M, "N": N, "K": K, "batch": batch, "ms": ms.value,
               "tflops_complex_equiv": fl / ms.value / 1e9, "bf16_tflops_executed": 6.0 * fl / ms.value / 1e9,
               "rel_err": float(np.linalg.norm(got - ref) / np.linalg.norm(ref))}
    elif what == "batch":
        # the batched engine on requests of the batched distribution with one chi_max class
        import time
        from qrochet import serve as S
        from qrochet.batch import Batch
        chi, nreq, prec = int(argv[1]), int(argv[2]), argv[3]
        e = int(round(np.log2(chi)))
        reqs = S.batched_requests(nreq, seed=4, chi_log2=(e, e), nobs=1)
        with Batch(precision=prec) as b:
            for r in reqs:
                b.add(r)
            t0 = time.perf_counter()
            b.run()
            dt = time.perf_counter() - t0
            out = {"op": "batch", "chi_max": chi, "requests": nreq, "precision": prec,
                   "gates": sum(len(r.gates) for r in reqs), "wall_s": dt, **b.info()}
    elif what == "mpo_env":
        # <psi|H_XXZ|psi> environment sweep on an n-site chain with bonds min(chi, 2^i) mirrored
        import time
        import qrochet as Q
        n, chi, prec = int(argv[1]), int(argv[2]), argv[3]
        reps = int(argv[4]) if len(argv) > 4 else 1
        arrays = []
        for i in range(n):
            cl = 1 if i == 0 else min(chi, 2 ** i, 2 ** (n - i))
            cr = 1 if i == n - 1 else min(chi, 2 ** (i + 1), 2 ** (n - i - 1))
            a = R.complex_gaussian(g, (2, cl, cr)) / np.sqrt(2.0 * cl)
            arrays.append(np.asfortranarray(a[:, 0, :] if i == 0 else a[:, :, 0] if i == n - 1 else a))
        psi = Q.MPS(arrays)
        psi.set_precision("mixed+split" if prec == "split" else "fp64")
        H = Q.MPO(R.xxz_mpo_arrays(n, 1.0, 0.7))
        Q.mpo_expect(psi, H)
        psi.sync()
        t0 = time.perf_counter()
        for _ in range(reps):
            e = Q.mpo_expect(psi, H)
        dt = (time.perf_counter() - t0) / reps
        out = {"op": "mpo_env", "n": n, "chi": chi, "precision": prec, "ms": 1e3 * dt, "energy": [e.real, e.imag]}
    elif what == "upload":
        # a 3-site chain whose middle site is (2, chi, chi) in the reference's (o, l, r) order: the
        # upload permutes it to the device layout (l, o, r)
        import qrochet as Q
        chi = int(argv[1])
        arrays = [R.complex_gaussian(g, (2, chi)), R.complex_gaussian(g, (2, chi, chi)), R.complex_gaussian(g, (2, chi))]
        psi = Q.MPS(arrays)
        psi.sync()
        back = psi.site_array(2)
        out = {"op": "upload", "chi": chi, "bytes_per_permute": 2 * 16 * 2 * chi * chi,
               "roundtrip_exact": bool(np.array_equal(back, arrays[1]))}
    else:
        raise SystemExit(__doc__)
    print(json.dumps(out))


if __name__ == "__main__":
    main(sys.argv[1:])
