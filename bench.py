#!/usr/bin/env python
"""Benchmark of the Chain hot path: TEBD gate+SVD steps/s at chi=1024.

One step = one ``evolve!`` of a Haar-random two-site gate on a bond whose neighbours both have
chi = 1024: theta (2048 x 2048 complex) = A_l diag(Lambda) A_r, gate, thin SVD, truncate! to
maxdim = 1024 with the 1e-10 cutoff.  The chain is n = 24 random isometric sites (bonds
min(1024, 2^i) mirrored), so bonds 10..14 carry chi = 1024; steps cycle over the three bonds whose
neighbours are both full.  Every step touches > 129 MB (sites 64 MB, theta 64 MB, SVD buffers
several x 64 MB), so inputs are larger than L2.

Prints one JSON line (driver contract): ``value`` = gate-steps/s of the mixed path with the state
resident in HBM; ``e2e`` = the same through the C ABI with pinned host buffers copied in and out
every step; ``fp64`` = the plain all-FP64 path; ``roofline`` for the dominant kernel;
``cpu_baseline`` = the oracle (NumPy/LAPACK) on the host cores.

``--impl reference`` times the CPU restatement (the reference itself is Julia and is not
installed), on the same workload, with all host threads.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "qrochet.jl_gb300")
sys.path.insert(0, PKG)
sys.path.insert(0, ROOT)

METRIC = "TEBD gate+SVD steps/s at χ=1024; batched solves/s, p50/p99; mixed vs FP64 path"
N_SITES, CHI, MAXDIM, CUTOFF = 24, 1024, 1024, 1e-10
BONDS = (11, 12, 13)  # 1-based left sites of the gate bonds with chi=1024 on both sides


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=6)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--fp64-steps", type=int, default=6)
    p.add_argument("--cpu-steps", type=int, default=2)
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--quick", action="store_true", help="small chi for a fast functional run")
    p.add_argument("--launch-list", action="store_true",
                   help="only the warm-up and timed steps of the mixed path (for ncu launch lists)")
    p.add_argument("--batched", type=int, default=128, help="requests in the batched sample (0: skip)")
    p.add_argument("--canonize-full", action="store_true",
                   help="also time the whole canonize! of the MPO leg's chain (about a minute)")
    p.add_argument("--batched-full", type=int, default=8,
                   help="requests of the full batched distribution, chi_max up to 512 (0: skip)")
    p.add_argument("--serve", type=int, default=24, help="requests in the serving sample (0: skip)")
    p.add_argument("--serve-sat", type=int, default=64,
                   help="requests in the saturated mixed-precision serving sample (0: skip)")
    p.add_argument("--serve-full", type=int, default=64,
                   help="requests in the mixed-precision sample over every chi_max class (0: skip)")
    p.add_argument("--mpo-sites", type=int, default=128, help="sites of the MPO environment sweep (0: skip)")
    p.add_argument("--workers", type=int, default=16)
    p.add_argument("--no-tebd", action="store_true", help="skip the n=64, chi_max=256, depth-40 TEBD leg")
    return p.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    local = int(os.environ.get("LOCAL_RANK", 0))
    return rank, world, local


class Dist:
    """Barrier and max-reduce across replicas (gloo; no data-path collective)."""

    def __init__(self, world):
        self.world = world
        if world > 1:
            import torch.distributed as td

            td.init_process_group("gloo")
            self.td = td

    def barrier(self):
        if self.world > 1:
            self.td.barrier()

    def _reduce(self, x, op):
        if self.world == 1:
            return x
        import torch

        t = torch.tensor([float(x)], dtype=torch.float64)
        self.td.all_reduce(t, op=getattr(self.td.ReduceOp, op))
        return float(t.item())

    def max(self, x):
        return self._reduce(x, "MAX")

    def sum(self, x):
        return self._reduce(x, "SUM")

    def gather(self, values):
        """Concatenation of every rank's list (rank order)."""
        if self.world == 1:
            return list(values)
        out = [None] * self.world
        self.td.all_gather_object(out, list(values))
        return [v for part in out for v in part]


def shard(items, rank, world):
    """Replica partition of independent requests: rank r takes items r, r + world, ...  Every item
    goes to exactly one rank and no data moves between ranks."""
    return list(items)[rank::world]


class DevTimer:
    """CUDA events recorded on the stream the chain's kernels run on (device time of the timed
    region; the host-side synchronisations inside a step are part of it)."""

    def __init__(self, stream_handle, device):
        import torch

        torch.cuda.set_device(device)
        self.stream = torch.cuda.ExternalStream(stream_handle, device=device)
        self.e0 = torch.cuda.Event(enable_timing=True)
        self.e1 = torch.cuda.Event(enable_timing=True)

    def start(self):
        self.e0.record(self.stream)

    def stop(self):
        self.e1.record(self.stream)
        self.e1.synchronize()
        return self.e0.elapsed_time(self.e1) * 1e-3


# DRAM bytes (read + write) per launch (one Jacobi sweep, or one GEMM) from one ncu capture of each
# kernel on a 1024 x 1024 mixed SVD: jacobi_block_reg_k for jacobi_fp32, jacobi_block_df_k (the
# full double-float sweeps) for jacobi_df, zgemm_df_k for zgemm_df.  A sweep's traffic is the first
# touch of B and V and a GEMM's the first touch of its operands, so it scales with the operand
# size: (k / 1024)^2 at k columns.
NCU_TRAFFIC_1024 = {"jacobi_fp32": 16.937472e6 + 15.872e3, "jacobi_df": 34.0e6 + 5.3e6,
                    "zgemm_df": 16.850432e6}


def workload(chi):
    from qrochet import random as R

    g = R.rng(2024)
    arrays = R.rand_chain_state_arrays(g, N_SITES, chi, p=2)
    gates = [R.haar_unitary(g, 4) for _ in range(64)]
    return arrays, gates


class Clocks:
    """nvidia-smi sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except Exception:
            self.proc.kill()
            out = ""
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def gate_flops(chi):
    """Algorithmic flops of one gate step (theta GEMM + gate + R-SVD count of an m x n SVD,
    m = n = 2 chi, 4 (4 m^2 n + 8 m n^2 + 9 n^3) real flops for complex)."""
    m = n = 2 * chi
    gemm = 8.0 * (2 * chi) * (2 * chi) * chi
    gate = 8.0 * chi * chi * 16
    svd = 4.0 * (4 * m * m * n + 8 * m * n * n + 9 * n ** 3)
    return gemm + gate + svd


def cpu_gate_step(al, ar, lam, u, maxdim):
    """Oracle gate step (NumPy/LAPACK): the same arithmetic as evolve_2site! + truncate!."""
    from oracle import chain_oracle as O

    ch = O.OChain([np.ones((1, 2, al.shape[0]), dtype=complex)] + [al, ar] +
                  [np.ones((ar.shape[2], 2, 1), dtype=complex)])
    ch.lam[1] = lam
    O.evolve_2site_(ch, 1, u, threshold=CUTOFF, maxdim=maxdim)
    return ch


def guarded(name, fn, world):
    """Run a secondary leg; in a single process a failure is reported in the line (an "error"
    entry) instead of losing the headline measurement.  With several ranks the exception
    propagates, so that no rank is left waiting in a collective the failed one never joins."""
    if world > 1:
        return fn()
    try:
        return fn()
    except Exception as x:  # noqa: BLE001 -- any failure of a secondary leg
        print(f"bench: the {name} leg failed: {x!r}", file=sys.stderr, flush=True)
        return {"error": f"{type(x).__name__}: {x}"}


def run_batched(args, Q, dist, rank, world):
    """Batched solves/s on requests of the batched distribution (n ~ U[8,96], depth ~ U[4,32],
    cutoff 1e-10) with chi_max log-uniform in {16, 32, 64}: the bond classes the batched engine
    takes (theta up to 128 x 128).  Two paths on the same requests:
      - engine: qr_batch -- every layer of all requests one fused launch, device-side truncation,
        the whole circuit one CUDA graph; mixed (FP32-preconditioned SVD, FP64 finish) and FP64;
      - server: the continuous-batching request server, one chain and stream per request, mixed
        precision.
    The chi_max in {128, 256, 512} part of the distribution is outside the engine's bond limit and
    takes minutes per request on the server: not in this sample."""
    from qrochet import serve as S
    from qrochet.batch import Batch

    reqs = shard(S.batched_requests(args.batched, seed=4, chi_log2=(4, 6), nobs=1), rank, world)
    gates = dist.sum(sum(len(r.gates) for r in reqs))
    out = {"requests": int(dist.sum(len(reqs))), "gates": int(gates),
           "sample": f"{args.batched} requests: n~U[8,96], depth~U[4,32], chi_max log-uniform in {{16,32,64}}, "
                     f"cutoff 1e-10, 1 Pauli string each, seed 4"}
    vals_engine = None
    for prec in ("mixed", "fp64"):
        with Batch(device=0, precision=prec) as bt:
            for r in reqs:
                bt.add(r)
            dist.barrier()
            t0 = time.perf_counter()
            bt.run()
            dt = dist.max(time.perf_counter() - t0)
            info = bt.info()
            if prec == "mixed":
                vals_engine = [bt.values(i) for i in range(len(reqs))]
        out["engine" if prec == "mixed" else "engine_fp64"] = {
            "solves_per_s": out["requests"] / dt, "gate_steps_per_s": gates / dt, "wall_s": dt,
            "graph_ms": info["graph_ms"], "autotune_ms": info["tune_ms"], "layers": info["layers"],
            "launches": info["launches"], "graph_nodes": info["graph_nodes"],
            "warps_per_cta": info["warps_per_cta"], "precision": prec}
    with S.Server(workers=args.workers, precision="mixed") as sv:
        dist.barrier()
        t0 = time.perf_counter()
        tickets = [sv.submit(r) for r in reqs]
        res = [sv.wait(t) for t in tickets]
        dt = dist.max(time.perf_counter() - t0)
    lat = dist.gather([x["latency_ms"] for x in res])
    out["server"] = {"solves_per_s": out["requests"] / dt, "gate_steps_per_s": gates / dt, "wall_s": dt,
                     "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                     "workers": args.workers, "precision": "mixed"}
    diffs = [float(np.max(np.abs(a - x["values"])) / max(1e-300, float(np.max(np.abs(x["values"])))))
             for a, x in zip(vals_engine, res)]
    out["max_rel_diff_engine_vs_server"] = dist.max(max(diffs) if diffs else 0.0)
    out["engine_over_server"] = out["engine"]["solves_per_s"] / out["server"]["solves_per_s"]
    return out


def run_batched_full(args, Q, dist, rank, world):
    """Batched solves/s on a sample of the whole batched distribution: n ~ U[8,96], depth ~ U[4,32],
    chi_max log-uniform in {16, ..., 512}, cutoff 1e-10 (`--batched-full` requests, seed 12: chi_max
    512, 256, 3 x 128, 64, 2 x 32).  Requests with chi_max <= 64 run on the batched engine (one
    graph), the larger ones on the request server (one chain and stream per request; their gates take
    the multi-CTA SVD), one after the other; solves/s = requests / the two wall times.  A sample:
    per-request cost is heavy-tailed (a chi_max = 512 request with n ~ 90 runs ~1000 gates, most at
    theta 1024 x 1024), so the 512-request distribution would take tens of minutes at these rates."""
    from qrochet import serve as S
    from qrochet.batch import Batch

    reqs = shard(S.batched_requests(args.batched_full, seed=12, chi_log2=(4, 9), nobs=1), rank, world)
    small = [r for r in reqs if r.chi_max <= 64]
    large = [r for r in reqs if r.chi_max > 64]
    gates = dist.sum(sum(len(r.gates) for r in reqs))
    t_eng = t_srv = 0.0
    if small:
        with Batch(device=0, precision="mixed") as bt:
            for r in small:
                bt.add(r)
            dist.barrier()
            t0 = time.perf_counter()
            bt.run()
            t_eng = dist.max(time.perf_counter() - t0)
    lat = []
    if large:
        with S.Server(workers=args.workers, precision="mixed") as sv:
            dist.barrier()
            t0 = time.perf_counter()
            tickets = [sv.submit(r) for r in large]
            res = [sv.wait(t) for t in tickets]
            t_srv = dist.max(time.perf_counter() - t0)
        lat = [x["latency_ms"] for x in res]
    n_all = int(dist.sum(len(reqs)))
    return {"requests": n_all, "gates": int(gates), "chi_max": sorted((r.chi_max for r in reqs), reverse=True),
            "solves_per_s": n_all / max(1e-9, t_eng + t_srv), "gate_steps_per_s": gates / max(1e-9, t_eng + t_srv),
            "engine_s": t_eng, "engine_requests": len(small), "server_s": t_srv, "server_requests": len(large),
            "server_latency_ms": sorted(float(x) for x in lat), "precision": "mixed",
            "sample": f"{args.batched_full} requests of the full batched distribution (chi_max 16..512), seed 12"}


def run_serving(args, Q, dist, rank, world):
    """Serving: Poisson arrivals at 200 req/s of random brick-wall circuits with 8 Pauli strings of
    weight 1-4; p50/p99 latency and solves/s.  Bounded samples:
      - fp64 / mixed: `--serve` requests, n ~ U[16,64], depth ~ U[4,16], chi_max in {32, 128}; the
        two forms' expectation values are compared;
      - mixed_saturated: `--serve-sat` requests of the same distribution (~4x the workers), so a
        queue stands in front of every worker for most of the run;
      - mixed_full_chi: `--serve-full` requests over every chi_max class {32, 128, 512, 1024} of the
        serving distribution, on n ~ U[16,32], depth ~ U[4,10]."""
    from qrochet import serve as S
    from qrochet import random as R

    out = {}
    small = dict(n_range=(16, 64), depth_range=(4, 16), chi_choices=(32, 128))
    runs = [("fp64", "fp64", args.serve, small), ("mixed", "mixed", args.serve, small)]
    if args.serve_sat > 0:
        runs.append(("mixed_saturated", "mixed", args.serve_sat, small))
    if args.serve_full > 0:
        # every chi_max class of the serving distribution, on shorter and shallower circuits so the
        # chi_max = 512 / 1024 requests take seconds, not minutes
        runs.append(("mixed_full_chi", "mixed", args.serve_full,
                     dict(n_range=(16, 32), depth_range=(4, 10), chi_choices=(32, 128, 512, 1024))))
    for name, prec, nreq, dist_kw in runs:
        g = R.rng(5)
        reqs = [S.random_request(g, nobs=8, **dist_kw) for _ in range(nreq)]
        # arrivals at 200 req/s in total: each replica sees its share of the Poisson stream
        gaps = shard(g.exponential(1.0 / 200.0, size=len(reqs)).cumsum(), rank, world)
        reqs = shard(reqs, rank, world)
        with S.Server(workers=args.workers, precision=prec) as sv:
            tickets = []
            dist.barrier()
            t0 = time.perf_counter()
            for r, at in zip(reqs, gaps):
                wait = at - (time.perf_counter() - t0)
                if wait > 0:
                    time.sleep(wait)
                tickets.append(sv.submit(r))
            res = [sv.wait(t) for t in tickets]
            dt = dist.max(time.perf_counter() - t0)
        lat = np.array(dist.gather([x["latency_ms"] for x in res]))
        out[name] = {"requests": len(lat), "solves_per_s": len(lat) / dt, "p50_ms": float(np.percentile(lat, 50)),
                     "p99_ms": float(np.percentile(lat, 99)),
                     "p99_over_p50": float(np.percentile(lat, 99) / np.percentile(lat, 50)),
                     "values": [x["values"] for x in res]}
    err = max(float(np.max(np.abs(a - b))) for a, b in zip(out["fp64"]["values"], out["mixed"]["values"]))
    for prec in out:
        del out[prec]["values"]
    if "mixed_full_chi" in out:
        out["mixed_full_chi"]["sample"] = (f"{args.serve_full} requests: n~U[16,32], depth~U[4,10], "
                                           f"chi_max in {{32,128,512,1024}}, 8 Pauli strings of weight 1-4, seed 5")
    out["max_abs_expectation_diff_mixed_vs_fp64"] = err
    out["arrival_rate_per_s"] = 200
    out["workers"] = args.workers
    out["sample"] = ("fp64 / mixed / mixed_saturated: n~U[16,64], depth~U[4,16], chi_max in {32,128}, 8 Pauli "
                     "strings of weight 1-4, seed 5")
    return out


def run_mpo_env(args, Q):
    """MPS-MPO expectation of the Heisenberg XXZ MPO (Jz=1, Jxy=0.7, w=5) on an n-site chi=1024
    MPS: one left-to-right environment sweep in split precision (BF16x3 tensor cores) and in FP64.
    The state has complex Gaussian sites scaled by 1/sqrt(2 chi) (norm O(1)); canonize! is not
    timed (the sweep's cost does not depend on the gauge).  Each site is scaled by
    1/sqrt(2 chi_l) so the transfer operator keeps the environments O(1) along the chain."""
    from qrochet import random as R

    n, chi = args.mpo_sites, 1024
    g = R.rng(3)
    arrays = []
    for i in range(n):
        cl = 1 if i == 0 else min(chi, 2 ** i, 2 ** (n - i))
        cr = 1 if i == n - 1 else min(chi, 2 ** (i + 1), 2 ** (n - i - 1))
        a = (g.standard_normal((2, cl, cr), dtype=np.float32) + 1j * g.standard_normal((2, cl, cr),
                                                                                   dtype=np.float32))
        a = (a.astype(np.complex128) * (1.0 / np.sqrt(2.0 * 2 * cl)))
        arrays.append(np.asfortranarray(a[:, 0, :] if i == 0 else a[:, :, 0] if i == n - 1 else a))
    psi = Q.MPS(arrays)
    del arrays
    H = Q.MPO(R.xxz_mpo_arrays(n, 1.0, 0.7))
    res = {}
    for prec in ("mixed+split", "fp64"):
        psi.set_precision(prec)
        Q.mpo_expect(psi, H) if prec == "mixed+split" else None  # warm-up of the split path
        psi.sync()
        t0 = time.perf_counter()
        e = Q.mpo_expect(psi, H)
        res[prec] = (time.perf_counter() - t0, e)
    (ts, es), (td, ed) = res["mixed+split"], res["fp64"]
    # canonize! of this chain is 127 QR steps and 127 SVD steps of up to 2048 x 1024 (Chain.jl:469-497);
    # one of each on a middle site (chi = 1024 on both sides), per precision, on a copy
    mid = n // 2 + 1
    canon = {}
    for prec in ("fp64", "mixed"):
        c = psi.copy()
        c.set_precision(prec)
        c.sync()
        t0 = time.perf_counter()
        Q.canonize_site_(c, mid, "left", "qr")
        c.sync()
        t1 = time.perf_counter()
        Q.canonize_site_(c, mid, "left", "svd")
        c.sync()
        t2 = time.perf_counter()
        canon[prec] = {"qr_step_ms": 1e3 * (t1 - t0), "svd_step_ms": 1e3 * (t2 - t1)}
        del c
    if args.canonize_full:
        # the whole canonize! (Chain.jl:469-497) of this chain, per precision, on a copy
        for prec in ("mixed", "fp64"):
            c = psi.copy()
            c.set_precision(prec)
            c.sync()
            t0 = time.perf_counter()
            Q.canonize_(c)
            c.sync()
            canon[prec]["canonize_s"] = time.perf_counter() - t0
            del c
    bonds = [1] + [min(chi, 2 ** (i + 1), 2 ** (n - i - 1)) for i in range(n - 1)] + [1]
    wdim = [1] + [5] * (n - 1) + [1]
    flops = sum(8.0 * (wdim[i] * bonds[i] * 2 * bonds[i + 1] * bonds[i] + bonds[i + 1] * bonds[i + 1] * 2 * bonds[i] *
                       wdim[i + 1]) for i in range(n))
    return {"n": n, "chi": chi, "w": 5, "split_ms_per_sweep": 1e3 * ts, "fp64_ms_per_sweep": 1e3 * td,
            "canonize_site_at_chi1024": canon,
            "canonize_note": "one canonize_site!(; direction=:left) step of each method on site n/2+1 "
                             "(a 2048 x 1024 factorisation); canonize! runs 127 of each, most at this size",
            "split_over_fp64": td / ts, "rel_err_split_vs_fp64": abs(es - ed) / abs(ed),
            "energy_fp64": [ed.real, ed.imag], "split_tflops_complex_equiv": flops / ts / 1e12,
            "note": "sites complex Gaussian / sqrt(2 chi_l); bond dims min(1024, 2^i) mirrored; "
                    "flops = algorithmic count of both contractions over the actual bond dims"}


def run_tebd(args, Q, local):
    """TEBD at full size: n = 64 qubits from |0...0>, a depth-40 brick wall of Haar 4 x 4 gates
    (seed 2), maxdim 256, cutoff 1e-10; each layer through evolve_layer_ (its gates several at a time).
      - mixed: all 40 layers; every bond's Lambda spectrum and <X_i> against the oracle's golden
        results for the same gates (tests/golden/tebd_n64_chi256_d40.npz, made by
        make_tebd_golden.py next to it);
      - fp64 vs mixed: from the mixed state after layer 30 (bonds saturated at chi = 256), the last
        10 layers in both precisions: gate-steps/s of each and the mixed path's error against the
        FP64 path on the same start state.  (The FP64 path's full 40 layers take ~160 s; the
        GPU test suite runs them against the golden results.)"""
    from qrochet import random as R

    gold = np.load(os.path.join(ROOT, "tests", "golden", "tebd_n64_chi256_d40.npz"))
    n, depth, maxdim, split_at = 64, 40, 256, 30
    layers = R.brickwall_layers(n, depth, seed=2)
    lam_gold = np.split(gold["lambdas"], np.cumsum(gold["bond_dims"])[:-1])
    nrm2 = float(gold["norm"]) ** 2
    out = {"n": n, "depth": depth, "chi_max": maxdim, "threshold": 1e-10, "gates": sum(len(x) for x in layers),
           "note": "evolve! defaults (iscanonical=false): Lambdas stay on the bonds and theta is truncated "
                   "without the neighbouring weights, so the norm decays (oracle: %.3g) and the maxdim "
                   "truncation amplifies rounding differences over the 40 layers; <X_i> errors are relative to "
                   "<psi|psi>" % float(gold["norm"])}

    def run_layers(psi, ls):
        # each brick-wall layer through evolve_layer_ (its gates on disjoint sites, several at a
        # time on their own streams); wall time, since the lanes' streams are not the chain's
        psi.sync()
        t0 = time.perf_counter()
        for layer in ls:
            Q.evolve_layer_(psi, [Q.gate_from_matrix(u, [s_, s_ + 1]) for s_, u in layer], threshold=1e-10,
                            maxdim=maxdim)
        psi.sync()
        return time.perf_counter() - t0, sum(len(x) for x in ls)

    def xs(psi):
        return np.array([Q.expect(psi, [Q.gate_from_matrix(R.PAULI["X"], [i])]) for i in range(1, n + 1)])

    psi = Q.MPS(R.zero_product_arrays(n))
    psi.set_precision("mixed")
    t1, g1 = run_layers(psi, layers[:split_at])
    mid = psi.copy()
    t2, g2 = run_layers(psi, layers[split_at:])
    bonds = psi.bond_dims()
    same = bonds == [int(b) for b in gold["bond_dims"]]
    xm = xs(psi)
    out["mixed"] = {"gate_steps_per_s": (g1 + g2) / (t1 + t2), "s": t1 + t2, "bond_dims_match_oracle": same,
                    "lambda_max_rel_err_vs_oracle": (max(
                        float(np.max(np.abs(psi.lambda_between(b + 1, b + 2) - lam_gold[b])) / lam_gold[b][0])
                        for b in range(n - 1)) if same else None),
                    "x_max_abs_err_vs_oracle_over_norm2": float(np.max(np.abs(xm - gold["x"]))) / nrm2,
                    "norm_rel_err_vs_oracle": abs(Q.norm(psi) - float(gold["norm"])) / float(gold["norm"])}
    mid.set_precision("fp64")
    t3, g3 = run_layers(mid, layers[split_at:])
    xf = xs(mid)
    nf2 = Q.norm(mid) ** 2
    same2 = mid.bond_dims() == bonds
    out["last_layers_fp64_vs_mixed"] = {
        "layers": f"{split_at + 1}-{depth}", "gates": g3,
        "fp64_gate_steps_per_s": g3 / t3, "mixed_gate_steps_per_s": g2 / t2, "mixed_over_fp64": (g2 / t2) / (g3 / t3),
        "bond_dims_match": same2,
        "lambda_max_rel_err_mixed_vs_fp64": (max(
            float(np.max(np.abs(psi.lambda_between(b + 1, b + 2) - mid.lambda_between(b + 1, b + 2))) /
                  mid.lambda_between(b + 1, b + 2)[0]) for b in range(n - 1)) if same2 else None),
        "x_max_abs_err_mixed_vs_fp64_over_norm2": float(np.max(np.abs(xm - xf))) / nf2}
    del psi, mid
    return out


def run_reference(args, chi):
    """CPU restatement on all host threads (the Julia reference is not installed).  Runs the
    requested --steps gate steps (one untimed warm-up step: the CPU path needs no more)."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    arrays, gates = workload(chi)
    from oracle import chain_oracle as O

    ch = O.from_reference_arrays(arrays)
    steps = max(1, args.steps)
    warm = min(args.warmup, 1)
    b = BONDS[0] - 1
    al, ar = ch.sites[b], ch.sites[b + 1]
    lam = np.ones(al.shape[2])
    for i in range(warm):
        cpu_gate_step(al, ar, lam, gates[i], MAXDIM if chi == CHI else chi)
    t0 = time.perf_counter()
    for i in range(steps):
        cpu_gate_step(al, ar, lam, gates[i % len(gates)], MAXDIM if chi == CHI else chi)
    dt = time.perf_counter() - t0
    v = steps / dt
    cores = os.cpu_count()
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "gate-steps/s", "n_gpus": args.gpus,
            "steps": steps, "warmup": warm, "ms_per_step": 1e3 * dt / steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "complex128", "data": "synthetic",
            "config": {"workload": f"tebd_gate_step_chi{chi}", "chi": chi, "theta": f"{2 * chi}x{2 * chi}",
                       "maxdim": MAXDIM if chi == CHI else chi, "threshold": CUTOFF, "n_sites": N_SITES},
            "cpu_baseline": {"value": v, "unit": "gate-steps/s", "cores": cores, "kind": "port",
                             "sample": f"{steps} gate-steps, {warm} untimed warm-up (NumPy/LAPACK restatement of "
                                       f"Chain.jl evolve_2site!+truncate!, zgesdd on all host threads; Qrochet.jl "
                                       f"is Julia and is not installed)"},
            "e2e": {"value": v, "unit": "gate-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args, chi):
    import qrochet as Q
    from qrochet import random as R

    rank, world, local = dist_env()
    dist = Dist(world)
    Q.set_device(local)
    arrays, gates = workload(chi)
    maxdim = MAXDIM if chi == CHI else chi
    b0 = BONDS[0]

    def make(prec):
        psi = Q.MPS(arrays)
        psi.set_precision(prec)
        return psi

    def step(psi, i):
        b = BONDS[i % len(BONDS)]
        Q.evolve_(psi, Q.gate_from_matrix(gates[i % len(gates)], [b, b + 1]), threshold=CUTOFF, maxdim=maxdim)

    def local_z(psi):
        return np.array([Q.expect(psi, [Q.gate_from_matrix(R.PAULI["Z"], [s])]) for s in (b0, b0 + 1)])

    # ---- mixed path, state resident in HBM -------------------------------------------------------
    # Step 0 (gate 0 on bond (b0, b0 + 1) of the initial state) is also the accuracy sample: the
    # FP64 path and the oracle run the same gate on the same theta below.
    psi = make("mixed")
    step(psi, 0)
    acc_mixed = (psi.lambda_between(b0, b0 + 1).copy(), local_z(psi), psi.bond_dims()[b0 - 1])
    for i in range(1, args.warmup):
        step(psi, i)
    psi.sync()
    clocks = Clocks(local)
    clocks.start()
    l0 = Q.launch_count()
    timer = DevTimer(psi.stream(), local)
    dist.barrier()
    psi.sync()
    timer.start()
    for i in range(args.steps):
        step(psi, args.warmup + i)
    dt = timer.stop()
    launches = Q.launch_count() - l0
    dist.barrier()
    clk = clocks.stop()
    dt_max = dist.max(dt)
    value = world * args.steps / dt_max
    del psi
    if args.launch_list:
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value, "unit": "gate-steps/s", "steps": args.steps,
                              "warmup": args.warmup, "gpu_launches": launches, "mode": "launch-list"}), flush=True)
        return

    # ---- plain FP64 path ---------------------------------------------------------------------------
    fp64 = None
    acc_fp64 = None
    if args.fp64_steps > 0:
        p64 = make("fp64")
        step(p64, 0)
        acc_fp64 = (p64.lambda_between(b0, b0 + 1).copy(), local_z(p64), p64.bond_dims()[b0 - 1])
        p64.sync()
        t64 = DevTimer(p64.stream(), local)
        dist.barrier()
        t64.start()
        for i in range(args.fp64_steps):
            step(p64, 1 + i)
        d64 = dist.max(t64.stop())
        fp64 = {"value": world * args.fp64_steps / d64, "unit": "gate-steps/s",
                "ms_per_step": 1e3 * d64 / args.fp64_steps, "steps": args.fp64_steps}
        # how the FP64 arm uses its pipe: two more steps under the kernel-class profiler
        Q.prof_enable(True)
        for i in range(2):
            step(p64, 1 + args.fp64_steps + i)
        p64.sync()
        st64 = {k: Q.prof_read(k) for k in Q.PROF_KINDS}
        Q.prof_enable(False)
        dfma = Q.probe_peak("dfma")
        ms64 = sum(v["ms"] for v in st64.values())
        ex64 = sum(v["flops"] for v in st64.values())
        fp64["pipe"] = {
            "peak_dfma_tflops": dfma,
            "algorithmic_frac_of_dfma": (gate_flops(chi) / (fp64["ms_per_step"] * 1e-3)) / (dfma * 1e12),
            "executed_tflops": ex64 / (ms64 * 1e-3) / 1e12 if ms64 > 0 else 0.0,
            "executed_frac_of_dfma": ex64 / (ms64 * 1e-3) / (dfma * 1e12) if ms64 > 0 else 0.0,
            "time_share": {k: round(v["ms"] / max(1e-9, ms64), 4) for k, v in st64.items() if v["ms"] > 0},
            "note": "executed = the FP64 operations the kernels count (Jacobi inner products and rotations, "
                    "Householder QR, DMMA GEMMs) over their event time: one-sided Jacobi does ~4x the "
                    "Golub-Van Loan R-SVD count, so the executed rate, not the algorithmic one, shows how "
                    "busy the FP64 pipe is"}
        del p64

    # ---- e2e through the C ABI with pinned host buffers --------------------------------------------
    # The same state sequence as `value`: the same warm-up and gates, with the two sites of every
    # step uploaded from page-locked host copies of the current state before it and downloaded
    # into them after it (plus the bond's Lambda), so each step moves the state through the host.
    pe = make("mixed")
    for i in range(args.warmup):
        step(pe, i)
    pin = {}
    for s_ in sorted({x for bb in BONDS for x in (bb, bb + 1)}):
        cl, d, cr = pe.site_dims(s_)
        pa = Q.PinnedArray((d, cl, cr))
        pe.download_site(s_, pa.array)
        pin[s_] = pa
    pe.sync()
    h2d = d2h = 0
    te = DevTimer(pe.stream(), local)
    dist.barrier()
    te.start()
    for i in range(args.steps):
        b = BONDS[(args.warmup + i) % len(BONDS)]
        for s_ in (b, b + 1):
            pe.upload_site(s_, pin[s_].array)
        step(pe, args.warmup + i)
        for s_ in (b, b + 1):
            pe.download_site(s_, pin[s_].array)
        lam = pe.lambda_between(b, b + 1)
        if i == 0:
            h2d = pin[b].array.nbytes + pin[b + 1].array.nbytes + 16 * 16
            d2h = pin[b].array.nbytes + pin[b + 1].array.nbytes + lam.nbytes
    de = dist.max(te.stop())
    e2e = {"value": world * args.steps / de, "unit": "gate-steps/s", "h2d_bytes_per_step": int(h2d),
           "d2h_bytes_per_step": int(d2h), "ms_per_step": 1e3 * de / args.steps,
           "note": "same gates and state sequence as value; both sites of each step uploaded from and "
                   "downloaded to page-locked host memory, plus the gate and the bond's Lambda"}
    del pe

    # ---- roofline: algorithmic work of the whole gate step, plus the dominant kernel's pipe use ----
    Q.prof_enable(True)
    pr = make("mixed")
    nprof = min(3, args.steps)
    for i in range(nprof):
        step(pr, i)
    pr.sync()
    stats = {k: Q.prof_read(k) for k in Q.PROF_KINDS}
    Q.prof_enable(False)
    del pr
    dom = max(stats, key=lambda k: stats[k]["ms"])
    try:
        mp = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        mp = {}
    ffma = Q.probe_peak("ffma")
    st = stats[dom]
    executed = st["flops"] / (st["ms"] * 1e-3) / 1e12 if st["ms"] > 0 else 0.0
    shares = {k: round(v["ms"] / max(1e-9, sum(x["ms"] for x in stats.values())), 4) for k, v in stats.items()}
    ms_step = 1e3 * dt_max / args.steps
    alg = gate_flops(chi)
    achieved = alg / (ms_step * 1e-3) / 1e12
    # DRAM traffic per gate step: ncu bytes per launch (per sweep for the Jacobi kernels) times the
    # launches (sweeps) per step of each profiled class
    traffic = sum(NCU_TRAFFIC_1024[k] * (2 * chi / 1024) ** 2 * stats[k]["launches"] / nprof
                  for k in NCU_TRAFFIC_1024)
    roofline = {"bound": "fp32", "kernel": "gate step (all kernels of one evolve!)", "achieved": achieved,
                "peak": ffma, "unit": "TFLOP/s", "frac": achieved / ffma if ffma else None,
                "traffic": traffic, "launches": launches / max(1, args.steps), "avg_launch_ms": ms_step,
                "achieved_source": f"algorithmic count {alg:.3e} flop per gate step (theta GEMM + gate + "
                                   f"Golub-Van Loan R-SVD count of a {2 * chi}x{2 * chi} complex SVD) / ms_per_step",
                "peak_source": "FP32 FFMA rate measured in-process (loop kernel, best of 3): the mixed path runs "
                               "on the FP32 pipes; MEASURED_PEAKS.json holds only HBM and cuBLAS BF16",
                "traffic_source": "DRAM bytes per gate step: ncu dram__bytes_read.sum + dram__bytes_write.sum per "
                                  "launch (one Jacobi sweep, one GEMM) at k = 1024 scaled by (k / 1024)^2, times "
                                  "the launches per step of jacobi_fp32, jacobi_df and zgemm_df",
                "units": "launches and traffic per gate step; avg_launch_ms = ms per gate step",
                "pipe_busy": {"kernel": dom, "executed_tflops": executed, "frac_of_ffma": executed / ffma if ffma else None,
                              "sweeps_per_step": st["launches"] / nprof,
                              "avg_sweep_ms": st["ms"] / max(1, st["launches"]),
                              "traffic_per_sweep": (NCU_TRAFFIC_1024.get(dom, 0.0) * (2 * chi / 1024) ** 2) or None,
                              "note": "FP32 instructions the kernel class executes (compensated inner products and "
                                      "rotations) per second, not algorithmic work"},
                "time_share": shares}
    if mp:
        roofline["measured_peaks_json"] = {"hbm_gbs": mp.get("hbm_gbs"), "bf16_tflops": mp.get("bf16_tflops")}

    # ---- CPU baseline (rank 0, bounded sample) and the oracle's spectrum of gate 0 ---------------
    cpu = None
    lam_oracle = None
    if rank == 0 and not args.no_cpu and args.cpu_steps > 0:
        from oracle import chain_oracle as O

        ch = O.from_reference_arrays(arrays)
        b = b0 - 1
        al, ar = ch.sites[b], ch.sites[b + 1]
        lam = np.ones(al.shape[2])
        t3 = time.perf_counter()
        for i in range(args.cpu_steps):
            res = cpu_gate_step(al, ar, lam, gates[i], maxdim)
            if i == 0:
                lam_oracle = res.lam[1].copy()
        dc = time.perf_counter() - t3
        cpu = {"value": args.cpu_steps / dc, "unit": "gate-steps/s", "cores": os.cpu_count(), "kind": "port",
               "sample": f"{args.cpu_steps} gate-steps at chi={chi} (NumPy/LAPACK zgesdd restatement, all host "
                         f"threads)"}

    accuracy = None
    if acc_fp64 is not None:
        lm, zm, bm = acc_mixed
        lf, zf, bf = acc_fp64
        smax = float(lf[0])
        accuracy = {"sample": f"gate 0 on bond ({b0},{b0 + 1}) of the initial state, chi = {chi} both sides",
                    "bond_dim": {"mixed": int(bm), "fp64": int(bf)},
                    "lambda_max_abs_err_mixed_vs_fp64_over_sigma_max":
                        float(np.max(np.abs(lm - lf)) / smax) if lm.size == lf.size else None,
                    "z_local_max_abs_err_mixed_vs_fp64": float(np.max(np.abs(zm - zf))),
                    "z_local_fp64": [float(x.real) for x in zf]}
        if lam_oracle is not None:
            accuracy["bond_dim"]["oracle"] = int(lam_oracle.size)
            for nm, lv in (("mixed", lm), ("fp64", lf)):
                accuracy[f"lambda_max_abs_err_{nm}_vs_oracle_over_sigma_max"] = (
                    float(np.max(np.abs(lv - lam_oracle)) / lam_oracle[0]) if lv.size == lam_oracle.size else None)

    batched = (guarded("batched", lambda: run_batched(args, Q, dist, rank, world), world)
               if (args.batched > 0 and not args.quick) else None)
    if args.batched_full > 0 and not args.quick:
        batched = batched or {}
        batched["full_distribution"] = guarded("batched_full", lambda: run_batched_full(args, Q, dist, rank, world),
                                               world)
    serving = (guarded("serving", lambda: run_serving(args, Q, dist, rank, world), world)
               if (args.serve > 0 and not args.quick) else None)
    mpo_env = guarded("mpo_env", lambda: run_mpo_env(args, Q), world) if (args.mpo_sites > 0 and not args.quick) else None
    tebd = guarded("tebd", lambda: run_tebd(args, Q, local), world) if not (args.no_tebd or args.quick) else None

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "gate-steps/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": 1e3 * dt_max / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None,
                "dtype": "complex64 Jacobi preconditioner + double-float (FP32-pair) theta GEMM, Newton-Schulz, B = A X and Jacobi polish; complex128 gate and results",
                "data": "synthetic",
                "config": {"workload": f"tebd_gate_step_chi{chi}", "chi": chi, "theta": f"{2 * chi}x{2 * chi}",
                           "maxdim": maxdim, "threshold": CUTOFF, "n_sites": N_SITES, "precision": "mixed",
                           "parallelism": "replicas" if world > 1 else "single",
                           "l2": "inputs larger than L2 (>129 MB touched per step)"},
                "fp64": fp64, "mixed_over_fp64": (value / fp64["value"]) if fp64 else None, "accuracy": accuracy,
                "gflop_per_step": gate_flops(chi) / 1e9, "e2e": e2e, "gpu_launches": launches,
                "roofline": roofline, "cpu_baseline": cpu, "clocks": clk,
                "batched": batched, "serving": serving, "mpo_env": mpo_env, "tebd_n64_chi256": tebd}
        print(json.dumps(line), flush=True)


def main():
    args = parse()
    chi = 128 if args.quick else CHI
    if args.impl == "reference":
        run_reference(args, chi)
    else:
        run_ours(args, chi)


if __name__ == "__main__":
    main()
