#!/usr/bin/env python
"""Benchmark of Muscle.jl's binary_einsum on one GB300: ComplexF64 contraction
in the emulated (Ozaki, tcgen05) form versus native FP64 (DMMA).

Workload (precision form): A(i,k1,k2) = 8192x128x64, B(k2,j,k1) = 64x8192x128,
ComplexF64 with log-uniform magnitudes over 2^-20..2^20 and uniform phase
(PCG64 seed 0); the contraction over k1, k2 gives C(i,j) with M = N = K = 8192,
8 M N K = 4.40e12 algorithmic flops. Operands are 1 GiB each, larger than L2,
so no flush is needed between steps.

One JSON line on rank 0:
  value        algorithmic TFLOP/s of the Ozaki form (device-resident inputs)
  e2e          same metric through the public API with host buffers, the
               host->device copies of A, B and the device->host copy of C
               inside the timed region
  native       the plain form (FP64 DMMA) on the same shapes
  rel_err      ||C_ozaki - C_fp64|| / ||C_fp64|| (Frobenius), C_fp64 = plain form
  roofline     the Ozaki GEMM kernel: tensor-pipe flops per launch / its
               CUDA-event duration, against the measured dense bf16 peak
  cpu_baseline the CPU oracle (permute -> OpenBLAS zgemm -> permute) on a
               bounded row sample of the same workload, all host threads

--impl reference times that CPU path alone (the reference's own host path
restated; Muscle.jl itself is Julia, which this machine does not have).
Multi-GPU: each rank runs an independent replica of the workload (the
contraction is not sharded), value = total flops of all ranks / max time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (os.path.join(ROOT, "muscle.jl_gb300", "python"), ROOT):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

METRIC = "C64 einsum TFLOP/s, emulated vs native FP64 @1e-13 rel err; served p50/p99 ms"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--slices", type=int, default=0,
                    help="Ozaki slice count of the headline; 0: adaptive (chosen on the device per call)")
    ap.add_argument("--n", type=int, default=8192, help="M = N of the precision workload")
    ap.add_argument("--native-steps", type=int, default=1)
    ap.add_argument("--cpu-seconds", type=float, default=10.0, help="target CPU work of the baseline sample")
    ap.add_argument("--workload", default="precision",
                    choices=["precision", "peps", "serve", "config2", "kernel", "permute", "hadamard", "unary", "fp64",
                             "blocks", "shortk", "simple_update"],
                    help="precision: the headline line; peps / serve: batching and serving forms; config2: "
                         "plain shapes that permute; kernel / permute: one contraction of the precision "
                         "workload at --n / the permutation of A(a,b,c,d,e) with e = --perm-e (profiling cases); "
                         "hadamard / unary: broadcast product / partial sums of a 4.3 GB array; blocks: the "
                         "precision workload at --n/2 contracted whole and block by block; shortk: 8192 x --k x 8192 "
                         "(GEMM epilogue rate); simple_update: one MPS bond update (contractions, SVD, absorb)")
    ap.add_argument("--form", default="ozaki", help="form of --workload kernel")
    ap.add_argument("--band", type=int, default=0, help="rasterisation band of --workload kernel (0: default)")
    ap.add_argument("--perm-e", type=int, default=32, help="extent of label e in --workload permute")
    ap.add_argument("--k", type=int, default=8, help="contracted extent of --workload shortk")
    ap.add_argument("--chi", type=int, default=0, help="bond dimension of --workload simple_update (0: 16, 32, 64, 128)")
    ap.add_argument("--serve-seconds", type=float, default=1.5, help="per offered rate in the serving sweep")
    ap.add_argument("--instances", type=int, default=4096)
    ap.add_argument("--serve-pool", type=int, default=4096, help="distinct requests of the serving workload")
    return ap.parse_args()


def workload_config(n):
    return {"workload": "precision form: ComplexF64 A(i,k1,k2) x B(k2,j,k1) -> C(i,j)",
            "A": [n, 128, 64], "B": [64, n, 128], "M": n, "N": n, "K": 128 * 64,
            "inputs": "log-uniform |z| in 2^-20..2^20, uniform phase, PCG64 seed 0",
            "l2": "operands 1 GiB each > 129 MB L2; no flush"}


class Clocks:
    """Samples SM clocks and throttle reasons with nvidia-smi while running."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            # the timed region starts once sampling runs (nvidia-smi takes a
            # moment to start), so that its samples cover all of it
            t0 = time.perf_counter()
            while not self.lines and time.perf_counter() - t0 < 3.0:
                time.sleep(0.01)
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
            except ValueError:
                continue
            for nm, v in zip(names, f[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return p["bf16_tflops"], p["hbm_gbs"], "measured"
    except (OSError, KeyError, ValueError):
        return 1900.0, 6800.0, "fallback"


def ncu_traffic(slices):
    """DRAM bytes per launch of the Ozaki GEMM at `slices` slices, from the
    committed ncu summary (lines `traffic_bytes_per_full_launch S=<s>: <bytes>`)."""
    path = os.path.join(ROOT, "profiles", "ozaki_gemm_c64_8192.md")
    key = f"traffic_bytes_per_full_launch S={slices}:"
    try:
        for line in open(path):
            if line.startswith(key):
                return float(line.split(":", 1)[1])
    except OSError:
        pass
    return None


def cpu_sample(n, slices_target_s, seed=0):
    """Times the CPU oracle on the first rows of A (same columns of B)."""
    import oracle.muscle_ref as ref
    from muscle_gb300 import workloads as wl

    rng = np.random.Generator(np.random.PCG64(seed))

    def run(rows):
        a = np.asfortranarray(wl.loguniform_complex(rng, (rows, 128, 64)))
        b = np.asfortranarray(wl.loguniform_complex(rng, (64, n, 128)))
        t0 = time.perf_counter()
        ref.contract(a, ["i", "k1", "k2"], b, ["k2", "j", "k1"], ["i", "j"])
        dt = time.perf_counter() - t0
        return 8.0 * rows * n * 8192 / dt, dt

    rate, _ = run(64)  # calibration (includes B's permutation)
    rows = int(max(64, min(n, rate * slices_target_s / (8.0 * n * 8192))))
    rate, dt = run(rows)
    return {"value": rate / 1e12, "unit": "TFLOP/s", "cores": os.cpu_count(), "kind": "port", "rows": rows,
            "seconds": dt,
            "sample": f"rows i=1..{rows} of A (of {n}), full B; {dt:.1f} s; permute -> OpenBLAS zgemm -> permute"}


def sampled_exact_error(a, ia, b, ib, ic, results, n, count=64, seed=1):
    """Relative error of each result over `count` sampled output entries
    against their correctly rounded values (the oracle's exact dot products:
    the checker, not the measured path)."""
    import oracle.muscle_ref as ref

    rng = np.random.default_rng(seed)
    pos = [tuple(int(x) for x in rng.integers(0, n, size=2)) for _ in range(count)]
    exact = np.array(ref.exact_entries_fast(a, ia, b, ib, ic, pos))
    out = {"entries": count, "reference": "correctly rounded sampled entries (exact dot products)"}
    for name, c in results.items():
        got = np.array([c[p] for p in pos])
        out[name] = float(np.linalg.norm(got - exact) / np.linalg.norm(exact))
    return out


def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if os.environ.get("MGB_BENCH_BACKEND", "nccl") == "nccl" else "gloo")
    return ws, rank, local


def max_over_ranks(x, ws):
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64, device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist

        dist.barrier()


# ----------------------------------------------------------------------------- serving
def _device_requests(n, seed, dev, flops_hi=1e10, req_cap=128 << 20, mem_cap=48 << 30):
    """Serving-form requests with device-resident operands (shapes from the
    seeded generator, values from a seeded device generator). Requests whose
    operands and output exceed `req_cap` bytes (mostly outer products whose
    output is gigabytes for few flops) are redrawn; drawing stops at n
    requests or when the next one would pass `mem_cap` bytes in total.
    Returns the requests and the draw statistics."""
    import torch

    import muscle_gb300 as m
    from muscle_gb300 import workloads as wl

    rng = np.random.default_rng(seed)
    gen = torch.Generator(device=dev)
    gen.manual_seed(seed)
    tdt = {np.complex128: torch.complex128, np.float64: torch.float64, np.complex64: torch.complex64}
    out, used, draws, flops_drawn = [], 0, 0, []
    while len(out) < n:
        sa, ia, sb, ib, ic, dt, fl = wl.serve_request(rng, 1e4, flops_hi)
        draws += 1
        flops_drawn.append(fl)
        ext = dict(zip(ia + ib, sa + sb))
        t = tdt[dt]
        nbytes = int(np.prod(sa) + np.prod(sb) + np.prod([ext[i] for i in ic])) * torch.empty((), dtype=t).element_size()
        if nbytes > req_cap:
            continue
        if used + nbytes > mem_cap:
            break
        used += nbytes
        A = m.Tensor(torch.randn(list(reversed(sa)), dtype=t, device=dev, generator=gen).permute(*reversed(range(len(sa)))), ia)
        B = m.Tensor(torch.randn(list(reversed(sb)), dtype=t, device=dev, generator=gen).permute(*reversed(range(len(sb)))), ib)
        C = m.Tensor(m.empty_colmajor([ext[i] for i in ic], t, dev), ic)
        out.append((A, B, C, fl))
    torch.cuda.synchronize(dev)
    stats = {"draws": draws, "redrawn": draws - len(out), "request_cap_bytes": req_cap, "pool_bytes": used,
             "flops_mean_of_all_draws": float(np.mean(flops_drawn))}
    return out, stats


def serve_bench(dev, rates, seconds, n_requests=4096, seed=5, budget=120 * 10**9, quick=False, streams=4,
                max_batch=256):
    """Serving form: a Poisson stream of distinct seeded requests (each with
    its own operands and output; the backlog stays below the pool size, so
    no two requests in flight share a buffer) served by the continuous
    batching server in the emulated and the plain form, against
    one-at-a-time launches of the same request sequence in each form."""
    import torch

    import muscle_gb300 as m
    from muscle_gb300 import _lib

    def progress(msg):
        print(f"[serve {time.strftime('%H:%M:%S')}] {msg}", file=sys.stderr, flush=True)

    reqs, draw = _device_requests(n_requests, seed, dev, mem_cap=48 << 30)
    progress(f"{len(reqs)} requests generated")
    res = {"requests_in_pool": len(reqs), "flops_mean": float(np.mean([r[3] for r in reqs])),
           "flops_median": float(np.median([r[3] for r in reqs])), "draws": draw, "streams": streams,
           "max_batch": max_batch}
    plans = {}
    for form in ("plain", "auto"):
        plans[form] = [m.contraction_plan(A.data, A.inds, B.data, B.inds, C.data, C.inds, form) for A, B, C, _ in reqs]
    ws = torch.empty(max(max(p.workspace_bytes for p in plans["auto"]), 1), dtype=torch.uint8, device=dev)
    lib = _lib.load()
    st = torch.cuda.current_stream(dev).cuda_stream

    def one_at_a_time(form, budget_s):
        """Launch, wait, next: the same request sequence the server is offered."""
        t0 = time.perf_counter()
        n_done = 0
        while time.perf_counter() - t0 < budget_s or n_done < 8:
            i = n_done % len(reqs)
            A, B, C, _ = reqs[i]
            p = plans[form][i]
            _lib.check(lib.mgb_contract(p.handle, A.data.data_ptr(), B.data.data_ptr(), C.data.data_ptr(),
                                        ws.data_ptr(), ws.numel(), st), lib)
            torch.cuda.synchronize(dev)
            n_done += 1
        return n_done / (time.perf_counter() - t0), n_done

    serial = {}
    for form in ("auto", "plain"):
        rate, cnt = one_at_a_time(form, 0.5 if quick else 2.0)
        serial[form] = {"per_s": rate, "requests": cnt}
        progress(f"one at a time, {form}: {rate:.1f}/s over {cnt} requests")
    res["one_at_a_time"] = {"emulated_per_s": serial["auto"]["per_s"], "plain_per_s": serial["plain"]["per_s"],
                            "requests_timed": {"emulated": serial["auto"]["requests"],
                                               "plain": serial["plain"]["requests"]},
                            "sequence": "requests 0, 1, 2, ... of the pool, the order the server is offered"}
    # Request i + len(reqs) reuses the buffers of request i, so fewer than
    # len(reqs) may be unfinished when it is submitted; the backlog is checked
    # every 64 submissions.
    backlog_cap = len(reqs) - 128
    sweeps = []
    for form in ("auto", "plain"):
        # the native FP64 form saturates far earlier
        form_rates = rates if form == "auto" else [r / 50.0 for r in rates]
        with m.Server(budget_bytes=budget, streams=streams, max_batch=max_batch, form=form, device=dev) as srv:
            for rate in form_rates:
                srv.reset_stats()
                rng = np.random.default_rng(seed + int(rate))
                t_start = time.perf_counter()
                t_next = t_start
                sent, pend = 0, []
                overloaded = False
                while True:
                    now = time.perf_counter()
                    if now - t_start >= seconds:
                        break
                    if now < t_next:
                        continue
                    if sent % 64 == 0 and sent - srv.stats()["completed"] > backlog_cap:
                        overloaded = True  # backlog near the pool size: stop offering
                        break
                    i = sent % len(reqs)
                    A, B, C, _ = reqs[i]
                    pend.append(srv.submit_planned(plans[form][i], A, B, C))
                    sent += 1
                    t_next += rng.exponential(1.0 / rate)
                for q in pend:
                    q.wait(timeout=120.0)  # raises when a request does not finish
                elapsed = time.perf_counter() - t_start
                sts = srv.stats()
                progress(f"{form} at {rate}/s: {sent} sent, {sts['completed']} completed, p99 {sts['p99_ms']:.2f} ms, "
                         f"{sts['batches']} batches")
                flops = sum(reqs[k % len(reqs)][3] for k in range(sent))
                offered_elapsed = min(seconds, elapsed)
                done_rate = sts["completed"] / elapsed
                sweeps.append({"form": "emulated" if form == "auto" else "plain", "offered_per_s": rate,
                               "submitted_per_s": sent / offered_elapsed, "completed_per_s": done_rate,
                               "overloaded": overloaded,
                               "unsaturated": (not overloaded) and done_rate >= 0.95 * sent / offered_elapsed,
                               "tflops": flops / elapsed / 1e12, "p50_ms": sts["p50_ms"], "p99_ms": sts["p99_ms"],
                               "max_ms": sts["max_ms"], "batches": sts["batches"], "requests": sent})
    res["sweep"] = sweeps

    def best(form):
        ok = [x for x in sweeps if x["form"] == form and x["unsaturated"]]
        return max(ok, key=lambda x: x["completed_per_s"]) if ok else None

    res["served_emulated_best"] = best("emulated") or max(
        (x for x in sweeps if x["form"] == "emulated"), key=lambda x: x["completed_per_s"])
    res["served_plain_best"] = best("plain") or max(
        (x for x in sweeps if x["form"] == "plain"), key=lambda x: x["completed_per_s"])
    e, p = res["served_emulated_best"], res["served_plain_best"]
    res["ratios"] = {
        "served_emulated_vs_one_at_a_time_plain": e["completed_per_s"] / serial["plain"]["per_s"],
        "served_emulated_vs_one_at_a_time_emulated": e["completed_per_s"] / serial["auto"]["per_s"],
        "served_plain_vs_one_at_a_time_plain": p["completed_per_s"] / serial["plain"]["per_s"],
        "basis": "highest unsaturated offered rate of each form (completions keep up with >= 95 % of the "
                 "submissions, no backlog stop)"}
    return res


def fp64_peaks(dev, target_ms=40.0):
    """Measured FP64 pipe rates of this GPU (the library's roofline probes):
    DMMA (mma.sync m16n8k16 .f64), DFMA and DADD, each the best over a few
    grid shapes, every launch sized to about `target_ms`."""
    import torch

    from muscle_gb300 import _lib

    lib = _lib.load()
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    scratch = torch.empty(sms * 16 * 1024 * 8, dtype=torch.uint8, device=dev)
    st = torch.cuda.current_stream(dev).cuda_stream
    out = {"sms": sms}
    import ctypes

    for op, name in ((0, "dmma_tflops"), (1, "dfma_tflops"), (2, "dadd_tflops")):
        best = 0.0
        for blocks_per_sm, threads in ((1, 128), (2, 256), (4, 256), (8, 256)):
            blocks = sms * blocks_per_sm
            iters = 64
            r = ctypes.c_double(0.0)
            _lib.check(lib.mgb_probe_fp64(op, iters, blocks, threads, scratch.data_ptr(), scratch.numel(), st,
                                          ctypes.byref(r)), lib)
            # flops of one iteration of the grid, and iterations for target_ms at the first rate
            per_iter = (blocks * threads / 32 * 4 * 4096) if op == 0 else blocks * threads * 8 * (2 if op == 1 else 1)
            iters = int(max(64, r.value * 1e12 * target_ms / 1e3 / per_iter))
            _lib.check(lib.mgb_probe_fp64(op, iters, blocks, threads, scratch.data_ptr(), scratch.numel(), st,
                                          ctypes.byref(r)), lib)
            best = max(best, r.value)
        out[name] = best
    out["how"] = "tight loops of independent chains, CUDA events, best of 1/2/4/8 blocks per SM"
    return out


def _group_phases_ms(dev, g, steps):
    """Device time of a group's two phases, each replayed as its own graph:
    the pre-passes (and plain buckets), then the persistent tensor-core
    launches."""
    import torch

    from muscle_gb300 import _lib

    lib = _lib.load()
    wsp, wsb = g.workspace.data_ptr(), g.workspace_bytes
    out = {}
    for name, fn in (("prepass_and_plain", lambda st: lib.mgb_group_prepare_part(g.handle, 0, 1, wsp, wsb, st)),
                     ("persistent_gemm", lambda st: lib.mgb_group_finish(g.handle, wsp, wsb, st))):
        side = torch.cuda.Stream(dev)
        side.wait_stream(torch.cuda.current_stream(dev))
        with torch.cuda.stream(side):
            _lib.check(fn(side.cuda_stream), lib)
        torch.cuda.current_stream(dev).wait_stream(side)
        torch.cuda.synchronize(dev)
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph):
            _lib.check(fn(torch.cuda.current_stream(dev).cuda_stream), lib)
        graph.replay()
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(steps):
            graph.replay()
        e1.record()
        torch.cuda.synchronize(dev)
        out[name] = e0.elapsed_time(e1) / steps
        del graph
    return out


def peps_bench(dev, instances, cap=1 << 22, seed=10000, steps=5, quick=False, check=0):
    """Batching form: PEPS-style pairs, one group per element type, replayed
    as one CUDA graph whose schedule the autotuner chose on the group's own
    data. quick: no per-class breakdown, a shorter one-at-a-time sample.
    check: members whose results are compared with the CPU oracle (the
    checker) after the timed replays."""
    import torch

    import muscle_gb300 as m
    from muscle_gb300 import workloads as wl
    from muscle_gb300.autotune import Autotuner

    out = {"instances": instances, "cap_elements": cap}
    rng_np = []
    shapes = []
    rej = 0
    for i in range(instances):
        (a, ia), (b, ib), ic, tries = wl.peps_instance(seed + i, cap=cap, dtype=np.complex64)
        shapes.append((a.shape, ia, b.shape, ib, ic))
        rej += tries - 1
    out["redraws_per_instance"] = rej / instances
    gen = torch.Generator(device=dev)
    gen.manual_seed(seed)
    for tdt in (torch.complex128, torch.complex64):
        items, flops = [], 0.0
        for sa, ia, sb, ib, ic in shapes:
            chi = sa[1]
            sc = (1.0 / chi) ** 0.5
            A = m.Tensor((torch.randn(list(reversed(sa)), dtype=tdt, device=dev, generator=gen) * sc).permute(4, 3, 2, 1, 0), ia)
            B = m.Tensor((torch.randn(list(reversed(sb)), dtype=tdt, device=dev, generator=gen) * sc).permute(4, 3, 2, 1, 0), ib)
            ext = dict(zip(ia + ib, sa + sb))
            C = m.Tensor(m.empty_colmajor([ext[x] for x in ic], tdt, dev), ic)
            items.append((C, A, B))
        tuner = Autotuner(os.environ.get("MGB_AUTOTUNE_CACHE"), reps=2)
        g = tuner.group(items)
        flops = g.flops
        # the schedule: (branches, persistent) chosen by the autotuner from
        # the candidates timed on this group; then timed again on its own
        best_parts, by_parts = tuner.schedule(g)
        ms = Autotuner.time_schedule(g, best_parts[0], best_parts[1], steps)
        # the persistent form's two phases on their own: pre-passes (and plain
        # buckets), then the persistent tensor-core launches
        phase_ms = {} if quick else _group_phases_ms(dev, g, steps)
        by_class = []
        errs = []
        if check:
            import oracle.muscle_ref as ref  # the checker

            graph = g.capture()
            graph.replay()
            torch.cuda.synchronize(dev)
            del graph
            for idx in np.linspace(0, len(items) - 1, check).astype(int):
                C, A, B = items[idx]
                want = ref.contract(A.data.cpu().numpy(), [i.tag for i in A.inds], B.data.cpu().numpy(),
                                    [i.tag for i in B.inds], [i.tag for i in C.inds])
                errs.append(ref.rel_fro(C.data.cpu().numpy(), want))
        if tdt == torch.complex128 and not quick:
            # every (M, N, K) class as a group of its own: where the time goes
            classes = {}
            for it, (sa, ia, sb, ib, ic) in zip(items, shapes):
                ext = dict(zip(ia + ib, sa + sb))
                mnk = tuple(int(np.prod([ext[x] for x in lab if x in ext])) for lab in
                            ([x for x in ia if x not in ib], [x for x in ib if x not in ia],
                             [x for x in ia if x in ib and x not in ic]))
                classes.setdefault(mnk, []).append(it)
            for (M, N, K), its in sorted(classes.items(), key=lambda kv: -kv[0][0] * kv[0][1] * kv[0][2] * len(kv[1])):
                gc = m.Group(its, "ozaki")
                ph = _group_phases_ms(dev, gc, 3)
                kb = -(-M // 128) * -(-2 * N // 32) * -(-2 * K // 32) * len(its)
                by_class.append({"M": M, "N": N, "K": K, "members": len(its), "k_blocks": kb, **ph,
                                 "k_blocks_per_ms": kb / ph["persistent_gemm"]})
                del gc
                torch.cuda.empty_cache()
        # one at a time, plain form, on the first instances
        sub = items[:64 if quick else 256]
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        for C, A, B in sub:
            with m.with_backend(m.BackendGB300("plain")):
                m.binary_einsum_(C, A, B)
            torch.cuda.synchronize(dev)
        one = len(sub) / (time.perf_counter() - t0)
        forms = {}
        for f in g.forms:
            forms[f] = forms.get(f, 0) + 1
        key = "c64" if tdt == torch.complex128 else "c32"
        out[key] = {"graph_ms": ms, "graph_branches": best_parts[0], "persistent": best_parts[1],
                    "graph_ms_by_branches": {f"{k[0]}{'p' if k[1] else ''}": v for k, v in by_parts.items()},
                    "persistent_phases_ms": phase_ms, "by_class": by_class,
                    "tflops": flops / (ms / 1e3) / 1e12, "contractions_per_s": len(items) / (ms / 1e3),
                    "one_at_a_time_plain_per_s": one, "forms_chosen": forms, "gflop": flops / 1e9,
                    "distinct_plans": len({id(p) for p in g.plans}),
                    "schedule_chosen_by": "autotuner (timed)" if by_parts else "autotuner cache"}
        if errs:
            out[key]["max_rel_err_vs_oracle"] = max(errs)
            out[key]["members_checked"] = len(errs)
        del g, items
        torch.cuda.empty_cache()
    return out


def config2_bench(dev, steps=3):
    """Plain native FP64/ComplexF64 contractions, and the emulated form beside
    them: (1) A(i,j,k,l) x B(k,m,l,n) -> (i,j,m,n), every extent 32 (the
    reference's own CPU-sized case; B needs a permutation on the host path);
    with index orders that force permutation, (2a) A(a,b,c,d,e) 64x96x64x48x32,
    B(e,c,f,a) 32x64x128x64 -> (b,d,f) and (2b) the MPS bond A(l,p,r) 512x4x512,
    B(r,q,s) 512x4x512 -> (l,p,q,s). Reports the permutation kernel's HBM
    bandwidth on 2a's A (the permute BackendBase does) and each form's time;
    the plain form reads the strided operands directly."""
    import ctypes

    import torch

    import muscle_gb300 as m
    from muscle_gb300 import _lib

    lib = _lib.load()
    stream = torch.cuda.current_stream(dev)
    gen = torch.Generator(device=dev)
    gen.manual_seed(0)
    res = {}
    cases = {"1": (["i", "j", "k", "l"], [32, 32, 32, 32], ["k", "m", "l", "n"], [32, 32, 32, 32],
                   ["i", "j", "m", "n"]),
             "2a": (["a", "b", "c", "d", "e"], [64, 96, 64, 48, 32], ["e", "c", "f", "a"], [32, 64, 128, 64],
                    ["b", "d", "f"]),
             "2b": (["l", "p", "r"], [512, 4, 512], ["r", "q", "s"], [512, 4, 512], ["l", "p", "q", "s"])}

    def colmajor_randn(shape, dt):
        return torch.randn(list(reversed(shape)), dtype=dt, device=dev, generator=gen).permute(
            *reversed(range(len(shape))))

    def timed(fn, reps):
        fn()
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize(dev)
        return e0.elapsed_time(e1) / reps

    for name, (ia, ea, ib, eb, ic) in cases.items():
        for tdt in (torch.complex128, torch.float64):
            A = m.Tensor(colmajor_randn(ea, tdt), ia)
            B = m.Tensor(colmajor_randn(eb, tdt), ib)
            ext = dict(zip(ia + ib, ea + eb))
            row = {}
            outs = {}
            for form in ("plain", "ozaki"):
                C = m.Tensor(m.empty_colmajor([ext[i] for i in ic], tdt, dev), ic)
                plan = m.contraction_plan(A.data, A.inds, B.data, B.inds, C.data, C.inds, form, 7)
                ws = torch.empty(max(plan.workspace_bytes, 1), dtype=torch.uint8, device=dev)

                def run(plan=plan, C=C, ws=ws):
                    _lib.check(lib.mgb_contract(plan.handle, A.data.data_ptr(), B.data.data_ptr(), C.data.data_ptr(),
                                                ws.data_ptr(), ws.numel(), stream.cuda_stream), lib)

                ms = timed(run, 1 if (form == "plain" and name == "2a") else steps)
                row[form] = {"ms": ms, "tflops": plan.flops / (ms / 1e3) / 1e12}
                outs[form] = C.data
                del ws
            row["rel_err_ozaki_vs_plain"] = (torch.linalg.vector_norm((outs["ozaki"] - outs["plain"]).flatten()) /
                                             torch.linalg.vector_norm(outs["plain"].flatten())).item()
            if name == "2a":
                # the permutation BackendBase stages: A(a,b,c,d,e) -> (b,d,a,c,e)
                perm = ["b", "d", "a", "c", "e"]
                Y = m.empty_colmajor([ext[i] for i in perm], tdt, dev)
                modes = {lab: k for k, lab in enumerate(A.inds)}
                (xd, kx) = _lib.make_desc(*m.ops._desc_args(A.data, A.inds, modes))
                (yd, ky) = _lib.make_desc(_lib.C64 if tdt == torch.complex128 else _lib.F64,
                                          tuple(modes[m.Index(i)] for i in perm), tuple(Y.shape), tuple(Y.stride()))

                def perm_run():
                    _lib.check(lib.mgb_permute(ctypes.byref(xd), ctypes.byref(yd), A.data.data_ptr(), Y.data_ptr(),
                                               stream.cuda_stream), lib)

                ms = timed(perm_run, steps)
                nbytes = 2 * A.data.numel() * A.data.element_size()
                _, hbm, kind = peaks()
                row["permute"] = {"ms": ms, "gbs": nbytes / (ms / 1e3) / 1e9, "bytes": nbytes,
                                  "frac_of_hbm": nbytes / (ms / 1e3) / 1e9 / hbm, "peak_kind": kind}
                del Y
            res[f"{name}_{'c64' if tdt == torch.complex128 else 'f64'}"] = row
            del A, B, outs
            torch.cuda.empty_cache()
    return res


def simple_update_bench(dev, steps=20, warmup=3, chis=(16, 32, 64, 128)):
    """Muscle's simple_update (src/Operations/simple_update.jl:35-82) on one
    MPS bond: A(p1, l, b) and B(p2, b, r) ComplexF64 with bond chi, a random
    two-site gate G(p1, p2, q1, q2), truncation to chi, normalisation and an
    equal absorb. Device time per update (CUDA events around `steps` updates
    issued from the host, plan creation included) against the CPU
    restatement of the same update (numpy contractions, LAPACK SVD), and the
    error of the reconstructed two-site tensor against it."""
    import torch

    import muscle_gb300 as m
    from oracle import muscle_ref as ref

    ia, ib, ig = ["p1", "l", "b"], ["p2", "b", "r"], ["p1", "p2", "q1", "q2"]
    kw = dict(maxdim=None, normalize=True, absorb="equally")
    res = {}
    for chi in chis:
        rng = np.random.default_rng(chi)

        def r(shape):
            return np.asfortranarray(rng.standard_normal(shape) + 1j * rng.standard_normal(shape))

        a, b, g = r((2, chi, chi)), r((2, chi, chi)), r((2, 2, 2, 2))
        A, B, G = (m.Tensor(torch.from_numpy(x).to(dev), i) for x, i in ((a, ia), (b, ib), (g, ig)))
        kw["maxdim"] = chi
        for _ in range(warmup):
            m.simple_update(A, "p1", B, "p2", "b", G, "q1", "q2", **kw)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(steps):
            U, V = m.simple_update(A, "p1", B, "p2", "b", G, "q1", "q2", **kw)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / steps
        reps, t0 = 0, time.perf_counter()
        while reps < 3 or (time.perf_counter() - t0 < 1.0 and reps < steps):
            (Uo, lu), (Vo, lv) = ref.simple_update(a, ia, "p1", b, ib, "p2", "b", g, ig, "q1", "q2", **kw)
            reps += 1
        cpu_ms = (time.perf_counter() - t0) / reps * 1e3
        out = ["p1", "l", "p2", "r"]
        got = ref.contract(U.data.cpu().numpy(), lu, V.data.cpu().numpy(), lv, out)
        err = ref.rel_fro(got, ref.contract(Uo, lu, Vo, lv, out))
        # the SVD step alone on the same 2chi x 2chi matrix: this library's
        # Jacobi kernel, and torch.linalg.svd (cuSOLVER) for comparison
        theta = m.Tensor(torch.from_numpy(r((2, chi, 2, chi))).to(dev), ["p1", "l", "p2", "r"])
        reps_svd = 3

        def timed(f):
            f()
            torch.cuda.synchronize()
            e0.record()
            for _ in range(reps_svd):
                f()
            e1.record()
            torch.cuda.synchronize()
            return e0.elapsed_time(e1) / reps_svd

        svd_ms = timed(lambda: m.tensor_svd_thin(theta, ["p1", "l"], ["p2", "r"]))
        mat = theta.data.reshape(2 * chi, 2 * chi)
        lib_ms = timed(lambda: torch.linalg.svd(mat, full_matrices=False))
        res[f"chi{chi}"] = {"theta": [2 * chi, 2 * chi], "ms_per_update": ms, "cpu_ms_per_update": cpu_ms,
                            "cpu_reps": reps, "speedup_vs_cpu": cpu_ms / ms, "rel_err_vs_cpu": err,
                            "svd_ms": svd_ms, "torch_linalg_svd_ms": lib_ms, "status": m.device_status(dev)}
    return {"cpu_baseline": {"kind": "port", "cores": os.cpu_count(),
                             "sample": "the same update through numpy (OpenBLAS) and LAPACK's SVD"},
            "updates": res}


def blocks_bench(dev, n=4096, steps=3, warmup=1):
    """The precision workload at M = N = n (K = 8192) contracted whole and
    block by block (block_einsum: every block pair in one group, partial
    products of contracted-label blocks summed by the unary kernel), TFLOP/s
    of the whole contraction's flops, and the block result's distance from
    the whole one."""
    import torch

    import muscle_gb300 as m
    from muscle_gb300 import workloads as wl

    (a, ia), (b, ib), ic = wl.gen_config3(seed=0, n=n)
    A = m.Tensor(torch.from_numpy(a).to(dev), ia)
    B = m.Tensor(torch.from_numpy(b).to(dev), ib)
    del a, b
    k1 = A.data.shape[ia.index("k1")]  # contracted labels k1, k2 (K = k1 k2)
    splits = {"whole": {}, "K in 4": {"k1": k1 // 4}, "C in 2x2": {"i": n // 2, "j": n // 2},
              "C in 2x2, K in 2": {"i": n // 2, "j": n // 2, "k1": k1 // 2}}
    res, whole = {}, None
    for name, bs in splits.items():
        bc = m.BlockContraction(A, B, bs, out=ic)
        for _ in range(warmup):
            bc.execute()
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(steps):
            bc.execute()
        e1.record()
        torch.cuda.synchronize(dev)
        ms = e0.elapsed_time(e1) / steps
        if whole is None:
            whole = bc.c.data.clone()
            err = 0.0
        else:
            err = float(torch.linalg.norm(bc.c.data - whole) / torch.linalg.norm(whole))
        res[name] = {"ms": ms, "tflops": bc.flops / (ms / 1e3) / 1e12, "members": len(bc.group.items),
                     "reductions": len(bc.reductions), "rel_diff_vs_whole": err}
        del bc
        torch.cuda.empty_cache()
    return {"M": n, "N": n, "K": k1 * A.data.shape[ia.index("k2")], "dtype": "c64", "splits": res}


def kernel_case(dev, n, form, slices, steps, warmup, band=0):
    """One contraction of the precision workload at M = N = n (K = 8192),
    launched warmup + steps times; phase timing from the plan."""
    import ctypes

    import torch

    import muscle_gb300 as m
    from muscle_gb300 import _lib
    from muscle_gb300 import workloads as wl

    (a, ia), (b, ib), ic = wl.gen_config3(seed=0, n=n)
    A = torch.from_numpy(a).to(dev)
    B = torch.from_numpy(b).to(dev)
    del a, b
    C = m.empty_colmajor([n, n], torch.complex128, dev)
    idx = [[m.Index(x) for x in ls] for ls in (ia, ib, ic)]
    p = m.contraction_plan(A, idx[0], B, idx[1], C, idx[2], form, slices)
    ws = torch.empty(max(p.workspace_bytes, 1), dtype=torch.uint8, device=dev)
    lib = _lib.load()
    st = torch.cuda.current_stream(dev).cuda_stream
    lib.mgb_plan_set_timing(p.handle, 1)
    _lib.check(lib.mgb_plan_set_band(p.handle, band), lib)
    pre, main = [], []
    for r in range(warmup + steps):
        _lib.check(lib.mgb_contract(p.handle, A.data_ptr(), B.data_ptr(), C.data_ptr(), ws.data_ptr(), ws.numel(),
                                    st), lib)
        fp, fm = ctypes.c_float(), ctypes.c_float()
        _lib.check(lib.mgb_plan_timing(p.handle, ctypes.byref(fp), ctypes.byref(fm)), lib)
        if r >= warmup:
            pre.append(fp.value)
            main.append(fm.value)
    ms = statistics.mean(main)
    return {"n": n, "form": form, "slices": slices, "band": band, "prepass_ms": statistics.mean(pre), "main_ms": ms,
            "tflops_alg": p.flops / ((statistics.mean(pre) + ms) / 1e3) / 1e12, "status": m.device_status(dev)}


def shortk_case(dev, k, steps, warmup, n=8192, slices=6):
    """C(i,j) = A(i,k) B(k,j), ComplexF64, M = N = n and a short contracted
    extent k: tiles with one or few k blocks, whose time is the GEMM
    epilogue's (profiling case); fixed slice count, phase timing from the plan."""
    import ctypes

    import torch

    import muscle_gb300 as m
    from muscle_gb300 import _lib

    g = torch.Generator(device=dev)
    g.manual_seed(0)
    A = m.empty_colmajor([n, k], torch.complex128, dev)
    A.copy_(torch.randn(n, k, dtype=torch.complex128, device=dev, generator=g))
    B = m.empty_colmajor([k, n], torch.complex128, dev)
    B.copy_(torch.randn(k, n, dtype=torch.complex128, device=dev, generator=g))
    C = m.empty_colmajor([n, n], torch.complex128, dev)
    I = [m.Index(x) for x in ("i", "k", "j")]
    p = m.contraction_plan(A, [I[0], I[1]], B, [I[1], I[2]], C, [I[0], I[2]], "ozaki", slices)
    ws = torch.empty(max(p.workspace_bytes, 1), dtype=torch.uint8, device=dev)
    lib = _lib.load()
    st = torch.cuda.current_stream(dev).cuda_stream
    lib.mgb_plan_set_timing(p.handle, 1)
    pre, main = [], []
    for r in range(warmup + steps):
        _lib.check(lib.mgb_contract(p.handle, A.data_ptr(), B.data_ptr(), C.data_ptr(), ws.data_ptr(), ws.numel(),
                                    st), lib)
        fp, fm = ctypes.c_float(), ctypes.c_float()
        _lib.check(lib.mgb_plan_timing(p.handle, ctypes.byref(fp), ctypes.byref(fm)), lib)
        if r >= warmup:
            pre.append(fp.value)
            main.append(fm.value)
    gemm = statistics.median(main)
    tiles = (n // 128) * (2 * n // 32)
    return {"n": n, "k": k, "slices": slices, "tiles": tiles, "prepass_ms": statistics.median(pre), "gemm_ms": gemm,
            "gemm_cycles_per_tile_per_sm_at_2070mhz": gemm * 1e-3 * 2.07e9 * 152 / tiles,
            "status": m.device_status(dev)}


def permute_case(dev, e, steps, warmup, dtype="c64"):
    """Permutation of A(a,b,c,d,e) = 64x96x64x48xe ComplexF64 (or Float64) to
    (b,d,a,c,e), the reordering the host backend stages for the permuting
    plain shapes."""
    import torch

    import muscle_gb300 as m

    ia, ea = ["a", "b", "c", "d", "e"], [64, 96, 64, 48, e]
    perm = ["b", "d", "a", "c", "e"]
    g = torch.Generator(device=dev)
    g.manual_seed(0)
    tdt = torch.complex128 if dtype == "c64" else torch.float64
    x = torch.randn(list(reversed(ea)), dtype=tdt, device=dev, generator=g).permute(4, 3, 2, 1, 0)
    X = m.Tensor(x, ia)
    for _ in range(warmup):
        Y = m.permutedims(X, perm)
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        Y = m.permutedims(X, perm)
    e1.record()
    torch.cuda.synchronize(dev)
    ms = e0.elapsed_time(e1) / steps
    nb = 2 * x.numel() * x.element_size()
    _, hbm, kind = peaks()
    return {"dtype": dtype, "bytes": nb, "ms": ms, "gbs": nb / (ms / 1e3) / 1e9,
            "frac_of_hbm": nb / (ms / 1e3) / 1e9 / hbm, "peak_kind": kind,
            "bit_exact": bool(torch.equal(Y.data, x.permute(1, 3, 0, 2, 4)))}


def hadamard_case(dev, steps, warmup):
    """hadamard(a, b) of a(x, y) = 2^16 x 2^12 with a vector b(y), the scaling
    step that follows a contraction in a simple update, in ComplexF64 and
    ComplexF32. Algorithmic bytes = read a + write c (+ b). ComplexF64 does 6
    FP64 flops per element (4 instructions with FMA) on GB300's ~1.25 TFLOP/s
    FP64 pipe, so it is bound by that pipe rather than HBM; ComplexF32 is
    HBM-bound."""
    import torch

    import muscle_gb300 as m

    out = {}
    _, hbm, kind = peaks()
    for tdt, name in ((torch.complex128, "c64"), (torch.complex64, "c32")):
        g = torch.Generator(device=dev)
        g.manual_seed(0)
        n0, n1 = 1 << 16, 1 << 12
        a = torch.randn(n1, n0, dtype=tdt, device=dev, generator=g).t()
        b = torch.randn(n1, dtype=tdt, device=dev, generator=g)
        A, B = m.Tensor(a, ["x", "y"]), m.Tensor(b, ["y"])
        C = m.Tensor(m.empty_colmajor([n0, n1], tdt, dev), ["x", "y"])
        for _ in range(warmup):
            m.hadamard_(C, A, B)
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(steps):
            m.hadamard_(C, A, B)
        e1.record()
        torch.cuda.synchronize(dev)
        ms = e0.elapsed_time(e1) / steps
        es = a.element_size()
        nb = 2 * a.numel() * es + b.numel() * es
        want = a * b[None, :]
        tol = 1e-15 if tdt == torch.complex128 else 1e-6
        ok = bool((C.data - want).abs().max().item() <= tol * want.abs().max().item())
        out[name] = {"bytes": nb, "ms": ms, "gbs": nb / (ms / 1e3) / 1e9, "frac_of_hbm": nb / (ms / 1e3) / 1e9 / hbm,
                     "peak_kind": kind, "matches_torch": ok}
        if tdt == torch.complex128:
            out[name]["fp64_tflops"] = 6.0 * a.numel() / (ms / 1e3) / 1e12
        del a, b, A, B, C, want
        torch.cuda.empty_cache()
    return out


def unary_case(dev, steps, warmup):
    """unary_einsum partial sums of a ComplexF64 X(a,b,c) = 4096 x 1024 x 64
    (4.3 GB): over the middle label b (a thread per output, coalesced over a)
    and over the contiguous label a (a warp per output). Fractions are of the
    copy rate: algorithmic bytes = read X + write Y. The Float64 sums run as
    fixed-point integers, bound by the integer ALU pipe short of HBM."""
    import torch

    import muscle_gb300 as m

    g = torch.Generator(device=dev)
    g.manual_seed(0)
    ea = [4096, 1024, 64]
    x = torch.randn(list(reversed(ea)), dtype=torch.complex128, device=dev, generator=g).permute(2, 1, 0)
    X = m.Tensor(x, ["a", "b", "c"])
    _, hbm, kind = peaks()
    out = {}
    for name, keep, dim in (("sum_over_b", ["a", "c"], 1), ("sum_over_a", ["b", "c"], 0)):
        Y = m.Tensor(m.empty_colmajor([ea[["a", "b", "c"].index(i)] for i in keep], torch.complex128, dev), keep)
        for _ in range(warmup):
            m.unary_einsum_(Y, X)
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(steps):
            m.unary_einsum_(Y, X)
        e1.record()
        torch.cuda.synchronize(dev)
        ms = e0.elapsed_time(e1) / steps
        nb = (x.numel() + Y.data.numel()) * 16
        want = x.sum(dim=dim)
        ok = bool((Y.data - want).abs().max().item() <= 1e-12 * want.abs().max().item())
        out[name] = {"bytes": nb, "ms": ms, "gbs": nb / (ms / 1e3) / 1e9, "frac_of_hbm": nb / (ms / 1e3) / 1e9 / hbm,
                     "peak_kind": kind, "matches_torch": ok}
    return out


def run_reference(args, ws, rank):
    if rank != 0:
        return
    cb = cpu_sample(args.n, args.cpu_seconds)
    for _ in range(args.warmup):  # untimed
        cpu_sample(args.n, args.cpu_seconds / 4)
    steps = []
    for _ in range(max(1, args.steps)):
        steps.append(cpu_sample(args.n, args.cpu_seconds / 2))
    val = statistics.median(x["value"] for x in steps)
    # a step is one timed row sample of the contraction (its rows stated)
    step_ms = statistics.median(x["seconds"] for x in steps) * 1e3
    line = {"impl": "reference", "metric": METRIC, "value": val, "unit": "TFLOP/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_ms,
            "ms_per_step_basis": f"one timed row sample ({steps[0]['rows']} of {args.n} rows of A, full B)",
            "full_contraction_ms_at_this_rate": 8.0 * args.n * args.n * 8192 / (val * 1e12) * 1e3,
            "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "c64", "data": "synthetic",
            "config": workload_config(args.n),
            "cpu_baseline": {**cb, "value": val},
            "e2e": {"value": val, "unit": "TFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "CPU restatement of Muscle.jl's BackendBase (Julia is not installed on this machine)"}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    ws, rank, local = dist_init()
    if args.impl == "reference":
        run_reference(args, ws, rank)
        return
    import torch

    import muscle_gb300 as m
    from muscle_gb300 import _lib
    from muscle_gb300 import workloads as wl

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if args.workload != "precision":
        if args.workload == "peps":
            res = peps_bench(dev, args.instances, check=8)
            metric = "PEPS batch: contractions/s and TFLOP/s, one graph-captured group"
        elif args.workload == "config2":
            res = config2_bench(dev)
            metric = "plain vs emulated TFLOP/s on permuting shapes; permutation kernel GB/s"
        elif args.workload == "kernel":
            res = kernel_case(dev, args.n, args.form, args.slices, args.steps, args.warmup, args.band)
            metric = "one contraction of the precision workload (profiling case)"
        elif args.workload == "shortk":
            res = shortk_case(dev, args.k, args.steps, args.warmup)
            metric = "short-K contraction: GEMM epilogue rate (profiling case)"
        elif args.workload == "permute":
            res = {d: permute_case(dev, args.perm_e, args.steps, args.warmup, d) for d in ("c64", "f64")}
            metric = "permutation kernel GB/s (profiling case)"
        elif args.workload == "unary":
            res = unary_case(dev, args.steps, args.warmup)
            metric = "unary_einsum partial sums GB/s"
        elif args.workload == "fp64":
            res = fp64_peaks(dev)
            metric = "measured FP64 pipe rates (roofline probes)"
        elif args.workload == "hadamard":
            res = hadamard_case(dev, args.steps, args.warmup)
            metric = "hadamard (broadcast product) GB/s"
        elif args.workload == "simple_update":
            res = simple_update_bench(dev, max(args.steps, 1), args.warmup,
                                      (args.chi,) if args.chi > 0 else (16, 32, 64, 128))
            metric = "simple_update ms per MPS bond update (ComplexF64) against the CPU restatement"
        elif args.workload == "blocks":
            res = blocks_bench(dev, args.n // 2)
            metric = "block-partitioned contraction TFLOP/s against the whole contraction"
        else:
            res = serve_bench(dev, [1000, 3000, 10000, 30000, 100000], args.serve_seconds, n_requests=args.serve_pool)
            metric = "served contractions/s with p50/p99 ms (Poisson arrivals)"
        if rank == 0:
            print(json.dumps({"metric": metric, "workload": args.workload, "n_gpus": ws, **res}), flush=True)
        return
    n = args.n
    (a, ia), (b, ib), ic = wl.gen_config3(seed=0, n=n)
    # column-major operands as flat pinned host buffers and strided device views
    def flat_pinned(arr):
        return torch.from_numpy(arr.reshape(-1, order="F")).pin_memory()

    def colmajor_view(flat, shape):
        strides, acc = [], 1
        for e in shape:
            strides.append(acc)
            acc *= e
        return flat.as_strided(tuple(shape), tuple(strides))

    a_f, b_f = flat_pinned(a), flat_pinned(b)
    A = colmajor_view(a_f.to(dev), a.shape)
    B = colmajor_view(b_f.to(dev), b.shape)
    C = m.empty_colmajor([n, n], torch.complex128, dev)
    Cn = m.empty_colmajor([n, n], torch.complex128, dev)
    labels = ([m.Index(x) for x in ia], [m.Index(x) for x in ib], [m.Index(x) for x in ic])

    def oz_plan(S, out=C):
        return m.contraction_plan(A, labels[0], B, labels[1], out, labels[2], "ozaki", S)

    pln = m.contraction_plan(A, labels[0], B, labels[1], Cn, labels[2], "plain", 0)
    sweep_s = (5, 6, 7, 8)
    ws_t = torch.empty(max(max(oz_plan(S).workspace_bytes for S in (0,) + sweep_s), 1), dtype=torch.uint8,
                       device=dev)
    lib = _lib.load()
    stream = torch.cuda.current_stream(dev)

    def launch(p, out):
        _lib.check(lib.mgb_contract(p.handle, A.data_ptr(), B.data_ptr(), out.data_ptr(), ws_t.data_ptr(),
                                    ws_t.numel(), stream.cuda_stream), lib)

    def rel(x, y):
        return (torch.linalg.vector_norm((x - y).flatten()) / torch.linalg.vector_norm(y.flatten())).item()

    # native FP64 (DMMA) on the same shapes: the FP64 reference for every error
    launch(pln, Cn)  # warm-up
    torch.cuda.synchronize()
    en0, en1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    en0.record(stream)
    for _ in range(args.native_steps):
        launch(pln, Cn)
    en1.record(stream)
    torch.cuda.synchronize()
    native_ms = en0.elapsed_time(en1) / args.native_steps

    # slice count swept 5..8: time and error of each
    sweep = []
    for S in sweep_s:
        p = oz_plan(S)
        launch(p, C)
        torch.cuda.synchronize()
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        for _ in range(2):
            launch(p, C)
        t1.record(stream)
        torch.cuda.synchronize()
        sms = t0.elapsed_time(t1) / 2
        sweep.append({"slices": S, "ms": sms, "tflops": p.flops / (sms / 1e3) / 1e12, "rel_err": rel(C, Cn)})
    # the headline: the adaptive plan (the library's default), which measures
    # the operands and picks the slice count on the device in every step
    plan = oz_plan(args.slices)
    launch(plan, C)
    torch.cuda.synchronize()
    choice = plan.report(ws_t, stream.cuda_stream) if plan.adaptive else {"slices": args.slices}
    S = choice["slices"]

    def step(p=plan, out=C):
        launch(p, out)

    # End to end through the public API with host buffers: every step copies
    # its inputs from pinned host memory, contracts, and copies the result back
    # (byte-for-byte copies of the column-major arrays as flat buffers).
    # Steps rotate over four device buffer sets. One copy stream carries both
    # directions in order: once step i has computed, its result goes back and
    # then step i + 4's inputs come in, while the next three steps compute
    # (about 15 ms of copies at ~200 GB/s against about 78 ms of compute per
    # step). On the shared GB300 hosts, copies were slowed periodically (a
    # result copy of ~70 ms followed by an input copy of ~130 ms about every
    # half second, instead of 5 and 10 ms); three steps of slack keep such a
    # pair off the critical path. This runs before the device-timed loop and its clock
    # sampler: host copies in the first few hundred milliseconds after
    # nvidia-smi started also ran at a fraction of their usual rate.
    NSET = 4
    cset = []
    for _ in range(NSET):
        af = torch.empty(a_f.numel(), dtype=torch.complex128, device=dev)
        bf = torch.empty(b_f.numel(), dtype=torch.complex128, device=dev)
        cf = torch.empty(n * n, dtype=torch.complex128, device=dev)
        ch = torch.empty(n * n, dtype=torch.complex128).pin_memory()
        cset.append((af, bf, cf, ch))
    cps = torch.cuda.Stream(dev)

    def tev():
        return torch.cuda.Event(enable_timing=True)

    def e2e_run(nsteps, log=None):
        marks = [[tev() for _ in range(6)] for _ in range(nsteps)] if log is not None else None
        ev_in = [torch.cuda.Event() for _ in range(nsteps)]
        ev_comp = [torch.cuda.Event() for _ in range(nsteps)]

        def h2d(i):  # on the copy stream
            af, bf, _, _ = cset[i % NSET]
            if marks:
                marks[i][0].record(cps)
            af.copy_(a_f, non_blocking=True)
            bf.copy_(b_f, non_blocking=True)
            if marks:
                marks[i][1].record(cps)
            ev_in[i].record(cps)

        cps.wait_stream(stream)  # no copy starts before the timer
        with torch.cuda.stream(cps):
            for i in range(min(NSET, nsteps)):
                h2d(i)
        for i in range(nsteps):
            af, bf, cf, ch = cset[i % NSET]
            stream.wait_event(ev_in[i])
            if marks:
                marks[i][2].record(stream)
            _lib.check(lib.mgb_contract(plan.handle, af.data_ptr(), bf.data_ptr(), cf.data_ptr(), ws_t.data_ptr(),
                                        ws_t.numel(), stream.cuda_stream), lib)
            if marks:
                marks[i][3].record(stream)
            ev_comp[i].record(stream)
            cps.wait_event(ev_comp[i])
            with torch.cuda.stream(cps):
                if marks:
                    marks[i][4].record(cps)
                ch.copy_(cf, non_blocking=True)
                if marks:
                    marks[i][5].record(cps)
                if i + NSET < nsteps:
                    h2d(i + NSET)  # into the set step i has finished with
        stream.wait_stream(cps)
        if log is not None:
            log.extend(marks)

    e2e_run(3)
    torch.cuda.synchronize()
    barrier(ws)
    ee0, ee1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    # at least twenty steps, so that the first inputs' copy and the last
    # result's copy (outside the pipeline's overlap) weigh a twentieth of the
    # total or less
    e2e_steps = max(args.steps, 20)
    e2e_log = []
    ee0.record(stream)
    e2e_run(e2e_steps, e2e_log)
    ee1.record(stream)
    torch.cuda.synchronize()
    e2e_ms = max_over_ranks(ee0.elapsed_time(ee1), ws)
    # per step: the host->device copies, the contraction and the device->host
    # copy, each timed on its own stream
    e2e_phases = {name: [round(mk[2 * j].elapsed_time(mk[2 * j + 1]), 3) for mk in e2e_log]
                  for j, name in enumerate(("h2d_ms", "contract_ms", "d2h_ms"))}
    e2e = plan.flops * ws * e2e_steps / (e2e_ms / 1e3) / 1e12
    # the last step's host copy (what the caller receives) against the device-timed result
    e2e_ok = bool(torch.equal(cset[(e2e_steps - 1) % NSET][3].view(n, n), C.t().cpu()))
    del cset
    torch.cuda.empty_cache()

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    barrier(ws)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks(local) as clk:
        e0.record(stream)
        for _ in range(args.steps):
            step()
        e1.record(stream)
        torch.cuda.synchronize()
    ms = max_over_ranks(e0.elapsed_time(e1), ws)
    barrier(ws)
    flops = plan.flops
    value = flops * ws * args.steps / (ms / 1e3) / 1e12
    # kernels of one adaptive step: 2 exponent scans, 2 statistics passes, the
    # estimate and the choice, 2 slicers, then one tcgen05 GEMM per candidate
    # slice count (5-8 at 1e-13) and the plain DMMA candidate, of which all but
    # the chosen one return at once (plus 3 memsets)
    launches_per_step = 2 + 2 + 1 + 1 + 2 + 4 + 1

    # kernel timing for the roofline: phase events around the GEMM launch
    lib.mgb_plan_set_timing(plan.handle, 1)
    pre, mainv = [], []
    import ctypes

    for _ in range(args.steps):
        step()
        fp, fm = ctypes.c_float(), ctypes.c_float()
        _lib.check(lib.mgb_plan_timing(plan.handle, ctypes.byref(fp), ctypes.byref(fm)), lib)
        pre.append(fp.value)
        mainv.append(fm.value)
    lib.mgb_plan_set_timing(plan.handle, 0)
    gemm_ms = statistics.mean(mainv)
    pairs = S * (S + 1) // 2
    tensor_flops = 2.0 * pairs * n * (2 * n) * (2 * 8192)
    bf16_peak, hbm_peak, peak_kind = peaks()
    achieved = tensor_flops / (gemm_ms / 1e3) / 1e12
    traffic = ncu_traffic(S)
    # pre-pass bytes: both operands read by the exponent scan and again by the
    # slicer, S bf16 digit planes written (A: M x 2K, B embedded: 2N x 2K)
    prepass_bytes = 2.0 * (A.numel() + B.numel()) * 16 + S * 2.0 * (n * 2 * 8192 + 2 * n * 2 * 8192)
    prepass_ms = statistics.mean(pre)

    native = flops / (native_ms / 1e3) / 1e12
    fp64 = fp64_peaks(dev, target_ms=20.0)
    step()
    torch.cuda.synchronize()
    rel_err = rel(C, Cn)
    if plan.adaptive:
        choice = plan.report(ws_t, stream.cuda_stream)
    # checker: correctly rounded values of sampled entries (the oracle's exact
    # dot products) against the emulated and the native results
    C_host, Cn_host = C.cpu().numpy(), Cn.cpu().numpy()
    exact_check = sampled_exact_error(a, ia, b, ib, ic, {"emulated": C_host, "native_fp64": Cn_host}, n)
    del C_host, Cn_host

    # Float32 variant (ComplexF32, BF16x3) on the same shapes; its FP64
    # reference is the plain form on the same rounded inputs
    A32, B32 = A.to(torch.complex64), B.to(torch.complex64)
    C32 = m.empty_colmajor([n, n], torch.complex64, dev)
    p32 = m.contraction_plan(A32, labels[0], B32, labels[1], C32, labels[2], "bf16x3", 0)
    ws32 = torch.empty(max(p32.workspace_bytes, 1), dtype=torch.uint8, device=dev)

    def run32():
        _lib.check(lib.mgb_contract(p32.handle, A32.data_ptr(), B32.data_ptr(), C32.data_ptr(), ws32.data_ptr(),
                                    ws32.numel(), stream.cuda_stream), lib)

    run32()
    torch.cuda.synchronize()
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f0.record(stream)
    for _ in range(args.steps):
        run32()
    f1.record(stream)
    torch.cuda.synchronize()
    ms32 = f0.elapsed_time(f1) / args.steps
    A.copy_(A32)
    B.copy_(B32)
    launch(pln, Cn)
    torch.cuda.synchronize()
    f32 = {"form": "bf16x3", "dtype": "c32", "ms_per_step": ms32, "value": p32.flops / (ms32 / 1e3) / 1e12,
           "unit": "TFLOP/s", "rel_err": rel(C32.to(torch.complex128), Cn),
           "rel_err_reference": "plain FP64 DMMA on the ComplexF32 inputs widened"}
    del A32, B32, C32, ws32

    # batching form: a PEPS group of 1024 instances (the full one is --workload peps)
    peps = peps_bench(dev, 1024, quick=True, check=8)
    torch.cuda.empty_cache()
    # block-partitioned form of the same workload at half the output extents
    blocks = blocks_bench(dev, n // 2)
    torch.cuda.empty_cache()

    # served mixed-size stream (short sweep; the full one is --workload serve)
    del a_f, b_f
    torch.cuda.empty_cache()
    # 4096 distinct requests: at 30 k/s with tens of ms in flight, a smaller
    # pool fills its backlog cap before the rate is measured
    serving = serve_bench(dev, [1000, 3000, 10000, 30000, 100000], 1.0, n_requests=4096, quick=True)

    status = m.device_status(dev)
    cpu = None
    if rank == 0 and ws == 1:
        cpu = cpu_sample(n, args.cpu_seconds)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "c64", "data": "synthetic", "config": workload_config(n),
            "form": f"ozaki, slice count {'adaptive' if plan.adaptive else 'fixed'}: S={S} (bf16 digits of "
                    f"{8 if S <= 6 else 7} bits on tcgen05.mma kind::f16, exact int accumulation)",
            "adaptive_choice": choice,
            "rel_err": rel_err, "rel_err_reference": "plain FP64 DMMA result on the same inputs",
            "rel_err_vs_exact": exact_check,
            "slice_sweep": sweep, "float32_variant": f32,
            "native": {"value": native, "unit": "TFLOP/s", "ms_per_step": native_ms, "form": "plain FP64 DMMA (4M)",
                       "fp64_peaks_measured": fp64, "frac_of_dmma_peak": native / fp64["dmma_tflops"]},
            "speedup_vs_native": value / native,
            "e2e": {"value": e2e, "unit": "TFLOP/s", "ms_per_step": e2e_ms / e2e_steps, "steps": e2e_steps,
                    "h2d_bytes_per_step": A.numel() * 16 + B.numel() * 16, "d2h_bytes_per_step": C.numel() * 16,
                    "pipelined": "result of step i, then inputs of step i + 4, on one copy stream while the next "
                                 "three steps compute (four buffer sets)",
                    "result_matches_device_run": e2e_ok, "phases": e2e_phases},
            "roofline": {"bound": "tensor", "achieved": achieved, "peak": bf16_peak, "unit": "TFLOP/s",
                         "frac": achieved / bf16_peak, "traffic": traffic, "peak_kind": f"bf16 dense burst ({peak_kind})",
                         "kernel": "k_oz_gemm", "kernel_ms": gemm_ms, "prepass_ms": prepass_ms,
                         "prepass_bytes": prepass_bytes, "prepass_gbs": prepass_bytes / (prepass_ms / 1e3) / 1e9,
                         "prepass_frac_of_hbm": prepass_bytes / (prepass_ms / 1e3) / 1e9 / hbm_peak,
                         "work": f"2 x {pairs} slice pairs x M x 2N x 2K bf16 flops per launch"},
            "serving": {"p50_ms": serving["served_emulated_best"]["p50_ms"],
                        "p99_ms": serving["served_emulated_best"]["p99_ms"],
                        "completed_per_s": serving["served_emulated_best"]["completed_per_s"],
                        "offered_per_s": serving["served_emulated_best"]["offered_per_s"],
                        "one_at_a_time": serving["one_at_a_time"],
                        "ratios": serving["ratios"],
                        "requests_in_pool": serving["requests_in_pool"],
                        "sweep": serving["sweep"]},
            "batching": {k: {kk: peps[k][kk] for kk in ("graph_ms", "graph_branches", "persistent", "tflops",
                                                          "contractions_per_s", "one_at_a_time_plain_per_s",
                                                          "max_rel_err_vs_oracle", "members_checked", "forms_chosen",
                                                          "graph_ms_by_branches")}
                         for k in ("c64", "c32")} | {"instances": peps["instances"],
                                                     "redraws_per_instance": peps["redraws_per_instance"],
                                                     "cap_elements": peps["cap_elements"]},
            "blocks": blocks,
            "gpu_launches": launches_per_step * args.steps,
            "device_status": status,
            "clocks": clk.summary(),
        }
        if cpu:
            line["cpu_baseline"] = cpu
        print(json.dumps(line), flush=True)
    if ws > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
