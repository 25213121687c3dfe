"""Benchmark: single large PRP test, degree D = 2^16, b uniform in [2^20, 2^21).

One step = one Gerbicz-Li block of the Fermat test: B_GL squarings of the real
exponent bits (one resident-kernel launch: the residue stays in the shared
memory of a 64-CTA cooperative grid) followed by the Gerbicz-Li multiply
d <- d * x, exactly the work cyclo::check does between two checkpoints
(cyclo/src/cyclo.h:277-308).

  value  squarings/s with the residue and exponent resident in HBM (CUDA events
         on the engine's stream, per step, L2 flushed between steps)
  e2e    same metric through the C ABI with host buffers: per step the exponent
         slice is copied host->device and the residue read back device->host
  roofline  32-bit integer multiply-add work per launch (4 IMAD per Montgomery
         multiply, P (D log2 D + 3 D) multiplies per squaring for P NTT primes:
         P = 2 when b keeps the product exact in two primes, as here, else 3)
         / launch time, against the IMAD throughput probed on the same GPU in this run
  cpu_baseline  the oracle's C restatement of the reference transform (the
         reference has no CPU PRP path), one candidate per host core

Two more workloads print their own line (not the default):
  --workload batch  4096 candidates of degree 2^k, k uniform in {12..15}, b uniform in
         [2^16, 2^22) seed 3, resident in one pool per degree and prime class (b within
         the degree's two-prime bound or above it), driven by one batch: one step = one
         tick (B squarings + the Gerbicz-Li multiply of every candidate), the squarings
         of all degrees in one persistent launch with per-degree work queues; CSIZE
         and CTAs per SM autotuned; compared per degree with the plain
         one-candidate-per-launch-sequence path
  --workload sieve  sieved b/s of the GPU sieve on n = 20, b < 2^30, p < 2^40 (and the
         n = 11 both-form sieve of b in [10^5, 3 10^5) to 2^32 beside it)
  --workload config1  the reference's workflow at n = 11: sieve b in [10^5, 3 10^5) to
         2^32 (both forms), then base-3 PRP of every survivor and of its twin partner N-
  --workload serve  a seeded Poisson stream of full PRP tests, degree 2^k with k
         log-uniform in [12, --serve-max-degree], b uniform in [2^16, 2^24), through the
         server (continuous batching by degree, admission by pool bytes; degrees 2^16
         and up in its grid lane); tests/s and p50/p99 latency per degree, beside the
         plain path run for real on the first arrivals (one test at a time)

python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference] [--workload single|batch|serve]
"""
from __future__ import annotations

import argparse
import json
import math
import os
import random
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

LOG2_D = 16
B_LO, B_HI = 2 ** 20, 2 ** 21
SEED = 1
METRIC = "PRP squarings/s"
UNIT = "squarings/s"


def exponent(b: int, ln: int) -> int:
    d = 1 << ln
    h = b ** (d // 2)
    return h * h - h


def workload(rank: int):
    rng = random.Random(SEED + 1000003 * rank)
    b = rng.randrange(B_LO, B_HI)
    E = exponent(b, LOG2_D)
    i0 = E.bit_length() - 1
    L = 2 << ((i0.bit_length() - 1) // 2)
    B_GL = (i0 - 1) // L + 1
    words = np.frombuffer(E.to_bytes((E.bit_length() + 31) // 32 * 4, "little"), dtype=np.uint32).copy()
    return b, E, i0, B_GL, words


TRAFFIC_PER_LAUNCH = 2.62e6     # ncu dram read+write bytes of one 651-squaring launch at 2^16 (64-CTA grid)
TRAFFIC_SOURCE = ("ncu dram__bytes_read.sum + dram__bytes_write.sum of one 651-squaring launch of the "
                  "default split (profiles/prp_kernel_grid2_d65536_full.md)")


def hbm_line(traffic: float, seconds: float) -> dict:
    """Achieved DRAM GB/s beside the measured copy bandwidth (MEASURED_PEAKS.json)."""
    peak = None
    try:
        peak = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))).get("hbm_gbs")
    except (OSError, ValueError):
        pass
    ach = traffic / seconds / 1e9
    return {"achieved_gbs": ach, "peak_gbs": peak, "frac": ach / peak if peak else None,
            "peak_source": "MEASURED_PEAKS.json" if peak else None}


def imad_per_squaring(D: int, primes: int = 3) -> float:
    """4 IMAD per modular multiply; per NTT prime D log2 D + 3 D multiplies per squaring
    (three primes: 4 (3 D log2 D + 9 D), the algorithmic count of one squaring)."""
    return 4.0 * primes * (D * math.log2(D) + 3 * D)


def roofline_single(achieved, executed, peak_imad, peak_mont, peak_shoup, t_launch, geo, sms, have_traffic):
    """Roofline of the resident squaring launch.  achieved: algorithmic IMAD/s
    (three-prime count); executed: the same count for the primes run.  The
    denominators are probes run in this process: plain 32-bit IMAD chains, and
    Montgomery / Shoup modular-product chains (4 IMAD-equivalents each, the
    count's charge per modular multiply)."""
    fr = {}
    for wname, w in (("algorithmic", achieved), ("executed_primes", executed)):
        fr[wname] = {"vs_imad_probe": w / peak_imad if peak_imad else None,
                     "vs_montgomery_probe": w / (4 * peak_mont) if peak_mont else None,
                     "vs_shoup_probe": w / (4 * peak_shoup) if peak_shoup else None}
    used = geo["ctas_per_lane"]
    out = {"bound": "imad", "achieved": achieved / 1e12, "peak": peak_imad / 1e12, "unit": "T IMAD/s",
           "frac": achieved / peak_imad if peak_imad else None,
           "traffic": TRAFFIC_PER_LAUNCH if have_traffic else None,
           "traffic_source": TRAFFIC_SOURCE,
           "peak_source": "32-bit IMAD probe kernel run on this GPU in this process",
           "fractions": fr,
           "peaks": {"imad_per_s": peak_imad, "montgomery_products_per_s": peak_mont,
                     "shoup_products_per_s": peak_shoup},
           "executed_t_imad_per_s": executed / 1e12,
           "sms_used": used, "sms": sms,
           "frac_of_used_sms": (achieved / peak_imad) * sms / used if peak_imad else None,
           "kernel_ms": t_launch * 1000.0,
           "hbm": hbm_line(TRAFFIC_PER_LAUNCH, t_launch) if have_traffic else None}
    return out


def secondary():
    """Other workloads, timed in the same process so that one bench line carries
    them: batched over plain at degrees 2^12..2^14 (256 candidates per degree,
    b uniform in [2^16, 2^22) seed 3, one batch tick against the one-candidate
    launch sequence), one pass of the large sieve (n = 20, b < 2^30, p < 2^40)
    and the n = 11 sieve of b in [10^5, 3 10^5) to 2^32, both forms."""
    import torch
    from ctwin_gb300 import Batch, sieve_pass
    out = {"batched_over_plain": {}}
    rng = random.Random(3)
    t_start = time.perf_counter()
    for k in (12, 13, 14):
        bs = [rng.randrange(1 << 16, 1 << 22) for _ in range(256)]
        pools = batch_pools({(k, 2): bs}, 16)
        p = pools[(k, 2)]
        with Batch([p]) as bt:
            bt.run(1)
            torch.cuda.synchronize()
            batched = statistics.median(batch_tick_rate(bt, [p]) for _ in range(3))
        p.close()
        plain = plain_rate(k, bs[0])
        out["batched_over_plain"][str(k)] = {"candidates": len(bs), "batched_sq_per_s": batched,
                                             "plain_sq_per_s": plain, "ratio": batched / plain,
                                             "path": "batch of one pool (persistent launch), CSIZE 16"}
    n, b_min, b_max = 20, 2, (1 << 30) - 1
    sieve_pass(n, b_min, b_max, 3 * (1 << n) + 1, 1 << 40, 1)
    t0 = time.perf_counter()
    struck, p_last = sieve_pass(n, b_min, b_max, 3 * (1 << n) + 1, 1 << 40, 1)
    t4 = time.perf_counter() - t0
    out["large_sieve"] = {"workload": "n = 20, b in [2, 2^30), p < 2^40, + form, one pass through the C ABI "
                                      "(bitmap copied in and out)", "seconds": t4,
                          "sieved_b_per_s": (b_max - b_min + 1) / t4, "p_last": p_last}
    c1 = {}
    for name, mode, pmn in (("pos", 1, 3 * 2048 + 1), ("neg", -1, 11)):
        sieve_pass(11, 100000, 299999, pmn, 1 << 32, mode)
        t0 = time.perf_counter()
        sieve_pass(11, 100000, 299999, pmn, 1 << 32, mode)
        c1[name] = time.perf_counter() - t0
    out["n11_sieve_s"] = c1
    out["seconds"] = time.perf_counter() - t_start
    return out


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
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
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------
# CPU arm: the oracle's restatement of the reference transform
# ---------------------------------------------------------------------------

def single_config(world: int = 1) -> dict:
    """The single-test workload's config, the same in both arms."""
    b, E, i0, B_GL, _ = workload(0)
    return {"workload": f"single large PRP, degree 2^{LOG2_D} (N = b^{1 << LOG2_D} - b^{1 << (LOG2_D - 1)} + 1), "
                        "b uniform in [2^20, 2^21) seed 1, Fermat base 3, one candidate per launch sequence",
            "degree": 1 << LOG2_D, "b": b, "base": 3, "seed": SEED, "exponent_bits": i0 + 1,
            "squarings_per_step": B_GL, "step": "one Gerbicz-Li block: B_GL resident squarings + one multiply",
            "l2": "flushed between steps (256 MiB write)", "parallelism": f"replicas{world}"}


def cpu_squarings_per_s(threads: int, seconds: float = 12.0):
    """Every host thread squares its own copy of the workload's candidate (b of
    seed 1, base 3) from the exponent's top bit; bounded sample."""
    from oracle import oracle as O
    O.build()
    per = [0] * threads
    stop = time.perf_counter() + seconds
    tabs = O.Tables(LOG2_D)
    lock = threading.Lock()

    def work(t):
        b, E, i0, _, words = workload(0)
        x = np.zeros(1 << LOG2_D, dtype=np.int32)
        x[0] = 1
        i = i0
        n = 0
        while time.perf_counter() < stop:
            tabs.square_loop(x, b, 3, 16, words, i, 4)        # Fermat base 3
            i -= 4
            n += 4
        with lock:
            per[t] = n

    t0 = time.perf_counter()
    th = [threading.Thread(target=work, args=(t,)) for t in range(threads)]
    for x in th:
        x.start()
    for x in th:
        x.join()
    dt = time.perf_counter() - t0
    tabs.close()
    total = sum(per)
    return total / dt, {"value": total / dt, "unit": UNIT, "cores": threads, "kind": "port",
                        "sample": f"{threads} copies of the degree-2^{LOG2_D} candidate (one per thread), "
                                  f"{total} squarings in {dt:.1f} s with the oracle C restatement"}


def run_reference(args, rank, world):
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    # one sample over all steps: 12 s at least (thread start-up is noise below that)
    total = args.cpu_seconds if args.cpu_seconds > 0 else min(120.0, max(12.0, 0.5 * max(1, args.steps)))
    v, cb = cpu_squarings_per_s(threads, seconds=total)
    b, E, i0, B_GL, _ = workload(0)
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 * B_GL / v, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
            "impl": "reference",
            "config": single_config(world),
            "cpu_baseline": cb,
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


# ---------------------------------------------------------------------------
# Batched and served workloads
# ---------------------------------------------------------------------------

def gl_block(i0: int) -> int:
    L = 2 << ((i0.bit_length() - 1) // 2)
    return (i0 - 1) // L + 1


def plain_rate(ln: int, b: int, reps: int = 2):
    """Plain path: one candidate per launch sequence, default split, CSIZE 8:
    squarings/s over Gerbicz-Li blocks (B squarings + the multiply)."""
    import torch
    from ctwin_gb300 import PrpEngine
    from ctwin_gb300._native import check, lib, ptr
    L = lib()
    E = exponent(b, ln)
    i0 = E.bit_length() - 1
    B = gl_block(((20 << ln) - 1))
    words = np.frombuffer(E.to_bytes((E.bit_length() + 31) // 32 * 4, "little"), dtype=np.uint32).copy()
    with PrpEngine(ln, 1) as eng:
        eng.set_b([b])
        eng.set(1)
        eng.copy(1, 0)
        check(L.ctw_prp_load_exponent(eng._h, ptr(words), words.size))
        st = torch.cuda.ExternalStream(eng.stream)
        i = i0
        check(L.ctw_prp_square_resident(eng._h, i, B))
        eng.sync()
        ts = []
        for _ in range(reps):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(st)
            check(L.ctw_prp_square_resident(eng._h, i, B))
            check(L.ctw_prp_mul_regs(eng._h, 1, 0, 1))
            e1.record(st)
            e1.synchronize()
            ts.append(e0.elapsed_time(e1) / 1000.0)
            i -= B
        eng.sync()
    return (B + 1) / statistics.median(ts)


def batch_pools(groups, csize):
    """One pool per (degree, prime class) on CTAs of 4096 coefficients, slots
    rounded up to whole work items, every b admitted."""
    from ctwin_gb300 import Pool
    pools = {}
    for c, bl in groups.items():
        lg = c[0] - 12
        unit = 8 >> lg
        slots = (len(bl) + unit - 1) // unit * unit
        pools[c] = Pool(c[0], slots, log2_ctas=lg, csize=csize)
        assert pools[c].admit_many(bl) == len(bl)
    return pools


def batch_tick_rate(bt, pools, ticks: int = 1):
    """Squarings per second of `ticks` batch ticks, CUDA events on the batch's stream."""
    import torch
    st = torch.cuda.ExternalStream(bt.stream)
    sq = sum(p.info()["active"] * (p.info()["gl_block"] + 1) for p in pools) * ticks
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    bt.run(ticks)
    e1.record(st)
    e1.synchronize()
    return sq / (e0.elapsed_time(e1) / 1000.0)


def run_batch(args):
    import torch
    from ctwin_gb300 import Batch, two_primes
    from ctwin_gb300._native import lib
    L = lib()
    rng = random.Random(3)
    N = args.candidates
    ks = [rng.choice((12, 13, 14, 15)) for _ in range(N)]
    bs = [rng.randrange(1 << 16, 1 << 22) for _ in range(N)]
    # one pool per (degree, prime class): b within the degree's two-prime bound,
    # or above it ("w": three primes)
    cls = [(k, 2 if two_primes(k, b) else 3) for k, b in zip(ks, bs)]
    groups = {}
    for c, b in zip(cls, bs):
        groups.setdefault(c, []).append(b)
    groups = dict(sorted(groups.items()))
    name = {c: f"{c[0]}" + ("" if c[1] == 2 else "w") for c in groups}
    # autotune (CSIZE, CTAs per SM of the batch kernel) on a sample of 64 candidates per class
    t0 = time.perf_counter()
    sample = {c: bl[:64] for c, bl in groups.items()}
    tune = []
    for cs in (8, 16, 32):
        pools = batch_pools(sample, cs)
        for occ in (2, 1):
            with Batch(list(pools.values()), ctas_per_sm=occ) as bt:
                bt.run(1)
                torch.cuda.synchronize()
                tune.append((batch_tick_rate(bt, list(pools.values())), cs, occ))
        for p in pools.values():
            p.close()
    _, csize, occ = max(tune)
    t_tune = time.perf_counter() - t0
    t0 = time.perf_counter()
    pools = batch_pools(groups, csize)
    t_admit = time.perf_counter() - t0
    plist = list(pools.values())
    info = {c: p.info() for c, p in pools.items()}
    sq_per_step = {c: info[c]["active"] * (info[c]["gl_block"] + 1) for c in pools}
    peak_imad = L.ctw_imad_peak()
    bt = Batch(plist, ctas_per_sm=occ)
    st = torch.cuda.ExternalStream(bt.stream)
    for _ in range(args.warmup):
        bt.run(1)
    torch.cuda.synchronize()
    times = []
    launches0 = bt.launches
    with ClockSampler(0) as clk:
        torch.cuda.synchronize()
        for _ in range(args.steps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            bt.run(1)
            e1.record(st)
            e1.synchronize()
            times.append(e0.elapsed_time(e1) / 1000.0)
        torch.cuda.synchronize()
    persistent = bt.launches - launches0
    t_dev = sum(times)
    total_sq = sum(sq_per_step.values()) * args.steps
    value = total_sq / t_dev
    imad = sum(sq_per_step[c] * imad_per_squaring(1 << c[0], 3) for c in pools) * args.steps / t_dev
    imad_exec = sum(sq_per_step[c] * imad_per_squaring(1 << c[0], c[1]) for c in pools) * args.steps / t_dev

    # e2e through the public API: host planning + graph launch + collect per step (wall clock)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        bt.run(1)
        for p in plist:
            p.collect(wait=True)
    t_e2e = time.perf_counter() - t0
    bt.close()
    h2d = sum(info[c]["slots"] * 2 * 8 + info[c]["slots"] * ((info[c]["gl_block"] + 31) // 32) * 4 for c in pools)
    # per degree: the pool alone in a batch of its own vs the plain path (one candidate per launch sequence)
    per_degree = {}
    for c, p in pools.items():
        with Batch([p], ctas_per_sm=occ) as b1:
            alone = batch_tick_rate(b1, [p])
        plain = plain_rate(c[0], groups[c][0])
        bits = (1 << c[0]) * statistics.mean(math.log2(b) for b in groups[c])
        per_degree[name[c]] = {"candidates": len(groups[c]), "gl_block": info[c]["gl_block"], "ntt_primes": c[1],
                               "b_range": [min(groups[c]), max(groups[c])],
                               "batched_alone_sq_per_s": alone, "plain_sq_per_s": plain,
                               "batched_over_plain": alone / plain,
                               "tests_per_s_projected": alone / bits, "plain_tests_per_s_projected": plain / bits}
    for p in plist:
        p.close()
    # residues: the first candidate of every class of degree 2^12 and 2^13 run
    # to completion in a batch of its own, against the same test on the plain
    # engine (PrpEngine.run, another launch path); tolerance 0
    from ctwin_gb300 import PrpEngine
    vpools = batch_pools({c: bl[:1] for c, bl in groups.items() if c[0] <= 13}, csize)
    with Batch(list(vpools.values()), ctas_per_sm=occ) as bv:
        vres = bv.run_to_completion()
    for p in vpools.values():
        p.close()
    for r in vres:
        with PrpEngine(r["log2_degree"], 1) as eng:
            prp, r64, gl = eng.run([r["b"]])
        if not (r["status"] == 0 and r["gl_ok"] and gl[0] and (r["is_prp"], r["res64"]) == (bool(prp[0]), int(r64[0]))):
            raise SystemExit(f"batch result differs from the engine's for b={r['b']} at 2^{r['log2_degree']}")
    line = {
        "metric": "PRP squarings/s (batched, uneven degrees)", "value": value, "unit": "squarings/s",
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * t_dev / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": {"workload": f"{N} candidates, degree 2^k with k uniform in {{12..15}}, b uniform in [2^16, 2^22) "
                               "seed 3, one pool per degree and prime class (b within the two-prime bound, or "
                               "above it: 'w'), all driven by one batch: per tick one persistent launch of every "
                               "pool's squarings (per-degree work queues) and one of every multiply",
                   "l2": "inputs larger than L2 (registers of all candidates resident)",
                   "autotune": {"csize": csize, "ctas_per_sm": occ,
                                "tried": [{"sq_per_s": r, "csize": c_, "ctas_per_sm": o} for r, c_, o in tune]},
                   "setup_s": {"autotune": t_tune, "admit": t_admit}},
        "per_degree": per_degree,
        "e2e": {"value": total_sq / t_e2e, "unit": "squarings/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": 0},
        "roofline": {"bound": "imad", "achieved": imad / 1e12, "peak": peak_imad / 1e12, "unit": "T IMAD/s",
                     "frac": imad / peak_imad if peak_imad else None, "traffic": None,
                     "executed_t_imad_per_s": imad_exec / 1e12,
                     "frac_executed_primes": imad_exec / peak_imad if peak_imad else None,
                     "peak_source": "32-bit IMAD probe kernel run on this GPU in this process"},
        "cpu_baseline": None, "gpu_launches": persistent + 2 * len(plist) * args.steps,
        "persistent_launches": persistent, "clocks": clk.summary(),
        "verified": {"tests": len(vres), "against": "PrpEngine.run (RES64, PRP flag, Gerbicz-Li)",
                     "b": sorted(r["b"] for r in vres)},
    }
    print(json.dumps(line))
    return 0


def plain_replay(reqs, limit_s: float):
    """The plain path, run for real: the same arrivals (time, degree, b) replayed
    through one FIFO worker that tests one candidate at a time with
    PrpEngine.run on the default split.  Stops admitting new requests once the
    replay has run limit_s; returns per-request latencies of those it served."""
    from ctwin_gb300 import PrpEngine
    engines = {}
    t0 = time.perf_counter()
    lat = []
    for ta, k, b in reqs:
        now = time.perf_counter() - t0
        if now > limit_s:
            break
        if now < ta:
            time.sleep(ta - now)
        eng = engines.get(k)
        if eng is None:
            eng = engines[k] = PrpEngine(k, 1)
        eng.run([b])
        lat.append((k, b, time.perf_counter() - t0 - ta))
    for e in engines.values():
        e.close()
    return lat


def pct(v, q):
    v = sorted(v)
    return v[min(len(v) - 1, int(q * len(v)))] if v else None


def run_serve(args):
    import torch  # noqa: F401  (CUDA context for the library)
    from ctwin_gb300 import Pool, PrpEngine, Server, autotune, two_primes
    rng = random.Random(11)
    kmax = args.serve_max_degree
    degrees = tuple(range(12, kmax + 1))
    lo, hi = math.log(12), math.log(kmax + 1)
    lane = 16                             # the server's grid lane: degrees 2^16 and up
    # capacity from the pools themselves: device time per lane-squaring of a
    # pool tick of each degree and prime class (squarings, multiply, register
    # moves, graph launch), 64 slots; for the grid lane's degrees the device
    # time per squaring of one test on the one-lane engine (the lane runs one
    # test at a time and takes turns with the pools)
    us, frac2 = {}, {}
    words = np.array([rng.getrandbits(32) for _ in range(64)], dtype=np.uint32)
    for k in degrees:
        slots = 64
        lim = max([b for b in range(1 << 16, 1 << 24, 1 << 12) if two_primes(k, b)] or [(1 << 16) - 1])
        frac2[k] = max(0.0, (lim - (1 << 16)) / ((1 << 24) - (1 << 16)))
        for primes, (b_lo, b_hi) in ((2, (1 << 16, lim)), (3, (lim + (1 << 12), 1 << 24))):
            if b_hi <= b_lo:
                continue
            if k >= lane:
                with PrpEngine(k, 1) as eng:
                    eng.set_b([rng.randrange(b_lo, b_hi)])
                    assert eng.prime_count == primes
                    eng.set(1)
                    eng.square_bits(words, 2047, 256)
                    eng.sync()
                    st = torch.cuda.ExternalStream(eng.stream)
                    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    e0.record(st)
                    eng.square_bits(words, 2047, 1024)
                    e1.record(st)
                    e1.synchronize()
                    us[(k, primes)] = e0.elapsed_time(e1) * 1e3 / 1024
                continue
            lg, cs, _ = autotune(k, slots, primes)
            with Pool(k, slots, log2_ctas=lg, csize=cs) as p:
                p.admit_many([rng.randrange(b_lo, b_hi) for _ in range(slots)])
                assert p.prime_count == primes
                p.run(1)
                p.collect(wait=True)
                B = p.info()["gl_block"]
                st = torch.cuda.ExternalStream(p.stream)
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(st)
                p.run(2)
                e1.record(st)
                e1.synchronize()
                us[(k, primes)] = e0.elapsed_time(e1) * 1e3 / (2 * (B + 1) * slots)
    mean_bits = {k: (1 << k) * statistics.mean(math.log2(rng.randrange(1 << 16, 1 << 24)) for _ in range(2000))
                 for k in degrees}
    w = {k: (math.log(k + 1) - math.log(k)) / (hi - lo) for k in degrees}
    demand = sum(w[k] * mean_bits[k] * 1e-6 * (frac2[k] * us.get((k, 2), 0.0) + (1 - frac2[k]) * us[(k, 3)])
                 for k in degrees)
    lam = args.load / demand
    n = args.requests or max(50, int(lam * args.serve_seconds))
    reqs, t = [], 0.0
    for i in range(n):
        t += rng.expovariate(lam)
        k = int(math.exp(rng.uniform(lo, hi)))
        reqs.append((t, k, rng.randrange(1 << 16, 1 << 24)))
    srv = Server(hbm_budget_bytes=args.hbm_budget << 30, max_slots=256, ticks_per_launch=1, autotune=True,
                 grid_lane=lane)
    for k in degrees:
        if k < lane:
            srv.prepare(k, 0)
    last, still = -1, 0
    while still < 10:                     # pools created and tuned: bytes stable for 1 s
        nb = srv.stats()["pool_bytes"]
        still = still + 1 if (nb == last and nb > 0) else 0
        last = nb
        time.sleep(0.1)
    res = []
    with ClockSampler(0) as clk:
        t0 = srv.clock()
        for i, (ta, k, b) in enumerate(reqs):
            while srv.clock() - t0 < ta:
                res += srv.poll(256, 0)
                time.sleep(0.0005)
            srv.submit(k, b, tag=i)
        res += srv.drain(n - len(res), timeout_s=args.serve_drain)
        t_end = srv.clock()
    srv.close()
    lat = [r["t_done"] - r["t_submit"] for r in res]
    bad = sum(1 for r in res if r["status"] != 0 or not r["gl_ok"])
    span = max(r["t_done"] for r in res) - (t0 + reqs[0][0])
    per = {}
    for k in degrees:
        lk = [r["t_done"] - r["t_submit"] for r in res if r["log2_degree"] == k]
        if lk:
            per[str(k)] = {"count": len(lk), "p50_s": pct(lk, 0.5), "p99_s": pct(lk, 0.99), "max_s": max(lk)}
    # the plain path, run: the first arrivals replayed through one test at a time
    plain = plain_replay(reqs, args.plain_seconds)
    served_same = [r["t_done"] - r["t_submit"] for r in res if r["tag"] < len(plain)]
    plat = [x[2] for x in plain]
    line = {
        "metric": "PRP tests/s (served, mixed degrees)", "value": len(res) / span, "unit": "tests/s",
        "n_gpus": 1, "steps": n, "warmup": 0, "ms_per_step": 1000.0 * span / max(1, len(res)),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": {"workload": f"{n} Poisson arrivals (seed 11, rate {lam:.3f}/s = {args.load:.0%} of the capacity "
                               f"measured on pool ticks and on the grid lane's engine), degree 2^k, k log-uniform "
                               f"in [12, {kmax}], b uniform in [2^16, 2^24); degrees 2^{lane} and up in the "
                               "server's grid lane (one test at a time on the cooperative grid kernel, taking "
                               "turns with the pools)",
                   "us_per_lane_squaring": {f"{k}" + ("" if c == 2 else "w"): v for (k, c), v in us.items()},
                   "two_prime_fraction": {str(k): v for k, v in frac2.items()},
                   "hbm_budget_gib": args.hbm_budget, "ticks_per_launch": 1},
        "latency_s": {"p50": pct(lat, 0.5), "p99": pct(lat, 0.99), "max": max(lat)},
        "per_degree": per, "failed": bad, "completed": len(res),
        "plain_path": {"requests": len(plain), "p50_s": pct(plat, 0.5), "p99_s": pct(plat, 0.99),
                       "served_p50_s_same_requests": pct(served_same, 0.5),
                       "served_p99_s_same_requests": pct(served_same, 0.99),
                       "method": f"the first {len(plain)} arrivals replayed at their arrival times through one FIFO "
                                 "worker (PrpEngine.run, one test at a time, default split), measured"},
        "wall_s": t_end,
        "e2e": {"value": len(res) / span, "unit": "tests/s", "h2d_bytes_per_step": None, "d2h_bytes_per_step": None},
        "clocks": clk.summary(),
    }
    print(json.dumps(line))
    return 0


def _is_prime64(p: int) -> bool:
    if p < 2:
        return False
    for q in (2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37):
        if p % q == 0:
            return p == q
    d, r = p - 1, 0
    while d % 2 == 0:
        d //= 2
        r += 1
    for a in (2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37):
        x = pow(a, d, p)
        if x in (1, p - 1):
            continue
        for _ in range(r - 1):
            x = x * x % p
            if x == p - 1:
                break
        else:
            return False
    return True


def run_sieve(args):
    """Sieved b/s: config 4 (n = 20, b < 2^30, p = 3k 2^20 + 1 < 2^40) on the GPU,
    config 1 (n = 11, b in [10^5, 3 10^5), both forms to 2^32) beside it, the
    oracle's C restatement of the CPU sieve timed on a bounded sample."""
    import torch  # noqa: F401  (CUDA context)
    from ctwin_gb300 import sieve_pass
    from ctwin_gb300._native import lib
    from ctwin_gb300.sieve import unpack
    L = lib()
    n, b_min, b_max = 20, 2, (1 << 30) - 1
    p_min, p_max = 3 * (1 << n) + 1, 1 << 40
    for _ in range(args.warmup):
        sieve_pass(n, b_min, b_max, p_min, p_max, 1)
    times, launches0 = [], L.ctw_sieve_launches()
    with ClockSampler(0) as clk:
        for _ in range(args.steps):
            t0 = time.perf_counter()
            struck, p_last = sieve_pass(n, b_min, b_max, p_min, p_max, 1)
            times.append(time.perf_counter() - t0)
    launches = L.ctw_sieve_launches() - launches0
    t = statistics.median(times)
    size = b_max - b_min + 1
    survivors = int((unpack(struck, size) == 0).sum())
    # algorithmic work: 2^(n-1) root products per prime (0.5 mulmod per root) + an
    # Euler/PRP test of log2 p squarings per candidate k
    step = 3 << n
    ks = list(range(1, (p_max - 1) // step + 1))
    primes = sum(1 for k in ks if _is_prime64(k * step + 1))
    work = primes * (1 << (n - 1)) + len(ks) * 40
    peak = L.ctw_mulmod64_peak()
    # config 1, both forms
    c1 = {}
    for name, mode, pmn in (("pos", 1, 3 * 2048 + 1), ("neg", -1, 11)):
        sieve_pass(11, 100000, 299999, pmn, 1 << 32, mode)
        t0 = time.perf_counter()
        sieve_pass(11, 100000, 299999, pmn, 1 << 32, mode)
        c1[name] = time.perf_counter() - t0
    cpu = None
    if not args.no_cpu_baseline:
        from oracle import oracle as O
        O.build()
        cores = os.cpu_count() or 1
        p_s = 1 << 34                       # bounded sample: primes below 2^34 of config 4
        t0 = time.perf_counter()
        O.sieve(n, b_min, b_max, p_min, p_s, 1, threads=cores)
        dt = time.perf_counter() - t0
        frac = (p_s - p_min) / (p_max - p_min)
        t0 = time.perf_counter()
        O.sieve(11, 100000, 299999, 3 * 2048 + 1, 1 << 32, 1, threads=cores)
        dt1 = time.perf_counter() - t0
        cpu = {"value": size * frac / dt, "unit": "sieved b/s", "cores": cores, "kind": "port",
               "sample": f"config 4 primes below 2^34 ({frac:.4f} of the p range) in {dt:.1f} s; "
                         f"config 1 '+' form in {dt1:.2f} s",
               "config1_pos_s": dt1}
    line = {
        "metric": "sieved b/s", "value": size / t, "unit": "sieved b/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000.0 * t, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u64", "data": "synthetic (the full b and p ranges)",
        "config": {"workload": "n = 20 (N = b^(2^20) - b^(2^19) + 1), b in [2, 2^30), p = 3k 2^20 + 1 < 2^40, + form",
                   "survivors": survivors, "p_last": p_last, "primes": primes, "candidates_k": len(ks),
                   "config1_s": c1, "config1_sieved_b_per_s": {k: 200000 / v for k, v in c1.items()}},
        "e2e": {"value": size / t, "unit": "sieved b/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": int(struck.nbytes)},
        "roofline": {"bound": "mulmod64", "achieved": work / t / 1e12, "peak": peak / 1e12,
                     "unit": "T mulmod64/s", "frac": work / t / peak if peak else None,
                     "work_per_step": work, "traffic": None,
                     "peak_source": "64-bit Montgomery probe kernel run on this GPU in this process",
                     "hbm": hbm_line(struck.nbytes, t)},
        "cpu_baseline": cpu, "gpu_launches": launches // max(1, args.steps), "clocks": clk.summary(),
    }
    print(json.dumps(line))
    return 0


def run_pool_all(pool, bs, ticks: int = 8):
    """Every b through one pool, admitting as slots free up; results by b."""
    queue, res = list(bs), []
    while queue or pool.info()["active"]:
        free = pool.slots - pool.info()["active"]
        if queue and free:
            k = pool.admit_many(queue[:free])
            queue = queue[k:]
        pool.run(ticks)
        pool.collect(wait=True)
        res += pool.results()
    return {r["b"]: r for r in res}


def run_config1(args):
    """The reference's own workflow at n = 11: the GPU sieve of b in
    [100000, 300000) to p < 2^32 for both forms, then the base-3 Fermat test of
    every survivor N+ and of its twin partner N- (cyclo's PRP and the N- test)."""
    import torch  # noqa: F401
    from ctwin_gb300 import Pool, sieve_pass
    from ctwin_gb300.sieve import unpack
    n, b0, b1 = 11, 100000, 299999
    t0 = time.perf_counter()
    struck, _ = sieve_pass(n, b0, b1, 3 * (1 << n) + 1, 1 << 32, 1)
    struck, _ = sieve_pass(n, b0, b1, 11, 1 << 32, -1, struck)
    t_sieve = time.perf_counter() - t0
    surv = [b0 + int(i) for i in np.flatnonzero(unpack(struck, b1 - b0 + 1) == 0)]
    t0 = time.perf_counter()
    with Pool(n, 2048, base=3) as pp:
        plus = run_pool_all(pp, surv)
    t_plus = time.perf_counter() - t0
    t0 = time.perf_counter()
    with Pool(n, 2048, base=3, minus=True) as pm:
        minus = run_pool_all(pm, surv)
    t_minus = time.perf_counter() - t0
    bad = sum(1 for r in list(plus.values()) + list(minus.values()) if r["status"] != 0 or not r["gl_ok"])
    twins = [b for b in surv if plus[b]["is_prp"] and minus[b]["is_prp"]]
    # parity sample: the survivors with a GMP residue in tests/golden (N+, base 3; the first 256)
    gold = {}
    try:
        for x in json.load(open(os.path.join(ROOT, "tests", "golden", "prp_gmp.json"))):
            if x["n"] == n and x["form"] == "+" and x["base"] == 3:
                gold[x["b"]] = int(x["res64"], 16)
    except OSError:
        pass
    checked = [b for b in surv if b in gold]
    agree = sum(1 for b in checked if plus[b]["res64"] == gold[b])
    tests = 2 * len(surv)
    cpu = None
    if not args.no_cpu_baseline:
        from oracle import oracle as O
        O.build()
        cores = os.cpu_count() or 1
        sample = surv[:cores]
        t1 = time.perf_counter()
        threads = [threading.Thread(target=O.prp_check, args=(b, n, 3)) for b in sample]
        for th in threads:
            th.start()
        for th in threads:
            th.join()
        dt = time.perf_counter() - t1
        cpu = {"value": len(sample) / dt, "unit": "PRP tests/s", "cores": cores, "kind": "port",
               "sample": f"{len(sample)} N+ base-3 tests of degree 2^11 (oracle C restatement, one per core) "
                         f"in {dt:.1f} s"}
    line = {
        "metric": "PRP tests/s (config 1: N+ and N- of every sieve survivor)", "value": tests / (t_plus + t_minus),
        "unit": "tests/s", "n_gpus": 1, "steps": 1, "warmup": 0, "ms_per_step": 1000.0 * (t_plus + t_minus),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": {"workload": "n = 11, b in [100000, 300000), sieve to p < 2^32 (both forms), base-3 Fermat "
                               "test of N+ and N- for every survivor, pools of 2048 slots",
                   "survivors": len(surv), "sieve_s": t_sieve, "plus_s": t_plus, "minus_s": t_minus,
                   "twin_prps": twins, "failed": bad, "gmp_checked": len(checked), "gmp_agree": agree},
        "e2e": {"value": tests / (t_sieve + t_plus + t_minus), "unit": "tests/s", "h2d_bytes_per_step": None,
                "d2h_bytes_per_step": None},
        "cpu_baseline": cpu,
    }
    print(json.dumps(line))
    return 0


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------

def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-secondary", action="store_true",
                    help="single: skip the secondary block (batched/plain, sieves) of the bench line")
    ap.add_argument("--workload", default="single", choices=["single", "batch", "serve", "sieve", "config1"])
    ap.add_argument("--candidates", type=int, default=4096, help="batch: candidates")
    ap.add_argument("--requests", type=int, default=0, help="serve: requests (0: rate x --serve-seconds)")
    ap.add_argument("--serve-seconds", type=float, default=60.0)
    ap.add_argument("--load", type=float, default=0.8, help="serve: offered load / tuned capacity")
    ap.add_argument("--hbm-budget", type=int, default=64, help="serve: pool budget in GiB")
    ap.add_argument("--serve-max-degree", type=int, default=14, choices=range(12, 19),
                    help="serve: degrees 2^12 .. 2^this (log-uniform)")
    ap.add_argument("--serve-drain", type=float, default=1800.0, help="serve: seconds to wait for the last tests")
    ap.add_argument("--plain-seconds", type=float, default=120.0,
                    help="serve: seconds of the plain-path replay (the first arrivals, one test at a time)")
    ap.add_argument("--log2-degree", type=int, default=16, choices=range(12, 19),
                    help="single: degree of the candidate (2^16 is the headline configuration)")
    ap.add_argument("--cpu-seconds", type=float, default=0.0,
                    help="reference arm: seconds of CPU work in all (0: 0.5 s per step, 12 s to 120 s)")
    ap.add_argument("--log2-ctas", type=int, default=-1,
                    help="single: CTAs per candidate as a power of two (-1: the library's default split)")
    args = ap.parse_args()
    global LOG2_D
    LOG2_D = args.log2_degree

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        if args.impl == "ours":
            import torch
            torch.cuda.set_device(local)
            dist.init_process_group("nccl")
        else:
            dist.init_process_group("gloo")      # the reference arm runs on the host cores only

    if args.impl == "reference":
        rc = run_reference(args, rank, world)
        if dist:
            dist.destroy_process_group()
        return rc

    import torch
    torch.cuda.set_device(local)
    if args.workload == "batch":
        return run_batch(args) if rank == 0 else 0
    if args.workload == "serve":
        return run_serve(args) if rank == 0 else 0
    if args.workload == "sieve":
        return run_sieve(args) if rank == 0 else 0
    if args.workload == "config1":
        return run_config1(args) if rank == 0 else 0
    import ctwin_gb300
    from ctwin_gb300 import PrpEngine
    from ctwin_gb300._native import lib

    b, E, i0, B_GL, words = workload(rank)
    D = 1 << LOG2_D
    eng = PrpEngine(LOG2_D, 1, base=3, log2_ctas=args.log2_ctas)          # Fermat base 3
    eng.set_b([b])
    eng.set(1)
    eng.copy(1, 0)
    # exponent bits resident in HBM for the device-side arm
    L = lib()
    stream = torch.cuda.ExternalStream(eng.stream)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.int32, device="cuda")
    peak_imad = L.ctw_imad_peak()

    from ctwin_gb300._native import check, ptr
    check(L.ctw_prp_load_exponent(eng._h, ptr(words), words.size))

    def device_step(i_hi):
        check(L.ctw_prp_square_resident(eng._h, i_hi, B_GL))
        check(L.ctw_prp_mul_regs(eng._h, 1, 0, 1))

    i = i0
    for w in range(args.warmup):
        device_step(i)
        i -= B_GL
    eng.sync()

    launches0 = eng.launches
    times = []
    with ClockSampler(local) as clk:
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        for s in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            device_step(i)
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
            i -= B_GL
        torch.cuda.synchronize()
    launches = eng.launches - launches0
    t_dev = sum(times) / 1000.0
    if dist:
        t = torch.tensor([t_dev], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_dev = float(t.item())
    squarings = args.steps * B_GL * world
    value = squarings / t_dev

    # dominant kernel: the resident squaring launch alone
    sq_times = []
    for s in range(5):
        flush.zero_()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        check(L.ctw_prp_square_resident(eng._h, i, B_GL))
        e1.record(stream)
        e1.synchronize()
        sq_times.append(e0.elapsed_time(e1) / 1000.0)
        i -= B_GL
    t_launch = statistics.median(sq_times)
    primes = eng.prime_count
    # algorithmic work: the three-prime count 4 (3 D log2 D + 9 D) IMAD per squaring;
    # executed work: the same count for the primes the launch ran
    achieved = imad_per_squaring(D, 3) * B_GL / t_launch
    executed = imad_per_squaring(D, primes) * B_GL / t_launch
    geo = eng.geometry()
    sms = torch.cuda.get_device_properties(local).multi_processor_count
    peak_mont, peak_shoup = L.ctw_modmul_peak(0), L.ctw_modmul_peak(1)

    # e2e through the C ABI with host buffers: exponent slice in, residue out
    reg_host = np.zeros((1, 1, D), dtype=np.int32)
    t0 = time.perf_counter()
    h2d = d2h = 0
    for s in range(args.steps):
        lo = max(0, i - B_GL + 1)
        w0 = lo // 32
        w1 = i // 32 + 1
        sl = np.ascontiguousarray(words[w0:w1])
        check(L.ctw_prp_square_bits(eng._h, ptr(sl), sl.size, i - 32 * w0, B_GL))
        check(L.ctw_prp_mul_regs(eng._h, 1, 0, 1))
        check(L.ctw_prp_read_regs(eng._h, 0, 1, ptr(reg_host)))
        h2d = sl.nbytes
        d2h = reg_host.nbytes
        i -= B_GL
    t_e2e = time.perf_counter() - t0
    if dist:
        t = torch.tensor([t_e2e], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_e2e = float(t.item())
    e2e = squarings / t_e2e
    eng.sync()
    eng.close()

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return 0

    cpu = None
    if not args.no_cpu_baseline:
        _, cpu = cpu_squarings_per_s(os.cpu_count() or 1)

    clocks = clk.summary()
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000.0 * t_dev / args.steps, "higher_is_better": True,
        "step_ms": {"min": min(times), "median": statistics.median(times), "max": max(times),
                    "first": times[0], "last": times[-1]},
        "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": single_config(world),
        "launch": {"ctas_per_candidate": geo["ctas_per_lane"], "threads_per_cta": geo["threads"],
                   "smem_per_cta": geo["smem_bytes"], "ntt_primes": primes},
        "tests_per_s_projected": value / (i0 + 1),
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
        "roofline": roofline_single(achieved, executed, peak_imad, peak_mont, peak_shoup, t_launch, geo, sms,
                                    LOG2_D == 16 and args.log2_ctas < 0),
        "cpu_baseline": cpu,
        "gpu_launches": int(launches),
        "clocks": clocks,
    }
    if not args.no_secondary and LOG2_D == 16 and world == 1:
        line["secondary"] = secondary()
    print(json.dumps(line))
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
