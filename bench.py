"""Benchmark: single large PRP test, degree D = 2^16, b uniform in [2^20, 2^21).

One step = one Gerbicz-Li block of the Fermat test: B_GL squarings of the real
exponent bits (one resident-kernel launch, the residue stays in shared memory of
a 16-CTA cluster) followed by the Gerbicz-Li multiply d <- d * x, exactly the
work cyclo::check does between two checkpoints (cyclo/src/cyclo.h:277-308).

  value  squarings/s with the residue and exponent resident in HBM (CUDA events
         on the engine's stream, per step, L2 flushed between steps)
  e2e    same metric through the C ABI with host buffers: per step the exponent
         slice is copied host->device and the residue read back device->host
  roofline  32-bit integer multiply-add work per launch (4 IMAD per Montgomery
         multiply, 3 D log2 D + 9 D multiplies per squaring) / launch time,
         against the IMAD throughput probed on the same GPU in this run
  cpu_baseline  the oracle's C restatement of the reference transform (the
         reference has no CPU PRP path), one candidate per host core

python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
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


def imad_per_squaring(D: int) -> float:
    return 4.0 * (3 * D * math.log2(D) + 9 * D)


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

def cpu_squarings_per_s(threads: int, seconds: float = 12.0):
    """Each host thread squares its own degree-2^16 candidate; bounded sample."""
    from oracle import oracle as O
    O.build()
    per = [0] * threads
    stop = time.perf_counter() + seconds
    tabs = O.Tables(LOG2_D)
    lock = threading.Lock()

    def work(t):
        b, E, i0, _, words = workload(100 + t)
        x = np.zeros(1 << LOG2_D, dtype=np.int32)
        x[0] = 1
        i = i0
        n = 0
        while time.perf_counter() < stop:
            tabs.square_loop(x, b, 2, 16, words, i, 4)
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
                        "sample": f"{threads} candidates of degree 2^16 (b in [2^20,2^21)), "
                                  f"{total} squarings in {dt:.1f} s with the oracle C restatement"}


def run_reference(args, rank, world):
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    samples = []
    for _ in range(args.warmup if args.warmup < 1 else 1):
        pass
    for _ in range(max(1, args.steps)):
        v, cb = cpu_squarings_per_s(threads, seconds=max(2.0, 20.0 / max(1, args.steps)))
        samples.append(v)
    v = statistics.median(samples)
    cb["value"] = v
    b, E, i0, B_GL, _ = workload(0)
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 * B_GL / v, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": "single large PRP, degree 2^16, b in [2^20, 2^21), one candidate per core",
                       "degree": 1 << LOG2_D, "squarings_per_step": B_GL},
            "cpu_baseline": cb,
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
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
    args = ap.parse_args()

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        import torch
        torch.cuda.set_device(local)
        dist.init_process_group("nccl" if args.impl == "ours" else "gloo")

    if args.impl == "reference":
        rc = run_reference(args, rank, world)
        if dist:
            dist.destroy_process_group()
        return rc

    import torch
    torch.cuda.set_device(local)
    import ctwin_gb300
    from ctwin_gb300 import PrpEngine
    from ctwin_gb300._native import lib

    b, E, i0, B_GL, words = workload(rank)
    D = 1 << LOG2_D
    eng = PrpEngine(LOG2_D, 1)
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
    achieved = imad_per_squaring(D) * B_GL / t_launch
    geo = eng.geometry()

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
        "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": {"workload": "single large PRP, degree 2^16 (N = b^65536 - b^32768 + 1), b uniform in "
                               "[2^20, 2^21) seed 1, one candidate per launch sequence",
                   "degree": D, "b": b, "exponent_bits": i0 + 1, "squarings_per_step": B_GL,
                   "step": "one Gerbicz-Li block: B_GL resident squarings + one multiply",
                   "l2": "flushed between steps (256 MiB write)", "parallelism": f"replicas{world}",
                   "cluster_ctas": geo["ctas_per_lane"], "threads_per_cta": geo["threads"],
                   "smem_per_cta": geo["smem_bytes"]},
        "tests_per_s_projected": value / (i0 + 1),
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
        "roofline": {"bound": "imad", "achieved": achieved / 1e12, "peak": peak_imad / 1e12, "unit": "T IMAD/s",
                     "frac": achieved / peak_imad if peak_imad else None, "traffic": None,
                     "peak_source": "32-bit IMAD probe kernel run on this GPU in this process",
                     "sms_used": geo["ctas_per_lane"],
                     "frac_of_used_sms": (achieved / peak_imad) * 152 / geo["ctas_per_lane"] if peak_imad else None,
                     "kernel_ms": t_launch * 1000.0},
        "cpu_baseline": cpu,
        "gpu_launches": int(launches),
        "clocks": clocks,
    }
    print(json.dumps(line))
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
