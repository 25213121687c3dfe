"""Pools and the request server: many resident PRP tests at once.

Neither has a counterpart in the reference, whose cyclog runs one vector of
64 candidates of one degree to completion (cyclo/src/cyclo.h:457-478); both
return, per test, the same verdict and RES64 as PrpEngine.run.  Every call goes
through the C ABI of libctwin_gb300.so.
"""
from __future__ import annotations

import ctypes

import numpy as np

from ._native import CtwError, CtwResult, check, lib, ptr

CTW_E_FULL = -6


def result_dict(r: CtwResult) -> dict:
    return {"tag": int(r.tag), "b": int(r.b), "log2_degree": int(r.log2_degree), "is_prp": bool(r.is_prp),
            "res64": int(r.res64), "gl_ok": bool(r.gl_ok), "status": int(r.status), "slot": int(r.slot),
            "t_submit": r.t_submit, "t_admit": r.t_admit, "t_done": r.t_done, "squarings": int(r.squarings)}


def autotune(log2_degree: int, lanes: int, primes: int = 2):
    """(log2_ctas, csize, us_per_squaring) the device picks for `lanes` candidates of
    degree 2^log2_degree whose b runs on `primes` NTT primes (2: within the bound)."""
    lg, cs, us = ctypes.c_int(), ctypes.c_int(), ctypes.c_double()
    check(lib().ctw_prp_autotune_primes(log2_degree, lanes, primes, ctypes.byref(lg), ctypes.byref(cs),
                                        ctypes.byref(us)))
    return lg.value, cs.value, us.value


def two_primes(log2_degree: int, b: int, minus: bool = False) -> bool:
    """Whether a test of this degree and b runs on two NTT primes (default split; host only)."""
    return bool(lib().ctw_prp_two_primes(log2_degree, 1 if minus else 0, b))


def schedule(log2_degree: int, b: int, gl_block: int = 0):
    """Tick program of one test (host only): (int32 array [ticks, 4] of
    {moves before, moves after, source 0 = E / 1 = block sum, lowest bit}, B)."""
    L = lib()
    blk = ctypes.c_int()
    n = L.ctw_pool_schedule(log2_degree, b, gl_block, None, 0, ctypes.byref(blk))
    if n < 0:
        check(n)
    out = np.zeros((n, 4), dtype=np.int32)
    check(0 if L.ctw_pool_schedule(log2_degree, b, gl_block, ptr(out), n, ctypes.byref(blk)) == n else -1)
    return out, blk.value


def slot_bytes(log2_degree: int) -> int:
    return int(lib().ctw_pool_slot_bytes(log2_degree))


class Pool:
    """`slots` resident tests of degree 2^log2_degree (continuous batching)."""

    def __init__(self, log2_degree: int, slots: int, log2_ctas: int = -1, csize: int = 0, base: int = 2,
                 gl_block: int = 0, minus: bool = False):
        """minus=True: tests of the twin partners N- = b^D - b^{D/2} - 1 (the
        split is then chosen as for PrpEngine(minus=True))."""
        h = ctypes.c_void_p()
        if minus:
            check(lib().ctw_pool_create_minus(log2_degree, slots, csize, base, gl_block, ctypes.byref(h)))
        else:
            check(lib().ctw_pool_create(log2_degree, slots, log2_ctas, csize, base, gl_block, ctypes.byref(h)))
        self._h = h
        self.ln = log2_degree
        self.D = 1 << log2_degree
        self.regD = self.D * (2 if minus else 1)
        self.slots = slots

    def close(self):
        if self._h:
            lib().ctw_pool_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def admit(self, b: int, tag: int = 0) -> int | None:
        """Slot of the new test, or None when the pool is full."""
        rc = lib().ctw_pool_admit(self._h, int(b), int(tag))
        if rc == CTW_E_FULL:
            return None
        if rc < 0:
            check(rc)
        return rc

    def admit_many(self, bs, tags=None, threads: int = 0) -> int:
        """Admit as many of bs as there are free slots (exponents prepared on
        `threads` host threads); returns the number admitted."""
        b = np.ascontiguousarray(bs, dtype=np.uint32)
        t = None if tags is None else np.ascontiguousarray(tags, dtype=np.uint64)
        n = lib().ctw_pool_admit_many(self._h, ptr(b), ptr(t) if t is not None else None, b.size, threads)
        if n < 0:
            check(n)
        return n

    def run(self, ticks: int = 1):
        check(lib().ctw_pool_run(self._h, ticks))

    def collect(self, wait: bool = False) -> int:
        n = lib().ctw_pool_collect(self._h, 1 if wait else 0)
        if n < 0:
            check(n)
        return n

    def results(self) -> list[dict]:
        out = []
        buf = (CtwResult * 256)()
        while True:
            n = lib().ctw_pool_results(self._h, ctypes.cast(buf, ctypes.c_void_p), 256)
            if n < 0:
                check(n)
            out += [result_dict(buf[i]) for i in range(n)]
            if n < 256:
                return out

    def info(self) -> dict:
        v = [ctypes.c_int() for _ in range(6)]
        sq = ctypes.c_longlong()
        check(lib().ctw_pool_info(self._h, *[ctypes.byref(x) for x in v], ctypes.byref(sq)))
        keys = ["slots", "active", "in_flight", "gl_block", "log2_ctas", "csize"]
        d = {k: x.value for k, x in zip(keys, v)}
        d["squarings"] = sq.value
        return d

    def set_prime_count(self, count: int):
        """0: two NTT primes for launches whose lanes allow it (default); 3: always three."""
        check(lib().ctw_pool_set_prime_count(self._h, count))

    @property
    def prime_count(self) -> int:
        """NTT primes of the next launch over the current slots (2 or 3)."""
        return int(lib().ctw_pool_prime_count(self._h))

    def read_slot(self, slot: int, reg: int) -> np.ndarray:
        out = np.zeros(self.regD, dtype=np.int32)
        check(lib().ctw_pool_read_slot(self._h, slot, reg, ptr(out)))
        return out

    @property
    def stream(self) -> int:
        return lib().ctw_pool_stream(self._h) or 0

    def run_to_completion(self, ticks_per_call: int = 8) -> list[dict]:
        """Run until every admitted test has finished; return their results."""
        res = []
        while True:
            self.collect(wait=False)
            res += self.results()
            if self.info()["active"] == 0:
                return res
            self.run(ticks_per_call)
            self.collect(wait=True)
            res += self.results()


class Batch:
    """Pools of degrees 2^12..2^15 (CTAs of 4096 coefficients) driven together:
    per tick, every pool's squarings in one persistent launch with per-degree
    work queues (and every pool's Gerbicz-Li multiply in a second), replayed
    from CUDA graphs.  Results stay the pools' own (Pool.collect / results)."""

    def __init__(self, pools, ctas_per_sm: int = 2):
        self.pools = list(pools)
        arr = (ctypes.c_void_p * len(self.pools))(*[p._h.value for p in self.pools])
        h = ctypes.c_void_p()
        check(lib().ctw_batch_create(ctypes.cast(arr, ctypes.c_void_p), len(self.pools), ctypes.byref(h)))
        self._h = h
        self.set_ctas_per_sm(ctas_per_sm)

    def set_ctas_per_sm(self, ctas: int):
        check(lib().ctw_batch_set_ctas_per_sm(self._h, ctas))
        self.ctas_per_sm = ctas

    def close(self):
        if self._h:
            lib().ctw_batch_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def run(self, ticks: int = 1):
        check(lib().ctw_batch_run(self._h, ticks))

    @property
    def stream(self) -> int:
        return lib().ctw_batch_stream(self._h) or 0

    @property
    def launches(self) -> int:
        return int(lib().ctw_batch_launches(self._h))

    def run_to_completion(self, ticks_per_call: int = 8) -> list[dict]:
        """Run until every admitted test of every pool has finished."""
        res = []
        while True:
            for p in self.pools:
                p.collect(wait=False)
                res += p.results()
            if all(p.info()["active"] == 0 for p in self.pools):
                return res
            self.run(ticks_per_call)
            for p in self.pools:
                p.collect(wait=True)
                res += p.results()


class Server:
    """Request loop over pools of every degree (continuous batching by size class)."""

    def __init__(self, hbm_budget_bytes: int = 0, max_slots: int = 256, base: int = 2, ticks_per_launch: int = 2,
                 autotune: bool = False, grid_lane: int = 16, grid_lanes: int = 1):
        """grid_lane: tests of degree >= 2^grid_lane run on the cooperative grid
        kernel, one per lane at a time, taking turns with the pools (0: pools
        only); grid_lanes: lanes taking requests (1: first come, first served;
        2: two large tests in flight)."""
        h = ctypes.c_void_p()
        check(lib().ctw_server_create(hbm_budget_bytes, max_slots, base, ticks_per_launch, 1 if autotune else 0,
                                      ctypes.byref(h)))
        self._h = h
        try:
            check(lib().ctw_server_set_grid_lane(h, grid_lane))
            check(lib().ctw_server_set_grid_lanes(h, grid_lanes))
        except Exception:
            self.close()
            raise

    def close(self):
        if self._h:
            lib().ctw_server_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, log2_degree: int, b: int, tag: int = 0):
        check(lib().ctw_server_submit(self._h, log2_degree, int(b), int(tag)))

    def prepare(self, log2_degree: int, slots: int = 0):
        check(lib().ctw_server_prepare(self._h, log2_degree, slots))

    def poll(self, max_results: int = 256, timeout_ms: int = 0) -> list[dict]:
        buf = (CtwResult * max_results)()
        n = lib().ctw_server_poll(self._h, ctypes.cast(buf, ctypes.c_void_p), max_results, timeout_ms)
        if n < 0:
            check(n)
        return [result_dict(buf[i]) for i in range(n)]

    def stats(self) -> dict:
        v = [ctypes.c_longlong() for _ in range(4)]
        nb = ctypes.c_size_t()
        check(lib().ctw_server_stats(self._h, *[ctypes.byref(x) for x in v], ctypes.byref(nb)))
        d = dict(zip(["submitted", "pending", "active", "finished"], [x.value for x in v]))
        d["pool_bytes"] = nb.value
        return d

    def clock(self) -> float:
        return float(lib().ctw_server_clock(self._h))

    def drain(self, count: int, timeout_s: float = 600.0) -> list[dict]:
        """Wait for `count` results (or raise after timeout_s of no progress)."""
        import time
        out: list[dict] = []
        last = time.monotonic()
        while len(out) < count:
            got = self.poll(256, 50)
            if got:
                out += got
                last = time.monotonic()
            elif time.monotonic() - last > timeout_s:
                raise CtwError(-2, f"server drain: {len(out)} of {count} results after {timeout_s} s without progress")
        return out


def _main(argv=None) -> int:
    """Tick throughput of one pool: python -m ctwin_gb300.pool <log2_degree> <slots>
    [--ticks T] [--b-min B] [--b-max B] [--seed S] [--primes 0|3].  Admits `slots`
    tests with seeded b in [b_min, b_max), runs T ticks and prints squarings/s
    (wall clock, one line of JSON)."""
    import argparse
    import json
    import random
    import time
    ap = argparse.ArgumentParser(prog="python -m ctwin_gb300.pool")
    ap.add_argument("log2_degree", type=int)
    ap.add_argument("slots", type=int)
    ap.add_argument("--ticks", type=int, default=4)
    ap.add_argument("--b-min", type=int, default=1 << 16)
    ap.add_argument("--b-max", type=int, default=1 << 22)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--primes", type=int, default=0, choices=(0, 3))
    a = ap.parse_args(argv)
    rng = random.Random(a.seed)
    bs = [rng.randrange(a.b_min, a.b_max) for _ in range(a.slots)]
    with Pool(a.log2_degree, a.slots) as p:
        p.set_prime_count(a.primes)
        p.admit_many(bs)
        p.run(1)
        p.collect(wait=True)
        t0 = time.perf_counter()
        p.run(a.ticks)
        p.collect(wait=True)
        dt = time.perf_counter() - t0
        info = p.info()
        print(json.dumps({"log2_degree": a.log2_degree, "slots": a.slots, "ticks": a.ticks,
                          "ntt_primes": p.prime_count, "log2_ctas": info["log2_ctas"], "csize": info["csize"],
                          "squarings_per_s": a.slots * a.ticks * (info["gl_block"] + 1) / dt}))
    return 0


if __name__ == "__main__":
    import sys
    sys.exit(_main())
