"""The reference's GPU sieve driver and candidate merge over the C ABI.

    python -m ctwin_gb300.gfsieve <n> <p_min> <p_max> <+|-> [-w <dir>]

mirrors ctsieveg (sieve/GPU/src/main.cpp:121-166, ctsieve.h:326-421): p_min and
p_max in P (10^15) for the + form and in T (10^12) for the - form, factor pairs
appended to fp<n>_<pmin_T>_<pmax_T>.txt / fn..., progress kept in ctx<...> and
resumed.  merge() restates the factor-file reading of tools/ctools.cpp:177-248:
every verified factor removes its b from a candidate list.
"""
from __future__ import annotations

import argparse
import ctypes
import signal
import sys

import numpy as np

from ._native import check, lib, ptr

CTW_STOPPED = 1
PETA, TERA = 10 ** 15, 10 ** 12


def factors(n: int, k_begin: int, k_end: int, mode: int, b_max: int) -> np.ndarray:
    """(p, b) pairs [m, 2] of the primes with k in [k_begin, k_end), roots b <= b_max."""
    L = lib()
    cnt = ctypes.c_uint64(0)
    cap = 1 << 20
    while True:
        buf = np.zeros((cap, 2), dtype=np.uint64)
        rc = L.ctw_sieve_factors(n, k_begin, k_end, mode, b_max, ptr(buf), cap, ctypes.byref(cnt))
        if rc == 0:
            return buf[:cnt.value]
        if rc == -3 and cnt.value > cap:
            cap = int(cnt.value)
            continue
        check(rc)


def check_range(n: int, p_min: int, p_max: int, mode: int, workdir: str = ".", stop_after_blocks: int = 0,
                quit_flag: ctypes.c_int | None = None):
    """Run ctsieveg's loop over [p_min, p_max] (absolute p): (done, factors written)."""
    w = ctypes.c_uint64(0)
    rc = lib().ctw_gfsieve_check(n, p_min, p_max, mode, workdir.encode(),
                                 ctypes.byref(quit_flag) if quit_flag is not None else None, stop_after_blocks,
                                 ctypes.byref(w))
    if rc == CTW_STOPPED:
        return False, w.value
    check(rc)
    return True, w.value


def divides(p: int, b: int, n: int, mode: int) -> bool:
    x = pow(b, 1 << (n - 1), p)
    r = (x * x - x) % p
    return r == p - 1 if mode > 0 else r == 1


def merge(n: int, candidates, factor_files, mode_of_file, b_min: int, b_max: int):
    """Remove from `candidates` (iterable of b) every b in [b_min, b_max] with a
    verified factor in the files: (remaining sorted list, factors used, bad lines)."""
    cand = set(int(b) for b in candidates)
    used = bad = 0
    for fname in factor_files:
        mode = mode_of_file(fname)
        prev = None
        with open(fname) as f:
            for line in f:
                parts = line.split()
                if len(parts) != 2:
                    continue
                p, b = int(parts[0]), int(parts[1])
                if (p, b) == prev:
                    continue
                prev = (p, b)
                if b_min <= b <= b_max:
                    if divides(p, b, n, mode):
                        cand.discard(b)
                        used += 1
                    else:
                        bad += 1
    return sorted(cand), used, bad


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(prog="ctwin_gb300.gfsieve",
                                 description="GPU sieve of b^(2^n) - b^(2^(n-1)) +- 1 (factor files)")
    ap.add_argument("n", type=int)
    ap.add_argument("p_min", type=int, help="P (10^15) for +, T (10^12) for -")
    ap.add_argument("p_max", type=int)
    ap.add_argument("sign", choices=["+", "-"])
    ap.add_argument("-w", dest="workdir", default=".")
    args = ap.parse_args(argv)
    mode = 1 if args.sign == "+" else -1
    unit = PETA if mode > 0 else TERA
    if not 8 <= args.n <= 24 or args.p_max <= args.p_min:
        ap.print_usage()
        return 2
    quit_flag = ctypes.c_int(0)

    def on_signal(signum, frame):
        quit_flag.value = 1

    signal.signal(signal.SIGINT, on_signal)
    signal.signal(signal.SIGTERM, on_signal)
    done, nf = check_range(args.n, args.p_min * unit, args.p_max * unit, mode, args.workdir, quit_flag=quit_flag)
    print(f"{nf} factors written; {'done' if done else 'stopped, resume with the same command'}")
    return 0 if done else 1


if __name__ == "__main__":
    sys.exit(main())
