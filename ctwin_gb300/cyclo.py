"""The cyclog file loop over the C ABI (cyclo/src/cyclo.h:416-480, cyclo/src/main.cpp).

    python -m ctwin_gb300.cyclo -n <n> -f <file> [-minus] [-w <dir>]

tests every b of <file> (one per line) for N = b^(2^n) - b^(2^(n-1)) + 1 (or
the twin partner N- with -minus), appends the reference's result lines to
result_c.txt and PRPs to prp_<n>.txt, keeps <file>.ini (CSIZE) and resumes
from cyclo.ctx (the reference's context format) after an interruption.
"""
from __future__ import annotations

import argparse
import ctypes
import signal
import sys

import numpy as np

from ._native import check, lib, ptr

CTW_STOPPED = 1


def check_file(n: int, filename: str, workdir: str = ".", minus: bool = False, save_every_s: float = 600.0,
               stop_after: int = 0, quit_flag: ctypes.c_int | None = None) -> bool:
    """Run the file; True when every vector is done, False when stopped (context saved)."""
    rc = lib().ctw_cyclo_check_file(n, filename.encode(), workdir.encode(), 1 if minus else 0, save_every_s,
                                    ctypes.byref(quit_flag) if quit_flag is not None else None, stop_after)
    if rc == CTW_STOPPED:
        return False
    check(rc)
    return True


def context_encode(digits: np.ndarray, k: int, i: int, elapsed: float) -> bytes:
    """Context bytes of digits shaped [nregs, lanes, D] (no device needed)."""
    d = np.ascontiguousarray(digits, dtype=np.int32)
    nregs, lanes, D = d.shape
    ln = D.bit_length() - 1
    out = np.zeros(lib().ctw_context_bytes(ln, lanes, nregs), dtype=np.uint8)
    check(lib().ctw_context_encode(ln, lanes, nregs, ptr(d), k, i, elapsed, ptr(out)))
    return out.tobytes()


def context_decode(data: bytes, log2_degree: int, lanes: int, nregs: int = 2):
    """(digits [nregs, lanes, D], k, i, elapsed) of context bytes."""
    buf = np.frombuffer(data, dtype=np.uint8).copy()
    d = np.zeros((nregs, lanes, 1 << log2_degree), dtype=np.int32)
    k, i, el = ctypes.c_int(), ctypes.c_int(), ctypes.c_double()
    check(lib().ctw_context_decode(log2_degree, lanes, nregs, ptr(buf), buf.size, ptr(d), ctypes.byref(k),
                                   ctypes.byref(i), ctypes.byref(el)))
    return d, k.value, i.value, el.value


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(prog="ctwin_gb300.cyclo", description="Fermat PRP test of b^(2^n) - b^(2^(n-1)) +- 1")
    ap.add_argument("-n", type=int, required=True, help="exponent (b^{2^n} - b^{2^{n-1}} + 1)")
    ap.add_argument("-f", dest="filename", required=True, help="input text file (one b per line)")
    ap.add_argument("-w", dest="workdir", default=".", help="directory of cyclo.ctx and the result files")
    ap.add_argument("-minus", action="store_true", help="test the twin partners b^{2^n} - b^{2^{n-1}} - 1")
    args = ap.parse_args(argv)
    quit_flag = ctypes.c_int(0)

    def on_signal(signum, frame):
        quit_flag.value = 1

    signal.signal(signal.SIGINT, on_signal)
    signal.signal(signal.SIGTERM, on_signal)
    done = check_file(args.n, args.filename, args.workdir, args.minus, quit_flag=quit_flag)
    return 0 if done else 1


if __name__ == "__main__":
    sys.exit(main())
