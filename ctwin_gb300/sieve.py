"""Host mirror of the reference sieve interface.

`Sieve(n, b_min, b_max)` follows the reference CPU sieve class
(sieve/CPU/ctsieve.cpp:454-812): check_pos / check_neg extend the sieve limit
of one form, check(mode) is the "ini" / "+" / "-" entry point, write() produces
sv_*.dat and cand_*.txt.  All striking happens on the GPU through
ctw_sieve_run; nothing here computes a root.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from ._native import check, lib, ptr


def words_for(size: int) -> int:
    return (size + 31) // 32


def sieve_pass(n: int, b_min: int, b_max: int, p_min: int, p_max: int, mode: int,
               struck: np.ndarray | None = None, p_last: int = 0):
    """One GPU pass; struck is the packed uint32 bitmap (updated in place)."""
    size = b_max - b_min + 1
    if struck is None:
        struck = np.zeros(words_for(size), dtype=np.uint32)
    pl = ctypes.c_uint64(p_last)
    check(lib().ctw_sieve_run(n, b_min, b_max, p_min, p_max, mode, ptr(struck), ctypes.byref(pl)))
    return struck, pl.value


def unpack(struck: np.ndarray, size: int) -> np.ndarray:
    """uint8 array, 1 where b_min + i is struck (the reference's _bsieve)."""
    return np.unpackbits(struck.view(np.uint8), bitorder="little")[:size]


class Sieve:
    """b in [b_min, b_max] (inclusive, b_min >= 2 as ctsieve.cpp:847-848)."""

    def __init__(self, n: int, b_min: int, b_max: int):
        if not 8 <= n <= 24:
            raise ValueError("n must be in [8, 24]")
        self.n = n
        self.b_min = max(2, b_min)
        self.b_max = max(b_max, self.b_min)
        self.size = self.b_max - self.b_min + 1
        self.struck = np.zeros(words_for(self.size), dtype=np.uint32)
        self.p_min_pos = 3 * (1 << n) + 1
        self.p_min_neg = 11

    def check_pos(self, p_max: int):
        self.struck, self.p_min_pos = sieve_pass(self.n, self.b_min, self.b_max, self.p_min_pos, p_max, 1,
                                                 self.struck, self.p_min_pos)

    def check_neg(self, p_max: int):
        self.struck, self.p_min_neg = sieve_pass(self.n, self.b_min, self.b_max, self.p_min_neg, p_max, -1,
                                                 self.struck, self.p_min_neg)

    def check(self, mode: int = 0, p_max_pos: int | None = None, p_max_neg: int | None = None):
        """mode 0 = "ini" with the reference's default limits (ctsieve.cpp:798-802),
        +1 / -1 extend one form."""
        if p_max_pos is None:
            p_max_pos = 3 * (100000000 << self.n) + 1
        if p_max_neg is None:
            p_max_neg = 10000000001
        if mode >= 0:
            self.check_pos(p_max_pos)
        if mode <= 0:
            self.check_neg(p_max_neg)

    def bits(self) -> np.ndarray:
        return unpack(self.struck, self.size)

    def survivors(self) -> np.ndarray:
        return self.b_min + np.flatnonzero(self.bits() == 0)

    def write(self, directory: str = "."):
        os.makedirs(directory, exist_ok=True)
        check(lib().ctw_sieve_write_files(self.n, self.b_min, self.b_max, ptr(self.struck), self.p_min_pos,
                                          self.p_min_neg, directory.encode()))
        tag = f"_{self.n}_{self.b_min}_{self.b_max}"
        return os.path.join(directory, "sv" + tag + ".dat"), os.path.join(directory, "cand" + tag + ".txt")
