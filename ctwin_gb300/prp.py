"""Host mirror of the reference PRP engine interface.

PrpEngine follows the reference's engine/transform calls (cyclo/src/engine.h,
cyclo/src/transform.h) one for one: set_b, set, copy, square_dup(mask), mul,
get_int (canonical digits), is_prime (PRP flag, RES64), and run (the whole
cyclo::check of cyclo/src/cyclo.h:252-408).  Every call goes through the C ABI
of libctwin_gb300.so; nothing here computes a residue.
"""
from __future__ import annotations

import ctypes

import numpy as np

from ._native import check, lib, ptr


_CHECKPOINT_FN = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_longlong)


class PrpEngine:
    """Fermat-test engine for `lanes` candidates of degree D = 2^log2_degree."""

    def __init__(self, log2_degree: int, lanes: int = 1, csize: int = 8, base: int = 2, minus: bool = False,
                 log2_ctas: int = -1):
        """minus=True tests the twin partner N- = b^D - b^{D/2} - 1 (no reference
        counterpart; its registers hold 2D words, its digits D).  log2_ctas >= 0
        picks the cluster split (2^log2_ctas CTAs per candidate) of an N+ engine."""
        h = ctypes.c_void_p()
        if minus:
            check(lib().ctw_prp_create_minus(log2_degree, lanes, ctypes.byref(h)))
        elif log2_ctas >= 0:
            check(lib().ctw_prp_create_split(log2_degree, lanes, log2_ctas, ctypes.byref(h)))
        else:
            check(lib().ctw_prp_create(log2_degree, lanes, ctypes.byref(h)))
        self._h = h
        self.ln = log2_degree
        self.D = 1 << log2_degree
        self.minus = minus
        self.regD = self.D * (2 if minus else 1)
        self.lanes = lanes
        self.set_csize(csize)
        self.set_base(base)

    # -- lifetime --
    def close(self):
        if self._h:
            lib().ctw_prp_destroy(self._h)
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

    # -- configuration --
    def set_csize(self, csize: int):
        check(lib().ctw_prp_set_csize(self._h, csize))
        self.csize = csize

    def set_base(self, base: int):
        check(lib().ctw_prp_set_base(self._h, base))
        self.base = base

    def set_b(self, b):
        arr = np.ascontiguousarray(b, dtype=np.uint32)
        check(lib().ctw_prp_set_b(self._h, ptr(arr), arr.size))
        self.b = arr.copy()

    def set_prime_count(self, count: int):
        """0: two NTT primes whenever they keep the product exact (default); 3: always three."""
        check(lib().ctw_prp_set_prime_count(self._h, count))

    @property
    def prime_count(self) -> int:
        """NTT primes of the next launch (2 or 3)."""
        return int(lib().ctw_prp_prime_count(self._h))

    # -- register operations (reference engine.h) --
    def set(self, a: int):
        check(lib().ctw_prp_set(self._h, a))

    def copy(self, dst: int, src: int):
        check(lib().ctw_prp_copy(self._h, dst, src))

    def square_dup(self, dup_lanes=None):
        """reg0 <- reg0^2 * base^bit; dup_lanes: int bitmask or iterable of bools per lane."""
        nw = (self.lanes + 63) // 64
        words = np.zeros(nw, dtype=np.uint64)
        if dup_lanes is None:
            pass
        elif isinstance(dup_lanes, (int, np.integer)):
            v = int(dup_lanes)
            for w in range(nw):
                words[w] = (v >> (64 * w)) & 0xFFFFFFFFFFFFFFFF
        else:
            for i, f in enumerate(dup_lanes):
                if f:
                    words[i // 64] |= np.uint64(1) << np.uint64(i % 64)
        check(lib().ctw_prp_square_dup(self._h, ptr(words)))

    def mul(self):
        check(lib().ctw_prp_mul(self._h))

    def mul_regs(self, out: int, a: int, b: int):
        check(lib().ctw_prp_mul_regs(self._h, out, a, b))

    def square_bits(self, e_words: np.ndarray, i_hi: int, count: int):
        """count squarings over exponent bits i_hi .. i_hi-count+1; e_words is (lanes, nwords) uint32."""
        w = np.ascontiguousarray(e_words, dtype=np.uint32)
        if w.ndim == 1:
            w = np.tile(w, (self.lanes, 1))
        check(lib().ctw_prp_square_bits(self._h, ptr(w), w.shape[1], i_hi, count))

    # -- results (reference transform.h) --
    def get_int(self, reg: int = 0) -> np.ndarray:
        out = np.zeros((self.lanes, self.D), dtype=np.uint32)
        check(lib().ctw_prp_get_digits(self._h, reg, ptr(out)))
        return out

    def is_prime(self, reg: int = 0):
        prp = np.zeros(self.lanes, dtype=np.uint8)
        r64 = np.zeros(self.lanes, dtype=np.uint64)
        check(lib().ctw_prp_is_prime(self._h, reg, ptr(prp), ptr(r64)))
        return prp.astype(bool), r64

    def read_regs(self, first: int = 0, nregs: int = 1) -> np.ndarray:
        out = np.zeros((nregs, self.lanes, self.regD), dtype=np.int32)
        check(lib().ctw_prp_read_regs(self._h, first, nregs, ptr(out)))
        return out

    def write_regs(self, regs: np.ndarray, first: int = 0):
        arr = np.ascontiguousarray(regs, dtype=np.int32)
        nregs = arr.size // (self.lanes * self.regD)
        check(lib().ctw_prp_write_regs(self._h, first, nregs, ptr(arr)))

    def run(self, b):
        """Whole test with Gerbicz-Li of up to `lanes` values of b: (is_prp, res64, gl_ok)."""
        arr = np.ascontiguousarray(b, dtype=np.uint32)
        n = arr.size
        prp = np.zeros(n, dtype=np.uint8)
        r64 = np.zeros(n, dtype=np.uint64)
        gl = np.zeros(n, dtype=np.uint8)
        check(lib().ctw_prp_run(self._h, ptr(arr), n, ptr(prp), ptr(r64), ptr(gl)))
        return prp.astype(bool), r64, gl.astype(bool)

    def run_ex(self, b, checkpoint=None, i_start: int = -1):
        """run() with checkpoints and resume, as cyclo::check(b, ctx, k, ri)
        (cyclo/src/cyclo.h:252-377): checkpoint(i) is called on the host after
        every Gerbicz-Li multiply, i being the next exponent bit, with the device
        idle (registers 0 = x and 1 = d may be read or written there); a true
        return stops the run (CtwError with CTW_STOPPED).  i_start >= 0 resumes
        before bit i_start from registers 0 and 1 as they are."""
        arr = np.ascontiguousarray(b, dtype=np.uint32)
        n = arr.size
        prp = np.zeros(n, dtype=np.uint8)
        r64 = np.zeros(n, dtype=np.uint64)
        gl = np.zeros(n, dtype=np.uint8)
        errors = []

        def trampoline(_user, i):
            try:
                return 1 if checkpoint(int(i)) else 0
            except Exception as e:      # stop the run, re-raise below
                errors.append(e)
                return 1

        cb = _CHECKPOINT_FN(trampoline) if checkpoint else None
        rc = lib().ctw_prp_run_ex(self._h, ptr(arr), n, i_start, ctypes.cast(cb, ctypes.c_void_p) if cb else None,
                                  None, ptr(prp), ptr(r64), ptr(gl))
        if errors:
            raise errors[0]
        check(rc)
        return prp.astype(bool), r64, gl.astype(bool)

    # -- plumbing --
    def sync(self):
        check(lib().ctw_prp_sync(self._h))

    @property
    def stream(self) -> int:
        return lib().ctw_prp_stream(self._h) or 0

    def geometry(self):
        c, t, s = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        check(lib().ctw_prp_geometry(self._h, ctypes.byref(c), ctypes.byref(t), ctypes.byref(s)))
        return {"ctas_per_lane": c.value, "threads": t.value, "smem_bytes": s.value}

    @property
    def launches(self) -> int:
        return int(lib().ctw_prp_launches(self._h))


def prp_test(b_values, n: int, base: int = 2, lanes: int | None = None, csize: int = 8, minus: bool = False):
    """Fermat-test b^(2^n) - b^(2^(n-1)) + 1 (minus: ... - 1) for every b: list of (b, is_prp, res64, gl_ok)."""
    b_values = [int(x) for x in b_values]
    lanes = lanes or min(64, max(1, len(b_values)))
    out = []
    with PrpEngine(n, lanes, csize=csize, base=base, minus=minus) as eng:
        for i in range(0, len(b_values), lanes):
            chunk = b_values[i:i + lanes]
            prp, r64, gl = eng.run(chunk)
            out += [(bb, bool(p), int(r), bool(g)) for bb, p, r, g in zip(chunk, prp, r64, gl)]
    return out


def res64_string(r: int) -> str:
    """RES64 as the reference prints it (cyclo/src/cyclo.h:50-56)."""
    return f"{r:016X}"
