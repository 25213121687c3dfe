"""ORACLE — test infrastructure only.

Python access to the CPU restatement of the reference (``cpu_prp.c``,
``cpu_sieve.c``), to the reference CPU sieve compiled unchanged (``_ref/``,
present only where the reference source was available at build time), and to
GMP (``libgmp.so.10``, prototypes declared here; the header is not installed).

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline / reference
legs of ``bench.py`` may import this module.  The product never does.

Canonical results follow the reference's definitions:
  * N+ = b^D - b^{D/2} + 1 (= Phi_{3D}(b)), N- = b^D - b^{D/2} - 1, D = 2^n
    (cyclo/src/cyclo.h:261-267, sieve/CPU/ctsieve.cpp:434-439);
  * the Fermat residue r = base^(N-1) mod N, RES64 = r mod 2^64, PRP iff r == 1
    (cyclo/src/transform.h:600-636).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
_REF_PATH = os.path.join(HERE, "_ref", "libctsieve_ref.so")
_lock = threading.Lock()
_lib = None
_ref = None
_gmp = None


def build(force: bool = False) -> str:
    """Compile the C restatement (make -C oracle)."""
    if force or not os.path.exists(_LIB_PATH):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return _LIB_PATH


def build_ref(ref_dir: str | None) -> str | None:
    """Compile the reference CPU sieve from its own source, ``ref_dir`` being the
    reference checkout (the directory holding ``sieve/``); None or a missing
    source leaves it unbuilt (a machine without the reference)."""
    if os.path.exists(_REF_PATH):
        return _REF_PATH
    if not ref_dir or not os.path.exists(os.path.join(ref_dir, "sieve", "CPU", "ctsieve.cpp")):
        return None
    subprocess.run(["make", "-s", "-C", HERE, "ref", "REF=" + ref_dir], check=True)
    return _REF_PATH if os.path.exists(_REF_PATH) else None


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = ctypes.CDLL(_LIB_PATH)
            vp, i32, u32, u64, sz = ctypes.c_void_p, ctypes.c_int, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_size_t
            L.orc_prp_tables_create.restype = vp
            L.orc_prp_tables_create.argtypes = [i32]
            L.orc_prp_tables_destroy.argtypes = [vp]
            L.orc_square_dup.argtypes = [vp, vp, u32, i32, i32]
            L.orc_mul.argtypes = [vp, vp, vp, u32, i32]
            L.orc_poly_mul_coeffs.argtypes = [vp, vp, vp, vp]
            L.orc_get_int.argtypes = [sz, vp, u32, vp]
            L.orc_get_int.restype = i32
            L.orc_is_prime.argtypes = [sz, vp, u32, vp, vp]
            L.orc_is_prime.restype = i32
            L.orc_prp_check.argtypes = [i32, u32, u32, vp, sz, i32, vp, vp, vp, vp]
            L.orc_prp_check.restype = i32
            L.orc_square_loop.argtypes = [vp, vp, u32, i32, i32, vp, sz, ctypes.c_long, ctypes.c_long]
            L.orc_sieve.argtypes = [i32, u64, u64, u64, u64, i32, vp, i32, vp, vp]
            L.orc_sieve.restype = i32
            L.orc_crc32.argtypes = [u32, vp, sz]
            L.orc_crc32.restype = u32
            _lib = L
    return _lib


def ref_lib():
    """The reference CPU sieve library, or None where it was not built."""
    global _ref
    with _lock:
        if _ref is None:
            path = _REF_PATH if os.path.exists(_REF_PATH) else None
            if path is None:
                return None
            L = ctypes.CDLL(path)
            u64 = ctypes.c_uint64
            L.ref_sieve.argtypes = [ctypes.c_int, u64, u64, u64, u64, u64, u64, ctypes.c_int,
                                    ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
            L.ref_sieve.restype = ctypes.c_int
            _ref = L
    return _ref


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


# ----------------------------------------------------------------------------
# Numbers
# ----------------------------------------------------------------------------

def n_plus(b: int, ln: int) -> int:
    d = 1 << ln
    return b ** d - b ** (d // 2) + 1


def n_minus(b: int, ln: int) -> int:
    d = 1 << ln
    return b ** d - b ** (d // 2) - 1


def exponent(b: int, ln: int) -> int:
    """E = N+ - 1 = b^D - b^{D/2} (cyclo/src/cyclo.h:261-267)."""
    d = 1 << ln
    h = b ** (d // 2)
    return h * h - h


def int_to_words(e: int) -> np.ndarray:
    nb = max(1, (e.bit_length() + 31) // 32)
    return np.frombuffer(e.to_bytes(nb * 4, "little"), dtype=np.uint32).copy()


def digits_to_int(d, b: int) -> int:
    """sum d_j b^j for a digit sequence (signed digits allowed)."""
    d = [int(x) for x in d]

    def rec(lo, hi):
        if hi - lo <= 32:
            v = 0
            for j in range(hi - 1, lo - 1, -1):
                v = v * b + d[j]
            return v, b ** (hi - lo)
        mid = (lo + hi) // 2
        a, pa = rec(lo, mid)
        c, pc = rec(mid, hi)
        return a + c * pa, pa * pc

    return rec(0, len(d))[0]


def int_to_digits(v: int, b: int, n: int) -> list[int]:
    """Canonical base-b digits (n of them) of 0 <= v < b^n."""
    if n <= 64:
        out = []
        for _ in range(n):
            v, r = divmod(v, b)
            out.append(r)
        return out
    h = n // 2
    hi, lo = divmod(v, b ** h)
    return int_to_digits(lo, b, h) + int_to_digits(hi, b, n - h)


# ----------------------------------------------------------------------------
# GMP (libgmp.so.10), prototypes declared by hand
# ----------------------------------------------------------------------------

class _Mpz(ctypes.Structure):
    _fields_ = [("alloc", ctypes.c_int), ("size", ctypes.c_int), ("d", ctypes.c_void_p)]


def gmp():
    global _gmp
    with _lock:
        if _gmp is None:
            for name in ("libgmp.so.10", "libgmp.so"):
                try:
                    g = ctypes.CDLL(name)
                    break
                except OSError:
                    g = None
            if g is None:
                _gmp = False
            else:
                p = ctypes.POINTER(_Mpz)
                g.__gmpz_init.argtypes = [p]
                g.__gmpz_clear.argtypes = [p]
                g.__gmpz_import.argtypes = [p, ctypes.c_size_t, ctypes.c_int, ctypes.c_size_t, ctypes.c_int,
                                            ctypes.c_size_t, ctypes.c_void_p]
                g.__gmpz_export.restype = ctypes.c_void_p
                g.__gmpz_export.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_size_t), ctypes.c_int,
                                            ctypes.c_size_t, ctypes.c_int, ctypes.c_size_t, p]
                g.__gmpz_powm.argtypes = [p, p, p, p]
                g.__gmpz_sizeinbase.restype = ctypes.c_size_t
                g.__gmpz_sizeinbase.argtypes = [p, ctypes.c_int]
                _gmp = g
    return _gmp or None


def _to_mpz(g, z, v: int):
    assert v >= 0
    nb = max(1, (v.bit_length() + 7) // 8)
    buf = v.to_bytes(nb, "little")
    g.__gmpz_import(ctypes.byref(z), nb, -1, 1, 0, 0, buf)


def _from_mpz(g, z) -> int:
    nbits = g.__gmpz_sizeinbase(ctypes.byref(z), 2)
    nb = (nbits + 7) // 8 + 1
    buf = ctypes.create_string_buffer(nb)
    cnt = ctypes.c_size_t(0)
    g.__gmpz_export(buf, ctypes.byref(cnt), -1, 1, 0, 0, ctypes.byref(z))
    return int.from_bytes(buf.raw[:cnt.value], "little")


def powmod(base: int, e: int, m: int) -> int:
    """base^e mod m with GMP when available, else Python's pow."""
    g = gmp()
    if not g:
        return pow(base, e, m)
    zs = [_Mpz() for _ in range(4)]
    for z in zs:
        g.__gmpz_init(ctypes.byref(z))
    try:
        _to_mpz(g, zs[1], base)
        _to_mpz(g, zs[2], e)
        _to_mpz(g, zs[3], m)
        g.__gmpz_powm(ctypes.byref(zs[0]), ctypes.byref(zs[1]), ctypes.byref(zs[2]), ctypes.byref(zs[3]))
        return _from_mpz(g, zs[0])
    finally:
        for z in zs:
            g.__gmpz_clear(ctypes.byref(z))


def fermat(b: int, ln: int, base: int = 2, minus: bool = False):
    """(r, res64, is_prp) for N = N+ (or N-) with r = base^(N-1) mod N."""
    N = n_minus(b, ln) if minus else n_plus(b, ln)
    r = powmod(base, N - 1, N)
    return r, r & (2 ** 64 - 1), r == 1


def partial_residue(b: int, ln: int, base: int, k: int) -> int:
    """Register value after the first k squarings of the left-to-right loop:
    base^(E >> (L - k)) mod N+, L = bit length of E."""
    E = exponent(b, ln)
    L = E.bit_length()
    N = n_plus(b, ln)
    return pow(base, E >> (L - k), N) if k <= L else None


# ----------------------------------------------------------------------------
# PRP restatement
# ----------------------------------------------------------------------------

class Tables:
    def __init__(self, ln: int):
        self.ln = ln
        self.n = 1 << ln
        self._h = lib().orc_prp_tables_create(ln)

    def close(self):
        if self._h:
            lib().orc_prp_tables_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def square_dup(self, x: np.ndarray, b: int, mult: int = 1, csize: int = 16):
        assert x.dtype == np.int32 and x.size == self.n
        lib().orc_square_dup(self._h, _ptr(x), b, mult, csize)

    def mul(self, x: np.ndarray, y: np.ndarray, b: int, csize: int = 16):
        lib().orc_mul(self._h, _ptr(x), _ptr(y), b, csize)

    def poly_mul(self, x: np.ndarray, y: np.ndarray) -> list[int]:
        out = np.zeros(2 * self.n, dtype=np.int64)
        lib().orc_poly_mul_coeffs(self._h, _ptr(x), _ptr(y), _ptr(out))
        lo = out[0::2].view(np.uint64)
        hi = out[1::2]
        return [int(h) * 2 ** 64 + int(l) for l, h in zip(lo, hi)]

    def square_loop(self, x, b, mult, csize, ewords, i_hi, count):
        lib().orc_square_loop(self._h, _ptr(x), b, mult, csize, _ptr(ewords), ewords.size, i_hi, count)


def get_int(x: np.ndarray, b: int) -> np.ndarray:
    out = np.zeros(x.size, dtype=np.uint32)
    rc = lib().orc_get_int(x.size, _ptr(np.ascontiguousarray(x, dtype=np.int32)), b, _ptr(out))
    if rc != 0:
        raise RuntimeError("getInt failed")
    return out


def is_prime(c: np.ndarray, b: int):
    prm = ctypes.c_int(0)
    r64 = ctypes.c_uint64(0)
    err = lib().orc_is_prime(c.size, _ptr(c), b, ctypes.byref(prm), ctypes.byref(r64))
    return bool(prm.value), r64.value, bool(err)


def prp_check(b: int, ln: int, base: int = 2, csize: int = 16):
    """Whole test as cyclo::check does for one lane: (is_prp, res64, gl_ok, digits)."""
    E = exponent(b, ln)
    ew = int_to_words(E)
    prm = ctypes.c_int(0)
    r64 = ctypes.c_uint64(0)
    gl = ctypes.c_int(0)
    digits = np.zeros(1 << ln, dtype=np.uint32)
    rc = lib().orc_prp_check(ln, b, base, _ptr(ew), ew.size, csize, ctypes.byref(prm), ctypes.byref(r64),
                             ctypes.byref(gl), _ptr(digits))
    if rc != 0:
        raise RuntimeError("oracle PRP computation failed")
    return bool(prm.value), r64.value, bool(gl.value), digits


# ----------------------------------------------------------------------------
# Sieve restatement and the reference sieve
# ----------------------------------------------------------------------------

def pos_p_default(n: int) -> tuple[int, int]:
    """'ini' limits of the + sieve (ctsieve.cpp:800-802): (p_min, p_max)."""
    return 3 * (1 << n) + 1, 3 * (100000000 << n) + 1


def sieve(n: int, b_min: int, b_max: int, p_min: int, p_max: int, mode: int,
          bits: np.ndarray | None = None, threads: int = 1):
    """Strike b in [b_min, b_max] for mode +1 (p = 3k2^n+1) or -1 (p = 10k+-1).
    Returns (bits uint8 array, p_last)."""
    size = b_max - b_min + 1
    if bits is None:
        bits = np.zeros(size, dtype=np.uint8)
    p_last = ctypes.c_uint64(0)
    err = np.zeros(2, dtype=np.uint64)
    rc = lib().orc_sieve(n, b_min, b_max, p_min, p_max, mode, _ptr(bits), threads, ctypes.byref(p_last), _ptr(err))
    if rc != 0:
        raise RuntimeError(f"Calculation error: p = {int(err[0])}, b = {int(err[1])}")
    return bits, p_last.value


def ref_sieve(n: int, b_min: int, b_max: int, p_max_pos: int, p_max_neg: int, mode: int,
              p_min_pos: int | None = None, p_min_neg: int = 11, write_dir: str | None = None):
    """Run the reference CPU sieve itself.  Returns (bits, p_last_pos, p_last_neg) or None."""
    L = ref_lib()
    if L is None:
        return None
    if p_min_pos is None:
        p_min_pos = 3 * (1 << n) + 1
    bits = np.zeros(b_max - b_min + 1, dtype=np.uint8)
    lp, ln_ = ctypes.c_uint64(0), ctypes.c_uint64(0)
    cwd = os.getcwd()
    try:
        if write_dir:
            os.chdir(write_dir)
        rc = L.ref_sieve(n, b_min, b_max, p_min_pos, p_max_pos, p_min_neg, p_max_neg, mode, _ptr(bits),
                         ctypes.byref(lp), ctypes.byref(ln_), 1 if write_dir else 0)
    finally:
        os.chdir(cwd)
    if rc != 0:
        raise RuntimeError("reference sieve raised")
    return bits, lp.value, ln_.value


def crc32(data: bytes, crc: int = 0) -> int:
    buf = np.frombuffer(data, dtype=np.uint8)
    return lib().orc_crc32(crc, _ptr(buf) if buf.size else None, buf.size)


def sv_bytes(bits: np.ndarray, p_min_pos: int, p_min_neg: int) -> bytes:
    """sv_<n>_<bmin>_<bmax>.dat as the reference writes it (ctsieve.cpp:591-626)."""
    idx = np.flatnonzero(bits == 0).astype(np.uint32)
    head = np.array([p_min_pos, p_min_neg, idx.size], dtype=np.uint64).tobytes()
    body = idx.tobytes()
    c = crc32(head[0:8])
    c = crc32(head[8:16], c)
    c = crc32(head[16:24], c)
    c = crc32(body, c)
    c = (~c & 0xffffffff) ^ 0xa23777ac
    return head + body + np.array([c], dtype=np.uint32).tobytes()


def cand_text(bits: np.ndarray, b_min: int) -> str:
    idx = np.flatnonzero(bits == 0)
    return "".join(f"{b_min + int(i)}\n" for i in idx)
