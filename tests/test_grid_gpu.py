"""The grid kernel (degrees 2^16..2^18 on 32 to 128 CTAs of one cooperative
launch) on the GPU: registers bit-exact with the oracle and with the cluster
kernel, on two and three primes, one and two lanes, and partial residues of
the real exponent against GMP.  Integer work: tolerance 0."""
import hashlib
import json
import os
import random

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _digits(rng, lanes, D, b):
    return np.array([[rng.randint(-(b[l] - 1), b[l] - 1) for _ in range(D)] for l in range(lanes)], dtype=np.int32)


@pytest.mark.parametrize("ln,lanes,csize,primes", [(17, 1, 8, 2), (17, 2, 32, 3), (18, 1, 16, 2), (18, 2, 64, 3)])
def test_grid_registers_bit_exact(native, ln, lanes, csize, primes):
    from ctwin_gb300 import PrpEngine
    rng = random.Random(ln * 100 + lanes * 10 + primes)
    D = 1 << ln
    b = [rng.randrange(1 << 16, 1 << 20) for _ in range(lanes)]        # within the two-prime bound
    x0 = _digits(rng, lanes, D, b)
    y0 = _digits(rng, lanes, D, b)
    masks = [rng.getrandbits(lanes) for _ in range(3)]
    with PrpEngine(ln, lanes, csize=csize) as eng:
        # the grid split: 2048 coefficients per CTA where the lanes fit (one lane of 2^18), else 4096
        assert eng.geometry()["ctas_per_lane"] == (128 if (ln == 18 and lanes == 1) else 64)
        eng.set_b(b)
        eng.set_prime_count(0 if primes == 2 else 3)
        assert eng.prime_count == primes
        eng.write_regs(np.stack([x0, y0]), 0)
        for m in masks:
            eng.square_dup(m)
        eng.mul()
        got = eng.read_regs(0, 1)[0]
    with O.Tables(ln) as t:
        for l in range(lanes):
            x = x0[l].copy()
            for m in masks:
                t.square_dup(x, b[l], 2 if (m >> l) & 1 else 1, csize)
            t.mul(x, y0[l], b[l], csize)
            assert np.array_equal(got[l], x), f"lane {l} differs from the oracle"


@pytest.mark.parametrize("ln,lg,csize,primes", [(16, 5, 16, 2), (17, 6, 32, 3), (18, 7, 16, 3), (18, 7, 8, 2)])
def test_grid_2048_registers_bit_exact(native, ln, lg, csize, primes):
    """The grid kernel with 2048 coefficients per CTA (2^16 on 32 CTAs, 2^17 on
    64, 2^18 on 128 with 16-column runs)."""
    from ctwin_gb300 import PrpEngine
    rng = random.Random(ln * 11 + lg)
    D = 1 << ln
    b = [rng.randrange(1 << 16, 1 << 20)]
    x0 = _digits(rng, 1, D, b)
    y0 = _digits(rng, 1, D, b)
    with PrpEngine(ln, 1, csize=csize, log2_ctas=lg) as eng:
        assert eng.geometry()["ctas_per_lane"] == 1 << lg
        eng.set_b(b)
        eng.set_prime_count(0 if primes == 2 else 3)
        assert eng.prime_count == primes
        eng.write_regs(np.stack([x0, y0]), 0)
        for m in (1, 0, 1):
            eng.square_dup(m)
        eng.mul()
        got = eng.read_regs(0, 1)[0]
    with O.Tables(ln) as t:
        x = x0[0].copy()
        for m in (1, 0, 1):
            t.square_dup(x, b[0], 2 if m else 1, csize)
        t.mul(x, y0[0], b[0], csize)
    assert np.array_equal(got[0], x)


@pytest.mark.parametrize("ln", [17, 18])
def test_grid_matches_cluster_kernel(native, ln):
    """The same squarings with b near 2^30 (three primes, 128-bit carries) on the
    grid split and on the 16-CTA cluster split give the same registers."""
    from ctwin_gb300 import PrpEngine
    rng = random.Random(ln)
    D = 1 << ln
    b = [rng.randrange(1 << 30, 1 << 31)]
    x0 = _digits(rng, 1, D, b)
    out = []
    for lg in (-1, 4):
        with PrpEngine(ln, 1, csize=16, log2_ctas=lg) as eng:
            assert eng.geometry()["ctas_per_lane"] == ((1 << (ln - 11)) if lg < 0 else 16)
            eng.set_b(b)
            eng.write_regs(x0[None], 0)
            for m in (1, 0, 1):
                eng.square_dup(m)
            out.append(eng.read_regs(0, 1)[0])
    assert np.array_equal(out[0], out[1])


@pytest.mark.parametrize("ln,base", [(17, 3), (18, 2)])
def test_grid_partial_residue_matches_gmp(native, ln, base):
    """The first K squarings of the real exponent on the grid give base^(E >> (L-K)) mod N+."""
    from ctwin_gb300 import PrpEngine
    rng = random.Random(ln * 7 + base)
    b = rng.randrange(2 ** 20, 2 ** 21)
    E = O.exponent(b, ln)
    L = E.bit_length()
    K = 40
    with PrpEngine(ln, 1, base=base) as eng:
        assert eng.geometry()["ctas_per_lane"] == 1 << (ln - 11)
        eng.set_b([b])
        eng.set(1)
        eng.square_bits(O.int_to_words(E), L - 1, K)
        dig = eng.get_int(0)[0]
    assert O.digits_to_int(dig, b) == O.powmod(base, E >> (L - K), O.n_plus(b, ln))


@pytest.mark.parametrize("ln,primes", [(17, 2), (18, 3)])
def test_grid_prefix_4096_matches_gmp(native, golden_dir, ln, primes):
    """The first 4096 squarings of the single-test workload's exponent
    (b = 1330358) on the default grid split, against GMP through a hash of the
    whole residue (tests/golden/prefix_gmp.json)."""
    from ctwin_gb300 import PrpEngine
    c = next(c for c in json.load(open(os.path.join(golden_dir, "prefix_gmp.json"))) if c["n"] == ln)
    b, K = c["b"], c["K"]
    E = O.exponent(b, ln)
    L = E.bit_length()
    with PrpEngine(ln, 1) as eng:
        assert eng.geometry()["ctas_per_lane"] == 1 << (ln - 11)
        eng.set_b([b])
        assert eng.prime_count == primes
        eng.set(1)
        eng.square_bits(O.int_to_words(E), L - 1, K)
        dig = eng.get_int(0)[0]
    assert all(0 <= int(v) < b for v in dig)
    r = O.digits_to_int(dig, b)
    raw = r.to_bytes((O.n_plus(b, ln).bit_length() + 7) // 8, "little")
    assert f"{r & (2 ** 64 - 1):016X}" == c["low64"]
    assert hashlib.sha256(raw).hexdigest() == c["sha256"]


def test_grid_too_many_lanes_falls_back_to_clusters(native):
    """More lanes than one cooperative launch holds: the default split is the
    16-CTA cluster; an explicit grid split is refused."""
    from ctwin_gb300 import CtwError, PrpEngine
    with PrpEngine(18, 8) as eng:
        assert eng.geometry()["ctas_per_lane"] == 16
    with pytest.raises(CtwError):
        PrpEngine(18, 8, log2_ctas=6)


@pytest.mark.parametrize("csize,ctas", [(8, 64), (32, 32), (64, 32)])
def test_grid_reshapes_for_long_chunks(native, csize, ctas):
    """One lane of degree 2^16 runs on 64 CTAs of 1024 coefficients (column runs
    of 16); a longer carry chunk moves the handle to 32 CTAs of 2048 (runs of
    64) without losing its registers, which stay bit-exact with the oracle."""
    from ctwin_gb300 import PrpEngine
    rng = random.Random(csize)
    ln, D = 16, 1 << 16
    b = [rng.randrange(1 << 18, 1 << 20)]
    x0 = _digits(rng, 1, D, b)
    with PrpEngine(ln, 1) as eng:
        assert eng.geometry()["ctas_per_lane"] == 64
        eng.set_b(b)
        eng.write_regs(x0[None], 0)
        eng.set_csize(csize)                      # may re-split the handle
        assert eng.geometry()["ctas_per_lane"] == ctas
        assert np.array_equal(eng.read_regs(0, 1)[0], x0)
        for m in (1, 1, 0):
            eng.square_dup(m)
        got = eng.read_regs(0, 1)[0]
    with O.Tables(ln) as t:
        x = x0[0].copy()
        for m in (1, 1, 0):
            t.square_dup(x, b[0], 2 if m else 1, csize)
    assert np.array_equal(got[0], x)
