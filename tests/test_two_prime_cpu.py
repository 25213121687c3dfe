"""The two-prime launches, checked without a GPU.

Two NTT primes (q0 q1 = 2^59.89) give the exact product of two residues when
every coefficient of the ring product lies in (-q0 q1 / 2, q0 q1 / 2).  The
engines take two primes when 2 * terms * (b + 1)^2 < q0 q1, with terms = 1.5 D
for N+ and Dn for the exact N- product, relying on |digit| <= b.  These tests
check on the oracle that the bound holds and is attained, that the reference's
carry keeps |digit| <= b, the two-prime CRT, and the library's decision."""
import random

import numpy as np
import pytest

from oracle import oracle as O

Q0, Q1 = 1053818881, 1012924417
P2 = Q0 * Q1


@pytest.mark.parametrize("ln", [8, 10])
def test_ring_product_bound_is_attained(ln):
    """|c_m| <= 1.5 D max|x| max|y| for X^D - X^{D/2} + 1, with equality for x = y = b."""
    D = 1 << ln
    b = 1000
    with O.Tables(ln) as t:
        full = np.full(D, b, dtype=np.int32)
        c = t.poly_mul(full, full)
        assert max(abs(v) for v in c) == 3 * D // 2 * b * b
        rng = np.random.default_rng(ln)
        for _ in range(3):
            x = rng.integers(-b, b + 1, D).astype(np.int32)
            y = rng.integers(-b, b + 1, D).astype(np.int32)
            assert max(abs(v) for v in t.poly_mul(x, y)) <= 3 * D // 2 * b * b


def test_minus_product_bound():
    """The exact product of two degree < Dn polynomials: |c_k| <= Dn b^2."""
    Dn, b = 256, 5000
    x = np.full(Dn, b, dtype=object)
    c = np.convolve(x, x)
    assert max(abs(v) for v in c) == Dn * b * b


@pytest.mark.parametrize("csize", [8, 16, 64])
def test_carry_keeps_digits_within_b(csize):
    """After each reference carry (normalize1 + normalize2) every digit has |d| <= b."""
    rng = random.Random(csize)
    ln = 10
    D = 1 << ln
    with O.Tables(ln) as t:
        for b in (65, 70001, 1330358, (1 << 30) + 3):
            x = np.array([rng.randint(-(b - 1), b - 1) for _ in range(D)], dtype=np.int32)
            for step in range(6):
                t.square_dup(x, b, 2 if step % 2 else 1, csize)
                assert int(np.abs(x.astype(np.int64)).max()) <= b


def garner2(r0, r1):
    """The device's two-prime CRT: x = r1 + q1 ((r0 - r1) q1^-1 mod q0), balanced."""
    a1 = ((r0 - r1) * pow(Q1, -1, Q0)) % Q0
    x = r1 + Q1 * a1
    return x - P2 if 2 * x > P2 else x


def test_garner2_recovers_balanced_values():
    rng = random.Random(3)
    vals = [0, 1, -1, (P2 - 1) // 2, -(P2 - 1) // 2] + [rng.randrange(-(P2 // 2), P2 // 2) for _ in range(2000)]
    for v in vals:
        assert garner2(v % Q0, v % Q1) == v


def _rule(ln, minus, b):
    terms = (1 << ln) if minus else 3 * (1 << ln) // 2
    return 2 * terms * (b + 1) ** 2 < P2


def test_library_decision_matches_the_bound(native_lib):
    """ctw_prp_two_primes follows 2 terms (b + 1)^2 < q0 q1 on the splits with a
    two-prime kernel (one CTA, or 4096 coefficients per CTA, clusters or grid)."""
    L = native_lib
    # N+: every degree; 2^17 and 2^18 run one candidate on the grid kernel, which has both counts
    for ln in range(8, 19):
        for b in (64, 65537, 1 << 20, (1 << 21) - 1, 2330079, 2330081, 6590461, 9320320, 9320322, (1 << 31) - 1):
            assert L.ctw_prp_two_primes(ln, 0, b) == int(_rule(ln, False, b)), (ln, b)
    # N-: transform degree 2^(ln+1) on one CTA up to 2^12 coefficients, else on
    # >= 4 CTAs; 4096 coefficients per CTA for ln = 13..15, 8192 on 16 CTAs for
    # ln = 16 (both have two-prime kernels), 2048 for ln = 12 (none)
    for ln in range(8, 17):
        split = ln != 12
        for b in (64, 300000, 1 << 21, 3 << 20, (1 << 31) - 1):
            assert L.ctw_prp_two_primes(ln, 1, b) == int(split and _rule(ln, True, b)), (ln, b)


def test_workloads_that_take_two_primes(native_lib):
    """One candidate of degree 2^16 with b < 2^21, and both forms at degree 2^11
    with b < 3 * 10^5, run on two primes; b = 2^24 at degree 2^12 does not."""
    L = native_lib
    assert L.ctw_prp_two_primes(16, 0, (1 << 21) - 1) == 1
    assert L.ctw_prp_two_primes(11, 0, 300000) == 1 and L.ctw_prp_two_primes(11, 1, 300000) == 1
    assert L.ctw_prp_two_primes(12, 0, 1 << 24) == 0
    assert L.ctw_prp_two_primes(15, 0, (1 << 22) - 1) == 0
