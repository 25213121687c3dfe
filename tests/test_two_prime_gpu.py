"""Two-prime launches on the GPU: registers bit-exact with the oracle and with
the same engine held to three primes, the switch between two and three primes
in a pool as tests come and go, and whole tests against GMP on both sides of
the bound (tests/golden/pool_gmp.json).  Integer work: tolerance 0."""
import json
import math
import os
import random

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

Q0, Q1 = 1053818881, 1012924417
HERE = os.path.dirname(os.path.abspath(__file__))


def b_limit(ln):
    """Largest b that runs on two primes at degree 2^ln (N+): 3 D (b + 1)^2 < q0 q1."""
    b = math.isqrt(Q0 * Q1 // (3 << ln))
    while 3 * (1 << ln) * (b + 1) ** 2 >= Q0 * Q1:
        b -= 1
    return b


def gold():
    d = json.load(open(os.path.join(HERE, "golden", "pool_gmp.json")))
    return {(x["b"], x["n"], x["base"]): x for x in d if x["form"] == "+"}


@pytest.mark.parametrize("ln,lg,csize", [(8, 0, 8), (10, 0, 16), (11, 0, 8), (12, 0, 8), (12, 0, 16), (13, 0, 8),
                                         (13, 1, 8), (14, 0, 32), (14, 2, 16), (15, 3, 8), (16, 4, 8), (16, 4, 16),
                                         (17, 4, 16)])
def test_two_prime_registers_bit_exact(native, ln, lg, csize):
    """square_dup and mul on two primes give the reference's registers, with b up
    to the bound (digits at the bound's extreme included)."""
    from ctwin_gb300 import PrpEngine
    rng = random.Random(70 + ln * 8 + lg)
    lanes, D = 3, 1 << ln
    top = min(b_limit(ln), (1 << 31) - 1)
    b = [top, rng.randrange(1 << 16, top), rng.randrange(64, 1 << 12)]
    x0 = np.array([[rng.choice((-1, 1)) * (b[l] - 1) if rng.random() < 0.3 else rng.randint(-(b[l] - 1), b[l] - 1)
                    for _ in range(D)] for l in range(lanes)], dtype=np.int32)
    y0 = np.array([[rng.randint(-(b[l] - 1), b[l] - 1) for _ in range(D)] for l in range(lanes)], dtype=np.int32)
    masks = [rng.getrandbits(lanes) for _ in range(4)]
    got = {}
    for count in (0, 3):
        with PrpEngine(ln, lanes, csize=csize, log2_ctas=lg) as eng:
            eng.set_b(b)
            eng.set_prime_count(count)
            assert eng.prime_count == (2 if count == 0 else 3)
            eng.write_regs(np.stack([x0, y0]), 0)
            for m in masks:
                eng.square_dup(m)
            eng.mul()
            got[count] = eng.read_regs(0, 1)[0]
    assert np.array_equal(got[0], got[3]), "two and three primes differ"
    with O.Tables(ln) as t:
        for l in range(lanes):
            x = x0[l].copy()
            for m in masks:
                t.square_dup(x, b[l], 2 if (m >> l) & 1 else 1, csize)
            t.mul(x, y0[l], b[l], csize)
            assert np.array_equal(got[0][l], x), f"lane {l} differs from the oracle"


def test_engine_takes_three_primes_above_the_bound(native):
    from ctwin_gb300 import PrpEngine
    with PrpEngine(16, 2) as eng:
        eng.set_b([1 << 20, b_limit(16)])
        assert eng.prime_count == 2
        eng.set_b([1 << 20, b_limit(16) + 1])
        assert eng.prime_count == 3
    with PrpEngine(18, 1, log2_ctas=4) as eng:    # no two-prime kernel for 16384 coefficients per CTA
        eng.set_b([1000])
        assert eng.prime_count == 3
    with PrpEngine(17, 1) as eng:                 # the grid kernel has one
        eng.set_b([1000])
        assert eng.prime_count == 2


@pytest.mark.parametrize("ln", [12, 13])
def test_engine_runs_both_sides_of_the_bound_match_gmp(native, ln):
    from ctwin_gb300 import PrpEngine
    g = gold()
    cases = sorted(b for (b, n, base) in g if n == ln and base == 2 and b > 6000000)
    assert len(cases) >= 2
    for b in cases:
        with PrpEngine(ln, 1) as eng:
            eng.set_b([b])
            want_np = 2 if b <= b_limit(ln) else 3
            assert eng.prime_count == want_np, b
            prp, r64, ok = eng.run([b])
        want = g[(b, ln, 2)]
        assert ok[0] and (bool(prp[0]), int(r64[0])) == (want["prp"], int(want["res64"], 16)), b


def test_pool_switches_prime_count(native):
    """A pool launches on two primes while its tests allow it, on three while a
    test above the bound is resident, and on two again once it has finished."""
    from ctwin_gb300 import Pool
    g = gold()
    small = [65537, 70001, 100003]
    big = 16777213
    with Pool(12, 8) as p:
        assert p.prime_count == 2
        for i, b in enumerate(small):
            p.admit(b, tag=i)
        assert p.prime_count == 2
        p.admit(big, tag=99)
        assert p.prime_count == 3
        res = p.run_to_completion()
        assert p.prime_count == 2           # finished slots compute on zeros with b = 2^16 + 1
        p.admit(9000001, tag=7)
        assert p.prime_count == 2
        res += p.run_to_completion()
    assert sorted(r["b"] for r in res) == sorted(small + [big, 9000001])
    for r in res:
        want = g[(r["b"], 12, 2)]
        assert r["status"] == 0 and r["gl_ok"], r
        assert (r["is_prp"], r["res64"]) == (want["prp"], int(want["res64"], 16)), r


def test_pool_two_and_three_primes_agree(native):
    """The same 40 tests at degree 2^14 on two primes and held to three.  40
    lanes of 4 CTAs fill the GPU, so the two-prime launches run at two CTAs per
    SM (roots from L2) while the three-prime ones keep one."""
    from ctwin_gb300 import Pool
    bs = [(1 << 21) + 2 * i + 1 for i in range(38)] + [4000037, 4600003]
    out = {}
    for count in (0, 3):
        with Pool(14, 40) as p:
            p.set_prime_count(count)
            p.admit_many(bs)
            assert p.prime_count == (2 if count == 0 else 3)
            out[count] = {r["b"]: (r["is_prp"], r["res64"], r["status"], r["gl_ok"]) for r in p.run_to_completion()}
    assert out[0] == out[3]
    assert all(v[2] == 0 and v[3] for v in out[0].values())


def test_minus_two_primes_match_three(native):
    """N- at degrees 2^11 (one CTA) and 2^13 (4 CTAs of 4096) on two primes."""
    from ctwin_gb300 import PrpEngine
    for ln in (11, 13):
        bs = [300007, 1000003]
        res = {}
        for count in (0, 3):
            with PrpEngine(ln, len(bs), minus=True) as eng:
                eng.set_b(bs)
                eng.set_prime_count(count)
                assert eng.prime_count == (2 if count == 0 else 3)
                res[count] = eng.run(bs)
        for a, c in zip(res[0], res[3]):
            assert list(a) == list(c)
        assert all(res[0][2])


def test_server_separates_prime_classes(native):
    """Degree-2^12 requests on both sides of the bound, interleaved: every result
    equals GMP's; the server holds them in pools of their own class (b above
    the bound never holds the others at three primes)."""
    from ctwin_gb300 import Server, two_primes
    g = gold()
    bs = [65537, 9999991, 70001, 16777213, 100003, 9000001]
    assert [two_primes(12, b) for b in bs] == [True, False, True, False, True, True]
    with Server(hbm_budget_bytes=1 << 30, max_slots=8, ticks_per_launch=2) as s:
        for i, b in enumerate(bs):
            s.submit(12, b, tag=i)
        res = s.drain(len(bs), timeout_s=300)
    assert sorted(r["tag"] for r in res) == list(range(len(bs)))
    for r in res:
        want = g[(r["b"], 12, 2)]
        assert r["status"] == 0 and r["gl_ok"], r
        assert (r["is_prp"], r["res64"]) == (want["prp"], int(want["res64"], 16)), r


@pytest.mark.parametrize("minus,ln,csize", [(True, 13, 16), (False, 15, 32)])
def test_dense_pool_matches_single_engine(native, minus, ln, csize):
    """A pool whose lanes fill the GPU (40 lanes of 4 or 8 CTAs: the dense
    two-CTA-per-SM build, roots from L2) gives every test the verdict and
    RES64 of the same test alone in an engine (one lane: the one-CTA-per-SM
    build), for N- at 2^13 and N+ at 2^15 with a longer carry chunk."""
    from ctwin_gb300 import Pool, PrpEngine
    rng = random.Random(ln + (100 if minus else 0))
    bs = sorted({rng.randrange(1 << 17, 1 << 20) for _ in range(40)})
    with Pool(ln, len(bs), csize=csize, minus=minus) as p:
        assert p.admit_many(bs) == len(bs)
        assert p.prime_count == 2
        res = {r["b"]: r for r in p.run_to_completion()}
    assert sorted(res) == bs
    for b in bs[:1] + bs[-1:]:
        with PrpEngine(ln, 1, csize=csize, minus=minus) as eng:
            prp, r64, ok = eng.run([b])
        r = res[b]
        assert r["status"] == 0 and r["gl_ok"] and ok[0], r
        assert (r["is_prp"], r["res64"]) == (bool(prp[0]), int(r64[0])), r
    assert all(r["status"] == 0 and r["gl_ok"] for r in res.values())
