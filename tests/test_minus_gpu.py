"""Twin partner N- = b^D - b^{D/2} - 1 on the GPU.  The reference has no PRP
path for N- (it only sieves it, sieve/CPU/ctsieve.cpp:434-439, 728-787), so
parity is pinned by GMP: full Fermat tests against the GMP residues of
tests/golden/prp_gmp.json, and partial residues base^(E >> (L - K)) mod N- at
degrees up to 2^16."""
import json
import os
import random

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


def minus_cases(n, base=2):
    d = json.load(open(os.path.join(HERE, "golden", "prp_gmp.json")))
    return [(x["b"], int(x["res64"], 16), x["prp"]) for x in d if x["n"] == n and x["form"] == "-" and x["base"] == base]


@pytest.mark.parametrize("n,lanes", [(8, 64), (11, 64)])
def test_minus_run_matches_gmp(native, n, lanes):
    from ctwin_gb300 import PrpEngine
    cases = minus_cases(n)[:lanes]
    assert cases
    with PrpEngine(n, lanes, minus=True) as eng:
        prp, r64, gl = eng.run([c[0] for c in cases])
    for (b, want64, want_prp), p, r, g in zip(cases, prp, r64, gl):
        assert g, b
        assert (bool(p), int(r)) == (want_prp, want64), b


@pytest.mark.parametrize("base", [2, 3])
def test_minus_config1_survivors_match_gmp(native, base):
    """N- of the first 256 twin-sieve survivors of b in [100000, 300000) at
    n = 11, base 2 and 3, in vectors of 64 lanes."""
    from ctwin_gb300 import PrpEngine
    cases = minus_cases(11, base)
    assert len(cases) == 256
    for i in range(0, len(cases), 64):
        part = cases[i:i + 64]
        with PrpEngine(11, 64, base=base, minus=True) as eng:
            prp, r64, gl = eng.run([c[0] for c in part])
        for (b, want64, want_prp), p, r, g in zip(part, prp, r64, gl):
            assert g, b
            assert (bool(p), int(r)) == (want_prp, want64), b


def test_minus_finds_prps(native):
    """Every N- PRP of the golden n = 8 list comes out as residue 1."""
    from ctwin_gb300 import prp_test
    cases = minus_cases(8)
    hits = [c for c in cases if c[2]]
    assert hits, "golden list has no N- PRP at n = 8"
    res = prp_test([c[0] for c in hits], 8, minus=True)
    assert all(p and r == 1 and g for _, p, r, g in res)


@pytest.mark.parametrize("n", [9, 12, 13, 14, 15, 16])
def test_minus_partial_residue(native, n):
    """K squarings of the left-to-right loop: base^(E >> (L - K)) mod N-."""
    from ctwin_gb300 import PrpEngine
    rng = random.Random(n)
    b = rng.randrange(1 << 16, 1 << 21)
    D = 1 << n
    E = b ** D - b ** (D // 2) - 2
    L = E.bit_length()
    K = 200
    words = O.int_to_words(E)
    with PrpEngine(n, 1, minus=True) as eng:
        eng.set_b([b])
        eng.set(1)
        eng.square_bits(words, L - 1, K)
        got = eng.get_int(0)[0]
    N = b ** D - b ** (D // 2) - 1
    want = O.powmod(2, E >> (L - K), N)
    assert O.digits_to_int(got, b) == want
    assert all(int(v) < b for v in got)


def test_minus_mul(native):
    """ctw_prp_mul on N- registers: x * y mod N- for random residues."""
    from ctwin_gb300 import PrpEngine
    n, lanes = 12, 3
    rng = np.random.default_rng(7)
    bs = [70001, 100003, 1 << 20]
    with PrpEngine(n, lanes, minus=True) as eng:
        eng.set_b(bs)
        regs = np.zeros((2, lanes, 2 << n), dtype=np.int32)
        for l, b in enumerate(bs):
            regs[:, l, : 1 << n] = rng.integers(-(b // 2), b // 2, size=(2, 1 << n))
        eng.write_regs(regs, 0)
        eng.mul()
        got = eng.get_int(0)
    for l, b in enumerate(bs):
        N = b ** (1 << n) - b ** (1 << (n - 1)) - 1
        x = O.digits_to_int([int(v) for v in regs[0, l, : 1 << n]], b)
        y = O.digits_to_int([int(v) for v in regs[1, l, : 1 << n]], b)
        assert O.digits_to_int(got[l], b) == x * y % N


@pytest.mark.parametrize("n", [8, 11])
def test_minus_pool_matches_gmp(native, n):
    """N- tests in a pool (continuous batching on the degree-2D transform)."""
    from ctwin_gb300 import Pool
    cases = minus_cases(n)[:40]
    with Pool(n, 16, minus=True) as p:
        queue = [c[0] for c in cases]
        res = []
        while queue or p.info()["active"]:
            take = min(len(queue), 16 - p.info()["active"])
            if take:
                assert p.admit_many(queue[:take]) == take
                queue = queue[take:]
            p.run(4)
            p.collect(wait=True)
            res += p.results()
    want = {b: (prp, r64) for b, r64, prp in cases}
    assert sorted(r["b"] for r in res) == sorted(want)
    for r in res:
        assert r["status"] == 0 and r["gl_ok"] and r["log2_degree"] == n
        assert (r["is_prp"], r["res64"]) == want[r["b"]], r
