"""The PRP oracle (CPU restatement) pinned against the reference's own
known-answer vectors (cyclo/algo/algo.cpp:173-177) and against GMP."""
import json
import os
import random

import numpy as np
import pytest

from oracle import oracle as O


def test_algo_kat(golden_dir):
    kat = json.load(open(os.path.join(golden_dir, "algo_kat.json")))
    assert set(kat) == {"8", "16"}
    for n_str, expected in kat.items():
        n = int(n_str)
        ln = n.bit_length() - 1
        for e in (1, 2, 3):
            f = 10 ** e
            x = np.array([(i + 1) * f for i in range(n)], dtype=np.int32)
            with O.Tables(ln) as t:
                sq = t.poly_mul(x, x)
            assert [c // (f * f) for c in sq] == expected
            assert all(c % (f * f) == 0 for c in sq)


@pytest.mark.parametrize("ln", [3, 5, 8, 11])
def test_poly_square_matches_schoolbook(ln):
    rng = random.Random(ln)
    n = 1 << ln
    x = np.array([rng.randint(-2 ** 20, 2 ** 20) for _ in range(n)], dtype=np.int32)
    full = [0] * (2 * n)
    for i in range(n):
        for j in range(n):
            full[i + j] += int(x[i]) * int(x[j])
    for k in range(2 * n - 1, n - 1, -1):
        c = full[k]
        full[k] = 0
        full[k - n // 2] += c
        full[k - n] -= c
    with O.Tables(ln) as t:
        assert t.poly_mul(x, x) == full[:n]


@pytest.mark.parametrize("ln,b,csize", [(8, 100003, 8), (9, 2 ** 20 + 7, 16), (10, 65537, 32), (11, 299999, 64)])
def test_square_dup_value(ln, b, csize):
    rng = random.Random(b)
    n = 1 << ln
    N = O.n_plus(b, ln)
    x = np.zeros(n, dtype=np.int32)
    x[0] = 1
    v = 1
    with O.Tables(ln) as t:
        for it in range(40):
            m = rng.choice([1, 2, 3])
            t.square_dup(x, b, m, csize)
            v = v * v * m % N
    assert O.digits_to_int(O.get_int(x, b), b) == v


def test_gmp_fixture_small(golden_dir):
    cases = [c for c in json.load(open(os.path.join(golden_dir, "prp_gmp.json"))) if c["n"] == 8 and c["form"] == "+"]
    assert len(cases) > 100
    rng = random.Random(1)
    for c in rng.sample(cases, 12) + [c for c in cases if c["prp"]]:
        prp, r64, gl, _ = O.prp_check(c["b"], c["n"], c["base"], 16)
        assert gl
        assert prp == c["prp"]
        assert f"{r64:016X}" == c["res64"]


def test_gmp_matches_python_pow():
    for b, ln in ((1000, 8), (70001, 8)):
        N = O.n_plus(b, ln)
        assert O.powmod(3, N - 1, N) == pow(3, N - 1, N)


@pytest.mark.parametrize("ln,b,base", [(16, 1330358, 2), (16, 1330358, 3), (17, 1048583, 2)])
def test_square_loop_prefix_matches_gmp(ln, b, base):
    """The oracle's left-to-right loop at the headline degrees: after K squarings
    (digits doubled or tripled where E has a one) the register is
    base^(E >> (L - K)) mod N+, computed by GMP."""
    import numpy as np
    from oracle import oracle as O
    K = 96
    E = O.exponent(b, ln)
    L = E.bit_length()
    x = np.zeros(1 << ln, dtype=np.int32)
    x[0] = 1
    with O.Tables(ln) as t:
        t.square_loop(x, b, base, 16, O.int_to_words(E), L - 1, K)
    got = O.digits_to_int(O.get_int(x, b), b)
    assert got == O.powmod(base, E >> (L - K), O.n_plus(b, ln))
