"""N- = b^D - b^{D/2} - 1 arithmetic, without a GPU.

The kernels take the exact product of two degree < D polynomials on the
transform of degree 2D and fold it with X^D = X^{D/2} + 1:
  j <  D/2:  c_j + c_{j+D} + c_{j+3D/2}
  j >= D/2:  c_j + c_{j+D/2} + 2 c_{j+D}
This restates that rule in Python and checks it against the residue mod N-,
and pins the GMP golden residues of the twin partners against Python's pow."""
import json
import os
import random

from oracle import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))


def fold(c, D):
    c = list(c) + [0] * (2 * D - len(c))
    out = []
    for j in range(D):
        if j < D // 2:
            out.append(c[j] + c[j + D] + c[j + 3 * D // 2])
        else:
            out.append(c[j] + c[j + D // 2] + 2 * c[j + D])
    return out


def test_fold_rule():
    rng = random.Random(1)
    for D in (8, 16, 64, 256):
        b = rng.randrange(64, 1 << 20)
        N = b ** D - b ** (D // 2) - 1
        for _ in range(5):
            x = [rng.randrange(-b // 2, b // 2) for _ in range(D)]
            y = [rng.randrange(-b // 2, b // 2) for _ in range(D)]
            c = [0] * (2 * D - 1)
            for i, xi in enumerate(x):
                for k, yk in enumerate(y):
                    c[i + k] += xi * yk
            f = fold(c, D)
            assert O.digits_to_int(f, b) % N == O.digits_to_int(x, b) * O.digits_to_int(y, b) % N
            # the folded coefficients stay within D b^2 (< 2^89 for D <= 2^16, b < 2^31)
            assert max(abs(v) for v in f) <= D * b * b


def test_minus_golden_pinned():
    """The GMP N- residues of the golden list agree with Python's pow (n = 8)."""
    d = json.load(open(os.path.join(HERE, "golden", "prp_gmp.json")))
    cases = [x for x in d if x["n"] == 8 and x["form"] == "-"][:12]
    assert cases
    for x in cases:
        b = x["b"]
        N = b ** 256 - b ** 128 - 1
        r = pow(x["base"], N - 1, N)
        assert f"{r & (2 ** 64 - 1):016X}" == x["res64"] and (r == 1) == x["prp"]
