"""Degree 2^16 against GMP (tests/golden/prp16_gmp.json): whole Fermat tests
with Gerbicz-Li of small b (N+ base 2 and 3, N-), and the first 4096
squarings of the single-test workload's exponent (b = 1330358, the 64-CTA
grid, two primes), compared through a hash of the whole residue.  Integer
work: tolerance 0."""
import hashlib
import json
import os

import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


def cases():
    return json.load(open(os.path.join(HERE, "golden", "prp16_gmp.json")))


@pytest.mark.parametrize("base,form", [(2, "+"), (3, "+"), (2, "-")])
def test_whole_tests_degree_65536(native, base, form):
    from ctwin_gb300 import PrpEngine
    sel = [c for c in cases() if "K" not in c and c["base"] == base and c["form"] == form]
    assert sel
    with PrpEngine(16, len(sel), base=base, minus=form == "-") as eng:
        prp, r64, gl = eng.run([c["b"] for c in sel])
    for c, p, r, g in zip(sel, prp, r64, gl):
        assert g, c
        assert (bool(p), f"{int(r):016X}") == (c["prp"], c["res64"]), c


@pytest.mark.parametrize("base", [2, 3])
def test_prefix_4096_single_workload(native, base):
    from ctwin_gb300 import PrpEngine
    c = next(c for c in cases() if c.get("K") and c["base"] == base)
    b, K = c["b"], c["K"]
    E = O.exponent(b, 16)
    L = E.bit_length()
    with PrpEngine(16, 1, base=base) as eng:
        assert eng.geometry()["ctas_per_lane"] == 64
        eng.set_b([b])
        assert eng.prime_count == 2
        eng.set(1)
        eng.square_bits(O.int_to_words(E), L - 1, K)
        dig = eng.get_int(0)[0]
    assert all(0 <= int(v) < b for v in dig)
    r = O.digits_to_int(dig, b)
    N = O.n_plus(b, 16)
    raw = r.to_bytes((N.bit_length() + 7) // 8, "little")
    assert f"{r & (2 ** 64 - 1):016X}" == c["low64"]
    assert hashlib.sha256(raw).hexdigest() == c["sha256"]
