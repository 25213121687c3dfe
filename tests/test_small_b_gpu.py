"""Small bases (64 <= b < 2^16, the bottom of the accepted range): the engine and
a pool against GMP (tests/golden/pool_gmp.json)."""
import json
import os

import pytest

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


def gold():
    d = json.load(open(os.path.join(HERE, "golden", "pool_gmp.json")))
    return {(x["b"], x["n"], x["base"]): x for x in d if x["form"] == "+"}


@pytest.mark.parametrize("n", [12, 13])
def test_engine_small_b(native, n):
    from ctwin_gb300 import PrpEngine
    g = gold()
    bs = [64, 65, 100, 1000]
    with PrpEngine(n, 4) as eng:
        prp, r64, ok = eng.run(bs)
    for b, p, r, k in zip(bs, prp, r64, ok):
        want = g[(b, n, 2)]
        assert k and (bool(p), int(r)) == (want["prp"], int(want["res64"], 16)), b


def test_pool_small_b(native):
    from ctwin_gb300 import Pool
    g = gold()
    bs = [64, 65, 100, 1000]
    with Pool(12, 4) as p:
        p.admit_many(bs)
        res = p.run_to_completion()
    for r in res:
        want = g[(r["b"], 12, 2)]
        assert r["status"] == 0 and r["gl_ok"]
        assert (r["is_prp"], r["res64"]) == (want["prp"], int(want["res64"], 16))
