"""Batches of pools of uneven degrees (2^12..2^15) on the GPU: every pool's
squarings of a tick in one persistent launch with per-degree work queues.
Each test's verdict and RES64 equal GMP's (tests/golden/pool_gmp.json) and the
same pool run on its own; integer work, tolerance 0."""
import json
import os

import pytest

pytestmark = pytest.mark.gpu


def gold():
    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "pool_gmp.json")
    return {(d["b"], d["n"]): (d["prp"], int(d["res64"], 16)) for d in json.load(open(here))
            if d["form"] == "+" and d["base"] == 2}


# (degree, slots, b values): two-prime pools of every degree and one three-prime
# pool (b above the two-prime bound at 2^12)
MIX = [
    (15, 2, [64, 1000]),
    (14, 2, [65, 100]),
    (13, 4, [64, 65537, 70001, 6500003]),
    (12, 8, [64, 65, 100, 1000, 65537, 70001, 100003, 9000001]),
    (12, 8, [9999991, 16777213]),
]


@pytest.mark.parametrize("ctas_per_sm", [2, 1])
def test_batch_mixed_degrees_match_gmp(native, ctas_per_sm):
    from ctwin_gb300 import Batch, Pool
    want = gold()
    pools = [Pool(ln, slots, log2_ctas=ln - 12, csize=16 if ln % 2 else 8) for ln, slots, _ in MIX]
    try:
        for p, (ln, _, bs) in zip(pools, MIX):
            for i, b in enumerate(bs):
                assert p.admit(b, tag=ln * 1000 + i) is not None
        assert [p.prime_count for p in pools] == [2, 2, 2, 2, 3]
        with Batch(pools, ctas_per_sm=ctas_per_sm) as bt:
            res = bt.run_to_completion(4)
            assert bt.launches > 0
        got = {(r["b"], r["log2_degree"]): r for r in res}
        assert len(got) == sum(len(bs) for _, _, bs in MIX)
        for (b, ln), r in got.items():
            assert r["status"] == 0 and r["gl_ok"], r
            assert (r["is_prp"], r["res64"]) == want[(b, ln)], r
    finally:
        for p in pools:
            p.close()


def test_batch_continuous_admission_equals_pool_alone(native):
    """Tests admitted into a batched pool while the others run give the same
    results as the pool run on its own."""
    from ctwin_gb300 import Batch, Pool
    bs13 = [65537, 70001, 100003, 64]
    with Pool(13, 4, log2_ctas=1) as alone:
        for b in bs13:
            alone.admit(b)
        ref = {r["b"]: (r["is_prp"], r["res64"]) for r in alone.run_to_completion()}
    p15 = Pool(15, 1, log2_ctas=3)
    p13 = Pool(13, 4, log2_ctas=1)
    try:
        p15.admit(1000)
        p13.admit(bs13[0])
        res = []
        queue = bs13[1:]
        with Batch([p13, p15]) as bt:
            while queue or p13.info()["active"] or p15.info()["active"]:
                bt.run(2)
                for p in (p13, p15):
                    p.collect(wait=True)
                    res += p.results()
                if queue and p13.info()["active"] < 4:
                    p13.admit(queue.pop(0))
        got = {r["b"]: (r["is_prp"], r["res64"]) for r in res if r["log2_degree"] == 13}
        assert got == ref
        r15 = [r for r in res if r["log2_degree"] == 15]
        assert len(r15) == 1 and (r15[0]["is_prp"], r15[0]["res64"]) == gold()[(1000, 15)]
    finally:
        p15.close()
        p13.close()


def test_batch_rejects_other_splits(native):
    from ctwin_gb300 import Batch, CtwError, Pool
    with Pool(13, 4, log2_ctas=2) as p:        # 2048 coefficients per CTA
        with pytest.raises(CtwError):
            Batch([p])
    with Pool(14, 3, log2_ctas=2) as p:        # 3 slots: not whole work items of 2 lanes
        with pytest.raises(CtwError):
            Batch([p])
