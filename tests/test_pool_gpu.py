"""Pools and the server on the GPU: every test's verdict and RES64 equal GMP's
(tests/golden/pool_gmp.json), whatever the cluster split, carry chunk, slot
or admission time, and a test's result is the same alone and in a mix."""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLD = None


def gold():
    global GOLD
    if GOLD is None:
        here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "pool_gmp.json")
        GOLD = {(d["b"], d["n"], d["base"]): d for d in json.load(open(here)) if d["form"] == "+"}
    return GOLD


def expect(b, ln, base=2):
    d = gold()[(b, ln, base)]
    return d["prp"], int(d["res64"], 16)


def check_results(res, ln, base=2):
    for r in res:
        assert r["status"] == 0, r
        assert r["gl_ok"], r
        assert (r["is_prp"], r["res64"]) == expect(r["b"], ln, base), r


def server_cases(ln):
    return sorted(b for (b, n, base) in gold() if n == ln and base == 2 and b >= 1 << 16)


@pytest.mark.parametrize("ln,lg", [(12, 0), (12, 1), (12, 2), (12, 3), (13, 0), (13, 1), (13, 2), (13, 3), (13, 4)])
def test_pool_splits_match_gmp(native, ln, lg):
    from ctwin_gb300 import Pool
    bs = [65537, 70001, 100003]
    csize = 8 if lg % 2 == 0 else 16
    with Pool(ln, 4, log2_ctas=lg, csize=csize) as p:
        for i, b in enumerate(bs):
            assert p.admit(b, tag=i) == i
        res = p.run_to_completion()
    assert sorted(r["b"] for r in res) == bs
    check_results(res, ln)


@pytest.mark.parametrize("ln,lg", [(14, 0), (14, 1), (14, 3), (14, 4), (15, 2), (15, 4)])
def test_pool_splits_match_engine(native, ln, lg):
    """Degrees 2^14 and 2^15 on every kind of split against the engine's own
    test of the same b (default split; the engine is GMP-pinned elsewhere)."""
    from ctwin_gb300 import Pool, PrpEngine
    bs = [65537, 65539]
    with PrpEngine(ln, len(bs)) as eng:
        prp, r64, gl = eng.run(bs)
    want = {b: (bool(p), int(r)) for b, p, r in zip(bs, prp, r64)}
    with Pool(ln, 2, log2_ctas=lg, csize=32 if lg % 2 else 8) as p:
        for b in bs:
            p.admit(b)
        res = p.run_to_completion()
    for r in res:
        assert r["status"] == 0 and r["gl_ok"], r
        assert (r["is_prp"], r["res64"]) == want[r["b"]], r


def test_pool_base3(native):
    from ctwin_gb300 import Pool
    with Pool(12, 2, base=3) as p:
        p.admit(65539, 1)
        res = p.run_to_completion()
    check_results(res, 12, base=3)


def test_pool_continuous_admission(native):
    """Tests admitted while others run, into slots freed by finished tests."""
    from ctwin_gb300 import Pool
    bs = server_cases(10)[:12]
    got = []
    with Pool(10, 4) as p:
        queue = list(bs)
        for _ in range(2):
            p.admit(queue.pop(0))
        while queue or p.info()["active"]:
            p.run(3)
            p.collect(wait=True)
            got += p.results()
            if queue and p.info()["active"] < 4:
                assert p.admit(queue.pop(0)) is not None
        got += p.results()
    assert sorted(r["b"] for r in got) == sorted(bs)
    check_results(got, 10)
    assert max(r["slot"] for r in got) < 4


def test_pool_full_and_args(native):
    from ctwin_gb300 import Pool, CtwError
    with Pool(9, 2) as p:
        assert p.admit(100000) == 0 and p.admit(100001) == 1
        assert p.admit(100002) is None
        with pytest.raises(CtwError):
            p.admit(63)
    with pytest.raises(CtwError):
        Pool(12, 2, log2_ctas=4)          # 256 coefficients per CTA on 16 CTAs: no kernel
    with pytest.raises(CtwError):
        Pool(13, 2, log2_ctas=4, csize=64)  # run of 32 columns shorter than the chunk


def test_autotune(native):
    from ctwin_gb300 import Pool, autotune
    lg, cs, us = autotune(12, 64)
    assert 0 <= lg <= 3 and cs in (8, 16, 32, 64) and us > 0
    assert autotune(12, 64) == (lg, cs, us)           # cached
    with Pool(12, 2, log2_ctas=lg, csize=cs) as p:
        p.admit(65537)
        p.admit(100003)
        check_results(p.run_to_completion(), 12)


def test_server_mix_and_alone(native):
    """Requests of degrees 2^9..2^11 interleaved; each result equals GMP and
    equals the same request served alone."""
    from ctwin_gb300 import Server
    reqs = [(ln, b) for ln in (9, 10, 11) for b in server_cases(ln)]
    rng = np.random.default_rng(3)
    order = rng.permutation(len(reqs))
    with Server(hbm_budget_bytes=1 << 30, max_slots=16, ticks_per_launch=2) as s:
        for i in order:
            ln, b = reqs[i]
            s.submit(ln, b, tag=int(i))
        res = s.drain(len(reqs), timeout_s=300)
        st = s.stats()
    assert st["finished"] == len(reqs) and st["pending"] == 0
    by_tag = {r["tag"]: r for r in res}
    assert sorted(by_tag) == list(range(len(reqs)))
    for t, r in by_tag.items():
        ln, b = reqs[t]
        assert (r["log2_degree"], r["b"]) == (ln, b)
        check_results([r], ln)
        assert r["t_submit"] <= r["t_admit"] <= r["t_done"]
    alone = {}
    with Server(hbm_budget_bytes=1 << 30, max_slots=16) as s:
        for t in (0, len(reqs) // 2, len(reqs) - 1):
            ln, b = reqs[t]
            s.submit(ln, b, tag=t)
            r = s.drain(1, timeout_s=120)[0]
            alone[t] = (r["is_prp"], r["res64"], r["gl_ok"])
    for t, v in alone.items():
        assert v == (by_tag[t]["is_prp"], by_tag[t]["res64"], by_tag[t]["gl_ok"])


def test_server_budget_admission(native):
    """A budget that holds one pool at a time: degrees take turns, all finish."""
    from ctwin_gb300 import Server
    from ctwin_gb300.pool import slot_bytes
    # one one-slot pool of degree 2^10 (its slot plus 2 x 3 x 1024 words of
    # root tables) fits, a second pool next to it does not
    budget = slot_bytes(10) + 24 * 1024 + 1024
    reqs = [(9, b) for b in server_cases(9)[:4]] + [(10, b) for b in server_cases(10)[:4]]
    with Server(hbm_budget_bytes=budget, max_slots=4) as s:
        for i, (ln, b) in enumerate(reqs):
            s.submit(ln, b, tag=i)
        res = s.drain(len(reqs), timeout_s=300)
        assert s.stats()["pool_bytes"] <= budget
    for r in res:
        check_results([r], reqs[r["tag"]][0])
    with Server(hbm_budget_bytes=1 << 16, max_slots=4) as s:
        s.submit(12, 100003, tag=7)                 # no pool of degree 2^12 fits in 64 KiB
        r = s.drain(1, timeout_s=60)[0]
        assert r["status"] == -3 and r["tag"] == 7


def test_pool_admit_many(native):
    """Parallel admission (exponents prepared on several host threads)."""
    from ctwin_gb300 import Pool
    bs = server_cases(11)[:10]
    with Pool(11, 8) as p:
        assert p.admit_many(bs, tags=list(range(len(bs))), threads=4) == 8   # as many as there are slots
        res = p.run_to_completion()
        assert p.admit_many(bs[8:]) == 2
        res += p.run_to_completion()
    assert sorted(r["b"] for r in res) == sorted(bs)
    check_results(res, 11)


def test_server_admits_arrivals_while_others_run(native):
    """Continuous batching: requests that arrive while a test is on the device
    are admitted before it finishes, and their device work overlaps it (pools
    of other degrees running beside it).  Every result equals GMP's and the
    same request served alone (tolerance 0)."""
    import time

    from ctwin_gb300 import Server
    first = (12, 9999991)                                   # about 95 k squarings
    later = [(9, server_cases(9)[0]), (10, server_cases(10)[1]), (11, server_cases(11)[2]), (12, 65537)]
    with Server(hbm_budget_bytes=1 << 30, max_slots=8, ticks_per_launch=1) as s:
        for ln in (9, 10, 11, 12):
            s.prepare(ln, 4)
        s.submit(*first, tag=0)
        t0 = time.time()
        while s.stats()["active"] < 1:                      # the first test is on the device
            assert time.time() - t0 < 60
            time.sleep(0.001)
        for i, (ln, b) in enumerate(later):
            s.submit(ln, b, tag=i + 1)
            time.sleep(0.002)
        res = {r["tag"]: r for r in s.drain(1 + len(later), timeout_s=300)}
    reqs = [first] + later
    assert sorted(res) == list(range(len(reqs)))
    for t, r in res.items():
        check_results([r], reqs[t][0])
    a = res[0]
    for t in range(1, len(reqs)):
        r = res[t]
        assert a["t_admit"] < r["t_admit"] < a["t_done"], (a, r)        # admitted while the first ran
        assert r["t_admit"] < a["t_done"] and a["t_admit"] < r["t_done"]   # intervals overlap
    with Server(hbm_budget_bytes=1 << 30, max_slots=8) as s:
        for t, (ln, b) in enumerate(reqs):
            s.submit(ln, b, tag=t)
            r = s.drain(1, timeout_s=120)[0]
            assert (r["is_prp"], r["res64"], r["gl_ok"]) == (res[t]["is_prp"], res[t]["res64"], res[t]["gl_ok"])


def test_server_grid_lane_beside_pools(native):
    """The grid lane: a request of degree 2^16 runs on the one-lane engine (the
    64-CTA cooperative grid) while requests of 2^10..2^12 run in pools; the two
    take turns on the device at the lane test's Gerbicz-Li checkpoints, so pool
    tests are admitted and finish while the lane test runs.  The lane's result
    equals PrpEngine.run's for the same b, the pools' equal GMP's (tolerance 0)."""
    import time

    from ctwin_gb300 import PrpEngine, Server
    big = (16, 1330358)                                     # about 1.33 M squarings
    small = [(10, server_cases(10)[0]), (11, server_cases(11)[1]), (12, server_cases(12)[0]),
             (12, server_cases(12)[1])]
    with Server(hbm_budget_bytes=1 << 30, max_slots=8, ticks_per_launch=1) as s:
        for ln in (10, 11, 12):
            s.prepare(ln, 4)
        s.submit(*big, tag=0)
        t0 = time.time()
        while s.stats()["active"] < 1:                      # the lane test is on the device
            assert time.time() - t0 < 60
            time.sleep(0.001)
        for i, (ln, b) in enumerate(small):
            s.submit(ln, b, tag=i + 1)
        res = {r["tag"]: r for r in s.drain(1 + len(small), timeout_s=600)}
    assert sorted(res) == list(range(1 + len(small)))
    lane = res[0]
    assert lane["slot"] == -2 and lane["status"] == 0 and lane["gl_ok"]
    with PrpEngine(16, 1) as eng:
        assert eng.geometry()["ctas_per_lane"] == 64
        prp, r64, gl = eng.run([big[1]])
    assert gl[0] and (lane["is_prp"], lane["res64"]) == (bool(prp[0]), int(r64[0]))
    for t in range(1, 1 + len(small)):
        r = res[t]
        assert r["slot"] >= 0
        check_results([r], small[t - 1][0])
        assert lane["t_admit"] < r["t_admit"] and r["t_done"] < lane["t_done"], (lane, r)


def test_server_two_grid_lanes_run_together(native):
    """Two requests of degree 2^16 (64 CTAs each) hold the device together in
    the two grid lanes: their admit-done intervals overlap and each result
    equals PrpEngine.run's for its b."""
    from ctwin_gb300 import PrpEngine, Server
    bs = [65, 127]                                          # about 0.4 M squarings each
    with Server(hbm_budget_bytes=1 << 30, max_slots=8, grid_lanes=2) as s:
        for i, b in enumerate(bs):
            s.submit(16, b, tag=i)
        res = {r["tag"]: r for r in s.drain(len(bs), timeout_s=600)}
    assert sorted(res) == [0, 1]
    a, c = res[0], res[1]
    assert a["slot"] == c["slot"] == -2
    assert a["t_admit"] < c["t_done"] and c["t_admit"] < a["t_done"], (a, c)   # both on the device at once
    with PrpEngine(16, 1) as eng:
        for i, b in enumerate(bs):
            prp, r64, gl = eng.run([b])
            r = res[i]
            assert r["status"] == 0 and r["gl_ok"] and gl[0]
            assert (r["is_prp"], r["res64"]) == (bool(prp[0]), int(r64[0]))
