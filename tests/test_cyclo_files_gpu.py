"""The cyclog file loop on the GPU: result lines and PRP lists in the
reference's words against GMP, the <file>.ini CSIZE, and a run stopped at a
Gerbicz-Li checkpoint then resumed from cyclo.ctx giving the same lines."""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


def golden(n, form="+"):
    d = json.load(open(os.path.join(HERE, "golden", "prp_gmp.json")))
    return {x["b"]: x for x in d if x["n"] == n and x["form"] == form and x["base"] == 2}


def expected_lines(bs, n, gold, sign="+"):
    out = []
    for b in bs:
        g = gold[b]
        tail = "a probable prime." if g["prp"] else f"composite. RES64: {g['res64']}"
        out.append(f"{b}^{1 << n} - {b}^{1 << (n - 1)} {sign} 1 is {tail}")
    return out


def test_file_loop_results(native, tmp_path):
    from ctwin_gb300.cyclo import check_file
    gold = golden(8)
    bs = sorted(gold)[:70]                         # two vectors, the second padded
    f = tmp_path / "cand.txt"
    f.write_text("".join(f"{b}\n" for b in bs))
    assert check_file(8, str(f), str(tmp_path))
    lines = (tmp_path / "result_c.txt").read_text().splitlines()
    assert lines == expected_lines(bs, 8, gold)
    prps = [b for b in bs if gold[b]["prp"]]
    if prps:
        assert [int(x) for x in (tmp_path / "prp_8.txt").read_text().split()] == prps
    assert int((tmp_path / "cand.txt.ini").read_text().split()[0]) in (8, 16, 32, 64)
    assert not (tmp_path / "cyclo.ctx").exists()


def test_file_loop_stop_and_resume(native, tmp_path):
    from ctwin_gb300.cyclo import check_file, context_decode
    gold = golden(8)
    bs = sorted(gold)[:64]
    f = tmp_path / "cand.txt"
    f.write_text("".join(f"{b}\n" for b in bs))
    assert not check_file(8, str(f), str(tmp_path), stop_after=5)
    ctx = (tmp_path / "cyclo.ctx").read_bytes()
    d, k, i, el = context_decode(ctx, 8, 64)
    assert k == 0 and i > 0 and np.abs(d).max() < 2 ** 31
    assert not (tmp_path / "result_c.txt").exists()
    assert check_file(8, str(f), str(tmp_path))
    assert (tmp_path / "result_c.txt").read_text().splitlines() == expected_lines(bs, 8, gold)


def test_file_loop_minus(native, tmp_path):
    from ctwin_gb300.cyclo import check_file
    gold = golden(8, "-")
    bs = sorted(gold)[:20]
    f = tmp_path / "cand.txt"
    f.write_text("".join(f"{b}\n" for b in bs))
    assert check_file(8, str(f), str(tmp_path), minus=True)
    assert (tmp_path / "result_c.txt").read_text().splitlines() == expected_lines(bs, 8, gold, "-")


def test_context_save_read_engine(native, tmp_path):
    """ctw_prp_save_context / ctw_prp_read_context move registers 0 and 1 exactly."""
    import ctypes
    from ctwin_gb300 import PrpEngine
    from ctwin_gb300._native import check, lib
    rng = np.random.default_rng(3)
    with PrpEngine(10, 4) as eng:
        eng.set_b([70001, 80021, 90001, 100003])
        regs = rng.integers(-35000, 35000, size=(2, 4, 1024)).astype(np.int32)
        eng.write_regs(regs, 0)
        p = str(tmp_path / "c.ctx").encode()
        check(lib().ctw_prp_save_context(eng._h, p, 7, 4242, 3.5))
        eng.write_regs(np.zeros_like(regs), 0)
        k, i, el = ctypes.c_int(), ctypes.c_int(), ctypes.c_double()
        assert lib().ctw_prp_read_context(eng._h, p, ctypes.byref(k), ctypes.byref(i), ctypes.byref(el)) == 0
        assert (k.value, i.value, el.value) == (7, 4242, 3.5)
        assert np.array_equal(eng.read_regs(0, 2), regs)
