"""GPU parity of the sieve (through the C ABI) against the reference CPU sieve's
own outputs (golden fixtures) and the oracle.  Bit-exact."""
import hashlib
import json
import os
import tempfile

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _golden(golden_dir):
    meta = json.load(open(os.path.join(golden_dir, "sieve_files.json")))
    arrs = np.load(os.path.join(golden_dir, "sieve_ref.npz"))
    return meta, arrs


@pytest.mark.parametrize("name", ["n8_small", "n9_small", "n10_mid", "cfg1_pos", "n12_pos", "n14_pos", "n16_pos",
                                  "n20_pos_s0", "cfg1_twin"])
def test_sieve_matches_reference(native, golden_dir, name):
    from ctwin_gb300 import Sieve
    meta, arrs = _golden(golden_dir)
    m = meta["cases"][name]
    s = Sieve(m["n"], m["b_min"], m["b_max"])
    if m["mode"] >= 0:
        s.check_pos(m["p_max_pos"])
        assert s.p_min_pos == m["p_last_pos"]
    if m["mode"] <= 0:
        s.check_neg(m["p_max_neg"])
        assert s.p_min_neg == m["p_last_neg"]
    want = np.unpackbits(arrs[name], bitorder="little")[: m["size"]]
    got = s.bits()
    assert np.array_equal(got, want), f"{int((got != want).sum())} b differ"
    assert int((got == 0).sum()) == m["survivors"]
    if name in meta["files"] and meta["files"][name]:
        d = tempfile.mkdtemp()
        sv, cand = s.write(d)
        files = meta["files"][name]
        assert hashlib.md5(open(cand, "rb").read()).hexdigest() == files[os.path.basename(cand)]
        assert hashlib.md5(open(sv, "rb").read()).hexdigest() == files[os.path.basename(sv)]


@pytest.mark.parametrize("n,b_min,b_max,p_max,mode", [
    (8, 2, 2, 10 ** 6, 1),                 # single b
    (8, 2, 2, 10 ** 5, -1),
    (11, 123, 4567, 2 ** 33, 1),           # ragged range, p past 2^32
    (13, 10 ** 6, 10 ** 6 + 99, 2 ** 34, 1),
    (12, 5, 70000, 3 * 10 ** 6, -1),       # small p: many strikes per root
    (24, 2, 5000, 2 ** 38, 1),             # n at the reference's maximum
])
def test_sieve_matches_oracle_edges(native, n, b_min, b_max, p_max, mode):
    from ctwin_gb300 import sieve_pass
    from ctwin_gb300.sieve import unpack
    p_min = 3 * (1 << n) + 1 if mode > 0 else 11
    struck, pl = sieve_pass(n, b_min, b_max, p_min, p_max, mode)
    want, wpl = O.sieve(n, b_min, b_max, p_min, p_max, mode, threads=8)
    assert np.array_equal(unpack(struck, b_max - b_min + 1), want)
    assert pl == wpl


def test_sieve_split_ranges_agree(native):
    """Size-independent property: one pass over [b0, b1] equals passes over its halves
    and over the two halves of the p range."""
    from ctwin_gb300 import sieve_pass
    from ctwin_gb300.sieve import unpack
    n, b0, b1, pmax = 20, 2, 2 ** 22 + 1, 2 ** 40
    whole, pl = sieve_pass(n, b0, b1, 3 * (1 << n) + 1, pmax, 1)
    mid = (b0 + b1) // 2
    lo, _ = sieve_pass(n, b0, mid, 3 * (1 << n) + 1, pmax, 1)
    hi, _ = sieve_pass(n, mid + 1, b1, 3 * (1 << n) + 1, pmax, 1)
    bits = unpack(whole, b1 - b0 + 1)
    assert np.array_equal(bits[: mid - b0 + 1], unpack(lo, mid - b0 + 1))
    assert np.array_equal(bits[mid - b0 + 1:], unpack(hi, b1 - mid))
    p_split = 2 ** 36
    a, pa = sieve_pass(n, b0, b1, 3 * (1 << n) + 1, p_split, 1)
    a, pb = sieve_pass(n, b0, b1, pa, pmax, 1, a, pa)
    assert np.array_equal(a, whole) and pb == pl


def test_sieve_argument_errors(native):
    from ctwin_gb300 import CtwError, sieve_pass
    with pytest.raises(CtwError):
        sieve_pass(7, 2, 100, 10, 1000, 1)
    with pytest.raises(CtwError):
        sieve_pass(11, 1, 100, 10, 1000, 1)
    with pytest.raises(CtwError):
        sieve_pass(11, 100, 99, 10, 1000, 1)
    with pytest.raises(CtwError):
        sieve_pass(11, 2, 100, 10, 1000, 0)
