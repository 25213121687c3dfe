"""The sieve oracle (CPU restatement) pinned against the reference CPU sieve's
own outputs (survivor bitmaps, last p, cand/sv file digests)."""
import hashlib
import json
import os

import numpy as np
import pytest

from oracle import oracle as O

FAST = ["n8_small", "n9_small", "n10_mid", "cfg1_pos"]


def _golden(golden_dir):
    meta = json.load(open(os.path.join(golden_dir, "sieve_files.json")))
    arrs = np.load(os.path.join(golden_dir, "sieve_ref.npz"))
    return meta, arrs


def _bits(arrs, meta, name):
    m = meta["cases"][name]
    return np.unpackbits(arrs[name], bitorder="little")[: m["size"]]


@pytest.mark.parametrize("name", FAST)
def test_sieve_oracle_matches_reference(golden_dir, name):
    meta, arrs = _golden(golden_dir)
    m = meta["cases"][name]
    n = m["n"]
    bits = np.zeros(m["size"], dtype=np.uint8)
    lp = ln_ = None
    if m["mode"] >= 0:
        bits, lp = O.sieve(n, m["b_min"], m["b_max"], 3 * (1 << n) + 1, m["p_max_pos"], 1, bits, threads=4)
        assert lp == m["p_last_pos"]
    if m["mode"] <= 0:
        bits, ln_ = O.sieve(n, m["b_min"], m["b_max"], 11, m["p_max_neg"], -1, bits, threads=4)
        assert ln_ == m["p_last_neg"]
    assert np.array_equal(bits, _bits(arrs, meta, name))


def test_sv_cand_format(golden_dir):
    meta, arrs = _golden(golden_dir)
    m = meta["cases"]["cfg1_twin"]
    bits = _bits(arrs, meta, "cfg1_twin")
    files = meta["files"]["cfg1_twin"]
    tag = f"_{m['n']}_{m['b_min']}_{m['b_max']}"
    cand = O.cand_text(bits, m["b_min"]).encode()
    sv = O.sv_bytes(bits, m["p_last_pos"], m["p_last_neg"])
    assert hashlib.md5(cand).hexdigest() == files["cand" + tag + ".txt"]
    assert hashlib.md5(sv).hexdigest() == files["sv" + tag + ".dat"]
    assert m["survivors"] == 8800


def test_reference_sieve_if_available():
    """Where the reference CPU sieve was built (oracle/_ref), run it directly."""
    if O.build_ref(os.environ.get("CTWIN_REFERENCE")) is None:
        pytest.skip("reference source not present on this machine")
    r = O.ref_sieve(9, 100, 5000, 10 ** 6, 10 ** 5, 0)
    bits = np.zeros(4901, dtype=np.uint8)
    bits, _ = O.sieve(9, 100, 5000, 3 * 512 + 1, 10 ** 6, 1, bits)
    bits, _ = O.sieve(9, 100, 5000, 11, 10 ** 5, -1, bits)
    assert np.array_equal(bits, r[0])
