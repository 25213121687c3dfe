"""The large sieve on the GPU at its own size, against the reference CPU sieve.

n = 20 (N = b^(2^20) - b^(2^19) + 1), p = 3k 2^20 + 1 up to 2^40, + form, over
four seeded sub-ranges [s, s + 2^24) of [2, 2^30).  The fixture
(tests/golden/sieve_cfg4.json, written by tests/golden/make_golden.py --only cfg4)
holds what the reference CPU sieve itself (sieve/CPU/ctsieve.cpp:678-726,
check_pos, compiled unchanged) produced on those ranges: the SHA-256 of the
packed struck bitmap, the survivor count, the last p it recorded and the md5 of
the sv_*.dat / cand_*.txt it writes.  Bit-exact.
"""
import hashlib
import json
import os
import tempfile

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _ranges(golden_dir):
    return json.load(open(os.path.join(golden_dir, "sieve_cfg4.json")))["ranges"]


@pytest.mark.parametrize("idx", range(4))
def test_sieve_n20_p40_subrange_matches_reference(native, golden_dir, idx):
    from ctwin_gb300 import Sieve
    g = _ranges(golden_dir)[idx]
    s = Sieve(g["n"], g["b_min"], g["b_max"])
    s.check_pos(g["p_max_pos"])
    assert s.p_min_pos == g["p_last_pos"]
    bits = s.bits()
    surv = np.flatnonzero(bits == 0)
    assert [g["b_min"] + int(i) for i in surv[:64]] == g["first_survivors"]
    assert int(surv.size) == g["survivors"]
    packed = np.packbits(bits, bitorder="little")
    assert hashlib.sha256(packed.tobytes()).hexdigest() == g["sha256_bits"]
    if idx == 0:
        d = tempfile.mkdtemp()
        sv, cand = s.write(d)
        assert hashlib.md5(open(sv, "rb").read()).hexdigest() == g["files"][os.path.basename(sv)]
        assert hashlib.md5(open(cand, "rb").read()).hexdigest() == g["files"][os.path.basename(cand)]


def test_sieve_n20_whole_range_contains_subranges(native, golden_dir):
    """One pass over all of [2, 2^30) (the large-sieve workload itself) restricted
    to each sub-range equals the reference's bitmap of that sub-range."""
    from ctwin_gb300 import sieve_pass
    n, b_min, b_max = 20, 2, (1 << 30) - 1
    struck, p_last = sieve_pass(n, b_min, b_max, 3 * (1 << n) + 1, 1 << 40, 1)
    raw = struck.view(np.uint8)
    for g in _ranges(golden_dir):
        lo, hi = g["b_min"] - b_min, g["b_max"] - b_min + 1          # bit offsets in the whole bitmap
        sub = np.unpackbits(raw[lo // 8: (hi + 7) // 8], bitorder="little")[lo % 8: lo % 8 + (hi - lo)]
        assert hashlib.sha256(np.packbits(sub, bitorder="little").tobytes()).hexdigest() == g["sha256_bits"]
        assert p_last == g["p_last_pos"]
