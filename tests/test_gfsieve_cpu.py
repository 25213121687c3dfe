"""Candidate merge of factor files (tools/ctools.cpp:177-248 restated), without a GPU."""
from ctwin_gb300.gfsieve import divides, merge


def test_merge_removes_verified_factors(tmp_path):
    n = 8
    # real factors found by brute force for a few b, plus a bad line and a duplicate
    lines, struck = [], set()
    for p in (7681, 10753, 12289, 14593):           # primes = 1 (mod 3 * 2^8)
        for b in range(2, 3000):
            if divides(p, b, n, 1):
                lines.append(f"{p} {b}")
                struck.add(b)
    lines.insert(1, lines[0])                         # repeated line (skipped like the reference's p_prev/b_prev)
    lines.append("7681 5")                           # not a factor
    f = tmp_path / "fp8_0_0.txt"
    f.write_text("\n".join(lines) + "\n")
    cand = range(2, 3000)
    rem, used, bad = merge(n, cand, [str(f)], lambda name: 1, 2, 2999)
    assert set(rem) == set(cand) - struck and bad == 1 and used == len(lines) - 2
