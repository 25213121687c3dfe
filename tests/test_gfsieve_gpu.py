"""Factor-pair mode of the GPU sieve (the reference's ctsieveg output) against
the oracle's sieve over the same k range, and the file driver: every line a
verified factor, a run stopped after one block and resumed equal to an
uninterrupted run."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mode", [1, -1])
def test_factor_pairs_match_oracle(native, mode):
    from ctwin_gb300.gfsieve import divides, factors
    n, b_max = 8, 1 << 22
    if mode > 0:
        k_b, k_e = 1 << 20, (1 << 20) + (1 << 13)
        p_min, p_max = 3 * (k_b << n) + 1, 3 * ((k_e - 1) << n) + 1
    else:
        k_b, k_e = 1 << 21, (1 << 21) + (1 << 12)
        p_min, p_max = 10 * k_b, 10 * (k_e - 1)
    pairs = factors(n, k_b, k_e, mode, b_max)
    assert len(pairs) > 0
    assert all(p > b_max for p, _ in pairs)
    for p, b in pairs[:: max(1, len(pairs) // 200)]:
        assert divides(int(p), int(b), n, mode)
    assert np.all(np.diff(pairs[:, 0].astype(np.int64)) >= 0)
    bits, _ = O.sieve(n, 2, b_max, p_min, p_max, mode, threads=8)
    struck = set(int(b) for b in np.flatnonzero(bits) + 2)
    assert set(int(b) for b in pairs[:, 1]) == struck


def test_gfsieve_file_resume(native, tmp_path):
    from ctwin_gb300.gfsieve import check_range, divides
    n, mode = 8, 1
    p_min, p_max = 10 ** 12, 10 ** 12 + 3 * 10 ** 9
    a = tmp_path / "a"
    a.mkdir()
    done, nf = check_range(n, p_min, p_max, mode, str(a))
    assert done and nf > 0
    full = (a / f"fp{n}_1_1.txt").read_text().splitlines()
    assert len(full) == nf
    for line in full[:: max(1, len(full) // 100)]:
        p, b = map(int, line.split())
        assert p_min <= p <= p_max and b <= 5 * 10 ** 9 and divides(p, b, n, mode)
    b_dir = tmp_path / "b"
    b_dir.mkdir()
    done, _ = check_range(n, p_min, p_max, mode, str(b_dir), stop_after_blocks=1)
    assert not done and (b_dir / f"ctx{n}_1_1.txt").exists()
    done, _ = check_range(n, p_min, p_max, mode, str(b_dir))
    assert done
    assert (b_dir / f"fp{n}_1_1.txt").read_text().splitlines() == full
