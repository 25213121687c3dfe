"""GPU parity of the PRP engine (through the C ABI) against the oracle and GMP.

Integer work: every comparison is bit-exact (tolerance 0)."""
import json
import os
import random

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _rand_digits(rng, lanes, D, b):
    return np.array([[rng.randint(-(b[l] // 2), b[l] // 2) for _ in range(D)] for l in range(lanes)], dtype=np.int32)


@pytest.mark.parametrize("ln,csize", [(8, 8), (9, 16), (10, 32), (11, 16), (12, 64), (13, 16), (14, 8),
                                      (15, 16), (16, 16), (17, 32), (18, 16)])
def test_square_dup_registers_bit_exact(native, ln, csize):
    """Device registers after each square_dup equal the reference's normalize1/2
    digits (oracle restatement) for the same CSIZE."""
    from ctwin_gb300 import PrpEngine
    rng = random.Random(1000 + ln)
    lanes = 2 if ln >= 16 else 3
    D = 1 << ln
    b = [rng.randrange(2 ** 16, 2 ** 24) for _ in range(lanes)]
    b[0] = rng.randrange(2 ** 30, 2 ** 31)          # large b near the Barrett limit
    x0 = _rand_digits(rng, lanes, D, b)
    steps = 3 if ln >= 17 else 5
    masks = [rng.getrandbits(lanes) for _ in range(steps)]
    with PrpEngine(ln, lanes, csize=csize) as eng:
        eng.set_b(b)
        eng.write_regs(x0[None], 0)
        for m in masks:
            eng.square_dup(m)
        got = eng.read_regs(0, 1)[0]
    with O.Tables(ln) as t:
        for l in range(lanes):
            x = x0[l].copy()
            for m in masks:
                t.square_dup(x, b[l], 2 if (m >> l) & 1 else 1, csize)
            assert np.array_equal(got[l], x), f"lane {l} differs"


@pytest.mark.parametrize("ln", [8, 11, 13, 16])
def test_mul_regs_bit_exact(native, ln):
    from ctwin_gb300 import PrpEngine
    rng = random.Random(7 + ln)
    lanes, D = 2, 1 << ln
    b = [rng.randrange(2 ** 17, 2 ** 22) for _ in range(lanes)]
    x = _rand_digits(rng, lanes, D, b)
    y = _rand_digits(rng, lanes, D, b)
    with PrpEngine(ln, lanes, csize=16) as eng:
        eng.set_b(b)
        eng.write_regs(np.stack([x, y]), 0)
        eng.mul()                     # reg0 <- reg0 * reg1
        got = eng.read_regs(0, 2)
    with O.Tables(ln) as t:
        for l in range(lanes):
            xx = x[l].copy()
            t.mul(xx, y[l], b[l], 16)
            assert np.array_equal(got[0, l], xx)
            assert np.array_equal(got[1, l], y[l])


@pytest.mark.parametrize("ln,base", [(12, 2), (14, 3), (16, 2)])
def test_partial_residue_canonical(native, ln, base):
    """First K squarings of the real exponent give base^(E >> (L-K)) mod N+."""
    from ctwin_gb300 import PrpEngine
    rng = random.Random(ln * 31 + base)
    b = rng.randrange(2 ** 20, 2 ** 21)
    E = O.exponent(b, ln)
    L = E.bit_length()
    K = 48
    with PrpEngine(ln, 1, base=base) as eng:
        eng.set_b([b])
        eng.set(1)
        eng.square_bits(O.int_to_words(E), L - 1, K)
        dig = eng.get_int(0)[0]
    want = O.powmod(base, E >> (L - K), O.n_plus(b, ln))
    assert O.digits_to_int(dig, b) == want


def test_run_vs_gmp_n8(native, golden_dir):
    """Whole tests (with Gerbicz-Li) of 64 candidates, base 2 and 3, against GMP."""
    from ctwin_gb300 import PrpEngine
    cases = [c for c in json.load(open(os.path.join(golden_dir, "prp_gmp.json"))) if c["n"] == 8 and c["form"] == "+"]
    for base in (2, 3):
        sel = [c for c in cases if c["base"] == base][:64]
        with PrpEngine(8, 64, base=base) as eng:
            prp, r64, gl = eng.run([c["b"] for c in sel])
        assert gl.all()
        for c, p, r in zip(sel, prp, r64):
            assert p == c["prp"] and f"{int(r):016X}" == c["res64"], c


def test_run_vs_gmp_config1_survivors(native, golden_dir):
    """The first 256 twin-sieve survivors of b in [100000, 300000) at n = 11,
    base 2 and 3, in vectors of 64 lanes."""
    from ctwin_gb300 import PrpEngine
    cases = [c for c in json.load(open(os.path.join(golden_dir, "prp_gmp.json")))
             if c["n"] == 11 and c["form"] == "+"]
    for base in (2, 3):
        sel = [c for c in cases if c["base"] == base]
        assert len(sel) == 256
        for i in range(0, len(sel), 64):
            part = sel[i:i + 64]
            with PrpEngine(11, 64, base=base) as eng:
                prp, r64, gl = eng.run([c["b"] for c in part])
            assert gl.all()
            assert [f"{int(r):016X}" for r in r64] == [c["res64"] for c in part]
            assert list(prp) == [c["prp"] for c in part]


def test_run_pads_lanes_with_last_b(native):
    from ctwin_gb300 import PrpEngine
    with PrpEngine(8, 8) as eng:
        prp, r64, gl = eng.run([298, 300, 302])
    for b, p, r in zip([298, 300, 302], prp, r64):
        _, rr, pp = O.fermat(b, 8, 2)
        assert p == pp and int(r) == rr
    assert prp[0]   # 298^256 - 298^128 + 1 is a probable prime


def test_argument_errors(native):
    from ctwin_gb300 import CtwError, PrpEngine
    with pytest.raises(CtwError):
        PrpEngine(19, 1)
    with PrpEngine(8, 2) as eng:
        with pytest.raises(CtwError):
            eng.set_b([10, 1000])          # b below 64
        with pytest.raises(CtwError):
            eng.set_b([2 ** 31, 1000])     # b >= 2^31
        with pytest.raises(CtwError):
            eng.copy(0, 3)
        with pytest.raises(CtwError):
            eng.set_csize(12)
