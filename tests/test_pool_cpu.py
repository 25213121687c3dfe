"""Host logic of the pools, without a GPU: the tick program that every slot
runs (ctw_pool_schedule) replayed on the oracle's CPU restatement of the
transform, against GMP.  The program restates cyclo::check
(cyclo/src/cyclo.h:252-377) with the exponent padded to whole Gerbicz-Li
blocks; its verdict, RES64 and Gerbicz-Li check must be the reference's."""
import numpy as np
import pytest

from oracle import oracle as O


def _lib_or_skip():
    try:
        from ctwin_gb300.pool import schedule  # noqa: F401
        from ctwin_gb300._native import lib
        lib()
    except ImportError as e:
        pytest.skip(f"native library not built: {e}")


def replay(ln, b, base=2, gl_block=0, csize=16, corrupt_tick=None):
    """Run the tick program of one test on the oracle: (is_prp, res64, gl_ok)."""
    from ctwin_gb300.pool import schedule
    prog, r0 = schedule(ln, b, gl_block)
    D = 1 << ln
    E = O.exponent(b, ln)
    B = int(prog[0, 1])
    res = 0
    e = E
    while e:
        res += e & ((1 << B) - 1)
        e >>= B
    words = np.zeros(r0 // 32 + (res.bit_length() + 31) // 32 + 2, dtype=np.uint32)
    ew = O.int_to_words(E)
    words[:ew.size] = ew
    rw = O.int_to_words(res)
    words[r0 // 32:r0 // 32 + rw.size] = rw
    one = np.zeros(D, dtype=np.int32)
    one[0] = 1
    regs = [np.zeros(D, dtype=np.int32) for _ in range(4)]
    with O.Tables(ln) as T:
        for t, (aux, sq_n, sq_hi, mul_n, m_in, m_y, m_out, _) in enumerate(prog):
            if aux & 1:
                regs[3] = regs[0].copy()
            if aux & 2:
                regs[0] = one.copy()
            if aux & 4:
                regs[1] = one.copy()
            if sq_n > 0:
                T.square_loop(regs[0], b, base, csize, words, int(sq_hi), int(sq_n))
            if t == corrupt_tick:
                regs[0][5] += 1          # a planted arithmetic error on the CPU
            if mul_n > 0:
                x = regs[m_in].copy()
                T.mul(x, regs[m_y], b, csize)
                regs[m_out] = x
    c3 = O.get_int(regs[3], b)
    prp, r64, _ = O.is_prime(c3, b)
    gl_ok = bool(np.array_equal(O.get_int(regs[0], b), O.get_int(regs[2], b)))
    return prp, r64, gl_ok


@pytest.mark.parametrize("ln,b,base", [(8, 100002, 2), (8, 300000, 3), (9, 65536 + 1234, 2), (8, 64, 2)])
def test_schedule_matches_gmp(ln, b, base):
    _lib_or_skip()
    prp, r64, gl_ok = replay(ln, b, base)
    _, want64, want_prp = O.fermat(b, ln, base)
    assert (prp, r64) == (want_prp, want64)
    assert gl_ok


def test_schedule_finds_a_prp():
    """A known PRP from the n = 8 golden list (GMP-pinned)."""
    _lib_or_skip()
    for b in range(100000, 100400):
        if O.fermat(b, 8, 2)[2]:
            prp, r64, gl_ok = replay(8, b, 2)
            assert prp and r64 == 1 and gl_ok
            return
    pytest.skip("no PRP in the scanned range")


@pytest.mark.parametrize("gl_block", [1, 7, 64, 5000])
def test_schedule_any_block(gl_block):
    """The result does not depend on the Gerbicz-Li block; the check passes."""
    _lib_or_skip()
    prp, r64, gl_ok = replay(8, 123457, 2, gl_block=gl_block)
    assert r64 == O.fermat(123457, 8, 2)[1] and gl_ok


def test_schedule_detects_error():
    """An error planted in the middle of the main phase fails the Gerbicz-Li check."""
    _lib_or_skip()
    _, r64, gl_ok = replay(8, 123457, 2, corrupt_tick=20)
    assert not gl_ok


def test_schedule_structure():
    """Blocks are whole: the first squaring sits at a multiple of B minus one,
    every main tick but the last multiplies into d, the last into d(t+1)."""
    _lib_or_skip()
    from ctwin_gb300.pool import schedule
    for ln, b in [(8, 100002), (12, 1 << 20), (16, 1330358)]:
        prog, r0 = schedule(ln, b)
        B = int(prog[0, 1])
        L = O.exponent(b, ln).bit_length()
        main = prog[:-2]
        assert (int(main[0, 2]) + 1) % B == 0 and int(main[0, 2]) + 1 >= L > int(main[0, 2]) + 1 - B
        assert main[0, 0] == 6 and all(main[1:, 0] == 0)
        assert all(main[:-1, 6] == 1) and main[-1, 6] == 2
        assert list(np.diff(main[:, 2])) == [-B] * (len(main) - 1) and main[-1, 2] == B - 1
        assert prog[-2, 0] == 3 and prog[-2, 6] == 0 and prog[-1, 3] == 0
        assert prog[-1, 2] == r0 + B - 1 and prog[-1, 1] == B
