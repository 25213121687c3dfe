"""Host logic of the pools, without a GPU: the tick program that every slot
runs (ctw_pool_schedule) replayed on the oracle's CPU restatement of the
transform, against GMP.  The program restates cyclo::check
(cyclo/src/cyclo.h:252-377) with the exponent padded to whole Gerbicz-Li
blocks and with the pool's uniform launches (every tick: register moves, B
squarings of register 0, d <- x * d into register 1, register moves); its
verdict, RES64 and Gerbicz-Li check must be the reference's."""
import numpy as np
import pytest

from oracle import oracle as O

INIT, SAVE_D, SAVE_X, SAVE_D1, SET_Y, LOAD_D, TAKE, SAVE_Y = (1 << k for k in range(8))


def _lib_or_skip():
    try:
        from ctwin_gb300._native import lib
        lib()
    except ImportError as e:
        pytest.skip(f"native library not built: {e}")


def block_sum(E, B):
    res = 0
    while E:
        res += E & ((1 << B) - 1)
        E >>= B
    return res


def moves(r, ops):
    one = np.zeros_like(r[0])
    one[0] = 1
    if ops & INIT:
        r[0], r[1] = one.copy(), one.copy()
    if ops & SAVE_D:
        r[3] = r[1].copy()
    if ops & SAVE_X:
        r[2] = r[0].copy()
    if ops & SAVE_D1:
        r[4] = r[1].copy()
    if ops & SET_Y:
        r[0] = one.copy()
    if ops & LOAD_D:
        r[1] = r[3].copy()
    if ops & TAKE:
        r[0] = r[1].copy()
    if ops & SAVE_Y:
        r[5] = r[0].copy()


def replay(ln, b, base=2, gl_block=0, csize=16, corrupt_tick=None):
    """Run the tick program of one test on the oracle: (is_prp, res64, gl_ok)."""
    from ctwin_gb300.pool import schedule
    prog, B = schedule(ln, b, gl_block)
    D = 1 << ln
    E = O.exponent(b, ln)
    src = [E, block_sum(E, B)]
    regs = [np.zeros(D, dtype=np.int32) for _ in range(6)]
    with O.Tables(ln) as T:
        for t, (before, after, source, lo) in enumerate(prog):
            moves(regs, int(before))
            bits = (src[source] >> int(lo)) & ((1 << B) - 1)
            words = O.int_to_words(bits) if bits else np.zeros(1, dtype=np.uint32)
            T.square_loop(regs[0], b, base, csize, words, B - 1, B)
            if t == corrupt_tick:
                regs[0][5] += 1          # a planted arithmetic error on the CPU
            x = regs[0].copy()
            T.mul(x, regs[1], b, csize)
            regs[1] = x
            moves(regs, int(after))
    c = O.get_int(regs[2], b)
    prp, r64, _ = O.is_prime(c, b)
    gl_ok = bool(np.array_equal(O.get_int(regs[5], b), O.get_int(regs[4], b)))
    return prp, r64, gl_ok


@pytest.mark.parametrize("ln,b,base", [(8, 100002, 2), (8, 300000, 3), (9, 65536 + 1234, 2), (8, 64, 2)])
def test_schedule_matches_gmp(ln, b, base):
    _lib_or_skip()
    prp, r64, gl_ok = replay(ln, b, base)
    _, want64, want_prp = O.fermat(b, ln, base)
    assert (prp, r64) == (want_prp, want64)
    assert gl_ok


def test_schedule_finds_a_prp():
    """A PRP of degree 2^8 (GMP-pinned) comes out as residue 1."""
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
    """Blocks are whole and aligned from the top of the padded exponent; the
    register moves sit where the Gerbicz-Li program needs them."""
    _lib_or_skip()
    from ctwin_gb300.pool import schedule
    for ln, b in [(8, 100002), (12, 1 << 20), (16, 1330358)]:
        prog, B = schedule(ln, b)
        E = O.exponent(b, ln)
        nb = (E.bit_length() + B - 1) // B
        main, ver = prog[:nb], prog[nb:]
        assert list(main[:, 3]) == [(nb - 1 - t) * B for t in range(nb)] and all(main[:, 2] == 0)
        assert main[0, 0] & INIT and main[-1, 0] & SAVE_D and not any(main[1:-1, 0])
        assert all(ver[:, 2] == 1) and ver[-1, 3] == 0 and ver[-1, 1] == SAVE_Y
        assert ver[0, 0] & (SAVE_X | SAVE_D1 | SET_Y) == SAVE_X | SAVE_D1 | SET_Y
        assert ver[-2, 0] & LOAD_D and ver[-2, 1] == TAKE
        kh = len(ver) - 1
        assert block_sum(E, B) < 1 << ((kh + 1) * B)
