"""Failure detection on the GPU, without a GPU fault.

* Gerbicz-Li (cyclo/src/cyclo.h:301-377, the check the reference's commented
  fault injection at cyclo.h:298 exercises): one digit of the residue x is
  changed on the host between two Gerbicz-Li blocks (read with
  ctw_prp_read_regs, written back with ctw_prp_write_regs at a checkpoint);
  the run must end with the check failed.  Run on the 64-CTA grid of degree
  2^16 and on a one-CTA engine of degree 2^12.
* Grid waits: every wait of the grid kernel (barrier, carry count, poll of a
  published word) is bounded (50 ms of %globaltimer).  A test hook starts the
  barrier counter of one launch out of reach and has CTA 0 skip its first
  publication of columns, so that the other CTAs' polls run out; the launch
  must end within a few wait budgets with CTW_E_COMPUTE, and the same handle
  must then square bit-exactly again.
"""
import time

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _flip_run(eng, b, at_checkpoint, seen):
    def cp(i):
        seen.append(i)
        if len(seen) == at_checkpoint:
            x = eng.read_regs(0, 1)
            j = x.shape[-1] // 3
            x[0, 0, j] = x[0, 0, j] + 1 if x[0, 0, j] < b // 2 else x[0, 0, j] - 1
            eng.write_regs(x, 0)
        return False

    return eng.run_ex([b], cp)


@pytest.mark.parametrize("ln,b", [(16, 65), (12, 1000003)])
def test_gerbicz_li_catches_a_flipped_digit(native, ln, b):
    from ctwin_gb300 import CtwError, PrpEngine
    with PrpEngine(ln, 1, base=3) as eng:
        prp, r64, gl = eng.run([b])            # clean run: the check passes
        assert gl[0]
        seen = []
        # the reference treats a failed check as a fatal error (cyclo/src/cyclo.h:376-377): CTW_E_GERBICZ
        with pytest.raises(CtwError) as ei:
            _flip_run(eng, b, 2, seen)
        assert ei.value.code == -5, "Gerbicz-Li missed a changed digit"
        assert len(seen) > 2
        # the engine is unharmed: a clean run again passes
        prp3, r643, gl3 = eng.run([b])
        assert gl3[0] and int(r643[0]) == int(r64[0])


def test_grid_barrier_wait_runs_out_and_engine_recovers(native):
    from ctwin_gb300 import CtwError, PrpEngine
    from ctwin_gb300._native import lib
    ln, b = 16, 1330358
    D = 1 << ln
    rng = np.random.default_rng(7)
    x0 = rng.integers(-(b // 2), b // 2 + 1, size=(1, 1, D), dtype=np.int64).astype(np.int32)
    with PrpEngine(ln, 1, base=3) as eng:
        assert eng.geometry()["ctas_per_lane"] == 64
        eng.set_b([b])
        eng.write_regs(x0, 0)
        eng.sync()
        assert lib().ctw_prp_test_unreachable_barrier(eng._h) == 0
        t0 = time.perf_counter()
        with pytest.raises(CtwError) as ei:
            eng.square_dup(1)
            eng.get_int(0)                     # reads the launch status
        dt = time.perf_counter() - t0
        assert "barrier" in str(ei.value)
        assert dt < 2.0, f"timed-out launch took {dt:.2f} s"
        # the same handle squares bit-exactly afterwards
        eng.write_regs(x0, 0)
        eng.square_dup(1)
        eng.square_dup(0)
        got = eng.read_regs(0, 1)[0, 0]
    with O.Tables(ln) as t:
        x = x0[0, 0].copy()
        t.square_dup(x, b, 3, 8)
        t.square_dup(x, b, 1, 8)
    assert np.array_equal(got, x)


def test_unreachable_barrier_hook_rejects_non_grid(native):
    from ctwin_gb300 import PrpEngine
    from ctwin_gb300._native import lib
    with PrpEngine(12, 1) as eng:
        assert lib().ctw_prp_test_unreachable_barrier(eng._h) != 0
