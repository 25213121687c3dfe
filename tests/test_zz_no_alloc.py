"""The allocation-free multiply (ctw_prp_mul_noalloc) against the handle-based
multiply (ctw_prp_mul_regs), through the C ABI, on two calls in a row.

It serves callers that cannot allocate device memory (a host that owns the
GPU's memory budget, a pooling allocator that forbids cudaMalloc): the test
allocates the input/output buffers itself, as such a caller would from its own
pool, and the entry point must give the same digits (integer work, tolerance 0).
This file is collected last so that a failure here leaves every other test run."""
import ctypes
import random

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


# (degree, lanes, CSIZE, b range, NTT primes the b range selects, z aliases x)
CASES = [
    (11, 3, 16, (2 ** 17, 2 ** 30), 3, False),
    (13, 2, 8, (2 ** 17, 2 ** 30), 3, False),
    (14, 2, 16, (2 ** 24, 2 ** 30), 3, False),   # three primes at the largest degree
    (14, 3, 8, (2 ** 16, 2 ** 21), 2, False),    # two primes (3 D (b+1)^2 < q0 q1)
    (11, 4, 16, (64, 2 ** 18), 2, True),         # two primes, z written over x
]


@pytest.mark.parametrize("ln,lanes,csize,brange,primes,alias", CASES)
def test_mul_noalloc_matches_engine(native, ln, lanes, csize, brange, primes, alias):
    import torch

    from ctwin_gb300 import PrpEngine
    from ctwin_gb300._native import check, lib

    rng = random.Random(4242 + ln + 7 * lanes)
    D = 1 << ln
    L = lib()
    stream = torch.cuda.current_stream()
    for call in range(2):
        b = np.array([rng.randrange(*brange) for _ in range(lanes)], dtype=np.uint32)
        x = np.array([[rng.randint(-(int(bb) // 2), int(bb) // 2) for _ in range(D)] for bb in b], dtype=np.int32)
        y = np.array([[rng.randint(-(int(bb) // 2), int(bb) // 2) for _ in range(D)] for bb in b], dtype=np.int32)
        with PrpEngine(ln, lanes, csize=csize) as eng:
            eng.set_b(b)
            assert eng.prime_count == primes
            eng.write_regs(np.stack([x, y]), 0)
            eng.mul_regs(2, 0, 1)
            want = eng.read_regs(2, 1)[0]
        xd = torch.from_numpy(x).cuda()
        yd = torch.from_numpy(y).cuda()
        zd = xd if alias else torch.zeros_like(xd)
        torch.cuda.synchronize()
        check(L.ctw_prp_mul_noalloc(ln, lanes, ctypes.c_void_p(b.ctypes.data), ctypes.c_void_p(xd.data_ptr()),
                                    ctypes.c_void_p(yd.data_ptr()), ctypes.c_void_p(zd.data_ptr()), csize,
                                    ctypes.c_void_p(stream.cuda_stream)))
        got = zd.cpu().numpy()
        assert np.array_equal(got, want), f"call {call}: {int((got != want).sum())} digits differ"


def test_mul_noalloc_rejects_oversize(native):
    from ctwin_gb300._native import lib
    L = lib()
    b = np.full(64, 1000003, dtype=np.uint32)
    null = ctypes.c_void_p(8)   # never dereferenced: the size check comes first
    assert L.ctw_prp_mul_noalloc(14, 64, ctypes.c_void_p(b.ctypes.data), null, null, null, 16, None) == -1
    assert b"exceed the fixed scratch" in L.ctw_last_error()
    assert L.ctw_prp_mul_noalloc(15, 1, ctypes.c_void_p(b.ctypes.data), null, null, null, 16, None) == -1


def test_mul_noalloc_rejects_stream_capture(native):
    """The call synchronises its stream, so it refuses a stream under capture
    (CTW_E_ARG) instead of recording a copy from its own stack frame."""
    import torch

    from ctwin_gb300._native import lib
    L = lib()
    b = np.full(1, 1000003, dtype=np.uint32)
    x = torch.zeros(1 << 11, dtype=torch.int32, device="cuda")
    keep = torch.zeros(16, device="cuda")
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        keep.add_(1.0)                     # the graph holds one node of its own
        st = torch.cuda.current_stream().cuda_stream
        rc = L.ctw_prp_mul_noalloc(11, 1, ctypes.c_void_p(b.ctypes.data), ctypes.c_void_p(x.data_ptr()),
                                   ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(x.data_ptr()), 16,
                                   ctypes.c_void_p(st))
    assert rc == -1
    assert b"being captured" in L.ctw_last_error()
    g.replay()                             # the captured add runs once, at replay
    torch.cuda.synchronize()
    assert float(keep[0]) == 1.0
