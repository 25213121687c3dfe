"""The grid kernel's one-step carry division (reduce_b64 in
ctwin_gb300/csrc/prp_device.cuh) against the reference's two 29-bit Barrett
steps (reduce64 of cyclo/ocl/kernel.cl:480-510, restated as reduce() in
oracle/cpu_prp.c) on 64-bit values: same quotient and remainder for every b
the engine takes (64 <= b < 2^31) and |f| < 2^63, including values next to
multiples of b and the extremes.  Integer work: exact."""
import random


def barrett(a, b, b_inv, b_s):
    d = (((a >> b_s) & 0xFFFFFFFF) * b_inv) >> 32
    r = (a - d * b) & 0xFFFFFFFF
    return (d + 1, r - b) if r >= b else (d, r)


def reduce_ref(f, b):
    s = (b.bit_length() - 1) - 1
    b_inv = (1 << (s + 32)) // b
    t = -f if f < 0 else f
    assert ((t >> 29) >> s) >> 32 == 0            # the reference's range check never fires here
    d_h, r_h = barrett(t >> 29, b, b_inv, s)
    d_l, r_l = barrett((r_h << 29) | (t & ((1 << 29) - 1)), b, b_inv, s)
    d = (d_h << 29) | d_l
    return (-d, -r_l) if f < 0 else (d, r_l)


def reduce_one_step(f, b):
    m = ((1 << 64) - 1) // b
    t = -f if f < 0 else f
    q = (t * m) >> 64
    r = (t - q * b) & 0xFFFFFFFF
    if r >= b:
        r -= b
        q += 1
    return (-q, -r) if f < 0 else (q, r)


def test_one_step_division_equals_reference_barrett():
    rng = random.Random(11)
    bs = [64, 65, 127, 128, 1330358, 2 ** 21 - 1, 2 ** 30 + 1, 2 ** 31 - 1] + [rng.randrange(64, 2 ** 31) for _ in range(60)]
    for b in bs:
        vals = [0, 1, -1, b - 1, b, b + 1, -b, 2 ** 63 - 1, -(2 ** 63 - 1)]
        for _ in range(400):
            e = rng.randrange(1, 63)
            vals.append(rng.randrange(-(2 ** e), 2 ** e))
            k = rng.randrange(0, (2 ** 63 - 1) // b)
            vals += [k * b, k * b - 1, -(k * b), -(k * b) + 1]
        for f in vals:
            q, r = reduce_one_step(f, b)
            assert (q, r) == reduce_ref(f, b), (f, b)
            assert q * b + r == f and abs(r) < b and (r == 0 or (r < 0) == (f < 0))
