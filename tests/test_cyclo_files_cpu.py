"""The reference's context format (cyclo.ctx), without a GPU: an independent
Python restatement of cyclo/src/cyclo.h:146-177, cyclo/src/transform.h:458-468
and the file class's CRC32 trailer (cyclo/src/file.h) against the library's
encoder and decoder."""
import struct
import zlib

import numpy as np
import pytest

P = (4293918721, 4253024257, 4231004161)


def ref_bytes(digits, k, i, elapsed):
    nregs, lanes, D = digits.shape
    head = struct.pack("<Iiid", 1, k, i, elapsed)
    x12 = bytearray()
    x3 = bytearray()
    for r in range(nregs):
        for j in range(D):
            for l in range(lanes):
                d = int(digits[r, l, j])
                x12 += struct.pack("<II", d % P[0], d % P[1])
                x3 += struct.pack("<I", d % P[2])
    body = head + bytes(x12) + bytes(x3)
    trailer = (~zlib.crc32(body) ^ 0xA23777AC) & 0xFFFFFFFF
    return body + struct.pack("<I", trailer)


@pytest.fixture(scope="module")
def cyclo():
    try:
        from ctwin_gb300 import cyclo as C
        from ctwin_gb300._native import lib
        lib()
        return C
    except ImportError as e:
        pytest.skip(f"native library not built: {e}")


def test_context_encode_matches_reference_layout(cyclo):
    rng = np.random.default_rng(1)
    d = rng.integers(-(1 << 30), 1 << 30, size=(2, 64, 256), dtype=np.int64).astype(np.int32)
    data = cyclo.context_encode(d, 3, 12345, 678.5)
    assert data == ref_bytes(d, 3, 12345, 678.5)


def test_context_roundtrip_and_crc(cyclo):
    rng = np.random.default_rng(2)
    d = rng.integers(-70000, 70000, size=(2, 4, 512)).astype(np.int32)
    data = cyclo.context_encode(d, 0, 99, 1.25)
    back, k, i, el = cyclo.context_decode(data, 9, 4)
    assert np.array_equal(back, d) and (k, i, el) == (0, 99, 1.25)
    from ctwin_gb300 import CtwError
    bad = bytearray(data)
    bad[40] ^= 1
    with pytest.raises(CtwError):
        cyclo.context_decode(bytes(bad), 9, 4)          # CRC32 mismatch
    # a consistent CRC over residues that name no 32-bit digit
    raw = bytearray(data[:-4])
    raw[20:24] = struct.pack("<I", 123)
    raw[24:28] = struct.pack("<I", 456)
    raw += struct.pack("<I", (~zlib.crc32(bytes(raw)) ^ 0xA23777AC) & 0xFFFFFFFF)
    with pytest.raises(CtwError):
        cyclo.context_decode(bytes(raw), 9, 4)
