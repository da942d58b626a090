"""Plan-file format helpers on the CPU: the checksum and the header reader
that mirror fl_cache.cu (the GPU tests check the library's own files against
them)."""
import struct

import numpy as np
import pytest

from fastload_gb300 import plan as P

HEADER = dict(magic=b"FLGBPLAN", version=1, header_bytes=128, byte_order=0x01020304, m=5, n=3, nnz=4,
              tilenum=3, steps=2, with_ref=1, heavy=-1, nforms=1, reserved0=0)


def fnv_words_reference(data: bytes) -> int:
    """The checksum spelled out byte by byte: FNV-1a over 64-bit words."""
    h = 0xCBF29CE484222325
    for i in range(0, len(data), 8):
        w = 0
        for j, b in enumerate(data[i:i + 8]):
            w |= b << (8 * j)
        h = ((h ^ w) * 0x100000001B3) % (1 << 64)
    return h ^ len(data)


@pytest.mark.parametrize("size", [0, 1, 7, 8, 9, 64, 1001])
def test_hash_matches_bytewise_statement(size):
    data = bytes((i * 37 + 11) % 256 for i in range(size))
    assert P.plan_file_hash(data) == fnv_words_reference(data)


def test_hash_depends_on_length_and_content():
    assert P.plan_file_hash(b"") != P.plan_file_hash(b"\0")
    assert P.plan_file_hash(b"\1" + b"\0" * 15) != P.plan_file_hash(b"\0" * 8 + b"\1" + b"\0" * 7)


def test_header_round_trip(tmp_path):
    f = tmp_path / "a.flplan"
    sec = dict(perm=[2, 0, 1], sortnnz=[1, 1, 2], row=[4, 0, 1, 3], val=[1.5, -2, 3, 4],
               forms=np.array([[1, -2, 0]]))
    P.write_plan_file(f, HEADER, sec)
    assert f.stat().st_size == 128 + 8 * 3 + 12 * 4 + 12
    h = P.plan_file_header(f)
    for k, v in HEADER.items():
        assert h[k] == v, k
    s = P.plan_file_sections(f)
    np.testing.assert_array_equal(s["perm"], [2, 0, 1])
    np.testing.assert_array_equal(s["val"], [1.5, -2, 3, 4])
    np.testing.assert_array_equal(s["forms"], [[1, -2, 0]])
    assert h["hashes"]["row"] == P.plan_file_hash(np.array([4, 0, 1, 3], "<i4").tobytes())


def test_header_rejects_corruption(tmp_path):
    f = tmp_path / "a.flplan"
    P.write_plan_file(f, HEADER, dict(perm=[0, 1, 2], sortnnz=[1, 1, 2], row=[0, 1, 2, 3], val=[1.0] * 4,
                                      forms=np.array([[0, 0, 0]])))
    raw = bytearray(f.read_bytes())
    raw[20] ^= 1  # m
    f.write_bytes(bytes(raw))
    with pytest.raises(ValueError, match="checksum"):
        P.plan_file_header(f)
    f.write_bytes(b"NOTAPLAN" + bytes(raw[8:]))
    with pytest.raises(ValueError, match="not a plan file"):
        P.plan_file_header(f)
    f.write_bytes(bytes(raw[:40]))
    with pytest.raises(ValueError, match="not a plan file"):
        P.plan_file_header(f)


def test_header_struct_is_128_bytes():
    assert P._HEADER.size == 128
    assert struct.calcsize("<8sIII9i") == 56
