"""MRC reader and writer (CPU): round trip, byte order, and clear errors for
malformed files instead of a failed memory map."""
import struct

import numpy as np
import pytest

from gisapr_gb300.mrc import read_mrc, read_mrc_volume, write_mrc


def test_round_trip_2d_and_3d(tmp_path):
    rng = np.random.default_rng(3)
    for shape in ((5, 7), (3, 5, 7)):
        a = rng.normal(size=shape).astype(np.float32)
        p = tmp_path / f"a{len(shape)}.mrc"
        write_mrc(p, a, voxel_size=1.5)
        np.testing.assert_array_equal(read_mrc(p), a)
        np.testing.assert_array_equal(read_mrc(p, mmap=False), a)
    assert read_mrc_volume(tmp_path / "a3.mrc").flags["C_CONTIGUOUS"]


def test_big_endian_int16(tmp_path):
    a = np.arange(24, dtype=">i2").reshape(2, 3, 4)
    h = bytearray(1024)
    struct.pack_into(">4i", h, 0, 4, 3, 2, 1)
    h[212:214] = b"\x11\x11"
    p = tmp_path / "be.mrc"
    p.write_bytes(bytes(h) + a.tobytes())
    np.testing.assert_array_equal(read_mrc(p), a.astype(np.int16))


@pytest.mark.parametrize("dims,extra,cut", [((0, 4, 4), 0, 0), ((4, 4, -1), 0, 0), ((4, 4, 1), -8, 0),
                                            ((4, 4, 2), 0, 4)])
def test_malformed_headers_raise(tmp_path, dims, extra, cut):
    h = bytearray(1024)
    struct.pack_into("<4i", h, 0, *dims, 2)
    struct.pack_into("<i", h, 92, extra)
    body = np.zeros(max(0, dims[0] * dims[1] * dims[2]), np.float32).tobytes()
    p = tmp_path / "bad.mrc"
    p.write_bytes(bytes(h) + body[:len(body) - cut])
    with pytest.raises(ValueError):
        read_mrc(p)


def test_short_header_and_unknown_mode(tmp_path):
    p = tmp_path / "short.mrc"
    p.write_bytes(b"\0" * 100)
    with pytest.raises(ValueError, match="short header"):
        read_mrc(p)
    h = bytearray(1024)
    struct.pack_into("<4i", h, 0, 2, 2, 1, 4)  # mode 4 (complex) is not a search input
    p.write_bytes(bytes(h) + b"\0" * 32)
    with pytest.raises(ValueError, match="mode 4"):
        read_mrc(p)
