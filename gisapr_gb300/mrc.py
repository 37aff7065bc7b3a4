"""Minimal MRC2014 reader/writer for the volumes and particle stacks the search
reads (the reference uses the ``mrcfile`` package: v606:1054-1060,
1259-1318). Supported data modes: 0 (int8), 1 (int16), 2 (float32),
6 (uint16), 12 (float16); little- or big-endian by the machine stamp.
"""
from __future__ import annotations

import struct
from pathlib import Path

import numpy as np

_MODES = {0: np.int8, 1: np.int16, 2: np.float32, 6: np.uint16, 12: np.float16}


def _header(raw: bytes):
    stamp = raw[212:214]
    endian = ">" if stamp[:1] == b"\x11" else "<"
    nx, ny, nz, mode = struct.unpack(endian + "4i", raw[0:16])
    nsymbt = struct.unpack(endian + "i", raw[92:96])[0]
    if mode not in _MODES:
        raise ValueError(f"Unsupported MRC data mode {mode}")
    return endian, nx, ny, nz, mode, nsymbt


def read_mrc(path, mmap: bool = True) -> np.ndarray:
    """Data array shaped (nz, ny, nx) (2-D images as (ny, nx))."""
    path = Path(path)
    with open(path, "rb") as fh:
        raw = fh.read(1024)
    if len(raw) < 1024:
        raise ValueError(f"{path} is not an MRC file (short header)")
    endian, nx, ny, nz, mode, nsymbt = _header(raw)
    if min(nx, ny, nz) <= 0 or nsymbt < 0:
        raise ValueError(f"{path}: invalid MRC header (size {nx} x {ny} x {nz}, extended header {nsymbt} bytes)")
    dtype = np.dtype(_MODES[mode]).newbyteorder(endian)
    offset = 1024 + nsymbt
    count = nx * ny * nz
    if path.stat().st_size < offset + count * dtype.itemsize:
        raise ValueError(f"{path} is truncated: the header announces {nx} x {ny} x {nz} values")
    if mmap:
        data = np.memmap(path, dtype=dtype, mode="r", offset=offset, shape=(count,))
    else:
        data = np.fromfile(path, dtype=dtype, count=count, offset=offset)
    shape = (ny, nx) if nz == 1 else (nz, ny, nx)
    return data.reshape(shape)


def read_mrc_volume(path) -> np.ndarray:
    return np.array(read_mrc(path), dtype=np.float32, copy=True, order="C")


def write_mrc(path, data: np.ndarray, voxel_size: float = 1.0) -> None:
    """Write float32 data as a mode-2 little-endian MRC2014 file."""
    a = np.ascontiguousarray(data, dtype="<f4")
    if a.ndim == 2:
        nz, ny, nx = 1, a.shape[0], a.shape[1]
    elif a.ndim == 3:
        nz, ny, nx = a.shape
    else:
        raise ValueError("MRC data must be 2-D or 3-D")
    h = bytearray(1024)
    struct.pack_into("<4i", h, 0, nx, ny, nz, 2)
    struct.pack_into("<3i", h, 16, 0, 0, 0)
    struct.pack_into("<3i", h, 28, nx, ny, nz)
    struct.pack_into("<3f", h, 40, nx * voxel_size, ny * voxel_size, nz * voxel_size)
    struct.pack_into("<3f", h, 52, 90.0, 90.0, 90.0)
    struct.pack_into("<3i", h, 64, 1, 2, 3)
    struct.pack_into("<3f", h, 76, float(a.min()) if a.size else 0.0, float(a.max()) if a.size else 0.0,
                     float(a.mean()) if a.size else 0.0)
    struct.pack_into("<i", h, 92, 0)
    h[208:212] = b"MAP "
    h[212:216] = b"\x44\x44\x00\x00"
    struct.pack_into("<i", h, 104, 20140)
    with open(path, "wb") as fh:
        fh.write(bytes(h))
        fh.write(a.tobytes())
