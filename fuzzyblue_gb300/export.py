"""Export of the precomputed tables: the files the crate's dump example writes
(examples/dump.rs:205-227, 331-367) and NumPy arrays.

`export_atmosphere(atmosphere, directory)` writes
  transmittance.exr   RGBA FLOAT, width x height = transmittance extent
  irradiance.exr      RGBA FLOAT
  scattering.exr      RGBA HALF, one layer per depth slice (r), channel names
                      "<layer>.R" ... "<layer>.A" (plain "R" ... "A" for depth 1)
as examples/dump.rs does (the scattering table is read back as RGBA16F there,
the transmittance and irradiance tables as RGBA32F), or the same three tables
as .npy files (`fmt="npy"`, float32, scattering also as float16).

The EXR writer emits single-part scanline files without compression, in the
layout of the published OpenEXR file format: magic number and version, the
header attributes (channels, compression, dataWindow, displayWindow,
lineOrder, pixelAspectRatio, screenWindowCenter, screenWindowWidth), the line
offset table, then one block per scanline holding each channel's row, channels
in byte order of their names. `read_exr` reads such files back.
"""
from __future__ import annotations

import os
import struct
from typing import Dict, Tuple

import numpy as np

_MAGIC = 20000630
_VERSION = 2  # single-part scanline file
_PIXEL_TYPE = {np.dtype(np.uint32): 0, np.dtype(np.float16): 1, np.dtype(np.float32): 2}
_DTYPE_OF = {0: np.dtype("<u4"), 1: np.dtype("<f2"), 2: np.dtype("<f4")}


def _attr(name: str, type_name: str, value: bytes) -> bytes:
    return name.encode() + b"\0" + type_name.encode() + b"\0" + struct.pack("<i", len(value)) + value


def _chlist(channels) -> bytes:
    out = b""
    for name, ptype in channels:
        # name, pixel type, pLinear (1 byte) + 3 reserved bytes, xSampling, ySampling
        out += name.encode() + b"\0" + struct.pack("<iB3xii", ptype, 0, 1, 1)
    return out + b"\0"


def write_exr(path: str, channels: Dict[str, np.ndarray]) -> None:
    """Writes 2D arrays of one shape (height, width) as the named channels
    (float32 -> FLOAT, float16 -> HALF, uint32 -> UINT)."""
    if not channels:
        raise ValueError("no channels")
    names = sorted(channels, key=lambda n: n.encode())
    shapes = {channels[n].shape for n in names}
    if len(shapes) != 1 or len(next(iter(shapes))) != 2:
        raise ValueError("channels must be 2D arrays of one shape")
    height, width = next(iter(shapes))
    data = []
    for n in names:
        a = np.asarray(channels[n])
        if a.dtype not in _PIXEL_TYPE:
            raise ValueError("unsupported pixel type %s" % a.dtype)
        data.append(np.ascontiguousarray(a, a.dtype.newbyteorder("<")))
    header = b"".join([
        _attr("channels", "chlist", _chlist([(n, _PIXEL_TYPE[d.dtype.newbyteorder("=")]) for n, d in zip(names, data)])),
        _attr("compression", "compression", bytes([0])),
        _attr("dataWindow", "box2i", struct.pack("<iiii", 0, 0, width - 1, height - 1)),
        _attr("displayWindow", "box2i", struct.pack("<iiii", 0, 0, width - 1, height - 1)),
        _attr("lineOrder", "lineOrder", bytes([0])),
        _attr("pixelAspectRatio", "float", struct.pack("<f", 1.0)),
        _attr("screenWindowCenter", "v2f", struct.pack("<ff", 0.0, 0.0)),
        _attr("screenWindowWidth", "float", struct.pack("<f", 1.0)),
    ]) + b"\0"
    prefix = struct.pack("<ii", _MAGIC, _VERSION) + header
    row_bytes = sum(width * d.dtype.itemsize for d in data)
    block = 8 + row_bytes  # y, data size, pixel data
    start = len(prefix) + 8 * height
    offsets = struct.pack("<%dQ" % height, *[start + y * block for y in range(height)])
    with open(path, "wb") as f:
        f.write(prefix)
        f.write(offsets)
        for y in range(height):
            f.write(struct.pack("<ii", y, row_bytes))
            for d in data:
                f.write(d[y].tobytes())


def read_exr(path: str) -> Tuple[Dict[str, np.ndarray], Dict[str, bytes]]:
    """Reads an uncompressed single-part scanline EXR written by write_exr:
    returns the channels (2D arrays) and the raw header attributes."""
    with open(path, "rb") as f:
        buf = f.read()
    magic, version = struct.unpack_from("<ii", buf, 0)
    if magic != _MAGIC or (version & 0xFF) != 2 or version & 0x200:
        raise ValueError("not a single-part scanline EXR")
    pos, attrs = 8, {}
    while buf[pos] != 0:
        end = buf.index(b"\0", pos)
        name = buf[pos:end].decode()
        tend = buf.index(b"\0", end + 1)
        (size,) = struct.unpack_from("<i", buf, tend + 1)
        attrs[name] = buf[tend + 5:tend + 5 + size]
        pos = tend + 5 + size
    pos += 1
    if attrs["compression"] != bytes([0]):
        raise ValueError("compressed EXR")
    chans, p = [], 0
    raw = attrs["channels"]
    while raw[p] != 0:
        end = raw.index(b"\0", p)
        ptype = struct.unpack_from("<i", raw, end + 1)[0]
        chans.append((raw[p:end].decode(), _DTYPE_OF[ptype]))
        p = end + 1 + 16
    x0, y0, x1, y1 = struct.unpack_from("<iiii", attrs["dataWindow"])
    width, height = x1 - x0 + 1, y1 - y0 + 1
    offsets = struct.unpack_from("<%dQ" % height, buf, pos)
    out = {n: np.empty((height, width), d) for n, d in chans}
    for y, off in enumerate(offsets):
        row, size = struct.unpack_from("<ii", buf, off)
        q = off + 8
        for n, d in chans:
            out[n][row - y0] = np.frombuffer(buf, d, width, q)
            q += width * d.itemsize
    return out, attrs


def channel_name(color: str, layer: int, layers: int) -> str:
    """examples/dump.rs:362-367: "<layer>.<color>" for layered images."""
    return color if layers == 1 else "%d.%s" % (layer, color)


def write_table_exr(path: str, table: np.ndarray) -> None:
    """An RGBA table shaped (height, width, 4) or (depth, height, width, 4)
    as one EXR, one layer per depth slice."""
    t = table if table.ndim == 4 else table[None]
    depth = t.shape[0]
    ch = {}
    for layer in range(depth):
        for c, color in enumerate("RGBA"):
            ch[channel_name(color, layer, depth)] = t[layer, :, :, c]
    write_exr(path, ch)


def export_atmosphere(atmosphere, directory: str, fmt: str = "exr") -> Dict[str, str]:
    """Writes the three tables of `atmosphere` (fuzzyblue_gb300.api.Atmosphere)
    into `directory`; returns the paths written."""
    os.makedirs(directory, exist_ok=True)
    t = atmosphere.to_host()
    paths = {}
    if fmt == "exr":
        for name in ("transmittance", "irradiance"):
            paths[name] = os.path.join(directory, name + ".exr")
            write_table_exr(paths[name], t[name].astype(np.float32))
        paths["scattering"] = os.path.join(directory, "scattering.exr")
        write_table_exr(paths["scattering"], atmosphere.export_scattering_f16())
    elif fmt == "npy":
        for name in ("transmittance", "irradiance", "scattering"):
            paths[name] = os.path.join(directory, name + ".npy")
            np.save(paths[name], t[name])
        paths["scattering_f16"] = os.path.join(directory, "scattering_f16.npy")
        np.save(paths["scattering_f16"], atmosphere.export_scattering_f16())
    else:
        raise ValueError("fmt must be 'exr' or 'npy'")
    return paths
