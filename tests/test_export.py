"""LUT export (fuzzyblue_gb300.export): OpenEXR files as the crate's dump
example writes them (examples/dump.rs:331-367) and NumPy arrays."""
import struct

import numpy as np
import pytest

from fuzzyblue_gb300 import export
from fuzzyblue_gb300.params import smoke_parameters


def test_exr_round_trip_and_layout(tmp_path):
    rng = np.random.default_rng(0)
    ch = {"R": rng.random((5, 7), dtype=np.float32), "G": rng.random((5, 7), dtype=np.float32),
          "B": rng.random((5, 7)).astype(np.float16), "ID": np.arange(35, dtype=np.uint32).reshape(5, 7)}
    path = str(tmp_path / "t.exr")
    export.write_exr(path, ch)
    raw = open(path, "rb").read()
    assert struct.unpack_from("<ii", raw, 0) == (20000630, 2)
    back, attrs = export.read_exr(path)
    assert set(back) == set(ch)
    for k in ch:
        assert back[k].dtype == ch[k].dtype and np.array_equal(back[k], ch[k]), k
    assert struct.unpack("<iiii", attrs["dataWindow"]) == (0, 0, 6, 4)
    assert attrs["compression"] == bytes([0])
    # channel list sorted by name bytes
    names = []
    p = 0
    while attrs["channels"][p] != 0:
        e = attrs["channels"].index(b"\0", p)
        names.append(attrs["channels"][p:e].decode())
        p = e + 17
    assert names == sorted(names, key=str.encode)


def test_layered_channel_names(tmp_path):
    t = np.random.default_rng(1).random((12, 3, 4, 4)).astype(np.float16)
    path = str(tmp_path / "s.exr")
    export.write_table_exr(path, t)
    back, _ = export.read_exr(path)
    assert "10.R" in back and "2.A" in back and len(back) == 48
    for layer in range(12):
        for c, color in enumerate("RGBA"):
            assert np.array_equal(back["%d.%s" % (layer, color)], t[layer, :, :, c])
    flat = np.random.default_rng(2).random((3, 4, 4), dtype=np.float32)
    export.write_table_exr(str(tmp_path / "f.exr"), flat)
    back, _ = export.read_exr(str(tmp_path / "f.exr"))
    assert sorted(back) == ["A", "B", "G", "R"]


@pytest.mark.gpu
def test_export_atmosphere(builder, tmp_path):
    from fuzzyblue_gb300.api import Atmosphere
    pend = Atmosphere.build(builder, smoke_parameters())
    pend.wait()
    atm = pend.atmosphere()
    tables = atm.to_host()
    half = atm.export_scattering_f16()
    paths = export.export_atmosphere(atm, str(tmp_path / "exr"))
    for name in ("transmittance", "irradiance"):
        back, _ = export.read_exr(paths[name])
        for c, color in enumerate("RGBA"):
            assert np.array_equal(back[color], tables[name][..., c]), (name, color)
    back, _ = export.read_exr(paths["scattering"])
    depth = tables["scattering"].shape[0]
    for layer in range(depth):
        for c, color in enumerate("RGBA"):
            assert np.array_equal(back["%d.%s" % (layer, color)], half[layer, :, :, c])
    npy = export.export_atmosphere(atm, str(tmp_path / "npy"), fmt="npy")
    for name in ("transmittance", "irradiance", "scattering"):
        assert np.array_equal(np.load(npy[name]), tables[name])
    assert np.array_equal(np.load(npy["scattering_f16"]), half)
    pend.release()


def test_exr_bytes_match_the_file_format(tmp_path):
    """A two-channel 2 x 2 file assembled byte by byte from the published
    OpenEXR layout (magic number, version field, attributes as name, type
    name, size and value, header terminator, one 64-bit offset per scanline,
    then per scanline its y, its byte count and each channel's row with the
    channels in name order), independent of `write_exr` and `read_exr`."""
    a = np.array([[1.0, 2.0], [3.0, 4.0]], np.float32)          # FLOAT
    b = np.array([[0.5, -2.0], [65504.0, 0.0]], np.float16)     # HALF
    path = str(tmp_path / "k.exr")
    export.write_exr(path, {"B": b, "A": a})  # given out of name order
    got = open(path, "rb").read()

    def attr(name, typ, value_hex):
        v = bytes.fromhex(value_hex)
        return name + b"\0" + typ + b"\0" + len(v).to_bytes(4, "little") + v

    chlist = ("41 00" "02000000" "00 000000" "01000000" "01000000"     # "A", FLOAT, pLinear 0, sampling 1 1
              "42 00" "01000000" "00 000000" "01000000" "01000000"     # "B", HALF
              "00")
    header = b"".join([
        bytes.fromhex("762f3101"),          # magic 20000630
        bytes.fromhex("02000000"),          # version 2, single-part scanline, no flags
        attr(b"channels", b"chlist", chlist),
        attr(b"compression", b"compression", "00"),                     # NO_COMPRESSION
        attr(b"dataWindow", b"box2i", "00000000" "00000000" "01000000" "01000000"),
        attr(b"displayWindow", b"box2i", "00000000" "00000000" "01000000" "01000000"),
        attr(b"lineOrder", b"lineOrder", "00"),                         # INCREASING_Y
        attr(b"pixelAspectRatio", b"float", "0000803f"),                # 1.0
        attr(b"screenWindowCenter", b"v2f", "00000000" "00000000"),
        attr(b"screenWindowWidth", b"float", "0000803f"),
        b"\0",
    ])
    row = 2 * 4 + 2 * 2                      # A: two floats, B: two halves
    first = len(header) + 2 * 8              # after the offset table
    expect = header + (first).to_bytes(8, "little") + (first + 8 + row).to_bytes(8, "little")
    # scanline 0: A = 1.0 2.0, B = 0.5 -2.0; scanline 1: A = 3.0 4.0, B = 65504 0
    expect += bytes.fromhex("00000000" "0c000000" "0000803f" "00000040" "0038" "00c0")
    expect += bytes.fromhex("01000000" "0c000000" "00004040" "00008040" "ff7b" "0000")
    assert got == expect
