"""Film output (pbrtgpu_write_image): write_img's 8-bit values
(src/camera/film.rs:15-33) in PNG and PPM, linear floats in PFM."""
import struct
import zlib

import numpy as np
import pytest

from pbrt_rust_gb300.gpu import image_bytes, write_image


@pytest.fixture
def rgb():
    r = np.random.default_rng(3).uniform(-0.2, 1.6, size=(7, 11, 3)).astype(np.float32)
    r[0, 0] = [np.nan, 0.0, 1.0]
    r[0, 1] = [np.inf, -np.inf, 0.5]
    return r


def expected_bytes(rgb):
    with np.errstate(invalid="ignore"):
        v = np.float32(255.0) * np.power(rgb, np.float32(1.0) / np.float32(2.2)) + np.float32(0.5)
    v = np.where(np.isnan(v), 0, np.clip(v, 0, 255))
    return v.astype(np.uint8)


def test_bytes_follow_write_img(lib, rgb):
    got = image_bytes(rgb)
    want = expected_bytes(rgb)
    assert np.abs(got.astype(int) - want.astype(int)).max() <= 1  # numpy's and libm's powf may differ by an ulp
    # NaN -> 0 (clamp keeps NaN, `as u8` makes it 0); pow(-inf, 1/2.2) = +inf -> 255
    assert got[0, 0, 0] == 0 and got[0, 1, 0] == 255 and got[0, 1, 1] == 255 and got[0, 0, 2] == 255


def read_png(path):
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat, ihdr = 8, b"", None
    while pos < len(data):
        n, = struct.unpack(">I", data[pos:pos + 4])
        typ = data[pos + 4:pos + 8]
        body = data[pos + 8:pos + 8 + n]
        crc, = struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])
        assert crc == zlib.crc32(typ + body) & 0xffffffff
        if typ == b"IHDR":
            ihdr = struct.unpack(">IIBBBBB", body)
        elif typ == b"IDAT":
            idat += body
        pos += 12 + n
    w, h, depth, color = ihdr[:4]
    assert (depth, color) == (8, 2)
    raw = zlib.decompress(idat)
    rows = np.frombuffer(raw, np.uint8).reshape(h, 1 + 3 * w)
    assert not rows[:, 0].any()  # filter 0
    return rows[:, 1:].reshape(h, w, 3)


def test_png_ppm_pfm_round_trip(lib, rgb, tmp_path):
    want = image_bytes(rgb)
    write_image(rgb, tmp_path / "a.png")
    assert np.array_equal(read_png(tmp_path / "a.png"), want)
    write_image(rgb, tmp_path / "a.ppm")
    data = open(tmp_path / "a.ppm", "rb").read()
    assert data.startswith(b"P6\n11 7\n255\n")
    assert np.array_equal(np.frombuffer(data[len(b"P6\n11 7\n255\n"):], np.uint8).reshape(7, 11, 3), want)
    write_image(rgb, tmp_path / "a.pfm")
    data = open(tmp_path / "a.pfm", "rb").read()
    head = b"PF\n11 7\n-1.0\n"
    assert data.startswith(head)
    back = np.frombuffer(data[len(head):], "<f4").reshape(7, 11, 3)[::-1]
    assert np.array_equal(back.view(np.uint32), rgb.view(np.uint32))


def read_exr(path):
    """A reader of the OpenEXR layout (magic, version, header attributes,
    scanline offset table, uncompressed one-line blocks) written from the
    published file-format description: returns (attributes, channels,
    (h, w, 3) RGB)."""
    import struct
    data = open(path, "rb").read()
    assert data[:4] == bytes([0x76, 0x2F, 0x31, 0x01]) and struct.unpack("<I", data[4:8])[0] == 2
    pos, attrs = 8, {}
    while data[pos] != 0:
        end = data.index(b"\0", pos)
        name = data[pos:end].decode()
        tend = data.index(b"\0", end + 1)
        typ = data[end + 1:tend].decode()
        size = struct.unpack("<i", data[tend + 1:tend + 5])[0]
        attrs[name] = (typ, data[tend + 5:tend + 5 + size])
        pos = tend + 5 + size
    pos += 1
    chl = attrs["channels"][1]
    chans, q = [], 0
    while chl[q] != 0:
        e = chl.index(b"\0", q)
        ptype, _, xs, ys = struct.unpack("<iIii", chl[e + 1:e + 17])
        chans.append((chl[q:e].decode(), ptype, xs, ys))
        q = e + 17
    x0, y0, x1, y1 = struct.unpack("<4i", attrs["dataWindow"][1])
    w, h = x1 - x0 + 1, y1 - y0 + 1
    offsets = struct.unpack(f"<{h}Q", data[pos:pos + 8 * h])
    planes = {c[0]: np.zeros((h, w), np.float32) for c in chans}
    for off in offsets:
        y, nbytes = struct.unpack("<iI", data[off:off + 8])
        assert nbytes == 4 * w * len(chans)
        row = np.frombuffer(data[off + 8:off + 8 + nbytes], "<f4").reshape(len(chans), w)
        for k, c in enumerate(chans):
            planes[c[0]][y - y0] = row[k]
    return attrs, chans, np.stack([planes["R"], planes["G"], planes["B"]], axis=-1)


def test_exr_holds_the_linear_floats(lib, rgb, tmp_path):
    write_image(rgb, tmp_path / "a.exr")
    attrs, chans, back = read_exr(tmp_path / "a.exr")
    assert [c[0] for c in chans] == ["B", "G", "R"] and all(c[1:] == (2, 1, 1) for c in chans)  # FLOAT
    assert attrs["compression"] == ("compression", b"\x00") and attrs["lineOrder"] == ("lineOrder", b"\x00")
    assert attrs["displayWindow"] == attrs["dataWindow"]
    assert np.array_equal(back.view(np.uint32), rgb.view(np.uint32))


def test_big_png_uses_several_deflate_blocks(lib, tmp_path):
    rgb = np.random.default_rng(1).uniform(0, 1, size=(200, 150, 3)).astype(np.float32)  # 90 kB of scanlines
    write_image(rgb, tmp_path / "b.png")
    assert np.array_equal(read_png(tmp_path / "b.png"), image_bytes(rgb))


def test_unknown_format_is_refused(lib, rgb, tmp_path):
    from pbrt_rust_gb300 import abi
    with pytest.raises(abi.PbrtError) as e:
        write_image(rgb, tmp_path / "a.tiff")
    assert e.value.status == 4  # PBRT_ERR_UNSUPPORTED
