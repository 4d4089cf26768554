"""Map ingest and frame output: PNG decoding/encoding and the Futhark binary
data format (futspace_gb300/csrc/fs_io.c), checked against independent Python
restatements, the reference's own data-format reader (tools/data2png.py) and
the reference's map images when they are present."""
import importlib.util
import struct
import sys
import types
import zlib
from pathlib import Path

import numpy as np
import pytest

from conftest import reference_dir

# the reference checkout (FUTSPACE_REFERENCE_DIR), None when absent
REF = reference_dir()


# ---- an independent PNG encoder/decoder in numpy + zlib (test side) ----------

def _filter_rows(raw: np.ndarray, chans: int, kinds) -> bytes:
    """PNG filtering of [H][stride] u8 rows with the given filter type per row."""
    H, stride = raw.shape
    out = bytearray()
    prev = np.zeros(stride, np.int32)
    for y in range(H):
        row = raw[y].astype(np.int32)
        a = np.concatenate([np.zeros(chans, np.int32), row[:-chans]])
        c = np.concatenate([np.zeros(chans, np.int32), prev[:-chans]])
        b = prev
        k = kinds[y % len(kinds)]
        if k == 0:
            f = row
        elif k == 1:
            f = row - a
        elif k == 2:
            f = row - b
        elif k == 3:
            f = row - ((a + b) >> 1)
        else:
            p = a + b - c
            pa, pb, pc = np.abs(p - a), np.abs(p - b), np.abs(p - c)
            pred = np.where((pa <= pb) & (pa <= pc), a, np.where(pb <= pc, b, c))
            f = row - pred
        out.append(k)
        out += (f & 0xFF).astype(np.uint8).tobytes()
        prev = row
    return bytes(out)


def _chunk(t: bytes, body: bytes) -> bytes:
    return struct.pack(">I", len(body)) + t + body + struct.pack(">I", zlib.crc32(t + body))


def make_png(pixels: np.ndarray, ctype: int, palette=None, kinds=(0,), level=6,
             strategy=zlib.Z_DEFAULT_STRATEGY, split=8192) -> bytes:
    H, W = pixels.shape[:2]
    chans = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    raw = pixels.reshape(H, W * chans).astype(np.uint8)
    co = zlib.compressobj(level, zlib.DEFLATED, 15, 9, strategy)
    z = co.compress(_filter_rows(raw, chans, kinds)) + co.flush()
    png = b"\x89PNG\r\n\x1a\n" + _chunk(b"IHDR", struct.pack(">IIBBBBB", W, H, 8, ctype, 0, 0, 0))
    if palette is not None:
        png += _chunk(b"PLTE", palette.astype(np.uint8).tobytes())
    png += _chunk(b"tEXt", b"Comment\x00ancillary chunks are skipped")
    for i in range(0, len(z), split):
        png += _chunk(b"IDAT", z[i:i + split])
    return png + _chunk(b"IEND", b"")


def decode_png_numpy(data: bytes) -> np.ndarray:
    """Independent decoder for 8-bit non-interlaced PNGs -> 0xFFRRGGBB."""
    pos, idat, pal = 8, b"", None
    while pos < len(data):
        ln, t = struct.unpack(">I4s", data[pos:pos + 8])
        body = data[pos + 8:pos + 8 + ln]
        if t == b"IHDR":
            W, H, depth, ctype, _, _, il = struct.unpack(">IIBBBBB", body)
        elif t == b"PLTE":
            pal = np.frombuffer(body, np.uint8).reshape(-1, 3)
        elif t == b"IDAT":
            idat += body
        pos += 12 + ln
    chans = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    stride = W * chans
    raw = np.frombuffer(zlib.decompress(idat), np.uint8).reshape(H, stride + 1)
    img = np.zeros((H, stride), np.int32)
    prev = np.zeros(stride, np.int32)
    for y in range(H):
        k, f = raw[y, 0], raw[y, 1:].astype(np.int32)
        row = np.zeros(stride, np.int32)
        for i in range(stride):  # sequential: Sub/Avg/Paeth depend on the left byte
            a = row[i - chans] if i >= chans else 0
            b = prev[i]
            c = prev[i - chans] if i >= chans else 0
            if k == 0:
                pr = 0
            elif k == 1:
                pr = a
            elif k == 2:
                pr = b
            elif k == 3:
                pr = (a + b) >> 1
            else:
                p = a + b - c
                pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
                pr = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
            row[i] = (f[i] + pr) & 0xFF
        img[y], prev = row, row
    px = img.reshape(H, W, chans).astype(np.uint32)
    if ctype in (0, 4):
        r = g = b = px[:, :, 0]
    elif ctype == 3:
        rgb = pal[px[:, :, 0]].astype(np.uint32)
        r, g, b = rgb[:, :, 0], rgb[:, :, 1], rgb[:, :, 2]
    else:
        r, g, b = px[:, :, 0], px[:, :, 1], px[:, :, 2]
    return (np.uint32(0xFF000000) | (r << 16) | (g << 8) | b).astype(np.uint32)


def _expected(pixels, ctype, palette=None):
    p = pixels.astype(np.uint32)
    if ctype == 0:
        v = p
        return np.uint32(0xFF000000) | (v << 16) | (v << 8) | v
    if ctype == 4:
        v = p[:, :, 0]
        return np.uint32(0xFF000000) | (v << 16) | (v << 8) | v
    if ctype == 3:
        rgb = palette[p].astype(np.uint32)
        return np.uint32(0xFF000000) | (rgb[..., 0] << 16) | (rgb[..., 1] << 8) | rgb[..., 2]
    return np.uint32(0xFF000000) | (p[..., 0] << 16) | (p[..., 1] << 8) | p[..., 2]


@pytest.mark.parametrize("ctype", [0, 2, 3, 4, 6])
@pytest.mark.parametrize("kinds", [(0,), (1,), (2,), (3,), (4,), (0, 1, 2, 3, 4)])
def test_png_decode_colour_types_and_filters(fs, ctype, kinds):
    rng = np.random.default_rng(ctype * 10 + len(kinds) + kinds[0])
    H, W = 37, 53
    chans = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    palette = None
    if ctype == 3:
        palette = rng.integers(0, 256, (200, 3))
        pixels = rng.integers(0, 200, (H, W))
    else:
        # smooth ramps plus noise: exercises matches (copies) and literals alike
        base = (np.add.outer(np.arange(H), np.arange(W)) * 3) % 256
        pixels = (base[..., None] + rng.integers(0, 4, (H, W, chans))) % 256
        if chans == 1:
            pixels = pixels[..., 0]
    png = make_png(pixels, ctype, palette, kinds)
    got = fs.png_decode(png)
    np.testing.assert_array_equal(got, _expected(pixels, ctype, palette))
    np.testing.assert_array_equal(got, decode_png_numpy(png))


@pytest.mark.parametrize("level,strategy", [(0, zlib.Z_DEFAULT_STRATEGY), (1, zlib.Z_FIXED),
                                            (9, zlib.Z_DEFAULT_STRATEGY), (6, zlib.Z_RLE),
                                            (6, zlib.Z_HUFFMAN_ONLY)])
def test_png_inflate_block_kinds(fs, level, strategy):
    """Stored, fixed-Huffman and dynamic-Huffman deflate blocks, long matches."""
    rng = np.random.default_rng(level + strategy)
    H, W = 96, 300
    pix = np.repeat(rng.integers(0, 256, (H, 1, 3)), W, axis=1)
    pix[::7] = rng.integers(0, 256, (len(pix[::7]), W, 3))
    png = make_png(pix, 2, kinds=(0, 2), level=level, strategy=strategy, split=1000)
    np.testing.assert_array_equal(fs.png_decode(png), _expected(pix, 2))


def test_png_rejects_corrupt_input(fs):
    pix = np.arange(12 * 10 * 3).reshape(12, 10, 3) % 256
    png = bytearray(make_png(pix, 2))
    for bad in (bytes(png[:40]), b"GIF89a" + bytes(png[6:]),
                bytes(png[:33]) + bytes([png[33] ^ 1]) + bytes(png[34:])):
        with pytest.raises(fs.FsError) as e:
            fs.png_decode(bad)
        assert e.value.code == 7
    # 16-bit samples and interlacing are outside the supported forms
    ihdr16 = b"\x89PNG\r\n\x1a\n" + _chunk(b"IHDR", struct.pack(">IIBBBBB", 4, 4, 16, 2, 0, 0, 0))
    with pytest.raises(fs.FsError):
        fs.png_decode(ihdr16 + _chunk(b"IEND", b""))


def test_png_write_round_trip(fs, tmp_path):
    rng = np.random.default_rng(5)
    img = rng.integers(0, 2**32, (70, 130), dtype=np.uint64).astype(np.uint32)
    p = tmp_path / "frame.png"
    fs.png_write(p, img)
    data = p.read_bytes()
    want = (img & np.uint32(0x00FFFFFF)) | np.uint32(0xFF000000)  # alpha is not stored
    np.testing.assert_array_equal(decode_png_numpy(data), want)
    np.testing.assert_array_equal(fs.png_read(p), want)
    # more than one stored block and IDAT chunk
    big = rng.integers(0, 2**24, (700, 900), dtype=np.uint32)
    fs.png_write(p, big)
    np.testing.assert_array_equal(fs.png_read(p), big | np.uint32(0xFF000000))


@pytest.mark.skipif(REF is None or not (REF / "data").exists(),
                    reason="reference map images not present (set FUTSPACE_REFERENCE_DIR)")
@pytest.mark.parametrize("name", ["converted-maps/C1W.png", "converted-maps/D1.png",
                                  "unconverted-maps/C1W.png", "unconverted-maps/D1.png",
                                  "custom-maps/testmap.png"])
def test_png_decode_reference_maps(fs, name):
    """The reference's own map images (RGB, palette and greyscale PNGs)."""
    path = REF / "data" / name
    got = fs.png_read(path)
    assert got.shape == (1024, 1024)
    np.testing.assert_array_equal(got[:48], decode_png_numpy(path.read_bytes())[:48])
    # whole image through zlib + numpy for the filter-free fast check of bytes
    assert got.dtype == np.uint32 and np.all(got >> 24 == 0xFF)


def _reference_data_reader():
    """tools/data2png.py's read_image, imported with its image-writing module
    stubbed out (only the reader is used)."""
    if REF is None or not (REF / "tools" / "data2png.py").exists():
        pytest.skip("reference tools not present (set FUTSPACE_REFERENCE_DIR)")
    path = REF / "tools" / "data2png.py"
    sys.modules.setdefault("png", types.ModuleType("png"))
    spec = importlib.util.spec_from_file_location("ref_data2png", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.read_image


@pytest.mark.parametrize("dtype,tname", [(np.int32, " i32"), (np.uint32, " u32"),
                                         (np.uint8, "  u8")])
def test_data_format_write_read(fs, tmp_path, dtype, tname):
    rng = np.random.default_rng(3)
    a = rng.integers(0, 255 if dtype == np.uint8 else 2**31 - 1, (17, 29)).astype(dtype)
    p = tmp_path / "v.data"
    fs.data_write(p, a)
    raw = p.read_bytes()
    # header as tools/png2data.py:46-53 writes it
    assert raw[:7] == b"b" + bytes([2, 2]) + tname.encode()
    assert struct.unpack("<QQ", raw[7:23]) == (17, 29)
    b = fs.data_read(p)
    assert b.dtype == a.dtype and b.shape == a.shape
    np.testing.assert_array_equal(a, b)


def test_data_format_against_reference_reader(fs, tmp_path):
    read_image = _reference_data_reader()
    rng = np.random.default_rng(9)
    img = (rng.integers(0, 2**24, (23, 31)) | 0xFF000000).astype(np.uint32)
    p = tmp_path / "img.data"
    fs.data_write(p, img)
    with open(p, "rb") as f:
        w, h, rgb = read_image(f)
    assert (w, h) == (31, 23)
    rgb = np.asarray(rgb).reshape(23, 31, 3).astype(np.uint32)
    np.testing.assert_array_equal((rgb[..., 0] << 16) | (rgb[..., 1] << 8) | rgb[..., 2],
                                  img & np.uint32(0xFFFFFF))
    heights = rng.integers(0, 256, (19, 11)).astype(np.uint8)
    fs.data_write(p, heights)
    with open(p, "rb") as f:
        w, h, arr = read_image(f)
    np.testing.assert_array_equal(np.asarray(arr), heights)


def test_data_format_reads_png2data_layout(fs, tmp_path):
    """Bytes laid out as tools/png2data.py:46-53 writes an [h][w]i32 value."""
    rng = np.random.default_rng(4)
    arr = rng.integers(-2**31, 2**31 - 1, (5, 7)).astype(np.int32)
    p = tmp_path / "p.data"
    with open(p, "wb") as f:
        f.write(b"b" + np.int8(2).tobytes() + np.int8(2).tobytes() + b" i32")
        f.write(np.uint64(5).tobytes() + np.uint64(7).tobytes())
        arr.tofile(f)
    np.testing.assert_array_equal(fs.data_read(p), arr)
    p.write_bytes(p.read_bytes()[:-1])
    with pytest.raises(fs.FsError):
        fs.data_read(p)


@pytest.mark.gpu
def test_map_from_png_renders_like_arrays(fs, orc, gpu_ctx, tmp_path):
    """fs_map_load_png: a colour PNG and a height PNG give the same frames as the
    arrays they hold (heights from the low byte of each word)."""
    hm = fs.gen_heights(61, 256, 0.55)
    cm = fs.gen_colors(62, hm, 12)
    grey = (np.uint32(0xFF000000) | (hm.astype(np.uint32) * np.uint32(0x010101))).astype(np.uint32)
    fs.png_write(tmp_path / "c.png", cm)
    fs.png_write(tmp_path / "d.png", grey)
    fmap = fs.Map.from_png(gpu_ctx, tmp_path / "c.png", tmp_path / "d.png")
    assert fmap.shape == (256, 256)
    cm_file = cm | np.uint32(0xFF000000)
    for cam in fs.gen_cameras(63, hm, 3, above=(30, 60), distance=(300, 500), screen_h=60):
        got = gpu_ctx.render(fmap, cam, 80, 60)
        want = orc.render(cam, orc.make_params(), hm, cm_file, 80, 60)
        assert int(np.count_nonzero(got != want)) == 0
