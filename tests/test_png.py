"""PNG texture ingest (Texture::from_png_file, src/texture.rs:26-45)."""
import os
import zlib

import numpy as np
import pytest

from rusterizer_gb300 import png

# the reference crate's demo asset (images/checkerboard.png), when a copy of the crate is at
# hand: RUSTERIZER_REFERENCE names the crate's root directory; the tests that need it skip
# otherwise
REF_CHECKERBOARD = os.path.join(os.environ.get("RUSTERIZER_REFERENCE", ""), "images", "checkerboard.png")


@pytest.mark.parametrize("filters", [(0,), (1,), (2,), (3,), (4,), (0, 1, 2, 3, 4), (4, 3, 2, 1)])
def test_round_trip_every_filter(filters):
    rng = np.random.default_rng(len(filters) * 7 + filters[0])
    for h, w in [(1, 1), (3, 5), (17, 9), (32, 33)]:
        img = rng.integers(0, 256, (h, w, 4), dtype=np.uint8)
        data = png.encode_png_rgba8(img, filters=filters)
        assert (png.decode_png_rgba8(data) == img).all()


def test_smooth_image_all_filters_and_split_idat():
    y, x = np.mgrid[0:40, 0:50]
    img = np.stack([x * 5, y * 6, (x + y) * 2, 255 - x], -1).astype(np.uint8)
    data = png.encode_png_rgba8(img, filters=(0, 1, 2, 3, 4))
    # split the IDAT payload into three chunks, as encoders may do
    sig, rest = data[:8], data[8:]
    ihdr_len = 12 + 13
    ihdr, idat_chunk, iend = rest[:ihdr_len], rest[ihdr_len:-12], rest[-12:]
    payload = idat_chunk[8:-4]
    parts = [payload[:5], payload[5:11], payload[11:]]

    def chunk(t, body):
        import struct
        return struct.pack(">I", len(body)) + t + body + struct.pack(">I", zlib.crc32(t + body) & 0xFFFFFFFF)

    split = sig + ihdr + b"".join(chunk(b"IDAT", p) for p in parts) + iend
    assert (png.decode_png_rgba8(split) == img).all()


def test_rejects_what_the_reference_only_debug_asserts():
    img = np.zeros((2, 2, 4), np.uint8)
    good = bytearray(png.encode_png_rgba8(img))
    # colour type 2 (RGB): rewrite IHDR and its CRC
    import struct
    bad = bytearray(good)
    bad[8 + 8 + 9] = 2
    bad[8 + 8 + 13:8 + 8 + 17] = struct.pack(">I", zlib.crc32(bytes(bad[8 + 4:8 + 8 + 13])) & 0xFFFFFFFF)
    with pytest.raises(ValueError, match="RGBA"):
        png.decode_png_rgba8(bytes(bad))
    inter = bytearray(good)
    inter[8 + 8 + 12] = 1
    inter[8 + 8 + 13:8 + 8 + 17] = struct.pack(">I", zlib.crc32(bytes(inter[8 + 4:8 + 8 + 13])) & 0xFFFFFFFF)
    with pytest.raises(ValueError, match="interlaced"):
        png.decode_png_rgba8(bytes(inter))
    corrupt = bytearray(good)
    corrupt[8 + 8 + 2] ^= 0x40  # width byte, CRC now wrong
    with pytest.raises(ValueError, match="corrupt"):
        png.decode_png_rgba8(bytes(corrupt))
    with pytest.raises(ValueError, match="signature"):
        png.decode_png_rgba8(b"GIF89a" + bytes(good[6:]))


@pytest.mark.skipif(not os.path.exists(REF_CHECKERBOARD), reason="reference assets not mounted")
def test_reference_checkerboard_asset():
    """The crate's demo texture (images/checkerboard.png, Sub/Up/Paeth rows) decodes to a
    400x400 black/white checkerboard of 100-pixel squares, black at the top-left."""
    img = png.read_png_rgba8(REF_CHECKERBOARD)
    assert img.shape == (400, 400, 4)
    y, x = np.mgrid[0:400, 0:400]
    white = ((x // 100) + (y // 100)) % 2 == 1
    expect = np.where(white[..., None], np.uint8(255), np.array([0, 0, 0, 255], np.uint8))
    assert (img == expect).all()


def test_argb_to_rgba8():
    argb = np.array([[0xFF191919, 0x80FF0010]], np.uint32)
    assert png.argb_to_rgba8(argb).tolist() == [[[0x19, 0x19, 0x19, 0xFF], [0xFF, 0x00, 0x10, 0x80]]]


@pytest.mark.gpu
def test_png_texture_renders_like_the_oracle(tmp_path):
    """A PNG-ingested checkerboard on the demo cube: GPU frame == oracle frame."""
    import oracle
    from rusterizer_gb300 import renderer, scenes
    y, x = np.mgrid[0:96, 0:96]
    white = ((x // 24) + (y // 24)) % 2 == 1
    img = np.where(white[..., None], np.uint8(255), np.array([0, 0, 0, 255], np.uint8))
    path = tmp_path / "checker.png"
    path.write_bytes(png.encode_png_rgba8(img, filters=(1, 2, 4)))
    tex = renderer.Texture.from_png_file(str(path))
    assert (tex.buf == img).all()
    scene = scenes.config0()
    scene["textures"] = [tex.buf]
    argb, status, _ = renderer.render_scene(scene)
    ref, *_ = oracle.render_scene(scene)
    assert (argb == ref).all()
