"""Image files packed on the GPU (cy_encode_image): byte for byte what the
reference's own writers make of the same get_image_data pixels -- the test
harness's uncompressed PNG (test/test.cpp:2415-2511) and the tiger demo's
TGA (demos/tiger/tiger.cpp:4336-4343), restated here with zlib's CRC-32 and
Adler-32.  The restatements are pinned to the files the reference's writers
made (SHA-256 in tests/golden/manifest.json): the PNG of every recorded
reference test and the tiger demo's tiger.tga."""
import ctypes
import hashlib
import struct
import zlib

import numpy as np
import pytest

from canvas_ity_gb300 import native, scenes
from canvas_ity_gb300 import trace as T
import golden_util as G


def ref_png(rgba: bytes, w: int, h: int) -> bytes:
    ihdr = b"IHDR" + struct.pack(">II", w, h) + bytes([8, 6, 0, 0, 0])
    out = bytearray(b"\x89PNG\r\n\x1a\n" + struct.pack(">I", 13) + ihdr + struct.pack(">I", zlib.crc32(ihdr)))
    out += bytes([0, 0, 0, 1, 115, 82, 71, 66, 0, 174, 206, 28, 233])
    size = 1 + 4 * w
    data = bytearray(b"\x78\x01")
    raw = bytearray()
    for y in range(h):
        row = rgba[y * 4 * w:(y + 1) * 4 * w]
        data += bytes([1 if y + 1 == h else 0, size & 255, size >> 8, ~size & 255, (~size >> 8) & 255, 0]) + row
        raw += b"\x00" + row
    data += struct.pack(">I", zlib.adler32(bytes(raw)))
    idat = b"IDAT" + bytes(data)
    out += struct.pack(">I", len(data)) + idat + struct.pack(">I", zlib.crc32(idat))
    out += b"\x00\x00\x00\x00IEND\xaeB`\x82"
    return bytes(out)


def ref_tga(rgba: bytes, w: int, h: int) -> bytes:
    px = np.frombuffer(rgba, np.uint8).reshape(-1, 4)[:, [2, 1, 0, 3]]
    return bytes([0, 0, 2, 0, 0, 0, 0, 0, 0, 0, 0, 0, w & 255, w >> 8, h & 255, h >> 8, 32, 40]) + px.tobytes()


def test_reference_png_restatement_is_a_valid_stream():
    """The restated writer's IDAT inflates back to the filtered rows."""
    w, h = 5, 3
    rgba = bytes(range(w * h * 4))
    png = ref_png(rgba, w, h)
    at = 33 + 13
    n = struct.unpack(">I", png[at:at + 4])[0]
    rows = zlib.decompress(png[at + 8:at + 8 + n])
    assert rows == b"".join(b"\x00" + rgba[y * 20:(y + 1) * 20] for y in range(h))


def sha(b: bytes) -> str:
    return hashlib.sha256(b).hexdigest()


MANIFEST = G.manifest()
DEMOS = G.demos()


@pytest.mark.parametrize("entry", MANIFEST, ids=[e["name"] for e in MANIFEST])
def test_png_restatement_is_the_reference_writer(entry):
    """ref_png of a test's final image is the file the reference's own
    write_png made of it (test.cpp --pngs)."""
    img = G.final_image(G.load_fixture(entry))
    h, w = img.shape[:2]
    png = ref_png(img.tobytes(), w, h)
    assert len(png) == entry["reference_png_bytes"]
    assert sha(png) == entry["reference_png_sha256"]


@pytest.mark.parametrize("demo", DEMOS, ids=[d["name"] for d in DEMOS])
def test_tga_restatement_is_the_tiger_writer(demo):
    img = G.final_image(G.load_fixture(demo))
    tga = ref_tga(img.tobytes(), demo["width"], demo["height"])
    assert len(tga) == demo["reference_tga_bytes"]
    assert sha(tga) == demo["reference_tga_sha256"]


# small reference tests whose canvases the GPU packs as PNG (exact coverage,
# where the canvas is the reference's byte for byte)
PNG_CASES = [e for e in MANIFEST if e["name"] in ("fill_rectangle", "linear_gradient", "shadow_blur", "fill_text",
                                                  "example_smiley", "draw_image")]


@pytest.mark.gpu
@pytest.mark.parametrize("entry", PNG_CASES, ids=[e["name"] for e in PNG_CASES])
def test_gpu_png_is_the_reference_file(entry):
    tb = G.load_fixture(entry)
    w, h = T.canvas_size(tb)
    G.use_mode("tile_exact")
    try:
        got = native.encode_image(tb, native.PNG, 0, 0, w, h)
    finally:
        G.use_mode("tile")
    assert sha(got) == entry["reference_png_sha256"]


@pytest.mark.gpu
@pytest.mark.parametrize("demo", DEMOS, ids=[d["name"] for d in DEMOS])
def test_gpu_tga_is_the_tiger_file(demo):
    tb = G.load_fixture(demo)
    G.use_mode("tile_exact")
    try:
        got = native.encode_image(tb, native.TGA, 0, 0, demo["width"], demo["height"])
    finally:
        G.use_mode("tile")
    assert sha(got) == demo["reference_tga_sha256"]


def test_encode_rejects_bad_arguments():
    fn = native.load().cy_encode_image
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                   ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]
    assert fn(None, 1, 0, 0, 4, 4, None, 0, None) == -1


CASES = [("c0_small", 0, (0, 0, None, None)), ("mixed_small", 1, (-7, 5, 61, 40)), ("c2_small", 2, (30, -3, 17, 90))]


@pytest.mark.gpu
@pytest.mark.parametrize("fmt", [native.TGA, native.PNG], ids=["tga", "png"])
@pytest.mark.parametrize("config,seed,rect", CASES)
def test_encode_matches_reference_writers(fmt, config, seed, rect):
    tb = scenes.small_scene(config, seed)
    W, H = T.canvas_size(tb)
    x, y, w, h = rect
    w = w or W
    h = h or H
    got = native.encode_image(tb, fmt, x, y, w, h)
    # the same pixels through get_image_data, appended before the list's end
    rgba = native.replay(_append_read(tb, w, h, x, y))[0][-w * h * 4:]
    want = ref_png(rgba, w, h) if fmt == native.PNG else ref_tga(rgba, w, h)
    assert got == want


def _append_read(tb: bytes, w: int, h: int, x: int, y: int) -> bytes:
    """The call list with one more get_image_data(w, h, x, y) before its
    END record (the last 4 bytes)."""
    assert struct.unpack("<i", tb[-4:])[0] == T.END
    return tb[:-4] + struct.pack("<i6i", T.GET_IMAGE_DATA, w, h, x, y, 1, 0) + tb[-4:]


@pytest.mark.gpu
def test_encode_blank_canvas():
    t = T.TraceWriter(9, 4)
    tb = t.finish(read_back=False)
    got = native.encode_image(tb, native.PNG, 0, 0, 9, 4)
    assert got == ref_png(bytes(9 * 4 * 4), 9, 4)
