"""Host utilities that need no GPU: PPM and PNG output and the frame driver's
keyboard state (callbacksPBO.cpp:104-143)."""
import numpy as np
import pytest

import photonmap


def test_write_ppm(tmp_path):
    rs = np.random.RandomState(0)
    img = rs.randint(0, 256, size=(7, 5, 4)).astype(np.uint8)
    p = str(tmp_path / "f.ppm")
    photonmap.write_ppm(p, img)
    data = open(p, "rb").read()
    header = b"P6\n5 7\n255\n"
    assert data.startswith(header)
    body = np.frombuffer(data[len(header):], np.uint8).reshape(7, 5, 3)
    np.testing.assert_array_equal(body, img[..., :3])


@pytest.mark.parametrize("h,w", [(7, 5), (1, 1), (300, 257)])
def test_write_png_decodes_to_the_pixels(tmp_path, h, w):
    """An independent decoder (zlib + the PNG chunk rules) reads the file
    back to the image's RGB bytes; every chunk's CRC checks out. 300 x 257
    pixels span two stored deflate blocks."""
    import struct
    import zlib
    rs = np.random.RandomState(h * w)
    img = rs.randint(0, 256, size=(h, w, 4)).astype(np.uint8)
    p = str(tmp_path / "f.png")
    photonmap.write_png(p, img)
    data = open(p, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    at, chunks = 8, []
    while at < len(data):
        n, = struct.unpack(">I", data[at:at + 4])
        kind, body = data[at + 4:at + 8], data[at + 8:at + 8 + n]
        crc, = struct.unpack(">I", data[at + 8 + n:at + 12 + n])
        assert zlib.crc32(kind + body) & 0xffffffff == crc
        chunks.append((kind, body))
        at += 12 + n
    assert [c[0] for c in chunks] == [b"IHDR", b"IDAT", b"IEND"]
    assert struct.unpack(">IIBBBBB", chunks[0][1]) == (w, h, 8, 2, 0, 0, 0)
    raw = np.frombuffer(zlib.decompress(chunks[1][1]), np.uint8).reshape(h, 1 + 3 * w)
    assert (raw[:, 0] == 0).all()
    np.testing.assert_array_equal(raw[:, 1:].reshape(h, w, 3), img[..., :3])


def test_viewer_keys_follow_the_reference():
    v = photonmap.Viewer(64, 48)
    s = v.state()
    assert (s.anim_flag, s.emit_flag, s.interpolate, s.media, s.iter) == (0, 1, 0, 0, 0)
    assert s.anim_inc == np.float32(0.1) and s.anim_time == 0.0
    for k in "aeipAEIP":
        v.key(k)
    s = v.state()
    assert (s.anim_flag, s.emit_flag, s.interpolate, s.media) == (0, 1, 0, 0)
    v.key("i")
    v.key("p")
    v.key("a")
    s = v.state()
    assert (s.anim_flag, s.interpolate, s.media) == (1, 1, 1)
    # animInc -= 0.01 on a float with a double literal (callbacksPBO.cpp:134)
    v.key("-")
    assert v.state().anim_inc == np.float32(np.float64(np.float32(0.1)) - 0.01)
    v.key("+")
    v.key("+")
    expect = np.float32(np.float64(np.float32(np.float64(np.float32(np.float64(np.float32(0.1)) - 0.01)) + 0.01)) + 0.01)
    assert v.state().anim_inc == expect
    v.key("r")
    assert v.state().anim_inc == np.float32(0.01)
    v.key(27)
    assert v.state().quit == 1
    v.close()
