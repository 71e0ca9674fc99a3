"""Host utilities that need no GPU: PPM output and the frame driver's
keyboard state (callbacksPBO.cpp:104-143)."""
import numpy as np

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
