"""The C restatement of the reference (oracle/legacy_oracle.c) against
golden vectors produced by the reference's own code
(tests/golden/make_golden.py). Bit-exact: grids, float radiance, images and
generator state are compared by SHA-256 of their bytes."""
import hashlib
import os

import numpy as np
import pytest

from oracle import LegacyOracle

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "legacy_ref.npz"))


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def test_emission_before_random_table():
    # simplePBO.cpp:203 emits once before callbacksPBO.cpp:55 fills the table:
    # every direction is normalize(0) = NaN and nothing lands in the grid.
    o = LegacyOracle()
    o.emit(0.0, 0, 0)
    assert sha(o.grid()) == str(GOLD["pre_init_grid_sha"])
    img, _ = o.render(512, 512, 0.0, 0, 0)
    assert sha(img) == str(GOLD["pre_init_img_sha"])


def test_random_table_matches_reference():
    o = LegacyOracle()
    o.init_random()
    t = o.table()
    np.testing.assert_array_equal(t[:64].view(np.uint32), GOLD["table_head"].view(np.uint32))
    assert sha(t) == str(GOLD["table_sha"])
    np.testing.assert_array_equal(o.rng(), GOLD["rng_after_init"])


def test_frame_sequence_matches_reference():
    o = LegacyOracle()
    o.init_random()
    for i, (t, interp, media, w, h) in enumerate(GOLD["frames"]):
        t, interp, media, w, h = float(t), int(interp), int(media), int(w), int(h)
        o.emit(t, interp, media)
        g = o.grid()
        if "f%d_grid" % i in GOLD:
            np.testing.assert_array_equal(g.view(np.uint32), GOLD["f%d_grid" % i].view(np.uint32))
        assert sha(g) == str(GOLD["f%d_grid_sha" % i]), "grid of frame %d" % i
        img, rgb = o.render(w, h, t, interp, media)
        np.testing.assert_array_equal(img[::8, ::8], GOLD["f%d_img_sub" % i])
        assert sha(img) == str(GOLD["f%d_img_sha" % i]), "image of frame %d" % i
        assert sha(rgb) == str(GOLD["f%d_rgb_sha" % i]), "radiance of frame %d" % i
        np.testing.assert_array_equal(o.rng(), GOLD["f%d_rng" % i])


def test_planted_error_is_detected():
    # A one-ulp change in a single voxel must change the golden digest.
    o = LegacyOracle()
    o.init_random()
    o.emit(0.0, 0, 0)
    g = o.grid()
    g.view(np.uint32)[31, 16, 16, 0] += 1
    assert sha(g) != str(GOLD["f0_grid_sha"])
