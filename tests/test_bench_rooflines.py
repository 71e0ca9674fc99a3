"""The bench line's roofline arithmetic (no GPU): the estimate-pass and the
whole-frame byte formulas on a measured preset-3 frame's figures."""
import bench

# one timed preset-3 frame: both 8M-record maps, 1.06 M diffuse and 19.71 M
# volume gathers, 45.5 ms in the estimate pass of a 119.3 ms frame
FRAME = {"map_sizes": [8000000, 8000000], "surf": 1063193.0, "vol": 19706980.0,
         "gather_ms": [45.5], "frame_ms": [119.3]}
PEAK = 6685.5


def test_estimate_pass_roofline():
    r = bench.estimate_roofline(FRAME, 1, 128, PEAK, "measured", 1418367744.0)
    q = 1063193.0 + 19706980.0
    assert r["algorithmic_bytes_per_launch"] == q * (32 * 128 + 52)
    assert abs(r["achieved"] - q * (32 * 128 + 52) / 0.0455 / 1e9) < 1e-6
    assert abs(r["frac"] - r["achieved"] / PEAK) < 1e-12
    assert 0.27 < r["frac"] < 0.30
    assert r["traffic"] == 1418367744.0


def test_frame_roofline():
    r = bench.frame_roofline(FRAME, 1, 128, PEAK, "measured")
    q = 1063193.0 + 19706980.0
    want = 32.0 * 16e6 + 116.0 * 16e6 + q * (32 * 128 + 16)
    assert r["algorithmic_bytes_per_frame"] == want
    assert abs(r["achieved"] - want / 0.1193 / 1e9) < 1e-6
    assert abs(r["frac"] - r["achieved"] / PEAK) < 1e-12
    assert 0.10 < r["frac"] < 0.12
    # two timed frames average their times; the bytes are per frame
    two = dict(FRAME, surf=2 * FRAME["surf"], vol=2 * FRAME["vol"], frame_ms=[119.0, 119.6])
    r2 = bench.frame_roofline(two, 2, 128, PEAK, "measured")
    assert r2["algorithmic_bytes_per_frame"] == want
    assert abs(r2["achieved"] - r["achieved"]) < 1e-6
