"""The radiance-cache oracle (oracle/cache_oracle.py) checked on its own:
bf16 rounding, grid indexing, the spherical-harmonic basis, and its
gradients against central finite differences in float64."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import cache_oracle as co  # noqa: E402


def test_bf16_rounding_ties_to_even():
    one = 1.0
    ulp = 2.0 ** -7
    vals = np.array([one, one + ulp / 2, one + 3 * ulp / 2, -2.5, 3.0e38, 1e-40])
    got = co.bf16(vals)
    assert got[0] == 1.0
    assert got[1] == 1.0                 # halfway, even mantissa kept
    assert got[2] == one + 2 * ulp       # halfway, rounds to even
    assert got[3] == -2.5
    assert np.isfinite(got[4])


def test_dense_levels_index_every_vertex_once():
    r, log2_t = 7, 12                    # 8^3 = 512 vertices <= 4096: dense
    g = np.stack(np.meshgrid(*[np.arange(r + 1) / r] * 3, indexing="ij"), -1).reshape(-1, 3)
    idx, w = co.level_corners(g, r, log2_t)
    assert idx.max() < (r + 1) ** 3 and idx.min() >= 0
    np.testing.assert_allclose(w.sum(1), 1.0, rtol=0, atol=1e-12)


def test_hash_levels_stay_in_the_table():
    rng = np.random.default_rng(1)
    p = rng.random((4096, 3))
    idx, w = co.level_corners(p, 2048, 10)
    assert idx.min() >= 0 and idx.max() < 1024
    np.testing.assert_allclose(w.sum(1), 1.0, atol=1e-12)


def test_spherical_harmonics_are_orthonormal():
    n = 200000
    k = np.arange(n) + 0.5
    z = 1 - 2 * k / n
    phi = np.pi * (1 + 5 ** 0.5) * k
    rr = np.sqrt(1 - z * z)
    d = np.stack([rr * np.cos(phi), rr * np.sin(phi), z], 1)
    Y = co.sh16(d)
    gram = Y.T @ Y * (4 * np.pi / n)
    np.testing.assert_allclose(gram, np.eye(16), atol=2e-3)


def _net(rng, n=9):
    w = rng.uniform(-0.3, 0.3, co.split_weights(np.zeros(4 * 4096 + 1024)).__len__() and 4 * 4096 + 1024)
    x = rng.uniform(-1, 1, (n, 64))
    t = rng.uniform(0, 2, (n, 3))
    return x, w, t


def test_weight_gradients_match_finite_differences():
    rng = np.random.default_rng(2)
    x, w, t = _net(rng)
    base = co.mlp_step(x, w, t, bf16_ops=False)
    y0 = base["y"]
    h = 1e-6
    for j in rng.choice(len(w), 40, replace=False):
        wp, wm = w.copy(), w.copy()
        wp[j] += h
        wm[j] -= h
        fd = (co.loss_fixed_den(x, wp, t, y0) - co.loss_fixed_den(x, wm, t, y0)) / (2 * h)
        assert abs(fd - base["w_grad"][j]) <= 1e-6 * max(1.0, abs(fd)), j


def test_input_gradients_match_finite_differences():
    rng = np.random.default_rng(3)
    x, w, t = _net(rng)
    base = co.mlp_step(x, w, t, bf16_ops=False)
    y0 = base["y"]
    h = 1e-6
    for i, j in zip(rng.integers(0, len(x), 30), rng.integers(0, 64, 30)):
        xp, xm = x.copy(), x.copy()
        xp[i, j] += h
        xm[i, j] -= h
        fd = (co.loss_fixed_den(xp, w, t, y0) - co.loss_fixed_den(xm, w, t, y0)) / (2 * h)
        assert abs(fd - base["dx"][i, j]) <= 1e-6 * max(1.0, abs(fd))


def test_table_gradients_match_finite_differences():
    rng = np.random.default_rng(4)
    res, log2_t = [3, 9], 8
    table = rng.uniform(-1, 1, (2, 1 << log2_t, 2))
    p = rng.random((6, 3))
    w = rng.uniform(-0.3, 0.3, 4 * 4096 + 1024)
    t = rng.uniform(0, 2, (6, 3))
    other = rng.uniform(-1, 1, (6, 64))

    def inputs(tab):
        x = other.copy()
        x[:, :4] = co.encode_hash(p, tab, res, log2_t)
        x[:, 4:32] = 0.0
        return x

    base = co.mlp_step(inputs(table), w, t, bf16_ops=False)
    g = co.table_grad(p, base["dx"], res, log2_t)
    touched = np.argwhere(np.abs(g) > 0)
    h = 1e-6
    for l, e, f in touched[rng.choice(len(touched), 25, replace=False)]:
        tp, tm = table.copy(), table.copy()
        tp[l, e, f] += h
        tm[l, e, f] -= h
        fd = (co.loss_fixed_den(inputs(tp), w, t, base["y"]) -
              co.loss_fixed_den(inputs(tm), w, t, base["y"])) / (2 * h)
        assert abs(fd - g[l, e, f]) <= 1e-6 * max(1.0, abs(fd))


def test_bf16_model_stays_close_to_fp64():
    rng = np.random.default_rng(5)
    x, w, t = _net(rng, n=256)
    a = co.mlp_step(x, w, t, bf16_ops=True)
    b = co.mlp_step(x, w, t, bf16_ops=False)
    rel = np.linalg.norm(a["w_grad"] - b["w_grad"]) / np.linalg.norm(b["w_grad"])
    assert rel < 5e-2
