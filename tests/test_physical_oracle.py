"""Known-answer tests of the physically based CPU oracle (no GPU): the
deterministic math, Philox, the samplers against their analytic
distributions, energy bookkeeping in a closed box, point-light irradiance,
free-flight distances, and exact k-NN against numpy brute force."""
import ctypes
import math

import numpy as np
import pytest

import oracle
import photonmap


# ---- deterministic math (include/pm_math.h) --------------------------------

def ulp_err(got, ref):
    got = np.asarray(got, np.float64)
    ulp = np.spacing(np.abs(ref).astype(np.float32)).astype(np.float64)
    return np.abs(got - ref) / ulp


def test_logf_within_few_ulp():
    lib = oracle.phys_lib()
    rs = np.random.RandomState(0)
    x = np.concatenate([rs.randint(1, 1 << 24, 20000) / float(1 << 24),
                        np.geomspace(6e-8, 1.0, 2000)]).astype(np.float32)
    got = np.array([lib.pmo_logf(float(v)) for v in x])
    ref = np.log(x.astype(np.float64))
    err = np.abs(got - ref) / np.maximum(np.abs(ref), 1e-30)
    big = np.abs(ref) > 1e-3
    assert ulp_err(got[big], ref[big]).max() <= 4
    assert np.abs(got[~big] - ref[~big]).max() < 3e-10 + 0 * err.max()


def test_expf_within_few_ulp():
    lib = oracle.phys_lib()
    x = np.linspace(-87.0, 0.0, 20001).astype(np.float32)
    got = np.array([lib.pmo_expf(float(v)) for v in x])
    ref = np.exp(x.astype(np.float64))
    assert ulp_err(got, ref).max() <= 4


def test_sincos2pi_accuracy():
    lib = oracle.phys_lib()
    u = (np.arange(0, 1 << 24, 997) / float(1 << 24)).astype(np.float32)
    s = ctypes.c_float()
    c = ctypes.c_float()
    gs, gc = [], []
    for v in u:
        lib.pmo_sincos2pi(float(v), ctypes.byref(s), ctypes.byref(c))
        gs.append(s.value)
        gc.append(c.value)
    ang = 2.0 * math.pi * u.astype(np.float64)
    assert np.abs(np.array(gs) - np.sin(ang)).max() < 2.5e-7
    assert np.abs(np.array(gc) - np.cos(ang)).max() < 2.5e-7


def philox_py(ctr, key):
    """Philox4x32-10 restated in Python from Salmon et al. (SC 2011)."""
    c = list(ctr)
    k0, k1 = key
    for _ in range(10):
        p0 = 0xD2511F53 * c[0]
        p1 = 0xCD9E8D57 * c[2]
        hi0, lo0 = p0 >> 32, p0 & 0xFFFFFFFF
        hi1, lo1 = p1 >> 32, p1 & 0xFFFFFFFF
        c = [hi1 ^ c[1] ^ k0, lo1, hi0 ^ c[3] ^ k1, lo0]
        k0 = (k0 + 0x9E3779B9) & 0xFFFFFFFF
        k1 = (k1 + 0xBB67AE85) & 0xFFFFFFFF
    return c


def test_philox_matches_triton_philox():
    """The generator the GPU kernels and the oracle share, against another
    project's Philox4x32-10: Triton's philox_impl run in its CPU interpreter
    on the all-zero and all-ones patterns and 256 random counters and keys
    (tests/golden/make_philox_golden.py wrote the vectors)."""
    import os
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "philox_triton.npz"))
    lib = oracle.phys_lib()
    out = np.zeros(4, np.uint32)
    assert len(d["ctr"]) == 258
    for ctr, key, want in zip(d["ctr"], d["key"], d["out"]):
        ctr = np.ascontiguousarray(ctr, np.uint32)
        seed = int(key[0]) | (int(key[1]) << 32)
        lib.pmo_philox(seed, ctr.ctypes.data, out.ctypes.data)
        assert [int(v) for v in out] == [int(v) for v in want], (ctr, key)
        assert philox_py([int(v) for v in ctr], (int(key[0]), int(key[1]))) == [int(v) for v in want]


def test_philox_matches_independent_restatement():
    # The C implementation (shared by GPU and oracle) against a separate
    # Python restatement on more inputs than the Triton vectors hold.
    lib = oracle.phys_lib()
    rs = np.random.RandomState(1)
    out = np.zeros(4, np.uint32)
    for _ in range(500):
        ctr = rs.randint(0, 2 ** 32, 4, dtype=np.uint64).astype(np.uint32)
        seed = int(rs.randint(0, 2 ** 63, dtype=np.int64))
        lib.pmo_philox(seed, ctr.ctypes.data, out.ctypes.data)
        ref = philox_py([int(v) for v in ctr], (seed & 0xFFFFFFFF, seed >> 32))
        assert [int(v) for v in out] == ref


def test_philox_uniformity():
    lib = oracle.phys_lib()
    out = np.zeros(4, np.uint32)
    vals = []
    for i in range(50000):
        ctr = np.array([i, 7, 0, 3], np.uint32)
        lib.pmo_philox(0x5EED, ctr.ctypes.data, out.ctypes.data)
        vals.extend(out.tolist())
    u = np.array(vals, np.float64) / 2 ** 32
    h, _ = np.histogram(u, bins=64, range=(0, 1))
    e = len(u) / 64.0
    chi2 = ((h - e) ** 2 / e).sum()
    assert chi2 < 120  # 63 dof; p ~ 1e-5 threshold


# ---- samplers -----------------------------------------------------------------

def chi2_hist(samples, pdf, lo, hi, bins=40, cdf=None):
    h, edges = np.histogram(samples, bins=bins, range=(lo, hi))
    if cdf is not None:
        e = np.diff(cdf(edges)) * len(samples)
    else:
        mids = 0.5 * (edges[1:] + edges[:-1])
        e = pdf(mids) * (edges[1] - edges[0]) * len(samples)
    keep = e > 5
    return (((h[keep] - e[keep]) ** 2) / e[keep]).sum()


def test_uniform_sphere_distribution():
    d = oracle.sample(0, 40000)
    np.testing.assert_allclose(np.linalg.norm(d, axis=1), 1.0, atol=2e-6)
    assert chi2_hist(d[:, 2], lambda z: 0.5 * np.ones_like(z), -1, 1) < 80


def test_cosine_hemisphere_distribution():
    n = np.array([0.3, -0.5, 0.8], np.float32)
    n /= np.linalg.norm(n)
    d = oracle.sample(1, 40000, direction=n)
    mu = d @ n
    assert (mu >= -1e-6).all()
    assert chi2_hist(mu, lambda m: 2 * m, 0, 1) < 80


@pytest.mark.parametrize("g", [0.0, 0.3, -0.6, 0.9])
def test_henyey_greenstein_distribution(g):
    n = np.array([0.0, 0.6, -0.8], np.float32)
    d = oracle.sample(2, 40000, g=g, direction=n)
    mu = np.clip(d @ n, -1, 1)
    if g == 0.0:
        cdf = lambda m: (m + 1) / 2  # noqa: E731
    else:
        cdf = lambda m: (1 - g * g) / (2 * g) * (1 / np.sqrt(1 + g * g - 2 * g * m) - 1 / (1 + g))  # noqa: E731,E501
    assert chi2_hist(mu, None, -1, 1, cdf=cdf) < 80
    lib = oracle.phys_lib()
    # phase function integrates to 1 over the sphere
    m = np.linspace(-1, 1, 20001)
    ph = np.array([lib.pmo_hg_phase(g, float(x)) for x in m])
    integral = np.trapezoid(ph, m) * 2 * math.pi
    assert abs(integral - 1.0) < 2e-3


def test_fresnel_limits():
    lib = oracle.phys_lib()
    # normal incidence, n = 1.5: ((1 - 1.5) / (1 + 1.5))^2 = 0.04
    assert abs(lib.pmo_fresnel(1.0, 1.0 / 1.5) - 0.04) < 1e-6
    # total internal reflection from inside glass beyond the critical angle
    assert lib.pmo_fresnel(0.3, 1.5) == 1.0
    # grazing incidence reflects almost everything
    assert lib.pmo_fresnel(1e-4, 1.0 / 1.5) > 0.99


# ---- emission known answers ----------------------------------------------------

def box_scene(closed=True, albedo=0.5, sigma_s=0.0, sigma_a=0.0):
    sc, cf = photonmap.preset(1, 1)
    sc.num_spheres = 0
    sc.sigma_s, sc.sigma_a = sigma_s, sigma_a
    for i in range(5):
        sc.plane_mat[i].kind = photonmap.MAT_DIFFUSE
        for c in range(3):
            sc.plane_mat[i].albedo[c] = albedo
    if closed:
        sc.num_planes = 6
        sc.planes[5][0], sc.planes[5][1] = 2.0, -0.5
        sc.plane_mat[5].kind = photonmap.MAT_DIFFUSE
        for c in range(3):
            sc.plane_mat[5].albedo[c] = albedo
    return sc, cf


def test_furnace_without_roulette_is_exact():
    # Closed box, no medium, survival 1: every path stores exactly B records
    # of power a^b / N, so the map's total power is sum_b a^b.
    a, B = 0.5, 5
    sc, cf = box_scene(albedo=a)
    cf.max_bounces, cf.rr_survival = B, 1.0
    cf.surface_photons, cf.volume_photons = 20000 * B, 0
    m = oracle.emit(sc, cf)
    # a path can slip out through a box edge between two walls when rounding
    # puts its hit just outside both rectangles; that is rare
    assert 20000 <= m.paths[0] <= 20020
    total = m.spow[:, :3].astype(np.float64).sum(axis=0)
    expect = sum(a ** b for b in range(B))
    np.testing.assert_allclose(total, expect, rtol=2e-3)


def test_furnace_with_roulette_is_unbiased():
    a, B = 0.6, 8
    sc, cf = box_scene(albedo=a)
    cf.max_bounces, cf.rr_survival = B, 0.8
    cf.surface_photons, cf.volume_photons = 200000, 0
    m = oracle.emit(sc, cf)
    total = m.spow[:, 0].astype(np.float64).sum()
    expect = sum(a ** b for b in range(B))
    # per-path totals have std < expect; 5 standard errors
    assert abs(total - expect) < 5 * expect / math.sqrt(m.paths[0])


def test_point_light_irradiance_on_floor():
    # Only the floor: the first hits inside a disc of radius R below the
    # light take the solid-angle fraction (1 - h / sqrt(h^2 + R^2)) / 2.
    sc, cf = box_scene(closed=False)
    sc.num_planes = 1
    sc.planes[0][0], sc.planes[0][1] = 1.0, 0.0
    for a in (0, 2):
        sc.box_min[a], sc.box_max[a] = -50.0, 50.0
    cf.max_bounces, cf.rr_survival = 1, 1.0
    cf.surface_photons, cf.volume_photons = 200000, 0
    cf.max_paths = 400000
    m = oracle.emit(sc, cf)
    h, R = 0.95, 0.5
    n_paths = m.paths[0]
    r = np.hypot(m.spos[:, 0], m.spos[:, 2])
    frac = (r < R).sum() / float(n_paths)
    expect = (1 - h / math.hypot(h, R)) / 2
    assert abs(frac - expect) < 5 * math.sqrt(expect * (1 - expect) / n_paths)


def test_free_flight_distances_are_exponential():
    # Homogeneous medium, no surfaces inside a huge box: a photon's first
    # record is its first collision, at distance ~ Exp(sigma_t).
    sc, cf = box_scene(closed=False, sigma_s=2.0, sigma_a=0.5)
    sc.num_planes = 0
    for a in range(3):
        sc.box_min[a], sc.box_max[a] = -100.0, 100.0
    cf.max_bounces, cf.rr_survival = 1, 1.0
    cf.surface_photons, cf.volume_photons = 0, 50000
    m = oracle.emit(sc, cf)
    light = np.array(sc.light[:], np.float64)
    d = np.linalg.norm(m.vpos[:, :3] - light, axis=1)
    st = 2.5
    assert abs(d.mean() - 1 / st) < 5 * (1 / st) / math.sqrt(len(d))
    assert chi2_hist(d, lambda x: st * np.exp(-st * x), 0, 3.0 / st) < 80


def test_float32_and_float64_emission_agree():
    sc, cf = photonmap.preset(2, 7)
    cf.surface_photons = cf.volume_photons = 5000
    m = oracle.emit(sc, cf)
    m64 = oracle.emit(sc, cf, double=True)
    assert list(m.sizes) == list(m64.sizes)
    same = (np.abs(m.spos[:, :3] - m64.spos[:, :3]) < 1e-4).all(axis=1)
    assert same.mean() > 0.97


# ---- k-NN ------------------------------------------------------------------

def brute_knn(pos, q, k, radius):
    r2 = np.float32(radius) * np.float32(radius)
    d = pos[None, :, :3] - q[:, None, :3]
    d2 = (d[..., 0] * d[..., 0] + d[..., 1] * d[..., 1]) + d[..., 2] * d[..., 2]
    idx = pos[:, 3].view(np.uint32)
    out_i = np.full((len(q), k), 0xFFFFFFFF, np.uint32)
    out_d = np.full((len(q), k), r2, np.float32)
    for j in range(len(q)):
        ok = np.nonzero(d2[j] <= r2)[0]
        order = np.lexsort((idx[ok], d2[j][ok]))[:k]
        out_i[j, :len(order)] = idx[ok][order]
        out_d[j, :len(order)] = d2[j][ok][order]
    return out_i, out_d


@pytest.mark.parametrize("ties", [False, True])
def test_oracle_knn_matches_brute_force(ties):
    rs = np.random.RandomState(5)
    if ties:
        g = rs.randint(0, 6, size=(3000, 3)).astype(np.float32) * 0.05
    else:
        g = rs.uniform(0, 0.5, size=(3000, 3)).astype(np.float32)
    pos = np.zeros((3000, 4), np.float32)
    pos[:, :3] = g
    pos[:, 3] = np.arange(3000, dtype=np.uint32).view(np.float32)
    q = np.zeros((200, 4), np.float32)
    q[:, :3] = rs.uniform(-0.05, 0.55, size=(200, 3))
    if ties:
        q[:100, :3] = g[:100] + np.float32(0.025)
    for k, r in [(1, 0.1), (16, 0.08), (64, 0.2), (128, 0.3)]:
        oi, od = oracle.knn(pos, q, k, r)
        bi, bd = brute_knn(pos, q, k, r)
        np.testing.assert_array_equal(oi, bi)
        np.testing.assert_array_equal(od.view(np.uint32), bd.view(np.uint32))
        # the CPU kd-tree (the benchmark's CPU gather) finds the same sets
        ki, kd = oracle.knn_kd(pos, q, k, r)
        np.testing.assert_array_equal(ki, bi)
        np.testing.assert_array_equal(kd.view(np.uint32), bd.view(np.uint32))


@pytest.mark.parametrize("n", [0, 1, 16, 17, 1000, 60000])
def test_kdtree_knn_equals_grid_knn(n):
    """Leaf-sized, just-above-leaf and large maps, a fifth of the points on a
    lattice (exact distance ties), queries inside and outside the box."""
    rs = np.random.RandomState(n + 3)
    pos = np.zeros((n, 4), np.float32)
    pos[:, :3] = rs.uniform(0.0, 1.0, (n, 3))
    pos[: n // 5, :3] = np.round(pos[: n // 5, :3] * 10) / 10
    pos[:, 3] = np.arange(n, dtype=np.uint32).view(np.float32)
    q = np.zeros((2000, 4), np.float32)
    q[:, :3] = rs.uniform(-0.1, 1.1, (2000, 3))
    q[:200, :3] = np.round(q[:200, :3] * 10) / 10
    for k, r in [(1, 0.05), (64, 0.1), (128, 0.2)]:
        gi, gd = oracle.knn(pos, q, k, r)
        ki, kd = oracle.knn_kd(pos, q, k, r)
        np.testing.assert_array_equal(ki, gi)
        np.testing.assert_array_equal(kd.view(np.uint32), gd.view(np.uint32))


def test_render_is_the_same_with_either_neighbour_index():
    """pmo_render through kd-trees (the default) and through grids: the
    same k-NN sets, so the same bits."""
    sc, cf = oracle.preset(2, 0x5EED0002)
    cf.surface_photons = cf.volume_photons = 20000
    cf.width, cf.height = 40, 30
    maps = oracle.emit(sc, cf, None)
    try:
        oracle.set_gather_index("grid")
        a = oracle.render(sc, cf, None, maps)
    finally:
        oracle.set_gather_index("kdtree")
    b = oracle.render(sc, cf, None, maps)
    np.testing.assert_array_equal(a.view(np.uint32), b.view(np.uint32))


# ---- presets (host only) -------------------------------------------------------

@pytest.mark.parametrize("which,ns", [(1, 2), (2, 8), (3, 64)])
def test_presets(which, ns):
    sc, cf = photonmap.preset(which, 0x5EED0000 + which)
    assert sc.num_spheres == ns and sc.num_planes == 5
    light = np.array(sc.light[:])
    kinds = [sc.sphere_mat[i].kind for i in range(ns)]
    for i in range(ns):
        c = np.array(sc.spheres[i][:3])
        rad = sc.spheres[i][3]
        assert np.linalg.norm(c - light) > rad
        assert (c - rad >= np.array(sc.box_min[:]) - 1e-6).all()
        assert (c + rad <= np.array(sc.box_max[:]) + 1e-6).all()
    if which >= 2:
        assert kinds.count(photonmap.MAT_DIFFUSE) >= 1
    again = photonmap.preset(which, 0x5EED0000 + which)[0]
    assert bytes(again) == bytes(sc)


@pytest.mark.parametrize("which", [1, 2, 3])
def test_oracle_presets_equal_the_library_presets(which):
    """The oracle's restatement of the scene generator (used where the
    product library must not be loaded) writes the same bytes as pm_preset."""
    for seed in (0x5EED0000 + which, 0, 2 ** 64 - 1):
        a, b = oracle.preset(which, seed)
        c, d = photonmap.preset(which, seed)
        assert bytes(a) == bytes(c)
        assert bytes(b) == bytes(d)


def test_fixed_sum_is_order_independent_and_close_to_exact():
    """The estimate sum: any order of the terms gives the same bits, within
    one rounding of the exact sum (here within 1 ulp of the correctly rounded
    float of the exact rational sum)."""
    from fractions import Fraction
    rng = np.random.default_rng(7)
    for trial in range(200):
        n = int(rng.integers(0, 129))
        scale = 10.0 ** rng.uniform(-30, 3)
        t = (rng.exponential(1.0, n) * scale).astype(np.float32)
        if trial % 5 == 0 and n:
            t[rng.integers(0, n, max(1, n // 4))] = 0.0  # back-facing photons
        if trial % 7 == 0 and n:
            t[0] = np.float32(1e-41)  # a subnormal term
        s = oracle.fixed_sum(t)
        for _ in range(3):
            assert oracle.fixed_sum(rng.permutation(t)).view(np.uint32) == s.view(np.uint32)
        exact = sum((Fraction(float(x)) for x in t), Fraction(0))
        ref = np.float32(float(exact))
        if ref == 0:
            assert s == 0
        else:
            assert abs(int(s.view(np.int32)) - int(ref.view(np.int32))) <= 1, (trial, s, ref)
    assert oracle.fixed_sum(np.zeros(0, np.float32)) == 0.0
    assert oracle.fixed_sum(np.zeros(5, np.float32)) == 0.0
    one = np.ones(100, np.float32)
    assert oracle.fixed_sum(one) == np.float32(100.0)
