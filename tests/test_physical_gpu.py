"""Physically based mode on the GPU against the single-precision CPU oracle
(bit for bit) and the double-precision oracle (relative RMSE), through the
C ABI."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
import photonmap  # noqa: E402
import oracle  # noqa: E402

pytestmark = pytest.mark.gpu


def small(preset, surface=20000, volume=20000, size=(48, 40), k=None, radius=None, seed=0x5EED0001):
    sc, cf = photonmap.preset(preset, seed)
    cf.surface_photons, cf.volume_photons = surface, volume
    cf.width, cf.height = size
    if k is not None:
        cf.k = k
    if radius is not None:
        cf.radius = radius
    return sc, cf


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


@pytest.fixture
def ctx():
    c = photonmap.Context(0)
    yield c
    c.close()


def gpu_frame(ctx, sc, cf):
    ctx.set_scene(sc, cf)
    ctx.emit()
    ctx.build()
    rad = torch.zeros((cf.height * cf.width, 4), dtype=torch.float32, device="cuda")
    rgba = torch.zeros((cf.height * cf.width, 4), dtype=torch.uint8, device="cuda")
    ctx.render(rad.data_ptr(), rgba.data_ptr())
    torch.cuda.synchronize()
    return rad.cpu().numpy(), rgba.cpu().numpy()


@pytest.mark.parametrize("preset", [1, 2, 3])
def test_emission_bit_exact(ctx, preset):
    sc, cf = small(preset, 30000, 30000)
    ctx.set_scene(sc, cf)
    ctx.emit()
    het = oracle.noise_grid(sc, cf)
    m = oracle.emit(sc, cf, het)
    st = ctx.stats()
    assert list(st.map_size) == list(m.sizes)
    assert list(st.map_paths) == list(m.paths)
    for mid, (op, ow) in enumerate([(m.spos, m.spow), (m.vpos, m.vpow)]):
        pos, pw = ctx.photons_soa(mid)
        np.testing.assert_array_equal(bits(pos), bits(op))
        np.testing.assert_array_equal(bits(pw), bits(ow))


def test_emission_close_to_float64(ctx):
    sc, cf = small(2, 30000, 30000)
    ctx.set_scene(sc, cf)
    ctx.emit()
    m64 = oracle.emit(sc, cf, None, double=True)
    pos, pw = ctx.photons_soa(0)
    assert len(pos) == len(m64.spos)
    rel = np.abs(pos[:, :3] - m64.spos[:, :3]) / np.maximum(np.abs(m64.spos[:, :3]), 1e-3)
    # Paths that take a different branch in float32 (a grazing hit or a
    # threshold draw) diverge; all others agree to 1e-5 relative.
    ok = (rel < 1e-5).all(axis=1)
    assert ok.mean() > 0.97, ok.mean()
    prel = np.abs(pw[:, :3] - m64.spow[:, :3]) / np.abs(m64.spow[:, :3])
    assert np.median(prel) < 1e-5


@pytest.mark.parametrize("k,radius", [(1, 0.05), (17, 0.08), (32, 0.1), (64, 0.1), (100, 0.05),
                                      (128, 0.2)])
def test_knn_bit_exact(ctx, k, radius):
    sc, cf = small(1, 40000, 10000)
    ctx.set_scene(sc, cf)
    ctx.emit()
    ctx.build()
    rs = np.random.RandomState(k)
    q = np.zeros((3000, 4), np.float32)
    q[:, 0] = rs.uniform(-0.55, 0.55, 3000)
    q[:, 1] = rs.uniform(-0.05, 1.05, 3000)
    q[:, 2] = rs.uniform(-0.55, 0.55, 3000)
    for mid in (0, 1):
        pos, _ = ctx.photons_soa(mid)
        qd = torch.from_numpy(q).cuda()
        idx = torch.zeros((3000, k), dtype=torch.int32, device="cuda")
        d2 = torch.zeros((3000, k), dtype=torch.float32, device="cuda")
        ctx.knn(mid, qd.data_ptr(), 3000, k, radius, idx.data_ptr(), d2.data_ptr())
        torch.cuda.synchronize()
        oi, od = oracle.knn(pos, q, k, radius)
        np.testing.assert_array_equal(idx.cpu().numpy().view(np.uint32), oi)
        np.testing.assert_array_equal(bits(d2.cpu().numpy()), bits(od))


def test_knn_ties_broken_by_index(ctx):
    # A lattice with every point repeated three times: many neighbours at
    # exactly equal distance; the answer must follow the photon index.
    sc, cf = small(1, 1000, 1000)
    ctx.set_scene(sc, cf)
    g = np.stack(np.meshgrid(np.arange(-0.5, 0.51, 0.05), np.arange(0.0, 1.01, 0.05),
                             np.arange(-0.5, 0.51, 0.05), indexing="ij"), -1).reshape(-1, 3)
    g = np.repeat(g, 3, axis=0).astype(np.float32)
    rs = np.random.RandomState(3)
    perm = rs.permutation(len(g))
    pos = np.zeros((len(g), 4), np.float32)
    pos[:, :3] = g[perm]
    pos[:, 3] = np.arange(len(g), dtype=np.uint32).view(np.float32)  # record index bits
    pw = np.ones((len(g), 4), np.float32)
    ctx.set_photons(0, pos, pw)
    ctx.build()
    q = np.zeros((500, 4), np.float32)
    q[:, :3] = g[rs.randint(0, len(g), 500)]
    q[250:, 0] += 0.025  # midway between lattice planes: equal distances to both
    for k in (7, 27, 64, 128):
        qd = torch.from_numpy(q).cuda()
        idx = torch.zeros((500, k), dtype=torch.int32, device="cuda")
        d2 = torch.zeros((500, k), dtype=torch.float32, device="cuda")
        ctx.knn(0, qd.data_ptr(), 500, k, 0.12, idx.data_ptr(), d2.data_ptr())
        torch.cuda.synchronize()
        oi, od = oracle.knn(pos, q, k, 0.12)
        np.testing.assert_array_equal(idx.cpu().numpy().view(np.uint32), oi)
        np.testing.assert_array_equal(bits(d2.cpu().numpy()), bits(od))


def test_knn_empty_and_tiny_maps(ctx):
    sc, cf = small(1, 1000, 1000)
    ctx.set_scene(sc, cf)
    q = torch.zeros((4, 4), dtype=torch.float32, device="cuda")
    idx = torch.zeros((4, 8), dtype=torch.int32, device="cuda")
    d2 = torch.zeros((4, 8), dtype=torch.float32, device="cuda")
    for n in (0, 1, 5, 33):
        pos = np.zeros((n, 4), np.float32)
        pos[:, 0] = np.linspace(-0.1, 0.1, n)
        pos[:, 3] = np.arange(n, dtype=np.uint32).view(np.float32)
        ctx.set_photons(1, pos, np.ones((n, 4), np.float32))
        ctx.build()
        ctx.knn(1, q.data_ptr(), 4, 8, 0.5, idx.data_ptr(), d2.data_ptr())
        torch.cuda.synchronize()
        oi, od = oracle.knn(pos, np.zeros((4, 4), np.float32), 8, 0.5)
        np.testing.assert_array_equal(idx.cpu().numpy().view(np.uint32), oi)
        np.testing.assert_array_equal(bits(d2.cpu().numpy()), bits(od))


@pytest.mark.parametrize("preset,size", [(1, (48, 40)), (2, (40, 40)), (3, (64, 36))])
def test_render_bit_exact(ctx, preset, size):
    sc, cf = small(preset, 20000, 20000, size)
    rad, rgba = gpu_frame(ctx, sc, cf)
    het = oracle.noise_grid(sc, cf)
    m = oracle.emit(sc, cf, het)
    orad = oracle.render(sc, cf, het, m)
    np.testing.assert_array_equal(bits(rad), bits(orad))
    assert rad[:, :3].max() > 0.0
    st = ctx.stats()
    assert st.surface_gathers > 0 and st.volume_gathers > 0


@pytest.mark.parametrize("preset,size,k,radius,photons", [
    (1, (48, 40), None, None, 20000), (2, (64, 48), None, None, 20000),
    (3, (64, 36), None, None, 20000), (2, (40, 30), 1, None, 20000), (3, (40, 30), 64, None, 20000),
    (2, (48, 40), 100, 0.02, 20000),   # the radius cap binds: fewer than k found
    (2, (40, 30), 32, None, 300),      # tiny maps
    (2, (96, 72), 100, None, 60000)])
def test_query_list_render_equals_single_kernel(ctx, preset, size, k, radius, photons):
    """pm_render (query list in spatial order, shared candidate sets) and
    pm_render_single_kernel (warp-per-pixel march with the list search)
    give the same bits, the same 8-bit image and the same gather counts."""
    sc, cf = small(preset, photons, photons, size, k=k, radius=radius)
    rad, rgba = gpu_frame(ctx, sc, cf)
    st = ctx.stats()
    rad1 = torch.zeros_like(torch.from_numpy(rad)).cuda()
    rgba1 = torch.zeros_like(torch.from_numpy(rgba)).cuda()
    ctx.render_single_kernel(rad1.data_ptr(), rgba1.data_ptr())
    torch.cuda.synchronize()
    np.testing.assert_array_equal(bits(rad1.cpu().numpy()), bits(rad))
    np.testing.assert_array_equal(rgba1.cpu().numpy(), rgba)
    st1 = ctx.stats()
    assert (st1.surface_gathers, st1.volume_gathers) == (st.surface_gathers, st.volume_gathers)
    assert st.surface_gathers > 0


def test_render_with_massive_distance_ties(ctx):
    """Maps whose records sit on a lattice, every point 40 times: the k-th
    distance of most queries is shared by dozens of records, so the
    shared-candidate selection has to rank more than 32 records at one
    distance by photon index. The image equals the single-kernel render's."""
    sc, cf = small(1, 1000, 1000, (40, 32), k=64, radius=0.1)
    ctx.set_scene(sc, cf)
    g = np.stack(np.meshgrid(np.arange(-0.5, 0.51, 0.1), np.arange(0.0, 1.01, 0.1),
                             np.arange(-0.5, 0.51, 0.1), indexing="ij"), -1).reshape(-1, 3)
    g = np.repeat(g, 40, axis=0).astype(np.float32)
    rs = np.random.RandomState(11)
    for mid in (0, 1):
        perm = rs.permutation(len(g))
        pos = np.zeros((len(g), 4), np.float32)
        pos[:, :3] = g[perm]
        pos[:, 3] = np.arange(len(g), dtype=np.uint32).view(np.float32)
        pw = np.zeros((len(g), 4), np.float32)
        pw[:, :3] = rs.uniform(1e-4, 1e-3, (len(g), 3))
        pw[:, 3] = rs.randint(0, 2**32, len(g), dtype=np.uint64).astype(np.uint32).view(np.float32)
        ctx.set_photons(mid, pos, pw)
    ctx.build()
    n = cf.width * cf.height
    rad = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
    rad1 = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
    ctx.render(rad.data_ptr(), None)
    ctx.render_single_kernel(rad1.data_ptr(), None)
    torch.cuda.synchronize()
    a, b = rad.cpu().numpy(), rad1.cpu().numpy()
    np.testing.assert_array_equal(bits(a), bits(b))
    assert a[:, :3].max() > 0.0


def test_gather_stats_of_the_shared_candidate_sets(ctx):
    """The k-NN estimates of a frame mostly come from shared candidate
    sets, and no result contradicts its distance bound."""
    sc, cf = small(2, 100000, 100000, (128, 96))
    gpu_frame(ctx, sc, cf)
    g = ctx.gather_stats()
    st = ctx.stats()
    assert g["tiled"] + g["list"] == st.surface_gathers + st.volume_gathers
    assert g["violations"] == 0
    assert g["tiled"] > 0.9 * (g["tiled"] + g["list"]), g
    assert g["groups"] > 0 and g["candidates"] >= 50 * g["groups"]


def test_render_against_float64(ctx):
    sc, cf = small(2, 30000, 30000, (40, 40))
    rad, _ = gpu_frame(ctx, sc, cf)
    m64 = oracle.emit(sc, cf, None, double=True)
    r64 = oracle.render(sc, cf, None, m64, double=True)
    err = np.sqrt(np.mean((rad[:, :3] - r64[:, :3]) ** 2)) / np.sqrt(np.mean(r64[:, :3] ** 2))
    # tolerance: float32 trajectories and neighbour sets vs float64 ones
    assert err < 2e-2, err


def test_emit_build_render_repeatable(ctx):
    sc, cf = small(1, 20000, 20000, (32, 32))
    a, _ = gpu_frame(ctx, sc, cf)
    ctx.emit()
    ctx.build()
    rad = torch.zeros((32 * 32, 4), dtype=torch.float32, device="cuda")
    ctx.render(rad.data_ptr(), None)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(bits(rad.cpu().numpy()), bits(a))


def test_record_layout_export(ctx):
    sc, cf = small(1, 5000, 5000)
    ctx.set_scene(sc, cf)
    ctx.emit()
    rec = ctx.photon_records(0)
    pos, pw = ctx.photons_soa(0)
    np.testing.assert_array_equal(rec[:, 0:3], pos[:, :3])
    np.testing.assert_array_equal(rec[:, 6:9], pw[:, :3])
    nrm = np.linalg.norm(rec[:, 3:6], axis=1)
    np.testing.assert_allclose(nrm, 1.0, atol=1e-5)


def test_state_errors(ctx):
    lib = photonmap.load()
    assert lib.pm_emit(ctx.h, None) == 4
    sc, cf = small(1, 1000, 1000)
    ctx.set_scene(sc, cf)
    assert lib.pm_render(ctx.h, None, None, None) == 4
    cf.k = 0
    with pytest.raises(photonmap.PMError):
        ctx.set_scene(sc, cf)


def test_radius_gather_matches_reference_weighting(ctx):
    # kernelPBO.cu:165-182 weighting over the surface map; float32 sums in
    # tree order against float64 sums in index order: 1e-4 relative.
    sc, cf = small(1, 20000, 1000)
    ctx.set_scene(sc, cf)
    ctx.emit()
    ctx.build()
    pos, pw = ctx.photons_soa(0)
    rs = np.random.RandomState(9)
    nq = 600
    pts = np.zeros((nq, 4), np.float32)
    nrm = np.zeros((nq, 4), np.float32)
    pts[:, 0] = rs.uniform(-0.5, 0.5, nq)
    pts[:, 2] = rs.uniform(-0.5, 0.5, nq)
    pts[:300, 1] = 0.0          # on the floor, facing up
    nrm[:300, 1] = 1.0
    pts[300:, 1] = rs.uniform(0.0, 1.0, 300)
    v = rs.standard_normal((300, 3)).astype(np.float32)
    nrm[300:, :3] = v / np.linalg.norm(v, axis=1, keepdims=True)
    for sq, expo in [(0.01, 50.0), (0.0025, 1.0)]:
        pd, nd = torch.from_numpy(pts).cuda(), torch.from_numpy(nrm).cuda()
        out = torch.zeros((nq, 4), dtype=torch.float32, device="cuda")
        ctx.radius_gather(0, pd.data_ptr(), nd.data_ptr(), nq, sq, expo, out.data_ptr())
        torch.cuda.synchronize()
        got = out.cpu().numpy()[:, :3].astype(np.float64)
        ref = oracle.radius_gather(pos, pw, pts, nrm, sq, expo)
        scale = np.abs(ref).max()
        assert scale > 0
        np.testing.assert_allclose(got, ref, rtol=1e-4, atol=1e-6 * scale)


@pytest.mark.parametrize("leaf", [64, 128])
def test_leaf_size_does_not_change_the_render(ctx, leaf):
    sc, cf = small(2, 30000, 30000, (40, 32))
    a, _ = gpu_frame(ctx, sc, cf)
    cf.leaf_size = leaf
    b, _ = gpu_frame(ctx, sc, cf)
    np.testing.assert_array_equal(bits(b), bits(a))
