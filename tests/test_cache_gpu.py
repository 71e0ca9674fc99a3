"""Learned radiance cache on the GPU, through the C ABI: the query-list
render against pm_render, the encoding and the tensor-core forward/backward
against the FP64 oracle (oracle/cache_oracle.py), training, files."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
import photonmap  # noqa: E402
import cache_oracle as co  # noqa: E402

pytestmark = pytest.mark.gpu


def small(preset, surface=20000, volume=20000, size=(48, 40), seed=0x5EED0001):
    sc, cf = photonmap.preset(preset, seed)
    cf.surface_photons, cf.volume_photons = surface, volume
    cf.width, cf.height = size
    return sc, cf


@pytest.fixture
def ctx():
    c = photonmap.Context(0)
    yield c
    c.close()


def frame(ctx, sc, cf):
    ctx.set_scene(sc, cf)
    ctx.emit()
    ctx.build()


def render(ctx, cf, cached=None):
    rad = torch.zeros((cf.height * cf.width, 4), dtype=torch.float32, device="cuda")
    if cached is None:
        ctx.render(rad.data_ptr(), None)
    else:
        ctx.render_cached(rad.data_ptr(), None, cached)
    torch.cuda.synchronize()
    return rad.cpu().numpy()


def rel_rmse(a, b):
    return float(np.sqrt(np.mean((a[:, :3] - b[:, :3]) ** 2)) / np.sqrt(np.mean(b[:, :3] ** 2)))


def scene_geometry(sc):
    spheres = np.array([list(sc.spheres[i]) for i in range(sc.num_spheres)], np.float64)
    axes = [int(sc.planes[i][0]) for i in range(sc.num_planes)]
    return spheres, axes


@pytest.mark.parametrize("preset,size", [(1, (48, 40)), (2, (40, 40)), (3, (64, 36))])
def test_query_list_render_equals_render(ctx, preset, size):
    sc, cf = small(preset, size=size)
    frame(ctx, sc, cf)
    ref = render(ctx, cf)
    ctx.cache_enable(log2_table=12)
    via = render(ctx, cf, cached=1)
    # same queries, same per-pixel order and arithmetic: the same bits
    np.testing.assert_array_equal(via.view(np.uint32), ref.view(np.uint32))
    st = ctx.stats()
    assert ctx.cache_stats().queries == st.surface_gathers + st.volume_gathers


def enable_small(ctx, sc, log2_table=12, table_seed=7, table_scale=0.5):
    cfg = ctx.cache_enable(log2_table=log2_table)
    w, t, res = ctx.cache_params()
    rng = np.random.default_rng(table_seed)
    t = rng.uniform(-table_scale, table_scale, t.shape).astype(np.float32)
    ctx.cache_set_params(table=t)
    return cfg, w, t, res


def sample_queries(ctx, n, seed=3):
    qa, qd = ctx.cache_queries()
    rng = np.random.default_rng(seed)
    pick = rng.choice(len(qa), n, replace=len(qa) < n)
    return qa[pick], qd[pick]


def test_encoding_matches_oracle(ctx):
    sc, cf = small(2, size=(40, 40))
    frame(ctx, sc, cf)
    cfg, w, t, res = enable_small(ctx, sc)
    qa, qd = sample_queries(ctx, 700)
    kinds = qa[:, 3].view(np.int32) != co.KNONE
    assert kinds.any() and (~kinds).any()
    out = ctx.cache_debug_step(qa, qd, np.ones((len(qa), 4), np.float32))
    lo, inv = co.grid_box(sc.box_min, sc.box_max)
    spheres, axes = scene_geometry(sc)
    x = co.features(qa, qd, lo, inv, t, res, cfg.log2_table, spheres, axes)
    np.testing.assert_allclose(out["x"][:, :32], x[:, :32], rtol=0, atol=2e-5)
    np.testing.assert_allclose(out["x"][:, 32:], x[:, 32:], rtol=0, atol=2e-6)


@pytest.mark.parametrize("n", [128, 1000, 5000])
def test_forward_backward_matches_oracle(ctx, n):
    sc, cf = small(2, size=(40, 40))
    frame(ctx, sc, cf)
    cfg, w, t, res = enable_small(ctx, sc, table_scale=0.3)
    qa, qd = sample_queries(ctx, n, seed=n)
    rng = np.random.default_rng(11)
    target = np.zeros((n, 4), np.float32)
    target[:, :3] = rng.uniform(0.0, 2.0, (n, 3))
    scale = 1.7
    out = ctx.cache_debug_step(qa, qd, target, target_scale=scale)
    assert ctx.cache_stats().tc_status == 0
    ref = co.mlp_step(out["x"].astype(np.float64), w, target[:, :3] / np.float32(scale),
                      eps=cfg.loss_eps)
    y = out["y"][:, :3]
    assert np.linalg.norm(y - ref["y"]) / np.linalg.norm(ref["y"]) < 1e-2
    assert abs(out["loss"] - ref["loss"]) / ref["loss"] < 1e-2
    gw = out["w_grad"]
    for l, (a, b) in enumerate(zip(co.split_weights(gw), co.split_weights(ref["w_grad"]))):
        err = np.linalg.norm(a - b) / np.linalg.norm(b)
        assert err < 2e-2, (l, err)
    lo, inv = co.grid_box(sc.box_min, sc.box_max)
    tg = co.table_grad(co.unit_pos(qa[:, :3], lo, inv), ref["dx"], res, cfg.log2_table)
    err = np.linalg.norm(out["table_grad"] - tg) / np.linalg.norm(tg)
    assert err < 2e-2, err


def test_training_learns_the_knn_estimate(ctx):
    """What the trained network gains: the untrained cache renders with
    ~100 % error against the k-NN render; after training it is within a few
    per cent."""
    sc, cf = small(1, 30000, 30000, size=(64, 48))
    frame(ctx, sc, cf)
    ctx.cache_enable(train_samples=1 << 16, batch=1 << 12)
    knn = render(ctx, cf, cached=1)
    untrained = rel_rmse(render(ctx, cf, cached=0), knn)
    ctx.cache_train(2)
    first = ctx.cache_stats().loss
    ctx.cache_train(78)
    st = ctx.cache_stats()
    assert st.tc_status == 0
    assert st.train_steps == 80 * 16
    trained = rel_rmse(render(ctx, cf, cached=0), knn)
    print("untrained %.4f trained %.4f loss %.4g -> %.4g" % (untrained, trained, first, st.loss))
    assert st.loss < 0.5 * first, (first, st.loss)
    assert trained < 0.25 * untrained, (untrained, trained)
    assert trained < 0.1, trained


def test_training_is_deterministic(ctx):
    """Training adds its table gradients as exact fixed-point integers and
    reduces the weight gradients, the loss and the target scale in a fixed
    order, so the same frames give the same network bit for bit, however
    the atomics of the many CTAs interleave."""
    sc, cf = small(2, 30000, 30000, size=(64, 48))
    frame(ctx, sc, cf)
    runs = []
    for _ in range(2):
        ctx.cache_enable(train_samples=1 << 16, batch=1 << 13)
        ctx.cache_train(6)
        w, t, _ = ctx.cache_params()
        runs.append((w, t, ctx.cache_stats().loss, render(ctx, cf, cached=0)))
    (w0, t0, l0, i0), (w1, t1, l1, i1) = runs
    np.testing.assert_array_equal(w0.view(np.uint32), w1.view(np.uint32))
    np.testing.assert_array_equal(t0.view(np.uint32), t1.view(np.uint32))
    assert np.float32(l0).view(np.uint32) == np.float32(l1).view(np.uint32)
    np.testing.assert_array_equal(i0.view(np.uint32), i1.view(np.uint32))


def test_bounded_wait_gives_up_reports_and_recovers(ctx):
    """Every tensor-core and copy wait of the cache kernels is bounded. With
    the first bound set to zero polls each wait gives up at once: the kernel
    records tc_status, waits out the MMA or copy it issued under the default
    bound (nothing stays in flight) and stops after its tile. The context
    stays usable: with the default bound back, training and inference run
    clean again."""
    sc, cf = small(1, 20000, 20000, size=(48, 40))
    frame(ctx, sc, cf)
    ctx.cache_enable(log2_table=12, train_samples=1 << 13, batch=1 << 12)
    ctx.cache_train(1)
    assert ctx.cache_stats().tc_status == 0
    ctx.cache_set_wait_limit(0)
    ctx.cache_train(1)
    assert ctx.cache_stats().tc_status == 1
    ctx.cache_clear_status()
    render(ctx, cf, cached=0)
    assert ctx.cache_stats().tc_status == 1
    ctx.cache_set_wait_limit(-1)
    ctx.cache_clear_status()
    ctx.cache_train(2)
    img = render(ctx, cf, cached=0)
    assert ctx.cache_stats().tc_status == 0
    assert np.isfinite(img).all()


def test_cached_values_are_the_network_of_each_query(ctx):
    """The query list holds each block of 32 consecutive pixels
    sample-major, and pm_render_cached runs inference in list order; every
    query's value must land in its own slot: it equals the network output
    for that query from the training kernel's forward pass (same weights
    and table), and not the output of its neighbour in the list. 40 x 40
    pixels: blocks that straddle image rows and a short last block."""
    sc, cf = small(2, size=(40, 40))
    frame(ctx, sc, cf)
    ctx.cache_enable(log2_table=12, train_samples=1 << 14, batch=1 << 12)
    ctx.cache_train(8)
    render(ctx, cf, cached=0)
    vals = ctx.cache_values()[:, :3]
    qa, qd = ctx.cache_queries()
    scale = np.float32(ctx.cache_stats().target_scale)
    out = ctx.cache_debug_step(qa, qd, np.zeros((len(qa), 4), np.float32))
    assert ctx.cache_stats().tc_status == 0
    ref = np.maximum(out["y"][:, :3], 0.0) * scale

    def rel(a, b):
        return float(np.linalg.norm(a - b) / np.linalg.norm(b))

    err = rel(vals, ref)
    shifted = rel(vals, np.roll(ref, 1, axis=0))
    print("cached values vs forward pass %.3g (neighbour's: %.3g)" % (err, shifted))
    assert err < 1e-3, err
    assert shifted > 20 * err + 1e-3, (err, shifted)


def test_cache_file_round_trip(ctx, tmp_path):
    sc, cf = small(1, size=(32, 32))
    frame(ctx, sc, cf)
    ctx.cache_enable(log2_table=12, train_samples=1 << 12, batch=1 << 11)
    ctx.cache_train(3)
    a = render(ctx, cf, cached=0)
    path = str(tmp_path / "cache.bin")
    ctx.cache_save(path)
    w0, t0, _ = ctx.cache_params()
    ctx.cache_enable(log2_table=12, train_samples=1 << 12, batch=1 << 11, seed=99)
    ctx.cache_load(path)
    w1, t1, _ = ctx.cache_params()
    np.testing.assert_array_equal(w0, w1)
    np.testing.assert_array_equal(t0, t1)
    b = render(ctx, cf, cached=0)
    np.testing.assert_array_equal(a, b)
    assert ctx.cache_stats().train_steps == 6
    ctx.cache_enable(log2_table=13)
    with pytest.raises(photonmap.PMError):
        ctx.cache_load(path)


def test_cached_render_against_float64_at_bench_scale(ctx):
    """The A/B of the benchmark scene (preset 2: 1M + 1M photons, 1024^2,
    k = 100): the cached render after 384 online training frames (2^20
    samples and 8 Adam steps each, the default settings) and the k-NN
    render, both against the FP64 oracle render on 8192 random pixels. The
    target: the cached render within 1e-2 relative RMSE of the FP64 render
    (the k-NN render's own error is ~0.3 %). Training is deterministic
    (fixed-point table gradient, fixed-order reductions), so every run of
    this build on a GB300 gives the same image."""
    import oracle
    sc, cf = photonmap.preset(2, 0x5EED0002)
    frame(ctx, sc, cf)
    knn = render(ctx, cf)
    ctx.cache_enable()
    ctx.cache_train(384)
    cached = render(ctx, cf, cached=0)
    assert ctx.cache_stats().tc_status == 0
    rng = np.random.default_rng(2024)
    pix = np.sort(rng.choice(cf.width * cf.height, 8192, replace=False)).astype(np.uint32)
    m64 = oracle.emit(sc, cf, None, double=True)
    r64 = oracle.render(sc, cf, None, m64, pixels=pix, double=True)
    e_knn = rel_rmse(knn[pix], r64)
    e_cache = rel_rmse(cached[pix], r64)
    e_ab = rel_rmse(cached, knn)
    print("rel RMSE vs FP64: k-NN %.4f cached %.4f; cached vs k-NN %.4f" % (e_knn, e_cache, e_ab))
    assert e_cache < 1e-2, (e_knn, e_cache)
    assert e_ab < 1.5e-2, e_ab


@pytest.mark.parametrize("preset", [1, 2])
def test_training_targets_equal_per_query_knn(ctx, preset):
    """The warm-started runs of spatially sorted samples give exactly the
    per-query k-NN estimates (the values the k-NN render path sums)."""
    sc, cf = small(preset, 30000, 30000, size=(48, 40))
    frame(ctx, sc, cf)
    ctx.cache_enable(log2_table=12, train_samples=1 << 14, batch=1 << 12)
    render(ctx, cf, cached=1)
    raw = ctx.cache_values()  # flux sums and squared radii
    qa, _ = ctx.cache_queries()
    targets, query = ctx.cache_debug_targets()
    # the estimate from the raw values, in float32 with the kernel's operations
    f = np.float32
    e, r2 = raw[query, :3], raw[query, 3:4]
    vol = (qa[query, 3].view(np.int32) == co.KNONE)[:, None]
    with np.errstate(divide="ignore", invalid="ignore"):
        s_surf = (f(1.0) / (f(3.14159265) * r2)) * f(0.318309886)
        s_vol = f(1.0) / ((f(4.18879020) * r2) * np.sqrt(r2))
    want = np.where(r2 >= 0, e * np.where(vol, s_vol, s_surf), f(0.0)).astype(np.float32)
    assert (r2 >= 0).mean() > 0.9
    np.testing.assert_array_equal(targets[:, :3].view(np.uint32), want.view(np.uint32))
