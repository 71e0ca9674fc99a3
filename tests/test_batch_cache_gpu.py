"""Per-scene radiance caches of a batch (pm_batch_cache_*) on the GPU: each
scene's network learns that scene's k-NN image, a replayed CUDA graph keeps
training exactly like eager frames (schedule, target scale and frame
counter in device memory), and the caches keep every scene on the
query-list render."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
import photonmap  # noqa: E402

pytestmark = pytest.mark.gpu


def small_batch(n=3, seed=0x5EED0005):
    scenes, cfgs = [], []
    for i in range(n):
        sc, cf = photonmap.batch_scene(i, seed)
        f = 1.0 / 40.0
        cf.surface_photons = max(int(cf.surface_photons * f), 20000)
        cf.volume_photons = max(int(cf.volume_photons * f), 20000) if cf.volume_photons else 0
        cf.width = cf.height = cf.width // 16
        cf.max_paths = 8 * max(cf.surface_photons, cf.volume_photons)
        scenes.append(sc)
        cfgs.append(cf)
    return scenes, cfgs


CACHE = dict(log2_table=14, train_samples=1 << 14, batch=1 << 13, lr_half_life=200.0)


def rel_rmse(a, b):
    a = a[:, :3].astype(np.float64)
    b = b[:, :3].astype(np.float64)
    return float(np.sqrt(np.mean((a - b) ** 2)) / np.sqrt(np.mean(b ** 2)))


@pytest.fixture
def ctx():
    c = photonmap.Context(0)
    yield c
    c.close()


def test_batch_caches_learn_each_scene(ctx):
    scenes, cfgs = small_batch()
    b = photonmap.Batch(ctx, scenes, cfgs)
    b.frame()
    knn = [b.read(i)[0] for i in range(len(cfgs))]
    b.cache_enable(**CACHE)
    b.frame()
    first = [rel_rmse(b.read(i)[0], knn[i]) for i in range(len(cfgs))]
    for _ in range(59):
        b.frame()
    last = [rel_rmse(b.read(i)[0], knn[i]) for i in range(len(cfgs))]
    print("cached vs k-NN after 1 / 60 frames:", ["%.3f / %.3f" % fl for fl in zip(first, last)])
    for i, (f, l) in enumerate(zip(first, last)):
        assert np.isfinite(b.read(i)[0]).all()
        assert l < 0.5 * f, (i, f, l)
        assert l < 0.2, (i, l)
    # back to the k-NN render: the same images as before the caches
    b.cache_disable()
    b.frame()
    for i in range(len(cfgs)):
        np.testing.assert_array_equal(b.read(i)[0].view(np.uint32), knn[i].view(np.uint32))
    b.close()


def test_replayed_frames_train_like_eager_frames(ctx):
    scenes, cfgs = small_batch()
    eager = photonmap.Batch(ctx, scenes, cfgs)
    eager.cache_enable(**CACHE)
    for _ in range(5):
        eager.frame()
    want = [eager.read(i)[0] for i in range(len(cfgs))]
    eager.close()
    replay = photonmap.Batch(ctx, scenes, cfgs)
    replay.cache_enable(**CACHE)
    stream = torch.cuda.Stream()
    replay.capture(stream.cuda_stream)
    replay.launch(stream.cuda_stream)
    stream.synchronize()
    after1 = [replay.read(i)[0] for i in range(len(cfgs))]
    for _ in range(4):
        replay.launch(stream.cuda_stream)
    stream.synchronize()
    for i in range(len(cfgs)):
        got = replay.read(i)[0]
        np.testing.assert_array_equal(got.view(np.uint32), want[i].view(np.uint32), err_msg="scene %d" % i)
        assert not np.array_equal(got, after1[i])  # the replays kept training
    replay.close()


def test_caches_keep_the_query_list_render(ctx):
    scenes, cfgs = small_batch(2)
    b = photonmap.Batch(ctx, scenes, cfgs)
    b.set_tune(0, query_list=0)
    b.cache_enable(**CACHE)
    assert b.get_tune(0).query_list == 1
    with pytest.raises(photonmap.PMError):
        b.set_tune(1, query_list=0)
    with pytest.raises(photonmap.PMError):
        b.autotune()
    b.frame()
    assert np.isfinite(b.read(0)[0]).all()
    b.close()
