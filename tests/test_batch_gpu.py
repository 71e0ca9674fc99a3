"""Batched scenes on the GPU through the C ABI: every scene of a batch
renders exactly as the single-scene path renders it, the CUDA-graph replay
equals the eager frame, the search knobs leave results unchanged, and the
autotuner records its trials."""
import json

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import photonmap  # noqa: E402

pytestmark = pytest.mark.gpu


def small_batch(n=6, seed=0x5EED0005):
    scenes, cfgs = [], []
    for i in range(n):
        sc, cf = photonmap.batch_scene(i, seed)
        # keep the workload's variety (spheres, medium, k, aspect of the
        # photon split) at test sizes
        f = 1.0 / 40.0
        cf.surface_photons = max(int(cf.surface_photons * f), 2000)
        cf.volume_photons = max(int(cf.volume_photons * f), 2000) if cf.volume_photons else 0
        cf.width = cf.height = cf.width // 16
        cf.max_paths = 8 * max(cf.surface_photons, cf.volume_photons)
        scenes.append(sc)
        cfgs.append(cf)
    return scenes, cfgs


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def batch_images(b, cfgs):
    return [b.read(i)[0] for i in range(len(cfgs))]


@pytest.fixture
def ctx():
    c = photonmap.Context(0)
    yield c
    c.close()


def single(ctx, sc, cf):
    ctx.set_scene(sc, cf)
    ctx.emit()
    ctx.build()
    rad = torch.zeros((cf.width * cf.height, 4), dtype=torch.float32, device="cuda")
    ctx.render(rad.data_ptr(), None)
    torch.cuda.synchronize()
    return rad.cpu().numpy(), ctx.stats()


def test_batch_scenes_equal_single_scene_renders(ctx):
    scenes, cfgs = small_batch()
    assert len({cf.k for cf in cfgs}) > 1
    b = photonmap.Batch(ctx, scenes, cfgs)
    b.frame()
    imgs = batch_images(b, cfgs)
    for i, (sc, cf) in enumerate(zip(scenes, cfgs)):
        ref, st = single(ctx, sc, cf)
        bs = b.stats(i)
        assert list(bs.map_size) == list(st.map_size), i
        assert list(bs.map_paths) == list(st.map_paths), i
        assert bs.surface_gathers == st.surface_gathers and bs.volume_gathers == st.volume_gathers
        np.testing.assert_array_equal(bits(imgs[i]), bits(ref), err_msg="scene %d" % i)
        assert imgs[i][:, :3].max() > 0
    b.close()


def test_graph_replay_equals_eager_frame(ctx):
    scenes, cfgs = small_batch(4)
    b = photonmap.Batch(ctx, scenes, cfgs)
    b.frame()
    eager = batch_images(b, cfgs)
    stream = torch.cuda.Stream()
    b.capture(stream.cuda_stream)
    l0 = ctx.lib.pm_kernel_launches()
    for _ in range(2):
        b.launch(stream.cuda_stream)
    stream.synchronize()
    assert ctx.lib.pm_kernel_launches() - l0 > 4 * 2
    replay = batch_images(b, cfgs)
    for a, r in zip(eager, replay):
        np.testing.assert_array_equal(bits(a), bits(r))
    b.close()


def test_frame_launches_do_not_grow_with_scenes(ctx):
    """Every stage of the frame runs over all scenes in shared launches: a
    batch of the same two scenes three times over replays exactly as many
    kernels per frame as the two scenes alone, and each copy renders like
    the original."""
    scenes, cfgs = small_batch(2)
    counts, imgs = [], []
    for rep in (1, 3):
        b = photonmap.Batch(ctx, scenes * rep, cfgs * rep)
        stream = torch.cuda.Stream()
        b.capture(stream.cuda_stream)
        l0 = ctx.lib.pm_kernel_launches()
        b.launch(stream.cuda_stream)
        stream.synchronize()
        counts.append(ctx.lib.pm_kernel_launches() - l0)
        imgs.append(batch_images(b, cfgs * rep))
        b.close()
    print("kernels per replayed frame, 2 and 6 scenes:", counts)
    assert counts[0] == counts[1], counts
    for i in range(6):
        np.testing.assert_array_equal(bits(imgs[1][i]), bits(imgs[0][i % 2]), err_msg="copy %d" % i)


def test_search_knobs_do_not_change_images(ctx):
    scenes, cfgs = small_batch(4)
    b = photonmap.Batch(ctx, scenes, cfgs)
    b.frame()
    ref = batch_images(b, cfgs)
    for leaf, tile, collect, merge, ql in [(64, 4, 32, 8, 0), (128, 2, 64, 33, 0), (32, 8, 128, 1, 0),
                                           (64, 1, 128, 16, 1), (128, 1, 128, 16, 1)]:
        for i in range(len(cfgs)):
            # mixed: odd scenes in the other render mode
            b.set_tune(i, leaf, tile, collect, merge, ql if i % 2 == 0 else 1 - ql)
        b.frame()
        got = batch_images(b, cfgs)
        for i, (a, r) in enumerate(zip(got, ref)):
            np.testing.assert_array_equal(bits(a), bits(r), err_msg="scene %d %s" % (
                i, (leaf, tile, collect, merge, ql)))
    b.close()


def test_autotune_writes_its_trials(ctx, tmp_path):
    scenes, cfgs = small_batch(6)
    b = photonmap.Batch(ctx, scenes, cfgs)
    b.frame()
    ref = batch_images(b, cfgs)
    path = str(tmp_path / "tune.json")
    b.autotune(path)
    doc = json.load(open(path))
    ks = sorted({cf.k for cf in cfgs})
    assert [c["k"] for c in doc["classes"]] == ks
    for c in doc["classes"]:
        assert len(c["trials"]) == 12 + 9 + 3
        assert sorted({t["query_list"] for t in c["trials"]}) == [0, 1]
        assert c["choice"]["ms"] == min(t["ms"] for t in c["trials"])
        for i, cf in enumerate(cfgs):
            if cf.k == c["k"]:
                t = b.get_tune(i)
                assert (t.leaf_size, t.tile, t.collect_max, t.merge_min, t.query_list) == (
                    c["choice"]["leaf_size"], c["choice"]["tile"], c["choice"]["collect_max"],
                    c["choice"]["merge_min"], c["choice"]["query_list"])
    got = batch_images(b, cfgs)
    for a, r in zip(got, ref):
        np.testing.assert_array_equal(bits(a), bits(r))
    b.close()


def test_batch_of_the_three_presets(ctx):
    """Presets 1-3 side by side (preset 3's heterogeneous medium included):
    each scene of the batch equals its single-scene render."""
    scenes, cfgs = [], []
    for i, p in enumerate((1, 2, 3)):
        sc, cf = photonmap.preset(p, 0x5EED0001 + p)
        cf.surface_photons = cf.volume_photons = 15000
        cf.width, cf.height = 40, 30
        cf.scene_id = i
        cf.max_paths = 8 * 15000
        scenes.append(sc)
        cfgs.append(cf)
    b = photonmap.Batch(ctx, scenes, cfgs)
    b.frame()
    imgs = batch_images(b, cfgs)
    for i, (sc, cf) in enumerate(zip(scenes, cfgs)):
        ref, _ = single(ctx, sc, cf)
        np.testing.assert_array_equal(bits(imgs[i]), bits(ref), err_msg="preset %d" % (i + 1))
    b.close()
