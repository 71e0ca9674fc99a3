"""Photon-map files and the headless frame driver on the GPU."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
import photonmap  # noqa: E402
from oracle import LegacyOracle  # noqa: E402

pytestmark = pytest.mark.gpu


def test_map_file_round_trip(tmp_path):
    sc, cf = photonmap.preset(1, 3)
    cf.surface_photons = cf.volume_photons = 20000
    a = photonmap.Context(0)
    a.set_scene(sc, cf)
    a.emit()
    path = str(tmp_path / "surface.pmap")
    a.save_map(0, path)
    b = photonmap.Context(0)
    b.set_scene(sc, cf)
    b.load_map(0, path)
    pa, wa = a.photons_soa(0)
    pb, wb = b.photons_soa(0)
    np.testing.assert_array_equal(pa.view(np.uint32), pb.view(np.uint32))
    np.testing.assert_array_equal(wa.view(np.uint32), wb.view(np.uint32))
    a.build()
    b.build()
    q = torch.rand((500, 4), device="cuda") - torch.tensor([0.5, 0.0, 0.5, 0.0], device="cuda")
    out = []
    for c in (a, b):
        idx = torch.zeros((500, 32), dtype=torch.int32, device="cuda")
        d2 = torch.zeros((500, 32), dtype=torch.float32, device="cuda")
        c.knn(0, q.data_ptr(), 500, 32, 0.1, idx.data_ptr(), d2.data_ptr())
        torch.cuda.synchronize()
        out.append(idx.cpu().numpy())
    np.testing.assert_array_equal(out[0], out[1])


def test_viewer_matches_reference_frame_loop():
    v = photonmap.Viewer(128, 96)
    o = LegacyOracle()
    img = torch.zeros((96, 128, 4), dtype=torch.uint8, device="cuda")
    o.emit(0.0, 0, 0)  # initCuda's early emission
    keys = ["", "a", "p", "", "i", "e", "", "a", "e", ""]
    t, inc, interp, media, anim, emit = 0.0, np.float32(0.1), 0, 0, 0, 1
    for i, k in enumerate(keys):
        if k:
            v.key(k)
            anim ^= k == "a"
            media ^= k == "p"
            interp ^= k == "i"
            emit ^= k == "e"
        v.display(img.data_ptr())
        torch.cuda.synchronize()
        if i == 0:
            o.init_random()
        if emit:
            o.emit(float(t), interp, media)
        oimg, _ = o.render(128, 96, float(t), interp, media)
        np.testing.assert_array_equal(img.cpu().numpy(), oimg, err_msg="frame %d" % i)
        if anim:
            t = np.float32(np.float32(t) + inc)
    assert v.state().frames == len(keys)
    v.close()


def test_physical_driver_reuses_maps_until_the_scene_changes():
    """The physically based frame loop: the first display emits and builds;
    displays of an unchanged scene reuse the maps and trees (the same image
    as a fresh frame); an animation step that moves sphere 0 re-emits; the
    'e' key forces re-emission every frame; with the cache enabled a
    display trains it online and renders through it."""
    ctx = photonmap.Context(0)
    sc, cf = photonmap.preset(2, 0x5EED0002)
    cf.surface_photons = cf.volume_photons = 20000
    cf.width, cf.height = 48, 40
    v = photonmap.PhysViewer(ctx, sc, cf)
    v.key("c")  # plain k-NN renders first
    rad = torch.zeros((cf.width * cf.height, 4), dtype=torch.float32, device="cuda")

    def show():
        v.display(rad.data_ptr(), None)
        torch.cuda.synchronize()
        return rad.cpu().numpy().copy()

    a = show()
    b = show()
    s = v.state()
    assert (s.frames, s.emissions, s.reuses) == (2, 1, 1)
    np.testing.assert_array_equal(a.view(np.uint32), b.view(np.uint32))
    fresh = photonmap.Context(0)
    fresh.set_scene(sc, cf)
    fresh.emit()
    fresh.build()
    rf = torch.zeros_like(rad)
    fresh.render(rf.data_ptr(), None)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(rf.cpu().numpy().view(np.uint32), a.view(np.uint32))
    fresh.close()
    v.key("a")  # animation on: this display is still at anim_time 0
    show()
    assert v.state().emissions == 1
    c = show()  # sphere 0 moved by 0.05 * sin(0.1)
    s = v.state()
    assert s.emissions == 2 and abs(s.anim_time - 0.2) < 1e-6
    assert not np.array_equal(c, a)
    v.key("a")  # animation off, re-emission forced
    v.key("e")
    d = show()
    e = show()
    s = v.state()
    assert s.emissions == 4 and s.reuses == 2
    np.testing.assert_array_equal(d.view(np.uint32), e.view(np.uint32))
    v.key("e")
    ctx.cache_enable(log2_table=12, train_samples=1 << 12, batch=1 << 12)
    v.key("c")
    show()
    show()
    s = v.state()
    assert s.cached_frames == 2 and s.emissions == 4
    assert ctx.cache_stats().train_frames == 2
    v.key(27)
    assert v.state().quit == 1
    v.close()
    ctx.close()
