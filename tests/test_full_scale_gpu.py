"""Parity at the benchmark's own sizes: preset 2 (1M + 1M photons, 1024^2,
k = 100) and preset 3 (8M + 8M photons with up to 8 bounces through the
heterogeneous medium, 1920x1080, k = 128), through the C ABI.

Per preset: the full GPU frame (pm_emit + pm_build + pm_render) against the
FP32 oracle's own emission (every record of both maps, bit for bit), the
radiance of 2048 random pixels against the oracle's render of them (bit for
bit), the k-NN sets and squared distances of 4096 random queries on each
full map (bit for bit, the oracle's kd-tree search), and the relative RMSE
of those pixels against the FP64 oracle (printed, bounded)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
import photonmap  # noqa: E402
import oracle  # noqa: E402

pytestmark = pytest.mark.gpu


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def rel_rmse(a, b):
    a = np.asarray(a, np.float64)[:, :3]
    b = np.asarray(b, np.float64)[:, :3]
    return float(np.sqrt(np.mean((a - b) ** 2)) / np.sqrt(np.mean(b ** 2)))


@pytest.fixture
def ctx():
    c = photonmap.Context(0)
    yield c
    c.close()


@pytest.mark.parametrize("preset,fp64_bound", [(2, 1e-2), (3, 2e-2)])
def test_full_frame_parity(ctx, preset, fp64_bound):
    sc, cf = photonmap.preset(preset, 0x5EED0000 + preset)
    ctx.set_scene(sc, cf)
    ctx.emit()
    ctx.build()
    npix = cf.width * cf.height
    rad_d = torch.zeros((npix, 4), dtype=torch.float32, device="cuda")
    ctx.render(rad_d.data_ptr(), None)
    torch.cuda.synchronize()
    rad = rad_d.cpu().numpy()
    st = ctx.stats()

    # the maps: the oracle's emission of the same paths, every record
    het = oracle.noise_grid(sc, cf)
    m = oracle.emit(sc, cf, het)
    assert list(st.map_size) == list(m.sizes) == [cf.surface_photons, cf.volume_photons]
    assert list(st.map_paths) == list(m.paths)
    gpu_pos = []
    for mid, (op, ow) in enumerate([(m.spos, m.spow), (m.vpos, m.vpow)]):
        pos, pw = ctx.photons_soa(mid)
        np.testing.assert_array_equal(bits(pos), bits(op))
        np.testing.assert_array_equal(bits(pw), bits(ow))
        gpu_pos.append(pos)

    # sampled pixels of the frame
    rs = np.random.RandomState(preset)
    pix = np.sort(rs.choice(npix, 2048, replace=False)).astype(np.uint32)
    r32 = oracle.render(sc, cf, het, m, pixels=pix)
    np.testing.assert_array_equal(bits(rad[pix]), bits(r32))
    assert (rad[pix, :3] > 0).any()

    # k-NN sets on the full maps: half the queries at records (dense
    # neighbourhoods), half uniform in the box
    for mid in (0, 1):
        pos = gpu_pos[mid]
        q = np.zeros((4096, 4), np.float32)
        at = rs.choice(len(pos), 2048, replace=False)
        q[:2048, :3] = pos[at, :3] + rs.normal(0.0, 0.01, (2048, 3)).astype(np.float32)
        q[2048:, :3] = rs.uniform(sc.box_min[:], sc.box_max[:], (2048, 3))
        qd = torch.from_numpy(q).cuda()
        idx = torch.zeros((4096, cf.k), dtype=torch.int32, device="cuda")
        d2 = torch.zeros((4096, cf.k), dtype=torch.float32, device="cuda")
        ctx.knn(mid, qd.data_ptr(), 4096, cf.k, cf.radius, idx.data_ptr(), d2.data_ptr())
        torch.cuda.synchronize()
        oi, od = oracle.knn_kd(pos, q, cf.k, cf.radius)
        np.testing.assert_array_equal(idx.cpu().numpy().view(np.uint32), oi)
        np.testing.assert_array_equal(bits(d2.cpu().numpy()), bits(od))
        assert (oi[:2048] != 0xFFFFFFFF).all(axis=1).mean() > 0.5  # full k-sets exercised

    # the FP32 frame against the FP64 oracle on the same pixels
    m64 = oracle.emit(sc, cf, het, double=True)
    r64 = oracle.render(sc, cf, het, m64, pixels=pix, double=True)
    err = rel_rmse(rad[pix], r64)
    print("preset %d: relative RMSE vs FP64 on %d pixels: %.5f" % (preset, len(pix), err))
    assert err < fp64_bound, err
