"""pm_knn_noalloc -- the k-NN entry point for callers that cannot allocate
device memory (code inside another framework's memory pool, plug-ins whose
host forbids allocation after start-up, real-time loops) -- against the
allocating path pm_set_photons + pm_build + pm_knn, through the C ABI.

Results must be identical (k-NN index sets and squared distances are exact
in both paths), on two calls in a row that share the entry point's fixed
scratch array. This file is collected last on purpose."""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import photonmap  # noqa: E402

pytestmark = pytest.mark.gpu

MAX_POINTS = 1 << 17
PM_ERR_LIMIT = 5


def points(rs, n):
    p = np.zeros((n, 4), np.float32)
    p[:, :3] = rs.uniform([-0.5, 0.0, -0.5], [0.5, 1.0, 0.5], size=(n, 3))
    p[: n // 10, :3] = np.round(p[: n // 10, :3] * 20) / 20  # lattice points: exact ties
    p[:, 3] = rs.uniform(size=n)  # ignored: the array position is the index
    return p


def allocating_knn(pos, q, k, radius):
    ctx = photonmap.Context(0)
    sc, cf = photonmap.preset(1)
    ctx.set_scene(sc, cf)
    ctx.set_photons(0, pos, np.ones_like(pos))
    ctx.build()
    qd = torch.from_numpy(q).cuda()
    idx = torch.zeros((len(q), k), dtype=torch.int32, device="cuda")
    d2 = torch.zeros((len(q), k), dtype=torch.float32, device="cuda")
    ctx.knn(0, qd.data_ptr(), len(q), k, radius, idx.data_ptr(), d2.data_ptr())
    torch.cuda.synchronize()
    out = idx.cpu().numpy().view(np.uint32), d2.cpu().numpy()
    ctx.close()
    return out


def noalloc_knn(pos, q, k, radius):
    lib = photonmap.load()
    pd = torch.from_numpy(pos).cuda()
    qd = torch.from_numpy(q).cuda()
    idx = torch.zeros((len(q), k), dtype=torch.int32, device="cuda")
    d2 = torch.zeros((len(q), k), dtype=torch.float32, device="cuda")
    s = lib.pm_knn_noalloc(pd.data_ptr(), len(pos), qd.data_ptr(), len(q), k, radius,
                           idx.data_ptr(), d2.data_ptr(), None)
    torch.cuda.synchronize()
    assert s == 0, s
    return idx.cpu().numpy().view(np.uint32), d2.cpu().numpy()


def test_noalloc_matches_allocating_path_on_consecutive_calls():
    torch.cuda.set_device(0)
    rs = np.random.RandomState(11)
    cases = [(points(rs, 60000), 8, 0.05), (points(rs, MAX_POINTS), 100, 0.1)]
    for pos, k, radius in cases:  # two calls in a row on the shared scratch
        q = np.zeros((2000, 4), np.float32)
        q[:, :3] = rs.uniform([-0.55, -0.05, -0.55], [0.55, 1.05, 0.55], size=(2000, 3))
        ai, ad = allocating_knn(pos, q, k, radius)
        bi, bd = noalloc_knn(pos, q, k, radius)
        np.testing.assert_array_equal(bi, ai)
        np.testing.assert_array_equal(bd.view(np.uint32), ad.view(np.uint32))


def test_noalloc_allocates_no_device_memory():
    """The device's free memory (cudaMemGetInfo) is the same before and
    after calls: the scratch is the library's static array, not an
    allocation. The first call may load the library's kernels and its
    static array on this device (a one-time module load, not an allocation
    by the entry point), so the check covers the calls after it."""
    torch.cuda.set_device(0)
    rs = np.random.RandomState(5)
    for n, k in [(4096, 16), (MAX_POINTS, 64), (1000, 128)]:
        pos = points(rs, n)
        q = np.zeros((4096, 4), np.float32)
        q[:, :3] = rs.uniform([-0.5, 0.0, -0.5], [0.5, 1.0, 0.5], size=(4096, 3))
        pd = torch.from_numpy(pos).cuda()
        qd = torch.from_numpy(q).cuda()
        idx = torch.zeros((len(q), k), dtype=torch.int32, device="cuda")
        d2 = torch.zeros((len(q), k), dtype=torch.float32, device="cuda")
        lib = photonmap.load()

        def call():
            s = lib.pm_knn_noalloc(pd.data_ptr(), n, qd.data_ptr(), len(q), k, 0.1,
                                   idx.data_ptr(), d2.data_ptr(), None)
            torch.cuda.synchronize()
            assert s == 0, s

        call()
        free_before, _ = torch.cuda.mem_get_info()
        for _ in range(3):
            call()
        free_after, _ = torch.cuda.mem_get_info()
        assert free_after == free_before, (n, free_before, free_after)


def test_noalloc_rejects_more_points_than_its_scratch_holds():
    lib = photonmap.load()
    dummy = torch.zeros(4, dtype=torch.float32, device="cuda")
    p = dummy.data_ptr()
    s = lib.pm_knn_noalloc(p, MAX_POINTS + 1, p, 1, 8, 0.1, p, p, None)
    assert s == PM_ERR_LIMIT
    assert lib.pm_abi_struct_size(0) == ctypes.sizeof(photonmap.Scene)
