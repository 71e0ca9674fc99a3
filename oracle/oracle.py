"""ctypes bindings of oracle/liboracle.so, the CPU restatements used as the
parity checker.

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
benchmark's CPU-baseline leg. The product never imports it.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
_lib = None


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("oracle/liboracle.so is not built (run __graft_entry__.build())")
        lib = ctypes.CDLL(LIB_PATH)
        vp, f, i, u = ctypes.c_void_p, ctypes.c_float, ctypes.c_int, ctypes.c_uint
        lib.pmo_legacy_create.restype = vp
        for n in ["pmo_legacy_destroy", "pmo_legacy_reset", "pmo_legacy_init_random"]:
            getattr(lib, n).argtypes = [vp]
            getattr(lib, n).restype = None
        for n in ["pmo_legacy_get_grid", "pmo_legacy_set_grid", "pmo_legacy_get_table", "pmo_legacy_get_rng"]:
            getattr(lib, n).argtypes = [vp, vp]
            getattr(lib, n).restype = None
        lib.pmo_legacy_emit.argtypes = [vp, f, i, i]
        lib.pmo_legacy_emit.restype = None
        lib.pmo_legacy_render.argtypes = [vp, u, u, f, i, i, vp, vp]
        lib.pmo_legacy_render.restype = None
        lib.pmo_legacy_position_spheres.argtypes = [f, vp]
        lib.pmo_legacy_position_spheres.restype = None
        _lib = lib
    return _lib


class LegacyOracle:
    """Serial CPU run of the reference's voxel photon mapper."""

    def __init__(self):
        self.lib = load()
        self.h = self.lib.pmo_legacy_create()

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.pmo_legacy_destroy(self.h)
            self.h = None

    def init_random(self):
        self.lib.pmo_legacy_init_random(self.h)

    def emit(self, anim_time=0.0, interp=0, media=0):
        self.lib.pmo_legacy_emit(self.h, anim_time, int(interp), int(media))

    def render(self, width, height, anim_time=0.0, interp=0, media=0):
        img = np.zeros((height, width, 4), np.uint8)
        rgb = np.zeros((height, width, 3), np.float32)
        self.lib.pmo_legacy_render(self.h, width, height, anim_time, int(interp), int(media),
                                   img.ctypes.data, rgb.ctypes.data)
        return img, rgb

    def grid(self):
        g = np.zeros((32, 32, 32, 3), np.float32)
        self.lib.pmo_legacy_get_grid(self.h, g.ctypes.data)
        return g

    def set_grid(self, g):
        g = np.ascontiguousarray(g, np.float32)
        self.lib.pmo_legacy_set_grid(self.h, g.ctypes.data)

    def table(self):
        t = np.zeros((10000, 3), np.float32)
        self.lib.pmo_legacy_get_table(self.h, t.ctypes.data)
        return t

    def rng(self):
        r = np.zeros(2, np.uint32)
        self.lib.pmo_legacy_get_rng(self.h, r.ctypes.data)
        return r


# ---- physically based mode ---------------------------------------------------

def _phys_protos(lib):
    vp, u32, i, f = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_int, ctypes.c_float
    lib.pmo_emit.argtypes = [vp, vp, vp, vp, vp, vp, vp, vp, vp]
    lib.pmo_emit.restype = i
    lib.pmo_fixed_sum.argtypes = [vp, i]
    lib.pmo_fixed_sum.restype = f
    lib.pmo_knn.argtypes = [vp, u32, vp, u32, i, f, vp, vp]
    lib.pmo_knn.restype = None
    lib.pmo_render.argtypes = [vp, vp, vp, vp, vp, u32, vp, vp, u32, vp, u32, vp, vp]
    lib.pmo_render.restype = None
    lib.pmo_render_timed.argtypes = [vp, vp, vp, vp, vp, u32, vp, vp, u32, vp, u32, vp, vp, vp]
    lib.pmo_render_timed.restype = None
    lib.pmo_noise_grid.argtypes = [vp, i, ctypes.c_uint64, f, f]
    lib.pmo_noise_grid.restype = None
    lib.pmo_philox.argtypes = [ctypes.c_uint64, vp, vp]
    lib.pmo_philox.restype = None
    lib.pmo_logf.argtypes = [f]
    lib.pmo_logf.restype = f
    lib.pmo_expf.argtypes = [f]
    lib.pmo_expf.restype = f
    lib.pmo_sincos2pi.argtypes = [f, vp, vp]
    lib.pmo_sincos2pi.restype = None
    lib.pmo_oct_encode.argtypes = [vp]
    lib.pmo_oct_encode.restype = u32
    lib.pmo_oct_decode.argtypes = [u32, vp]
    lib.pmo_oct_decode.restype = None
    lib.pmo_sizeof_scene.restype = ctypes.c_size_t
    lib.pmo_sizeof_config.restype = ctypes.c_size_t
    lib.pmo64_emit.argtypes = [vp, vp, vp, vp, vp, vp, vp, vp, vp]
    lib.pmo64_emit.restype = i
    lib.pmo64_render.argtypes = [vp, vp, vp, vp, vp, u32, vp, vp, u32, vp, u32, vp]
    lib.pmo64_render.restype = None
    lib.pmo_preset.argtypes = [i, ctypes.c_uint64, vp, vp]
    lib.pmo_preset.restype = i
    lib.pmo_knn_kd.argtypes = [vp, u32, vp, u32, i, f, vp, vp]
    lib.pmo_knn_kd.restype = None
    lib.pmo_set_gather_index.argtypes = [i]
    lib.pmo_set_gather_index.restype = None
    lib.pmo_render_create.argtypes = [vp, vp, vp, vp, vp, u32, vp, vp, u32]
    lib.pmo_render_create.restype = vp
    lib.pmo_render_pixels.argtypes = [vp, vp, u32, vp, vp]
    lib.pmo_render_pixels.restype = None
    lib.pmo_render_free.argtypes = [vp]
    lib.pmo_render_free.restype = None
    lib.pmo_trace_sample.argtypes = [vp, vp, vp, u32, u32]
    lib.pmo_trace_sample.restype = ctypes.c_uint64
    lib.pmo_trace_path.argtypes = [vp, vp, vp, u32, vp, vp, vp, vp, vp, vp]
    lib.pmo_trace_path.restype = None
    lib.pmo64_radius_gather.argtypes = [vp, vp, vp, u32, vp, vp, u32, f, f, vp]
    lib.pmo64_radius_gather.restype = None
    lib.pmo_sample.argtypes = [i, vp, f, f, f, vp]
    lib.pmo_sample.restype = None
    lib.pmo_fresnel.argtypes = [f, f]
    lib.pmo_fresnel.restype = f
    lib.pmo_hg_phase.argtypes = [f, f]
    lib.pmo_hg_phase.restype = f


def phys_lib():
    lib = load()
    if not getattr(lib, "_phys_ready", False):
        _phys_protos(lib)
        lib._phys_ready = True
    return lib


NOISE_SEED_SALT = 0x6E6F697365


class Material(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("albedo", ctypes.c_float * 3), ("ior", ctypes.c_float)]


class Scene(ctypes.Structure):
    """pmo_scene: the memory layout of the product's pm_scene (float4
    members 16-byte aligned, float2 8-byte), declared here so that CPU-only
    callers need not load the product library."""
    _fields_ = [
        ("num_spheres", ctypes.c_int), ("_pad0", ctypes.c_byte * 12),
        ("spheres", (ctypes.c_float * 4) * 64),
        ("sphere_mat", Material * 64),
        ("num_planes", ctypes.c_int), ("_pad1", ctypes.c_byte * 4),
        ("planes", (ctypes.c_float * 2) * 8),
        ("plane_mat", Material * 8),
        ("box_min", ctypes.c_float * 3), ("box_max", ctypes.c_float * 3),
        ("light", ctypes.c_float * 3), ("light_power", ctypes.c_float),
        ("sigma_s", ctypes.c_float), ("sigma_a", ctypes.c_float), ("hg_g", ctypes.c_float),
        ("het_res", ctypes.c_int), ("het_min", ctypes.c_float), ("het_max", ctypes.c_float),
        ("cam_pos", ctypes.c_float * 3), ("focal", ctypes.c_float),
        ("_pad2", ctypes.c_byte * 8),
    ]


class Config(ctypes.Structure):
    """pmo_config: the memory layout of the product's pm_config."""
    _fields_ = [
        ("seed", ctypes.c_uint64), ("scene_id", ctypes.c_uint32),
        ("surface_photons", ctypes.c_uint32), ("volume_photons", ctypes.c_uint32),
        ("max_paths", ctypes.c_uint32), ("max_bounces", ctypes.c_int),
        ("rr_survival", ctypes.c_float), ("width", ctypes.c_int), ("height", ctypes.c_int),
        ("k", ctypes.c_int), ("radius", ctypes.c_float), ("march_step", ctypes.c_float),
        ("leaf_size", ctypes.c_int), ("exposure", ctypes.c_float), ("_pad", ctypes.c_byte * 4),
    ]


def preset(which, seed):
    """Benchmark preset `which` (1, 2, 3) from the oracle's restatement of
    the product's scene generator: (Scene, Config), byte-equal to
    pm_preset's."""
    lib = phys_lib()
    assert ctypes.sizeof(Scene) == lib.pmo_sizeof_scene()
    assert ctypes.sizeof(Config) == lib.pmo_sizeof_config()
    sc, cf = Scene(), Config()
    if lib.pmo_preset(which, seed & (2 ** 64 - 1), ctypes.byref(sc), ctypes.byref(cf)) != 0:
        raise ValueError("no preset %r" % (which,))
    return sc, cf


def set_gather_index(which):
    """'kdtree' (default) or 'grid': the neighbour index of render()."""
    phys_lib().pmo_set_gather_index({"grid": 0, "kdtree": 1}[which])


def noise_grid(scene, cfg):
    """The heterogeneous medium's sigma_s grid (None for a homogeneous one)."""
    if scene.het_res <= 0:
        return None
    r = scene.het_res
    g = np.zeros(r * r * r, np.float32)
    phys_lib().pmo_noise_grid(g.ctypes.data, r, (cfg.seed ^ NOISE_SEED_SALT) & (2 ** 64 - 1),
                              scene.het_min, scene.het_max)
    return g


def _ptr(a):
    return None if a is None else a.ctypes.data


class PhysicalMaps:
    def __init__(self, spos, spow, vpos, vpow, sizes, paths):
        self.spos, self.spow, self.vpos, self.vpow = spos, spow, vpos, vpow
        self.sizes, self.paths = sizes, paths


def emit(scene, cfg, het=None, double=False):
    """Photon maps as the GPU compacts them (float32) or their float64
    counterpart (pos [n,4], pow [n,6] with the direction in pow[:,3:])."""
    lib = phys_lib()
    ns, nv = cfg.surface_photons, cfg.volume_photons
    dt, w = (np.float64, 6) if double else (np.float32, 4)
    spos = np.zeros((max(ns, 1), 4), dt)
    spow = np.zeros((max(ns, 1), w), dt)
    vpos = np.zeros((max(nv, 1), 4), dt)
    vpow = np.zeros((max(nv, 1), w), dt)
    sizes = np.zeros(2, np.uint32)
    paths = np.zeros(2, np.uint32)
    fn = lib.pmo64_emit if double else lib.pmo_emit
    fn(ctypes.byref(scene), ctypes.byref(cfg), _ptr(het), spos.ctypes.data, spow.ctypes.data,
       vpos.ctypes.data, vpow.ctypes.data, sizes.ctypes.data, paths.ctypes.data)
    return PhysicalMaps(spos[:sizes[0]], spow[:sizes[0]], vpos[:sizes[1]], vpow[:sizes[1]], sizes,
                        paths)


def fixed_sum(terms):
    """The estimate sum of non-negative float32 terms (order-independent)."""
    t = np.ascontiguousarray(terms, np.float32)
    return np.float32(phys_lib().pmo_fixed_sum(t.ctypes.data, len(t)))


def knn(pos, queries, k, radius):
    pos = np.ascontiguousarray(pos, np.float32)
    q = np.ascontiguousarray(queries, np.float32)
    idx = np.zeros((len(q), k), np.uint32)
    d2 = np.zeros((len(q), k), np.float32)
    phys_lib().pmo_knn(pos.ctypes.data, len(pos), q.ctypes.data, len(q), k, radius,
                       idx.ctypes.data, d2.ctypes.data)
    return idx, d2


def knn_kd(pos, queries, k, radius):
    """knn() through the CPU kd-tree (the same sets)."""
    pos = np.ascontiguousarray(pos, np.float32)
    q = np.ascontiguousarray(queries, np.float32)
    idx = np.zeros((len(q), k), np.uint32)
    d2 = np.zeros((len(q), k), np.float32)
    phys_lib().pmo_knn_kd(pos.ctypes.data, len(pos), q.ctypes.data, len(q), k, radius,
                          idx.ctypes.data, d2.ctypes.data)
    return idx, d2


def render_timed(scene, cfg, het, maps, pixels):
    """float32 render of `pixels`; returns (radiance, gathers[2], seconds[2]
    = neighbour-index build, shading)."""
    pixels = np.ascontiguousarray(pixels, np.uint32)
    out = np.zeros((len(pixels), 4), np.float32)
    gathers = np.zeros(2, np.uint64)
    secs = np.zeros(2, np.float64)
    phys_lib().pmo_render_timed(ctypes.byref(scene), ctypes.byref(cfg), _ptr(het),
                                maps.spos.ctypes.data, maps.spow.ctypes.data, len(maps.spos),
                                maps.vpos.ctypes.data, maps.vpow.ctypes.data, len(maps.vpos),
                                pixels.ctypes.data, len(pixels), out.ctypes.data,
                                gathers.ctypes.data, secs.ctypes.data)
    return out, gathers, secs


class Renderer:
    """float32 renders of pixel samples over fixed maps: the neighbour
    indexes are built once (build_s) and reused by every pixels() call."""

    def __init__(self, scene, cfg, het, maps):
        import time
        self.lib = phys_lib()
        self.keep = (scene, cfg, het, maps)
        t0 = time.perf_counter()
        self.h = self.lib.pmo_render_create(
            ctypes.byref(scene), ctypes.byref(cfg), _ptr(het), maps.spos.ctypes.data,
            maps.spow.ctypes.data, len(maps.spos), maps.vpos.ctypes.data, maps.vpow.ctypes.data,
            len(maps.vpos))
        self.build_s = time.perf_counter() - t0

    def pixels(self, pixels):
        """(radiance [n, 4], gathers [2]) of the given pixel indices."""
        pixels = np.ascontiguousarray(pixels, np.uint32)
        out = np.zeros((len(pixels), 4), np.float32)
        gathers = np.zeros(2, np.uint64)
        self.lib.pmo_render_pixels(self.h, pixels.ctypes.data, len(pixels), out.ctypes.data,
                                   gathers.ctypes.data)
        return out, gathers

    def close(self):
        if self.h:
            self.lib.pmo_render_free(self.h)
            self.h = None

    def __del__(self):
        self.close()


def trace_sample(scene, cfg, het, first, count):
    """Traces paths first .. first + count - 1 on all threads (timing sample
    of the emission); returns the records they produced."""
    return int(phys_lib().pmo_trace_sample(ctypes.byref(scene), ctypes.byref(cfg), _ptr(het),
                                           first, count))


def maps_from_arrays(spos, spow, vpos, vpow):
    """PhysicalMaps over given float32 [n, 4] record arrays (e.g. a GPU
    map copied to the host)."""
    a = [np.ascontiguousarray(x, np.float32) for x in (spos, spow, vpos, vpow)]
    sizes = np.array([len(a[0]), len(a[2])], np.uint32)
    return PhysicalMaps(a[0], a[1], a[2], a[3], sizes, np.zeros(2, np.uint32))


def render(scene, cfg, het, maps, pixels=None, double=False):
    """Radiance float[npix, 4] for the given pixel indices (all by default)."""
    lib = phys_lib()
    if pixels is None:
        pixels = np.arange(cfg.width * cfg.height, dtype=np.uint32)
    pixels = np.ascontiguousarray(pixels, np.uint32)
    if double:
        out = np.zeros((len(pixels), 4), np.float64)
        lib.pmo64_render(ctypes.byref(scene), ctypes.byref(cfg), _ptr(het), maps.spos.ctypes.data,
                         maps.spow.ctypes.data, len(maps.spos), maps.vpos.ctypes.data,
                         maps.vpow.ctypes.data, len(maps.vpos), pixels.ctypes.data, len(pixels),
                         out.ctypes.data)
        return out
    out = np.zeros((len(pixels), 4), np.float32)
    gathers = np.zeros(2, np.uint64)
    lib.pmo_render(ctypes.byref(scene), ctypes.byref(cfg), _ptr(het), maps.spos.ctypes.data,
                   maps.spow.ctypes.data, len(maps.spos), maps.vpos.ctypes.data,
                   maps.vpow.ctypes.data, len(maps.vpos), pixels.ctypes.data, len(pixels),
                   out.ctypes.data, gathers.ctypes.data)
    return out


def sample(which, n, g=0.0, direction=(0.0, 0.0, 1.0), seed=0):
    """n directions from sampler `which` (0 sphere, 1 cosine, 2 HG) with
    uniforms from a seeded numpy stream."""
    lib = phys_lib()
    rs = np.random.RandomState(seed)
    u = rs.randint(0, 1 << 24, size=(n, 2)).astype(np.float64) / float(1 << 24)
    d = np.asarray(direction, np.float32)
    out = np.zeros((n, 3), np.float32)
    o = np.zeros(3, np.float32)
    for i in range(n):
        lib.pmo_sample(which, d.ctypes.data, g, float(u[i, 0]), float(u[i, 1]), o.ctypes.data)
        out[i] = o
    return out


def radius_gather(pos, pw, points, normals, sq_radius, exposure):
    """The reference's radius gather over records in index order (float64)."""
    lib = phys_lib()
    pos = np.ascontiguousarray(pos, np.float32)
    pw = np.ascontiguousarray(pw, np.float32)
    dirs = np.zeros((len(pw), 3), np.float32)
    d = np.zeros(3, np.float32)
    for i in range(len(pw)):
        lib.pmo_oct_decode(int(pw[i, 3:4].view(np.uint32)[0]), d.ctypes.data)
        dirs[i] = d
    pts = np.ascontiguousarray(points, np.float32)
    nrm = np.ascontiguousarray(normals, np.float32)
    out = np.zeros((len(pts), 3), np.float64)
    lib.pmo64_radius_gather(pos.ctypes.data, pw.ctypes.data, dirs.ctypes.data, len(pos),
                            pts.ctypes.data, nrm.ctypes.data, len(pts), sq_radius, exposure,
                            out.ctypes.data)
    return out


# ---- the reference's own GPU kernels (measurement only) ---------------------

class ReferenceGPU:
    """The reference's photonMappingKernel.cu, compiled unmodified for the GPU
    (oracle/_ref/ref_kernels.cubin), replayed through its three launch
    wrappers by oracle/_ref/libpmref_gpu.so (ref_gpu_runner.cpp) and timed.
    Its kernels are racy by design (shared generator, non-atomic grid
    adds): timed, never compared. Raises OSError when either file is
    missing."""

    def __init__(self):
        d = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_ref")
        cubin = os.path.join(d, "ref_kernels.cubin")
        if not os.path.exists(cubin):
            raise OSError("the reference's GPU module was not built (needs the reference checkout)")
        self.lib = ctypes.CDLL(os.path.join(d, "libpmref_gpu.so"))
        f, u, i = ctypes.c_float, ctypes.c_uint, ctypes.c_int
        self.lib.pmref_gpu_load.argtypes = [ctypes.c_char_p]
        self.lib.pmref_gpu_init_rng.argtypes = [ctypes.POINTER(f)]
        self.lib.pmref_gpu_frame.argtypes = [u, u, f, i, i, i, ctypes.POINTER(f), ctypes.POINTER(f)]
        if self.lib.pmref_gpu_load(cubin.encode()) != 0:
            raise OSError("loading the reference's GPU module failed")

    def init_random(self):
        ms = ctypes.c_float()
        if self.lib.pmref_gpu_init_rng(ctypes.byref(ms)) != 0:
            raise OSError("init_random_numbers_kernel failed")
        return ms.value

    def frame(self, w, h, anim_time, interpolate, media, emit=True):
        """(emit ms, render ms) of one frame."""
        me, mr = ctypes.c_float(), ctypes.c_float()
        if self.lib.pmref_gpu_frame(w, h, anim_time, int(interpolate), int(media), int(emit),
                                    ctypes.byref(me), ctypes.byref(mr)) != 0:
            raise OSError("reference frame failed")
        return me.value, mr.value
