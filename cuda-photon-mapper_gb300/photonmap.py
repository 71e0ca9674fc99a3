"""Python bindings of libphotonmap.so (include/pm.h) through ctypes.

The library is the product; this module only declares its C ABI for Python
callers (tests, the benchmark, scripts). Buffers are passed as device or
host addresses (ints). Importing fails loudly when the library has not been
built: there is no fallback implementation.
"""
import ctypes
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libphotonmap.so")

PM_OK = 0
PM_LEGACY_INTERPOLATE = 1
PM_LEGACY_MEDIA = 2
LEGACY_GRID = 32
LEGACY_PHOTONS = 10000

_c = ctypes


class Material(_c.Structure):
    _fields_ = [("kind", _c.c_int), ("albedo", _c.c_float * 3), ("ior", _c.c_float)]


class Scene(_c.Structure):
    """pm_scene (include/pm.h); padding mirrors float4/float2 alignment."""
    _fields_ = [
        ("num_spheres", _c.c_int), ("_pad0", _c.c_byte * 12),
        ("spheres", (_c.c_float * 4) * 64),
        ("sphere_mat", Material * 64),
        ("num_planes", _c.c_int), ("_pad1", _c.c_byte * 4),
        ("planes", (_c.c_float * 2) * 8),
        ("plane_mat", Material * 8),
        ("box_min", _c.c_float * 3), ("box_max", _c.c_float * 3),
        ("light", _c.c_float * 3), ("light_power", _c.c_float),
        ("sigma_s", _c.c_float), ("sigma_a", _c.c_float), ("hg_g", _c.c_float),
        ("het_res", _c.c_int), ("het_min", _c.c_float), ("het_max", _c.c_float),
        ("cam_pos", _c.c_float * 3), ("focal", _c.c_float),
        ("_pad2", _c.c_byte * 8),
    ]


class Config(_c.Structure):
    _fields_ = [
        ("seed", _c.c_uint64), ("scene_id", _c.c_uint32),
        ("surface_photons", _c.c_uint32), ("volume_photons", _c.c_uint32),
        ("max_paths", _c.c_uint32), ("max_bounces", _c.c_int), ("rr_survival", _c.c_float),
        ("width", _c.c_int), ("height", _c.c_int), ("k", _c.c_int), ("radius", _c.c_float),
        ("march_step", _c.c_float), ("leaf_size", _c.c_int), ("exposure", _c.c_float),
        ("_pad", _c.c_byte * 4),
    ]


class PhotonRecord(_c.Structure):
    _fields_ = [("location", _c.c_float * 3), ("direction", _c.c_float * 3),
                ("energy", _c.c_float * 3)]


class FrameStats(_c.Structure):
    _fields_ = [
        ("paths_traced", _c.c_uint64), ("map_size", _c.c_uint32 * 2),
        ("map_paths", _c.c_uint32 * 2), ("surface_gathers", _c.c_uint64),
        ("volume_gathers", _c.c_uint64), ("ms_emit", _c.c_float), ("ms_build", _c.c_float),
        ("ms_render", _c.c_float), ("ms_gather", _c.c_float),
    ]


class ViewerState(_c.Structure):
    _fields_ = [("width", _c.c_uint), ("height", _c.c_uint), ("anim_flag", _c.c_int),
                ("emit_flag", _c.c_int), ("interpolate", _c.c_int), ("media", _c.c_int),
                ("iter", _c.c_int), ("quit", _c.c_int), ("anim_time", _c.c_float),
                ("anim_inc", _c.c_float), ("frames", _c.c_ulonglong)]


class PhysViewerState(_c.Structure):
    _fields_ = [("anim_flag", _c.c_int), ("emit_flag", _c.c_int), ("use_cache", _c.c_int),
                ("cache_frames", _c.c_int), ("anim_time", _c.c_float), ("anim_inc", _c.c_float),
                ("anim_radius", _c.c_float), ("quit", _c.c_int), ("frames", _c.c_ulonglong),
                ("emissions", _c.c_ulonglong), ("reuses", _c.c_ulonglong),
                ("cached_frames", _c.c_ulonglong)]


class CacheConfig(_c.Structure):
    _fields_ = [("levels", _c.c_int), ("log2_table", _c.c_int), ("base_res", _c.c_int),
                ("max_res", _c.c_int), ("train_samples", _c.c_uint32), ("batch", _c.c_uint32),
                ("lr", _c.c_float), ("beta1", _c.c_float), ("beta2", _c.c_float),
                ("eps", _c.c_float), ("lr_min", _c.c_float), ("lr_half_life", _c.c_float),
                ("loss_eps", _c.c_float), ("surface_fraction", _c.c_float), ("seed", _c.c_uint64)]


class CacheStats(_c.Structure):
    _fields_ = [("queries", _c.c_ulonglong), ("train_steps", _c.c_ulonglong),
                ("train_frames", _c.c_ulonglong), ("loss", _c.c_float),
                ("target_scale", _c.c_float), ("ms_queries", _c.c_float),
                ("ms_values", _c.c_float), ("ms_composite", _c.c_float),
                ("ms_targets", _c.c_float), ("ms_train", _c.c_float), ("tc_status", _c.c_int)]


class BatchTune(_c.Structure):
    _fields_ = [("leaf_size", _c.c_int), ("tile", _c.c_int), ("collect_max", _c.c_int),
                ("merge_min", _c.c_int), ("query_list", _c.c_int)]


CACHE_WEIGHTS = 4 * 64 * 64 + 64 * 16
MAP_SURFACE = 0
MAP_VOLUME = 1
MAT_DIFFUSE, MAT_MIRROR, MAT_DIELECTRIC = 0, 1, 2
NOISE_SEED_SALT = 0x6E6F697365

_vp = _c.c_void_p
_u = _c.c_uint
_f = _c.c_float
_i = _c.c_int

# name: (restype, argtypes)
PROTOTYPES = {
    "launch_init_random_numbers_kernel": (None, []),
    "launch_emit_photons_kernel": (None, [_vp, _u, _u, _f, _c.c_bool, _c.c_bool]),
    "launch_photon_mapping_kernel": (None, [_vp, _u, _u, _f, _c.c_bool, _c.c_bool]),
    "pm_legacy_set_exit_on_error": (None, [_i]),
    "pm_legacy_last_status": (_i, []),
    "pm_legacy_last_error": (_c.c_char_p, []),
    "pm_legacy_release": (None, []),
    "pm_create": (_i, [_c.POINTER(_vp), _i]),
    "pm_destroy": (None, [_vp]),
    "pm_last_error": (_c.c_char_p, [_vp]),
    "pm_status_string": (_c.c_char_p, [_i]),
    "pm_legacy_init_random": (_i, [_vp, _vp]),
    "pm_legacy_emit": (_i, [_vp, _f, _i, _vp]),
    "pm_legacy_render": (_i, [_vp, _vp, _u, _u, _f, _i, _vp, _vp]),
    "pm_legacy_get_grid": (_i, [_vp, _vp]),
    "pm_legacy_set_grid": (_i, [_vp, _vp]),
    "pm_legacy_get_random_numbers": (_i, [_vp, _vp]),
    "pm_legacy_rng_draws": (_i, [_vp, _c.POINTER(_c.c_ulonglong)]),
    "pm_preset": (_i, [_i, _c.c_uint64, _c.POINTER(Scene), _c.POINTER(Config)]),
    "pm_set_scene": (_i, [_vp, _c.POINTER(Scene), _c.POINTER(Config)]),
    "pm_update_scene": (_i, [_vp, _c.POINTER(Scene)]),
    "pm_emit": (_i, [_vp, _vp]),
    "pm_build": (_i, [_vp, _vp]),
    "pm_render": (_i, [_vp, _vp, _vp, _vp]),
    "pm_render_single_kernel": (_i, [_vp, _vp, _vp, _vp]),
    "pm_get_gather_stats": (_i, [_vp, _vp, _i]),
    "pm_knn": (_i, [_vp, _i, _vp, _c.c_uint32, _i, _f, _vp, _vp, _vp]),
    "pm_radius_gather": (_i, [_vp, _i, _vp, _vp, _c.c_uint32, _f, _f, _vp, _vp]),
    "pm_get_photons": (_i, [_vp, _i, _vp, _c.c_uint32, _c.POINTER(_c.c_uint32)]),
    "pm_get_photons_soa": (_i, [_vp, _i, _vp, _vp, _c.c_uint32, _c.POINTER(_c.c_uint32)]),
    "pm_get_stats": (_i, [_vp, _c.POINTER(FrameStats)]),
    "pm_abi_struct_size": (_c.c_size_t, [_i]),
    "pm_set_photons": (_i, [_vp, _i, _vp, _vp, _c.c_uint32]),
    "pm_kernel_launches": (_c.c_ulonglong, []),
    "pm_knn_noalloc": (_i, [_vp, _c.c_uint32, _vp, _c.c_uint32, _i, _f, _vp, _vp, _vp]),
    "pm_save_map": (_i, [_vp, _i, _c.c_char_p]),
    "pm_load_map": (_i, [_vp, _i, _c.c_char_p]),
    "pm_write_ppm": (_i, [_c.c_char_p, _vp, _u, _u]),
    "pm_write_png": (_i, [_c.c_char_p, _vp, _u, _u]),
    "pm_viewer_create": (_i, [_c.POINTER(_vp), _u, _u]),
    "pm_viewer_destroy": (None, [_vp]),
    "pm_viewer_key": (None, [_vp, _c.c_ubyte]),
    "pm_viewer_state_get": (_i, [_vp, _c.POINTER(ViewerState)]),
    "pm_viewer_display": (_i, [_vp, _vp]),
    "pm_phys_viewer_create": (_i, [_vp, _c.POINTER(Scene), _c.POINTER(Config), _c.POINTER(_vp)]),
    "pm_phys_viewer_destroy": (None, [_vp]),
    "pm_phys_viewer_key": (None, [_vp, _c.c_ubyte]),
    "pm_phys_viewer_state_get": (_i, [_vp, _c.POINTER(PhysViewerState)]),
    "pm_phys_viewer_display": (_i, [_vp, _vp, _vp, _vp]),
    "pm_cache_default_config": (None, [_c.POINTER(CacheConfig)]),
    "pm_cache_enable": (_i, [_vp, _c.POINTER(CacheConfig)]),
    "pm_cache_disable": (_i, [_vp]),
    "pm_cache_train": (_i, [_vp, _i, _vp]),
    "pm_render_cached": (_i, [_vp, _vp, _vp, _i, _vp]),
    "pm_cache_get_stats": (_i, [_vp, _c.POINTER(CacheStats)]),
    "pm_cache_get_params": (_i, [_vp, _vp, _vp, _vp]),
    "pm_cache_set_params": (_i, [_vp, _vp, _vp]),
    "pm_cache_debug_step": (_i, [_vp, _vp, _vp, _vp, _c.c_uint32, _f, _vp, _vp, _vp, _vp, _vp]),
    "pm_cache_get_queries": (_i, [_vp, _vp, _vp, _c.c_uint32, _c.POINTER(_c.c_uint32)]),
    "pm_cache_get_values": (_i, [_vp, _vp, _c.c_uint32, _c.POINTER(_c.c_uint32)]),
    "pm_cache_debug_targets": (_i, [_vp, _vp, _vp]),
    "pm_batch_scene": (_i, [_i, _c.c_uint64, _c.POINTER(Scene), _c.POINTER(Config)]),
    "pm_batch_create": (_i, [_vp, _i, _vp, _vp, _c.POINTER(_vp)]),
    "pm_batch_destroy": (None, [_vp]),
    "pm_batch_frame": (_i, [_vp, _vp]),
    "pm_batch_capture": (_i, [_vp, _vp]),
    "pm_batch_launch": (_i, [_vp, _vp]),
    "pm_batch_image": (_i, [_vp, _i, _c.POINTER(_vp), _c.POINTER(_vp)]),
    "pm_batch_read": (_i, [_vp, _i, _vp, _vp]),
    "pm_batch_stats": (_i, [_vp, _i, _c.POINTER(FrameStats)]),
    "pm_batch_set_tune": (_i, [_vp, _i, _c.POINTER(BatchTune)]),
    "pm_batch_get_tune": (_i, [_vp, _i, _c.POINTER(BatchTune)]),
    "pm_batch_autotune": (_i, [_vp, _c.c_char_p, _vp]),
    "pm_batch_cache_enable": (_i, [_vp, _vp]),
    "pm_batch_cache_disable": (_i, [_vp]),
    "pm_cache_set_wait_limit": (_i, [_vp, _i]),
    "pm_cache_clear_status": (_i, [_vp]),
    "pm_cache_save": (_i, [_vp, _c.c_char_p]),
    "pm_cache_load": (_i, [_vp, _c.c_char_p]),
}

_lib = None


def load():
    """Loads libphotonmap.so once; raises if it is missing."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libphotonmap.so is not built (run __graft_entry__.build())")
        lib = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in PROTOTYPES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


class PMError(RuntimeError):
    pass


class Context:
    """An explicit pm_ctx on one device."""

    def __init__(self, device=0):
        self.lib = load()
        h = _vp()
        s = self.lib.pm_create(_c.byref(h), device)
        if s != PM_OK:
            raise PMError("pm_create(%d): %s" % (device, self.lib.pm_status_string(s).decode()))
        self.h = h

    def close(self):
        if self.h:
            self.lib.pm_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, s, what):
        if s != PM_OK:
            raise PMError("%s: %s (%s)" % (what, self.lib.pm_status_string(s).decode(),
                                           self.lib.pm_last_error(self.h).decode()))

    # legacy mode -------------------------------------------------------------
    def legacy_init_random(self, stream=0):
        self._check(self.lib.pm_legacy_init_random(self.h, stream), "pm_legacy_init_random")

    def legacy_emit(self, anim_time=0.0, flags=0, stream=0):
        self._check(self.lib.pm_legacy_emit(self.h, anim_time, flags, stream), "pm_legacy_emit")

    def legacy_render(self, pos, width, height, anim_time=0.0, flags=0, rgb=None, stream=0):
        self._check(self.lib.pm_legacy_render(self.h, pos, width, height, anim_time, flags,
                                              rgb, stream), "pm_legacy_render")

    def legacy_grid(self):
        g = np.zeros((LEGACY_GRID, LEGACY_GRID, LEGACY_GRID, 3), np.float32)
        self._check(self.lib.pm_legacy_get_grid(self.h, g.ctypes.data), "pm_legacy_get_grid")
        return g

    def legacy_set_grid(self, grid):
        g = np.ascontiguousarray(grid, np.float32)
        assert g.size == LEGACY_GRID ** 3 * 3
        self._check(self.lib.pm_legacy_set_grid(self.h, g.ctypes.data), "pm_legacy_set_grid")

    def legacy_random_numbers(self):
        t = np.zeros((LEGACY_PHOTONS, 3), np.float32)
        self._check(self.lib.pm_legacy_get_random_numbers(self.h, t.ctypes.data),
                    "pm_legacy_get_random_numbers")
        return t

    def legacy_rng_draws(self):
        n = _c.c_ulonglong()
        self._check(self.lib.pm_legacy_rng_draws(self.h, _c.byref(n)), "pm_legacy_rng_draws")
        return n.value


    # physically based mode --------------------------------------------------
    def set_scene(self, scene, cfg):
        self.scene, self.cfg = scene, cfg
        self._check(self.lib.pm_set_scene(self.h, _c.byref(scene), _c.byref(cfg)), "pm_set_scene")

    def update_scene(self, scene):
        self.scene = scene
        self._check(self.lib.pm_update_scene(self.h, _c.byref(scene)), "pm_update_scene")

    def emit(self, stream=0):
        self._check(self.lib.pm_emit(self.h, stream), "pm_emit")

    def build(self, stream=0):
        self._check(self.lib.pm_build(self.h, stream), "pm_build")

    def render(self, radiance=None, rgba=None, stream=0):
        self._check(self.lib.pm_render(self.h, radiance, rgba, stream), "pm_render")

    def gather_stats(self):
        """Counters of the last render's k-NN estimates (pm_get_gather_stats)."""
        out = (_c.c_uint64 * 7)()
        self._check(self.lib.pm_get_gather_stats(self.h, out, 7), "pm_get_gather_stats")
        names = ("tiled", "list", "shrunk", "violations", "groups", "candidates", "halvings")
        return dict(zip(names, [int(v) for v in out]))

    def render_single_kernel(self, radiance=None, rgba=None, stream=0):
        self._check(self.lib.pm_render_single_kernel(self.h, radiance, rgba, stream),
                    "pm_render_single_kernel")

    def knn(self, map_id, queries, nq, k, radius, idx, d2, stream=0):
        self._check(self.lib.pm_knn(self.h, map_id, queries, nq, k, radius, idx, d2, stream),
                    "pm_knn")

    def radius_gather(self, map_id, points, normals, nq, sq_radius, exposure, out, stream=0):
        self._check(self.lib.pm_radius_gather(self.h, map_id, points, normals, nq, sq_radius,
                                              exposure, out, stream), "pm_radius_gather")

    def photons_soa(self, map_id):
        """Map `map_id` in index order: (pos float32[n,4], pow float32[n,4])."""
        n = _c.c_uint32()
        self._check(self.lib.pm_get_photons_soa(self.h, map_id, None, None, 0, _c.byref(n)),
                    "pm_get_photons_soa")
        pos = np.zeros((n.value, 4), np.float32)
        pw = np.zeros((n.value, 4), np.float32)
        self._check(self.lib.pm_get_photons_soa(self.h, map_id, pos.ctypes.data, pw.ctypes.data,
                                                n.value, _c.byref(n)), "pm_get_photons_soa")
        return pos, pw

    def photon_records(self, map_id):
        """Map `map_id` in the reference's record layout, float32[n, 9]
        (location, direction, energy)."""
        n = _c.c_uint32()
        self._check(self.lib.pm_get_photons(self.h, map_id, None, 0, _c.byref(n)), "pm_get_photons")
        out = np.zeros((n.value, 9), np.float32)
        self._check(self.lib.pm_get_photons(self.h, map_id, out.ctypes.data, n.value, _c.byref(n)),
                    "pm_get_photons")
        return out

    def set_photons(self, map_id, pos, pw):
        pos = np.ascontiguousarray(pos, np.float32)
        pw = np.ascontiguousarray(pw, np.float32)
        assert pos.shape == pw.shape and pos.shape[1] == 4
        self._check(self.lib.pm_set_photons(self.h, map_id, pos.ctypes.data, pw.ctypes.data,
                                            len(pos)), "pm_set_photons")

    def save_map(self, map_id, path):
        self._check(self.lib.pm_save_map(self.h, map_id, path.encode()), "pm_save_map")

    def load_map(self, map_id, path):
        self._check(self.lib.pm_load_map(self.h, map_id, path.encode()), "pm_load_map")

    def stats(self):
        st = FrameStats()
        self._check(self.lib.pm_get_stats(self.h, _c.byref(st)), "pm_get_stats")
        return st

    # ---- learned radiance cache (pm_cache_*) ----
    def cache_enable(self, cfg=None, **overrides):
        if cfg is None:
            cfg = cache_default_config()
        for k, v in overrides.items():
            setattr(cfg, k, v)
        self._check(self.lib.pm_cache_enable(self.h, _c.byref(cfg)), "pm_cache_enable")
        self.cache_cfg = cfg
        return cfg

    def cache_disable(self):
        self._check(self.lib.pm_cache_disable(self.h), "pm_cache_disable")

    def cache_train(self, frames=1, stream=0):
        self._check(self.lib.pm_cache_train(self.h, frames, stream), "pm_cache_train")

    def render_cached(self, radiance=None, rgba=None, source=0, stream=0):
        self._check(self.lib.pm_render_cached(self.h, radiance, rgba, source, stream),
                    "pm_render_cached")

    def cache_stats(self):
        st = CacheStats()
        self._check(self.lib.pm_cache_get_stats(self.h, _c.byref(st)), "pm_cache_get_stats")
        return st

    def cache_set_wait_limit(self, polls):
        self._check(self.lib.pm_cache_set_wait_limit(self.h, polls), "pm_cache_set_wait_limit")

    def cache_clear_status(self):
        self._check(self.lib.pm_cache_clear_status(self.h), "pm_cache_clear_status")

    def cache_params(self):
        """(weights [PM_CACHE_WEIGHTS], table [levels, 2^log2, 2], res [levels])."""
        cfg = self.cache_cfg
        w = np.zeros(CACHE_WEIGHTS, np.float32)
        t = np.zeros((cfg.levels, 1 << cfg.log2_table, 2), np.float32)
        r = np.zeros(cfg.levels, np.int32)
        self._check(self.lib.pm_cache_get_params(self.h, w.ctypes.data, t.ctypes.data, r.ctypes.data),
                    "pm_cache_get_params")
        return w, t, r

    def cache_set_params(self, weights=None, table=None):
        w = None if weights is None else np.ascontiguousarray(weights, np.float32)
        t = None if table is None else np.ascontiguousarray(table, np.float32)
        self._check(self.lib.pm_cache_set_params(self.h, None if w is None else w.ctypes.data,
                                                 None if t is None else t.ctypes.data),
                    "pm_cache_set_params")

    def cache_debug_step(self, qa, qd, target, target_scale=1.0):
        """Forward + backward on host queries: dict of x, y, loss, w_grad, table_grad."""
        cfg = self.cache_cfg
        qa = np.ascontiguousarray(qa, np.float32)
        qd = np.ascontiguousarray(qd, np.float32)
        tg = np.ascontiguousarray(target, np.float32)
        n = len(qa)
        x = np.zeros((n, 64), np.float32)
        y = np.zeros((n, 4), np.float32)
        loss = np.zeros(1, np.float32)
        wg = np.zeros(CACHE_WEIGHTS, np.float32)
        tgr = np.zeros((cfg.levels, 1 << cfg.log2_table, 2), np.float32)
        self._check(self.lib.pm_cache_debug_step(self.h, qa.ctypes.data, qd.ctypes.data, tg.ctypes.data,
                                                 n, target_scale, x.ctypes.data, y.ctypes.data,
                                                 loss.ctypes.data, wg.ctypes.data, tgr.ctypes.data),
                    "pm_cache_debug_step")
        return {"x": x, "y": y, "loss": float(loss[0]), "w_grad": wg, "table_grad": tgr}

    def cache_queries(self):
        n = _c.c_uint32(0)
        self._check(self.lib.pm_cache_get_queries(self.h, None, None, 0, _c.byref(n)),
                    "pm_cache_get_queries")
        qa = np.zeros((n.value, 4), np.float32)
        qd = np.zeros((n.value, 4), np.float32)
        self._check(self.lib.pm_cache_get_queries(self.h, qa.ctypes.data, qd.ctypes.data, n.value,
                                                  _c.byref(n)), "pm_cache_get_queries")
        return qa, qd

    def cache_values(self):
        n = _c.c_uint32(0)
        self._check(self.lib.pm_cache_get_values(self.h, None, 0, _c.byref(n)), "pm_cache_get_values")
        v = np.zeros((n.value, 4), np.float32)
        self._check(self.lib.pm_cache_get_values(self.h, v.ctypes.data, n.value, _c.byref(n)),
                    "pm_cache_get_values")
        return v

    def cache_debug_targets(self):
        """(targets [train_samples, 4], query index of each) of the next training frame."""
        n = self.cache_cfg.train_samples
        t = np.zeros((n, 4), np.float32)
        q = np.zeros(n, np.uint32)
        self._check(self.lib.pm_cache_debug_targets(self.h, t.ctypes.data, q.ctypes.data),
                    "pm_cache_debug_targets")
        return t, q

    def cache_save(self, path):
        self._check(self.lib.pm_cache_save(self.h, path.encode()), "pm_cache_save")

    def cache_load(self, path):
        self._check(self.lib.pm_cache_load(self.h, path.encode()), "pm_cache_load")


class Viewer:
    """Headless frame driver (pm_viewer_*): the reference's display()/keyboard()."""

    def __init__(self, width=512, height=512):
        self.lib = load()
        h = _vp()
        if self.lib.pm_viewer_create(_c.byref(h), width, height) != PM_OK:
            raise PMError("pm_viewer_create")
        self.h = h

    def key(self, k):
        self.lib.pm_viewer_key(self.h, ord(k) if isinstance(k, str) else int(k))

    def state(self):
        st = ViewerState()
        self.lib.pm_viewer_state_get(self.h, _c.byref(st))
        return st

    def display(self, pos):
        s = self.lib.pm_viewer_display(self.h, pos)
        if s != PM_OK:
            raise PMError("pm_viewer_display: %s" % self.lib.pm_status_string(s).decode())

    def close(self):
        if self.h:
            self.lib.pm_viewer_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class PhysViewer:
    """pm_phys_viewer: the frame loop over a context's physically based
    pipeline with temporal reuse of the maps, trees and cache."""

    def __init__(self, ctx, scene, cfg):
        self.lib = load()
        self.ctx = ctx
        h = _c.c_void_p()
        ctx._check(self.lib.pm_phys_viewer_create(ctx.h, _c.byref(scene), _c.byref(cfg),
                                                  _c.byref(h)), "pm_phys_viewer_create")
        self.h = h

    def key(self, k):
        self.lib.pm_phys_viewer_key(self.h, ord(k) if isinstance(k, str) else k)

    def state(self):
        st = PhysViewerState()
        self.ctx._check(self.lib.pm_phys_viewer_state_get(self.h, _c.byref(st)),
                        "pm_phys_viewer_state_get")
        return st

    def display(self, radiance=None, rgba=None, stream=0):
        self.ctx._check(self.lib.pm_phys_viewer_display(self.h, radiance, rgba, stream),
                        "pm_phys_viewer_display")

    def close(self):
        if self.h:
            self.lib.pm_phys_viewer_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()


def batch_scene(index, seed=0x5EED0005):
    """Scene `index` of the batched benchmark workload (pm_batch_scene)."""
    sc, cf = Scene(), Config()
    s = load().pm_batch_scene(index, seed, _c.byref(sc), _c.byref(cf))
    if s != PM_OK:
        raise PMError("pm_batch_scene(%d): %s" % (index, load().pm_status_string(s).decode()))
    return sc, cf


class Batch:
    """Many scenes per frame (pm_batch_*), owned by a Context."""

    def __init__(self, ctx, scenes, cfgs):
        self.ctx = ctx
        self.lib = ctx.lib
        self.n = len(scenes)
        arr_s = (Scene * self.n)(*scenes)
        arr_c = (Config * self.n)(*cfgs)
        self.cfgs = list(cfgs)
        h = _vp()
        ctx._check(self.lib.pm_batch_create(ctx.h, self.n, _c.addressof(arr_s), _c.addressof(arr_c),
                                            _c.byref(h)), "pm_batch_create")
        self.h = h

    def close(self):
        if self.h:
            self.lib.pm_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def frame(self, stream=0):
        self.ctx._check(self.lib.pm_batch_frame(self.h, stream), "pm_batch_frame")

    def capture(self, stream):
        self.ctx._check(self.lib.pm_batch_capture(self.h, stream), "pm_batch_capture")

    def launch(self, stream):
        self.ctx._check(self.lib.pm_batch_launch(self.h, stream), "pm_batch_launch")

    def image_ptrs(self, i):
        r, g = _vp(), _vp()
        self.ctx._check(self.lib.pm_batch_image(self.h, i, _c.byref(r), _c.byref(g)), "pm_batch_image")
        return r.value, g.value

    def read(self, i):
        """(radiance float32 [pixels, 4], rgba uint8 [pixels, 4]) of scene i."""
        cf = self.cfgs[i]
        rad = np.zeros((cf.width * cf.height, 4), np.float32)
        rgba = np.zeros((cf.width * cf.height, 4), np.uint8)
        self.ctx._check(self.lib.pm_batch_read(self.h, i, rad.ctypes.data, rgba.ctypes.data),
                        "pm_batch_read")
        return rad, rgba

    def stats(self, i):
        st = FrameStats()
        self.ctx._check(self.lib.pm_batch_stats(self.h, i, _c.byref(st)), "pm_batch_stats")
        return st

    def set_tune(self, i, leaf_size=32, tile=1, collect_max=128, merge_min=16, query_list=1):
        t = BatchTune(leaf_size, tile, collect_max, merge_min, query_list)
        self.ctx._check(self.lib.pm_batch_set_tune(self.h, i, _c.byref(t)), "pm_batch_set_tune")

    def get_tune(self, i):
        t = BatchTune()
        self.ctx._check(self.lib.pm_batch_get_tune(self.h, i, _c.byref(t)), "pm_batch_get_tune")
        return t

    def autotune(self, json_path=None, stream=0):
        self.ctx._check(self.lib.pm_batch_autotune(
            self.h, json_path.encode() if json_path else None, stream), "pm_batch_autotune")

    def cache_enable(self, cfg=None, **overrides):
        """Per-scene radiance caches (pm_batch_cache_enable); overrides set
        fields of the default (or given) CacheConfig."""
        if cfg is None:
            cfg = cache_default_config()
        for k, v in overrides.items():
            setattr(cfg, k, v)
        self.ctx._check(self.lib.pm_batch_cache_enable(self.h, _c.byref(cfg)), "pm_batch_cache_enable")
        return cfg

    def cache_disable(self):
        self.ctx._check(self.lib.pm_batch_cache_disable(self.h), "pm_batch_cache_disable")


def cache_default_config():
    cfg = CacheConfig()
    load().pm_cache_default_config(_c.byref(cfg))
    return cfg


def write_ppm(path, rgba):
    """rgba: uint8 [h, w, 4] host array."""
    a = np.ascontiguousarray(rgba, np.uint8)
    s = load().pm_write_ppm(path.encode(), a.ctypes.data, a.shape[1], a.shape[0])
    if s != PM_OK:
        raise PMError("pm_write_ppm(%s)" % path)


def write_png(path, rgba):
    """rgba: uint8 [h, w, 4] host array (alpha dropped)."""
    a = np.ascontiguousarray(rgba, np.uint8)
    s = load().pm_write_png(path.encode(), a.ctypes.data, a.shape[1], a.shape[0])
    if s != PM_OK:
        raise PMError("pm_write_png(%s)" % path)


def preset(which, seed=0x5EED0000):
    """Benchmark preset `which` (1, 2, 3): returns (Scene, Config)."""
    sc, cf = Scene(), Config()
    s = load().pm_preset(which, seed, _c.byref(sc), _c.byref(cf))
    if s != PM_OK:
        raise PMError("pm_preset(%d): %s" % (which, load().pm_status_string(s).decode()))
    return sc, cf


# The reference's three exports (photonMappingKernel.cu:1523,1549,1569).
def launch_init_random_numbers_kernel():
    load().launch_init_random_numbers_kernel()


def launch_emit_photons_kernel(pos, image_width, image_height, animTime, interpolateFlag,
                               participatingMediaFlag):
    load().launch_emit_photons_kernel(pos, image_width, image_height, animTime,
                                      bool(interpolateFlag), bool(participatingMediaFlag))


def launch_photon_mapping_kernel(pos, image_width, image_height, animTime, interpolateFlag,
                                 participatingMediaFlag):
    load().launch_photon_mapping_kernel(pos, image_width, image_height, animTime,
                                        bool(interpolateFlag), bool(participatingMediaFlag))
