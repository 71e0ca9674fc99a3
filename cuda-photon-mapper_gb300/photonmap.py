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
