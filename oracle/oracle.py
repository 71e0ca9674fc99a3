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
