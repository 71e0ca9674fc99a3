"""Generate the legacy-mode golden vectors from the reference's own code.

Builds oracle/_ref/libpmref.so from the reference checkout (oracle/ref.mk),
runs the reference's frame sequence serially on this machine's CPU and
writes tests/golden/legacy_ref.npz. The vectors pin the C restatement in
oracle/legacy_oracle.c (tests/test_oracle_golden.py) and, through it, the
GPU kernels.

Usage: python tests/golden/make_golden.py [--ref /path/to/reference]
"""
import argparse
import ctypes
import hashlib
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))

# (animTime, interpolateFlag, participatingMediaFlag, width, height):
# the four keyboard modes of callbacksPBO.cpp:104-143 at animTime 0, two
# animated frames, and a non-square image size.
FRAMES = [
    (0.0, 0, 0, 512, 512),
    (0.0, 1, 0, 512, 512),
    (0.0, 0, 1, 512, 512),
    (0.0, 1, 1, 512, 512),
    (0.7, 0, 1, 512, 512),
    (2.3, 1, 0, 512, 512),
    (0.0, 0, 0, 300, 200),
]


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def load_ref(ref_dir):
    subprocess.check_call(["make", "-s", "-f", "oracle/ref.mk", "REF=" + ref_dir], cwd=ROOT)
    lib = ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", "libpmref.so"))
    for n in ["ref_get_grid", "ref_get_random_numbers", "ref_get_rng_state", "ref_get_spheres"]:
        getattr(lib, n).argtypes = [ctypes.c_void_p]
    lib.ref_emit.argtypes = [ctypes.c_float, ctypes.c_int, ctypes.c_int]
    lib.ref_render.argtypes = [ctypes.c_uint, ctypes.c_uint, ctypes.c_float, ctypes.c_int,
                               ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    return lib


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("PM_REFERENCE_DIR")
                    or os.path.join(os.path.dirname(ROOT), "reference"),
                    help="reference checkout (default: $PM_REFERENCE_DIR, else ../reference)")
    args = ap.parse_args()
    lib = load_ref(args.ref)
    out = {}

    # Sequence A: the reference's own start-up order (simplePBO.cpp:203 runs
    # one emission before callbacksPBO.cpp:55 fills the random table).
    lib.ref_reset()
    lib.ref_emit(0.0, 0, 0)
    g = np.zeros((32, 32, 32, 3), np.float32)
    lib.ref_get_grid(g.ctypes.data)
    img = np.zeros((512, 512, 4), np.uint8)
    rgb = np.zeros((512, 512, 3), np.float32)
    lib.ref_render(512, 512, 0.0, 0, 0, img.ctypes.data, rgb.ctypes.data)
    out["pre_init_grid_sha"] = sha(g)
    out["pre_init_img_sha"] = sha(img)

    # Sequence B: init once, then FRAMES in order (emit + render each).
    lib.ref_reset()
    lib.ref_init_random_numbers()
    table = np.zeros((10000, 3), np.float32)
    lib.ref_get_random_numbers(table.ctypes.data)
    st = np.zeros(2, np.uint32)
    lib.ref_get_rng_state(st.ctypes.data)
    out["table_sha"] = sha(table)
    out["table_head"] = table[:64].copy()
    out["rng_after_init"] = st.copy()
    out["frames"] = np.array(FRAMES, np.float64)
    for i, (t, interp, media, w, h) in enumerate(FRAMES):
        lib.ref_emit(t, interp, media)
        lib.ref_get_grid(g.ctypes.data)
        img = np.zeros((h, w, 4), np.uint8)
        rgb = np.zeros((h, w, 3), np.float32)
        lib.ref_render(w, h, t, interp, media, img.ctypes.data, rgb.ctypes.data)
        lib.ref_get_rng_state(st.ctypes.data)
        if i in (0, 2):
            out["f%d_grid" % i] = g.copy()
        out["f%d_grid_sha" % i] = sha(g)
        out["f%d_img_sha" % i] = sha(img)
        out["f%d_rgb_sha" % i] = sha(rgb)
        out["f%d_img_sub" % i] = img[::8, ::8].copy()
        out["f%d_rng" % i] = st.copy()
        print("frame", i, (t, interp, media, w, h), "grid sum %.3f" % g.sum(dtype=np.float64),
              "img mean %.3f" % img[..., :3].mean())
    path = os.path.join(HERE, "legacy_ref.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    sys.exit(main())
