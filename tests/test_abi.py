"""The C ABI library loads on a machine without a GPU and exports every
entry point include/pm.h declares; calls that need no GPU behave."""
import ctypes
import os
import re
import subprocess
import sys

import photonmap

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = []
    for h in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if h.endswith(".h"):
            text = open(os.path.join(ROOT, "include", h)).read()
            names += re.findall(r"^PM_API[^(;]*?\b(\w+)\(", text, re.M)
    return names


def test_header_declares_reference_exports():
    names = declared_symbols()
    for n in ["launch_init_random_numbers_kernel", "launch_emit_photons_kernel",
              "launch_photon_mapping_kernel"]:
        assert n in names


def test_every_declared_symbol_is_exported():
    lib = ctypes.CDLL(photonmap.LIB_PATH)
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing


def test_bindings_cover_header():
    assert set(declared_symbols()) <= set(photonmap.PROTOTYPES)


def test_status_strings():
    lib = photonmap.load()
    assert lib.pm_status_string(0) == b"ok"
    assert lib.pm_status_string(5).startswith(b"size")


def test_create_rejects_bad_device():
    lib = photonmap.load()
    h = ctypes.c_void_p()
    assert lib.pm_create(ctypes.byref(h), -1) == 1
    assert lib.pm_create(None, 0) == 1


def test_reference_exports_exit_like_the_reference_without_device():
    # checkCUDAError (photonMappingKernel.cu:49-55) prints and exits with
    # EXIT_FAILURE; on a machine without a usable GPU the exports do the same.
    code = ("import sys; sys.path.insert(0, %r); import photonmap; "
            "photonmap.launch_init_random_numbers_kernel(); print('survived')" % photonmap.PKG)
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env)
    assert r.returncode == 1
    assert "Cuda error" in r.stderr
    assert "survived" not in r.stdout


def test_reference_exports_record_error_when_asked():
    code = ("import sys; sys.path.insert(0, %r); import photonmap; lib = photonmap.load(); "
            "lib.pm_legacy_set_exit_on_error(0); photonmap.launch_init_random_numbers_kernel(); "
            "print(lib.pm_legacy_last_status())" % photonmap.PKG)
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env)
    assert r.returncode == 0, r.stderr
    assert int(r.stdout.strip().splitlines()[-1]) != 0


def test_struct_layouts_match_the_library():
    lib = photonmap.load()
    structs = [photonmap.Scene, photonmap.Config, photonmap.PhotonRecord, photonmap.FrameStats,
               photonmap.CacheConfig, photonmap.CacheStats]
    for which, st in enumerate(structs):
        assert lib.pm_abi_struct_size(which) == ctypes.sizeof(st), st.__name__


def test_cache_default_config():
    cfg = photonmap.cache_default_config()
    assert (cfg.levels, cfg.log2_table, cfg.base_res, cfg.max_res) == (16, 19, 16, 2048)
    assert cfg.train_samples == 1 << 20 and cfg.batch % 128 == 0


def test_batch_scene_generator_ranges():
    spheres, sig, photons, res, ks = [], [], [], set(), set()
    for i in range(64):
        sc, cf = photonmap.batch_scene(i)
        spheres.append(sc.num_spheres)
        sig.append(sc.sigma_s)
        photons.append(cf.surface_photons + cf.volume_photons if sc.sigma_s > 0 else 2 * cf.surface_photons)
        res.add((cf.width, cf.height))
        ks.add(cf.k)
        assert cf.scene_id == i
        assert cf.volume_photons == (cf.surface_photons if sc.sigma_s > 0 else 0)
    assert 2 <= min(spheres) and max(spheres) <= 32 and len(set(spheres)) > 10
    assert 0.0 <= min(sig) and max(sig) <= 0.2
    assert 1e5 * 0.99 <= min(photons) and max(photons) <= 4e6
    assert res == {(256, 256), (512, 512), (1024, 1024)}
    assert ks == {32, 64, 128}
    a, _ = photonmap.batch_scene(5)
    b, _ = photonmap.batch_scene(5)
    assert bytes(a) == bytes(b)
