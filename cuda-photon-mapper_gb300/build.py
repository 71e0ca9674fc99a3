"""Builds libphotonmap.so (the CUDA kernels and the C ABI of include/pm.h)
in-tree for sm_103a, plus the CPU oracle library used by the tests.

    python cuda-photon-mapper_gb300/build.py          # library + oracle
"""
import concurrent.futures as cf
import glob
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libphotonmap.so")
ORACLE_DIR = os.path.join(ROOT, "oracle")
ORACLE_LIB = os.path.join(ORACLE_DIR, "liboracle.so")
# The reference checkout, when present: $PM_REFERENCE_DIR, else a directory
# named `reference` beside the repository.
REF_DIR = os.environ.get("PM_REFERENCE_DIR") or os.path.join(os.path.dirname(ROOT), "reference")

NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-std=c++17", "-O3", "-lineinfo", "-fmad=false", "-Xcompiler", "-fPIC",
           "-Xcompiler", "-ffp-contract=off",
           "-Xcompiler", "-fvisibility=hidden", "-I", os.path.join(ROOT, "include"), "-I", CSRC]


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s" % (" ".join(cmd), r.stdout))
    return r.stdout


def build_library(force=False):
    os.makedirs(BUILD, exist_ok=True)
    sources = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    headers = glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(ROOT, "include", "*.h"))
    objs, jobs = [], []
    for src in sources:
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        objs.append(obj)
        if force or _newer(obj, [src] + headers):
            jobs.append([NVCC] + ARCH + NVFLAGS + ["-c", src, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        list(ex.map(_run, jobs))
    if force or jobs or _newer(LIB, objs):
        _run([NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"])
    return LIB


def build_oracle(force=False):
    sources = sorted(glob.glob(os.path.join(ORACLE_DIR, "*.c")))
    headers = glob.glob(os.path.join(ORACLE_DIR, "*.h"))
    if force or _newer(ORACLE_LIB, sources + headers):
        _run(["gcc", "-O2", "-std=gnu11", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC",
              "-shared", "-o", ORACLE_LIB] + sources + ["-lm"])
    return ORACLE_LIB


REF_CUBIN = os.path.join(ORACLE_DIR, "_ref", "ref_kernels.cubin")
REF_GPU_LIB = os.path.join(ORACLE_DIR, "_ref", "libpmref_gpu.so")


def build_reference():
    """Compiles the reference's own code into oracle/_ref (needs the checkout):
    its photon-mapping code as serial host C++ (the legacy oracle's pin) and
    its CUDA file unmodified as an sm_103a module (the measured reference-GPU
    bar; the module travels to GPU hosts, the checkout does not)."""
    if not os.path.isdir(REF_DIR):
        return None
    _run(["make", "-s", "-C", ROOT, "-f", "oracle/ref.mk", "REF=" + REF_DIR])
    src = os.path.join(REF_DIR, "photonMappingKernel.cu")
    shims = glob.glob(os.path.join(ORACLE_DIR, "ref_gpu", "*.h"))
    if _newer(REF_CUBIN, [src] + shims):
        _run([NVCC] + ARCH + ["-O3", "-cubin", "-w", "-I", os.path.join(ORACLE_DIR, "ref_gpu"), "-o",
                              REF_CUBIN, src])
    return os.path.join(ORACLE_DIR, "_ref", "libpmref.so")


def build_ref_gpu_runner():
    """The loader that times the reference's GPU module (oracle/ref_gpu_runner.cpp)."""
    src = os.path.join(ORACLE_DIR, "ref_gpu_runner.cpp")
    if not _newer(REF_GPU_LIB, [src]):
        return REF_GPU_LIB
    os.makedirs(os.path.dirname(REF_GPU_LIB), exist_ok=True)
    cuda = os.path.dirname(os.path.dirname(NVCC))
    _run(["g++", "-O2", "-fPIC", "-shared", "-I", os.path.join(cuda, "include"), src, "-o", REF_GPU_LIB,
          "-L", os.path.join(cuda, "lib64"), "-L", os.path.join(cuda, "lib64", "stubs"), "-lcudart",
          "-lcuda"])
    return REF_GPU_LIB


def build_all(force=False):
    build_library(force)
    build_oracle(force)
    build_reference()
    try:
        build_ref_gpu_runner()
    except RuntimeError as e:  # measurement infrastructure: never fails the product build
        print("build: reference-GPU runner not built:", str(e).splitlines()[0], file=sys.stderr)


if __name__ == "__main__":
    build_all(force="--force" in sys.argv)
    print("built", LIB, ORACLE_LIB)
