"""Generate Philox4x32-10 vectors from an independent implementation.

Runs Triton's own Philox4x32-10 (`triton.language.philox_impl`, 10 rounds)
in Triton's CPU interpreter on the all-zero and all-ones counter/key
patterns and 256 seeded random (counter, key) pairs, and writes
tests/golden/philox_triton.npz. The vectors check the generator the GPU
kernels and the CPU oracle share (include/pm_math.h, pm_philox4x32_10)
against code written by someone else (tests/test_physical_oracle.py).

Usage: python tests/golden/make_philox_golden.py   (needs triton and torch)
"""
import os

os.environ["TRITON_INTERPRET"] = "1"  # before triton is imported: run on the CPU

import numpy as np  # noqa: E402
import torch  # noqa: E402
import triton  # noqa: E402
import triton.language as tl  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))


@triton.jit
def _philox_kernel(ctr_ptr, key_ptr, out_ptr, N: tl.constexpr):
    i = tl.arange(0, N)
    c0 = tl.load(ctr_ptr + 4 * i + 0)
    c1 = tl.load(ctr_ptr + 4 * i + 1)
    c2 = tl.load(ctr_ptr + 4 * i + 2)
    c3 = tl.load(ctr_ptr + 4 * i + 3)
    k0 = tl.load(key_ptr + 2 * i + 0)
    k1 = tl.load(key_ptr + 2 * i + 1)
    r0, r1, r2, r3 = tl.philox_impl(c0, c1, c2, c3, k0, k1, 10)
    tl.store(out_ptr + 4 * i + 0, r0)
    tl.store(out_ptr + 4 * i + 1, r1)
    tl.store(out_ptr + 4 * i + 2, r2)
    tl.store(out_ptr + 4 * i + 3, r3)


def inputs():
    rs = np.random.RandomState(0x9411)
    n = 256
    ctr = np.zeros((n + 2, 4), np.uint32)
    key = np.zeros((n + 2, 2), np.uint32)
    ctr[1] = 0xFFFFFFFF
    key[1] = 0xFFFFFFFF
    ctr[2:] = rs.randint(0, 2 ** 32, (n, 4), dtype=np.uint64).astype(np.uint32)
    key[2:] = rs.randint(0, 2 ** 32, (n, 2), dtype=np.uint64).astype(np.uint32)
    return ctr, key


def main():
    ctr, key = inputs()
    n = len(ctr)
    size = 1 << (n - 1).bit_length()  # tl.arange wants a power of two
    c = torch.zeros((size, 4), dtype=torch.uint32)
    k = torch.zeros((size, 2), dtype=torch.uint32)
    c[:n] = torch.from_numpy(ctr.view(np.int32)).view(torch.uint32)
    k[:n] = torch.from_numpy(key.view(np.int32)).view(torch.uint32)
    out = torch.zeros((size, 4), dtype=torch.uint32)
    _philox_kernel[(1,)](c, k, out, N=size)
    res = out[:n].view(torch.int32).numpy().view(np.uint32)
    path = os.path.join(HERE, "philox_triton.npz")
    np.savez_compressed(path, ctr=ctr, key=key, out=res, source=np.array("triton %s philox_impl, 10 rounds, "
                                                                         "CPU interpreter" % triton.__version__))
    print("wrote %s (%d vectors)" % (path, n))


if __name__ == "__main__":
    main()
