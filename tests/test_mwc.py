"""Jump-ahead of the reference's Marsaglia generator
(photonMappingKernel.cu:1029-1036), which the GPU uses to fill the random
table and to position each photon's medium draws in parallel."""
import numpy as np

AZ, AW = 36969, 18000
MZ, MW = AZ * 65536 - 1, AW * 65536 - 1


def step(z, a):
    return (a * (z & 65535) + (z >> 16)) & 0xFFFFFFFF


def jump(z, a, m, n):
    return (pow(a, n, m) * z) % m


def test_jump_equals_serial_steps():
    for seed, a, m in [(316, AZ, MZ), (6548, AW, MW), (1, AZ, MZ), (MZ - 1, AZ, MZ)]:
        z = seed
        for n in range(1, 5000):
            z = step(z, a)
            assert z == jump(seed, a, m, n), (seed, n)


def test_jump_composes():
    z = 316
    for n in [3, 30000, 90000, 10 ** 9]:
        assert jump(jump(z, AZ, MZ, n), AZ, MZ, 7) == jump(z, AZ, MZ, n + 7)
