"""Known-answer tests of the random-number generator every transport stream is drawn from:
Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as 1, 2, 3", SC'11),
against the published known-answer vectors of the Random123 library (counter, key -> output, 10
rounds).  The library's host copy (mqi_philox4x32_10, the same __host__ __device__ function the
kernels inline) and the oracle's restatement are checked on the CPU; the GPU test checks device
blocks against the host copy through the plan sampler, whose source vertices are a fixed function
of two Philox blocks per history.
"""
import numpy as np
import pytest

from moquimc_gb300 import capi

# (counter[4], key[2]) -> output[4], Random123 philox4x32 10-round known answers
KAT = [
    ((0x00000000, 0x00000000, 0x00000000, 0x00000000), (0x00000000, 0x00000000),
     (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
    ((0xFFFFFFFF, 0xFFFFFFFF, 0xFFFFFFFF, 0xFFFFFFFF), (0xFFFFFFFF, 0xFFFFFFFF),
     (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
    ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
     (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
]


@pytest.mark.parametrize("ctr,key,expect", KAT)
def test_library_philox_known_answers(built_lib, ctr, key, expect):
    np.testing.assert_array_equal(capi.philox4x32_10(ctr, key), np.array(expect, np.uint32))


@pytest.mark.parametrize("ctr,key,expect", KAT)
def test_oracle_philox_known_answers(oracle, ctr, key, expect):
    np.testing.assert_array_equal(oracle.philox(ctr, key), np.array(expect, np.uint32))


def test_library_and_oracle_agree_on_random_blocks(built_lib, oracle):
    rng = np.random.default_rng(123)
    for _ in range(200):
        c = rng.integers(0, 2 ** 32, 4, dtype=np.uint64).astype(np.uint32)
        k = rng.integers(0, 2 ** 32, 2, dtype=np.uint64).astype(np.uint32)
        np.testing.assert_array_equal(capi.philox4x32_10(c, k), oracle.philox(c, k))


def test_philox_rejects_null_pointers(built_lib):
    assert built_lib.mqi_philox4x32_10(None, None, None) == capi.MQI_ERR_INVALID


def _u01(w):
    return ((w >> np.uint32(8)).astype(np.float64) + 0.5) / 16777216.0


@pytest.mark.gpu
def test_device_blocks_match_the_host_copy(gpu_ctx_factory):
    """mqi_sample_plan draws history h's vertex from the blocks (0, h, ~0, ~0) and (1, h, ~0, ~0)
    under the plan's source key (the run seed with its high word XOR 0xA5A5A5A5): six Box-Muller normals z = sqrt(-2 ln u(w2k)) * {cos, sin}(2 pi u(w2k+1)).
    With unit sigmas, no correlation, an identity frame and a unit energy spread, the vertex is the
    normals themselves: x = z0, x' = z1, y = z2, y' = z3, z = z4, E = 100 + z5.  A wrong word or
    round would move them by O(1); the tolerance covers the device's and numpy's libm."""
    n, seed = 4096, 0x1234_5678_9ABC_DEF0
    sp = np.zeros(1, capi.SPOT_DTYPE)
    sp["energy"] = 100.0
    sp["energy_sigma"] = 1.0
    sp["sigma"][0, :] = (1.0, 1.0, 1.0, 0.01, 0.01)
    sp["rot"] = np.eye(3, dtype=np.float32).ravel()
    sp["histories"] = n
    c = gpu_ctx_factory()
    c.set_spot_plan(sp)
    v, spots = c.sample_plan(0, n, seed)
    k = (seed & 0xFFFFFFFF, (seed >> 32) ^ 0xA5A5A5A5)
    z = np.zeros((n, 6))
    for h in range(n):
        w = np.concatenate([capi.philox4x32_10((0, h, 0xFFFFFFFF, 0xFFFFFFFF), k),
                            capi.philox4x32_10((1, h, 0xFFFFFFFF, 0xFFFFFFFF), k)[:2]])
        u = _u01(w)
        r = np.sqrt(-2.0 * np.log(u[0::2]))
        z[h, 0::2] = r * np.cos(2.0 * np.pi * u[1::2])
        z[h, 1::2] = r * np.sin(2.0 * np.pi * u[1::2])
    np.testing.assert_allclose(v["pos"][:, 0], z[:, 0], atol=2e-5, rtol=2e-5)
    np.testing.assert_allclose(v["pos"][:, 1], z[:, 2], atol=2e-5, rtol=2e-5)
    np.testing.assert_allclose(v["pos"][:, 2], z[:, 4], atol=2e-5, rtol=2e-5)
    np.testing.assert_allclose(v["dir"][:, 0], 0.01 * z[:, 1], atol=2e-7, rtol=2e-5)
    np.testing.assert_allclose(v["dir"][:, 1], 0.01 * z[:, 3], atol=2e-7, rtol=2e-5)
    np.testing.assert_allclose(v["ke"], 100.0 + z[:, 5], atol=2e-5, rtol=0)
