"""One tcgen05 MMA (128 x N x 16, BF16 operands from shared memory, FP32
accumulator in tensor memory) against a host product: checks the
descriptor encoders, the K-major canonical layout without swizzle (leading
offset = distance of core matrices along K, stride offset = along M/N) and
the accumulator's lane/column layout, before any GEMM relies on them."""
import ctypes

import numpy as np
import pytest

from elastic_gb300._lib import load

pytestmark = pytest.mark.gpu


def to_bf16_bits(x):
    """float32 -> bfloat16 bit patterns, round to nearest even."""
    b = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) >> 16
    return b.astype(np.uint16)


def from_bf16_bits(h):
    return (h.astype(np.uint32) << 16).view(np.float32)


def probe(N, lbo, sbo, A, B):
    D = np.zeros((128, N), np.float32)
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    st = load().rtm_debug_umma_probe(N, lbo, sbo, P(A), P(B), P(D))
    assert st == 0, load().rtm_last_error()
    return D


@pytest.mark.parametrize("N", [64, 128, 256])
def test_umma_probe_matches_host_product(N):
    rng = np.random.default_rng(N)
    A = to_bf16_bits(rng.standard_normal((128, 16)))
    B = to_bf16_bits(rng.standard_normal((N, 16)))
    want = from_bf16_bits(A).astype(np.float64) @ from_bf16_bits(B).astype(np.float64).T
    got = probe(N, 128, 256, A, B)
    err = np.linalg.norm(got - want) / np.linalg.norm(want)
    swapped = probe(N, 256, 128, A, B)
    err_sw = np.linalg.norm(swapped - want) / np.linalg.norm(want)
    print("N=%d: rel. L2 with (LBO=128 along K, SBO=256 along M/N) %.2e, swapped %.2e" % (N, err, err_sw))
    assert err < 1e-6


@pytest.mark.parametrize("K", [64, 32])
@pytest.mark.parametrize("N", [32, 96, 256])
def test_umma_swizzled_probe_matches_host_product(N, K):
    """The swizzled K-major layouts of the convolution kernels (128-byte
    swizzle for 64-channel chunks, 64-byte for 32-channel chunks) with the
    descriptor advanced 32 bytes per 16-wide K step."""
    rng = np.random.default_rng(N + K)
    A = to_bf16_bits(rng.standard_normal((128, K)))
    B = to_bf16_bits(rng.standard_normal((N, K)))
    want = from_bf16_bits(A).astype(np.float64) @ from_bf16_bits(B).astype(np.float64).T
    D = np.zeros((128, N), np.float32)
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    st = load().rtm_debug_umma_probe_sw(N, K, P(A), P(B), P(D))
    assert st == 0, load().rtm_last_error()
    err = np.linalg.norm(D - want) / np.linalg.norm(want)
    print("N=%d K=%d swizzled: rel. L2 %.2e" % (N, K, err))
    assert err < 1e-6
