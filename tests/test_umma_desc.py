"""The tcgen05 descriptor encoders (elastic_gb300/csrc/umma.cuh) against the
PTX ISA field layouts, on the CPU, before any kernel uses them.

Instruction descriptor for .kind::f16: bits 4-5 D type (1 = F32), 7-9 A
type and 10-12 B type (1 = BF16), 15/16 A/B major (0 = K-major), 17-22 N/8,
24-28 M/16, everything else zero for a dense, unnegated, unsaturated MMA.
Shared-memory matrix descriptor: bits 0-13 start address / 16, 16-29 leading
byte offset / 16, 32-45 stride byte offset / 16, 46-47 the constant 0b01,
61-63 the swizzle mode."""
import ctypes

import numpy as np
import pytest

from elastic_gb300._lib import load


def idesc_ref(M, N, bf16=True, f32=True):
    d = 0
    d |= (1 if f32 else 0) << 4
    d |= (1 if bf16 else 0) << 7
    d |= (1 if bf16 else 0) << 10
    d |= (N // 8) << 17
    d |= (M // 16) << 24
    return d


def sdesc_ref(addr, lbo, sbo, swizzle=0):
    return ((addr & 0x3FFFF) >> 4) | ((lbo >> 4) << 16) | ((sbo >> 4) << 32) | (1 << 46) | (swizzle << 61)


def encode(M, N, bf16, f32, addr, lbo, sbo, sw):
    out = np.zeros(2, np.uint64)
    assert load().rtm_debug_umma_desc(M, N, int(bf16), int(f32), addr, lbo, sbo, sw,
                                      out.ctypes.data_as(ctypes.c_void_p)) == 0
    return int(out[0]), int(out[1])


@pytest.mark.parametrize("M", [64, 128])
@pytest.mark.parametrize("N", [16, 32, 64, 96, 128, 256])
def test_instruction_descriptor(M, N):
    i, _ = encode(M, N, True, True, 0, 16, 16, 0)
    assert i == idesc_ref(M, N)
    # field by field
    assert (i >> 4) & 3 == 1 and (i >> 7) & 7 == 1 and (i >> 10) & 7 == 1
    assert (i >> 15) & 3 == 0 and (i >> 17) & 63 == N // 8 and (i >> 24) & 31 == M // 16
    assert i & 0b1111 == 0 and (i >> 13) & 3 == 0 and (i >> 23) & 1 == 0 and (i >> 29) == 0
    i16, _ = encode(M, N, False, False, 0, 16, 16, 0)
    assert i16 == idesc_ref(M, N, bf16=False, f32=False)


@pytest.mark.parametrize("addr,lbo,sbo,sw", [(0, 128, 256, 0), (0x400, 128, 1024, 0), (0x2FFF0, 256, 128, 0),
                                             (0x1000, 16, 1024, 2)])
def test_shared_memory_descriptor(addr, lbo, sbo, sw):
    _, s = encode(128, 64, True, True, addr, lbo, sbo, sw)
    assert s == sdesc_ref(addr, lbo, sbo, sw)
    assert s & 0x3FFF == (addr >> 4) & 0x3FFF
    assert (s >> 16) & 0x3FFF == lbo >> 4 and (s >> 32) & 0x3FFF == sbo >> 4
    assert (s >> 46) & 3 == 1 and (s >> 49) & 7 == 0 and (s >> 52) & 1 == 0 and (s >> 61) == sw
