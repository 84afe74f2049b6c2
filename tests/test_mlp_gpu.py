"""Radiance-cache MLP on the tensor cores: operand-layout products, forward and gradients
against a numpy FP32 statement of the same network (the CPU oracle of the learned part)."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def to_bf16_bits(x):
    u = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    return ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)


def from_bf16_bits(b):
    return (b.astype(np.uint32) << 16).view(np.float32)


@pytest.fixture(scope="module")
def ctx(built_lib):
    import lighttransportsimulation_gb300 as lts
    c = lts.Context(0)
    yield c
    c.close()


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_umma_operand_layouts(ctx, mode):
    """One tcgen05 product per operand arrangement equals the FP32 product of the bf16 inputs."""
    rng = np.random.default_rng(mode)
    shapes = {0: ((128, 64), (64, 64)), 1: ((128, 64), (64, 96)), 2: ((128, 96), (128, 64))}
    (ar, ac), (br, bc) = shapes[mode]
    a = to_bf16_bits(rng.standard_normal((ar, ac)).astype(np.float32))
    b = to_bf16_bits(rng.standard_normal((br, bc)).astype(np.float32))
    af, bf = from_bf16_bits(a).astype(np.float64), from_bf16_bits(b).astype(np.float64)
    want = {0: lambda: af @ bf.T, 1: lambda: af @ bf, 2: lambda: af.T @ bf}[mode]()
    res = {}
    for swap in (0, 1):
        d = np.zeros((128, 96 if mode == 1 else 64), np.float32)
        ctx.check(ctx.lib.lts_debug_umma_probe(ctx.h, mode, swap, a.ctypes.data_as(ctypes.c_void_p),
                                                b.ctypes.data_as(ctypes.c_void_p), d.ctypes.data_as(ctypes.c_void_p)))
        got = d[:want.shape[0]]
        res[swap] = np.max(np.abs(got - want)) / np.max(np.abs(want))
    print(f"mode {mode}: max rel err, offsets as documented {res[0]:.2e}, swapped {res[1]:.2e}")
    assert res[0] < 1e-5
