"""GPU known-answer tests: the renderer's float device functions (lts_debug_kat, one record per
thread on cuda:0) against the reference's own functions on the same inputs
(tests/golden/kat_reference.npz, made by oracle/_ref/lts_ref kat from the reference's sources).

Tolerance: the FP32 parity bar, 1e-4 relative, plus 1e-6 absolute for values near zero.
The device code rounds with FMA contraction and CUDA's transcendentals, the reference's host
build without FMA and with glibc's, so values agree to a few ulps, not bit for bit; the worst
relative error of each function is printed."""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from test_oracle import KAT_FUNCS, kat_compare_mask

pytestmark = pytest.mark.gpu

RTOL, ATOL = 1e-4, 1e-6


@pytest.fixture(scope="module")
def ctx(built_lib):
    import lighttransportsimulation_gb300 as lts
    c = lts.Context(0)
    yield c
    c.close()


@pytest.mark.parametrize("name", list(KAT_FUNCS))
def test_device_function_matches_reference(ctx, name):
    import ctypes
    z = np.load(os.path.join(GOLDEN, "kat_reference.npz"))
    a = np.ascontiguousarray(z[f"in_{name}"], np.float32)
    ref = z[f"out_{name}"]
    got = np.zeros_like(ref)
    ctx.check(ctx.lib.lts_debug_kat(ctx.h, KAT_FUNCS[name], ctypes.c_void_p(a.ctypes.data), len(a),
                                    ctypes.c_void_p(got.ctypes.data)))
    m = kat_compare_mask(name, ref)
    err = np.abs(got - ref)
    tol = RTOL * np.abs(ref) + ATOL
    rel = np.where(m, err / (np.abs(ref) + ATOL), 0)
    print(f"{name}: max relative error {rel.max():.3g}, bit-exact {np.mean((got.view(np.uint32) == ref.view(np.uint32)) | ~m):.4f}")
    assert np.isfinite(got[m]).all()
    assert np.all((err <= tol) | ~m)
