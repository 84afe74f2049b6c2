"""GPU test of the allocation-free LBVH entry point (lts_bvh_build_noalloc).

It exists for callers that may not allocate device memory -- code running inside an allocator or
memory-pool callback, render loops that forbid cudaMalloc/cudaFree because they synchronise the
device, plugins whose host application owns every allocation.  It keeps its scratch in one fixed
device array, so this test checks, through the C-ABI, that two calls in a row give exactly the
output of the allocating entry point for the same inputs, and that sizes beyond the array's limit
are refused.  The file is named to be collected last.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LIMIT = 262144  # LTS_NOALLOC_MAX_PRIMITIVES


def _canonical(n, nodes_raw, root):
    """Raw 64-byte nodes -> the reference's flattened arrays (interior 0..n-2, leaves n-1..2n-2)."""
    f = nodes_raw.view(np.float32).reshape(-1, 16)
    d = nodes_raw.view(np.int32).reshape(-1, 16)[:, 12:16]
    flat = lambda c: np.where(c < 0, (n - 1) + ~c, c)
    nodes = 2 * n - 1
    left = np.full(nodes, -1, np.int32)
    right = np.full(nodes, -1, np.int32)
    bounds = np.zeros((nodes, 6), np.float32)
    bounds[0] = root
    if n > 1:
        lc, rc = flat(d[:, 0]), flat(d[:, 1])
        left[: n - 1], right[: n - 1] = lc, rc
        bounds[lc] = f[:, 0:6]
        bounds[rc] = f[:, 6:12]
    return left, right, bounds.reshape(-1)


def _noalloc(lib, tris, mode, code_limit):
    import torch
    n = tris.shape[0]
    t = torch.from_numpy(np.ascontiguousarray(tris.reshape(-1))).cuda()
    codes = torch.empty(n, dtype=torch.int32, device="cuda")
    ids = torch.empty(n, dtype=torch.int32, device="cuda")
    nodes = torch.empty(max(n - 1, 1) * 16, dtype=torch.int32, device="cuda")
    leaf = torch.empty(n, dtype=torch.int32, device="cuda")
    root = torch.empty(6, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    rc = lib.lts_bvh_build_noalloc(ctypes.c_void_p(t.data_ptr()), n, mode, code_limit,
                                   ctypes.c_void_p(codes.data_ptr()), ctypes.c_void_p(ids.data_ptr()),
                                   ctypes.c_void_p(nodes.data_ptr()), ctypes.c_void_p(leaf.data_ptr()),
                                   ctypes.c_void_p(root.data_ptr()), None)
    assert rc == 0, rc
    return (codes.cpu().numpy().view(np.uint32), ids.cpu().numpy(), nodes.cpu().numpy()[: (n - 1) * 16],
            leaf.cpu().numpy(), root.cpu().numpy())


@pytest.mark.parametrize("first", [(50_000, 1, -1, 5)])
def test_noalloc_matches_allocating_build_twice(built_lib, first):
    import lighttransportsimulation_gb300 as lts
    from lighttransportsimulation_gb300 import scenes
    lib = lts.library()
    ctx = lts.Context(0)
    cases = [first, (120_001, 0, 65_536, 6)]  # two calls in a row: sorted mode, then reference mode
    for n, mode, limit, seed in cases:
        tris = scenes.random_triangles(n, seed=seed)
        want = lts.build_bvh_triangles(ctx, tris, mode, limit)
        codes, ids, nodes, leaf, root = _noalloc(lib, tris, mode, limit)
        assert np.array_equal(codes, want["sorted_codes"]) and np.array_equal(ids, want["sorted_ids"])
        left, right, bounds = _canonical(n, nodes, root)
        assert np.array_equal(left, want["node_left"]) and np.array_equal(right, want["node_right"])
        assert np.array_equal(bounds.view(np.uint32), want["node_bounds"].view(np.uint32))
        assert np.array_equal(leaf, np.arange(n) if mode == 0 else want["sorted_ids"])
    ctx.close()


def test_noalloc_rejects_sizes_beyond_its_array(built_lib):
    import lighttransportsimulation_gb300 as lts
    lib = lts.library()
    one = ctypes.c_void_p(1)
    assert lib.lts_bvh_build_noalloc(one, LIMIT + 1, 1, -1, one, one, one, one, one, None) == 1
    assert lib.lts_bvh_build_noalloc(one, 0, 1, -1, one, one, one, one, one, None) == 1
