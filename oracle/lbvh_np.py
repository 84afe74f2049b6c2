"""Test infrastructure (oracle): numpy statement of the reference's LBVH arithmetic, used to
check GPU builds at sizes the host reference build is too slow for.

  morton_codes   BVH.cuh:92-97 (AABB, centroid), Bound.cuh:169-175 (offset), BVH.cuh:101-116,
                 134-137 (x1024, truncation, 10-bit interleave)
  karras_topology  BVH.cuh:173-236 (delta with the +40 index tie-break, lMax = 128*4^k,
                 ceil-halving split search), vectorised over all interior nodes
  flatten        BVH.cuh:311-329 (interior 0..N-2, leaves N-1..2N-2)
Pinned against the reference's own dumps by tests/test_lbvh_gpu.py and tests/test_port.py.
"""
import numpy as np


def tri_bounds(tris):
    t = np.asarray(tris, np.float32).reshape(-1, 3, 3)
    return t.min(axis=1), t.max(axis=1)


def _shift3(x):
    x = x.astype(np.uint32)
    x[x == 1024] = 1023
    x = (x | (x << 16)) & np.uint32(0b00000011000000000000000011111111)
    x = (x | (x << 8)) & np.uint32(0b00000011000000001111000000001111)
    x = (x | (x << 4)) & np.uint32(0b00000011000011000011000011000011)
    x = (x | (x << 2)) & np.uint32(0b00001001001001001001001001001001)
    return x


def morton_codes(tris, code_limit=-1):
    mn, mx = tri_bounds(tris)
    gmn, gmx = mn.min(axis=0), mx.max(axis=0)
    c = mn * np.float32(0.5) + mx * np.float32(0.5)
    o = (c - gmn).astype(np.float32)
    ext = (gmx - gmn).astype(np.float32)
    for k in range(3):
        if gmx[k] > gmn[k]:
            o[:, k] = o[:, k] / ext[k]
    s = (np.float32(1024) * o).astype(np.float32)
    q = s.astype(np.uint32)  # truncation toward zero; values lie in [0, 1024]
    codes = _shift3(q[:, 0]) | (_shift3(q[:, 1]) << np.uint32(1)) | (_shift3(q[:, 2]) << np.uint32(2))
    ids = np.arange(len(codes), dtype=np.int32)
    if code_limit >= 0:
        codes[code_limit:] = 0
        ids[code_limit:] = 0
    return codes.astype(np.uint32), ids


def stable_sort(codes, ids):
    order = np.argsort(codes, kind="stable")
    return codes[order], ids[order]


def _clz32(x):
    x = x.astype(np.uint64)
    out = np.full(x.shape, 32, np.int64)
    nz = x != 0
    _, e = np.frexp(x[nz].astype(np.float64))  # x = m * 2^e, m in [0.5, 1): msb index = e - 1
    out[nz] = 32 - e
    return out


def _delta(codes, i, j):
    n = len(codes)
    ok = (j >= 0) & (j < n)
    jj = np.where(ok, j, 0)
    x = codes[i].astype(np.uint64) ^ codes[jj].astype(np.uint64)
    tie = x == 0
    xi = np.where(tie, (i ^ jj).astype(np.uint64) & 0xFFFFFFFF, x)
    d = _clz32(xi) + np.where(tie, 40, 0)
    return np.where(ok, d, -1)


def karras_topology(codes):
    """(left, right) of every interior node in flattened indices (leaf l -> N-1+l)."""
    n = len(codes)
    i = np.arange(n - 1, dtype=np.int64)
    d = np.where(_delta(codes, i, i + 1) - _delta(codes, i, i - 1) > 0, 1, -1)
    dmin = _delta(codes, i, i - d)
    lmax = np.full(n - 1, 128, np.int64)
    while True:
        grow = _delta(codes, i, i + lmax * d) > dmin
        if not grow.any():
            break
        lmax[grow] *= 4
    l = np.zeros(n - 1, np.int64)
    t = lmax // 2
    while (t >= 1).any():
        act = t >= 1
        ok = act & (_delta(codes, i, i + (l + t) * d) > dmin)
        l[ok] += t[ok]
        t = np.where(act, t // 2, 0)
    j = i + l * d
    dnode = _delta(codes, i, j)
    s = np.zeros(n - 1, np.int64)
    t = (l + 1) // 2
    while (t >= 1).any():
        act = t >= 1
        ok = act & (_delta(codes, i, i + (s + t) * d) > dnode)
        s[ok] += t[ok]
        t = np.where(act, np.where(t == 1, 0, (t + 1) // 2), 0)
    gamma = i + s * d + np.minimum(d, 0)
    lo, hi = np.minimum(i, j), np.maximum(i, j)
    left = np.where(lo == gamma, n - 1 + gamma, gamma)
    right = np.where(hi == gamma + 1, n - 1 + gamma + 1, gamma + 1)
    return left.astype(np.int32), right.astype(np.int32)


def check_tree(left, right, bounds, leaf_bounds):
    """Structural checks of a flattened LBVH: every non-root node has exactly one parent, every
    interior box is the union of its children's boxes and every leaf box is its primitive's."""
    n = len(leaf_bounds)
    nodes = 2 * n - 1
    parents = np.zeros(nodes, np.int64)
    np.add.at(parents, left[: n - 1], 1)
    np.add.at(parents, right[: n - 1], 1)
    assert parents[0] == 0 and np.all(parents[1:] == 1), "not a binary tree over all nodes"
    b = bounds.reshape(-1, 6)
    lb, rb = b[left[: n - 1]], b[right[: n - 1]]
    union = np.concatenate([np.minimum(lb[:, :3], rb[:, :3]), np.maximum(lb[:, 3:], rb[:, 3:])], axis=1)
    assert np.array_equal(union.view(np.uint32), b[: n - 1].view(np.uint32)), "interior box != union of children"
    assert np.array_equal(b[n - 1:].view(np.uint32), leaf_bounds.view(np.uint32)), "leaf box != primitive box"
