"""Decoder and structural checker of the compressed wide-BVH layout (test helper).

Node of width W: 24-byte header {float p[3]; u8 e[3]; u8 imask; u32 child_base;
u32 tri_base}, meta[W], qlo[3][W], qhi[3][W], padded to 16 bytes.  Internal
slots have meta low 5 bits = 24 + octant code; leaf slots have
meta = unary(count) << 5 | triangle offset.
"""
from __future__ import annotations

import numpy as np


def node_bytes(W):
    return ((24 + 7 * W) + 15) // 16 * 16


def decode(wide: np.ndarray, W: int):
    nb = node_bytes(W)
    n = wide.size // nb
    raw = wide.reshape(n, nb)
    p = raw[:, 0:12].copy().view(np.float32).reshape(n, 3)
    e = raw[:, 12:15].astype(np.int32) - 127
    imask = raw[:, 15]
    child_base = raw[:, 16:20].copy().view(np.uint32).reshape(n)
    tri_base = raw[:, 20:24].copy().view(np.uint32).reshape(n)
    meta = raw[:, 24:24 + W]
    qlo = raw[:, 24 + W:24 + 4 * W].reshape(n, 3, W)
    qhi = raw[:, 24 + 4 * W:24 + 7 * W].reshape(n, 3, W)
    return dict(n=n, p=p, e=e, imask=imask, child_base=child_base, tri_base=tri_base, meta=meta, qlo=qlo, qhi=qhi)


def slot_box(d, k, s):
    scale = np.ldexp(1.0, d["e"][k])
    lo = d["p"][k].astype(np.float64) + scale * d["qlo"][k, :, s]
    hi = d["p"][k].astype(np.float64) + scale * d["qhi"][k, :, s]
    return lo, hi


def empty_slots_inverted(d, W):
    """Empty slots (meta 0) must carry qlo = 255, qhi = 0 on every axis."""
    empty = d["meta"] == 0
    return bool((d["qlo"].transpose(0, 2, 1)[empty] == 255).all() and (d["qhi"].transpose(0, 2, 1)[empty] == 0).all())


def children(d, k, W):
    """[(slot, kind, index, count)] kind 'node' (index = child node) or 'tris' (index = first slot)."""
    out = []
    for s in range(W):
        m = int(d["meta"][k, s])
        if m == 0:
            continue
        lo5 = m & 31
        if lo5 >= 24:
            code = lo5 - 24
            assert d["imask"][k] & (1 << code), f"node {k} slot {s}: internal code {code} not in imask"
            rank = bin(int(d["imask"][k]) & ((1 << code) - 1)).count("1")
            out.append((s, "node", int(d["child_base"][k]) + rank, 0))
        else:
            unary = m >> 5
            cnt = {1: 1, 3: 2, 7: 3}[unary]
            out.append((s, "tris", int(d["tri_base"][k]) + lo5, cnt))
    return out


def validate(wide: np.ndarray, tris: np.ndarray, W: int, ntri: int, verts: np.ndarray | None = None):
    """Raises AssertionError on any structural fault; returns depth."""
    if ntri == 0:
        assert wide.size == 0
        return 0
    d = decode(wide, W)
    n = d["n"]
    assert empty_slots_inverted(d, W), "an empty slot does not carry the inverted box"
    seen_nodes = np.zeros(n, np.int32)
    seen_tris = np.zeros(ntri, np.int32)
    seen_nodes[0] = 1
    tri_xyz = tris.reshape(-1, 12)
    prims = tri_xyz[:, 3].copy().view(np.uint32)
    assert sorted(prims.tolist()) == list(range(ntri)), "triangle array is not a permutation of the primitives"
    if verts is not None:
        v = verts.reshape(-1, 9)
        assert np.array_equal(tri_xyz[:, [0, 1, 2, 4, 5, 6, 8, 9, 10]], v[prims]), "triangle copies differ from the input"
    # subtree boxes bottom-up (children always have larger indices)
    sub_lo = np.full((n, 3), np.inf)
    sub_hi = np.full((n, 3), -np.inf)
    kids = [children(d, k, W) for k in range(n)]
    for k in range(n):
        for s, kind, idx, cnt in kids[k]:
            if kind == "node":
                assert k < idx < n, f"node {k}: child {idx} out of order/range"
                seen_nodes[idx] += 1
            else:
                assert 0 <= idx and idx + cnt <= ntri, f"node {k}: triangle range out of bounds"
                seen_tris[idx:idx + cnt] += 1
    assert (seen_nodes == 1).all(), "some node is unreachable or shared"
    assert (seen_tris == 1).all(), "some triangle slot is unreachable or shared"
    for k in range(n - 1, -1, -1):
        for s, kind, idx, cnt in kids[k]:
            if kind == "node":
                clo, chi = sub_lo[idx], sub_hi[idx]
            else:
                t = tri_xyz[idx:idx + cnt][:, [0, 1, 2, 4, 5, 6, 8, 9, 10]].reshape(-1, 3).astype(np.float64)
                clo, chi = t.min(0), t.max(0)
            lo, hi = slot_box(d, k, s)
            assert (lo <= clo).all() and (chi <= hi).all(), f"node {k} slot {s}: quantized box not conservative"
            sub_lo[k] = np.minimum(sub_lo[k], clo)
            sub_hi[k] = np.maximum(sub_hi[k], chi)
    # depth
    depth = np.zeros(n, np.int32)
    for k in range(n):
        for s, kind, idx, cnt in kids[k]:
            if kind == "node":
                depth[idx] = depth[k] + 1
    return int(depth.max()) + 1
