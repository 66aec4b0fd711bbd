"""The 4-wide traversal nodes: the even-depth collapse of the binary LBVH.

CPU: the oracle's collapse keeps every leaf exactly once and every box it copies.
GPU: the device collapse of BLAS and TLAS equals the oracle's, bit for bit.
"""
import numpy as np
import pytest

import luz_gb300 as L
import oracle as O
from tests.pathutil import oracle_scene


def _leaves(wide: np.ndarray) -> list[int]:
    ch = wide.view(np.int32)[:, 24:28].ravel()
    return sorted(int(~c) for c in ch if c < 0 and c != O.K_EMPTY_CHILD)


def test_oracle_collapse_keeps_leaves_and_boxes():
    s = L.HostScene(2, width=32, height=32, meshes=2, instances=40, subdivisions=3)
    ob, tl = oracle_scene(s)
    for o in ob:
        nodes, tris, _, _ = o.arrays()
        w = O.collapse_wide(nodes)
        assert _leaves(w) == list(range(len(tris)))
        # internal slots point to rows of the collapse; the tree is about half as deep
        ch = w.view(np.int32)[:, 24:28]
        inner = ch[ch >= 0]
        assert inner.size == len(w) - 1 and len(set(inner.tolist())) == inner.size
        assert inner.max() < len(w)
    tn, _, _ = tl.arrays()
    assert _leaves(O.collapse_wide(tn)) == list(range(s.instance_count))


@pytest.mark.gpu
def test_wide_nodes_bit_exact():
    ctx = L.Context(0)
    try:
        s = L.HostScene(2, width=64, height=36, meshes=5, instances=300, subdivisions=4)
        g = L.GPUScene(ctx, s)
        g.update_resources_gpu()
        ob, tl = oracle_scene(s)
        for gb, o in zip(g.blas, ob):
            want = O.collapse_wide(o.arrays()[0])
            got = gb.download_wide()[: len(want)]
            assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
        want = O.collapse_wide(tl.arrays()[0])
        got = g.tlas.download_wide()[: len(want)]
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
        # single-triangle and two-triangle meshes
        tiny = [(np.array([[0, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 0], [1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 0],
                           [0, 1, 0, 0, 0, 1, 0, 0, 0, 0, 0, 0], [1, 1, 0, 0, 0, 1, 0, 0, 0, 0, 0, 0]], np.float32),
                 idx) for idx in (np.array([0, 1, 2], np.uint32), np.array([0, 1, 2, 1, 3, 2], np.uint32))]
        for b, (v, i) in zip(ctx.build_blas(tiny), tiny):
            want = O.collapse_wide(O.OracleBlas(v, i).arrays()[0])
            assert np.array_equal(b.download_wide()[: len(want)].view(np.uint32), want.view(np.uint32))
        mem = g.blas[0].memory()
        assert mem["wide_nodes"] >= (g.blas[0].prims - 1) * 128 and mem["nodes"] >= (g.blas[0].prims - 1) * 64
        assert g.tlas.memory()["leaves"] > 0
    finally:
        ctx.close()
