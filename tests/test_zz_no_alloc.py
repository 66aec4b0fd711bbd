"""luz_blas_build_noalloc: the BLAS build for callers that cannot allocate device
memory (a fixed up-front memory budget, no allocation-induced synchronisation inside
a frame, or a host that owns every allocation). The test owns all device buffers
(allocated with torch, outside the entry point), calls the entry point through the
C ABI twice in a row on different meshes, and checks each result byte for byte
against the allocating build, luz_blas_build, downloaded with luz_blas_download.

The file name sorts last so that a run stopping at the first failure has run every
other test first; it also passes alone in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

import luz_gb300 as L

pytestmark = pytest.mark.gpu


def _noalloc_build(mesh, stream):
    import torch

    v, idx = mesh
    n = idx.size // 3
    m = max(n, 2) - 1
    dev = torch.device("cuda", 0)
    d_v = torch.from_numpy(np.ascontiguousarray(v, np.float32)).to(dev)
    d_i = torch.from_numpy(np.ascontiguousarray(idx, np.uint32).view(np.int32)).to(dev)
    nodes = torch.zeros((m, 16), dtype=torch.float32, device=dev)
    tris = torch.zeros((max(n, 1), 12), dtype=torch.float32, device=dev)
    mort = torch.zeros(max(n, 1), dtype=torch.int32, device=dev)
    order = torch.zeros(max(n, 1), dtype=torch.int32, device=dev)
    torch.cuda.synchronize()
    st = L.lib.luz_blas_build_noalloc(C.c_void_p(d_v.data_ptr()), v.shape[0], C.c_void_p(d_i.data_ptr()),
                                      idx.size, C.c_void_p(nodes.data_ptr()), C.c_void_p(tris.data_ptr()),
                                      C.c_void_p(mort.data_ptr()), C.c_void_p(order.data_ptr()),
                                      C.c_void_p(stream))
    assert st == 0, st
    return (nodes.cpu().numpy(), tris.cpu().numpy()[:n], mort.cpu().numpy().view(np.uint32)[:n],
            order.cpu().numpy().view(np.uint32)[:n])


def test_noalloc_blas_matches_allocating_build_twice():
    torch = pytest.importorskip("torch")
    ctx = L.Context(0)
    sphere = L.HostScene(2, width=16, height=16, meshes=1, instances=1, subdivisions=5).meshes()[0]
    cube = L.HostScene(1, width=16, height=16).meshes()[1]
    stream = torch.cuda.Stream()
    try:
        for mesh in (sphere, cube):      # two calls in a row; the second must not see the first's scratch
            ref = ctx.build_blas([mesh])[0].download()
            got = _noalloc_build(mesh, stream.cuda_stream)
            for name, a, b in zip(("nodes", "triangles", "morton", "order"), got, ref):
                assert np.array_equal(np.ascontiguousarray(a).view(np.uint32),
                                      np.ascontiguousarray(b).view(np.uint32)), name
    finally:
        ctx.close()


def test_noalloc_rejects_more_than_the_maximum():
    n = (1 << 17) + 1
    st = L.lib.luz_blas_build_noalloc(C.c_void_p(16), 3, C.c_void_p(16), 3 * n, C.c_void_p(16), C.c_void_p(16),
                                      C.c_void_p(16), C.c_void_p(16), None)
    assert st == 5   # LUZ_ERR_LIMIT, returned before any GPU work
