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


class _Buffers:
    """Device buffers of one call, owned by the caller (allocated here with torch)."""

    def __init__(self, mesh):
        import torch

        v, idx = mesh
        self.n = idx.size // 3
        m = max(self.n, 2) - 1
        dev = torch.device("cuda", 0)
        self.vertex_count, self.index_count = v.shape[0], idx.size
        self.v = torch.from_numpy(np.ascontiguousarray(v, np.float32).reshape(-1, 12)).to(dev)
        self.i = torch.from_numpy(np.ascontiguousarray(idx, np.uint32).view(np.int32).reshape(-1)).to(dev)
        self.nodes = torch.zeros((m, 16), dtype=torch.float32, device=dev)
        self.tris = torch.zeros((max(self.n, 1), 12), dtype=torch.float32, device=dev)
        self.mort = torch.zeros(max(self.n, 1), dtype=torch.int32, device=dev)
        self.order = torch.zeros(max(self.n, 1), dtype=torch.int32, device=dev)
        torch.cuda.synchronize()

    def call(self, stream):
        return L.lib.luz_blas_build_noalloc(
            C.c_void_p(self.v.data_ptr()), self.vertex_count, C.c_void_p(self.i.data_ptr()), self.index_count,
            C.c_void_p(self.nodes.data_ptr()), C.c_void_p(self.tris.data_ptr()), C.c_void_p(self.mort.data_ptr()),
            C.c_void_p(self.order.data_ptr()), C.c_void_p(stream))

    def result(self):
        n = self.n
        return (self.nodes.cpu().numpy(), self.tris.cpu().numpy()[:n], self.mort.cpu().numpy().view(np.uint32)[:n],
                self.order.cpu().numpy().view(np.uint32)[:n])


def _noalloc_build(mesh, stream):
    b = _Buffers(mesh)
    st = b.call(stream)
    assert st == 0, st
    return b.result()


def _same(got, ref):
    for name, a, b in zip(("nodes", "triangles", "morton", "order"), got, ref):
        assert np.array_equal(np.ascontiguousarray(a).view(np.uint32), np.ascontiguousarray(b).view(np.uint32)), name


def test_noalloc_blas_matches_allocating_build_twice():
    torch = pytest.importorskip("torch")
    ctx = L.Context(0)
    sphere = L.HostScene(2, width=16, height=16, meshes=1, instances=1, subdivisions=5).meshes()[0]
    cube = L.HostScene(1, width=16, height=16).meshes()[1]
    stream = torch.cuda.Stream()
    try:
        for mesh in (sphere, cube):      # two calls in a row; the second must not see the first's scratch
            ref = ctx.build_blas([mesh])[0].download()
            _same(_noalloc_build(mesh, stream.cuda_stream), ref)
    finally:
        ctx.close()


def test_noalloc_empty_and_single_triangle_meshes():
    """n = 0 writes one root with two empty (inverted) slots; n = 1 one root whose first
    child is the leaf; both as the allocating build writes them."""
    torch = pytest.importorskip("torch")
    ctx = L.Context(0)
    v = np.zeros((3, 12), np.float32)
    v[:, :3] = [[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.5]]
    stream = torch.cuda.Stream()
    try:
        for idx in (np.zeros(0, np.uint32), np.array([0, 1, 2], np.uint32)):
            ref = ctx.build_blas([(v, idx)])[0].download()
            got = _noalloc_build((v, idx), stream.cuda_stream)
            _same(got, ref)
            child0 = got[0].reshape(-1)[12:13].view(np.int32)[0]
            assert child0 == (~0 if idx.size else np.int32(-2147483647))
    finally:
        ctx.close()


def test_noalloc_index_outside_the_vertex_buffer_is_invalid():
    """The index check runs on the device (the bad index is never dereferenced); the call
    returns LUZ_ERR_INVALID, and the next good call builds correctly again."""
    torch = pytest.importorskip("torch")
    ctx = L.Context(0)
    cube = L.HostScene(1, width=16, height=16).meshes()[1]
    bad = (cube[0], np.where(np.arange(cube[1].size) == 7, cube[0].shape[0], cube[1]).astype(np.uint32))
    stream = torch.cuda.Stream()
    try:
        assert _Buffers(bad).call(stream.cuda_stream) == 1     # LUZ_ERR_INVALID
        _same(_noalloc_build(cube, stream.cuda_stream), ctx.build_blas([cube])[0].download())
    finally:
        ctx.close()


def test_noalloc_call_leaves_device_memory_unchanged():
    """The defining property: with its buffers in place, a call takes no device memory
    (free bytes of the device before and after are equal)."""
    torch = pytest.importorskip("torch")
    sphere = L.HostScene(2, width=16, height=16, meshes=1, instances=1, subdivisions=5).meshes()[0]
    stream = torch.cuda.Stream()
    b = _Buffers(sphere)
    assert b.call(stream.cuda_stream) == 0          # first call: module set-up, address look-up
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info(0)
    for _ in range(3):
        assert b.call(stream.cuda_stream) == 0
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info(0)
    assert free1 == free0, (free0, free1)


def test_noalloc_rejects_more_than_the_maximum():
    n = (1 << 17) + 1
    st = L.lib.luz_blas_build_noalloc(C.c_void_p(16), 3, C.c_void_p(16), 3 * n, C.c_void_p(16), C.c_void_p(16),
                                      C.c_void_p(16), C.c_void_p(16), None)
    assert st == 5   # LUZ_ERR_LIMIT, returned before any GPU work
