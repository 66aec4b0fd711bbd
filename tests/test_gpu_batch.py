"""Batched rendering: the frame kernel (one persistent launch per frame over every
scene: TLAS builds, G-buffers, traversal, light passes) and the staged launches give
the same bits as rendering each scene alone, through CUDA graph capture/replay and the
autotuner; the frame kernel's planes match the CPU oracle scene by scene."""
import numpy as np
import pytest

import luz_gb300 as L
from tests.pathutil import bits_mismatch, oracle_frame, oracle_scene

pytestmark = pytest.mark.gpu

RADIANCE_RTOL = 1e-4


def _scenes():
    return [L.HostScene(1, width=128, height=96),
            L.HostScene(6, width=96, height=64, triangles=30000, seed=11),
            L.HostScene(2, width=160, height=90, meshes=3, instances=120, subdivisions=3)]


def _planes(frame):
    return (frame.read(L.PLANE_SHADOW_BITS).copy(), frame.read(L.PLANE_AO_BITS).copy(),
            frame.read(L.PLANE_LIGHT).copy(), frame.read(L.PLANE_NORMAL).copy(), frame.read(L.PLANE_DEPTH).copy(),
            frame.read(L.PLANE_ALBEDO).copy(), frame.read(L.PLANE_MATERIAL).copy(),
            frame.read(L.PLANE_PRIMARY_HIT).copy())


def _same(a, b):
    return all(np.array_equal(x.view(np.uint32), y.view(np.uint32)) for x, y in zip(a, b))


def _clobber(b):
    for fr in b.frames:
        fr.write(L.PLANE_LIGHT, np.zeros((fr.height, fr.width, 4), np.float32))
        fr.write(L.PLANE_NORMAL, np.full((fr.height, fr.width, 4), 7.0, np.float32))


def test_batch_matches_single_scene_renders():
    torch = pytest.importorskip("torch")
    ctx = L.Context(0)
    try:
        stream = torch.cuda.Stream()
        ctx.set_stream(stream.cuda_stream)
        scenes = _scenes()
        singles = []
        for sc in scenes:
            g = L.GPUScene(ctx, sc)
            g.render(3)
            ctx.synchronize()
            singles.append(_planes(g.frame))
        ctx.set_blue_noise(L.blue_noise())
        b = L.Batch(ctx, scenes)
        assert b.fused
        stats = {}
        for fused in (True, False):
            b.set_fused(fused)
            _clobber(b)
            b.render(3)
            ctx.synchronize()
            assert ctx.device_status() == 0
            for fr, ref in zip(b.frames, singles):
                assert _same(_planes(fr), ref)
            stats[fused] = b.stats(3)
            for fr, ref in zip(b.frames, singles):
                assert _same(_planes(fr), ref)
            # graph capture + replay
            b.capture(3)
            _clobber(b)
            b.replay()
            ctx.synchronize()
            for fr, ref in zip(b.frames, singles):
                assert _same(_planes(fr), ref)
        # both forms trace the same rays and visit the same nodes
        assert stats[True] == stats[False]
        lit = sum(int((np.linalg.norm(f.read(L.PLANE_NORMAL)[..., :3], axis=-1) > 0).sum()) for f in b.frames)
        assert stats[True]["rays"] > lit
        # autotuner on the frame kernel: a valid shape, and the same bits afterwards
        b.set_fused(True)
        tun, ms = b.autotune(reps=1)
        assert 1 <= tun["refill"] <= 32 and tun["ctas_per_sm"] >= 1 and ms > 0
        _clobber(b)
        b.render(3)
        ctx.synchronize()
        for fr, ref in zip(b.frames, singles):
            assert _same(_planes(fr), ref)
        assert ctx.device_status() == 0
    finally:
        ctx.close()


def test_batch_frame_kernel_matches_oracle():
    """A mix of scene kinds and sizes rendered by the frame kernel, each scene against
    the CPU oracle: G-buffer planes and hit/miss masks bit for bit, radiance within
    1e-4 relative."""
    ctx = L.Context(0)
    try:
        scenes = [L.HostScene(1, width=72, height=40, seed=21),
                  L.HostScene(6, width=48, height=48, triangles=8000, seed=22),
                  L.HostScene(2, width=64, height=36, meshes=2, instances=40, subdivisions=2, seed=23),
                  L.HostScene(1, width=17, height=9, seed=24)]
        ctx.set_blue_noise(L.blue_noise())
        b = L.Batch(ctx, scenes)
        assert b.fused
        b.render(5)
        ctx.synchronize()
        assert ctx.device_status() == 0
        for sc, fr in zip(scenes, b.frames):
            _, tl = oracle_scene(sc)
            f = oracle_frame(sc, tl, frame=5)
            assert np.array_equal(fr.read(L.PLANE_ALBEDO).ravel(), f.albedo)
            assert np.array_equal(fr.read(L.PLANE_MATERIAL).ravel(), f.material)
            assert np.array_equal(fr.read(L.PLANE_DEPTH).ravel().view(np.uint32), f.depth.view(np.uint32))
            assert np.array_equal(fr.read(L.PLANE_NORMAL).reshape(-1, 4).view(np.uint32), f.normal.view(np.uint32))
            assert bits_mismatch(fr.read(L.PLANE_SHADOW_BITS), f.shadow_bits[: f.shadow_slots]) == 0
            assert bits_mismatch(fr.read(L.PLANE_AO_BITS), f.ao_bits[: f.ao_samples]) == 0
            gl = fr.read(L.PLANE_LIGHT)
            ol = f.light_pass()
            rel = np.abs(gl - ol) / np.maximum(np.abs(ol), 1e-6)
            assert rel.max() <= RADIANCE_RTOL, rel.max()
    finally:
        ctx.close()


def test_batch_with_a_scene_beyond_the_frame_kernel_renders_staged():
    ctx = L.Context(0)
    try:
        big = L.HostScene(2, width=32, height=24, meshes=1, instances=4100, subdivisions=1, seed=31)
        small = L.HostScene(1, width=32, height=24, seed=32)
        ctx.set_blue_noise(L.blue_noise())
        b = L.Batch(ctx, [small, big])
        assert not b.fused
        with pytest.raises(L.LuzError):
            b.set_fused(True)
        b.render(0)
        ctx.synchronize()
        assert ctx.device_status() == 0
        g = L.GPUScene(ctx, big)
        g.render(0)
        ctx.synchronize()
        assert _same(_planes(b.frames[1]), _planes(g.frame))
    finally:
        ctx.close()
