"""Batched rendering: one visibility launch over several uneven scenes, CUDA graph
capture/replay and the autotuner give the same bits as rendering each scene alone."""
import numpy as np
import pytest

import luz_gb300 as L

pytestmark = pytest.mark.gpu


def _scenes():
    return [L.HostScene(1, width=128, height=96),
            L.HostScene(6, width=96, height=64, triangles=30000, seed=11),
            L.HostScene(2, width=160, height=90, meshes=3, instances=120, subdivisions=3)]


def _planes(frame):
    return (frame.read(L.PLANE_SHADOW_BITS).copy(), frame.read(L.PLANE_AO_BITS).copy(),
            frame.read(L.PLANE_LIGHT).copy())


def _same(a, b):
    return all(np.array_equal(x.view(np.uint32), y.view(np.uint32)) for x, y in zip(a, b))


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
        b.render(3)
        ctx.synchronize()
        assert ctx.device_status() == 0
        for fr, ref in zip(b.frames, singles):
            assert _same(_planes(fr), ref)
        st = b.stats(3)
        lit = sum(int((np.linalg.norm(f.read(L.PLANE_NORMAL)[..., :3], axis=-1) > 0).sum()) for f in b.frames)
        assert st["rays"] > lit
        # graph capture + replay
        b.capture(3)
        for fr in b.frames:
            fr.write(L.PLANE_LIGHT, np.zeros((fr.height, fr.width, 4), np.float32))
        b.replay()
        ctx.synchronize()
        for fr, ref in zip(b.frames, singles):
            assert _same(_planes(fr), ref)
        # autotuner: a valid shape, and the same bits afterwards
        tun, ms = b.autotune(reps=1)
        assert 1 <= tun["refill"] <= 32 and tun["ctas_per_sm"] >= 1 and ms > 0
        b.render(3)
        ctx.synchronize()
        for fr, ref in zip(b.frames, singles):
            assert _same(_planes(fr), ref)
        assert ctx.device_status() == 0
    finally:
        ctx.close()
