"""Temporal anti-aliasing (taa.comp) on the GPU against the oracle, bit for bit:
first frame (zero history), jittered static camera, moving camera, reconstruct on
and off, history carried across frames, NaN in the light image."""
import numpy as np
import pytest

import luz_gb300 as L
import oracle as O

pytestmark = pytest.mark.gpu


def _frame(g, s):
    g.update_resources()
    g.render(0)
    light = g.frame.read(L.PLANE_LIGHT).reshape(s.height, s.width, 4).copy()
    depth = g.frame.read(L.PLANE_DEPTH).reshape(s.height, s.width).copy()
    return light, depth


@pytest.mark.parametrize("size", [(96, 72), (13, 10), (3, 2)])   # partial blocks; images narrower than a tile
@pytest.mark.parametrize("reconstruct", [True, False])
def test_taa_sequence_matches_oracle(reconstruct, size):
    ctx = L.Context(0)
    try:
        s = L.HostScene(1, width=size[0], height=size[1])
        g = L.GPUScene(ctx, s)
        hist = np.zeros((s.height, s.width, 4), np.float32)
        cam = s.camera()
        for k in range(4):
            if k == 2:   # move the camera: reprojection with real motion
                cam = s.camera()
                cam.eye[0] += 0.3
                cam.eye[1] -= 0.2
                s.set_camera(cam)
            s.next_frame(jitter=True)
            light, depth = _frame(g, s)
            if k == 3:
                light[5 % s.height, 7 % s.width, 1] = np.nan   # a NaN source texel
                g.frame.write(L.PLANE_LIGHT, light)
            g.frame.taa(reconstruct)
            ctx.synchronize()
            got = g.frame.read(L.PLANE_TAA).reshape(s.height, s.width, 4)
            want = O.taa(s.block(), light, hist, depth, reconstruct)
            same = (got.view(np.uint32) == want.view(np.uint32)) | (np.isnan(got) & np.isnan(want))
            assert same.all(), (k, np.argwhere(~same)[:5])
            hist = want
        assert ctx.device_status() == 0
    finally:
        ctx.close()
