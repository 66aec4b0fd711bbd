"""Compose (present.frag) and the luminance histogram on the GPU against the oracle.

Compose output is BGRA8: the ACES curve ends in pow(x, 1/2.2), whose last-bit rounding
differs between CUDA's powf and the host's, so a channel may differ by 1 LSB on a few
pixels; every other view (G-buffer planes, grid) is bit-exact. Histogram bins come
from log2 of the luminance: counts agree except for pixels within a rounding of a bin
edge (at most 0.01 % of pixels move).
"""
import numpy as np
import pytest

import luz_gb300 as L
import oracle as O

pytestmark = pytest.mark.gpu


def _planes(fr, s):
    H, W = s.height, s.width
    return (fr.read(L.PLANE_LIGHT).reshape(H, W, 4), fr.read(L.PLANE_ALBEDO).reshape(H, W),
            fr.read(L.PLANE_NORMAL).reshape(H, W, 4), fr.read(L.PLANE_MATERIAL).reshape(H, W),
            fr.read(L.PLANE_EMISSION).reshape(H, W), fr.read(L.PLANE_DEPTH).reshape(H, W))


def test_compose_views_match_oracle():
    ctx = L.Context(0)
    try:
        s = L.HostScene(1, width=120, height=90)
        g = L.GPUScene(ctx, s)
        g.render(0)
        planes = _planes(g.frame, s)
        for image_type in range(7):
            g.frame.compose(False, image_type)
            ctx.synchronize()
            got = g.frame.read(L.PLANE_COMPOSE).reshape(s.height, s.width)
            want = O.compose(*planes, image_type=image_type)
            d = np.abs(got.view(np.uint8).astype(int) - want.view(np.uint8).astype(int))
            if image_type in (0, 6):
                assert d.max() <= 1 and (d > 0).mean() < 0.01, (image_type, d.max(), (d > 0).mean())
            else:
                assert d.max() == 0, image_type
        rgba = g.frame.composed_rgba()
        assert rgba.shape == (s.height, s.width, 4) and (rgba[..., 3] == 255).all()
    finally:
        ctx.close()


def test_luminance_histogram_matches_oracle():
    ctx = L.Context(0)
    try:
        s = L.HostScene(1, width=160, height=120)
        g = L.GPUScene(ctx, s)
        state = np.zeros(1, np.float32)
        for k in range(3):
            g.render(k)
            light = g.frame.read(L.PLANE_LIGHT)
            got = g.frame.luminance_histogram(False, 1.0 / 60.0)
            want, state = O.histogram(light, 1.0 / 60.0, state)
            assert got["bins"].sum() == s.width * s.height
            assert np.abs(got["bins"].astype(int) - want["bins"].astype(int)).sum() <= 4
            for key in ("weighted_sum", "log_average", "average_luminance", "adapted_luminance"):
                assert np.isclose(got[key], want[key], rtol=1e-4), (key, got[key], want[key])
    finally:
        ctx.close()
