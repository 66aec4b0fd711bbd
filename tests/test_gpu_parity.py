"""GPU parity: the sm_103a path through the C ABI against the CPU oracle.

Bit-exact: Morton codes, sort order, BVH topology and boxes, G-buffer planes,
per-ray hit/miss masks. Radiance: within 1e-4 relative per channel.
"""
import numpy as np
import pytest

import luz_gb300 as L
from tests.pathutil import bits_mismatch, gpu_frame, oracle_frame, oracle_scene

pytestmark = pytest.mark.gpu

RADIANCE_RTOL = 1e-4


@pytest.fixture(scope="module")
def ctx():
    c = L.Context(0)
    yield c
    c.close()


def _cfg1(w=512, h=512, **kw):
    return L.HostScene(1, width=w, height=h, **kw)


def test_blas_bit_exact(ctx):
    s = _cfg1(64, 64)
    meshes = s.meshes()
    gb = ctx.build_blas(meshes)
    ob, _ = oracle_scene(s)
    for g, o in zip(gb, ob):
        gn, gt, gm, go = g.download()
        on, ot, om, oo = o.arrays()
        assert np.array_equal(gm, om), "morton codes"
        assert np.array_equal(go, oo), "sort order"
        assert np.array_equal(gn.view(np.uint32), on.view(np.uint32)), "nodes (topology + boxes)"
        assert np.array_equal(gt.view(np.uint32), ot.view(np.uint32)), "triangles"


def test_blas_batch_icospheres_bit_exact(ctx):
    s = L.HostScene(2, width=64, height=36, meshes=6, instances=32, subdivisions=4)
    meshes = s.meshes()
    gb = ctx.build_blas(meshes)
    ob, _ = oracle_scene(s)
    for g, o in zip(gb, ob):
        gn, gt, gm, go = g.download()
        on, ot, om, oo = o.arrays()
        assert np.array_equal(gm, om)
        assert np.array_equal(go, oo)
        assert np.array_equal(gn.view(np.uint32), on.view(np.uint32))
        assert np.array_equal(gt.view(np.uint32), ot.view(np.uint32))


@pytest.mark.parametrize("instances", [1, 2, 300, 4096, 5000])
def test_tlas_bit_exact(ctx, instances):
    # up to 4096 instances: the single-CTA build; above: the multi-kernel build
    s = L.HostScene(2, width=64, height=36, meshes=4, instances=instances, subdivisions=3 if instances <= 300 else 1)
    g = L.GPUScene(ctx, s)
    g.update_resources_gpu()
    gn, gm, go = g.tlas.download()
    _, tl = oracle_scene(s)
    on, om, oo = tl.arrays()
    assert np.array_equal(gm[: s.instance_count], om)
    assert np.array_equal(go[: s.instance_count], oo)
    assert np.array_equal(gn.view(np.uint32), on.view(np.uint32))


@pytest.mark.parametrize("sampler", [L.SAMPLER_PARITY, L.SAMPLER_STRATIFIED])
def test_config1_frame_parity(ctx, sampler):
    s = _cfg1(sampler=sampler)
    g = gpu_frame(ctx, s)
    _, tl = oracle_scene(s)
    f = oracle_frame(s, tl)
    fr = g.frame
    # G-buffer planes, bit for bit
    assert np.array_equal(fr.read(L.PLANE_ALBEDO).ravel(), f.albedo)
    assert np.array_equal(fr.read(L.PLANE_MATERIAL).ravel(), f.material)
    assert np.array_equal(fr.read(L.PLANE_EMISSION).ravel(), f.emission)
    assert np.array_equal(fr.read(L.PLANE_DEPTH).ravel().view(np.uint32), f.depth.view(np.uint32))
    assert np.array_equal(fr.read(L.PLANE_NORMAL).reshape(-1, 4).view(np.uint32), f.normal.view(np.uint32))
    assert np.array_equal(fr.read(L.PLANE_PRIMARY_HIT).reshape(-1, 2), f.primary_hit)
    # hit / miss masks, bit for bit
    assert bits_mismatch(fr.read(L.PLANE_SHADOW_BITS), f.shadow_bits[: f.shadow_slots]) == 0
    assert bits_mismatch(fr.read(L.PLANE_AO_BITS), f.ao_bits[: f.ao_samples]) == 0
    # radiance within 1e-4 relative per channel
    gl = fr.read(L.PLANE_LIGHT)
    ol = f.light_pass()
    rel = np.abs(gl - ol) / np.maximum(np.abs(ol), 1e-6)
    assert rel.max() <= RADIANCE_RTOL, rel.max()


def test_config1_masks_match_bruteforce(ctx):
    s = _cfg1(256, 256)
    g = gpu_frame(ctx, s)
    _, tl = oracle_scene(s)
    f = oracle_frame(s, tl, brute=True)
    assert bits_mismatch(g.frame.read(L.PLANE_SHADOW_BITS), f.shadow_bits[: f.shadow_slots]) == 0
    assert bits_mismatch(g.frame.read(L.PLANE_AO_BITS), f.ao_bits[: f.ao_samples]) == 0


def test_config2_reduced_resolution_parity(ctx):
    s = L.HostScene(2, width=240, height=136, meshes=8, instances=256, subdivisions=5)
    g = gpu_frame(ctx, s)
    _, tl = oracle_scene(s)
    f = oracle_frame(s, tl)
    fr = g.frame
    assert np.array_equal(fr.read(L.PLANE_NORMAL).reshape(-1, 4).view(np.uint32), f.normal.view(np.uint32))
    assert np.array_equal(fr.read(L.PLANE_DEPTH).ravel().view(np.uint32), f.depth.view(np.uint32))
    assert bits_mismatch(fr.read(L.PLANE_SHADOW_BITS), f.shadow_bits[: f.shadow_slots]) == 0
    assert bits_mismatch(fr.read(L.PLANE_AO_BITS), f.ao_bits[: f.ao_samples]) == 0
    gl = fr.read(L.PLANE_LIGHT)
    ol = f.light_pass()
    rel = np.abs(gl - ol) / np.maximum(np.abs(ol), 1e-6)
    assert rel.max() <= RADIANCE_RTOL, rel.max()


@pytest.mark.parametrize("place", ["inside_cube", "inside_field"])
def test_gbuffer_tile_lists_camera_inside_scene(ctx, place):
    """The G-buffer traces each 8x8 tile through the TLAS leaves its corner-ray cone
    keeps. With the camera inside an instance's box (every cone keeps that box) or in
    the middle of the cube field (instances behind the camera and beside it) the planes
    are still the oracle's bit for bit."""
    s = _cfg1(96, 64)
    tr = s.transforms().reshape(-1, 3, 4)
    c = s.camera()
    if place == "inside_cube":
        c.eye[:] = [float(v) for v in tr[1][:, 3]]
        c.center[:] = [0.0, 0.0, 0.0]
    else:
        c.eye[:] = [0.0, 1.0, 0.0]
        c.center[:] = [8.0, 1.5, 8.0]
    s.set_camera(c)
    g = gpu_frame(ctx, s)
    _, tl = oracle_scene(s)
    f = oracle_frame(s, tl)
    fr = g.frame
    assert np.array_equal(fr.read(L.PLANE_DEPTH).ravel().view(np.uint32), f.depth.view(np.uint32))
    assert np.array_equal(fr.read(L.PLANE_NORMAL).reshape(-1, 4).view(np.uint32), f.normal.view(np.uint32))
    assert np.array_equal(fr.read(L.PLANE_PRIMARY_HIT).reshape(-1, 2), f.primary_hit)
    assert (f.primary_hit[:, 0] != 0xFFFFFFFF).sum() > 0
    assert bits_mismatch(fr.read(L.PLANE_SHADOW_BITS), f.shadow_bits[: f.shadow_slots]) == 0
    assert bits_mismatch(fr.read(L.PLANE_AO_BITS), f.ao_bits[: f.ao_samples]) == 0


@pytest.mark.parametrize("ao_max", [0.5, 3.0, 12.0])
def test_short_rays_near_lists_match_oracle(ctx, ao_max):
    """AO rays whose segment stays within 1.5 AO radii of their own instance's box start
    at that instance's TLAS leaf, with the near instances whose boxes the segment
    overlaps on the stack; a list of more than 8 instances falls back to the TLAS root.
    On the config-1 cubes a short radius gives few near instances, a medium one masks
    near instances in and out, a long one overflows most lists: the masks stay the
    oracle's."""
    s = _cfg1(160, 160)
    s.set_sampling(8, ao_max=ao_max)
    g = gpu_frame(ctx, s)
    _, tl = oracle_scene(s)
    f = oracle_frame(s, tl)
    assert bits_mismatch(g.frame.read(L.PLANE_AO_BITS), f.ao_bits[: f.ao_samples]) == 0
    assert bits_mismatch(g.frame.read(L.PLANE_SHADOW_BITS), f.shadow_bits[: f.shadow_slots]) == 0


def test_short_rays_skip_the_tlas(ctx):
    """AO rays of the sparse two-level scene all start at their own instance's leaf: the
    counting build of the traversal sees almost no TLAS node per ray, and the masks are
    the oracle's."""
    s = L.HostScene(2, width=240, height=136, meshes=8, instances=256, subdivisions=4)
    s.set_sampling(4, light_samples=0)
    g = gpu_frame(ctx, s)
    st = g.frame.trace_stats(g.tlas, 0)
    assert st["rays"] > 0
    assert st["tlas_nodes"] < 0.5 * st["rays"], st
    _, tl = oracle_scene(s)
    f = oracle_frame(s, tl)
    assert bits_mismatch(g.frame.read(L.PLANE_AO_BITS), f.ao_bits[: f.ao_samples]) == 0


@pytest.mark.parametrize("light_samples", [1, 3])
def test_shadow_beams_skip_the_tlas(ctx, light_samples):
    """Shadow rays start at their group's beam list (the TLAS leaves the capsule around
    32 neighbouring rays of one light sample reaches): on the sparse two-level scene
    few TLAS nodes are visited per traversed ray, and the masks are the oracle's, with
    one and with several samples per light (groups then also span slot ends)."""
    s = L.HostScene(2, width=960, height=540, meshes=8, instances=256, subdivisions=4)
    s.set_sampling(2, light_samples=light_samples)
    g = gpu_frame(ctx, s)
    st = g.frame.trace_stats(g.tlas, 0)
    assert st["rays"] > 0
    # 1.5-1.6 measured at this size (the lists get shorter as the pixels get smaller:
    # 6.0 per ray at 240x136)
    assert st["tlas_nodes"] < 2.5 * st["rays"], st
    _, tl = oracle_scene(s)
    f = oracle_frame(s, tl)
    assert bits_mismatch(g.frame.read(L.PLANE_SHADOW_BITS), f.shadow_bits[: f.shadow_slots]) == 0
    assert bits_mismatch(g.frame.read(L.PLANE_AO_BITS), f.ao_bits[: f.ao_samples]) == 0


def test_render_frame_single_call_matches_stages(ctx):
    s = _cfg1(128, 128)
    g = gpu_frame(ctx, s)
    staged = g.frame.read(L.PLANE_LIGHT).copy()
    g.render_frame(0)
    ctx.synchronize()
    assert np.array_equal(g.frame.read(L.PLANE_LIGHT).view(np.uint32), staged.view(np.uint32))


def test_deterministic_rebuild(ctx):
    s = _cfg1(128, 128)
    g1 = gpu_frame(ctx, s)
    a = g1.frame.read(L.PLANE_AO_BITS).copy()
    n1 = g1.tlas.download()[0].copy()
    g1.render(0)
    ctx.synchronize()
    assert np.array_equal(a, g1.frame.read(L.PLANE_AO_BITS))
    assert np.array_equal(n1.view(np.uint32), g1.tlas.download()[0].view(np.uint32))


def test_negative_ao_min_is_rejected(ctx):
    # aoMin is the AO rays' tMin; a ray query's tMin must not be negative.
    s = _cfg1(32, 32)
    s.set_sampling(4, ao_min=-0.5)
    g = L.GPUScene(ctx, s)
    with pytest.raises(L.LuzError, match="ao_min is negative"):
        g.update_resources_gpu()


@pytest.mark.parametrize("scene", ["config1", "config2_small"])
def test_every_shadow_ray_traced_matches_oracle(ctx, scene):
    """With the shadow-ray cull off, every shadow sample light.frag traces is traced
    (light.frag:93-107): the bit planes equal the oracle's full trace (cull=False) bit
    for bit, and the light pass output is bit-identical to the culled frame's."""
    if scene == "config1":
        s = _cfg1(256, 256)
    else:
        s = L.HostScene(2, width=160, height=90, meshes=6, instances=128, subdivisions=4)
    g = gpu_frame(ctx, s)
    culled_light = g.frame.read(L.PLANE_LIGHT).copy()
    culled_bits = g.frame.read(L.PLANE_SHADOW_BITS).copy()
    g.frame.set_shadow_cull(False)
    g.render(0)
    ctx.synchronize()
    assert ctx.device_status() == 0
    _, tl = oracle_scene(s)
    f = oracle_frame(s, tl)
    f.shadow_bits[:] = 0
    f.ao_bits[:] = 0
    f.visibility(0, L.blue_noise(), cull=False)
    full_bits = g.frame.read(L.PLANE_SHADOW_BITS)
    assert bits_mismatch(full_bits, f.shadow_bits[: f.shadow_slots]) == 0
    assert bits_mismatch(g.frame.read(L.PLANE_AO_BITS), f.ao_bits[: f.ao_samples]) == 0
    assert bits_mismatch(full_bits, culled_bits) > 0          # the culled samples do hit
    assert np.array_equal(g.frame.read(L.PLANE_LIGHT).view(np.uint32), culled_light.view(np.uint32))
    g.frame.set_shadow_cull(True)


def test_config2_full_size_frame_parity(ctx):
    """The benchmark frame itself: 1920x1080, 64 displaced icospheres x 1024 instances, 41
    lights, 1 shadow ray per light and 16 AO rays per pixel. G-buffer planes and every
    hit/miss mask bit-exact against the oracle, radiance within 1e-4 relative."""
    s = L.HostScene(2)
    assert (s.width, s.height, s.instance_count, s.light_count) == (1920, 1080, 1024, 41)
    g = gpu_frame(ctx, s)
    _, tl = oracle_scene(s)
    f = oracle_frame(s, tl)
    fr = g.frame
    assert np.array_equal(fr.read(L.PLANE_ALBEDO).ravel(), f.albedo)
    assert np.array_equal(fr.read(L.PLANE_MATERIAL).ravel(), f.material)
    assert np.array_equal(fr.read(L.PLANE_NORMAL).reshape(-1, 4).view(np.uint32), f.normal.view(np.uint32))
    assert np.array_equal(fr.read(L.PLANE_DEPTH).ravel().view(np.uint32), f.depth.view(np.uint32))
    assert np.array_equal(fr.read(L.PLANE_PRIMARY_HIT).reshape(-1, 2), f.primary_hit)
    assert bits_mismatch(fr.read(L.PLANE_SHADOW_BITS), f.shadow_bits[: f.shadow_slots]) == 0
    assert bits_mismatch(fr.read(L.PLANE_AO_BITS), f.ao_bits[: f.ao_samples]) == 0
    gl = fr.read(L.PLANE_LIGHT)
    ol = f.light_pass()
    rel = np.abs(gl - ol) / np.maximum(np.abs(ol), 1e-6)
    assert rel.max() <= RADIANCE_RTOL, rel.max()


def test_config5_reduced_resolution_parity(ctx):
    """The stress scene (4096 instances of the 64 displaced icospheres, 145 lights, 64 AO
    rays per pixel; the TLAS at the single-CTA build's 4096-instance limit) at 960x540:
    G-buffer planes and every hit/miss mask bit-exact against the oracle, radiance within
    1e-4 relative."""
    s = L.HostScene(5, width=960, height=540)
    assert (s.instance_count, s.light_count, s.block().ao_num_samples) == (4096, 145, 64)
    g = gpu_frame(ctx, s)
    _, tl = oracle_scene(s)
    f = oracle_frame(s, tl)
    fr = g.frame
    assert np.array_equal(fr.read(L.PLANE_NORMAL).reshape(-1, 4).view(np.uint32), f.normal.view(np.uint32))
    assert np.array_equal(fr.read(L.PLANE_DEPTH).ravel().view(np.uint32), f.depth.view(np.uint32))
    assert np.array_equal(fr.read(L.PLANE_PRIMARY_HIT).reshape(-1, 2), f.primary_hit)
    assert bits_mismatch(fr.read(L.PLANE_SHADOW_BITS), f.shadow_bits[: f.shadow_slots]) == 0
    assert bits_mismatch(fr.read(L.PLANE_AO_BITS), f.ao_bits[: f.ao_samples]) == 0
    gl = fr.read(L.PLANE_LIGHT)
    ol = f.light_pass()
    rel = np.abs(gl - ol) / np.maximum(np.abs(ol), 1e-6)
    assert rel.max() <= RADIANCE_RTOL, rel.max()
