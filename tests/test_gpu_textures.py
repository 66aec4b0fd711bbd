"""Textured G-buffer parity: colour, metallic-roughness, occlusion, emission and
normal maps sampled at the primary hit (bilinear, repeat), the colour-map alpha test
that lets primary rays continue behind discarded texels, and an imported glTF scene
end to end — bit-exact against the CPU oracle (radiance within 1e-4)."""
import os

import numpy as np
import pytest

import luz_gb300 as L
from tests.pathutil import bits_mismatch, oracle_frame, oracle_scene

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ingest")


def _scene(w=160, h=120):
    s = L.HostScene.import_file(os.path.join(GOLD, "synth.gltf"), w, h)
    cam = s.camera()
    cam.mode = 2
    cam.eye[:] = (2.5, 3.0, 5.0)
    cam.center[:] = (2.0, 1.0, -1.0)
    cam.horizontal_fov = 60.0
    s.set_camera(cam)
    return s


def _compare(g, s, tl, models=None, textures=None):
    f = oracle_frame(s, tl, models=models, textures=textures)
    fr = g.frame
    assert np.array_equal(fr.read(L.PLANE_ALBEDO).ravel(), f.albedo)
    assert np.array_equal(fr.read(L.PLANE_MATERIAL).ravel(), f.material)
    assert np.array_equal(fr.read(L.PLANE_EMISSION).ravel(), f.emission)
    assert np.array_equal(fr.read(L.PLANE_DEPTH).ravel().view(np.uint32), f.depth.view(np.uint32))
    assert np.array_equal(fr.read(L.PLANE_NORMAL).reshape(-1, 4).view(np.uint32), f.normal.view(np.uint32))
    assert np.array_equal(fr.read(L.PLANE_PRIMARY_HIT).reshape(-1, 2), f.primary_hit)
    assert bits_mismatch(fr.read(L.PLANE_SHADOW_BITS), f.shadow_bits[: f.shadow_slots]) == 0
    assert bits_mismatch(fr.read(L.PLANE_AO_BITS), f.ao_bits[: f.ao_samples]) == 0
    gl, ol = fr.read(L.PLANE_LIGHT), f.light_pass()
    rel = np.abs(gl - ol) / np.maximum(np.abs(ol), 1e-6)
    assert rel.max() <= 1e-4, rel.max()
    return f


def test_imported_gltf_scene_parity():
    ctx = L.Context(0)
    try:
        s = _scene()
        g = L.GPUScene(ctx, s)
        g.render(0)
        ctx.synchronize()
        assert ctx.device_status() == 0
        _, tl = oracle_scene(s)
        f = _compare(g, s, tl)
        # the checker texture shows in the albedo plane of the box
        alb = g.frame.read(L.PLANE_ALBEDO).ravel()
        box = f.primary_hit.reshape(-1, 2)[:, 0] == 0
        assert len(np.unique(alb[box])) > 4
    finally:
        ctx.close()


def test_all_maps_and_alpha_test_parity():
    ctx = L.Context(0)
    try:
        s = _scene()
        g = L.GPUScene(ctx, s)
        rng = np.random.default_rng(3)
        checker = s.textures()[0].copy()
        holes = checker.copy()
        yy, xx = np.mgrid[0:16, 0:16]
        holes[..., 3] = np.where(((xx // 2 + yy // 2) % 3) == 0, 40, 255).astype(np.uint8)   # alpha holes
        nmap = rng.integers(60, 255, size=(9, 13, 4), dtype=np.uint8)                      # odd size: wraps
        nmap[2, 3, :3] = 255                                                               # a white texel
        mr = rng.integers(0, 256, size=(5, 7, 4), dtype=np.uint8)
        textures = [holes, nmap, mr]
        g.frame.set_textures(textures)
        models = g.models
        for k in range(s.instance_count):
            models[k].color_map = 0
            models[k].normal_map = 1
            models[k].metallic_roughness_map = 2
            models[k].ao_map = 2
            models[k].emission_map = 2 if k == 0 else -1
            models[k].emission[0] = 0.5
        g.render(0)
        ctx.synchronize()
        assert ctx.device_status() == 0
        _, tl = oracle_scene(s)
        f = _compare(g, s, tl, models=models, textures=textures)
        # discarded texels let rays through: fewer box hits than without the holes
        g.frame.set_textures([checker, nmap, mr])
        g.render(0)
        ctx.synchronize()
        solid = g.frame.read(L.PLANE_PRIMARY_HIT).reshape(-1, 2)[:, 0]
        assert (f.primary_hit.reshape(-1, 2)[:, 0] == 0).sum() < (solid == 0).sum()
    finally:
        ctx.close()


def test_map_index_beyond_textures_is_an_error():
    ctx = L.Context(0)
    try:
        s = _scene(32, 24)
        g = L.GPUScene(ctx, s)
        g.models[0].normal_map = 5
        g.update_resources_gpu()
        with pytest.raises(L.LuzError, match="beyond the frame's textures"):
            g.frame.gbuffer(g.tlas)
    finally:
        ctx.close()
