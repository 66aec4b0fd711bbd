"""Edge cases through the C ABI against the oracle: degenerate and tiny meshes in one
batched BLAS build, instances hidden by their mask, frames with nothing lit, no
lights and no AO samples, and a camera inside geometry-free space."""
import numpy as np
import pytest

import luz_gb300 as L
import oracle as O
from tests.pathutil import bits_mismatch, oracle_frame, oracle_scene

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = L.Context(0)
    yield c
    c.close()


def _mesh(tris):
    tris = np.asarray(tris, np.float32).reshape(-1, 3, 3)
    v = np.zeros((tris.shape[0] * 3, 12), np.float32)
    v[:, :3] = tris.reshape(-1, 3)
    v[:, 5] = 1.0   # normal +z
    return v, np.arange(v.shape[0], dtype=np.uint32)


def test_degenerate_and_tiny_meshes_bit_exact(ctx):
    rng = np.random.default_rng(7)
    tri = [[0, 0, 0], [1, 0, 0], [0, 1, 0]]
    meshes = [
        (np.zeros((0, 12), np.float32), np.zeros(0, np.uint32)),              # empty
        _mesh([tri]),                                                          # one triangle
        _mesh([tri, [[1, 1, 0], [1, 0, 0], [0, 1, 0]]]),                      # two
        _mesh([[[2, 2, 2]] * 3] * 5),                                          # points only
        _mesh([tri] * 40),                                                     # identical keys
        _mesh([[[0, 0, 0], [1e-7, 0, 0], [2e-7, 0, 0]]] * 3 + [tri]),          # slivers
        _mesh(rng.uniform(-1e4, 1e4, size=(300, 3, 3))),                       # large coordinates
    ]
    gb = ctx.build_blas(meshes)
    assert ctx.device_status() == 0
    for (v, i), g in zip(meshes, gb):
        o = O.OracleBlas(v, i)
        gn, gt, gm, go = g.download()
        on, ot, om, oo = o.arrays()
        assert np.array_equal(gm, om) and np.array_equal(go, oo)
        assert np.array_equal(gn.view(np.uint32), on.view(np.uint32))
        assert np.array_equal(gt.view(np.uint32), ot.view(np.uint32))


def test_instances_hidden_by_mask(ctx):
    s = L.HostScene(1, width=96, height=96)
    g = L.GPUScene(ctx, s)
    mask = np.full(s.instance_count, 0xFF, np.uint32)
    mask[::3] = 0                                   # every third instance invisible to all rays
    g.instances, g.n_instances = L.Tlas.make_instances(g.blas, s.instance_mesh(), s.transforms(), mask=mask)
    g.render(0)
    ctx.synchronize()
    assert ctx.device_status() == 0
    ob, _ = oracle_scene(s)
    tl = O.OracleTlas([ob[m] for m in s.instance_mesh()], s.transforms(), mask=mask)
    f = oracle_frame(s, tl)
    fr = g.frame
    assert np.array_equal(fr.read(L.PLANE_PRIMARY_HIT).reshape(-1, 2), f.primary_hit)
    assert bits_mismatch(fr.read(L.PLANE_SHADOW_BITS), f.shadow_bits[: f.shadow_slots]) == 0
    assert bits_mismatch(fr.read(L.PLANE_AO_BITS), f.ao_bits[: f.ao_samples]) == 0
    hidden = set(np.nonzero(mask == 0)[0].tolist())
    hits = f.primary_hit[:, 0]
    assert not (set(hits[hits != 0xFFFFFFFF].tolist()) & hidden)


def _ambient(s):
    b = s.block()
    return np.array(b.ambient_light_color[:3], np.float32) * np.float32(b.ambient_light_intensity)


def test_nothing_lit(ctx):
    s = L.HostScene(1, width=64, height=48)
    cam = s.camera()
    cam.mode = 2
    cam.eye[:] = (0.0, 50.0, 0.0)
    cam.center[:] = (0.0, 100.0, 1.0)       # looking up into empty sky
    s.set_camera(cam)
    g = L.GPUScene(ctx, s)
    g.render(0)
    ctx.synchronize()
    assert ctx.device_status() == 0
    assert g.frame.lit_count() == 0
    light = g.frame.read(L.PLANE_LIGHT).reshape(-1, 4)
    assert np.allclose(light[:, :3], _ambient(s)[None, :]) and np.all(light[:, 3] == 1.0)


def test_no_lights_no_ao(ctx):
    s = L.HostScene(1, width=64, height=64)
    s.set_sampling(0, light_samples=0)
    g = L.GPUScene(ctx, s)
    g.render(0)
    ctx.synchronize()
    assert ctx.device_status() == 0
    _, tl = oracle_scene(s)
    f = oracle_frame(s, tl)
    gl, ol = g.frame.read(L.PLANE_LIGHT), f.light_pass()
    rel = np.abs(gl - ol) / np.maximum(np.abs(ol), 1e-6)
    assert rel.max() <= 1e-4
    assert g.frame.trace_stats(g.tlas, 0)["rays"] == 0
