"""Pins the oracle against the reference's own light-pass shader code.

oracle/_ref holds light.frag's main, EvaluateShadow, TraceShadowRay, TraceAORays,
the samplers and GGX terms, and utils.glsl's DepthToWorld, compiled for the CPU under
the reference's glm by the recipe oracle/ref_shaders.py, with ray queries answered by
the oracle's BVH. It runs where the reference tree is available (this build's CPU
test environment); elsewhere the test skips.

The reference evaluates normalize() as v * inversesqrt(dot(v, v)), pow() and cos/sin
through libm, so its rays and radiance agree with the oracle's to float rounding, not
bit for bit; a grazing ray may therefore flip between hit and miss.
"""
import ctypes as C

import numpy as np
import pytest

import luz_gb300 as L
import oracle as O
from tests.pathutil import oracle_frame, oracle_scene

REF = O.load_ref()
pytestmark = pytest.mark.skipif(REF is None, reason="oracle/_ref not built (reference tree absent)")


def _run_ref(s, f, bn, frame=0, log_cap=0, shadow=None):
    """shadow: (luz_shadow_light array, [maps], resolution) for a shadow-map scene."""
    lib = O.load()
    W, H = s.width, s.height
    out = np.zeros((H, W, 4), np.float32)
    log = np.zeros((max(log_cap, 1), 8), np.float32)
    cnt = C.c_uint64()
    fn = C.cast(lib.oracle_trace_ray, C.c_void_p)
    sl, maps, res = shadow if shadow else (None, None, 0)
    flat = np.ascontiguousarray(np.concatenate([m.reshape(-1) for m in maps])) if maps else None
    st = REF.ref_light_pass(C.byref(f.scene), C.cast(f.lights, C.c_void_p), f.nl, O._p(f.albedo),
                            O._p(f.normal), O._p(f.material), O._p(f.emission), O._p(f.depth), O._p(bn),
                            bn.shape[0], W, H, frame, fn, f.tlas.handle, O._p(out), O._p(log), log_cap,
                            C.byref(cnt), C.cast(sl, C.c_void_p) if sl is not None else None, O._p(flat),
                            len(sl) if sl is not None else 0, res)
    assert st == 0
    return out, log[: min(cnt.value, log_cap)], cnt.value


def test_reference_rays_match_oracle_rays():
    s = L.HostScene(1, width=48, height=48)
    _, tl = oracle_scene(s)
    f = oracle_frame(s, tl)
    bn = L.blue_noise()
    cap = 48 * 48 * 9
    _, ref_rays, n_ref = _run_ref(s, f, bn, log_cap=cap)
    mine = np.zeros((cap, 8), np.float32)
    n = O.load().oracle_generate_rays(C.byref(f.scene), C.cast(f.lights, C.c_void_p), f.nl, O._p(f.normal),
                                      O._p(f.depth), s.width, s.height, 0, O._p(bn), bn.shape[0], O._p(mine), cap)
    assert n == n_ref and n > 1000
    mine = mine[:n]
    scale = np.maximum(np.abs(ref_rays), 1.0)
    err = np.abs(mine - ref_rays) / scale
    assert err[:, :3].max() < 1e-5      # origins
    assert err[:, 4:7].max() < 1e-5     # directions
    assert np.array_equal(mine[:, 3], ref_rays[:, 3]) and np.abs(err[:, 7]).max() < 1e-5


def test_reference_light_pass_matches_oracle():
    s = L.HostScene(1, width=96, height=96)
    _, tl = oracle_scene(s)
    f = oracle_frame(s, tl)
    ref, _, _ = _run_ref(s, f, L.blue_noise())
    mine = f.light_pass()
    rel = np.abs(ref - mine) / np.maximum(np.abs(mine), 1e-6)
    close = (rel[..., :3] <= 1e-4).all(axis=-1)
    # a handful of pixels may see a grazing ray flip between hit and miss
    assert close.mean() > 0.995, close.mean()
    assert np.median(rel[..., :3]) < 1e-6


def test_reference_shadow_map_lookups_match_oracle():
    """light.frag:147-165 from the reference's code: the point lights' cube-map test
    (distance - 0.05 against depth x zFar) and the directional light's 2D map test
    (NDC depth of the biased origin through viewProj[0]), over the oracle's rasterised
    maps, against the oracle's light pass with the same maps. The cube texture
    lookup (face selection, bilinear within a face) is the shim's, the rest is the
    reference's."""
    s = L.HostScene(1, width=96, height=96)
    s.set_shadow_type(L._abi.SHADOW_MAP)
    _, tl = oracle_scene(s)
    lights = s.shadow_lights()
    res = 256
    maps = O.render_shadow_maps(tl, lights, res)
    try:
        f = oracle_frame(s, tl)
        ref, _, _ = _run_ref(s, f, L.blue_noise(), shadow=(lights, maps, res))   # only AO rays are traced
        mine = f.light_pass()
        rel = np.abs(ref - mine) / np.maximum(np.abs(mine), 1e-6)
        close = (rel[..., :3] <= 1e-4).all(axis=-1)
        assert close.mean() > 0.995, close.mean()
        # the maps shadow some pixels: the frame differs from the one without maps
        O.clear_shadow_maps()
        unshadowed = f.light_pass()
        assert (np.abs(unshadowed - mine)[..., :3].max(axis=-1) > 1e-3).mean() > 0.01
    finally:
        O.clear_shadow_maps()


# ---------------------------------------------------------------- post-processing passes
# taa.comp and present.frag from the reference tree, compiled the same way; their
# texture() reads go through the shim's bilinear, repeat-addressed sampler (the one
# piece defined here rather than taken from the reference). glm evaluates mat4 * vec4
# as (c0 x + c1 y) + (c2 z + c3 w), the oracle as ((c0 x + c1 y) + c2 z) + c3 w, so the
# reprojected history differs in the last bits once the camera moves.

def _post_fns():
    REF.ref_taa.argtypes = [C.c_void_p] * 4 + [C.c_int, C.c_int, C.c_int, C.c_void_p]
    REF.ref_compose.argtypes = [C.c_void_p] * 6 + [C.c_int, C.c_int, C.c_int, C.c_void_p]
    return REF.ref_taa, REF.ref_compose


def test_taa_matches_reference_shader():
    ref_taa, _ = _post_fns()
    W, H = 96, 72
    s = L.HostScene(1, width=W, height=H)
    _, tl = oracle_scene(s)
    hist = np.zeros((H, W, 4), np.float32)
    for k in range(3):
        if k == 1:   # camera motion: real reprojection
            cam = s.camera()
            cam.eye[0] += 0.4
            s.set_camera(cam)
        s.next_frame(True)
        f = oracle_frame(s, tl)
        light = f.light_pass().reshape(H, W, 4)
        depth = f.depth.reshape(H, W)
        b = s.block()
        for rec in (True, False):
            ours = O.taa(b, light, hist, depth, rec)
            ref = np.zeros_like(ours)
            ref_taa(C.cast(C.pointer(b), C.c_void_p), O._p(light), O._p(hist), O._p(depth), W, H, int(rec), O._p(ref))
            rel = np.abs(ours - ref) / np.maximum(np.abs(ref), 1e-3)
            # the history lookup moves with the motion vector's last bits: 5e-4 relative
            assert rel.max() <= 5e-4, (k, rec, rel.max())
            if k == 0:
                assert np.array_equal(ours.view(np.uint32), ref.view(np.uint32))
        hist = O.taa(b, light, hist, depth, True)


def test_compose_matches_reference_shader():
    _, ref_compose = _post_fns()
    W, H = 96, 72
    s = L.HostScene(1, width=W, height=H)
    _, tl = oracle_scene(s)
    f = oracle_frame(s, tl)
    planes = [np.ascontiguousarray(p) for p in (f.light_pass().reshape(H, W, 4), f.albedo.reshape(H, W),
                                                 f.normal.reshape(H, W, 4), f.material.reshape(H, W),
                                                 f.emission.reshape(H, W), f.depth.reshape(H, W))]
    for t in range(7):
        ours = O.compose(*planes, image_type=t)
        ref = np.zeros((H, W, 4), np.float32)
        ref_compose(*[O._p(p) for p in planes], W, H, t, O._p(ref))
        q = (np.clip(np.nan_to_num(ref, nan=0.0), 0, 1) * 255 + 0.5).astype(np.uint32)
        words = q[..., 2] | (q[..., 1] << 8) | (q[..., 0] << 16) | (255 << 24)
        assert np.array_equal(words, ours), t


def test_histogram_matches_reference_shaders():
    """histogram.comp and histogramAverage.comp from the reference tree. The bin of every
    pixel comes from the shader's HDRToHistogramBin: the oracle's counts equal the
    count of the reference's bins, bin for bin. histogramAverage.comp's workgroup runs
    phase by phase over those counts: its weighted sum, log average, average and adapted
    luminance equal the oracle's. Two deliberate deviations are checked as such: the
    shader stores the weighted bin sum where the next frame reads its adapted luminance
    (here the adapted luminance is carried), and every workgroup of histogram.comp
    zeroes the global bins before adding its own (here the bins are exact counts)."""
    lib = REF
    lib.ref_histogram_bins.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
    lib.ref_histogram_average.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_float, C.c_float, C.c_void_p]
    rng = np.random.default_rng(3)
    H, W = 48, 64
    img = np.zeros((H, W, 4), np.float32)
    img[..., :3] = np.exp2(rng.uniform(-14.0, 5.0, size=(H, W, 3))).astype(np.float32)
    img[:2] = 0.0                                   # below LUZ_EPS: bin 0
    img[2, :8, :3] = 1e30                           # clamped to the top bin
    ref_bins = np.zeros(H * W, np.uint32)
    lib.ref_histogram_bins(O._p(img), H * W, O._p(ref_bins))
    counts = np.bincount(ref_bins, minlength=256).astype(np.uint32)
    state = np.array([0.37], np.float32)
    want, _ = O.histogram(img, 1.0 / 60.0, state.copy())
    assert np.array_equal(want["bins"], counts)
    assert counts[0] >= 2 * W and counts[255] >= 8
    out = np.zeros(5, np.float32)
    lib.ref_histogram_average(O._p(counts), W, H, C.c_float(1.0 / 60.0), C.c_float(state[0]), O._p(out))
    assert out[0] == np.float32(want["weighted_sum"])
    assert out[1] == np.float32(want["log_average"])
    assert np.isclose(out[2], want["average_luminance"], rtol=1e-6)
    assert np.isclose(out[3], want["adapted_luminance"], rtol=1e-6)
    assert out[4] == out[0] and out[4] != np.float32(want["adapted_luminance"])   # what the shader stores
