"""CPU checks of the oracle itself: BVH any-hit against the brute-force all-triangles
any-hit, analytic known answers, the project sin/cos against libm, BVH invariants."""
import math

import numpy as np
import pytest

import luz_gb300 as L
import oracle as O
from tests.pathutil import oracle_frame, oracle_scene


@pytest.mark.parametrize("sampler", [L.SAMPLER_PARITY, L.SAMPLER_STRATIFIED])
def test_bvh_anyhit_equals_bruteforce_config1(sampler):
    s = L.HostScene(1, width=96, height=96, sampler=sampler)
    _, tl = oracle_scene(s)
    a = oracle_frame(s, tl)
    b = oracle_frame(s, tl, brute=True)
    assert np.array_equal(a.shadow_bits, b.shadow_bits)
    assert np.array_equal(a.ao_bits, b.ao_bits)
    assert a.shadow_bits.any() and a.ao_bits.any()


def test_bvh_anyhit_equals_bruteforce_spheres():
    s = L.HostScene(2, width=64, height=36, meshes=3, instances=40, subdivisions=3)
    _, tl = oracle_scene(s)
    a = oracle_frame(s, tl)
    b = oracle_frame(s, tl, brute=True)
    assert np.array_equal(a.shadow_bits, b.shadow_bits)
    assert np.array_equal(a.ao_bits, b.ao_bits)


@pytest.mark.parametrize("cfg", [1, 2])
def test_culled_shadow_rays_leave_the_image_unchanged(cfg):
    # Shadow rays of lights with max(dot(N, L), 0) = 0 are not traced (bit 0): the
    # light pass weights them by that 0, so its output equals tracing every ray.
    kw = dict(width=96, height=96) if cfg == 1 else dict(width=80, height=48, meshes=3, instances=60,
                                                            subdivisions=3)
    s = L.HostScene(cfg, **kw)
    _, tl = oracle_scene(s)
    b, lights, models = s.block(), s.lights(), s.models()
    frames = []
    for cull in (True, False):
        f = O.OracleFrame(tl, b, lights, s.light_count, models, s.instance_count, s.width, s.height)
        f.gbuffer()
        n = f.visibility(0, L.blue_noise(), cull=cull)
        frames.append((f, n, f.light_pass()))
    (fc, nc, oc), (fa, na, oa) = frames
    assert nc < na                                          # some rays were left out
    assert np.array_equal(fc.ao_bits, fa.ao_bits)
    assert not (fc.shadow_bits & ~fa.shadow_bits).any()     # culling only clears bits
    assert (fc.shadow_bits != fa.shadow_bits).any()         # and some culled rays were occluded
    same = (oc.view(np.uint32) == oa.view(np.uint32)) | (np.isnan(oc) & np.isnan(oa))
    assert same.all()


def test_random_rays_bvh_vs_bruteforce():
    s = L.HostScene(1, width=16, height=16)
    _, tl = oracle_scene(s)
    rng = np.random.default_rng(3)
    for _ in range(3000):
        o = rng.uniform([-10, -1, -10], [10, 6, 10]).astype(np.float32)
        d = rng.normal(size=3).astype(np.float32)
        tmax = float(rng.uniform(0.1, 30))
        assert tl.ray(o, d, 0.0, tmax)[0] == tl.ray(o, d, 0.0, tmax, brute=True)[0]


def test_sincos_error_bound():
    x = np.linspace(-20.0, 20.0, 200001, dtype=np.float32)
    s = np.zeros_like(x)
    c = np.zeros_like(x)
    O.load().oracle_sincos(O._p(x), O._p(s), O._p(c), x.size)
    xs = x.astype(np.float64)
    assert np.abs(s - np.sin(xs)).max() < 4e-7
    assert np.abs(c - np.cos(xs)).max() < 4e-7


def test_samplers_known_values():
    lib = O.load()
    import ctypes as C
    dx, dy = C.c_float(), C.c_float()
    for rx, ry in [(0.0, 0.3), (1.0, 0.0), (0.25, 0.25), (0.81, 0.5)]:
        lib.oracle_disk_sample(rx, ry, 2.0, C.byref(dx), C.byref(dy))
        assert abs(math.hypot(dx.value, dy.value) - 2.0 * math.sqrt(rx)) < 1e-6
        h = np.zeros(3, np.float32)
        lib.oracle_hemisphere_sample(rx, ry, O._p(h))
        assert abs(float(np.linalg.norm(h)) - 1.0) < 1e-6
        assert abs(h[2] - math.sqrt(max(0.0, 1.0 - rx))) < 1e-7


def test_ggx_known_answers():
    lib = O.load()
    import ctypes as C
    N = np.array([0, 0, 1], np.float32)
    F0 = np.array([0.04, 0.5, 0.9], np.float32)
    D, G = C.c_float(), C.c_float()
    F = np.zeros(3, np.float32)
    for rough in (0.1, 0.5, 1.0):
        # V = L = N  =>  H = N: D = 1/(pi a^2), a = rough^2; G = 1; F = F0
        lib.oracle_ggx_terms(O._p(N), O._p(N), O._p(N), rough, O._p(F0), C.byref(D), C.byref(G), O._p(F))
        a2 = rough ** 4
        # light.frag:23 evaluates (NdotH2*(a2-1)+1) in float: at NdotH = 1 it cancels to
        # a2 with an absolute error of ~ulp(1), i.e. a relative error of ~1.2e-7 / a2.
        rel_tol = 2.4e-7 / a2 + 1e-6
        assert abs(D.value - 1.0 / (math.pi * a2)) <= rel_tol * D.value
        assert abs(G.value - 1.0) < 1e-6
        assert np.allclose(F, F0, atol=1e-7)
    # grazing: V . H = 0 => F = 1
    V = np.array([1, 0, 0], np.float32)
    Lv = np.array([-1, 0, 0], np.float32)
    lib.oracle_ggx_terms(O._p(N), O._p(V), O._p(np.array([0, 1, 0], np.float32)), 0.5, O._p(F0),
                         C.byref(D), C.byref(G), O._p(F))
    assert np.all(F <= 1.0) and np.all(F >= F0 - 1e-7)
    del Lv


def _quad_scene(with_slab: bool):
    """Ground quad (and optionally an opaque slab above part of it) as raw oracle input."""
    quad = np.zeros((4, 12), np.float32)
    quad[:, :3] = [[-10, 0, -10], [10, 0, -10], [10, 0, 10], [-10, 0, 10]]
    quad[:, 3:6] = [0, 1, 0]
    qi = np.array([0, 2, 1, 0, 3, 2], np.uint32)
    blas = [O.OracleBlas(quad, qi)]
    tr = [np.array([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 1, 0]], np.float32)]
    if with_slab:
        tr.append(np.array([[1, 0, 0, 0], [0, 1, 0, 2.0], [0, 0, 1, 0]], np.float32))
        blas.append(blas[0])
    return O.OracleTlas(blas, np.stack(tr))


def test_open_plane_ao_is_one():
    tl = _quad_scene(False)
    rng = np.random.default_rng(0)
    for _ in range(500):
        o = np.array([rng.uniform(-5, 5), 0.01, rng.uniform(-5, 5)], np.float32)
        d = rng.normal(size=3).astype(np.float32)
        d[1] = abs(d[1]) + 0.05
        assert not tl.ray(o, d, 1e-4, 1.0)[0]          # every AO ray misses


def test_point_under_slab_is_shadowed():
    tl = _quad_scene(True)
    o = np.array([0.5, 0.05, -0.5], np.float32)
    hit, t = tl.ray(o, np.array([0, 1, 0], np.float32), 0.001, 100.0, closest=True)
    assert hit and abs(t - 1.95) < 1e-5
    assert tl.ray(o, np.array([0.1, 1, 0.2], np.float32), 0.001, 100.0)[0]
    # the slab is two-sided: a ray from above hits it too
    assert tl.ray(np.array([0, 5, 0], np.float32), np.array([0, -1, 0], np.float32), 0.0, 100.0)[0]


def _box_contains(outer_lo, outer_hi, inner_lo, inner_hi):
    return np.all(outer_lo <= inner_lo) and np.all(outer_hi >= inner_hi)


def test_blas_invariants():
    s = L.HostScene(2, width=16, height=16, meshes=1, instances=1, subdivisions=3)
    (v, idx), = s.meshes()
    b = O.OracleBlas(v, idx)
    nodes, tris, mort, order = b.arrays()
    assert np.all(np.diff(mort.astype(np.int64)) >= 0)
    assert np.array_equal(np.sort(order), np.arange(len(order)))
    ch = nodes[:, 12:14].view(np.int32)
    leaves = ch[ch < 0]
    assert np.array_equal(np.sort(~leaves), np.arange(len(order)))
    internal = ch[ch >= 0]
    assert np.array_equal(np.sort(internal), np.arange(1, nodes.shape[0]))
    for j in range(len(order)):
        t = tris[j].reshape(3, 4)[:, :3]
        p = order[j]
        assert np.array_equal(t, v[idx[3 * p:3 * p + 3], :3])


def test_light_pass_f32_vs_f64_reported():
    s = L.HostScene(1, width=64, height=64)
    _, tl = oracle_scene(s)
    f = oracle_frame(s, tl)
    a = f.light_pass()
    b = f.light_pass(f64=True)
    assert np.isfinite(a).all() and np.isfinite(b).all()
    rel = np.abs(a - b) / np.maximum(np.abs(b), 1e-6)
    assert rel.max() < 1e-2
