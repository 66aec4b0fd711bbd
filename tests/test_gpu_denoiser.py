"""The BF16 tensor-core denoiser against its FP64 oracle, on the GPU."""
import numpy as np
import pytest

import luz_gb300 as L
from oracle import denoiser as OD

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def setup():
    torch = pytest.importorskip("torch")
    from luz_gb300 import denoiser as D
    ctx = L.Context(0)
    pairs = D.render_pairs(ctx, 4, size=64, seed0=777, target_spp=64)
    den = D.Denoiser(ctx, seed=3)
    yield ctx, D, pairs, den, torch
    ctx.close()


def _host(pairs, n):
    return (pairs.feat[:n].cpu().numpy().view(np.uint16), pairs.lin_depth[:n].cpu().numpy(),
            pairs.noisy[:n].cpu().numpy(), pairs.unshadowed[:n].cpu().numpy(), pairs.target[:n].cpu().numpy())


def test_gradient_matches_fp64_oracle(setup):
    ctx, D, pairs, den, torch = setup
    g, loss = den.gradient(pairs.batch(0, 4))
    feat, ld, sig, uns, tgt = _host(pairs, 4)
    _, loss64, g64 = OD.forward_backward(den.weights(), feat, ld, sig, uns, tgt)
    assert abs(loss - loss64) <= 2e-2 * loss64
    cos = float(g @ g64 / (np.linalg.norm(g) * np.linalg.norm(g64)))
    rel = float(np.linalg.norm(g - g64) / np.linalg.norm(g64))
    assert cos > 0.995 and rel < 6e-2, (cos, rel)


def test_weighted_gradient_matches_fp64_oracle(setup):
    """Per-pixel, per-output loss weights (the radiance-aligned weights of training)."""
    ctx, D, pairs, den, torch = setup
    g0 = torch.Generator(device="cpu").manual_seed(5)
    w = torch.rand((4, 64, 64, 4), generator=g0).mul_(3.0).to("cuda")
    b = pairs.batch(0, 4)
    b.weight = w.data_ptr()
    g, loss = den.gradient(b)
    feat, ld, sig, uns, tgt = _host(pairs, 4)
    _, loss64, g64 = OD.forward_backward(den.weights(), feat, ld, sig, uns, tgt, weight=w.cpu().numpy())
    assert abs(loss - loss64) <= 2e-2 * loss64
    cos = float(g @ g64 / (np.linalg.norm(g) * np.linalg.norm(g64)))
    rel = float(np.linalg.norm(g - g64) / np.linalg.norm(g64))
    assert cos > 0.995 and rel < 6e-2, (cos, rel)


def test_gradient_is_deterministic(setup):
    ctx, D, pairs, den, torch = setup
    g1, l1 = den.gradient(pairs.batch(0, 4))
    g2, l2 = den.gradient(pairs.batch(0, 4))
    assert np.array_equal(g1.view(np.uint32), g2.view(np.uint32)) and l1 == l2


def test_inference_matches_fp64_oracle(setup):
    ctx, D, pairs, den, torch = setup
    out = torch.zeros((2, 64, 64, 4), dtype=torch.float32, device="cuda")
    den.infer(pairs.batch(0, 2, with_target=False), out.data_ptr())
    torch.cuda.synchronize()
    feat, ld, sig, uns, tgt = _host(pairs, 2)
    y64, _, _ = OD.forward_backward(den.weights(), feat, ld, sig, uns, tgt)
    assert np.abs(out.cpu().numpy() - y64).max() < 2e-2


def test_training_reduces_loss(setup):
    ctx, D, pairs, den, torch = setup
    d2 = D.Denoiser(ctx, seed=5)
    first = d2.train_step(pairs.batch(0, 4), 3e-3)
    for _ in range(60):
        last = d2.train_step(pairs.batch(0, 4), 3e-3)
    assert last < 0.7 * first, (first, last)
    d2.close()


def test_trained_network_beats_plain_one_sample():
    """What the trained network gains over the method without it, on a held-out
    config-3 scene, against 1024 samples: the AO RMSE and the radiance RMSE (shadows
    of every light and AO together) of the denoised single sample against the plain
    single-sample frame, and the plain sample count the denoised frame matches."""
    pytest.importorskip("torch")
    from luz_gb300 import denoiser as D
    if not D.DEFAULT_WEIGHTS.exists():
        pytest.skip("no trained weights committed")
    ctx = L.Context(0)
    try:
        den = D.Denoiser(ctx)
        den.load(D.DEFAULT_WEIGHTS)
        g = L.GPUScene(ctx, L.HostScene(3, seed=987654, width=256, height=256))
        r = D.evaluate(g, den, spps=(2, 4, 16), target_spp=1024)
        assert r["denoised_1spp_ao"] < 0.5 * r["raw_1spp_ao"], r
        assert r["denoised_1spp_radiance"] < 0.75 * r["raw_1spp_radiance"], r
        assert r["equal_rmse_spp_ao"] > 4 and r["equal_rmse_spp_radiance"] > 2, r
    finally:
        ctx.close()


@pytest.mark.parametrize("size", [(200, 120), (64, 64)])
def test_frame_path_over_lit_pixels_matches_dense_batch(size):
    """luz_denoise filters only the frame's lit pixels (its compacted list) and leaves 0
    at the background; the batch entry point runs over every pixel of the same planes.
    Both must agree bit for bit."""
    torch = pytest.importorskip("torch")
    from luz_gb300 import denoiser as D
    from luz_gb300 import _abi
    ctx = L.Context(0)
    try:
        w, h = size
        g = L.GPUScene(ctx, L.HostScene(1, width=w, height=h))
        g.render(0)
        fr = g.frame
        first, second = D.Denoiser(ctx, seed=21), D.Denoiser(ctx, seed=22)
        first.denoise(fr)            # leaves other values in the plane for the second pass to replace
        second.denoise(fr)
        b = _abi.DenoiseBatch()
        b.features = fr.device_ptr(L.PLANE_FEATURES)
        b.lin_depth = fr.device_ptr(L.PLANE_LIN_DEPTH)
        b.noisy = fr.device_ptr(L.PLANE_SIGNAL)
        b.unshadowed = fr.device_ptr(L.PLANE_UNSHADOWED)
        b.target = None
        b.width, b.height, b.images = w, h, 1
        out = torch.full((h, w, 4), float("nan"), dtype=torch.float32, device="cuda")
        second.infer(b, out.data_ptr())
        ctx.synchronize()
        assert ctx.device_status() == 0
        dense = out.cpu().numpy().reshape(-1, 4)
        framed = fr.read(L.PLANE_DENOISED).reshape(-1, 4)
        assert np.array_equal(dense.view(np.uint32), framed.view(np.uint32))
        ao = fr.read(L.PLANE_AO_DENOISED).reshape(-1)
        assert np.array_equal(ao.view(np.uint32), framed[:, 3].copy().view(np.uint32))
        lit = fr.read(L.PLANE_LIN_DEPTH).reshape(-1) > 0
        assert lit.sum() > 0 and np.all(framed[~lit] == 0.0)
    finally:
        ctx.close()


def test_features_count_the_sample_bits():
    """The network inputs per lit pixel: the AO value is the mean of the AO miss bits over
    all sample planes (40 here), the shadow feature the unoccluded fraction of all shadow
    samples, both rounded to BF16; background pixels are zero."""
    from oracle import denoiser as OD
    ctx = L.Context(0)
    try:
        w, h = 200, 120
        s = L.HostScene(1, width=w, height=h)
        s.set_sampling(40, light_samples=8)           # 40 AO planes, 5 lights x 8 shadow planes
        g = L.GPUScene(ctx, s)
        g.render(0)
        fr = g.frame
        fr.denoise_features()
        ctx.synchronize()
        assert ctx.device_status() == 0
        P, words = w * h, (w * h + 31) // 32

        def counts(plane):
            raw = fr.read(plane).reshape(-1).view(np.uint32)
            planes = raw.size // words
            bits = (raw.reshape(planes, words)[:, :, None] >> np.arange(32, dtype=np.uint32)) & 1
            return bits.reshape(planes, -1)[:, :P].sum(0), planes

        ao_hits, n_ao = counts(L.PLANE_AO_BITS)
        _, n_sh = counts(L.PLANE_SHADOW_BITS)
        assert n_ao == 40 and n_sh == 40
        lit = np.linalg.norm(fr.read(L.PLANE_NORMAL).reshape(-1, 4)[:, :3], axis=1) > 0
        assert lit.any()
        ao = np.where(lit, ao_hits.astype(np.float32) / np.float32(n_ao), np.float32(0)).astype(np.float32)
        assert np.array_equal(fr.read(L.PLANE_AO).reshape(-1), ao)
        assert np.array_equal(fr.read(L.PLANE_SIGNAL).reshape(-1, 4)[:, 3], ao)
        feat = fr.read(L.PLANE_FEATURES).reshape(-1, 8)
        sh_hits, _ = counts(L.PLANE_SHADOW_BITS)
        shadow = np.float32(1) - sh_hits.astype(np.float32) / np.float32(n_sh)
        assert np.array_equal(fr.read(L.PLANE_UNSHADOWED).reshape(-1, 4)[lit, 3], shadow[lit])
        assert np.array_equal(OD.bf16_bits_to_f32(feat[lit, 0]), OD.bf16_round(ao[lit]))
        assert np.array_equal(OD.bf16_bits_to_f32(feat[lit, 1]), OD.bf16_round(shadow[lit]))
        assert np.all(feat[~lit] == 0)
    finally:
        ctx.close()


def test_frame_with_nothing_lit_denoises_to_zero():
    """An empty lit-pixel list: the network runs over no tile and every pixel of the
    denoised plane is the background's 0."""
    ctx = L.Context(0)
    try:
        from luz_gb300 import denoiser as D
        s = L.HostScene(1, width=64, height=48)
        cam = s.camera()
        cam.mode = 2
        cam.eye[:] = (0.0, 50.0, 0.0)
        cam.center[:] = (0.0, 100.0, 1.0)       # looking up into empty sky
        s.set_camera(cam)
        g = L.GPUScene(ctx, s)
        g.render(0)
        den = D.Denoiser(ctx, seed=4)
        den.denoise(g.frame)
        ctx.synchronize()
        assert ctx.device_status() == 0
        assert g.frame.lit_count() == 0
        assert np.all(g.frame.read(L.PLANE_AO_DENOISED) == 0.0)
        assert np.all(g.frame.read(L.PLANE_DENOISED) == 0.0)
    finally:
        ctx.close()


def test_split_of_the_direct_light_matches_oracle():
    """The denoiser's input pass: per lit pixel light.frag's direct light S (shadowed)
    and U (every shadow factor 0), the AO value and the unoccluded fraction of the
    shadow samples, against the oracle's restatement on the same frame (bit-exact
    visibility). S and U within 1e-4 relative, as the radiance; the counts exact."""
    from tests.pathutil import oracle_frame, oracle_scene
    ctx = L.Context(0)
    try:
        s = L.HostScene(1, width=160, height=120)
        s.set_sampling(4, light_samples=3)
        g = L.GPUScene(ctx, s)
        g.render(0)
        g.frame.denoise_features()
        ctx.synchronize()
        assert ctx.device_status() == 0
        _, tl = oracle_scene(s)
        f = oracle_frame(s, tl)
        assert np.array_equal(g.frame.read(L.PLANE_SHADOW_BITS), f.shadow_bits[: f.shadow_slots])
        o_sig, o_u = f.light_split()
        sig, u = g.frame.read(L.PLANE_SIGNAL), g.frame.read(L.PLANE_UNSHADOWED)
        lit = np.linalg.norm(g.frame.read(L.PLANE_NORMAL)[..., :3], axis=-1) > 0
        assert lit.sum() > 1000 and np.all(sig[~lit] == 0) and np.all(u[~lit] == 0)
        for a, b in ((u[..., :3], o_u[..., :3]), (sig[..., :3], o_sig[..., :3])):
            rel = np.abs(a - b) / np.maximum(np.abs(b), 1e-6)
            assert rel[lit].max() <= 1e-4, rel[lit].max()
        assert np.array_equal(u[..., 3][lit], o_u[..., 3][lit])
        assert np.array_equal(sig[..., 3][lit], o_sig[..., 3][lit])          # AO = misses / samples
        ratio = u[..., 3][lit]
        assert (ratio < 1).any() and (ratio == 1).any()                        # shadowed and lit pixels
    finally:
        ctx.close()


def test_denoised_frame_is_composed_from_the_filtered_signal():
    """LUZ_LIGHT_PASS_DENOISED: ambient * AO + U * R + emission per channel from the
    denoised plane; unlit pixels keep the background colour."""
    from luz_gb300 import denoiser as D
    ctx = L.Context(0)
    try:
        s = L.HostScene(1, width=96, height=80)
        s.set_sampling(1, light_samples=1, sampler=L.SAMPLER_STRATIFIED)
        g = L.GPUScene(ctx, s)
        g.render(0)
        fr = g.frame
        den = D.Denoiser(ctx, seed=8)
        den.denoise(fr)
        fr.light_pass(L.LIGHT_PASS_DENOISED)
        ctx.synchronize()
        assert ctx.device_status() == 0
        d, u = fr.read(L.PLANE_DENOISED), fr.read(L.PLANE_UNSHADOWED)
        albedo = fr.read(L.PLANE_ALBEDO).view(np.uint8).reshape(80, 96, 4)
        mat = fr.read(L.PLANE_MATERIAL).view(np.uint8).reshape(80, 96, 4)
        emi = fr.read(L.PLANE_EMISSION).view(np.uint8).reshape(80, 96, 4)
        b = s.block()
        amb = np.array(b.ambient_light_color, np.float64) * b.ambient_light_intensity
        lut = np.array([np.float32(np.float64(np.float32(i / 255.0)) ** 2.2) for i in range(256)], np.float64)
        want = (amb * lut[albedo[..., :3]] * (mat[..., 2:3] / 255.0) * d[..., 3:4] + u[..., :3] * d[..., :3] +
                emi[..., :3] / 255.0)
        got = fr.read(L.PLANE_LIGHT)
        lit = np.linalg.norm(fr.read(L.PLANE_NORMAL)[..., :3], axis=-1) > 0
        assert lit.sum() > 500
        assert np.abs(got[..., :3] - want)[lit].max() <= 1e-5 * max(1.0, np.abs(want[lit]).max())
        assert np.allclose(got[~lit][:, :3], amb, rtol=1e-6) and np.all(got[..., 3] == 1.0)
        # the ratio estimator keeps every output ratio in [0, 1]
        assert np.all((d[..., :3][lit] >= 0) & (d[..., :3][lit] <= 1))
    finally:
        ctx.close()
