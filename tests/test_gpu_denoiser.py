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
            pairs.noisy[:n].cpu().numpy(), pairs.target[:n].cpu().numpy())


def test_gradient_matches_fp64_oracle(setup):
    ctx, D, pairs, den, torch = setup
    g, loss = den.gradient(pairs.batch(0, 4))
    feat, ld, ao, tgt = _host(pairs, 4)
    _, loss64, g64 = OD.forward_backward(den.weights(), feat, ld, ao, tgt)
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
    out = torch.zeros((2, 64, 64), dtype=torch.float32, device="cuda")
    den.infer(pairs.batch(0, 2, with_target=False), out.data_ptr())
    torch.cuda.synchronize()
    feat, ld, ao, tgt = _host(pairs, 2)
    y64, _, _ = OD.forward_backward(den.weights(), feat, ld, ao, tgt)
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
    """What the trained network gains over the method without it: AO RMSE against
    1024 samples, denoised 1 sample vs the plain 1-sample estimate, on a held-out
    config-3 scene."""
    pytest.importorskip("torch")
    from luz_gb300 import denoiser as D
    if not D.DEFAULT_WEIGHTS.exists():
        pytest.skip("no trained weights committed")
    ctx = L.Context(0)
    try:
        den = D.Denoiser(ctx)
        den.load(D.DEFAULT_WEIGHTS)
        g = L.GPUScene(ctx, L.HostScene(3, seed=987654, width=256, height=256))
        r = D.evaluate(g, den, spps=(4, 16), target_spp=1024)
        assert r["denoised_1spp"] < 0.5 * r["raw_1spp"], r
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
        b.noisy_ao = fr.device_ptr(L.PLANE_AO)
        b.target_ao = None
        b.width, b.height, b.images = w, h, 1
        out = torch.full((h, w), float("nan"), dtype=torch.float32, device="cuda")
        second.infer(b, out.data_ptr())
        ctx.synchronize()
        assert ctx.device_status() == 0
        dense = out.cpu().numpy().reshape(-1)
        framed = fr.read(L.PLANE_AO_DENOISED).reshape(-1)
        assert np.array_equal(dense.view(np.uint32), framed.view(np.uint32))
        lit = fr.read(L.PLANE_LIN_DEPTH).reshape(-1) > 0
        assert lit.sum() > 0 and np.all(framed[~lit] == 0.0)
    finally:
        ctx.close()


def test_features_count_the_sample_bits():
    """The features pass counts, per lit pixel, the set AO bits and the occluded shadow
    bits over all sample planes (more than 32 of each: two groups of the per-lane load)."""
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
        sh_hits, n_sh = counts(L.PLANE_SHADOW_BITS)
        assert n_ao == 40 and n_sh == 40
        lit = np.linalg.norm(fr.read(L.PLANE_NORMAL).reshape(-1, 4)[:, :3], axis=1) > 0
        assert lit.any()
        ao = np.where(lit, ao_hits.astype(np.float32) / np.float32(n_ao), np.float32(0)).astype(np.float32)
        assert np.array_equal(fr.read(L.PLANE_AO).reshape(-1), ao)
        feat = fr.read(L.PLANE_FEATURES).reshape(-1, 8)
        lit_frac = np.float32(1) - sh_hits.astype(np.float32) / np.float32(n_sh)
        assert np.array_equal(OD.bf16_bits_to_f32(feat[lit, 0]), OD.bf16_round(ao[lit]))
        assert np.array_equal(OD.bf16_bits_to_f32(feat[lit, 1]), OD.bf16_round(lit_frac[lit]))
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
    finally:
        ctx.close()
