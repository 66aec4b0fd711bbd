"""CPU: the FP64 denoiser oracle's analytic gradient against central differences
(ratio-estimator shadow outputs and AO, weighted loss)."""
import numpy as np

from oracle import denoiser as OD


def _problem(seed=0, n=1, h=9, w=10):
    rng = np.random.default_rng(seed)
    feat = OD.bf16_round(rng.uniform(-1, 1, size=(n, h, w, 8)).astype(np.float32))
    bits = (feat.view(np.uint32) >> 16).astype(np.uint16)
    ld = rng.uniform(5, 6, size=(n, h, w)).astype(np.float32)
    ld[0, 0, :3] = 0   # a few background pixels
    # split of the direct light: unshadowed U > 0 (a few 0 channels), shadowed S = U x a
    # 1-sample visibility mix, and a 1-sample AO (0 or 1)
    uns = rng.uniform(0.1, 3.0, size=(n, h, w, 4)).astype(np.float32)
    uns[0, 1, 1:4, 0] = 0.0
    sig = np.empty_like(uns)
    sig[..., :3] = uns[..., :3] * rng.choice([0.0, 0.4, 1.0], size=(n, h, w, 3)).astype(np.float32)
    sig[..., 3] = (rng.uniform(size=(n, h, w)) < 0.6).astype(np.float32)
    tgt = rng.uniform(0.3, 0.9, size=(n, h, w, 4)).astype(np.float32)
    params = (rng.normal(size=16177) * 0.2).astype(np.float32)
    params = OD.bf16_round(params)   # exactly representable: the oracle rounds weights to BF16
    return params, bits, ld, (sig, uns), tgt


def test_fp64_gradient_matches_central_differences():
    params, bits, ld, ao, tgt = _problem()
    _, loss, g = OD.forward_backward(params, bits, ld, ao[0], ao[1], tgt)
    rng = np.random.default_rng(1)
    # biases are not rounded to BF16, so they admit small perturbations
    layout = [(64 * 72, 64), (64 * 64, 64), (64 * 64, 64), (49 * 64, 49)]
    starts, o = [], 0
    for nw, nb in layout:
        starts.append(o + nw)
        o += nw + nb
    idx = np.concatenate([s + rng.choice(nb, 6, replace=False) for s, (_, nb) in zip(starts, layout)])
    eps = 1e-4
    for i in idx:
        p1 = params.astype(np.float64).copy()
        p2 = params.astype(np.float64).copy()
        p1[i] += eps
        p2[i] -= eps
        l1 = OD.forward_backward(p1, bits, ld, ao[0], ao[1], tgt)[1]
        l2 = OD.forward_backward(p2, bits, ld, ao[0], ao[1], tgt)[1]
        num = (l1 - l2) / (2 * eps)
        assert abs(num - g[i]) <= 1e-6 + 1e-4 * abs(g[i]), (i, num, g[i])


def test_gather_clamps_and_zeroes_background():
    params, bits, ld, ao, tgt = _problem(h=4, w=5)
    X, valid = OD.gather(bits, ld)
    assert X.shape == (1, 4, 5, 72)
    assert not valid[0, 0, 0] and np.all(X[0, 0, 0] == 0)
    # centre tap channel 5 (relative depth to itself) is zero
    assert np.all(X[valid][:, 4 * 8 + 5] == 0)
