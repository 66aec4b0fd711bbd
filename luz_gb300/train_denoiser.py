"""Trains the shadow + AO denoiser on the GPU and writes a checkpoint (FP32 weights + JSON).

    python -m luz_gb300.train_denoiser --scenes 2000 --size 256 --epochs 20 \
        --out luz_gb300/weights/denoiser_config3.bin

Pairs: config-3 scenes (config-1 generator, seeded cameras), 256x256 images (crops
of 1920x1080 images with --crops), 1-sample input (1 AO ray and 1 shadow ray per light) and the
1024-sample target (shadow ratio of the direct light and AO). Evaluation: a held-out
config-3 scene at 1920x1080, AO and radiance RMSE against 1024 samples for the
denoised single sample and the plain path (AO and shadow rays per light alike).
"""
from __future__ import annotations

import argparse
import json
import time

import luz_gb300 as L
from luz_gb300 import denoiser as D


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--scenes", type=int, default=2000)
    ap.add_argument("--size", type=int, default=256)
    ap.add_argument("--target-spp", type=int, default=1024)
    ap.add_argument("--epochs", type=int, default=20)
    ap.add_argument("--batch", type=int, default=16)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--shadow-weight", type=float, default=0.0,
                    help="loss weight of each shadow-ratio output (the AO output weighs 1)")
    ap.add_argument("--radiance-weights", action="store_true",
                    help="weight each pixel's shadow-ratio error by its squared unshadowed direct light "
                         "(relative to the set's RMS), so that it counts as the radiance error it causes")
    ap.add_argument("--crops", action="store_true",
                    help="train on size x size crops of 1920x1080 images instead of whole size x size images")
    ap.add_argument("--out", default=str(D.DEFAULT_WEIGHTS))
    ap.add_argument("--resume", default=None, help="checkpoint to start from")
    ap.add_argument("--no-eval", action="store_true")
    a = ap.parse_args()
    import torch

    ctx = L.Context(0)
    log = lambda m: print(m, flush=True)  # noqa: E731
    t0 = time.perf_counter()
    pairs = D.render_pairs(ctx, a.scenes, size=a.size, seed0=20000, target_spp=a.target_spp,
                           crop_of=(1920, 1080) if a.crops else None, log=log)
    t_pairs = time.perf_counter() - t0
    den = D.Denoiser(ctx, seed=a.seed)
    if a.resume:
        den.load(a.resume)
    den.set_shadow_weight(a.shadow_weight)
    if a.radiance_weights:
        pairs.radiance_weights(a.shadow_weight)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    hist = D.train(den, pairs, a.epochs, batch=a.batch, lr=a.lr, seed=a.seed, log=log)
    ctx.synchronize()
    t_train = time.perf_counter() - t1
    steps = a.epochs * (a.scenes // a.batch)
    px = steps * a.batch * a.size * a.size
    record = {"scenes": a.scenes, "size": a.size, "target_spp": a.target_spp, "epochs": a.epochs,
              "batch": a.batch, "lr": a.lr, "seed": a.seed, "shadow_weight": a.shadow_weight,
              "radiance_weights": a.radiance_weights, "crops_of": [1920, 1080] if a.crops else None,
              "loss_history": hist,
              "pair_generation_s": t_pairs, "train_s": t_train, "train_steps": steps,
              "train_pixels_per_s": px / t_train,
              "train_tflops_bf16": px * 3 * 31872 / t_train / 1e12}
    if not a.no_eval:
        g = L.GPUScene(ctx, L.HostScene(3, seed=424242, width=1920, height=1080))
        record["eval_1080p_config3"] = D.evaluate(g, den, target_spp=1024)
        # a held-out scene of the two-level icosphere generator (the benchmark frame uses
        # seed 1002): how the network trained on cube scenes carries over
        g2 = L.GPUScene(ctx, L.HostScene(2, seed=7777))
        record["eval_1080p_config2_validation"] = D.evaluate(g2, den, target_spp=1024)
    den.save(a.out, **record)
    print(json.dumps({k: v for k, v in record.items() if k != "loss_history"}), flush=True)
    ctx.close()


if __name__ == "__main__":
    main()
