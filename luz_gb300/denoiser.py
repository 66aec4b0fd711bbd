"""The learned AO denoiser: handle, checkpoints, training pairs, training and RMSE.

Pairs follow the training recipe of the path: scenes of the config-1 generator with
seeded cameras (config 3), 256x256; input = 1 AO sample and 1 shadow sample per
light per pixel, target = the 1024-sample AO of the same pixels. Samples come from
the stratified sequence (LUZ_SAMPLER_STRATIFIED): the reference's float recurrence
repeats values long before 1024 samples.

The dataset lives in device memory (torch tensors as plain buffers); every compute
step is a libluz_gb300 kernel.
"""
from __future__ import annotations

import ctypes as C
import json
import math
import time
from pathlib import Path

import numpy as np

from . import (PLANE_AO, PLANE_AO_DENOISED, PLANE_NORMAL, SAMPLER_STRATIFIED, Context, GPUScene, HostScene, Tlas,
               _abi, _check, blue_noise, lib)

WEIGHTS_DIR = Path(__file__).resolve().parent / "weights"
DEFAULT_WEIGHTS = WEIGHTS_DIR / "denoiser_config3.bin"


class Denoiser:
    def __init__(self, ctx: Context, seed: int = 1):
        self.ctx = ctx
        h = C.c_void_p()
        _check(lib.luz_denoiser_create(ctx.handle, seed, C.byref(h)), ctx.handle, "denoiser create")
        self._h = h
        self.meta: dict = {"seed": seed, "step": 0}
        ctx._adopt(self)

    @property
    def handle(self):
        return self._h

    def weights(self) -> np.ndarray:
        w = np.zeros(_abi.DENOISER_PARAMS, np.float32)
        _check(lib.luz_denoiser_get_weights(self.ctx.handle, self._h, _abi.ptr(w, _abi.c_float_p)), self.ctx.handle)
        return w

    def set_weights(self, w: np.ndarray) -> None:
        w = np.ascontiguousarray(w, np.float32)
        assert w.size == _abi.DENOISER_PARAMS
        _check(lib.luz_denoiser_set_weights(self.ctx.handle, self._h, _abi.ptr(w, _abi.c_float_p)), self.ctx.handle)

    # checkpoint: FP32 parameters + JSON header (step, seed, shapes, training record)
    def save(self, path: Path, **meta) -> None:
        path = Path(path)
        path.parent.mkdir(parents=True, exist_ok=True)
        self.weights().tofile(path)
        m = dict(self.meta, **meta)
        m["params"] = _abi.DENOISER_PARAMS
        m["layout"] = "W1[64][72] b1[64] W2[64][64] b2[64] W3[64][64] b3[64] W4[49][64] b4[49], FP32"
        path.with_suffix(".json").write_text(json.dumps(m, indent=1))

    def load(self, path: Path = DEFAULT_WEIGHTS) -> None:
        path = Path(path)
        self.set_weights(np.fromfile(path, np.float32))
        js = path.with_suffix(".json")
        if js.exists():
            self.meta = json.loads(js.read_text())

    def denoise(self, frame) -> None:
        _check(lib.luz_denoise(self.ctx.handle, self._h, frame.handle), self.ctx.handle, "denoise")

    def gradient(self, batch: _abi.DenoiseBatch):
        g = np.zeros(_abi.DENOISER_PARAMS, np.float32)
        loss = C.c_float()
        _check(lib.luz_denoiser_gradient(self.ctx.handle, self._h, C.byref(batch), _abi.ptr(g, _abi.c_float_p),
                                         C.byref(loss)), self.ctx.handle, "denoiser gradient")
        return g, loss.value

    def train_step(self, batch: _abi.DenoiseBatch, lr: float) -> float:
        loss = C.c_float()
        _check(lib.luz_denoiser_train_step(self.ctx.handle, self._h, C.byref(batch), lr, C.byref(loss)),
               self.ctx.handle, "denoiser train step")
        self.meta["step"] = self.meta.get("step", 0) + 1
        return loss.value

    def infer(self, batch: _abi.DenoiseBatch, out_ptr: int) -> None:
        _check(lib.luz_denoise_batch_infer(self.ctx.handle, self._h, C.byref(batch), C.c_void_p(out_ptr)),
               self.ctx.handle, "denoiser infer")

    def close(self):
        if self._h:
            lib.luz_denoiser_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()


class PairSet:
    """N images of W x H in device memory: features, distances, noisy AO, target AO."""

    def __init__(self, n: int, width: int, height: int, device: int = 0):
        import torch
        dev = torch.device("cuda", device)
        self.n, self.width, self.height = n, width, height
        self.feat = torch.zeros((n, height, width, 8), dtype=torch.int16, device=dev)
        self.lin_depth = torch.zeros((n, height, width), dtype=torch.float32, device=dev)
        self.noisy = torch.zeros((n, height, width), dtype=torch.float32, device=dev)
        self.target = torch.zeros((n, height, width), dtype=torch.float32, device=dev)

    def batch(self, i0: int, count: int, with_target: bool = True) -> _abi.DenoiseBatch:
        b = _abi.DenoiseBatch()
        b.features = self.feat[i0].data_ptr()
        b.lin_depth = self.lin_depth[i0].data_ptr()
        b.noisy_ao = self.noisy[i0].data_ptr()
        b.target_ao = self.target[i0].data_ptr() if with_target else None
        b.width, b.height, b.images = self.width, self.height, count
        return b


def _trace_ao(frame, tlas, scene: HostScene, ao_spp: int, light_spp: int, frame_index: int):
    scene.set_sampling(ao_spp, light_samples=light_spp, sampler=SAMPLER_STRATIFIED)
    frame.upload(scene.block(), scene.lights(), scene.light_count, scene.models(), scene.instance_count)
    frame.trace(tlas, frame_index)


def render_pairs(ctx: Context, n: int, size: int = 256, seed0: int = 20000, target_spp: int = 1024,
                 log=None) -> PairSet:
    """Renders n config-3 scenes (one BLAS set, a fresh TLAS per scene)."""
    import torch
    first = HostScene(3, seed=seed0, width=size, height=size)
    blas = ctx.build_blas(first.meshes())
    tlas = ctx.tlas(256)
    frame = ctx.frame(size, size)
    ctx.set_blue_noise(blue_noise())
    pairs = PairSet(n, size, size)
    t0 = time.perf_counter()
    for s in range(n):
        sc = HostScene(3, seed=seed0 + s, width=size, height=size)
        inst, cnt = Tlas.make_instances(blas, sc.instance_mesh(), sc.transforms())
        sc.set_sampling(1, light_samples=1, sampler=SAMPLER_STRATIFIED)
        frame.upload(sc.block(), sc.lights(), sc.light_count, sc.models(), sc.instance_count)
        tlas.build(inst, cnt)
        frame.gbuffer(tlas)
        frame.trace(tlas, s)
        frame.denoise_features()
        pairs.feat[s] = torch.from_numpy(frame.read(_abi.PLANE_FEATURES).view(np.int16))
        pairs.lin_depth[s] = torch.from_numpy(frame.read(_abi.PLANE_LIN_DEPTH))
        pairs.noisy[s] = torch.from_numpy(frame.read(PLANE_AO))
        _trace_ao(frame, tlas, sc, target_spp, 0, 1_000_000 + s)
        frame.ao_resolve()
        pairs.target[s] = torch.from_numpy(frame.read(PLANE_AO))
        if log and (s + 1) % max(1, n // 10) == 0:
            log(f"pairs {s + 1}/{n} ({time.perf_counter() - t0:.1f} s)")
    ctx.synchronize()
    return pairs


def train(den: Denoiser, pairs: PairSet, epochs: int, batch: int = 16, lr: float = 2e-3, seed: int = 0,
          log=None) -> list[float]:
    """Adam over shuffled batches of consecutive images, cosine-decayed learning rate."""
    rng = np.random.default_rng(seed)
    nb = pairs.n // batch
    steps = epochs * nb
    hist = []
    k = 0
    for e in range(epochs):
        losses = []
        for bi in rng.permutation(nb):
            cur = lr * 0.5 * (1.0 + math.cos(math.pi * k / max(steps, 1)))
            losses.append(den.train_step(pairs.batch(int(bi) * batch, batch), cur))
            k += 1
        hist.append(float(np.mean(losses)))
        if log:
            log(f"epoch {e + 1}/{epochs} mse {hist[-1]:.6f}")
    return hist


def lit_rmse(a: np.ndarray, b: np.ndarray, lit: np.ndarray) -> float:
    d = (a - b)[lit]
    return float(np.sqrt(np.mean(d.astype(np.float64) ** 2))) if d.size else 0.0


def evaluate(g: GPUScene, den: Denoiser | None, spps=(16, 64, 256), target_spp: int = 1024,
             frame_index: int = 7) -> dict:
    """AO RMSE against target_spp samples over lit pixels: denoised 1 spp, raw 1 spp,
    plain N spp (stratified samples, shadows off for the AO-only passes)."""
    fr, tl, sc = g.frame, g.tlas, g.scene
    g.update_resources_gpu()
    fr.gbuffer(tl)
    lit = np.linalg.norm(fr.read(PLANE_NORMAL)[..., :3], axis=-1) > 0
    _trace_ao(fr, tl, sc, target_spp, 0, 1_000_000 + frame_index)
    fr.ao_resolve()
    target = fr.read(PLANE_AO).copy()
    out = {"lit_pixels": int(lit.sum()), "target_spp": target_spp, "plain": {}}
    for n in spps:
        _trace_ao(fr, tl, sc, n, 0, frame_index)
        fr.ao_resolve()
        out["plain"][int(n)] = lit_rmse(fr.read(PLANE_AO), target, lit)
    _trace_ao(fr, tl, sc, 1, 1, frame_index)
    fr.ao_resolve()
    out["raw_1spp"] = lit_rmse(fr.read(PLANE_AO), target, lit)
    if den is not None:
        den.denoise(fr)
        out["denoised_1spp"] = lit_rmse(fr.read(PLANE_AO_DENOISED), target, lit)
        # equal-RMSE sample count of the plain path, from RMSE ~ c / sqrt(N) fitted on spps
        ns = np.array(sorted(out["plain"]), np.float64)
        rs = np.array([out["plain"][int(k)] for k in ns])
        c = float(np.exp(np.mean(np.log(rs) + 0.5 * np.log(ns))))
        out["equal_rmse_spp"] = (c / out["denoised_1spp"]) ** 2 if out["denoised_1spp"] > 0 else float("inf")
    return out
