"""The learned shadow + AO denoiser: handle, checkpoints, training pairs, training
and RMSE.

Pairs follow the training recipe of the path: scenes of the config-1 generator with
seeded cameras (config 3), 256x256 (whole images by default; crops of 1920x1080
images on request); input = 1 AO sample and 1 shadow sample per light per pixel,
target = the 1024-sample estimate of the same pixels (shadow ratio of the direct
light and AO). Samples come from the
stratified sequence (LUZ_SAMPLER_STRATIFIED): the reference's float recurrence
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

from . import (LIGHT_PASS_DENOISED, LIGHT_PASS_PLAIN, PLANE_AO, PLANE_AO_DENOISED, PLANE_LIGHT, PLANE_NORMAL,
               PLANE_SIGNAL, PLANE_UNSHADOWED, SAMPLER_STRATIFIED, Context, GPUScene, HostScene, Tlas, _abi, _check,
               blue_noise, lib)

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

    def set_shadow_weight(self, w: float) -> None:
        """Training loss weight of each shadow-ratio output (AO weighs 1)."""
        _check(lib.luz_denoiser_set_shadow_weight(self.ctx.handle, self._h, w), self.ctx.handle, "shadow weight")
        self.meta["shadow_weight"] = w

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
    """N images of W x H in device memory: features, distances, the noisy split of the
    direct light (S r, g, b and AO; U r, g, b and the lit shadow fraction) and the many-sample
    target (shadow ratio r, g, b and AO)."""

    def __init__(self, n: int, width: int, height: int, device: int = 0):
        import torch
        dev = torch.device("cuda", device)
        self.n, self.width, self.height = n, width, height
        self.feat = torch.zeros((n, height, width, 8), dtype=torch.int16, device=dev)
        self.lin_depth = torch.zeros((n, height, width), dtype=torch.float32, device=dev)
        self.noisy = torch.zeros((n, height, width, 4), dtype=torch.float32, device=dev)
        self.unshadowed = torch.zeros((n, height, width, 4), dtype=torch.float32, device=dev)
        self.target = torch.zeros((n, height, width, 4), dtype=torch.float32, device=dev)
        self.weight = None

    def radiance_weights(self, shadow_weight: float) -> None:
        """Per-pixel loss weights that make the shadow-ratio error count as the direct
        radiance error it causes: shadow_weight x (U_c / rms U)^2 for ratio output c,
        with U the unshadowed direct light and rms over the lit pixels of the set; AO 1."""
        import torch
        lit = self.lin_depth > 0
        u = self.unshadowed[..., :3]
        rms = torch.sqrt((u[lit].double() ** 2).mean()).float().clamp_min(1e-12)
        w = torch.ones_like(self.target)
        w[..., :3] = shadow_weight * (u / rms) ** 2
        self.weight = w

    def batch(self, i0: int, count: int, with_target: bool = True) -> _abi.DenoiseBatch:
        b = _abi.DenoiseBatch()
        b.features = self.feat[i0].data_ptr()
        b.lin_depth = self.lin_depth[i0].data_ptr()
        b.noisy = self.noisy[i0].data_ptr()
        b.unshadowed = self.unshadowed[i0].data_ptr()
        b.target = self.target[i0].data_ptr() if with_target else None
        b.weight = self.weight[i0].data_ptr() if (with_target and self.weight is not None) else None
        b.width, b.height, b.images = self.width, self.height, count
        return b


def set_samples(frame, scene: HostScene, ao_spp: int, light_spp: int) -> None:
    """Stratified sampling with ao_spp AO rays and light_spp shadow rays per light (the
    reference's one knob, GPUScene.cpp:248) for the next trace."""
    scene.set_sampling(ao_spp, light_samples=light_spp, sampler=SAMPLER_STRATIFIED)
    frame.upload(scene.block(), scene.lights(), scene.light_count, scene.models(), scene.instance_count)


class _DevicePlane:
    """A frame plane as a CUDA array (__cuda_array_interface__) for torch.as_tensor;
    no copy. Reading it from torch needs torch's stream to be the context's stream."""

    def __init__(self, frame, plane: int, dtype=None):
        dt, comps = _abi.PLANE_DTYPES[plane]
        dt = dtype or dt
        shape = (frame.height, frame.width, comps) if comps > 1 else (frame.height, frame.width)
        self.__cuda_array_interface__ = {"shape": shape, "typestr": np.dtype(dt).str,
                                         "data": (frame.device_ptr(plane), False), "version": 2}


def plane_tensor(frame, plane: int, dtype=None):
    import torch
    return torch.as_tensor(_DevicePlane(frame, plane, dtype), device="cuda")


def shared_stream(ctx: Context):
    """A torch stream that the context also runs on, so that torch reads of frame
    planes are ordered after the library's kernels."""
    import torch
    st = torch.cuda.Stream()
    torch.cuda.set_stream(st)
    ctx.set_stream(st.cuda_stream)
    return st


def reference(frame, tlas, scene: HostScene, spp: int = 1024, per_trace: int = 16, frame0: int = 1_000_000):
    """The many-sample estimate of a frame whose G-buffer is in place: spp AO samples
    and spp shadow samples per light, as spp / per_trace traces of per_trace samples
    each (independent sample rotations per trace). Returns (radiance [H, W, 3],
    signal [H, W, 4]: shadowed direct light r, g, b and AO) as host arrays. The context
    and torch must share a stream (shared_stream)."""
    import torch
    traces = max(1, spp // per_trace)
    set_samples(frame, scene, per_trace, per_trace)
    light = torch.zeros((frame.height, frame.width, 3), dtype=torch.float64, device="cuda")
    sig = torch.zeros((frame.height, frame.width, 4), dtype=torch.float64, device="cuda")
    lp, sp = plane_tensor(frame, PLANE_LIGHT), plane_tensor(frame, PLANE_SIGNAL)
    for t in range(traces):
        frame.trace(tlas, frame0 + t)
        frame.light_pass(LIGHT_PASS_PLAIN)
        frame.denoise_features()           # the split: shadowed direct light and AO
        light += lp[..., :3]
        sig += sp
    return (light / traces).float().cpu().numpy(), (sig / traces).float().cpu().numpy()


def crop_camera(scene: HostScene, full=(1920, 1080), rng=None) -> None:
    """Turns the scene's camera into a width x height crop of a full[0] x full[1] image
    of the same camera (the full image's pixel footprint): the vertical field of view
    shrinks to the crop's rows and the projection is shifted (the camera's NDC jitter)
    to a crop window at a random place of the full image."""
    cam = scene.camera()
    w, h = scene.width, scene.height
    fw, fh = full
    half = math.radians(cam.horizontal_fov) * 0.5
    cam.horizontal_fov = math.degrees(2.0 * math.atan(math.tan(half) * h / fh))
    rng = rng or np.random.default_rng(0)
    cx = rng.uniform(-1.0 + w / fw, 1.0 - w / fw)   # crop centre in the full image's NDC
    cy = rng.uniform(-1.0 + h / fh, 1.0 - h / fh)
    cam.jitter[0] = -cx * fw / w
    cam.jitter[1] = -cy * fh / h
    scene.set_camera(cam)


def render_pairs(ctx: Context, n: int, size: int = 256, seed0: int = 20000, target_spp: int = 1024,
                 per_trace: int = 32, crop_of=None, log=None) -> PairSet:
    """Renders n config-3 scenes (one BLAS set, a fresh TLAS per scene) as size x size
    crops of crop_of-sized images (None: whole size x size images): the 1-sample input
    (1 AO ray, 1 shadow ray per light) and the target_spp-sample target."""
    import torch
    saved = torch.cuda.current_stream()
    shared_stream(ctx)
    first = HostScene(3, seed=seed0, width=size, height=size)
    blas = ctx.build_blas(first.meshes())
    tlas = ctx.tlas(256)
    frame = ctx.frame(size, size)
    ctx.set_blue_noise(blue_noise())
    pairs = PairSet(n, size, size)
    feat, lin = plane_tensor(frame, _abi.PLANE_FEATURES, np.int16), plane_tensor(frame, _abi.PLANE_LIN_DEPTH)
    sig, uns = plane_tensor(frame, PLANE_SIGNAL), plane_tensor(frame, PLANE_UNSHADOWED)
    t0 = time.perf_counter()
    traces = max(1, target_spp // per_trace)
    acc = torch.zeros((size, size, 4), dtype=torch.float64, device="cuda")
    crop_rng = np.random.default_rng(seed0)
    for s in range(n):
        sc = HostScene(3, seed=seed0 + s, width=size, height=size)
        if crop_of:
            crop_camera(sc, crop_of, crop_rng)
        inst, cnt = Tlas.make_instances(blas, sc.instance_mesh(), sc.transforms())
        set_samples(frame, sc, 1, 1)
        tlas.build(inst, cnt)
        frame.gbuffer(tlas)
        frame.trace(tlas, s)
        frame.denoise_features()
        pairs.feat[s].copy_(feat)
        pairs.lin_depth[s].copy_(lin)
        pairs.noisy[s].copy_(sig)
        pairs.unshadowed[s].copy_(uns)
        set_samples(frame, sc, per_trace, per_trace)
        acc.zero_()
        for t in range(traces):
            frame.trace(tlas, 1_000_000 + s * traces + t)
            frame.denoise_features()
            acc += sig
        mean = acc / traces          # (S r, g, b, AO) of target_spp samples
        u = pairs.unshadowed[s, ..., :3].double()
        ratio = torch.where(u > 0, (mean[..., :3] / torch.where(u > 0, u, torch.ones_like(u))).clamp(0, 1),
                            torch.ones_like(u))
        pairs.target[s, ..., :3].copy_(ratio)
        pairs.target[s, ..., 3].copy_(mean[..., 3])
        if log and (s + 1) % max(1, n // 10) == 0:
            log(f"pairs {s + 1}/{n} ({time.perf_counter() - t0:.1f} s)")
    ctx.synchronize()
    torch.cuda.synchronize()
    ctx.set_stream_default()
    torch.cuda.set_stream(saved)
    frame.close()
    tlas.close()
    for b in blas:
        b.close()
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
            log(f"epoch {e + 1}/{epochs} loss {hist[-1]:.6f}")
    return hist


def lit_rmse(a: np.ndarray, b: np.ndarray, lit: np.ndarray) -> float:
    d = (a - b)[lit]
    return float(np.sqrt(np.mean(d.astype(np.float64) ** 2))) if d.size else 0.0


def equal_rmse_spp(curve: dict, r: float) -> float:
    """The plain sample count whose RMSE equals r: log-log interpolation on the measured
    curve {N: RMSE}, extrapolated as RMSE ~ 1 / sqrt(N) past its ends."""
    ns = np.array(sorted(curve), np.float64)
    rs = np.array([curve[int(k)] for k in ns])
    if r >= rs[0]:
        return float(ns[0] * (rs[0] / r) ** 2)
    if r <= rs[-1]:
        return float(ns[-1] * (rs[-1] / r) ** 2)
    i = int(np.nonzero(rs <= r)[0][0])
    a, b = i - 1, i
    f = np.log(rs[a] / r) / np.log(rs[a] / rs[b]) if rs[a] != rs[b] else 1.0
    return float(np.exp(np.log(ns[a]) + f * (np.log(ns[b]) - np.log(ns[a]))))


def evaluate(g: GPUScene, den: Denoiser | None, spps=(2, 4, 8, 16, 64), target_spp: int = 1024,
             frame_index: int = 7) -> dict:
    """RMSE against target_spp samples over lit pixels, for the AO value and for the
    radiance (light pass output, RGB): denoised 1 spp, raw 1 spp and the plain path at
    N spp (N AO rays and N shadow rays per light, stratified samples)."""
    import torch
    fr, tl, sc = g.frame, g.tlas, g.scene
    saved = torch.cuda.current_stream()
    shared_stream(g.ctx)
    g.update_resources_gpu()
    fr.gbuffer(tl)
    lit = np.linalg.norm(fr.read(PLANE_NORMAL)[..., :3], axis=-1) > 0
    t_rad, t_sig = reference(fr, tl, sc, target_spp)
    g.ctx.synchronize()
    g.ctx.set_stream_default()
    torch.cuda.set_stream(saved)
    t_ao = t_sig[..., 3]
    out = {"lit_pixels": int(lit.sum()), "target_spp": target_spp, "plain_ao": {}, "plain_radiance": {}}

    def plain(n):
        set_samples(fr, sc, n, n)
        fr.trace(tl, frame_index)
        fr.light_pass(LIGHT_PASS_PLAIN)
        fr.ao_resolve()
        return lit_rmse(fr.read(PLANE_AO), t_ao, lit), lit_rmse(fr.read(PLANE_LIGHT)[..., :3], t_rad, lit)

    for n in spps:
        out["plain_ao"][int(n)], out["plain_radiance"][int(n)] = plain(n)
    out["raw_1spp_ao"], out["raw_1spp_radiance"] = plain(1)
    if den is not None:
        set_samples(fr, sc, 1, 1)
        fr.trace(tl, frame_index)
        den.denoise(fr)
        fr.light_pass(LIGHT_PASS_DENOISED)
        out["denoised_1spp_ao"] = lit_rmse(fr.read(PLANE_AO_DENOISED), t_ao, lit)
        out["denoised_1spp_radiance"] = lit_rmse(fr.read(PLANE_LIGHT)[..., :3], t_rad, lit)
        for key in ("ao", "radiance"):
            curve = dict(out["plain_" + key])
            curve[1] = out["raw_1spp_" + key]
            out["equal_rmse_spp_" + key] = equal_rmse_spp(curve, out["denoised_1spp_" + key])
    return out
