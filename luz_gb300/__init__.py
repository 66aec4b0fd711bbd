"""luz_gb300 — GB300-native (sm_103a) ray-traced visibility and deferred lighting.

Python face of the C ABI in include/luz.h and include/luz_scene.h. Every compute
call goes to libluz_gb300.so (hand-written CUDA kernels); there is no CPU or
PyTorch fallback, and importing the package fails when the library is missing.

The classes mirror the reference renderer's host interface for this path
(hadryansalles/Luz): ``GPUScene`` follows GPUScene::AddMesh / UpdateResources /
UpdateResourcesGPU (source/Graphics/GPUScene.cpp:108-366) and ``light_pass``
follows DeferredRenderer::LightPass (source/Graphics/DeferredRenderer.cpp:324-345).
"""
from __future__ import annotations

import ctypes as C
import time
import weakref

import numpy as np

from . import _abi
from ._abi import (BLUE_NOISE_SIZE, LIGHT_DIRECTIONAL, LIGHT_POINT, LIGHT_SPOT, PLANE_ALBEDO, PLANE_AO,
                   PLANE_AO_BITS, PLANE_AO_DENOISED, PLANE_DEPTH, PLANE_DTYPES, PLANE_EMISSION, PLANE_LIGHT,
                   PLANE_MATERIAL, PLANE_NORMAL, PLANE_PRIMARY_HIT, PLANE_SHADOW_BITS, PLANE_TAA, PLANE_COMPOSE,
                   PLANE_FEATURES, PLANE_LIN_DEPTH, PLANE_SIGNAL, PLANE_UNSHADOWED, PLANE_DENOISED,
                   LIGHT_PASS_PLAIN, LIGHT_PASS_DENOISED_AO, LIGHT_PASS_DENOISED, SAMPLER_PARITY,
                   SAMPLER_STRATIFIED, SHADOW_RAYTRACING, BlasDesc, Camera, GenParams, Instance, Light, Model,
                   Scene, Vertex)

lib = _abi.load()

__all__ = ["LuzError", "HostScene", "Context", "GPUScene", "lib", "blue_noise"]


class LuzError(RuntimeError):
    def __init__(self, status: int, message: str = ""):
        self.status = status
        super().__init__(f"{_abi.STATUS_NAMES.get(status, status)}: {message}")


def _check(status: int, ctx_handle=None, what: str = "") -> None:
    if status != _abi.LUZ_OK:
        msg = lib.luz_last_error(ctx_handle).decode() if ctx_handle else what
        raise LuzError(status, f"{what}: {msg}" if what else msg)


def blue_noise(seed: int = 7, size: int = BLUE_NOISE_SIZE) -> np.ndarray:
    """Seeded RGBA8 substitute for the reference's missing assets/blue_noise.png."""
    out = np.zeros((size, size, 4), np.uint8)
    _check(lib.luz_blue_noise_generate(seed, size, _abi.ptr(out, _abi.c_u8_p)), what="blue noise")
    return out


# ---------------------------------------------------------------------------- host scenes
class HostScene:
    """A generated scene (meshes, instances with ModelBlocks, lights, SceneBlock)."""

    def __init__(self, config: int, seed: int | None = None, width: int | None = None,
                 height: int | None = None, **overrides):
        p = GenParams()
        _check(lib.luz_scene_default_params(config, C.byref(p)), what="default params")
        if seed is not None:
            p.seed = seed
        if width:
            p.width = width
        if height:
            p.height = height
        for k, v in overrides.items():
            setattr(p, k, v)
        self.params = p
        h = C.c_void_p()
        _check(lib.luz_scene_generate(C.byref(p), C.byref(h)), what="scene generate")
        self._h = h

    @classmethod
    def _adopt(cls, h) -> "HostScene":
        obj = cls.__new__(cls)
        obj.params = None
        obj._h = h
        return obj

    @classmethod
    def load_project(cls, luz_path, luzbin_path, width: int = 1920, height: int = 1080) -> "HostScene":
        """The initial scene of a .luz / .luzbin project (AssetManager::LoadProject)."""
        h, err = C.c_void_p(), C.create_string_buffer(512)
        st = lib.luz_scene_load_project(str(luz_path).encode(), str(luzbin_path).encode(), width, height,
                                        C.byref(h), err, len(err))
        if st != _abi.LUZ_OK:
            raise LuzError(st, f"load project {luz_path}: {err.value.decode()}")
        return cls._adopt(h)

    @classmethod
    def import_file(cls, path, width: int = 1920, height: int = 1080) -> "HostScene":
        """A .gltf / .glb / .obj file in an empty default scene (AssetIO::Import)."""
        h, err = C.c_void_p(), C.create_string_buffer(512)
        st = lib.luz_scene_import(str(path).encode(), width, height, C.byref(h), err, len(err))
        if st != _abi.LUZ_OK:
            raise LuzError(st, f"import {path}: {err.value.decode()}")
        return cls._adopt(h)

    def save_project(self, luz_path, luzbin_path) -> None:
        err = C.create_string_buffer(512)
        st = lib.luz_scene_save_project(self._h, str(luz_path).encode(), str(luzbin_path).encode(), err, len(err))
        if st != _abi.LUZ_OK:
            raise LuzError(st, f"save project {luz_path}: {err.value.decode()}")

    def textures(self) -> list[np.ndarray]:
        """RGBA8 textures (h, w, 4) indexed by the ModelBlocks' map fields (copies)."""
        out = []
        for i in range(lib.luz_scene_texture_count(self._h)):
            p, w, hh = _abi.c_u8_p(), C.c_uint32(), C.c_uint32()
            _check(lib.luz_scene_texture(self._h, i, C.byref(p), C.byref(w), C.byref(hh)))
            out.append(np.ctypeslib.as_array(p, shape=(hh.value, w.value, 4)).copy())
        return out

    def __del__(self):
        if getattr(self, "_h", None):
            lib.luz_scene_destroy(self._h)
            self._h = None

    @property
    def handle(self):
        return self._h

    @property
    def width(self) -> int:
        return lib.luz_scene_width(self._h)

    @property
    def height(self) -> int:
        return lib.luz_scene_height(self._h)

    def meshes(self) -> list[tuple[np.ndarray, np.ndarray]]:
        """[(vertices float32 (nv, 12), indices uint32 (ni,))], copies owned by the caller."""
        out = []
        for i in range(lib.luz_scene_mesh_count(self._h)):
            vp = C.POINTER(Vertex)()
            ip = _abi.c_u32_p()
            nv, ni = C.c_uint32(), C.c_uint32()
            _check(lib.luz_scene_mesh(self._h, i, C.byref(vp), C.byref(nv), C.byref(ip), C.byref(ni)))
            v = np.ctypeslib.as_array(C.cast(vp, _abi.c_float_p), shape=(nv.value, 12)).copy() if nv.value else \
                np.zeros((0, 12), np.float32)
            idx = np.ctypeslib.as_array(ip, shape=(ni.value,)).copy() if ni.value else np.zeros(0, np.uint32)
            out.append((v, idx))
        return out

    @property
    def instance_count(self) -> int:
        return lib.luz_scene_instance_count(self._h)

    def instance_mesh(self) -> np.ndarray:
        n = self.instance_count
        return np.ctypeslib.as_array(lib.luz_scene_instance_mesh(self._h), shape=(n,)).copy()

    def models(self) -> C.Array:
        n = self.instance_count
        arr = (Model * n)()
        C.memmove(arr, lib.luz_scene_models(self._h), C.sizeof(Model) * n)
        return arr

    def lights(self) -> C.Array:
        n = lib.luz_scene_light_count(self._h)
        arr = (Light * max(n, 1))()
        if n:
            C.memmove(arr, lib.luz_scene_lights(self._h), C.sizeof(Light) * n)
        return arr

    @property
    def light_count(self) -> int:
        return lib.luz_scene_light_count(self._h)

    def block(self) -> Scene:
        s = Scene()
        C.memmove(C.byref(s), lib.luz_scene_block(self._h), C.sizeof(Scene))
        return s

    def transforms(self) -> np.ndarray:
        out = np.zeros((self.instance_count, 3, 4), np.float32)
        _check(lib.luz_scene_instance_transforms(self._h, _abi.ptr(out, _abi.c_float_p)))
        return out

    def set_sampling(self, ao_samples: int, ao_min: float | None = None, ao_max: float | None = None,
                     light_samples: int = 1, sampler: int | None = None) -> None:
        b = self.block()
        _check(lib.luz_scene_set_sampling(self._h, ao_samples, b.ao_min if ao_min is None else ao_min,
                                          b.ao_max if ao_max is None else ao_max, light_samples,
                                          b.sampler if sampler is None else sampler))

    def shadow_lights(self) -> C.Array:
        """luz_shadow_light per light: the shadow-map matrices GPUScene computes."""
        n = self.light_count
        arr = (_abi.ShadowLight * max(n, 1))()
        _check(lib.luz_scene_shadow_lights(self._h, arr), what="shadow lights")
        return arr if n else (_abi.ShadowLight * 0)()

    def set_shadow_type(self, shadow_type: int) -> None:
        _check(lib.luz_scene_set_shadow_type(self._h, shadow_type), what="shadow type")

    def next_frame(self, jitter: bool = True) -> None:
        """One frame on: prev matrices / jitter <- current, next jitter (GPUScene::UpdateResources)."""
        _check(lib.luz_scene_next_frame(self._h, int(jitter)), what="next frame")

    def camera(self) -> Camera:
        c = Camera()
        _check(lib.luz_scene_get_camera(self._h, C.byref(c)))
        return c

    def set_camera(self, cam: Camera) -> None:
        _check(lib.luz_scene_set_camera(self._h, C.byref(cam)))

    def triangle_count(self) -> int:
        per = [len(i) // 3 for _, i in self.meshes()]
        return int(sum(per[m] for m in self.instance_mesh()))


# ---------------------------------------------------------------------------- device objects
class Blas:
    def __init__(self, ctx: "Context", handle):
        self.ctx, self._h = ctx, handle

    @property
    def handle(self):
        return self._h

    @property
    def prims(self) -> int:
        return lib.luz_blas_primitive_count(self._h)

    def download(self):
        n = self.prims
        m = max(n, 2) - 1
        nodes = np.zeros((m, 16), np.float32)
        tris = np.zeros((max(n, 1), 12), np.float32)
        mort = np.zeros(max(n, 1), np.uint32)
        order = np.zeros(max(n, 1), np.uint32)
        _check(lib.luz_blas_download(self.ctx.handle, self._h, _abi.ptr(nodes), _abi.ptr(tris),
                                     _abi.ptr(mort, _abi.c_u32_p), _abi.ptr(order, _abi.c_u32_p)),
               self.ctx.handle, "blas download")
        return nodes, tris[:n], mort[:n], order[:n]

    def download_wide(self) -> np.ndarray:
        """The 4-wide traversal nodes, (max(n-1,1), 32) float32 (children as int bits
        in columns 24..27); the leading even-depth-count rows are the nodes."""
        m = max(self.prims, 2) - 1
        nodes4 = np.zeros((m, 32), np.float32)
        _check(lib.luz_blas_download_wide(self.ctx.handle, self._h, _abi.ptr(nodes4)), self.ctx.handle,
               "blas download wide")
        return nodes4

    def memory(self) -> dict:
        m = _abi.Memory()
        _check(lib.luz_blas_memory(self._h, C.byref(m)), what="blas memory")
        return m.as_dict()

    def close(self):
        if self._h:
            lib.luz_blas_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()


class Tlas:
    def __init__(self, ctx: "Context", max_instances: int):
        self.ctx = ctx
        h = C.c_void_p()
        _check(lib.luz_tlas_create(ctx.handle, max_instances, C.byref(h)), ctx.handle, "tlas create")
        self._h = h
        self._instances = None

    @property
    def handle(self):
        return self._h

    @staticmethod
    def make_instances(blas: list[Blas], instance_mesh, transforms: np.ndarray, custom=None, mask=None):
        n = len(instance_mesh)
        arr = (Instance * max(n, 1))()
        for i in range(n):
            arr[i].blas = blas[int(instance_mesh[i])].handle
            C.memmove(arr[i].transform, transforms[i].astype(np.float32).ctypes.data, 48)
            arr[i].custom_index = i if custom is None else int(custom[i])
            arr[i].mask = 0xFF if mask is None else int(mask[i])
        return arr, n

    def build(self, instances, count: int) -> None:
        self._instances = instances   # keep alive until the next build
        _check(lib.luz_tlas_build(self.ctx.handle, self._h, instances, count), self.ctx.handle, "tlas build")

    def download(self):
        cnt = C.c_uint32()
        _check(lib.luz_tlas_download(self.ctx.handle, self._h, None, None, None, C.byref(cnt)))
        m = cnt.value
        nodes = np.zeros((max(m, 1), 16), np.float32)
        n = len(self._instances) if self._instances is not None else 0
        mort = np.zeros(max(n, 1), np.uint32)
        order = np.zeros(max(n, 1), np.uint32)
        _check(lib.luz_tlas_download(self.ctx.handle, self._h, _abi.ptr(nodes), _abi.ptr(mort, _abi.c_u32_p),
                                     _abi.ptr(order, _abi.c_u32_p), C.byref(cnt)), self.ctx.handle, "tlas download")
        return nodes[:m], mort, order

    def download_wide(self) -> np.ndarray:
        cnt = C.c_uint32()
        _check(lib.luz_tlas_download(self.ctx.handle, self._h, None, None, None, C.byref(cnt)))
        nodes4 = np.zeros((max(cnt.value, 1), 32), np.float32)
        _check(lib.luz_tlas_download_wide(self.ctx.handle, self._h, _abi.ptr(nodes4)), self.ctx.handle,
               "tlas download wide")
        return nodes4[:cnt.value]

    def memory(self) -> dict:
        m = _abi.Memory()
        _check(lib.luz_tlas_memory(self._h, C.byref(m)), what="tlas memory")
        return m.as_dict()

    def close(self):
        if self._h:
            lib.luz_tlas_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()


class Frame:
    def __init__(self, ctx: "Context", width: int, height: int):
        self.ctx, self.width, self.height = ctx, width, height
        h = C.c_void_p()
        _check(lib.luz_frame_create(ctx.handle, width, height, C.byref(h)), ctx.handle, "frame create")
        self._h = h

    @property
    def handle(self):
        return self._h

    def upload(self, scene: Scene, lights, light_count: int, models, model_count: int) -> None:
        _check(lib.luz_frame_upload(self.ctx.handle, self._h, C.byref(scene), lights, light_count, models,
                                    model_count), self.ctx.handle, "frame upload")

    def set_textures(self, textures) -> None:
        """RGBA8 arrays (h, w, 4) that the ModelBlocks' map fields index."""
        tex = [np.ascontiguousarray(t, np.uint8) for t in textures]
        descs = (_abi.TextureDesc * max(len(tex), 1))()
        for k, t in enumerate(tex):
            descs[k].rgba8 = t.ctypes.data
            descs[k].width = t.shape[1]
            descs[k].height = t.shape[0]
        _check(lib.luz_frame_set_textures(self.ctx.handle, self._h, descs, len(tex)), self.ctx.handle,
               "set textures")

    def render_shadow_maps(self, tlas: Tlas, lights, resolution: int = 1024) -> None:
        self._shadow_faces = [int(l.faces) for l in lights]
        self._shadow_res = resolution
        _check(lib.luz_frame_render_shadow_maps(self.ctx.handle, self._h, tlas.handle, C.cast(lights, C.c_void_p),
                                                len(lights), resolution), self.ctx.handle, "shadow maps")

    def read_shadow_map(self, light: int) -> np.ndarray:
        f, r = self._shadow_faces[light], self._shadow_res
        out = np.zeros((f, r, r), np.float32)
        _check(lib.luz_frame_read_shadow_map(self.ctx.handle, self._h, light, _abi.ptr(out), out.nbytes),
               self.ctx.handle, "read shadow map")
        return out

    def gbuffer(self, tlas: Tlas) -> None:
        _check(lib.luz_gbuffer_primary(self.ctx.handle, self._h, tlas.handle), self.ctx.handle, "gbuffer")

    def trace(self, tlas: Tlas, frame_index: int = 0) -> None:
        _check(lib.luz_trace_visibility(self.ctx.handle, self._h, tlas.handle, frame_index), self.ctx.handle,
               "trace visibility")

    def trace_stats(self, tlas: Tlas, frame_index: int = 0) -> dict:
        out = (C.c_uint64 * 5)()
        _check(lib.luz_trace_visibility_stats(self.ctx.handle, self._h, tlas.handle, frame_index, out),
               self.ctx.handle, "trace stats")
        return {"rays": out[0], "tlas_nodes": out[1], "blas_nodes": out[2], "tris": out[3], "instances": out[4]}

    def set_shadow_cull(self, enable: bool) -> None:
        """False: trace every shadow sample light.frag traces (exact per-ray bit planes);
        True (default): leave out the samples whose light's term cannot depend on them."""
        _check(lib.luz_frame_set_shadow_cull(self._h, int(enable)), self.ctx.handle, "shadow cull")

    def ao_resolve(self) -> None:
        _check(lib.luz_ao_resolve(self.ctx.handle, self._h), self.ctx.handle, "ao resolve")

    def lit_count(self) -> int:
        n = C.c_uint32()
        _check(lib.luz_frame_lit_count(self.ctx.handle, self._h, C.byref(n)), self.ctx.handle, "lit count")
        return n.value

    def light_pass(self, mode: int = LIGHT_PASS_PLAIN) -> None:
        """mode: LIGHT_PASS_PLAIN (light.frag from the bit planes), LIGHT_PASS_DENOISED_AO
        (AO from the denoised plane; True also selects it), LIGHT_PASS_DENOISED (the frame
        composed from the denoiser's filtered shadow ratio and AO)."""
        _check(lib.luz_light_pass(self.ctx.handle, self._h, int(mode)), self.ctx.handle, "light pass")

    def taa(self, reconstruct: bool = True) -> None:
        """Temporal anti-aliasing of the light image into PLANE_TAA (the next history)."""
        _check(lib.luz_taa(self.ctx.handle, self._h, int(reconstruct)), self.ctx.handle, "taa")

    def compose(self, source_taa: bool = False, image_type: int = 0) -> None:
        """present.frag into PLANE_COMPOSE (BGRA8): 0 tone-mapped light, 1-5 G-buffer views, 6 grid."""
        _check(lib.luz_compose(self.ctx.handle, self._h, int(source_taa), image_type), self.ctx.handle, "compose")

    def composed_rgba(self) -> np.ndarray:
        """PLANE_COMPOSE as an (H, W, 4) RGBA8 array."""
        bgra = self.read(PLANE_COMPOSE).view(np.uint8).reshape(self.height, self.width, 4)
        return bgra[..., [2, 1, 0, 3]].copy()

    def luminance_histogram(self, source_taa: bool = False, delta_time: float = 1.0 / 60.0) -> dict:
        h = _abi.Histogram()
        _check(lib.luz_luminance_histogram(self.ctx.handle, self._h, int(source_taa), delta_time, C.byref(h)),
               self.ctx.handle, "luminance histogram")
        return {"bins": np.array(h.bins, np.uint32), "weighted_sum": h.weighted_sum, "log_average": h.log_average,
                "average_luminance": h.average_luminance, "adapted_luminance": h.adapted_luminance}

    def taa_reset(self) -> None:
        _check(lib.luz_taa_reset(self.ctx.handle, self._h), self.ctx.handle, "taa reset")

    def device_ptr(self, plane: int) -> int:
        return lib.luz_frame_plane_device_ptr(self._h, plane) or 0

    def denoise_features(self) -> None:
        _check(lib.luz_denoise_features(self.ctx.handle, self._h), self.ctx.handle, "denoise features")

    def plane_bytes(self, plane: int) -> int:
        return lib.luz_frame_plane_bytes(self._h, plane)

    def read(self, plane: int) -> np.ndarray:
        dt, comps = PLANE_DTYPES[plane]
        nbytes = self.plane_bytes(plane)
        raw = np.zeros(max(nbytes, 16), np.uint8)
        if nbytes:
            _check(lib.luz_frame_read(self.ctx.handle, self._h, plane, _abi.ptr(raw), nbytes), self.ctx.handle,
                   "frame read")
        out = raw[:nbytes].view(dt)
        if plane in (PLANE_SHADOW_BITS, PLANE_AO_BITS):
            words = (self.width * self.height + 31) // 32
            return out.reshape(-1, words)
        if comps > 1:
            return out.reshape(self.height, self.width, comps)
        return out.reshape(self.height, self.width)

    def write(self, plane: int, data: np.ndarray) -> None:
        data = np.ascontiguousarray(data)
        _check(lib.luz_frame_write(self.ctx.handle, self._h, plane, _abi.ptr(data), data.nbytes), self.ctx.handle,
               "frame write")

    def close(self):
        if self._h:
            lib.luz_frame_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()


class Context:
    """One CUDA device and stream (the reference's global Vulkan context)."""

    def __init__(self, device: int = 0):
        h = C.c_void_p()
        _check(lib.luz_ctx_create(device, C.byref(h)), what="luz_ctx_create")
        self._h = h
        self._children = weakref.WeakSet()   # handles that must be destroyed before the context

    def _adopt(self, obj):
        self._children.add(obj)
        return obj

    @property
    def handle(self):
        return self._h

    def set_blue_noise(self, tex: np.ndarray) -> None:
        tex = np.ascontiguousarray(tex, np.uint8)
        _check(lib.luz_ctx_set_blue_noise(self._h, _abi.ptr(tex, _abi.c_u8_p), tex.shape[0]), self._h, "blue noise")

    def build_blas(self, meshes: list[tuple[np.ndarray, np.ndarray]]) -> list[Blas]:
        descs = (BlasDesc * len(meshes))()
        keep = []
        for i, (v, idx) in enumerate(meshes):
            v = np.ascontiguousarray(v, np.float32)
            idx = np.ascontiguousarray(idx, np.uint32)
            keep += [v, idx]
            descs[i].vertices = v.ctypes.data
            descs[i].vertex_count = v.shape[0]
            descs[i].vertex_stride = v.shape[1] * 4 if v.ndim == 2 else 48
            descs[i].indices = idx.ctypes.data
            descs[i].index_count = idx.size
        outs = (C.c_void_p * len(meshes))()
        _check(lib.luz_blas_build_batch(self._h, len(meshes), descs, outs), self._h, "blas build")
        return [self._adopt(Blas(self, C.c_void_p(outs[i]))) for i in range(len(meshes))]

    def tlas(self, max_instances: int) -> Tlas:
        return self._adopt(Tlas(self, max_instances))

    def frame(self, width: int, height: int) -> Frame:
        return self._adopt(Frame(self, width, height))

    def set_vis_tuning(self, smem_nodes: int = 0, refill: int = 0, steps: int = 0, ctas_per_sm: int = 0) -> None:
        """Launch shape of the visibility kernel; all zero restores the defaults."""
        arr = (C.c_uint32 * 4)(smem_nodes, refill, steps, ctas_per_sm)
        _check(lib.luz_ctx_set_vis_tuning(self._h, C.byref(arr)), self._h, "vis tuning")

    def vis_tuning(self) -> dict:
        arr = (C.c_uint32 * 4)()
        _check(lib.luz_ctx_get_vis_tuning(self._h, C.byref(arr)), self._h, "vis tuning")
        return dict(zip(("smem_nodes", "refill", "steps", "ctas_per_sm"), list(arr)))

    def set_stream(self, cuda_stream: int) -> None:
        """Runs all later work on `cuda_stream` (a cudaStream_t value, not 0: the
        legacy default stream would not order against the context's own stream)."""
        if not cuda_stream:
            raise ValueError("pass an explicit (non-default) CUDA stream")
        _check(lib.luz_ctx_set_stream(self._h, C.c_void_p(cuda_stream)), self._h, "set stream")

    def synchronize(self) -> None:
        _check(lib.luz_ctx_synchronize(self._h), self._h, "synchronize")

    def device_status(self) -> int:
        bits = C.c_uint32()
        _check(lib.luz_ctx_device_status(self._h, C.byref(bits)), self._h, "device status")
        return bits.value

    def launch_count(self) -> int:
        return lib.luz_ctx_launch_count(self._h)

    def last_blas_build_ms(self) -> float:
        """Device time of the last BLAS build, host->device copies excluded."""
        ms = C.c_float()
        _check(lib.luz_ctx_last_blas_build_ms(self._h, C.byref(ms)), self._h, "build timing")
        return ms.value

    KERNELS = {"tlas_build": 0, "gbuffer": 1, "raygen": 2, "traversal": 3, "light_pass": 4, "features": 5,
               "denoise": 6, "taa": 7, "denoise_train": 8, "batch_frame": 9}

    def profile(self, on: bool) -> None:
        """Per-kernel event timing of the instrumented kernels (on clears the records)."""
        _check(lib.luz_ctx_profile(self._h, 1 if on else 0), self._h, "profile")

    def profile_read(self, kernel: str) -> tuple[float, int]:
        """(summed ms, launches) of one kernel since profiling was switched on."""
        ms, n = C.c_float(), C.c_uint32()
        _check(lib.luz_ctx_profile_read(self._h, self.KERNELS[kernel], C.byref(ms), C.byref(n)), self._h,
               "profile read")
        return ms.value, n.value

    def probe_l2_read_gbs(self, nbytes: int = 48 << 20, reps: int = 50) -> float:
        """L2 read bandwidth (GB/s) from L2-only 16-B loads over an nbytes buffer."""
        g = C.c_float()
        _check(lib.luz_ctx_probe_l2_read(self._h, nbytes, reps, C.byref(g)), self._h, "L2 probe")
        return g.value

    def set_debug_step_cap(self, steps: int) -> None:
        """Debug: traversal steps per shadow / AO ray before it is ended with
        LUZ_DEV_TRAVERSAL_CAP raised; 0 restores the library's cap."""
        _check(lib.luz_ctx_set_debug_step_cap(self._h, steps), self._h, "debug step cap")

    def set_stream_default(self) -> None:
        """Back to the context's own stream."""
        _check(lib.luz_ctx_set_stream(self._h, None), self._h, "set stream")

    def close(self):
        if self._h:
            for child in list(self._children):
                child.close()
            lib.luz_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()


class _BorrowedFrame(Frame):
    """A frame owned by a batch (not destroyed by this handle)."""

    def __init__(self, ctx: "Context", handle, width: int, height: int):
        self.ctx, self.width, self.height, self._h = ctx, width, height, handle

    def close(self):
        self._h = None


class Batch:
    """Many scenes rendered as one unit (luz_batch_*): one batched BLAS build over the
    meshes of every scene at creation, then per render ONE persistent launch (the frame
    kernel: every TLAS build, G-buffer, the traversal of all scenes' rays and every
    light pass), or the staged launches (set_fused(False)); optionally as one CUDA
    graph."""

    def __init__(self, ctx: "Context", scenes: list[HostScene]):
        self.ctx, self.scenes = ctx, scenes
        meshes, first = [], []
        for sc in scenes:
            first.append(len(meshes))
            meshes += sc.meshes()
        self.blas = ctx.build_blas(meshes)
        self.triangles = sum(sc.triangle_count() for sc in scenes)
        n = len(scenes)
        descs = (_abi.BatchScene * n)()
        keep = []
        for i, sc in enumerate(scenes):
            nm = lib.luz_scene_mesh_count(sc.handle)
            inst, cnt = Tlas.make_instances(self.blas[first[i]:first[i] + nm], sc.instance_mesh(), sc.transforms())
            models, lights, block = sc.models(), sc.lights(), sc.block()
            keep += [inst, models, lights, block]
            descs[i].instances = C.addressof(inst)
            descs[i].instance_count = cnt
            descs[i].scene = C.addressof(block)
            descs[i].lights = C.addressof(lights)
            descs[i].light_count = sc.light_count
            descs[i].models = C.addressof(models)
            descs[i].model_count = sc.instance_count
            descs[i].width, descs[i].height = sc.width, sc.height
        h = C.c_void_p()
        _check(lib.luz_batch_create(ctx.handle, n, descs, C.byref(h)), ctx.handle, "batch create")
        self._h = h
        ctx._adopt(self)
        self.frames = [_BorrowedFrame(ctx, C.c_void_p(lib.luz_batch_frame(h, i)), sc.width, sc.height)
                       for i, sc in enumerate(scenes)]

    @property
    def handle(self):
        return self._h

    def render(self, frame_index: int = 0) -> None:
        _check(lib.luz_batch_render(self.ctx.handle, self._h, frame_index), self.ctx.handle, "batch render")

    def stats(self, frame_index: int = 0) -> dict:
        out = (C.c_uint64 * 5)()
        _check(lib.luz_batch_stats(self.ctx.handle, self._h, frame_index, out), self.ctx.handle, "batch stats")
        return {"rays": out[0], "tlas_nodes": out[1], "blas_nodes": out[2], "tris": out[3], "instances": out[4]}

    def capture(self, frame_index: int = 0) -> None:
        _check(lib.luz_batch_capture(self.ctx.handle, self._h, frame_index), self.ctx.handle, "batch capture")

    def replay(self) -> None:
        _check(lib.luz_batch_replay(self.ctx.handle, self._h), self.ctx.handle, "batch replay")

    @property
    def fused(self) -> bool:
        """True when renders run the frame kernel."""
        return bool(lib.luz_batch_fused(self._h))

    def set_fused(self, on: bool) -> None:
        _check(lib.luz_batch_set_fused(self.ctx.handle, self._h, 1 if on else 0), self.ctx.handle, "batch mode")

    def autotune(self, reps: int = 3):
        arr = (C.c_uint32 * 4)()
        ms = C.c_float()
        _check(lib.luz_batch_autotune(self.ctx.handle, self._h, reps, C.byref(arr), C.byref(ms)), self.ctx.handle,
               "batch autotune")
        return dict(zip(("smem_nodes", "refill", "steps", "ctas_per_sm"), list(arr))), ms.value

    def close(self):
        if self._h:
            for f in self.frames:
                f.close()
            lib.luz_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()


# ---------------------------------------------------------------------------- GPUScene mirror
class GPUScene:
    """Host orchestration of the path, mirroring the reference's GPUScene
    (AddMesh / UpdateResources / UpdateResourcesGPU, GPUScene.cpp:108-366) and the
    frame order of LuzApplication::RenderFrame (main.cpp:223-311): TLAS rebuild,
    opaque (primary-ray G-buffer) pass, light pass with ray-traced visibility."""

    def __init__(self, ctx: Context, scene: HostScene, blue_noise_seed: int = 7):
        self.ctx, self.scene = ctx, scene
        ctx.set_blue_noise(blue_noise(blue_noise_seed))
        meshes = scene.meshes()
        t0 = time.perf_counter()
        self.blas = ctx.build_blas(meshes)                          # AddMesh for every mesh
        self.blas_build_ms = (time.perf_counter() - t0) * 1e3       # synchronous, host copies included
        self.blas_build_device_ms = ctx.last_blas_build_ms() if meshes else 0.0
        self.blas_prims = sum(len(i) // 3 for _, i in meshes)
        self.tlas = ctx.tlas(max(scene.instance_count, 1))          # CreateTLAS
        self.frame = ctx.frame(scene.width, scene.height)           # DeferredRenderer::CreateImages
        self.textures = scene.textures()                            # one RGBA8 image per texture asset
        if self.textures:
            self.frame.set_textures(self.textures)
        self.update_resources()

    def update_resources(self) -> None:
        """UpdateResources: pack ModelBlocks, SceneBlock and LightBlocks (host)."""
        s = self.scene
        self.models = s.models()
        self.lights = s.lights()
        self.block = s.block()
        self.instances, self.n_instances = Tlas.make_instances(self.blas, s.instance_mesh(), s.transforms())

    def update_resources_gpu(self) -> None:
        """UpdateResourcesGPU: copy the blocks to the device and rebuild the TLAS."""
        self.frame.upload(self.block, self.lights, self.scene.light_count, self.models, self.scene.instance_count)
        self.tlas.build(self.instances, self.n_instances)

    def render(self, frame_index: int = 0, use_denoised_ao: bool = False) -> None:
        self.update_resources_gpu()
        self.frame.gbuffer(self.tlas)
        self.frame.trace(self.tlas, frame_index)
        self.frame.light_pass(use_denoised_ao)

    def render_frame(self, frame_index: int = 0) -> None:
        """The whole frame in one C call (TLAS build + G-buffer + visibility + light pass)."""
        _check(lib.luz_render_frame(self.ctx.handle, self.frame.handle, self.tlas.handle, self.instances,
                                    self.n_instances, frame_index), self.ctx.handle, "render frame")
