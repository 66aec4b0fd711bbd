"""ctypes mirror of include/luz.h and include/luz_scene.h.

The structures below are byte-for-byte the C structs of the C ABI; tests assert
their sizes against the header's static assertions.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "libluz_gb300.so"

c_float_p = C.POINTER(C.c_float)
c_u32_p = C.POINTER(C.c_uint32)
c_u8_p = C.POINTER(C.c_uint8)

LUZ_OK = 0
STATUS_NAMES = {0: "LUZ_OK", 1: "LUZ_ERR_INVALID", 2: "LUZ_ERR_CUDA", 3: "LUZ_ERR_OOM",
                4: "LUZ_ERR_DEVICE", 5: "LUZ_ERR_LIMIT", 6: "LUZ_ERR_NO_DEVICE"}

LIGHT_POINT, LIGHT_SPOT, LIGHT_DIRECTIONAL = 0, 1, 2
SHADOW_DISABLED, SHADOW_RAYTRACING, SHADOW_MAP = 0, 1, 2
SAMPLER_PARITY, SAMPLER_STRATIFIED = 0, 1
BLUE_NOISE_SIZE = 128

PLANE_ALBEDO, PLANE_NORMAL, PLANE_MATERIAL, PLANE_EMISSION, PLANE_DEPTH, PLANE_LIGHT = range(6)
PLANE_SHADOW_BITS, PLANE_AO_BITS, PLANE_AO, PLANE_AO_DENOISED, PLANE_PRIMARY_HIT = range(6, 11)
PLANE_TAA, PLANE_COMPOSE = 13, 14
PLANE_SIGNAL, PLANE_UNSHADOWED, PLANE_DENOISED = 15, 16, 17
LIGHT_PASS_PLAIN, LIGHT_PASS_DENOISED_AO, LIGHT_PASS_DENOISED = 0, 1, 2
PLANE_DTYPES = {PLANE_ALBEDO: (np.uint32, 1), PLANE_NORMAL: (np.float32, 4), PLANE_MATERIAL: (np.uint32, 1),
                PLANE_EMISSION: (np.uint32, 1), PLANE_DEPTH: (np.float32, 1), PLANE_LIGHT: (np.float32, 4),
                PLANE_SHADOW_BITS: (np.uint32, 1), PLANE_AO_BITS: (np.uint32, 1), PLANE_AO: (np.float32, 1),
                PLANE_AO_DENOISED: (np.float32, 1), PLANE_PRIMARY_HIT: (np.uint32, 2),
                PLANE_TAA: (np.float32, 4), PLANE_COMPOSE: (np.uint32, 1), PLANE_SIGNAL: (np.float32, 4),
                PLANE_UNSHADOWED: (np.float32, 4), PLANE_DENOISED: (np.float32, 4)}


class Vertex(C.Structure):
    _fields_ = [("position", C.c_float * 3), ("normal", C.c_float * 3), ("tangent", C.c_float * 4),
                ("texcoord", C.c_float * 2)]


class Light(C.Structure):
    _fields_ = [("color", C.c_float * 3), ("intensity", C.c_float), ("position", C.c_float * 3),
                ("inner_angle", C.c_float), ("direction", C.c_float * 3), ("outer_angle", C.c_float),
                ("type", C.c_int32), ("num_shadow_samples", C.c_int32), ("radius", C.c_float),
                ("shadow_map", C.c_int32)]


class Model(C.Structure):
    _fields_ = [("model_mat", C.c_float * 16), ("color", C.c_float * 4), ("emission", C.c_float * 3),
                ("metallic", C.c_float), ("roughness", C.c_float), ("ao_map", C.c_int32),
                ("color_map", C.c_int32), ("normal_map", C.c_int32), ("emission_map", C.c_int32),
                ("metallic_roughness_map", C.c_int32), ("vertex_buffer", C.c_int32),
                ("index_buffer", C.c_int32)]


class Scene(C.Structure):
    _fields_ = [("ambient_light_color", C.c_float * 3), ("ambient_light_intensity", C.c_float),
                ("proj", C.c_float * 16), ("view", C.c_float * 16), ("view_proj", C.c_float * 16),
                ("prev_view_proj", C.c_float * 16), ("inverse_proj", C.c_float * 16),
                ("inverse_view", C.c_float * 16), ("jitter", C.c_float * 2), ("prev_jitter", C.c_float * 2),
                ("cam_pos", C.c_float * 3), ("num_lights", C.c_int32), ("ao_min", C.c_float),
                ("ao_max", C.c_float), ("exposure", C.c_float), ("ao_num_samples", C.c_int32),
                ("white_texture", C.c_int32), ("black_texture", C.c_int32),
                ("blue_noise_texture", C.c_int32), ("tlas_rid", C.c_int32), ("shadow_type", C.c_int32),
                ("sampler", C.c_int32), ("pad", C.c_int32 * 2)]


class Instance(C.Structure):
    _fields_ = [("blas", C.c_void_p), ("transform", (C.c_float * 4) * 3), ("custom_index", C.c_uint32),
                ("mask", C.c_uint32)]


class Histogram(C.Structure):
    _fields_ = [("bins", C.c_uint32 * 256), ("weighted_sum", C.c_float), ("log_average", C.c_float),
                ("average_luminance", C.c_float), ("adapted_luminance", C.c_float)]


class ShadowLight(C.Structure):
    _fields_ = [("view_proj", (C.c_float * 16) * 6), ("z_far", C.c_float), ("faces", C.c_uint32),
                ("position", C.c_float * 3), ("pad", C.c_uint32)]


class TextureDesc(C.Structure):
    _fields_ = [("rgba8", C.c_void_p), ("width", C.c_uint32), ("height", C.c_uint32)]


class Memory(C.Structure):
    _fields_ = [("nodes", C.c_uint64), ("wide_nodes", C.c_uint64), ("leaves", C.c_uint64), ("other", C.c_uint64)]

    def as_dict(self) -> dict:
        d = {k: int(getattr(self, k)) for k, _ in self._fields_}
        d["total"] = sum(d.values())
        return d


class BlasDesc(C.Structure):
    _fields_ = [("vertices", C.c_void_p), ("vertex_count", C.c_uint32), ("vertex_stride", C.c_uint32),
                ("indices", C.c_void_p), ("index_count", C.c_uint32)]


class Camera(C.Structure):
    _fields_ = [("camera_type", C.c_int32), ("mode", C.c_int32), ("eye", C.c_float * 3),
                ("center", C.c_float * 3), ("rotation", C.c_float * 3), ("zoom", C.c_float),
                ("far_distance", C.c_float), ("near_distance", C.c_float), ("horizontal_fov", C.c_float),
                ("ortho_far_distance", C.c_float), ("ortho_near_distance", C.c_float),
                ("extent", C.c_float * 2), ("jitter", C.c_float * 2)]


class GenParams(C.Structure):
    _fields_ = [("config", C.c_int32), ("pad0", C.c_uint32), ("seed", C.c_uint64), ("width", C.c_uint32),
                ("height", C.c_uint32), ("ao_samples", C.c_int32), ("ao_max", C.c_float),
                ("light_samples", C.c_int32), ("sampler", C.c_int32), ("meshes", C.c_uint32),
                ("instances", C.c_uint32), ("subdivisions", C.c_uint32), ("point_lights", C.c_uint32),
                ("spot_lights", C.c_uint32), ("directional_lights", C.c_uint32), ("triangles", C.c_uint32),
                ("pad1", C.c_uint32)]


class BatchScene(C.Structure):
    _fields_ = [("instances", C.c_void_p), ("instance_count", C.c_uint32), ("scene", C.c_void_p),
                ("lights", C.c_void_p), ("light_count", C.c_uint32), ("models", C.c_void_p),
                ("model_count", C.c_uint32), ("width", C.c_uint32), ("height", C.c_uint32)]


class DenoiseBatch(C.Structure):
    _fields_ = [("features", C.c_void_p), ("lin_depth", C.c_void_p), ("noisy", C.c_void_p),
                ("unshadowed", C.c_void_p), ("target", C.c_void_p), ("weight", C.c_void_p), ("width", C.c_uint32),
                ("height", C.c_uint32), ("images", C.c_uint32)]


DENOISER_PARAMS = 16177
PLANE_FEATURES, PLANE_LIN_DEPTH = 11, 12
PLANE_DTYPES[PLANE_FEATURES] = (np.uint16, 8)
PLANE_DTYPES[PLANE_LIN_DEPTH] = (np.float32, 1)


# (name, restype, argtypes) of every entry point declared in include/*.h
P = C.c_void_p
SIGNATURES = [
    ("luz_ctx_create", C.c_int32, [C.c_int, C.POINTER(P)]),
    ("luz_ctx_destroy", None, [P]),
    ("luz_last_error", C.c_char_p, [P]),
    ("luz_ctx_synchronize", C.c_int32, [P]),
    ("luz_ctx_device_status", C.c_int32, [P, c_u32_p]),
    ("luz_ctx_launch_count", C.c_uint64, [P]),
    ("luz_ctx_set_stream", C.c_int32, [P, P]),
    ("luz_ctx_set_debug_step_cap", C.c_int32, [P, C.c_uint32]),
    ("luz_ctx_set_blue_noise", C.c_int32, [P, c_u8_p, C.c_uint32]),
    ("luz_ctx_set_vis_tuning", C.c_int32, [P, C.POINTER(C.c_uint32 * 4)]),
    ("luz_ctx_get_vis_tuning", C.c_int32, [P, C.POINTER(C.c_uint32 * 4)]),
    ("luz_ctx_last_blas_build_ms", C.c_int32, [P, c_float_p]),
    ("luz_ctx_probe_l2_read", C.c_int32, [P, C.c_uint64, C.c_uint32, c_float_p]),
    ("luz_ctx_profile", C.c_int32, [P, C.c_int32]),
    ("luz_ctx_profile_read", C.c_int32, [P, C.c_int32, c_float_p, c_u32_p]),
    ("luz_blas_build", C.c_int32, [P, C.POINTER(BlasDesc), C.POINTER(P)]),
    ("luz_blas_build_batch", C.c_int32, [P, C.c_uint32, C.POINTER(BlasDesc), C.POINTER(P)]),
    ("luz_blas_destroy", None, [P]),
    ("luz_blas_primitive_count", C.c_uint32, [P]),
    ("luz_blas_download", C.c_int32, [P, P, P, P, c_u32_p, c_u32_p]),
    ("luz_blas_download_wide", C.c_int32, [P, P, P]),
    ("luz_frame_set_textures", C.c_int32, [P, P, P, C.c_uint32]),
    ("luz_taa", C.c_int32, [P, P, C.c_int32]),
    ("luz_compose", C.c_int32, [P, P, C.c_int32, C.c_int32]),
    ("luz_luminance_histogram", C.c_int32, [P, P, C.c_int32, C.c_float, P]),
    ("luz_taa_reset", C.c_int32, [P, P]),
    ("luz_blas_memory", C.c_int32, [P, P]),
    ("luz_blas_build_noalloc", C.c_int32, [P, C.c_uint32, P, C.c_uint32, P, P, P, P, P]),
    ("luz_tlas_create", C.c_int32, [P, C.c_uint32, C.POINTER(P)]),
    ("luz_tlas_build", C.c_int32, [P, P, C.POINTER(Instance), C.c_uint32]),
    ("luz_tlas_destroy", None, [P]),
    ("luz_tlas_download", C.c_int32, [P, P, P, c_u32_p, c_u32_p, c_u32_p]),
    ("luz_tlas_download_wide", C.c_int32, [P, P, P]),
    ("luz_tlas_memory", C.c_int32, [P, P]),
    ("luz_frame_create", C.c_int32, [P, C.c_uint32, C.c_uint32, C.POINTER(P)]),
    ("luz_frame_destroy", None, [P]),
    ("luz_frame_upload", C.c_int32, [P, P, C.POINTER(Scene), C.POINTER(Light), C.c_uint32,
                                     C.POINTER(Model), C.c_uint32]),
    ("luz_gbuffer_primary", C.c_int32, [P, P, P]),
    ("luz_trace_visibility", C.c_int32, [P, P, P, C.c_int32]),
    ("luz_trace_visibility_stats", C.c_int32, [P, P, P, C.c_int32, C.POINTER(C.c_uint64)]),
    ("luz_ao_resolve", C.c_int32, [P, P]),
    ("luz_frame_set_shadow_cull", C.c_int32, [P, C.c_int32]),
    ("luz_frame_lit_count", C.c_int32, [P, P, c_u32_p]),
    ("luz_light_pass", C.c_int32, [P, P, C.c_int32]),
    ("luz_render_frame", C.c_int32, [P, P, P, C.POINTER(Instance), C.c_uint32, C.c_int32]),
    ("luz_frame_plane_bytes", C.c_size_t, [P, C.c_int32]),
    ("luz_frame_read", C.c_int32, [P, P, C.c_int32, P, C.c_size_t]),
    ("luz_frame_write", C.c_int32, [P, P, C.c_int32, P, C.c_size_t]),
    ("luz_frame_plane_device_ptr", P, [P, C.c_int32]),
    ("luz_batch_create", C.c_int32, [P, C.c_uint32, C.POINTER(BatchScene), C.POINTER(P)]),
    ("luz_batch_destroy", None, [P]),
    ("luz_batch_count", C.c_uint32, [P]),
    ("luz_batch_frame", P, [P, C.c_uint32]),
    ("luz_batch_render", C.c_int32, [P, P, C.c_int32]),
    ("luz_batch_stats", C.c_int32, [P, P, C.c_int32, C.POINTER(C.c_uint64)]),
    ("luz_batch_capture", C.c_int32, [P, P, C.c_int32]),
    ("luz_batch_replay", C.c_int32, [P, P]),
    ("luz_batch_autotune", C.c_int32, [P, P, C.c_uint32, C.POINTER(C.c_uint32 * 4), C.POINTER(C.c_float)]),
    ("luz_batch_set_fused", C.c_int32, [P, P, C.c_int32]),
    ("luz_batch_fused", C.c_int32, [P]),
    ("luz_denoiser_create", C.c_int32, [P, C.c_uint64, C.POINTER(P)]),
    ("luz_denoiser_destroy", None, [P]),
    ("luz_denoiser_set_weights", C.c_int32, [P, P, c_float_p]),
    ("luz_denoiser_get_weights", C.c_int32, [P, P, c_float_p]),
    ("luz_denoiser_set_shadow_weight", C.c_int32, [P, P, C.c_float]),
    ("luz_denoise_features", C.c_int32, [P, P]),
    ("luz_denoise", C.c_int32, [P, P, P]),
    ("luz_denoise_batch_infer", C.c_int32, [P, P, C.POINTER(DenoiseBatch), P]),
    ("luz_denoiser_gradient", C.c_int32, [P, P, C.POINTER(DenoiseBatch), c_float_p, c_float_p]),
    ("luz_denoiser_train_step", C.c_int32, [P, P, C.POINTER(DenoiseBatch), C.c_float, c_float_p]),
    # luz_scene.h
    ("luz_scene_default_params", C.c_int32, [C.c_int32, C.POINTER(GenParams)]),
    ("luz_scene_generate", C.c_int32, [C.POINTER(GenParams), C.POINTER(P)]),
    ("luz_scene_destroy", None, [P]),
    ("luz_scene_mesh_count", C.c_uint32, [P]),
    ("luz_scene_mesh", C.c_int32, [P, C.c_uint32, C.POINTER(C.POINTER(Vertex)), c_u32_p,
                                   C.POINTER(c_u32_p), c_u32_p]),
    ("luz_scene_instance_count", C.c_uint32, [P]),
    ("luz_scene_instance_mesh", c_u32_p, [P]),
    ("luz_scene_models", C.POINTER(Model), [P]),
    ("luz_scene_light_count", C.c_uint32, [P]),
    ("luz_scene_lights", C.POINTER(Light), [P]),
    ("luz_scene_block", C.POINTER(Scene), [P]),
    ("luz_scene_width", C.c_uint32, [P]),
    ("luz_scene_height", C.c_uint32, [P]),
    ("luz_scene_instance_transforms", C.c_int32, [P, c_float_p]),
    ("luz_scene_set_camera", C.c_int32, [P, C.POINTER(Camera)]),
    ("luz_scene_get_camera", C.c_int32, [P, C.POINTER(Camera)]),
    ("luz_scene_set_sampling", C.c_int32, [P, C.c_int32, C.c_float, C.c_float, C.c_int32, C.c_int32]),
    ("luz_scene_load_project", C.c_int32, [C.c_char_p, C.c_char_p, C.c_uint32, C.c_uint32, C.POINTER(P),
                                           C.c_char_p, C.c_uint32]),
    ("luz_scene_import", C.c_int32, [C.c_char_p, C.c_uint32, C.c_uint32, C.POINTER(P), C.c_char_p, C.c_uint32]),
    ("luz_scene_save_project", C.c_int32, [P, C.c_char_p, C.c_char_p, C.c_char_p, C.c_uint32]),
    ("luz_scene_texture_count", C.c_uint32, [P]),
    ("luz_scene_next_frame", C.c_int32, [P, C.c_int32]),
    ("luz_scene_shadow_lights", C.c_int32, [P, P]),
    ("luz_scene_set_shadow_type", C.c_int32, [P, C.c_int32]),
    ("luz_frame_render_shadow_maps", C.c_int32, [P, P, P, P, C.c_uint32, C.c_uint32]),
    ("luz_frame_read_shadow_map", C.c_int32, [P, P, C.c_uint32, P, C.c_size_t]),
    ("luz_scene_texture", C.c_int32, [P, C.c_uint32, C.POINTER(c_u8_p), c_u32_p, c_u32_p]),
    ("luz_compose_transform", None, [c_float_p, c_float_p, c_float_p, c_float_p, c_float_p]),
    ("luz_camera_matrices", None, [C.POINTER(Camera), c_float_p, c_float_p]),
    ("luz_blue_noise_generate", C.c_int32, [C.c_uint64, C.c_uint32, c_u8_p]),
]

_lib = None


def load() -> C.CDLL:
    """Loads the in-tree libluz_gb300.so. Raises if it was not built: there is no
    fallback implementation of any entry point."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise ImportError(f"{LIB_PATH} is missing: run luz_gb300.build.build() (needs nvcc)")
    lib = C.CDLL(str(LIB_PATH))
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def ptr(a: np.ndarray, t=C.c_void_p):
    return C.cast(a.ctypes.data, t)
