"""Python handle on the CPU oracle (oracle/luz_oracle.cpp).

TEST INFRASTRUCTURE: imported only by tests/, the smoke check and the CPU-baseline
leg of bench.py, as the checker. The product never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "libluz_oracle.so"

P = C.c_void_p


def build() -> Path:
    src = HERE / "luz_oracle.cpp"
    if not LIB.exists() or LIB.stat().st_mtime < src.stat().st_mtime:
        subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB


_lib = None


def load() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        lib = C.CDLL(str(LIB))
        sig = {
            "oracle_blas_build": (C.c_int, [P, C.c_uint32, C.c_uint32, P, C.c_uint32, C.POINTER(P)]),
            "oracle_blas_prims": (C.c_uint32, [P]),
            "oracle_blas_get": (None, [P, P, P, P, P]),
            "oracle_blas_destroy": (None, [P]),
            "oracle_tlas_build": (C.c_int, [P, P, P, P, C.c_uint32, C.POINTER(P)]),
            "oracle_tlas_get": (None, [P, P, P, P, P]),
            "oracle_tlas_destroy": (None, [P]),
            "oracle_gbuffer": (C.c_int, [P, P, P, C.c_uint32, C.c_uint32, C.c_uint32, P, P, P, P, P, P, C.c_int,
                                         C.c_uint32, C.c_uint32, P, P, C.c_uint32]),
            "oracle_visibility": (C.c_uint64, [P, P, P, C.c_uint32, P, P, C.c_uint32, C.c_uint32, C.c_uint32,
                                               C.c_uint32, C.c_int, P, C.c_uint32, P, P, C.c_int, C.c_int,
                                               C.c_int]),
            "oracle_light_pass": (C.c_int, [P, P, C.c_uint32, P, P, P, P, P, P, P, P, C.c_uint32, C.c_uint32, P,
                                            C.c_int, C.c_uint32, C.c_uint32]),
            "oracle_light_split": (C.c_int, [P, P, C.c_uint32, P, P, P, P, P, P, P, C.c_uint32, C.c_uint32, P,
                                             C.c_int]),
            "oracle_light_pass_f64": (C.c_int, [P, P, C.c_uint32, P, P, P, P, P, P, P, P, C.c_uint32, C.c_uint32,
                                                P, C.c_int, C.c_uint32, C.c_uint32]),
            "oracle_trace_ray": (C.c_int, [P, P, P, C.c_float, C.c_float, C.c_int, C.c_int, P]),
            "oracle_generate_rays": (C.c_uint64, [P, P, C.c_uint32, P, P, C.c_uint32, C.c_uint32, C.c_int, P,
                                                  C.c_uint32, P, C.c_uint64]),
            "oracle_sincos": (None, [P, P, P, C.c_uint32]),
            "oracle_taa": (None, [P, P, P, P, C.c_uint32, C.c_uint32, C.c_int, P, C.c_int]),
            "oracle_compose": (None, [P, P, P, P, P, P, C.c_uint32, C.c_uint32, C.c_int, P]),
            "oracle_render_shadow_maps": (None, [P, P, C.c_uint32, C.c_uint32, P, C.c_int]),
            "oracle_clear_shadow_maps": (None, []),
            "oracle_histogram": (None, [P, C.c_uint32, C.c_float, P, P]),
            "oracle_disk_sample": (None, [C.c_float, C.c_float, C.c_float, P, P]),
            "oracle_hemisphere_sample": (None, [C.c_float, C.c_float, P]),
            "oracle_ggx_terms": (None, [P, P, P, C.c_float, P, P, P, P]),
            "oracle_depth_to_world": (None, [P, C.c_float, C.c_float, C.c_float, P]),
        }
        for name, (res, args) in sig.items():
            f = getattr(lib, name)
            f.restype, f.argtypes = res, args
        _lib = lib
    return _lib


def _p(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


REF_LIB = HERE / "_ref" / "libluz_ref_shaders.so"


def load_ref():
    """The reference's own light-pass shader compiled for the CPU (oracle/_ref), or
    None where the reference tree was not available to build it."""
    if not REF_LIB.exists():
        return None
    lib = C.CDLL(str(REF_LIB))
    f = lib.ref_light_pass
    f.restype = C.c_int
    f.argtypes = [P, P, C.c_int, P, P, P, P, P, P, C.c_int, C.c_int, C.c_int, C.c_int, P, P, P, P, C.c_uint64,
                  C.POINTER(C.c_uint64), P, P, C.c_int, C.c_int]
    return lib


def threads() -> int:
    return max(1, len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count() or 1)


class OracleBlas:
    def __init__(self, vertices: np.ndarray, indices: np.ndarray):
        lib = load()
        v = np.ascontiguousarray(vertices, np.float32)
        i = np.ascontiguousarray(indices, np.uint32)
        h = C.c_void_p()
        st = lib.oracle_blas_build(_p(v), v.shape[0], v.shape[1] * 4, _p(i), i.size, C.byref(h))
        if st != 0:
            raise ValueError(f"oracle_blas_build failed ({st})")
        self._h = h
        self.prims = i.size // 3

    @property
    def handle(self):
        return self._h

    def arrays(self):
        n = self.prims
        m = max(n, 2) - 1
        nodes = np.zeros((m, 16), np.float32)
        tris = np.zeros((max(n, 1), 12), np.float32)
        mort = np.zeros(max(n, 1), np.uint32)
        order = np.zeros(max(n, 1), np.uint32)
        load().oracle_blas_get(self._h, _p(nodes), _p(tris), _p(mort), _p(order))
        return nodes, tris[:n], mort[:n], order[:n]

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.oracle_blas_destroy(self._h)
            self._h = None


class OracleTlas:
    def __init__(self, blas_per_instance: list[OracleBlas], transforms: np.ndarray, custom=None, mask=None):
        lib = load()
        n = len(blas_per_instance)
        arr = (C.c_void_p * max(n, 1))(*[b.handle.value for b in blas_per_instance])
        tr = np.ascontiguousarray(transforms, np.float32).reshape(n, 12)
        cu = None if custom is None else np.ascontiguousarray(custom, np.uint32)
        ma = None if mask is None else np.ascontiguousarray(mask, np.uint32)
        h = C.c_void_p()
        lib.oracle_tlas_build(C.cast(arr, C.c_void_p), _p(tr), _p(cu), _p(ma), n, C.byref(h))
        self._h = h
        self.n = n
        self._keep = blas_per_instance

    @property
    def handle(self):
        return self._h

    def arrays(self):
        lib = load()
        cnt = C.c_uint32()
        lib.oracle_tlas_get(self._h, None, None, None, C.byref(cnt))
        nodes = np.zeros((max(cnt.value, 1), 16), np.float32)
        mort = np.zeros(max(self.n, 1), np.uint32)
        order = np.zeros(max(self.n, 1), np.uint32)
        lib.oracle_tlas_get(self._h, _p(nodes), _p(mort), _p(order), C.byref(cnt))
        return nodes[: cnt.value], mort[: self.n], order[: self.n]

    def ray(self, o, d, tmin, tmax, closest=False, brute=False):
        o = np.asarray(o, np.float32)
        d = np.asarray(d, np.float32)
        t = C.c_float()
        r = load().oracle_trace_ray(self._h, _p(o), _p(d), tmin, tmax, int(closest), int(brute), C.byref(t))
        return bool(r), t.value

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.oracle_tlas_destroy(self._h)
            self._h = None


def scene_bytes(scene) -> C.c_void_p:
    return C.cast(C.byref(scene), C.c_void_p)


class OracleFrame:
    """G-buffer, visibility and light pass of one frame on the CPU."""

    def __init__(self, tlas: OracleTlas, scene, lights, n_lights: int, models, n_models: int, width: int,
                 height: int):
        self.tlas, self.scene, self.lights, self.nl = tlas, scene, lights, n_lights
        self.models, self.nm, self.W, self.H = models, n_models, width, height
        P_ = width * height
        self.albedo = np.zeros(P_, np.uint32)
        self.normal = np.zeros((P_, 4), np.float32)
        self.material = np.zeros(P_, np.uint32)
        self.emission = np.zeros(P_, np.uint32)
        self.depth = np.zeros(P_, np.float32)
        self.primary_hit = np.zeros((P_, 2), np.uint32)
        self.words = (P_ + 31) // 32
        ns = sum(max(0, lights[i].num_shadow_samples) for i in range(n_lights)) \
            if scene.shadow_type == 1 else 0
        self.shadow_slots = ns
        self.ao_samples = max(0, scene.ao_num_samples)
        self.shadow_bits = np.zeros((max(ns, 1), self.words), np.uint32)
        self.ao_bits = np.zeros((max(self.ao_samples, 1), self.words), np.uint32)

    def gbuffer(self, nthreads=None, y0: int = 0, y1: int | None = None, textures=()):
        """textures: RGBA8 arrays (h, w, 4) indexed by the ModelBlocks' map fields."""
        tex = [np.ascontiguousarray(t, np.uint8) for t in textures]
        ptrs = (C.c_void_p * max(len(tex), 1))(*[t.ctypes.data for t in tex])
        dims = np.array([[t.shape[1], t.shape[0]] for t in tex] or [[0, 0]], np.uint32)
        load().oracle_gbuffer(self.tlas.handle, scene_bytes(self.scene), C.cast(self.models, C.c_void_p), self.nm,
                              self.W, self.H, _p(self.albedo), _p(self.normal), _p(self.material),
                              _p(self.emission), _p(self.depth), _p(self.primary_hit), nthreads or threads(),
                              y0, self.H if y1 is None else y1, C.cast(ptrs, C.c_void_p), _p(dims), len(tex))

    def visibility(self, frame: int, bn: np.ndarray, y0: int = 0, y1: int | None = None, brute: bool = False,
                   nthreads=None, cull: bool = True) -> int:
        """Shadow/AO bit planes. cull: leave out the shadow rays whose light has a zero
        max(dot(N, L), 0) weight in the light pass, as the device does; False traces
        every ray of light.frag. Returns the rays traced."""
        bn = np.ascontiguousarray(bn, np.uint8)
        y1 = self.H if y1 is None else y1
        return load().oracle_visibility(self.tlas.handle, scene_bytes(self.scene), C.cast(self.lights, C.c_void_p),
                                        self.nl, _p(self.normal), _p(self.depth), self.W, self.H, y0, y1, frame,
                                        _p(bn), bn.shape[0], _p(self.shadow_bits), _p(self.ao_bits),
                                        nthreads or threads(), int(brute), int(cull))

    def light_pass(self, ao_override=None, f64=False, nthreads=None, y0: int = 0, y1: int | None = None) -> np.ndarray:
        P_ = self.W * self.H
        out = np.zeros((P_, 4), np.float64 if f64 else np.float32)
        fn = load().oracle_light_pass_f64 if f64 else load().oracle_light_pass
        ao = None if ao_override is None else np.ascontiguousarray(ao_override, np.float32)
        fn(scene_bytes(self.scene), C.cast(self.lights, C.c_void_p), self.nl, _p(self.albedo), _p(self.normal),
           _p(self.material), _p(self.emission), _p(self.depth), _p(self.shadow_bits), _p(self.ao_bits), _p(ao),
           self.W, self.H, _p(out), nthreads or threads(), y0, self.H if y1 is None else y1)
        return out.reshape(self.H, self.W, 4)

    def light_split(self, nthreads=None) -> tuple[np.ndarray, np.ndarray]:
        """The denoiser's split of the direct light: (signal [H, W, 4] = shadowed direct
        light S r, g, b and AO; unshadowed [H, W, 4] = U r, g, b and the unoccluded
        fraction of all shadow samples)."""
        out = np.zeros((self.W * self.H, 8), np.float32)
        load().oracle_light_split(scene_bytes(self.scene), C.cast(self.lights, C.c_void_p), self.nl, _p(self.albedo),
                                  _p(self.normal), _p(self.material), _p(self.emission), _p(self.depth),
                                  _p(self.shadow_bits), _p(self.ao_bits), self.W, self.H, _p(out),
                                  nthreads or threads())
        out = out.reshape(self.H, self.W, 8)
        return out[..., :4].copy(), out[..., 4:].copy()


K_EMPTY_CHILD = -2147483647   # 0x80000001: a child slot with an inverted box


def _child_box(node: np.ndarray, side: int):
    """Box of child `side` of a binary node (64 B: see the BVH layout of the library)."""
    if side == 0:
        return (node[0], node[2], node[8]), (node[1], node[3], node[9])
    return (node[4], node[6], node[10]), (node[5], node[7], node[11])


def collapse_wide(nodes: np.ndarray) -> np.ndarray:
    """Even-depth 4-wide collapse of a binary BVH (rows of 16 float32, root at 0).

    Every binary node at even depth becomes a 4-wide node; its slots are its
    grandchildren, or its children where a child is a leaf (or an empty slot), in
    left-to-right order, padded with inverted boxes and the empty-child id. Internal
    slot ids are ranks among the even-depth nodes in index order. Rows of 32 float32:
    lo.x[4] hi.x[4] lo.y[4] hi.y[4] lo.z[4] hi.z[4] child[4] (int bits) 0[4].
    """
    m = len(nodes)
    iv = nodes.view(np.int32)
    depth = np.full(m, -1, np.int64)
    depth[0] = 0
    stack = [0]
    while stack:
        q = stack.pop()
        for side in (0, 1):
            c = int(iv[q, 12 + side])
            if c >= 0:
                depth[c] = depth[q] + 1
                stack.append(c)
    even = np.nonzero(depth % 2 == 0)[0]
    rank = np.full(m, -1, np.int64)
    rank[even] = np.arange(len(even))
    out = np.zeros((len(even), 32), np.float32)
    oi = out.view(np.int32)
    for q in even:
        slots = []
        for side in (0, 1):
            c = int(iv[q, 12 + side])
            if c < 0:
                slots.append((_child_box(nodes[q], side), c))
                continue
            for s2 in (0, 1):
                g = int(iv[c, 12 + s2])
                slots.append((_child_box(nodes[c], s2), g if g < 0 else int(rank[g])))
        row = int(rank[q])
        for k in range(4):
            if k < len(slots):
                (lo, hi), cid = slots[k]
            else:
                lo, hi, cid = (np.inf,) * 3, (-np.inf,) * 3, K_EMPTY_CHILD
            for a in range(3):
                out[row, 8 * a + k] = lo[a]
                out[row, 8 * a + 4 + k] = hi[a]
            oi[row, 24 + k] = cid
    return out


def taa(scene, light: np.ndarray, history: np.ndarray, depth: np.ndarray, reconstruct: bool = True,
        nthreads=None) -> np.ndarray:
    """One TAA pass (taa.comp) over (H, W, 4) float32 images and an (H, W) depth."""
    H, W = depth.shape
    light = np.ascontiguousarray(light, np.float32)
    history = np.ascontiguousarray(history, np.float32)
    depth = np.ascontiguousarray(depth, np.float32)
    out = np.zeros((H, W, 4), np.float32)
    load().oracle_taa(scene_bytes(scene), _p(light), _p(history), _p(depth), W, H, int(bool(reconstruct)), _p(out),
                      nthreads or threads())
    return out


def compose(light, albedo, normal, material, emission, depth, image_type: int = 0) -> np.ndarray:
    """present.frag over (H, W) images -> BGRA8 words (H, W) uint32."""
    H, W = depth.shape
    arrs = [np.ascontiguousarray(a) for a in (light, albedo, normal, material, emission, depth)]
    out = np.zeros((H, W), np.uint32)
    load().oracle_compose(*[_p(a) for a in arrs], W, H, image_type, _p(out))
    return out


def histogram(img, delta_time: float = 1.0 / 60.0, state=None):
    """Luminance histogram + averages of an (..., 4) float32 image; state: [adapted]."""
    img = np.ascontiguousarray(img, np.float32).reshape(-1, 4)
    st = np.zeros(1, np.float32) if state is None else state
    out = np.zeros(260, np.uint32)
    load().oracle_histogram(_p(img), img.shape[0], delta_time, _p(st), _p(out))
    f = out[256:].view(np.float32)
    return {"bins": out[:256].copy(), "weighted_sum": float(f[0]), "log_average": float(f[1]),
            "average_luminance": float(f[2]), "adapted_luminance": float(f[3])}, st


def render_shadow_maps(tlas, lights, res: int, nthreads=None):
    """Shadow maps of every light (a ctypes array of luz_shadow_light); returns a list of
    (faces, res, res) float32 arrays and registers them for OracleFrame.light_pass."""
    n = len(lights)
    total = sum(int(l.faces) for l in lights) * res * res
    buf = np.zeros(max(total, 1), np.float32)
    load().oracle_render_shadow_maps(tlas.handle, C.cast(lights, C.c_void_p), n, res, _p(buf), nthreads or threads())
    out, off = [], 0
    for l in lights:
        k = int(l.faces) * res * res
        out.append(buf[off:off + k].reshape(int(l.faces), res, res))
        off += k
    _keep_maps[:] = [buf]
    return out


_keep_maps = []


def clear_shadow_maps():
    load().oracle_clear_shadow_maps()
    _keep_maps.clear()
