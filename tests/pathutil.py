"""Shared helpers: run one scene through the CUDA path (C ABI) and the CPU oracle."""
from __future__ import annotations

import numpy as np

import luz_gb300 as L
import oracle as O


def oracle_scene(scene: L.HostScene):
    meshes = scene.meshes()
    ob = [O.OracleBlas(v, i) for v, i in meshes]
    im = scene.instance_mesh()
    tl = O.OracleTlas([ob[m] for m in im], scene.transforms())
    return ob, tl


def oracle_frame(scene: L.HostScene, tlas: "O.OracleTlas", frame: int = 0, bn=None, brute=False, models=None,
                 textures=None):
    b, lights = scene.block(), scene.lights()
    models = scene.models() if models is None else models
    f = O.OracleFrame(tlas, b, lights, scene.light_count, models, scene.instance_count, scene.width, scene.height)
    f.gbuffer(textures=scene.textures() if textures is None else textures)
    f.visibility(frame, L.blue_noise() if bn is None else bn, brute=brute)
    return f


def gpu_frame(ctx: L.Context, scene: L.HostScene, frame: int = 0) -> L.GPUScene:
    g = L.GPUScene(ctx, scene)
    g.render(frame)
    ctx.synchronize()
    assert ctx.device_status() == 0
    return g


def bits_mismatch(a: np.ndarray, b: np.ndarray) -> int:
    return int(np.unpackbits((a ^ b).view(np.uint8)).sum())
