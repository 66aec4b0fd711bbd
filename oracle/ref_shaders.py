#!/usr/bin/env python3
"""Recipe: compile the reference's own light-pass shader code for the CPU.

Reads source/Shaders/light.frag and source/Shaders/utils.glsl from the reference tree
(where they lie; nothing is copied into the repository), keeps the functions of the
ray-traced light pass (main, EvaluateShadow, TraceShadowRay, TraceAORays,
BlueNoiseSample, DiskSample, HemisphereSample, the GGX terms, DepthToWorld), rewrites
the GLSL-only syntax so that it compiles as C++ under the reference's vendored glm:

  * unsuffixed float literals get an `f` (GLSL literals are single precision),
  * multi-component swizzles .xyz/.rgb/.xy/.rg become vec3(...)/vec2(...) of the operand,
  * `void main()` becomes `void light_main()`,

and writes oracle/_ref/ref_shaders.cpp: the shim (oracle/ref_shim.hpp), the shader
globals, the transformed functions, compile-time checks of the C ABI data contract
(include/luz.h) against the reference's LuzCommon.h layouts, and one C entry point
that runs the shader's main over a G-buffer with the oracle's BVH as the ray-query
backend. TEST INFRASTRUCTURE: the product never uses it.
"""
from __future__ import annotations

import argparse
import re
from pathlib import Path

LIGHT_FUNCS = ["DistributionGGX", "GeometrySchlickGGX", "GeometrySmith", "FresnelSchlick", "DiskSample",
               "HemisphereSample", "BlueNoiseSample", "TraceShadowRay", "TraceAORays", "EvaluateShadow", "main"]
UTIL_FUNCS = ["DepthToWorld"]


def extract(src: str, name: str) -> str:
    m = re.search(r"^[A-Za-z_][\w]*\s+" + name + r"\s*\(", src, re.M)
    if not m:
        raise SystemExit(f"function {name} not found")
    i = src.index("{", m.end())
    depth = 0
    for j in range(i, len(src)):
        if src[j] == "{":
            depth += 1
        elif src[j] == "}":
            depth -= 1
            if depth == 0:
                return src[m.start():j + 1]
    raise SystemExit(f"unbalanced braces in {name}")


def float_literals(s: str) -> str:
    return re.sub(r"(?<![\w.])(\d+\.\d*|\.\d+)([eE][-+]?\d+)?(?![\w.])", lambda m: m.group(0) + "f", s)


def swizzles(s: str) -> str:
    pat = re.compile(r"\.(xyz|rgb|xy|rg)\b")
    out = s
    while True:
        m = pat.search(out)
        if not m:
            return out
        end = m.start()
        i = end
        # walk back over the operand: identifiers, member dots, balanced () and [] groups
        while i > 0:
            c = out[i - 1]
            if c.isalnum() or c in "_.":
                i -= 1
            elif c in ")]":
                close, open_ = c, "(" if c == ")" else "["
                depth, j = 0, i - 1
                while j >= 0:
                    if out[j] == close:
                        depth += 1
                    elif out[j] == open_:
                        depth -= 1
                        if depth == 0:
                            break
                    j -= 1
                i = j
            else:
                break
        operand = out[i:end]
        ctor = "vec3" if m.group(1) in ("xyz", "rgb") else "vec2"
        out = out[:i] + f"{ctor}({operand})" + out[m.end():]


WRAPPER = r"""
#undef scene
#undef tlas

// The C ABI's data contract (include/luz.h) against the reference layouts (LuzCommon.h).
static_assert(sizeof(LightBlock) == 480, "LightBlock size");
static_assert(sizeof(ModelBlock) == sizeof(luz_model), "ModelBlock vs luz_model");
static_assert(offsetof(LightBlock, shadowMap) == offsetof(luz_light, shadow_map), "LightBlock head vs luz_light");
static_assert(offsetof(LightBlock, radius) == offsetof(luz_light, radius), "LightBlock radius");
static_assert(offsetof(ModelBlock, metallicRoughnessMap) == offsetof(luz_model, metallic_roughness_map), "ModelBlock");
#define LUZ_SB(f, g) static_assert(offsetof(SceneBlock, f) - sizeof(LightBlock) * LUZ_MAX_LIGHTS == offsetof(luz_scene, g), #f)
LUZ_SB(ambientLightColor, ambient_light_color); LUZ_SB(proj, proj); LUZ_SB(inverseProj, inverse_proj);
LUZ_SB(inverseView, inverse_view); LUZ_SB(camPos, cam_pos); LUZ_SB(numLights, num_lights); LUZ_SB(aoMin, ao_min);
LUZ_SB(aoNumSamples, ao_num_samples); LUZ_SB(blueNoiseTexture, blue_noise_texture); LUZ_SB(shadowType, shadow_type);
static_assert(sizeof(SceneBlock) - sizeof(LightBlock) * LUZ_MAX_LIGHTS == sizeof(luz_scene), "SceneBlock tail");

extern "C" int ref_light_pass(const luz_scene* S, const luz_light* L, int nl, const uint32_t* albedo,
                              const float* normal, const uint32_t* material, const uint32_t* emission,
                              const float* depth, const uint8_t* bn, int bn_size, int W, int H, int frame,
                              refshim::AnyHitFn fn, const void* user, float* out, float* ray_log,
                              uint64_t ray_log_cap, uint64_t* ray_count) {
    if (nl < 0 || nl > LUZ_MAX_LIGHTS) return 1;
    SceneBlock& sb = g_scene;
    memset(&sb, 0, sizeof(sb));
    for (int i = 0; i < nl; ++i) memcpy(&sb.lights[i], &L[i], sizeof(luz_light));   // head of LightBlock
    memcpy((char*)&sb + sizeof(LightBlock) * LUZ_MAX_LIGHTS, S, sizeof(luz_scene));
    sb.numLights = nl;
    sb.blueNoiseTexture = 5;
    textures[0] = {albedo, W, H, 0};
    textures[1] = {normal, W, H, 1};
    textures[2] = {material, W, H, 0};
    textures[3] = {emission, W, H, 0};
    textures[4] = {depth, W, H, 2};
    textures[5] = {bn, bn_size, bn_size, 0};
    memset(&ctx, 0, sizeof(ctx));
    ctx.frame = frame;
    ctx.albedoRID = 0; ctx.normalRID = 1; ctx.materialRID = 2; ctx.emissionRID = 3; ctx.depthRID = 4;
    refshim::g_env = refshim::Env{fn, user, ray_log, ray_log_cap, 0};
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            gl_FragCoord = vec4(x + 0.5f, y + 0.5f, 0.0f, 1.0f);
            fragTexCoord = vec2((x + 0.5f) / (float)W, (y + 0.5f) / (float)H);
            light_main();
            float* o = out + 4 * ((size_t)y * W + x);
            o[0] = outColor.x; o[1] = outColor.y; o[2] = outColor.z; o[3] = outColor.w;
        }
    if (ray_count) *ray_count = refshim::g_env.ray_count;
    return 0;
}
"""


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", required=True)
    ap.add_argument("--out", required=True)
    a = ap.parse_args()
    ref = Path(a.reference) / "source" / "Shaders"
    light = (ref / "light.frag").read_text()
    utils = (ref / "utils.glsl").read_text()
    parts = [extract(utils, f) for f in UTIL_FUNCS] + [extract(light, f) for f in LIGHT_FUNCS]
    body = "\n\n".join(parts)
    body = body.replace("void main()", "void light_main()")
    body = swizzles(float_literals(body))
    out = Path(a.out)
    out.mkdir(parents=True, exist_ok=True)
    head = "\n".join([
        "// Generated by oracle/ref_shaders.py from the reference's light.frag and utils.glsl.",
        "#include <cstddef>",
        '#include "ref_shim.hpp"',
        '#include "luz.h"',
        "namespace refshim { Env g_env; }",
        "SceneBlock g_scene;",
        "sampler2D textures[8];",
        "samplerCube cubeTextures[1];",
        "LightConstants ctx;",
        "vec2 fragTexCoord;",
        "vec4 outColor;",
        "vec4 gl_FragCoord;",
        "#define scene g_scene",
        "#define tlas tlas_dummy",
        "",
    ])
    (out / "ref_shaders.cpp").write_text(head + body + "\n" + WRAPPER)


if __name__ == "__main__":
    main()
