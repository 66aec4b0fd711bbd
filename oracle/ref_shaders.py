#!/usr/bin/env python3
"""Recipe: compile the reference's own light-pass shader code for the CPU.

Reads source/Shaders/light.frag and source/Shaders/utils.glsl from the reference tree
(and taa.comp, present.frag, histogram.comp, histogramAverage.comp for the post passes)
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
TAA_UTIL_FUNCS = ["DepthToWorld", "MitchellFilter", "rcp", "Luminance"]
TAA_FUNCS = ["get_uv", "get_motion_vector", "get_neighbor_3x3", "find_closest_3x3", "clip_aabb", "anti_flicker",
             "main"]
COMPOSE_FUNCS = ["LinearizeDepth", "Tonemap", "TonemapACES", "TonemapExposure", "main"]
HIST_UTIL_FUNCS = ["Luminance"]
HIST_FUNCS = ["HDRToHistogramBin"]


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


def params(s: str) -> str:
    """GLSL `out T x` / `inout T x` parameters become C++ references."""
    return re.sub(r"\b(?:inout|out)\s+(\w+)\s+(\w+)", r"\1& \2", s)


def divide_by_w(s: str) -> str:
    """`v.xyz /= v.w;` (a swizzle assignment) -> `v = vec4(vec3(v) / v.w, v.w);`."""
    return re.sub(r"(\w+)\.xyz\s*/=\s*(\w+)\.w\s*;", r"\1 = vec4(vec3(\1) / \2.w, \1.w);", s)


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


TAA_HEAD = """// Generated by oracle/ref_shaders.py from the reference's taa.comp and utils.glsl.
#include <cstddef>
#include "ref_shim.hpp"
#include "luz.h"
static SceneBlock t_scene;
static sampler2D t_textures[4];
static image2D t_images[1];
static PostProcessingConstants t_ctx;
static uvec3 gl_GlobalInvocationID;
#define scene t_scene
#define textures t_textures
#define images t_images
#define ctx t_ctx
"""

TAA_WRAPPER = r"""
#undef scene
#undef textures
#undef images
#undef ctx
extern "C" void ref_taa(const luz_scene* S, const float* input, const float* history, const float* depth, int W,
                        int H, int reconstruct, float* out) {
    memset(&t_scene, 0, sizeof(t_scene));
    memcpy((char*)&t_scene + sizeof(LightBlock) * LUZ_MAX_LIGHTS, S, sizeof(luz_scene));
    t_textures[0] = {input, W, H, 1, 1};
    t_textures[1] = {history, W, H, 1, 1};
    t_textures[2] = {depth, W, H, 2, 1};
    t_images[0] = {out, W, H};
    memset(&t_ctx, 0, sizeof(t_ctx));
    t_ctx.lightInputRID = 0; t_ctx.lightHistoryRID = 1; t_ctx.depthRID = 2; t_ctx.lightOutputRID = 0;
    t_ctx.size = vec2((float)W, (float)H);
    t_ctx.reconstruct = reconstruct;
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            gl_GlobalInvocationID = uvec3(x, y, 0);
            taa_main();
        }
}
"""

COMPOSE_HEAD = """// Generated by oracle/ref_shaders.py from the reference's present.frag.
#include <cstddef>
#include "ref_shim.hpp"
#include "luz.h"
static sampler2D c_textures[8];
static ComposeConstants c_ctx;
static vec2 fragTexCoord;
static vec4 outColor;
#define textures c_textures
#define ctx c_ctx
"""

COMPOSE_WRAPPER = r"""
#undef textures
#undef ctx
extern "C" void ref_compose(const float* light, const uint32_t* albedo, const float* normal, const uint32_t* material,
                            const uint32_t* emission, const float* depth, int W, int H, int image_type, float* out) {
    c_textures[0] = {light, W, H, 1, 1};
    c_textures[1] = {albedo, W, H, 0, 1};
    c_textures[2] = {normal, W, H, 1, 1};
    c_textures[3] = {material, W, H, 0, 1};
    c_textures[4] = {emission, W, H, 0, 1};
    c_textures[5] = {depth, W, H, 2, 1};
    c_textures[6] = {nullptr, 1, 1, 0, 1};   // the debug-line overlay: empty
    memset(&c_ctx, 0, sizeof(c_ctx));
    c_ctx.lightRID = 0; c_ctx.albedoRID = 1; c_ctx.normalRID = 2; c_ctx.materialRID = 3; c_ctx.emissionRID = 4;
    c_ctx.depthRID = 5; c_ctx.debugRID = 6; c_ctx.imageType = image_type;
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            fragTexCoord = vec2((x + 0.5f) / (float)W, (y + 0.5f) / (float)H);
            compose_main();
            float* o = out + 4 * ((size_t)y * W + x);
            o[0] = outColor.x; o[1] = outColor.y; o[2] = outColor.z; o[3] = outColor.w;
        }
}
"""

HIST_HEAD = """// Generated by oracle/ref_shaders.py from the reference's histogram.comp,
// histogramAverage.comp and utils.glsl.
#include <cstddef>
#include "ref_shim.hpp"
#include "luz.h"
static PostProcessingConstants h_ctx;
struct HistFloatBuffer { float* data; };
static HistFloatBuffer h_floatBuffers[2];
static float HistogramShared[LUZ_HISTOGRAM_BINS];
#define ctx h_ctx
#define floatBuffers h_floatBuffers
"""

HIST_WRAPPER = r"""
#undef ctx
#undef floatBuffers
// DeferredRenderer.cpp:447-466: histogramMinLog -10, histogramOneOverLog 1/12.
static void hist_constants(float width, float height, float delta_time) {
    memset(&h_ctx, 0, sizeof(h_ctx));
    h_ctx.size = vec2(width, height);
    h_ctx.deltaTime = delta_time;
    h_ctx.histogramMinLog = -10.0f;
    h_ctx.histogramOneOverLog = 1.0f / 12.0f;
    h_ctx.histogramRID = 0;
    h_ctx.histogramAverageRID = 1;
}

// The bin of every pixel of an RGBA32F image (histogram.comp's HDRToHistogramBin).
extern "C" void ref_histogram_bins(const float* rgba, int n, uint32_t* bins) {
    hist_constants((float)n, 1.0f, 0.0f);
    for (int i = 0; i < n; ++i) bins[i] = HDRToHistogramBin(vec3(rgba[4 * i], rgba[4 * i + 1], rgba[4 * i + 2]));
}

// histogramAverage.comp's one workgroup of 256 threads over the bin counts, run phase
// by phase between its barriers: each thread's count x bin index, the halving tree
// sum, then thread 0's block. out: the weighted sum, weightedLogAverage,
// weightedAverageLuminance, adaptedLuminance and the value the shader stores in the
// average buffer.
extern "C" void ref_histogram_average(const uint32_t* counts, int width, int height, float delta_time,
                                      float last_luminance, float* out) {
    hist_constants((float)width, (float)height, delta_time);
    float bins[LUZ_HISTOGRAM_BINS * 4] = {}, average[4] = {last_luminance, 0.0f, 0.0f, 0.0f};
    for (int i = 0; i < LUZ_HISTOGRAM_BINS; ++i) bins[i * 4] = (float)counts[i];
    h_floatBuffers[0].data = bins;
    h_floatBuffers[1].data = average;
    for (uint32_t g = 0; g < LUZ_HISTOGRAM_BINS; ++g) hist_avg_init(g);
    for (uint32_t k = (LUZ_HISTOGRAM_BINS >> 1); k > 0; k >>= 1)
        for (uint32_t g = 0; g < LUZ_HISTOGRAM_BINS; ++g) hist_avg_step(g, k);
    hist_average_final(bins[0], out);
    out[4] = average[0];
}
"""

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
                              uint64_t ray_log_cap, uint64_t* ray_count, const luz_shadow_light* sl,
                              const float* maps, int sl_count, int map_res) {
    if (nl < 0 || nl > LUZ_MAX_LIGHTS) return 1;
    SceneBlock& sb = g_scene;
    memset(&sb, 0, sizeof(sb));
    for (int i = 0; i < nl; ++i) memcpy(&sb.lights[i], &L[i], sizeof(luz_light));   // head of LightBlock
    // Shadow maps (scene shadow type MAP): the LightBlock tail (viewProj, zFar) and the
    // map as a cube texture (point lights) or a 2D texture read through the bilinear,
    // repeat-addressed sampler; maps of the lights are concatenated in light order.
    for (int i = 0; i < nl; ++i) {
        sb.lights[i].shadowMap = -1;
        cubeTextures[i] = samplerCube{};
    }
    const float* m = maps;
    for (int i = 0; sl && maps && i < sl_count && i < nl; ++i) {
        if (!sl[i].faces) continue;
        for (int f = 0; f < 6; ++f) memcpy(&sb.lights[i].viewProj[f], sl[i].view_proj[f], 64);
        sb.lights[i].zFar = sl[i].z_far;
        if (sl[i].faces == 6) {
            cubeTextures[i] = samplerCube{m, map_res};
            sb.lights[i].shadowMap = i;
        } else {
            textures[8 + i] = {m, map_res, map_res, 2, 1};
            sb.lights[i].shadowMap = 8 + i;
        }
        m += (size_t)sl[i].faces * map_res * map_res;
    }
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
        "sampler2D textures[8 + LUZ_MAX_LIGHTS];",
        "samplerCube cubeTextures[LUZ_MAX_LIGHTS];",
        "LightConstants ctx;",
        "vec2 fragTexCoord;",
        "vec4 outColor;",
        "vec4 gl_FragCoord;",
        "#define scene g_scene",
        "#define tlas tlas_dummy",
        "",
    ])
    (out / "ref_shaders.cpp").write_text(head + body + "\n" + WRAPPER)

    # taa.comp (+ utils.glsl helpers) and present.frag
    taa = (ref / "taa.comp").read_text()
    tbody = "\n\n".join([extract(utils, f) for f in TAA_UTIL_FUNCS] + [extract(taa, f) for f in TAA_FUNCS])
    tbody = tbody.replace("void main()", "void taa_main()")
    tbody = tbody.replace("greaterThanEqual(pixelPos, ctx.size)", "greaterThanEqual(vec2(pixelPos), ctx.size)")
    tbody = swizzles(float_literals(divide_by_w(params(tbody))))
    (out / "ref_taa.cpp").write_text(TAA_HEAD + "namespace {\n" + tbody + "\n}  // namespace\n" + TAA_WRAPPER)
    present = (ref / "present.frag").read_text()
    cbody = "\n\n".join(extract(present, f) for f in COMPOSE_FUNCS)
    cbody = cbody.replace("void main()", "void compose_main()")
    cbody = cbody.replace("LinearizeDepth(value.r).xxxx", "vec4(LinearizeDepth(value.r))")
    cbody = swizzles(float_literals(cbody))
    (out / "ref_compose.cpp").write_text(COMPOSE_HEAD + "namespace {\n" + cbody + "\n}  // namespace\n" +
                                         COMPOSE_WRAPPER)

    # histogram.comp's bin function and histogramAverage.comp's phases
    hist = (ref / "histogram.comp").read_text()
    havg = (ref / "histogramAverage.comp").read_text()
    hbody = "\n\n".join([extract(utils, f) for f in HIST_UTIL_FUNCS] + [extract(hist, f) for f in HIST_FUNCS])
    amain = extract(havg, "main")
    init = re.search(r"float countForThisBin = (.*?);\s*HistogramShared\[groupIndex\] = (.*?);", amain, re.S)
    step = re.search(r"if \(groupIndex < histogramSampleIndex\) \{\s*(.*?;)\s*\}", amain, re.S)
    blk = re.search(r"if \(groupIndex == 0\) \{", amain)
    if not (init and step and blk):
        raise SystemExit("histogramAverage.comp: unexpected main")
    i = amain.index("{", blk.start())
    depth, j = 0, i
    for j in range(i, len(amain)):
        depth += {"{": 1, "}": -1}.get(amain[j], 0)
        if depth == 0:
            break
    final = amain[i + 1:j]
    phases = "\n".join([
        "void hist_avg_init(uint groupIndex) { float countForThisBin = " + init.group(1) +
        "; HistogramShared[groupIndex] = " + init.group(2) + "; }",
        "void hist_avg_step(uint groupIndex, uint histogramSampleIndex) { if (groupIndex < histogramSampleIndex) { " +
        step.group(1) + " } }",
        "void hist_average_final(float countForThisBin, float* out) {" + final +
        "\n    out[0] = HistogramShared[0]; out[1] = weightedLogAverage; out[2] = weightedAverageLuminance;"
        " out[3] = adaptedLuminance;\n}",
    ])
    hsrc = swizzles(float_literals(hbody + "\n\n" + phases))
    (out / "ref_histogram.cpp").write_text(HIST_HEAD + "namespace {\n" + hsrc + "\n}  // namespace\n" +
                                           HIST_WRAPPER)


if __name__ == "__main__":
    main()
