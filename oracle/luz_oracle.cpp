// luz_oracle.cpp — CPU oracle of the ray-traced visibility and deferred-lighting path.
//
// TEST INFRASTRUCTURE ONLY. Tests, the smoke check and the benchmark's CPU-baseline
// leg call this library as the checker; the product (libluz_gb300) never links,
// loads or calls it.
//
// It restates, one step per line, the reference's shader functions
// (hadryansalles/Luz, source/Shaders/light.frag:17-235, utils.glsl:1-7,
// opaque.vert:21-31, opaque.frag:21-58) in plain C++ over its own CPU build of the
// same two-level LBVH (Morton codes, stable sort, Karras hierarchy, refit). The
// reference's acceleration-structure build and traversal live in a closed Vulkan
// driver, so the LBVH here is the project's own algorithm restated, not the
// driver's. The reference ships no tests and no golden vectors: parity unpinned by
// reference tests. Pinning comes from analytic known-answer tests, from a
// brute-force all-triangles any-hit, and from the reference's own shader functions
// compiled under glm (recipe in oracle/Makefile, outputs in oracle/_ref/).
//
// Arithmetic rules (shared with the device code so that rays are bit-identical):
// no FMA contraction (-ffp-contract=off), IEEE division and sqrt, the operation
// order of the GLSL expressions, and the project's own sin/cos (Cody–Waite
// reduction + Taylor polynomials) where the shaders call cos/sin.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <functional>
#include <limits>
#include <thread>
#include <vector>

#include "../include/luz.h"

namespace oracle {

// ---------------------------------------------------------------- scalar helpers
static inline float fmin_(float a, float b) { return a < b ? a : b; }
static inline float fmax_(float a, float b) { return a > b ? a : b; }
static inline float clamp01(float x) { return fmin_(fmax_(x, 0.0f), 1.0f); }
static inline float fract_(float x) { return x - std::floor(x); }

template <typename T>
struct vec3 {
    T x, y, z;
};
template <typename T> static inline vec3<T> operator+(vec3<T> a, vec3<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <typename T> static inline vec3<T> operator-(vec3<T> a, vec3<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <typename T> static inline vec3<T> operator-(vec3<T> a) { return {-a.x, -a.y, -a.z}; }
template <typename T> static inline vec3<T> operator*(vec3<T> a, T s) { return {a.x * s, a.y * s, a.z * s}; }
template <typename T> static inline vec3<T> operator*(T s, vec3<T> a) { return {s * a.x, s * a.y, s * a.z}; }
template <typename T> static inline vec3<T> operator*(vec3<T> a, vec3<T> b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
template <typename T> static inline vec3<T> operator/(vec3<T> a, T s) { return {a.x / s, a.y / s, a.z / s}; }
template <typename T> static inline T dot(vec3<T> a, vec3<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <typename T> static inline vec3<T> cross(vec3<T> a, vec3<T> b) {
    return {a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y};
}
template <typename T> static inline T length(vec3<T> a) { return std::sqrt(dot(a, a)); }
template <typename T> static inline vec3<T> normalize(vec3<T> a) {   // pathmath.cuh normalize
    T inv = T(1) / length(a);
    return {a.x * inv, a.y * inv, a.z * inv};
}
template <typename T> static inline T tmax_(T a, T b) { return a > b ? a : b; }
template <typename T> static inline T tmin_(T a, T b) { return a < b ? a : b; }
template <typename T> static inline T tclamp01(T x) { return tmin_(tmax_(x, T(0)), T(1)); }

using v3 = vec3<float>;

// LuzCommon.h:10-12 (single-precision GLSL literals); light.frag:65.
static const float PI_F = 3.14159265359f;
static const float GOLDEN_RATIO_F = 2.118033988749895f;

// ---------------------------------------------------------------- sin / cos
// Cody–Waite reduction by pi/2 (three-part constant) + Taylor polynomials on
// |r| <= pi/4 (sin to r^9, cos to r^10), coefficients 1/n!.
static void sincos_cw(float x, float* s, float* c) {
    const float two_over_pi = 0x1.45f306p-1f;
    const float p1 = 0x1.92p+0f, p2 = 0x1.fb5p-12f, p3 = 0x1.110b46p-26f;
    float k = std::rint(x * two_over_pi);
    float r = x - k * p1;
    r = r - k * p2;
    r = r - k * p3;
    float r2 = r * r;
    const float s3 = -1.0f / 6.0f, s5 = 1.0f / 120.0f, s7 = -1.0f / 5040.0f, s9 = 1.0f / 362880.0f;
    const float c2 = -0.5f, c4 = 1.0f / 24.0f, c6 = -1.0f / 720.0f, c8 = 1.0f / 40320.0f, c10 = -1.0f / 3628800.0f;
    float sp = r + r * (r2 * (s3 + r2 * (s5 + r2 * (s7 + r2 * s9))));
    float cp = 1.0f + r2 * (c2 + r2 * (c4 + r2 * (c6 + r2 * (c8 + r2 * c10))));
    int q = ((int)k) & 3;
    if (q == 0) { *s = sp; *c = cp; }
    else if (q == 1) { *s = cp; *c = -sp; }
    else if (q == 2) { *s = -sp; *c = -cp; }
    else { *s = -cp; *c = sp; }
}

// ---------------------------------------------------------------- samplers
// DiskSample, light.frag:57-61
static void DiskSample(float rx, float ry, float radius, float* dx, float* dy) {
    float pointRadius = radius * std::sqrt(rx);
    float pointAngle = ry * 2.0f * PI_F;
    float s, c;
    sincos_cw(pointAngle, &s, &c);
    *dx = pointRadius * c;
    *dy = pointRadius * s;
}
// HemisphereSample, light.frag:63-69
static v3 HemisphereSample(float rx, float ry) {
    float r = std::sqrt(rx);
    float theta = 6.283f * ry;
    float s, c;
    sincos_cw(theta, &s, &c);
    float x = r * c;
    float y = r * s;
    return {x, y, std::sqrt(fmax_(0.0f, 1.0f - rx))};
}
// BlueNoiseSample(i).rg, light.frag:71-75 over the substitute texture.
static void BlueNoiseSample(const uint8_t* bn, uint32_t size, uint32_t px, uint32_t py, int i, int frame,
                            float* rx, float* ry) {
    const uint8_t* t = bn + 4 * ((size_t)(py % size) * size + (px % size));
    float offs = GOLDEN_RATIO_F * (float)(128 * i + frame % 128);
    *rx = fract_((float)t[0] / 255.0f + offs);
    *ry = fract_((float)t[1] / 255.0f + offs);
}
static uint32_t hash32(uint32_t x) {
    x ^= x >> 16; x *= 0x7feb352du;
    x ^= x >> 15; x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}
// Stratified: R2 sequence in 32-bit fixed point; the 64 pixels of an 8x8 block
// share one rotation and take interleaved points (sample i of pixel j: point 64 i + j).
static void StratifiedSample(uint32_t px, uint32_t py, int i, int frame, uint32_t stream, float* rx, float* ry) {
    uint32_t h = hash32((px >> 3) * 0x9E3779B1u ^ hash32((py >> 3) + 0x632BE5ABu * (uint32_t)(frame + 1)) ^
                        (stream * 0x85EBCA77u));
    uint32_t h2 = hash32(h ^ 0x27D4EB2Fu);
    uint32_t k = (uint32_t)i * 64u + (((py & 7u) << 3) | (px & 7u));
    uint32_t ux = h + k * 0xC13FA9A9u;
    uint32_t uy = h2 + k * 0x91E10DA5u;
    *rx = (float)(ux >> 8) * (1.0f / 16777216.0f);
    *ry = (float)(uy >> 8) * (1.0f / 16777216.0f);
}

struct Sampler {
    int kind;
    const uint8_t* bn;
    uint32_t bn_size;
    int frame;
    void rg(uint32_t px, uint32_t py, int i, uint32_t stream, float* rx, float* ry) const {
        if (kind == LUZ_SAMPLER_STRATIFIED) StratifiedSample(px, py, i, frame, stream, rx, ry);
        else BlueNoiseSample(bn, bn_size, px, py, i, frame, rx, ry);
    }
};

// ---------------------------------------------------------------- matrices
static void mat4_vec4(const float* m, const float v[4], float o[4]) {
    for (int r = 0; r < 4; ++r) o[r] = m[0 * 4 + r] * v[0] + m[1 * 4 + r] * v[1] + m[2 * 4 + r] * v[2] + m[3 * 4 + r] * v[3];
}
// DepthToWorld, utils.glsl:1-7
static v3 DepthToWorld(const luz_scene& S, float u, float v, float depth) {
    float clip[4] = {u * 2.0f - 1.0f, v * 2.0f - 1.0f, depth, 1.0f};
    float view[4];
    mat4_vec4(S.inverse_proj, clip, view);
    float w = view[3];
    for (int k = 0; k < 4; ++k) view[k] = view[k] / w;
    float world[4];
    mat4_vec4(S.inverse_view, view, world);
    return {world[0], world[1], world[2]};
}
static float pixel_uv(uint32_t x, uint32_t n) { return ((float)x + 0.5f) / (float)n; }

static void affine_inverse(const float m[12], float o[12]) {
    float a = m[0], b = m[1], c = m[2], d = m[4], e = m[5], f = m[6], g = m[8], h = m[9], k = m[10];
    float c00 = e * k - f * h;
    float c01 = f * g - d * k;
    float c02 = d * h - e * g;
    float det = a * c00 + b * c01 + c * c02;
    float inv = 1.0f / det;
    float r00 = c00 * inv, r01 = (c * h - b * k) * inv, r02 = (b * f - c * e) * inv;
    float r10 = c01 * inv, r11 = (a * k - c * g) * inv, r12 = (c * d - a * f) * inv;
    float r20 = c02 * inv, r21 = (b * g - a * h) * inv, r22 = (a * e - b * d) * inv;
    float tx = m[3], ty = m[7], tz = m[11];
    o[0] = r00; o[1] = r01; o[2] = r02; o[3] = -(r00 * tx + r01 * ty + r02 * tz);
    o[4] = r10; o[5] = r11; o[6] = r12; o[7] = -(r10 * tx + r11 * ty + r12 * tz);
    o[8] = r20; o[9] = r21; o[10] = r22; o[11] = -(r20 * tx + r21 * ty + r22 * tz);
}
static v3 xpoint(const float m[12], v3 p) {
    return {m[0] * p.x + m[1] * p.y + m[2] * p.z + m[3], m[4] * p.x + m[5] * p.y + m[6] * p.z + m[7],
            m[8] * p.x + m[9] * p.y + m[10] * p.z + m[11]};
}
static v3 xdir(const float m[12], v3 d) {
    return {m[0] * d.x + m[1] * d.y + m[2] * d.z, m[4] * d.x + m[5] * d.y + m[6] * d.z, m[8] * d.x + m[9] * d.y + m[10] * d.z};
}

// ---------------------------------------------------------------- LBVH
struct Box {
    v3 lo, hi;
};
static Box empty_box() {
    const float inf = std::numeric_limits<float>::infinity();
    return {{inf, inf, inf}, {-inf, -inf, -inf}};
}
static Box unite(const Box& a, const Box& b) {
    return {{fmin_(a.lo.x, b.lo.x), fmin_(a.lo.y, b.lo.y), fmin_(a.lo.z, b.lo.z)},
            {fmax_(a.hi.x, b.hi.x), fmax_(a.hi.y, b.hi.y), fmax_(a.hi.z, b.hi.z)}};
}
static bool finite3(v3 a) { return std::isfinite(a.x) && std::isfinite(a.y) && std::isfinite(a.z); }

static uint32_t expand10(uint32_t v) {
    // spread the low 10 bits of v to every third bit
    uint32_t r = 0;
    for (int b = 0; b < 10; ++b) r |= ((v >> b) & 1u) << (3 * b);
    return r;
}
static uint32_t quant10(float c, float lo, float ext) {
    float n = ext > 0.0f ? (c - lo) / ext : 0.0f;
    float q = fmin_(fmax_(n * 1024.0f, 0.0f), 1023.0f);
    return (uint32_t)q;
}
static v3 centroid(const Box& b) {
    return {(b.lo.x + b.hi.x) * 0.5f + 0.0f, (b.lo.y + b.hi.y) * 0.5f + 0.0f, (b.lo.z + b.hi.z) * 0.5f + 0.0f};
}
static uint32_t morton30(const Box& b, v3 cmin, v3 ext) {
    float cx = (b.lo.x + b.hi.x) * 0.5f, cy = (b.lo.y + b.hi.y) * 0.5f, cz = (b.lo.z + b.hi.z) * 0.5f;
    return (expand10(quant10(cx, cmin.x, ext.x)) << 2) | (expand10(quant10(cy, cmin.y, ext.y)) << 1) |
           expand10(quant10(cz, cmin.z, ext.z));
}

static const int32_t EMPTY_CHILD = (int32_t)0x80000001;

struct Tree {
    std::vector<float> nodes;      // 16 floats per node
    std::vector<uint32_t> morton;  // sorted
    std::vector<uint32_t> order;   // sorted primitive order
};

static void set_child(float* node, int slot, int32_t c) { memcpy(&node[12 + slot], &c, 4); }
static int32_t child(const float* node, int slot) {
    int32_t c;
    memcpy(&c, &node[12 + slot], 4);
    return c;
}
static void set_slot(float* node, int slot, const Box& b) {
    if (slot == 0) {
        node[0] = b.lo.x; node[1] = b.hi.x; node[2] = b.lo.y; node[3] = b.hi.y; node[8] = b.lo.z; node[9] = b.hi.z;
    } else {
        node[4] = b.lo.x; node[5] = b.hi.x; node[6] = b.lo.y; node[7] = b.hi.y; node[10] = b.lo.z; node[11] = b.hi.z;
    }
}
static Box get_slot(const float* node, int slot) {
    if (slot == 0) return {{node[0], node[2], node[8]}, {node[1], node[3], node[9]}};
    return {{node[4], node[6], node[10]}, {node[5], node[7], node[11]}};
}
// Centre of a BLAS root box (the union of the root node's two slots), as
// lbvh.cu root_centre.
static v3 root_centre(const float* root) {
    Box rb = unite(get_slot(root, 0), get_slot(root, 1));
    return {(rb.lo.x + rb.hi.x) * 0.5f + 0.0f, (rb.lo.y + rb.hi.y) * 0.5f + 0.0f, (rb.lo.z + rb.hi.z) * 0.5f + 0.0f};
}

// Karras delta: common prefix length of keys i and j, index-extended for equal keys.
static int kdelta(const std::vector<uint32_t>& k, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    if (k[i] != k[j]) return __builtin_clz(k[i] ^ k[j]);
    return 32 + __builtin_clz((uint32_t)i ^ (uint32_t)j);
}

// Builds a binary LBVH over `boxes` (leaf boxes in primitive order) with Morton keys
// from the centroid boxes `cboxes`. Leaves are ~sorted position.
static void build_tree(const std::vector<Box>& cboxes, const std::vector<Box>& leaf_boxes_in_prim_order, Tree& t) {
    int n = (int)cboxes.size();
    int m = std::max(n, 2) - 1;
    t.nodes.assign((size_t)m * 16, 0.0f);
    t.morton.assign(n, 0);
    t.order.assign(n, 0);
    if (n <= 1) {
        set_slot(&t.nodes[0], 0, empty_box());
        set_slot(&t.nodes[0], 1, empty_box());
        set_child(&t.nodes[0], 0, n == 1 ? ~0 : EMPTY_CHILD);
        set_child(&t.nodes[0], 1, EMPTY_CHILD);
        if (n == 1) {
            // One centroid: the centroid bounds have zero (or no finite) extent, so
            // every axis quantises to 0.
            set_slot(&t.nodes[0], 0, leaf_boxes_in_prim_order[0]);
            t.order[0] = 0;
            t.morton[0] = 0;
        }
        return;
    }
    // centroid bounds (finite centroids only)
    const float inf = std::numeric_limits<float>::infinity();
    v3 cmin = {inf, inf, inf}, cmax = {-inf, -inf, -inf};
    for (int i = 0; i < n; ++i) {
        v3 c = centroid(cboxes[i]);
        if (!finite3(c)) continue;
        cmin = {fmin_(c.x, cmin.x), fmin_(c.y, cmin.y), fmin_(c.z, cmin.z)};
        cmax = {fmax_(c.x, cmax.x), fmax_(c.y, cmax.y), fmax_(c.z, cmax.z)};
    }
    v3 ext = cmax - cmin;
    std::vector<uint32_t> keys(n);
    for (int i = 0; i < n; ++i) keys[i] = morton30(cboxes[i], cmin, ext);
    std::vector<uint32_t> idx(n);
    for (int i = 0; i < n; ++i) idx[i] = (uint32_t)i;
    std::stable_sort(idx.begin(), idx.end(), [&](uint32_t a, uint32_t b) { return keys[a] < keys[b]; });
    for (int i = 0; i < n; ++i) { t.order[i] = idx[i]; t.morton[i] = keys[idx[i]]; }
    const std::vector<uint32_t>& k = t.morton;
    std::vector<int32_t> parent_node(m, -1), parent_leaf(n, -1);
    std::vector<int8_t> side_node(m, 0), side_leaf(n, 0);
    for (int i = 0; i < m; ++i) {
        int d = (kdelta(k, n, i, i + 1) - kdelta(k, n, i, i - 1)) >= 0 ? 1 : -1;
        int dmin = kdelta(k, n, i, i - d);
        int lmax = 2;
        while (kdelta(k, n, i, i + lmax * d) > dmin) lmax <<= 1;
        int l = 0;
        for (int tt = lmax >> 1; tt >= 1; tt >>= 1)
            if (kdelta(k, n, i, i + (l + tt) * d) > dmin) l += tt;
        int j = i + l * d;
        int dnode = kdelta(k, n, i, j);
        int split = 0, step = l;
        do {
            step = (step + 1) >> 1;
            if (kdelta(k, n, i, i + (split + step) * d) > dnode) split += step;
        } while (step > 1);
        int gamma = i + split * d + std::min(d, 0);
        float* node = &t.nodes[(size_t)i * 16];
        if (std::min(i, j) == gamma) { set_child(node, 0, ~gamma); parent_leaf[gamma] = i; side_leaf[gamma] = 0; }
        else { set_child(node, 0, gamma); parent_node[gamma] = i; side_node[gamma] = 0; }
        if (std::max(i, j) == gamma + 1) { set_child(node, 1, ~(gamma + 1)); parent_leaf[gamma + 1] = i; side_leaf[gamma + 1] = 1; }
        else { set_child(node, 1, gamma + 1); parent_node[gamma + 1] = i; side_node[gamma + 1] = 1; }
    }
    // refit: post-order over the tree from the root
    std::vector<Box> nb(m);
    std::vector<std::pair<int, int>> st;   // (node, state)
    st.push_back({0, 0});
    while (!st.empty()) {
        auto [nd, s] = st.back();
        float* node = &t.nodes[(size_t)nd * 16];
        if (s == 0) {
            st.back().second = 1;
            for (int c = 1; c >= 0; --c) {
                int32_t ch = child(node, c);
                if (ch >= 0) st.push_back({ch, 0});
            }
        } else {
            st.pop_back();
            Box b[2];
            for (int c = 0; c < 2; ++c) {
                int32_t ch = child(node, c);
                b[c] = ch >= 0 ? nb[ch] : leaf_boxes_in_prim_order[t.order[~ch]];
                set_slot(node, c, b[c]);
            }
            nb[nd] = unite(b[0], b[1]);
        }
    }
}

// Breadth-first relayout (children of a level in their parents' order, left first).
static void bfs_relayout(Tree& t) {
    size_t m = t.nodes.size() / 16;
    std::vector<uint32_t> queue = {0}, newidx(m, 0);
    for (size_t h = 0; h < queue.size(); ++h) {
        const float* node = &t.nodes[(size_t)queue[h] * 16];
        for (int c = 0; c < 2; ++c) {
            int32_t ch = child(node, c);
            if (ch >= 0) { newidx[ch] = (uint32_t)queue.size(); queue.push_back((uint32_t)ch); }
        }
    }
    std::vector<float> out(t.nodes.size());
    for (size_t old = 0; old < m; ++old) {
        float* d = &out[(size_t)newidx[old] * 16];
        memcpy(d, &t.nodes[old * 16], 64);
        for (int c = 0; c < 2; ++c) {
            int32_t ch = child(&t.nodes[old * 16], c);
            if (ch >= 0) set_child(d, c, (int32_t)newidx[ch]);
        }
    }
    t.nodes.swap(out);
}

struct Blas {
    Tree tree;
    std::vector<float> tris;        // 12 floats per triangle, sorted order
    std::vector<luz_vertex> vertices;
    std::vector<uint32_t> indices;
    uint32_t prims = 0;
};

static Box tri_box(v3 a, v3 b, v3 c) {
    return {{fmin_(fmin_(a.x, b.x), c.x), fmin_(fmin_(a.y, b.y), c.y), fmin_(fmin_(a.z, b.z), c.z)},
            {fmax_(fmax_(a.x, b.x), c.x), fmax_(fmax_(a.y, b.y), c.y), fmax_(fmax_(a.z, b.z), c.z)}};
}
static float leaf_pad(float lo, float hi) { return fmax_(std::fabs(lo), std::fabs(hi)) * 0x1p-20f + 0x1p-100f; }
static float inst_pad(float lo, float hi) {
    float m = fmax_(std::fabs(lo), std::fabs(hi));
    return m * 0x1p-14f + (hi - lo) * 0x1p-16f + 0x1p-60f;
}

static v3 vpos(const Blas& b, uint32_t i) {
    const float* p = b.vertices[i].position;
    return {p[0], p[1], p[2]};
}

struct Instance {
    float w2o[12];
    float o2w[12];
    const Blas* blas;
    uint32_t custom, mask, input;
};

struct Tlas {
    Tree tree;
    std::vector<Instance> inst;    // leaf order
    std::vector<Instance> by_input;
};

// ---------------------------------------------------------------- watertight test
struct WtRay {
    v3 o;
    int kx, ky, kz;
    float sx, sy, sz;
};
static float comp(v3 v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }
static WtRay wt_setup(v3 o, v3 d) {
    WtRay r;
    r.o = o;
    float ax = std::fabs(d.x), ay = std::fabs(d.y), az = std::fabs(d.z);
    r.kz = ax >= ay ? (ax >= az ? 0 : 2) : (ay >= az ? 1 : 2);
    r.kx = r.kz == 2 ? 0 : r.kz + 1;
    r.ky = r.kx == 2 ? 0 : r.kx + 1;
    float dz = comp(d, r.kz);
    if (dz < 0.0f) std::swap(r.kx, r.ky);
    r.sx = comp(d, r.kx) / dz;
    r.sy = comp(d, r.ky) / dz;
    r.sz = 1.0f / dz;
    return r;
}
// S. Woop, C. Benthin, I. Wald, "Watertight Ray/Triangle Intersection", JCGT 2013;
// two-sided; edge functions recomputed in double when one is exactly zero.
static bool wt_test(const WtRay& r, v3 v0, v3 v1, v3 v2, float& t, float& U, float& V, float& W, float& det) {
    v3 A = v0 - r.o, B = v1 - r.o, C = v2 - r.o;
    float Ax = comp(A, r.kx) - r.sx * comp(A, r.kz), Ay = comp(A, r.ky) - r.sy * comp(A, r.kz);
    float Bx = comp(B, r.kx) - r.sx * comp(B, r.kz), By = comp(B, r.ky) - r.sy * comp(B, r.kz);
    float Cx = comp(C, r.kx) - r.sx * comp(C, r.kz), Cy = comp(C, r.ky) - r.sy * comp(C, r.kz);
    U = Cx * By - Cy * Bx;
    V = Ax * Cy - Ay * Cx;
    W = Bx * Ay - By * Ax;
    if (U == 0.0f || V == 0.0f || W == 0.0f) {
        U = (float)((double)Cx * (double)By - (double)Cy * (double)Bx);
        V = (float)((double)Ax * (double)Cy - (double)Ay * (double)Cx);
        W = (float)((double)Bx * (double)Ay - (double)By * (double)Ax);
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
    det = U + V + W;
    if (det == 0.0f) return false;
    float Az = r.sz * comp(A, r.kz), Bz = r.sz * comp(B, r.kz), Cz = r.sz * comp(C, r.kz);
    float T = U * Az + V * Bz + W * Cz;
    t = T / det;
    return true;
}

// ---------------------------------------------------------------- traversal
static v3 safe_inv(v3 d) {
    auto f = [](float x) { return std::fabs(x) > 1e-20f ? x : std::copysign(1e-20f, x); };
    return {1.0f / f(d.x), 1.0f / f(d.y), 1.0f / f(d.z)};
}
// Conservative slab test (interval widened by a relative 2^-18).
static bool slab(const Box& b, v3 o, v3 id, float tmin, float tmax, float& tn_out) {
    float tx0 = (b.lo.x - o.x) * id.x, tx1 = (b.hi.x - o.x) * id.x;
    float ty0 = (b.lo.y - o.y) * id.y, ty1 = (b.hi.y - o.y) * id.y;
    float tz0 = (b.lo.z - o.z) * id.z, tz1 = (b.hi.z - o.z) * id.z;
    float tn = std::fmax(std::fmax(std::fmin(tx0, tx1), std::fmin(ty0, ty1)), std::fmax(std::fmin(tz0, tz1), tmin));
    float tf = std::fmin(std::fmin(std::fmax(tx0, tx1), std::fmax(ty0, ty1)), std::fmin(std::fmax(tz0, tz1), tmax));
    tn_out = tn;
    const float e = 0x1p-18f;
    return tn - std::fabs(tn) * e <= tf + std::fabs(tf) * e;
}

struct Hit {
    float t;
    uint32_t input, prim, custom;
    float b0, b1, b2;
};

// Per-hit alpha test of the primary rays (opaque.frag:29-34 discard).
struct AlphaTest {
    virtual bool accept(uint32_t input, uint32_t custom, uint32_t prim, float b0, float b1, float b2) const = 0;
    virtual ~AlphaTest() {}
};

// Object-space closest/any hit inside one BLAS. Returns true if any accepted hit.
template <bool kClosest>
static bool trace_blas(const Blas& b, v3 o, v3 d, float tmin, float& tmax, uint32_t input, uint32_t custom,
                       bool& found, Hit* hit, uint64_t& best_key, const AlphaTest* alpha = nullptr) {
    if (b.prims == 0) return false;
    v3 id = safe_inv(d);
    WtRay wt = wt_setup(o, d);
    int32_t stack[256];
    int sp = 0;
    stack[sp++] = 0;
    bool any = false;
    while (sp) {
        int32_t nd = stack[--sp];
        const float* node = &b.tree.nodes[(size_t)nd * 16];
        for (int c = 0; c < 2; ++c) {
            int32_t ch = child(node, c);
            if (ch == EMPTY_CHILD) continue;
            float tn;
            if (!slab(get_slot(node, c), o, id, tmin, tmax, tn)) continue;
            if (ch >= 0) { stack[sp++] = ch; continue; }
            const float* tr = &b.tris[(size_t)(~ch) * 12];
            float t, U, V, W, det;
            if (!wt_test(wt, {tr[0], tr[1], tr[2]}, {tr[4], tr[5], tr[6]}, {tr[8], tr[9], tr[10]}, t, U, V, W, det)) continue;
            if (!(t >= tmin && t <= tmax)) continue;
            if (!kClosest) return true;
            uint32_t prim;
            memcpy(&prim, &tr[3], 4);
            uint64_t key = ((uint64_t)input << 32) | prim;
            if ((!found || t < tmax || key < best_key) &&
                (!alpha || alpha->accept(input, custom, prim, U / det, V / det, W / det))) {
                found = true;
                any = true;
                tmax = t;
                best_key = key;
                hit->t = t; hit->input = input; hit->prim = prim; hit->custom = custom;
                hit->b0 = U / det; hit->b1 = V / det; hit->b2 = W / det;
            }
        }
    }
    return any;
}

static bool ray_ok(v3 o, v3 d, float tmin, float tmax) {
    if (!finite3(o) || !finite3(d) || !(tmin <= tmax)) return false;
    if (d.x == 0.0f && d.y == 0.0f && d.z == 0.0f) return false;
    return true;
}

// skip[custom]: 1 = instance never hit by closest-hit rays, 2 = every hit alpha-tested.
template <bool kClosest>
static bool trace(const Tlas& T, v3 o, v3 d, float tmin, float tmax, const uint8_t* skip, uint32_t skip_n, Hit* hit,
                  const AlphaTest* alpha = nullptr) {
    if (T.inst.empty() || !ray_ok(o, d, tmin, tmax)) return false;
    v3 id = safe_inv(d);
    int32_t stack[256];
    int sp = 0;
    stack[sp++] = 0;
    bool found = false;
    uint64_t best_key = ~0ull;
    while (sp) {
        int32_t nd = stack[--sp];
        const float* node = &T.tree.nodes[(size_t)nd * 16];
        for (int c = 0; c < 2; ++c) {
            int32_t ch = child(node, c);
            if (ch == EMPTY_CHILD) continue;
            float tn;
            if (!slab(get_slot(node, c), o, id, tmin, tmax, tn)) continue;
            if (ch >= 0) { stack[sp++] = ch; continue; }
            const Instance& I = T.inst[~ch];
            // the rays' cull mask is 0xFF (light.frag:100,126): an instance whose mask
            // shares no bit with it is invisible
            if ((I.mask & 0xFFu) == 0) continue;
            const bool tested = kClosest && skip && I.custom < skip_n && skip[I.custom] == 2;
            if (kClosest && skip && I.custom < skip_n && skip[I.custom] == 1) continue;
            v3 oo = xpoint(I.w2o, o), od = xdir(I.w2o, d);
            bool h = trace_blas<kClosest>(*I.blas, oo, od, tmin, tmax, I.input, I.custom, found, hit, best_key,
                                          tested ? alpha : nullptr);
            if (h && !kClosest) return true;
        }
    }
    return found;
}

// Every triangle of every instance, no BVH: an independent any-hit oracle.
static bool trace_bruteforce(const Tlas& T, v3 o, v3 d, float tmin, float tmax) {
    if (!ray_ok(o, d, tmin, tmax)) return false;
    for (const Instance& I : T.by_input) {
        if ((I.mask & 0xFFu) == 0) continue;   // invisible to the 0xFF cull mask
        const Blas& b = *I.blas;
        v3 oo = xpoint(I.w2o, o), od = xdir(I.w2o, d);
        WtRay wt = wt_setup(oo, od);
        for (uint32_t p = 0; p < b.prims; ++p) {
            v3 a = vpos(b, b.indices[3 * p]), bb = vpos(b, b.indices[3 * p + 1]), c = vpos(b, b.indices[3 * p + 2]);
            float t, U, V, W, det;
            if (wt_test(wt, a, bb, c, t, U, V, W, det) && t >= tmin && t <= tmax) return true;
        }
    }
    return false;
}

// ---------------------------------------------------------------- ray generation
// EvaluateShadow (light.frag:137-146) + TraceShadowRay (light.frag:86-109), one sample.
static void ShadowRay(const luz_light& L, v3 p, v3 N, v3 cam, float rx, float ry, v3& O, v3& dir, float& tMax) {
    v3 lpos = {L.position[0], L.position[1], L.position[2]};
    v3 ldir = {L.direction[0], L.direction[1], L.direction[2]};
    v3 Ln = normalize(lpos - p);                                   // light.frag:194-195
    if (L.type == LUZ_LIGHT_DIRECTIONAL) Ln = normalize(-ldir);    // light.frag:197-198
    float shadowBias = fmax_(length(p - cam) * 0.01f, 0.05f);      // light.frag:138
    v3 shadowOrigin = p + N * shadowBias;                          // light.frag:139
    float dist = length(lpos - p);                                 // light.frag:140
    v3 Lv = L.type == LUZ_LIGHT_DIRECTIONAL ? (ldir * dot(ldir, Ln)) * dist : Ln * dist;   // 143 / 145
    v3 lightTangent = normalize(cross(Lv, v3{0.0f, 1.0f, 0.0f}));  // light.frag:90
    v3 lightBitangent = normalize(cross(lightTangent, Lv));       // light.frag:91
    float dx, dy;
    DiskSample(rx, ry, L.radius, &dx, &dy);                        // light.frag:96
    tMax = length(Lv);                                             // light.frag:97
    dir = normalize((Lv + dx * lightTangent) + dy * lightBitangent);   // light.frag:98
    O = shadowOrigin;
}
// light.frag:229-231 origin + TraceAORays (light.frag:111-135), one sample.
static void AORay(v3 p, v3 N, v3 cam, float rx, float ry, v3& O, v3& dir) {
    float shadowBias = length(p - cam) * 0.01f;
    O = p + N * shadowBias;
    v3 tangent = std::fabs(N.z) > 0.5f ? v3{0.0f, -N.z, N.y} : v3{-N.y, N.x, 0.0f};
    v3 bitangent = cross(N, tangent);
    v3 h = HemisphereSample(rx, ry);
    dir = (tangent * h.x + bitangent * h.y) + N * h.z;
}

static void parallel_for(uint32_t n, int threads, const std::function<void(uint32_t, uint32_t)>& fn) {
    if (threads <= 1 || n < 2) { fn(0, n); return; }
    std::atomic<uint32_t> next{0};
    const uint32_t chunk = std::max(1u, n / (uint32_t)(threads * 16));
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; ++t)
        pool.emplace_back([&]() {
            for (;;) {
                uint32_t b = next.fetch_add(chunk);
                if (b >= n) break;
                fn(b, std::min(n, b + chunk));
            }
        });
    for (auto& th : pool) th.join();
}

static uint32_t unorm8(float x) { return (uint32_t)(clamp01(x) * 255.0f + 0.5f); }
static uint32_t pack8(float r, float g, float b, float a) { return unorm8(r) | (unorm8(g) << 8) | (unorm8(b) << 16) | (unorm8(a) << 24); }

// ---------------------------------------------------------------- light pass
// light.frag:17-49 in precision T.
template <typename T> static T DistributionGGX(vec3<T> N, vec3<T> H, T roughness, T pi) {
    T a = roughness * roughness;
    T a2 = a * a;
    T NdotH = tmax_(dot(N, H), T(0));
    T NdotH2 = NdotH * NdotH;
    T nom = a2;
    T denom = (NdotH2 * (a2 - T(1)) + T(1));
    denom = pi * denom * denom;
    return nom / denom;
}
template <typename T> static T GeometrySchlickGGX(T NdotV, T roughness) {
    T r = (roughness + T(1));
    T k = (r * r) / T(8);
    T nom = NdotV;
    T denom = NdotV * (T(1) - k) + k;
    return nom / denom;
}
template <typename T> static T GeometrySmith(vec3<T> N, vec3<T> V, vec3<T> L, T roughness) {
    T NdotV = tmax_(dot(N, V), T(0));
    T NdotL = tmax_(dot(N, L), T(0));
    T ggx2 = GeometrySchlickGGX(NdotV, roughness);
    T ggx1 = GeometrySchlickGGX(NdotL, roughness);
    return ggx1 * ggx2;
}
template <typename T> static vec3<T> FresnelSchlick(T cosTheta, vec3<T> F0) {
    T x = tclamp01(T(1) - cosTheta);
    T x2 = x * x;
    T p5 = (x2 * x2) * x;   // pow(x, 5.0)
    return F0 + (vec3<T>{T(1), T(1), T(1)} - F0) * p5;
}

// ---------------------------------------------------------------- shadow maps
// The shadow-map pass (shadowMap.vert/.geom/.frag) as a depth rasteriser and the
// lookups of EvaluateShadow's map branch (light.frag:147-165), restated with the same
// single-precision steps as the device: clip to w >= 1e-5 for cube faces, pixel-centre
// edge functions with a top-left rule, front faces (counter-clockwise) culled, depth
// LESS from 1.0; bilinear lookups (repeat for 2D maps, clamp per cube face).
struct OShadow {
    const float* map = nullptr;
    float vp0[16];
    float pos[3];
    float zfar = 1.0f;
    uint32_t faces = 0, res = 0;
};
static std::vector<OShadow> g_shadow;

static uint32_t sm_wrap(float f, uint32_t n) {
    float m = std::fmod(f, (float)n);
    if (m < 0.0f) m += (float)n;
    uint32_t i = (uint32_t)m;
    return i < n ? i : 0u;
}
static uint32_t sm_clamp(float f, uint32_t n) {
    if (!(f > 0.0f)) return 0u;
    if (f >= (float)(n - 1)) return n - 1;
    return (uint32_t)f;
}
static float sm_sample(const float* face, uint32_t res, float u, float v, bool repeat) {
    float x = u * (float)res - 0.5f, y = v * (float)res - 0.5f;
    if (!std::isfinite(x)) x = 0.0f;
    if (!std::isfinite(y)) y = 0.0f;
    float fx = std::floor(x), fy = std::floor(y);
    float ax = x - fx, ay = y - fy, bx = 1.0f - ax, by = 1.0f - ay;
    uint32_t x0, x1, y0, y1;
    if (repeat) {
        x0 = sm_wrap(fx, res); y0 = sm_wrap(fy, res);
        x1 = x0 + 1 == res ? 0u : x0 + 1; y1 = y0 + 1 == res ? 0u : y0 + 1;
    } else {
        x0 = sm_clamp(fx, res); y0 = sm_clamp(fy, res); x1 = sm_clamp(fx + 1.0f, res); y1 = sm_clamp(fy + 1.0f, res);
    }
    float c00 = face[(size_t)y0 * res + x0], c10 = face[(size_t)y0 * res + x1];
    float c01 = face[(size_t)y1 * res + x0], c11 = face[(size_t)y1 * res + x1];
    return (c00 * bx + c10 * ax) * by + (c01 * bx + c11 * ax) * ay;
}
static float shadow_map_factor(const OShadow& S, v3 frag, v3 origin) {
    if (S.faces == 6) {
        v3 d = frag - v3{S.pos[0], S.pos[1], S.pos[2]};
        float ax = std::fabs(d.x), ay = std::fabs(d.y), az = std::fabs(d.z), ma, sc, tc;
        uint32_t face;
        if (ax >= ay && ax >= az) { face = d.x >= 0.0f ? 0u : 1u; ma = ax; sc = d.x >= 0.0f ? -d.z : d.z; tc = -d.y; }
        else if (ay >= az) { face = d.y >= 0.0f ? 2u : 3u; ma = ay; sc = d.x; tc = d.y >= 0.0f ? d.z : -d.z; }
        else { face = d.z >= 0.0f ? 4u : 5u; ma = az; sc = d.z >= 0.0f ? d.x : -d.x; tc = -d.y; }
        float s_, t_;
        if (ma == 0.0f) { face = 0; s_ = t_ = 0.5f; }
        else { s_ = 0.5f * (sc / ma + 1.0f); t_ = 0.5f * (tc / ma + 1.0f); }
        float depth = sm_sample(S.map + (size_t)face * S.res * S.res, S.res, s_, t_, false);
        return length(d) - 0.05f >= depth * S.zfar ? 1.0f : 0.0f;
    }
    float p4[4] = {origin.x, origin.y, origin.z, 1.0f}, fl[4];
    mat4_vec4(S.vp0, p4, fl);
    float depth = sm_sample(S.map, S.res, fl[0] * 0.5f + 0.5f, fl[1] * 0.5f + 0.5f, true);
    return fl[2] >= depth ? 1.0f : 0.0f;
}

struct RV {
    float x, y, z, iw, wx, wy, wz;
};
static float r_edge(const RV& a, const RV& b, float px, float py) {
    return (b.x - a.x) * (py - a.y) - (b.y - a.y) * (px - a.x);
}
static bool r_top_left(const RV& a, const RV& b) {
    float dy = b.y - a.y, dx = b.x - a.x;
    return dy > 0.0f || (dy == 0.0f && dx < 0.0f);
}
static void r_tri(const RV* v, uint32_t faces, uint32_t res, const float light[3], float inv_zfar, uint32_t* face_map) {
    float sarea = (v[0].x * v[1].y - v[1].x * v[0].y) + (v[1].x * v[2].y - v[2].x * v[1].y) + (v[2].x * v[0].y - v[0].x * v[2].y);
    float a = -0.5f * sarea;
    if (!(a < 0.0f)) return;
    float area2 = (v[1].x - v[0].x) * (v[2].y - v[0].y) - (v[1].y - v[0].y) * (v[2].x - v[0].x);
    if (!(area2 > 0.0f)) return;
    float mnx = std::fmin(std::fmin(v[0].x, v[1].x), v[2].x), mxx = std::fmax(std::fmax(v[0].x, v[1].x), v[2].x);
    float mny = std::fmin(std::fmin(v[0].y, v[1].y), v[2].y), mxy = std::fmax(std::fmax(v[0].y, v[1].y), v[2].y);
    float lx = std::fmax(std::floor(mnx - 0.5f), 0.0f), ly = std::fmax(std::floor(mny - 0.5f), 0.0f);
    float hx = std::fmin(std::ceil(mxx - 0.5f), (float)res - 1.0f), hy = std::fmin(std::ceil(mxy - 0.5f), (float)res - 1.0f);
    if (!(lx <= hx && ly <= hy)) return;
    for (uint32_t py = (uint32_t)ly; py <= (uint32_t)hy; ++py)
        for (uint32_t px = (uint32_t)lx; px <= (uint32_t)hx; ++px) {
            float sx = (float)px + 0.5f, sy = (float)py + 0.5f;
            float e0 = r_edge(v[1], v[2], sx, sy), e1 = r_edge(v[2], v[0], sx, sy), e2 = r_edge(v[0], v[1], sx, sy);
            bool in0 = e0 > 0.0f || (e0 == 0.0f && r_top_left(v[1], v[2]));
            bool in1 = e1 > 0.0f || (e1 == 0.0f && r_top_left(v[2], v[0]));
            bool in2 = e2 > 0.0f || (e2 == 0.0f && r_top_left(v[0], v[1]));
            if (!(in0 && in1 && in2)) continue;
            float b0 = e0 / area2, b1 = e1 / area2, b2 = e2 / area2, depth;
            if (faces == 6) {
                float w0 = b0 * v[0].iw, w1 = b1 * v[1].iw, w2 = b2 * v[2].iw;
                float iw = (w0 + w1) + w2;
                float fx = ((w0 * v[0].wx + w1 * v[1].wx) + w2 * v[2].wx) / iw;
                float fy = ((w0 * v[0].wy + w1 * v[1].wy) + w2 * v[2].wy) / iw;
                float fz = ((w0 * v[0].wz + w1 * v[1].wz) + w2 * v[2].wz) / iw;
                float dx = light[0] - fx, dy = light[1] - fy, dz = light[2] - fz;
                depth = std::sqrt(dx * dx + dy * dy + dz * dz) * inv_zfar;
            } else {
                depth = (b0 * v[0].z + b1 * v[1].z) + b2 * v[2].z;
            }
            if (!(depth >= 0.0f && depth < 1.0f)) continue;
            uint32_t bits;
            memcpy(&bits, &depth, 4);
            uint32_t& m = face_map[(size_t)py * res + px];
            if (bits < m) m = bits;
        }
}
static RV r_screen(const float c[4], const float w[3], uint32_t res) {
    float iw = 1.0f / c[3];
    return RV{(c[0] * iw * 0.5f + 0.5f) * (float)res, (c[1] * iw * 0.5f + 0.5f) * (float)res, c[2] * iw, iw, w[0], w[1], w[2]};
}

struct Planes {
    const uint32_t* albedo;
    const float* normal;
    const uint32_t* material;
    const uint32_t* emission;
    const float* depth;
    const uint32_t* shadow_bits;
    const uint32_t* ao_bits;
    const float* ao_override;
};

// light.frag:194-198: the light vector L.
template <typename T>
static vec3<T> light_vector(const luz_light& lt, vec3<T> p) {
    vec3<T> lpos = {(T)lt.position[0], (T)lt.position[1], (T)lt.position[2]};
    vec3<T> ldir = {(T)lt.direction[0], (T)lt.direction[1], (T)lt.direction[2]};
    vec3<T> L = normalize(lpos - p);
    if (lt.type == LUZ_LIGHT_DIRECTIONAL) L = normalize(-ldir);
    return L;
}
// light.frag:199-208: 1 (directional), 1/d^2 (point), 1/d^2 times the cone term (spot).
template <typename T>
static T light_attenuation(const luz_light& lt, vec3<T> p, vec3<T> L) {
    vec3<T> lpos = {(T)lt.position[0], (T)lt.position[1], (T)lt.position[2]};
    vec3<T> ldir = {(T)lt.direction[0], (T)lt.direction[1], (T)lt.direction[2]};
    T attenuation = T(1);
    if (lt.type == LUZ_LIGHT_SPOT) {
        T dist = length(lpos - p);
        attenuation = T(1) / (dist * dist);
        T theta = dot(L, normalize(-ldir));
        T epsilon = (T)lt.inner_angle - (T)lt.outer_angle;
        attenuation *= tclamp01((theta - (T)lt.outer_angle) / epsilon);
    } else if (lt.type == LUZ_LIGHT_POINT) {
        T dist = length(lpos - p);
        attenuation = T(1) / (dist * dist);
    }
    return attenuation;
}
// The light pass's term of this light cannot depend on its shadow factor: zero
// weight max(dot(N, L), 0) or zero unshadowed radiance in every channel
// (light.frag:209-226; the device's shadow_has_no_effect).
static bool shadow_has_no_effect(const luz_light& lt, v3 p, v3 N, v3 L) {
    if (!(dot(N, L) > 0.0f)) return true;
    const float a = light_attenuation<float>(lt, p, L);
    const v3 c = (v3{lt.color[0], lt.color[1], lt.color[2]} * lt.intensity) * a;
    return c.x == 0.0f && c.y == 0.0f && c.z == 0.0f;
}

template <typename T>
static void light_pixel(const luz_scene& S, const luz_light* lights, uint32_t nl, const std::vector<uint32_t>& first_slot,
                        const Planes& P, uint32_t W, uint32_t H, uint32_t words, uint32_t ao_n, uint32_t pix,
                        T out[4], const std::vector<T>& lut, T* split = nullptr) {
    const T pi = std::is_same<T, float>::value ? (T)PI_F : (T)3.14159265359;
    vec3<T> N = {(T)P.normal[4 * pix], (T)P.normal[4 * pix + 1], (T)P.normal[4 * pix + 2]};
    vec3<T> amb = {(T)S.ambient_light_color[0], (T)S.ambient_light_color[1], (T)S.ambient_light_color[2]};
    if (length(N) == T(0)) {   // light.frag:178-181
        vec3<T> c = amb * (T)S.ambient_light_intensity;
        out[0] = c.x; out[1] = c.y; out[2] = c.z; out[3] = T(1);
        if (split)
            for (int k = 0; k < 8; ++k) split[k] = T(0);
        return;
    }
    uint32_t a8 = P.albedo[pix], m8 = P.material[pix], e8 = P.emission[pix];
    vec3<T> albedo = {lut[a8 & 0xFF], lut[(a8 >> 8) & 0xFF], lut[(a8 >> 16) & 0xFF]};     // light.frag:172
    T roughness = (T)(m8 & 0xFF) / (T)255, metallic = (T)((m8 >> 8) & 0xFF) / (T)255;      // light.frag:183-185
    T occlusion = (T)((m8 >> 16) & 0xFF) / (T)255;
    vec3<T> emission = {(T)(e8 & 0xFF) / (T)255, (T)((e8 >> 8) & 0xFF) / (T)255, (T)((e8 >> 16) & 0xFF) / (T)255};
    uint32_t x = pix % W, y = pix / W;
    vec3<T> fragPos;
    {
        T u = ((T)x + (T)0.5) / (T)W, v = ((T)y + (T)0.5) / (T)H;
        T clip[4] = {u * T(2) - T(1), v * T(2) - T(1), (T)P.depth[pix], T(1)};
        T view[4], world[4];
        for (int r = 0; r < 4; ++r) view[r] = (T)S.inverse_proj[r] * clip[0] + (T)S.inverse_proj[4 + r] * clip[1] + (T)S.inverse_proj[8 + r] * clip[2] + (T)S.inverse_proj[12 + r] * clip[3];
        T w = view[3];
        for (int k = 0; k < 4; ++k) view[k] = view[k] / w;
        for (int r = 0; r < 4; ++r) world[r] = (T)S.inverse_view[r] * view[0] + (T)S.inverse_view[4 + r] * view[1] + (T)S.inverse_view[8 + r] * view[2] + (T)S.inverse_view[12 + r] * view[3];
        fragPos = {world[0], world[1], world[2]};
    }
    vec3<T> cam = {(T)S.cam_pos[0], (T)S.cam_pos[1], (T)S.cam_pos[2]};
    vec3<T> V = normalize(cam - fragPos);                                                   // light.frag:187
    vec3<T> F0 = vec3<T>{(T)0.04f, (T)0.04f, (T)0.04f} * (T(1) - metallic) + albedo * metallic;   // 188-189
    vec3<T> Lo = {T(0), T(0), T(0)};
    vec3<T> Lu = {T(0), T(0), T(0)};   // the same sum with every shadow factor 0 (for `split`)
    uint32_t hits_all = 0, slots_all = 0;   // occluded shadow samples over all lights (for `split`)
    T shadow_sum = T(0);
    for (uint32_t i = 0; i < nl; ++i) {                                                    // light.frag:192
        const luz_light& lt = lights[i];
        vec3<T> L = light_vector<T>(lt, fragPos);                                           // light.frag:194-198
        T attenuation = light_attenuation<T>(lt, fragPos, L);                                // light.frag:199-208
        T shadow = T(1);                                                                     // light.frag:166-167
        if (S.shadow_type == LUZ_SHADOW_RAYTRACING) {
            int ns = lt.num_shadow_samples;
            if (ns <= 0) shadow = T(0);                                                      // light.frag:87-89
            else {
                uint32_t hits = 0;
                for (int s = 0; s < ns; ++s)
                    hits += (P.shadow_bits[(size_t)(first_slot[i] + s) * words + (pix >> 5)] >> (pix & 31)) & 1u;
                shadow = (T)hits / (T)ns;                                                    // light.frag:108
                hits_all += hits;
                slots_all += (uint32_t)ns;
            }
        } else if (S.shadow_type == LUZ_SHADOW_MAP && i < g_shadow.size() && g_shadow[i].faces) {   // 147-164
            v3 fp = {(float)fragPos.x, (float)fragPos.y, (float)fragPos.z};
            v3 nf = {(float)N.x, (float)N.y, (float)N.z};
            v3 camf = {S.cam_pos[0], S.cam_pos[1], S.cam_pos[2]};
            v3 origin = fp + nf * fmax_(length(fp - camf) * 0.01f, 0.05f);
            shadow = (T)shadow_map_factor(g_shadow[i], fp, origin);
        }
        shadow_sum += shadow;
        vec3<T> color = {(T)lt.color[0], (T)lt.color[1], (T)lt.color[2]};
        vec3<T> radiance = ((color * (T)lt.intensity) * attenuation) * (T(1) - shadow);    // light.frag:210
        vec3<T> Hh = normalize(V + L);
        T NDF = DistributionGGX(N, Hh, roughness, pi);
        T G = GeometrySmith(N, V, L, roughness);
        vec3<T> F = FresnelSchlick(tclamp01(dot(Hh, V)), F0);
        vec3<T> num = (NDF * G) * F;
        T denom = (T(4) * tmax_(dot(N, V), T(0))) * tmax_(dot(N, L), T(0)) + (T)0.0001f;
        vec3<T> spec = num / denom;
        vec3<T> kD = (vec3<T>{T(1), T(1), T(1)} - F) * (T(1) - metallic);
        T NdotL = tmax_(dot(N, L), T(0));
        Lo = Lo + ((kD * albedo) / pi + spec) * radiance * NdotL;                           // light.frag:226
        if (split) Lu = Lu + ((kD * albedo) / pi + spec) * ((color * (T)lt.intensity) * attenuation) * NdotL;
    }
    T ao;
    if (P.ao_override) ao = (T)P.ao_override[pix];
    else if (ao_n == 0) ao = T(1);                                                          // light.frag:112-114
    else {
        uint32_t misses = 0;
        for (uint32_t s = 0; s < ao_n; ++s) misses += (P.ao_bits[(size_t)s * words + (pix >> 5)] >> (pix & 31)) & 1u;
        ao = (T)misses / (T)ao_n;                                                            // light.frag:134
    }
    if (split) {   // S, AO, U, unoccluded fraction of all shadow samples
        T lit_fraction = T(1);
        if (S.shadow_type == LUZ_SHADOW_RAYTRACING) {
            if (slots_all) lit_fraction = T(1) - (T)hits_all / (T)slots_all;
        } else if (nl) {
            lit_fraction = T(1) - shadow_sum / (T)nl;
        }
        split[0] = Lo.x; split[1] = Lo.y; split[2] = Lo.z; split[3] = ao;
        split[4] = Lu.x; split[5] = Lu.y; split[6] = Lu.z; split[7] = lit_fraction;
    }
    vec3<T> ambient = (((amb * (T)S.ambient_light_intensity) * albedo) * occlusion) * ao;   // light.frag:232
    vec3<T> c = (ambient + Lo) + emission;                                                  // light.frag:233
    out[0] = c.x; out[1] = c.y; out[2] = c.z; out[3] = T(1);
}

}  // namespace oracle

using namespace oracle;

struct oracle_blas { Blas b; };
struct oracle_tlas { Tlas t; };

extern "C" {

int oracle_blas_build(const void* vertices, uint32_t nv, uint32_t stride, const uint32_t* idx, uint32_t ni,
                      oracle_blas** out) {
    if (!out || ni % 3 || stride < 12) return LUZ_ERR_INVALID;
    for (uint32_t k = 0; k < ni; ++k)
        if (idx[k] >= nv) return LUZ_ERR_INVALID;
    oracle_blas* ob = new oracle_blas();
    Blas& b = ob->b;
    b.vertices.resize(nv);
    for (uint32_t v = 0; v < nv; ++v) {
        memset(&b.vertices[v], 0, sizeof(luz_vertex));
        memcpy(&b.vertices[v], (const char*)vertices + (size_t)v * stride, std::min<uint32_t>(stride, sizeof(luz_vertex)));
    }
    b.indices.assign(idx, idx + ni);
    b.prims = ni / 3;
    std::vector<Box> boxes(b.prims), leaf(b.prims);
    for (uint32_t p = 0; p < b.prims; ++p) {
        boxes[p] = tri_box(vpos(b, idx[3 * p]), vpos(b, idx[3 * p + 1]), vpos(b, idx[3 * p + 2]));
        Box l = boxes[p];
        float px = leaf_pad(l.lo.x, l.hi.x), py = leaf_pad(l.lo.y, l.hi.y), pz = leaf_pad(l.lo.z, l.hi.z);
        leaf[p] = {{l.lo.x - px, l.lo.y - py, l.lo.z - pz}, {l.hi.x + px, l.hi.y + py, l.hi.z + pz}};
    }
    build_tree(boxes, leaf, b.tree);
    b.tris.assign((size_t)b.prims * 12, 0.0f);
    for (uint32_t j = 0; j < b.prims; ++j) {
        uint32_t p = b.tree.order[j];
        float* t = &b.tris[(size_t)j * 12];
        for (int k = 0; k < 3; ++k) {
            v3 v = vpos(b, idx[3 * p + k]);
            t[4 * k] = v.x; t[4 * k + 1] = v.y; t[4 * k + 2] = v.z;
        }
        int32_t pi = (int32_t)p;
        memcpy(&t[3], &pi, 4);
    }
    if (b.prims) {
        // Bounding sphere about the root box centre: the largest squared vertex
        // distance, as float bits in the root's spare word (lbvh.cu blas_radius_kernel).
        float* root = b.tree.nodes.data();
        v3 c = root_centre(root);
        uint32_t r2 = 0;
        for (size_t k = 0; k < (size_t)b.prims * 3; ++k) {
            const float* v = &b.tris[4 * k];
            float dx = v[0] - c.x, dy = v[1] - c.y, dz = v[2] - c.z;
            float d2 = dx * dx + dy * dy + dz * dz;
            uint32_t u;
            memcpy(&u, &d2, 4);
            r2 = std::max(r2, u);
        }
        memcpy(&root[14], &r2, 4);
    }
    *out = ob;
    return LUZ_OK;
}

uint32_t oracle_blas_prims(const oracle_blas* b) { return b ? b->b.prims : 0; }

void oracle_blas_get(const oracle_blas* ob, float* nodes, float* tris, uint32_t* morton, uint32_t* order) {
    const Blas& b = ob->b;
    if (nodes) memcpy(nodes, b.tree.nodes.data(), b.tree.nodes.size() * 4);
    if (tris) memcpy(tris, b.tris.data(), b.tris.size() * 4);
    if (morton) memcpy(morton, b.tree.morton.data(), b.tree.morton.size() * 4);
    if (order) memcpy(order, b.tree.order.data(), b.tree.order.size() * 4);
}

void oracle_blas_destroy(oracle_blas* b) { delete b; }

int oracle_tlas_build(const oracle_blas* const* blas, const float* transforms, const uint32_t* custom,
                      const uint32_t* mask, uint32_t n, oracle_tlas** out) {
    if (!out) return LUZ_ERR_INVALID;
    oracle_tlas* ot = new oracle_tlas();
    Tlas& T = ot->t;
    T.by_input.resize(n);
    std::vector<Box> boxes(n);
    for (uint32_t i = 0; i < n; ++i) {
        Instance& I = T.by_input[i];
        memcpy(I.o2w, transforms + 12 * (size_t)i, 48);
        affine_inverse(I.o2w, I.w2o);
        I.blas = &blas[i]->b;
        I.custom = custom ? custom[i] : i;
        I.mask = mask ? mask[i] : 0xFFu;
        I.input = i;
        Box wb = empty_box();
        if (I.blas->prims > 0) {
            const float* root = I.blas->tree.nodes.data();
            Box rb = unite(get_slot(root, 0), get_slot(root, 1));
            for (int c = 0; c < 8; ++c) {
                v3 p = {(c & 1) ? rb.hi.x : rb.lo.x, (c & 2) ? rb.hi.y : rb.lo.y, (c & 4) ? rb.hi.z : rb.lo.z};
                v3 w = xpoint(I.o2w, p);
                wb.lo = {fmin_(wb.lo.x, w.x), fmin_(wb.lo.y, w.y), fmin_(wb.lo.z, w.z)};
                wb.hi = {fmax_(wb.hi.x, w.x), fmax_(wb.hi.y, w.y), fmax_(wb.hi.z, w.z)};
            }
            // Clip with the axis box of the transformed bounding sphere (lbvh.cu
            // tlas_instance_kernel): extent r * |row_a(M)| along world axis a.
            uint32_t r2;
            memcpy(&r2, &root[14], 4);
            if (r2 < 0x7F800000u) {
                v3 cw = xpoint(I.o2w, root_centre(root));
                float r2f;
                memcpy(&r2f, &r2, 4);
                float r = std::sqrt(r2f);
                const float* m = I.o2w;
                float ex = r * std::sqrt(m[0] * m[0] + m[1] * m[1] + m[2] * m[2]);
                float ey = r * std::sqrt(m[4] * m[4] + m[5] * m[5] + m[6] * m[6]);
                float ez = r * std::sqrt(m[8] * m[8] + m[9] * m[9] + m[10] * m[10]);
                wb.lo = {fmax_(wb.lo.x, cw.x - ex), fmax_(wb.lo.y, cw.y - ey), fmax_(wb.lo.z, cw.z - ez)};
                wb.hi = {fmin_(wb.hi.x, cw.x + ex), fmin_(wb.hi.y, cw.y + ey), fmin_(wb.hi.z, cw.z + ez)};
            }
            float px = inst_pad(wb.lo.x, wb.hi.x), py = inst_pad(wb.lo.y, wb.hi.y), pz = inst_pad(wb.lo.z, wb.hi.z);
            wb = {{wb.lo.x - px, wb.lo.y - py, wb.lo.z - pz}, {wb.hi.x + px, wb.hi.y + py, wb.hi.z + pz}};
        }
        boxes[i] = wb;
    }
    if (n) {
        build_tree(boxes, boxes, T.tree);
        bfs_relayout(T.tree);
        T.inst.resize(n);
        for (uint32_t j = 0; j < n; ++j) T.inst[j] = T.by_input[T.tree.order[j]];
    }
    *out = ot;
    return LUZ_OK;
}

void oracle_tlas_get(const oracle_tlas* ot, float* nodes, uint32_t* morton, uint32_t* order, uint32_t* node_count) {
    const Tlas& T = ot->t;
    if (node_count) *node_count = T.inst.empty() ? 0 : (uint32_t)(T.tree.nodes.size() / 16);
    if (nodes) memcpy(nodes, T.tree.nodes.data(), T.tree.nodes.size() * 4);
    if (morton) memcpy(morton, T.tree.morton.data(), T.tree.morton.size() * 4);
    if (order) memcpy(order, T.tree.order.data(), T.tree.order.size() * 4);
}

void oracle_tlas_destroy(oracle_tlas* t) { delete t; }

// ---------------------------------------------------------------- textures
// One RGBA8 UNORM level sampled bilinearly with repeat addressing (the reference's
// sampler, VulkanWrapper.cpp:2429-2454): u*width - 0.5 to texel space, weights from
// the fractional part, texels as c / 255.
struct Tex {
    const uint32_t* texels;
    uint32_t w, h;
};
static uint32_t tex_wrap(float f, uint32_t n) {
    float m = std::fmod(f, (float)n);
    if (m < 0.0f) m += (float)n;
    uint32_t i = (uint32_t)m;
    return i < n ? i : 0u;
}
static void tex_texel(const Tex& t, uint32_t x, uint32_t y, float c[4]) {
    uint32_t v = t.texels[(size_t)y * t.w + x];
    for (int k = 0; k < 4; ++k) c[k] = (float)((v >> (8 * k)) & 255u) / 255.0f;
}
static void tex_sample(const Tex& t, float u, float v, float out[4]) {
    float x = u * (float)t.w - 0.5f, y = v * (float)t.h - 0.5f;
    if (!std::isfinite(x)) x = 0.0f;
    if (!std::isfinite(y)) y = 0.0f;
    float fx = std::floor(x), fy = std::floor(y);
    float ax = x - fx, ay = y - fy;
    uint32_t x0 = tex_wrap(fx, t.w), y0 = tex_wrap(fy, t.h);
    uint32_t x1 = x0 + 1 == t.w ? 0u : x0 + 1, y1 = y0 + 1 == t.h ? 0u : y0 + 1;
    float c00[4], c10[4], c01[4], c11[4];
    tex_texel(t, x0, y0, c00);
    tex_texel(t, x1, y0, c10);
    tex_texel(t, x0, y1, c01);
    tex_texel(t, x1, y1, c11);
    float bx = 1.0f - ax, by = 1.0f - ay;
    for (int k = 0; k < 4; ++k) out[k] = (c00[k] * bx + c10[k] * ax) * by + (c01[k] * bx + c11[k] * ax) * ay;
}

static void hit_uv(const Blas& b, uint32_t prim, float b0, float b1, float b2, float& u, float& v) {
    const luz_vertex& v0 = b.vertices[b.indices[3 * prim]];
    const luz_vertex& v1 = b.vertices[b.indices[3 * prim + 1]];
    const luz_vertex& v2 = b.vertices[b.indices[3 * prim + 2]];
    u = (v0.texcoord[0] * b0 + v1.texcoord[0] * b1) + v2.texcoord[0] * b2;
    v = (v0.texcoord[1] * b0 + v1.texcoord[1] * b1) + v2.texcoord[1] * b2;
}

struct ColourAlpha : AlphaTest {
    const Tlas* T;
    const luz_model* models;
    uint32_t nmodels;
    const std::vector<Tex>* tex;
    bool accept(uint32_t input, uint32_t custom, uint32_t prim, float b0, float b1, float b2) const override {
        if (custom >= nmodels) return true;
        const luz_model& m = models[custom];
        if (m.color_map < 0 || (uint32_t)m.color_map >= tex->size()) return !(m.color[3] < 0.5f);
        float u, v, c[4];
        hit_uv(*T->by_input[input].blas, prim, b0, b1, b2, u, v);
        tex_sample((*tex)[(size_t)m.color_map], u, v, c);
        return !(m.color[3] * c[3] < 0.5f);
    }
};

// Primary-ray G-buffer (opaque.vert:21-31 + opaque.frag:21-58 at the closest hit).
// textures: ntex pointers to RGBA8 texel arrays, dims: width, height per texture.
int oracle_gbuffer(const oracle_tlas* ot, const luz_scene* S, const luz_model* models, uint32_t nmodels, uint32_t W,
                   uint32_t H, uint32_t* albedo, float* normal, uint32_t* material, uint32_t* emission, float* depth,
                   uint32_t* primary_hit, int threads, uint32_t y0, uint32_t y1, const uint32_t* const* textures,
                   const uint32_t* dims, uint32_t ntex) {
    const Tlas& T = ot->t;
    std::vector<Tex> tex(ntex);
    for (uint32_t k = 0; k < ntex; ++k) tex[k] = Tex{textures[k], dims[2 * k], dims[2 * k + 1]};
    std::vector<uint8_t> skip(std::max(nmodels, 1u), 0);
    for (uint32_t m = 0; m < nmodels; ++m)
        skip[m] = models[m].color_map >= 0 ? 2 : (models[m].color[3] < 0.5f ? 1 : 0);
    ColourAlpha alpha;
    alpha.T = &T;
    alpha.models = models;
    alpha.nmodels = nmodels;
    alpha.tex = &tex;
    // Normal matrices transpose(inverse(model)) = transpose of the w2o 3x3, per input instance.
    y1 = std::min(y1, H);
    const uint32_t p0 = std::min(y0, y1) * W;
    parallel_for(y1 * W - p0, threads, [&](uint32_t b, uint32_t e) {
        for (uint32_t pix = p0 + b; pix < p0 + e; ++pix) {
            uint32_t x = pix % W, y = pix / W;
            v3 cam = {S->cam_pos[0], S->cam_pos[1], S->cam_pos[2]};
            v3 target = DepthToWorld(*S, pixel_uv(x, W), pixel_uv(y, H), 1.0f);
            v3 dir = normalize(target - cam);
            Hit h{};
            bool hit = trace<true>(T, cam, dir, 0.0f, std::numeric_limits<float>::infinity(), skip.data(), nmodels, &h,
                                   &alpha);
            if (!hit) {
                albedo[pix] = 0; material[pix] = 0; emission[pix] = 0; depth[pix] = 1.0f;
                for (int k = 0; k < 4; ++k) normal[4 * pix + k] = 0.0f;
                primary_hit[2 * pix] = primary_hit[2 * pix + 1] = 0xFFFFFFFFu;
                continue;
            }
            v3 p = cam + dir * h.t;
            float pw[4] = {p.x, p.y, p.z, 1.0f}, clip[4];
            mat4_vec4(S->view_proj, pw, clip);
            float color[4] = {1, 1, 1, 1}, em[4] = {0, 0, 0, 1}, metallic = 0.0f, roughness = 0.5f, occl = 1.0f;
            int32_t cmap = -1, mrmap = -1, aomap = -1, nmap = -1, emap = -1;
            if (h.custom < nmodels) {
                const luz_model& m = models[h.custom];
                for (int k = 0; k < 4; ++k) color[k] = m.color[k];
                for (int k = 0; k < 3; ++k) em[k] = m.emission[k];
                metallic = m.metallic;
                roughness = m.roughness;
                auto ok = [&](int32_t i) { return i >= 0 && (uint32_t)i < ntex ? i : -1; };
                cmap = ok(m.color_map);
                mrmap = ok(m.metallic_roughness_map);
                aomap = ok(m.ao_map);
                nmap = ok(m.normal_map);
                emap = ok(m.emission_map);
            }
            const Instance& I = T.by_input[h.input];
            const Blas& bl = *I.blas;
            const float* w = I.w2o;
            // transpose(inverse(modelMat)) * vec4(x, 0): rows of the transposed inverse
            auto tim = [&](const float* n) {
                return v3{w[0] * n[0] + w[4] * n[1] + w[8] * n[2], w[1] * n[0] + w[5] * n[1] + w[9] * n[2],
                          w[2] * n[0] + w[6] * n[1] + w[10] * n[2]};
            };
            v3 nv[3], tv[3], bv[3];
            for (int k = 0; k < 3; ++k) {
                const luz_vertex& vx = bl.vertices[bl.indices[3 * h.prim + k]];
                nv[k] = normalize(tim(vx.normal));
                if (nmap >= 0) {   // opaque.vert:27-30
                    v3 tg = normalize(tim(vx.tangent));
                    tv[k] = normalize(tg - nv[k] * dot(tg, nv[k]));
                    bv[k] = cross(nv[k], tv[k]) * vx.tangent[3];
                }
            }
            v3 Ni = (nv[0] * h.b0 + nv[1] * h.b1) + nv[2] * h.b2;
            v3 N = normalize(Ni);
            float u = 0.0f, v = 0.0f, c[4];
            if (cmap >= 0 || mrmap >= 0 || aomap >= 0 || nmap >= 0 || emap >= 0) hit_uv(bl, h.prim, h.b0, h.b1, h.b2, u, v);
            if (cmap >= 0) {
                tex_sample(tex[cmap], u, v, c);
                for (int k = 0; k < 4; ++k) color[k] *= c[k];
            }
            if (mrmap >= 0) {
                tex_sample(tex[mrmap], u, v, c);
                roughness *= c[1];
                metallic *= c[2];
            }
            if (aomap >= 0) {
                tex_sample(tex[aomap], u, v, c);
                occl = c[0];
            }
            if (emap >= 0) {
                tex_sample(tex[emap], u, v, c);
                for (int k = 0; k < 4; ++k) em[k] *= c[k];
            }
            if (nmap >= 0) {   // opaque.frag:45-50
                tex_sample(tex[nmap], u, v, c);
                v3 ti = (tv[0] * h.b0 + tv[1] * h.b1) + tv[2] * h.b2;
                v3 bi = (bv[0] * h.b0 + bv[1] * h.b1) + bv[2] * h.b2;
                bool flat_t = ti.x == 0.0f && ti.y == 0.0f && ti.z == 0.0f;
                bool white = c[0] == 1.0f && c[1] == 1.0f && c[2] == 1.0f;
                if (!flat_t && !white) {
                    v3 ns = normalize(v3{c[0] * 2.0f - 1.0f, c[1] * 2.0f - 1.0f, c[2] * 2.0f - 1.0f});
                    N = normalize((ti * ns.x + bi * ns.y) + Ni * ns.z);
                }
            }
            albedo[pix] = pack8(color[0], color[1], color[2], color[3]);
            normal[4 * pix] = N.x; normal[4 * pix + 1] = N.y; normal[4 * pix + 2] = N.z; normal[4 * pix + 3] = 1.0f;
            material[pix] = pack8(roughness, metallic, occl, 1.0f);
            emission[pix] = pack8(em[0], em[1], em[2], em[3]);
            depth[pix] = clip[2] / clip[3];
            primary_hit[2 * pix] = h.custom;
            primary_hit[2 * pix + 1] = h.prim;
        }
    });
    return LUZ_OK;
}

// ---------------------------------------------------------------- TAA (taa.comp)
// The reference's sampler (linear, repeat, one level) on float images.
struct Bil {
    uint32_t x0, x1, y0, y1;
    float ax, ay, bx, by;
};
static Bil bil(float u, float v, uint32_t w, uint32_t h) {
    float x = u * (float)w - 0.5f, y = v * (float)h - 0.5f;
    if (!std::isfinite(x)) x = 0.0f;
    if (!std::isfinite(y)) y = 0.0f;
    float fx = std::floor(x), fy = std::floor(y);
    Bil b;
    b.ax = x - fx;
    b.ay = y - fy;
    b.bx = 1.0f - b.ax;
    b.by = 1.0f - b.ay;
    b.x0 = tex_wrap(fx, w);
    b.y0 = tex_wrap(fy, h);
    b.x1 = b.x0 + 1 == w ? 0u : b.x0 + 1;
    b.y1 = b.y0 + 1 == h ? 0u : b.y0 + 1;
    return b;
}
static float bl(float c00, float c10, float c01, float c11, const Bil& b) {
    return (c00 * b.bx + c10 * b.ax) * b.by + (c01 * b.bx + c11 * b.ax) * b.ay;
}
struct f4 {
    float v[4];
};
static f4 samp4(const float* img, uint32_t w, uint32_t h, float u, float v) {
    Bil b = bil(u, v, w, h);
    const float* c00 = img + 4 * ((size_t)b.y0 * w + b.x0);
    const float* c10 = img + 4 * ((size_t)b.y0 * w + b.x1);
    const float* c01 = img + 4 * ((size_t)b.y1 * w + b.x0);
    const float* c11 = img + 4 * ((size_t)b.y1 * w + b.x1);
    f4 r;
    for (int k = 0; k < 4; ++k) r.v[k] = bl(c00[k], c10[k], c01[k], c11[k], b);
    return r;
}
static float samp1(const float* img, uint32_t w, uint32_t h, float u, float v) {
    Bil b = bil(u, v, w, h);
    return bl(img[(size_t)b.y0 * w + b.x0], img[(size_t)b.y0 * w + b.x1], img[(size_t)b.y1 * w + b.x0],
              img[(size_t)b.y1 * w + b.x1], b);
}
static float gmin(float x, float y) { return y < x ? y : x; }   // GLSL min / max
static float gmax(float x, float y) { return x < y ? y : x; }
static f4 op(const f4& a, const f4& b, int o) {
    f4 r;
    for (int k = 0; k < 4; ++k)
        r.v[k] = o == 0 ? gmin(a.v[k], b.v[k]) : o == 1 ? gmax(a.v[k], b.v[k]) : o == 2 ? a.v[k] + b.v[k] : a.v[k] - b.v[k];
    return r;
}
static f4 scale(const f4& a, float s) { f4 r; for (int k = 0; k < 4; ++k) r.v[k] = a.v[k] * s; return r; }
static f4 divide(const f4& a, float s) { f4 r; for (int k = 0; k < 4; ++k) r.v[k] = a.v[k] / s; return r; }
static bool anynan(const f4& a) { return std::isnan(a.v[0]) || std::isnan(a.v[1]) || std::isnan(a.v[2]) || std::isnan(a.v[3]); }
static float MitchellFilter(float x) {   // utils.glsl
    const float B = 1.0f / 3.0f, C = 1.0f / 3.0f;
    float x2 = x * x;
    float x3 = x2 * x;
    return (6.0f - 2.0f * B) * x3 - (6.0f - 2.0f * B - 3.0f * C) * x2 + 1.0f;
}

// One TAA pass over rgba images (4 floats per pixel): taa.comp main (taa.comp:288-307).
void oracle_taa(const luz_scene* S, const float* input, const float* history, const float* depth, uint32_t W,
                uint32_t H, int reconstruct, float* out, int threads) {
    parallel_for(W * H, threads, [&](uint32_t b0, uint32_t e0) {
        for (uint32_t pix = b0; pix < e0; ++pix) {
            uint32_t x = pix % W, y = pix / W;
            const float su = ((float)x + 0.5f) / (float)W, sv = ((float)y + 0.5f) / (float)H;
            // find_closest_3x3
            const float ddx = std::fabs(1.0f / (float)W), ddy = std::fabs(1.0f / (float)H);
            float bx = 0, by = 0, bz = 0;
            bool first = true;
            for (int dy = -1; dy <= 1; ++dy)
                for (int dx = -1; dx <= 1; ++dx) {
                    float u = dx < 0 ? su - ddx : (dx > 0 ? su + ddx : su);
                    float v = dy < 0 ? sv - ddy : (dy > 0 ? sv + ddy : sv);
                    float z = samp1(depth, W, H, u, v);
                    if (first || bz > z) { bx = (float)dx; by = (float)dy; bz = z; first = false; }
                }
            float cu = su + ddx * bx, cv = sv + ddy * by;
            // get_motion_vector
            float d = samp1(depth, W, H, cu, cv);
            v3 wp = DepthToWorld(*S, cu, cv, d);
            float p4[4] = {wp.x, wp.y, wp.z, 1.0f}, prev[4], cur[4];
            mat4_vec4(S->prev_view_proj, p4, prev);
            mat4_vec4(S->view_proj, p4, cur);
            float mx = ((cur[0] / cur[3] - S->jitter[0]) - (prev[0] / prev[3] - S->prev_jitter[0])) * 0.5f;
            float my = ((cur[1] / cur[3] - S->jitter[1]) - (prev[1] / prev[3] - S->prev_jitter[1])) * 0.5f;
            const float hu = su - mx, hv = sv - my;
            f4 hist = samp4(history, W, H, hu, hv);
            // get_neighbor_3x3
            const float du = 1.0f / (float)W, dv = 1.0f / (float)H;
            f4 c[9];
            for (int k = 0; k < 9; ++k) {
                int dx = k % 3 - 1, dy = k / 3 - 1;
                float u = dx < 0 ? su - du : (dx > 0 ? su + du : su);
                float v = dy < 0 ? sv - dv : (dy > 0 ? sv + dv : sv);
                c[k] = samp4(input, W, H, u, v);
            }
            f4 cmin = c[8], cmax = c[8];
            for (int k = 7; k >= 0; --k) { cmin = op(c[k], cmin, 0); cmax = op(c[k], cmax, 1); }
            f4 cavg = c[0];
            for (int k = 1; k < 9; ++k) cavg = op(cavg, c[k], 2);
            cavg = divide(cavg, 9.0f);
            f4 cmin5 = op(c[1], op(c[3], op(c[4], op(c[5], c[7], 0), 0), 0), 0);
            f4 cmax5 = op(c[1], op(c[3], op(c[4], op(c[5], c[7], 1), 1), 1), 1);
            f4 cavg5 = divide(op(op(op(op(c[1], c[3], 2), c[4], 2), c[5], 2), c[7], 2), 5.0f);
            cmin = scale(op(cmin, cmin5, 2), 0.5f);
            cmax = scale(op(cmax, cmax5, 2), 0.5f);
            cavg = scale(op(cavg, cavg5, 2), 0.5f);
            f4 src = {{0, 0, 0, 0}};
            if (reconstruct == 1) {
                float wsum = 0.0f;
                for (int k = 0; k < 9; ++k) {
                    float dx = (float)(k % 3 - 1), dy = (float)(k / 3 - 1);
                    float wgt = MitchellFilter(std::sqrt(dx * dx + dy * dy));
                    src = op(src, scale(c[k], wgt), 2);
                    wsum += wgt;
                }
                src = divide(src, wsum);
            }
            if (reconstruct == 0 || anynan(src)) src = samp4(input, W, H, su, sv);
            f4 res;
            if (hu > 1.0f || hv > 1.0f || hu < 0.0f || hv < 0.0f) {
                res = src;
            } else {
                f4 p = op(op(cavg, cmin, 1), cmax, 0);   // clamp(cavg, cmin, cmax)
                f4 r = op(hist, p, 3);
                const float eps = 0.00000001f;
                float rmax[3], rmin[3];
                for (int k = 0; k < 3; ++k) { rmax[k] = cmax.v[k] - p.v[k]; rmin[k] = cmin.v[k] - p.v[k]; }
                for (int k = 0; k < 3; ++k) if (r.v[k] > rmax[k] + eps) r = scale(r, rmax[k] / r.v[k]);
                for (int k = 0; k < 3; ++k) if (r.v[k] < rmin[k] - eps) r = scale(r, rmin[k] / r.v[k]);
                hist = op(p, r, 2);
                float sw = 0.05f, hw = 1.0f - sw;
                float rs = 1.0f / (gmax(gmax(src.v[0], src.v[1]), src.v[2]) + 1.0f);
                float rh = 1.0f / (gmax(gmax(hist.v[0], hist.v[1]), hist.v[2]) + 1.0f);
                float ls = (src.v[0] * rs) * 0.2127f + (src.v[1] * rs) * 0.7152f + (src.v[2] * rs) * 0.0722f;
                float lh = (hist.v[0] * rh) * 0.2127f + (hist.v[1] * rh) * 0.7152f + (hist.v[2] * rh) * 0.0722f;
                sw *= 1.0f / (1.0f + ls);
                hw *= 1.0f / (1.0f + lh);
                res = divide(op(scale(src, sw), scale(hist, hw), 2), gmax(sw + hw, 0.0000001f));
                if (anynan(res)) res = src;
            }
            for (int k = 0; k < 4; ++k) out[4 * (size_t)pix + k] = res.v[k];
        }
    });
}

// ---------------------------------------------------------------- compose (present.frag)
static f4 samp_rgba8(const uint32_t* img, uint32_t w, uint32_t h, float u, float v) {
    Bil b = bil(u, v, w, h);
    uint32_t t[4] = {img[(size_t)b.y0 * w + b.x0], img[(size_t)b.y0 * w + b.x1], img[(size_t)b.y1 * w + b.x0],
                     img[(size_t)b.y1 * w + b.x1]};
    f4 r;
    for (int k = 0; k < 4; ++k) {
        float c[4];
        for (int q = 0; q < 4; ++q) c[q] = (float)((t[q] >> (8 * k)) & 255u) / 255.0f;
        r.v[k] = bl(c[0], c[1], c[2], c[3], b);
    }
    return r;
}
static float aces(float x) {
    const float a = 2.51f, b = 0.03f, c = 2.43f, d = 0.59f, e = 0.14f;
    x = (x * (a * x + b)) / (x * (c * x + d) + e);
    return std::pow(x, 1.0f / 2.2f);
}
static uint32_t unorm8c(float x) {
    x = gmin(gmax(x, 0.0f), 1.0f);
    return (uint32_t)(x * 255.0f + 0.5f);
}

// present.frag main over every pixel into BGRA8 words.
void oracle_compose(const float* light, const uint32_t* albedo, const float* normal, const uint32_t* material,
                    const uint32_t* emission, const float* depth, uint32_t W, uint32_t H, int image_type,
                    uint32_t* out) {
    for (uint32_t y = 0; y < H; ++y)
        for (uint32_t x = 0; x < W; ++x) {
            float tu = ((float)x + 0.5f) / (float)W, tv = ((float)y + 0.5f) / (float)H;
            int type = image_type;
            float fu = tu, fv = tv;
            if (type == 6) {
                fu = tu * 3.0f;
                fv = tv * 2.0f;
                if (tv < 0.5f) {
                    if (tu < 1.0f / 3.0f) type = 0;
                    else if (tu < 2.0f / 3.0f) { type = 1; fu -= 1.0f; }
                    else { type = 2; fu -= 2.0f; }
                } else {
                    fv -= 1.0f;
                    if (tu < 1.0f / 3.0f) type = 3;
                    else if (tu < 2.0f / 3.0f) { type = 4; fu -= 1.0f; }
                    else { type = 5; fu -= 2.0f; }
                }
                fu = 1.0f / 6.0f + fu * 2.0f / 3.0f;
            }
            f4 v;
            switch (type) {
                case 1: v = samp_rgba8(albedo, W, H, fu, fv); break;
                case 2: v = samp4(normal, W, H, fu, fv); break;
                case 3: v = samp_rgba8(material, W, H, fu, fv); break;
                case 4: v = samp_rgba8(emission, W, H, fu, fv); break;
                case 5: v = f4{{samp1(depth, W, H, fu, fv), 0.0f, 0.0f, 1.0f}}; break;
                default: v = samp4(light, W, H, fu, fv); break;
            }
            if (type == 0) {
                v = f4{{aces(v.v[0]), aces(v.v[1]), aces(v.v[2]), 1.0f}};
            } else if (type == 2) {
                for (int k = 0; k < 4; ++k) v.v[k] = (v.v[k] + 1.0f) / 2.0f;
            } else if (type == 5) {
                const float nearp = 0.01f, farp = 5.0f;
                float l = (2.0f * nearp) / (farp + nearp - v.v[0] * (farp - nearp));
                v = f4{{l, l, l, l}};
            }
            out[(size_t)y * W + x] = unorm8c(v.v[2]) | (unorm8c(v.v[1]) << 8) | (unorm8c(v.v[0]) << 16) | (255u << 24);
        }
}

// histogram.comp + histogramAverage.comp (DeferredRenderer.cpp:447-466 constants).
// out: 256 bins then 4 floats (weighted sum, log average, average, adapted).
void oracle_histogram(const float* img, uint32_t n, float delta_time, float* state, uint32_t* out) {
    const float min_log = -10.0f, one_over_log = 1.0f / 12.0f;
    std::vector<uint32_t> bins(256, 0);
    for (uint32_t i = 0; i < n; ++i) {
        const float* c = img + 4 * (size_t)i;
        float lum = c[0] * 0.2127f + c[1] * 0.7152f + c[2] * 0.0722f;
        uint32_t bin = 0;
        if (!(lum < 0.000001f)) {
            float t = (std::log2(lum) - min_log) * one_over_log;
            t = gmin(gmax(t, 0.0f), 1.0f);
            bin = (uint32_t)(t * 254.0f + 1.0f);
        }
        bins[bin]++;
    }
    float sh[256];
    for (int i = 0; i < 256; ++i) sh[i] = (float)bins[i] * (float)i;
    for (int k = 128; k > 0; k >>= 1)
        for (int i = 0; i < k; ++i) sh[i] += sh[i + k];
    float wla = (sh[0] / gmax((float)n - (float)bins[0], 1.0f)) - 1.0f;
    float avg = std::exp2(((wla / 254.0f) * one_over_log) + min_log);
    float adapted = state[0] + (avg - state[0]) * (1.0f - std::exp(-delta_time * 1.1f));
    state[0] = adapted;
    for (int i = 0; i < 256; ++i) out[i] = bins[i];
    float f[4] = {sh[0], wla, avg, adapted};
    memcpy(out + 256, f, 16);
}

// Shadow maps of every light into out (per light faces * res * res floats, lights in
// order) and registered for the light pass (oracle_clear_shadow_maps drops them).
void oracle_render_shadow_maps(const oracle_tlas* ot, const luz_shadow_light* lights, uint32_t count, uint32_t res,
                               float* out, int threads) {
    const Tlas& T = ot->t;
    g_shadow.assign(count, OShadow{});
    size_t off = 0;
    for (uint32_t l = 0; l < count; ++l) {
        const luz_shadow_light& L = lights[l];
        OShadow& o = g_shadow[l];
        o.map = out + off;
        memcpy(o.vp0, L.view_proj[0], 64);
        memcpy(o.pos, L.position, 12);
        o.zfar = L.z_far;
        o.faces = L.faces;
        o.res = res;
        const size_t face_px = (size_t)res * res;
        std::vector<uint32_t> bits((size_t)L.faces * face_px, 0x3F800000u);
        const float inv_zfar = 1.0f / L.z_far;
        // faces in parallel (each face's map is its own)
        parallel_for(L.faces, std::min<int>(threads, (int)L.faces), [&](uint32_t f0, uint32_t f1) {
            for (uint32_t face = f0; face < f1; ++face)
                for (const Instance& I : T.by_input) {
                    const Blas& b = *I.blas;
                    for (uint32_t t = 0; t < b.prims; ++t) {
                        float clip[3][4], world[3][3];
                        for (int k = 0; k < 3; ++k) {
                            const float* p = b.vertices[b.indices[3 * t + k]].position;
                            const float* m = I.o2w;
                            for (int r = 0; r < 3; ++r)
                                world[k][r] = m[r * 4 + 0] * p[0] + m[r * 4 + 1] * p[1] + m[r * 4 + 2] * p[2] + m[r * 4 + 3];
                            float w4[4] = {world[k][0], world[k][1], world[k][2], 1.0f};
                            mat4_vec4(L.view_proj[face], w4, clip[k]);
                        }
                        uint32_t* fm = bits.data() + face * face_px;
                        if (L.faces != 6) {
                            RV v[3] = {r_screen(clip[0], world[0], res), r_screen(clip[1], world[1], res),
                                       r_screen(clip[2], world[2], res)};
                            r_tri(v, L.faces, res, L.position, inv_zfar, fm);
                            continue;
                        }
                        const float kNearW = 1e-5f;
                        float pc[4][4], pw[4][3];
                        int n = 0;
                        for (int k = 0; k < 3; ++k) {
                            const int j = (k + 1) % 3;
                            const bool ink = clip[k][3] >= kNearW, inj = clip[j][3] >= kNearW;
                            if (ink) {
                                for (int q = 0; q < 4; ++q) pc[n][q] = clip[k][q];
                                for (int q = 0; q < 3; ++q) pw[n][q] = world[k][q];
                                ++n;
                            }
                            if (ink != inj) {
                                float tt = (kNearW - clip[k][3]) / (clip[j][3] - clip[k][3]);
                                for (int q = 0; q < 4; ++q) pc[n][q] = clip[k][q] + (clip[j][q] - clip[k][q]) * tt;
                                for (int q = 0; q < 3; ++q) pw[n][q] = world[k][q] + (world[j][q] - world[k][q]) * tt;
                                ++n;
                            }
                        }
                        if (n < 3) continue;
                        RV sv[4];
                        for (int k = 0; k < n; ++k) sv[k] = r_screen(pc[k], pw[k], res);
                        RV t0[3] = {sv[0], sv[1], sv[2]};
                        r_tri(t0, 6, res, L.position, inv_zfar, fm);
                        if (n == 4) {
                            RV t1[3] = {sv[0], sv[2], sv[3]};
                            r_tri(t1, 6, res, L.position, inv_zfar, fm);
                        }
                    }
                }
        });
        memcpy(out + off, bits.data(), bits.size() * 4);
        off += bits.size();
    }
}

void oracle_clear_shadow_maps() { g_shadow.clear(); }

// Shadow + AO visibility bits for the pixel rows [y0, y1). brute != 0 uses the
// all-triangles oracle instead of the BVH. cull != 0 leaves out (bit 0) the shadow
// rays of a light whose term in the light pass cannot depend on its shadow factor
// (shadow_has_no_effect), as the device's ray generation does; cull = 0 traces every
// ray light.frag traces.
// Returns the number of rays traced.
uint64_t oracle_visibility(const oracle_tlas* ot, const luz_scene* S, const luz_light* lights, uint32_t nl,
                           const float* normal, const float* depth, uint32_t W, uint32_t H, uint32_t y0, uint32_t y1,
                           int frame, const uint8_t* bn, uint32_t bn_size, uint32_t* shadow_bits, uint32_t* ao_bits,
                           int threads, int brute, int cull) {
    const Tlas& T = ot->t;
    uint32_t words = (W * H + 31) / 32;
    Sampler smp{S->sampler, bn, bn_size, frame};
    std::vector<uint32_t> first(nl + 1, 0);
    for (uint32_t l = 0; l < nl; ++l)
        first[l + 1] = first[l] + (S->shadow_type == LUZ_SHADOW_RAYTRACING ? (uint32_t)std::max(0, lights[l].num_shadow_samples) : 0u);
    uint32_t ao_n = (uint32_t)std::max(0, S->ao_num_samples);
    std::atomic<uint64_t> rays{0};
    v3 cam = {S->cam_pos[0], S->cam_pos[1], S->cam_pos[2]};
    // bits are written per 32-pixel word: split the work on word boundaries
    uint32_t p0 = y0 * W, p1 = y1 * W;
    uint32_t w0 = p0 / 32, w1 = (p1 + 31) / 32;
    parallel_for(w1 - w0, threads, [&](uint32_t b, uint32_t e) {
        uint64_t local = 0;
        for (uint32_t wd = w0 + b; wd < w0 + e; ++wd) {
            for (uint32_t pix = std::max(wd * 32, p0); pix < std::min(wd * 32 + 32, p1); ++pix) {
                v3 N = {normal[4 * pix], normal[4 * pix + 1], normal[4 * pix + 2]};
                if (length(N) == 0.0f) continue;
                uint32_t x = pix % W, y = pix / W;
                v3 p = DepthToWorld(*S, pixel_uv(x, W), pixel_uv(y, H), depth[pix]);
                uint32_t bit = 1u << (pix & 31);
                for (uint32_t l = 0; l < nl; ++l) {
                    if (cull && first[l + 1] > first[l] &&
                        shadow_has_no_effect(lights[l], p, N, light_vector<float>(lights[l], p)))
                        continue;
                    for (uint32_t s = 0; s < first[l + 1] - first[l]; ++s) {
                        float rx, ry;
                        smp.rg(x, y, (int)s, l + 1, &rx, &ry);
                        v3 O, dir;
                        float tMax;
                        ShadowRay(lights[l], p, N, cam, rx, ry, O, dir, tMax);
                        bool hit = brute ? trace_bruteforce(T, O, dir, 0.001f, tMax)
                                         : trace<false>(T, O, dir, 0.001f, tMax, nullptr, 0, nullptr);
                        ++local;
                        if (hit) shadow_bits[(size_t)(first[l] + s) * words + (pix >> 5)] |= bit;
                    }
                }
                for (uint32_t s = 0; s < ao_n; ++s) {
                    float rx, ry;
                    smp.rg(x, y, (int)s, 0u, &rx, &ry);
                    v3 O, dir;
                    AORay(p, N, cam, rx, ry, O, dir);
                    bool hit = brute ? trace_bruteforce(T, O, dir, S->ao_min, S->ao_max)
                                     : trace<false>(T, O, dir, S->ao_min, S->ao_max, nullptr, 0, nullptr);
                    ++local;
                    if (!hit) ao_bits[(size_t)s * words + (pix >> 5)] |= bit;
                }
            }
        }
        rays += local;
    });
    return rays.load();
}

static void light_pass_impl(const luz_scene* S, const luz_light* lights, uint32_t nl, const uint32_t* albedo,
                            const float* normal, const uint32_t* material, const uint32_t* emission, const float* depth,
                            const uint32_t* shadow_bits, const uint32_t* ao_bits, const float* ao_override, uint32_t W,
                            uint32_t H, float* outf, double* outd, int threads, uint32_t y0, uint32_t y1) {
    uint32_t words = (W * H + 31) / 32;
    std::vector<uint32_t> first(nl, 0);
    uint32_t acc = 0;
    for (uint32_t l = 0; l < nl; ++l) {
        first[l] = acc;
        acc += S->shadow_type == LUZ_SHADOW_RAYTRACING ? (uint32_t)std::max(0, lights[l].num_shadow_samples) : 0u;
    }
    std::vector<float> lutf(256);
    std::vector<double> lutd(256);
    for (int i = 0; i < 256; ++i) {
        lutf[i] = (float)std::pow((double)((float)i / 255.0f), 2.2);
        lutd[i] = std::pow((double)i / 255.0, 2.2);
    }
    Planes P{albedo, normal, material, emission, depth, shadow_bits, ao_bits, ao_override};
    uint32_t ao_n = (uint32_t)std::max(0, S->ao_num_samples);
    y1 = std::min(y1, H);
    const uint32_t p0 = std::min(y0, y1) * W;
    parallel_for(y1 * W - p0, threads, [&](uint32_t b, uint32_t e) {
        for (uint32_t pix = p0 + b; pix < p0 + e; ++pix) {
            if (outf) light_pixel<float>(*S, lights, nl, first, P, W, H, words, ao_n, pix, &outf[4 * (size_t)pix], lutf);
            if (outd) light_pixel<double>(*S, lights, nl, first, P, W, H, words, ao_n, pix, &outd[4 * (size_t)pix], lutd);
        }
    });
}

// The split of the direct light that feeds the denoiser, per pixel 8 values: S (r, g,
// b), the AO value, U (r, g, b), the unoccluded fraction of all shadow samples; S is
// light.frag's shadowed sum over the lights, U the same with every shadow factor 0.
// Background pixels get zeros.
int oracle_light_split(const luz_scene* S, const luz_light* lights, uint32_t nl, const uint32_t* albedo,
                       const float* normal, const uint32_t* material, const uint32_t* emission, const float* depth,
                       const uint32_t* shadow_bits, const uint32_t* ao_bits, uint32_t W, uint32_t H, float* out8,
                       int threads) {
    uint32_t words = (W * H + 31) / 32;
    std::vector<uint32_t> first(nl, 0);
    uint32_t acc = 0;
    for (uint32_t l = 0; l < nl; ++l) {
        first[l] = acc;
        acc += S->shadow_type == LUZ_SHADOW_RAYTRACING ? (uint32_t)std::max(0, lights[l].num_shadow_samples) : 0u;
    }
    std::vector<float> lutf(256);
    for (int i = 0; i < 256; ++i) lutf[i] = (float)std::pow((double)((float)i / 255.0f), 2.2);
    Planes P{albedo, normal, material, emission, depth, shadow_bits, ao_bits, nullptr};
    uint32_t ao_n = (uint32_t)std::max(0, S->ao_num_samples);
    parallel_for(W * H, threads, [&](uint32_t b, uint32_t e) {
        float rgba[4];
        for (uint32_t pix = b; pix < e; ++pix)
            light_pixel<float>(*S, lights, nl, first, P, W, H, words, ao_n, pix, rgba, lutf, &out8[8 * (size_t)pix]);
    });
    return LUZ_OK;
}

int oracle_light_pass(const luz_scene* S, const luz_light* lights, uint32_t nl, const uint32_t* albedo,
                      const float* normal, const uint32_t* material, const uint32_t* emission, const float* depth,
                      const uint32_t* shadow_bits, const uint32_t* ao_bits, const float* ao_override, uint32_t W,
                      uint32_t H, float* out, int threads, uint32_t y0, uint32_t y1) {
    light_pass_impl(S, lights, nl, albedo, normal, material, emission, depth, shadow_bits, ao_bits, ao_override, W, H,
                    out, nullptr, threads, y0, y1);
    return LUZ_OK;
}

int oracle_light_pass_f64(const luz_scene* S, const luz_light* lights, uint32_t nl, const uint32_t* albedo,
                          const float* normal, const uint32_t* material, const uint32_t* emission, const float* depth,
                          const uint32_t* shadow_bits, const uint32_t* ao_bits, const float* ao_override, uint32_t W,
                          uint32_t H, double* out, int threads, uint32_t y0, uint32_t y1) {
    light_pass_impl(S, lights, nl, albedo, normal, material, emission, depth, shadow_bits, ao_bits, ao_override, W, H,
                    nullptr, out, threads, y0, y1);
    return LUZ_OK;
}

// The shadow and AO rays of every lit pixel in the order light.frag main issues them
// (lights in order, their samples, then the AO samples): 8 floats per ray (o, tmin,
// d, tmax). Returns the number of rays (written up to cap).
uint64_t oracle_generate_rays(const luz_scene* S, const luz_light* lights, uint32_t nl, const float* normal,
                              const float* depth, uint32_t W, uint32_t H, int frame, const uint8_t* bn,
                              uint32_t bn_size, float* out, uint64_t cap) {
    Sampler smp{S->sampler, bn, bn_size, frame};
    v3 cam = {S->cam_pos[0], S->cam_pos[1], S->cam_pos[2]};
    uint64_t n = 0;
    auto put = [&](v3 o, float tmin, v3 d, float tmax) {
        if (n < cap) {
            float* r = out + 8 * n;
            r[0] = o.x; r[1] = o.y; r[2] = o.z; r[3] = tmin; r[4] = d.x; r[5] = d.y; r[6] = d.z; r[7] = tmax;
        }
        ++n;
    };
    for (uint32_t pix = 0; pix < W * H; ++pix) {
        v3 N = {normal[4 * pix], normal[4 * pix + 1], normal[4 * pix + 2]};
        if (length(N) == 0.0f) continue;
        uint32_t x = pix % W, y = pix / W;
        v3 p = DepthToWorld(*S, pixel_uv(x, W), pixel_uv(y, H), depth[pix]);
        for (uint32_t l = 0; l < nl; ++l) {
            int ns = S->shadow_type == LUZ_SHADOW_RAYTRACING ? lights[l].num_shadow_samples : 0;
            for (int s = 0; s < ns; ++s) {
                float rx, ry, tMax;
                smp.rg(x, y, s, l + 1, &rx, &ry);
                v3 O, dir;
                ShadowRay(lights[l], p, N, cam, rx, ry, O, dir, tMax);
                put(O, 0.001f, dir, tMax);
            }
        }
        for (int s = 0; s < S->ao_num_samples; ++s) {
            float rx, ry;
            smp.rg(x, y, s, 0u, &rx, &ry);
            v3 O, dir;
            AORay(p, N, cam, rx, ry, O, dir);
            put(O, S->ao_min, dir, S->ao_max);
        }
    }
    return n;
}

// Single rays, for known-answer tests: any-hit (closest = 0) or closest-hit t.
int oracle_trace_ray(const oracle_tlas* ot, const float o[3], const float d[3], float tmin, float tmax, int closest,
                     int brute, float* t_out) {
    const Tlas& T = ot->t;
    v3 O = {o[0], o[1], o[2]}, D = {d[0], d[1], d[2]};
    if (closest) {
        Hit h{};
        bool r = trace<true>(T, O, D, tmin, tmax, nullptr, 0, &h);
        if (t_out) *t_out = r ? h.t : -1.0f;
        return r ? 1 : 0;
    }
    return (brute ? trace_bruteforce(T, O, D, tmin, tmax) : trace<false>(T, O, D, tmin, tmax, nullptr, 0, nullptr)) ? 1 : 0;
}

// The project sin/cos and the two samplers, exposed for error-bound tests.
void oracle_sincos(const float* x, float* s, float* c, uint32_t n) {
    for (uint32_t i = 0; i < n; ++i) sincos_cw(x[i], &s[i], &c[i]);
}
void oracle_disk_sample(float rx, float ry, float radius, float* dx, float* dy) { DiskSample(rx, ry, radius, dx, dy); }
void oracle_hemisphere_sample(float rx, float ry, float* out3) {
    v3 h = HemisphereSample(rx, ry);
    out3[0] = h.x; out3[1] = h.y; out3[2] = h.z;
}
// GGX terms for known-answer tests (light.frag:17-49).
void oracle_ggx_terms(const float N[3], const float V[3], const float L[3], float roughness, const float F0[3],
                      float* D, float* G, float F[3]) {
    v3 n = {N[0], N[1], N[2]}, v = {V[0], V[1], V[2]}, l = {L[0], L[1], L[2]};
    v3 h = normalize(v + l);
    *D = DistributionGGX<float>(n, h, roughness, PI_F);
    *G = GeometrySmith<float>(n, v, l, roughness);
    v3 f = FresnelSchlick<float>(tclamp01(dot(h, v)), {F0[0], F0[1], F0[2]});
    F[0] = f.x; F[1] = f.y; F[2] = f.z;
}
void oracle_depth_to_world(const luz_scene* S, float u, float v, float depth, float out[3]) {
    v3 p = DepthToWorld(*S, u, v, depth);
    out[0] = p.x; out[1] = p.y; out[2] = p.z;
}

}  // extern "C"
