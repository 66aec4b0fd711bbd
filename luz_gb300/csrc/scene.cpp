// scene.cpp — host scene layer: synthetic generators, the reference's transform and
// camera math, SceneBlock/LightBlock/ModelBlock packing. C++17, no CUDA.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <new>
#include <stdexcept>
#include <utility>
#include <vector>

#include "../../include/luz_scene.h"
#include "pathmath.cuh"
#include "scene_internal.hpp"

namespace {

using luz::host::Mesh;

// ---------------------------------------------------------------- PRNG
// SplitMix64 (S. Vigna): integer-only, identical on every platform.
struct Rng {
    uint64_t s;
    explicit Rng(uint64_t seed) : s(seed * 0x9E3779B97F4A7C15ull + 0x632BE59BD9B4E019ull) {}
    uint64_t next() {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    float uniform() { return (float)(next() >> 40) * (1.0f / 16777216.0f); }   // [0,1)
    float uniform(float a, float b) { return a + (b - a) * uniform(); }
    uint32_t below(uint32_t n) { return (uint32_t)((next() >> 32) % n); }
};

// ---------------------------------------------------------------- 4x4 column-major math
using M4 = std::array<float, 16>;

M4 identity() {
    M4 m{};
    m[0] = m[5] = m[10] = m[15] = 1.0f;
    return m;
}
M4 mul(const M4& a, const M4& b) {
    M4 c{};
    for (int col = 0; col < 4; ++col)
        for (int row = 0; row < 4; ++row) {
            float s = 0.0f;
            for (int k = 0; k < 4; ++k) s += a[k * 4 + row] * b[col * 4 + k];
            c[col * 4 + row] = s;
        }
    return c;
}
// General inverse by Gauss-Jordan elimination in double precision.
M4 inverse(const M4& m) {
    double a[4][8];
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) {
            a[r][c] = m[c * 4 + r];
            a[r][c + 4] = r == c ? 1.0 : 0.0;
        }
    for (int c = 0; c < 4; ++c) {
        int piv = c;
        for (int r = c + 1; r < 4; ++r)
            if (std::fabs(a[r][c]) > std::fabs(a[piv][c])) piv = r;
        if (piv != c)
            for (int k = 0; k < 8; ++k) std::swap(a[c][k], a[piv][k]);
        double d = a[c][c];
        if (d == 0.0) return identity();
        for (int k = 0; k < 8; ++k) a[c][k] /= d;
        for (int r = 0; r < 4; ++r) {
            if (r == c) continue;
            double f = a[r][c];
            for (int k = 0; k < 8; ++k) a[r][k] -= f * a[c][k];
        }
    }
    M4 out{};
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) out[c * 4 + r] = (float)a[r][c + 4];
    return out;
}

struct F3 {
    float x, y, z;
};
F3 sub(F3 a, F3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
F3 crossf(F3 a, F3 b) { return {a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y}; }
float dotf(F3 a, F3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
F3 normf(F3 a) {
    float l = std::sqrt(dotf(a, a));
    return {a.x / l, a.y / l, a.z / l};
}

// glm::lookAt, right-handed.
M4 look_at(F3 eye, F3 center, F3 up) {
    F3 f = normf(sub(center, eye));
    F3 s = normf(crossf(f, up));
    F3 u = crossf(s, f);
    M4 r = identity();
    r[0] = s.x; r[4] = s.y; r[8] = s.z;
    r[1] = u.x; r[5] = u.y; r[9] = u.z;
    r[2] = -f.x; r[6] = -f.y; r[10] = -f.z;
    r[12] = -dotf(s, eye);
    r[13] = -dotf(u, eye);
    r[14] = dotf(f, eye);
    return r;
}
// glm::perspective, right-handed, depth zero-to-one (Luzpch.hpp: GLM_FORCE_DEPTH_ZERO_TO_ONE).
M4 perspective_zo(float fovy, float aspect, float zn, float zf) {
    float t = std::tan(fovy / 2.0f);
    M4 r{};
    r[0] = 1.0f / (aspect * t);
    r[5] = 1.0f / t;
    r[10] = zf / (zn - zf);
    r[11] = -1.0f;
    r[14] = -(zf * zn) / (zf - zn);
    return r;
}
// glm::ortho, right-handed, zero-to-one.
M4 ortho_zo(float l, float rgt, float b, float t, float zn, float zf) {
    M4 r = identity();
    r[0] = 2.0f / (rgt - l);
    r[5] = 2.0f / (t - b);
    r[10] = -1.0f / (zf - zn);
    r[12] = -(rgt + l) / (rgt - l);
    r[13] = -(t + b) / (t - b);
    r[14] = -zn / (zf - zn);
    return r;
}
M4 rotate(const M4& m, float angle, F3 axis) {
    float c = std::cos(angle), s = std::sin(angle);
    F3 a = normf(axis);
    F3 t = {(1.0f - c) * a.x, (1.0f - c) * a.y, (1.0f - c) * a.z};
    float R[3][3];
    R[0][0] = c + t.x * a.x; R[0][1] = t.x * a.y + s * a.z; R[0][2] = t.x * a.z - s * a.y;
    R[1][0] = t.y * a.x - s * a.z; R[1][1] = c + t.y * a.y; R[1][2] = t.y * a.z + s * a.x;
    R[2][0] = t.z * a.x + s * a.y; R[2][1] = t.z * a.y - s * a.x; R[2][2] = c + t.z * a.z;
    M4 r = m;
    for (int row = 0; row < 4; ++row)
        for (int col = 0; col < 3; ++col)
            r[col * 4 + row] = m[0 * 4 + row] * R[col][0] + m[1 * 4 + row] * R[col][1] + m[2 * 4 + row] * R[col][2];
    return r;
}

// Quaternion (w, x, y, z) -> rotation matrix, as glm::mat3_cast.
M4 quat_to_mat(float w, float x, float y, float z) {
    float qxx = x * x, qyy = y * y, qzz = z * z, qxz = x * z, qxy = x * y, qyz = y * z,
          qwx = w * x, qwy = w * y, qwz = w * z;
    M4 r = identity();
    r[0] = 1.0f - 2.0f * (qyy + qzz); r[1] = 2.0f * (qxy + qwz); r[2] = 2.0f * (qxz - qwy);
    r[4] = 2.0f * (qxy - qwz); r[5] = 1.0f - 2.0f * (qxx + qzz); r[6] = 2.0f * (qyz + qwx);
    r[8] = 2.0f * (qxz + qwy); r[9] = 2.0f * (qyz - qwx); r[10] = 1.0f - 2.0f * (qxx + qyy);
    return r;
}

M4 compose(const float pos[3], const float rot_deg[3], const float scl[3], const M4& parent) {
    const float d2r = 3.14159265358979323846f / 180.0f;
    float ex = rot_deg[0] * d2r * 0.5f, ey = rot_deg[1] * d2r * 0.5f, ez = rot_deg[2] * d2r * 0.5f;
    float cx = std::cos(ex), cy = std::cos(ey), cz = std::cos(ez);
    float sx = std::sin(ex), sy = std::sin(ey), sz = std::sin(ez);
    // glm::quat(vec3 eulerAngles)
    float w = cx * cy * cz + sx * sy * sz;
    float x = sx * cy * cz - cx * sy * sz;
    float y = cx * sy * cz + sx * cy * sz;
    float z = cx * cy * sz - sx * sy * cz;
    M4 R = quat_to_mat(w, x, y, z);
    M4 T = identity();
    T[12] = pos[0]; T[13] = pos[1]; T[14] = pos[2];
    M4 S = identity();
    S[0] = scl[0]; S[5] = scl[1]; S[10] = scl[2];
    return mul(parent, mul(mul(T, R), S));
}

void camera_matrices(const luz_camera& cam, luz_camera& updated, M4& view, M4& proj) {
    updated = cam;
    const float d2r = 3.14159265358979323846f / 180.0f;
    if (cam.mode == 0) {   // Orbit
        float rx = (cam.rotation[0] + 90.0f) * d2r, ry = (cam.rotation[1] + 90.0f) * d2r;
        F3 vd;
        vd.x = std::cos(-ry) * std::sin(rx);
        vd.z = std::sin(-ry) * std::sin(rx);
        vd.y = std::cos(rx);
        if (cam.camera_type == 0) vd = {vd.x * cam.zoom, vd.y * cam.zoom, vd.z * cam.zoom};
        F3 c = {cam.center[0], cam.center[1], cam.center[2]};
        F3 e = sub(c, vd);
        updated.eye[0] = e.x; updated.eye[1] = e.y; updated.eye[2] = e.z;
        view = look_at(e, c, {0.0f, 1.0f, 0.0f});
    } else if (cam.mode == 1) {   // Fly
        float rx = cam.rotation[0] * d2r, ry = (cam.rotation[1] + 180.0f) * d2r, rz = cam.rotation[2] * d2r;
        M4 rot = identity();
        rot = rotate(rot, rz, {0.0f, 0.0f, 1.0f});
        rot = rotate(rot, ry, {0.0f, 1.0f, 0.0f});
        rot = rotate(rot, rx, {1.0f, 0.0f, 0.0f});
        F3 e = {cam.eye[0], cam.eye[1], cam.eye[2]};
        F3 f = {rot[8], rot[9], rot[10]};
        view = look_at(e, {e.x + f.x, e.y + f.y, e.z + f.z}, {0.0f, 1.0f, 0.0f});
    } else {   // look-at
        view = look_at({cam.eye[0], cam.eye[1], cam.eye[2]}, {cam.center[0], cam.center[1], cam.center[2]},
                       {0.0f, 1.0f, 0.0f});
    }
    if (cam.camera_type == 0) {
        proj = perspective_zo(cam.horizontal_fov * d2r, cam.extent[0] / cam.extent[1], cam.near_distance,
                              cam.far_distance);
    } else {
        float sx = cam.zoom, sy = cam.extent[1] / cam.extent[0] * cam.zoom;
        proj = ortho_zo(-sx, sx, -sy, sy, cam.ortho_near_distance, cam.ortho_far_distance);
    }
    proj[5] *= -1.0f;   // AssetManager.cpp:375
    M4 jit = identity();
    jit[12] = cam.jitter[0];
    jit[13] = cam.jitter[1];
    proj = mul(jit, proj);   // GetProjJittered
}

// ---------------------------------------------------------------- meshes

luz_vertex vert(float px, float py, float pz, float nx, float ny, float nz) {
    luz_vertex v;
    memset(&v, 0, sizeof(v));
    v.position[0] = px; v.position[1] = py; v.position[2] = pz;
    v.normal[0] = nx; v.normal[1] = ny; v.normal[2] = nz;
    return v;
}

Mesh make_quad(float half) {
    Mesh m;
    m.v = {vert(-half, 0, -half, 0, 1, 0), vert(half, 0, -half, 0, 1, 0), vert(half, 0, half, 0, 1, 0),
           vert(-half, 0, half, 0, 1, 0)};
    m.i = {0, 2, 1, 0, 3, 2};
    return m;
}

// Unit cube [-0.5, 0.5]^3, 24 vertices with face normals, 12 triangles.
Mesh make_cube() {
    Mesh m;
    const float h = 0.5f;
    const float faces[6][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
    for (int f = 0; f < 6; ++f) {
        F3 n = {faces[f][0], faces[f][1], faces[f][2]};
        F3 u = std::fabs(n.y) > 0.5f ? F3{1, 0, 0} : F3{0, 1, 0};
        F3 t = crossf(u, n);
        F3 b = crossf(n, t);
        uint32_t base = (uint32_t)m.v.size();
        const float sgn[4][2] = {{-1, -1}, {1, -1}, {1, 1}, {-1, 1}};
        for (int k = 0; k < 4; ++k) {
            float px = (n.x + sgn[k][0] * t.x + sgn[k][1] * b.x) * h;
            float py = (n.y + sgn[k][0] * t.y + sgn[k][1] * b.y) * h;
            float pz = (n.z + sgn[k][0] * t.z + sgn[k][1] * b.z) * h;
            m.v.push_back(vert(px, py, pz, n.x, n.y, n.z));
        }
        m.i.insert(m.i.end(), {base, base + 1, base + 2, base, base + 2, base + 3});
    }
    return m;
}

// Icosphere: icosahedron subdivided `level` times by edge midpoints projected to the
// unit sphere (20 * 4^level triangles, 10 * 4^level + 2 vertices).
Mesh make_icosphere(int level) {
    const float t = (1.0f + std::sqrt(5.0f)) / 2.0f;
    std::vector<F3> p = {{-1, t, 0}, {1, t, 0}, {-1, -t, 0}, {1, -t, 0}, {0, -1, t}, {0, 1, t},
                         {0, -1, -t}, {0, 1, -t}, {t, 0, -1}, {t, 0, 1}, {-t, 0, -1}, {-t, 0, 1}};
    for (auto& q : p) q = normf(q);
    std::vector<uint32_t> tri = {0, 11, 5, 0, 5, 1, 0, 1, 7, 0, 7, 10, 0, 10, 11, 1, 5, 9, 5, 11, 4,
                                 11, 10, 2, 10, 7, 6, 7, 1, 8, 3, 9, 4, 3, 4, 2, 3, 2, 6, 3, 6, 8,
                                 3, 8, 9, 4, 9, 5, 2, 4, 11, 6, 2, 10, 8, 6, 7, 9, 8, 1};
    for (int l = 0; l < level; ++l) {
        std::map<std::pair<uint32_t, uint32_t>, uint32_t> mid;
        auto midpoint = [&](uint32_t a, uint32_t b) {
            auto key = std::make_pair(std::min(a, b), std::max(a, b));
            auto it = mid.find(key);
            if (it != mid.end()) return it->second;
            F3 m = {(p[a].x + p[b].x) * 0.5f, (p[a].y + p[b].y) * 0.5f, (p[a].z + p[b].z) * 0.5f};
            p.push_back(normf(m));
            uint32_t id = (uint32_t)p.size() - 1;
            mid.emplace(key, id);
            return id;
        };
        std::vector<uint32_t> nt;
        nt.reserve(tri.size() * 4);
        for (size_t k = 0; k < tri.size(); k += 3) {
            uint32_t a = tri[k], b = tri[k + 1], c = tri[k + 2];
            uint32_t ab = midpoint(a, b), bc = midpoint(b, c), ca = midpoint(c, a);
            nt.insert(nt.end(), {a, ab, ca, b, bc, ab, c, ca, bc, ab, bc, ca});
        }
        tri.swap(nt);
    }
    Mesh m;
    m.v.resize(p.size());
    for (size_t k = 0; k < p.size(); ++k) m.v[k] = vert(p[k].x, p[k].y, p[k].z, p[k].x, p[k].y, p[k].z);
    m.i = tri;
    return m;
}

// Radial displacement by a sum of 8 spherical sinusoids, then area-weighted normals.
Mesh displace(const Mesh& base, Rng& rng, float amplitude) {
    struct Wave { F3 axis; float freq, phase; };
    Wave w[8];
    for (auto& wv : w) {
        float z = rng.uniform(-1.0f, 1.0f), a = rng.uniform(0.0f, 2.0f * luz::kPi);
        float r = std::sqrt(std::max(0.0f, 1.0f - z * z));
        float s, c;
        luz::sincos_(a, &s, &c);
        wv.axis = {r * c, r * s, z};
        wv.freq = (float)(1 + rng.below(8));
        wv.phase = rng.uniform(0.0f, 2.0f * luz::kPi);
    }
    Mesh m = base;
    for (auto& v : m.v) {
        F3 u = {v.position[0], v.position[1], v.position[2]};
        float r = 1.0f;
        for (auto& wv : w) {
            float s, c;
            luz::sincos_(wv.freq * dotf(u, wv.axis) + wv.phase, &s, &c);
            r += amplitude * s;
        }
        v.position[0] = u.x * r; v.position[1] = u.y * r; v.position[2] = u.z * r;
        v.normal[0] = v.normal[1] = v.normal[2] = 0.0f;
    }
    for (size_t k = 0; k < m.i.size(); k += 3) {
        luz_vertex &a = m.v[m.i[k]], &b = m.v[m.i[k + 1]], &c = m.v[m.i[k + 2]];
        F3 pa = {a.position[0], a.position[1], a.position[2]};
        F3 n = crossf(sub({b.position[0], b.position[1], b.position[2]}, pa),
                      sub({c.position[0], c.position[1], c.position[2]}, pa));
        for (luz_vertex* q : {&a, &b, &c}) {
            q->normal[0] += n.x; q->normal[1] += n.y; q->normal[2] += n.z;
        }
    }
    for (auto& v : m.v) {
        F3 n = normf({v.normal[0], v.normal[1], v.normal[2]});
        v.normal[0] = n.x; v.normal[1] = n.y; v.normal[2] = n.z;
    }
    return m;
}

}  // namespace

namespace {

luz_model default_model() {   // GPUScene.cpp:19-30
    luz_model m;
    memset(&m, 0, sizeof(m));
    M4 I = identity();
    memcpy(m.model_mat, I.data(), 64);
    m.color[0] = m.color[1] = m.color[2] = m.color[3] = 1.0f;
    m.roughness = 0.5f;
    m.ao_map = m.color_map = m.normal_map = m.emission_map = m.metallic_roughness_map = -1;
    m.vertex_buffer = m.index_buffer = -1;
    return m;
}

void random_material(luz_model& m, Rng& rng) {
    m.color[0] = rng.uniform();
    m.color[1] = rng.uniform();
    m.color[2] = rng.uniform();
    m.color[3] = 1.0f;
    m.metallic = rng.uniform();
    m.roughness = rng.uniform(0.05f, 1.0f);
}

luz_light make_light(int type, F3 pos, F3 dir, F3 color, float intensity, int samples) {
    luz_light l;
    memset(&l, 0, sizeof(l));
    l.color[0] = color.x; l.color[1] = color.y; l.color[2] = color.z;
    l.intensity = intensity;
    l.position[0] = pos.x; l.position[1] = pos.y; l.position[2] = pos.z;
    l.direction[0] = dir.x; l.direction[1] = dir.y; l.direction[2] = dir.z;
    const float d2r = 3.14159265358979323846f / 180.0f;
    l.inner_angle = 60.0f * d2r;   // LightNode defaults (AssetManager.hpp:201-202), GPUScene.cpp:244
    l.outer_angle = 50.0f * d2r;
    l.type = type;
    l.num_shadow_samples = samples;
    l.radius = 2.0f;               // LightNode default radius (AssetManager.hpp:200)
    l.shadow_map = -1;
    return l;
}

// Non-vertical unit direction pointing down at elevation in [30, 60] degrees.
F3 sun_direction(Rng& rng) {
    float az = rng.uniform(0.0f, 2.0f * luz::kPi);
    float el = rng.uniform(30.0f, 60.0f) * luz::kPi / 180.0f;
    float sa, ca, se, ce;
    luz::sincos_(az, &sa, &ca);
    luz::sincos_(el, &se, &ce);
    return normf({ce * ca, -se, ce * sa});
}

void set_model_matrix(luz_model& m, const M4& mat) { memcpy(m.model_mat, mat.data(), 64); }

M4 trs(F3 pos, const M4& rot, float scale) {
    M4 T = identity();
    T[12] = pos.x; T[13] = pos.y; T[14] = pos.z;
    M4 S = identity();
    S[0] = S[5] = S[10] = scale;
    return mul(mul(T, rot), S);
}

// Uniform random rotation (K. Shoemake, "Uniform random rotations", Graphics Gems III).
M4 random_rotation(Rng& rng) {
    float u1 = rng.uniform(), u2 = rng.uniform(), u3 = rng.uniform();
    float a = std::sqrt(1.0f - u1), b = std::sqrt(u1);
    float s2, c2, s3, c3;
    luz::sincos_(2.0f * luz::kPi * u2, &s2, &c2);
    luz::sincos_(2.0f * luz::kPi * u3, &s3, &c3);
    return quat_to_mat(b * c3, a * s2, a * c2, b * s3);
}

void update_block(luz_host_scene* s) {
    luz_camera upd;
    M4 view, proj;
    camera_matrices(s->camera, upd, view, proj);
    s->camera = upd;
    luz_scene& b = s->block;
    M4 vp = mul(proj, view);
    memcpy(b.prev_view_proj, s->prev_view_proj, 64);
    memcpy(b.proj, proj.data(), 64);
    memcpy(b.view, view.data(), 64);
    memcpy(b.view_proj, vp.data(), 64);
    M4 ip = inverse(proj), iv = inverse(view);
    memcpy(b.inverse_proj, ip.data(), 64);
    memcpy(b.inverse_view, iv.data(), 64);
    b.prev_jitter[0] = b.jitter[0];
    b.prev_jitter[1] = b.jitter[1];
    b.jitter[0] = s->camera.jitter[0];
    b.jitter[1] = s->camera.jitter[1];
    b.cam_pos[0] = s->camera.eye[0];
    b.cam_pos[1] = s->camera.eye[1];
    b.cam_pos[2] = s->camera.eye[2];
    b.num_lights = (int32_t)s->lights.size();
    memcpy(s->prev_view_proj, vp.data(), 64);
}

luz_camera look_camera(F3 eye, F3 center, float fovy, uint32_t w, uint32_t h, float zn, float zf) {
    luz_camera c;
    memset(&c, 0, sizeof(c));
    c.camera_type = 0;
    c.mode = 2;
    c.eye[0] = eye.x; c.eye[1] = eye.y; c.eye[2] = eye.z;
    c.center[0] = center.x; c.center[1] = center.y; c.center[2] = center.z;
    c.zoom = 10.0f;
    c.far_distance = zf;
    c.near_distance = zn;
    c.horizontal_fov = fovy;
    c.ortho_far_distance = 10.0f;
    c.ortho_near_distance = -100.0f;
    c.extent[0] = (float)w;
    c.extent[1] = (float)h;
    return c;
}

void gen_cubes(luz_host_scene* s, const luz_gen_params& p, Rng& rng, bool random_camera) {
    s->meshes.push_back(make_quad(10.0f));
    s->meshes.push_back(make_cube());
    luz_model ground = default_model();
    random_material(ground, rng);
    s->models.push_back(ground);
    s->instance_mesh.push_back(0);
    uint32_t cubes = p.instances ? p.instances : 64;
    for (uint32_t k = 0; k < cubes; ++k) {
        luz_model m = default_model();
        float pos[3] = {rng.uniform(-8.0f, 8.0f), rng.uniform(0.0f, 4.0f), rng.uniform(-8.0f, 8.0f)};
        float rot[3] = {0.0f, rng.uniform(0.0f, 360.0f), 0.0f};
        float scl[3] = {1.0f, 1.0f, 1.0f};
        set_model_matrix(m, compose(pos, rot, scl, identity()));
        random_material(m, rng);
        s->models.push_back(m);
        s->instance_mesh.push_back(1);
    }
    int ls = p.light_samples > 0 ? p.light_samples : 1;
    uint32_t ndir = p.directional_lights ? p.directional_lights : 1;
    uint32_t npt = p.point_lights ? p.point_lights : 4;
    for (uint32_t k = 0; k < ndir; ++k) {
        F3 d = sun_direction(rng);
        F3 pos = {-d.x * 1e4f, -d.y * 1e4f, -d.z * 1e4f};   // node far up-light
        s->lights.push_back(make_light(LUZ_LIGHT_DIRECTIONAL, pos, d, {1, 1, 1}, rng.uniform(1.0f, 3.0f), ls));
    }
    for (uint32_t k = 0; k < npt; ++k) {
        F3 pos = {rng.uniform(-8.0f, 8.0f), rng.uniform(3.0f, 8.0f), rng.uniform(-8.0f, 8.0f)};
        F3 col = {rng.uniform(0.5f, 1.0f), rng.uniform(0.5f, 1.0f), rng.uniform(0.5f, 1.0f)};
        s->lights.push_back(make_light(LUZ_LIGHT_POINT, pos, {0, -1, 0}, col, rng.uniform(1.0f, 10.0f), ls));
    }
    F3 eye = {0.0f, 10.0f, 16.0f}, center = {0.0f, 0.0f, 0.0f};
    if (random_camera) {
        float az = rng.uniform(0.0f, 2.0f * luz::kPi), el = rng.uniform(15.0f, 60.0f) * luz::kPi / 180.0f;
        float dist = rng.uniform(10.0f, 22.0f);
        float sa, ca, se, ce;
        luz::sincos_(az, &sa, &ca);
        luz::sincos_(el, &se, &ce);
        eye = {dist * ce * ca, dist * se, dist * ce * sa};
        center = {rng.uniform(-3.0f, 3.0f), rng.uniform(0.0f, 1.5f), rng.uniform(-3.0f, 3.0f)};
    }
    s->camera = look_camera(eye, center, 60.0f, s->width, s->height, 0.01f, 1000.0f);
}

std::vector<Mesh> displaced_spheres(uint32_t count, int level, Rng& rng) {
    Mesh base = make_icosphere(level);
    std::vector<Mesh> out;
    out.reserve(count);
    for (uint32_t k = 0; k < count; ++k) out.push_back(displace(base, rng, 0.05f));
    return out;
}

void gen_spheres(luz_host_scene* s, const luz_gen_params& p, Rng& rng, uint32_t def_instances,
                 uint32_t def_point, uint32_t def_spot) {
    uint32_t nmesh = p.meshes ? p.meshes : 64;
    int level = p.subdivisions ? (int)p.subdivisions : 6;
    s->meshes = displaced_spheres(nmesh, level, rng);
    uint32_t ninst = p.instances ? p.instances : def_instances;
    const float half = 100.0f;
    for (uint32_t k = 0; k < ninst; ++k) {
        luz_model m = default_model();
        F3 pos = {rng.uniform(-half, half), rng.uniform(-half, half), rng.uniform(-half, half)};
        M4 R = random_rotation(rng);
        float sc = rng.uniform(0.5f, 2.0f);
        set_model_matrix(m, trs(pos, R, sc));
        random_material(m, rng);
        s->models.push_back(m);
        s->instance_mesh.push_back(rng.below(nmesh));
    }
    int ls = p.light_samples > 0 ? p.light_samples : 1;
    uint32_t ndir = p.directional_lights ? p.directional_lights : 1;
    uint32_t npt = p.point_lights ? p.point_lights : def_point;
    uint32_t nspot = p.spot_lights ? p.spot_lights : def_spot;
    for (uint32_t k = 0; k < ndir; ++k) {
        F3 d = sun_direction(rng);
        F3 pos = {-d.x * 1e4f, -d.y * 1e4f, -d.z * 1e4f};
        s->lights.push_back(make_light(LUZ_LIGHT_DIRECTIONAL, pos, d, {1, 1, 1}, rng.uniform(1.0f, 3.0f), ls));
    }
    for (uint32_t k = 0; k < npt; ++k) {
        F3 pos = {rng.uniform(-half, half), rng.uniform(-half, half), rng.uniform(-half, half)};
        F3 col = {rng.uniform(0.5f, 1.0f), rng.uniform(0.5f, 1.0f), rng.uniform(0.5f, 1.0f)};
        s->lights.push_back(make_light(LUZ_LIGHT_POINT, pos, {0, -1, 0}, col, rng.uniform(100.0f, 1000.0f), ls));
    }
    for (uint32_t k = 0; k < nspot; ++k) {
        F3 pos = {rng.uniform(-half, half), rng.uniform(-half, half), rng.uniform(-half, half)};
        F3 tgt = {rng.uniform(-half, half) * 0.5f, rng.uniform(-half, half) * 0.5f, rng.uniform(-half, half) * 0.5f};
        F3 dir = normf(sub(tgt, pos));
        F3 col = {rng.uniform(0.5f, 1.0f), rng.uniform(0.5f, 1.0f), rng.uniform(0.5f, 1.0f)};
        s->lights.push_back(make_light(LUZ_LIGHT_SPOT, pos, dir, col, rng.uniform(100.0f, 1000.0f), ls));
    }
    // Camera at the centre of the instance cloud looking along +z (about 23% of the
    // pixels see geometry; from outside the box only about 4% would).
    s->camera = look_camera({0.0f, 0.0f, 0.0f}, {0.0f, 0.0f, 100.0f}, 60.0f, s->width, s->height, 0.1f, 2000.0f);
}

// One scene of the batched workload: a triangle budget filled either with cubes on a
// quad (small budgets) or with displaced icospheres of the needed subdivision.
void gen_budget(luz_host_scene* s, const luz_gen_params& p, Rng& rng) {
    uint32_t budget = p.triangles ? p.triangles : 100000;
    if (budget < 20000) {
        luz_gen_params q = p;
        q.instances = std::max(1u, (budget - 2) / 12);
        gen_cubes(s, q, rng, false);
        return;
    }
    int level = 2;
    while (level < 7 && 20u * (1u << (2 * (level + 1))) <= budget / 8) ++level;
    uint32_t per = 20u * (1u << (2 * level));
    uint32_t nmesh = std::max(1u, std::min(64u, budget / per));
    luz_gen_params q = p;
    q.meshes = nmesh;
    q.subdivisions = (uint32_t)level;
    q.instances = std::max(1u, (budget + per / 2) / per);   // instanced triangles ~ the budget
    gen_spheres(s, q, rng, q.instances, 8, 2);
}

}  // namespace

namespace luz {
namespace host {
luz_model default_model() { return ::default_model(); }
void refresh_block(luz_host_scene* s) {
    update_block(s);
    update_block(s);   // prevViewProj = viewProj for a static camera
}
void compose_transform(const float pos[3], const float rot_deg[3], const float scl[3], const float parent[16],
                       float out[16]) {
    M4 par = identity();
    if (parent) memcpy(par.data(), parent, 64);
    M4 r = compose(pos, rot_deg, scl, par);
    memcpy(out, r.data(), 64);
}
}  // namespace host
}  // namespace luz

extern "C" {

luz_status luz_scene_default_params(int32_t config, luz_gen_params* out) {
    if (!out) return LUZ_ERR_INVALID;
    memset(out, 0, sizeof(*out));
    out->config = config;
    out->seed = 1000 + (uint64_t)config;
    out->ao_samples = -1;
    out->light_samples = 1;
    out->sampler = LUZ_SAMPLER_PARITY;
    switch (config) {
        case 1: case 3: out->width = 512; out->height = 512; break;
        case 2: out->width = 1920; out->height = 1080; break;
        case 5: out->width = 3840; out->height = 2160; break;
        case 6: out->width = 512; out->height = 512; out->triangles = 100000; break;
        default: return LUZ_ERR_INVALID;
    }
    return LUZ_OK;
}

}  // extern "C"

namespace {
constexpr uint32_t kMaxSubdivisions = 10;   // luz_gen_params::subdivisions

// The generator behind luz_scene_generate; throws std::bad_alloc when the scene the
// parameters ask for does not fit in host memory.
luz_status generate_scene(const luz_gen_params* p, luz_host_scene** out) {
    std::unique_ptr<luz_host_scene> owner(new luz_host_scene());
    luz_host_scene* s = owner.get();
    s->width = p->width;
    s->height = p->height;
    Rng rng(p->seed);
    int ao_default = 4;
    float ao_max_default = 1.0f;
    switch (p->config) {
        case 1: gen_cubes(s, *p, rng, false); break;
        case 3: gen_cubes(s, *p, rng, true); break;
        case 2: gen_spheres(s, *p, rng, 1024, 32, 8); ao_default = 16; ao_max_default = 2.0f; break;
        case 5: gen_spheres(s, *p, rng, 4096, 128, 16); ao_default = 64; ao_max_default = 2.0f; break;
        case 6: gen_budget(s, *p, rng); break;
        default: return LUZ_ERR_INVALID;
    }
    luz_scene& b = s->block;
    memset(&b, 0, sizeof(b));
    b.ambient_light_color[0] = b.ambient_light_color[1] = b.ambient_light_color[2] = 1.0f;
    b.ambient_light_intensity = 0.2f;
    b.ao_min = 0.0001f;
    b.ao_max = p->ao_max > 0.0f ? p->ao_max : ao_max_default;
    b.ao_num_samples = p->ao_samples >= 0 ? p->ao_samples : ao_default;
    b.exposure = 2.0f;
    b.white_texture = b.black_texture = -1;
    b.blue_noise_texture = 0;
    b.tlas_rid = 0;
    b.shadow_type = LUZ_SHADOW_RAYTRACING;
    b.sampler = p->sampler;
    s->light_samples = p->light_samples > 0 ? p->light_samples : 1;
    for (auto& l : s->lights) l.num_shadow_samples = s->light_samples;
    update_block(s);
    update_block(s);   // prevViewProj = viewProj for a static camera
    *out = owner.release();
    return LUZ_OK;
}
}  // namespace

extern "C" {

luz_status luz_scene_generate(const luz_gen_params* p, luz_host_scene** out) {
    if (!p || !out) return LUZ_ERR_INVALID;
    *out = nullptr;
    if (p->width == 0 || p->height == 0) return LUZ_ERR_INVALID;
    // 20 x 4^10 triangles per icosphere at most (its vertex count stays far inside
    // the 32-bit index range)
    if (p->subdivisions > kMaxSubdivisions) return LUZ_ERR_LIMIT;
    try {
        return generate_scene(p, out);
    } catch (const std::bad_alloc&) {
        return LUZ_ERR_OOM;
    } catch (const std::exception&) {
        return LUZ_ERR_INVALID;
    }
}


void luz_scene_destroy(luz_host_scene* s) { delete s; }

uint32_t luz_scene_texture_count(const luz_host_scene* s) { return s ? (uint32_t)s->textures.size() : 0; }

luz_status luz_scene_texture(const luz_host_scene* s, uint32_t i, const uint8_t** rgba8, uint32_t* width,
                             uint32_t* height) {
    if (!s || i >= s->textures.size()) return LUZ_ERR_INVALID;
    const luz::host::Texture& t = s->textures[i];
    if (rgba8) *rgba8 = t.rgba.data();
    if (width) *width = t.width;
    if (height) *height = t.height;
    return LUZ_OK;
}

uint32_t luz_scene_mesh_count(const luz_host_scene* s) { return s ? (uint32_t)s->meshes.size() : 0; }

luz_status luz_scene_mesh(const luz_host_scene* s, uint32_t i, const luz_vertex** v, uint32_t* nv,
                          const uint32_t** idx, uint32_t* ni) {
    if (!s || i >= s->meshes.size()) return LUZ_ERR_INVALID;
    const Mesh& m = s->meshes[i];
    if (v) *v = m.v.data();
    if (nv) *nv = (uint32_t)m.v.size();
    if (idx) *idx = m.i.data();
    if (ni) *ni = (uint32_t)m.i.size();
    return LUZ_OK;
}

uint32_t luz_scene_instance_count(const luz_host_scene* s) { return s ? (uint32_t)s->models.size() : 0; }
const uint32_t* luz_scene_instance_mesh(const luz_host_scene* s) { return s ? s->instance_mesh.data() : nullptr; }
const luz_model* luz_scene_models(const luz_host_scene* s) { return s ? s->models.data() : nullptr; }
uint32_t luz_scene_light_count(const luz_host_scene* s) { return s ? (uint32_t)s->lights.size() : 0; }
const luz_light* luz_scene_lights(const luz_host_scene* s) { return s ? s->lights.data() : nullptr; }
const luz_scene* luz_scene_block(const luz_host_scene* s) { return s ? &s->block : nullptr; }
uint32_t luz_scene_width(const luz_host_scene* s) { return s ? s->width : 0; }
uint32_t luz_scene_height(const luz_host_scene* s) { return s ? s->height : 0; }

luz_status luz_scene_instance_transforms(const luz_host_scene* s, float* out) {
    if (!s || !out) return LUZ_ERR_INVALID;
    for (size_t k = 0; k < s->models.size(); ++k) {
        const float* m = s->models[k].model_mat;
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 4; ++c) out[k * 12 + r * 4 + c] = m[c * 4 + r];
    }
    return LUZ_OK;
}

luz_status luz_scene_set_camera(luz_host_scene* s, const luz_camera* cam) {
    if (!s || !cam) return LUZ_ERR_INVALID;
    s->camera = *cam;
    update_block(s);
    return LUZ_OK;
}

luz_status luz_scene_get_camera(const luz_host_scene* s, luz_camera* cam) {
    if (!s || !cam) return LUZ_ERR_INVALID;
    *cam = s->camera;
    return LUZ_OK;
}

luz_status luz_scene_set_shadow_type(luz_host_scene* s, int32_t shadow_type) {
    if (!s || shadow_type < LUZ_SHADOW_DISABLED || shadow_type > LUZ_SHADOW_MAP) return LUZ_ERR_INVALID;
    s->block.shadow_type = shadow_type;
    for (auto& l : s->lights) l.num_shadow_samples = shadow_type == LUZ_SHADOW_RAYTRACING ? s->light_samples : 0;
    return LUZ_OK;
}

luz_status luz_scene_shadow_lights(const luz_host_scene* s, luz_shadow_light* out) {
    if (!s || (!out && !s->lights.empty())) return LUZ_ERR_INVALID;
    const float d2r = 0.01745329251994329576923690768489f;
    const luz_camera& cam = s->camera;
    M4 view;
    memcpy(view.data(), s->block.view, 64);
    for (size_t k = 0; k < s->lights.size(); ++k) {
        const luz_light& l = s->lights[k];
        luz_shadow_light& o = out[k];
        memset(&o, 0, sizeof(o));
        float range = k < s->shadow_range.size() ? s->shadow_range[k] : 3.0f;
        float zfar = k < s->shadow_far.size() ? s->shadow_far[k] : 2000.0f;
        o.z_far = zfar;
        memcpy(o.position, l.position, 12);
        F3 pos = {l.position[0], l.position[1], l.position[2]};
        if (l.type == LUZ_LIGHT_POINT) {
            o.faces = 6;
            M4 proj = perspective_zo(90.0f * d2r, 1.0f, 0.0f, zfar);
            const F3 dirs[6] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
            const F3 ups[6] = {{0, -1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}, {0, -1, 0}, {0, -1, 0}};
            for (int f = 0; f < 6; ++f) {
                M4 vp = mul(proj, look_at(pos, {pos.x + dirs[f].x, pos.y + dirs[f].y, pos.z + dirs[f].z}, ups[f]));
                memcpy(o.view_proj[f], vp.data(), 64);
            }
        } else {
            o.faces = 1;
            // camera->GetProj(near, far / range): no jitter, y flipped
            M4 cp;
            if (cam.camera_type == 0) {
                cp = perspective_zo(cam.horizontal_fov * d2r, cam.extent[0] / cam.extent[1], cam.near_distance,
                                    cam.far_distance / range);
            } else {
                float sx = cam.zoom, sy = cam.extent[1] / cam.extent[0] * cam.zoom;
                cp = ortho_zo(-sx, sx, -sy, sy, cam.ortho_near_distance, cam.ortho_far_distance);
            }
            cp[5] *= -1.0f;
            M4 inv = inverse(mul(cp, view));
            float corners[8][4];
            int c = 0;
            for (int i = 0; i < 2; ++i)
                for (int j = 0; j < 2; ++j)
                    for (int kk = 0; kk < 2; ++kk, ++c) {
                        float pt[4] = {2.0f * i - 1.0f, 2.0f * j - 1.0f, 2.0f * kk - 1.0f, 1.0f};
                        float r[4];
                        for (int q = 0; q < 4; ++q)
                            r[q] = inv[q] * pt[0] + inv[4 + q] * pt[1] + inv[8 + q] * pt[2] + inv[12 + q] * pt[3];
                        for (int q = 0; q < 4; ++q) corners[c][q] = r[q] / r[3];
                    }
            F3 center = {0.0f, 0.0f, 0.0f};
            for (int q = 0; q < 8; ++q) center = {center.x + corners[q][0], center.y + corners[q][1], center.z + corners[q][2]};
            center = {center.x / 8.0f, center.y / 8.0f, center.z / 8.0f};
            F3 front = {l.direction[0], l.direction[1], l.direction[2]};
            M4 lv = look_at({center.x + front.x, center.y + front.y, center.z + front.z}, center, {0.0f, 1.0f, 0.0f});
            // the reference starts min / max at the world-space corner 0 (GPUScene.cpp:292-293)
            float mn[3] = {corners[0][0], corners[0][1], corners[0][2]}, mx[3] = {mn[0], mn[1], mn[2]};
            for (int q = 0; q < 8; ++q) {
                float v[3];
                for (int a = 0; a < 3; ++a)
                    v[a] = lv[a] * corners[q][0] + lv[4 + a] * corners[q][1] + lv[8 + a] * corners[q][2] +
                           lv[12 + a] * corners[q][3];
                for (int a = 0; a < 3; ++a) {
                    mn[a] = mn[a] < v[a] ? mn[a] : v[a];
                    mx[a] = v[a] < mx[a] ? mx[a] : v[a];
                }
            }
            mn[2] = mn[2] < 0 ? mn[2] * range : mn[2] / range;
            mx[2] = mx[2] < 0 ? mx[2] / range : mx[2] * range;
            M4 proj = ortho_zo(mn[0], mx[0], mn[1], mx[1], mx[2], mn[2]);
            M4 vp = mul(proj, lv);
            memcpy(o.view_proj[0], vp.data(), 64);
        }
    }
    return LUZ_OK;
}

// Util.hpp Halton(i, b), single precision.
static float halton(uint32_t i, uint32_t b) {
    float f = 1.0f, r = 0.0f;
    while (i > 0) {
        f /= (float)b;
        r = r + f * (float)(i % b);
        i = (uint32_t)std::floor((float)i / (float)b);
    }
    return r;
}

luz_status luz_scene_next_frame(luz_host_scene* s, int32_t use_jitter) {
    if (!s) return LUZ_ERR_INVALID;
    luz_camera& c = s->camera;
    if (use_jitter) {   // CameraNode::NextJitter (AssetManager.cpp:383-392)
        s->jitter_index = (s->jitter_index + 1) % 16;
        float jx = halton(s->jitter_index + 1, 2), jy = halton(s->jitter_index + 1, 3);
        c.jitter[0] = (2.0f * jx - 1.0f) / c.extent[0];
        c.jitter[1] = (2.0f * jy - 1.0f) / c.extent[1];
    } else {
        c.jitter[0] = c.jitter[1] = 0.0f;
    }
    update_block(s);
    return LUZ_OK;
}

luz_status luz_scene_set_sampling(luz_host_scene* s, int32_t ao_samples, float ao_min, float ao_max,
                                  int32_t light_samples, int32_t sampler) {
    if (!s || ao_samples < 0 || light_samples < 0) return LUZ_ERR_INVALID;
    s->block.ao_num_samples = ao_samples;
    s->block.ao_min = ao_min;
    s->block.ao_max = ao_max;
    s->block.sampler = sampler;
    s->light_samples = light_samples;
    for (auto& l : s->lights) l.num_shadow_samples = light_samples;
    return LUZ_OK;
}

void luz_compose_transform(const float pos[3], const float rot_deg[3], const float scale[3],
                           const float* parent, float out[16]) {
    if (!out) return;
    static const float zero[3] = {0.0f, 0.0f, 0.0f}, one[3] = {1.0f, 1.0f, 1.0f};   // a Node's defaults
    M4 par = identity();
    if (parent) memcpy(par.data(), parent, 64);
    M4 r = compose(pos ? pos : zero, rot_deg ? rot_deg : zero, scale ? scale : one, par);
    memcpy(out, r.data(), 64);
}

void luz_camera_matrices(const luz_camera* cam, float view[16], float proj[16]) {
    if (!cam) return;
    luz_camera upd;
    M4 v, p;
    camera_matrices(*cam, upd, v, p);
    if (view) memcpy(view, v.data(), 64);
    if (proj) memcpy(proj, p.data(), 64);
}

luz_status luz_blue_noise_generate(uint64_t seed, uint32_t size, uint8_t* rgba8) {
    if (!rgba8 || size == 0) return LUZ_ERR_INVALID;
    for (uint32_t y = 0; y < size; ++y)
        for (uint32_t x = 0; x < size; ++x) {
            uint32_t h = luz::hash32(x + 0x9E3779B9u * (y + 1) + (uint32_t)seed * 0x85EBCA6Bu + (uint32_t)(seed >> 32));
            uint32_t h2 = luz::hash32(h ^ 0xC2B2AE35u);
            uint8_t* px = rgba8 + 4 * ((size_t)y * size + x);
            px[0] = (uint8_t)(h & 0xFF);
            px[1] = (uint8_t)((h >> 8) & 0xFF);
            px[2] = (uint8_t)(h2 & 0xFF);
            px[3] = 255;
        }
    return LUZ_OK;
}

}  // extern "C"
