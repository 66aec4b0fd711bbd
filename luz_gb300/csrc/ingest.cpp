// ingest.cpp — scene files into host scenes: the reference's project format (.luz
// JSON + .luzbin binary storage), glTF 2.0 (.gltf / .glb) and Wavefront OBJ (+ MTL),
// and the .luz/.luzbin writer. C++17, no CUDA, no third-party code.
//
// The object model mirrors the reference's asset manager
// (source/Resources/AssetManager.hpp:14-300): texture, mesh and material assets
// referenced by 64-bit UUIDs, and scenes holding trees of nodes (Node, MeshNode,
// LightNode, CameraNode) with position / Euler rotation in degrees / scale. A loaded
// scene becomes a luz_host_scene the way GPUScene::UpdateResources packs one
// (source/Graphics/GPUScene.cpp:181-346): every MeshNode of a pre-order walk is an
// instance with a ModelBlock, every LightNode a LightBlock.
#include <algorithm>
#include <array>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <functional>
#include <map>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>

#include "json.hpp"
#include "png.hpp"
#include "scene_internal.hpp"

namespace luz {
namespace ingest {

using json::Value;

// Deepest node tree a scene may have (project files and glTF alike): the readers
// and the packing walk recurse once per level.
constexpr int kMaxNodeDepth = 512;

// ---------------------------------------------------------------- object model
enum ObjType : int {   // ObjectType (AssetManager.hpp:14-25)
    kTexture = 1, kMesh = 2, kMaterial = 3, kScene = 4, kNode = 5, kMeshNode = 6, kLightNode = 7, kCameraNode = 8
};

struct TextureAsset {
    uint64_t uuid = 0;
    std::string name;
    int32_t width = 0, height = 0, channels = 4;
    std::vector<uint8_t> data;   // RGBA8
};

struct MeshAsset {
    uint64_t uuid = 0;
    std::string name;
    std::vector<luz_vertex> vertices;
    std::vector<uint32_t> indices;
};

struct MaterialAsset {   // defaults: AssetManager.hpp:101-111
    uint64_t uuid = 0;
    std::string name;
    float color[4] = {1, 1, 1, 1};
    float emission[3] = {0, 0, 0};
    float metallic = 0.0f, roughness = 0.5f;
    uint64_t ao_map = 0, color_map = 0, normal_map = 0, emission_map = 0, mr_map = 0;
};

struct Node {
    int type = kNode;
    uint64_t uuid = 0;
    std::string name;
    float position[3] = {0, 0, 0}, rotation[3] = {0, 0, 0}, scale[3] = {1, 1, 1};
    bool has_matrix = false;     // exact local matrix (written by this library's saver)
    float matrix[16] = {};
    std::vector<Node> children;
    // MeshNode
    uint64_t mesh = 0, material = 0;
    // LightNode (AssetManager.hpp:200-227)
    float color[3] = {1, 1, 1};
    float intensity = 10.0f;
    int32_t light_type = 0;
    float radius = 2.0f, inner_angle = 60.0f, outer_angle = 50.0f;
    float shadow_map_range = 3.0f, shadow_map_far = 2000.0f;
    int32_t volumetric_type = 1;
    bool has_direction = false;  // exact direction (this library's saver)
    float direction[3] = {0, -1, 0};
    // CameraNode (AssetManager.hpp:246-261)
    int32_t camera_type = 0, mode = 0;
    float eye[3] = {0, 0, 0}, center[3] = {0, 0, 0};
    float zoom = 10.0f, far_distance = 1000.0f, near_distance = 0.01f, horizontal_fov = 60.0f;
    float ortho_far = 10.0f, ortho_near = -100.0f;
};

struct SceneAsset {   // defaults: AssetManager.hpp:280-296
    uint64_t uuid = 0;
    std::string name;
    std::vector<Node> nodes;
    float ambient_color[3] = {1, 1, 1};
    float ambient_light = 0.01f;
    int32_t ao_samples = 4, light_samples = 2;
    float ao_min = 0.0001f, ao_max = 1.0f, exposure = 2.0f;
    int32_t shadow_type = 1;
    bool taa_enabled = true, taa_reconstruct = true;
    uint64_t main_camera = 0;
};

struct Project {
    std::vector<TextureAsset> textures;
    std::vector<MeshAsset> meshes;
    std::vector<MaterialAsset> materials;
    std::vector<SceneAsset> scenes;
    uint64_t initial_scene = 0;

    const TextureAsset* texture(uint64_t id) const {
        for (const auto& t : textures) if (t.uuid == id) return &t;
        return nullptr;
    }
    const MeshAsset* mesh(uint64_t id) const {
        for (const auto& m : meshes) if (m.uuid == id) return &m;
        return nullptr;
    }
    const MaterialAsset* material(uint64_t id) const {
        for (const auto& m : materials) if (m.uuid == id) return &m;
        return nullptr;
    }
};

[[noreturn]] void fail(const std::string& what) { throw std::runtime_error(what); }

// Deterministic UUIDs in [2^61, 2^62] (the reference draws them at random in that range).
struct UuidGen {
    uint64_t s;
    explicit UuidGen(uint64_t seed) : s(seed) {}
    uint64_t next() {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        return (1ull << 61) + z % (1ull << 61);
    }
};

// ---------------------------------------------------------------- files
std::vector<uint8_t> read_bytes(const std::string& path) {
    std::ifstream f(path, std::ios::binary);
    if (!f) fail("cannot open " + path);
    return std::vector<uint8_t>((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
}
std::string read_text(const std::string& path) {
    std::vector<uint8_t> b = read_bytes(path);
    return std::string(b.begin(), b.end());
}
void write_bytes(const std::string& path, const void* data, size_t n) {
    std::ofstream f(path, std::ios::binary);
    if (!f) fail("cannot write " + path);
    f.write((const char*)data, (std::streamsize)n);
    if (!f) fail("write failed: " + path);
}
std::string dir_of(const std::string& path) {
    size_t k = path.find_last_of('/');
    return k == std::string::npos ? std::string() : path.substr(0, k + 1);
}
std::string stem_of(const std::string& path) {
    size_t a = path.find_last_of('/');
    std::string f = a == std::string::npos ? path : path.substr(a + 1);
    size_t d = f.find_last_of('.');
    return d == std::string::npos ? f : f.substr(0, d);
}
std::string ext_of(const std::string& path) {
    size_t d = path.find_last_of('.');
    size_t a = path.find_last_of('/');
    if (d == std::string::npos || (a != std::string::npos && d < a)) return "";
    std::string e = path.substr(d);
    for (auto& c : e) c = (char)tolower((unsigned char)c);
    return e;
}

// ---------------------------------------------------------------- .luz reader
// Field readers of the reference's Serializer (source/Resources/Serializer.hpp:8-31):
// a vec3 / vec4 is read only from an array of exactly that length.
void get_f(const Value& j, const char* k, float& out) { if (const Value* v = j.find(k)) if (v->is_num()) out = v->f32(); }
void get_i(const Value& j, const char* k, int32_t& out) { if (const Value* v = j.find(k)) if (v->is_num()) out = (int32_t)v->i64(); }
void get_b(const Value& j, const char* k, bool& out) {
    if (const Value* v = j.find(k)) out = v->kind == Value::Bool ? v->b : v->num() != 0.0;
}
void get_u(const Value& j, const char* k, uint64_t& out) { if (const Value* v = j.find(k)) if (v->is_num()) out = v->u64(); }
void get_v(const Value& j, const char* k, float* out, size_t n) {
    const Value* v = j.find(k);
    if (!v || !v->is_arr() || v->size() != n) return;
    for (size_t a = 0; a < n; ++a) out[a] = (*v)[a].f32();
}
void get_s(const Value& j, const char* k, std::string& out) {
    if (const Value* v = j.find(k)) if (v->kind == Value::String) out = v->s;
}

// Serializer::Vector (Serializer.hpp:93-109): {offset, size} into the binary storage.
template <typename T>
void get_blob(const Value& j, const char* k, const std::vector<uint8_t>& bin, std::vector<T>& out) {
    const Value* v = j.find(k);
    if (!v) return;
    uint64_t off = v->at("offset").u64(), size = v->at("size").u64();
    if (off > bin.size() || size > bin.size() - off) fail(std::string("binary range of '") + k + "' is outside the .luzbin file");
    if (size % sizeof(T)) fail(std::string("binary size of '") + k + "' is not a whole number of elements");
    out.resize(size / sizeof(T));
    if (size) memcpy(out.data(), bin.data() + off, size);
}

Node read_node(const Value& j, int depth) {
    if (depth > kMaxNodeDepth) fail("node tree too deep");
    Node n;
    n.type = (int)j.at("type").i64();
    get_s(j, "name", n.name);
    get_u(j, "uuid", n.uuid);
    get_v(j, "position", n.position, 3);
    get_v(j, "rotation", n.rotation, 3);
    get_v(j, "scale", n.scale, 3);
    if (const Value* m = j.find("luzMatrix"))
        if (m->is_arr() && m->size() == 16) {
            n.has_matrix = true;
            for (int k = 0; k < 16; ++k) n.matrix[k] = (*m)[k].f32();
        }
    if (const Value* c = j.find("children"))
        if (c->is_arr())
            for (const auto& cj : c->items) n.children.push_back(read_node(cj, depth + 1));
    switch (n.type) {
        case kNode: break;
        case kMeshNode:
            get_u(j, "mesh", n.mesh);
            get_u(j, "material", n.material);
            break;
        case kLightNode:
            get_v(j, "color", n.color, 3);
            get_f(j, "intensity", n.intensity);
            get_i(j, "lightType", n.light_type);
            get_f(j, "innerAngle", n.inner_angle);
            get_f(j, "outerAngle", n.outer_angle);
            get_f(j, "radius", n.radius);
            get_f(j, "shadowMapRange", n.shadow_map_range);
            get_f(j, "shadowMapFar", n.shadow_map_far);
            get_i(j, "volumetricType", n.volumetric_type);
            if (const Value* d = j.find("luzDirection"))
                if (d->is_arr() && d->size() == 3) {
                    n.has_direction = true;
                    for (int k = 0; k < 3; ++k) n.direction[k] = (*d)[k].f32();
                }
            break;
        case kCameraNode:
            get_i(j, "cameraType", n.camera_type);
            get_i(j, "mode", n.mode);
            get_v(j, "eye", n.eye, 3);
            get_v(j, "center", n.center, 3);
            get_f(j, "zoom", n.zoom);
            get_f(j, "farDistance", n.far_distance);
            get_f(j, "nearDistance", n.near_distance);
            get_f(j, "horizontalFov", n.horizontal_fov);
            get_f(j, "orthoFarDistance", n.ortho_far);
            get_f(j, "orthoNearDistance", n.ortho_near);
            break;
        default: fail("unknown node type " + std::to_string(n.type));
    }
    return n;
}

SceneAsset read_scene(const Value& j) {
    SceneAsset s;
    get_s(j, "name", s.name);
    get_u(j, "uuid", s.uuid);
    if (const Value* ns = j.find("nodes"))
        if (ns->is_arr())
            for (const auto& nj : ns->items) s.nodes.push_back(read_node(nj, 0));
    get_f(j, "ambientLight", s.ambient_light);
    get_v(j, "ambientLightColor", s.ambient_color, 3);
    get_i(j, "lightSamples", s.light_samples);
    get_i(j, "aoSamples", s.ao_samples);
    get_f(j, "aoMin", s.ao_min);
    get_f(j, "aoMax", s.ao_max);
    get_f(j, "exposure", s.exposure);
    get_i(j, "shadowType", s.shadow_type);
    get_b(j, "taaEnabled", s.taa_enabled);
    get_b(j, "taaReconstruct", s.taa_reconstruct);
    get_u(j, "mainCamera", s.main_camera);
    return s;
}

// AssetManager::LoadProject (AssetManager.cpp:183-211).
Project load_project(const std::string& luz_path, const std::string& bin_path) {
    Project p;
    Value j = json::parse(read_text(luz_path));
    std::vector<uint8_t> bin = read_bytes(bin_path);
    if (const Value* assets = j.find("assets"))
        for (const auto& a : assets->items) {
            int type = (int)a.at("type").i64();
            if (type == kTexture) {
                TextureAsset t;
                get_s(a, "name", t.name);
                get_u(a, "uuid", t.uuid);
                get_blob(a, "data", bin, t.data);
                get_i(a, "width", t.width);
                get_i(a, "height", t.height);
                get_i(a, "channels", t.channels);
                p.textures.push_back(std::move(t));
            } else if (type == kMesh) {
                MeshAsset m;
                get_s(a, "name", m.name);
                get_u(a, "uuid", m.uuid);
                get_blob(a, "vertices", bin, m.vertices);
                get_blob(a, "indices", bin, m.indices);
                p.meshes.push_back(std::move(m));
            } else if (type == kMaterial) {
                MaterialAsset m;
                get_s(a, "name", m.name);
                get_u(a, "uuid", m.uuid);
                get_v(a, "color", m.color, 4);
                get_v(a, "emission", m.emission, 3);
                get_f(a, "metallic", m.metallic);
                get_f(a, "roughness", m.roughness);
                get_u(a, "colorMap", m.color_map);
                get_u(a, "aoMap", m.ao_map);
                get_u(a, "emissionMap", m.emission_map);
                get_u(a, "normalMap", m.normal_map);
                get_u(a, "metallicRoughnessMap", m.mr_map);
                p.materials.push_back(std::move(m));
            } else if (type == kScene) {
                p.scenes.push_back(read_scene(a));
            } else {
                fail("unknown asset type " + std::to_string(type));
            }
        }
    if (const Value* scenes = j.find("scenes")) {
        if (scenes->is_obj())
            for (const auto& m : scenes->members) p.scenes.push_back(read_scene(m.second));
        else if (scenes->is_arr())
            for (const auto& sj : scenes->items) p.scenes.push_back(read_scene(sj));
    }
    get_u(j, "initialScene", p.initial_scene);
    return p;
}

// ---------------------------------------------------------------- .luz writer
Value vec(const float* v, int n) {
    Value a = Value::array();
    for (int k = 0; k < n; ++k) a.push(Value::of((double)v[k]));
    return a;
}

struct BinaryStorage {   // Serializer.hpp:33-46
    std::vector<uint8_t> data;
    Value push(const void* p, size_t n) {
        Value v = Value::object();
        v.set("offset", Value::of_u64(data.size()));
        v.set("size", Value::of_u64(n));
        const uint8_t* b = (const uint8_t*)p;
        data.insert(data.end(), b, b + n);
        return v;
    }
};

Value write_node(const Node& n) {
    Value j = Value::object();
    Value ch = Value::array();
    for (const auto& c : n.children) ch.push(write_node(c));
    j.set("children", std::move(ch));
    j.set("name", Value::of_str(n.name));
    j.set("position", vec(n.position, 3));
    j.set("rotation", vec(n.type == kCameraNode ? n.rotation : n.rotation, 3));
    j.set("scale", vec(n.scale, 3));
    j.set("type", Value::of_i64(n.type));
    j.set("uuid", Value::of_u64(n.uuid));
    if (n.has_matrix) j.set("luzMatrix", vec(n.matrix, 16));
    if (n.type == kMeshNode) {
        j.set("mesh", Value::of_u64(n.mesh));
        j.set("material", Value::of_u64(n.material));
    } else if (n.type == kLightNode) {
        j.set("color", vec(n.color, 3));
        j.set("intensity", Value::of((double)n.intensity));
        j.set("lightType", Value::of_i64(n.light_type));
        j.set("innerAngle", Value::of((double)n.inner_angle));
        j.set("outerAngle", Value::of((double)n.outer_angle));
        j.set("radius", Value::of((double)n.radius));
        j.set("shadowMapRange", Value::of((double)n.shadow_map_range));
        j.set("shadowMapFar", Value::of((double)n.shadow_map_far));
        j.set("volumetricType", Value::of_i64(n.volumetric_type));
        if (n.has_direction) j.set("luzDirection", vec(n.direction, 3));
    } else if (n.type == kCameraNode) {
        j.set("cameraType", Value::of_i64(n.camera_type));
        j.set("mode", Value::of_i64(n.mode));
        j.set("eye", vec(n.eye, 3));
        j.set("center", vec(n.center, 3));
        j.set("zoom", Value::of((double)n.zoom));
        j.set("farDistance", Value::of((double)n.far_distance));
        j.set("nearDistance", Value::of((double)n.near_distance));
        j.set("horizontalFov", Value::of((double)n.horizontal_fov));
        j.set("orthoFarDistance", Value::of((double)n.ortho_far));
        j.set("orthoNearDistance", Value::of((double)n.ortho_near));
    }
    return j;
}

// AssetManager::SaveProject (AssetManager.cpp:216-258): assets by type, scenes keyed
// by their UUID as a string, the initial scene's UUID.
void save_project(const Project& p, const std::string& luz_path, const std::string& bin_path) {
    BinaryStorage bin;
    Value assets = Value::array();
    for (const auto& t : p.textures) {
        Value a = Value::object();
        a.set("channels", Value::of_i64(t.channels));
        a.set("data", bin.push(t.data.data(), t.data.size()));
        a.set("height", Value::of_i64(t.height));
        a.set("name", Value::of_str(t.name));
        a.set("type", Value::of_i64(kTexture));
        a.set("uuid", Value::of_u64(t.uuid));
        a.set("width", Value::of_i64(t.width));
        assets.push(std::move(a));
    }
    for (const auto& m : p.meshes) {
        Value a = Value::object();
        a.set("indices", bin.push(m.indices.data(), m.indices.size() * 4));
        a.set("name", Value::of_str(m.name));
        a.set("type", Value::of_i64(kMesh));
        a.set("uuid", Value::of_u64(m.uuid));
        a.set("vertices", bin.push(m.vertices.data(), m.vertices.size() * sizeof(luz_vertex)));
        assets.push(std::move(a));
    }
    for (const auto& m : p.materials) {
        Value a = Value::object();
        a.set("aoMap", Value::of_u64(m.ao_map));
        a.set("color", vec(m.color, 4));
        a.set("colorMap", Value::of_u64(m.color_map));
        a.set("emission", vec(m.emission, 3));
        a.set("emissionMap", Value::of_u64(m.emission_map));
        a.set("metallic", Value::of((double)m.metallic));
        a.set("metallicRoughnessMap", Value::of_u64(m.mr_map));
        a.set("name", Value::of_str(m.name));
        a.set("normalMap", Value::of_u64(m.normal_map));
        a.set("roughness", Value::of((double)m.roughness));
        a.set("type", Value::of_i64(kMaterial));
        a.set("uuid", Value::of_u64(m.uuid));
        assets.push(std::move(a));
    }
    Value scenes = Value::object();
    for (const auto& s : p.scenes) {
        Value j = Value::object();
        j.set("ambientLight", Value::of((double)s.ambient_light));
        j.set("ambientLightColor", vec(s.ambient_color, 3));
        j.set("aoMax", Value::of((double)s.ao_max));
        j.set("aoMin", Value::of((double)s.ao_min));
        j.set("aoSamples", Value::of_i64(s.ao_samples));
        j.set("exposure", Value::of((double)s.exposure));
        j.set("lightSamples", Value::of_i64(s.light_samples));
        j.set("mainCamera", Value::of_u64(s.main_camera));
        j.set("name", Value::of_str(s.name));
        Value ns = Value::array();
        for (const auto& n : s.nodes) ns.push(write_node(n));
        j.set("nodes", std::move(ns));
        j.set("shadowType", Value::of_i64(s.shadow_type));
        j.set("taaEnabled", Value::of_bool(s.taa_enabled));
        j.set("taaReconstruct", Value::of_bool(s.taa_reconstruct));
        j.set("type", Value::of_i64(kScene));
        j.set("uuid", Value::of_u64(s.uuid));
        scenes.set(std::to_string(s.uuid), std::move(j));
    }
    Value root = Value::object();
    root.set("assets", std::move(assets));
    root.set("initialScene", Value::of_u64(p.initial_scene));
    root.set("scenes", std::move(scenes));
    std::string text = json::dump(root);
    write_bytes(bin_path, bin.data.data(), bin.data.size());
    write_bytes(luz_path, text.data(), text.size());
}

// ---------------------------------------------------------------- quaternion / Euler
// glm conventions: quat (w, x, y, z); eulerAngles returns (pitch, yaw, roll) in
// radians; quat(vec3 euler) composes them (as in Node::ComposeTransform).
void quat_to_euler_deg(float w, float x, float y, float z, float out[3]) {
    // glm::pitch / yaw / roll of a unit quaternion
    float py = 2.0f * (y * z + w * x), px = w * w - x * x - y * y + z * z;
    const float eps = 1.1920928955078125e-07f;   // FLT_EPSILON
    float pitch = (std::fabs(px) <= eps && std::fabs(py) <= eps) ? 2.0f * std::atan2(x, w) : std::atan2(py, px);
    float sy = -2.0f * (x * z - w * y);
    sy = std::min(std::max(sy, -1.0f), 1.0f);
    float yaw = std::asin(sy);
    float roll = std::atan2(2.0f * (x * y + w * z), w * w + x * x - y * y - z * z);
    const float r2d = 57.295779513082320876798154814105f;
    out[0] = pitch * r2d;
    out[1] = yaw * r2d;
    out[2] = roll * r2d;
}

// Rotation part of a column-major matrix with positive scales -> unit quaternion
// (Shepperd's method on the scale-normalised 3x3).
void matrix_to_trs(const float m[16], float pos[3], float rot_deg[3], float scl[3]) {
    pos[0] = m[12]; pos[1] = m[13]; pos[2] = m[14];
    float c[3][3];
    for (int k = 0; k < 3; ++k) {
        float l = std::sqrt(m[k * 4] * m[k * 4] + m[k * 4 + 1] * m[k * 4 + 1] + m[k * 4 + 2] * m[k * 4 + 2]);
        scl[k] = l;
        for (int r = 0; r < 3; ++r) c[k][r] = l > 0.0f ? m[k * 4 + r] / l : (r == k ? 1.0f : 0.0f);
    }
    // a reflection goes into the x scale
    float det = c[0][0] * (c[1][1] * c[2][2] - c[2][1] * c[1][2]) - c[1][0] * (c[0][1] * c[2][2] - c[2][1] * c[0][2]) +
                c[2][0] * (c[0][1] * c[1][2] - c[1][1] * c[0][2]);
    if (det < 0.0f) {
        scl[0] = -scl[0];
        for (int r = 0; r < 3; ++r) c[0][r] = -c[0][r];
    }
    // R[row][col] = c[col][row]
    float tr = c[0][0] + c[1][1] + c[2][2], w, x, y, z;
    if (tr > 0.0f) {
        float s = std::sqrt(tr + 1.0f) * 2.0f;
        w = 0.25f * s;
        x = (c[1][2] - c[2][1]) / s;
        y = (c[2][0] - c[0][2]) / s;
        z = (c[0][1] - c[1][0]) / s;
    } else if (c[0][0] > c[1][1] && c[0][0] > c[2][2]) {
        float s = std::sqrt(1.0f + c[0][0] - c[1][1] - c[2][2]) * 2.0f;
        w = (c[1][2] - c[2][1]) / s;
        x = 0.25f * s;
        y = (c[1][0] + c[0][1]) / s;
        z = (c[2][0] + c[0][2]) / s;
    } else if (c[1][1] > c[2][2]) {
        float s = std::sqrt(1.0f + c[1][1] - c[0][0] - c[2][2]) * 2.0f;
        w = (c[2][0] - c[0][2]) / s;
        x = (c[1][0] + c[0][1]) / s;
        y = 0.25f * s;
        z = (c[2][1] + c[1][2]) / s;
    } else {
        float s = std::sqrt(1.0f + c[2][2] - c[0][0] - c[1][1]) * 2.0f;
        w = (c[0][1] - c[1][0]) / s;
        x = (c[2][0] + c[0][2]) / s;
        y = (c[2][1] + c[1][2]) / s;
        z = 0.25f * s;
    }
    quat_to_euler_deg(w, x, y, z, rot_deg);
}

// ---------------------------------------------------------------- base64 / data URIs
std::vector<uint8_t> base64_decode(const std::string& s, size_t from) {
    auto val = [](char c) -> int {
        if (c >= 'A' && c <= 'Z') return c - 'A';
        if (c >= 'a' && c <= 'z') return c - 'a' + 26;
        if (c >= '0' && c <= '9') return c - '0' + 52;
        if (c == '+' || c == '-') return 62;
        if (c == '/' || c == '_') return 63;
        return -1;
    };
    std::vector<uint8_t> out;
    uint32_t acc = 0;
    int bits = 0;
    for (size_t k = from; k < s.size(); ++k) {
        int v = val(s[k]);
        if (v < 0) {
            if (s[k] == '=') break;
            continue;
        }
        acc = (acc << 6) | (uint32_t)v;
        bits += 6;
        if (bits >= 8) {
            bits -= 8;
            out.push_back((uint8_t)(acc >> bits));
        }
    }
    return out;
}

std::vector<uint8_t> load_uri(const std::string& uri, const std::string& base) {
    if (uri.compare(0, 5, "data:") == 0) {
        size_t comma = uri.find(',');
        if (comma == std::string::npos || uri.find(";base64") == std::string::npos || uri.find(";base64") > comma)
            fail("unsupported data URI (base64 expected)");
        return base64_decode(uri, comma + 1);
    }
    std::string path;
    for (size_t k = 0; k < uri.size(); ++k) {   // %XX escapes
        if (uri[k] == '%' && k + 2 < uri.size()) {
            path += (char)strtol(uri.substr(k + 1, 2).c_str(), nullptr, 16);
            k += 2;
        } else {
            path += uri[k];
        }
    }
    return read_bytes(base + path);
}

void decode_image(const std::vector<uint8_t>& bytes, TextureAsset& t, const std::string& what) {
    if (!png::is_png(bytes.data(), bytes.size()))
        fail(what + ": only PNG images are decoded (JPEG and other formats are not supported)");
    png::Image img = png::decode(bytes.data(), bytes.size());
    t.width = (int32_t)img.width;
    t.height = (int32_t)img.height;
    t.channels = 4;
    t.data = std::move(img.rgba);
}

// ---------------------------------------------------------------- glTF 2.0
// AssetIO::ImportSceneGLTF (source/Resources/AssetIO.cpp:117-402), written from the
// glTF 2.0 specification: one texture asset per texture, one material asset per
// material, one mesh asset per primitive (tangents computed when absent), and per
// glTF node a Node holding a MeshNode and/or a LightNode child plus its glTF
// children. As in the reference, a node's mesh index selects from the flat list of
// primitives, and KHR_lights_punctual lights become default LightNodes.
struct GltfAccessor {
    const uint8_t* base = nullptr;
    size_t count = 0, stride = 0, comps = 0;
    int ctype = 0;
};

SceneAsset import_gltf(const std::string& path, Project& p, UuidGen& ids) {
    std::vector<uint8_t> file = read_bytes(path);
    std::string base = dir_of(path);
    Value j;
    std::vector<uint8_t> glb_bin;
    if (file.size() >= 12 && memcmp(file.data(), "glTF", 4) == 0) {
        uint32_t version, length;
        memcpy(&version, file.data() + 4, 4);
        memcpy(&length, file.data() + 8, 4);
        if (version != 2) fail("only glTF 2.0 binaries are supported");
        size_t pos = 12;
        bool have_json = false;
        while (pos + 8 <= std::min<size_t>(file.size(), length)) {
            uint32_t clen, ctype;
            memcpy(&clen, file.data() + pos, 4);
            memcpy(&ctype, file.data() + pos + 4, 4);
            if (pos + 8 + clen > file.size()) fail("truncated GLB chunk");
            if (ctype == 0x4E4F534Au) {
                j = json::parse(std::string((const char*)file.data() + pos + 8, clen));
                have_json = true;
            } else if (ctype == 0x004E4942u && glb_bin.empty()) {
                glb_bin.assign(file.data() + pos + 8, file.data() + pos + 8 + clen);
            }
            pos += 8 + ((clen + 3) & ~3u);
        }
        if (!have_json) fail("GLB without a JSON chunk");
    } else {
        j = json::parse(std::string(file.begin(), file.end()));
    }
    // buffers
    std::vector<std::vector<uint8_t>> buffers;
    if (const Value* bs = j.find("buffers"))
        for (const auto& b : bs->items) {
            if (const Value* uri = b.find("uri")) buffers.push_back(load_uri(uri->str(), base));
            else buffers.push_back(glb_bin);
            if (const Value* bl = b.find("byteLength"))
                if (buffers.back().size() < bl->u64()) fail("glTF buffer shorter than its byteLength");
        }
    const Value* views = j.find("bufferViews");
    const Value* accs = j.find("accessors");
    auto view_bytes = [&](size_t vi, size_t& len) -> const uint8_t* {
        if (!views || vi >= views->size()) fail("bad bufferView index");
        const Value& v = (*views)[vi];
        size_t bi = (size_t)v.at("buffer").u64();
        if (bi >= buffers.size()) fail("bad buffer index");
        size_t off = v.has("byteOffset") ? (size_t)v.at("byteOffset").u64() : 0;
        len = (size_t)v.at("byteLength").u64();
        if (off > buffers[bi].size() || len > buffers[bi].size() - off) fail("bufferView outside its buffer");
        return buffers[bi].data() + off;
    };
    auto accessor = [&](size_t ai) {
        if (!accs || ai >= accs->size()) fail("bad accessor index");
        const Value& a = (*accs)[ai];
        if (a.has("sparse")) fail("sparse accessors are not supported");
        GltfAccessor r;
        r.ctype = (int)a.at("componentType").i64();
        r.count = (size_t)a.at("count").u64();
        const std::string& type = a.at("type").str();
        r.comps = type == "SCALAR" ? 1 : type == "VEC2" ? 2 : type == "VEC3" ? 3 : type == "VEC4" ? 4 : 0;
        if (!r.comps) fail("unsupported accessor type " + type);
        size_t csize = (r.ctype == 5120 || r.ctype == 5121) ? 1 : (r.ctype == 5122 || r.ctype == 5123) ? 2 : 4;
        size_t vlen;
        const uint8_t* vb = view_bytes((size_t)a.at("bufferView").u64(), vlen);
        const Value& v = (*views)[(size_t)a.at("bufferView").u64()];
        r.stride = v.has("byteStride") ? (size_t)v.at("byteStride").u64() : csize * r.comps;
        size_t off = a.has("byteOffset") ? (size_t)a.at("byteOffset").u64() : 0;
        const size_t elem = csize * r.comps;
        if (r.stride < elem) fail("bufferView byteStride smaller than the accessor's element");
        // off + (count - 1) * stride + elem <= vlen, without overflow
        if (r.count && (off > vlen || elem > vlen - off || r.count - 1 > (vlen - off - elem) / r.stride))
            fail("accessor outside its bufferView");
        r.base = vb + off;
        return r;
    };
    auto read_f = [&](const GltfAccessor& a, size_t k, int c) -> float {
        if (a.ctype != 5126) fail("only float vertex attributes are supported");
        float f;
        memcpy(&f, a.base + k * a.stride + 4 * c, 4);
        return f;
    };
    // textures
    std::vector<uint64_t> tex_ids;
    if (const Value* ts = j.find("textures")) {
        const Value* images = j.find("images");
        for (size_t ti = 0; ti < ts->size(); ++ti) {
            const Value& t = (*ts)[ti];
            TextureAsset ta;
            ta.uuid = ids.next();
            get_s(t, "name", ta.name);
            if (!t.has("source") || !images || t.at("source").u64() >= images->size())
                fail("texture without an image source");
            const Value& im = (*images)[(size_t)t.at("source").u64()];
            std::vector<uint8_t> bytes;
            if (const Value* uri = im.find("uri")) {
                bytes = load_uri(uri->str(), base);
            } else {
                size_t len;
                const uint8_t* b = view_bytes((size_t)im.at("bufferView").u64(), len);
                bytes.assign(b, b + len);
            }
            decode_image(bytes, ta, "glTF image " + std::to_string(t.at("source").u64()));
            tex_ids.push_back(ta.uuid);
            p.textures.push_back(std::move(ta));
        }
    }
    auto tex_ref = [&](const Value* info) -> uint64_t {
        if (!info || !info->has("index")) return 0;
        size_t k = (size_t)info->at("index").u64();
        if (k >= tex_ids.size()) fail("bad texture index");
        return tex_ids[k];
    };
    // materials
    std::vector<uint64_t> mat_ids;
    if (const Value* ms = j.find("materials"))
        for (const auto& m : ms->items) {
            MaterialAsset ma;
            ma.uuid = ids.next();
            get_s(m, "name", ma.name);
            if (const Value* pbr = m.find("pbrMetallicRoughness")) {
                ma.color_map = tex_ref(pbr->find("baseColorTexture"));
                ma.mr_map = tex_ref(pbr->find("metallicRoughnessTexture"));
                get_v(*pbr, "baseColorFactor", ma.color, 4);
                get_f(*pbr, "roughnessFactor", ma.roughness);
                get_f(*pbr, "metallicFactor", ma.metallic);
            }
            ma.normal_map = tex_ref(m.find("normalTexture"));
            ma.emission_map = tex_ref(m.find("emissiveTexture"));
            ma.ao_map = tex_ref(m.find("occlusionTexture"));
            get_v(m, "emissiveFactor", ma.emission, 3);
            mat_ids.push_back(ma.uuid);
            p.materials.push_back(std::move(ma));
        }
    // meshes: one asset per primitive
    std::vector<uint64_t> prim_mesh;
    std::vector<int64_t> prim_material;
    if (const Value* meshes = j.find("meshes"))
        for (const auto& mesh : meshes->items) {
            std::string mname;
            get_s(mesh, "name", mname);
            const Value& prims = mesh.at("primitives");
            for (size_t pi = 0; pi < prims.size(); ++pi) {
                const Value& prim = prims[pi];
                if (prim.has("mode") && prim.at("mode").i64() != 4) fail("only triangle-list primitives are supported");
                MeshAsset ma;
                ma.uuid = ids.next();
                ma.name = (mname.empty() ? stem_of(path) : mname) + "_" + std::to_string(pi);
                prim_material.push_back(prim.has("material") ? prim.at("material").i64() : -1);
                const Value& attr = prim.at("attributes");
                GltfAccessor pos = accessor((size_t)attr.at("POSITION").u64());
                GltfAccessor nrm, tan, uv;
                bool has_n = attr.has("NORMAL"), has_t = attr.has("TANGENT"), has_uv = attr.has("TEXCOORD_0");
                if (has_n) nrm = accessor((size_t)attr.at("NORMAL").u64());
                if (has_t) tan = accessor((size_t)attr.at("TANGENT").u64());
                if (has_uv) uv = accessor((size_t)attr.at("TEXCOORD_0").u64());
                size_t nv = pos.count;
                if ((has_n && nrm.count < nv) || (has_t && tan.count < nv) || (has_uv && uv.count < nv))
                    fail("vertex attribute shorter than POSITION");
                ma.vertices.resize(nv);
                for (size_t v = 0; v < nv; ++v) {
                    luz_vertex& x = ma.vertices[v];
                    memset(&x, 0, sizeof(x));
                    for (int c = 0; c < 3; ++c) x.position[c] = read_f(pos, v, c);
                    if (has_n) for (int c = 0; c < 3; ++c) x.normal[c] = read_f(nrm, v, c);
                    if (has_uv) for (int c = 0; c < 2; ++c) x.texcoord[c] = read_f(uv, v, c);
                    if (has_t) for (int c = 0; c < 4; ++c) x.tangent[c] = read_f(tan, v, c);
                }
                if (!prim.has("indices")) fail("non-indexed primitives are not supported");
                GltfAccessor ia = accessor((size_t)prim.at("indices").u64());
                ma.indices.resize(ia.count);
                for (size_t k = 0; k < ia.count; ++k) {
                    const uint8_t* q = ia.base + k * ia.stride;
                    uint32_t v;
                    if (ia.ctype == 5125) memcpy(&v, q, 4);
                    else if (ia.ctype == 5123) { uint16_t h; memcpy(&h, q, 2); v = h; }
                    else if (ia.ctype == 5121) v = q[0];
                    else fail("unsupported index type");
                    ma.indices[k] = v;
                }
                if (!has_t) {
                    // per-vertex tangent from UV gradients (AssetIO.cpp:325-357): the
                    // triangle (i0, i2, i1), sdir/tdir summed per vertex, then
                    // Gram-Schmidt against the normal and the handedness sign.
                    std::vector<float> t1(nv * 3, 0.0f), t2(nv * 3, 0.0f);
                    for (size_t k = 0; k + 2 < ma.indices.size(); k += 3) {
                        uint32_t a = ma.indices[k], b = ma.indices[k + 2], c = ma.indices[k + 1];
                        if (a >= nv || b >= nv || c >= nv) fail("index outside the vertex buffer");
                        const luz_vertex &v1 = ma.vertices[a], &v2 = ma.vertices[b], &v3 = ma.vertices[c];
                        float e1[3], e2[3];
                        for (int q = 0; q < 3; ++q) {
                            e1[q] = v2.position[q] - v1.position[q];
                            e2[q] = v3.position[q] - v1.position[q];
                        }
                        float d1x = v2.texcoord[0] - v1.texcoord[0], d1y = v2.texcoord[1] - v1.texcoord[1];
                        float d2x = v3.texcoord[0] - v1.texcoord[0], d2y = v3.texcoord[1] - v1.texcoord[1];
                        float f = 1.0f / (d1x * d2y - d2x * d1y);
                        float sdir[3], tdir[3];
                        for (int q = 0; q < 3; ++q) {
                            sdir[q] = f * (d2y * e1[q] - d1y * e2[q]);
                            tdir[q] = f * (d1x * e2[q] - d2x * e1[q]);
                        }
                        for (uint32_t vi : {a, b, c})
                            for (int q = 0; q < 3; ++q) {
                                t1[vi * 3 + q] += sdir[q];
                                t2[vi * 3 + q] += tdir[q];
                            }
                    }
                    for (size_t v = 0; v < nv; ++v) {
                        luz_vertex& x = ma.vertices[v];
                        const float* t = &t1[v * 3];
                        const float* n = x.normal;
                        float d = t[0] * n[0] + t[1] * n[1] + t[2] * n[2];
                        float g[3] = {t[0] - n[0] * d, t[1] - n[1] * d, t[2] - n[2] * d};
                        // glm::normalize: v * inversesqrt(dot(v, v))
                        float inv = 1.0f / std::sqrt(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]);
                        x.tangent[0] = g[0] * inv;
                        x.tangent[1] = g[1] * inv;
                        x.tangent[2] = g[2] * inv;
                        float cr[3] = {n[1] * t[2] - t[1] * n[2], n[2] * t[0] - t[2] * n[0], n[0] * t[1] - t[0] * n[1]};
                        float s = cr[0] * t2[v * 3] + cr[1] * t2[v * 3 + 1] + cr[2] * t2[v * 3 + 2];
                        x.tangent[3] = s < 0.0f ? -1.0f : 1.0f;
                    }
                }
                prim_mesh.push_back(ma.uuid);
                p.meshes.push_back(std::move(ma));
            }
        }
    // nodes
    std::vector<Node> gnodes;
    const Value* nodes = j.find("nodes");
    if (nodes)
        for (const auto& n : nodes->items) {
            Node g;
            g.type = kNode;
            g.uuid = ids.next();
            get_s(n, "name", g.name);
            if (n.has("mesh")) {
                size_t mi = (size_t)n.at("mesh").u64();
                if (mi >= prim_mesh.size()) fail("node mesh index outside the primitive list");
                Node mn;
                mn.type = kMeshNode;
                mn.uuid = ids.next();
                mn.name = g.name;
                mn.mesh = prim_mesh[mi];
                int64_t mat = prim_material[mi];
                if (mat >= 0) {
                    if ((size_t)mat >= mat_ids.size()) fail("bad material index");
                    mn.material = mat_ids[(size_t)mat];
                }
                g.children.push_back(std::move(mn));
            }
            bool has_light = false;
            if (const Value* ex = n.find("extensions"))
                if (const Value* kl = ex->find("KHR_lights_punctual")) has_light = kl->has("light");
            if (has_light) {
                Node ln;
                ln.type = kLightNode;
                ln.uuid = ids.next();
                ln.name = g.name;
                g.children.push_back(std::move(ln));
            }
            if (const Value* t = n.find("translation"))
                if (t->size() == 3) for (int c = 0; c < 3; ++c) g.position[c] = (*t)[c].f32();
            if (const Value* r = n.find("rotation"))
                if (r->size() == 4)
                    quat_to_euler_deg((*r)[3].f32(), (*r)[0].f32(), (*r)[1].f32(), (*r)[2].f32(), g.rotation);
            if (const Value* s = n.find("scale"))
                if (s->size() == 3) for (int c = 0; c < 3; ++c) g.scale[c] = (*s)[c].f32();
            if (const Value* m = n.find("matrix"))
                if (m->size() == 16) {
                    float mm[16];
                    for (int c = 0; c < 16; ++c) mm[c] = (*m)[c].f32();
                    matrix_to_trs(mm, g.position, g.rotation, g.scale);
                }
            gnodes.push_back(std::move(g));
        }
    // hierarchy: children attach after the node's own mesh / light child
    std::vector<std::vector<size_t>> kids(gnodes.size());
    std::vector<int> parent(gnodes.size(), -1);
    if (nodes)
        for (size_t i = 0; i < nodes->size(); ++i)
            if (const Value* ch = (*nodes)[i].find("children"))
                for (const auto& c : ch->items) {
                    size_t k = (size_t)c.u64();
                    if (k >= gnodes.size() || parent[k] >= 0 || k == i) fail("bad glTF node hierarchy");
                    parent[k] = (int)i;
                    kids[i].push_back(k);
                }
    std::vector<int> state(gnodes.size(), 0);
    std::function<Node(size_t, int)> build = [&](size_t i, int depth) -> Node {
        if (depth > kMaxNodeDepth) fail("node tree too deep");
        if (state[i] == 1) fail("cycle in the glTF node hierarchy");
        state[i] = 1;
        Node n = gnodes[i];
        for (size_t k : kids[i]) n.children.push_back(build(k, depth + 1));
        state[i] = 2;
        return n;
    };
    SceneAsset scene;
    scene.uuid = ids.next();
    // the first glTF scene (the reference returns loadedScenes[0])
    if (const Value* scenes = j.find("scenes")) {
        if (scenes->size() > 0) {
            const Value& s0 = (*scenes)[0];
            get_s(s0, "name", scene.name);
            if (const Value* ns = s0.find("nodes"))
                for (const auto& n : ns->items) {
                    size_t k = (size_t)n.u64();
                    if (k >= gnodes.size()) fail("bad scene node index");
                    scene.nodes.push_back(build(k, 0));
                }
        }
    }
    return scene;
}

// ---------------------------------------------------------------- OBJ + MTL
// AssetIO::ImportSceneOBJ (source/Resources/AssetIO.cpp:404-529), written from the
// OBJ/MTL formats: one mesh asset per shape with vertices merged on equal (position,
// normal, texcoord), v flipped (1 - v), no tangents; a parent Node named after the
// file holding the MeshNodes. Polygons: triangles as given, quads split along the
// shorter diagonal, larger polygons by ear clipping in their dominant plane.
struct ObjIndex { int v = -1, vt = -1, vn = -1; };
struct ObjMaterial {
    std::string name;
    float kd[3] = {0.6f, 0.6f, 0.6f}, ks[3] = {0, 0, 0}, ke[3] = {0, 0, 0};
    float pm = 0.0f, pr = 0.0f;
    std::string map_kd, norm;
};

std::vector<std::string> split_ws(const std::string& line) {
    std::vector<std::string> out;
    std::istringstream ss(line);
    std::string tok;
    while (ss >> tok) out.push_back(tok);
    return out;
}

void read_mtl(const std::string& path, std::vector<ObjMaterial>& mats, std::map<std::string, int>& by_name) {
    std::ifstream f(path);
    if (!f) return;   // a missing material library leaves the faces without materials
    std::string line;
    ObjMaterial* cur = nullptr;
    while (std::getline(f, line)) {
        if (!line.empty() && line.back() == '\r') line.pop_back();
        auto t = split_ws(line);
        if (t.empty() || t[0][0] == '#') continue;
        auto num = [&](size_t k) { return k < t.size() ? strtof(t[k].c_str(), nullptr) : 0.0f; };
        if (t[0] == "newmtl") {
            ObjMaterial m;
            m.name = t.size() > 1 ? t[1] : "";
            by_name[m.name] = (int)mats.size();
            mats.push_back(m);
            cur = &mats.back();
        } else if (!cur) {
            continue;
        } else if (t[0] == "Kd") {
            for (int c = 0; c < 3; ++c) cur->kd[c] = num(1 + c);
        } else if (t[0] == "Ks") {
            for (int c = 0; c < 3; ++c) cur->ks[c] = num(1 + c);
        } else if (t[0] == "Ke") {
            for (int c = 0; c < 3; ++c) cur->ke[c] = num(1 + c);
        } else if (t[0] == "Pm") {
            cur->pm = num(1);
        } else if (t[0] == "Pr") {
            cur->pr = num(1);
        } else if (t[0] == "map_Kd" && t.size() > 1) {
            cur->map_kd = t.back();
        } else if (t[0] == "norm" && t.size() > 1) {
            cur->norm = t.back();
        }
    }
}

// Ear clipping of one polygon (indices into pts, counter-clockwise or clockwise).
std::vector<std::array<size_t, 3>> ear_clip(const std::vector<std::array<float, 2>>& pts) {
    std::vector<std::array<size_t, 3>> tris;
    std::vector<size_t> idx(pts.size());
    for (size_t k = 0; k < idx.size(); ++k) idx[k] = k;
    double area = 0.0;
    for (size_t k = 0; k < pts.size(); ++k) {
        const auto &a = pts[k], &b = pts[(k + 1) % pts.size()];
        area += (double)a[0] * b[1] - (double)b[0] * a[1];
    }
    const double orient = area >= 0.0 ? 1.0 : -1.0;
    auto cross = [&](size_t a, size_t b, size_t c) {
        return ((double)pts[b][0] - pts[a][0]) * ((double)pts[c][1] - pts[a][1]) -
               ((double)pts[b][1] - pts[a][1]) * ((double)pts[c][0] - pts[a][0]);
    };
    size_t guard = 0;
    while (idx.size() > 3 && guard < pts.size() * pts.size() + 8) {
        ++guard;
        bool clipped = false;
        for (size_t k = 0; k < idx.size(); ++k) {
            size_t a = idx[(k + idx.size() - 1) % idx.size()], b = idx[k], c = idx[(k + 1) % idx.size()];
            if (cross(a, b, c) * orient <= 0.0) continue;   // reflex or degenerate corner
            bool inside = false;
            for (size_t q : idx) {
                if (q == a || q == b || q == c) continue;
                if (cross(a, b, q) * orient >= 0.0 && cross(b, c, q) * orient >= 0.0 && cross(c, a, q) * orient >= 0.0) {
                    inside = true;
                    break;
                }
            }
            if (inside) continue;
            tris.push_back({a, b, c});
            idx.erase(idx.begin() + (long)k);
            clipped = true;
            break;
        }
        if (!clipped) break;   // degenerate remainder: fan it
    }
    for (size_t k = 1; k + 1 < idx.size(); ++k) tris.push_back({idx[0], idx[k], idx[k + 1]});
    return tris;
}

SceneAsset import_obj(const std::string& path, Project& p, UuidGen& ids) {
    std::ifstream f(path);
    if (!f) fail("cannot open " + path);
    std::string base = dir_of(path), filename = stem_of(path);
    std::vector<float> v, vt, vn;
    std::vector<ObjMaterial> mats;
    std::map<std::string, int> mat_by_name;
    struct Shape {
        std::string name;
        std::vector<ObjIndex> idx;   // triangulated
        std::vector<int> mat;        // per triangle
    };
    std::vector<Shape> shapes(1);
    int cur_mat = -1;
    std::string line;
    // 1-based, or negative from the end of what was read so far; 0 is "none" (-1).
    // An index outside that range maps to INT_MAX, which the checks below reject.
    auto resolve = [&](long i, size_t n) -> int {
        if (i > 0) return (unsigned long)i <= n ? (int)(i - 1) : INT_MAX;
        if (i < 0) return (unsigned long)(-(i + 1)) < n ? (int)((long)n + i) : INT_MAX;
        return -1;
    };
    while (std::getline(f, line)) {
        if (!line.empty() && line.back() == '\r') line.pop_back();
        auto t = split_ws(line);
        if (t.empty() || t[0][0] == '#') continue;
        if (t[0] == "v") {
            for (int c = 0; c < 3; ++c) v.push_back(1 + c < (int)t.size() ? strtof(t[1 + c].c_str(), nullptr) : 0.0f);
        } else if (t[0] == "vn") {
            for (int c = 0; c < 3; ++c) vn.push_back(1 + c < (int)t.size() ? strtof(t[1 + c].c_str(), nullptr) : 0.0f);
        } else if (t[0] == "vt") {
            for (int c = 0; c < 2; ++c) vt.push_back(1 + c < (int)t.size() ? strtof(t[1 + c].c_str(), nullptr) : 0.0f);
        } else if (t[0] == "o" || t[0] == "g") {
            if (!shapes.back().idx.empty()) shapes.emplace_back();
            shapes.back().name = t.size() > 1 ? t[1] : "";
        } else if (t[0] == "mtllib" && t.size() > 1) {
            for (size_t k = 1; k < t.size(); ++k) read_mtl(base + t[k], mats, mat_by_name);
        } else if (t[0] == "usemtl") {
            auto it = t.size() > 1 ? mat_by_name.find(t[1]) : mat_by_name.end();
            cur_mat = it == mat_by_name.end() ? -1 : it->second;
        } else if (t[0] == "f") {
            std::vector<ObjIndex> poly;
            for (size_t k = 1; k < t.size(); ++k) {
                ObjIndex oi;
                const std::string& s = t[k];
                size_t a = s.find('/');
                oi.v = resolve(strtol(s.substr(0, a).c_str(), nullptr, 10), v.size() / 3);
                if (a != std::string::npos) {
                    size_t b = s.find('/', a + 1);
                    std::string st = s.substr(a + 1, b == std::string::npos ? std::string::npos : b - a - 1);
                    if (!st.empty()) oi.vt = resolve(strtol(st.c_str(), nullptr, 10), vt.size() / 2);
                    if (b != std::string::npos && b + 1 < s.size())
                        oi.vn = resolve(strtol(s.substr(b + 1).c_str(), nullptr, 10), vn.size() / 3);
                }
                if (oi.v < 0 || (size_t)oi.v * 3 + 2 >= v.size()) fail("OBJ face references a missing vertex");
                if (oi.vt >= 0 && (size_t)oi.vt * 2 + 1 >= vt.size()) fail("OBJ face references a missing texcoord");
                if (oi.vn >= 0 && (size_t)oi.vn * 3 + 2 >= vn.size()) fail("OBJ face references a missing normal");
                poly.push_back(oi);
            }
            if (poly.size() < 3) continue;
            Shape& sh = shapes.back();
            auto P = [&](const ObjIndex& q, int c) { return v[(size_t)q.v * 3 + c]; };
            auto emit = [&](size_t a, size_t b, size_t c) {
                sh.idx.push_back(poly[a]);
                sh.idx.push_back(poly[b]);
                sh.idx.push_back(poly[c]);
                sh.mat.push_back(cur_mat);
            };
            if (poly.size() == 3) {
                emit(0, 1, 2);
            } else if (poly.size() == 4) {
                float d02 = 0, d13 = 0;
                for (int c = 0; c < 3; ++c) {
                    float a = P(poly[2], c) - P(poly[0], c), b = P(poly[3], c) - P(poly[1], c);
                    d02 += a * a;
                    d13 += b * b;
                }
                if (d02 < d13) { emit(0, 1, 2); emit(0, 2, 3); }
                else { emit(0, 1, 3); emit(1, 2, 3); }
            } else {
                // dominant plane from Newell's normal
                double nx = 0, ny = 0, nz = 0;
                for (size_t k = 0; k < poly.size(); ++k) {
                    const ObjIndex &a = poly[k], &b = poly[(k + 1) % poly.size()];
                    nx += ((double)P(a, 1) - P(b, 1)) * ((double)P(a, 2) + P(b, 2));
                    ny += ((double)P(a, 2) - P(b, 2)) * ((double)P(a, 0) + P(b, 0));
                    nz += ((double)P(a, 0) - P(b, 0)) * ((double)P(a, 1) + P(b, 1));
                }
                int ax = 0, ay = 1;
                if (std::fabs(nx) >= std::fabs(ny) && std::fabs(nx) >= std::fabs(nz)) { ax = 1; ay = 2; }
                else if (std::fabs(ny) >= std::fabs(nz)) { ax = 2; ay = 0; }
                std::vector<std::array<float, 2>> pts;
                for (const auto& q : poly) pts.push_back({P(q, ax), P(q, ay)});
                for (const auto& tri : ear_clip(pts)) emit(tri[0], tri[1], tri[2]);
            }
        }
    }
    // materials (AssetIO.cpp:426-459)
    std::vector<uint64_t> mat_ids;
    std::map<std::string, uint64_t> tex_by_name;
    auto texture = [&](const std::string& name) -> uint64_t {
        if (name.empty()) return 0;
        auto it = tex_by_name.find(name);
        if (it != tex_by_name.end()) return it->second;
        TextureAsset ta;
        ta.uuid = ids.next();
        ta.name = name;
        decode_image(read_bytes(base + name), ta, "OBJ texture " + name);
        tex_by_name[name] = ta.uuid;
        p.textures.push_back(std::move(ta));
        return tex_by_name[name];
    };
    for (const auto& m : mats) {
        MaterialAsset ma;
        ma.uuid = ids.next();
        ma.name = filename + ":" + m.name;
        ma.color[0] = m.kd[0]; ma.color[1] = m.kd[1]; ma.color[2] = m.kd[2]; ma.color[3] = 1.0f;
        for (int c = 0; c < 3; ++c) ma.emission[c] = m.ke[c];
        ma.metallic = m.pm;
        // The reference tests `materials[i].specular != 0`, an array against null,
        // which always holds: roughness is 1 - mean(Ks) and Pr is never used.
        ma.roughness = 1.0f - (m.ks[0] + m.ks[1] + m.ks[2]) / 3.0f;
        ma.color_map = texture(m.map_kd);
        ma.normal_map = texture(m.norm);
        mat_ids.push_back(ma.uuid);
        p.materials.push_back(std::move(ma));
    }
    SceneAsset scene;
    scene.uuid = ids.next();
    scene.name = filename;
    Node parent;
    parent.type = kNode;
    parent.uuid = ids.next();
    parent.name = filename;
    for (const Shape& sh : shapes) {
        if (sh.idx.empty()) continue;
        // Runs of faces with one material become MeshNodes. The reference keeps
        // appending every run to the same mesh asset, so each of its MeshNodes draws
        // the whole shape; here each run is its own mesh.
        size_t start = 0;
        while (start < sh.mat.size()) {
            size_t end = start;
            while (end < sh.mat.size() && sh.mat[end] == sh.mat[start]) ++end;
            MeshAsset ma;
            ma.uuid = ids.next();
            ma.name = filename + ":" + sh.name + "_0";
            struct Key {
                float p[3], n[3], t[2];
                bool operator<(const Key& o) const { return memcmp(this, &o, sizeof(Key)) < 0; }
            };
            std::map<Key, uint32_t> unique;
            for (size_t k = start * 3; k < end * 3; ++k) {
                const ObjIndex& q = sh.idx[k];
                luz_vertex x;
                memset(&x, 0, sizeof(x));
                for (int c = 0; c < 3; ++c) x.position[c] = v[(size_t)q.v * 3 + c];
                if (q.vn >= 0) for (int c = 0; c < 3; ++c) x.normal[c] = vn[(size_t)q.vn * 3 + c];
                if (q.vt >= 0) {
                    x.texcoord[0] = vt[(size_t)q.vt * 2];
                    x.texcoord[1] = 1.0f - vt[(size_t)q.vt * 2 + 1];
                }
                Key key;
                memset(&key, 0, sizeof(key));
                // +0.0 and -0.0 compare equal in the reference's float comparison
                for (int c = 0; c < 3; ++c) { key.p[c] = x.position[c] + 0.0f; key.n[c] = x.normal[c] + 0.0f; }
                key.t[0] = x.texcoord[0] + 0.0f;
                key.t[1] = x.texcoord[1] + 0.0f;
                auto it = unique.find(key);
                if (it == unique.end()) {
                    it = unique.emplace(key, (uint32_t)ma.vertices.size()).first;
                    ma.vertices.push_back(x);
                }
                ma.indices.push_back(it->second);
            }
            Node mn;
            mn.type = kMeshNode;
            mn.uuid = ids.next();
            mn.name = ma.name;
            mn.mesh = ma.uuid;
            if (sh.mat[start] >= 0) mn.material = mat_ids[(size_t)sh.mat[start]];
            parent.children.push_back(std::move(mn));
            p.meshes.push_back(std::move(ma));
            start = end;
        }
    }
    scene.nodes.push_back(std::move(parent));
    return scene;
}

// ---------------------------------------------------------------- project -> host scene
// GPUScene::UpdateResources (GPUScene.cpp:181-346) over a pre-order walk of the scene
// (SceneAsset::GetAll, AssetManager.hpp:305-325).
struct Walker {
    const Project& p;
    luz_host_scene* s;
    std::map<uint64_t, uint32_t> mesh_index, tex_index;
    std::vector<const Node*> lights;
    std::vector<std::array<float, 16>> light_world;

    uint32_t mesh_of(uint64_t id) {
        auto it = mesh_index.find(id);
        if (it != mesh_index.end()) return it->second;
        const MeshAsset* m = p.mesh(id);
        if (!m) fail("MeshNode references a missing mesh " + std::to_string(id));
        for (uint32_t k : m->indices)
            if (k >= m->vertices.size()) fail("mesh '" + m->name + "' has an index outside its vertex buffer");
        if (m->indices.size() % 3) fail("mesh '" + m->name + "' index count is not a multiple of 3");
        luz::host::Mesh hm;
        hm.v = m->vertices;
        hm.i = m->indices;
        s->meshes.push_back(std::move(hm));
        uint32_t k = (uint32_t)s->meshes.size() - 1;
        mesh_index[id] = k;
        return k;
    }
    int32_t tex_of(uint64_t id) {
        if (!id) return -1;
        auto it = tex_index.find(id);
        if (it != tex_index.end()) return (int32_t)it->second;
        const TextureAsset* t = p.texture(id);
        if (!t) fail("material references a missing texture " + std::to_string(id));
        if (t->width <= 0 || t->height <= 0 || t->data.size() < (size_t)t->width * t->height * 4)
            fail("texture '" + t->name + "' is not width*height RGBA8");
        luz::host::Texture ht;
        ht.width = (uint32_t)t->width;
        ht.height = (uint32_t)t->height;
        ht.rgba.assign(t->data.begin(), t->data.begin() + (size_t)t->width * t->height * 4);
        s->textures.push_back(std::move(ht));
        uint32_t k = (uint32_t)s->textures.size() - 1;
        tex_index[id] = k;
        return (int32_t)k;
    }
    void walk(const Node& n, const float parent[16], int depth) {
        if (depth > kMaxNodeDepth) fail("node tree too deep");
        float world[16];
        if (n.has_matrix) {
            float id[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
            const float* par = parent ? parent : id;
            for (int c = 0; c < 4; ++c)
                for (int r = 0; r < 4; ++r) {
                    float acc = 0.0f;
                    for (int k = 0; k < 4; ++k) acc += par[k * 4 + r] * n.matrix[c * 4 + k];
                    world[c * 4 + r] = acc;
                }
            if (!parent) memcpy(world, n.matrix, 64);
        } else {
            luz::host::compose_transform(n.position, n.rotation, n.scale, parent, world);
        }
        if (n.type == kMeshNode) {
            uint32_t mi = mesh_of(n.mesh);
            luz_model m = luz::host::default_model();
            if (n.material) {
                const MaterialAsset* mat = p.material(n.material);
                if (!mat) fail("MeshNode references a missing material " + std::to_string(n.material));
                memcpy(m.color, mat->color, 16);
                memcpy(m.emission, mat->emission, 12);
                m.metallic = mat->metallic;
                m.roughness = mat->roughness;
                m.color_map = tex_of(mat->color_map);
                m.normal_map = tex_of(mat->normal_map);
                m.metallic_roughness_map = tex_of(mat->mr_map);
                m.emission_map = tex_of(mat->emission_map);
                // aoMap is not packed (GPUScene.cpp:197-213)
            }
            memcpy(m.model_mat, world, 64);
            s->models.push_back(m);
            s->instance_mesh.push_back(mi);
        } else if (n.type == kLightNode) {
            lights.push_back(&n);
            std::array<float, 16> w;
            memcpy(w.data(), world, 64);
            light_world.push_back(w);
        }
        for (const Node& c : n.children) walk(c, world, depth + 1);
    }
};

const Node* find_top(const SceneAsset& s, uint64_t id) {   // SceneAsset::Get: top-level nodes only
    for (const auto& n : s.nodes)
        if (n.uuid == id) return &n;
    return nullptr;
}

luz_host_scene* to_host_scene(const Project& p, const SceneAsset& sc, uint32_t width, uint32_t height) {
    std::unique_ptr<luz_host_scene> s(new luz_host_scene());
    s->width = width;
    s->height = height;
    Walker w{p, s.get(), {}, {}, {}, {}};
    for (const Node& n : sc.nodes) w.walk(n, nullptr, 0);
    for (size_t k = 0; k < w.lights.size(); ++k) {
        const Node& n = *w.lights[k];
        const float* m = w.light_world[k].data();
        luz_light l;
        memset(&l, 0, sizeof(l));
        memcpy(l.color, n.color, 12);
        l.intensity = n.intensity;
        // GetWorldPosition = parent transform * position; the light's own transform
        // applied to (0,-1,0,0) is its direction (GPUScene.cpp:239-246).
        for (int r = 0; r < 3; ++r) l.position[r] = m[12 + r];
        for (int r = 0; r < 3; ++r) l.direction[r] = n.has_direction ? n.direction[r] : -m[4 + r];
        const float d2r = 0.01745329251994329576923690768489f;
        l.inner_angle = n.inner_angle * d2r;
        l.outer_angle = n.outer_angle * d2r;
        l.type = n.light_type;
        l.num_shadow_samples = sc.shadow_type == LUZ_SHADOW_RAYTRACING ? sc.light_samples : 0;
        l.radius = n.radius;
        l.shadow_map = -1;
        s->lights.push_back(l);
        s->shadow_range.push_back(n.shadow_map_range);
        s->shadow_far.push_back(n.shadow_map_far);
    }
    luz_scene& b = s->block;
    memset(&b, 0, sizeof(b));
    memcpy(b.ambient_light_color, sc.ambient_color, 12);
    b.ambient_light_intensity = sc.ambient_light;
    b.ao_max = sc.ao_max;
    b.ao_min = sc.ao_min;
    b.ao_num_samples = sc.ao_samples > 0 ? sc.ao_samples : 0;
    b.exposure = sc.exposure;
    b.white_texture = b.black_texture = -1;
    b.shadow_type = sc.shadow_type;
    b.sampler = LUZ_SAMPLER_PARITY;
    s->light_samples = sc.light_samples;
    // camera: the scene's main camera (a top-level CameraNode) or a default one
    luz_camera& cam = s->camera;
    memset(&cam, 0, sizeof(cam));
    Node def;
    def.type = kCameraNode;
    const Node* cn = sc.main_camera ? find_top(sc, sc.main_camera) : nullptr;
    if (!cn || cn->type != kCameraNode) cn = &def;
    cam.camera_type = cn->camera_type;
    cam.mode = cn->mode;
    memcpy(cam.eye, cn->eye, 12);
    memcpy(cam.center, cn->center, 12);
    memcpy(cam.rotation, cn->rotation, 12);
    cam.zoom = cn->zoom;
    cam.far_distance = cn->far_distance;
    cam.near_distance = cn->near_distance;
    cam.horizontal_fov = cn->horizontal_fov;
    cam.ortho_far_distance = cn->ortho_far;
    cam.ortho_near_distance = cn->ortho_near;
    cam.extent[0] = (float)width;
    cam.extent[1] = (float)height;
    luz::host::refresh_block(s.get());
    return s.release();
}

// ---------------------------------------------------------------- host scene -> project
Project from_host_scene(const luz_host_scene* s) {
    Project p;
    UuidGen ids(0x5EEDull + s->models.size() * 131 + s->lights.size());
    std::vector<uint64_t> tex_ids, mesh_ids;
    for (size_t k = 0; k < s->textures.size(); ++k) {
        TextureAsset t;
        t.uuid = ids.next();
        t.name = "texture" + std::to_string(k);
        t.width = (int32_t)s->textures[k].width;
        t.height = (int32_t)s->textures[k].height;
        t.channels = 4;
        t.data = s->textures[k].rgba;
        tex_ids.push_back(t.uuid);
        p.textures.push_back(std::move(t));
    }
    for (size_t k = 0; k < s->meshes.size(); ++k) {
        MeshAsset m;
        m.uuid = ids.next();
        m.name = "mesh" + std::to_string(k);
        m.vertices = s->meshes[k].v;
        m.indices = s->meshes[k].i;
        mesh_ids.push_back(m.uuid);
        p.meshes.push_back(std::move(m));
    }
    auto tex = [&](int32_t i) -> uint64_t { return i >= 0 && (size_t)i < tex_ids.size() ? tex_ids[(size_t)i] : 0; };
    SceneAsset sc;
    sc.uuid = ids.next();
    sc.name = "Scene";
    memcpy(sc.ambient_color, s->block.ambient_light_color, 12);
    sc.ambient_light = s->block.ambient_light_intensity;
    sc.ao_samples = s->block.ao_num_samples;
    sc.light_samples = s->light_samples;
    sc.ao_min = s->block.ao_min;
    sc.ao_max = s->block.ao_max;
    sc.exposure = s->block.exposure;
    sc.shadow_type = s->block.shadow_type;
    // camera first, as the main camera
    Node cam;
    cam.type = kCameraNode;
    cam.uuid = ids.next();
    cam.name = "Camera";
    const luz_camera& c = s->camera;
    cam.camera_type = c.camera_type;
    cam.mode = c.mode == 2 ? 0 : c.mode;
    memcpy(cam.eye, c.eye, 12);
    memcpy(cam.center, c.center, 12);
    memcpy(cam.rotation, c.rotation, 12);
    cam.zoom = c.zoom;
    cam.far_distance = c.far_distance;
    cam.near_distance = c.near_distance;
    cam.horizontal_fov = c.horizontal_fov;
    cam.ortho_far = c.ortho_far_distance;
    cam.ortho_near = c.ortho_near_distance;
    if (c.mode == 2) {
        // a look-at camera becomes an orbit camera around `center` with the same eye
        float d[3] = {c.center[0] - c.eye[0], c.center[1] - c.eye[1], c.center[2] - c.eye[2]};
        float len = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
        const float r2d = 57.295779513082320876798154814105f;
        if (len > 0.0f) {
            // viewDir = center - eye = zoom * (cos(-ry) sin(rx), cos(rx), sin(-ry) sin(rx))
            float rx = std::acos(std::min(std::max(d[1] / len, -1.0f), 1.0f));
            float ry = -std::atan2(d[2], d[0]);
            cam.rotation[0] = rx * r2d - 90.0f;
            cam.rotation[1] = ry * r2d - 90.0f;
            cam.rotation[2] = 0.0f;
            cam.zoom = len;
        }
    }
    sc.main_camera = cam.uuid;
    sc.nodes.push_back(cam);
    // one material per instance, identical ones shared
    std::vector<MaterialAsset> mats;
    for (size_t k = 0; k < s->models.size(); ++k) {
        const luz_model& m = s->models[k];
        MaterialAsset ma;
        memcpy(ma.color, m.color, 16);
        memcpy(ma.emission, m.emission, 12);
        ma.metallic = m.metallic;
        ma.roughness = m.roughness;
        ma.color_map = tex(m.color_map);
        ma.normal_map = tex(m.normal_map);
        ma.mr_map = tex(m.metallic_roughness_map);
        ma.emission_map = tex(m.emission_map);
        uint64_t mid = 0;
        for (const auto& e : p.materials)
            if (!memcmp(e.color, ma.color, 16) && !memcmp(e.emission, ma.emission, 12) && e.metallic == ma.metallic &&
                e.roughness == ma.roughness && e.color_map == ma.color_map && e.normal_map == ma.normal_map &&
                e.mr_map == ma.mr_map && e.emission_map == ma.emission_map) {
                mid = e.uuid;
                break;
            }
        if (!mid) {
            ma.uuid = ids.next();
            ma.name = "material" + std::to_string(p.materials.size());
            mid = ma.uuid;
            p.materials.push_back(ma);
        }
        Node n;
        n.type = kMeshNode;
        n.uuid = ids.next();
        n.name = "instance" + std::to_string(k);
        n.mesh = mesh_ids.at(s->instance_mesh[k]);
        n.material = mid;
        n.has_matrix = true;
        memcpy(n.matrix, m.model_mat, 64);
        matrix_to_trs(m.model_mat, n.position, n.rotation, n.scale);
        sc.nodes.push_back(std::move(n));
    }
    const float r2d = 57.295779513082320876798154814105f;
    for (size_t k = 0; k < s->lights.size(); ++k) {
        const luz_light& l = s->lights[k];
        Node n;
        n.type = kLightNode;
        n.uuid = ids.next();
        n.name = "light" + std::to_string(k);
        memcpy(n.position, l.position, 12);
        memcpy(n.color, l.color, 12);
        n.intensity = l.intensity;
        n.light_type = l.type;
        n.radius = l.radius;
        n.inner_angle = l.inner_angle * r2d;
        n.outer_angle = l.outer_angle * r2d;
        n.has_direction = true;
        memcpy(n.direction, l.direction, 12);
        if (k < s->shadow_range.size()) n.shadow_map_range = s->shadow_range[k];
        if (k < s->shadow_far.size()) n.shadow_map_far = s->shadow_far[k];
        // a rotation that takes (0,-1,0) to the direction, for readers of the plain format:
        // pitch about x, then yaw about y
        float dl = std::sqrt(l.direction[0] * l.direction[0] + l.direction[1] * l.direction[1] +
                             l.direction[2] * l.direction[2]);
        if (dl > 0.0f) {
            float dx = l.direction[0] / dl, dy = l.direction[1] / dl, dz = l.direction[2] / dl;
            float pitch = std::acos(std::min(std::max(-dy, -1.0f), 1.0f));
            float yaw = std::atan2(-dx, -dz);
            n.rotation[0] = pitch * r2d;
            n.rotation[1] = yaw * r2d;
        }
        sc.nodes.push_back(std::move(n));
    }
    p.initial_scene = sc.uuid;
    p.scenes.push_back(std::move(sc));
    return p;
}

int copy_error(const std::exception& e, char* err, uint32_t err_len) {
    if (err && err_len) {
        strncpy(err, e.what(), err_len - 1);
        err[err_len - 1] = 0;
    }
    return 0;
}

}  // namespace ingest
}  // namespace luz

using namespace luz::ingest;

extern "C" {

luz_status luz_scene_load_project(const char* luz_path, const char* luzbin_path, uint32_t width, uint32_t height,
                                  luz_host_scene** out, char* err, uint32_t err_len) {
    if (!luz_path || !luzbin_path || !out || width == 0 || height == 0) return LUZ_ERR_INVALID;
    *out = nullptr;
    try {
        Project p = load_project(luz_path, luzbin_path);
        const SceneAsset* sc = nullptr;
        for (const auto& s : p.scenes)
            if (s.uuid == p.initial_scene) sc = &s;
        if (!sc && !p.scenes.empty()) sc = &p.scenes.front();
        if (!sc) fail("project without a scene");
        *out = to_host_scene(p, *sc, width, height);
        return LUZ_OK;
    } catch (const std::bad_alloc&) {
        return LUZ_ERR_OOM;
    } catch (const std::exception& e) {
        copy_error(e, err, err_len);
        return LUZ_ERR_INVALID;
    }
}

luz_status luz_scene_import(const char* path, uint32_t width, uint32_t height, luz_host_scene** out, char* err,
                            uint32_t err_len) {
    if (!path || !out || width == 0 || height == 0) return LUZ_ERR_INVALID;
    *out = nullptr;
    try {
        Project p;
        UuidGen ids(0x1D5EEDull);
        std::string ext = ext_of(path);
        SceneAsset imported;
        if (ext == ".gltf" || ext == ".glb") imported = import_gltf(path, p, ids);
        else if (ext == ".obj") imported = import_obj(path, p, ids);
        else fail(std::string("unsupported scene file ") + path);
        // AssetManager::AddAssetsToScene into the default scene
        SceneAsset scene;
        scene.uuid = ids.next();
        scene.name = "DefaultScene";
        scene.nodes = imported.nodes;
        *out = to_host_scene(p, scene, width, height);
        return LUZ_OK;
    } catch (const std::bad_alloc&) {
        return LUZ_ERR_OOM;
    } catch (const std::exception& e) {
        copy_error(e, err, err_len);
        return LUZ_ERR_INVALID;
    }
}

luz_status luz_scene_save_project(const luz_host_scene* s, const char* luz_path, const char* luzbin_path, char* err,
                                  uint32_t err_len) {
    if (!s || !luz_path || !luzbin_path) return LUZ_ERR_INVALID;
    try {
        save_project(from_host_scene(s), luz_path, luzbin_path);
        return LUZ_OK;
    } catch (const std::bad_alloc&) {
        return LUZ_ERR_OOM;
    } catch (const std::exception& e) {
        copy_error(e, err, err_len);
        return LUZ_ERR_INVALID;
    }
}

}  // extern "C"
