// ref_ingest.cpp — TEST INFRASTRUCTURE. Drives the reference renderer's own scene
// importers and project (de)serialiser (hadryansalles/Luz source/Resources/AssetIO.cpp,
// AssetManager.cpp, compiled from the reference tree by `make ref` into oracle/_ref/)
// and dumps what they produce as JSON, packed the way GPUScene::UpdateResources packs
// a scene (source/Graphics/GPUScene.cpp:181-346): per MeshNode of a pre-order walk
// its world matrix, material and mesh; per LightNode its LightBlock fields; the
// scene settings and the main camera. tests/golden/make_ingest_golden.py turns these
// dumps into committed fixtures.
//
// The editor and profiler symbols the two translation units reference (ImGui tree
// widgets, TimeScope's destructor) are stubbed here; they are not on the import path.
#include <cstdio>
#include <fstream>
#include <string>
#include <vector>

#include "AssetIO.hpp"
#include "AssetManager.hpp"

namespace ImGui {
bool TreeNode(const void*, const char*, ...) { return false; }
void TreePop() {}
}  // namespace ImGui
TimeScope::~TimeScope() {}

namespace {

uint32_t crc32(const uint8_t* p, size_t n) {
    uint32_t c = 0xFFFFFFFFu;
    for (size_t k = 0; k < n; ++k) {
        c ^= p[k];
        for (int b = 0; b < 8; ++b) c = (c >> 1) ^ (0xEDB88320u & (0u - (c & 1u)));
    }
    return ~c;
}

struct Out {
    std::string s;
    void f(float v) {
        char b[48];
        snprintf(b, sizeof b, "%.9g", (double)v);
        std::string t(b);
        if (t == "nan" || t == "-nan" || t == "inf" || t == "-inf") t = "\"" + t + "\"";
        else if (t.find_first_of(".e") == std::string::npos) t += ".0";   // keeps -0.0 a float
        s += t;
    }
    void fs(const float* v, int n) {
        s += "[";
        for (int k = 0; k < n; ++k) {
            if (k) s += ",";
            f(v[k]);
        }
        s += "]";
    }
    void u(uint64_t v) { s += std::to_string(v); }
    void i(int64_t v) { s += std::to_string(v); }
    void str(const std::string& v) {
        s += "\"";
        for (char c : v) {
            if (c == '"' || c == '\\') s += '\\';
            s += c;
        }
        s += "\"";
    }
};

void dump_scene(const Ref<SceneAsset>& scene, const Ref<CameraNode>& camera, const std::string& path) {
    Out o;
    std::vector<Ref<MeshNode>> meshNodes;
    scene->GetAll<MeshNode>(ObjectType::MeshNode, meshNodes);
    std::vector<UUID> meshes, textures;
    std::vector<Ref<MeshAsset>> meshRefs;
    std::vector<Ref<TextureAsset>> texRefs;
    auto meshIndex = [&](const Ref<MeshAsset>& m) {
        for (size_t k = 0; k < meshes.size(); ++k)
            if (meshes[k] == m->uuid) return (int)k;
        meshes.push_back(m->uuid);
        meshRefs.push_back(m);
        return (int)meshes.size() - 1;
    };
    auto texIndex = [&](const Ref<TextureAsset>& t) {
        if (!t) return -1;
        for (size_t k = 0; k < textures.size(); ++k)
            if (textures[k] == t->uuid) return (int)k;
        textures.push_back(t->uuid);
        texRefs.push_back(t);
        return (int)textures.size() - 1;
    };
    o.s += "{\"instances\":[";
    for (size_t k = 0; k < meshNodes.size(); ++k) {
        const auto& n = meshNodes[k];
        if (k) o.s += ",";
        glm::mat4 w = n->GetWorldTransform();
        o.s += "{\"world\":";
        o.fs(&w[0][0], 16);
        o.s += ",\"mesh\":";
        o.i(meshIndex(n->mesh));
        o.s += ",\"name\":";
        o.str(n->name);
        if (n->material) {
            const auto& m = n->material;
            o.s += ",\"material\":{\"color\":";
            o.fs(&m->color[0], 4);
            o.s += ",\"emission\":";
            o.fs(&m->emission[0], 3);
            o.s += ",\"metallic\":";
            o.f(m->metallic);
            o.s += ",\"roughness\":";
            o.f(m->roughness);
            o.s += ",\"colorMap\":";
            o.i(texIndex(m->colorMap));
            o.s += ",\"normalMap\":";
            o.i(texIndex(m->normalMap));
            o.s += ",\"metallicRoughnessMap\":";
            o.i(texIndex(m->metallicRoughnessMap));
            o.s += ",\"emissionMap\":";
            o.i(texIndex(m->emissionMap));
            o.s += "}";
        }
        o.s += "}";
    }
    o.s += "],\"meshes\":[";
    for (size_t k = 0; k < meshRefs.size(); ++k) {
        const auto& m = meshRefs[k];
        if (k) o.s += ",";
        o.s += "{\"name\":";
        o.str(m->name);
        o.s += ",\"vertices\":[";
        for (size_t v = 0; v < m->vertices.size(); ++v) {
            if (v) o.s += ",";
            o.fs(&m->vertices[v].position[0], 12);
        }
        o.s += "],\"indices\":[";
        for (size_t i = 0; i < m->indices.size(); ++i) {
            if (i) o.s += ",";
            o.u(m->indices[i]);
        }
        o.s += "]}";
    }
    o.s += "],\"textures\":[";
    for (size_t k = 0; k < texRefs.size(); ++k) {
        const auto& t = texRefs[k];
        if (k) o.s += ",";
        o.s += "{\"width\":";
        o.i(t->width);
        o.s += ",\"height\":";
        o.i(t->height);
        o.s += ",\"channels\":";
        o.i(t->channels);
        o.s += ",\"crc32\":";
        o.u(crc32(t->data.data(), t->data.size()));
        o.s += "}";
    }
    o.s += "],\"lights\":[";
    auto lights = scene->GetAll<LightNode>(ObjectType::LightNode);
    for (size_t k = 0; k < lights.size(); ++k) {
        const auto& l = lights[k];
        if (k) o.s += ",";
        glm::vec3 pos = l->GetWorldPosition();
        glm::vec3 dir = l->GetWorldTransform() * glm::vec4(0, -1, 0, 0);
        o.s += "{\"color\":";
        o.fs(&l->color[0], 3);
        o.s += ",\"intensity\":";
        o.f(l->intensity);
        o.s += ",\"position\":";
        o.fs(&pos[0], 3);
        o.s += ",\"direction\":";
        o.fs(&dir[0], 3);
        o.s += ",\"innerAngle\":";
        o.f(glm::radians(l->innerAngle));
        o.s += ",\"outerAngle\":";
        o.f(glm::radians(l->outerAngle));
        o.s += ",\"type\":";
        o.i((int)l->lightType);
        o.s += ",\"radius\":";
        o.f(l->radius);
        o.s += "}";
    }
    o.s += "],\"scene\":{\"ambientLight\":";
    o.f(scene->ambientLight);
    o.s += ",\"ambientLightColor\":";
    o.fs(&scene->ambientLightColor[0], 3);
    o.s += ",\"aoSamples\":";
    o.i(scene->aoSamples);
    o.s += ",\"lightSamples\":";
    o.i(scene->lightSamples);
    o.s += ",\"aoMin\":";
    o.f(scene->aoMin);
    o.s += ",\"aoMax\":";
    o.f(scene->aoMax);
    o.s += ",\"exposure\":";
    o.f(scene->exposure);
    o.s += ",\"shadowType\":";
    o.i((int)scene->shadowType);
    o.s += "}";
    if (camera) {
        o.s += ",\"camera\":{\"cameraType\":";
        o.i((int)camera->cameraType);
        o.s += ",\"mode\":";
        o.i((int)camera->mode);
        o.s += ",\"eye\":";
        o.fs(&camera->eye[0], 3);
        o.s += ",\"center\":";
        o.fs(&camera->center[0], 3);
        o.s += ",\"rotation\":";
        o.fs(&camera->rotation[0], 3);
        o.s += ",\"zoom\":";
        o.f(camera->zoom);
        o.s += ",\"farDistance\":";
        o.f(camera->farDistance);
        o.s += ",\"nearDistance\":";
        o.f(camera->nearDistance);
        o.s += ",\"horizontalFov\":";
        o.f(camera->horizontalFov);
        o.s += "}";
    }
    o.s += "}";
    std::ofstream f(path);
    f << o.s;
}

bool g_logger = false;
void init_logger() {
    if (!g_logger) {
        Logger::Init();
        g_logger = true;
    }
}

}  // namespace

extern "C" {

// AssetManager::AddAssetsToScene of one file into a fresh default scene, dumped.
int ref_import_dump(const char* path, const char* out_json) {
    init_logger();
    AssetManager manager;
    Ref<SceneAsset> scene = manager.CreateAsset<SceneAsset>("DefaultScene");
    auto added = manager.AddAssetsToScene(scene, {std::string(path)});
    dump_scene(scene, nullptr, out_json);
    return (int)added.size();
}

// The same import saved with AssetManager::SaveProject.
int ref_save_import(const char* path, const char* out_luz, const char* out_luzbin) {
    init_logger();
    AssetManager manager;
    Ref<SceneAsset> scene = manager.CreateAsset<SceneAsset>("DefaultScene");
    manager.AddAssetsToScene(scene, {std::string(path)});
    manager.SaveProject(out_luz, out_luzbin);
    return 0;
}

// AssetManager::LoadProject, then the initial scene dumped (main camera when set).
int ref_load_dump(const char* luz, const char* luzbin, const char* out_json) {
    init_logger();
    AssetManager manager;
    manager.LoadProject(luz, luzbin);
    Ref<SceneAsset> scene = manager.GetInitialScene();
    dump_scene(scene, scene->mainCamera, out_json);
    return 0;
}

}  // extern "C"
