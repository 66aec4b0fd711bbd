// scene_internal.hpp — the host scene object shared by the generators (scene.cpp)
// and the scene-file importers (ingest.cpp).
#pragma once
#include <cstdint>
#include <vector>

#include "../../include/luz_scene.h"

namespace luz {
namespace host {

struct Mesh {
    std::vector<luz_vertex> v;
    std::vector<uint32_t> i;
};

struct Texture {             // RGBA8, rows top to bottom
    uint32_t width = 0, height = 0;
    std::vector<uint8_t> rgba;
};

luz_model default_model();   // GPUScene's default ModelBlock: white, roughness 0.5, no maps
// Recomputes the SceneBlock matrices from the camera (view, proj, inverses, prev = current).
void refresh_block(luz_host_scene* s);
// Node::ComposeTransform: parent * T * R(quat(radians(rot))) * S, column-major.
void compose_transform(const float pos[3], const float rot_deg[3], const float scl[3], const float parent[16],
                       float out[16]);

}  // namespace host
}  // namespace luz

struct luz_host_scene {
    std::vector<luz::host::Mesh> meshes;
    std::vector<uint32_t> instance_mesh;
    std::vector<luz_model> models;
    std::vector<luz_light> lights;
    std::vector<luz::host::Texture> textures;   // indexed by the ModelBlocks' map fields
    luz_scene block{};
    luz_camera camera{};
    uint32_t width = 0, height = 0;
    int32_t light_samples = 1;
    uint32_t jitter_index = 0;   // CameraNode::jitterIndex
    std::vector<float> shadow_range, shadow_far;   // per light; defaults 3 and 2000 when missing
    float prev_view_proj[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
};
