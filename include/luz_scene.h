/*
 * luz_scene.h — host-side scene layer of the path (C++17 behind a C ABI).
 *
 * It stands where the reference's GPUScene::UpdateResources
 * (source/Graphics/GPUScene.cpp:181-346) and the scene graph math of
 * source/Resources/AssetManager.cpp sit: it turns a scene description into the
 * inputs of include/luz.h (meshes, instances with ModelBlocks, LightBlocks and the
 * SceneBlock constants). It also holds the seeded synthetic scene generators the
 * benchmarks and tests use. No GPU work happens here.
 */
#ifndef LUZ_GB300_SCENE_H
#define LUZ_GB300_SCENE_H

#include "luz.h"

#ifdef __cplusplus
extern "C" {
#endif

/* CameraNode (source/Resources/AssetManager.hpp:229-275). mode: 0 = Orbit, 1 = Fly
 * (CameraNode::GetView, AssetManager.cpp:334-355), 2 = look-at from eye to center. */
typedef struct luz_camera {
    int32_t camera_type;      /* 0 perspective, 1 orthographic */
    int32_t mode;
    float eye[3];
    float center[3];
    float rotation[3];        /* degrees */
    float zoom;
    float far_distance;
    float near_distance;
    float horizontal_fov;     /* degrees; passed to perspective() as fovy (AssetManager.cpp:368) */
    float ortho_far_distance;
    float ortho_near_distance;
    float extent[2];          /* viewport size in pixels */
    float jitter[2];          /* NDC jitter (CameraNode::NextJitter); 0 = off */
} luz_camera;

/* Parameters of the synthetic scene generators (the configs are listed at
 * luz_scene_default_params). Fields left 0 take the config's default. */
typedef struct luz_gen_params {
    int32_t config;
    uint32_t pad0;
    uint64_t seed;
    uint32_t width, height;
    int32_t ao_samples;       /* -1 = config default */
    float ao_max;             /* 0 = config default  */
    int32_t light_samples;    /* 0 = 1               */
    int32_t sampler;          /* LUZ_SAMPLER_*       */
    uint32_t meshes, instances, subdivisions;
    uint32_t point_lights, spot_lights, directional_lights;
    uint32_t triangles;       /* config 6 */
    uint32_t pad1;
} luz_gen_params;

typedef struct luz_host_scene luz_host_scene;

/* Default parameters of a generated workload (seed 1000 + config, 1 shadow sample per
 * light, the parity sampler); nonzero fields of the params override the defaults:
 *   1  512x512: 64 unit cubes on a 20x20 quad, 1 directional + 4 point lights,
 *      4 AO rays per pixel (aoMax 1), fixed camera;
 *   2  1920x1080: 64 displaced icospheres of 81,920 triangles, 1024 instances in a
 *      200-unit box, 1 directional + 32 point + 8 spot lights, 16 AO rays (aoMax 2),
 *      camera at the centre of the instance cloud;
 *   3  as 1 with a random camera (training and held-out scenes of the denoiser);
 *   5  3840x2160: as 2 with 4096 instances, 1 + 128 + 16 lights and 64 AO rays;
 *   6  512x512: a triangle budget (params.triangles, default 100,000) filled with
 *      cubes below 20,000 triangles, else with icospheres of the needed subdivision
 *      (one scene of the many-scene batch).
 * Any other config returns LUZ_ERR_INVALID. */
luz_status luz_scene_default_params(int32_t config, luz_gen_params* out);
/* Generates the scene the params describe. subdivisions above 10 return
 * LUZ_ERR_LIMIT; a scene that does not fit in host memory returns LUZ_ERR_OOM. */
luz_status luz_scene_generate(const luz_gen_params* params, luz_host_scene** out);
void luz_scene_destroy(luz_host_scene* scene);

uint32_t luz_scene_mesh_count(const luz_host_scene* s);
luz_status luz_scene_mesh(const luz_host_scene* s, uint32_t i, const luz_vertex** vertices,
                          uint32_t* vertex_count, const uint32_t** indices, uint32_t* index_count);
uint32_t luz_scene_instance_count(const luz_host_scene* s);
/* Mesh index of each instance. */
const uint32_t* luz_scene_instance_mesh(const luz_host_scene* s);
/* ModelBlock of each instance (custom index i = model i, as GPUScene.cpp:188-191). */
const luz_model* luz_scene_models(const luz_host_scene* s);
uint32_t luz_scene_light_count(const luz_host_scene* s);
const luz_light* luz_scene_lights(const luz_host_scene* s);
const luz_scene* luz_scene_block(const luz_host_scene* s);
uint32_t luz_scene_width(const luz_host_scene* s);
uint32_t luz_scene_height(const luz_host_scene* s);
/* Instance transforms as VkTransformMatrixKHR rows (VulkanWrapper.cpp:1122-1126):
 * count*12 floats, row-major 3x4 = the first three rows of modelMat. */
luz_status luz_scene_instance_transforms(const luz_host_scene* s, float* out);
luz_status luz_scene_set_camera(luz_host_scene* s, const luz_camera* cam);
luz_status luz_scene_get_camera(const luz_host_scene* s, luz_camera* cam);
/* Sample counts: aoSamples/aoMin/aoMax (GPUScene.cpp:333-335) and lightSamples,
 * which becomes every light's numShadowSamples (GPUScene.cpp:248). */
luz_status luz_scene_set_sampling(luz_host_scene* s, int32_t ao_samples, float ao_min, float ao_max,
                                  int32_t light_samples, int32_t sampler);

/* Shadow-map matrices of every light (GPUScene.cpp:266-303): point lights six
 * 90-degree perspective cube faces (near 0, far = shadowMapFar), others an
 * orthographic box fitted to the camera frustum cut at farDistance / shadowMapRange,
 * including the reference's start of the fit's min/max at a world-space corner.
 * out holds luz_scene_light_count entries. */
luz_status luz_scene_shadow_lights(const luz_host_scene* s, luz_shadow_light* out);
/* SceneAsset::shadowType (LUZ_SHADOW_*); lights trace lightSamples shadow rays only
 * under LUZ_SHADOW_RAYTRACING (GPUScene.cpp:248). */
luz_status luz_scene_set_shadow_type(luz_host_scene* s, int32_t shadow_type);

/* Advances one frame as GPUScene::UpdateResources does (GPUScene.cpp:223-233):
 * prevViewProj / prevJitter take the current values, the camera steps its jitter
 * (CameraNode::NextJitter: Halton(2,3) over 16 frames, scaled to +-1 pixel; zero
 * when use_jitter is 0) and the SceneBlock matrices are recomputed. */
luz_status luz_scene_next_frame(luz_host_scene* s, int32_t use_jitter);

/* Node::ComposeTransform (AssetManager.cpp:38-43): parent * T * R(quat(radians(rot))) * S.
 * parent may be NULL (identity); a NULL pos, rot_deg or scale takes a Node's default
 * (0, 0, 1); nothing is written when out is NULL. Column-major 4x4 out. */
void luz_compose_transform(const float pos[3], const float rot_deg[3], const float scale[3],
                           const float* parent, float out[16]);
/* CameraNode::GetView and GetProjJittered (AssetManager.cpp:334-377). */
void luz_camera_matrices(const luz_camera* cam, float view[16], float proj[16]);
/* Seeded RGBA8 substitute for the missing assets/blue_noise.png. */
luz_status luz_blue_noise_generate(uint64_t seed, uint32_t size, uint8_t* rgba8);

/* ------------------------------------------------------------------ scene files
 * The reference's project files and importers: AssetManager::LoadProject /
 * SaveProject (source/Resources/AssetManager.cpp:183-258, format of
 * source/Resources/Serializer.hpp: a .luz JSON document plus a .luzbin binary
 * store) and AssetIO::ImportSceneGLTF / ImportSceneOBJ
 * (source/Resources/AssetIO.cpp:117-529). A loaded scene is packed as
 * GPUScene::UpdateResources packs one (GPUScene.cpp:181-346): MeshNodes of a
 * pre-order walk become instances with ModelBlocks, LightNodes LightBlocks; the
 * project's main camera (or a default CameraNode) gets extent width x height.
 * Textures (RGBA8) are numbered by first use and the ModelBlocks' map fields index
 * them. Images in glTF / OBJ files must be PNG. On failure a message goes to err
 * (err_len bytes, may be NULL). */
luz_status luz_scene_load_project(const char* luz_path, const char* luzbin_path, uint32_t width, uint32_t height,
                                  luz_host_scene** out, char* err, uint32_t err_len);
/* A .gltf / .glb / .obj file added to an empty default scene (AssetManager::
 * AddAssetsToScene, AssetManager.cpp:273-288). */
luz_status luz_scene_import(const char* path, uint32_t width, uint32_t height, luz_host_scene** out, char* err,
                            uint32_t err_len);
/* Writes a scene as a .luz / .luzbin pair the reference's LoadProject reads (one
 * MeshNode per instance, one LightNode per light, the camera as the main camera).
 * Nodes also carry their exact matrix ("luzMatrix") and lights their exact direction
 * ("luzDirection"), which luz_scene_load_project prefers, so scenes round-trip
 * bit for bit through this library. */
luz_status luz_scene_save_project(const luz_host_scene* s, const char* luz_path, const char* luzbin_path, char* err,
                                  uint32_t err_len);
uint32_t luz_scene_texture_count(const luz_host_scene* s);
luz_status luz_scene_texture(const luz_host_scene* s, uint32_t i, const uint8_t** rgba8, uint32_t* width,
                             uint32_t* height);

#ifdef __cplusplus
}
#endif
#endif /* LUZ_GB300_SCENE_H */
