// Headless scene loading for the C ABI: the part of Lumen's LumenScene that produces the flat arrays the
// path reads (src/RayTracer/LumenScene.cpp:52-229 for the arrays and light list, :231-513 for the JSON + OBJ
// scene format, :732-751 for the scene bounds). The loader is our own code for the same file format.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "lgb.h"

namespace lgbh {

struct TextureData {
    uint32_t width = 0, height = 0;
    std::vector<float> rgba;  // linear FP32, row-major
};

struct CameraSettings {  // SceneConfig.h:6-11
    float fov = 45.0f;
    float pos[3] = {0, 0, 0};
    float dir[3] = {0, 0, 1};
    // Mitsuba sensors give a matrix instead (LumenScene.cpp:64-68): the camera-to-world matrix the render loop
    // uses, column-major, after Lumen's Euler-angle round trip (see LumenScene::load_mitsuba).
    bool use_matrix = false;
    float cam_matrix[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
};

struct SceneConfig {  // SceneConfig.h:15-63 (the fields the Path and VCM integrators read)
    std::string integrator = "path";
    int path_length = 6;
    bool enable_vm = false;        // VCMConfig
    float radius_factor = 0.025f;  // VCMConfig
    float base_radius = 0.03f;     // SPPMConfig (SceneConfig.h:34)
    float sky_col[3] = {0, 0, 0};
    CameraSettings cam;
};

class LumenScene {
  public:
    // Loads a Lumen JSON scene and the OBJ it names, or a Mitsuba XML scene and its OBJ shapes (by extension,
    // as LumenScene::load_scene, LumenScene.cpp:52-57). Throws std::runtime_error with a message on failure.
    void load(const std::string& path);

    // Flat arrays, exactly as the C ABI takes them.
    std::vector<float> positions, normals, uvs;  // 3, 3, 2 floats per vertex
    std::vector<uint32_t> indices;
    std::vector<lgb_mesh> meshes;
    std::vector<std::string> mesh_names;
    std::vector<lgb_material> materials;
    std::vector<lgb_light> lights;          // area lights of emissive meshes first, then JSON lights
    std::vector<TextureData> textures;
    uint32_t total_light_triangle_cnt = 0;  // LumenScene.cpp:94,106
    float total_light_area = 0.0f;
    uint32_t dir_light_idx = 0xFFFFFFFFu;
    float bbox_min[3] = {0, 0, 0}, bbox_max[3] = {0, 0, 0}, radius = 0.0f;
    SceneConfig config;

    lgb_scene_desc desc() const;  // points into the vectors above
    std::vector<lgb_texture> texture_views() const;

  private:
    void load_json(const std::string& path);
    void load_mitsuba(const std::string& path);
    void finish_lights(const std::vector<lgb_light>& listed);
    void load_obj(const std::string& path);
    mutable std::vector<lgb_texture> tex_views_;
};

// Reads a PFM image ("PF" colour or "Pf" grey, either endianness) into linear RGBA.
TextureData read_pfm(const std::string& path);
// Writes RGB of an RGBA32F host film as a little-endian colour PFM (rows bottom-up as PFM stores them).
void write_pfm(const std::string& path, const float* rgba, uint32_t width, uint32_t height);
// OpenEXR (uncompressed FLOAT B, G, R scanlines), the format Lumen saves its film in (ImageUtils.cpp:22-89).
void write_exr(const std::string& path, const float* rgba, uint32_t width, uint32_t height);
// By extension: ".exr" -> write_exr, otherwise write_pfm.
void write_image(const std::string& path, const float* rgba, uint32_t width, uint32_t height);

}  // namespace lgbh
