#include "integrator.h"

#include <cuda_runtime.h>

#include <stdexcept>
#include <string>

namespace lgbh {

void Integrator::check(lgb_status st, const char* what) {
    if (st != LGB_OK) throw LgbCallError(st, std::string(what) + ": " + lgb_last_error(ctx));
}

void Integrator::init() {
    const lgb_scene_desc d = lumen_scene->desc();
    check(lgb_scene_create(ctx, &d, &scene), "lgb_scene_create");
    const size_t bytes = sizeof(float) * 4 * (size_t)width * height;
    if (cudaMalloc((void**)&output_film, bytes) != cudaSuccess) throw std::runtime_error("film allocation failed");
    cudaMemset(output_film, 0, bytes);
    update();
}

bool Integrator::update() {
    const CameraSettings& c = lumen_scene->config.cam;
    if (c.use_matrix)
        check(lgb_camera_from_matrix(c.cam_matrix, c.fov, width, height, &cam), "lgb_camera_from_matrix");
    else
        check(lgb_camera_lookat(c.pos, c.dir, c.fov, width, height, &cam), "lgb_camera_lookat");
    return updated;
}

void Integrator::destroy() {
    if (output_film) cudaFree(output_film);
    output_film = nullptr;
    if (scene) lgb_scene_destroy(scene);
    scene = nullptr;
}

void Integrator::create_accel(const lgb_build_opts* opts) { check(lgb_bvh_build(scene, opts, &accel_stats), "lgb_bvh_build"); }

void GpuPath::init() {
    Integrator::init();
    frame_num = 0;
    path_length = (uint32_t)lumen_scene->config.path_length;  // Path::init (Path.cpp:24)
}

void GpuPath::render() {  // Path::render (Path.cpp:27-59)
    lgb_path_params p{};
    for (int i = 0; i < 3; i++) p.sky_col[i] = lumen_scene->config.sky_col[i];
    p.max_depth = (int32_t)path_length;
    p.num_lights = (int32_t)lumen_scene->lights.size();
    p.light_triangle_count = (int32_t)lumen_scene->total_light_triangle_cnt;
    p.dir_light_idx = lumen_scene->dir_light_idx;
    p.direct_lighting = direct_lighting ? 1u : 0u;
    check(lgb_render_path(scene, &cam, &p, frame_num, 1, output_film, stream), "lgb_render_path");
}

bool GpuPath::update() {  // Path::update (Path.cpp:61-68)
    frame_num++;
    const bool changed = Integrator::update();
    if (changed) frame_num = 0;
    return changed;
}

static uint32_t hash32(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}

void vcm_seeds(uint32_t seed, uint32_t frame, uint32_t* light_seed, uint32_t* eye_seed) {
    *light_seed = hash32(seed * 0x9e3779b9u + 2u * frame + 1u);
    *eye_seed = hash32(seed * 0x9e3779b9u + 2u * frame + 2u);
}

void GpuVCM::init() {
    Integrator::init();
    frame_num = 0;
    path_length = (uint32_t)lumen_scene->config.path_length;
}

void GpuVCM::render() {  // VCM::render (VCM.cpp:131-265)
    lgb_vcm_params p{};
    for (int i = 0; i < 3; i++) {
        p.sky_col[i] = lumen_scene->config.sky_col[i];
        p.scene_min[i] = lumen_scene->bbox_min[i];
        p.scene_max[i] = lumen_scene->bbox_max[i];
    }
    p.max_depth = (int32_t)path_length;
    p.num_lights = (int32_t)lumen_scene->lights.size();
    p.light_triangle_count = (int32_t)lumen_scene->total_light_triangle_cnt;
    p.dir_light_idx = lumen_scene->dir_light_idx;
    p.radius = lgb_vcm_radius(lumen_scene->radius, lumen_scene->config.radius_factor, frame_num, 2.0f / 3.0f);
    p.use_vm = lumen_scene->config.enable_vm ? 1 : 0;
    p.use_vc = 1;
    vcm_seeds(seed, frame_num, &p.light_seed, &p.eye_seed);
    p.frame_num = frame_num;
    check(lgb_vcm_iteration(scene, &cam, &p, output_film, stream), "lgb_vcm_iteration");
}

bool GpuVCM::update() {  // VCM::update (VCM.cpp:267-274)
    frame_num++;
    const bool changed = Integrator::update();
    if (changed) frame_num = 0;
    return changed;
}

void GpuSPPM::init() {
    Integrator::init();
    frame_num = 0;
    path_length = (uint32_t)lumen_scene->config.path_length;
    base_radius = lumen_scene->config.base_radius;
}

void GpuSPPM::render() {  // SPPM::render (SPPM.cpp:78-184)
    lgb_sppm_params p{};
    for (int i = 0; i < 3; i++) p.sky_col[i] = lumen_scene->config.sky_col[i];
    p.max_depth = (int32_t)path_length;
    p.num_lights = (int32_t)lumen_scene->lights.size();
    p.light_triangle_count = (int32_t)lumen_scene->total_light_triangle_cnt;
    p.dir_light_idx = lumen_scene->dir_light_idx;
    p.base_radius = base_radius;
    uint32_t unused;
    vcm_seeds(seed, frame_num, &p.seed, &unused);
    p.frame_num = frame_num;
    check(lgb_sppm_iteration(scene, &cam, &p, output_film, stream), "lgb_sppm_iteration");
}

bool GpuSPPM::update() {  // SPPM::update (SPPM.cpp:186-192)
    frame_num++;
    const bool changed = Integrator::update();
    if (changed) frame_num = 0;
    return changed;
}

void GpuBDPT::init() {
    Integrator::init();
    frame_num = 0;
    path_length = (uint32_t)lumen_scene->config.path_length;
}

void GpuBDPT::render() {  // BDPT::render (BDPT.cpp:55-88)
    lgb_bdpt_params p{};
    for (int i = 0; i < 3; i++) p.sky_col[i] = lumen_scene->config.sky_col[i];
    p.max_depth = (int32_t)path_length;
    p.num_lights = (int32_t)lumen_scene->lights.size();
    p.light_triangle_count = (int32_t)lumen_scene->total_light_triangle_cnt;
    p.dir_light_idx = lumen_scene->dir_light_idx;
    uint32_t unused;
    vcm_seeds(seed, frame_num, &p.seed, &unused);
    p.frame_num = frame_num;
    check(lgb_bdpt_iteration(scene, &cam, &p, output_film, stream), "lgb_bdpt_iteration");
}

bool GpuBDPT::update() {  // BDPT::update (BDPT.cpp:90-97)
    frame_num++;
    const bool changed = Integrator::update();
    if (changed) frame_num = 0;
    return changed;
}

void GpuReSTIR::init() {
    Integrator::init();
    frame_num = 0;
    do_spatiotemporal = false;
    prev_cam_ = cam;
}

void GpuReSTIR::render() {  // ReSTIR::render (ReSTIR.cpp:74-157)
    lgb_restir_params p{};
    for (int i = 0; i < 3; i++) p.sky_col[i] = lumen_scene->config.sky_col[i];
    p.max_depth = lumen_scene->config.path_length;
    p.num_lights = (int32_t)lumen_scene->lights.size();
    p.light_triangle_count = (int32_t)lumen_scene->total_light_triangle_cnt;
    p.dir_light_idx = lumen_scene->dir_light_idx;
    uint32_t unused;
    vcm_seeds(seed, frame_num, &p.seed, &unused);
    p.frame_num = frame_num;
    p.do_spatiotemporal = do_spatiotemporal ? 1u : 0u;
    p.enable_accumulation = enable_accumulation ? 1u : 0u;
    p.flags = flags;
    check(lgb_restir_di_iteration(scene, &cam, &prev_cam_, &p, output_film, stream), "lgb_restir_di_iteration");
    do_spatiotemporal = true;
    prev_cam_ = cam;
}

bool GpuReSTIR::update() {  // ReSTIR::update (ReSTIR.cpp:159-165)
    frame_num++;
    const bool changed = Integrator::update();
    if (changed) frame_num = 0;
    return changed;
}

}  // namespace lgbh
