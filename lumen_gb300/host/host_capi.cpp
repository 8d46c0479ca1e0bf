// C entry points of include/lgb_host.h.
#include <cuda_runtime.h>

#include <cstring>
#include <exception>
#include <stdexcept>
#include <string>
#include <vector>

#include <memory>

#include "integrator.h"
#include "lgb_host.h"
#include "lumen_scene.h"

struct lgbh_scene {
    lgbh::LumenScene scene;
};

namespace {
void put_err(const std::string& msg, char* err, size_t errlen) {
    if (!err || errlen == 0) return;
    std::strncpy(err, msg.c_str(), errlen - 1);
    err[errlen - 1] = '\0';
}
}  // namespace

extern "C" {

LGB_API lgb_status lgbh_scene_load(const char* json_path, lgbh_scene** out, char* err, size_t errlen) {
    if (!json_path || !out) return LGB_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    lgbh_scene* s = new lgbh_scene();
    try {
        s->scene.load(json_path);
    } catch (const std::exception& e) {
        put_err(e.what(), err, errlen);
        delete s;
        return LGB_ERR_INVALID_ARGUMENT;
    }
    *out = s;
    return LGB_OK;
}

LGB_API void lgbh_scene_free(lgbh_scene* s) { delete s; }

LGB_API lgb_status lgbh_scene_desc(lgbh_scene* s, lgb_scene_desc* out) {
    if (!s || !out) return LGB_ERR_INVALID_ARGUMENT;
    *out = s->scene.desc();
    return LGB_OK;
}

LGB_API lgb_status lgbh_scene_get_info(lgbh_scene* s, lgbh_scene_info* out) {
    if (!s || !out) return LGB_ERR_INVALID_ARGUMENT;
    const lgbh::LumenScene& sc = s->scene;
    std::memset(out, 0, sizeof(*out));
    for (int a = 0; a < 3; a++) {
        out->cam_pos[a] = sc.config.cam.pos[a];
        out->cam_dir[a] = sc.config.cam.dir[a];
        out->sky_col[a] = sc.config.sky_col[a];
        out->bbox_min[a] = sc.bbox_min[a];
        out->bbox_max[a] = sc.bbox_max[a];
    }
    out->fov = sc.config.cam.fov;
    out->path_length = sc.config.path_length;
    out->light_triangle_count = sc.total_light_triangle_cnt;
    out->dir_light_idx = sc.dir_light_idx;
    out->total_light_area = sc.total_light_area;
    out->radius = sc.radius;
    out->base_radius = sc.config.base_radius;
    out->radius_factor = sc.config.radius_factor;
    out->enable_vm = sc.config.enable_vm ? 1 : 0;
    out->cam_use_matrix = sc.config.cam.use_matrix ? 1 : 0;
    for (int i = 0; i < 16; i++) out->cam_matrix[i] = sc.config.cam.cam_matrix[i];
    return LGB_OK;
}

LGB_API lgb_status lgbh_write_image(const char* path, const float* rgba, uint32_t width, uint32_t height, char* err,
                                    size_t errlen) {
    if (!path || !rgba || width == 0 || height == 0) return LGB_ERR_INVALID_ARGUMENT;
    try {
        lgbh::write_image(path, rgba, width, height);
    } catch (const std::exception& e) {
        put_err(e.what(), err, errlen);
        return LGB_ERR_INVALID_ARGUMENT;
    }
    return LGB_OK;
}

LGB_API lgb_status lgbh_render_path(const char* json_path, int device, uint32_t width, uint32_t height, uint32_t spp,
                                    const char* out_pfm, float* host_rgba, char* err, size_t errlen) {
    if (!json_path || width == 0 || height == 0) return LGB_ERR_INVALID_ARGUMENT;
    lgb_ctx* ctx = nullptr;
    lgb_status st = lgb_create(&ctx, device, nullptr);
    if (st != LGB_OK) {
        put_err("lgb_create failed", err, errlen);
        return st;
    }
    try {
        lgbh::LumenScene scene;
        scene.load(json_path);
        // RayTracer::init picks the integrator named in the scene (RayTracer.cpp:45-60)
        std::unique_ptr<lgbh::Integrator> integrator;
        if (scene.config.integrator == "vcm") integrator.reset(new lgbh::GpuVCM(&scene, ctx, width, height));
        else if (scene.config.integrator == "sppm") integrator.reset(new lgbh::GpuSPPM(&scene, ctx, width, height));
        else if (scene.config.integrator == "restir") integrator.reset(new lgbh::GpuReSTIR(&scene, ctx, width, height));
        else if (scene.config.integrator == "bdpt") integrator.reset(new lgbh::GpuBDPT(&scene, ctx, width, height));
        else if (scene.config.integrator == "path") integrator.reset(new lgbh::GpuPath(&scene, ctx, width, height));
        else throw std::runtime_error("integrator \"" + scene.config.integrator + "\" is not supported (path, vcm, sppm, restir, bdpt)");
        integrator->init();           // RayTracer::init -> integrator->init (RayTracer.cpp:61-65)
        integrator->create_accel();   // integrator->create_accel
        for (uint32_t f = 0; f < spp; f++) {  // the frame loop: render, then update (RayTracer.cpp:167-197)
            integrator->render();
            integrator->update();
        }
        st = lgb_sync(integrator->gpu_scene(), nullptr);
        if (st != LGB_OK) throw std::runtime_error(lgb_last_error(ctx));
        std::vector<float> film((size_t)width * height * 4);
        if (cudaMemcpy(film.data(), integrator->output_film, film.size() * 4, cudaMemcpyDeviceToHost) != cudaSuccess)
            throw std::runtime_error("film read-back failed");
        if (out_pfm) lgbh::write_image(out_pfm, film.data(), width, height);
        if (host_rgba) std::memcpy(host_rgba, film.data(), film.size() * 4);
    } catch (const lgbh::LgbCallError& e) {
        put_err(e.what(), err, errlen);
        lgb_destroy(ctx);
        return e.status;
    } catch (const std::exception& e) {
        put_err(e.what(), err, errlen);
        lgb_destroy(ctx);
        return st != LGB_OK ? st : LGB_ERR_INVALID_ARGUMENT;
    }
    lgb_destroy(ctx);
    return LGB_OK;
}

}  // extern "C"
