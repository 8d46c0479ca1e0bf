/* lgb_host.h -- C entry points of the headless host layer (liblgb_host.so) above the lgb.h ABI.
 *
 * These mirror the caller side of Lumen's path: LumenScene::load_scene (src/RayTracer/LumenScene.cpp:52-513)
 * and the Path integrator's frame loop (src/RayTracer/Path.cpp, RayTracer.cpp:167-197), without a window.
 * They exist so that C, Python or a command line can load a Lumen JSON scene and render it headless.
 */
#ifndef LGB_HOST_H
#define LGB_HOST_H

#include "lgb.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct lgbh_scene lgbh_scene;

typedef struct lgbh_scene_info {
    float cam_pos[3];
    float cam_dir[3];
    float fov;
    int32_t path_length;
    float sky_col[3];
    uint32_t light_triangle_count;
    uint32_t dir_light_idx;
    float total_light_area;
    float bbox_min[3];
    float bbox_max[3];
    float radius;
    float base_radius;    /* SPPM integrator block (SPPMConfig::base_radius) */
    float radius_factor;  /* VCM integrator block (VCMConfig::radius_factor) */
    int32_t enable_vm;    /* VCM integrator block (VCMConfig::enable_vm) */
    int32_t cam_use_matrix;   /* 1: the camera is cam_matrix (Mitsuba sensors), not cam_pos / cam_dir */
    float cam_matrix[16];     /* camera-to-world, column-major, for lgb_camera_from_matrix */
} lgbh_scene_info;

/* Loads a Lumen JSON scene and its OBJ (LumenScene::load_lumen_scene, LumenScene.cpp:231-513), or a Mitsuba
 * XML scene and its OBJ shapes when the path ends in ".xml" (LumenScene::load_mitsuba_scene,
 * LumenScene.cpp:514-690). On failure returns LGB_ERR_INVALID_ARGUMENT and copies the message into err (up to
 * errlen bytes). */
LGB_API lgb_status lgbh_scene_load(const char* json_path, lgbh_scene** out, char* err, size_t errlen);
LGB_API void lgbh_scene_free(lgbh_scene* s);
/* The loaded arrays as an lgb_scene_desc (pointers stay valid until lgbh_scene_free). */
LGB_API lgb_status lgbh_scene_desc(lgbh_scene* s, lgb_scene_desc* out);
LGB_API lgb_status lgbh_scene_get_info(lgbh_scene* s, lgbh_scene_info* out);
/* Writes an RGBA32F film (width*height*4 floats, row 0 at the top) as OpenEXR when the path ends in ".exr"
 * (uncompressed FLOAT B, G, R: Lumen saves its film as EXR, ImageUtils.cpp:22-89), else as RGB PFM. */
LGB_API lgb_status lgbh_write_image(const char* path, const float* rgba, uint32_t width, uint32_t height, char* err,
                                    size_t errlen);
/* Headless render with the scene's integrator (Path; VCM with seeds from the deterministic sequence of GpuVCM,
 * light_seed / eye_seed = vcm_seeds(0, frame); SPPM, BDPT and ReSTIR DI with seed = the light seed of
 * vcm_seeds(0, frame)): init, create_accel, then `spp` frames of render/update, film
 * written to out_pfm (OpenEXR if it ends in ".exr", else RGB PFM; skipped when null) and copied to host_rgba (width*height*4 floats; skipped when
 * null). */
LGB_API lgb_status lgbh_render_path(const char* json_path, int device, uint32_t width, uint32_t height, uint32_t spp,
                                    const char* out_pfm, float* host_rgba, char* err, size_t errlen);

#ifdef __cplusplus
}
#endif
#endif /* LGB_HOST_H */
