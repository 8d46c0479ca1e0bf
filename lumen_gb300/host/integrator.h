// Host-side mirror of Lumen's integrator interface (src/RayTracer/Integrator.h:14-33, Path.h:4-20) over the
// C ABI, headless: the output is an RGBA32F device film instead of a Vulkan texture.
#pragma once
#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>

#include "lgb.h"
#include "lumen_scene.h"

namespace lgbh {

// A failed lgb_* call inside an integrator, with its status.
struct LgbCallError : std::runtime_error {
    LgbCallError(lgb_status s, const std::string& msg) : std::runtime_error(msg), status(s) {}
    lgb_status status;
};

class Integrator {
  public:
    Integrator(LumenScene* scene, lgb_ctx* ctx, uint32_t width, uint32_t height)
        : lumen_scene(scene), ctx(ctx), width(width), height(height) {}
    virtual ~Integrator() { destroy(); }
    // Integrator::init (Integrator.cpp:8-50): uploads the scene, allocates the output film, sets the camera.
    virtual void init();
    virtual void render() = 0;
    // Integrator::update (Integrator.cpp:74-125) without input handling: refreshes the camera matrices.
    virtual bool update();
    virtual void destroy();
    // Integrator::create_accel (Integrator.cpp:137-160): one 8-wide BVH over every mesh.
    virtual void create_accel(const lgb_build_opts* opts = nullptr);

    float* output_film = nullptr;  // device RGBA32F, width * height
    bool updated = false;
    uint32_t frame_num = 0;
    lgb_build_stats accel_stats{};
    lgb_scene* gpu_scene() const { return scene; }
    const lgb_camera& camera() const { return cam; }

  protected:
    void check(lgb_status st, const char* what);
    LumenScene* lumen_scene = nullptr;
    lgb_ctx* ctx = nullptr;
    lgb_scene* scene = nullptr;
    lgb_camera cam{};
    uint32_t width = 0, height = 0;
};

// The Path integrator (Path.cpp): one sample per pixel per render(), progressive mean in the film.
class GpuPath final : public Integrator {
  public:
    using Integrator::Integrator;
    void init() override;
    void render() override;
    bool update() override;
    uint32_t path_length = 6;
    bool direct_lighting = true;
    void* stream = nullptr;
};

// The VCM integrator (VCM.cpp:131-275): one iteration per render(); the merge radius shrinks with the frame
// (VCM.cpp:137-138) and VC is always on (VCM.cpp:8). Lumen seeds each iteration with host rand(); here the
// seeds are the deterministic sequence vcm_seeds(seed, frame_num).
class GpuVCM final : public Integrator {
  public:
    using Integrator::Integrator;
    void init() override;
    void render() override;
    bool update() override;
    uint32_t path_length = 6;
    uint32_t seed = 0;
    void* stream = nullptr;
};

// The SPPM integrator (SPPM.cpp:78-192): one frame per render(); the per-pixel state restarts at frame 0, which
// update() returns to when the camera changed. Lumen draws each frame's RNG offset with host rand(); here it is
// the light seed of vcm_seeds(seed, frame_num).
class GpuSPPM final : public Integrator {
  public:
    using Integrator::Integrator;
    void init() override;
    void render() override;
    bool update() override;
    uint32_t path_length = 6;
    float base_radius = 0.03f;
    uint32_t seed = 0;
    void* stream = nullptr;
};

// The BDPT integrator (BDPT.cpp:55-99): one frame per render(); frame 0 again after a camera change. Lumen draws
// each frame's RNG offset with host rand(); here it is the light seed of vcm_seeds(seed, frame_num).
class GpuBDPT final : public Integrator {
  public:
    using Integrator::Integrator;
    void init() override;
    void render() override;
    bool update() override;
    uint32_t path_length = 6;
    uint32_t seed = 0;
    void* stream = nullptr;
};

// The ReSTIR DI integrator (ReSTIR.cpp:74-165): one frame per render(); spatiotemporal reuse is off for the
// first frame and on afterwards (ReSTIR.cpp:154-156); the previous camera feeds the temporal reprojection test.
class GpuReSTIR final : public Integrator {
  public:
    using Integrator::Integrator;
    void init() override;
    void render() override;
    bool update() override;
    bool do_spatiotemporal = false;
    bool enable_accumulation = true;
    uint32_t flags = 0;  // LGB_RESTIR_*
    uint32_t seed = 0;
    void* stream = nullptr;

  private:
    lgb_camera prev_cam_{};
};

// Light and eye seeds of VCM iteration `frame` (PCG-style integer hash of (seed, frame, stream)).
void vcm_seeds(uint32_t seed, uint32_t frame, uint32_t* light_seed, uint32_t* eye_seed);

}  // namespace lgbh
