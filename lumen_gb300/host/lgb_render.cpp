// Headless Lumen-style renderer: lgb_render <scene.json> <width> <height> <spp> <out.pfm> [device]
// The window, GUI and swapchain of src/main.cpp / RayTracer.cpp are replaced by a PFM written at the end.
#include <cstdio>
#include <cstdlib>

#include "lgb_host.h"

int main(int argc, char** argv) {
    if (argc < 6) {
        std::fprintf(stderr, "usage: %s <scene.json> <width> <height> <spp> <out.pfm> [device]\n", argv[0]);
        return 2;
    }
    char err[512] = {0};
    const lgb_status st = lgbh_render_path(argv[1], argc > 6 ? std::atoi(argv[6]) : 0, (uint32_t)std::atoi(argv[2]),
                                           (uint32_t)std::atoi(argv[3]), (uint32_t)std::atoi(argv[4]), argv[5], nullptr,
                                           err, sizeof(err));
    if (st != LGB_OK) {
        std::fprintf(stderr, "lgb_render: error %d: %s\n", st, err);
        return 1;
    }
    std::printf("wrote %s\n", argv[5]);
    return 0;
}
