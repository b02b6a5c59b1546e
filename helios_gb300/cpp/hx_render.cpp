// hx_render — headless C++ driver over the hx C-ABI (the role of the
// reference's viewer loop, src/viewer/main.cpp:66-76, without a window):
// uploads a procedural scene, renders N progressive frames through
// helios::PathIntegrator / helios::Renderer and writes the tone-mapped image;
// with a parameter file of the learned denoiser (raw FP32, hx.h layout) it
// also writes the denoised image next to it (<out>.denoised.png).
//
//   hx_render <box|icospheres> <width> <height> <frames> <out.png> [denoiser.f32]
#include "helios_gb300.hpp"

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>

int main(int argc, char** argv) {
    if (argc < 6) {
        std::fprintf(stderr, "usage: %s <box|icospheres> <width> <height> <frames> <out.png> [denoiser.f32]\n", argv[0]);
        return 2;
    }
    const bool box = std::strcmp(argv[1], "box") == 0;
    const uint32_t w = (uint32_t)std::atoi(argv[2]), h = (uint32_t)std::atoi(argv[3]), frames = (uint32_t)std::atoi(argv[4]);
    try {
        hx_procedural_params pp;
        hx_procedural_defaults(box ? HX_SCENE_BOX : HX_SCENE_ICOSPHERES, &pp);
        hx_host_scene* hs = nullptr;
        helios::hx_check(hx_procedural_scene_create(&pp, &hs));
        auto ctx = std::make_shared<helios::Context>(0);
        auto scene = std::make_shared<helios::GpuScene>(ctx, *hx_host_scene_desc(hs));
        hx_policy pol;
        if (box) hx_policy_spec(&pol);
        else {
            hx_policy_reference(&pol);
            pol.env_sampling = HX_ENV_SAMPLE_IMPORTANCE;
        }
        auto integrator = std::make_shared<helios::PathIntegrator>(ctx, scene, w, h, &pol);
        integrator->set_max_ray_bounces(box ? 5 : 8);
        helios::Renderer renderer(integrator);
        hx_camera cam;
        helios::hx_check(hx_host_scene_camera(hs, &cam));
        hx_frame_desc frame;
        helios::hx_check(hx_camera_to_frame_desc(&cam, w, h, &frame));
        auto t0 = std::chrono::steady_clock::now();
        for (uint32_t f = 0; f < frames; ++f) renderer.render(frame);
        ctx->synchronize();
        double s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        renderer.save_image_to_disk(argv[5], w, h);
        std::printf("rendered %u frames of %ux%u (%u samples accumulated) in %.3f s: %.1f Mpaths/s\n", frames, w, h,
                    integrator->num_accumulated_samples(), s, (double)frames * w * h / s / 1e6);
        if (argc > 6) {
            helios::Denoiser dn(ctx);
            std::vector<float> params(dn.num_params());
            FILE* f = std::fopen(argv[6], "rb");
            if (!f || std::fread(params.data(), 4, params.size(), f) != params.size())
                throw std::runtime_error(std::string("cannot read ") + std::to_string(params.size()) +
                                         " parameters from " + argv[6]);
            std::fclose(f);
            dn.set_params(params);
            std::vector<uint8_t> px = dn.denoise(*integrator, frame, w, h);
            std::string out = std::string(argv[5]) + ".denoised.png";
            helios::hx_check(hx_save_png(out.c_str(), px.data(), w, h));
            std::printf("denoised image: %s\n", out.c_str());
        }
        hx_host_scene_destroy(hs);
    } catch (const std::exception& e) {
        std::fprintf(stderr, "hx_render: %s\n", e.what());
        return 1;
    }
    return 0;
}
