// helios_gb300.hpp — header-only C++ surface over the hx C-ABI, shaped like
// the engine classes it replaces so a renderer can swap its integrator:
//   helios::PathIntegrator  <- include/gfx/path_integrator.h:9-62
//   helios::Renderer        <- include/gfx/renderer.h:37-122 (render / tone map /
//                              exposure / save image surface)
//   helios::GpuScene        <- the GPU buffers of Scene::create_gpu_resources
//                              (src/engine/resource/scene.cpp:915-1311)
// Errors become std::runtime_error on this side of the ABI (the reference
// threw on Vulkan errors, src/engine/gfx/vk.cpp:2306-2310); the ABI itself
// never throws.
#pragma once

#include "hx.h"

#include <cstdint>
#include <cstdio>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace helios {

inline void hx_check(hx_status s) {
    if (s != HX_OK) throw std::runtime_error(std::string("hx: ") + hx_last_error_string());
}

class Context {
public:
    using Ptr = std::shared_ptr<Context>;
    explicit Context(int device = 0, uint64_t hbm_budget_bytes = 0) { hx_check(hx_context_create(device, hbm_budget_bytes, &m_ctx)); }
    ~Context() { hx_context_destroy(m_ctx); }
    Context(const Context&) = delete;
    Context& operator=(const Context&) = delete;
    hx_context* handle() const { return m_ctx; }
    void synchronize() { hx_check(hx_context_synchronize(m_ctx)); }

private:
    hx_context* m_ctx = nullptr;
};

class GpuScene {
public:
    using Ptr = std::shared_ptr<GpuScene>;
    GpuScene(Context::Ptr ctx, const hx_scene_desc& desc) : m_ctx(std::move(ctx)) {
        hx_check(hx_scene_upload(m_ctx->handle(), &desc, &m_scene));
    }
    ~GpuScene() { hx_scene_destroy(m_scene); }
    GpuScene(const GpuScene&) = delete;
    GpuScene& operator=(const GpuScene&) = delete;
    const hx_scene* handle() const { return m_scene; }
    hx_scene_info info() const {
        hx_scene_info i;
        hx_check(hx_scene_info_get(m_scene, &i));
        return i;
    }
    uint32_t num_lights() const { return info().num_lights; }

private:
    Context::Ptr m_ctx;
    hx_scene* m_scene = nullptr;
};

// Same members and defaults as the reference PathIntegrator
// (path_integrator.h:18-51); render() takes the per-frame constants the
// reference pulled from RenderState (camera matrices, focal plane, aperture).
class PathIntegrator {
public:
    using Ptr = std::shared_ptr<PathIntegrator>;
    PathIntegrator(Context::Ptr ctx, GpuScene::Ptr scene, uint32_t width, uint32_t height, const hx_policy* policy = nullptr)
        : m_ctx(std::move(ctx)), m_scene(std::move(scene)) {
        hx_integrator_desc d{};
        d.width = width;
        d.height = height;
        d.max_ray_bounces = 7;
        d.max_samples = 5000;
        d.shadow_ray_bias = 0.0f;
        d.tiled = 0;
        if (policy) d.policy = *policy;
        else hx_policy_reference(&d.policy);
        hx_check(hx_integrator_create(m_ctx->handle(), m_scene->handle(), &d, &m_it));
    }
    ~PathIntegrator() { hx_integrator_destroy(m_it); }
    PathIntegrator(const PathIntegrator&) = delete;
    PathIntegrator& operator=(const PathIntegrator&) = delete;

    uint32_t num_accumulated_samples() const { return progress(0); }
    uint32_t tile_idx() const { return progress(1); }
    uint32_t num_target_samples() const { return progress(2); }
    void restart_bake() { hx_check(hx_integrator_restart_bake(m_it)); }
    void set_max_ray_bounces(const uint32_t& n) { hx_check(hx_integrator_set_max_ray_bounces(m_it, n)); }
    void set_max_samples(const uint32_t& n) { hx_check(hx_integrator_set_max_samples(m_it, n)); }
    void set_shadow_ray_bias(const float& b) { hx_check(hx_integrator_set_shadow_ray_bias(m_it, b)); }
    void set_tiled(bool tiled) { hx_check(hx_integrator_set_tiled(m_it, tiled ? 1u : 0u)); }
    void render(const hx_frame_desc& frame) { hx_check(hx_integrator_render(m_it, &frame)); }
    void render(const hx_camera& camera, uint32_t width, uint32_t height) {
        hx_frame_desc f;
        hx_check(hx_camera_to_frame_desc(&camera, width, height, &f));
        render(f);
    }
    hx_integrator* handle() const { return m_it; }

private:
    uint32_t progress(int which) const {
        uint32_t v[3];
        hx_check(hx_integrator_progress(m_it, &v[0], &v[1], &v[2]));
        return v[which];
    }
    Context::Ptr m_ctx;
    GpuScene::Ptr m_scene;
    hx_integrator* m_it = nullptr;
};

enum ToneMapOperator { TONE_MAP_OPERATOR_ACES = HX_TONEMAP_ACES, TONE_MAP_OPERATOR_REINHARD = HX_TONEMAP_REINHARD };

// The render / tone-map / save part of helios::Renderer (renderer.h:83-97).
class Renderer {
public:
    explicit Renderer(PathIntegrator::Ptr integrator) : m_integrator(std::move(integrator)) {}
    void set_tone_map_operator(ToneMapOperator op) { m_op = op; }
    void set_exposure(float e) { m_exposure = e; }
    void render(const hx_frame_desc& frame) {
        m_integrator->render(frame);
        hx_check(hx_integrator_tonemap(m_integrator->handle(), (uint32_t)m_op, m_exposure, nullptr));
    }
    // Tone-mapped RGBA8 (vertically flipped like the negative-height viewport).
    std::vector<uint8_t> read_ldr(uint32_t width, uint32_t height) {
        std::vector<uint8_t> px((size_t)width * height * 4);
        hx_check(hx_integrator_tonemap(m_integrator->handle(), (uint32_t)m_op, m_exposure, px.data()));
        return px;
    }
    // Binary PPM instead of stb's PNG (no image-library dependency).
    void save_image_to_disk(const std::string& path, uint32_t width, uint32_t height) {
        std::vector<uint8_t> px = read_ldr(width, height);
        FILE* f = std::fopen(path.c_str(), "wb");
        if (!f) throw std::runtime_error("cannot open " + path);
        std::fprintf(f, "P6\n%u %u\n255\n", width, height);
        for (size_t i = 0; i < (size_t)width * height; ++i) std::fwrite(&px[4 * i], 1, 3, f);
        std::fclose(f);
    }

private:
    PathIntegrator::Ptr m_integrator;
    ToneMapOperator m_op = TONE_MAP_OPERATOR_ACES;
    float m_exposure = 1.0f;
};

}  // namespace helios
