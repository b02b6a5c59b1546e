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

#include <algorithm>
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
    // Bake checkpoint / resume (progressive state to host memory and back).
    std::vector<uint8_t> save_checkpoint() {
        size_t n = 0;
        hx_check(hx_integrator_checkpoint_size(m_it, &n));
        std::vector<uint8_t> buf(n);
        hx_check(hx_integrator_save_checkpoint(m_it, buf.data(), buf.size()));
        return buf;
    }
    void load_checkpoint(const std::vector<uint8_t>& buf) {
        hx_check(hx_integrator_load_checkpoint(m_it, buf.data(), buf.size()));
    }
    void set_max_ray_bounces(const uint32_t& n) { hx_check(hx_integrator_set_max_ray_bounces(m_it, n)); }
    void set_max_samples(const uint32_t& n) { hx_check(hx_integrator_set_max_samples(m_it, n)); }
    void set_shadow_ray_bias(const float& b) { hx_check(hx_integrator_set_shadow_ray_bias(m_it, b)); }
    void set_tiled(bool tiled) { hx_check(hx_integrator_set_tiled(m_it, tiled ? 1u : 0u)); }
    void render(const hx_frame_desc& frame) { hx_check(hx_integrator_render(m_it, &frame)); }
    // Segments of num_debug_rays paths through a display pixel
    // (path_integrator.h:35), two vertices per segment.
    std::vector<hx_debug_ray_vertex> gather_debug_rays(const hx_frame_desc& frame, uint32_t pixel_x, uint32_t pixel_y,
                                                       uint32_t num_debug_rays, uint32_t max_ray_bounces) {
        std::vector<hx_debug_ray_vertex> v((size_t)2 * num_debug_rays * (max_ray_bounces ? max_ray_bounces : 1));
        uint32_t n = 0;
        hx_check(hx_integrator_gather_debug_rays(m_it, &frame, pixel_x, pixel_y, num_debug_rays, v.data(),
                                                 (uint32_t)v.size(), &n));
        v.resize(std::min<size_t>(n, v.size()));
        return v;
    }
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
// renderer.h:27-35
enum OutputBuffer {
    OUTPUT_BUFFER_ALBEDO = HX_OUTPUT_ALBEDO,
    OUTPUT_BUFFER_NORMALS = HX_OUTPUT_NORMALS,
    OUTPUT_BUFFER_ROUGHNESS = HX_OUTPUT_ROUGHNESS,
    OUTPUT_BUFFER_METALLIC = HX_OUTPUT_METALLIC,
    OUTPUT_BUFFER_EMISSIVE = HX_OUTPUT_EMISSIVE,
    OUTPUT_BUFFER_FINAL = HX_OUTPUT_FINAL
};

// The render / tone-map / save part of helios::Renderer (renderer.h:83-97).
class Renderer {
public:
    explicit Renderer(PathIntegrator::Ptr integrator) : m_integrator(std::move(integrator)) {}
    void set_tone_map_operator(ToneMapOperator op) { m_op = op; }
    void set_exposure(float e) { m_exposure = e; }
    void set_current_output_buffer(OutputBuffer b) { m_output = b; }
    OutputBuffer current_output_buffer() const { return m_output; }
    // The current output buffer as RGBA32F in display order: a debug view, or
    // for OUTPUT_BUFFER_FINAL the accumulated radiance (renderer.cpp:329-333).
    std::vector<float> read_output(const hx_frame_desc& frame, uint32_t width, uint32_t height) {
        std::vector<float> px((size_t)width * height * 4);
        hx_check(hx_integrator_render_output(m_integrator->handle(), &frame, (uint32_t)m_output, px.data()));
        return px;
    }
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
    // The tone-mapped frame as an RGBA PNG (renderer.cpp:637-713).
    void save_image_to_disk(const std::string& path, uint32_t width, uint32_t height) {
        std::vector<uint8_t> px = read_ldr(width, height);
        hx_check(hx_save_png(path.c_str(), px.data(), width, height));
    }

private:
    PathIntegrator::Ptr m_integrator;
    ToneMapOperator m_op = TONE_MAP_OPERATOR_ACES;
    OutputBuffer m_output = OUTPUT_BUFFER_FINAL;
    float m_exposure = 1.0f;
};

// The learned denoiser (no reference counterpart): parameters in, denoised
// tone-mapped frames out of a PathIntegrator's accumulation.
class Denoiser {
public:
    using Ptr = std::shared_ptr<Denoiser>;
    explicit Denoiser(Context::Ptr ctx) : m_ctx(std::move(ctx)) { hx_check(hx_denoiser_create(m_ctx->handle(), &m_dn)); }
    ~Denoiser() { hx_denoiser_destroy(m_dn); }
    Denoiser(const Denoiser&) = delete;
    Denoiser& operator=(const Denoiser&) = delete;
    uint64_t num_params() const {
        uint64_t n = 0;
        hx_check(hx_denoiser_num_params(m_dn, &n));
        return n;
    }
    void set_params(const std::vector<float>& p) { hx_check(hx_denoiser_set_params(m_dn, p.data(), p.size())); }
    std::vector<float> params() const {
        std::vector<float> p(num_params());
        hx_check(hx_denoiser_get_params(m_dn, p.data(), p.size()));
        return p;
    }
    // Denoised, tone-mapped RGBA8 of the integrator's current accumulation.
    std::vector<uint8_t> denoise(PathIntegrator& it, const hx_frame_desc& frame, uint32_t width, uint32_t height,
                                 ToneMapOperator op = TONE_MAP_OPERATOR_ACES, float exposure = 1.0f) {
        std::vector<uint8_t> px((size_t)width * height * 4);
        hx_check(hx_integrator_denoise(it.handle(), m_dn, &frame, (uint32_t)op, exposure, px.data(), nullptr));
        return px;
    }
    hx_denoiser* handle() const { return m_dn; }

private:
    Context::Ptr m_ctx;
    hx_denoiser* m_dn = nullptr;
};

// Resident render-serving loop over several GpuScenes.
class Server {
public:
    Server(Context::Ptr ctx, const hx_server_desc& desc) : m_ctx(std::move(ctx)) {
        hx_check(hx_server_create(m_ctx->handle(), &desc, &m_srv));
    }
    ~Server() { hx_server_destroy(m_srv); }
    Server(const Server&) = delete;
    Server& operator=(const Server&) = delete;
    uint32_t add_scene(const GpuScene::Ptr& scene) {
        uint32_t id = 0;
        hx_check(hx_server_add_scene(m_srv, scene->handle(), &id));
        m_scenes.push_back(scene);
        return id;
    }
    void set_denoiser(const Denoiser::Ptr& dn) {
        hx_check(hx_server_set_denoiser(m_srv, dn->handle()));
        m_dn = dn;
    }
    void start() { hx_check(hx_server_start(m_srv)); }
    uint64_t submit(const hx_request_desc& r) {
        uint64_t id = 0;
        hx_check(hx_server_submit(m_srv, &r, &id));
        return id;
    }
    std::vector<hx_request_result> poll(double wait_seconds, uint32_t capacity = 64) {
        std::vector<hx_request_result> out(capacity);
        uint32_t n = 0;
        hx_check(hx_server_poll(m_srv, out.data(), capacity, &n, wait_seconds));
        out.resize(n);
        return out;
    }
    std::vector<uint8_t> fetch(uint64_t id, uint32_t width, uint32_t height) {
        std::vector<uint8_t> px((size_t)width * height * 4);
        hx_check(hx_server_fetch(m_srv, id, px.data()));
        return px;
    }

private:
    Context::Ptr m_ctx;
    hx_server* m_srv = nullptr;
    std::vector<GpuScene::Ptr> m_scenes;
    Denoiser::Ptr m_dn;
};

}  // namespace helios
