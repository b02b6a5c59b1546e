// context.cu — context (device + stream + HBM budget), errors, policies and
// the camera helper.  The context plays the role of vk::Backend
// (src/engine/gfx/vk.cpp) for this path: one device, one ordered queue, a
// budgeted allocator.
#include "hx_internal.h"

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>

static thread_local char g_last_error[1024] = "";

void hx_set_error(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
    va_end(ap);
}

extern "C" const char* hx_last_error_string(void) { return g_last_error; }
extern "C" const char* hx_version(void) { return "helios-gb300 0.1 (sm_103a)"; }

hx_status hx_alloc(hx_context* ctx, void** ptr, size_t bytes) {
    *ptr = nullptr;
    if (bytes == 0) bytes = 16;
    {
        std::lock_guard<std::mutex> lk(ctx->mu);
        if (ctx->budget && ctx->used + bytes > ctx->budget) {
            hx_set_error("HBM budget exceeded: %llu + %llu > %llu bytes", (unsigned long long)ctx->used,
                         (unsigned long long)bytes, (unsigned long long)ctx->budget);
            return HX_ERR_OOM_BUDGET;
        }
        ctx->used += bytes;
    }
    cudaError_t e = cudaMalloc(ptr, bytes);
    if (e != cudaSuccess) {
        std::lock_guard<std::mutex> lk(ctx->mu);
        ctx->used -= bytes;
        *ptr = nullptr;
        hx_set_error("cudaMalloc(%zu): %s", bytes, cudaGetErrorString(e));
        return e == cudaErrorMemoryAllocation ? HX_ERR_OOM_BUDGET : HX_ERR_DEVICE;
    }
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->sizes[*ptr] = bytes;
    return HX_OK;
}

void hx_free(hx_context* ctx, void* ptr) {
    if (!ptr) return;
    cudaFree(ptr);
    std::lock_guard<std::mutex> lk(ctx->mu);
    auto it = ctx->sizes.find(ptr);
    if (it != ctx->sizes.end()) {
        ctx->used -= it->second;
        ctx->sizes.erase(it);
    }
}

extern "C" hx_status hx_context_create(int device, uint64_t budget, hx_context** out) {
    HX_CHECK_ARG(out, "hx_context_create: null out");
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) {
        hx_set_error("no CUDA device available (%s)", cudaGetErrorString(e));
        return HX_ERR_UNSUPPORTED;
    }
    HX_CHECK_ARG(device >= 0 && device < n, "hx_context_create: device %d of %d", device, n);
    HX_CUDA(cudaSetDevice(device));
    cudaDeviceProp prop;
    HX_CUDA(cudaGetDeviceProperties(&prop, device));
    if (prop.major < 10) {
        hx_set_error("device %d is sm_%d%d; this build targets sm_103a", device, prop.major, prop.minor);
        return HX_ERR_UNSUPPORTED;
    }
    hx_context* ctx = new hx_context();
    ctx->device = device;
    ctx->budget = budget;
    ctx->num_sms = prop.multiProcessorCount;
    // highest priority: the serving loop's denoiser and short requests share
    // the device with long ticks on low-priority streams
    int lo_prio = 0, hi_prio = 0;
    cudaDeviceGetStreamPriorityRange(&lo_prio, &hi_prio);
    e = cudaStreamCreateWithPriority(&ctx->stream, cudaStreamNonBlocking, hi_prio);
    if (e != cudaSuccess) {
        delete ctx;
        hx_set_error("cudaStreamCreate: %s", cudaGetErrorString(e));
        return HX_ERR_DEVICE;
    }
    *out = ctx;
    return HX_OK;
}

extern "C" hx_status hx_context_destroy(hx_context* ctx) {
    if (!ctx) return HX_OK;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    for (auto& kv : ctx->sizes) cudaFree(kv.first);
    cudaStreamDestroy(ctx->stream);
    delete ctx;
    return HX_OK;
}

extern "C" hx_status hx_context_synchronize(hx_context* ctx) {
    HX_CHECK_ARG(ctx, "null context");
    HX_CUDA(cudaStreamSynchronize(ctx->stream));
    return HX_OK;
}

extern "C" hx_status hx_context_memory(hx_context* ctx, uint64_t* used, uint64_t* budget) {
    HX_CHECK_ARG(ctx, "null context");
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (used) *used = ctx->used;
    if (budget) *budget = ctx->budget;
    return HX_OK;
}

// One pass = every 16-byte word of the buffer read once (ld.global.cg: L2,
// not L1); the XOR of the words is stored only if it equals a constant it
// practically never equals, which keeps the loads without writing.
__global__ void k_read_bandwidth(const uint4* __restrict__ buf, size_t n16, uint32_t passes, uint32_t* sink) {
    uint32_t acc = 0;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (uint32_t p = 0; p < passes; ++p)
        for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n16; i += stride) {
            const uint4 v = __ldcg(buf + i);
            acc ^= v.x ^ v.y ^ v.z ^ v.w;
        }
    if (acc == 0x9e3779b9u) sink[blockIdx.x] = acc;
}

extern "C" hx_status hx_measure_read_bandwidth(hx_context* ctx, uint64_t bytes, uint32_t passes, double* gbs) {
    HX_CHECK_ARG(ctx && gbs && passes > 0 && bytes >= (1u << 20) && bytes % 16 == 0,
                 "hx_measure_read_bandwidth: bad argument");
    HX_CUDA(cudaSetDevice(ctx->device));
    const int blocks = 8 * ctx->num_sms, threads = 256;
    DevBuffer buf, sink;
    HX_TRY(buf.reserve(ctx, bytes));
    HX_TRY(sink.reserve(ctx, 4 * (size_t)blocks));
    cudaStream_t st = ctx->stream;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    hx_status rs = HX_OK;
    float ms = 0.0f;
    if (cudaMemsetAsync(buf.ptr, 0x5a, bytes, st) != cudaSuccess || cudaEventCreate(&e0) != cudaSuccess ||
        cudaEventCreate(&e1) != cudaSuccess) {
        rs = HX_ERR_DEVICE;
    } else {
        k_read_bandwidth<<<blocks, threads, 0, st>>>(buf.as<uint4>(), bytes / 16, 1, sink.as<uint32_t>());  // warm-up
        cudaEventRecord(e0, st);
        k_read_bandwidth<<<blocks, threads, 0, st>>>(buf.as<uint4>(), bytes / 16, passes, sink.as<uint32_t>());
        cudaEventRecord(e1, st);
        if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess || ms <= 0.0f)
            rs = HX_ERR_DEVICE;
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    buf.release();
    sink.release();
    if (rs != HX_OK) {
        hx_set_error("hx_measure_read_bandwidth: CUDA error %s", cudaGetErrorString(cudaGetLastError()));
        return rs;
    }
    *gbs = (double)bytes * passes / (ms * 1e-3) / 1e9;
    return HX_OK;
}

struct hx_event {
    hx_context* ctx;
    cudaEvent_t ev;
};

extern "C" hx_status hx_event_create(hx_context* ctx, hx_event** out) {
    HX_CHECK_ARG(ctx && out, "hx_event_create: null argument");
    HX_CUDA(cudaSetDevice(ctx->device));
    cudaEvent_t e;
    HX_CUDA(cudaEventCreate(&e));
    *out = new hx_event{ctx, e};
    return HX_OK;
}

extern "C" hx_status hx_event_record(hx_event* ev) {
    HX_CHECK_ARG(ev, "hx_event_record: null event");
    HX_CUDA(cudaEventRecord(ev->ev, ev->ctx->stream));
    return HX_OK;
}

extern "C" hx_status hx_event_elapsed(hx_event* a, hx_event* b, float* ms) {
    HX_CHECK_ARG(a && b && ms, "hx_event_elapsed: null argument");
    HX_CUDA(cudaEventSynchronize(b->ev));
    HX_CUDA(cudaEventElapsedTime(ms, a->ev, b->ev));
    return HX_OK;
}

extern "C" hx_status hx_event_destroy(hx_event* ev) {
    if (!ev) return HX_OK;
    cudaEventDestroy(ev->ev);
    delete ev;
    return HX_OK;
}

extern "C" hx_status hx_pinned_alloc(size_t bytes, void** out) {
    HX_CHECK_ARG(out && bytes > 0, "hx_pinned_alloc: bad argument");
    HX_CUDA(cudaMallocHost(out, bytes));
    return HX_OK;
}

extern "C" hx_status hx_pinned_free(void* ptr) {
    if (ptr) HX_CUDA(cudaFreeHost(ptr));
    return HX_OK;
}

extern "C" hx_status hx_device_alloc(hx_context* ctx, uint64_t bytes, void** out) {
    HX_CHECK_ARG(ctx && out && bytes > 0, "hx_device_alloc: bad argument");
    HX_CUDA(cudaSetDevice(ctx->device));
    return hx_alloc(ctx, out, bytes);
}

extern "C" hx_status hx_device_free(hx_context* ctx, void* ptr) {
    HX_CHECK_ARG(ctx, "hx_device_free: null context");
    if (ptr) {
        HX_CUDA(cudaStreamSynchronize(ctx->stream));
        hx_free(ctx, ptr);
    }
    return HX_OK;
}

extern "C" hx_status hx_device_copy(hx_context* ctx, void* dst, const void* src, uint64_t bytes, uint32_t kind) {
    HX_CHECK_ARG(ctx && dst && src && kind <= HX_COPY_DEVICE_TO_DEVICE, "hx_device_copy: bad argument");
    if (bytes == 0) return HX_OK;
    const cudaMemcpyKind k = kind == HX_COPY_HOST_TO_DEVICE   ? cudaMemcpyHostToDevice
                             : kind == HX_COPY_DEVICE_TO_HOST ? cudaMemcpyDeviceToHost
                                                              : cudaMemcpyDeviceToDevice;
    HX_CUDA(cudaSetDevice(ctx->device));
    HX_CUDA(cudaMemcpyAsync(dst, src, bytes, k, ctx->stream));
    if (kind != HX_COPY_DEVICE_TO_DEVICE) HX_CUDA(cudaStreamSynchronize(ctx->stream));
    return HX_OK;
}

extern "C" void hx_policy_reference(hx_policy* p) {
    std::memset(p, 0, sizeof(*p));
    p->rng = HX_RNG_XOROSHIRO64STAR;
    p->rr_start_depth = 0;
    p->rr_clamp = 0;
    p->radiance_clamp = 1.0f;
    p->accumulation = HX_ACCUM_RUNNING_MEAN;
    p->area_count_from_x = 0;
    p->area_w_one = 0;
    p->env_sampling = HX_ENV_SAMPLE_COSINE;
    p->payload = HX_PAYLOAD_FP32;
}

extern "C" void hx_policy_spec(hx_policy* p) {
    hx_policy_reference(p);
    p->rng = HX_RNG_PCG;
    p->rr_start_depth = 3;
    p->rr_clamp = 1;
    p->area_count_from_x = 1;
    p->area_w_one = 1;
    p->env_sampling = HX_ENV_SAMPLE_IMPORTANCE;
}

// glm::lookAt / glm::perspective (right-handed, depth -1..1) in double,
// inverse(projection * view) rounded to float once.
static void mat_mul(const double* a, const double* b, double* o) {  // column-major o = a * b
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) {
            double s = 0;
            for (int k = 0; k < 4; ++k) s += a[k * 4 + r] * b[c * 4 + k];
            o[c * 4 + r] = s;
        }
}

static bool mat_inverse(const double* m, double* inv) {
    double a[4][8];
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) {
            a[r][c] = m[c * 4 + r];
            a[r][c + 4] = r == c ? 1.0 : 0.0;
        }
    for (int c = 0; c < 4; ++c) {
        int piv = c;
        for (int r = c + 1; r < 4; ++r)
            if (std::fabs(a[r][c]) > std::fabs(a[piv][c])) piv = r;
        if (a[piv][c] == 0.0) return false;
        if (piv != c)
            for (int k = 0; k < 8; ++k) std::swap(a[c][k], a[piv][k]);
        double d = a[c][c];
        for (int k = 0; k < 8; ++k) a[c][k] /= d;
        for (int r = 0; r < 4; ++r) {
            if (r == c) continue;
            double f = a[r][c];
            for (int k = 0; k < 8; ++k) a[r][k] -= f * a[c][k];
        }
    }
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) inv[c * 4 + r] = a[r][c + 4];
    return true;
}

extern "C" hx_status hx_camera_to_frame_desc(const hx_camera* cam, uint32_t width, uint32_t height, hx_frame_desc* out) {
    HX_CHECK_ARG(cam && out && width > 0 && height > 0, "hx_camera_to_frame_desc: bad argument");
    double eye[3] = {cam->position[0], cam->position[1], cam->position[2]};
    double ctr[3] = {cam->target[0], cam->target[1], cam->target[2]};
    double upv[3] = {cam->up[0], cam->up[1], cam->up[2]};
    auto norm = [](double* v) {
        double l = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        for (int k = 0; k < 3; ++k) v[k] /= l;
    };
    auto crs = [](const double* a, const double* b, double* o) {
        o[0] = a[1] * b[2] - a[2] * b[1];
        o[1] = a[2] * b[0] - a[0] * b[2];
        o[2] = a[0] * b[1] - a[1] * b[0];
    };
    double f[3] = {ctr[0] - eye[0], ctr[1] - eye[1], ctr[2] - eye[2]};
    norm(f);
    double s[3], u[3];
    crs(f, upv, s);
    norm(s);
    crs(s, f, u);
    double view[16] = {s[0], u[0], -f[0], 0, s[1], u[1], -f[1], 0, s[2], u[2], -f[2], 0,
                       -(s[0] * eye[0] + s[1] * eye[1] + s[2] * eye[2]), -(u[0] * eye[0] + u[1] * eye[1] + u[2] * eye[2]),
                       (f[0] * eye[0] + f[1] * eye[1] + f[2] * eye[2]), 1};
    double fovy = (double)cam->fov_y_degrees * 3.14159265358979323846 / 180.0;
    double aspect = (double)width / (double)height;
    double th = std::tan(fovy / 2.0);
    double n = cam->near_plane, fa = cam->far_plane;
    HX_CHECK_ARG(fa > n && n > 0 && th > 0, "hx_camera_to_frame_desc: bad projection");
    double proj[16] = {0};
    proj[0] = 1.0 / (aspect * th);
    proj[5] = 1.0 / th;
    proj[10] = -(fa + n) / (fa - n);
    proj[11] = -1.0;
    proj[14] = -(2.0 * fa * n) / (fa - n);
    double vp[16], inv[16];
    mat_mul(proj, view, vp);
    HX_CHECK_ARG(mat_inverse(vp, inv), "hx_camera_to_frame_desc: singular view-projection");
    std::memset(out, 0, sizeof(*out));
    for (int k = 0; k < 16; ++k) out->view_proj_inverse[k] = (float)inv[k];
    for (int k = 0; k < 3; ++k) {
        out->camera_pos[k] = cam->position[k];
        out->up_direction[k] = (float)u[k];
        out->right_direction[k] = (float)s[k];  // CameraNode::left() = orientation * +X (scene.cpp:220-223)
    }
    // focal plane (path_integrator.cpp:136-142): normal -forward through camera_pos + forward * focal_length
    float fw[3] = {(float)f[0], (float)f[1], (float)f[2]};
    float P[3];
    for (int k = 0; k < 3; ++k) P[k] = cam->position[k] + fw[k] * cam->focal_length;
    out->focal_plane[0] = -fw[0];
    out->focal_plane[1] = -fw[1];
    out->focal_plane[2] = -fw[2];
    out->focal_plane[3] = -(out->focal_plane[0] * P[0] + out->focal_plane[1] * P[1] + out->focal_plane[2] * P[2]);
    out->focal_length = cam->focal_length;
    out->aperture_radius = cam->aperture_radius;
    return HX_OK;
}
