/*
 * hx.h — C-ABI of the helios-gb300 path-tracing core (sm_103a).
 *
 * This is the drop-in boundary that replaces the Vulkan ray-tracing path of
 * helios (diharaw/helios): the ray-gen / closest-hit / any-hit / miss / shadow
 * shaders, the progressive accumulation and the tone-map pass.  The engine's
 * C++ surface (helios::PathIntegrator, helios::Renderer, the packed scene
 * buffers of helios::Scene) maps one-to-one onto the calls below; each
 * declaration names the reference interface it replaces (path within the
 * reference project, file:line).
 *
 * Rules of the ABI:
 *   - plain C types, plain pointers and sizes; no C++ or framework types;
 *   - every call returns hx_status; hx_last_error_string() gives the reason
 *     of the last failure on the calling thread (no exceptions cross the ABI;
 *     the reference logged and threw std::runtime_error, src/engine/gfx/vk.cpp:2306-2310);
 *   - caller-owned host arrays are copied during the call; device memory is
 *     owned by the library and charged to the context's HBM budget;
 *   - all work of a context is ordered on that context's CUDA stream; one
 *     context per host thread.
 *
 * Struct layouts marked "reference layout" keep the byte layout and field
 * meaning of the reference's GPU buffers (std430), so a maintainer can pass
 * the engine's packed arrays through unchanged.
 */
#ifndef HX_H
#define HX_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define HX_API __attribute__((visibility("default")))
#else
#define HX_API
#endif

/* ------------------------------------------------------------------------ */
/* Status codes                                                              */
/* ------------------------------------------------------------------------ */

typedef enum hx_status {
    HX_OK                = 0,
    HX_ERR_INVALID_ARG   = 1,  /* bad pointer, size or enum value            */
    HX_ERR_OOM_BUDGET    = 2,  /* allocation would exceed the HBM budget     */
    HX_ERR_TIMEOUT       = 3,  /* a bounded device wait gave up              */
    HX_ERR_DEVICE        = 4,  /* CUDA runtime error                         */
    HX_ERR_NOT_READY     = 5,  /* result not available yet                   */
    HX_ERR_UNSUPPORTED   = 6,  /* feature not built / not available          */
    HX_ERR_CANCELLED     = 7   /* request cancelled before completion        */
} hx_status;

typedef struct hx_context    hx_context;
typedef struct hx_scene      hx_scene;
typedef struct hx_integrator hx_integrator;
typedef struct hx_host_scene hx_host_scene;
typedef struct hx_denoiser   hx_denoiser;

/* ------------------------------------------------------------------------ */
/* Scene input — reference layouts                                           */
/* ------------------------------------------------------------------------ */

/* Vertex — reference layout include/resource/mesh.h:10-17 (5 x vec4 = 80 B).
 * position.w carries the submesh index as written by the resource loader
 * (src/engine/core/resource_manager.cpp:471-472). */
typedef struct hx_vertex {
    float position[4];
    float tex_coord[4];
    float normal[4];
    float tangent[4];
    float bitangent[4];
} hx_vertex;

/* Submesh flags. */
#define HX_SUBMESH_NON_OPAQUE 1u  /* alpha-tested or non-opaque material:
                                     the BLAS geometry lacks the OPAQUE bit
                                     (src/engine/resource/mesh.cpp:75-76), so
                                     any-hit alpha testing runs on it */

/* SubMesh — include/resource/mesh.h:20-29 (the fields the path uses). */
typedef struct hx_submesh {
    uint32_t base_index;   /* first index (multiple of 3)                    */
    uint32_t index_count;  /* number of indices (multiple of 3)              */
    uint32_t material;     /* index into hx_scene_desc.materials             */
    uint32_t flags;        /* HX_SUBMESH_*                                   */
} hx_submesh;

typedef struct hx_mesh_desc {
    const hx_vertex*  vertices;
    uint32_t          num_vertices;
    const uint32_t*   indices;       /* absolute vertex indices              */
    uint32_t          num_indices;
    const hx_submesh* submeshes;
    uint32_t          num_submeshes;
} hx_mesh_desc;

/* MaterialData — reference layout src/engine/resource/scene.cpp:25-32 and
 * common.glsl:80-87 (80 B).  texture_indices0 = (albedo, normal, roughness,
 * metallic), texture_indices1 = (emissive, -, roughness channel, metallic
 * channel); -1 = no texture.  albedo is linear (the host already applied the
 * sRGB->linear pow(2.2), scene.cpp:1017). */
typedef struct hx_material {
    int32_t texture_indices0[4];
    int32_t texture_indices1[4];
    float   albedo[4];
    float   emissive[4];
    float   roughness_metallic[4];
} hx_material;

/* Light types — src/engine/shader/common.glsl:12-16. */
#define HX_LIGHT_DIRECTIONAL 0
#define HX_LIGHT_SPOT        1
#define HX_LIGHT_POINT       2
#define HX_LIGHT_ENVIRONMENT 3
#define HX_LIGHT_AREA        4

/* LightData — reference layout src/engine/resource/scene.cpp:36-42,
 * common.glsl:89-95 (64 B).  Only DIRECTIONAL / POINT / SPOT entries are
 * passed in; the library derives the AREA and ENVIRONMENT entries and the
 * list order itself (scene.cpp:1111-1119,1269-1309). */
typedef struct hx_light {
    float data0[4];  /* x: type, yzw: colour | area: x type, y instance, z material, w primitive offset */
    float data1[4];  /* xyz: direction, w: intensity | area: x primitive count */
    float data2[4];  /* xyz: position, w: radius */
    float data3[4];  /* x: cos inner, y: cos outer */
} hx_light;

/* InstanceData — reference layout src/engine/resource/scene.cpp:46-52
 * (144 B).  Matrices are column-major (GLM).  material_override replaces
 * the submesh materials of this instance (-1 = none), the per-node
 * override of scene.cpp:1125-1127. */
typedef struct hx_instance {
    float    model_matrix[16];
    float    normal_matrix[16];
    uint32_t mesh_index;
    int32_t  material_override;
    float    padding[2];
} hx_instance;

/* RGBA8 texture, linear UNORM, sampled bilinearly with REPEAT addressing at
 * level 0 (textureLod(...,0) with the trilinear sampler, vk.cpp:3559-3580). */
/* srgb = 1: the texture's RGB is sRGB-encoded (the reference creates such
 * textures with *_SRGB formats, resource_manager.cpp:48-67), so samples
 * decode each texel's RGB with the sRGB transfer function before filtering;
 * alpha stays linear.  srgb = 0: UNORM.  Normal maps (texture_indices0[1])
 * use the vertex tangent and bitangent (path_trace_rchit.glsl:190-219).
 * format: HX_TEXTURE_RGBA8 (rgba8 = width * height * 4 bytes) or one of the
 * block-compressed formats of the reference's assets
 * (kCompressedFormats, resource_manager.cpp:14-30), then rgba8 points at
 * ceil(width / 4) * ceil(height / 4) blocks in row-major block order; they
 * are decoded to RGBA8 at upload (hx_texture_decode).  The half-float
 * formats (BC6H, the reference's VK_FORMAT_BC6H_SFLOAT_BLOCK, and
 * uncompressed RGBA16F, its R16G16B16A16_SFLOAT for FLOAT16 images) are kept
 * as RGBA16F texels on the device (hx_texture_decode_hdr) and sampled in
 * FP32; they take srgb = 0 (the reference has no sRGB variant of them).
 * HX_TEXTURE_RGBA8_SNORM is how the reference creates uncompressed 8-bit
 * images that are not sRGB (kNonSRGBFormats, resource_manager.cpp:32-36, 64:
 * R8G8B8A8_SNORM): each channel reads max(int8 / 127, -1), srgb = 0. */
#define HX_TEXTURE_RGBA8    0u
#define HX_TEXTURE_BC1_RGB  1u  /* 8-byte blocks, alpha 255                          */
#define HX_TEXTURE_BC1_RGBA 2u  /* 8-byte blocks, 1-bit alpha in the 3-colour mode   */
#define HX_TEXTURE_BC2      3u  /* 16-byte blocks: explicit 4-bit alpha + colour      */
#define HX_TEXTURE_BC3      4u  /* 16-byte blocks: interpolated alpha + colour        */
#define HX_TEXTURE_BC4      5u  /* 8-byte blocks: R (G = B = 0, A = 255)              */
#define HX_TEXTURE_BC5      6u  /* 16-byte blocks: R, G (B = 0, A = 255)              */
#define HX_TEXTURE_BC7      7u  /* 16-byte blocks: BPTC RGBA, 8 modes, 1-3 subsets     */
#define HX_TEXTURE_BC6H_SF16 8u /* 16-byte blocks: BPTC signed half-float RGB (A = 1)  */
#define HX_TEXTURE_BC6H_UF16 9u /* 16-byte blocks: BPTC unsigned half-float RGB (A = 1) */
#define HX_TEXTURE_RGBA16F 10u  /* width * height * 4 IEEE half floats (little-endian) */
#define HX_TEXTURE_RGBA8_SNORM 11u /* width * height * 4 signed bytes: max(c / 127, -1)  */
typedef struct hx_texture_desc {
    const uint8_t* rgba8;
    uint32_t       width;
    uint32_t       height;
    uint32_t       srgb;
    uint32_t       format;  /* HX_TEXTURE_* */
} hx_texture_desc;

/* Host-only: decodes a texture of an 8-bit HX_TEXTURE_* format to width *
 * height RGBA8 texels (rows top to bottom; RGBA8 and RGBA8_SNORM bytes are
 * returned as they are).  Colour endpoints expand from RGB565 by
 * bit replication; interpolated palette entries round to nearest:
 * (2a + b + 1) / 3 and (a + b + 1) / 2 for colour, ((8 - k) a + (k - 1) b + 3) / 7
 * and ((6 - k) a + (k - 1) b + 2) / 5 for BC4-style channels; BC2 alpha is
 * a4 * 17.  The 3-colour mode (c0 <= c1) exists in BC1 blocks only.  BC7
 * follows the BPTC specification exactly (its interpolation is integer:
 * ((64 - w) e0 + w e1 + 32) >> 6); a block with a reserved mode decodes to
 * zero.  Half-float formats are refused (hx_texture_decode_hdr). */
HX_API hx_status hx_texture_decode(const hx_texture_desc* texture, uint8_t* rgba8_out);

/* Host-only: decodes a half-float texture (HX_TEXTURE_BC6H_SF16 / _UF16 /
 * RGBA16F) to width * height RGBA16F texels (IEEE half bit patterns, rows top
 * to bottom).  BC6H follows the BPTC specification exactly: endpoints
 * unquantised to 16 bits, interpolated with the 6-bit weights in integers
 * (floor((64 - w) e0 + w e1 + 32) / 64), scaled to the half pattern (x 31/64
 * unsigned; signed: magnitude x 31/32 with the sign bit); alpha is 1.0; a
 * block with a reserved mode decodes to zero colour. */
HX_API hx_status hx_texture_decode_hdr(const hx_texture_desc* texture, uint16_t* rgba16f_out);

#define HX_ENV_NONE          0u  /* black environment                        */
#define HX_ENV_EQUIRECT      1u  /* caller-supplied RGBA32F lat-long map     */
#define HX_ENV_HOSEK_WILKIE  2u  /* sky baked on the device from the model   */

/* Environment.  The reference binds a 512^2 RGBA32F cubemap rendered by the
 * Hosek-Wilkie raster pass (src/engine/gfx/hosek_wilkie_sky_model.cpp:658-764)
 * or an IBL map.  Here the environment is a lat-long map (FP16 on the
 * device) with a marginal/conditional CDF for importance sampling. */
typedef struct hx_environment_desc {
    uint32_t     kind;            /* HX_ENV_*                                   */
    uint32_t     width, height;   /* lat-long resolution (e.g. 2048 x 1024)     */
    const float* rgba32f;         /* HX_ENV_EQUIRECT: width*height*4 floats      */
    float        sun_direction[4];/* HX_ENV_HOSEK_WILKIE: direction TO the sun  */
    float        coeffs[40];      /* HX_ENV_HOSEK_WILKIE: A..I,Z as 10 x vec4
                                     (the UBO of procedural_sky.frag:11-23)    */
} hx_environment_desc;

typedef struct hx_scene_desc {
    const hx_mesh_desc*    meshes;          uint32_t num_meshes;
    const hx_instance*     instances;       uint32_t num_instances;
    const hx_material*     materials;       uint32_t num_materials;
    const hx_texture_desc* textures;        uint32_t num_textures;
    const hx_light*        punctual_lights; uint32_t num_punctual_lights;
    hx_environment_desc    environment;
} hx_scene_desc;

/* ------------------------------------------------------------------------ */
/* Integrator policy — reference-faithful vs benchmark-spec behaviour        */
/* ------------------------------------------------------------------------ */

#define HX_RNG_XOROSHIRO64STAR 0u /* Wang-hash seeded xoroshiro64*, random.glsl:17-50 */
#define HX_RNG_PCG             1u /* PCG hash seeded per (pixel, sample)             */

#define HX_ACCUM_RUNNING_MEAN  0u /* prev + (c - prev)/num_frames, path_trace_rgen.glsl:221-247 */
#define HX_ACCUM_KAHAN         1u /* Kahan-compensated FP32 sum / n (precision form)            */

#define HX_ENV_SAMPLE_COSINE     0u /* cosine-lobe env NEE, path_trace_rchit.glsl:366-372 */
#define HX_ENV_SAMPLE_IMPORTANCE 1u /* lat-long CDF importance sampling                   */

#define HX_PAYLOAD_FP32 0u
#define HX_PAYLOAD_FP16 1u          /* 16-bit ray / hit payloads (precision form):
                                       direction = two snorm16 octahedral coords,
                                       barycentrics = FP16; traversal stays FP32 */
/* Origins of the rays a hit spawns (the next bounce's ray and the shadow ray). */
#define HX_RAY_OFFSET_REFERENCE 0u  /* the reference's: the interpolated hit position
                                       (+ shading normal * shadow_ray_bias for shadow
                                       rays), tmin 1e-4 (path_trace_rchit.glsl:293-295,
                                       518-520)                                      */
#define HX_RAY_OFFSET_SCALED 1u     /* that origin moved off the surface along the
                                       geometric normal, to the side the ray leaves
                                       on, by n_i * (2^-15 |p_i| + 2^-16) in each
                                       coordinate (a continuous form of Waechter and
                                       Binder's self-intersection offset, Ray Tracing
                                       Gems ch. 6, 2019); shadow-ray tmax shortened by
                                       the offset's L1 length.  The fixed tmin of 1e-4
                                       is below the FP32 rounding of hit positions far
                                       from the origin (ulp(2048) = 2.4e-4), so rays
                                       re-hit the surface they leave there; this
                                       removes that bias and keeps tmin as it is     */

typedef struct hx_policy {
    uint32_t rng;                 /* HX_RNG_*                                              */
    uint32_t rr_start_depth;      /* RR at hits with depth >= this (0 = every depth)        */
    uint32_t rr_clamp;            /* 1: RR probability clamped to <= 1                      */
    float    radiance_clamp;      /* per-sample clamp (1.0 = RADIANCE_CLAMP_COLOR); <=0 off */
    uint32_t accumulation;        /* HX_ACCUM_*                                            */
    uint32_t area_count_from_x;   /* 1: read the area-light triangle count from data1.x     */
    uint32_t area_w_one;          /* 1: transform area-light vertices with w = 1            */
    uint32_t env_sampling;        /* HX_ENV_SAMPLE_*                                       */
    uint32_t payload;             /* HX_PAYLOAD_*                                          */
    uint32_t visualize_nans;      /* 1: a sample whose radiance has a NaN stores (1, 0, 0)
                                     in its pixel (VISUALIZE_NANS, path_trace_rgen.glsl:
                                     225-244); running-mean accumulation only             */
    uint32_t ray_offset;          /* HX_RAY_OFFSET_*                                       */
    uint32_t reserved;
} hx_policy;

/* Reference-faithful policy (every reference quirk reproduced). */
HX_API void hx_policy_reference(hx_policy* out);
/* Benchmark-spec policy (PCG RNG, RR after depth 3 with p <= 1, area-light
 * count from .x, w = 1, importance-sampled environment). */
HX_API void hx_policy_spec(hx_policy* out);

/* ------------------------------------------------------------------------ */
/* Integrator (replaces helios::PathIntegrator, include/gfx/path_integrator.h:9-62) */
/* ------------------------------------------------------------------------ */

typedef struct hx_integrator_desc {
    uint32_t  width, height;       /* output extents (swap_chain_extents)          */
    uint32_t  max_ray_bounces;     /* default 7, path_integrator.h:47; 0..64 (0 shades
                                      the camera hit like 1: no indirect ray)     */
    uint32_t  max_samples;         /* default 5000, path_integrator.h:48            */
    float     shadow_ray_bias;     /* default 0, path_integrator.h:51               */
    uint32_t  tiled;               /* 128x128 tiles, path_integrator.cpp:7,312-336  */
    uint32_t  max_paths_in_flight; /* wavefront capacity in paths (0 = max(width*height,
                                      2^22)); k*width*height lets render_frames trace
                                      k frames per wavefront (same result)         */
    uint32_t  reserved;
    hx_policy policy;
} hx_integrator_desc;

/* Per-frame constants: the push-constant block of path_integrator.cpp:11-28
 * that launch_rays fills (path_integrator.cpp:136-161). */
typedef struct hx_frame_desc {
    float view_proj_inverse[16];  /* inverse(projection * view), column-major */
    float camera_pos[4];
    float up_direction[4];
    float right_direction[4];
    float focal_plane[4];
    float focal_length;
    float aperture_radius;
    float reserved[2];
} hx_frame_desc;

/* Camera description used to fill hx_frame_desc the way CameraNode::update
 * (src/engine/resource/scene.cpp:632-646) and launch_rays do: GLM
 * perspective (right-handed, depth -1..1) and lookAt. */
typedef struct hx_camera {
    float position[3];
    float target[3];
    float up[3];
    float fov_y_degrees;   /* default 60 (scene.h:258)            */
    float near_plane;      /* default 1 (scene.h:256)             */
    float far_plane;       /* default 1000 (scene.h:257)          */
    float focal_length;    /* default 8 (scene.h:259)             */
    float aperture_radius; /* default 0.1 (scene.h:260); 0 = pinhole */
} hx_camera;

HX_API hx_status hx_camera_to_frame_desc(const hx_camera* camera, uint32_t width,
                                         uint32_t height, hx_frame_desc* out);

#define HX_TONEMAP_ACES     0u  /* tone_map.frag:8-15 (Narkowicz fit) */
#define HX_TONEMAP_REINHARD 1u  /* tone_map.frag:17-20                */
#define HX_TONEMAP_NONE     2u  /* exposure + gamma only              */

/* Hit record of a closest-hit query: prim = index into the scene's flattened
 * triangle list (instance-major, submesh order), 0xFFFFFFFF on a miss. */
typedef struct hx_hit {
    float    t;
    uint32_t prim;
    float    u, v;   /* barycentric weights of vertex 1 and vertex 2 (b_HitAttribs) */
} hx_hit;

/* Compressed 8-wide BVH node (80 B).  Child boxes are stored as 8-bit
 * offsets on a per-node grid: lo = origin + q * 2^exponent (exact products,
 * one rounded add), quantised outward so every decoded child box contains
 * the exact one.  meta[i] holds the slot's hit-bit position in its low 5
 * bits: 0x10 = empty slot; 0x80 | (24 + i) = internal child (node
 * child_base + the number of internal slots below i); 0x20 | off = leaf
 * slot with one triangle at leaf-triangle index prim_base + off (off < 8). */
typedef struct hx_bvh8_node {
    float    origin[3];
    int8_t   exponent[3];
    uint8_t  internal_mask;
    uint32_t child_base;
    uint32_t prim_base;
    uint8_t  meta[8];
    uint8_t  qlo[3][8];
    uint8_t  qhi[3][8];
} hx_bvh8_node;

typedef struct hx_stats {
    uint64_t paths;            /* camera samples traced                      */
    uint64_t extension_rays;   /* closest-hit queries                        */
    uint64_t shadow_rays;      /* any-hit visibility queries                 */
    double   ms_total;         /* device time of the last render call        */
    double   ms_raygen, ms_trace, ms_shade, ms_shadow, ms_accumulate;  /* ms_trace covers the
                                  shadow rays too (one traversal launch per bounce); ms_shadow is 0 */
    uint32_t trace_launches;   /* traversal launches in the last call        */
    uint32_t kernel_launches;  /* all kernel launches in the last call       */
    uint64_t node_visits;      /* BVH8 nodes fetched by traversal (counting mode)             */
    uint64_t tri_tests;        /* triangles tested by traversal (counting mode)               */
    /* SIMD utilisation of the traversal launches (counting mode): warp-level
     * steps of the node phase and of the triangle phase (node_visits /
     * (32 * warp_node_steps) = lanes busy per node step), warp iterations of
     * the persistent loop and lane iterations that held a ray. */
    uint64_t warp_node_steps;
    uint64_t warp_tri_steps;
    uint64_t warp_loop_iters;
    uint64_t lane_loop_busy;
    uint64_t alpha_tests;      /* any-hit alpha tests (counting mode)                         */
} hx_stats;

/* Context: one CUDA device + stream + HBM budget (the role of vk::Backend). */
HX_API hx_status   hx_context_create(int device, uint64_t hbm_budget_bytes, hx_context** out);
HX_API hx_status   hx_context_destroy(hx_context* ctx);
HX_API hx_status   hx_context_synchronize(hx_context* ctx);
HX_API hx_status   hx_context_memory(hx_context* ctx, uint64_t* used_bytes, uint64_t* budget_bytes);
/* Read bandwidth of this GPU for a working set of `bytes` (a multiple of 16,
 * at least 1 MiB): one launch reads the buffer `passes` times with 16-byte
 * loads that bypass L1, timed with events on the context stream.  A working
 * set well under the L2 (129 MB) gives the L2 read bandwidth, one of
 * gigabytes the HBM read bandwidth: the denominators of the traversal's
 * cache-served and DRAM bytes.  The buffer is allocated and freed inside the
 * call (charged to the context's budget meanwhile). */
HX_API hx_status   hx_measure_read_bandwidth(hx_context* ctx, uint64_t bytes, uint32_t passes, double* gb_per_s);
HX_API const char* hx_last_error_string(void);
HX_API const char* hx_version(void);

/* Device timestamps on the context stream (the GPU half of the reference
 * profiler's timestamp queries, src/engine/utility/profiler.cpp:84-140). */
typedef struct hx_event hx_event;
HX_API hx_status hx_event_create(hx_context* ctx, hx_event** out);
HX_API hx_status hx_event_record(hx_event* ev);
/* Waits for `end` and returns the device time between the two records. */
HX_API hx_status hx_event_elapsed(hx_event* begin, hx_event* end, float* ms);
HX_API hx_status hx_event_destroy(hx_event* ev);

/* Page-locked host staging memory for fast host<->device copies. */
HX_API hx_status hx_pinned_alloc(size_t bytes, void** out);
HX_API hx_status hx_pinned_free(void* ptr);

/* Device buffers from the context's budgeted allocator, and copies ordered
 * on the context stream (host copies return when complete). */
#define HX_COPY_HOST_TO_DEVICE   0u
#define HX_COPY_DEVICE_TO_HOST   1u
#define HX_COPY_DEVICE_TO_DEVICE 2u
HX_API hx_status hx_device_alloc(hx_context* ctx, uint64_t bytes, void** out);
HX_API hx_status hx_device_free(hx_context* ctx, void* ptr);
HX_API hx_status hx_device_copy(hx_context* ctx, void* dst, const void* src, uint64_t bytes, uint32_t kind);

/* Scene upload (replaces Scene::create_gpu_resources, scene.cpp:915-1311, and
 * the BLAS/TLAS builds of mesh.cpp:61-117 and renderer.cpp:113-181): copies
 * the host arrays, flattens instances, builds the LBVH -> BVH8 on the device,
 * derives the light list, bakes the environment. */
HX_API hx_status hx_scene_upload(hx_context* ctx, const hx_scene_desc* desc, hx_scene** out);
HX_API hx_status hx_scene_destroy(hx_scene* scene);

typedef struct hx_scene_info {
    uint32_t num_triangles;    /* flattened triangles                       */
    uint32_t num_bvh8_nodes;
    uint32_t num_binary_nodes; /* internal nodes of the Karras tree (n-1)    */
    uint32_t num_lights;       /* light list length (render_state.num_lights) */
    uint64_t device_bytes;
    double   build_ms;         /* device time of the BVH build               */
    float    scene_min[3], scene_max[3];
} hx_scene_info;
HX_API hx_status hx_scene_info_get(const hx_scene* scene, hx_scene_info* out);

/* Diagnostic knob (no counterpart in the reference, whose traversal stack
 * lives in the driver): the number of traversal-stack entries a ray may use,
 * 1..32 (default 32).  A ray that needs more drops the extra entries and sets
 * the overflow bit of the device status word, which the next synchronising
 * call reports as HX_ERR_DEVICE.  Applies to launches issued after the call. */
HX_API hx_status hx_scene_set_traversal_stack_limit(hx_scene* scene, uint32_t entries);

/* Copies the light list the library derived (reference order, scene.cpp
 * 1111-1119,1269-1309) into out[0..capacity). */
HX_API hx_status hx_scene_lights(const hx_scene* scene, hx_light* out, uint32_t capacity,
                                 uint32_t* count);

/* Copies device BVH data for parity checks (any pointer may be NULL):
 * morton[n] (30-bit codes in input order), sorted_prims[n] (stable sort
 * order), binary nodes as (left,right) child pairs with leaf flag in bit 31
 * [2*(n-1)], BVH8 nodes (80 B each) [num_bvh8_nodes*80 bytes], BVH8 leaf
 * triangle order [n]. */
HX_API hx_status hx_scene_export_bvh(const hx_scene* scene, uint32_t* morton,
                                     uint32_t* sorted_prims, uint32_t* binary_children,
                                     void* bvh8_nodes, uint32_t* bvh8_prims);

/* PathIntegrator::PathIntegrator (path_integrator.cpp:32-38). */
HX_API hx_status hx_integrator_create(hx_context* ctx, const hx_scene* scene,
                                      const hx_integrator_desc* desc, hx_integrator** out);
HX_API hx_status hx_integrator_destroy(hx_integrator* integ);

/* PathIntegrator::render (path_integrator.cpp:48-84) + the accumulation of
 * Renderer::render (renderer.cpp:183-227): traces one progressive frame
 * (1 sample per pixel of the current tile) and accumulates it.
 * Device-side faults of a frame (traversal-stack overflow, a malformed tree,
 * a shading list that misses rays) set bits of a device status word; render
 * itself does not wait, and the next call that synchronises anyway
 * (tonemap to host memory, read_accumulation, primary_hits,
 * sample_radiance, render_output, gather_debug_rays) reads the word with its
 * own copy, returns HX_ERR_DEVICE and clears it. */
HX_API hx_status hx_integrator_render(hx_integrator* integ, const hx_frame_desc* frame);

/* n consecutive render() calls with the same frame constants, batched into
 * one wavefront.  Results are identical to n render() calls. */
HX_API hx_status hx_integrator_render_frames(hx_integrator* integ, const hx_frame_desc* frame,
                                             uint32_t num_frames);

/* PathIntegrator::restart_bake (path_integrator.h:25-29) + the image clear of
 * renderer.cpp:212-223. */
HX_API hx_status hx_integrator_restart_bake(hx_integrator* integ);
HX_API hx_status hx_integrator_set_max_ray_bounces(hx_integrator* integ, uint32_t n);
HX_API hx_status hx_integrator_set_max_samples(hx_integrator* integ, uint32_t n);
HX_API hx_status hx_integrator_set_shadow_ray_bias(hx_integrator* integ, float bias);
HX_API hx_status hx_integrator_set_tiled(hx_integrator* integ, uint32_t tiled);
HX_API hx_status hx_integrator_set_policy(hx_integrator* integ, const hx_policy* policy);
/* num_accumulated_samples / tile_idx / num_target_samples (path_integrator.h:20-22). */
HX_API hx_status hx_integrator_progress(const hx_integrator* integ, uint32_t* accumulated_samples,
                                        uint32_t* tile_idx, uint32_t* target_samples);

/* Renderer::tone_map (renderer.cpp:369-426) + tone_map.frag:22-51: exposure,
 * ACES/Reinhard, gamma 1/2.2, RGBA8, vertically flipped like the
 * negative-height viewport (renderer.cpp:394-399).  host_rgba8 may be NULL
 * (result stays on the device). */
HX_API hx_status hx_integrator_tonemap(hx_integrator* integ, uint32_t op, float exposure,
                                       uint8_t* host_rgba8);

/* Reads the RGBA32F accumulation image (the ping-pong output image of
 * renderer.cpp:1483-1506) into width*height*4 floats. */
HX_API hx_status hx_integrator_read_accumulation(hx_integrator* integ, float* host_rgba32f);

/* Bake checkpoint / resume.  The reference keeps its progressive state (the
 * accumulation image, num_accumulated_samples, tile_idx of
 * path_integrator.h:46-53) only for the life of the process; these calls
 * serialise it to host memory and restore it into an integrator of the same
 * size, so a bake can stop and continue (another process, another GPU) with a
 * result bit-identical to an uninterrupted one: the next frame's samples are
 * seeded from the restored sample count, like the reference's frame index.
 * Layout: one hx_bake_checkpoint header, then the payload — the accumulation
 * image (RGBA32F, the running mean or the Kahan sum), the Kahan compensation
 * image (RGBA32F), the per-pixel sample counts (uint32), and with AOV
 * accumulation on the first-hit albedo+depth and normal images (RGBA32F each),
 * every image width*height in launch-grid order.  checksum is a 64-bit hash of
 * the payload (four multiply-rotate lanes over little-endian 8-byte words,
 * folded through the SplitMix64 finaliser). */
#define HX_BAKE_CHECKPOINT_MAGIC   0x4B425848u  /* "HXBK" */
#define HX_BAKE_CHECKPOINT_VERSION 1u
typedef struct hx_bake_checkpoint {
    uint32_t magic, version;
    uint32_t width, height;
    uint32_t max_samples;      /* samples per tile */
    uint32_t tiled;
    uint32_t accumulation;     /* HX_ACCUM_* */
    uint32_t accumulated;      /* samples of the current tile */
    uint32_t tile_idx;
    uint32_t aov;              /* 1: the two AOV images follow the counts */
    uint32_t aov_frames;
    uint32_t reserved;
    uint64_t payload_bytes;
    uint64_t checksum;
} hx_bake_checkpoint;          /* 64 bytes */

/* Bytes hx_integrator_save_checkpoint writes for the integrator's current
 * state (header included). */
HX_API hx_status hx_integrator_checkpoint_size(const hx_integrator* integ, size_t* bytes);
/* Waits for the integrator's queued work, then writes the checkpoint into
 * host[0 .. checkpoint_size); HX_ERR_INVALID_ARG if `bytes` is smaller, and
 * HX_ERR_DEVICE (no checkpoint) if the device status word is set. */
HX_API hx_status hx_integrator_save_checkpoint(hx_integrator* integ, void* host, size_t bytes);
/* Restores a checkpoint.  HX_ERR_INVALID_ARG, with the state unchanged, when
 * the magic, version, sizes or checksum do not match or when its width,
 * height, max_samples, tiled flag or accumulation mode differ from the
 * integrator's; AOV accumulation is switched to the checkpoint's setting.
 * Other parameters (bounces, bias, RNG kind) are the caller's to keep equal
 * for a bit-identical continuation. */
HX_API hx_status hx_integrator_load_checkpoint(hx_integrator* integ, const void* host, size_t bytes);

/* Output buffers of Renderer::set_current_output_buffer (renderer.h:27-35,
 * 85) and its debug-visualization pass (renderer.cpp:491-545,
 * debug_visualization.frag:71-161).  Rendered headless: one camera ray
 * through each pixel centre, the closest triangle without alpha test (the
 * raster pass never discards), the fragment shader's value (albedo; normals
 * * 0.5 + 0.5; roughness; metallic; emissive), misses (0, 0, 0, 1); width *
 * height RGBA32F in display order, like hx_integrator_tonemap.
 * HX_OUTPUT_FINAL returns the resolved accumulation in that order. */
#define HX_OUTPUT_ALBEDO    0u
#define HX_OUTPUT_NORMALS   1u
#define HX_OUTPUT_ROUGHNESS 2u
#define HX_OUTPUT_METALLIC  3u
#define HX_OUTPUT_EMISSIVE  4u
#define HX_OUTPUT_FINAL     5u
HX_API hx_status hx_integrator_render_output(hx_integrator* integ, const hx_frame_desc* frame,
                                             uint32_t output_buffer, float* host_rgba32f);

/* Ray-debug capture: PathIntegrator::gather_debug_rays
 * (include/gfx/path_integrator.h:35, path_integrator.cpp:88-104) with the
 * RAY_DEBUG_VIEW shaders (path_trace_rgen.glsl:136-147,183-188,
 * path_trace_rchit.glsl:548-567).  Traces num_debug_rays paths through
 * display pixel (pixel_x, pixel_y) (launch row height - pixel_y, as
 * path_integrator.cpp:146), each with its own colour (three draws, each
 * * 0.5 + 0.5); every closest hit after the camera ray records a line
 * segment: ray origin and hit point, two DebugRayVertex records
 * (common.glsl:54-58).  Nothing is accumulated.  *count = vertices recorded;
 * at most capacity are copied to host_vertices.  FP32 payloads only
 * (HX_ERR_UNSUPPORTED otherwise). */
typedef struct hx_debug_ray_vertex {
    float position[4]; /* xyz, 1 */
    float color[4];    /* rgb, 1 */
} hx_debug_ray_vertex;
HX_API hx_status hx_integrator_gather_debug_rays(hx_integrator* integ, const hx_frame_desc* frame, uint32_t pixel_x,
                                                 uint32_t pixel_y, uint32_t num_debug_rays,
                                                 hx_debug_ray_vertex* host_vertices, uint32_t capacity,
                                                 uint32_t* count);

/* Device-timed statistics of the last render call (CUDA events on the
 * context stream when timing is on). */
HX_API hx_status hx_integrator_set_timing(hx_integrator* integ, uint32_t enabled);
/* Counting mode: traversal launches also count node fetches, triangle tests
 * and their warp-level steps (hx_stats.node_visits ... lane_loop_busy); used
 * to derive the algorithmic bytes and the SIMD utilisation of the traversal,
 * never in a timed run. */
HX_API hx_status hx_integrator_set_counting(hx_integrator* integ, uint32_t enabled);
HX_API hx_status hx_integrator_stats(const hx_integrator* integ, hx_stats* out);

/* Parity hook: primary-ray closest hits (with the any-hit alpha test) for
 * every pixel of frame `frame_index`, in pixel order (y*width + x). */
HX_API hx_status hx_integrator_primary_hits(hx_integrator* integ, const hx_frame_desc* frame,
                                            uint32_t frame_index, hx_hit* host_hits);

/* Parity hook: per-sample radiance (before clamping) of frame `frame_index`
 * for every pixel, RGB, in pixel order. */
HX_API hx_status hx_integrator_sample_radiance(hx_integrator* integ, const hx_frame_desc* frame,
                                               uint32_t frame_index, float* host_rgb);

/* Parity hook: closest-hit queries for caller rays (origin xyz, tmin,
 * direction xyz, tmax) x n, alpha testing when any_hit != 0, traced by the
 * same traversal kernel as a frame's bounces. */
HX_API hx_status hx_scene_trace(const hx_scene* scene, const float* host_rays, uint32_t n,
                                uint32_t any_hit, hx_hit* host_hits);

/* Parity hook: the baked environment as RGB floats (width*height*3), the
 * FP16 texels widened. */
HX_API hx_status hx_scene_export_env(const hx_scene* scene, float* host_rgb);

/* Parity hook: RNG streams on the device.  For stream i the seed pair is
 * (seeds[2i], seeds[2i+1]) = (pixel id, frame/sample index); writes
 * draws_per_stream raw 32-bit outputs per stream. */
HX_API hx_status hx_rng_streams(hx_context* ctx, uint32_t rng_kind, const uint32_t* seeds,
                                uint32_t num_streams, uint32_t draws_per_stream,
                                uint32_t* host_out);

/* ------------------------------------------------------------------------ */
/* Serving loop (no reference counterpart; the nearest hook is the per-frame   */
/* Renderer::render, src/engine/gfx/renderer.cpp:107, that the application    */
/* loop calls once per window frame, application.cpp:38-54)                   */
/* ------------------------------------------------------------------------ */

typedef struct hx_server hx_server;

typedef struct hx_server_desc {
    uint64_t  request_arena_bytes;  /* HBM for per-request images: the admission budget  */
    uint32_t  max_paths_per_tick;   /* wavefront capacity of one scene tick              */
    uint32_t  max_ray_bounces;
    hx_policy policy;
    uint64_t  result_arena_bytes;   /* pinned host memory for finished images (0: 1/4 of the HBM arena) */
    uint64_t  admitted_work_paths;  /* admit while admitted remaining work <= this (0: 4 ticks) */
    uint32_t  max_concurrent_ticks; /* scene ticks in flight at once (0: 4)                */
    uint32_t  max_paths_per_long_tick; /* paths of one tick of requests that do not fit in
                                          one tick (0: max_paths_per_tick); smaller long
                                          ticks bound the wait of a short request behind one */
} hx_server_desc;

typedef struct hx_request_desc {
    uint32_t      scene_id;          /* from hx_server_add_scene                  */
    uint32_t      width, height;
    uint32_t      spp;               /* progressive samples per pixel             */
    uint32_t      denoise;           /* 1: denoise with the attached denoiser     */
    uint32_t      tonemap_op;        /* HX_TONEMAP_*                              */
    float         exposure;
    uint32_t      reserved;
    hx_frame_desc frame;             /* camera constants of the view              */
    uint64_t      user_tag;
} hx_request_desc;

typedef struct hx_request_result {
    uint64_t  request_id, user_tag;
    uint64_t  paths;                 /* camera samples traced for the request     */
    double    queue_ms;              /* submit -> admitted                        */
    double    latency_ms;            /* submit -> tone-mapped image in host memory */
    hx_status status;
    uint32_t  reserved;
} hx_request_result;

typedef struct hx_server_stats {
    uint64_t paths, ticks, requests_done, requests_pending, requests_active;
    uint64_t arena_bytes, arena_used;
    double   seconds;
    uint64_t requests_denoised;
    uint64_t requests_active_peak;  /* most requests admitted at once        */
    uint64_t arena_used_peak;       /* most device-arena bytes in use at once */
} hx_server_stats;

HX_API hx_status hx_server_create(hx_context* ctx, const hx_server_desc* desc, hx_server** out);
/* Makes a resident scene servable (captures its tick as a CUDA graph). */
HX_API hx_status hx_server_add_scene(hx_server* server, const hx_scene* scene, uint32_t* scene_id);
/* Attaches the learned denoiser used for requests with denoise set (same
 * context; before hx_server_start).  Such a request accumulates first-hit
 * AOVs while it renders; when it finishes it is denoised on the context
 * stream before tone mapping. */
HX_API hx_status hx_server_set_denoiser(hx_server* server, hx_denoiser* denoiser);
/* Starts the worker thread (admission, batching, launches). */
HX_API hx_status hx_server_start(hx_server* server);
/* Thread-safe, non-blocking. */
HX_API hx_status hx_server_submit(hx_server* server, const hx_request_desc* request, uint64_t* request_id);
/* Completed requests since the last poll; waits up to wait_seconds for one. */
HX_API hx_status hx_server_poll(hx_server* server, hx_request_result* out, uint32_t capacity, uint32_t* count,
                                double wait_seconds);
/* Copies a finished request's RGBA8 image (width*height*4, may be NULL) and
 * releases it. */
HX_API hx_status hx_server_fetch(hx_server* server, uint64_t request_id, uint8_t* host_rgba8);
/* Cancels a request (thread-safe, non-blocking; the serving form's own
 * control, no counterpart in the reference).  A pending request ends at
 * once; an admitted one ends as soon as none of its samples is on the GPU,
 * releasing its slot and arena space.  Either way its result reports
 * HX_ERR_CANCELLED and hx_server_fetch returns HX_ERR_CANCELLED (no image).
 * A request whose image is already complete is not affected.  Unknown ids:
 * HX_ERR_INVALID_ARG. */
HX_API hx_status hx_server_cancel(hx_server* server, uint64_t request_id);
HX_API hx_status hx_server_stats_get(hx_server* server, hx_server_stats* out);
HX_API hx_status hx_server_destroy(hx_server* server);

/* Allocation-free Morton sort.  No counterpart in the reference.  For callers
 * that cannot allocate device memory (an engine whose own allocator owns all
 * device memory, a process that may not grow its footprint after start-up, a
 * latency-critical thread that must not take the allocator's locks): the
 * Morton-code + stable-sort stage of the LBVH build over the caller's device
 * buffers, with no cudaMalloc.  d_world_tris: n x 9 floats (world-space
 * vertices, flattened order); d_morton[n]: 30-bit codes in input order;
 * d_sorted[n]: the stable sort order — the same values hx_scene_upload
 * computes (hx_scene_export_bvh).  n must be 1..262144 (2^18); larger n is
 * rejected with HX_ERR_INVALID_ARG.  Scratch is one fixed device array of
 * about 5 MB in the library, held by every GPU that loads it until exit.
 * Every call looks up that array's address on the current device (valid
 * again after a cudaDeviceReset); with lazy module loading (the CUDA default)
 * the first call on a device is also when the array is committed there, so a
 * caller that must not grow its footprint later makes one warm-up call at
 * start-up, before any stream capture.  Work is ordered on cuda_stream (a
 * cudaStream_t, NULL = default stream); calls that overlap on the GPU race on
 * the shared scratch. */
HX_API hx_status hx_lbvh_sort_noalloc(const float* d_world_tris, uint32_t n, uint32_t* d_morton, uint32_t* d_sorted,
                                      void* cuda_stream);

/* ------------------------------------------------------------------------ */
/* Procedural scenes for the benchmark configurations (host side)            */
/* ------------------------------------------------------------------------ */

#define HX_SCENE_BOX          0u  /* 5-wall box + 2 boxes + quad light (36 tris)         */
#define HX_SCENE_ICOSPHERES   1u  /* 12 icospheres + ground + alpha quads + sky + lights */
#define HX_SCENE_TERRAIN      2u  /* spheres + fBm heightfield + sun and sky             */

typedef struct hx_procedural_params {
    uint32_t kind;           /* HX_SCENE_*                                   */
    uint64_t seed;
    uint32_t num_alpha_quads;/* HX_SCENE_ICOSPHERES: default 100000          */
    uint32_t mask_pool;      /* distinct 512^2 masks (default 64)            */
    uint32_t mask_size;      /* default 512                                  */
    uint32_t icosphere_level;/* default 6 (81,920 triangles)                 */
    uint32_t env_width, env_height; /* default 2048 x 1024                   */
    float    sun_elevation_deg;     /* default 30                             */
    float    turbidity;             /* default 3                              */
    uint32_t terrain_size;          /* HX_SCENE_TERRAIN: grid vertices per side (default 4096) */
    uint32_t num_spheres;           /* HX_SCENE_TERRAIN: sphere instances (default 200)        */
    float    ground_albedo;         /* sky model ground albedo 0..1 (default 0.1)              */
} hx_procedural_params;

HX_API void      hx_procedural_defaults(uint32_t kind, hx_procedural_params* out);
HX_API hx_status hx_procedural_scene_create(const hx_procedural_params* params, hx_host_scene** out);
HX_API const hx_scene_desc* hx_host_scene_desc(const hx_host_scene* scene);
HX_API hx_status hx_host_scene_camera(const hx_host_scene* scene, hx_camera* out);
HX_API hx_status hx_host_scene_destroy(hx_host_scene* scene);

/* PNG export: replaces the stb_image_write call behind
 * Renderer::save_image_to_disk (renderer.h:97, renderer.cpp:637-713), which
 * writes the tone-mapped RGBA8 frame as a PNG.  8-bit RGBA rows top to
 * bottom (the layout hx_integrator_tonemap returns).  hx_encode_png writes
 * the file bytes to out (out = NULL: only *size is set); hx_save_png writes
 * them to path.  Host-only: needs no GPU. */
HX_API hx_status hx_encode_png(const uint8_t* rgba8, uint32_t width, uint32_t height, uint8_t* out,
                               uint64_t capacity, uint64_t* size);
HX_API hx_status hx_save_png(const char* path, const uint8_t* rgba8, uint32_t width, uint32_t height);

/* Hosek-Wilkie RGB coefficients (A..I, Z; 10 x vec4): HosekWilkieSkyModel::
 * update (hosek_wilkie_sky_model.cpp:658-686) for the given sun direction,
 * turbidity (clamped to 1..10 and blended between integer turbidities) and
 * ground albedo (blended between 0 and 1), as the reference's evaluate
 * (hosek_wilkie_sky_model.cpp:48-67) does, normalised so the luminance toward
 * the sun is normalized_sun_y (0: raw). */
HX_API hx_status hx_hosek_wilkie_sky(const float sun_direction[3], float turbidity, float albedo,
                                     float normalized_sun_y, float out[40]);
/* The same with the reference's default ground albedo 0.1
 * (hosek_wilkie_sky_model.h:33). */
HX_API hx_status hx_hosek_wilkie_coefficients(const float sun_direction[3], float turbidity,
                                              float normalized_sun_y, float out[40]);

/* ------------------------------------------------------------------------
 * Learned denoiser (no counterpart in the reference engine; its auxiliary
 * inputs follow the reference's AOV definitions, renderer.h:27-35 and
 * debug_visualization.frag:142-161).  A 5-level convolutional
 * encoder-decoder (3x3 convolutions, 32 -> 128 channels, skip connections),
 * BF16 weights and activations with FP32 accumulation on the tensor cores,
 * trained by its own forward/backward kernels and Adam.
 *
 * Features: per pixel 12 floats, NHWC — radiance rgb, noise level
 * 1/sqrt(samples in the pixel), albedo rgb, depth feature log1p(t)/8 (0 on a
 * miss), shading normal xyz, 0.  Targets: per
 * pixel RGBA float radiance (alpha ignored).  The network predicts
 * log1p(radiance) as the input's log1p radiance plus a learned correction;
 * the loss is chosen by hx_denoiser_set_loss.  Parameters: one flat FP32 vector, per layer W[9][cout][cin]
 * (tap = ky*3 + kx) then b[cout].
 * ------------------------------------------------------------------------ */
HX_API hx_status hx_denoiser_create(hx_context* ctx, hx_denoiser** out);
HX_API hx_status hx_denoiser_destroy(hx_denoiser* dn);
HX_API hx_status hx_denoiser_num_params(hx_denoiser* dn, uint64_t* n);
/* Load parameters (host FP32) and reset the Adam state. */
HX_API hx_status hx_denoiser_set_params(hx_denoiser* dn, const float* host, uint64_t n);
HX_API hx_status hx_denoiser_get_params(hx_denoiser* dn, float* host, uint64_t n);
/* Forward + backward over n crops of h x w (multiples of 16) held on the
 * device; the parameter gradient stays on the device (get_gradients reads
 * it); *loss (optional) receives the batch loss. */
HX_API hx_status hx_denoiser_forward_backward(hx_denoiser* dn, const float* d_features, const float* d_targets,
                                              uint32_t n, uint32_t h, uint32_t w, float* loss);
HX_API hx_status hx_denoiser_get_gradients(hx_denoiser* dn, float* host, uint64_t n);
/* Training loss: mean over pixels and colour channels of |y - log1p(t)|
 * (default) or of (expm1(y) - t)^2 (squared error of the linear radiance). */
#define HX_DN_LOSS_L1_LOG    0u
#define HX_DN_LOSS_L2_LINEAR 1u
HX_API hx_status hx_denoiser_set_loss(hx_denoiser* dn, uint32_t kind);
HX_API hx_status hx_denoiser_adam_step(hx_denoiser* dn, float lr);
HX_API hx_status hx_denoiser_train_step(hx_denoiser* dn, const float* d_features, const float* d_targets,
                                        uint32_t n, uint32_t h, uint32_t w, float lr, float* loss);
/* Inference over n images of h x w (any size; padded to 16 internally):
 * d_out_rgba receives n*h*w RGBA floats of denoised radiance.  Ordered on
 * the context stream; call hx_denoiser_check to collect pipeline errors. */
HX_API hx_status hx_denoiser_infer(hx_denoiser* dn, const float* d_features, uint32_t n, uint32_t h, uint32_t w,
                                   float* d_out_rgba);
HX_API hx_status hx_denoiser_check(hx_denoiser* dn);
/* Untrained starting point for training: He-uniform weights (bound
 * sqrt(6 / (9 cin))) from a SplitMix64 stream of `seed`, zero biases; resets
 * the Adam state. */
HX_API hx_status hx_denoiser_init_params(hx_denoiser* dn, uint64_t seed);
/* Diagnostic knob (no counterpart in the reference): the clock-cycle budget
 * of each tensor-core pipeline wait of later launches (0 = the default, about
 * two seconds; at most that).  A wait that runs out sets the denoiser's error
 * word; the CTA still waits (with the default budget) for its own TMA copies
 * and MMAs in flight, frees its TMEM and exits, and hx_denoiser_check then
 * returns HX_ERR_TIMEOUT.  A budget of a few cycles makes the waits run out
 * on purpose, to exercise that path. */
HX_API hx_status hx_denoiser_set_wait_budget(hx_denoiser* dn, uint64_t cycles);
/* Test access: a stored BF16 tensor (activation, or its gradient) of the
 * last training (training = 1) or inference pass, by index in network order
 * (x, a0, a0b, p0, a1, p1, a2, p2, a3, p3, a4, a4b, u3, d3, u2, d2, u1, d1,
 * u0, d0, d0b, gy), and the FP32 network output (RGBA per padded pixel). */
HX_API hx_status hx_denoiser_read_tensor(hx_denoiser* dn, uint32_t training, uint32_t index, uint32_t gradient,
                                         void* host, uint64_t bytes);
HX_API hx_status hx_denoiser_read_output(hx_denoiser* dn, uint32_t training, float* host, uint64_t count);

/* First-hit AOV accumulation (albedo, shading normal, depth feature averaged
 * over the same frames as the image; off by default).  Switching it restarts
 * the progressive accumulation. */
HX_API hx_status hx_integrator_set_aov_accumulation(hx_integrator* it, uint32_t enabled);
/* Denoiser inputs from an integrator: the current accumulated image, its
 * noise level (1/sqrt of each pixel's sample count) and albedo / normal /
 * depth — the accumulated AOVs when AOV accumulation is on, else those of the
 * primary hits of sample frame_index — into d_features (width*height*12
 * floats, device memory). */
HX_API hx_status hx_integrator_features(hx_integrator* it, const hx_frame_desc* frame, uint32_t frame_index,
                                        float* d_features);
/* The accumulated image (resolved RGBA floats) into device memory. */
HX_API hx_status hx_integrator_resolve(hx_integrator* it, float* d_rgba);
/* Denoise the accumulated image (features of sample 0) and tone-map the
 * result like hx_integrator_tonemap; host_rgba8 (optional) receives it, and
 * host_rgba32f (optional) the denoised HDR radiance. */
HX_API hx_status hx_integrator_denoise(hx_integrator* it, hx_denoiser* dn, const hx_frame_desc* frame, uint32_t op,
                                       float exposure, uint8_t* host_rgba8, float* host_rgba32f);

#ifdef __cplusplus
}
#endif

#endif /* HX_H */
