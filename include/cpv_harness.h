/*
 * cpv_harness.h — C ABI of libcpv_harness.so: a headless application that
 * loads an ICD shared object the way the Vulkan loader does (dlopen,
 * vk_icdNegotiateLoaderICDInterfaceVersion, vk_icdGetInstanceProcAddr,
 * dispatch-word check) and renders plain-data scenes (cpv/scene.h) through
 * the Vulkan API only. It stands in for the loader and the LunarG samples,
 * neither of which exists on these machines.
 *
 * It also holds the seeded scene generators of the benchmark workloads.
 */
#ifndef CPV_HARNESS_H
#define CPV_HARNESS_H

#include <stdint.h>

#include "cpv/scene.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Scene configurations. */
enum cpvh_config {
    CPVH_CUBE = 1,        /* spinning cube, 500x500 BGRA8 + D16 (param0 = frame index)                         */
    CPVH_HEIGHTFIELD = 2, /* textured heightfield (param0 = grid side, default 1024; param1/2 = width/height)   */
    CPVH_BLEND = 3,       /* blend-bound overdraw quads (param0 = quad count, default 200000; param1/2 = w/h; param3 = 1: colour per corner, interpolated) */
    CPVH_BATCH = 4,       /* 4096 icosphere draws (param0 = draw count, param1 = max triangles, param2/3 = w/h) */
    CPVH_PROGRAM = 5,     /* small scene for one shader program (param0 = cpv_program, param1 = variant, param2/3 = w/h, param4 = triangles, param5 = colour attribute VkFormat of CUBE-family programs, or FETCH's specialisation constant, param6 = colour attachment VkFormat, 0 for RGBA8/BGRA8 by variant) */
    CPVH_SERVE = 6        /* one serving request (param0 = side px, param1 = triangles, param2 = client id)     */
};

/* Builds a scene; the harness owns every array it points to. */
cpv_scene* cpvh_scene_create(uint32_t config, uint64_t seed, const uint64_t* params, uint32_t num_params);
void cpvh_scene_destroy(cpv_scene* scene);
/* Updates the per-frame data of a scene (the cube's rotation for frame f). */
void cpvh_scene_set_frame(cpv_scene* scene, uint32_t frame);
/* Total triangles of all draws × instances. */
uint64_t cpvh_scene_triangles(const cpv_scene* scene);

typedef struct cpvh_context cpvh_context;
typedef struct cpvh_renderer cpvh_renderer;

/* Loads the ICD at icd_path and creates instance, device and queue.
 * Returns NULL and fills err on failure. */
cpvh_context* cpvh_open(const char* icd_path, char* err, uint32_t err_len);
void cpvh_close(cpvh_context* ctx);

/* Creates every Vulkan object the scene needs and records one command
 * buffer (clear + all draws). Vertex/index/uniform/texture data are uploaded
 * once into device-local memory through a staging buffer. */
cpvh_renderer* cpvh_renderer_create(cpvh_context* ctx, const cpv_scene* scene, char* err, uint32_t err_len);
void cpvh_renderer_destroy(cpvh_renderer* r);

/* Submits the recorded frame `frames` times, waiting on the fence after each
 * submission. device_ms: device time of all frames (queue events) or NULL;
 * latency_ms: per-frame host submit→fence times (array of `frames`) or NULL.
 * Returns a VkResult. */
int cpvh_render(cpvh_renderer* r, uint32_t frames, double* device_ms, double* latency_ms);

/* Device-timed frames: before each frame, a vkCmdFillBuffer over
 * `flush_bytes` of scratch memory evicts the L2 (untimed); the frame itself
 * is bracketed by queue events. frame_ms receives `frames` device times. */
int cpvh_render_timed(cpvh_renderer* r, uint32_t frames, uint64_t flush_bytes, double* frame_ms);

/* End-to-end frame through the public API: uploads the scene's vertex,
 * index and uniform bytes from host memory (map/copy/unmap + vkCmdCopyBuffer),
 * renders, copies the colour attachment to a host-visible buffer and reads
 * it back. Returns a VkResult; bytes moved are reported. */
int cpvh_render_e2e(cpvh_renderer* r, uint32_t frames, double* total_ms, uint64_t* h2d_bytes, uint64_t* d2h_bytes);

/* Creates (then destroys) only the scene's graphics pipelines: SPIR-V
 * translation and NVRTC compilation, without rendering. Returns a VkResult. */
int cpvh_compile_pipelines(cpvh_context* ctx, const cpv_scene* scene, char* err, uint32_t err_len);

/* Re-uploads the scene's uniform buffer and push constants (e.g. after
 * cpvh_scene_set_frame) and re-records the frame. */
int cpvh_renderer_update(cpvh_renderer* r);

/* With CPVH_INDIRECT=1 or 2 at creation: overwrites draw `draw`'s indirect record
 * (5 words; a non-indexed draw uses the first 4) through vkMapMemory /
 * vkUnmapMemory, without re-recording; the next frame reads it. Returns a
 * VkResult (VK_ERROR_INITIALIZATION_FAILED without indirect records). */
int cpvh_renderer_set_indirect(cpvh_renderer* r, uint32_t draw, const uint32_t record[5]);

/* With CPVH_INDIRECT=2 at creation (each draw an indirect-count draw of at
 * most one record): overwrites draw `draw`'s count word; 0 skips the draw,
 * any larger value draws its one record. Returns a VkResult. */
int cpvh_renderer_set_indirect_count(cpvh_renderer* r, uint32_t draw, uint32_t count);

/* Reads the attachments back (colour: width*height*4; depth: texel-sized). */
int cpvh_readback(cpvh_renderer* r, uint8_t* color, uint8_t* depth);
/* Colour attachment k (1 .. 7) of the scene's subpass after the last frame:
 * width * height texels of its format (zeros for an unused reference). */
int cpvh_readback_extra(cpvh_renderer* r, uint32_t k, uint8_t* out);

/* Creates and destroys one of each host object kind the ICD places in an
 * application allocator (buffer, device memory, image, image view, render
 * pass, framebuffer, sampler, pipeline cache, descriptor set layout,
 * pipeline layout, descriptor pool, command pool, fence), passing a counting
 * VkAllocationCallbacks to every call; reports the objects created and the
 * allocator's allocations and frees. Returns the first failing VkResult. */
int cpvh_allocator_check(cpvh_context* ctx, uint64_t* objects, uint64_t* allocations, uint64_t* frees);

/* One transfer / clear command of cpvh_image_ops on image 0 (image 1 is a
 * copy source). */
enum {
    CPVH_OP_CLEAR_COLOR_IMAGE = 0,         /* vkCmdClearColorImage of levels level .. level+level_count-1 */
    CPVH_OP_CLEAR_DEPTH_STENCIL_IMAGE = 1, /* vkCmdClearDepthStencilImage of those levels, aspects `aspect` */
    CPVH_OP_COPY_IMAGE = 2,                /* vkCmdCopyImage: image 1 level src_level at (src_x, src_y) → image 0 level `level` at (x, y), w x h */
    CPVH_OP_CLEAR_ATTACHMENTS = 3          /* vkCmdClearAttachments in a LOAD/STORE render pass over level `level`: rectangle (x, y, w, h) */
};
typedef struct cpvh_image_op {
    uint32_t kind;
    uint32_t aspect; /* VkImageAspectFlags of the range, region or clear */
    uint32_t level, level_count, src_level;
    int32_t x, y, src_x, src_y;
    uint32_t w, h;
    float colour[4];
    float depth;
    uint32_t stencil;
} cpvh_image_op;

/* Runs `ops` in order through the ICD on two 2D images of `format` (one
 * layer, `levels` mips of width x height halving), initialised from init0 /
 * init1 (every level packed in order, in the ICD's texel layout: 4 bytes for
 * colour, 2 for D16, 4 for D32, 8 for D32S8 with the stencil in byte 4;
 * init1 may be null: zeros), then reads image 0 back into `out` in the same
 * layout. Returns a VkResult. */
int cpvh_image_ops(cpvh_context* ctx, uint32_t format, uint32_t width, uint32_t height, uint32_t levels, const uint8_t* init0, const uint8_t* init1,
                   const cpvh_image_op* ops, uint32_t op_count, uint8_t* out, char* err, uint32_t err_len);

/* vkCmdBlitImage through the ICD. src (and dst when not null) hold every mip
 * level of an RGBA8 (37) / BGRA8 (44) image, level l being
 * max(w >> l, 1) x max(h >> l, 1) texels, packed one after another. Both
 * images are uploaded, one vkCmdBlitImage per region is recorded (each 10
 * ints: src level, src x0, y0, x1, y1, dst level, dst x0, y0, x1, y1) with a
 * barrier between regions, and the destination is read back into dst, or
 * into src when dst is null (the regions then blit within the source image,
 * as a mip chain is generated). filter: 0 NEAREST, 1 LINEAR. Returns a
 * VkResult. */
int cpvh_blit(cpvh_context* ctx, uint8_t* src, uint32_t src_w, uint32_t src_h, uint32_t src_levels, uint32_t src_format, uint8_t* dst,
              uint32_t dst_w, uint32_t dst_h, uint32_t dst_levels, uint32_t dst_format, const int32_t* regions, uint32_t region_count,
              uint32_t filter, char* err, uint32_t err_len);

/* The ICD's vkQueue (for the ICD's timing helpers). */
void* cpvh_queue(cpvh_context* ctx);
const char* cpvh_last_error(void);

/* ---- serving: continuous batching of offscreen clients ----
 *
 * Each client owns a seeded textured-icosphere scene (image side uniform over
 * {256, 512, 1024, 2048}, at most max_side when non-zero; triangles
 * log-uniform in [min_tris, max_tris]) whose pipelines, buffers, texture and
 * attachments are created once and stay resident while the resident total
 * fits hbm_budget_bytes. Requests arrive per client with exponential
 * inter-arrival times (mean mean_interarrival_ms) during duration_s; a
 * request renders one frame of its client. The loop admits the oldest
 * waiting request whose client is idle whenever one of `slots` queues is
 * free and the footprint of the requests in flight stays within the budget,
 * and retires requests as their fences signal. */
typedef struct cpvh_serve_config {
    uint32_t clients;
    uint32_t slots;
    double mean_interarrival_ms;
    double duration_s;
    uint64_t seed;
    uint64_t hbm_budget_bytes;   /* resident clients' footprint (attachments, buffers, texture) */
    uint32_t min_tris, max_tris;
    uint32_t max_side;
    /* 1: a request of a client that is not resident is admitted by making
     * the client resident, evicting idle resident clients (least recently
     * used first) until it fits the budget; 0: such clients are never made
     * resident and their requests are not generated */
    uint32_t admit_on_demand;
} cpvh_serve_config;

typedef struct cpvh_serve_result {
    uint64_t requests, completed, triangles;
    uint32_t resident_clients, max_in_flight;
    uint64_t resident_bytes;
    double wall_s, mtri_s;
    double latency_p50_ms, latency_p99_ms; /* arrival → fence signalled */
    double submit_p50_ms, submit_p99_ms;   /* vkQueueSubmit → fence signalled */
    double queue_p50_ms, queue_p99_ms;     /* arrival → vkQueueSubmit */
    uint64_t residencies, evictions;       /* clients made resident / evicted during the run */
    double residency_p50_ms, residency_p99_ms; /* time to make a client resident (objects, upload, recording) */
} cpvh_serve_result;

typedef struct cpvh_server cpvh_server;
cpvh_server* cpvh_server_create(cpvh_context* ctx, const cpvh_serve_config* cfg, char* err, uint32_t err_len);
int cpvh_server_run(cpvh_server* server, cpvh_serve_result* out);
/* Sets the mean inter-arrival time and the arrival window of later runs. */
void cpvh_server_set_load(cpvh_server* server, double mean_interarrival_ms, double duration_s);
uint32_t cpvh_server_clients(const cpvh_server* server);
/* The client's renderer (readback, or a frame rendered alone with
 * cpvh_render), or NULL when the client is not resident. */
cpvh_renderer* cpvh_server_client(cpvh_server* server, uint32_t client);
const cpv_scene* cpvh_server_scene(cpvh_server* server, uint32_t client);
void cpvh_server_destroy(cpvh_server* server);

#ifdef __cplusplus
}
#endif

#endif /* CPV_HARNESS_H */
