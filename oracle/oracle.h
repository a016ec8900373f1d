/*
 * oracle.h — CPU oracle for the draw hot path. TEST INFRASTRUCTURE ONLY.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
 * load this library, and only as the checker / the timed CPU baseline. The
 * product path (libcpvulkan_gb300.so) never calls it.
 *
 * What it is: a single-threaded C++ restatement of the reference ICD's CPU
 * draw path (CPVulkan/CommandBuffer.Draw.cpp, LLVMRuntime/PipelineCompiler.cpp,
 * LLVMRuntime/ImageCompiler.cpp, CPVulkan/ImageSampler.cpp,
 * CPVulkan/GlslFunctions.cpp), operating on the plain-data scene description
 * in include/cpv/scene.h. Shader programs are hand-written C++ restatements of
 * the SPIR-V modules the harness ships (one per cpv_program).
 *
 * Parity status: the reference as a whole cannot be built in this image (it
 * needs LLVM-C 8, the Khronos Vulkan headers, Microsoft GSL and glm >= 0.9.9,
 * none of which are present) and ships no tests, golden images or fixtures.
 * Its plain C++ parts of the path (edge function, fragment inputs, blend,
 * wrap / lerp / image sampling) are compiled from the reference's own files
 * by oracle/refpin and this restatement matches them bit for bit
 * (tests/test_oracle_pinned.py). The parts the reference generates as LLVM
 * IR at run time (pixel codecs, per-fragment operations, vertex fetch) and
 * glm's operand order in shaders are "parity unpinned": they are checked
 * against hand-derived known-answer tests (tests/golden/) only.
 */
#ifndef CPV_ORACLE_H
#define CPV_ORACLE_H

#include <stdint.h>

#include "../include/cpv/scene.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct cpv_oracle_stats {
    uint64_t triangles;        /* assembled triangles (all instances) */
    uint64_t vs_invocations;   /* vertex shader invocations (one per assembled vertex, as the reference) */
    uint64_t fragments;        /* covered pixels that ran the fragment shader */
    uint64_t fragments_written;/* fragments whose colour write happened */
} cpv_oracle_stats;

/* Renders draws [draw_begin, draw_end) of the scene (clear first when
 * do_clear != 0). color: width*height*4 bytes; depth: width*height*texel bytes
 * of depth_format (may be null when depth_format == 0). Both are read as the
 * initial attachment contents when do_clear == 0. Returns 0 on success,
 * negative on an unsupported scene. */
int cpv_oracle_render(const cpv_scene* scene, uint8_t* color, uint8_t* depth, uint32_t do_clear,
                      uint32_t draw_begin, uint32_t draw_end, cpv_oracle_stats* stats);

/* cpv_oracle_render with the scene's colour attachments after the first:
 * extra[k] is attachment k + 1 (width*height texels of its format), null
 * for an unused reference; extra may be null when the scene has none. */
int cpv_oracle_render_extra(const cpv_scene* scene, uint8_t* color, uint8_t* const* extra, uint8_t* depth, uint32_t do_clear,
                            uint32_t draw_begin, uint32_t draw_end, cpv_oracle_stats* stats);

/* The same render on `threads` host threads (the reference renders on one;
 * this is the oracle's own parallel form, for full-size checks): the
 * assembly of each draw instance is made once, vertex shading and triangle
 * set-up are split among the threads, and thread t writes the rows y with
 * y % threads == t, walking every triangle of every draw in API order, so
 * each pixel receives its fragments in the order of cpv_oracle_render and
 * the image is identical to it. */
int cpv_oracle_render_threaded(const cpv_scene* scene, uint8_t* color, uint8_t* depth, uint32_t do_clear,
                               uint32_t draw_begin, uint32_t draw_end, uint32_t threads, cpv_oracle_stats* stats);

/* Single-step helpers exposed for known-answer tests. */
/* A vertex attribute of `format` (32-bit float, normalised 8/16-bit, 16-bit
 * float, B8G8R8A8) decoded from its bytes into out (absent components
 * 0, 0, 0, 1); returns its component count, or -1 for another format. */
int cpv_oracle_decode_attribute(uint32_t format, const uint8_t* bytes, float out[4]);
float cpv_oracle_edge(float ax, float ay, float bx, float by, float cx, float cy);
uint8_t cpv_oracle_encode_unorm8(float value);
/* VkLogicOp `op` (0 CLEAR .. 15 SET) of an encoded source and destination byte. */
uint8_t cpv_oracle_logic_op(uint32_t op, uint8_t src, uint8_t dst);
uint16_t cpv_oracle_encode_unorm16(float value);
float cpv_oracle_decode_unorm8(uint8_t value);
/* Bilinear/nearest sample of level 0..levels-1 of an RGBA8 texture with the
 * reference sampler semantics; out = RGBA float. */
void cpv_oracle_sample(const uint8_t* texels, uint32_t width, uint32_t height, uint32_t levels,
                       const cpv_scene_sampler* sampler, float u, float v, float lod, float out[4]);
/* vkCmdBlitImage of one 2D colour region between RGBA8 (37) / BGRA8 (44)
 * images: region = src x0, y0, x1, y1, dst x0, y0, x1, y1; filter 0 NEAREST,
 * 1 LINEAR; dst is updated in place. */
void cpv_oracle_blit(const uint8_t* src, uint32_t src_w, uint32_t src_h, uint32_t src_format, uint8_t* dst, uint32_t dst_w, uint32_t dst_h,
                     uint32_t dst_format, const int32_t region[8], uint32_t filter);
/* Batch forms for the comparison with the reference's own functions
 * (oracle/refpin, tests/test_oracle_pinned.py); layouts as cpv_ref_*_n:
 * edge: 6 floats in, 1 out per case; wrap: value, size, address mode;
 * blend: 4 + 4 + 4 floats and 6 modes (src/dst colour factor, colour op,
 * src/dst alpha factor, alpha op) per case; fragment input: p0, p1, p2
 * (NDC x, y, z, clip w) and the pixel centre (14 floats), 27 vertex floats
 * (perspective vec4, linear vec4, flat float per vertex), cull mode and
 * provoking vertex in, covered, front, depth and 9 components out;
 * sample: 6 modes (mag, min, mipmap, address u, address v, border) and
 * u, v, λ in (no bias, no λ clamp), 4 floats out. */
/* 0.5 * log2(r) as the quad-derivative LOD mode computes it (own series,
 * the same binary32 steps as the GPU path). */
void cpv_oracle_half_log2_n(const float* in, float* out, uint64_t n);
/* λ_base of the quad-derivative LOD mode for n fragments: in[6 i ..] =
 * (u, v, u and v at the horizontal neighbour, u and v at the vertical one),
 * odd[i] bit 0 / bit 1 = x / y odd, on a width x height level 0. */
void cpv_oracle_quad_lambda_n(const float* in, const uint32_t* odd, uint32_t width, uint32_t height, float* out, uint64_t n);
void cpv_oracle_edge_n(const float* in, float* out, uint64_t n);
void cpv_oracle_wrap_n(const int32_t* v, const int32_t* size, const uint32_t* mode, int32_t* out, uint64_t n);
void cpv_oracle_blend_n(const float* src, const float* dst, const float* constant, const uint32_t* modes, float* out, uint64_t n);
void cpv_oracle_fragment_input_n(const float* pts, const float* vars, const uint32_t* cull, const uint32_t* provoking, float* out, uint64_t n);
void cpv_oracle_sample_n(const uint8_t* texels, uint32_t width, uint32_t height, uint32_t levels, const uint32_t* modes, const float* uvl,
                         float* out, uint64_t n);
/* Blend one colour against a destination with the reference blend equations. */
void cpv_oracle_blend(const float src[4], const float dst[4], const float constant[4],
                      uint32_t src_color, uint32_t dst_color, uint32_t color_op,
                      uint32_t src_alpha, uint32_t dst_alpha, uint32_t alpha_op, float out[4]);

#ifdef __cplusplus
}
#endif

#endif
