/*
 * scene.h — plain-data description of one frame of draws: the contract
 * between the headless application harness (which turns it into Vulkan calls
 * on the ICD) and the CPU oracle (which renders the same bytes with the
 * reference's CPU draw semantics).
 *
 * Nothing here is a Vulkan object. Enumerants reuse the Vulkan values (see
 * vk_subset.h) so that the harness passes them through unchanged.
 *
 * A frame = begin render pass (clear colour, clear depth) → draws in order →
 * end render pass. Every draw binds one pipeline, its vertex buffer offsets,
 * optional index buffer offset and push constants. One uniform block (set 0,
 * binding 0) and at most one combined image sampler (set 0, binding 1) are
 * shared by all draws of a scene.
 */
#ifndef CPV_SCENE_H
#define CPV_SCENE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Shader programs (vertex + fragment pair). The harness maps each to the
 * SPIR-V modules it ships; the oracle maps each to a hand-written C++
 * restatement of the same arithmetic. */
enum cpv_program {
    CPV_PROGRAM_CUBE = 0,        /* pos vec4 + colour vec4 → UBO mat4 MVP; FS passes colour                      */
    CPV_PROGRAM_TEXLIT = 1,      /* pos vec3 + uv vec2 + normal vec3 → UBO {MVP, light}; FS texture × Lambert  */
    CPV_PROGRAM_FLATQUAD = 2,    /* pos vec2 (NDC) + flat colour vec4 → FS passes colour                         */
    CPV_PROGRAM_MESHPC = 3,      /* pos vec3 + normal vec3 + per-instance offset vec4 → push {MVP, colour}; Lambert */
    CPV_PROGRAM_DISCARD = 4,     /* CUBE with a fragment discard when colour.r > 0.5 (OpKill coverage)          */
    CPV_PROGRAM_NOPERSP = 5,     /* CUBE with noperspective colour (InterpolationType::Linear coverage)         */
    CPV_PROGRAM_POINTS = 6,      /* CUBE that also writes gl_PointSize = colour.a * 16                          */
    CPV_PROGRAM_FETCH = 7,       /* TEXLIT's vertex shader; FS: texelFetch at uv * (K * 8 + 8) with K a
                                    specialisation constant (default 3), bitCount, a copy between variables */
    CPV_PROGRAM_MRT = 8,         /* CUBE's vertex shader; FS: eight outputs (locations 0-7), each a different
                                    function of the colour, one per colour attachment                         */
    CPV_PROGRAM_MRTI = 9,        /* CUBE's vertex shader; FS: vec4 colour, uvec4(c * 300), ivec4(c * 400 - 200)
                                    and floatBitsToUint(c) at locations 0-3 (integer attachments)            */
    CPV_PROGRAM_STORAGE = 10,    /* TEXLIT's vertex shader; FS: imageLoad of an rgba8 storage image at
                                    ivec2(uv * 64) (OpImageRead)                                              */
    CPV_PROGRAM_SEPARATE = 11,   /* TEXLIT with the texture and its sampler in separate bindings, joined by
                                    sampler2D(t, s) (OpSampledImage)                                          */
    CPV_PROGRAM_MATHX = 12,      /* CUBE's vertex shader; FS: GLSL.std.450 NMin/NMax/NClamp (with a NaN),
                                    FindSMsb/FindILsb/SSign/FindUMsb on integers from the colour, Reflect    */
    CPV_PROGRAM_CALLS = 13,      /* CUBE's vertex shader; FS: function calls (a pointer and a value parameter,
                                    a return value, a discard inside a called function)                      */
    CPV_PROGRAM_SSBO = 14,       /* CUBE's vertex shader; FS: colour × row 1 of a read-only storage buffer
                                    (the uniform buffer bound again at binding 3, cpv_scene::uniform_as_storage) */
    CPV_PROGRAM_COUNT = 15
};

/* How a scene's texture is bound (cpv_scene::texture_binding). */
enum cpv_texture_binding {
    CPV_TEXTURE_COMBINED = 0,  /* binding 1: a combined image sampler                   */
    CPV_TEXTURE_STORAGE = 1,   /* binding 1: a storage image (layout GENERAL)           */
    CPV_TEXTURE_SEPARATE = 2   /* binding 1: a sampled image; binding 2: its sampler     */
};

#define CPV_SCENE_MAX_BINDINGS 4
#define CPV_SCENE_MAX_ATTRIBUTES 8
#define CPV_SCENE_MAX_PUSH 128
#define CPV_SCENE_MAX_EXTRA_COLOR 7 /* colour attachments after the first */

/* Blend state of one colour attachment after the first. */
typedef struct cpv_scene_attachment_blend {
    uint32_t blend_enable;
    uint32_t src_color, dst_color, color_op;
    uint32_t src_alpha, dst_alpha, alpha_op;
    uint32_t color_write_mask; /* VkColorComponentFlags */
} cpv_scene_attachment_blend;

typedef struct cpv_scene_binding {
    uint32_t binding;
    uint32_t stride;
    uint32_t input_rate; /* VkVertexInputRate */
} cpv_scene_binding;

typedef struct cpv_scene_attribute {
    uint32_t location;
    uint32_t binding;
    uint32_t format; /* VkFormat */
    uint32_t offset;
} cpv_scene_attribute;

typedef struct cpv_scene_stencil {
    uint32_t fail_op, pass_op, depth_fail_op, compare_op;
    uint32_t compare_mask, write_mask, reference;
} cpv_scene_stencil;

typedef struct cpv_scene_pipeline {
    uint32_t program;    /* cpv_program */
    uint32_t topology;   /* VkPrimitiveTopology (point list, line list / strip, triangle list / strip / fan) */
    uint32_t cull_mode;  /* VkCullModeFlags */
    uint32_t front_face; /* VkFrontFace */
    uint32_t depth_test, depth_write, depth_compare;
    uint32_t stencil_test;
    cpv_scene_stencil stencil_front, stencil_back;
    uint32_t blend_enable;
    uint32_t src_color, dst_color, color_op;
    uint32_t src_alpha, dst_alpha, alpha_op;
    float blend_constants[4];
    uint32_t num_bindings;
    cpv_scene_binding bindings[CPV_SCENE_MAX_BINDINGS];
    uint32_t num_attributes;
    cpv_scene_attribute attributes[CPV_SCENE_MAX_ATTRIBUTES];
    float line_width;    /* VkPipelineRasterizationStateCreateInfo::lineWidth */
    uint32_t color_write_mask; /* VkColorComponentFlags: R 1, G 2, B 4, A 8 (0xF writes every channel) */
    uint32_t logic_op_enable;  /* VkPipelineColorBlendStateCreateInfo::logicOpEnable (blending then off) */
    uint32_t logic_op;         /* VkLogicOp, CLEAR (0) .. SET (15) */
    uint32_t depth_bounds_test;              /* VkPipelineDepthStencilStateCreateInfo::depthBoundsTestEnable */
    float min_depth_bounds, max_depth_bounds;
    uint32_t spec_k;           /* non-zero: the fragment shader's specialisation constant 0 (a 32-bit int) */
    cpv_scene_attachment_blend extra_blend[CPV_SCENE_MAX_EXTRA_COLOR]; /* colour attachments 1 .. */
} cpv_scene_pipeline;

typedef struct cpv_scene_draw {
    uint32_t pipeline;       /* index into pipelines */
    uint32_t indexed;        /* vkCmdDrawIndexed when non-zero */
    uint32_t count;          /* vertexCount or indexCount */
    uint32_t instance_count;
    uint32_t first;          /* firstVertex or firstIndex */
    int32_t vertex_offset;   /* vertexOffset (indexed only) */
    uint32_t first_instance;
    uint32_t push_size;
    uint64_t vertex_offsets[CPV_SCENE_MAX_BINDINGS]; /* byte offsets into vertex_data, per binding slot */
    uint64_t index_offset;   /* byte offset into index_data */
    uint8_t push[CPV_SCENE_MAX_PUSH];
} cpv_scene_draw;

typedef struct cpv_scene_sampler {
    uint32_t mag_filter, min_filter, mipmap_mode;
    uint32_t address_u, address_v, address_w;
    float mip_lod_bias, min_lod, max_lod;
    uint32_t border_color;
} cpv_scene_sampler;

typedef struct cpv_scene {
    uint32_t width, height;
    uint32_t color_format; /* VkFormat: R8G8B8A8_UNORM or B8G8R8A8_UNORM; 0: no colour attachment (depth-only) */
    uint32_t depth_format; /* VkFormat: 0 (none), D16_UNORM, D32_SFLOAT, D32_SFLOAT_S8_UINT */
    float clear_color[4];
    float clear_depth;
    uint32_t clear_stencil;
    float viewport[6]; /* x, y, width, height, minDepth, maxDepth */

    const uint8_t* vertex_data;
    uint64_t vertex_bytes;
    const uint8_t* index_data;
    uint64_t index_bytes;
    uint32_t index_type; /* VkIndexType */

    const uint8_t* uniform_data; /* set 0 binding 0 (may be null) */
    uint32_t uniform_bytes;

    /* set 0 binding 1: one 2D texture with a full linear mip chain, levels
     * concatenated level after level (the reference's linear image layout). */
    const uint8_t* texture_data;
    uint64_t texture_bytes;
    uint32_t texture_width, texture_height, texture_levels;
    uint32_t texture_format; /* VkFormat, R8G8B8A8_UNORM */
    cpv_scene_sampler sampler;

    uint32_t num_pipelines;
    const cpv_scene_pipeline* pipelines;
    uint32_t num_draws;
    const cpv_scene_draw* draws;

    /* colour attachments after the first (same size; 0 formats: unused
     * references), referenced by the subpass in order after it. An
     * integer-format attachment is cleared with the integers
     * round(clear_color * 100). */
    uint32_t extra_color_count;
    uint32_t extra_color_formats[CPV_SCENE_MAX_EXTRA_COLOR];

    /* 1: implicit-LOD sampling in fragment shaders takes λ from quad
     * derivatives (the ICD's CPV_SPEC_LOD=1 mode); 0: λ = 0 as the
     * reference computes it. */
    uint32_t spec_lod;

    /* cpv_texture_binding: the descriptors the texture is bound through */
    uint32_t texture_binding;

    /* 1: the uniform buffer is also bound at binding 3 as a storage buffer */
    uint32_t uniform_as_storage;
} cpv_scene;

#ifdef __cplusplus
}
#endif

#endif /* CPV_SCENE_H */
