/*
 * cpv_params.h — per-draw parameter block shared by the host runtime and
 * every draw kernel (plain C++ layout, no device code). Included by
 * cpv_device.cuh on the device side and by the runtime on the host side.
 */
#ifndef CPV_PARAMS_H
#define CPV_PARAMS_H

#ifdef __CUDACC_RTC__
typedef unsigned char uint8_t;
typedef signed char int8_t;
typedef unsigned short uint16_t;
typedef short int16_t;
typedef unsigned int uint32_t;
typedef int int32_t;
typedef unsigned long long uint64_t;
typedef long long int64_t;
#else
#include <stdint.h>
#endif

#define CPV_MAX_VB 8
#define CPV_MAX_UBO 8
#define CPV_MAX_TEX 4
#define CPV_MAX_VARYINGS 16
#define CPV_MAX_LEVELS 16
#define CPV_MAX_CA 8 /* colour attachments per subpass (the reference's MAX_FRAGMENT_OUTPUT_ATTACHMENTS) */

/* Status word bits written by kernels instead of trapping. */
#define CPV_STATUS_LIST_OVERFLOW 0x1u
#define CPV_STATUS_BAD_INPUT 0x2u
#define CPV_STATUS_TIMEOUT 0x4u

#define CPV_FMT_R8G8B8A8_UNORM 37u
#define CPV_FMT_B8G8R8A8_UNORM 44u
#define CPV_FMT_D16_UNORM 124u
#define CPV_FMT_D32_SFLOAT 126u
#define CPV_FMT_D32_SFLOAT_S8_UINT 130u

/* One sampled image + its sampler, resolved from a descriptor at draw time.
 * Levels follow the reference's linear layout: level after level, tightly
 * packed rows (CPVulkanBase/Formats.cpp:453-484). */
struct CpvTexture {
    const uint8_t* data;
    uint64_t bytes;
    uint64_t level_offset[CPV_MAX_LEVELS];
    uint32_t level_w[CPV_MAX_LEVELS];
    uint32_t level_h[CPV_MAX_LEVELS];
    uint32_t levels;
    uint32_t format;
    uint32_t mag_filter, min_filter, mipmap_mode;
    uint32_t address_u, address_v, border;
    float lod_bias, min_lod, max_lod;
};

/* Everything one draw's kernels read. Passed by value as a kernel argument. */
struct CpvDrawParams {
    /* geometry */
    const uint8_t* vb[CPV_MAX_VB];
    uint64_t vb_bytes[CPV_MAX_VB];
    const uint8_t* ib;
    uint64_t ib_bytes;
    uint32_t index_size; /* 0 = non-indexed, 2 or 4 */
    uint32_t count;      /* vertexCount or indexCount */
    uint32_t first;      /* firstVertex or firstIndex */
    int32_t vertex_offset;
    uint32_t first_instance;
    uint32_t instance_count;
    uint32_t prims_per_instance;
    uint32_t pad0;
    uint64_t total_prims;
    /* resources */
    const uint8_t* ubo[CPV_MAX_UBO];
    uint64_t ubo_bytes[CPV_MAX_UBO];
    CpvTexture tex[CPV_MAX_TEX];
    uint32_t push[32];
    /* attachments */
    uint8_t* color;
    uint8_t* depth;
    uint8_t* color_extra[CPV_MAX_CA - 1]; /* colour attachments 1 .. of the subpass (null: unused) */
    uint32_t fb_width, fb_height;
    float viewport[6];
    float blend_constants[4];
    /* screen tiling */
    uint32_t tile_shift;
    uint32_t tiles_x, tiles_y;
    uint32_t pad1;
    /* binning scratch (null in direct mode) */
    const uint32_t* tile_end;   /* tiles*spans cursor matrix after the write pass */
    const uint32_t* bin_list;   /* primitive ids, tile-major, primitive order within a tile */
    const uint32_t* pair_total; /* device word: pairs the draw needed */
    const uint16_t* rects;      /* per primitive tile rectangle (x0,y0,x1,y1), exclusive ends */
    /* the union of the draw's tile rectangles, 4 device words kept as maxima
     * of (0xFFFF - x0, 0xFFFF - y0, x1, y1) (zeroed before the draw): the
     * (tiles x spans) matrix covers only its tiles, row-major */
    uint32_t* tile_box;
    uint32_t spans;
    uint32_t list_capacity;
    uint32_t* status;
    /* per primitive 4 x 256 bytes: the blend result of each channel for each
     * destination byte (pipelines blending a constant colour; null: compute) */
    uint8_t* tables;
    /* vertex slots of the batched path's vertex stage: vertex ids
     * [vs_lo, vs_lo + vs_count) of every instance, shaded once per frame
     * (slot = local instance * vs_count + id - vs_lo). vs_pos holds NDC x, y,
     * z and clip w per slot, vs_var vs_stride floats of outputs per slot.
     * vs_count 0: no slots, the set-up shades its vertices itself. */
    float* vs_pos;
    float* vs_var;
    uint32_t vs_lo;
    uint32_t vs_count;
    uint32_t vs_stride;
    uint32_t pad2;
};

/* Primitives per set-up block of the batched path: every draw of a batch
 * starts at a multiple of this in the batch's primitive index space, so a
 * primitive index g belongs to block g / CPV_BATCH_BLOCK and that block to
 * exactly one draw. */
#define CPV_BATCH_BLOCK 256u

/* Everything the batched kernels read: the draws of one render pass, their
 * tables and the binning buffers. Passed by value as a kernel argument. */
struct CpvBatchParams {
    const struct CpvDrawParams* draws; /* per draw (device array) */
    const uint32_t* draw_pipeline;     /* per draw: pipeline index in the module */
    const uint32_t* draw_block;        /* per draw + 1: first set-up block */
    const uint32_t* block_draw;        /* per set-up block: its draw */
    uint32_t num_draws;
    uint32_t total_blocks;
    /* shared attachments and pixel-centre grid of the render pass */
    uint8_t* color;
    uint8_t* depth;
    uint8_t* color_extra[CPV_MAX_CA - 1];
    uint32_t fb_width, fb_height;
    float vw, vh;
    uint32_t tiles_x, tiles_y;
    /* binning */
    uint2* rects;                 /* per primitive tile rectangle, packed */
    uint32_t* block_pairs;        /* per set-up block: (primitive, tile) pairs */
    const uint32_t* block_offsets;/* exclusive scan of block_pairs */
    const uint32_t* pair_total;   /* device word: pairs of the batch */
    uint32_t pair_capacity;
    uint32_t pad0;
    const uint32_t* sorted_prims; /* pair primitives sorted by tile, API order within a tile */
    const uint32_t* tile_begin;   /* per tile: range in sorted_prims */
    const uint32_t* tile_end;
    uint32_t* tile_counter;       /* persistent raster work queue */
    uint32_t* status;
    /* pixel-centre NDC of every column (fb_width) and row (fb_height):
     * (x / vw + (1 / vw) * 0.5) * 2 - 1, each operation rounded once */
    const float* ndc_x;
    const float* ndc_y;
    /* vertex stage: draw d owns vertex blocks [vs_draw_block[d],
     * vs_draw_block[d+1]) of CPV_BATCH_BLOCK slots each */
    const uint32_t* vs_draw_block;
    const uint32_t* vs_block_draw;
    uint32_t vs_blocks;
    uint32_t pad1;
};

#endif /* CPV_PARAMS_H */
