/*
 * cpv_pipeline.cuh — the kernels of one graphics pipeline for the per-draw
 * path. Compiled by NVRTC at vkCreateGraphicsPipelines after cpv_device.cuh,
 * cpv_raster.cuh and the pipeline's stage functions (cpv_stage.cuh in
 * namespace cpv_p0).
 *
 * Kernels:
 *   cpv_setup_rects — one thread per primitive: runs the vertex shader for the
 *                     primitive's three vertices (positions only), the
 *                     reference's bounding box and cull test, and writes the
 *                     primitive's screen-tile rectangle for binning.
 *   cpv_raster      — one CTA per screen tile: walks the tile's primitives in
 *                     API order (cpv_raster_tile), evaluates coverage per pixel
 *                     with the reference's float edge functions, interpolates,
 *                     runs the fragment shader and the per-fragment operations
 *                     against colour/depth/stencil held in registers, and
 *                     writes the tile back once.
 * Parameters are __grid_constant__: device functions read them in place
 * through references, without a per-thread copy.
 */
#ifndef CPV_PIPELINE_CUH
#define CPV_PIPELINE_CUH

extern "C" __global__ void __launch_bounds__(256) cpv_setup_rects(const __grid_constant__ CpvDrawParams P) {
#if CPV_ANY_VS_SAMPLES
    cpv_lut8_init();  /* the vertex shader samples images */
    __syncthreads();
#endif
    const uint64_t g = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    uint2 r = make_uint2(0u, 0u);
    if (g < P.total_prims) {
        CpvTri t;
        cpv_p0::Stage::setup<false>(P, g, t);
        r = cpv_tile_rect(t, P.viewport[2], P.viewport[3]);
        reinterpret_cast<uint2*>(const_cast<uint16_t*>(P.rects))[g] = r;
    }
    /* the union of the draw's rectangles sizes its (tiles x spans) matrix
     * (P.tile_box is the same for every CTA, so all or none call it) */
    if (P.tile_box) cpv_tile_box_add(P.tile_box, r);
}

/* Blend tables (pipelines that blend a per-primitive constant colour): one
 * thread per primitive shades it (vertex shader, flat inputs, fragment
 * shader), then the CTA fills the 4 × 256-byte table of each live primitive
 * of its 256, one destination byte per thread. Primitives whose tile
 * rectangle is empty are skipped (the raster never reads their tables). */
extern "C" __global__ void __launch_bounds__(256) cpv_blend_tables(const __grid_constant__ CpvDrawParams P) {
    __shared__ float colours[256][4];
    __shared__ uint32_t live[256];
    cpv_lut8_init();
    const uint64_t g = static_cast<uint64_t>(blockIdx.x) * 256u + threadIdx.x;
    uint32_t ok = 0u;
    if (cpv_p0::kBlendTable && g < P.total_prims) {
        bool drawn = true;
        if (P.rects) {
            const uint2 r = reinterpret_cast<const uint2*>(P.rects)[g];
            drawn = r.x != r.y;  /* empty rectangles are all-zero */
        }
        if (drawn) {
            CpvTri t;
            cpv_p0::Stage::setup<true>(P, g, t);
            ok = cpv_tri_live(t) ? 1u : 0u;
#pragma unroll
            for (int c = 0; c < 4; c++) colours[threadIdx.x][c] = t.var[0][c];
        }
    }
    live[threadIdx.x] = ok;
    __syncthreads();
    const uint64_t first = static_cast<uint64_t>(blockIdx.x) * 256u;
    for (uint32_t k = 0; k < 256u; k++) {
        if (!live[k]) continue;
        const float colour[4] = {colours[k][0], colours[k][1], colours[k][2], colours[k][3]};
        uint8_t bytes[4];
        cpv_p0::cpv_blend_table_column(colour, P.blend_constants, threadIdx.x, bytes);
        uint8_t* table = P.tables + (first + k) * 1024u;
#pragma unroll
        for (int c = 0; c < 4; c++) table[c * 256 + threadIdx.x] = bytes[c];
    }
}

/* Primitives of one tile of a single draw: every primitive (direct mode), the
 * tile's bin list[begin, end) in API order, or — when the bin list overflowed
 * its capacity — every primitive whose tile rectangle covers the tile. */
struct CpvPlainSource {
    const CpvDrawParams& P;
    uint64_t begin, end;
    bool by_index, scan_rects;
    uint32_t tx, ty;
    float vw, vh;
    uint32_t fb_width, fb_height;

    __device__ __forceinline__ uint64_t count() const { return end > begin ? end - begin : 0; }
    __device__ __forceinline__ void setup(uint64_t i, CpvTri& t) const {
        uint64_t g;
        if (by_index) {
            g = begin + i;
            if (scan_rects) {
                const uint2 r = reinterpret_cast<const uint2*>(P.rects)[g];
                const uint32_t rx0 = r.x & 0xFFFFu, ry0 = r.x >> 16, rx1 = r.y & 0xFFFFu, ry1 = r.y >> 16;
                if (!(tx >= rx0 && tx < rx1 && ty >= ry0 && ty < ry1)) {
                    t.wf.w = __uint_as_float(0u);
                    return;
                }
            }
        } else {
            g = P.bin_list[begin + i];
        }
        cpv_p0::Stage::setup<true>(P, g, t);
    }
    __device__ __forceinline__ bool shade(const CpvTri& t, const float w[3], int32_t x, int32_t y, float* colour, float& mapped,
                                          const CpvPixel* early = nullptr) const {
        return cpv_p0::Stage::shade(P, t, w, x, y, colour, mapped, early);
    }
    __device__ __forceinline__ void rop(const CpvTri& t, const float* colour, float mapped, CpvPixel& s) const {
        cpv_p0::Stage::rop(P.blend_constants, cpv_tri_front(t), colour, mapped, s, cpv_p0::Stage::table(P, t));
    }
    /* A covered fragment of a table-only pipeline: the table lookup is the
     * whole of shade + rop (the colour is constant and nothing discards a
     * live primitive). Returns false when the general path must run. */
    __device__ __forceinline__ bool table_fragment(const CpvTri& t, CpvPixel& s) const {
        if (cpv_p0::kTableOnly) {
            const uint8_t* table = cpv_p0::Stage::table(P, t);
            if (table) {
                cpv_p0::cpv_apply_table(table, s);
                return true;
            }
        }
        return false;
    }
    __device__ __forceinline__ void load_pixel(uint64_t pix, CpvPixel& s) const { cpv_p0::Stage::load_pixel(P.color, P.depth, pix, s, P.color_extra); }
    __device__ __forceinline__ void store_pixel(uint64_t pix, const CpvPixel& s) const {
        cpv_p0::Stage::store_pixel(P.color, P.depth, pix, s, P.color_extra);
    }
};

/* Raster kernel: one CTA per screen tile (blockIdx.x = tile id).
 * direct != 0: the tile walks every primitive of the draw (small draws).
 * Otherwise it walks its bin. Dynamic shared memory: CPV_RASTER_SMEM_BYTES. */
#ifdef CPV_PLAIN_MIN_BLOCKS
/* a register budget for CPV_PLAIN_MIN_BLOCKS resident CTAs per SM */
#define CPV_PLAIN_BOUNDS __launch_bounds__(CPV_RT_THREADS, CPV_PLAIN_MIN_BLOCKS)
#else
#define CPV_PLAIN_BOUNDS __launch_bounds__(CPV_RT_THREADS)
#endif
extern "C" __global__ void CPV_PLAIN_BOUNDS cpv_raster(const __grid_constant__ CpvDrawParams P, uint32_t direct) {
    extern __shared__ float4 cpv_dyn_smem[];
    __shared__ uint32_t warp_sums[CPV_RT_THREADS / 32];
    const uint32_t tile = blockIdx.x;
    const uint32_t tx = tile % P.tiles_x, ty = tile / P.tiles_x;
    uint64_t begin = 0, end = P.total_prims;
    bool scan_rects = false;
    if (!direct) {
        /* tiles outside the union of the draw's rectangles have no primitive */
        const CpvTileBox b = cpv_tile_box(P.tile_box);
        if (tx - b.x0 >= b.w || ty - b.y0 >= b.h) return;
        if (*P.pair_total > P.list_capacity) {
            scan_rects = true;
        } else {
            const uint64_t local = static_cast<uint64_t>(ty - b.y0) * b.w + (tx - b.x0);
            end = P.tile_end[local * P.spans + P.spans - 1u];
            begin = local == 0u ? 0u : P.tile_end[local * P.spans - 1u];
        }
    }
    if (begin >= end) return;
    cpv_lut8_init();
    CpvPlainSource src{P, begin, end, direct != 0 || scan_rects, scan_rects, tx, ty, P.viewport[2], P.viewport[3], P.fb_width, P.fb_height};
    cpv_raster_tile(src, tx, ty, reinterpret_cast<CpvTri*>(cpv_dyn_smem), warp_sums);
}

#endif /* CPV_PIPELINE_CUH */

/* Launch shape of the raster kernel, read by the host at module load
 * (cudaLibraryGetGlobal): dynamic shared memory bytes and threads per CTA. */
extern "C" __device__ const uint32_t cpv_raster_smem_bytes = CPV_RASTER_SMEM_BYTES;
extern "C" __device__ const uint32_t cpv_raster_threads = CPV_RT_THREADS;
