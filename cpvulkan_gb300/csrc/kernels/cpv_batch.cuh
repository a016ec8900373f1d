/*
 * cpv_batch.cuh — batched kernels: all draws of one render pass in one
 * pass per stage, for a module holding every pipeline those draws bind
 * (namespaces cpv_p0 … cpv_p<n-1>, routed by cpv_dispatch).
 *
 * The draws' primitives share one index space: draw d owns the set-up
 * blocks [draw_block[d], draw_block[d+1]), CPV_BATCH_BLOCK primitives each,
 * so a primitive index g orders the batch in API order (draw, then primitive).
 *
 *   cpv_batch_setup  — one thread per primitive of every draw: vertex
 *                      positions, bounding box, cull and the tile rectangle;
 *                      per block, the number of (primitive, tile) pairs.
 *   (runtime)        — scan of the block pair counts, pair emission in
 *                      primitive order, stable radix sort of the pairs by
 *                      tile, per-tile ranges (cpv_bin.cuh).
 *   cpv_batch_raster — persistent CTAs take tiles from a work counter and
 *                      walk each tile's primitives (all draws, API order)
 *                      with cpv_raster_tile, switching pipeline per
 *                      primitive; each tile's texels stay in registers from
 *                      the first primitive of the first draw to the last of
 *                      the last draw and are written back once.
 *
 * The per-primitive and per-fragment arithmetic is the per-draw module's
 * (the same cpv_stage.cuh functions): a batched image equals the per-draw
 * image bit for bit.
 */
#ifndef CPV_BATCH_CUH
#define CPV_BATCH_CUH

/* Floats of vertex outputs per vertex slot (a multiple of 4, so that every
 * slot's outputs start on a 16-byte boundary). */
#define CPV_VS_STRIDE (((CPV_NV_MAX) + 3) & ~3)

/* Vertex stage: one thread per vertex slot of every draw that has slots —
 * vertex id vs_lo + v of local instance i, shaded once per frame for the
 * set-up and raster kernels that follow (cpv_setup reads the slot instead of
 * shading the vertex again for each triangle and tile that uses it). */
extern "C" __global__ void __launch_bounds__(CPV_BATCH_BLOCK) cpv_batch_vs(const __grid_constant__ CpvBatchParams B) {
#if CPV_ANY_VS_SAMPLES
    cpv_lut8_init();  /* the vertex shader samples images */
    __syncthreads();
#endif
    const uint32_t block = blockIdx.x;
    const uint32_t d = B.vs_block_draw[block];
    const CpvDrawParams& P = B.draws[d];
    /* the host gives a draw slots only when vs_count * instances < 2^32 */
    const uint32_t local = (block - B.vs_draw_block[d]) * CPV_BATCH_BLOCK + threadIdx.x;
    const uint32_t count = P.vs_count;
    const uint32_t instances = P.instance_count > 1u ? P.instance_count : 1u;
    if (count == 0u || local >= count * instances) return;
    const uint32_t inst = local / count;
    const uint32_t v = local - inst * count;
    cpv_dispatch(B.draw_pipeline[d], [&](auto S) { decltype(S)::vertex(P, P.vs_lo + v, P.first_instance + inst, local); });
}

/* register budget of the set-up: eight resident CTAs of 256 threads (32
 * registers a thread). Its dependent loads (draw table, indices, vertex
 * slots) leave it latency-bound: C4 set-up 11.8 ms at eight, 12.0 at six,
 * 13.4 at five */
#ifndef CPV_SETUP_MIN_BLOCKS
#define CPV_SETUP_MIN_BLOCKS 8
#endif
extern "C" __global__ void __launch_bounds__(CPV_BATCH_BLOCK, CPV_SETUP_MIN_BLOCKS) cpv_batch_setup(const __grid_constant__ CpvBatchParams B) {
    __shared__ uint32_t warp_pairs[CPV_BATCH_BLOCK / 32];
#if CPV_ANY_VS_SAMPLES
    cpv_lut8_init();  /* the vertex shader samples images */
    __syncthreads();
#endif
    const uint32_t block = blockIdx.x;
    const uint32_t d = B.block_draw[block];
    const CpvDrawParams& P = B.draws[d];
    const uint64_t local = static_cast<uint64_t>(block - B.draw_block[d]) * CPV_BATCH_BLOCK + threadIdx.x;
    uint2 rect = make_uint2(0u, 0u);
    if (local < P.total_prims) {
        CpvTri t;
        cpv_dispatch(B.draw_pipeline[d], [&](auto S) { decltype(S)::template setup<false>(P, local, t); });
        rect = cpv_tile_rect(t, B.vw, B.vh, B.ndc_x, B.ndc_y);
    }
    const uint64_t g = static_cast<uint64_t>(block) * CPV_BATCH_BLOCK + threadIdx.x;
    uint32_t pairs = ((rect.y & 0xFFFFu) - (rect.x & 0xFFFFu)) * ((rect.y >> 16) - (rect.x >> 16));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) pairs += __shfl_xor_sync(0xFFFFFFFFu, pairs, o);
    if ((threadIdx.x & 31u) == 0u) warp_pairs[threadIdx.x >> 5] = pairs;
    __syncthreads();
    uint32_t s = 0;
    for (uint32_t w = 0; w < CPV_BATCH_BLOCK / 32; w++) s += warp_pairs[w];
    /* a block without pairs (all culled or off screen) leaves its
     * rectangles unwritten: the emit kernel and the raster's rectangle scan
     * skip such blocks by their pair count */
    if (s != 0u) B.rects[g] = rect;
    if (threadIdx.x == 0) B.block_pairs[block] = s;
}

/* Primitives of one tile of the batch: the tile's range of the sorted pair
 * list, or — when the pairs overflowed their capacity — every primitive of
 * the batch whose tile rectangle covers the tile. Each primitive is routed
 * to its draw's parameters and its pipeline's stage functions. */
struct CpvBatchSource {
    const CpvBatchParams& B;
    uint64_t begin, end;
    bool scan_rects;
    uint32_t tx, ty;
    float vw, vh;
    uint32_t fb_width, fb_height;

    __device__ __forceinline__ uint64_t count() const { return end > begin ? end - begin : 0; }
    __device__ __forceinline__ void setup(uint64_t i, CpvTri& t) const {
        uint64_t g;
        if (scan_rects) {
            g = begin + i;
            if (B.block_pairs[g / CPV_BATCH_BLOCK] == 0u) {  /* its rectangles were not written */
                t.wf.w = __uint_as_float(0u);
                return;
            }
            const uint2 r = B.rects[g];
            const uint32_t rx0 = r.x & 0xFFFFu, ry0 = r.x >> 16, rx1 = r.y & 0xFFFFu, ry1 = r.y >> 16;
            if (!(tx >= rx0 && tx < rx1 && ty >= ry0 && ty < ry1)) {
                t.wf.w = __uint_as_float(0u);
                return;
            }
        } else {
            g = B.sorted_prims[begin + i];
        }
        const uint32_t block = static_cast<uint32_t>(g / CPV_BATCH_BLOCK);
        const uint32_t d = B.block_draw[block];
        const uint64_t local = g - static_cast<uint64_t>(B.draw_block[d]) * CPV_BATCH_BLOCK;
        const uint32_t pid = B.draw_pipeline[d];
        cpv_dispatch(pid, [&](auto S) { decltype(S)::template setup<true>(B.draws[d], local, t); });
        cpv_tri_tag(t, pid, d);
    }
    __device__ __forceinline__ bool shade(const CpvTri& t, const float w[3], int32_t x, int32_t y, float* colour, float& mapped,
                                          const CpvPixel* early = nullptr) const {
        bool discard = false;
        const CpvDrawParams& P = B.draws[cpv_tri_draw(t)];
        cpv_dispatch(cpv_tri_pipeline(t), [&](auto S) { discard = decltype(S)::shade(P, t, w, x, y, colour, mapped, early); });
        return discard;
    }
    __device__ __forceinline__ void rop(const CpvTri& t, const float* colour, float mapped, CpvPixel& s) const {
        const float* bc = B.draws[cpv_tri_draw(t)].blend_constants;
        const bool front = cpv_tri_front(t);
        cpv_dispatch(cpv_tri_pipeline(t), [&](auto S) { decltype(S)::rop(bc, front, colour, mapped, s); });
    }
    /* batched passes build no blend tables */
    __device__ __forceinline__ bool table_fragment(const CpvTri&, CpvPixel&) const { return false; }
    __device__ __forceinline__ void load_pixel(uint64_t pix, CpvPixel& s) const { cpv_p0::Stage::load_pixel(B.color, B.depth, pix, s, B.color_extra); }
    __device__ __forceinline__ void store_pixel(uint64_t pix, const CpvPixel& s) const {
        cpv_p0::Stage::store_pixel(B.color, B.depth, pix, s, B.color_extra);
    }
};

/* Persistent raster: CTAs take tiles from B.tile_counter (reset to zero
 * before the launch) until every tile is done. */
extern "C" __global__ void __launch_bounds__(CPV_RT_THREADS, CPV_RT_MIN_BLOCKS) cpv_batch_raster(const __grid_constant__ CpvBatchParams B) {
    extern __shared__ float4 cpv_dyn_smem[];
    __shared__ uint32_t warp_sums[CPV_RT_THREADS / 32];
    __shared__ uint32_t next_tile;
    cpv_lut8_init();
    const uint32_t tiles = B.tiles_x * B.tiles_y;
    const bool overflow = *B.pair_total > B.pair_capacity;
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) next_tile = atomicAdd(B.tile_counter, 1u);
        __syncthreads();
        const uint32_t tile = next_tile;
        if (tile >= tiles) break;
        const uint32_t tx = tile % B.tiles_x, ty = tile / B.tiles_x;
        uint64_t begin = 0, end = static_cast<uint64_t>(B.total_blocks) * CPV_BATCH_BLOCK;
        if (!overflow) {
            begin = B.tile_begin[tile];
            end = B.tile_end[tile];
        }
        CpvBatchSource src{B, begin, end, overflow, tx, ty, B.vw, B.vh, B.fb_width, B.fb_height};
        cpv_raster_tile(src, tx, ty, reinterpret_cast<CpvTri*>(cpv_dyn_smem), warp_sums);
    }
}

#endif /* CPV_BATCH_CUH */

extern "C" __device__ const uint32_t cpv_raster_smem_bytes = CPV_RASTER_SMEM_BYTES;
extern "C" __device__ const uint32_t cpv_raster_threads = CPV_RT_THREADS;
extern "C" __device__ const uint32_t cpv_vs_stride = CPV_VS_STRIDE;
