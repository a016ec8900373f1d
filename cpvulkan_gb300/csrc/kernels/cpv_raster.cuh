/*
 * cpv_raster.cuh — the pipeline-independent part of the tile rasteriser,
 * shared by the per-draw module (cpv_pipeline.cuh) and the batched module
 * (cpv_batch.cuh). Compiled by NVRTC after cpv_device.cuh; the module prefix
 * defines CPV_TILE_SHIFT, CPV_SCHEDULE, CPV_RT_WARPS, CPV_BATCH and
 * CPV_NV_MAX (the largest varying count over the module's pipelines).
 *
 * The per-pipeline part (primitive set-up, fragment shading and the
 * per-fragment operations, which depend on the pipeline's shaders and
 * fixed-function state) is cpv_stage.cuh, instantiated once per pipeline in
 * its own namespace. cpv_raster_tile() walks one screen tile's primitives
 * through a Source object that supplies the primitives in API order and
 * routes each to its pipeline's stage functions.
 */
#ifndef CPV_RASTER_CUH
#define CPV_RASTER_CUH

#ifndef CPV_TILE_SHIFT
#define CPV_TILE_SHIFT 4
#endif
#ifndef CPV_SCHEDULE
#define CPV_SCHEDULE 0 /* 0 immediate, 1 deferred, 2 sparse (see cpv_raster_tile) */
#endif
#define CPV_DEFERRED (CPV_SCHEDULE == 1)
#if CPV_DEFERRED && CPV_NUM_CA > 1
#error "the deferred schedule keeps one colour per recorded fragment: modules with several colour attachments use another"
#endif
#define CPV_SPARSE (CPV_SCHEDULE == 2)
#define CPV_WARP_LISTS (CPV_SCHEDULE == 0) /* immediate: each warp walks only the primitives reaching its rows */
#ifndef CPV_SLOT_DEPTH
#define CPV_SLOT_DEPTH 16 /* sparse: fragments a pixel takes per batch before its fallback */
#endif
#ifndef CPV_SMALL_PX
#define CPV_SMALL_PX 64 /* sparse: largest in-tile bounding box listed by the warp-spread tests (C4 raster 21.37 ms at 64, 21.65 at 32, 21.86 at 128) */
#endif
#ifndef CPV_RT_WARPS
#define CPV_RT_WARPS 8
#endif
#ifndef CPV_BATCH
#define CPV_BATCH 128
#endif
#ifndef CPV_ANY_FS_CONSTANT
#define CPV_ANY_FS_CONSTANT 0 /* some pipeline of the module shades once per primitive */
#endif
#define CPV_TILE (1 << CPV_TILE_SHIFT)
#define CPV_RT_THREADS ((CPV_TILE * CPV_TILE) < (32 * CPV_RT_WARPS) ? (CPV_TILE * CPV_TILE) : (32 * CPV_RT_WARPS))
#define CPV_PPT ((CPV_TILE * CPV_TILE) / CPV_RT_THREADS)
/* register budget of the persistent batched raster: 40 resident warps per
 * SM (48 registers a thread at 256 threads a CTA, the five CTAs shared
 * memory allows) */
#ifndef CPV_RT_MIN_BLOCKS
#define CPV_RT_MIN_BLOCKS (1280 / CPV_RT_THREADS)
#endif

#define CPV_ROWS_PER_PASS (CPV_RT_THREADS / CPV_TILE)
#define CPV_WARP_ROWS (32 / CPV_TILE > 0 ? 32 / CPV_TILE : 1) /* tile rows one warp covers per pass */
/* immediate schedule with one pixel a thread: each warp owns an 8 x 4 block
 * of the tile instead of whole rows (a compact block is more often wholly
 * inside or outside a primitive, so fewer visits cover few lanes) */
#define CPV_WARP_BLOCKS (CPV_WARP_LISTS && CPV_PPT == 1 && CPV_TILE >= 8)
#define CPV_BLOCK_W 8
#define CPV_BLOCK_H 4
#ifndef CPV_ANY_LINES
#define CPV_ANY_LINES 0 /* some pipeline of the module draws lines */
#endif
#ifndef CPV_NUM_CA
#define CPV_NUM_CA 1 /* colour attachments of the module's subpass (up to 8; 1 also for a depth-only pass) */
#endif
/* fragment shader outputs: 4 floats per colour attachment */
#define CPV_COLOUR_FLOATS (4 * CPV_NUM_CA)
#ifndef CPV_ANY_VS_SAMPLES
#define CPV_ANY_VS_SAMPLES 1 /* some pipeline's vertex shader samples images */
#endif
#define CPV_NV_ALLOC (CPV_NV_MAX > 0 ? CPV_NV_MAX : 1)
#define CPV_NV_ROOM0 (CPV_ANY_FS_CONSTANT && CPV_NV_ALLOC < 4 ? 4 : CPV_NV_ALLOC)
#define CPV_NV_ROOM (CPV_ANY_LINES && CPV_NV_ROOM0 < 7 ? 7 : CPV_NV_ROOM0)
#define CPV_NV_PAD ((CPV_NV_ROOM + 3) & ~3)
#define CPV_SLOTS 4
#define CPV_NSLOT (CPV_RT_THREADS * CPV_SLOTS)

/* One primitive after set-up, in the reference's terms
 * (CPVulkan/CommandBuffer.Draw.cpp:1510-1594, 874-954). 16-byte aligned
 * groups so that the coverage loop reads them with 128-bit loads.
 *
 * Points and lines reuse the record (Draw.cpp:1315-1508):
 *   point — box is exactly the set of pixels the reference covers and the
 *           edges are zero (every pixel of the box passes); za.x = NDC z,
 *           wf.x = clip w, var[0] = the vertex's outputs;
 *   line  — e[0..2] and za are the four edges of the line's quad, wf.x/y
 *           the two clip w, var[0..1] the vertices' outputs, var[2][0..6] =
 *           p0.x, p0.y, (p1 - p0).x, (p1 - p0).y, |p1 - p0|², z0, z1; the
 *           provoking slot field holds 3 (a line's provoking vertex is its
 *           first). */
struct __align__(16) CpvTri {
    float4 e[3];     /* edge k: start vertex (x, y) and b - a (dx, dy), NDC */
    int4 box;        /* pixel bounding box x0, y0, x1, y1 (end exclusive) */
    float4 za;       /* NDC z of p0..p2 (after the CW swap), |area| */
    float4 wf;       /* clip w of p0..p2, flags (see below) */
    float var[3][CPV_NV_PAD]; /* varyings per vertex; for a pipeline whose fragment
                                 shader is constant per primitive, var[0][0..3]
                                 holds the shaded colour instead */
};

/* Flag word (wf.w bits): 1 live, 2 front facing, bits 2-5 pipeline index in
 * the module, bits 6-7 provoking-vertex slot (3: a line), bits 8-31 draw
 * index in the batch (0 for a per-draw module). */
__device__ __forceinline__ uint32_t cpv_tri_flags(const CpvTri& t) { return __float_as_uint(t.wf.w); }
__device__ __forceinline__ bool cpv_tri_live(const CpvTri& t) { return (cpv_tri_flags(t) & 1u) != 0u; }
__device__ __forceinline__ bool cpv_tri_front(const CpvTri& t) { return (cpv_tri_flags(t) & 2u) != 0u; }
__device__ __forceinline__ uint32_t cpv_tri_pipeline(const CpvTri& t) { return (cpv_tri_flags(t) >> 2) & 15u; }
__device__ __forceinline__ uint32_t cpv_tri_pslot(const CpvTri& t) { return (cpv_tri_flags(t) >> 6) & 3u; }
__device__ __forceinline__ uint32_t cpv_tri_draw(const CpvTri& t) { return cpv_tri_flags(t) >> 8; }
__device__ __forceinline__ void cpv_tri_tag(CpvTri& t, uint32_t pipeline, uint32_t draw) {
    t.wf.w = __uint_as_float((cpv_tri_flags(t) & 0xC3u) | (pipeline << 2) | (draw << 8));
}

/* Pixel centre in NDC (CPVulkan/CommandBuffer.Draw.cpp:1524, 1573-1580):
 * (x / width + halfPixel) * 2 - 1, halfPixel = (1 / width) * 0.5. */
__device__ __forceinline__ float cpv_pixel_ndc(int32_t x, float extent) {
    const float half = __fmul_rn(__fdiv_rn(1.0f, extent), 0.5f);
    return __fsub_rn(__fmul_rn(__fadd_rn(__fdiv_rn(static_cast<float>(x), extent), half), 2.0f), 1.0f);
}

/* Edge functions at a pixel centre (CPVulkan/CommandBuffer.Draw.cpp:882-902):
 * w_k = (p.x - a.x) * (b.y - a.y) - (p.y - a.y) * (b.x - a.x); covered when
 * no w_k is negative (inclusive on every edge). */
__device__ __forceinline__ bool cpv_covers(const CpvTri& t, float xf, float yf, float w[3]) {
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const float4 e = t.e[k];
        const float t0 = __fmul_rn(__fsub_rn(xf, e.x), e.w);
        const float t1 = __fmul_rn(__fsub_rn(yf, e.y), e.z);
        w[k] = __fsub_rn(t0, t1);
    }
#if CPV_ANY_LINES
    /* a line's quad has a fourth edge (CPVulkan/CommandBuffer.Draw.cpp:1437):
     * every edge must be >= 0, which also rejects NaN */
    if (((__float_as_uint(t.wf.w) >> 6) & 3u) == 3u) {
        const float4 e = t.za;
        const float w3 = __fsub_rn(__fmul_rn(__fsub_rn(xf, e.x), e.w), __fmul_rn(__fsub_rn(yf, e.y), e.z));
        return w[0] >= 0.0f && w[1] >= 0.0f && w[2] >= 0.0f && w3 >= 0.0f;
    }
#endif
    return !(w[0] < 0.0f || w[1] < 0.0f || w[2] < 0.0f);
}

/* Tile rectangle of a set-up primitive (empty when culled, off screen, or
 * when a bounding box of at most four pixels covers none of its pixel
 * centres — the raster would find no fragment there either). Packed as
 * x0 | y0 << 16, x1 | y1 << 16 in tile units, end exclusive. */
__device__ __forceinline__ uint2 cpv_tile_rect(const CpvTri& t, float vw, float vh, const float* ndc_x = nullptr, const float* ndc_y = nullptr) {
    uint32_t r[4] = {0, 0, 0, 0};
    if (cpv_tri_live(t)) {
        bool any = true;
        const int4 b = t.box;
        if ((b.z - b.x) * (b.w - b.y) <= 4) {
            /* pixel centres from the tables when given (the box lies inside
             * the attachment), else computed */
            any = false;
            for (int32_t y = b.y; y < b.w; y++) {
                const float yf = ndc_y ? __ldg(ndc_y + y) : cpv_pixel_ndc(y, vh);
                for (int32_t x = b.x; x < b.z; x++) {
                    float w[3];
                    if (cpv_covers(t, ndc_x ? __ldg(ndc_x + x) : cpv_pixel_ndc(x, vw), yf, w)) any = true;
                }
            }
        }
        if (any) {
            r[0] = static_cast<uint32_t>(b.x >> CPV_TILE_SHIFT);
            r[1] = static_cast<uint32_t>(b.y >> CPV_TILE_SHIFT);
            r[2] = static_cast<uint32_t>(((b.z - 1) >> CPV_TILE_SHIFT) + 1);
            r[3] = static_cast<uint32_t>(((b.w - 1) >> CPV_TILE_SHIFT) + 1);
        }
    }
    return make_uint2(r[0] | (r[1] << 16), r[2] | (r[3] << 16));
}

/* Whether primitive t may cover a pixel of the rectangle [rx0, rx1) x
 * [ry0, ry1) (inside its box). Each rounded edge function
 * w = fl(fl(xf - a.x) * dy) - fl(fl(yf - a.y) * dx) is monotonic along a
 * row and along a column (the pixel-centre values are monotonic in the
 * pixel index, and IEEE subtraction and multiplication by a fixed value are
 * monotonic), so its largest value over the rectangle is at the corner
 * picked by the signs of dy and dx; if that value is negative, every pixel
 * of the rectangle fails the edge and none is covered. Exact: it only
 * drops pixels the coverage test rejects. Edges with a non-finite
 * coefficient keep the primitive (NaN counts as covered). col/row hold the
 * tile's pixel-centre NDC values, indexed from (tile_x0, tile_y0). */
__device__ __forceinline__ bool cpv_may_cover(const CpvTri& t, int32_t rx0, int32_t ry0, int32_t rx1, int32_t ry1, const float* col,
                                              const float* row, int32_t tile_x0, int32_t tile_y0) {
    /* the pixel-centre sequences are monotonic (in either direction for a
     * negative extent): their extremes over a range are its ends */
    const float c0 = col[rx0 - tile_x0], c1 = col[rx1 - 1 - tile_x0];
    const float r0 = row[ry0 - tile_y0], r1 = row[ry1 - 1 - tile_y0];
    const float xa = fminf(c0, c1), xb = fmaxf(c0, c1), ya = fminf(r0, r1), yb = fmaxf(r0, r1);
    if (!(fabsf(c0) <= 3.4e38f && fabsf(c1) <= 3.4e38f && fabsf(r0) <= 3.4e38f && fabsf(r1) <= 3.4e38f)) return true;
    bool may = true;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        float4 e;
        if (k < 3) {
            e = t.e[k];
        } else {
#if CPV_ANY_LINES
            if (((__float_as_uint(t.wf.w) >> 6) & 3u) != 3u) break;
            e = t.za; /* a line's fourth edge */
#else
            break;
#endif
        }
        if (!(fabsf(e.x) <= 3.4e38f && fabsf(e.y) <= 3.4e38f && fabsf(e.z) <= 3.4e38f && fabsf(e.w) <= 3.4e38f)) continue;
        const float xf = e.w > 0.0f ? xb : xa;
        const float yf = e.z > 0.0f ? ya : yb;
        const float w = __fsub_rn(__fmul_rn(__fsub_rn(xf, e.x), e.w), __fmul_rn(__fsub_rn(yf, e.y), e.z));
        may = may && !(w < 0.0f);
    }
    return may;
}

/* Whether triangle t covers every pixel of the rectangle [rx0, rx1) x
 * [ry0, ry1): by the monotonicity cpv_may_cover uses, each edge function's
 * smallest value over the rectangle is at the corner picked by the signs of
 * dy and dx, and a pixel whose value is not negative passes that edge.
 * Exact in the other direction: true only when the coverage test passes at
 * every pixel (a NaN corner value, a non-finite coefficient or a line's
 * fourth edge gives false, and the pixels are then tested one by one). */
__device__ __forceinline__ bool cpv_must_cover(const CpvTri& t, int32_t rx0, int32_t ry0, int32_t rx1, int32_t ry1, const float* col,
                                               const float* row, int32_t tile_x0, int32_t tile_y0) {
#if CPV_ANY_LINES
    if (((__float_as_uint(t.wf.w) >> 6) & 3u) == 3u) return false;
#endif
    const float c0 = col[rx0 - tile_x0], c1 = col[rx1 - 1 - tile_x0];
    const float r0 = row[ry0 - tile_y0], r1 = row[ry1 - 1 - tile_y0];
    const float xa = fminf(c0, c1), xb = fmaxf(c0, c1), ya = fminf(r0, r1), yb = fmaxf(r0, r1);
    if (!(fabsf(c0) <= 3.4e38f && fabsf(c1) <= 3.4e38f && fabsf(r0) <= 3.4e38f && fabsf(r1) <= 3.4e38f)) return false;
    bool must = true;
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const float4 e = t.e[k];
        if (!(fabsf(e.x) <= 3.4e38f && fabsf(e.y) <= 3.4e38f && fabsf(e.z) <= 3.4e38f && fabsf(e.w) <= 3.4e38f)) return false;
        const float xf = e.w > 0.0f ? xa : xb;
        const float yf = e.z > 0.0f ? yb : ya;
        const float w = __fsub_rn(__fmul_rn(__fsub_rn(xf, e.x), e.w), __fmul_rn(__fsub_rn(yf, e.y), e.z));
        must = must && w >= 0.0f;
    }
    return must;
}

/* ---- per-fragment operation helpers (LLVMRuntime/PipelineCompiler.cpp:1020-1429) ---- */

__device__ __forceinline__ bool cpv_fcompare(float a, float b, uint32_t op) {
    switch (op) {
    case 0: return false;
    case 1: return a < b;
    case 2: return a == b;
    case 3: return a <= b;
    case 4: return a > b;
    case 5: return (a < b) || (a > b);
    case 6: return a >= b;
    default: return true;
    }
}

__device__ __forceinline__ bool cpv_icompare(uint32_t a, uint32_t b, uint32_t op) {
    switch (op) {
    case 0: return false;
    case 1: return a < b;
    case 2: return a == b;
    case 3: return a <= b;
    case 4: return a > b;
    case 5: return a != b;
    case 6: return a >= b;
    default: return true;
    }
}

/* Stencil ops; increment/decrement-and-clamp saturate as signed i8
 * (LLVMRuntime/PipelineCompiler.cpp:1382-1413). */
__device__ __forceinline__ uint32_t cpv_stencil_op(uint32_t op, uint32_t cur, uint32_t ref) {
    const int32_t sc = static_cast<int8_t>(cur);
    switch (op) {
    case 0: return cur;
    case 1: return 0u;
    case 2: return ref & 0xFFu;
    case 3: return static_cast<uint32_t>(static_cast<uint8_t>(sc == 127 ? 127 : sc + 1));
    case 4: return static_cast<uint32_t>(static_cast<uint8_t>(sc == -128 ? -128 : sc - 1));
    case 5: return (~cur) & 0xFFu;
    case 6: return (cur + 1u) & 0xFFu;
    case 7: return (cur - 1u) & 0xFFu;
    default: return cur;
    }
}

/* ApplyBlendFactor / ApplyBlend (CPVulkan/CommandBuffer.Draw.cpp:956-1262). */
__device__ __forceinline__ void cpv_blend_factor(const float s[4], const float d[4], const float c[4], uint32_t cf, uint32_t af, float o[4]) {
#pragma unroll
    for (int i = 0; i < 4; i++) o[i] = 0.0f;
    switch (cf) {
    case 0: break;
    case 1: for (int i = 0; i < 4; i++) o[i] = 1.0f; break;
    case 2: for (int i = 0; i < 4; i++) o[i] = s[i]; break;
    case 3: for (int i = 0; i < 4; i++) o[i] = __fsub_rn(1.0f, s[i]); break;
    case 4: for (int i = 0; i < 4; i++) o[i] = d[i]; break;
    case 5: for (int i = 0; i < 4; i++) o[i] = __fsub_rn(1.0f, d[i]); break;
    case 6: for (int i = 0; i < 4; i++) o[i] = s[3]; break;
    case 7: { const float v = __fsub_rn(1.0f, s[3]); for (int i = 0; i < 4; i++) o[i] = v; break; }
    case 8: for (int i = 0; i < 4; i++) o[i] = d[3]; break;
    case 9: { const float v = __fsub_rn(1.0f, d[3]); for (int i = 0; i < 4; i++) o[i] = v; break; }
    case 10: for (int i = 0; i < 4; i++) o[i] = c[i]; break;
    case 11: for (int i = 0; i < 4; i++) o[i] = __fsub_rn(1.0f, c[i]); break;
    case 12: for (int i = 0; i < 4; i++) o[i] = c[3]; break;
    case 13: { const float v = __fsub_rn(1.0f, c[3]); for (int i = 0; i < 4; i++) o[i] = v; break; }
    case 14: { const float f = cpv_std_min(s[3], __fsub_rn(1.0f, d[3])); o[0] = f; o[1] = f; o[2] = f; o[3] = 1.0f; break; }
    default: break;
    }
    if (cf != af) {
        switch (af) {
        case 0: o[3] = 0.0f; break;
        case 1: case 14: o[3] = 1.0f; break;
        case 2: case 6: o[3] = s[3]; break;
        case 3: case 7: o[3] = __fsub_rn(1.0f, s[3]); break;
        case 4: case 8: o[3] = d[3]; break;
        case 5: case 9: o[3] = __fsub_rn(1.0f, d[3]); break;
        case 10: case 12: o[3] = c[3]; break;
        case 11: case 13: o[3] = __fsub_rn(1.0f, c[3]); break;
        default: break;
        }
    }
}

__device__ __forceinline__ float cpv_blend_op(float s, float sf, float d, float df, uint32_t op) {
    const float a = __fmul_rn(s, sf);
    const float b = __fmul_rn(d, df);
    switch (op) {
    case 0: return __fadd_rn(a, b);
    case 1: return __fsub_rn(a, b);
    case 2: return __fsub_rn(b, a);
    case 3: return cpv_std_min(s, d);
    case 4: return cpv_std_max(s, d);
    default: return 0.0f;
    }
}

/* Register-resident attachment state of one pixel. */
#ifndef CPV_COLOUR_WORDS
#define CPV_COLOUR_WORDS 1 /* 32-bit words of the module's widest first-attachment texel (8- and 16-byte formats: 2, 4) */
#endif
struct CpvPixel {
    uint32_t colour[CPV_COLOUR_WORDS];
    float depth;        /* decoded depth (D16: u16 / 65535) */
    uint32_t depth_raw; /* stored bits */
    uint32_t stencil;
#if CPV_NUM_CA > 1
    uint32_t extra[CPV_NUM_CA - 1]; /* texels of colour attachments 1 .. */
#endif
};

/* Block-wide exclusive sum over CPV_RT_THREADS threads. */
__device__ __forceinline__ uint32_t cpv_block_scan(uint32_t v, uint32_t& total, uint32_t* warp_sums) {
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    uint32_t incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= static_cast<uint32_t>(o)) incl += t;
    }
    if (lane == 31u) warp_sums[warp] = incl;
    __syncthreads();
    uint32_t base = 0, sum = 0;
    for (uint32_t k = 0; k < CPV_RT_THREADS / 32; k++) {
        const uint32_t s = warp_sums[k];
        if (k < warp) base += s;
        sum += s;
    }
    total = sum;
    return base + incl - v;
}

/* Sparse schedule: class of a primitive in the tile — 0 dead or outside the
 * tile, 1 small (its bounding box covers at most CPV_SMALL_PX pixels of the
 * tile), 2 large. */
__device__ __forceinline__ uint32_t cpv_tile_class(const CpvTri& t, int32_t tile_x0, int32_t tile_y0) {
    if (!cpv_tri_live(t)) return 0u;
    const int4 box = t.box;
    const int32_t x0 = max(box.x, tile_x0), x1 = min(box.z, tile_x0 + CPV_TILE);
    const int32_t y0 = max(box.y, tile_y0), y1 = min(box.w, tile_y0 + CPV_TILE);
    if (x1 <= x0 || y1 <= y0) return 0u;
    return (x1 - x0) * (y1 - y0) > CPV_SMALL_PX ? 2u : 1u;
}

/* Sparse schedule: the small primitives j0 .. j0 + 31 of a batch (one per
 * lane of the calling warp) test the pixels of their boxes inside the tile
 * and append each covered pixel's primitive to its list — as one list of
 * (primitive, pixel) tests spread evenly over the warp's lanes, so that a
 * lane's large box does not hold the other 31 lanes. Test i of the warp
 * belongs to the first lane whose inclusive box-size sum exceeds i (a
 * binary search over the lanes' sums) and is pixel i - (that lane's
 * exclusive sum) of its box, row-major. A pixel's list is applied in batch
 * order whatever the order of its appends. */
__device__ __forceinline__ void cpv_list_small_warp(const CpvTri* tris, uint32_t j0, uint32_t n, int32_t tile_x0, int32_t tile_y0,
                                                    const float* col_ndc, const float* row_ndc, uint32_t* list_count, uint8_t* list_j) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t j = j0 + lane;
    uint32_t size = 0u, geo = 0u, magic = 0u;
    if (j < n && cpv_tile_class(tris[j], tile_x0, tile_y0) == 1u) {
        const int4 box = tris[j].box;
        const int32_t x0 = max(box.x, tile_x0), x1 = min(box.z, tile_x0 + CPV_TILE);
        const int32_t y0 = max(box.y, tile_y0), y1 = min(box.w, tile_y0 + CPV_TILE);
        const uint32_t bw = static_cast<uint32_t>(x1 - x0);
        size = bw * static_cast<uint32_t>(y1 - y0);
        geo = static_cast<uint32_t>(x0 - tile_x0) | (static_cast<uint32_t>(y0 - tile_y0) << 8) | (bw << 16);
        /* row = (k * magic) >> 16 = floor(k / bw) for every k < 1024 and bw
         * <= 32: magic = ceil(2^16 / bw) exceeds 2^16 / bw by less than 1,
         * so the product exceeds k * 2^16 / bw by less than k < 2^16 / 64,
         * under the 2^16 / bw gap from a non-integer k / bw to the next
         * integer */
        magic = (65536u + bw - 1u) / bw;
    }
    uint32_t incl = size;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= static_cast<uint32_t>(o)) incl += t;
    }
    const uint32_t total = __shfl_sync(0xFFFFFFFFu, incl, 31);
    for (uint32_t base = 0; base < total; base += 32u) {
        const uint32_t i = base + lane;
        /* owner: the number of lanes whose inclusive sum is <= i */
        uint32_t owner = 0u;
#pragma unroll
        for (uint32_t s = 16u; s > 0u; s >>= 1) {
            const uint32_t v = __shfl_sync(0xFFFFFFFFu, incl, owner + s - 1u);
            if (v <= i) owner += s;
        }
        owner &= 31u;
        const uint32_t o_incl = __shfl_sync(0xFFFFFFFFu, incl, owner);
        const uint32_t o_size = __shfl_sync(0xFFFFFFFFu, size, owner);
        const uint32_t o_geo = __shfl_sync(0xFFFFFFFFu, geo, owner);
        const uint32_t o_magic = __shfl_sync(0xFFFFFFFFu, magic, owner);
        if (i >= total) continue;
        const uint32_t k = i - (o_incl - o_size);
        const uint32_t row = (k * o_magic) >> 16;
        const uint32_t col = k - row * (o_geo >> 16);
        const uint32_t lx = (o_geo & 0xFFu) + col, ly = ((o_geo >> 8) & 0xFFu) + row;
        float w[3];
        if (!cpv_covers(tris[j0 + owner], col_ndc[lx], row_ndc[ly], w)) continue;
        const uint32_t p = ly * CPV_TILE + lx;
        const uint32_t s = atomicAdd(&list_count[p], 1u);
        if (s < CPV_SLOT_DEPTH) list_j[p * CPV_SLOT_DEPTH + s] = static_cast<uint8_t>(j0 + owner);
    }
}

/* Dynamic shared memory of the raster kernels: CPV_BATCH primitives, then
 * the schedule's buffers (deferred: fragment slots; sparse: per-pixel
 * primitive lists, pixel-centre tables, the large-primitive list). */
#define CPV_TILE_PX (CPV_TILE * CPV_TILE)
#define CPV_SPARSE_BYTES (4u * CPV_TILE_PX + CPV_TILE_PX * CPV_SLOT_DEPTH + CPV_BATCH)
#define CPV_RASTER_SMEM_BYTES \
    (CPV_BATCH * sizeof(CpvTri) + (CPV_DEFERRED ? CPV_NSLOT * (4u + 20u + 2u) : 0u) + (CPV_SPARSE ? CPV_SPARSE_BYTES : 0u))

/* One screen tile (tx, ty): loads the tile's attachment texels into
 * registers, walks the tile's primitives from `src` in API order in batches
 * of CPV_BATCH (set-up into shared memory, then coverage, shading and the
 * per-fragment operations of each pixel in primitive order) and stores the
 * texels back once.
 *
 * Source supplies:
 *   uint64_t count()                         primitives of this tile
 *   void setup(uint64_t i, CpvTri& t)        set up the i-th (or mark it dead)
 *   bool shade(const CpvTri&, const float w[3], int x, int y, float colour[CPV_COLOUR_FLOATS], float& mapped, const CpvPixel* early)
 *                                            (true: discarded, or failed the early depth
 *                                            test against *early when given)
 *   void rop(const CpvTri&, const float colour[CPV_COLOUR_FLOATS], float mapped, CpvPixel&)
 *   bool table_fragment(const CpvTri&, CpvPixel&)  a covered fragment applied by a
 *                                            blend-table lookup alone (false: use shade + rop)
 *   void load_pixel(uint64_t pix, CpvPixel&) / store_pixel(uint64_t pix, const CpvPixel&)
 *   float vw, vh                             viewport extent (pixel centres)
 *   uint32_t fb_width, fb_height
 *
 * Three fragment schedules (CPV_SCHEDULE):
 *   0 immediate — each pixel's thread tests every primitive of the batch and
 *               shades its covered fragments as it finds them (cheap
 *               shaders, large primitives);
 *   1 deferred — per batch of primitives, threads first record up to
 *               CPV_SLOTS covered fragments each, the CTA then shades all
 *               recorded fragments densely (full warps, whatever the
 *               coverage pattern), and finally every pixel's thread applies
 *               its own fragments' per-fragment operations in primitive
 *               order (expensive shaders);
 *   2 sparse  — coverage is found per primitive instead of per pixel: a
 *               primitive whose bounding box covers at most CPV_SMALL_PX
 *               pixels of the tile is rasterised by one thread, which tests
 *               only those pixels; larger ones are tested by the pixels'
 *               threads. Either appends the primitive's batch index to each
 *               covered pixel's list (up to CPV_SLOT_DEPTH per batch); each
 *               pixel's thread then shades and applies its list in
 *               primitive order (tiny primitives, heavy overdraw). A pixel
 *               whose list overflowed walks the whole batch instead.
 * All apply each pixel's fragments in API primitive order, as the
 * reference's serial loop does. */
template <class Source>
__device__ __forceinline__ void cpv_raster_tile(Source& src, uint32_t tx, uint32_t ty, CpvTri* tris, uint32_t* warp_sums) {
    const uint64_t end = src.count();
    if (end == 0) return;
    /* pixel-centre NDC of the tile's columns and rows (the values of
     * cpv_pixel_ndc); the barrier keeps the previous tile's readers of a
     * persistent CTA ahead of the rewrite */
    __shared__ float col_ndc[CPV_TILE], row_ndc[CPV_TILE];
    const int32_t tile_x0 = static_cast<int32_t>(tx * CPV_TILE), tile_y0 = static_cast<int32_t>(ty * CPV_TILE);
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < CPV_TILE; i += CPV_RT_THREADS) {
        col_ndc[i] = cpv_pixel_ndc(tile_x0 + static_cast<int32_t>(i), src.vw);
        row_ndc[i] = cpv_pixel_ndc(tile_y0 + static_cast<int32_t>(i), src.vh);
    }
    int32_t px[CPV_PPT], py[CPV_PPT];
    float xf[CPV_PPT], yf[CPV_PPT];
    bool inside[CPV_PPT];
    CpvPixel st[CPV_PPT];
#pragma unroll
    for (int k = 0; k < CPV_PPT; k++) {
#if CPV_WARP_BLOCKS
        /* warp w: block (w % blocks a row, w / blocks a row); lane: x = lane % 8, y = lane / 8 */
        const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
        px[k] = static_cast<int32_t>(tx * CPV_TILE + (warp % (CPV_TILE / CPV_BLOCK_W)) * CPV_BLOCK_W + (lane % CPV_BLOCK_W));
        py[k] = static_cast<int32_t>(ty * CPV_TILE + (warp / (CPV_TILE / CPV_BLOCK_W)) * CPV_BLOCK_H + (lane / CPV_BLOCK_W));
#else
        px[k] = static_cast<int32_t>(tx * CPV_TILE + (threadIdx.x % CPV_TILE));
        py[k] = static_cast<int32_t>(ty * CPV_TILE + (threadIdx.x / CPV_TILE) + k * CPV_ROWS_PER_PASS);
#endif
        inside[k] = px[k] < static_cast<int32_t>(src.fb_width) && py[k] < static_cast<int32_t>(src.fb_height);
        xf[k] = cpv_pixel_ndc(px[k], src.vw);
        yf[k] = cpv_pixel_ndc(py[k], src.vh);
        if (inside[k]) src.load_pixel(static_cast<uint64_t>(py[k]) * src.fb_width + px[k], st[k]);
    }

#if CPV_DEFERRED
    uint8_t* slot_base = reinterpret_cast<uint8_t*>(tris + CPV_BATCH);
    uint32_t* slot_jk = reinterpret_cast<uint32_t*>(slot_base);          /* batch index | pixel k << 8 | discard << 31 */
    float* slot_f = reinterpret_cast<float*>(slot_jk + CPV_NSLOT);       /* 5 floats per slot: w0 w1 w2 → rgba + mapped */
    uint16_t* dense = reinterpret_cast<uint16_t*>(slot_f + 5 * CPV_NSLOT);
#endif
#if CPV_SPARSE
    static_assert(CPV_BATCH <= 256, "batch indices are stored in bytes");
    uint32_t* list_count = reinterpret_cast<uint32_t*>(tris + CPV_BATCH);  /* per tile pixel: fragments listed this batch */
    uint8_t* list_j = reinterpret_cast<uint8_t*>(list_count + CPV_TILE_PX);  /* per tile pixel: CPV_SLOT_DEPTH batch indices */
    uint8_t* large = list_j + CPV_TILE_PX * CPV_SLOT_DEPTH;                  /* batch indices of large primitives, in order */
    for (uint32_t i = threadIdx.x; i < CPV_TILE_PX; i += CPV_RT_THREADS) list_count[i] = 0u;
    uint32_t lp[CPV_PPT]; /* this thread's pixels, as tile pixel indices */
#pragma unroll
    for (int k = 0; k < CPV_PPT; k++) lp[k] = static_cast<uint32_t>((py[k] - tile_y0) * CPV_TILE + (px[k] - tile_x0));
#endif

#if CPV_WARP_LISTS
    /* immediate schedule: per warp, the batch's primitives reaching its rows
     * (batch index; bit 15: the primitive covers the warp's whole block) */
    __shared__ uint16_t warp_list[(CPV_RT_THREADS / 32) * CPV_BATCH];
#if CPV_WARP_BLOCKS
    const int32_t warp_x0 = static_cast<int32_t>(tx * CPV_TILE + ((threadIdx.x >> 5) % (CPV_TILE / CPV_BLOCK_W)) * CPV_BLOCK_W);
    const int32_t warp_y0 = static_cast<int32_t>(ty * CPV_TILE + ((threadIdx.x >> 5) / (CPV_TILE / CPV_BLOCK_W)) * CPV_BLOCK_H);
#else
    const int32_t warp_y0 = static_cast<int32_t>(ty * CPV_TILE + ((threadIdx.x & ~31u) / CPV_TILE));
#endif
#endif

    for (uint64_t base = 0; base < end; base += CPV_BATCH) {
        const uint32_t n = static_cast<uint32_t>((end - base) < CPV_BATCH ? (end - base) : CPV_BATCH);
        __syncthreads();
        /* a tile of 8 × 8 has fewer threads than CPV_BATCH: stride the set-up;
         * a primitive reaching beyond the tile that covers no pixel of it
         * (its box ∩ the tile) is dropped for this tile; one inside the tile
         * is left to the pixel tests, which is cheaper for small primitives */
        for (uint32_t i = threadIdx.x; i < n; i += CPV_RT_THREADS) {
            CpvTri& t = tris[i];
            src.setup(base + i, t);
            const int4 b = t.box;
            if (cpv_tri_live(t) && (b.x < tile_x0 || b.y < tile_y0 || b.z > tile_x0 + CPV_TILE || b.w > tile_y0 + CPV_TILE)) {
                const int32_t rx0 = max(b.x, tile_x0), ry0 = max(b.y, tile_y0);
                const int32_t rx1 = min(b.z, tile_x0 + CPV_TILE), ry1 = min(b.w, tile_y0 + CPV_TILE);
                /* worth a test when the primitive spans much of the tile */
                if (rx1 <= rx0 || ry1 <= ry0 ||
                    ((rx1 - rx0) * (ry1 - ry0) >= CPV_TILE_PX / 8 && !cpv_may_cover(t, rx0, ry0, rx1, ry1, col_ndc, row_ndc, tile_x0, tile_y0)))
                    t.wf.w = __uint_as_float(__float_as_uint(t.wf.w) & ~1u);
            }
        }
        __syncthreads();
#if CPV_SPARSE
        /* 1. classify: large primitives (box covering more than CPV_SMALL_PX
         *    pixels of the tile) are collected in batch order, in rounds of
         *    one primitive per thread */
        uint32_t nlarge = 0u;
        for (uint32_t round = 0; round < n; round += CPV_RT_THREADS) {
            const uint32_t j = round + threadIdx.x;
            const uint32_t is_large = j < n && cpv_tile_class(tris[j], tile_x0, tile_y0) == 2u ? 1u : 0u;
            uint32_t round_large;
            const uint32_t lpos = cpv_block_scan(is_large, round_large, warp_sums);
            if (is_large) large[nlarge + lpos] = static_cast<uint8_t>(j);
            nlarge += round_large;
            __syncthreads();
        }
        /* mostly large primitives: this batch runs the immediate schedule */
        const bool immediate_batch = nlarge * 4u >= 3u * n;
        if (!immediate_batch) {
            /* 2. small primitives: each warp lists the pixels its 32 cover */
            for (uint32_t j0 = threadIdx.x & ~31u; j0 < n; j0 += CPV_RT_THREADS)
                cpv_list_small_warp(tris, j0, n, tile_x0, tile_y0, col_ndc, row_ndc, list_count, list_j);
            /* 3. large primitives, in order: every pixel's thread tests its pixels */
            for (uint32_t m = 0; m < nlarge; m++) {
                const uint32_t j = large[m];
                const CpvTri& t = tris[j];
                const int4 box = t.box;
#pragma unroll
                for (int k = 0; k < CPV_PPT; k++) {
                    if (!inside[k]) continue;
                    if (px[k] < box.x || px[k] >= box.z || py[k] < box.y || py[k] >= box.w) continue;
                    float w[3];
                    if (!cpv_covers(t, xf[k], yf[k], w)) continue;
                    const uint32_t s = atomicAdd(&list_count[lp[k]], 1u);
                    if (s < CPV_SLOT_DEPTH) list_j[lp[k] * CPV_SLOT_DEPTH + s] = static_cast<uint8_t>(j);
                }
            }
            __syncthreads();
            /* 4. each pixel shades and applies its list in batch (API) order */
#pragma unroll
            for (int k = 0; k < CPV_PPT; k++) {
                const uint32_t c = list_count[lp[k]];
                if (c == 0u) continue;
                if (c <= CPV_SLOT_DEPTH) {
                    const uint8_t* lj = list_j + lp[k] * CPV_SLOT_DEPTH;
                    int32_t last = -1;
                    for (uint32_t it = 0; it < c; it++) {
                        /* next batch index after `last` (a primitive covers a pixel once) */
                        int32_t j = 0x7FFFFFFF;
                        for (uint32_t e = 0; e < c; e++) {
                            const int32_t v = lj[e];
                            if (v > last && v < j) j = v;
                        }
                        last = j;
                        const CpvTri& t = tris[j];
                        float w[3], colour[CPV_COLOUR_FLOATS], mapped;
                        cpv_covers(t, xf[k], yf[k], w);
                        if (src.shade(t, w, px[k], py[k], colour, mapped, &st[k])) continue;
                        src.rop(t, colour, mapped, st[k]);
                    }
                } else {
                    /* list overflow: walk the whole batch for this pixel */
                    for (uint32_t j = 0; j < n; j++) {
                        const CpvTri& t = tris[j];
                        if (!cpv_tri_live(t)) continue;
                        const int4 box = t.box;
                        if (px[k] < box.x || px[k] >= box.z || py[k] < box.y || py[k] >= box.w) continue;
                        float w[3], colour[CPV_COLOUR_FLOATS], mapped;
                        if (!cpv_covers(t, xf[k], yf[k], w)) continue;
                        if (src.shade(t, w, px[k], py[k], colour, mapped, &st[k])) continue;
                        src.rop(t, colour, mapped, st[k]);
                    }
                }
                list_count[lp[k]] = 0u;
            }
        }
#else
        const bool immediate_batch = true;
        (void)immediate_batch;
#endif
#if !CPV_DEFERRED
        /* immediate: every pixel's thread tests each primitive in order,
         * shading and applying what it covers. Each warp first lists, in
         * order, the batch's live primitives whose box reaches its rows, and
         * walks only those. */
        if (immediate_batch) {
#if CPV_WARP_LISTS
            const uint32_t lane = threadIdx.x & 31u;
            uint16_t* mine = warp_list + (threadIdx.x >> 5) * CPV_BATCH;
            uint32_t count = 0;
            for (uint32_t b = 0; b < n; b += 32u) {
                const uint32_t j = b + lane;
                bool hit = false;
                uint32_t full = 0u;
                if (j < n && cpv_tri_live(tris[j])) {
                    const CpvTri& t = tris[j];
                    const int4 box = t.box;
#if CPV_WARP_BLOCKS
                    /* the warp's block, within the box */
                    const int32_t rx0 = max(box.x, warp_x0), rx1 = min(box.z, warp_x0 + CPV_BLOCK_W);
                    const int32_t ry0 = max(box.y, warp_y0), ry1 = min(box.w, warp_y0 + CPV_BLOCK_H);
                    hit = rx1 > rx0 && ry1 > ry0 && cpv_may_cover(t, rx0, ry0, rx1, ry1, col_ndc, row_ndc, tile_x0, tile_y0);
                    /* a block inside the box (so inside the attachment) and
                     * inside every edge: its pixels skip the box and edge tests */
                    if (hit && rx0 == warp_x0 && rx1 == warp_x0 + CPV_BLOCK_W && ry0 == warp_y0 && ry1 == warp_y0 + CPV_BLOCK_H &&
                        cpv_must_cover(t, rx0, ry0, rx1, ry1, col_ndc, row_ndc, tile_x0, tile_y0))
                        full = 0x8000u;
#else
                    const int32_t rx0 = max(box.x, tile_x0), rx1 = min(box.z, tile_x0 + CPV_TILE);
#pragma unroll
                    for (int k = 0; k < CPV_PPT; k++) {
                        /* the warp's rows of pass k, within the box */
                        const int32_t ry0 = max(box.y, warp_y0 + k * CPV_ROWS_PER_PASS);
                        const int32_t ry1 = min(box.w, warp_y0 + k * CPV_ROWS_PER_PASS + CPV_WARP_ROWS);
                        hit = hit || (ry1 > ry0 && cpv_may_cover(t, rx0, ry0, rx1, ry1, col_ndc, row_ndc, tile_x0, tile_y0));
                    }
#endif
                }
                const uint32_t ballot = __ballot_sync(0xFFFFFFFFu, hit);
                if (hit) mine[count + __popc(ballot & ((1u << lane) - 1u))] = static_cast<uint16_t>(j | full);
                count += __popc(ballot);
            }
            __syncwarp();
#else
            const uint32_t count = n;
#endif
            for (uint32_t m = 0; m < count; m++) {
#if CPV_WARP_LISTS
                const uint32_t entry = mine[m];
                const uint32_t j = entry & 0x7FFFu;
#if CPV_WARP_BLOCKS
                if (entry & 0x8000u) {
                    /* the whole block is covered (one pixel a thread, all inside) */
                    const CpvTri& t = tris[j];
                    if (src.table_fragment(t, st[0])) continue;
                    float w[3], colour[CPV_COLOUR_FLOATS], mapped;
                    cpv_covers(t, xf[0], yf[0], w);
                    if (src.shade(t, w, px[0], py[0], colour, mapped, &st[0])) continue;
                    src.rop(t, colour, mapped, st[0]);
                    continue;
                }
#endif
#else
                const uint32_t j = m;
                if (!cpv_tri_live(tris[j])) continue;
#endif
                const CpvTri& t = tris[j];
                const int4 box = t.box;
#pragma unroll
                for (int k = 0; k < CPV_PPT; k++) {
                    if (!inside[k]) continue;
                    if (px[k] < box.x || px[k] >= box.z || py[k] < box.y || py[k] >= box.w) continue;
                    float w[3];
                    if (!cpv_covers(t, xf[k], yf[k], w)) continue;
                    if (src.table_fragment(t, st[k])) continue;
                    float colour[CPV_COLOUR_FLOATS], mapped;
                    if (src.shade(t, w, px[k], py[k], colour, mapped, &st[k])) continue;
                    src.rop(t, colour, mapped, st[k]);
                }
            }
        }
#else
        const uint32_t limit = n * CPV_PPT;
        uint32_t cursor = 0;
        while (__syncthreads_or(cursor < limit)) {
            /* 1. coverage: record up to CPV_SLOTS fragments, in primitive order */
            uint32_t cnt = 0;
            while (cursor < limit && cnt < CPV_SLOTS) {
                const uint32_t j = cursor / CPV_PPT, k = cursor - j * CPV_PPT;
                cursor++;
                const CpvTri& t = tris[j];
                if (!cpv_tri_live(t)) continue;
                int32_t pxk = px[0], pyk = py[0];
                float xfk = xf[0], yfk = yf[0];
                bool ink = inside[0];
#pragma unroll
                for (int kk = 1; kk < CPV_PPT; kk++)
                    if (k == static_cast<uint32_t>(kk)) { pxk = px[kk]; pyk = py[kk]; xfk = xf[kk]; yfk = yf[kk]; ink = inside[kk]; }
                const int4 box = t.box;
                if (!ink || pxk < box.x || pxk >= box.z || pyk < box.y || pyk >= box.w) continue;
                float w[3];
                if (!cpv_covers(t, xfk, yfk, w)) continue;
                const uint32_t s = threadIdx.x * CPV_SLOTS + cnt;
                slot_jk[s] = j | (k << 8);
                slot_f[5 * s + 0] = w[0];
                slot_f[5 * s + 1] = w[1];
                slot_f[5 * s + 2] = w[2];
                cnt++;
            }
            /* 2. dense shading of every recorded fragment */
            uint32_t total;
            const uint32_t pos = cpv_block_scan(cnt, total, warp_sums);
            for (uint32_t i = 0; i < cnt; i++) dense[pos + i] = static_cast<uint16_t>(threadIdx.x * CPV_SLOTS + i);
            __syncthreads();
            for (uint32_t d = threadIdx.x; d < total; d += CPV_RT_THREADS) {
                const uint32_t s = dense[d];
                const uint32_t owner = s / CPV_SLOTS;
                const uint32_t jk = slot_jk[s];
                const uint32_t j = jk & 0xFFu, k = (jk >> 8) & 0xFFu;
                const int32_t x = static_cast<int32_t>(tx * CPV_TILE + (owner % CPV_TILE));
                const int32_t y = static_cast<int32_t>(ty * CPV_TILE + (owner / CPV_TILE) + k * CPV_ROWS_PER_PASS);
                const float w[3] = {slot_f[5 * s + 0], slot_f[5 * s + 1], slot_f[5 * s + 2]};
                float colour[CPV_COLOUR_FLOATS], mapped;
                const bool discard = src.shade(tris[j], w, x, y, colour, mapped);
                slot_f[5 * s + 0] = colour[0];
                slot_f[5 * s + 1] = colour[1];
                slot_f[5 * s + 2] = colour[2];
                slot_f[5 * s + 3] = colour[3];
                slot_f[5 * s + 4] = mapped;
                if (discard) slot_jk[s] = jk | 0x80000000u;
            }
            __syncthreads();
            /* 3. per-fragment operations of this thread's pixels, in order */
            for (uint32_t i = 0; i < cnt; i++) {
                const uint32_t s = threadIdx.x * CPV_SLOTS + i;
                const uint32_t jk = slot_jk[s];
                if (jk >> 31) continue;
                const uint32_t j = jk & 0xFFu, k = (jk >> 8) & 0xFFu;
                const float colour[4] = {slot_f[5 * s + 0], slot_f[5 * s + 1], slot_f[5 * s + 2], slot_f[5 * s + 3]};
#pragma unroll
                for (int kk = 0; kk < CPV_PPT; kk++)
                    if (k == static_cast<uint32_t>(kk)) src.rop(tris[j], colour, slot_f[5 * s + 4], st[kk]);
            }
        }
#endif
    }
#pragma unroll
    for (int k = 0; k < CPV_PPT; k++) {
        if (inside[k]) src.store_pixel(static_cast<uint64_t>(py[k]) * src.fb_width + px[k], st[k]);
    }
}

#endif /* CPV_RASTER_CUH */
