/*
 * cpv_pipeline.cuh — the kernels of one graphics pipeline. Compiled by NVRTC
 * at vkCreateGraphicsPipelines after a prefix that defines the pipeline's
 * fixed-function state (CPV_* macros) and its translated shaders:
 *
 *   __device__ void cpv_vs_run(const CpvDrawParams&, uint32_t vertex_index,
 *                              uint32_t instance_index, float pos[4], float var[CPV_NV]);
 *   __device__ bool cpv_fs_run(const CpvDrawParams&, const float in[CPV_NV],
 *                              const float frag_coord[4], bool front, float colour[4]);
 *   __device__ int  cpv_interp(int component);  // 0 perspective, 1 linear, 2 flat
 *
 * Kernels:
 *   cpv_setup_rects — one thread per primitive: runs the vertex shader for the
 *                     primitive's three vertices (positions only), the
 *                     reference's bounding box and cull test, and writes the
 *                     primitive's screen-tile rectangle for binning.
 *   cpv_raster      — one CTA per screen tile: walks the tile's primitives in
 *                     API order, evaluates coverage per pixel with the
 *                     reference's float edge functions, interpolates, runs the
 *                     fragment shader and the per-fragment operations against
 *                     colour/depth/stencil held in registers, and writes the
 *                     tile back once.
 *
 * Two fragment schedules, chosen per pipeline (CPV_DEFERRED):
 *   immediate — each pixel's thread shades its covered fragments as it finds
 *               them (cheap shaders, large primitives);
 *   deferred  — per batch of primitives, threads first record up to
 *               CPV_SLOTS covered fragments each, the CTA then shades all
 *               recorded fragments densely (full warps, whatever the
 *               coverage pattern), and finally every pixel's thread applies
 *               its own fragments' per-fragment operations in primitive
 *               order. Used when the fragment shader is expensive and
 *               primitives are small (sampling, many varyings).
 * Both apply each pixel's fragments in API primitive order, as the
 * reference's serial loop does.
 *
 * Vertex shading is recomputed where it is needed (set-up and raster) instead
 * of being stored: a vertex shader is a pure function of its inputs, and the
 * reference itself shades every assembled vertex (one per index), so the
 * recomputation is arithmetic the reference also performs and costs no HBM
 * traffic for a vertex-output buffer.
 */
#ifndef CPV_PIPELINE_CUH
#define CPV_PIPELINE_CUH

#ifndef CPV_TILE_SHIFT
#define CPV_TILE_SHIFT 4
#endif
#ifndef CPV_DEFERRED
#define CPV_DEFERRED 0
#endif
#define CPV_TILE (1 << CPV_TILE_SHIFT)
#define CPV_RT_THREADS ((CPV_TILE * CPV_TILE) < 256 ? (CPV_TILE * CPV_TILE) : 256)
#define CPV_PPT ((CPV_TILE * CPV_TILE) / CPV_RT_THREADS)
#define CPV_ROWS_PER_PASS (CPV_RT_THREADS / CPV_TILE)
#define CPV_BATCH 128
#define CPV_NV_ALLOC (CPV_NV > 0 ? CPV_NV : 1)
#define CPV_NV_PAD ((CPV_NV_ALLOC + 3) & ~3)
#define CPV_SLOTS 4
#define CPV_NSLOT (CPV_RT_THREADS * CPV_SLOTS)

/* One primitive after set-up, in the reference's terms
 * (CPVulkan/CommandBuffer.Draw.cpp:1510-1594, 874-954). 16-byte aligned
 * groups so that the coverage loop reads them with 128-bit loads. */
struct __align__(16) CpvTri {
    float4 e[3];     /* edge k: start vertex (x, y) and b - a (dx, dy), NDC */
    int4 box;        /* pixel bounding box x0, y0, x1, y1 (end exclusive) */
    float4 za;       /* NDC z of p0..p2 (after the CW swap), |area| */
    float4 wf;       /* clip w of p0..p2, flags (bits: 1 live, 2 front, pslot << 8) */
    float var[3][CPV_NV_PAD];
};

__device__ __forceinline__ uint32_t cpv_tri_flags(const CpvTri& t) { return __float_as_uint(t.wf.w); }

/* Primitive set-up: vertex shading of the three vertices, perspective divide,
 * screen bounding box, area, facing and cull. */
template <bool WITH_VARYINGS>
__device__ __forceinline__ void cpv_setup(const CpvDrawParams& P, uint64_t g, CpvTri& t) {
    const uint32_t ppi = P.prims_per_instance;
    const uint32_t g32 = static_cast<uint32_t>(g);  /* draws hold < 2^32 primitives */
    const uint32_t inst = P.instance_count > 1u ? g32 / ppi : 0u;
    const uint32_t instance = P.first_instance + inst;
    const uint32_t p = g32 - inst * ppi;
    uint32_t raw[3], provoking;
    cpv_prim_vertices(CPV_TOPOLOGY, p, raw, provoking);
#if CPV_FRONT_CW
    { const uint32_t tmp = raw[0]; raw[0] = raw[2]; raw[2] = tmp; }
#endif
    const uint32_t pslot = raw[0] == provoking ? 0u : (raw[1] == provoking ? 1u : 2u);
    float Pn[3][4];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        float pos[4];
        float var[CPV_NV_ALLOC];
        cpv_vs_run(P, cpv_vertex_id(P, raw[k]), instance, pos, var);
        const float w = pos[3];
        Pn[k][0] = __fdiv_rn(pos[0], w);
        Pn[k][1] = __fdiv_rn(pos[1], w);
        Pn[k][2] = __fdiv_rn(pos[2], w);
        Pn[k][3] = w;
        if (WITH_VARYINGS) {
#pragma unroll
            for (int c = 0; c < CPV_NV; c++) t.var[k][c] = var[c];
        }
    }
    const float vw = P.viewport[2], vh = P.viewport[3];
    int32_t sx[3], sy[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        sx[k] = cpv_f2i(__fmul_rn(__fmul_rn(__fadd_rn(Pn[k][0], 1.0f), 0.5f), vw));
        sy[k] = cpv_f2i(__fmul_rn(__fmul_rn(__fadd_rn(Pn[k][1], 1.0f), 0.5f), vh));
    }
    const int64_t minx = min(sx[0], min(sx[1], sx[2]));
    const int64_t miny = min(sy[0], min(sy[1], sy[2]));
    const int64_t maxx = max(sx[0], max(sx[1], sx[2]));
    const int64_t maxy = max(sy[0], max(sy[1], sy[2]));
    int64_t x0 = minx > 0 ? minx : 0, y0 = miny > 0 ? miny : 0;
    int64_t x1 = maxx + 1, y1 = maxy + 1;
    const int64_t iw = cpv_f2i(vw), ih = cpv_f2i(vh);
    x1 = x1 < iw ? x1 : iw;
    y1 = y1 < ih ? y1 : ih;
    x1 = x1 < static_cast<int64_t>(P.fb_width) ? x1 : static_cast<int64_t>(P.fb_width);
    y1 = y1 < static_cast<int64_t>(P.fb_height) ? y1 : static_cast<int64_t>(P.fb_height);
    int4 box;
    box.x = static_cast<int32_t>(x0);
    box.y = static_cast<int32_t>(y0);
    box.z = static_cast<int32_t>(x1 > x0 ? x1 : x0);
    box.w = static_cast<int32_t>(y1 > y0 ? y1 : y0);
    t.box = box;

    float area = cpv_edge(Pn[0][0], Pn[0][1], Pn[1][0], Pn[1][1], Pn[2][0], Pn[2][1]);
    /* Edges (a → b): front (area >= 0) w0 = E(p1,p2), w1 = E(p2,p0), w2 = E(p0,p1);
     * back: w0 = E(p2,p1), w1 = E(p0,p2), w2 = E(p1,p0) (Draw.cpp:882-898).
     * Selected with constant indices so the vertices stay in registers. */
    const bool front = !(area < 0.0f);
    if (!front) area = -area;
    const int fa[3] = {1, 2, 0}, fb[3] = {2, 0, 1};
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const float ax = front ? Pn[fa[k]][0] : Pn[fb[k]][0];
        const float ay = front ? Pn[fa[k]][1] : Pn[fb[k]][1];
        const float bx = front ? Pn[fb[k]][0] : Pn[fa[k]][0];
        const float by = front ? Pn[fb[k]][1] : Pn[fa[k]][1];
        t.e[k] = make_float4(ax, ay, __fsub_rn(bx, ax), __fsub_rn(by, ay));
    }
    t.za = make_float4(Pn[0][2], Pn[1][2], Pn[2][2], area);
    bool live = box.z > box.x && box.w > box.y;
    if ((CPV_CULL_MODE & 2) && !front) live = false;
    if ((CPV_CULL_MODE & 1) && front) live = false;
    const uint32_t flags = (live ? 1u : 0u) | (front ? 2u : 0u) | (pslot << 8);
    t.wf = make_float4(Pn[0][3], Pn[1][3], Pn[2][3], __uint_as_float(flags));
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
    return !(w[0] < 0.0f || w[1] < 0.0f || w[2] < 0.0f);
}

/* Set-up kernel: tile rectangle per primitive (empty when culled, off
 * screen, or when a bounding box of at most four pixels covers none of its
 * pixel centres — the raster would find no fragment there either). */
extern "C" __global__ void __launch_bounds__(256) cpv_setup_rects(CpvDrawParams P) {
    cpv_lut8_init();
    __syncthreads();
    const uint64_t g = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (g >= P.total_prims) return;
    CpvTri t;
    cpv_setup<false>(P, g, t);
    uint32_t r[4] = {0, 0, 0, 0};
    if (cpv_tri_flags(t) & 1u) {
        bool any = true;
        const int4 b = t.box;
        if ((b.z - b.x) * (b.w - b.y) <= 4) {
            any = false;
            const float vw = P.viewport[2], vh = P.viewport[3];
            for (int32_t y = b.y; y < b.w; y++) {
                const float yf = cpv_pixel_ndc(y, vh);
                for (int32_t x = b.x; x < b.z; x++) {
                    float w[3];
                    if (cpv_covers(t, cpv_pixel_ndc(x, vw), yf, w)) any = true;
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
    uint2 packed;
    packed.x = r[0] | (r[1] << 16);
    packed.y = r[2] | (r[3] << 16);
    reinterpret_cast<uint2*>(const_cast<uint16_t*>(P.rects))[g] = packed;
}

/* ---- per-fragment operations (LLVMRuntime/PipelineCompiler.cpp:1020-1429) ---- */

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

__device__ __forceinline__ void cpv_blend(const float s[4], const float d[4], const float c[4], float out[4]) {
    float sf[4], df[4];
    cpv_blend_factor(s, d, c, CPV_SRC_COLOR, CPV_SRC_ALPHA, sf);
    cpv_blend_factor(s, d, c, CPV_DST_COLOR, CPV_DST_ALPHA, df);
#pragma unroll
    for (int i = 0; i < 4; i++) out[i] = cpv_blend_op(s[i], sf[i], d[i], df[i], CPV_COLOR_OP);
    if (CPV_COLOR_OP != CPV_ALPHA_OP) out[3] = cpv_blend_op(s[3], sf[3], d[3], df[3], CPV_ALPHA_OP);
}

/* Byte offset of channel i in the colour attachment texel
 * (CPVulkanBase/Formats.cpp:248,255). */
__device__ __forceinline__ int cpv_channel_shift(int i) {
#if CPV_COLOR_FORMAT == 44
    return i == 0 ? 16 : (i == 1 ? 8 : (i == 2 ? 0 : 24));
#else
    return 8 * i;
#endif
}

/* Register-resident attachment state of one pixel. */
struct CpvPixel {
    uint32_t colour;
    float depth;        /* decoded depth (D16: u16 / 65535) */
    uint32_t depth_raw; /* stored bits */
    uint32_t stencil;
};

__device__ __forceinline__ void cpv_load_pixel(const CpvDrawParams& P, uint64_t pix, CpvPixel& s) {
    s.colour = reinterpret_cast<const uint32_t*>(P.color)[pix];
#if CPV_DEPTH_FORMAT == 124
    s.depth_raw = reinterpret_cast<const uint16_t*>(P.depth)[pix];
    s.depth = cpv_decode_unorm16(s.depth_raw);
    s.stencil = 0u;
#elif CPV_DEPTH_FORMAT == 126
    s.depth_raw = reinterpret_cast<const uint32_t*>(P.depth)[pix];
    s.depth = __uint_as_float(s.depth_raw);
    s.stencil = 0u;
#elif CPV_DEPTH_FORMAT == 130
    const uint2 v = reinterpret_cast<const uint2*>(P.depth)[pix];
    s.depth_raw = v.x;
    s.depth = __uint_as_float(v.x);
    s.stencil = v.y & 0xFFu;
#else
    s.depth_raw = 0u;
    s.depth = 0.0f;
    s.stencil = 0u;
#endif
}

__device__ __forceinline__ void cpv_store_pixel(const CpvDrawParams& P, uint64_t pix, const CpvPixel& s) {
    reinterpret_cast<uint32_t*>(P.color)[pix] = s.colour;
#if CPV_DEPTH_FORMAT == 124
    reinterpret_cast<uint16_t*>(P.depth)[pix] = static_cast<uint16_t>(s.depth_raw);
#elif CPV_DEPTH_FORMAT == 126
    reinterpret_cast<uint32_t*>(P.depth)[pix] = s.depth_raw;
#elif CPV_DEPTH_FORMAT == 130
    uint2* p = reinterpret_cast<uint2*>(P.depth) + pix;
    uint2 v = *p;
    v.x = s.depth_raw;
    v.y = (v.y & ~0xFFu) | (s.stencil & 0xFFu);
    *p = v;
#endif
}

__device__ __forceinline__ void cpv_write_depth(CpvPixel& s, float mapped) {
#if CPV_DEPTH_FORMAT == 124
    s.depth_raw = cpv_encode_unorm(mapped, 65535.0f);
    s.depth = cpv_decode_unorm16(s.depth_raw);
#else
    s.depth_raw = __float_as_uint(mapped);
    s.depth = mapped;
#endif
}

/* Shading of one covered pixel: barycentrics (w_k / area), screen-linear
 * depth, varyings (perspective Σ w·v/p ÷ Σ w/p, linear Σ w·v, or flat from
 * the provoking vertex; CPVulkan/CommandBuffer.Draw.cpp:816-954), viewport
 * depth mapping (:1300-1313) and the fragment shader. Returns true when the
 * shader discards. */
__device__ __forceinline__ bool cpv_shade(const CpvDrawParams& P, const CpvTri& t, const float wr[3], int32_t x, int32_t y, float colour[4],
                                          float& mapped) {
    const float area = t.za.w;
    float w[3];
    w[0] = __fdiv_rn(wr[0], area);
    w[1] = __fdiv_rn(wr[1], area);
    w[2] = __fdiv_rn(wr[2], area);
    const float depth = __fadd_rn(__fadd_rn(__fmul_rn(t.za.x, w[0]), __fmul_rn(t.za.y, w[1])), __fmul_rn(t.za.z, w[2]));
    const float pw[3] = {t.wf.x, t.wf.y, t.wf.z};
    const uint32_t pslot = cpv_tri_flags(t) >> 8;
    float in[CPV_NV_ALLOC];
#pragma unroll
    for (int c = 0; c < CPV_NV; c++) {
        const int kind = cpv_interp(c);
        if (kind == 2) {
            in[c] = t.var[pslot][c];
        } else if (kind == 1) {
            float r = 0.0f;
#pragma unroll
            for (int k = 0; k < 3; k++) r = __fadd_rn(r, __fmul_rn(w[k], t.var[k][c]));
            in[c] = r;
        } else {
            float num = 0.0f, den = 0.0f;
#pragma unroll
            for (int k = 0; k < 3; k++) {
                num = __fadd_rn(num, __fdiv_rn(__fmul_rn(w[k], t.var[k][c]), pw[k]));
                den = __fadd_rn(den, __fdiv_rn(w[k], pw[k]));
            }
            in[c] = __fdiv_rn(num, den);
        }
    }
    const float min_d = P.viewport[4], max_d = P.viewport[5];
    mapped = __fadd_rn(__fmul_rn(__fsub_rn(max_d, min_d), depth), min_d);
    float frag_coord[4];
#if CPV_ORIGIN_UPPER
    frag_coord[0] = static_cast<float>(x);
#else
    frag_coord[0] = __fsub_rn(__fsub_rn(P.viewport[2], static_cast<float>(x)), 1.0f);
#endif
    frag_coord[1] = static_cast<float>(y);
    frag_coord[2] = depth;
    frag_coord[3] = 1.0f;
    const bool front = (cpv_tri_flags(t) & 2u) != 0u;
    return cpv_fs_run(P, in, frag_coord, front, colour);
}

/* Depth bounds are rejected at pipeline creation; order as the reference's
 * fragment wrapper: current values → stencil test → depth test → depth /
 * stencil write → colour write (blend, write mask, encode). */
__device__ __forceinline__ void cpv_rop(const CpvDrawParams& P, bool front, const float colour[4], float mapped, CpvPixel& s) {
    const bool has_depth = CPV_DEPTH_FORMAT != 0;
    const bool stencil_on = CPV_STENCIL_TEST && CPV_DEPTH_FORMAT == 130;
    const float current_depth = (CPV_DEPTH_TEST && has_depth) ? s.depth : 0.0f;
    const uint32_t current_stencil = stencil_on ? s.stencil : 0u;
    bool stencil_result = true;
    uint32_t ref = 0u;
    if (stencil_on) {
        ref = (front ? CPV_ST_F_REF : CPV_ST_B_REF) & 0xFFu;
        const uint32_t mask = (front ? CPV_ST_F_CMASK : CPV_ST_B_CMASK) & 0xFFu;
        stencil_result = cpv_icompare(ref & mask, current_stencil & mask, front ? CPV_ST_F_OP : CPV_ST_B_OP);
    }
    const bool depth_result = (CPV_DEPTH_TEST && has_depth) ? cpv_fcompare(mapped, current_depth, CPV_DEPTH_OP) : true;
    const bool attempt_depth_write = CPV_DEPTH_TEST && CPV_DEPTH_WRITE && has_depth;
    if (stencil_on) {
        const uint32_t fail = cpv_stencil_op(front ? CPV_ST_F_FAIL : CPV_ST_B_FAIL, current_stencil, ref);
        const uint32_t dfail = cpv_stencil_op(front ? CPV_ST_F_DFAIL : CPV_ST_B_DFAIL, current_stencil, ref);
        const uint32_t pass = cpv_stencil_op(front ? CPV_ST_F_PASS : CPV_ST_B_PASS, current_stencil, ref);
        uint32_t value = stencil_result ? (depth_result ? pass : dfail) : fail;
        const uint32_t wmask = (front ? CPV_ST_F_WMASK : CPV_ST_B_WMASK) & 0xFFu;
        value = ((value & wmask) | (current_stencil & ~wmask)) & 0xFFu;
        if (depth_result && attempt_depth_write) cpv_write_depth(s, mapped);
        s.stencil = value;
    } else if (attempt_depth_write && depth_result) {
        cpv_write_depth(s, mapped);
    }
    if (stencil_result && depth_result) {
        float out[4];
#if CPV_BLEND
        float dst[4];
#pragma unroll
        for (int i = 0; i < 4; i++) dst[i] = CPV_DECODE8((s.colour >> cpv_channel_shift(i)) & 0xFFu);
        cpv_blend(colour, dst, P.blend_constants, out);
#else
#pragma unroll
        for (int i = 0; i < 4; i++) out[i] = colour[i];
#endif
        uint32_t packed = 0u;
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const uint32_t byte = ((CPV_WRITE_MASK >> i) & 1u) ? cpv_encode_unorm(out[i], 255.0f) : ((s.colour >> cpv_channel_shift(i)) & 0xFFu);
            packed |= byte << cpv_channel_shift(i);
        }
        s.colour = packed;
    }
}

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

/* Raster kernel: one CTA per screen tile (blockIdx.x = tile id).
 * direct != 0: the tile walks every primitive of the draw (small draws).
 * Otherwise it walks its bin: bin_list[start, end) in API order, or — when
 * the bin list overflowed its capacity — every primitive whose tile
 * rectangle overlaps the tile. Dynamic shared memory: CPV_BATCH primitives,
 * then (deferred schedule) the fragment slots. */
extern "C" __global__ void __launch_bounds__(CPV_RT_THREADS) cpv_raster(CpvDrawParams P, uint32_t direct) {
    extern __shared__ float4 cpv_dyn_smem[];
    CpvTri* tris = reinterpret_cast<CpvTri*>(cpv_dyn_smem);
    __shared__ uint32_t warp_sums[CPV_RT_THREADS / 32];
    const uint32_t tile = blockIdx.x;
    const uint32_t tx = tile % P.tiles_x, ty = tile / P.tiles_x;
    uint64_t begin = 0, end = P.total_prims;
    bool scan_rects = false;
    if (!direct) {
        if (*P.pair_total > P.list_capacity) {
            scan_rects = true;
        } else {
            end = P.tile_end[static_cast<uint64_t>(tile) * P.spans + P.spans - 1u];
            begin = tile == 0u ? 0u : P.tile_end[static_cast<uint64_t>(tile) * P.spans - 1u];
        }
    }
    if (begin >= end) return;
    cpv_lut8_init();

    const float vw = P.viewport[2], vh = P.viewport[3];
    int32_t px[CPV_PPT], py[CPV_PPT];
    float xf[CPV_PPT], yf[CPV_PPT];
    bool inside[CPV_PPT];
    CpvPixel st[CPV_PPT];
#pragma unroll
    for (int k = 0; k < CPV_PPT; k++) {
        px[k] = static_cast<int32_t>(tx * CPV_TILE + (threadIdx.x % CPV_TILE));
        py[k] = static_cast<int32_t>(ty * CPV_TILE + (threadIdx.x / CPV_TILE) + k * CPV_ROWS_PER_PASS);
        inside[k] = px[k] < static_cast<int32_t>(P.fb_width) && py[k] < static_cast<int32_t>(P.fb_height);
        xf[k] = cpv_pixel_ndc(px[k], vw);
        yf[k] = cpv_pixel_ndc(py[k], vh);
        if (inside[k]) cpv_load_pixel(P, static_cast<uint64_t>(py[k]) * P.fb_width + px[k], st[k]);
    }

#if CPV_DEFERRED
    uint8_t* slot_base = reinterpret_cast<uint8_t*>(tris + CPV_BATCH);
    uint32_t* slot_jk = reinterpret_cast<uint32_t*>(slot_base);          /* batch index | pixel k << 8 | discard << 31 */
    float* slot_f = reinterpret_cast<float*>(slot_jk + CPV_NSLOT);       /* 5 floats per slot: w0 w1 w2 → rgba + mapped */
    uint16_t* dense = reinterpret_cast<uint16_t*>(slot_f + 5 * CPV_NSLOT);
#endif

    for (uint64_t base = begin; base < end; base += CPV_BATCH) {
        const uint32_t n = static_cast<uint32_t>((end - base) < CPV_BATCH ? (end - base) : CPV_BATCH);
        __syncthreads();
        /* a tile of 8 × 8 has fewer threads than CPV_BATCH: stride the set-up */
        for (uint32_t i = threadIdx.x; i < n; i += CPV_RT_THREADS) {
            CpvTri& t = tris[i];
            uint64_t g;
            bool skip = false;
            if (direct || scan_rects) {
                g = base + i;
                if (scan_rects) {
                    const uint2 r = reinterpret_cast<const uint2*>(P.rects)[g];
                    const uint32_t rx0 = r.x & 0xFFFFu, ry0 = r.x >> 16, rx1 = r.y & 0xFFFFu, ry1 = r.y >> 16;
                    skip = !(tx >= rx0 && tx < rx1 && ty >= ry0 && ty < ry1);
                }
            } else {
                g = P.bin_list[base + i];
            }
            if (skip) t.wf.w = __uint_as_float(0u);
            else cpv_setup<true>(P, g, t);
        }
        __syncthreads();
#if !CPV_DEFERRED
        for (uint32_t j = 0; j < n; j++) {
            const CpvTri& t = tris[j];
            const uint32_t flags = cpv_tri_flags(t);
            if (!(flags & 1u)) continue;
            const int4 box = t.box;
#pragma unroll
            for (int k = 0; k < CPV_PPT; k++) {
                if (!inside[k]) continue;
                if (px[k] < box.x || px[k] >= box.z || py[k] < box.y || py[k] >= box.w) continue;
                float w[3];
                if (!cpv_covers(t, xf[k], yf[k], w)) continue;
                float colour[4], mapped;
                if (cpv_shade(P, t, w, px[k], py[k], colour, mapped)) continue;
                cpv_rop(P, (flags & 2u) != 0u, colour, mapped, st[k]);
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
                if (!(cpv_tri_flags(t) & 1u)) continue;
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
                float colour[4], mapped;
                const bool discard = cpv_shade(P, tris[j], w, x, y, colour, mapped);
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
                const bool front = (cpv_tri_flags(tris[j]) & 2u) != 0u;
#pragma unroll
                for (int kk = 0; kk < CPV_PPT; kk++)
                    if (k == static_cast<uint32_t>(kk)) cpv_rop(P, front, colour, slot_f[5 * s + 4], st[kk]);
            }
        }
#endif
    }
#pragma unroll
    for (int k = 0; k < CPV_PPT; k++) {
        if (inside[k]) cpv_store_pixel(P, static_cast<uint64_t>(py[k]) * P.fb_width + px[k], st[k]);
    }
}

#endif /* CPV_PIPELINE_CUH */

/* Dynamic shared memory the raster kernel needs, read by the host at module
 * load (cudaLibraryGetGlobal) to size the launch. */
extern "C" __device__ const uint32_t cpv_raster_smem_bytes =
    CPV_BATCH * sizeof(CpvTri) + (CPV_DEFERRED ? CPV_NSLOT * (4u + 20u + 2u) : 0u);
