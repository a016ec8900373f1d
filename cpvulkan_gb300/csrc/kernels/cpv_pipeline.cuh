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
#define CPV_TILE (1 << CPV_TILE_SHIFT)
#define CPV_RT_THREADS ((CPV_TILE * CPV_TILE) < 256 ? (CPV_TILE * CPV_TILE) : 256)
#define CPV_PPT ((CPV_TILE * CPV_TILE) / CPV_RT_THREADS)
#define CPV_ROWS_PER_PASS (CPV_RT_THREADS / CPV_TILE)
#define CPV_BATCH 128
#define CPV_NV_ALLOC (CPV_NV > 0 ? CPV_NV : 1)

/* One primitive after set-up, in the reference's terms
 * (CPVulkan/CommandBuffer.Draw.cpp:1510-1594, 874-954). */
struct CpvTri {
    float ax[3], ay[3];   /* start vertex of edge k (NDC) */
    float dx[3], dy[3];   /* b - a of edge k */
    float z[3], w[3];     /* NDC z and clip w of p0..p2 (after the CW swap) */
    float area;           /* |EdgeFunction(p0, p1, p2)| */
    int32_t x0, y0, x1, y1; /* pixel bounding box, end exclusive */
    uint32_t flags;       /* 1 live, 2 front facing */
    uint32_t pslot;       /* which of p0..p2 is the provoking vertex */
    float var[3][CPV_NV_ALLOC];
};

/* Primitive set-up: vertex shading of the three vertices, perspective divide,
 * screen bounding box, area, facing and cull. */
template <bool WITH_VARYINGS>
__device__ __forceinline__ void cpv_setup(const CpvDrawParams& P, uint64_t g, CpvTri& t) {
    const uint32_t ppi = P.prims_per_instance;
    const uint32_t instance = P.first_instance + static_cast<uint32_t>(g / ppi);
    const uint32_t p = static_cast<uint32_t>(g % ppi);
    uint32_t raw[3], provoking;
    cpv_prim_vertices(CPV_TOPOLOGY, p, raw, provoking);
#if CPV_FRONT_CW
    { const uint32_t tmp = raw[0]; raw[0] = raw[2]; raw[2] = tmp; }
#endif
    t.pslot = raw[0] == provoking ? 0u : (raw[1] == provoking ? 1u : 2u);
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
    t.x0 = static_cast<int32_t>(x0);
    t.y0 = static_cast<int32_t>(y0);
    t.x1 = static_cast<int32_t>(x1 > x0 ? x1 : x0);
    t.y1 = static_cast<int32_t>(y1 > y0 ? y1 : y0);

    float area = cpv_edge(Pn[0][0], Pn[0][1], Pn[1][0], Pn[1][1], Pn[2][0], Pn[2][1]);
    bool front;
    int ea[3], eb[3];
    if (area < 0.0f) {
        area = -area;
        front = false;
        ea[0] = 2; eb[0] = 1; ea[1] = 0; eb[1] = 2; ea[2] = 1; eb[2] = 0;
    } else {
        front = true;
        ea[0] = 1; eb[0] = 2; ea[1] = 2; eb[1] = 0; ea[2] = 0; eb[2] = 1;
    }
    t.area = area;
#pragma unroll
    for (int k = 0; k < 3; k++) {
        t.ax[k] = Pn[ea[k]][0];
        t.ay[k] = Pn[ea[k]][1];
        t.dx[k] = __fsub_rn(Pn[eb[k]][0], Pn[ea[k]][0]);
        t.dy[k] = __fsub_rn(Pn[eb[k]][1], Pn[ea[k]][1]);
        t.z[k] = Pn[k][2];
        t.w[k] = Pn[k][3];
    }
    bool live = t.x1 > t.x0 && t.y1 > t.y0;
    if ((CPV_CULL_MODE & 2) && !front) live = false;
    if ((CPV_CULL_MODE & 1) && front) live = false;
    t.flags = (live ? 1u : 0u) | (front ? 2u : 0u);
}

/* Pixel centre in NDC (CPVulkan/CommandBuffer.Draw.cpp:1524, 1573-1580):
 * (x / width + halfPixel) * 2 - 1, halfPixel = (1 / width) * 0.5. */
__device__ __forceinline__ float cpv_pixel_ndc(int32_t x, float extent) {
    const float half = __fmul_rn(__fdiv_rn(1.0f, extent), 0.5f);
    return __fsub_rn(__fmul_rn(__fadd_rn(__fdiv_rn(static_cast<float>(x), extent), half), 2.0f), 1.0f);
}

__device__ __forceinline__ bool cpv_covers(const CpvTri& t, float xf, float yf, float w[3]) {
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const float t0 = __fmul_rn(__fsub_rn(xf, t.ax[k]), t.dy[k]);
        const float t1 = __fmul_rn(__fsub_rn(yf, t.ay[k]), t.dx[k]);
        w[k] = __fsub_rn(t0, t1);
    }
    return !(w[0] < 0.0f || w[1] < 0.0f || w[2] < 0.0f);
}

/* Set-up kernel: tile rectangle per primitive (empty when culled, off
 * screen, or when a bounding box of at most four pixels covers none of its
 * pixel centres — the raster would find no fragment there either). */
extern "C" __global__ void __launch_bounds__(256) cpv_setup_rects(CpvDrawParams P) {
    const uint64_t g = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (g >= P.total_prims) return;
    CpvTri t;
    cpv_setup<false>(P, g, t);
    uint16_t r[4] = {0, 0, 0, 0};
    if (t.flags & 1u) {
        bool any = true;
        if ((t.x1 - t.x0) * (t.y1 - t.y0) <= 4) {
            any = false;
            const float vw = P.viewport[2], vh = P.viewport[3];
            for (int32_t y = t.y0; y < t.y1; y++) {
                const float yf = cpv_pixel_ndc(y, vh);
                for (int32_t x = t.x0; x < t.x1; x++) {
                    float w[3];
                    if (cpv_covers(t, cpv_pixel_ndc(x, vw), yf, w)) any = true;
                }
            }
        }
        if (any) {
            r[0] = static_cast<uint16_t>(t.x0 >> CPV_TILE_SHIFT);
            r[1] = static_cast<uint16_t>(t.y0 >> CPV_TILE_SHIFT);
            r[2] = static_cast<uint16_t>(((t.x1 - 1) >> CPV_TILE_SHIFT) + 1);
            r[3] = static_cast<uint16_t>(((t.y1 - 1) >> CPV_TILE_SHIFT) + 1);
        }
    }
    uint2 packed;
    packed.x = static_cast<uint32_t>(r[0]) | (static_cast<uint32_t>(r[1]) << 16);
    packed.y = static_cast<uint32_t>(r[2]) | (static_cast<uint32_t>(r[3]) << 16);
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

/* One covered pixel: barycentrics, depth, varyings, fragment shader, then
 * the reference's per-fragment operations. Returns 1 when the colour write
 * happened. */
__device__ __forceinline__ void cpv_fragment(const CpvDrawParams& P, const CpvTri& t, float w[3], int32_t x, int32_t y, CpvPixel& s) {
    w[0] = __fdiv_rn(w[0], t.area);
    w[1] = __fdiv_rn(w[1], t.area);
    w[2] = __fdiv_rn(w[2], t.area);
    const float depth = __fadd_rn(__fadd_rn(__fmul_rn(t.z[0], w[0]), __fmul_rn(t.z[1], w[1])), __fmul_rn(t.z[2], w[2]));
    float in[CPV_NV_ALLOC];
#pragma unroll
    for (int c = 0; c < CPV_NV; c++) {
        const int kind = cpv_interp(c);
        if (kind == 2) {
            in[c] = t.var[t.pslot][c];
        } else if (kind == 1) {
            float r = 0.0f;
#pragma unroll
            for (int k = 0; k < 3; k++) r = __fadd_rn(r, __fmul_rn(w[k], t.var[k][c]));
            in[c] = r;
        } else {
            float num = 0.0f, den = 0.0f;
#pragma unroll
            for (int k = 0; k < 3; k++) {
                num = __fadd_rn(num, __fdiv_rn(__fmul_rn(w[k], t.var[k][c]), t.w[k]));
                den = __fadd_rn(den, __fdiv_rn(w[k], t.w[k]));
            }
            in[c] = __fdiv_rn(num, den);
        }
    }
    const float min_d = P.viewport[4], max_d = P.viewport[5];
    const float mapped = __fadd_rn(__fmul_rn(__fsub_rn(max_d, min_d), depth), min_d);
    float frag_coord[4];
#if CPV_ORIGIN_UPPER
    frag_coord[0] = static_cast<float>(x);
#else
    frag_coord[0] = __fsub_rn(__fsub_rn(P.viewport[2], static_cast<float>(x)), 1.0f);
#endif
    frag_coord[1] = static_cast<float>(y);
    frag_coord[2] = depth;
    frag_coord[3] = 1.0f;
    const bool front = (t.flags & 2u) != 0u;
    float colour[4];
    if (cpv_fs_run(P, in, frag_coord, front, colour)) return;

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
        float dst[4];
#pragma unroll
        for (int i = 0; i < 4; i++) dst[i] = cpv_decode_unorm8((s.colour >> cpv_channel_shift(i)) & 0xFFu);
        float out[4];
#if CPV_BLEND
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

/* Raster kernel: one CTA per screen tile (blockIdx.x = tile id).
 * direct != 0: the tile walks every primitive of the draw (small draws).
 * Otherwise it walks its bin: bin_list[start, end) in API order, or — when
 * the bin list overflowed its capacity — every primitive whose tile
 * rectangle overlaps the tile. */
extern "C" __global__ void __launch_bounds__(CPV_RT_THREADS) cpv_raster(CpvDrawParams P, uint32_t direct) {
    __shared__ CpvTri tris[CPV_BATCH];
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

    for (uint64_t base = begin; base < end; base += CPV_BATCH) {
        const uint32_t n = static_cast<uint32_t>((end - base) < CPV_BATCH ? (end - base) : CPV_BATCH);
        __syncthreads();
        if (threadIdx.x < n) {
            CpvTri& t = tris[threadIdx.x];
            uint64_t g;
            bool skip = false;
            if (direct || scan_rects) {
                g = base + threadIdx.x;
                if (scan_rects) {
                    const uint2 r = reinterpret_cast<const uint2*>(P.rects)[g];
                    const uint32_t rx0 = r.x & 0xFFFFu, ry0 = r.x >> 16, rx1 = r.y & 0xFFFFu, ry1 = r.y >> 16;
                    skip = !(tx >= rx0 && tx < rx1 && ty >= ry0 && ty < ry1);
                }
            } else {
                g = P.bin_list[base + threadIdx.x];
            }
            if (skip) t.flags = 0u;
            else cpv_setup<true>(P, g, t);
        }
        __syncthreads();
        for (uint32_t j = 0; j < n; j++) {
            const CpvTri& t = tris[j];
            if (!(t.flags & 1u)) continue;
#pragma unroll
            for (int k = 0; k < CPV_PPT; k++) {
                if (!inside[k]) continue;
                if (px[k] < t.x0 || px[k] >= t.x1 || py[k] < t.y0 || py[k] >= t.y1) continue;
                float w[3];
                if (!cpv_covers(t, xf[k], yf[k], w)) continue;
                cpv_fragment(P, t, w, px[k], py[k], st[k]);
            }
        }
    }
#pragma unroll
    for (int k = 0; k < CPV_PPT; k++) {
        if (inside[k]) cpv_store_pixel(P, static_cast<uint64_t>(py[k]) * P.fb_width + px[k], st[k]);
    }
}

#endif /* CPV_PIPELINE_CUH */
