/*
 * cpv_stage.cuh — the per-pipeline stage functions. Deliberately without an
 * include guard: the module source includes it once per pipeline, inside
 * that pipeline's namespace (cpv_p0, cpv_p1, …), after the pipeline's
 * fixed-function macros (CPV_TOPOLOGY, CPV_CULL_MODE, CPV_FRONT_CW,
 * CPV_DEPTH_*, CPV_STENCIL_TEST, CPV_ST_*, CPV_BLEND, CPV_SRC_* / CPV_DST_*,
 * CPV_*_OP, CPV_WRITE_MASK, CPV_LOGIC, CPV_LOGIC_OP, CPV_DEPTH_BOUNDS,
 * CPV_MIN_DEPTH_BOUNDS, CPV_MAX_DEPTH_BOUNDS, CPV_COLOR_FORMAT, CPV_DEPTH_FORMAT,
 * CPV_ORIGIN_UPPER, CPV_NV) and its translated shaders:
 *
 *   __device__ void cpv_vs_run(const CpvDrawParams&, uint32_t vertex_index,
 *                              uint32_t instance_index, float pos[4], float var[CPV_NV]);
 *   __device__ bool cpv_fs_run(const CpvDrawParams&, const float in[CPV_NV],
 *                              const float frag_coord[4], bool front, float colour[4 * CPV_NUM_CA]);
 *   __device__ int  cpv_interp(int component);  // 0 perspective, 1 linear, 2 flat
 *
 * Vertex shading is recomputed where it is needed (set-up and raster) instead
 * of being stored: a vertex shader is a pure function of its inputs, and the
 * reference itself shades every assembled vertex (one per index), so the
 * recomputation is arithmetic the reference also performs and costs no HBM
 * traffic for a vertex-output buffer.
 */

/* Primitive class of the pipeline's topology: 0 triangles, 1 lines (list,
 * strip), 2 points. */
#if CPV_TOPOLOGY == 0
#define CPV_PRIM_KIND 2
#elif CPV_TOPOLOGY == 1 || CPV_TOPOLOGY == 2
#define CPV_PRIM_KIND 1
#else
#define CPV_PRIM_KIND 0
#endif
#ifndef CPV_LINE_WIDTH
#define CPV_LINE_WIDTH 1.0f
#endif
/* logicOpEnable (blending is then off) and its VkLogicOp */
#ifndef CPV_LOGIC
#define CPV_LOGIC 0
#define CPV_LOGIC_OP 3
#endif
/* depthBoundsTestEnable with a depth attachment, and the static bounds */
#ifndef CPV_DEPTH_BOUNDS
#define CPV_DEPTH_BOUNDS 0
#define CPV_MIN_DEPTH_BOUNDS 0.0f
#define CPV_MAX_DEPTH_BOUNDS 1.0f
#endif

/* The fragment shader of a primitive whose shader is constant over it
 * (CPV_FS_CONSTANT): shaded once from the provoking vertex's outputs; the
 * colour goes to var[0][0..3] (a discard kills the primitive) and, with
 * blend tables, the primitive index to var[1][0]. */
template <bool WITH_VARYINGS>
__device__ __forceinline__ void cpv_shade_constant(const CpvDrawParams& P, const float* provoking, bool front, uint32_t g32, CpvTri& t, bool& live) {
#if CPV_FS_CONSTANT
    if (WITH_VARYINGS && live) {
        float in[CPV_NV_ALLOC];
#pragma unroll
        for (int c = 0; c < CPV_NV_ALLOC; c++) in[c] = c < CPV_NV ? provoking[c] : 0.0f;
        const float frag_coord[4] = {0.0f, 0.0f, 0.0f, 1.0f};  /* not read by this shader */
        float colour[CPV_COLOUR_FLOATS];
        if (cpv_fs_run(P, in, frag_coord, front, colour)) live = false;
#pragma unroll
        for (int c = 0; c < 4; c++) t.var[0][c] = colour[c];
#if CPV_BLEND_TABLE
        t.var[1][0] = __uint_as_float(g32);  /* the primitive's blend table */
#endif
    }
#else
    (void)P; (void)provoking; (void)front; (void)g32; (void)t; (void)live;
#endif
}

#if CPV_PRIM_KIND == 2
/* Point set-up (CPVulkan/CommandBuffer.Draw.cpp:1315-1380): screen position
 * (int)((ndc + 1) * 0.5 * (extent - 1)), half size ceil(size / 2), and the
 * pixels whose s = 0.5 + (x - sx) / size and t (likewise in y) lie in
 * [0, 1]. s is monotonic in x, so those pixels form a rectangle, found by
 * evaluating the reference's expression at the candidate range's ends; it
 * becomes the box, and the zero edges cover every pixel in it. */
template <bool WITH_VARYINGS>
__device__ __forceinline__ void cpv_setup(const CpvDrawParams& P, uint64_t g, CpvTri& t) {
    const uint32_t ppi = P.prims_per_instance;
    const uint32_t g32 = static_cast<uint32_t>(g);
    const uint32_t inst = P.instance_count > 1u ? g32 / ppi : 0u;
    const uint32_t p = g32 - inst * ppi;
    float pos[4], var[CPV_NV_ALLOC], size = 1.0f;
    cpv_vs_run(P, cpv_vertex_id(P, p), P.first_instance + inst, pos, var, &size);
    const float w = pos[3];
    const float nx = __fdiv_rn(pos[0], w), ny = __fdiv_rn(pos[1], w), nz = __fdiv_rn(pos[2], w);
    const float vw = P.viewport[2], vh = P.viewport[3];
    const int64_t sx = cpv_f2i(__fmul_rn(__fmul_rn(__fadd_rn(nx, 1.0f), 0.5f), __fsub_rn(vw, 1.0f)));
    const int64_t sy = cpv_f2i(__fmul_rn(__fmul_rn(__fadd_rn(ny, 1.0f), 0.5f), __fsub_rn(vh, 1.0f)));
    const int64_t half = cpv_f2i(ceilf(__fdiv_rn(size, 2.0f)));
    int64_t xe = min(static_cast<int64_t>(cpv_f2i(vw)), sx + half + 1), ye = min(static_cast<int64_t>(cpv_f2i(vh)), sy + half + 1);
    xe = min(xe, static_cast<int64_t>(P.fb_width));
    ye = min(ye, static_cast<int64_t>(P.fb_height));
    int64_t xb = max(static_cast<int64_t>(0), sx - half), yb = max(static_cast<int64_t>(0), sy - half);
    auto inside = [&](int64_t d) {
        const float s = __fadd_rn(0.5f, __fdiv_rn(static_cast<float>(static_cast<int32_t>(d)), size));
        return s >= 0.0f && s <= 1.0f;
    };
    /* the reference's loops cover at most a size-wide square plus one
     * pixel: shrink each end to its first covered pixel */
    while (xb < xe && !inside(xb - sx)) xb++;
    while (xe > xb && !inside(xe - 1 - sx)) xe--;
    while (yb < ye && !inside(yb - sy)) yb++;
    while (ye > yb && !inside(ye - 1 - sy)) ye--;
    bool live = xe > xb && ye > yb && size == size;
    t.box = make_int4(static_cast<int32_t>(xb), static_cast<int32_t>(yb), static_cast<int32_t>(live ? xe : xb), static_cast<int32_t>(live ? ye : yb));
#pragma unroll
    for (int k = 0; k < 3; k++) t.e[k] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    t.za = make_float4(nz, 0.0f, 0.0f, 1.0f);
    if (WITH_VARYINGS) {
#pragma unroll
        for (int c = 0; c < CPV_NV; c++) t.var[0][c] = var[c];
    }
    cpv_shade_constant<WITH_VARYINGS>(P, var, true, g32, t, live);
    t.wf = make_float4(w, w, w, __uint_as_float((live ? 1u : 0u) | 2u));
}
#elif CPV_PRIM_KIND == 1
/* Line set-up (CPVulkan/CommandBuffer.Draw.cpp:1382-1449): the quad around
 * p0 → p1 offset by ±(dir.y, -dir.x) * lineWidth / extent, dir the
 * normalised 4-component difference of the two (NDC xyz, clip w) points;
 * its four edges; a box around the quad's corners with a two-pixel margin
 * (the edge tests decide coverage; the reference tests every viewport
 * pixel, and pixels that far outside the quad fail an edge). */
template <bool WITH_VARYINGS>
__device__ __forceinline__ void cpv_setup(const CpvDrawParams& P, uint64_t g, CpvTri& t) {
    static_assert(CPV_ANY_LINES && CPV_NV_PAD >= 7, "a module with line pipelines defines CPV_ANY_LINES");
    const uint32_t ppi = P.prims_per_instance;
    const uint32_t g32 = static_cast<uint32_t>(g);
    const uint32_t inst = P.instance_count > 1u ? g32 / ppi : 0u;
    const uint32_t instance = P.first_instance + inst;
    const uint32_t p = g32 - inst * ppi;
    uint32_t raw[3], provoking;
    cpv_prim_vertices(CPV_TOPOLOGY, p, raw, provoking);
    (void)provoking;
    float Pn[2][4];
#pragma unroll
    for (int k = 0; k < 2; k++) {
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
    const float lwx = __fdiv_rn(CPV_LINE_WIDTH, vw), lwy = __fdiv_rn(CPV_LINE_WIDTH, vh);
    /* glm::normalize: v * (1 / sqrt(dot(v, v))), dot4 = (x + y) + (z + w) */
    float dv[4];
#pragma unroll
    for (int i = 0; i < 4; i++) dv[i] = __fsub_rn(Pn[1][i], Pn[0][i]);
    const float dot = __fadd_rn(__fadd_rn(__fmul_rn(dv[0], dv[0]), __fmul_rn(dv[1], dv[1])),
                                __fadd_rn(__fmul_rn(dv[2], dv[2]), __fmul_rn(dv[3], dv[3])));
    const float inv = __fdiv_rn(1.0f, __fsqrt_rn(dot));
    const float dir_x = __fmul_rn(dv[0], inv), dir_y = __fmul_rn(dv[1], inv);
    const float ox = __fmul_rn(dir_y, lwx), oy = __fmul_rn(-dir_x, lwy);
    const float c00x = __fadd_rn(Pn[0][0], ox), c00y = __fadd_rn(Pn[0][1], oy);
    const float c01x = __fsub_rn(Pn[0][0], ox), c01y = __fsub_rn(Pn[0][1], oy);
    const float c10x = __fadd_rn(Pn[1][0], ox), c10y = __fadd_rn(Pn[1][1], oy);
    const float c11x = __fsub_rn(Pn[1][0], ox), c11y = __fsub_rn(Pn[1][1], oy);
    /* edges (a, b): (p00, p01), (p11, p10), (p10, p00), (p01, p11) */
    t.e[0] = make_float4(c00x, c00y, __fsub_rn(c01x, c00x), __fsub_rn(c01y, c00y));
    t.e[1] = make_float4(c11x, c11y, __fsub_rn(c10x, c11x), __fsub_rn(c10y, c11y));
    t.e[2] = make_float4(c10x, c10y, __fsub_rn(c00x, c10x), __fsub_rn(c00y, c10y));
    t.za = make_float4(c01x, c01y, __fsub_rn(c11x, c01x), __fsub_rn(c11y, c01y));
    const float cx[4] = {c00x, c01x, c10x, c11x}, cy[4] = {c00y, c01y, c10y, c11y};
    bool nan = false, finite = true;
    float minx = cx[0], maxx = cx[0], miny = cy[0], maxy = cy[0];
#pragma unroll
    for (int i = 0; i < 4; i++) {
        nan = nan || cx[i] != cx[i] || cy[i] != cy[i];
        finite = finite && fabsf(cx[i]) <= 3.0e38f && fabsf(cy[i]) <= 3.0e38f;
        minx = fminf(minx, cx[i]); maxx = fmaxf(maxx, cx[i]);
        miny = fminf(miny, cy[i]); maxy = fmaxf(maxy, cy[i]);
    }
    /* the reference loops x < viewport.width (a float): ceil */
    const int64_t iw = min(static_cast<int64_t>(cpv_f2i(ceilf(vw))), static_cast<int64_t>(P.fb_width));
    const int64_t ih = min(static_cast<int64_t>(cpv_f2i(ceilf(vh))), static_cast<int64_t>(P.fb_height));
    int64_t x0 = 0, y0 = 0, x1 = iw, y1 = ih;
    if (finite) {
        /* pixel x has its centre at NDC (2x + 1) / W - 1 */
        auto lo = [](float v, float e) { return static_cast<int64_t>(floorf(fminf(fmaxf((v + 1.0f) * e * 0.5f - 0.5f, -4.0f), e + 4.0f))) - 2; };
        auto hi = [](float v, float e) { return static_cast<int64_t>(ceilf(fminf(fmaxf((v + 1.0f) * e * 0.5f - 0.5f, -4.0f), e + 4.0f))) + 3; };
        x0 = max(x0, lo(minx, vw));
        y0 = max(y0, lo(miny, vh));
        x1 = min(x1, hi(maxx, vw));
        y1 = min(y1, hi(maxy, vh));
    }
    bool live = !nan && x1 > x0 && y1 > y0;
    t.box = make_int4(static_cast<int32_t>(x0), static_cast<int32_t>(y0), static_cast<int32_t>(live ? x1 : x0), static_cast<int32_t>(live ? y1 : y0));
    const float dx = __fsub_rn(Pn[1][0], Pn[0][0]), dy = __fsub_rn(Pn[1][1], Pn[0][1]);
    const float len = __fsqrt_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)));
    if (WITH_VARYINGS) cpv_shade_constant<WITH_VARYINGS>(P, t.var[0], true, g32, t, live);
    t.var[2][0] = Pn[0][0];
    t.var[2][1] = Pn[0][1];
    t.var[2][2] = dx;
    t.var[2][3] = dy;
    t.var[2][4] = __fmul_rn(len, len);
    t.var[2][5] = Pn[0][2];
    t.var[2][6] = Pn[1][2];
    t.wf = make_float4(Pn[0][3], Pn[1][3], 0.0f, __uint_as_float((live ? 1u : 0u) | 2u | (3u << 6)));
}
#else
/* The per-vertex part of the set-up: the vertex shader and the perspective
 * divide of its position (CPVulkan/CommandBuffer.Draw.cpp:1541-1546), NDC
 * x, y, z and clip w. `var` receives the shader's outputs. */
__device__ __forceinline__ void cpv_vertex_ndc(const CpvDrawParams& P, uint32_t vertex_id, uint32_t instance, float Pn[4], float var[CPV_NV_ALLOC]) {
    float pos[4];
    cpv_vs_run(P, vertex_id, instance, pos, var);
    const float w = pos[3];
    Pn[0] = __fdiv_rn(pos[0], w);
    Pn[1] = __fdiv_rn(pos[1], w);
    Pn[2] = __fdiv_rn(pos[2], w);
    Pn[3] = w;
}

/* The per-triangle part of the set-up from its three vertices (after the CW
 * swap): screen bounding box, area, facing and cull, and with varyings the
 * constant fragment colour. t.var must hold the vertices' outputs when
 * WITH_VARYINGS. */
template <bool WITH_VARYINGS>
__device__ __forceinline__ void cpv_setup_tri(const CpvDrawParams& P, const float Pn[3][4], uint32_t pslot, uint32_t g32, CpvTri& t) {
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
    /* a fragment shader reading only flat inputs (the provoking vertex's)
     * gives every fragment of the primitive one colour; a discard discards
     * them all */
    if (WITH_VARYINGS) cpv_shade_constant<WITH_VARYINGS>(P, t.var[pslot], front, g32, t, live);
    const uint32_t flags = (live ? 1u : 0u) | (front ? 2u : 0u) | (pslot << 6);
    t.wf = make_float4(Pn[0][3], Pn[1][3], Pn[2][3], __uint_as_float(flags));
}

/* A triangle's instance and its three raw assembled vertices after the CW
 * swap (CPVulkan/CommandBuffer.Draw.cpp:567-760, 1532-1535), and the slot of
 * the provoking vertex among them. */
__device__ __forceinline__ void cpv_tri_vertices(const CpvDrawParams& P, uint32_t g32, uint32_t raw[3], uint32_t& instance, uint32_t& pslot,
                                                 uint32_t& inst) {
    const uint32_t ppi = P.prims_per_instance;
    inst = P.instance_count > 1u ? g32 / ppi : 0u;
    instance = P.first_instance + inst;
    const uint32_t p = g32 - inst * ppi;
    uint32_t provoking;
    cpv_prim_vertices(CPV_TOPOLOGY, p, raw, provoking);
#if CPV_FRONT_CW
    { const uint32_t tmp = raw[0]; raw[0] = raw[2]; raw[2] = tmp; }
#endif
    pslot = raw[0] == provoking ? 0u : (raw[1] == provoking ? 1u : 2u);
}

/* Primitive set-up: vertex shading of the three vertices, perspective divide,
 * screen bounding box, area, facing and cull. `g` is the primitive index
 * within the draw (all instances). A vertex with a slot of the vertex stage
 * (cpv_vertex_slot) is read from it instead of being shaded again: the slot
 * holds what cpv_vertex_ndc returns for the same vertex id and instance,
 * computed by the same function, so the bits are the same. */
template <bool WITH_VARYINGS>
__device__ __forceinline__ void cpv_setup(const CpvDrawParams& P, uint64_t g, CpvTri& t) {
    const uint32_t g32 = static_cast<uint32_t>(g);  /* draws hold < 2^32 primitives */
    uint32_t raw[3], instance, pslot, inst;
    cpv_tri_vertices(P, g32, raw, instance, pslot, inst);
    const uint32_t vs_count = P.vs_count;
    float Pn[3][4];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const uint32_t vid = cpv_vertex_id(P, raw[k]);
        const uint32_t rel = vid - P.vs_lo;
        if (rel < vs_count) {
            const uint64_t slot = static_cast<uint64_t>(inst) * vs_count + rel;
            const float4 p = __ldg(reinterpret_cast<const float4*>(P.vs_pos) + slot);
            Pn[k][0] = p.x;
            Pn[k][1] = p.y;
            Pn[k][2] = p.z;
            Pn[k][3] = p.w;
            if (WITH_VARYINGS) {
                const float4* v = reinterpret_cast<const float4*>(P.vs_var + slot * P.vs_stride);
#pragma unroll
                for (int q = 0; q < (CPV_NV + 3) / 4; q++) {
                    const float4 f = __ldg(v + q);
                    const float fs[4] = {f.x, f.y, f.z, f.w};
#pragma unroll
                    for (int c = 0; c < 4; c++)
                        if (4 * q + c < CPV_NV) t.var[k][4 * q + c] = fs[c];
                }
            }
        } else {
            float var[CPV_NV_ALLOC];
            cpv_vertex_ndc(P, vid, instance, Pn[k], var);
            if (WITH_VARYINGS) {
#pragma unroll
                for (int c = 0; c < CPV_NV; c++) t.var[k][c] = var[c];
            }
        }
    }
#if CPV_CULL_MODE != 0
    /* a culled triangle is dead whatever its box and edges: its facing is
     * the sign of the area cpv_setup_tri computes (the same expression),
     * so those are skipped for it. Nothing reads a dead primitive's other
     * fields. */
    {
        const float area = cpv_edge(Pn[0][0], Pn[0][1], Pn[1][0], Pn[1][1], Pn[2][0], Pn[2][1]);
        const bool front = !(area < 0.0f);
        if (((CPV_CULL_MODE & 2) && !front) || ((CPV_CULL_MODE & 1) && front)) {
            t.box = make_int4(0, 0, 0, 0);
            t.wf.w = __uint_as_float(0u);
            return;
        }
    }
#endif
    cpv_setup_tri<WITH_VARYINGS>(P, Pn, pslot, g32, t);
}

/* The vertex stage of the batched path: shades vertex id `vid` of
 * `instance` once and stores its NDC position and clip w, and its outputs,
 * in slot `slot` of P's vertex slots. */
__device__ __forceinline__ void cpv_vertex_slot(const CpvDrawParams& P, uint32_t vid, uint32_t instance, uint64_t slot) {
    float Pn[4], var[((CPV_NV_ALLOC + 3) / 4) * 4];
    cpv_vertex_ndc(P, vid, instance, Pn, var);
    reinterpret_cast<float4*>(P.vs_pos)[slot] = make_float4(Pn[0], Pn[1], Pn[2], Pn[3]);
    float4* v = reinterpret_cast<float4*>(P.vs_var + slot * P.vs_stride);
#pragma unroll
    for (int q = 0; q < (CPV_NV + 3) / 4; q++)
        v[q] = make_float4(var[4 * q], 4 * q + 1 < CPV_NV ? var[4 * q + 1] : 0.0f, 4 * q + 2 < CPV_NV ? var[4 * q + 2] : 0.0f,
                           4 * q + 3 < CPV_NV ? var[4 * q + 3] : 0.0f);
}

#endif /* CPV_PRIM_KIND */

/* The colour attachment's layout (from the reference's format table,
 * CPVulkanBase/Formats.cpp): texel bytes, channels, bits per channel, kind
 * (0 UNORM, 1 SNORM, 2 SFLOAT), red in byte 2. */
#ifndef CPV_CF_BYTES
#define CPV_CF_BYTES 4
#define CPV_CF_CHANNELS 4
#define CPV_CF_BITS 8
#define CPV_CF_KIND 0
#define CPV_CF_BGRA (CPV_COLOR_FORMAT == 44)
#endif
#define CPV_CF_MASK (CPV_CF_BITS >= 32 ? 0xFFFFFFFFu : ((1u << (CPV_CF_BITS & 31)) - 1u))

/* Where channel i of the colour attachment texel sits
 * (CPVulkanBase/Formats.cpp:248,255): 32-bit word i * bits / 32 of the
 * texel, at bit (i * bits) % 32; red in byte 2 for B8G8R8A8. */
#define CPV_CF_WORDS ((CPV_CF_BYTES + 3) / 4)
__device__ __forceinline__ int cpv_channel_shift(int i) {
#if CPV_CF_BGRA
    return i == 0 ? 16 : (i == 1 ? 8 : (i == 2 ? 0 : 24));
#else
    return (CPV_CF_BITS * i) & 31;
#endif
}
__device__ __forceinline__ int cpv_channel_word(int i) {
#if CPV_CF_BGRA
    (void)i;
    return 0;
#else
    return (CPV_CF_BITS * i) >> 5;
#endif
}
/* Stored bits of channel i of a texel (CPV_CF_WORDS words). */
__device__ __forceinline__ uint32_t cpv_channel_get(const uint32_t* t, int i) { return (t[cpv_channel_word(i)] >> cpv_channel_shift(i)) & CPV_CF_MASK; }

/* Stored channel bits → float, the reference's pixel decoder
 * (LLVMRuntime/ImageCompiler.cpp:161-230): UNORM and SNORM over their
 * maximum (signed codes not clamped), half floats widened, 32-bit floats
 * as stored. */
__device__ __forceinline__ float cpv_cf_decode(uint32_t raw) {
#if CPV_CF_KIND == 0 && CPV_CF_BITS == 8
    return CPV_DECODE8(raw);
#elif CPV_CF_KIND == 0
    return cpv_decode_unorm16(raw);
#elif CPV_CF_KIND == 1
    return cpv_decode_norm(raw, CPV_CF_BITS / 8, true);
#elif CPV_CF_KIND >= 3
    return __uint_as_float(raw); /* integer formats: not blended, never decoded to a value */
#elif CPV_CF_BITS == 16
    return cpv_half_to_float(raw);
#else
    return __uint_as_float(raw);
#endif
}

/* Float → stored channel bits, the reference's colour encoder
 * (LLVMRuntime/ImageCompiler.cpp:1077-1185): UNORM clamped to [0, 1] and
 * SNORM to [-1, 1] (minnum / maxnum), scaled, rounded half away from zero;
 * half floats rounded to nearest even; 32-bit floats as they are. */
__device__ __forceinline__ uint32_t cpv_cf_encode(float x) {
#if CPV_CF_KIND == 0
    return cpv_encode_unorm(x, CPV_CF_BITS == 8 ? 255.0f : 65535.0f);
#elif CPV_CF_KIND == 1
    const float v = roundf(__fmul_rn(fminf(fmaxf(x, -1.0f), 1.0f), CPV_CF_BITS == 8 ? 127.0f : 32767.0f));
    return static_cast<uint32_t>(static_cast<int32_t>(v)) & CPV_CF_MASK;
#elif CPV_CF_KIND == 3
    /* UINT: the output's 32 bits as an unsigned integer, clamped to the
     * channel's maximum (LLVMRuntime/ImageCompiler.cpp:1121-1144) */
    const uint32_t u = __float_as_uint(x);
    return CPV_CF_BITS >= 32 ? u : (u < CPV_CF_MASK ? u : CPV_CF_MASK);
#elif CPV_CF_KIND == 4
    /* SINT: as a signed integer, clamped to the channel's range (:1146-1175) */
    int32_t v = static_cast<int32_t>(__float_as_uint(x));
    if (CPV_CF_BITS < 32) {
        const int32_t hi = static_cast<int32_t>(CPV_CF_MASK >> 1), lo = -hi - 1;
        v = v > lo ? v : lo;
        v = v < hi ? v : hi;
    }
    return static_cast<uint32_t>(v) & CPV_CF_MASK;
#elif CPV_CF_BITS == 16
    return cpv_float_to_half(x);
#else
    return __float_as_uint(x);
#endif
}

/* The colour texel of pixel `pix` of this attachment into t[0 ..
 * CPV_CF_WORDS) (0 without one). */
__device__ __forceinline__ void cpv_load_colour(const uint8_t* color, uint64_t pix, uint32_t* t) {
#if CPV_COLOR_FORMAT != 0 && CPV_CF_BYTES == 1
    t[0] = color[pix];
#elif CPV_COLOR_FORMAT != 0 && CPV_CF_BYTES == 2
    t[0] = reinterpret_cast<const uint16_t*>(color)[pix];
#elif CPV_COLOR_FORMAT != 0 && CPV_CF_BYTES == 8
    const uint2 v = reinterpret_cast<const uint2*>(color)[pix];
    t[0] = v.x;
    t[1] = v.y;
#elif CPV_COLOR_FORMAT != 0 && CPV_CF_BYTES == 16
    const uint4 v = reinterpret_cast<const uint4*>(color)[pix];
    t[0] = v.x;
    t[1] = v.y;
    t[2] = v.z;
    t[3] = v.w;
#elif CPV_COLOR_FORMAT != 0
    t[0] = reinterpret_cast<const uint32_t*>(color)[pix];
#else
    (void)color; (void)pix; /* a depth-only pass, or an unused attachment */
    t[0] = 0u;
#endif
}

__device__ __forceinline__ void cpv_store_colour(uint8_t* color, uint64_t pix, const uint32_t* t) {
#if CPV_COLOR_FORMAT != 0 && CPV_CF_BYTES == 1
    color[pix] = static_cast<uint8_t>(t[0]);
#elif CPV_COLOR_FORMAT != 0 && CPV_CF_BYTES == 2
    reinterpret_cast<uint16_t*>(color)[pix] = static_cast<uint16_t>(t[0]);
#elif CPV_COLOR_FORMAT != 0 && CPV_CF_BYTES == 8
    reinterpret_cast<uint2*>(color)[pix] = make_uint2(t[0], t[1]);
#elif CPV_COLOR_FORMAT != 0 && CPV_CF_BYTES == 16
    reinterpret_cast<uint4*>(color)[pix] = make_uint4(t[0], t[1], t[2], t[3]);
#elif CPV_COLOR_FORMAT != 0
    reinterpret_cast<uint32_t*>(color)[pix] = t[0];
#else
    (void)color; (void)pix; (void)t;
#endif
}

#ifndef CPV_EXTRA_CA
#define CPV_EXTRA_CA 0 /* this pipeline's colour attachments after the first */
#endif
#if CPV_EXTRA_CA > 0
/* The attachments after the first: each has its own format, blend state and
 * write mask, compiled from this file again in a nested namespace
 * (cpv_ca1 …); these are defined after those namespaces. */
__device__ __forceinline__ void cpv_load_extra(const uint8_t* const* color, uint64_t pix, CpvPixel& s);
__device__ __forceinline__ void cpv_store_extra(uint8_t* const* color, uint64_t pix, const CpvPixel& s);
__device__ __forceinline__ void cpv_write_extra(const float blend_constants[4], const float* colour, CpvPixel& s);
#endif

__device__ __forceinline__ void cpv_load_pixel(const uint8_t* color, const uint8_t* depth, uint64_t pix, CpvPixel& s,
                                               const uint8_t* const* extra = nullptr) {
    cpv_load_colour(color, pix, s.colour);
#if CPV_EXTRA_CA > 0
    cpv_load_extra(extra, pix, s);
#else
    (void)extra;
#endif
#if CPV_DEPTH_FORMAT == 124
    s.depth_raw = reinterpret_cast<const uint16_t*>(depth)[pix];
    s.depth = cpv_decode_unorm16(s.depth_raw);
    s.stencil = 0u;
#elif CPV_DEPTH_FORMAT == 126
    s.depth_raw = reinterpret_cast<const uint32_t*>(depth)[pix];
    s.depth = __uint_as_float(s.depth_raw);
    s.stencil = 0u;
#elif CPV_DEPTH_FORMAT == 130
    const uint2 v = reinterpret_cast<const uint2*>(depth)[pix];
    s.depth_raw = v.x;
    s.depth = __uint_as_float(v.x);
    s.stencil = v.y & 0xFFu;
#else
    (void)depth;
    s.depth_raw = 0u;
    s.depth = 0.0f;
    s.stencil = 0u;
#endif
}

__device__ __forceinline__ void cpv_store_pixel(uint8_t* color, uint8_t* depth, uint64_t pix, const CpvPixel& s, uint8_t* const* extra = nullptr) {
    cpv_store_colour(color, pix, s.colour);
#if CPV_EXTRA_CA > 0
    cpv_store_extra(extra, pix, s);
#else
    (void)extra;
#endif
#if CPV_DEPTH_FORMAT == 124
    reinterpret_cast<uint16_t*>(depth)[pix] = static_cast<uint16_t>(s.depth_raw);
#elif CPV_DEPTH_FORMAT == 126
    reinterpret_cast<uint32_t*>(depth)[pix] = s.depth_raw;
#elif CPV_DEPTH_FORMAT == 130
    uint2* p = reinterpret_cast<uint2*>(depth) + pix;
    uint2 v = *p;
    v.x = s.depth_raw;
    v.y = (v.y & ~0xFFu) | (s.stencil & 0xFFu);
    *p = v;
#else
    (void)depth;
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

__device__ __forceinline__ void cpv_blend(const float s[4], const float d[4], const float c[4], float out[4]) {
    float sf[4], df[4];
    cpv_blend_factor(s, d, c, CPV_SRC_COLOR, CPV_SRC_ALPHA, sf);
    cpv_blend_factor(s, d, c, CPV_DST_COLOR, CPV_DST_ALPHA, df);
#pragma unroll
    for (int i = 0; i < 4; i++) out[i] = cpv_blend_op(s[i], sf[i], d[i], df[i], CPV_COLOR_OP);
    if (CPV_COLOR_OP != CPV_ALPHA_OP) out[3] = cpv_blend_op(s[3], sf[3], d[3], df[3], CPV_ALPHA_OP);
}

/* Early depth test. The fragment shader has no effect but its colour and
 * its discard (no storage writes, no FragDepth), so when it cannot discard
 * and no stencil test runs, a triangle fragment that fails the depth test
 * against the pixel's current depth changes nothing whatever its colour:
 * with the depth (the same arithmetic as below) known, the varyings and the
 * shader are skipped for it. The depth test, depth write and colour write
 * then run unchanged in cpv_rop for the fragments that pass. */
#ifndef CPV_FS_KILL
#define CPV_FS_KILL 1
#endif
#define CPV_EARLY_DEPTH (CPV_PRIM_KIND == 0 && CPV_DEPTH_TEST && CPV_DEPTH_FORMAT != 0 && !(CPV_STENCIL_TEST && CPV_DEPTH_FORMAT == 130) && !CPV_FS_KILL)

/* The varyings of a line's fragment at pixel (x, y): line parameter
 * t = dot(p - p0, d) / (|d| |d|) at the pixel centre, weights (1 - t, t),
 * depth p0.z * t + p1.z * (1 - t) as the reference writes it
 * (CPVulkan/CommandBuffer.Draw.cpp:1441-1486). Returns the NDC depth. */
__device__ __forceinline__ float cpv_line_inputs(const CpvDrawParams& P, const CpvTri& t, int32_t x, int32_t y, float* in) {
    const float xf = cpv_pixel_ndc(x, P.viewport[2]), yf = cpv_pixel_ndc(y, P.viewport[3]);
    const float num = __fadd_rn(__fmul_rn(__fsub_rn(xf, t.var[2][0]), t.var[2][2]), __fmul_rn(__fsub_rn(yf, t.var[2][1]), t.var[2][3]));
    const float lt = __fdiv_rn(num, t.var[2][4]);
    const float w[2] = {__fsub_rn(1.0f, lt), lt};
    const float depth = __fadd_rn(__fmul_rn(t.var[2][5], lt), __fmul_rn(t.var[2][6], w[0]));
    const float pw[2] = {t.wf.x, t.wf.y};
#pragma unroll
    for (int c = 0; c < CPV_NV; c++) {
        const int kind = cpv_interp(c);
        if (kind == 2) {
            in[c] = t.var[0][c];
        } else if (kind == 1) {
            in[c] = __fadd_rn(__fadd_rn(0.0f, __fmul_rn(w[0], t.var[0][c])), __fmul_rn(w[1], t.var[1][c]));
        } else {
            float n = 0.0f, d = 0.0f;
#pragma unroll
            for (int k = 0; k < 2; k++) {
                n = __fadd_rn(n, __fdiv_rn(__fmul_rn(w[k], t.var[k][c]), pw[k]));
                d = __fadd_rn(d, __fdiv_rn(w[k], pw[k]));
            }
            in[c] = __fdiv_rn(n, d);
        }
    }
    return depth;
}

/* A triangle's screen-linear NDC depth at barycentrics w (w_k / area). */
__device__ __forceinline__ float cpv_tri_depth(const CpvTri& t, const float w[3]) {
    return __fadd_rn(__fadd_rn(__fmul_rn(t.za.x, w[0]), __fmul_rn(t.za.y, w[1])), __fmul_rn(t.za.z, w[2]));
}

/* A triangle's varyings at barycentrics w: perspective Σ w·v/p ÷ Σ w/p,
 * linear Σ w·v, or flat from the provoking vertex
 * (CPVulkan/CommandBuffer.Draw.cpp:816-954). */
__device__ __forceinline__ void cpv_tri_inputs(const CpvTri& t, const float w[3], float* in) {
    const float pw[3] = {t.wf.x, t.wf.y, t.wf.z};
    const uint32_t pslot = cpv_tri_pslot(t);
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
}

/* gl_FragCoord of pixel (x, y) at NDC depth `depth`. */
__device__ __forceinline__ void cpv_frag_coord(const CpvDrawParams& P, int32_t x, int32_t y, float depth, float fc[4]) {
#if CPV_ORIGIN_UPPER
    (void)P;
    fc[0] = static_cast<float>(x);
#else
    fc[0] = __fsub_rn(__fsub_rn(P.viewport[2], static_cast<float>(x)), 1.0f);
#endif
    fc[1] = static_cast<float>(y);
    fc[2] = depth;
    fc[3] = 1.0f;
}

#ifndef CPV_LOD_SITES
#define CPV_LOD_SITES 0
#endif

#if CPV_LOD_SITES > 0 && !CPV_FS_CONSTANT
/* The quad-derivative mode's helper runs: the fragment shader at the
 * horizontal and the vertical neighbour of (x, y) within its 2x2 quad,
 * whatever their coverage, with the varyings, depth and gl_FragCoord the
 * primitive has there; they write nothing and only record their sampling
 * coordinates in q. */
__device__ __forceinline__ void cpv_quad_helpers(const CpvDrawParams& P, const CpvTri& t, int32_t x, int32_t y, CpvQuadLod& q) {
    q.odd = static_cast<uint32_t>(x & 1) | (static_cast<uint32_t>(y & 1) << 1);
    q.seen[0] = q.seen[1] = 0u;
#pragma unroll
    for (uint32_t n = 0; n < 2; n++) {
        const int32_t nx = n == 0 ? (x ^ 1) : x, ny = n == 0 ? y : (y ^ 1);
        float in[CPV_NV_ALLOC];
#if CPV_PRIM_KIND == 2
        const float depth = t.za.x;
#pragma unroll
        for (int c = 0; c < CPV_NV; c++) in[c] = t.var[0][c];
#elif CPV_PRIM_KIND == 1
        const float depth = cpv_line_inputs(P, t, nx, ny, in);
#else
        float w[3];
        (void)cpv_covers(t, cpv_pixel_ndc(nx, P.viewport[2]), cpv_pixel_ndc(ny, P.viewport[3]), w);
        const float area = t.za.w;
#pragma unroll
        for (int k = 0; k < 3; k++) w[k] = __fdiv_rn(w[k], area);
        const float depth = cpv_tri_depth(t, w);
        cpv_tri_inputs(t, w, in);
#endif
        float fc[4], scratch[CPV_COLOUR_FLOATS];
        cpv_frag_coord(P, nx, ny, depth, fc);
        q.mode = n + 1u;
        (void)cpv_fs_run(P, in, fc, cpv_tri_front(t), scratch, &q);
    }
    q.mode = 0u;
}
#endif

/* Shading of one covered pixel: barycentrics (w_k / area), screen-linear
 * depth, varyings (cpv_tri_inputs, cpv_line_inputs; a point's fragments
 * take its vertex's outputs as they are and its NDC z,
 * CPVulkan/CommandBuffer.Draw.cpp:1364-1374), viewport depth mapping
 * (:1300-1313) and the fragment shader. Returns true when the shader
 * discards, or when `early` (the pixel's current state) is given and the
 * fragment fails the early depth test. */
__device__ __forceinline__ bool cpv_shade(const CpvDrawParams& P, const CpvTri& t, const float wr[3], int32_t x, int32_t y, float* colour,
                                          float& mapped, const CpvPixel* early = nullptr) {
    float in[CPV_NV_ALLOC];
#if CPV_PRIM_KIND == 2
    (void)wr;
    const float depth = t.za.x;
#pragma unroll
    for (int c = 0; c < CPV_NV; c++) in[c] = t.var[0][c];
#elif CPV_PRIM_KIND == 1
    (void)wr;
    const float depth = cpv_line_inputs(P, t, x, y, in);
#else
    const float area = t.za.w;
    float w[3];
    w[0] = __fdiv_rn(wr[0], area);
    w[1] = __fdiv_rn(wr[1], area);
    w[2] = __fdiv_rn(wr[2], area);
    const float depth = cpv_tri_depth(t, w);
#if CPV_EARLY_DEPTH
    if (early) {
        const float early_mapped = __fadd_rn(__fmul_rn(__fsub_rn(P.viewport[5], P.viewport[4]), depth), P.viewport[4]);
        if (!cpv_fcompare(early_mapped, early->depth, CPV_DEPTH_OP)) return true;
    }
#else
    (void)early;
#endif
    cpv_tri_inputs(t, w, in);
#endif /* CPV_PRIM_KIND */
    const float min_d = P.viewport[4], max_d = P.viewport[5];
    mapped = __fadd_rn(__fmul_rn(__fsub_rn(max_d, min_d), depth), min_d);
    float frag_coord[4];
    cpv_frag_coord(P, x, y, depth, frag_coord);
#if CPV_FS_CONSTANT
    /* shaded once at set-up (a discarding primitive is not live) */
    (void)in;
    (void)frag_coord;
#pragma unroll
    for (int c = 0; c < 4; c++) colour[c] = t.var[0][c];
    return false;
#elif CPV_LOD_SITES > 0
    CpvQuadLod q;
    cpv_quad_helpers(P, t, x, y, q);
    return cpv_fs_run(P, in, frag_coord, cpv_tri_front(t), colour, &q);
#else
    return cpv_fs_run(P, in, frag_coord, cpv_tri_front(t), colour);
#endif
}

/* VkLogicOp CPV_LOGIC_OP of an encoded fragment channel s and the stored
 * channel d (Vulkan 1.1, "Logical Operations"); the switch folds to one
 * expression at compile time. */
__device__ __forceinline__ uint32_t cpv_logic(uint32_t s, uint32_t d) {
    uint32_t r;
    switch (CPV_LOGIC_OP) {
    case 0: r = 0u; break;
    case 1: r = s & d; break;
    case 2: r = s & ~d; break;
    case 3: r = s; break;
    case 4: r = ~s & d; break;
    case 5: r = d; break;
    case 6: r = s ^ d; break;
    case 7: r = s | d; break;
    case 8: r = ~(s | d); break;
    case 9: r = ~(s ^ d); break;
    case 10: r = ~d; break;
    case 11: r = s | ~d; break;
    case 12: r = ~s; break;
    case 13: r = ~s | d; break;
    case 14: r = ~(s & d); break;
    default: r = 0xFFu; break;
    }
    return r & 0xFFu;
}

/* The colour write of this attachment for a fragment that passed every
 * test (LLVMRuntime/PipelineCompiler.cpp:1528-1727): logic op, else blend
 * (CPVulkan/CommandBuffer.Draw.cpp:956-1262), else the colour; then the
 * write mask and the format's encoder. `colour` is this attachment's output. */
__device__ __forceinline__ void cpv_write_colour(const float blend_constants[4], const float colour[4], uint32_t* texel) {
#if CPV_COLOR_FORMAT == 0
    (void)blend_constants; (void)colour; (void)texel;
#else
#if CPV_LOGIC
    /* 8-bit normalised formats only (pipeline creation rejects others) */
    (void)blend_constants;
    uint32_t logic = 0u;
#pragma unroll
    for (int i = 0; i < CPV_CF_CHANNELS; i++) {
        const uint32_t d = (texel[0] >> cpv_channel_shift(i)) & 0xFFu;
        const uint32_t byte = ((CPV_WRITE_MASK >> i) & 1u) ? (cpv_logic(cpv_cf_encode(colour[i]), d) & 0xFFu) : d;
        logic |= byte << cpv_channel_shift(i);
    }
    texel[0] = logic;
#else
    float out[4];
#if CPV_BLEND
    /* the destination as the reference's decoder returns it: absent
     * channels read (0, 0, 0, 1) */
    float dst[4];
#pragma unroll
    for (int i = 0; i < 4; i++) dst[i] = i < CPV_CF_CHANNELS ? cpv_cf_decode(cpv_channel_get(texel, i)) : (i == 3 ? 1.0f : 0.0f);
    cpv_blend(colour, dst, blend_constants, out);
#else
    (void)blend_constants;
#pragma unroll
    for (int i = 0; i < 4; i++) out[i] = colour[i];
#endif
    /* the format's channels, each encoded or, outside the write mask, kept */
    uint32_t packed[CPV_CF_WORDS];
#pragma unroll
    for (int w = 0; w < CPV_CF_WORDS; w++) packed[w] = 0u;
#pragma unroll
    for (int i = 0; i < CPV_CF_CHANNELS; i++) {
        const uint32_t field = ((CPV_WRITE_MASK >> i) & 1u) ? cpv_cf_encode(out[i]) : cpv_channel_get(texel, i);
        packed[cpv_channel_word(i)] |= field << cpv_channel_shift(i);
    }
#pragma unroll
    for (int w = 0; w < CPV_CF_WORDS; w++) texel[w] = packed[w];
#endif
#endif
}

/* Order as the reference's fragment wrapper: current values → depth bounds
 * test → stencil test → depth test → depth / stencil write → colour write
 * (logic op or blend, write mask, encode). */
__device__ __forceinline__ void cpv_rop(const float blend_constants[4], bool front, const float* colour, float mapped, CpvPixel& s,
                                        const uint8_t* table = nullptr) {
    const bool has_depth = CPV_DEPTH_FORMAT != 0;
#if CPV_DEPTH_BOUNDS && CPV_DEPTH_FORMAT != 0
    /* the stored depth outside the bounds (unordered compares: NaN is
     * outside) ends the fragment with no write of any kind */
    if (!(s.depth >= CPV_MIN_DEPTH_BOUNDS) || !(s.depth <= CPV_MAX_DEPTH_BOUNDS)) return;
#endif
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
    if (CPV_COLOR_FORMAT == 0) return; /* a depth-only pass: no colour write */
    if (stencil_result && depth_result) {
#if CPV_BLEND_TABLE
        if (table) {
            /* the primitive's blend result for this destination byte, per channel */
            uint32_t packed = 0u;
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const uint32_t d = (s.colour[0] >> cpv_channel_shift(i)) & 0xFFu;
                packed |= static_cast<uint32_t>(table[i * 256 + d]) << cpv_channel_shift(i);
            }
            s.colour[0] = packed;
            return;
        }
#else
        (void)table;
#endif
        cpv_write_colour(blend_constants, colour, s.colour);
#if CPV_EXTRA_CA > 0
        cpv_write_extra(blend_constants, colour, s);
#endif
    }
}

/* One destination byte b of a blend table: the colour write of `colour`
 * (constant over the primitive) over a destination whose channels all hold
 * byte b, for each of the 4 channels (the same arithmetic as cpv_rop; with
 * no DST_ALPHA-based colour factor, channel i's result depends only on
 * destination channel i). */
__device__ __forceinline__ void cpv_blend_table_column(const float colour[4], const float blend_constants[4], uint32_t b, uint8_t out_bytes[4]) {
    const float d = CPV_DECODE8(b);
    const float dst[4] = {d, d, d, d};
    float out[4];
#if CPV_BLEND
    cpv_blend(colour, dst, blend_constants, out);
#else
    (void)dst;
    (void)blend_constants;
#pragma unroll
    for (int i = 0; i < 4; i++) out[i] = colour[i];
#endif
#pragma unroll
    for (int i = 0; i < 4; i++) out_bytes[i] = static_cast<uint8_t>(((CPV_WRITE_MASK >> i) & 1u) ? cpv_encode_unorm(out[i], 255.0f) : b);
}

constexpr bool kBlendTable = CPV_BLEND_TABLE != 0;
/* a blend-table pipeline without depth or stencil operations: a covered
 * fragment's whole effect is its table lookup */
constexpr bool kTableOnly = kBlendTable && !(CPV_DEPTH_TEST && CPV_DEPTH_FORMAT != 0) && !(CPV_STENCIL_TEST && CPV_DEPTH_FORMAT == 130) &&
                            !(CPV_DEPTH_BOUNDS && CPV_DEPTH_FORMAT != 0);

/* cpv_rop's colour write through a blend table, when every test passes */
__device__ __forceinline__ void cpv_apply_table(const uint8_t* table, CpvPixel& s) {
    uint32_t packed = 0u;
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const uint32_t d = (s.colour[0] >> cpv_channel_shift(i)) & 0xFFu;
        packed |= static_cast<uint32_t>(table[i * 256 + d]) << cpv_channel_shift(i);
    }
    s.colour[0] = packed;
}

/* The stage functions of this pipeline, as one type the module's
 * dispatcher (cpv_dispatch) hands to generic code. */
struct Stage {
    template <bool WITH_VARYINGS>
    static __device__ __forceinline__ void setup(const CpvDrawParams& P, uint64_t g, CpvTri& t) { cpv_setup<WITH_VARYINGS>(P, g, t); }
    /* the vertex stage (triangle topologies only; the host gives other
     * draws no slots) */
    static __device__ __forceinline__ void vertex(const CpvDrawParams& P, uint32_t vid, uint32_t instance, uint64_t slot) {
#if CPV_PRIM_KIND == 0
        cpv_vertex_slot(P, vid, instance, slot);
#else
        (void)P; (void)vid; (void)instance; (void)slot;
#endif
    }
    static __device__ __forceinline__ bool shade(const CpvDrawParams& P, const CpvTri& t, const float w[3], int32_t x, int32_t y, float* colour,
                                                 float& mapped, const CpvPixel* early = nullptr) {
        return cpv_shade(P, t, w, x, y, colour, mapped, early);
    }
    static __device__ __forceinline__ void rop(const float blend_constants[4], bool front, const float* colour, float mapped, CpvPixel& s,
                                               const uint8_t* table = nullptr) {
        cpv_rop(blend_constants, front, colour, mapped, s, table);
    }
    /* the primitive's blend table in P.tables, or null */
    static __device__ __forceinline__ const uint8_t* table(const CpvDrawParams& P, const CpvTri& t) {
#if CPV_BLEND_TABLE
        return P.tables ? P.tables + static_cast<uint64_t>(__float_as_uint(t.var[1][0])) * 1024u : nullptr;
#else
        (void)P;
        (void)t;
        return nullptr;
#endif
    }
    /* `extra`: the colour attachments after the first (unused without them) */
    static __device__ __forceinline__ void load_pixel(const uint8_t* c, const uint8_t* d, uint64_t pix, CpvPixel& s, const uint8_t* const* extra) {
        cpv_load_pixel(c, d, pix, s, extra);
    }
    static __device__ __forceinline__ void store_pixel(uint8_t* c, uint8_t* d, uint64_t pix, const CpvPixel& s, uint8_t* const* extra) {
        cpv_store_pixel(c, d, pix, s, extra);
    }
};
