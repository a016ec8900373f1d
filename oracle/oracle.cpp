/*
 * oracle.cpp — CPU oracle for the draw hot path. TEST INFRASTRUCTURE ONLY
 * (see oracle.h for who may call it and its parity status).
 *
 * Build: g++ -O2 -std=c++17 -ffp-contract=off (oracle/Makefile). Contraction
 * must stay off: the reference's arithmetic is plain IEEE single precision
 * with no fused multiply-add (its JIT emits separate fmul/fadd,
 * LLVMRuntime/Jit.cpp:44-71, and the ICD's own C++ was built for x86-64
 * without FMA), and GCC on aarch64 contracts by default.
 *
 * Every function cites the reference lines it restates. Paths are relative
 * to the reference project root.
 */
#include "oracle.h"

#include <algorithm>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <limits>
#include <mutex>
#include <thread>
#include <vector>

namespace {

enum : uint32_t {
    FMT_R8G8B8A8_UNORM = 37,
    FMT_B8G8R8A8_UNORM = 44,
    FMT_R32_SFLOAT = 100,
    FMT_R32G32_SFLOAT = 103,
    FMT_R32G32B32_SFLOAT = 106,
    FMT_R32G32B32A32_SFLOAT = 109,
    FMT_D16_UNORM = 124,
    FMT_D32_SFLOAT = 126,
    FMT_D32_SFLOAT_S8_UINT = 130,
};

enum : uint32_t { TOPO_POINT_LIST = 0, TOPO_LINE_LIST = 1, TOPO_LINE_STRIP = 2, TOPO_TRIANGLE_LIST = 3, TOPO_TRIANGLE_STRIP = 4, TOPO_TRIANGLE_FAN = 5 };
enum : uint32_t { CULL_FRONT = 1, CULL_BACK = 2 };
enum : uint32_t { FRONT_FACE_CW = 1 };
enum : uint32_t { RATE_VERTEX = 0, RATE_INSTANCE = 1 };

constexpr int kMaxVaryings = 16;

/* ---------------------------------------------------------------------- */
/* Scalar helpers                                                          */
/* ---------------------------------------------------------------------- */

/* static_cast<int32_t>(float) as both target machines execute it
 * (saturating, NaN → 0): the reference relies on this conversion for the
 * screen bounding box (CPVulkan/CommandBuffer.Draw.cpp:1548-1563). */
int32_t f2i(float f) {
    if (f != f) return 0;
    if (f >= 2147483648.0f) return std::numeric_limits<int32_t>::max();
    if (f < -2147483648.0f) return std::numeric_limits<int32_t>::min();
    return static_cast<int32_t>(f);
}

/* std::max / std::min / std::clamp as the reference's GLSL helpers call
 * them (CPVulkan/GlslFunctions.cpp:106-140). */
float fmax_std(float a, float b) { return (a < b) ? b : a; }
float fmin_std(float a, float b) { return (b < a) ? b : a; }

/* llvm.maxnum / llvm.minnum (NaN-ignoring), used by the pixel encoders
 * (LLVMRuntime/ImageCompiler.cpp:540-560). */
float maxnum(float a, float b) { if (a != a) return b; if (b != b) return a; return a > b ? a : b; }
float minnum(float a, float b) { if (a != a) return b; if (b != b) return a; return a < b ? a : b; }

/* UNORM encode: minnum(maxnum(x,0),1) * (2^n-1) → llvm.round (half away
 * from zero) → fptoui (LLVMRuntime/ImageCompiler.cpp:27-32, 1081-1095). */
uint32_t encode_unorm(float x, float maxv) {
    float v = minnum(maxnum(x, 0.0f), 1.0f);
    v = v * maxv;
    v = std::round(v);
    return static_cast<uint32_t>(v);
}

/* UNORM decode: uitofp / (2^n-1) (LLVMRuntime/ImageCompiler.cpp:43-53). */
float decode_unorm8(uint8_t u) { return static_cast<float>(u) / 255.0f; }
float decode_unorm16(uint16_t u) { return static_cast<float>(u) / 65535.0f; }

/* EdgeFunction (CPVulkan/CommandBuffer.Draw.cpp:410-418). */
float edge(float ax, float ay, float bx, float by, float cx, float cy) {
    const float t0 = (cx - ax) * (by - ay);
    const float t1 = (cy - ay) * (bx - ax);
    return t0 - t1;
}

/* ---------------------------------------------------------------------- */
/* Vector helpers with the operand order the reference's glm calls give.   */
/* glm is a third-party dependency absent from the mount; the order below  */
/* restates glm 0.9.9's published operator*(mat4, vec4) (pairwise column   */
/* sums), compute_dot (left-to-right for vec2/vec3, pairwise for vec4) and */
/* normalize (x * (1 / sqrt(dot(x, x)))). Parity unpinned.                 */
/* ---------------------------------------------------------------------- */

struct V4 { float x, y, z, w; };

V4 mat4_mul_vec4(const float* m /* column-major 16 */, const float v[4]) {
    float r[4];
    for (int i = 0; i < 4; i++) {
        const float mul0 = m[0 * 4 + i] * v[0];
        const float mul1 = m[1 * 4 + i] * v[1];
        const float add0 = mul0 + mul1;
        const float mul2 = m[2 * 4 + i] * v[2];
        const float mul3 = m[3 * 4 + i] * v[3];
        const float add1 = mul2 + mul3;
        r[i] = add0 + add1;
    }
    return V4{r[0], r[1], r[2], r[3]};
}

float dot3(const float a[3], const float b[3]) {
    const float t0 = a[0] * b[0];
    const float t1 = a[1] * b[1];
    const float t2 = a[2] * b[2];
    return (t0 + t1) + t2;
}

void normalize3(const float v[3], float out[3]) {
    const float d = dot3(v, v);
    const float inv = 1.0f / std::sqrt(d);
    out[0] = v[0] * inv;
    out[1] = v[1] * inv;
    out[2] = v[2] * inv;
}

/* ---------------------------------------------------------------------- */
/* Image sampler (CPVulkan/ImageSampler.cpp)                               */
/* ---------------------------------------------------------------------- */

struct Texture {
    const uint8_t* data = nullptr;
    uint64_t bytes = 0;
    uint32_t width = 0, height = 0, levels = 0;
    uint64_t level_offset[16] = {};
    uint32_t level_w[16] = {}, level_h[16] = {};
    uint32_t format = 37;  /* VkFormat: R8G8B8A8 (37) or B8G8R8A8 (44) UNORM */
};

/* wrap (CPVulkan/ImageSampler.cpp:12-38). */
int32_t wrap(int32_t v, int32_t size, uint32_t mode) {
    switch (mode) {
    case 0: /* REPEAT */
        return (v % size + size) % size;
    case 1: { /* MIRRORED_REPEAT */
        const int32_t two = 2 * size;
        const int32_t n = (v % two + two) % two - size;
        return size - 1 - (n >= 0 ? n : -(1 + n));
    }
    case 2: /* CLAMP_TO_EDGE */
        return std::clamp(v, 0, size - 1);
    case 3: /* CLAMP_TO_BORDER */
        return std::clamp(v, -1, size);
    case 4: /* MIRROR_CLAMP_TO_EDGE */
        return std::clamp(v >= 0 ? v : -(1 + v), 0, size - 1);
    default:
        return 0;
    }
}

/* Border colour table (CPVulkan/ImageSampler.cpp:409-417). */
void border_colour(uint32_t border, float out[4]) {
    static const float table[6][4] = {{0, 0, 0, 0}, {0, 0, 0, 0}, {0, 0, 0, 1}, {0, 0, 0, 1}, {1, 1, 1, 1}, {1, 1, 1, 1}};
    const uint32_t b = border < 6 ? border : 0;
    for (int i = 0; i < 4; i++) out[i] = table[b][i];
}

/* GetPixel<fvec4> for RGBA8 UNORM with the border check
 * (CPVulkan/ImageSampler.cpp:133-160). */
void get_texel(const Texture& t, uint32_t level, int32_t x, int32_t y, uint32_t border, float out[4]) {
    const int32_t w = static_cast<int32_t>(t.level_w[level]);
    const int32_t h = static_cast<int32_t>(t.level_h[level]);
    if (x < 0 || x >= w || y < 0 || y >= h) {
        border_colour(border, out);
        return;
    }
    const uint64_t off = t.level_offset[level] + (static_cast<uint64_t>(y) * static_cast<uint64_t>(w) + static_cast<uint64_t>(x)) * 4u;
    if (off + 4 > t.bytes) {
        for (int i = 0; i < 4; i++) out[i] = 0.0f;
        return;
    }
    /* B8G8R8A8 keeps red in byte 2 (CPVulkanBase/Formats.cpp:255) */
    for (int i = 0; i < 4; i++) out[i] = decode_unorm8(t.data[off + ((t.format == 44 && i < 3) ? 2 - i : i)]);
}

/* lerp with a double-precision delta (CPVulkan/ImageSampler.cpp:51-55):
 * dvec4(min) + dvec4(max - min) * delta, converted back to float. */
void lerp4(const float a[4], const float b[4], double delta, float out[4]) {
    for (int i = 0; i < 4; i++) {
        const float diff = b[i] - a[i];
        const double prod = static_cast<double>(diff) * delta;
        const double sum = static_cast<double>(a[i]) + prod;
        out[i] = static_cast<float>(sum);
    }
}

/* SampleImageOfLevel for 2D, NEAREST/LINEAR, weighted average
 * (CPVulkan/ImageSampler.cpp:403-531). */
void sample_level(const Texture& t, uint32_t level, float u, float v, uint32_t filter, const cpv_scene_sampler& s, float out[4]) {
    const uint32_t range[2] = {t.level_w[level], t.level_h[level]};
    const float coord[2] = {u, v};
    const uint32_t modes[2] = {s.address_u, s.address_v};
    if (filter == 0) {
        int32_t c[2];
        for (int i = 0; i < 2; i++) {
            const float scaled = coord[i] * static_cast<float>(range[i]) + 0.0f;
            c[i] = f2i(std::floor(scaled));
            c[i] = wrap(c[i], static_cast<int32_t>(range[i]), modes[i]);
        }
        get_texel(t, level, c[0], c[1], s.border_color, out);
        return;
    }
    int32_t c0[2], c1[2];
    float frac[2];
    for (int i = 0; i < 2; i++) {
        const float scaled = coord[i] * static_cast<float>(range[i]) - 0.5f;
        const float fl = std::floor(scaled);
        c0[i] = f2i(fl);
        c1[i] = wrap(c0[i] + 1, static_cast<int32_t>(range[i]), modes[i]);
        c0[i] = wrap(c0[i], static_cast<int32_t>(range[i]), modes[i]);
        frac[i] = scaled - fl;
    }
    float t00[4], t01[4], t10[4], t11[4];
    get_texel(t, level, c0[0], c0[1], s.border_color, t00);
    get_texel(t, level, c0[0], c1[1], s.border_color, t01);
    get_texel(t, level, c1[0], c0[1], s.border_color, t10);
    get_texel(t, level, c1[0], c1[1], s.border_color, t11);
    float ij0[4], ij1[4];
    lerp4(t00, t10, static_cast<double>(frac[0]), ij0);
    lerp4(t01, t11, static_cast<double>(frac[0]), ij1);
    lerp4(ij0, ij1, static_cast<double>(frac[1]), out);
}

/* SampleImage (CPVulkan/ImageSampler.cpp:562-673) after the λ computation of
 * ImageSampleExplicitLod (CPVulkan/GlslFunctions.cpp:598-646). */
void sample(const Texture& t, const cpv_scene_sampler& s, float u, float v, float lod_base, float out[4]) {
    const float bias = std::clamp(s.mip_lod_bias + 0.0f, -32.0f, 32.0f);
    const float lambda_prime = lod_base + bias;
    const float lambda = std::clamp(lambda_prime, s.min_lod, s.max_lod);
    if (lambda <= 0) {
        sample_level(t, 0, u, v, s.mag_filter, s, out);
    } else {
        const float max_level = static_cast<float>(t.levels - 1);
        const float mip = std::clamp(lambda, 0.0f, max_level);
        if (s.mipmap_mode == 0) {
            const uint32_t real = static_cast<uint32_t>(std::ceil(mip + 0.5f)) - 1;
            sample_level(t, real, u, v, s.min_filter, s, out);
        } else {
            const uint32_t l1 = static_cast<uint32_t>(std::floor(mip));
            const float delta = mip - static_cast<float>(l1);
            float p1[4];
            sample_level(t, l1, u, v, s.min_filter, s, p1);
            if (delta == 0) {
                for (int i = 0; i < 4; i++) out[i] = p1[i];
            } else {
                float p2[4];
                sample_level(t, l1 + 1, u, v, s.min_filter, s, p2);
                lerp4(p1, p2, static_cast<double>(delta), out);
            }
        }
    }
    /* RGBA8 carries all four channels: no channel forcing (:652-670). */
}

/* ---------------------------------------------------------------------- */
/* Blend (CPVulkan/CommandBuffer.Draw.cpp:956-1262, ApplyBlendFactor and   */
/* ApplyBlend). The reference never reaches these templates (blendEnable   */
/* aborts in LLVMRuntime/PipelineCompiler.cpp:1674-1684); they are adopted */
/* as its blend semantics.                                                 */
/* ---------------------------------------------------------------------- */

void blend_factor(const float s[4], const float d[4], const float c[4], uint32_t colour_factor, uint32_t alpha_factor, float out[4]) {
    for (int i = 0; i < 4; i++) out[i] = 0.0f;
    switch (colour_factor) {
    case 0: break;
    case 1: for (int i = 0; i < 4; i++) out[i] = 1.0f; break;
    case 2: for (int i = 0; i < 4; i++) out[i] = s[i]; break;
    case 3: for (int i = 0; i < 4; i++) out[i] = 1.0f - s[i]; break;
    case 4: for (int i = 0; i < 4; i++) out[i] = d[i]; break;
    case 5: for (int i = 0; i < 4; i++) out[i] = 1.0f - d[i]; break;
    case 6: for (int i = 0; i < 4; i++) out[i] = s[3]; break;
    case 7: { const float v = 1 - s[3]; for (int i = 0; i < 4; i++) out[i] = v; break; }
    case 8: for (int i = 0; i < 4; i++) out[i] = d[3]; break;
    case 9: { const float v = 1 - d[3]; for (int i = 0; i < 4; i++) out[i] = v; break; }
    case 10: for (int i = 0; i < 4; i++) out[i] = c[i]; break;
    case 11: for (int i = 0; i < 4; i++) out[i] = 1.0f - c[i]; break;
    case 12: for (int i = 0; i < 4; i++) out[i] = c[3]; break;
    case 13: { const float v = 1 - c[3]; for (int i = 0; i < 4; i++) out[i] = v; break; }
    case 14: { const float f = fmin_std(s[3], 1 - d[3]); out[0] = f; out[1] = f; out[2] = f; out[3] = 1; break; }
    default: break;
    }
    if (colour_factor != alpha_factor) {
        switch (alpha_factor) {
        case 0: out[3] = 0; break;
        case 1: case 14: out[3] = 1; break;
        case 2: case 6: out[3] = s[3]; break;
        case 3: case 7: out[3] = 1 - s[3]; break;
        case 4: case 8: out[3] = d[3]; break;
        case 5: case 9: out[3] = 1 - d[3]; break;
        case 10: case 12: out[3] = c[3]; break;
        case 11: case 13: out[3] = 1 - c[3]; break;
        default: break;
        }
    }
}

void blend(const float s[4], const float d[4], const float c[4], uint32_t src_color, uint32_t dst_color, uint32_t color_op,
           uint32_t src_alpha, uint32_t dst_alpha, uint32_t alpha_op, float out[4]) {
    float sf[4], df[4];
    blend_factor(s, d, c, src_color, src_alpha, sf);
    blend_factor(s, d, c, dst_color, dst_alpha, df);
    for (int i = 0; i < 4; i++) {
        const float a = s[i] * sf[i];
        const float b = d[i] * df[i];
        switch (color_op) {
        case 0: out[i] = a + b; break;
        case 1: out[i] = a - b; break;
        case 2: out[i] = b - a; break;
        case 3: out[i] = fmin_std(s[i], d[i]); break;
        case 4: out[i] = fmax_std(s[i], d[i]); break;
        default: out[i] = 0; break;
        }
    }
    if (color_op != alpha_op) {
        const float a = s[3] * sf[3];
        const float b = d[3] * df[3];
        switch (alpha_op) {
        case 0: out[3] = a + b; break;
        case 1: out[3] = a - b; break;
        case 2: out[3] = b - a; break;
        case 3: out[3] = fmin_std(s[3], d[3]); break;
        case 4: out[3] = fmax_std(s[3], d[3]); break;
        default: break;
        }
    }
}

/* ---------------------------------------------------------------------- */
/* Shader programs: C++ restatements of the SPIR-V modules the harness    */
/* ships (cpvulkan_gb300/shaders/gen_spirv.py), one op per SPIR-V op.     */
/* ---------------------------------------------------------------------- */

enum Interp { INTERP_PERSPECTIVE = 0, INTERP_LINEAR = 1, INTERP_FLAT = 2 };

struct ProgramInfo {
    int num_inputs;           /* fragment shader inputs, declaration order */
    int input_size[4];        /* components per input */
    Interp input_interp[4];
};

ProgramInfo program_info(uint32_t program) {
    switch (program) {
    case CPV_PROGRAM_CUBE: return {1, {4}, {INTERP_PERSPECTIVE}};
    case CPV_PROGRAM_TEXLIT:
    case CPV_PROGRAM_FETCH:
    case CPV_PROGRAM_STORAGE:
    case CPV_PROGRAM_SEPARATE: return {2, {2, 3}, {INTERP_PERSPECTIVE, INTERP_PERSPECTIVE}};
    case CPV_PROGRAM_FLATQUAD: return {1, {4}, {INTERP_FLAT}};
    case CPV_PROGRAM_MESHPC: return {1, {3}, {INTERP_PERSPECTIVE}};
    case CPV_PROGRAM_DISCARD: return {1, {4}, {INTERP_PERSPECTIVE}};
    case CPV_PROGRAM_NOPERSP: return {1, {4}, {INTERP_LINEAR}};
    case CPV_PROGRAM_POINTS: return {1, {4}, {INTERP_PERSPECTIVE}};
    case CPV_PROGRAM_MRT:
    case CPV_PROGRAM_MRTI:
    case CPV_PROGRAM_MATHX:
    case CPV_PROGRAM_CALLS:
    case CPV_PROGRAM_SSBO: return {1, {4}, {INTERP_PERSPECTIVE}};
    default: return {0, {0}, {INTERP_PERSPECTIVE}};
    }
}

struct Resources {
    const float* ubo = nullptr; /* set 0 binding 0 */
    uint32_t ubo_floats = 0;
    const Texture* texture = nullptr;
    const cpv_scene_sampler* sampler = nullptr;
    const float* push = nullptr; /* 32 floats */
};

float ubo_at(const Resources& r, uint32_t i) { return i < r.ubo_floats ? r.ubo[i] : 0.0f; }

struct VsOut {
    float pos[4];
    float var[kMaxVaryings];
    float point_size; /* gl_PointSize (1 when the shader does not write it) */
};

/* The quad-derivative LOD mode (cpv_scene::spec_lod): the inputs the
 * fragment's primitive has at its horizontal neighbour (x ^ 1, y) and its
 * vertical one (x, y ^ 1) in the 2x2 quad, whatever their coverage, for
 * fine derivatives dP/dx = P(x | 1) - P(x & ~1) (Vulkan 1.1, "Derivative
 * Operations"). The GPU path runs the shader there and records its
 * sampling coordinates (cpv_sample_quad); the restated programs sample at
 * coordinates that are their inputs, so the inputs suffice. */
struct Quad {
    uint32_t odd;       /* bit 0: x odd; bit 1: y odd */
    const float* in[2];
};

/* 0.5 * log2(r), the same binary32 steps as the GPU path's cpv_half_log2:
 * the series ln m = 2 (s + s³/3 + s⁵/5 + s⁷/7 + s⁹/9), s = (m - 1) / (m + 1),
 * on the mantissa reduced to [√½, √2]; 0 or NaN give -∞, +∞ gives +∞. */
float half_log2(float r) {
    if (!(r > 0.0f)) return -std::numeric_limits<float>::infinity();
    if (r == std::numeric_limits<float>::infinity()) return r;
    uint32_t b;
    std::memcpy(&b, &r, 4);
    int32_t e = 0;
    if (b < 0x00800000u) {
        const float scaled = r * 16777216.0f;
        std::memcpy(&b, &scaled, 4);
        e = -24;
    }
    e += static_cast<int32_t>(b >> 23) - 127;
    const uint32_t mb = (b & 0x007FFFFFu) | 0x3F800000u;
    float m;
    std::memcpy(&m, &mb, 4);
    if (m > 1.41421356f) {
        m = m * 0.5f;
        e += 1;
    }
    const float s = (m - 1.0f) / (m + 1.0f);
    const float s2 = s * s;
    float q = s2 * 0.111111111f + 0.142857143f;
    q = q * s2 + 0.2f;
    q = q * s2 + 0.333333333f;
    q = q * s2 + 1.0f;
    const float log2m = (s * q) * 2.88539008f;
    return (static_cast<float>(e) + log2m) * 0.5f;
}

/* λ_base = log2(max(ρx, ρy)) of implicit-LOD sampling at (u, v), with
 * ρ = |(du, dv)| scaled by the level-0 extent (Vulkan 1.1, "Scale Factor
 * Operation"); the derivatives are the differences with the neighbours'
 * coordinates (un[n], vn[n]), signed by the fragment's place in its quad. */
float quad_lambda(const Texture& t, float u, float v, const float un[2], const float vn[2], uint32_t odd) {
    const float w = static_cast<float>(t.level_w[0]), h = static_cast<float>(t.level_h[0]);
    float r2[2];
    for (uint32_t n = 0; n < 2; n++) {
        const bool o = ((odd >> n) & 1u) != 0u;
        const float du = o ? u - un[n] : un[n] - u;
        const float dv = o ? v - vn[n] : vn[n] - v;
        const float a = du * w, b = dv * h;
        r2[n] = a * a + b * b;
    }
    return half_log2(r2[0] >= r2[1] ? r2[0] : r2[1]);
}

/* attr[location][4] holds each attribute as fetched (missing components
 * default to 0,0,0,1). */
void run_vs(uint32_t program, const float attr[8][4], const Resources& r, VsOut& out) {
    out.point_size = 1.0f;
    switch (program) {
    case CPV_PROGRAM_CUBE:
    case CPV_PROGRAM_DISCARD:
    case CPV_PROGRAM_NOPERSP:
    case CPV_PROGRAM_POINTS:
    case CPV_PROGRAM_MRT:
    case CPV_PROGRAM_MRTI:
    case CPV_PROGRAM_MATHX:
    case CPV_PROGRAM_CALLS:
    case CPV_PROGRAM_SSBO: {
        float m[16];
        for (int i = 0; i < 16; i++) m[i] = ubo_at(r, i);
        for (int i = 0; i < 4; i++) out.var[i] = attr[1][i];
        const V4 p = mat4_mul_vec4(m, attr[0]);
        out.pos[0] = p.x; out.pos[1] = p.y; out.pos[2] = p.z; out.pos[3] = p.w;
        if (program == CPV_PROGRAM_POINTS) out.point_size = attr[1][3] * 16.0f;
        break;
    }
    case CPV_PROGRAM_TEXLIT:
    case CPV_PROGRAM_FETCH:
    case CPV_PROGRAM_STORAGE:
    case CPV_PROGRAM_SEPARATE: {
        float m[16];
        for (int i = 0; i < 16; i++) m[i] = ubo_at(r, i);
        out.var[0] = attr[1][0]; out.var[1] = attr[1][1];
        out.var[2] = attr[2][0]; out.var[3] = attr[2][1]; out.var[4] = attr[2][2];
        const float v[4] = {attr[0][0], attr[0][1], attr[0][2], 1.0f};
        const V4 p = mat4_mul_vec4(m, v);
        out.pos[0] = p.x; out.pos[1] = p.y; out.pos[2] = p.z; out.pos[3] = p.w;
        break;
    }
    case CPV_PROGRAM_FLATQUAD: {
        for (int i = 0; i < 4; i++) out.var[i] = attr[1][i];
        out.pos[0] = attr[0][0]; out.pos[1] = attr[0][1]; out.pos[2] = 0.0f; out.pos[3] = 1.0f;
        break;
    }
    case CPV_PROGRAM_MESHPC: {
        out.var[0] = attr[1][0]; out.var[1] = attr[1][1]; out.var[2] = attr[1][2];
        const float sum[3] = {attr[0][0] + attr[2][0], attr[0][1] + attr[2][1], attr[0][2] + attr[2][2]};
        const float v[4] = {sum[0], sum[1], sum[2], 1.0f};
        const V4 p = mat4_mul_vec4(r.push, v);
        out.pos[0] = p.x; out.pos[1] = p.y; out.pos[2] = p.z; out.pos[3] = p.w;
        break;
    }
    default:
        for (int i = 0; i < 4; i++) out.pos[i] = 0.0f;
        break;
    }
}

/* GLSL.std.450 functions the reference registers (CPVulkan/GlslFunctions.cpp:36-40,
 * 190-310): NMin / NMax give the second operand for a NaN first one, else
 * std::min / std::max; NClamp = NMin(NMax(x, lo), hi); FindILsb / FindUMsb /
 * FindSMsb return -1 without a set bit, FindSMsb looks at ~v for v < 0;
 * SSign = (0 < v) - (v < 0). */
float glsl_nmin(float a, float b) { return std::isnan(a) ? b : std::min(a, b); }
float glsl_nmax(float a, float b) { return std::isnan(a) ? b : std::max(a, b); }
float glsl_nclamp(float x, float lo, float hi) { return glsl_nmin(glsl_nmax(x, lo), hi); }
int32_t find_ilsb(uint32_t v) { return v == 0 ? -1 : __builtin_ctz(v); }
int32_t find_umsb(uint32_t v) { return v == 0 ? -1 : 31 - __builtin_clz(v); }
int32_t find_smsb(int32_t v) {
    if (v < 0) v = ~v;
    return v == 0 ? -1 : 31 - __builtin_clz(static_cast<uint32_t>(v));
}
int32_t ssign(int32_t v) { return (0 < v) - (v < 0); }

/* Returns true when the fragment is discarded (OpKill → return true,
 * LLVMRuntime/SPIRVCompiler.cpp:3308-3310, 3642-3651). colour holds 4
 * floats per output location (locations 0-7); a program fills the
 * locations it declares. */
bool run_fs(uint32_t program, const float* in, const Resources& r, float* colour, uint32_t spec_k, const Quad* quad) {
    switch (program) {
    case CPV_PROGRAM_MRT: {
        /* gen_spirv.py mrt_frag: one SPIR-V operation per float operation */
        const float* c = in;
        for (int i = 0; i < 4; i++) colour[i] = c[i];
        for (int i = 0; i < 3; i++) colour[4 + i] = 1.0f - c[i];
        colour[7] = c[3];
        colour[8] = c[2]; colour[9] = c[0]; colour[10] = c[1]; colour[11] = c[3];
        for (int i = 0; i < 4; i++) colour[12 + i] = c[i] * 0.5f;
        for (int i = 0; i < 4; i++) colour[16 + i] = c[i] * c[i];
        for (int i = 0; i < 4; i++) colour[20 + i] = c[i] * 2.0f - 1.0f;
        colour[24] = c[0] + c[1]; colour[25] = c[1] - c[2]; colour[26] = c[2]; colour[27] = 0.25f;
        colour[28] = c[3]; colour[29] = c[2]; colour[30] = c[1]; colour[31] = c[0];
        return false;
    }
    case CPV_PROGRAM_MRTI: {
        /* gen_spirv.py mrti_frag: integer outputs keep their bits in the
         * 32-bit output slots (OpConvertFToU / OpConvertFToS truncate) */
        const float* c = in;
        for (int i = 0; i < 4; i++) {
            colour[i] = c[i];
            const uint32_t u = static_cast<uint32_t>(c[i] * 300.0f);
            const int32_t v = static_cast<int32_t>(c[i] * 400.0f - 200.0f);
            std::memcpy(&colour[4 + i], &u, 4);
            std::memcpy(&colour[8 + i], &v, 4);
            colour[12 + i] = c[i];  /* OpBitcast: the same bits */
        }
        for (int i = 16; i < 32; i++) colour[i] = 0.0f;
        return false;
    }
    case CPV_PROGRAM_SSBO:
        /* gen_spirv.py ssbo_frag: colour times row 1 (bytes 16-31) of the
         * storage buffer, which is the uniform buffer bound again */
        for (int i = 0; i < 4; i++) colour[i] = in[i] * ubo_at(r, 4 + i);
        return false;
    case CPV_PROGRAM_CALLS: {
        /* gen_spirv.py calls_frag: scale() multiplies the variable it is
         * given by 0.5 and returns its x + 0.5; check() discards when y > 0.45 */
        float t[4];
        for (int i = 0; i < 4; i++) t[i] = in[i] * 0.5f;
        const float k = t[0] + 0.5f;
        if (t[1] > 0.45f) return true;
        colour[0] = t[0]; colour[1] = t[1]; colour[2] = t[2]; colour[3] = k;
        return false;
    }
    case CPV_PROGRAM_MATHX: {
        /* gen_spirv.py mathx_frag, one operation per SPIR-V instruction */
        const float* c = in;
        const float z = c[3] - c[3];
        const float nan = z / z;
        float r = glsl_nclamp(c[0] * 3.0f - 1.0f, 0.25f, 0.75f);
        r = glsl_nmin(nan, r);
        r = glsl_nmax(r, nan);
        const int32_t i = static_cast<int32_t>(c[1] * 1000.0f) - 500;  /* OpConvertFToS, OpISub */
        const uint32_t u = static_cast<uint32_t>(c[2] * 65535.0f);       /* OpConvertFToU */
        const int32_t bits = (find_smsb(i) + find_ilsb(static_cast<uint32_t>(i))) + ssign(i);
        const float n[3] = {0.6f, 0.0f, 0.8f};
        /* Reflect (glm::reflect): I - N * dot(N, I) * 2, dot left to right */
        const float d = (n[0] * c[0] + n[1] * c[1]) + n[2] * c[2];
        const float rx = c[0] - (n[0] * d) * 2.0f;
        colour[0] = r;
        colour[1] = static_cast<float>(bits) / 64.0f;
        colour[2] = static_cast<float>(find_umsb(u)) / 16.0f;
        colour[3] = rx * 0.5f + 0.5f;
        return false;
    }
    case CPV_PROGRAM_CUBE:
    case CPV_PROGRAM_NOPERSP:
    case CPV_PROGRAM_FLATQUAD:
    case CPV_PROGRAM_POINTS:
        for (int i = 0; i < 4; i++) colour[i] = in[i];
        return false;
    case CPV_PROGRAM_DISCARD:
        if (in[0] > 0.5f) return true;
        for (int i = 0; i < 4; i++) colour[i] = in[i];
        return false;
    case CPV_PROGRAM_STORAGE: {
        /* gen_spirv.py storage_frag: imageLoad at ivec2(uv * 64)
         * (OpVectorTimesScalar, OpConvertFToS), the reference's ImageFetch
         * (CPVulkan/GlslFunctions.cpp:740-744): level 0, zeros outside it */
        const int32_t px = static_cast<int32_t>(in[0] * 64.0f);
        const int32_t py = static_cast<int32_t>(in[1] * 64.0f);
        float t[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        if (r.texture && r.texture->levels > 0 && px >= 0 && py >= 0 && px < static_cast<int32_t>(r.texture->level_w[0]) &&
            py < static_cast<int32_t>(r.texture->level_h[0]))
            get_texel(*r.texture, 0, px, py, 0, t);
        for (int i = 0; i < 4; i++) colour[i] = t[i];
        return false;
    }
    case CPV_PROGRAM_TEXLIT:
    case CPV_PROGRAM_SEPARATE: {
        /* SEPARATE samples the same texture through a sampler in its own
         * binding (sampler2D(t, s)): the same arithmetic */
        float c[4] = {0, 0, 0, 1};
        if (r.texture && r.sampler) {
            /* implicit LOD: λ 0 as the reference computes it
             * (CPVulkan/GlslFunctions.cpp:657-672), or from the quad */
            float lod = 0.0f;
            if (quad && r.texture->levels != 0) {
                const float un[2] = {quad->in[0][0], quad->in[1][0]}, vn[2] = {quad->in[0][1], quad->in[1][1]};
                lod = quad_lambda(*r.texture, in[0], in[1], un, vn, quad->odd);
            }
            sample(*r.texture, *r.sampler, in[0], in[1], lod, c);
        }
        float n[3];
        normalize3(in + 2, n);
        const float light[3] = {ubo_at(r, 16), ubo_at(r, 17), ubo_at(r, 18)};
        const float d = dot3(n, light);
        const float l = fmax_std(d, 0.0f);
        colour[0] = c[0] * l; colour[1] = c[1] * l; colour[2] = c[2] * l; colour[3] = c[3];
        return false;
    }
    case CPV_PROGRAM_FETCH: {
        /* K: specialisation constant 0 (default 3); S = K * 8 + 8 folded in
         * 32-bit integers (OpSpecConstantOp IMul, IAdd). */
        const uint32_t k = spec_k ? spec_k : 3u;
        const int32_t scale = static_cast<int32_t>(k * 8u + 8u);
        const float sf = static_cast<float>(scale);                 /* OpConvertSToF */
        const int32_t px = static_cast<int32_t>(in[0] * sf);        /* OpVectorTimesScalar, OpConvertFToS */
        const int32_t py = static_cast<int32_t>(in[1] * sf);
        /* ImageFetch (CPVulkan/GlslFunctions.cpp:674-742): level 0 whatever
         * the Lod operand, zeros outside it; OpCopyMemory copies it as is */
        float t[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        if (r.texture && r.texture->levels > 0 && px >= 0 && py >= 0 && px < static_cast<int32_t>(r.texture->level_w[0]) &&
            py < static_cast<int32_t>(r.texture->level_h[0]))
            get_texel(*r.texture, 0, px, py, 0, t);
        const uint32_t bits = static_cast<uint32_t>(__builtin_popcount(static_cast<uint32_t>(px ^ py)));  /* OpBitCount */
        colour[0] = t[0]; colour[1] = t[1]; colour[2] = t[2];
        colour[3] = static_cast<float>(static_cast<int32_t>(bits)) / 16.0f;
        return false;
    }
    case CPV_PROGRAM_MESHPC: {
        float n[3];
        normalize3(in, n);
        const float light[3] = {0.48f, 0.6f, 0.64f};
        const float d = dot3(n, light);
        const float l0 = fmax_std(d, 0.0f);
        const float l1 = l0 * 0.8f;
        const float l = l1 + 0.2f;
        colour[0] = r.push[16] * l; colour[1] = r.push[17] * l; colour[2] = r.push[18] * l; colour[3] = r.push[19];
        return false;
    }
    default:
        for (int i = 0; i < 4; i++) colour[i] = 0.0f;
        return false;
    }
}

/* ---------------------------------------------------------------------- */
/* Attachments                                                             */
/* ---------------------------------------------------------------------- */

uint32_t depth_texel_size(uint32_t fmt) {
    switch (fmt) {
    case FMT_D16_UNORM: return 2;
    case FMT_D32_SFLOAT: return 4;
    case FMT_D32_SFLOAT_S8_UINT: return 8;
    default: return 0;
    }
}

bool has_stencil(uint32_t fmt) { return fmt == FMT_D32_SFLOAT_S8_UINT; }

/* Depth decode (LLVMRuntime/ImageCompiler.cpp:541-565). */
float get_depth(const uint8_t* texel, uint32_t fmt) {
    if (fmt == FMT_D16_UNORM) {
        uint16_t u;
        std::memcpy(&u, texel, 2);
        return decode_unorm16(u);
    }
    float f;
    std::memcpy(&f, texel, 4);
    return f;
}

/* Depth/stencil encode (LLVMRuntime/ImageCompiler.cpp:869-947). */
void set_depth(uint8_t* texel, uint32_t fmt, float d) {
    if (fmt == FMT_D16_UNORM) {
        const uint16_t u = static_cast<uint16_t>(encode_unorm(d, 65535.0f));
        std::memcpy(texel, &u, 2);
    } else {
        std::memcpy(texel, &d, 4);
    }
}

/* A colour attachment format (CPVulkanBase/Formats.cpp): bytes per texel,
 * channels, bytes per channel, kind (0 UNORM, 1 SNORM, 2 SFLOAT) and the
 * byte offset of each channel (B8G8R8A8: Formats.cpp:248,255). False for
 * formats the oracle does not write. */
struct ColourFormat {
    uint32_t bytes, channels, esize, kind;
    int off[4];
};
bool colour_format(uint32_t fmt, ColourFormat& cf) {
    switch (fmt) {
    case FMT_R8G8B8A8_UNORM: cf = {4, 4, 1, 0, {0, 1, 2, 3}}; return true;
    case FMT_B8G8R8A8_UNORM: cf = {4, 4, 1, 0, {2, 1, 0, 3}}; return true;
    case 9: cf = {1, 1, 1, 0, {0, 0, 0, 0}}; return true;    /* R8_UNORM */
    case 16: cf = {2, 2, 1, 0, {0, 1, 0, 0}}; return true;   /* R8G8_UNORM */
    case 38: cf = {4, 4, 1, 1, {0, 1, 2, 3}}; return true;   /* R8G8B8A8_SNORM */
    case 70: cf = {2, 1, 2, 0, {0, 0, 0, 0}}; return true;   /* R16_UNORM */
    case 77: cf = {4, 2, 2, 0, {0, 2, 0, 0}}; return true;   /* R16G16_UNORM */
    case 83: cf = {4, 2, 2, 2, {0, 2, 0, 0}}; return true;   /* R16G16_SFLOAT */
    case 100: cf = {4, 1, 4, 2, {0, 0, 0, 0}}; return true;  /* R32_SFLOAT */
    /* integer formats: kind 3 UINT, 4 SINT */
    case 13: cf = {1, 1, 1, 3, {0, 0, 0, 0}}; return true;   /* R8_UINT */
    case 14: cf = {1, 1, 1, 4, {0, 0, 0, 0}}; return true;   /* R8_SINT */
    case 20: cf = {2, 2, 1, 3, {0, 1, 0, 0}}; return true;   /* R8G8_UINT */
    case 21: cf = {2, 2, 1, 4, {0, 1, 0, 0}}; return true;   /* R8G8_SINT */
    case 41: cf = {4, 4, 1, 3, {0, 1, 2, 3}}; return true;   /* R8G8B8A8_UINT */
    case 42: cf = {4, 4, 1, 4, {0, 1, 2, 3}}; return true;   /* R8G8B8A8_SINT */
    case 74: cf = {2, 1, 2, 3, {0, 0, 0, 0}}; return true;   /* R16_UINT */
    case 75: cf = {2, 1, 2, 4, {0, 0, 0, 0}}; return true;   /* R16_SINT */
    case 81: cf = {4, 2, 2, 3, {0, 2, 0, 0}}; return true;   /* R16G16_UINT */
    case 82: cf = {4, 2, 2, 4, {0, 2, 0, 0}}; return true;   /* R16G16_SINT */
    case 98: cf = {4, 1, 4, 3, {0, 0, 0, 0}}; return true;   /* R32_UINT */
    case 99: cf = {4, 1, 4, 4, {0, 0, 0, 0}}; return true;   /* R32_SINT */
    /* 8- and 16-byte texels */
    case 91: cf = {8, 4, 2, 0, {0, 2, 4, 6}}; return true;   /* R16G16B16A16_UNORM */
    case 95: cf = {8, 4, 2, 3, {0, 2, 4, 6}}; return true;   /* R16G16B16A16_UINT */
    case 96: cf = {8, 4, 2, 4, {0, 2, 4, 6}}; return true;   /* R16G16B16A16_SINT */
    case 97: cf = {8, 4, 2, 2, {0, 2, 4, 6}}; return true;   /* R16G16B16A16_SFLOAT */
    case 101: cf = {8, 2, 4, 3, {0, 4, 0, 0}}; return true;  /* R32G32_UINT */
    case 102: cf = {8, 2, 4, 4, {0, 4, 0, 0}}; return true;  /* R32G32_SINT */
    case 103: cf = {8, 2, 4, 2, {0, 4, 0, 0}}; return true;  /* R32G32_SFLOAT */
    case 107: cf = {16, 4, 4, 3, {0, 4, 8, 12}}; return true;  /* R32G32B32A32_UINT */
    case 108: cf = {16, 4, 4, 4, {0, 4, 8, 12}}; return true;  /* R32G32B32A32_SINT */
    case 109: cf = {16, 4, 4, 2, {0, 4, 8, 12}}; return true;  /* R32G32B32A32_SFLOAT */
    default: return false;
    }
}

/* An integer channel from a 32-bit integer value: UINT clamped to the
 * channel's maximum, SINT to its range (LLVMRuntime/ImageCompiler.cpp:1121-1175). */
uint32_t encode_integer(uint32_t bits, const ColourFormat& cf) {
    const uint32_t width = 8 * cf.esize;
    if (width >= 32) return bits;
    if (cf.kind == 3) {
        const uint32_t m = (1u << width) - 1u;
        return bits < m ? bits : m;
    }
    const int32_t hi = (1 << (width - 1)) - 1, lo = -hi - 1;
    int32_t v = static_cast<int32_t>(bits);
    v = v > lo ? v : lo;
    v = v < hi ? v : hi;
    return static_cast<uint32_t>(v);
}

/* One stored channel → float: the reference's pixel decoder
 * (LLVMRuntime/ImageCompiler.cpp:161-230): UNORM and SNORM divided by
 * their type's maximum (SNORM not clamped), half floats widened through
 * the compiler's own binary16 type, 32-bit floats as stored. */
float decode_channel(const uint8_t* p, const ColourFormat& cf) {
    uint32_t raw = 0;
    std::memcpy(&raw, p, cf.esize);
    if (cf.kind == 2) {
        if (cf.esize == 2) {
            _Float16 h;
            const uint16_t r16 = static_cast<uint16_t>(raw);
            std::memcpy(&h, &r16, 2);
            return static_cast<float>(h);
        }
        float f;
        std::memcpy(&f, &raw, 4);
        return f;
    }
    if (cf.kind == 1) {
        const int32_t v = cf.esize == 1 ? static_cast<int8_t>(raw) : static_cast<int16_t>(raw);
        return static_cast<float>(v) / (cf.esize == 1 ? 127.0f : 32767.0f);
    }
    return cf.esize == 1 ? decode_unorm8(static_cast<uint8_t>(raw)) : decode_unorm16(static_cast<uint16_t>(raw));
}

/* float → stored channel: the reference's colour encoder
 * (LLVMRuntime/ImageCompiler.cpp:1077-1185): UNORM and SNORM clamped with
 * minnum / maxnum, scaled and rounded half away from zero; half floats by a
 * round-to-nearest-even narrowing; 32-bit floats unchanged. */
void encode_channel(float x, const ColourFormat& cf, uint8_t* p) {
    uint32_t raw;
    if (cf.kind >= 3) {
        /* an integer attachment reads the output's 32 bits as an integer */
        uint32_t bits;
        std::memcpy(&bits, &x, 4);
        raw = encode_integer(bits, cf);
    } else if (cf.kind == 0) {
        raw = encode_unorm(x, cf.esize == 1 ? 255.0f : 65535.0f);
    } else if (cf.kind == 1) {
        const float v = std::round(minnum(maxnum(x, -1.0f), 1.0f) * (cf.esize == 1 ? 127.0f : 32767.0f));
        raw = static_cast<uint32_t>(static_cast<int32_t>(v));
    } else if (cf.esize == 2) {
        const _Float16 h = static_cast<_Float16>(x);
        uint16_t r16;
        std::memcpy(&r16, &h, 2);
        raw = r16;
    } else {
        std::memcpy(&raw, &x, 4);
    }
    std::memcpy(p, &raw, cf.esize);
}

void set_colour(uint8_t* texel, uint32_t fmt, const float c[4]) {
    ColourFormat cf;
    if (!colour_format(fmt, cf)) return;
    for (uint32_t i = 0; i < cf.channels; i++) encode_channel(c[i], cf, texel + cf.off[i]);
}

/* The render pass's clear of one texel: an integer attachment is cleared
 * with the integer values round(clear * 100) (the scene contract; the
 * harness passes them as VkClearColorValue.int32), other formats with the
 * clear colour through their encoder. */
void clear_colour(uint8_t* texel, uint32_t fmt, const float c[4]) {
    ColourFormat cf;
    if (!colour_format(fmt, cf)) return;
    if (cf.kind < 3) {
        set_colour(texel, fmt, c);
        return;
    }
    for (uint32_t i = 0; i < cf.channels; i++) {
        const uint32_t raw = encode_integer(static_cast<uint32_t>(static_cast<int32_t>(std::lround(c[i] * 100.0f))), cf);
        std::memcpy(texel + cf.off[i], &raw, cf.esize);
    }
}

/* The texel as the reference decodes it; absent channels read 0, 0, 0, 1. */
void get_colour(const uint8_t* texel, uint32_t fmt, float c[4]) {
    ColourFormat cf;
    c[0] = c[1] = c[2] = 0.0f;
    c[3] = 1.0f;
    if (!colour_format(fmt, cf)) return;
    for (uint32_t i = 0; i < cf.channels; i++) c[i] = decode_channel(texel + cf.off[i], cf);
}

/* Stencil compare / ops (LLVMRuntime/PipelineCompiler.cpp:1194-1223,
 * 1382-1413, 1492-1526). Increment/decrement-and-clamp use the reference's
 * *signed* saturating i8 intrinsics. */
bool icompare(uint32_t a, uint32_t b, uint32_t op) {
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

bool fcompare(float a, float b, uint32_t op) {
    switch (op) {
    case 0: return false;
    case 1: return a < b;
    case 2: return a == b;
    case 3: return a <= b;
    case 4: return a > b;
    case 5: return (a < b) || (a > b); /* FCmpONE: ordered and not equal */
    case 6: return a >= b;
    default: return true;
    }
}

uint8_t stencil_op(uint32_t op, uint8_t current, uint8_t reference) {
    const int8_t sc = static_cast<int8_t>(current);
    switch (op) {
    case 0: return current;
    case 1: return 0;
    case 2: return reference;
    case 3: return static_cast<uint8_t>(sc == 127 ? 127 : sc + 1);
    case 4: return static_cast<uint8_t>(sc == -128 ? -128 : sc - 1);
    case 5: return static_cast<uint8_t>(~current);
    case 6: return static_cast<uint8_t>(current + 1);
    case 7: return static_cast<uint8_t>(current - 1);
    default: return current;
    }
}

/* ---------------------------------------------------------------------- */
/* Draw                                                                    */
/* ---------------------------------------------------------------------- */

struct Frame {
    const cpv_scene* s;
    uint8_t* colour;
    uint8_t* depth;
    uint32_t depth_size;
    uint32_t colour_size;  /* bytes per colour texel */
    uint8_t* extra[CPV_SCENE_MAX_EXTRA_COLOR] = {};       /* colour attachments 1 .. (null: unused or not given) */
    uint32_t extra_size[CPV_SCENE_MAX_EXTRA_COLOR] = {};  /* their bytes per texel */
    Resources res;
    cpv_oracle_stats* stats;
    /* Rows this frame writes: y % row_stride == row_index (1, 0: all rows).
     * The threaded entry gives each thread its own interleaved rows; every
     * pixel is then written by one thread, in API order. */
    uint32_t row_stride = 1, row_index = 0;
    bool count_prims = true;  /* count primitives (one thread of several) */
};

/* The first row >= start that the frame writes. */
int64_t first_row(const Frame& f, int64_t start) {
    const int64_t r = start % f.row_stride;
    return start + (static_cast<int64_t>(f.row_index) + f.row_stride - r) % f.row_stride;
}

/* Layout of a vertex attribute format: components, bytes per component,
 * kind (0 float32, 1 normalised 8/16-bit, 2 float16), signedness and
 * the B8G8R8A8 channel order (CPVulkanBase/Formats.cpp). False for formats
 * the oracle does not convert. */
bool attribute_layout(uint32_t format, int& comps, int& esize, int& kind, bool& sgn, bool& bgra) {
    sgn = bgra = false;
    kind = 1;
    switch (format) {
    case FMT_R32_SFLOAT: comps = 1; esize = 4; kind = 0; return true;
    case FMT_R32G32_SFLOAT: comps = 2; esize = 4; kind = 0; return true;
    case FMT_R32G32B32_SFLOAT: comps = 3; esize = 4; kind = 0; return true;
    case FMT_R32G32B32A32_SFLOAT: comps = 4; esize = 4; kind = 0; return true;
    case 9: comps = 1; esize = 1; return true;
    case 10: comps = 1; esize = 1; sgn = true; return true;
    case 16: comps = 2; esize = 1; return true;
    case 17: comps = 2; esize = 1; sgn = true; return true;
    case 23: comps = 3; esize = 1; return true;
    case 24: comps = 3; esize = 1; sgn = true; return true;
    case 37: comps = 4; esize = 1; return true;
    case 38: comps = 4; esize = 1; sgn = true; return true;
    case 44: comps = 4; esize = 1; bgra = true; return true;
    case 70: comps = 1; esize = 2; return true;
    case 71: comps = 1; esize = 2; sgn = true; return true;
    case 77: comps = 2; esize = 2; return true;
    case 78: comps = 2; esize = 2; sgn = true; return true;
    case 84: comps = 3; esize = 2; return true;
    case 85: comps = 3; esize = 2; sgn = true; return true;
    case 91: comps = 4; esize = 2; return true;
    case 92: comps = 4; esize = 2; sgn = true; return true;
    case 76: comps = 1; esize = 2; kind = 2; return true;
    case 83: comps = 2; esize = 2; kind = 2; return true;
    case 90: comps = 3; esize = 2; kind = 2; return true;
    case 97: comps = 4; esize = 2; kind = 2; return true;
    default: return false;
    }
}

/* IEEE binary16 → binary32 (exact; fpext of the reference's half loads). */
float half_to_float(uint16_t h) {
    const uint32_t sign = static_cast<uint32_t>(h & 0x8000u) << 16;
    const int exp = (h >> 10) & 0x1F;
    const uint32_t man = h & 0x3FFu;
    float f;
    if (exp == 0x1F) {
        const uint32_t bits = sign | 0x7F800000u | (man << 13) | (man ? 0x00400000u : 0u);
        std::memcpy(&f, &bits, 4);
        return f;
    }
    if (exp == 0) f = std::ldexp(static_cast<float>(man), -24);           /* zero or subnormal: man x 2^-24 */
    else f = std::ldexp(static_cast<float>(man | 0x400u), exp - 25);       /* (1024 + man) x 2^(exp - 25) */
    return sign ? -f : f;
}

/* One channel of a normalised 8/16-bit attribute as the reference's pixel
 * decoder returns it (LLVMRuntime/ImageCompiler.cpp:15-101, 161-230): the
 * integer converted to float and divided by its type's maximum; signed
 * values are not clamped, so the most negative code reads below -1. */
float decode_norm(uint32_t raw, int esize, bool sgn) {
    if (!sgn) return static_cast<float>(raw) / (esize == 1 ? 255.0f : 65535.0f);
    const int32_t v = esize == 1 ? static_cast<int8_t>(raw) : static_cast<int16_t>(raw);
    return static_cast<float>(v) / (esize == 1 ? 127.0f : 32767.0f);
}

/* An attribute's components from its bytes, into out[0..comps). */
void decode_attribute(const uint8_t* p, int comps, int esize, int kind, bool sgn, bool bgra, float out[4]) {
    for (int c = 0; c < comps; c++) {
        const int ch = (bgra && c < 3) ? 2 - c : c;
        const uint8_t* e = p + ch * esize;
        if (kind == 0) {
            std::memcpy(&out[c], e, 4);
        } else {
            const uint32_t raw = esize == 1 ? e[0] : static_cast<uint32_t>(e[0] | (e[1] << 8));
            out[c] = kind == 2 ? half_to_float(static_cast<uint16_t>(raw)) : decode_norm(raw, esize, sgn);
        }
    }
}

/* Attribute fetch (LLVMRuntime/PipelineCompiler.cpp:821-896): address =
 * binding base + stride * (vertex or instance id) + attribute offset; float
 * formats copy straight, normalised 8/16-bit formats go through the pixel
 * decoder, half floats are widened; components absent from the format read
 * 0,0,0,1. Reads outside the vertex blob return zeros. */
void fetch_attributes(const Frame& f, const cpv_scene_pipeline& p, const cpv_scene_draw& d, uint32_t vertex_id, uint32_t instance_id, float attr[8][4]) {
    for (int l = 0; l < 8; l++) { attr[l][0] = 0; attr[l][1] = 0; attr[l][2] = 0; attr[l][3] = 1; }
    for (uint32_t a = 0; a < p.num_attributes; a++) {
        const cpv_scene_attribute& at = p.attributes[a];
        if (at.location >= 8) continue;
        uint32_t slot = 0;
        const cpv_scene_binding* b = nullptr;
        for (uint32_t i = 0; i < p.num_bindings; i++) {
            if (p.bindings[i].binding == at.binding) { b = &p.bindings[i]; slot = i; }
        }
        if (!b) continue;
        int comps = 0, esize = 4, kind = 0;
        bool sgn = false, bgra = false;
        if (!attribute_layout(at.format, comps, esize, kind, sgn, bgra)) continue;
        const uint64_t index = (b->input_rate == RATE_VERTEX) ? vertex_id : instance_id;
        const uint64_t off = d.vertex_offsets[slot] + static_cast<uint64_t>(b->stride) * index + at.offset;
        if (off + static_cast<uint64_t>(comps) * esize > f.s->vertex_bytes) continue;
        decode_attribute(f.s->vertex_data + off, comps, esize, kind, sgn, bgra, attr[at.location]);
    }
}

struct Assembled {
    std::vector<uint32_t> vertex_id;   /* per assembled vertex (rawId order) */
    std::vector<uint32_t> prims;       /* provoking, v0, v1, v2 per triangle */
};

/* Primitives assemble() makes from `n` vertices. */
size_t primitive_count(uint32_t topology, uint32_t n) {
    switch (topology) {
    case TOPO_POINT_LIST: return n;
    case TOPO_LINE_LIST: return n / 2;
    case TOPO_LINE_STRIP: return n > 0 ? n - 1 : 0;
    case TOPO_TRIANGLE_LIST: return n / 3;
    default: return n > 1 ? n - 2 : 0;  /* strip, fan */
    }
}

/* Input assembly (CPVulkan/CommandBuffer.Draw.cpp:567-760) of vertices
 * [v0, v1) and primitives [p0, p1) into `out`, whose arrays are already
 * sized (d.count vertex ids, 4 entries per primitive); `base` is added to
 * every primitive entry. */
void assemble_range(const Frame& f, const cpv_scene_pipeline& p, const cpv_scene_draw& d, Assembled& out, size_t v0, size_t v1, size_t p0,
                    size_t p1, uint32_t base) {
    if (d.indexed) {
        const uint32_t isz = f.s->index_type == 0 ? 2 : 4;
        for (size_t i = v0; i < v1; i++) {
            const uint64_t off = d.index_offset + (static_cast<uint64_t>(d.first) + i) * isz;
            uint32_t index = 0;
            if (off + isz <= f.s->index_bytes) {
                if (isz == 2) { uint16_t v; std::memcpy(&v, f.s->index_data + off, 2); index = v; }
                else std::memcpy(&index, f.s->index_data + off, 4);
            }
            out.vertex_id[i] = static_cast<uint32_t>(d.vertex_offset) + index;
        }
    } else {
        for (size_t i = v0; i < v1; i++) out.vertex_id[i] = d.first + static_cast<uint32_t>(i);
    }
    for (size_t i = p0; i < p1; i++) {
        uint32_t* e = out.prims.data() + 4 * i;
        const uint32_t k = static_cast<uint32_t>(i);
        switch (p.topology) {
        case TOPO_POINT_LIST: e[0] = e[1] = e[2] = e[3] = k; break;
        case TOPO_LINE_LIST: e[0] = e[1] = 2 * k; e[2] = e[3] = 2 * k + 1; break;
        case TOPO_LINE_STRIP: e[0] = e[1] = k; e[2] = e[3] = k + 1; break;
        case TOPO_TRIANGLE_LIST: e[0] = e[1] = 3 * k; e[2] = 3 * k + 1; e[3] = 3 * k + 2; break;
        case TOPO_TRIANGLE_STRIP: e[0] = e[1] = k; e[2] = k + 1; e[3] = k + 2; break;
        default: /* fan */ e[0] = k + 1; e[1] = 0; e[2] = k + 1; e[3] = k + 2; break;
        }
        for (int j = 0; j < 4; j++) e[j] += base;
    }
}

/* Input assembly (CPVulkan/CommandBuffer.Draw.cpp:567-760): vertex ids per
 * assembled vertex and (provoking, v0, v1, v2) per primitive. */
void assemble(const Frame& f, const cpv_scene_pipeline& p, const cpv_scene_draw& d, Assembled& out) {
    const size_t prims = primitive_count(p.topology, d.count);
    out.vertex_id.resize(d.count);
    out.prims.resize(4 * prims);
    assemble_range(f, p, d, out, 0, d.count, 0, prims, 0);
}

/* The 16 logical operations on one UNORM8 channel (Vulkan 1.1, "Logical
 * Operations"): s is the fragment's encoded value, d the stored one. The
 * reference aborts on logicOpEnable (LLVMRuntime/PipelineCompiler.cpp:1687-1690). */
uint8_t logic_op(uint32_t op, uint8_t s, uint8_t d) {
    uint32_t r = 0;
    switch (op) {
    case 0: r = 0; break;                  // CLEAR
    case 1: r = s & d; break;              // AND
    case 2: r = s & ~d; break;             // AND_REVERSE
    case 3: r = s; break;                  // COPY
    case 4: r = ~s & d; break;             // AND_INVERTED
    case 5: r = d; break;                  // NO_OP
    case 6: r = s ^ d; break;              // XOR
    case 7: r = s | d; break;              // OR
    case 8: r = ~(s | d); break;           // NOR
    case 9: r = ~(s ^ d); break;           // EQUIVALENT
    case 10: r = ~d; break;                // INVERT
    case 11: r = s | ~d; break;            // OR_REVERSE
    case 12: r = ~s; break;                // COPY_INVERTED
    case 13: r = ~s | d; break;            // OR_INVERTED
    case 14: r = ~(s & d); break;          // NAND
    default: r = 0xFF; break;              // SET
    }
    return static_cast<uint8_t>(r);
}

/* Colour write of a fragment that passed its tests
 * (LLVMRuntime/PipelineCompiler.cpp:1415-1429, 1528-1727): a logic op on the
 * encoded channels, else the blend (the reference's ApplyBlend,
 * CPVulkan/CommandBuffer.Draw.cpp:956-1262), else the colour itself; then the
 * colour write mask keeps the stored byte of every channel it leaves out
 * (the reference aborts on a partial mask, PipelineCompiler.cpp:1693-1700;
 * this follows Vulkan 1.1, "Color Write Mask"). */
void write_colour(uint8_t* texel, uint32_t fmt, const cpv_scene_pipeline& p, const cpv_scene_attachment_blend& b, const float colour[4]) {
    ColourFormat cf;
    if (!colour_format(fmt, cf)) return;
    uint8_t enc[4][4];
    if (p.logic_op_enable) {
        /* 8-bit normalised formats only: the op on the encoded bytes */
        for (uint32_t i = 0; i < cf.channels; i++) {
            encode_channel(colour[i], cf, enc[i]);
            enc[i][0] = logic_op(p.logic_op, enc[i][0], texel[cf.off[i]]);
        }
    } else {
        float out[4];
        if (b.blend_enable && cf.kind < 3) {  /* integer attachments are not blended (Vulkan 1.1, "Blending") */
            float dst[4];
            get_colour(texel, fmt, dst);
            blend(colour, dst, p.blend_constants, b.src_color, b.dst_color, b.color_op, b.src_alpha, b.dst_alpha, b.alpha_op, out);
        } else {
            for (int i = 0; i < 4; i++) out[i] = colour[i];
        }
        for (uint32_t i = 0; i < cf.channels; i++) encode_channel(out[i], cf, enc[i]);
    }
    for (uint32_t i = 0; i < cf.channels; i++)
        if ((b.color_write_mask >> i) & 1u) std::memcpy(texel + cf.off[i], enc[i], cf.esize);
}

/* The first colour attachment's blend state, from the pipeline's fields. */
cpv_scene_attachment_blend first_blend(const cpv_scene_pipeline& p) {
    return {p.blend_enable, p.src_color, p.dst_color, p.color_op, p.src_alpha, p.dst_alpha, p.alpha_op, p.color_write_mask};
}

/* Interpolation (CPVulkan/CommandBuffer.Draw.cpp:816-871). */
float interp_persp(const float pw[3], const float v[3], const float w[3]) {
    float num = 0.0f, den = 0.0f;
    for (int i = 0; i < 3; i++) {
        const float wv = w[i] * v[i];
        num = num + wv / pw[i];
        den = den + w[i] / pw[i];
    }
    return num / den;
}

float interp_linear(const float v[3], const float w[3]) {
    float r = 0.0f;
    for (int i = 0; i < 3; i++) r = r + w[i] * v[i];
    return r;
}

/* Per-fragment operations (LLVMRuntime/PipelineCompiler.cpp:1020-1429). */
void fragment(Frame& f, const cpv_scene_pipeline& p, uint32_t x, uint32_t y, float depth_mapped, bool front, const float* inputs,
              const Quad* quad = nullptr) {
    const cpv_scene* s = f.s;
    f.stats->fragments++;
    float colour[32];
    if (run_fs(p.program, inputs, f.res, colour, p.spec_k, quad)) return;

    const uint64_t pix = static_cast<uint64_t>(y) * s->width + x;
    uint8_t* ds = f.depth ? f.depth + pix * f.depth_size : nullptr;
    const bool has_depth_att = ds != nullptr;

    float current_depth = 0.0f;
    if ((p.depth_test || p.depth_bounds_test) && has_depth_att) current_depth = get_depth(ds, s->depth_format);
    /* Depth bounds test (CompileDepthBoundsTest, :1128-1166): the stored
     * depth outside [min, max] (unordered compares: NaN is outside) ends the
     * fragment before the stencil test, with no write of any kind. */
    if (p.depth_bounds_test && has_depth_att && (!(current_depth >= p.min_depth_bounds) || !(current_depth <= p.max_depth_bounds))) return;
    uint8_t current_stencil = 0;
    const bool stencil_on = p.stencil_test && has_depth_att && has_stencil(s->depth_format);
    if (stencil_on) current_stencil = ds[4];

    bool stencil_result = true;
    uint8_t stencil_ref = 0;
    const cpv_scene_stencil& st = front ? p.stencil_front : p.stencil_back;
    if (stencil_on) {
        stencil_ref = static_cast<uint8_t>(st.reference);
        const uint8_t mask = static_cast<uint8_t>(st.compare_mask);
        stencil_result = icompare(stencil_ref & mask, current_stencil & mask, st.compare_op);
    }
    bool depth_result = true;
    if (p.depth_test && has_depth_att) depth_result = fcompare(depth_mapped, current_depth, p.depth_compare);

    const bool attempt_depth_write = p.depth_test && p.depth_write && has_depth_att;
    if (stencil_on) {
        /* CompileStencilWrite (:1382-1470): depth is written when the depth
         * test passes, independent of the stencil result. */
        const uint8_t fail = stencil_op(st.fail_op, current_stencil, stencil_ref);
        const uint8_t dfail = stencil_op(st.depth_fail_op, current_stencil, stencil_ref);
        const uint8_t pass = stencil_op(st.pass_op, current_stencil, stencil_ref);
        uint8_t value = stencil_result ? (depth_result ? pass : dfail) : fail;
        const uint8_t wmask = static_cast<uint8_t>(st.write_mask);
        value = static_cast<uint8_t>((value & wmask) | (current_stencil & static_cast<uint8_t>(~wmask)));
        if (depth_result && attempt_depth_write) set_depth(ds, s->depth_format, depth_mapped);
        ds[4] = value;
    } else if (attempt_depth_write && depth_result) {
        set_depth(ds, s->depth_format, depth_mapped);
    }

    if (stencil_result && depth_result) {
        /* every colour attachment of the subpass, each with its output and
         * blend state (CompileWriteFragment, PipelineCompiler.cpp:1415-1429) */
        if (s->color_format) {
            write_colour(f.colour + pix * f.colour_size, s->color_format, p, first_blend(p), colour);
            for (uint32_t k = 0; k < s->extra_color_count; k++)
                if (f.extra[k]) write_colour(f.extra[k] + pix * f.extra_size[k], s->extra_color_formats[k], p, p.extra_blend[k], colour + 4 * (k + 1));
        }
        f.stats->fragments_written++;
    }
}

/* One triangle after set-up (CPVulkan/CommandBuffer.Draw.cpp:1510-1569,
 * 874-897): NDC positions with clip w, the screen box, |area|, facing. */
struct TriSetup {
    float P[3][4];
    float area;
    uint32_t provoking, v[3];
    int32_t start_x, start_y, end_x, end_y;
    bool front, culled;
};

/* The area, facing and cull test of GetFragmentInput
 * (CPVulkan/CommandBuffer.Draw.cpp:879-900), once per triangle. */
void setup_facing(TriSetup& ts, uint32_t cull_mode) {
    const float (&P)[3][4] = ts.P;
    float area = edge(P[0][0], P[0][1], P[1][0], P[1][1], P[2][0], P[2][1]);
    if (area < 0) {
        area = -area;
        ts.front = false;
    } else {
        ts.front = true;
    }
    ts.area = area;
    ts.culled = ((cull_mode & CULL_BACK) && !ts.front) || ((cull_mode & CULL_FRONT) && ts.front);
}

/* ProcessTriangles up to the pixel loop (CPVulkan/CommandBuffer.Draw.cpp:1510-1569)
 * and the area / facing / cull part of GetFragmentInput (:874-897), for the
 * triangle at as.prims[t]. */
void setup_triangle(const Frame& f, const cpv_scene_pipeline& p, const Assembled& as, const std::vector<VsOut>& vs, size_t t, TriSetup& ts) {
    const cpv_scene* s = f.s;
    const float vw = s->viewport[2], vh = s->viewport[3];
    const int32_t iw = f2i(vw), ih = f2i(vh);
    const int32_t fb_w = static_cast<int32_t>(s->width), fb_h = static_cast<int32_t>(s->height);
    ts.provoking = as.prims[t];
    uint32_t i0 = as.prims[t + 1], i1 = as.prims[t + 2], i2 = as.prims[t + 3];
    if (p.front_face == FRONT_FACE_CW) std::swap(i0, i2);
    ts.v[0] = i0, ts.v[1] = i1, ts.v[2] = i2;
    float (&P)[3][4] = ts.P;
    for (int k = 0; k < 3; k++) {
        const VsOut& v = vs[ts.v[k]];
        const float w = v.pos[3];
        P[k][0] = v.pos[0] / w;
        P[k][1] = v.pos[1] / w;
        P[k][2] = v.pos[2] / w;
        P[k][3] = w;
    }
    int32_t sx[3], sy[3];
    for (int k = 0; k < 3; k++) {
        sx[k] = f2i(((P[k][0] + 1.0f) * 0.5f) * vw);
        sy[k] = f2i(((P[k][1] + 1.0f) * 0.5f) * vh);
    }
    ts.start_x = std::max<int32_t>(0, std::min({sx[0], sx[1], sx[2]}));
    ts.start_y = std::max<int32_t>(0, std::min({sy[0], sy[1], sy[2]}));
    int64_t end_x = std::min<int64_t>(iw, static_cast<int64_t>(std::max({sx[0], sx[1], sx[2]})) + 1);
    int64_t end_y = std::min<int64_t>(ih, static_cast<int64_t>(std::max({sy[0], sy[1], sy[2]})) + 1);
    /* Pixels outside the attachment are never written (the reference
     * assumes viewport == framebuffer; this bound keeps the restatement
     * memory safe). */
    ts.end_x = static_cast<int32_t>(std::min<int64_t>(end_x, fb_w));
    ts.end_y = static_cast<int32_t>(std::min<int64_t>(end_y, fb_h));

    setup_facing(ts, p.cull_mode);
}

/* GetFragmentInput up to the varyings (CPVulkan/CommandBuffer.Draw.cpp:874-909)
 * at the pixel centre (xf, yf) of a set-up, uncull triangle: the three edge
 * functions in the facing's order, rejection when any is negative, the
 * weights divided by |area| and the screen-linear NDC depth. */
bool fragment_weights(const TriSetup& ts, float xf, float yf, float w[3], float& depth) {
    static const int kFront[3][2] = {{1, 2}, {2, 0}, {0, 1}};
    static const int kBack[3][2] = {{2, 1}, {0, 2}, {1, 0}};
    const int (*e)[2] = ts.front ? kFront : kBack;
    const float (&P)[3][4] = ts.P;
    for (int k = 0; k < 3; k++) {
        const float* a = P[e[k][0]];
        const float* b = P[e[k][1]];
        w[k] = edge(a[0], a[1], b[0], b[1], xf, yf);
    }
    if (w[0] < 0 || w[1] < 0 || w[2] < 0) return false;
    w[0] = w[0] / ts.area;
    w[1] = w[1] / ts.area;
    w[2] = w[2] / ts.area;
    depth = (P[0][2] * w[0] + P[1][2] * w[1]) + P[2][2] * w[2];
    return true;
}

/* The weights of fragment_weights at any pixel centre, covered or not: a
 * quad neighbour's barycentrics. */
void helper_weights(const TriSetup& ts, float xf, float yf, float w[3]) {
    static const int kFront[3][2] = {{1, 2}, {2, 0}, {0, 1}};
    static const int kBack[3][2] = {{2, 1}, {0, 2}, {1, 0}};
    const int (*e)[2] = ts.front ? kFront : kBack;
    for (int k = 0; k < 3; k++) {
        const float* a = ts.P[e[k][0]];
        const float* b = ts.P[e[k][1]];
        w[k] = edge(a[0], a[1], b[0], b[1], xf, yf) / ts.area;
    }
}

/* The varyings of GetFragmentInput (SetDatum, CPVulkan/CommandBuffer.Draw.cpp:816-869,
 * 911-951): perspective, linear or the provoking vertex's value, per float
 * component in declaration order. */
void fragment_inputs(const ProgramInfo& info, const TriSetup& ts, const std::vector<VsOut>& vs, const float w[3], float* inputs) {
    const VsOut* v[3] = {&vs[ts.v[0]], &vs[ts.v[1]], &vs[ts.v[2]]};
    const float pw[3] = {ts.P[0][3], ts.P[1][3], ts.P[2][3]};
    int comp = 0;
    for (int in = 0; in < info.num_inputs; in++) {
        for (int c = 0; c < info.input_size[in]; c++, comp++) {
            const float val[3] = {v[0]->var[comp], v[1]->var[comp], v[2]->var[comp]};
            switch (info.input_interp[in]) {
            case INTERP_PERSPECTIVE: inputs[comp] = interp_persp(pw, val, w); break;
            case INTERP_LINEAR: inputs[comp] = interp_linear(val, w); break;
            case INTERP_FLAT: inputs[comp] = vs[ts.provoking].var[comp]; break;
            }
        }
    }
}

/* The pixel loop of ProcessTriangles (CPVulkan/CommandBuffer.Draw.cpp:1571-1594)
 * with GetFragmentInput (:874-954) and DrawPixel's depth map (:1300-1313),
 * over the frame's rows. */
void raster_triangle(Frame& f, const cpv_scene_pipeline& p, const ProgramInfo& info, const TriSetup& ts, const std::vector<VsOut>& vs) {
    const cpv_scene* s = f.s;
    const float vw = s->viewport[2], vh = s->viewport[3];
    const float min_d = s->viewport[4], max_d = s->viewport[5];
    const float half_x = (1.0f / vw) * 0.5f;
    const float half_y = (1.0f / vh) * 0.5f;
    for (int64_t y = first_row(f, ts.start_y); y < ts.end_y; y += f.row_stride) {
        const float yf = (static_cast<float>(y) / vh + half_y) * 2.0f - 1.0f;
        for (int64_t x = ts.start_x; x < ts.end_x; x++) {
            const float xf = (static_cast<float>(x) / vw + half_x) * 2.0f - 1.0f;
            float w[3], depth;
            if (!fragment_weights(ts, xf, yf, w, depth)) continue;
            float inputs[kMaxVaryings];
            fragment_inputs(info, ts, vs, w, inputs);
            const float mapped = (max_d - min_d) * depth + min_d;
            if (s->spec_lod) {
                float nin[2][kMaxVaryings];
                for (int n = 0; n < 2; n++) {
                    const int64_t nx = n == 0 ? (x ^ 1) : x, ny = n == 0 ? y : (y ^ 1);
                    const float nxf = (static_cast<float>(nx) / vw + half_x) * 2.0f - 1.0f;
                    const float nyf = (static_cast<float>(ny) / vh + half_y) * 2.0f - 1.0f;
                    float nw[3];
                    helper_weights(ts, nxf, nyf, nw);
                    fragment_inputs(info, ts, vs, nw, nin[n]);
                }
                const Quad quad = {static_cast<uint32_t>(x & 1) | (static_cast<uint32_t>(y & 1) << 1), {nin[0], nin[1]}};
                fragment(f, p, static_cast<uint32_t>(x), static_cast<uint32_t>(y), mapped, ts.front, inputs, &quad);
                continue;
            }
            fragment(f, p, static_cast<uint32_t>(x), static_cast<uint32_t>(y), mapped, ts.front, inputs);
        }
    }
}

/* ProcessTriangles + GetFragmentInput + DrawPixel
 * (CPVulkan/CommandBuffer.Draw.cpp:874-954, 1300-1313, 1510-1594). */
void rasterise(Frame& f, const cpv_scene_pipeline& p, const Assembled& as, const std::vector<VsOut>& vs) {
    const ProgramInfo info = program_info(p.program);
    TriSetup ts;
    for (size_t t = 0; t + 4 <= as.prims.size(); t += 4) {
        if (f.count_prims) f.stats->triangles++;
        setup_triangle(f, p, as, vs, t, ts);
        if (!ts.culled) raster_triangle(f, p, info, ts, vs);
    }
}

/* ProcessPoints (CPVulkan/CommandBuffer.Draw.cpp:1315-1380): the point's
 * screen position (int)((ndc + 1) * 0.5 * (extent - 1)), a square of
 * ceil(size / 2) around it, and the pixels whose s = 0.5 + (x - sx) / size
 * and t (likewise) lie in [0, 1]; every fragment takes the vertex's outputs
 * unchanged and its NDC z, facing front. */
void rasterise_points(Frame& f, const cpv_scene_pipeline& p, const Assembled& as, const std::vector<VsOut>& vs) {
    const cpv_scene* s = f.s;
    const float vw = s->viewport[2], vh = s->viewport[3];
    const float min_d = s->viewport[4], max_d = s->viewport[5];
    for (size_t t = 0; t + 4 <= as.prims.size(); t += 4) {
        const VsOut& v = vs[as.prims[t + 1]];
        if (f.count_prims) f.stats->triangles++;
        const float w = v.pos[3];
        const float p0[3] = {v.pos[0] / w, v.pos[1] / w, v.pos[2] / w};
        const int64_t sx = f2i(((p0[0] + 1.0f) * 0.5f) * (vw - 1.0f));
        const int64_t sy = f2i(((p0[1] + 1.0f) * 0.5f) * (vh - 1.0f));
        const float size = v.point_size;
        const int64_t half = f2i(std::ceil(size / 2.0f));
        const int64_t start_x = std::max<int64_t>(0, sx - half), start_y = std::max<int64_t>(0, sy - half);
        int64_t end_x = std::min<int64_t>(f2i(vw), sx + half + 1), end_y = std::min<int64_t>(f2i(vh), sy + half + 1);
        end_x = std::min<int64_t>(end_x, s->width);
        end_y = std::min<int64_t>(end_y, s->height);
        for (int64_t y = first_row(f, start_y); y < end_y; y += f.row_stride) {
            for (int64_t x = start_x; x < end_x; x++) {
                const float ps = 0.5f + static_cast<float>(static_cast<int32_t>(x - sx)) / size;
                const float pt = 0.5f + static_cast<float>(static_cast<int32_t>(y - sy)) / size;
                if (!(ps >= 0 && pt >= 0 && ps <= 1 && pt <= 1)) continue;
                const float mapped = (max_d - min_d) * p0[2] + min_d;
                /* a point's inputs are the same at its quad neighbours */
                const Quad quad = {static_cast<uint32_t>(x & 1) | (static_cast<uint32_t>(y & 1) << 1), {v.var, v.var}};
                fragment(f, p, static_cast<uint32_t>(x), static_cast<uint32_t>(y), mapped, true, v.var, s->spec_lod ? &quad : nullptr);
            }
        }
    }
}

/* ProcessLines, rectangular mode (CPVulkan/CommandBuffer.Draw.cpp:1382-1508):
 * the quad p0 ± o, p1 ± o with o = (dir.y, -dir.x) * lineWidth / extent and
 * dir = normalize(p1 - p0) over (NDC x, y, z, clip w); every viewport pixel
 * centre inside all four edges is a fragment, its line parameter
 * t = dot(p - p0, p1 - p0) / (|p1 - p0| |p1 - p0|) weighting the two
 * vertices (1 - t, t) and its depth p0.z * t + p1.z * (1 - t). */
void rasterise_lines(Frame& f, const cpv_scene_pipeline& p, const Assembled& as, const std::vector<VsOut>& vs) {
    const cpv_scene* s = f.s;
    const float vw = s->viewport[2], vh = s->viewport[3];
    const float min_d = s->viewport[4], max_d = s->viewport[5];
    const float half_x = (1.0f / vw) * 0.5f;
    const float half_y = (1.0f / vh) * 0.5f;
    const float lw_x = p.line_width / vw, lw_y = p.line_width / vh;
    const ProgramInfo info = program_info(p.program);
    for (size_t t = 0; t + 4 <= as.prims.size(); t += 4) {
        const uint32_t provoking = as.prims[t];
        const VsOut* v[2] = {&vs[as.prims[t + 1]], &vs[as.prims[t + 2]]};
        if (f.count_prims) f.stats->triangles++;
        float P[2][4];
        for (int k = 0; k < 2; k++) {
            const float w = v[k]->pos[3];
            P[k][0] = v[k]->pos[0] / w;
            P[k][1] = v[k]->pos[1] / w;
            P[k][2] = v[k]->pos[2] / w;
            P[k][3] = w;
        }
        float dv[4];
        for (int i = 0; i < 4; i++) dv[i] = P[1][i] - P[0][i];
        const float dot4 = (dv[0] * dv[0] + dv[1] * dv[1]) + (dv[2] * dv[2] + dv[3] * dv[3]);
        const float inv = 1.0f / std::sqrt(dot4);
        const float dir_x = dv[0] * inv, dir_y = dv[1] * inv;
        const float ox = dir_y * lw_x, oy = -dir_x * lw_y;
        const float c00[2] = {P[0][0] + ox, P[0][1] + oy}, c01[2] = {P[0][0] - ox, P[0][1] - oy};
        const float c10[2] = {P[1][0] + ox, P[1][1] + oy}, c11[2] = {P[1][0] - ox, P[1][1] - oy};
        const float dx = P[1][0] - P[0][0], dy = P[1][1] - P[0][1];
        /* the line parameter, weights, varyings and depth at a pixel centre */
        auto line_inputs = [&](float xf, float yf, float* inputs) {
            const float num = (xf - P[0][0]) * dx + (yf - P[0][1]) * dy;
            const float len = std::sqrt(dx * dx + dy * dy);
            const float lt = num / (len * len);
            const float wts[2] = {1.0f - lt, lt};
            int comp = 0;
            for (int in = 0; in < info.num_inputs; in++) {
                for (int c = 0; c < info.input_size[in]; c++, comp++) {
                    switch (info.input_interp[in]) {
                    case INTERP_PERSPECTIVE: {
                        float n = 0.0f, d = 0.0f;
                        for (int k = 0; k < 2; k++) {
                            n = n + wts[k] * v[k]->var[comp] / P[k][3];
                            d = d + wts[k] / P[k][3];
                        }
                        inputs[comp] = n / d;
                        break;
                    }
                    case INTERP_LINEAR: {
                        float r = 0.0f;
                        for (int k = 0; k < 2; k++) r = r + wts[k] * v[k]->var[comp];
                        inputs[comp] = r;
                        break;
                    }
                    case INTERP_FLAT: inputs[comp] = vs[provoking].var[comp]; break;
                    }
                }
            }
            return P[0][2] * lt + P[1][2] * (1.0f - lt);
        };
        for (uint32_t y = f.row_index; static_cast<float>(y) < vh && y < s->height; y += f.row_stride) {
            const float yf = (static_cast<float>(y) / vh + half_y) * 2.0f - 1.0f;
            for (uint32_t x = 0; static_cast<float>(x) < vw && x < s->width; x++) {
                const float xf = (static_cast<float>(x) / vw + half_x) * 2.0f - 1.0f;
                if (!(edge(c00[0], c00[1], c01[0], c01[1], xf, yf) >= 0 && edge(c11[0], c11[1], c10[0], c10[1], xf, yf) >= 0 &&
                      edge(c10[0], c10[1], c00[0], c00[1], xf, yf) >= 0 && edge(c01[0], c01[1], c11[0], c11[1], xf, yf) >= 0))
                    continue;
                float inputs[kMaxVaryings];
                const float depth = line_inputs(xf, yf, inputs);
                const float mapped = (max_d - min_d) * depth + min_d;
                if (s->spec_lod) {
                    float nin[2][kMaxVaryings];
                    for (int n = 0; n < 2; n++) {
                        const uint32_t nx = n == 0 ? (x ^ 1u) : x, ny = n == 0 ? y : (y ^ 1u);
                        line_inputs((static_cast<float>(nx) / vw + half_x) * 2.0f - 1.0f, (static_cast<float>(ny) / vh + half_y) * 2.0f - 1.0f, nin[n]);
                    }
                    const Quad quad = {(x & 1u) | ((y & 1u) << 1), {nin[0], nin[1]}};
                    fragment(f, p, x, y, mapped, true, inputs, &quad);
                    continue;
                }
                fragment(f, p, x, y, mapped, true, inputs);
            }
        }
    }
}

void draw(Frame& f, const cpv_scene_draw& d) {
    const cpv_scene* s = f.s;
    if (d.pipeline >= s->num_pipelines) return;
    const cpv_scene_pipeline& p = s->pipelines[d.pipeline];
    float push[32] = {};
    std::memcpy(push, d.push, std::min<uint32_t>(d.push_size, sizeof(push)));
    f.res.push = push;
    Assembled as;
    std::vector<VsOut> vs;
    for (uint32_t i = 0; i < d.instance_count; i++) {
        const uint32_t instance = d.first_instance + i;
        assemble(f, p, d, as);
        vs.resize(as.vertex_id.size());
        for (size_t k = 0; k < as.vertex_id.size(); k++) {
            float attr[8][4];
            fetch_attributes(f, p, d, as.vertex_id[k], instance, attr);
            std::memset(&vs[k], 0, sizeof(VsOut));
            run_vs(p.program, attr, f.res, vs[k]);
        }
        f.stats->vs_invocations += as.vertex_id.size();
        if (p.topology == TOPO_POINT_LIST) rasterise_points(f, p, as, vs);
        else if (p.topology == TOPO_LINE_LIST || p.topology == TOPO_LINE_STRIP) rasterise_lines(f, p, as, vs);
        else rasterise(f, p, as, vs);
    }
    f.res.push = nullptr;
}

/* A reusable barrier for the threads of one threaded render. */
class Barrier {
public:
    explicit Barrier(uint32_t n) : n_(n) {}
    void wait() {
        std::unique_lock<std::mutex> lock(m_);
        const uint64_t gen = generation_;
        if (++waiting_ == n_) {
            waiting_ = 0;
            generation_++;
            cv_.notify_all();
        } else {
            cv_.wait(lock, [&] { return generation_ != gen; });
        }
    }

private:
    std::mutex m_;
    std::condition_variable cv_;
    uint32_t n_, waiting_ = 0;
    uint64_t generation_ = 0;
};

/* One draw instance of a batch of the threaded render: its assembly (with
 * primitive entries offset to index the batch's vertex outputs), push
 * constants, and its ranges in the batch's vertex and triangle arrays. */
struct Unit {
    uint32_t draw = 0, instance = 0;
    bool triangles = true;
    size_t vs_base = 0, tri_base = 0, tri_count = 0, prim_base = 0, prim_count = 0;
    float push[32] = {};
    Assembled as;
};

/* What the threads of one threaded render share: the current batch of draw
 * instances (consecutive in API order) and their vertex outputs and
 * triangle set-ups. */
struct Shared {
    explicit Shared(uint32_t n) : bar(n) {}
    std::vector<Unit> units;
    size_t used = 0;            /* units of the current batch */
    size_t prims = 0;           /* primitives of the current batch */
    std::vector<VsOut> vs;
    std::vector<TriSetup> tri;
    std::vector<uint32_t> rows;  /* start_y << 16 | end_y per triangle, 0 if culled */
    std::vector<uint16_t> owner; /* per row: the thread that writes it (y % threads) */
    uint32_t next_draw = 0, next_instance = 0;
    Barrier bar;
};

/* Fills the next batch: draw instances in API order from the cursor until
 * about 64k triangles (one large instance forms a batch of its own). */
void build_batch(Frame& f, Shared& sh, uint32_t end) {
    const cpv_scene* s = f.s;
    sh.used = 0;
    size_t nv = 0, nt = 0, np = 0;
    while (sh.next_draw < end && nt < 65536 && nv < 3 * 65536) {
        const cpv_scene_draw& d = s->draws[sh.next_draw];
        if (d.pipeline >= s->num_pipelines || sh.next_instance >= d.instance_count) {
            sh.next_draw++;
            sh.next_instance = 0;
            continue;
        }
        const cpv_scene_pipeline& p = s->pipelines[d.pipeline];
        if (sh.used == sh.units.size()) sh.units.emplace_back();
        Unit& u = sh.units[sh.used++];
        u.draw = sh.next_draw;
        u.instance = d.first_instance + sh.next_instance;
        u.triangles = p.topology != TOPO_POINT_LIST && p.topology != TOPO_LINE_LIST && p.topology != TOPO_LINE_STRIP;
        std::memset(u.push, 0, sizeof(u.push));
        std::memcpy(u.push, d.push, std::min<uint32_t>(d.push_size, sizeof(u.push)));
        /* assembly makes d.count vertices and primitive_count() primitives */
        const uint32_t c = d.count;
        u.vs_base = nv;
        u.tri_base = nt;
        u.prim_base = np;
        u.prim_count = primitive_count(p.topology, c);
        u.tri_count = u.triangles ? u.prim_count : 0;
        nv += c;
        nt += u.tri_count;
        np += u.prim_count;
        f.stats->vs_invocations += c;
        if (++sh.next_instance >= d.instance_count) {
            sh.next_draw++;
            sh.next_instance = 0;
        }
    }
    sh.vs.resize(nv);
    sh.tri.resize(nt);
    sh.rows.resize(nt);
    sh.prims = np;
}

/* The unit of the current batch holding element k of a per-unit range:
 * vertex outputs (0), triangles (1) or primitives (2). */
size_t unit_of(const Shared& sh, size_t k, int kind) {
    size_t lo = 0, hi = sh.used;
    while (hi - lo > 1) {
        const size_t mid = (lo + hi) / 2;
        const Unit& u = sh.units[mid];
        if ((kind == 0 ? u.vs_base : (kind == 1 ? u.tri_base : u.prim_base)) <= k) lo = mid;
        else hi = mid;
    }
    return lo;
}

/* The render of draws [begin, end) by thread `tid` of `n`: per batch, vertex
 * shading and triangle set-up split into contiguous ranges, then every
 * thread walks all primitives of the batch in API order over its own rows. */
void render_threaded(Frame& f, Shared& sh, uint32_t tid, uint32_t n, uint32_t end) {
    const cpv_scene* s = f.s;
    for (;;) {
        if (tid == 0) build_batch(f, sh, end);
        sh.bar.wait();
        if (sh.used == 0) break;
        const size_t nv = sh.vs.size(), nt = sh.tri.size();
        /* assembly: the units' arrays sized a unit per thread in turn, then
         * every thread fills its share of the batch's vertices and
         * primitives, the entries offset to index the batch's outputs */
        for (size_t u = tid; u < sh.used; u += n) {
            Unit& unit = sh.units[u];
            unit.as.vertex_id.resize(s->draws[unit.draw].count);
            unit.as.prims.resize(4 * unit.prim_count);
        }
        sh.bar.wait();
        {
            const size_t v0 = nv * tid / n, v1 = nv * (tid + 1) / n;
            const size_t q0 = sh.prims * tid / n, q1 = sh.prims * (tid + 1) / n;
            for (size_t u = v0 < v1 ? unit_of(sh, v0, 0) : sh.used; u < sh.used && sh.units[u].vs_base < v1; u++) {
                Unit& unit = sh.units[u];
                const cpv_scene_draw& d = s->draws[unit.draw];
                const size_t a = std::max(v0, unit.vs_base) - unit.vs_base, b = std::min(v1, unit.vs_base + d.count) - unit.vs_base;
                assemble_range(f, s->pipelines[d.pipeline], d, unit.as, a, b, 0, 0, 0);
            }
            for (size_t u = q0 < q1 ? unit_of(sh, q0, 2) : sh.used; u < sh.used && sh.units[u].prim_base < q1; u++) {
                Unit& unit = sh.units[u];
                const cpv_scene_draw& d = s->draws[unit.draw];
                const size_t a = std::max(q0, unit.prim_base) - unit.prim_base, b = std::min(q1, unit.prim_base + unit.prim_count) - unit.prim_base;
                assemble_range(f, s->pipelines[d.pipeline], d, unit.as, 0, 0, a, b, static_cast<uint32_t>(unit.vs_base));
            }
        }
        sh.bar.wait();
        /* vertex shading */
        size_t k = nv * tid / n;
        const size_t k1 = nv * (tid + 1) / n;
        for (size_t u = k < k1 ? unit_of(sh, k, 0) : sh.used; u < sh.used && k < k1; u++) {
            const Unit& unit = sh.units[u];
            const cpv_scene_draw& d = s->draws[unit.draw];
            const cpv_scene_pipeline& p = s->pipelines[d.pipeline];
            f.res.push = unit.push;
            const size_t stop = std::min(k1, unit.vs_base + unit.as.vertex_id.size());
            for (; k < stop; k++) {
                float attr[8][4];
                fetch_attributes(f, p, d, unit.as.vertex_id[k - unit.vs_base], unit.instance, attr);
                std::memset(&sh.vs[k], 0, sizeof(VsOut));
                run_vs(p.program, attr, f.res, sh.vs[k]);
            }
        }
        sh.bar.wait();
        /* triangle set-up */
        size_t j = nt * tid / n;
        const size_t j1 = nt * (tid + 1) / n;
        for (size_t u = j < j1 ? unit_of(sh, j, 1) : sh.used; u < sh.used && j < j1; u++) {
            const Unit& unit = sh.units[u];
            const cpv_scene_pipeline& p = s->pipelines[s->draws[unit.draw].pipeline];
            const size_t stop = std::min(j1, unit.tri_base + unit.tri_count);
            for (; j < stop; j++) {
                TriSetup& ts = sh.tri[j];
                setup_triangle(f, p, unit.as, sh.vs, (j - unit.tri_base) * 4, ts);
                f.stats->triangles++;
                sh.rows[j] = (ts.culled || ts.end_y <= ts.start_y) ? 0u : (static_cast<uint32_t>(ts.start_y) << 16 | static_cast<uint32_t>(ts.end_y));
            }
        }
        sh.bar.wait();
        /* raster, in API order, over this thread's rows */
        for (size_t u = 0; u < sh.used; u++) {
            const Unit& unit = sh.units[u];
            const cpv_scene_pipeline& p = s->pipelines[s->draws[unit.draw].pipeline];
            f.res.push = unit.push;
            if (unit.triangles) {
                const ProgramInfo info = program_info(p.program);
                for (size_t t = unit.tri_base; t < unit.tri_base + unit.tri_count; t++) {
                    const uint32_t r = sh.rows[t];
                    if (!r) continue;
                    const uint32_t y0 = r >> 16, y1 = r & 0xFFFFu;
                    bool mine = y1 - y0 >= n;
                    for (uint32_t y = y0; !mine && y < y1; y++) mine = sh.owner[y] == tid;
                    if (mine) raster_triangle(f, p, info, sh.tri[t], sh.vs);
                }
            } else {
                f.count_prims = tid == 0;
                if (p.topology == TOPO_POINT_LIST) rasterise_points(f, p, unit.as, sh.vs);
                else rasterise_lines(f, p, unit.as, sh.vs);
                f.count_prims = true;
            }
        }
        f.res.push = nullptr;
        sh.bar.wait();  /* before thread 0 builds the next batch */
    }
}

/* Checks a scene and fills the parts of `f` and `tex` every render needs. */
int prepare(const cpv_scene* scene, uint8_t* color, uint8_t* depth, Frame& f, Texture& tex, uint8_t* const* extra = nullptr) {
    if (!scene || !color) return -1;
    if (scene->extra_color_count > CPV_SCENE_MAX_EXTRA_COLOR) return -2;
    for (uint32_t k = 0; k < scene->extra_color_count; k++) {
        ColourFormat ecf{};
        const uint32_t fmt = scene->extra_color_formats[k];
        if (!fmt) continue;
        if (!colour_format(fmt, ecf)) return -2;
        f.extra[k] = extra ? extra[k] : nullptr;
        f.extra_size[k] = ecf.bytes;
    }
    ColourFormat cf{};
    if (scene->color_format != 0 && !colour_format(scene->color_format, cf)) return -2;
    if (scene->color_format == 0 && scene->depth_format == 0) return -2;
    const uint32_t dsize = depth_texel_size(scene->depth_format);
    if (scene->depth_format != 0 && (dsize == 0 || !depth)) return -3;
    if (scene->height > 0xFFFFu) return -2;
    f.s = scene;
    f.colour = color;
    f.depth = scene->depth_format ? depth : nullptr;
    f.depth_size = dsize;
    f.colour_size = cf.bytes;
    if (scene->texture_data) {
        tex.data = scene->texture_data;
        tex.bytes = scene->texture_bytes;
        tex.width = scene->texture_width;
        tex.height = scene->texture_height;
        tex.levels = std::min<uint32_t>(scene->texture_levels, 16);
        uint64_t off = 0;
        uint32_t w = tex.width, h = tex.height;
        /* GetNormalImageSize (CPVulkanBase/Formats.cpp:453-484). */
        for (uint32_t l = 0; l < tex.levels; l++) {
            tex.level_offset[l] = off;
            tex.level_w[l] = w;
            tex.level_h[l] = h;
            off += static_cast<uint64_t>(w) * h * 4u;
            w = std::max(w / 2, 1u);
            h = std::max(h / 2, 1u);
        }
        f.res.texture = &tex;
        f.res.sampler = &scene->sampler;
    }
    f.res.ubo = reinterpret_cast<const float*>(scene->uniform_data);
    f.res.ubo_floats = scene->uniform_bytes / 4;
    return 0;
}

/* BeginRenderPassCommand + ClearImage (CPVulkan/CommandBuffer.cpp:591-646,
 * CPVulkan/CommandBuffer.Draw.cpp:117-149): every texel goes through the
 * format encoder. */
void clear(const Frame& f) {
    const cpv_scene* scene = f.s;
    const uint64_t pixels = static_cast<uint64_t>(scene->width) * scene->height;
    if (scene->color_format) {  // a depth-only pass leaves `color` untouched
        for (uint64_t i = 0; i < pixels; i++) clear_colour(f.colour + i * f.colour_size, scene->color_format, scene->clear_color);
        for (uint32_t k = 0; k < scene->extra_color_count; k++)
            if (f.extra[k])
                for (uint64_t i = 0; i < pixels; i++) clear_colour(f.extra[k] + i * f.extra_size[k], scene->extra_color_formats[k], scene->clear_color);
    }
    if (f.depth) {
        for (uint64_t i = 0; i < pixels; i++) {
            uint8_t* t = f.depth + i * f.depth_size;
            set_depth(t, scene->depth_format, scene->clear_depth);
            if (has_stencil(scene->depth_format)) { t[4] = static_cast<uint8_t>(scene->clear_stencil); t[5] = t[6] = t[7] = 0; }
        }
    }
}

} // namespace

extern "C" {

int cpv_oracle_render(const cpv_scene* scene, uint8_t* color, uint8_t* depth, uint32_t do_clear, uint32_t draw_begin,
                      uint32_t draw_end, cpv_oracle_stats* stats) {
    return cpv_oracle_render_extra(scene, color, nullptr, depth, do_clear, draw_begin, draw_end, stats);
}

int cpv_oracle_render_extra(const cpv_scene* scene, uint8_t* color, uint8_t* const* extra, uint8_t* depth, uint32_t do_clear,
                            uint32_t draw_begin, uint32_t draw_end, cpv_oracle_stats* stats) {
    cpv_oracle_stats local{};
    Frame f{};
    Texture tex;
    const int r = prepare(scene, color, depth, f, tex, extra);
    if (r != 0) return r;
    f.stats = stats ? stats : &local;
    if (do_clear) clear(f);
    const uint32_t end = std::min(draw_end, scene->num_draws);
    for (uint32_t i = draw_begin; i < end; i++) draw(f, scene->draws[i]);
    return 0;
}

int cpv_oracle_render_threaded(const cpv_scene* scene, uint8_t* color, uint8_t* depth, uint32_t do_clear, uint32_t draw_begin,
                               uint32_t draw_end, uint32_t threads, cpv_oracle_stats* stats) {
    Frame base{};
    Texture tex;
    const int r = prepare(scene, color, depth, base, tex);
    if (r != 0) return r;
    cpv_oracle_stats dummy{};
    base.stats = &dummy;
    if (do_clear) clear(base);
    const uint32_t n = std::max(1u, std::min(threads, 256u));
    const uint32_t end = std::min(draw_end, scene->num_draws);
    Shared sh(n);
    sh.next_draw = draw_begin;
    sh.owner.resize(scene->height);
    for (uint32_t y = 0; y < scene->height; y++) sh.owner[y] = static_cast<uint16_t>(y % n);
    std::vector<cpv_oracle_stats> per(n);
    std::vector<std::thread> pool;
    for (uint32_t t = 0; t < n; t++) {
        pool.emplace_back([&, t] {
            Frame f = base;
            if (f.res.texture) f.res.texture = &tex;
            cpv_oracle_stats local{};  /* counted per fragment: kept off the other threads' cache lines */
            f.stats = &local;
            f.row_stride = n;
            f.row_index = t;
            render_threaded(f, sh, t, n, end);
            per[t] = local;
        });
    }
    for (std::thread& th : pool) th.join();
    if (stats) {
        *stats = cpv_oracle_stats{};
        for (const cpv_oracle_stats& st : per) {
            stats->triangles += st.triangles;
            stats->vs_invocations += st.vs_invocations;
            stats->fragments += st.fragments;
            stats->fragments_written += st.fragments_written;
        }
    }
    return 0;
}

float cpv_oracle_edge(float ax, float ay, float bx, float by, float cx, float cy) { return edge(ax, ay, bx, by, cx, cy); }

int cpv_oracle_decode_attribute(uint32_t format, const uint8_t* bytes, float out[4]) {
    int comps = 0, esize = 4, kind = 0;
    bool sgn = false, bgra = false;
    if (!attribute_layout(format, comps, esize, kind, sgn, bgra)) return -1;
    out[0] = out[1] = out[2] = 0.0f;
    out[3] = 1.0f;
    decode_attribute(bytes, comps, esize, kind, sgn, bgra, out);
    return comps;
}

void cpv_oracle_quad_lambda_n(const float* in, const uint32_t* odd, uint32_t width, uint32_t height, float* out, uint64_t n) {
    Texture t;
    t.levels = 1;
    t.level_w[0] = width;
    t.level_h[0] = height;
    for (uint64_t i = 0; i < n; i++) {
        const float* p = in + 6 * i;
        const float un[2] = {p[2], p[4]}, vn[2] = {p[3], p[5]};
        out[i] = quad_lambda(t, p[0], p[1], un, vn, odd[i]);
    }
}

void cpv_oracle_half_log2_n(const float* in, float* out, uint64_t n) {
    for (uint64_t i = 0; i < n; i++) out[i] = half_log2(in[i]);
}

void cpv_oracle_edge_n(const float* in, float* out, uint64_t n) {
    for (uint64_t i = 0; i < n; i++) {
        const float* p = in + 6 * i;
        out[i] = edge(p[0], p[1], p[2], p[3], p[4], p[5]);
    }
}

void cpv_oracle_wrap_n(const int32_t* v, const int32_t* size, const uint32_t* mode, int32_t* out, uint64_t n) {
    for (uint64_t i = 0; i < n; i++) out[i] = wrap(v[i], size[i], mode[i]);
}

void cpv_oracle_blend_n(const float* src, const float* dst, const float* constant, const uint32_t* modes, float* out, uint64_t n) {
    for (uint64_t i = 0; i < n; i++) {
        const uint32_t* m = modes + 6 * i;
        blend(src + 4 * i, dst + 4 * i, constant + 4 * i, m[0], m[1], m[2], m[3], m[4], m[5], out + 4 * i);
    }
}

void cpv_oracle_fragment_input_n(const float* pts, const float* vars, const uint32_t* cull, const uint32_t* provoking, float* out, uint64_t n) {
    const ProgramInfo info{3, {4, 4, 1}, {INTERP_PERSPECTIVE, INTERP_LINEAR, INTERP_FLAT}};
    std::vector<VsOut> vs(3);
    for (uint64_t i = 0; i < n; i++) {
        const float* p = pts + 14 * i;
        TriSetup ts{};
        for (int k = 0; k < 3; k++) {
            for (int c = 0; c < 4; c++) ts.P[k][c] = p[4 * k + c];
            ts.v[k] = static_cast<uint32_t>(k);
            std::memset(&vs[k], 0, sizeof(VsOut));
            for (int c = 0; c < 9; c++) vs[k].var[c] = vars[27 * i + 9 * k + c];
        }
        ts.provoking = provoking[i];
        setup_facing(ts, cull[i]);
        float w[3], depth = 0.0f, inputs[kMaxVaryings] = {};
        const bool covered = !ts.culled && fragment_weights(ts, p[12], p[13], w, depth);
        if (covered) fragment_inputs(info, ts, vs, w, inputs);
        float* o = out + 12 * i;
        o[0] = covered ? 1.0f : 0.0f;
        o[1] = ts.front ? 1.0f : 0.0f;
        o[2] = covered ? depth : 0.0f;
        for (int k = 0; k < 9; k++) o[3 + k] = covered ? inputs[k] : 0.0f;
    }
}

void cpv_oracle_sample_n(const uint8_t* texels, uint32_t width, uint32_t height, uint32_t levels, const uint32_t* modes, const float* uvl, float* out,
                         uint64_t n) {
    for (uint64_t i = 0; i < n; i++) {
        const uint32_t* m = modes + 6 * i;
        cpv_scene_sampler s{};
        s.mag_filter = m[0];
        s.min_filter = m[1];
        s.mipmap_mode = m[2];
        s.address_u = m[3];
        s.address_v = m[4];
        s.address_w = m[3];
        s.border_color = m[5];
        s.mip_lod_bias = 0.0f;
        s.min_lod = -1000.0f;
        s.max_lod = 1000.0f;
        cpv_oracle_sample(texels, width, height, levels, &s, uvl[3 * i], uvl[3 * i + 1], uvl[3 * i + 2], out + 4 * i);
    }
}
uint8_t cpv_oracle_encode_unorm8(float value) { return static_cast<uint8_t>(encode_unorm(value, 255.0f)); }
uint8_t cpv_oracle_logic_op(uint32_t op, uint8_t src, uint8_t dst) { return logic_op(op, src, dst); }
uint16_t cpv_oracle_encode_unorm16(float value) { return static_cast<uint16_t>(encode_unorm(value, 65535.0f)); }
float cpv_oracle_decode_unorm8(uint8_t value) { return decode_unorm8(value); }

void cpv_oracle_sample(const uint8_t* texels, uint32_t width, uint32_t height, uint32_t levels, const cpv_scene_sampler* sampler,
                       float u, float v, float lod, float out[4]) {
    Texture tex;
    tex.data = texels;
    tex.width = width;
    tex.height = height;
    tex.levels = std::min<uint32_t>(levels, 16);
    uint64_t off = 0;
    uint32_t w = width, h = height;
    for (uint32_t l = 0; l < tex.levels; l++) {
        tex.level_offset[l] = off;
        tex.level_w[l] = w;
        tex.level_h[l] = h;
        off += static_cast<uint64_t>(w) * h * 4u;
        w = std::max(w / 2, 1u);
        h = std::max(h / 2, 1u);
    }
    tex.bytes = off;
    sample(tex, *sampler, u, v, lod, out);
}

void cpv_oracle_blend(const float src[4], const float dst[4], const float constant[4], uint32_t src_color, uint32_t dst_color,
                      uint32_t color_op, uint32_t src_alpha, uint32_t dst_alpha, uint32_t alpha_op, float out[4]) {
    blend(src, dst, constant, src_color, dst_color, color_op, src_alpha, dst_alpha, alpha_op, out);
}

/* BlitImageCommand::Process for one 2D colour region between RGBA8/BGRA8
 * levels (CPVulkan/CommandBuffer.cpp:57-232): for each destination texel of
 * the region (negative extents walk from offset 1), the source position
 * u = (dstX + 0.5 - dst0.x) * ((src1.x - src0.x) / (dst1.x - dst0.x)) + src0.x
 * (and v) is normalised by the level size and sampled as SampleImage does
 * for a blit (the level as a one-level image, CLAMP_TO_EDGE, the blit's
 * filter); SetPixel encodes the result. The third axis of the reference has
 * depth 1: its lerp by 0 changes nothing. */
void cpv_oracle_blit(const uint8_t* src, uint32_t src_w, uint32_t src_h, uint32_t src_format, uint8_t* dst, uint32_t dst_w, uint32_t dst_h,
                     uint32_t dst_format, const int32_t region[8], uint32_t filter) {
    Texture tex;
    tex.data = src;
    tex.width = src_w;
    tex.height = src_h;
    tex.levels = 1;
    tex.level_w[0] = src_w;
    tex.level_h[0] = src_h;
    tex.bytes = static_cast<uint64_t>(src_w) * src_h * 4u;
    tex.format = src_format;
    cpv_scene_sampler s{};
    s.address_u = s.address_v = s.address_w = 2; /* CLAMP_TO_EDGE */
    const int32_t* r0 = region;      /* src x0, y0, x1, y1 */
    const int32_t* d0 = region + 4;  /* dst x0, y0, x1, y1 */
    int32_t dw = d0[2] - d0[0], dh = d0[3] - d0[1];
    const bool neg_w = dw < 0, neg_h = dh < 0;
    dw = neg_w ? -dw : dw;
    dh = neg_h ? -dh : dh;
    for (int32_t y = 0; y < dh; y++) {
        for (int32_t x = 0; x < dw; x++) {
            const int32_t dst_x = neg_w ? x + d0[2] : x + d0[0];
            const int32_t dst_y = neg_h ? y + d0[3] : y + d0[1];
            if (dst_x < 0 || dst_y < 0 || dst_x >= static_cast<int32_t>(dst_w) || dst_y >= static_cast<int32_t>(dst_h)) continue;
            const float u = (static_cast<float>(dst_x) + 0.5f - static_cast<float>(d0[0])) *
                                (static_cast<float>(r0[2] - r0[0]) / static_cast<float>(d0[2] - d0[0])) + static_cast<float>(r0[0]);
            const float v = (static_cast<float>(dst_y) + 0.5f - static_cast<float>(d0[1])) *
                                (static_cast<float>(r0[3] - r0[1]) / static_cast<float>(d0[3] - d0[1])) + static_cast<float>(r0[1]);
            float value[4];
            sample_level(tex, 0, u / static_cast<float>(src_w), v / static_cast<float>(src_h), filter, s, value);
            uint8_t* texel = dst + (static_cast<uint64_t>(dst_y) * dst_w + dst_x) * 4u;
            for (int c = 0; c < 4; c++) texel[(dst_format == 44 && c < 3) ? 2 - c : c] = static_cast<uint8_t>(encode_unorm(value[c], 255.0f));
        }
    }
}

} // extern "C"
