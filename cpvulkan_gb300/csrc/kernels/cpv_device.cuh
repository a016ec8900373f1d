/*
 * cpv_device.cuh — device-side types and arithmetic shared by every kernel of
 * the draw path: per-draw parameters, attachment codecs, the image sampler,
 * the edge function and primitive set-up, plus the value types that
 * translated SPIR-V shaders use.
 *
 * Compiled twice: by nvcc into libcpvulkan_gb300.so (the generic binning,
 * scan and clear kernels) and by NVRTC at vkCreateGraphicsPipelines, where
 * the translated shaders and the pipeline's fixed-function state are
 * prepended and cpv_pipeline.cuh instantiates the pipeline's kernels.
 *
 * Every arithmetic step that decides a pixel follows the reference CPU path
 * operation for operation (cited per function) and must be compiled with
 * -fmad=false, IEEE division and square root, and no flush-to-zero, so that
 * results are bit-identical to the reference's uncontracted binary32 code.
 */
#ifndef CPV_DEVICE_CUH
#define CPV_DEVICE_CUH

#include "cpv_params.h"

/* ------------------------------------------------------------------------- */
/* Scalar helpers                                                            */
/* ------------------------------------------------------------------------- */

/* static_cast<int32_t>(float) with the saturating semantics of the target
 * (cvt.rzi.s32.f32): the reference's screen bounding box conversion
 * (CPVulkan/CommandBuffer.Draw.cpp:1548-1563). */
__device__ __forceinline__ int32_t cpv_f2i(float f) { return __float2int_rz(f); }

/* std::max / std::min as the reference's GLSL helpers use them
 * (CPVulkan/GlslFunctions.cpp:106-130). */
__device__ __forceinline__ float cpv_std_max(float a, float b) { return (a < b) ? b : a; }
__device__ __forceinline__ float cpv_std_min(float a, float b) { return (b < a) ? b : a; }
__device__ __forceinline__ float cpv_std_clamp(float v, float lo, float hi) { return (v < lo) ? lo : ((hi < v) ? hi : v); }

/* UNORM encode (LLVMRuntime/ImageCompiler.cpp:27-32, 1081-1095):
 * minnum(maxnum(x,0),1) * (2^n-1), round half away from zero, to unsigned. */
__device__ __forceinline__ uint32_t cpv_encode_unorm(float x, float maxv) {
    float v = fminf(fmaxf(x, 0.0f), 1.0f);
    v = __fmul_rn(v, maxv);
    v = roundf(v); /* half away from zero, as llvm.round */
    return __float2uint_rz(v);
}

/* UNORM decode: uitofp then IEEE divide (LLVMRuntime/ImageCompiler.cpp:43-53). */
__device__ __forceinline__ float cpv_decode_unorm8(uint32_t u) { return __fdiv_rn(__uint2float_rn(u), 255.0f); }
__device__ __forceinline__ float cpv_decode_unorm16(uint32_t u) { return __fdiv_rn(__uint2float_rn(u), 65535.0f); }

/* In pipeline modules the 256 UNORM8 decodes are a table in shared memory,
 * filled with exactly cpv_decode_unorm8(0..255) by each kernel before use:
 * one shared-memory read instead of an IEEE divide per channel. */
#ifdef CPV_PIPELINE_MODULE
__shared__ float cpv_lut8[256];
#define CPV_DECODE8(u) cpv_lut8[(u)]
__device__ __forceinline__ void cpv_lut8_init() {
    for (uint32_t i = threadIdx.x; i < 256u; i += blockDim.x) cpv_lut8[i] = cpv_decode_unorm8(i);
}
#else
#define CPV_DECODE8(u) cpv_decode_unorm8(u)
#endif

/* EdgeFunction (CPVulkan/CommandBuffer.Draw.cpp:410-418). */
__device__ __forceinline__ float cpv_edge(float ax, float ay, float bx, float by, float cx, float cy) {
    const float t0 = __fmul_rn(__fsub_rn(cx, ax), __fsub_rn(by, ay));
    const float t1 = __fmul_rn(__fsub_rn(cy, ay), __fsub_rn(bx, ax));
    return __fsub_rn(t0, t1);
}

/* Bounds-checked reads of application memory. Out-of-range reads return
 * zero (the oracle defines the same), so no input can make a kernel read
 * outside the buffers it was given. Plain (generic) loads: the same helpers
 * read push constants, which live in the kernel's parameter block, not in
 * global memory, so the global-only read-only path (ld.global.nc) must not
 * be used here. */
__device__ __forceinline__ float cpv_ld_f32(const uint8_t* base, uint64_t bytes, uint64_t off) {
    if (base == nullptr || off + 4u > bytes) return 0.0f;
    return *reinterpret_cast<const float*>(base + off);
}
__device__ __forceinline__ uint32_t cpv_ld_u32(const uint8_t* base, uint64_t bytes, uint64_t off) {
    if (base == nullptr || off + 4u > bytes) return 0u;
    return *reinterpret_cast<const uint32_t*>(base + off);
}
__device__ __forceinline__ int32_t cpv_ld_i32(const uint8_t* base, uint64_t bytes, uint64_t off) {
    return static_cast<int32_t>(cpv_ld_u32(base, bytes, off));
}
/* One element of `size` bytes (1 or 2), little endian, read byte by byte
 * (vertex attributes of 8- and 16-bit formats need no 4-byte alignment). */
__device__ __forceinline__ uint32_t cpv_ld_elem(const uint8_t* base, uint64_t bytes, uint64_t off, uint32_t size) {
    if (base == nullptr || off + size > bytes) return 0u;
    uint32_t v = base[off];
    if (size == 2u) v |= static_cast<uint32_t>(base[off + 1]) << 8;
    return v;
}

/* A vertex attribute channel of a normalised 8/16-bit format as the
 * reference's pixel decoder returns it (LLVMRuntime/ImageCompiler.cpp:15-101,
 * 161-230): the unsigned or signed integer converted to float and divided by
 * the type's maximum (255, 65535, 127, 32767) — for signed formats without
 * a clamp, so the most negative code reads slightly below -1. */
__device__ __forceinline__ float cpv_decode_norm(uint32_t raw, uint32_t size, bool is_signed) {
    if (!is_signed) return __fdiv_rn(__uint2float_rn(raw), size == 1u ? 255.0f : 65535.0f);
    const int32_t v = size == 1u ? static_cast<int32_t>(static_cast<int8_t>(raw)) : static_cast<int32_t>(static_cast<int16_t>(raw));
    return __fdiv_rn(__int2float_rn(v), size == 1u ? 127.0f : 32767.0f);
}

/* IEEE binary32 → binary16 rounded to nearest, ties to even (the
 * reference's fptrunc of half attachments): overflow to infinity, gradual
 * underflow through the subnormals, NaN kept quiet with its top payload
 * bits. */
__device__ __forceinline__ uint32_t cpv_float_to_half(float f) {
    const uint32_t x = __float_as_uint(f);
    const uint32_t sign = (x >> 16) & 0x8000u;
    const uint32_t e = (x >> 23) & 0xFFu, m = x & 0x7FFFFFu;
    if (e == 0xFFu) return sign | 0x7C00u | (m ? (0x200u | (m >> 13)) : 0u);
    const int32_t he = static_cast<int32_t>(e) - 112;  /* the half's biased exponent */
    if (he >= 31) return sign | 0x7C00u;
    if (he <= 0) {
        if (he < -10) return sign;  /* below half the smallest subnormal */
        const uint32_t mi = m | 0x800000u;
        const uint32_t shift = static_cast<uint32_t>(14 - he);
        uint32_t hm = mi >> shift;
        const uint32_t rem = mi & ((1u << shift) - 1u), half = 1u << (shift - 1u);
        if (rem > half || (rem == half && (hm & 1u))) hm++;
        return sign | hm;
    }
    uint32_t r = sign | (static_cast<uint32_t>(he) << 10) | (m >> 13);
    const uint32_t rem = m & 0x1FFFu;
    if (rem > 0x1000u || (rem == 0x1000u && (r & 1u))) r++;  /* a carry into the exponent is the correct rounding */
    return r;
}

/* IEEE binary16 → binary32, exact (the reference widens half attributes
 * with fpext): zero, subnormal, normal, infinity; a NaN keeps its payload
 * and becomes quiet. */
__device__ __forceinline__ float cpv_half_to_float(uint32_t h) {
    const uint32_t sign = (h & 0x8000u) << 16, exp = (h >> 10) & 0x1Fu, man = h & 0x3FFu;
    uint32_t bits;
    if (exp == 0x1Fu) {
        bits = sign | 0x7F800000u | (man << 13) | (man ? 0x00400000u : 0u);
    } else if (exp != 0u) {
        bits = sign | ((exp + 112u) << 23) | (man << 13);
    } else if (man == 0u) {
        bits = sign;
    } else {
        /* subnormal: man x 2^-24, normalised */
        uint32_t e = 113u, m = man;
        while ((m & 0x400u) == 0u) {
            m <<= 1;
            e--;
        }
        bits = sign | (e << 23) | ((m & 0x3FFu) << 13);
    }
    return __uint_as_float(bits);
}

/* ------------------------------------------------------------------------- */
/* Value types for translated shaders                                        */
/* ------------------------------------------------------------------------- */

template <typename T, int N>
struct cvec {
    T v[N];
};

template <int C, int R>
struct cmat {
    cvec<float, R> c[C];
};

/* Component-wise arithmetic, one IEEE operation per component. */
#define CPV_VEC_BINOP(NAME, EXPR)                                                          \
    __device__ __forceinline__ float NAME(float a, float b) { return EXPR; }               \
    template <int N>                                                                       \
    __device__ __forceinline__ cvec<float, N> NAME(const cvec<float, N>& a, const cvec<float, N>& b) { \
        cvec<float, N> r;                                                                  \
        _Pragma("unroll") for (int i = 0; i < N; i++) r.v[i] = NAME(a.v[i], b.v[i]);       \
        return r;                                                                          \
    }
CPV_VEC_BINOP(cpv_fadd, __fadd_rn(a, b))
CPV_VEC_BINOP(cpv_fsub, __fsub_rn(a, b))
CPV_VEC_BINOP(cpv_fmul, __fmul_rn(a, b))
CPV_VEC_BINOP(cpv_fdiv, __fdiv_rn(a, b))
#undef CPV_VEC_BINOP

__device__ __forceinline__ float cpv_fneg(float a) { return -a; }
template <int N>
__device__ __forceinline__ cvec<float, N> cpv_fneg(const cvec<float, N>& a) {
    cvec<float, N> r;
#pragma unroll
    for (int i = 0; i < N; i++) r.v[i] = -a.v[i];
    return r;
}

template <int N>
__device__ __forceinline__ cvec<float, N> cpv_vec_times_scalar(const cvec<float, N>& a, float s) {
    cvec<float, N> r;
#pragma unroll
    for (int i = 0; i < N; i++) r.v[i] = __fmul_rn(a.v[i], s);
    return r;
}

template <int C, int R>
__device__ __forceinline__ cmat<C, R> cpv_mat_times_scalar(const cmat<C, R>& m, float s) {
    cmat<C, R> r;
#pragma unroll
    for (int c = 0; c < C; c++) r.c[c] = cpv_vec_times_scalar(m.c[c], s);
    return r;
}

/* OpMatrixTimesVector for mat4 → glm operator*(mat4, vec4) order:
 * (m0*v0 + m1*v1) + (m2*v2 + m3*v3) per row (LLVMRuntime/SpirvFunctions.cpp:34-45;
 * glm 0.9.9 summation order, restated). */
__device__ __forceinline__ cvec<float, 4> cpv_mat_times_vec(const cmat<4, 4>& m, const cvec<float, 4>& v) {
    cvec<float, 4> r;
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const float mul0 = __fmul_rn(m.c[0].v[i], v.v[0]);
        const float mul1 = __fmul_rn(m.c[1].v[i], v.v[1]);
        const float add0 = __fadd_rn(mul0, mul1);
        const float mul2 = __fmul_rn(m.c[2].v[i], v.v[2]);
        const float mul3 = __fmul_rn(m.c[3].v[i], v.v[3]);
        const float add1 = __fadd_rn(mul2, mul3);
        r.v[i] = __fadd_rn(add0, add1);
    }
    return r;
}

/* mat3 * vec3 → glm order: (m0*v0 + m1*v1) + m2*v2. */
__device__ __forceinline__ cvec<float, 3> cpv_mat_times_vec(const cmat<3, 3>& m, const cvec<float, 3>& v) {
    cvec<float, 3> r;
#pragma unroll
    for (int i = 0; i < 3; i++) {
        const float mul0 = __fmul_rn(m.c[0].v[i], v.v[0]);
        const float mul1 = __fmul_rn(m.c[1].v[i], v.v[1]);
        const float mul2 = __fmul_rn(m.c[2].v[i], v.v[2]);
        r.v[i] = __fadd_rn(__fadd_rn(mul0, mul1), mul2);
    }
    return r;
}

/* OpDot → glm::dot: vec2/vec3 left to right, vec4 pairwise. */
__device__ __forceinline__ float cpv_dot(const cvec<float, 2>& a, const cvec<float, 2>& b) {
    return __fadd_rn(__fmul_rn(a.v[0], b.v[0]), __fmul_rn(a.v[1], b.v[1]));
}
__device__ __forceinline__ float cpv_dot(const cvec<float, 3>& a, const cvec<float, 3>& b) {
    const float t0 = __fmul_rn(a.v[0], b.v[0]);
    const float t1 = __fmul_rn(a.v[1], b.v[1]);
    const float t2 = __fmul_rn(a.v[2], b.v[2]);
    return __fadd_rn(__fadd_rn(t0, t1), t2);
}
__device__ __forceinline__ float cpv_dot(const cvec<float, 4>& a, const cvec<float, 4>& b) {
    const float t0 = __fmul_rn(a.v[0], b.v[0]);
    const float t1 = __fmul_rn(a.v[1], b.v[1]);
    const float t2 = __fmul_rn(a.v[2], b.v[2]);
    const float t3 = __fmul_rn(a.v[3], b.v[3]);
    return __fadd_rn(__fadd_rn(t0, t1), __fadd_rn(t2, t3));
}

/* GLSL.std.450 Normalize on vectors → glm::normalize: x * (1 / sqrt(dot(x, x)))
 * (CPVulkan/GlslFunctions.cpp:178-182). The scalar form is the reference's
 * sign-based variant (:172-176). */
template <int N>
__device__ __forceinline__ cvec<float, N> cpv_normalize(const cvec<float, N>& x) {
    const float inv = __fdiv_rn(1.0f, __fsqrt_rn(cpv_dot(x, x)));
    return cpv_vec_times_scalar(x, inv);
}
__device__ __forceinline__ float cpv_normalize(float x) { return signbit(x) ? 1.0f : -1.0f; }

#define CPV_VEC_FUNC2(NAME, SCALAR)                                                        \
    __device__ __forceinline__ float NAME(float a, float b) { return SCALAR(a, b); }       \
    template <int N>                                                                       \
    __device__ __forceinline__ cvec<float, N> NAME(const cvec<float, N>& a, const cvec<float, N>& b) { \
        cvec<float, N> r;                                                                  \
        _Pragma("unroll") for (int i = 0; i < N; i++) r.v[i] = SCALAR(a.v[i], b.v[i]);     \
        return r;                                                                          \
    }
/* NMin / NMax (CPVulkan/GlslFunctions.cpp:264-302): a NaN first operand
 * gives the second, else std::min / std::max (so a NaN second operand
 * gives the first). */
__device__ __forceinline__ float cpv_nmin(float a, float b) { return isnan(a) ? b : cpv_std_min(a, b); }
__device__ __forceinline__ float cpv_nmax(float a, float b) { return isnan(a) ? b : cpv_std_max(a, b); }
CPV_VEC_FUNC2(cpv_glsl_fmax, cpv_std_max)
CPV_VEC_FUNC2(cpv_glsl_fmin, cpv_std_min)
CPV_VEC_FUNC2(cpv_glsl_pow, powf)
CPV_VEC_FUNC2(cpv_glsl_nmin, cpv_nmin)
CPV_VEC_FUNC2(cpv_glsl_nmax, cpv_nmax)
#undef CPV_VEC_FUNC2

/* NClamp: NMin(NMax(x, lo), hi) (CPVulkan/GlslFunctions.cpp:306-310). */
__device__ __forceinline__ float cpv_glsl_nclamp(float v, float lo, float hi) { return cpv_nmin(cpv_nmax(v, lo), hi); }
template <int N>
__device__ __forceinline__ cvec<float, N> cpv_glsl_nclamp(const cvec<float, N>& v, const cvec<float, N>& lo, const cvec<float, N>& hi) {
    cvec<float, N> r;
#pragma unroll
    for (int i = 0; i < N; i++) r.v[i] = cpv_glsl_nclamp(v.v[i], lo.v[i], hi.v[i]);
    return r;
}

/* Reflect → glm::reflect: I - N * dot(N, I) * 2, each component one
 * rounded multiply, multiply and subtract (CPVulkan/GlslFunctions.cpp:184-188). */
__device__ __forceinline__ float cpv_glsl_reflect(float i, float n) {
    return __fsub_rn(i, __fmul_rn(__fmul_rn(n, __fmul_rn(n, i)), 2.0f));
}
template <int N>
__device__ __forceinline__ cvec<float, N> cpv_glsl_reflect(const cvec<float, N>& i, const cvec<float, N>& n) {
    const float d = cpv_dot(n, i);
    cvec<float, N> r;
#pragma unroll
    for (int k = 0; k < N; k++) r.v[k] = __fsub_rn(i.v[k], __fmul_rn(__fmul_rn(n.v[k], d), 2.0f));
    return r;
}

/* FindILsb / FindSMsb / FindUMsb on 32-bit integers (CPVulkan/GlslFunctions.cpp:190-262):
 * -1 for no set bit; FindSMsb looks at ~v for negative v. */
__device__ __forceinline__ int32_t cpv_find_ilsb(uint32_t v) { return v == 0u ? -1 : __ffs(static_cast<int>(v)) - 1; }
__device__ __forceinline__ int32_t cpv_find_umsb(uint32_t v) { return v == 0u ? -1 : 31 - __clz(static_cast<int>(v)); }
__device__ __forceinline__ int32_t cpv_find_smsb(int32_t v) {
    if (v < 0) v = ~v;
    return v == 0 ? -1 : 31 - __clz(v);
}

__device__ __forceinline__ float cpv_glsl_fclamp(float v, float lo, float hi) { return cpv_std_clamp(v, lo, hi); }
template <int N>
__device__ __forceinline__ cvec<float, N> cpv_glsl_fclamp(const cvec<float, N>& v, const cvec<float, N>& lo, const cvec<float, N>& hi) {
    cvec<float, N> r;
#pragma unroll
    for (int i = 0; i < N; i++) r.v[i] = cpv_std_clamp(v.v[i], lo.v[i], hi.v[i]);
    return r;
}
/* FMix: x * (1 - a) + y * a (CPVulkan/GlslFunctions.cpp:155-159). */
__device__ __forceinline__ float cpv_glsl_fmix(float x, float y, float a) {
    return __fadd_rn(__fmul_rn(x, __fsub_rn(1.0f, a)), __fmul_rn(y, a));
}
template <int N>
__device__ __forceinline__ cvec<float, N> cpv_glsl_fmix(const cvec<float, N>& x, const cvec<float, N>& y, const cvec<float, N>& a) {
    cvec<float, N> r;
#pragma unroll
    for (int i = 0; i < N; i++) r.v[i] = cpv_glsl_fmix(x.v[i], y.v[i], a.v[i]);
    return r;
}

/* ------------------------------------------------------------------------- */
/* Image sampler (CPVulkan/ImageSampler.cpp, CPVulkan/GlslFunctions.cpp)     */
/* ------------------------------------------------------------------------- */

/* wrap (CPVulkan/ImageSampler.cpp:12-38). */
__device__ __forceinline__ int32_t cpv_wrap(int32_t v, int32_t size, uint32_t mode) {
    switch (mode) {
    case 0: return (v % size + size) % size;
    case 1: {
        const int32_t two = 2 * size;
        const int32_t n = (v % two + two) % two - size;
        return size - 1 - (n >= 0 ? n : -(1 + n));
    }
    case 2: return v < 0 ? 0 : (v > size - 1 ? size - 1 : v);
    case 3: return v < -1 ? -1 : (v > size ? size : v);
    case 4: {
        const int32_t m = v >= 0 ? v : -(1 + v);
        return m < 0 ? 0 : (m > size - 1 ? size - 1 : m);
    }
    default: return 0;
    }
}

/* GetPixel<fvec4> of an RGBA8 UNORM texel with the border check
 * (CPVulkan/ImageSampler.cpp:133-160) and the border table (:409-417). */
__device__ __forceinline__ void cpv_texel(const CpvTexture& t, uint32_t level, int32_t x, int32_t y, float out[4]) {
    const int32_t w = static_cast<int32_t>(t.level_w[level]);
    const int32_t h = static_cast<int32_t>(t.level_h[level]);
    if (x < 0 || x >= w || y < 0 || y >= h) {
        const uint32_t b = t.border < 6u ? t.border : 0u;
        const float rgb = (b >= 4u) ? 1.0f : 0.0f;
        const float a = (b >= 2u) ? 1.0f : 0.0f;
        out[0] = rgb; out[1] = rgb; out[2] = rgb; out[3] = a;
        return;
    }
    const uint64_t off = t.level_offset[level] + (static_cast<uint64_t>(y) * static_cast<uint64_t>(w) + static_cast<uint64_t>(x)) * 4u;
    if (off + 4u > t.bytes) {
        out[0] = out[1] = out[2] = out[3] = 0.0f;
        return;
    }
    const uint32_t px = __ldg(reinterpret_cast<const uint32_t*>(t.data + off));
    /* B8G8R8A8 stores red in byte 2 (CPVulkanBase/Formats.cpp:255) */
    const bool bgra = t.format == CPV_FMT_B8G8R8A8_UNORM;
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const int byte = (bgra && i < 3) ? 2 - i : i;
        out[i] = CPV_DECODE8((px >> (8 * byte)) & 0xFFu);
    }
}

/* lerp with a double-precision delta (CPVulkan/ImageSampler.cpp:51-55):
 * float(double(a) + double(b - a) * delta). The product of two binary32
 * values is exact in binary64 (48 significant bits), so the reference's
 * multiply-then-add equals one binary64 fused multiply-add. */
__device__ __forceinline__ void cpv_lerp4(const float a[4], const float b[4], double delta, float out[4]) {
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const float diff = __fsub_rn(b[i], a[i]);
        const double sum = __fma_rn(static_cast<double>(diff), delta, static_cast<double>(a[i]));
        out[i] = __double2float_rn(sum);
    }
}

/* SampleImageOfLevel, 2D (CPVulkan/ImageSampler.cpp:403-531). */
__device__ __forceinline__ void cpv_sample_level(const CpvTexture& t, uint32_t level, float u, float v, uint32_t filter, float out[4]) {
    const float range_x = __uint2float_rn(t.level_w[level]);
    const float range_y = __uint2float_rn(t.level_h[level]);
    const int32_t wx = static_cast<int32_t>(t.level_w[level]);
    const int32_t wy = static_cast<int32_t>(t.level_h[level]);
    if (filter == 0u) {
        int32_t cx = cpv_f2i(floorf(__fadd_rn(__fmul_rn(u, range_x), 0.0f)));
        int32_t cy = cpv_f2i(floorf(__fadd_rn(__fmul_rn(v, range_y), 0.0f)));
        cx = cpv_wrap(cx, wx, t.address_u);
        cy = cpv_wrap(cy, wy, t.address_v);
        cpv_texel(t, level, cx, cy, out);
        return;
    }
    const float sx = __fsub_rn(__fmul_rn(u, range_x), 0.5f);
    const float sy = __fsub_rn(__fmul_rn(v, range_y), 0.5f);
    const float flx = floorf(sx), fly = floorf(sy);
    const int32_t x0r = cpv_f2i(flx), y0r = cpv_f2i(fly);
    const int32_t x1 = cpv_wrap(x0r + 1, wx, t.address_u);
    const int32_t y1 = cpv_wrap(y0r + 1, wy, t.address_v);
    const int32_t x0 = cpv_wrap(x0r, wx, t.address_u);
    const int32_t y0 = cpv_wrap(y0r, wy, t.address_v);
    const double fx = static_cast<double>(__fsub_rn(sx, flx));
    const double fy = static_cast<double>(__fsub_rn(sy, fly));
    float t00[4], t01[4], t10[4], t11[4];
    cpv_texel(t, level, x0, y0, t00);
    cpv_texel(t, level, x0, y1, t01);
    cpv_texel(t, level, x1, y0, t10);
    cpv_texel(t, level, x1, y1, t11);
    float ij0[4], ij1[4];
    cpv_lerp4(t00, t10, fx, ij0);
    cpv_lerp4(t01, t11, fx, ij1);
    cpv_lerp4(ij0, ij1, fy, out);
}

/* ImageSampleExplicitLod λ (CPVulkan/GlslFunctions.cpp:624-628) + SampleImage
 * (CPVulkan/ImageSampler.cpp:562-673). Implicit-LOD sampling passes lod 0
 * (CPVulkan/GlslFunctions.cpp:657-672). */
/* ImageFetch (CPVulkan/GlslFunctions.cpp:674-742): the texel at integer
 * coordinates of level 0 (the reference ignores the Lod operand), zeros
 * outside it (GetPixel's border argument is ReturnType{}). */
__device__ __forceinline__ cvec<float, 4> cpv_fetch(const CpvTexture& t, int32_t x, int32_t y) {
    cvec<float, 4> r;
    if (t.levels == 0u || x < 0 || y < 0 || x >= static_cast<int32_t>(t.level_w[0]) || y >= static_cast<int32_t>(t.level_h[0])) {
        r.v[0] = r.v[1] = r.v[2] = r.v[3] = 0.0f;
        return r;
    }
    cpv_texel(t, 0u, x, y, r.v);
    return r;
}

__device__ __forceinline__ cvec<float, 4> cpv_sample(const CpvTexture& t, float u, float v, float lod) {
    const float bias = cpv_std_clamp(__fadd_rn(t.lod_bias, 0.0f), -32.0f, 32.0f);
    const float lambda = cpv_std_clamp(__fadd_rn(lod, bias), t.min_lod, t.max_lod);
    float out[4];
    if (t.levels == 0u || t.data == nullptr) {
        out[0] = out[1] = out[2] = 0.0f;
        out[3] = 1.0f;
    } else if (lambda <= 0.0f) {
        cpv_sample_level(t, 0u, u, v, t.mag_filter, out);
    } else {
        const float max_level = __uint2float_rn(t.levels - 1u);
        const float mip = cpv_std_clamp(lambda, 0.0f, max_level);
        if (t.mipmap_mode == 0u) {
            const uint32_t real = __float2uint_rz(ceilf(__fadd_rn(mip, 0.5f))) - 1u;
            cpv_sample_level(t, real, u, v, t.min_filter, out);
        } else {
            const uint32_t l1 = __float2uint_rz(floorf(mip));
            const float delta = __fsub_rn(mip, __uint2float_rn(l1));
            float p1[4];
            cpv_sample_level(t, l1, u, v, t.min_filter, p1);
            if (delta == 0.0f) {
#pragma unroll
                for (int i = 0; i < 4; i++) out[i] = p1[i];
            } else {
                float p2[4];
                cpv_sample_level(t, l1 + 1u, u, v, t.min_filter, p2);
                cpv_lerp4(p1, p2, static_cast<double>(delta), out);
            }
        }
    }
    cvec<float, 4> r;
#pragma unroll
    for (int i = 0; i < 4; i++) r.v[i] = out[i];
    return r;
}

/* ------------------------------------------------------------------------- */
/* Per-draw binning over the union of the draw's tile rectangles             */
/* ------------------------------------------------------------------------- */

/* The union of a draw's tile rectangles (CpvDrawParams::tile_box): its
 * origin and extent in tiles; an empty union (no live primitive) has no
 * tiles. */
struct CpvTileBox {
    uint32_t x0, y0, w, h;
};
__device__ __forceinline__ CpvTileBox cpv_tile_box(const uint32_t* box) {
    CpvTileBox b;
    b.x0 = 0xFFFFu - box[0];
    b.y0 = 0xFFFFu - box[1];
    const uint32_t x1 = box[2], y1 = box[3];
    b.w = x1 > b.x0 ? x1 - b.x0 : 0u;
    b.h = y1 > b.y0 ? y1 - b.y0 : 0u;
    if (b.w == 0u || b.h == 0u) b.w = b.h = 0u;
    return b;
}

/* Adds each thread's non-empty tile rectangle to the union: the CTA's
 * maxima first (one atomic per word per CTA). Every thread of the CTA calls
 * it. */
__device__ __forceinline__ void cpv_tile_box_add(uint32_t* box, uint2 r) {
    __shared__ uint32_t m[4];
    if (threadIdx.x < 4u) m[threadIdx.x] = 0u;
    __syncthreads();
    const uint32_t x0 = r.x & 0xFFFFu, y0 = r.x >> 16, x1 = r.y & 0xFFFFu, y1 = r.y >> 16;
    const bool any = x1 > x0 && y1 > y0;
    const uint32_t v[4] = {any ? 0xFFFFu - x0 : 0u, any ? 0xFFFFu - y0 : 0u, any ? x1 : 0u, any ? y1 : 0u};
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const uint32_t w = __reduce_max_sync(0xFFFFFFFFu, v[i]);
        if ((threadIdx.x & 31u) == 0u && w) atomicMax(&m[i], w);
    }
    __syncthreads();
    if (threadIdx.x < 4u && m[threadIdx.x]) atomicMax(&box[threadIdx.x], m[threadIdx.x]);
}

/* ------------------------------------------------------------------------- */
/* Quad-derivative LOD: the labelled "spec LOD" mode (Vulkan 1.1, "Scale      */
/* Factor Operation, Level-of-Detail Operation and Image Level(s) Selection")*/
/* ------------------------------------------------------------------------- */

#define CPV_MAX_LOD_SITES 8

/* A fragment's 2x2 quad for implicit-LOD sampling. The fragment shader runs
 * first for the horizontal neighbour (mode 1: pixel (x ^ 1, y)) and the
 * vertical one (mode 2: (x, y ^ 1)), each recording the coordinates it
 * reaches at every implicit-LOD sampling instruction (site k) and sampling
 * nothing, then for the fragment itself (mode 0), whose sites take fine
 * derivatives within the quad: dP/dx = P(x | 1) - P(x & ~1), likewise in y.
 * A site a neighbour did not reach (it discarded first) has derivative 0
 * in that direction; a site inside a loop sees the neighbour's last value. */
struct CpvQuadLod {
    uint32_t mode;
    uint32_t odd;      /* bit 0: x odd; bit 1: y odd */
    uint32_t seen[2];  /* bit k: site k reached by neighbour 0 / 1 */
    float u[2][CPV_MAX_LOD_SITES], v[2][CPV_MAX_LOD_SITES];
};

/* 0.5 * log2(r) for r = ρ², so that λ_base = log2(max(ρx, ρy)) needs no
 * square root. Written from the series ln m = 2 atanh(s) = 2 (s + s³/3 +
 * s⁵/5 + s⁷/7 + s⁹/9 + ...), s = (m - 1) / (m + 1), with the mantissa m
 * reduced to [√½, √2] so |s| <= 0.1716 and the first omitted term is below
 * 2⁻²⁸ of the sum; every step is one rounded binary32 operation, so a host
 * restatement in the same order gives the same bits. r = 0 or NaN gives
 * -∞ (no derivative: the least λ), r = +∞ gives +∞. */
__device__ __forceinline__ float cpv_half_log2(float r) {
    if (!(r > 0.0f)) return __uint_as_float(0xFF800000u);
    if (r == __uint_as_float(0x7F800000u)) return r;
    uint32_t b = __float_as_uint(r);
    int32_t e = 0;
    if (b < 0x00800000u) {
        b = __float_as_uint(__fmul_rn(r, 16777216.0f));  /* subnormal: scale by 2^24 */
        e = -24;
    }
    e += static_cast<int32_t>(b >> 23) - 127;
    float m = __uint_as_float((b & 0x007FFFFFu) | 0x3F800000u);
    if (m > 1.41421356f) {
        m = __fmul_rn(m, 0.5f);
        e += 1;
    }
    const float s = __fdiv_rn(__fsub_rn(m, 1.0f), __fadd_rn(m, 1.0f));
    const float s2 = __fmul_rn(s, s);
    float q = __fadd_rn(__fmul_rn(s2, 0.111111111f), 0.142857143f);
    q = __fadd_rn(__fmul_rn(q, s2), 0.2f);
    q = __fadd_rn(__fmul_rn(q, s2), 0.333333333f);
    q = __fadd_rn(__fmul_rn(q, s2), 1.0f);
    const float log2m = __fmul_rn(__fmul_rn(s, q), 2.88539008f);  /* 2 / ln 2 */
    return __fmul_rn(__fadd_rn(static_cast<float>(e), log2m), 0.5f);
}

/* Implicit-LOD sampling at site k of a fragment shader compiled for the
 * quad-derivative mode: records the coordinates in a neighbour's run
 * (returning zeros), else samples with λ_base = log2(max(ρx, ρy)),
 * ρ = |(du/d·, dv/d·)| scaled by the level-0 extent, through the same bias,
 * clamp and level selection as explicit LOD. Without a quad (a shader run
 * once per primitive: its coordinates do not vary) λ_base is -∞. */
__device__ __forceinline__ cvec<float, 4> cpv_sample_quad(const CpvTexture& t, float u, float v, CpvQuadLod* q, uint32_t k) {
    if (q != nullptr && q->mode != 0u) {
        const uint32_t n = q->mode - 1u;
        q->u[n][k] = u;
        q->v[n][k] = v;
        q->seen[n] |= 1u << k;
        cvec<float, 4> r;
        r.v[0] = r.v[1] = r.v[2] = r.v[3] = 0.0f;
        return r;
    }
    float lambda = __uint_as_float(0xFF800000u);
    if (q != nullptr && t.levels != 0u) {
        const float w = __uint2float_rn(t.level_w[0]), h = __uint2float_rn(t.level_h[0]);
        float r2[2];
#pragma unroll
        for (uint32_t n = 0; n < 2; n++) {
            float du = 0.0f, dv = 0.0f;
            if ((q->seen[n] >> k) & 1u) {
                const bool odd = ((q->odd >> n) & 1u) != 0u;
                du = odd ? __fsub_rn(u, q->u[n][k]) : __fsub_rn(q->u[n][k], u);
                dv = odd ? __fsub_rn(v, q->v[n][k]) : __fsub_rn(q->v[n][k], v);
            }
            const float a = __fmul_rn(du, w), b = __fmul_rn(dv, h);
            r2[n] = __fadd_rn(__fmul_rn(a, a), __fmul_rn(b, b));
        }
        lambda = cpv_half_log2(r2[0] >= r2[1] ? r2[0] : r2[1]);
    }
    return cpv_sample(t, u, v, lambda);
}

/* ------------------------------------------------------------------------- */
/* Input assembly                                                            */
/* ------------------------------------------------------------------------- */

/* Assembled-vertex slots of primitive p for the topology
 * (CPVulkan/CommandBuffer.Draw.cpp:567-673): returns raw ids v[3] and the
 * provoking raw id. Points use v[0], lines v[0..1]. */
__device__ __forceinline__ void cpv_prim_vertices(uint32_t topology, uint32_t p, uint32_t v[3], uint32_t& provoking) {
    if (topology == 0u) { /* point list */
        v[0] = v[1] = v[2] = p; provoking = p;
    } else if (topology == 1u) { /* line list */
        v[0] = 2u * p; v[1] = 2u * p + 1u; v[2] = v[1]; provoking = 2u * p;
    } else if (topology == 2u) { /* line strip */
        v[0] = p; v[1] = p + 1u; v[2] = v[1]; provoking = p;
    } else if (topology == 4u) { /* strip */
        v[0] = p; v[1] = p + 1u; v[2] = p + 2u; provoking = p;
    } else if (topology == 5u) { /* fan */
        v[0] = 0u; v[1] = p + 1u; v[2] = p + 2u; provoking = p + 1u;
    } else { /* list */
        v[0] = 3u * p; v[1] = 3u * p + 1u; v[2] = 3u * p + 2u; provoking = 3u * p;
    }
}

/* Raw assembled vertex → vertex id (CPVulkan/CommandBuffer.Draw.cpp:675-760):
 * firstVertex + i, or vertexOffset + index[firstIndex + i]; an index outside
 * the bound index buffer reads as 0. */
__device__ __forceinline__ uint32_t cpv_vertex_id(const CpvDrawParams& P, uint32_t raw) {
    if (P.index_size == 0u) return P.first + raw;
    const uint64_t off = (static_cast<uint64_t>(P.first) + raw) * P.index_size;
    uint32_t index = 0u;
    if (off + P.index_size <= P.ib_bytes) {
        if (P.index_size == 2u) index = __ldg(reinterpret_cast<const uint16_t*>(P.ib + off));
        else index = __ldg(reinterpret_cast<const uint32_t*>(P.ib + off));
    }
    return static_cast<uint32_t>(P.vertex_offset) + index;
}

#endif /* CPV_DEVICE_CUH */
