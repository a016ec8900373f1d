/*
 * shim.h — TEST INFRASTRUCTURE ONLY. The environment in which the
 * reference's extracted functions (see extract.py) compile without the
 * reference's third-party dependencies, which are absent from this image:
 *
 *  - glm (version >= 0.9.9 in the reference's build, unpinned): a minimal
 *    vec<L, T> with the operations the pinned functions use, each one
 *    component-wise IEEE arithmetic as glm defines it (min(x, y) is
 *    (y < x) ? y : x, max(x, y) is (x < y) ? y : x, the defaulted default
 *    constructor value-initialises to zero under `T v{}`, conversions
 *    between element types are implicit);
 *  - gsl::span (Microsoft GSL): pointer + size;
 *  - the Vulkan names: include/cpv/vk_subset.h, plus the sampler
 *    reduction mode of VK_EXT_sampler_filter_minmax;
 *  - the reference's format table and pixel decode (CPVulkanBase/Formats.h,
 *    the JIT's GetPixelF32) for the formats the pinned cases use: the
 *    declarations mirror the reference's, the decode restates UNORM8 as
 *    u / 255.0f (LLVMRuntime/ImageCompiler.cpp:161-230).
 */
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <type_traits>
#include <vector>

#include "cpv/vk_subset.h"

#define TODO_ERROR() \
    if (1) {         \
        abort();     \
    } else           \
        (void)0
#define FATAL_ERROR() \
    if (1) {          \
        abort();      \
    } else            \
        (void)0

typedef enum VkSamplerReductionModeEXT {
    VK_SAMPLER_REDUCTION_MODE_WEIGHTED_AVERAGE_EXT = 0,
    VK_SAMPLER_REDUCTION_MODE_MIN_EXT = 1,
    VK_SAMPLER_REDUCTION_MODE_MAX_EXT = 2,
} VkSamplerReductionModeEXT;

namespace SPIRV {
class SPIRVType;
}

struct DeviceState;

namespace gsl {
template <typename T>
class span {
public:
    span() = default;
    span(T* p, size_t n) : p_(p), n_(n) {}
    T* data() const { return p_; }
    size_t size() const { return n_; }
    span subspan(size_t offset, size_t count) const { return span(p_ + offset, count); }

private:
    T* p_ = nullptr;
    size_t n_ = 0;
};
}  // namespace gsl

namespace glm {

template <int L, typename T>
struct vec;

#define CPV_GLM_COMMON(L)                                                                  \
    using value_type = T;                                                                  \
    static constexpr int length() { return L; }                                            \
    vec() = default;                                                                       \
    T& operator[](int i) { return reinterpret_cast<T*>(this)[i]; }                         \
    const T& operator[](int i) const { return reinterpret_cast<const T*>(this)[i]; }

template <typename T>
struct vec<1, T> {
    union { T x, r; };
    CPV_GLM_COMMON(1)
    explicit vec(T s) : x(s) {}
    template <typename U>
    vec(const vec<1, U>& v) : x(static_cast<T>(v.x)) {}
};

template <typename T>
struct vec<2, T> {
    union { T x, r; };
    union { T y, g; };
    CPV_GLM_COMMON(2)
    explicit vec(T s) : x(s), y(s) {}
    template <typename X, typename Y>
    vec(X a, Y b) : x(static_cast<T>(a)), y(static_cast<T>(b)) {}
    template <typename U>
    vec(const vec<2, U>& v) : x(static_cast<T>(v.x)), y(static_cast<T>(v.y)) {}
    template <typename U>
    vec(const vec<4, U>& v) : x(static_cast<T>(v.x)), y(static_cast<T>(v.y)) {}
};

template <typename T>
struct vec<3, T> {
    union { T x, r; };
    union { T y, g; };
    union { T z, b; };
    CPV_GLM_COMMON(3)
    explicit vec(T s) : x(s), y(s), z(s) {}
    template <typename X, typename Y, typename Z>
    vec(X a, Y b, Z c) : x(static_cast<T>(a)), y(static_cast<T>(b)), z(static_cast<T>(c)) {}
    template <typename U>
    vec(const vec<3, U>& v) : x(static_cast<T>(v.x)), y(static_cast<T>(v.y)), z(static_cast<T>(v.z)) {}
};

template <typename T>
struct vec<4, T> {
    union { T x, r; };
    union { T y, g; };
    union { T z, b; };
    union { T w, a; };
    CPV_GLM_COMMON(4)
    explicit vec(T s) : x(s), y(s), z(s), w(s) {}
    template <typename X, typename Y, typename Z, typename W>
    vec(X a_, Y b_, Z c_, W d_) : x(static_cast<T>(a_)), y(static_cast<T>(b_)), z(static_cast<T>(c_)), w(static_cast<T>(d_)) {}
    template <typename U>
    vec(const vec<4, U>& v) : x(static_cast<T>(v.x)), y(static_cast<T>(v.y)), z(static_cast<T>(v.z)), w(static_cast<T>(v.w)) {}
};

#undef CPV_GLM_COMMON

#define CPV_GLM_BINARY(op)                                                       \
    template <int L, typename T>                                                 \
    vec<L, T> operator op(const vec<L, T>& a, const vec<L, T>& b) {              \
        vec<L, T> r;                                                             \
        for (int i = 0; i < L; i++) r[i] = a[i] op b[i];                         \
        return r;                                                                \
    }                                                                            \
    template <int L, typename T>                                                 \
    vec<L, T> operator op(const vec<L, T>& a, T s) {                             \
        vec<L, T> r;                                                             \
        for (int i = 0; i < L; i++) r[i] = a[i] op s;                            \
        return r;                                                                \
    }                                                                            \
    template <int L, typename T>                                                 \
    vec<L, T> operator op(T s, const vec<L, T>& a) {                             \
        vec<L, T> r;                                                             \
        for (int i = 0; i < L; i++) r[i] = s op a[i];                            \
        return r;                                                                \
    }
CPV_GLM_BINARY(+)
CPV_GLM_BINARY(-)
CPV_GLM_BINARY(*)
CPV_GLM_BINARY(/)
#undef CPV_GLM_BINARY

template <int L, typename T>
vec<L, T> min(const vec<L, T>& x, const vec<L, T>& y) {
    vec<L, T> r;
    for (int i = 0; i < L; i++) r[i] = (y[i] < x[i]) ? y[i] : x[i];
    return r;
}

template <int L, typename T>
vec<L, T> max(const vec<L, T>& x, const vec<L, T>& y) {
    vec<L, T> r;
    for (int i = 0; i < L; i++) r[i] = (x[i] < y[i]) ? y[i] : x[i];
    return r;
}

using vec2 = vec<2, float>;
using vec3 = vec<3, float>;
using vec4 = vec<4, float>;
using fvec1 = vec<1, float>;
using fvec2 = vec<2, float>;
using fvec3 = vec<3, float>;
using fvec4 = vec<4, float>;
using dvec4 = vec<4, double>;
using ivec1 = vec<1, int32_t>;
using ivec2 = vec<2, int32_t>;
using ivec3 = vec<3, int32_t>;
using ivec4 = vec<4, int32_t>;
using uvec1 = vec<1, uint32_t>;
using uvec2 = vec<2, uint32_t>;
using uvec3 = vec<3, uint32_t>;
using uvec4 = vec<4, uint32_t>;

}  // namespace glm

/* CPVulkanBase/Formats.h: the fields of the format table the pinned code
 * reads. */
enum class FormatType { Normal, Packed, DepthStencil, Compressed, Planar, PlanarSamplable };
enum class BaseType { Unknown, UNorm, SNorm, UScaled, SScaled, UInt, SInt, UFloat, SFloat, SRGB };

struct FormatInformation {
    VkFormat Format;
    FormatType Type;
    VkColorComponentFlags Channels;
    uint32_t TotalSize;
    uint32_t ElementSize;
    BaseType Base;
    struct {
        uint32_t BlockWidth;
        uint32_t BlockHeight;
    } Compressed;
};

constexpr uint32_t MAX_MIP_LEVELS = 16;

const FormatInformation& GetFormatInformation(VkFormat format);

/* GetPixel<fvec4> for a 2D R8G8B8A8_UNORM level (CPVulkan/ImageSampler.cpp:105-145
 * with the JIT's decode): the border colour outside the level, else the
 * texel's four bytes divided by 255. */
template <typename ResultType, typename RangeType, typename CoordinateType>
ResultType GetPixel(DeviceState*, VkFormat, gsl::span<uint8_t> data, RangeType range, CoordinateType coordinates, ResultType borderColour) {
    if (coordinates.x < 0 || coordinates.x >= range.x || coordinates.y < 0 || coordinates.y >= range.y) return borderColour;
    const uint64_t offset = (static_cast<uint64_t>(coordinates.y) * range.x + static_cast<uint64_t>(coordinates.x)) * 4u;
    const uint8_t* p = data.data() + offset;
    return ResultType(static_cast<float>(p[0]) / 255.0f, static_cast<float>(p[1]) / 255.0f, static_cast<float>(p[2]) / 255.0f,
                      static_cast<float>(p[3]) / 255.0f);
}
