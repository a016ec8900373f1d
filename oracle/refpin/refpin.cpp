/*
 * refpin.cpp — TEST INFRASTRUCTURE ONLY. Batch entry points over the
 * reference's own functions, compiled from the reference's files by
 * extract.py into oracle/_ref/librefpin.so:
 *
 *   EdgeFunction, GetFragmentInput (with SetDatum), ApplyBlendFactor /
 *   ApplyBlend                          CPVulkan/CommandBuffer.Draw.cpp
 *   wrap, frac, lerp, GetPixelLinear, SampleImageOfLevel, SampleImage
 *                                       CPVulkan/ImageSampler.cpp
 *
 * tests/test_oracle_pinned.py compares the oracle's restatements with them
 * bit for bit on seeded and edge-case inputs.
 */
#include "shim.h"

#include "refpin_src.inc"

const FormatInformation& GetFormatInformation(VkFormat format) {
    static const FormatInformation rgba8{VK_FORMAT_R8G8B8A8_UNORM, FormatType::Normal,
                                         VK_COLOR_COMPONENT_R_BIT | VK_COLOR_COMPONENT_G_BIT | VK_COLOR_COMPONENT_B_BIT | VK_COLOR_COMPONENT_A_BIT,
                                         4, 1, BaseType::UNorm, {1, 1}};
    static const FormatInformation r32{VK_FORMAT_R32_SFLOAT, FormatType::Normal, VK_COLOR_COMPONENT_R_BIT, 4, 4, BaseType::SFloat, {1, 1}};
    static const FormatInformation rgba32{VK_FORMAT_R32G32B32A32_SFLOAT, FormatType::Normal,
                                          VK_COLOR_COMPONENT_R_BIT | VK_COLOR_COMPONENT_G_BIT | VK_COLOR_COMPONENT_B_BIT | VK_COLOR_COMPONENT_A_BIT,
                                          16, 4, BaseType::SFloat, {1, 1}};
    switch (format) {
    case VK_FORMAT_R32_SFLOAT: return r32;
    case VK_FORMAT_R32G32B32A32_SFLOAT: return rgba32;
    default: return rgba8;
    }
}

extern "C" {

/* in: 6 floats (a.x, a.y, b.x, b.y, c.x, c.y) per case; out[2 * i] from the
 * vec2 overload, out[2 * i + 1] from the vec4 one. */
void cpv_ref_edge_n(const float* in, float* out, uint64_t n) {
    for (uint64_t i = 0; i < n; i++) {
        const float* p = in + 6 * i;
        out[2 * i] = EdgeFunction(glm::vec2(p[0], p[1]), glm::vec2(p[2], p[3]), glm::vec2(p[4], p[5]));
        out[2 * i + 1] = EdgeFunction(glm::vec4(p[0], p[1], 0.5f, 2.0f), glm::vec4(p[2], p[3], 0.25f, 3.0f), glm::vec2(p[4], p[5]));
    }
}

/* wrap(v, size, mode) per case. */
void cpv_ref_wrap_n(const int32_t* v, const int32_t* size, const uint32_t* mode, int32_t* out, uint64_t n) {
    for (uint64_t i = 0; i < n; i++) out[i] = wrap(v[i], size[i], static_cast<VkSamplerAddressMode>(mode[i]));
}

/* ApplyBlend per case: src, dst, constant 4 floats each; modes = src colour,
 * dst colour, colour op, src alpha, dst alpha, alpha op factors. */
void cpv_ref_blend_n(const float* src, const float* dst, const float* constant, const uint32_t* modes, float* out, uint64_t n) {
    for (uint64_t i = 0; i < n; i++) {
        VkPipelineColorBlendAttachmentState st{};
        const uint32_t* m = modes + 6 * i;
        st.blendEnable = 1;
        st.srcColorBlendFactor = static_cast<VkBlendFactor>(m[0]);
        st.dstColorBlendFactor = static_cast<VkBlendFactor>(m[1]);
        st.colorBlendOp = static_cast<VkBlendOp>(m[2]);
        st.srcAlphaBlendFactor = static_cast<VkBlendFactor>(m[3]);
        st.dstAlphaBlendFactor = static_cast<VkBlendFactor>(m[4]);
        st.alphaBlendOp = static_cast<VkBlendOp>(m[5]);
        const float* s = src + 4 * i;
        const float* d = dst + 4 * i;
        const float* c = constant + 4 * i;
        const glm::vec4 r = ApplyBlend<glm::vec4>(glm::vec4(s[0], s[1], s[2], s[3]), glm::vec4(d[0], d[1], d[2], d[3]), glm::vec4(c[0], c[1], c[2], c[3]), st);
        for (int k = 0; k < 4; k++) out[4 * i + k] = r[k];
    }
}

/* GetFragmentInput per case. pts: p0, p1, p2 (NDC x, y, z, clip w) and the
 * pixel centre (x, y): 14 floats; vars: per vertex a perspective vec4, a
 * linear vec4 and a flat float (9 floats, 27 per case); cull: the cull mode;
 * provoking: 0..2. out: covered, front (as floats), depth, then the 9
 * interpolated components: 12 floats per case. */
void cpv_ref_fragment_input_n(const float* pts, const float* vars, const uint32_t* cull, const uint32_t* provoking, float* out, uint64_t n) {
    for (uint64_t i = 0; i < n; i++) {
        const float* p = pts + 14 * i;
        float result[9] = {};
        std::vector<VariableInOutData> inputs(3);
        inputs[0] = VariableInOutData{&result[0], 0, VK_FORMAT_R32G32B32A32_SFLOAT, nullptr, InterpolationType::Perspective, 16, 0};
        inputs[1] = VariableInOutData{&result[4], 1, VK_FORMAT_R32G32B32A32_SFLOAT, nullptr, InterpolationType::Linear, 16, 16};
        inputs[2] = VariableInOutData{&result[8], 2, VK_FORMAT_R32_SFLOAT, nullptr, InterpolationType::Flat, 4, 32};
        float depth = 0.0f;
        bool front = false;
        const bool covered = GetFragmentInput(inputs, reinterpret_cast<const uint8_t*>(vars + 27 * i), 36, provoking[i], 0, 1, 2,
                                              glm::vec4(p[0], p[1], p[2], p[3]), glm::vec4(p[4], p[5], p[6], p[7]),
                                              glm::vec4(p[8], p[9], p[10], p[11]), glm::vec2(p[12], p[13]), cull[i], depth, front);
        float* o = out + 12 * i;
        o[0] = covered ? 1.0f : 0.0f;
        o[1] = front ? 1.0f : 0.0f;
        o[2] = covered ? depth : 0.0f;
        for (int k = 0; k < 9; k++) o[3 + k] = covered ? result[k] : 0.0f;
    }
}

/* SampleImage of a 2D R8G8B8A8_UNORM texture with `levels` levels packed as
 * the reference lays them out (CPVulkanBase/Formats.cpp:453-484); modes =
 * mag filter, min filter, mipmap mode, address U, address V, border colour;
 * uvl = u, v, lod (the λ SampleImage receives) per case; out 4 floats. */
void cpv_ref_sample_n(const uint8_t* texels, uint32_t width, uint32_t height, uint32_t levels, const uint32_t* modes, const float* uvl, float* out,
                      uint64_t n) {
    gsl::span<uint8_t> data[MAX_MIP_LEVELS];
    glm::uvec2 range[MAX_MIP_LEVELS];
    uint64_t off = 0;
    uint32_t w = width, h = height;
    for (uint32_t l = 0; l < levels && l < MAX_MIP_LEVELS; l++) {
        data[l] = gsl::span<uint8_t>(const_cast<uint8_t*>(texels) + off, static_cast<size_t>(w) * h * 4u);
        range[l] = glm::uvec2(w, h);
        off += static_cast<uint64_t>(w) * h * 4u;
        w = std::max(w / 2, 1u);
        h = std::max(h / 2, 1u);
    }
    for (uint64_t i = 0; i < n; i++) {
        const uint32_t* m = modes + 6 * i;
        const float* c = uvl + 3 * i;
        const glm::fvec4 r = SampleImage<glm::fvec4, glm::uvec2, glm::vec2>(
            nullptr, VK_FORMAT_R8G8B8A8_UNORM, data, range, 0, levels, glm::vec2(c[0], c[1]), c[2], static_cast<VkFilter>(m[0]),
            static_cast<VkFilter>(m[1]), static_cast<VkSamplerMipmapMode>(m[2]), static_cast<VkSamplerAddressMode>(m[3]),
            static_cast<VkSamplerAddressMode>(m[4]), static_cast<VkSamplerAddressMode>(m[3]), false, false, VK_COMPARE_OP_NEVER,
            static_cast<VkBorderColor>(m[5]), false, VK_SAMPLER_REDUCTION_MODE_WEIGHTED_AVERAGE_EXT);
        for (int k = 0; k < 4; k++) out[4 * i + k] = r[k];
    }
}

}  // extern "C"
