// command.cpp — replay of a recorded command buffer on a queue's CUDA stream.
//
// Reference counterpart: CommandBuffer::Submit / RunCommands
// (CPVulkan/CommandBuffer.cpp:21-30, 964-968) and the Process() methods of
// the recorded commands (CommandBuffer.Binding.cpp, CommandBuffer.Draw.cpp,
// CommandBuffer.Copy.cpp). Where the reference executes each draw on the
// calling thread, this enqueues the draw's kernels on the stream and returns;
// the fence observes completion.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <thread>

#include "icd.h"

namespace cpv::icd {

// IEEE binary32 → binary16, round to nearest even (the encoder of half
// colour channels; the device code restates the same steps).
uint32_t float_to_half_host(float f) {
    uint32_t x;
    std::memcpy(&x, &f, 4);
    const uint32_t sign = (x >> 16) & 0x8000u;
    const uint32_t e = (x >> 23) & 0xFFu, m = x & 0x7FFFFFu;
    if (e == 0xFFu) return sign | 0x7C00u | (m ? (0x200u | (m >> 13)) : 0u);
    const int32_t he = static_cast<int32_t>(e) - 112;
    if (he >= 31) return sign | 0x7C00u;
    if (he <= 0) {
        if (he < -10) return sign;
        const uint32_t mi = m | 0x800000u;
        const uint32_t shift = static_cast<uint32_t>(14 - he);
        uint32_t hm = mi >> shift;
        const uint32_t rem = mi & ((1u << shift) - 1u), half = 1u << (shift - 1u);
        if (rem > half || (rem == half && (hm & 1u))) hm++;
        return sign | hm;
    }
    uint32_t r = sign | (static_cast<uint32_t>(he) << 10) | (m >> 13);
    const uint32_t rem = m & 0x1FFFu;
    if (rem > 0x1000u || (rem == 0x1000u && (r & 1u))) r++;
    return r;
}

// One colour channel through the reference's encoder for the format's kind
// (LLVMRuntime/ImageCompiler.cpp:1077-1185).
uint32_t encode_channel_host(float x, const ColourLayout& cl) {
    const uint32_t mask = cl.bits >= 32 ? 0xFFFFFFFFu : ((1u << cl.bits) - 1u);
    switch (cl.kind) {
    case 0: return encode_unorm_host(x, cl.bits == 8 ? 255.0f : 65535.0f);
    case 1: {
        float v = std::fmin(std::fmax(x, -1.0f), 1.0f) * (cl.bits == 8 ? 127.0f : 32767.0f);
        v = std::round(v);
        return static_cast<uint32_t>(static_cast<int32_t>(v)) & mask;
    }
    default:
        if (cl.bits == 16) return float_to_half_host(x);
        uint32_t b;
        std::memcpy(&b, &x, 4);
        return b;
    }
}

uint32_t encode_unorm_host(float x, float maxv) {
    float v = x;
    if (v != v) v = 0.0f;  // maxnum(NaN, 0) = 0
    if (v < 0.0f) v = 0.0f;
    if (v > 1.0f) v = 1.0f;
    v = v * maxv;
    return static_cast<uint32_t>(std::round(v));
}

namespace {

// Primitives of one instance of `count` assembled vertices
// (CPVulkan/CommandBuffer.Draw.cpp:567-673).
uint32_t primitives_per_instance(VkPrimitiveTopology topology, uint32_t count) {
    switch (topology) {
    case VK_PRIMITIVE_TOPOLOGY_POINT_LIST: return count;
    case VK_PRIMITIVE_TOPOLOGY_LINE_LIST: return count / 2;
    case VK_PRIMITIVE_TOPOLOGY_LINE_STRIP: return count > 1 ? count - 1 : 0;
    case VK_PRIMITIVE_TOPOLOGY_TRIANGLE_LIST: return count / 3;
    default: return count > 2 ? count - 2 : 0;  // strips and fans
    }
}

struct BoundVertex {
    Buffer* buffer = nullptr;
    VkDeviceSize offset = 0;
};

struct State {
    Pipeline* pipeline = nullptr;
    BoundVertex vertex[8];
    Buffer* index = nullptr;
    VkDeviceSize index_offset = 0;
    uint32_t index_size = 4;
    DescriptorSet* sets[8] = {};
    std::vector<uint32_t> dynamic_offsets[8];
    uint8_t push[128] = {};
    VkViewport viewport{};
    bool viewport_set = false;
    float blend_constants[4] = {0, 0, 0, 0};
    bool blend_set = false;
    RenderPass* pass = nullptr;
    Framebuffer* fb = nullptr;
    uint32_t subpass = 0;  // index into pass->subpasses
    const Subpass& sub() const { return pass->subpasses[subpass]; }
};

// Resolves the (set, binding) → dynamic offset index: dynamic descriptors are
// numbered in binding order within the set (Vulkan rule).
uint32_t dynamic_offset(const State& s, uint32_t set, uint32_t binding) {
    const DescriptorSet* ds = s.sets[set];
    if (!ds || !ds->layout) return 0;
    uint32_t index = 0;
    std::vector<VkDescriptorSetLayoutBinding> sorted = ds->layout->bindings;
    std::sort(sorted.begin(), sorted.end(), [](auto& a, auto& b) { return a.binding < b.binding; });
    for (const auto& b : sorted) {
        const bool dyn = b.descriptorType == VK_DESCRIPTOR_TYPE_UNIFORM_BUFFER_DYNAMIC || b.descriptorType == VK_DESCRIPTOR_TYPE_STORAGE_BUFFER_DYNAMIC;
        if (b.binding == binding) return dyn && index < s.dynamic_offsets[set].size() ? s.dynamic_offsets[set][index] : 0;
        if (dyn) index += b.descriptorCount;
    }
    return 0;
}

void fill_texture(CpvTexture& t, const ImageView* view, const Sampler* sampler) {
    std::memset(&t, 0, sizeof(t));
    if (!view || !view->image || !view->image->memory) return;
    const Image* img = view->image;
    const uint32_t base = view->range.baseMipLevel;
    uint32_t count = view->range.levelCount == VK_REMAINING_MIP_LEVELS ? img->levels - base : view->range.levelCount;
    if (count > CPV_MAX_LEVELS) count = CPV_MAX_LEVELS;
    const uint64_t layer_off = static_cast<uint64_t>(view->range.baseArrayLayer) * img->layer_size;
    const uint64_t base_off = layer_off + img->level[base].offset;
    t.data = img->device_ptr() + base_off;
    t.bytes = img->total_size - base_off;
    t.levels = count;
    t.format = static_cast<uint32_t>(view->format);
    for (uint32_t l = 0; l < count; l++) {
        t.level_offset[l] = img->level[base + l].offset - img->level[base].offset;
        t.level_w[l] = img->level[base + l].width;
        t.level_h[l] = img->level[base + l].height;
    }
    if (sampler) {
        const auto& s = sampler->info;
        t.mag_filter = s.magFilter;
        t.min_filter = s.minFilter;
        t.mipmap_mode = s.mipmapMode;
        t.address_u = s.addressModeU;
        t.address_v = s.addressModeV;
        t.border = s.borderColor;
        t.lod_bias = s.mipLodBias;
        t.min_lod = s.minLod;
        t.max_lod = s.maxLod;
    }
}

uint8_t* view_base(const ImageView* v, uint32_t& width, uint32_t& height) {
    const Image* img = v->image;
    const uint32_t level = v->range.baseMipLevel;
    width = img->level[level].width;
    height = img->level[level].height;
    return img->device_ptr() + static_cast<uint64_t>(v->range.baseArrayLayer) * img->layer_size + img->level[level].offset;
}

// The texel a clear value encodes to in `fmt`: colour through the UNORM8
// encoder in the format's byte order, D16 quantised, D32 as its bits, the
// stencil byte in the second word of a D32S8 texel (ClearImage → SetPixel,
// CPVulkan/CommandBuffer.Draw.cpp:117-149, 2398-2419). False for a format
// without a clear encoding here.
bool clear_texel(VkFormat fmt, const VkClearValue& cv, uint32_t words[4]) {
    for (int i = 0; i < 4; i++) words[i] = 0;
    uint32_t& lo = words[0];
    uint32_t& hi = words[1];
    ColourLayout cl;
    if (colour_layout(fmt, cl)) {
        // each channel through the format's encoder (UNORM, SNORM, half,
        // float), at its bit offset; red in byte 2 for B8G8R8A8
        const int shift_bgra[4] = {16, 8, 0, 24};
        for (uint32_t ch = 0; ch < cl.channels; ch++) {
            uint32_t field;
            if (cl.kind == 3) {  // UINT: the uint32 clear value, clamped to the channel's maximum
                const uint32_t m = cl.bits >= 32 ? 0xFFFFFFFFu : ((1u << cl.bits) - 1u);
                field = std::min(cv.color.uint32[ch], m);
            } else if (cl.kind == 4) {  // SINT: the int32 clear value, clamped to the channel's range
                const int32_t hi_v = cl.bits >= 32 ? INT32_MAX : ((1 << (cl.bits - 1)) - 1), lo_v = -hi_v - 1;
                const int32_t v = std::max(std::min(cv.color.int32[ch], hi_v), lo_v);
                field = static_cast<uint32_t>(v) & (cl.bits >= 32 ? 0xFFFFFFFFu : ((1u << cl.bits) - 1u));
            } else {
                field = encode_channel_host(cv.color.float32[ch], cl);
            }
            // channel ch in 32-bit word ch * bits / 32 (8- and 16-byte texels)
            if (cl.bgra) lo |= field << shift_bgra[ch];
            else words[(cl.bits * ch) >> 5] |= field << ((cl.bits * ch) & 31u);
        }
        return true;
    }
    switch (fmt) {
    case VK_FORMAT_D16_UNORM: lo = encode_unorm_host(cv.depthStencil.depth, 65535.0f); return true;
    case VK_FORMAT_D32_SFLOAT: std::memcpy(&lo, &cv.depthStencil.depth, 4); return true;
    case VK_FORMAT_D32_SFLOAT_S8_UINT:
        std::memcpy(&lo, &cv.depthStencil.depth, 4);
        hi = cv.depthStencil.stencil & 0xFFu;
        return true;
    default: return false;
    }
}

// Fills a rectangle of one layer and level of `img` with a clear value, in
// the aspects `aspects` selects (Vulkan: a clear writes only the aspects it
// names; the reference writes both, CPVulkan/CommandBuffer.Draw.cpp:2201-2203).
VkResult clear_rect(Queue* q, Image* img, uint32_t layer, uint32_t level, VkImageAspectFlags aspects, const VkClearValue& cv, int32_t x0, int32_t y0,
                    uint32_t w, uint32_t h) {
    if (!img || !img->memory || level >= img->levels || layer >= img->layers) return VK_ERROR_DEVICE_LOST;
    const ImageLevel& L = img->level[level];
    // the rectangle within the level
    const int64_t rows = static_cast<int64_t>(L.height) * std::max(1u, L.depth);
    const int64_t x1 = std::min<int64_t>(static_cast<int64_t>(x0) + w, L.width);
    const int64_t y1 = std::min<int64_t>(static_cast<int64_t>(y0) + h, rows);
    x0 = std::max(x0, 0);
    y0 = std::max(y0, 0);
    if (x1 <= x0 || y1 <= y0) return VK_SUCCESS;
    uint32_t words[4];
    if (!clear_texel(img->format, cv, words)) return VK_ERROR_DEVICE_LOST;
    const bool depth = format_is_depth(img->format);
    const bool write_lo = !depth || (aspects & VK_IMAGE_ASPECT_DEPTH_BIT) != 0;
    // the second word: a D32S8 texel's stencil, or an 8-byte colour texel's
    const bool write_hi = depth ? (aspects & VK_IMAGE_ASPECT_STENCIL_BIT) != 0 : true;
    if (!write_lo && (img->texel != 8 || !write_hi)) return VK_SUCCESS;
    uint8_t* base = img->device_ptr() + static_cast<uint64_t>(layer) * img->layer_size + L.offset + static_cast<uint64_t>(y0) * L.stride +
                    static_cast<uint64_t>(x0) * img->texel;
    return rt::fill_rect(q->stream, base, L.stride, static_cast<uint32_t>(x1 - x0), static_cast<uint32_t>(y1 - y0), img->texel, words[0], words[1], write_lo,
                         write_hi, words[2], words[3]) == rt::kOk
               ? VK_SUCCESS
               : VK_ERROR_DEVICE_LOST;
}

VkResult begin_render_pass(Queue* q, State& s, const Cmd& c, std::vector<DeviceMemory*>& written) {
    s.pass = static_cast<RenderPass*>(c.p[0]);
    s.fb = static_cast<Framebuffer*>(c.p[1]);
    s.subpass = 0;
    if (!s.pass || !s.fb || s.pass->subpasses.empty()) return VK_ERROR_DEVICE_LOST;
    for (size_t i = 0; i < s.pass->attachments.size() && i < s.fb->attachments.size(); i++) {
        const auto& a = s.pass->attachments[i];
        ImageView* v = s.fb->attachments[i];
        if (!v || !v->image || !v->image->memory) continue;
        written.push_back(v->image->memory);
        // loadOp CLEAR clears colour or depth, stencilLoadOp CLEAR the
        // stencil (ClearImage → SetPixel through the format encoder,
        // CPVulkan/CommandBuffer.Draw.cpp:117-149)
        const bool depth = format_is_depth(a.format);
        VkImageAspectFlags aspects = 0;
        if (a.loadOp == VK_ATTACHMENT_LOAD_OP_CLEAR) aspects |= depth ? VK_IMAGE_ASPECT_DEPTH_BIT : VK_IMAGE_ASPECT_COLOR_BIT;
        if (depth && format_has_stencil(a.format) && a.stencilLoadOp == VK_ATTACHMENT_LOAD_OP_CLEAR) aspects |= VK_IMAGE_ASPECT_STENCIL_BIT;
        if (!aspects || i >= c.clears.size()) continue;
        const ImageLevel& L = v->image->level[v->range.baseMipLevel];
        const VkResult r = clear_rect(q, v->image, v->range.baseArrayLayer, v->range.baseMipLevel, aspects, c.clears[i], 0, 0, L.width, L.height);
        if (r != VK_SUCCESS) return r;
    }
    return VK_SUCCESS;
}

// Parameters of one draw from the current state: the per-draw path launches
// them, the batched path collects them. `empty` when the draw has no
// primitive.
VkResult build_draw(State& s, uint32_t count, uint32_t instances, uint32_t first, int32_t vertex_offset, uint32_t first_instance, bool indexed,
                    CpvDrawParams& P, bool& empty) {
    Pipeline* p = s.pipeline;
    empty = true;
    if (!p || !s.pass || !s.fb) return VK_ERROR_DEVICE_LOST;
    std::memset(&P, 0, sizeof(P));
    for (int b = 0; b < 8; b++) {
        const BoundVertex& bv = s.vertex[b];
        if (!bv.buffer || !bv.buffer->memory) continue;
        P.vb[b] = bv.buffer->device_ptr(bv.offset);
        P.vb_bytes[b] = bv.offset < bv.buffer->size ? bv.buffer->size - bv.offset : 0;
    }
    if (indexed) {
        if (!s.index || !s.index->memory) return VK_ERROR_DEVICE_LOST;
        P.ib = s.index->device_ptr(s.index_offset);
        P.ib_bytes = s.index_offset < s.index->size ? s.index->size - s.index_offset : 0;
        P.index_size = s.index_size;
    }
    P.count = count;
    P.first = first;
    P.vertex_offset = vertex_offset;
    P.first_instance = first_instance;
    P.instance_count = instances;
    const uint32_t ppi = primitives_per_instance(p->topology, count);
    P.prims_per_instance = ppi;
    P.total_prims = static_cast<uint64_t>(ppi) * instances;
    if (P.total_prims == 0) return VK_SUCCESS;
    for (const auto& slot : p->slots) {
        if (slot.set >= 8 || !s.sets[slot.set]) continue;
        auto it = s.sets[slot.set]->bindings.find(slot.binding);
        if (it == s.sets[slot.set]->bindings.end() || it->second.empty()) continue;
        const Descriptor& d = it->second[0];
        if (slot.is_texture) {
            // a texture joined by OpSampledImage takes its sampler from the
            // sampler's own binding; a storage image has none
            const Sampler* sampler = d.sampler;
            if (slot.separate) {
                sampler = nullptr;
                if (slot.sampler_set < 8 && s.sets[slot.sampler_set]) {
                    auto st = s.sets[slot.sampler_set]->bindings.find(slot.sampler_binding);
                    if (st != s.sets[slot.sampler_set]->bindings.end() && !st->second.empty()) sampler = st->second[0].sampler;
                }
            }
            fill_texture(P.tex[slot.slot], d.view, sampler);
        } else if (d.buffer && d.buffer->memory) {
            const bool dynamic = d.type == VK_DESCRIPTOR_TYPE_UNIFORM_BUFFER_DYNAMIC || d.type == VK_DESCRIPTOR_TYPE_STORAGE_BUFFER_DYNAMIC;
            const uint64_t dyn = dynamic ? dynamic_offset(s, slot.set, slot.binding) : 0;
            const uint64_t off = d.offset + dyn;
            uint64_t range = d.range == VK_WHOLE_SIZE ? (d.buffer->size > off ? d.buffer->size - off : 0) : d.range;
            if (off + range > d.buffer->size) range = d.buffer->size > off ? d.buffer->size - off : 0;
            P.ubo[slot.slot] = d.buffer->device_ptr(off);
            P.ubo_bytes[slot.slot] = range;
        }
    }
    std::memcpy(P.push, s.push, sizeof(P.push));
    // Attachments of the current subpass (no colour attachment in a
    // depth-only one); attachment addressing uses the image row length.
    uint32_t w = 0, h = 0;
    const Subpass& sub = s.sub();
    if (!sub.colour.empty() && sub.colour[0] != VK_ATTACHMENT_UNUSED) P.color = view_base(s.fb->attachments[sub.colour[0]], w, h);
    // the further colour attachments, each the size of the first
    for (size_t k = 1; k < sub.colour.size() && k < CPV_MAX_CA; k++) {
        if (sub.colour[k] == VK_ATTACHMENT_UNUSED) continue;
        uint32_t ew, eh;
        P.color_extra[k - 1] = view_base(s.fb->attachments[sub.colour[k]], ew, eh);
        if (!P.color || ew != w || eh != h) return VK_ERROR_DEVICE_LOST;
    }
    if (sub.depth != VK_ATTACHMENT_UNUSED) {
        uint32_t dw, dh;
        P.depth = view_base(s.fb->attachments[sub.depth], dw, dh);
        if (!P.color) {
            w = dw;
            h = dh;
        } else if (dw != w || dh != h) {
            return VK_ERROR_DEVICE_LOST;
        }
    }
    if (!P.color && !P.depth) return VK_ERROR_DEVICE_LOST;
    P.fb_width = w;
    P.fb_height = h;
    const VkViewport vp = p->dynamic_viewport ? s.viewport : p->viewport;
    P.viewport[0] = vp.x;
    P.viewport[1] = vp.y;
    P.viewport[2] = vp.width;
    P.viewport[3] = vp.height;
    P.viewport[4] = vp.minDepth;
    P.viewport[5] = vp.maxDepth;
    for (int i = 0; i < 4; i++) P.blend_constants[i] = p->dynamic_blend_constants ? s.blend_constants[i] : p->blend_constants[i];
    empty = false;
    return VK_SUCCESS;
}

VkResult draw(Queue* q, State& s, uint32_t count, uint32_t instances, uint32_t first, int32_t vertex_offset, uint32_t first_instance, bool indexed,
              bool no_alloc) {
    CpvDrawParams P;
    bool empty = true;
    const VkResult vr = build_draw(s, count, instances, first, vertex_offset, first_instance, indexed, P, empty);
    if (vr != VK_SUCCESS || empty) return vr;
    Pipeline* p = s.pipeline;
    const int r = no_alloc ? rt::draw_plain_static(q->stream, p->module, P) : rt::draw_plain(q->stream, p->module, P, q->scratch);
    if (r == rt::kErrOutOfMemory) return VK_ERROR_OUT_OF_DEVICE_MEMORY;
    return r == rt::kOk ? VK_SUCCESS : VK_ERROR_DEVICE_LOST;
}

// vkCmdDrawIndirect / vkCmdDrawIndexedIndirect (CPVulkan/CommandBuffer.Draw.cpp:1874-2348):
// the reference reads each VkDraw(Indexed)IndirectCommand from the buffer on
// the CPU and runs the draw. Here too the records are read on the host at
// replay: from the pinned mirror of host-visible memory the device has not
// written, else from HBM after the queue's earlier work has finished.
// `size` bytes of buffer `b` at `offset` as the queue's work up to now
// leaves them: from the pinned mirror of host-visible memory the device has
// not written, else from HBM after the queue's earlier work has finished.
VkResult read_buffer(Queue* q, const Buffer* b, uint64_t offset, uint64_t size, const std::vector<DeviceMemory*>& written, uint8_t* out) {
    if (!b || !b->memory || offset + size > b->size) return VK_ERROR_DEVICE_LOST;
    DeviceMemory* m = b->memory;
    const uint64_t at = b->offset + offset;
    const bool device_newer = !m->host || m->device_dirty || std::find(written.begin(), written.end(), m) != written.end();
    if (!device_newer) {
        std::memcpy(out, m->host + at, size);
    } else if (cudaStreamSynchronize(q->stream) != cudaSuccess || cudaMemcpy(out, m->device + at, size, cudaMemcpyDeviceToHost) != cudaSuccess) {
        cudaGetLastError();
        return VK_ERROR_DEVICE_LOST;
    }
    return VK_SUCCESS;
}

VkResult read_indirect(Queue* q, const Cmd& c, const std::vector<DeviceMemory*>& written, std::vector<IndirectDraw>& out) {
    out.clear();
    const bool indexed = c.type == CmdType::DrawIndexedIndirect;
    uint32_t n = c.u[0];
    const uint32_t stride = c.u[1], record = indexed ? 20u : 16u;
    if (c.p[1]) {  // an indirect-count draw: min(maxDrawCount, the count word)
        uint32_t count = 0;
        const VkResult r = read_buffer(q, static_cast<const Buffer*>(c.p[1]), c.q[1], 4, written, reinterpret_cast<uint8_t*>(&count));
        if (r != VK_SUCCESS) return r;
        n = std::min(n, count);
    }
    if (n == 0) return VK_SUCCESS;
    const uint64_t span = static_cast<uint64_t>(n - 1) * stride + record;
    std::vector<uint8_t> bytes(span);
    const VkResult r = read_buffer(q, static_cast<const Buffer*>(c.p[0]), c.q[0], span, written, bytes.data());
    if (r != VK_SUCCESS) return r;
    out.resize(n);
    for (uint32_t i = 0; i < n; i++) {
        uint32_t v[5] = {0, 0, 0, 0, 0};
        std::memcpy(v, bytes.data() + static_cast<uint64_t>(i) * stride, record);
        if (indexed)  // indexCount, instanceCount, firstIndex, vertexOffset, firstInstance
            out[i] = {v[0], v[1], v[2], static_cast<int32_t>(v[3]), v[4]};
        else  // vertexCount, instanceCount, firstVertex, firstInstance
            out[i] = {v[0], v[1], v[2], 0, v[3]};
    }
    return VK_SUCCESS;
}

VkResult draw_indirect(Queue* q, State& s, const Cmd& c, const std::vector<DeviceMemory*>& written, bool no_alloc) {
    std::vector<IndirectDraw> records;
    const VkResult rr = read_indirect(q, c, written, records);
    if (rr != VK_SUCCESS) return rr;
    const bool indexed = c.type == CmdType::DrawIndexedIndirect;
    for (const IndirectDraw& d : records) {
        const VkResult r = draw(q, s, d.count, d.instances, d.first, d.vertex_offset, d.first_instance, indexed, no_alloc);
        if (r != VK_SUCCESS) return r;
    }
    return VK_SUCCESS;
}

bool is_indirect(const Cmd& c) { return c.type == CmdType::DrawIndirect || c.type == CmdType::DrawIndexedIndirect; }


// Applies a binding / dynamic-state command to `s`; false for any other.
bool apply_state(State& s, const Cmd& c) {
    switch (c.type) {
    case CmdType::NextSubpass:
        // the next subpass's attachments (CPVulkan/CommandBuffer.cpp:649-664)
        if (s.pass && s.subpass + 1 < s.pass->subpasses.size()) s.subpass++;
        return true;
    case CmdType::BindPipeline: s.pipeline = static_cast<Pipeline*>(c.p[0]); return true;
    case CmdType::BindVertexBuffers:
        for (uint32_t i = 0; i < c.u[1]; i++) {
            const uint32_t slot = c.u[0] + i;
            if (slot < 8) {
                s.vertex[slot].buffer = reinterpret_cast<Buffer*>(c.list[2 * i]);
                s.vertex[slot].offset = c.list[2 * i + 1];
            }
        }
        return true;
    case CmdType::BindIndexBuffer:
        s.index = static_cast<Buffer*>(c.p[0]);
        s.index_offset = c.q[0];
        s.index_size = c.u[0] == VK_INDEX_TYPE_UINT16 ? 2 : 4;
        return true;
    case CmdType::BindDescriptorSets: {
        const uint32_t first = c.u[0], count = c.u[1];
        uint32_t dyn_used = 0;
        for (uint32_t i = 0; i < count && first + i < 8; i++) {
            DescriptorSet* ds = reinterpret_cast<DescriptorSet*>(c.list[i]);
            s.sets[first + i] = ds;
            s.dynamic_offsets[first + i].clear();
            if (!ds || !ds->layout) continue;
            for (const auto& b : ds->layout->bindings)
                if (b.descriptorType == VK_DESCRIPTOR_TYPE_UNIFORM_BUFFER_DYNAMIC || b.descriptorType == VK_DESCRIPTOR_TYPE_STORAGE_BUFFER_DYNAMIC)
                    for (uint32_t k = 0; k < b.descriptorCount && dyn_used < c.u[2]; k++)
                        s.dynamic_offsets[first + i].push_back(static_cast<uint32_t>(c.list[count + dyn_used++]));
        }
        return true;
    }
    case CmdType::PushConstants: {
        const uint32_t off = c.u[0];
        const size_t n = c.bytes.size();
        if (off < 128) std::memcpy(s.push + off, c.bytes.data(), off + n <= 128 ? n : 128 - off);
        return true;
    }
    case CmdType::SetViewport: s.viewport = c.viewport; s.viewport_set = true; return true;
    case CmdType::SetScissor: return true;
    case CmdType::SetBlendConstants:
        std::memcpy(s.blend_constants, c.bytes.data(), 16);
        s.blend_set = true;
        return true;
    default: return false;
    }
}

uint32_t env_u32(const char* name, uint32_t dflt) {
    const char* v = std::getenv(name);
    return v && *v ? static_cast<uint32_t>(std::strtoul(v, nullptr, 0)) : dflt;
}

// Module configuration of a batch over `pipelines`.
ModuleConfig batch_config(const std::vector<Pipeline*>& pipelines) {
    bool dense = false, constant = true, samples = false;
    for (const Pipeline* p : pipelines) {
        dense = dense || p->prefers_deferred;
        constant = constant && p->fs_constant;
        samples = samples || p->samples;
    }
    return module_config(pipelines[0]->tile_shift, dense, constant, samples);
}

// ---- which render passes run batched ----
//
// A pass of at least CPV_BATCH_MIN_DRAWS (16) draws, or of at least
// CPV_BATCH_MIN_PRIMS (2^20) primitives when none of its pipelines uses
// blend tables (CPV_BATCH=0: none). The second rule exists because the
// per-draw path bins through a (tile x span) count matrix whose size grows
// with the tiles times the primitives / 256, while the batched path sorts
// the (tile, primitive) pairs: the 2.09 M-triangle heightfield renders in
// 0.59 ms batched against 0.74 ms per draw. Blend-table pipelines stay per
// draw, where their tables exist (the 400k-triangle blend scene: 2.84 ms per
// draw, 3.28 ms batched).
// Indirect draws count as the draws their records hold (at recording, where
// the records are not read yet, as their maximum draw count, with no
// primitives).
struct PassCensus {
    Pipeline* bound = nullptr;
    size_t draws = 0;
    uint64_t prims = 0;
    bool blend_tables = false;
    bool subpasses = false;  // a pass of several subpasses runs per draw
    void add(const Cmd& c, const std::vector<IndirectDraw>* records = nullptr) {
        if (c.type == CmdType::BindPipeline) bound = static_cast<Pipeline*>(c.p[0]);
        if (c.type == CmdType::NextSubpass) subpasses = true;
        if (is_indirect(c)) {
            draws += records ? records->size() : c.u[0];
            if (!bound) return;
            if (records)
                for (const IndirectDraw& d : *records) prims += static_cast<uint64_t>(primitives_per_instance(bound->topology, d.count)) * d.instances;
            blend_tables = blend_tables || ((records ? !records->empty() : c.u[0] > 0) && bound->blend_table);
            return;
        }
        if (c.type != CmdType::Draw && c.type != CmdType::DrawIndexed) return;
        draws++;
        if (!bound) return;
        prims += static_cast<uint64_t>(primitives_per_instance(bound->topology, c.u[0])) * c.u[1];
        blend_tables = blend_tables || bound->blend_table;
    }
    bool batches() const {
        if (env_u32("CPV_BATCH", 1u) == 0u || draws == 0 || subpasses) return false;
        if (draws >= env_u32("CPV_BATCH_MIN_DRAWS", 16u)) return true;
        return !blend_tables && prims >= env_u32("CPV_BATCH_MIN_PRIMS", 1u << 20);
    }
};

// ---- batch tuner ----
//
// The tile size and the warps per tile CTA change only the speed of a batch,
// never its image: every configuration applies each pixel's fragments in API
// order. The tuner therefore times the pass itself under each candidate and
// keeps the fastest (CPV_AUTOTUNE: 0 off, 1 every batched pass, default
// passes of at least CPV_AUTOTUNE_MIN_DRAWS = 256 draws; an explicit
// CPV_TILE or CPV_RT_WARPS turns it off).

thread_local std::string g_last_tuning;

bool tuning_enabled(size_t draws) {
    const uint32_t mode = env_u32("CPV_AUTOTUNE", 2u);
    if (mode == 0u || std::getenv("CPV_TILE") || std::getenv("CPV_RT_WARPS")) return false;
    return mode == 1u || draws >= env_u32("CPV_AUTOTUNE_MIN_DRAWS", 256u);
}

// Tile 8, 16 and 32 px, each with the warp counts that suit its pixels, and
// for 16 px tiles also 128-primitive batches and the other fast schedule
// (immediate for a sparse module, sparse for an immediate one).
std::vector<ModuleConfig> tune_candidates(const ModuleConfig& base) {
    static const uint32_t shapes[][2] = {{3, 2}, {4, 4}, {4, 8}, {5, 8}, {5, 16}};
    std::vector<ModuleConfig> out;
    for (const auto& s : shapes) {
        ModuleConfig mc = base;
        mc.tile_shift = s[0];
        mc.warps = s[1];
        out.push_back(mc);
    }
    ModuleConfig half = base;
    half.tile_shift = 4;
    half.warps = 8;
    half.batch = base.batch == 256u ? 128u : 256u;
    out.push_back(half);
    ModuleConfig other = base;
    other.tile_shift = 4;
    other.warps = 8;
    other.schedule = base.schedule == 0u ? 2u : 0u;
    other.batch = other.schedule == 0u ? 128u : 256u;
    out.push_back(other);
    // the sparse schedule's fragment-list depth per pixel and batch (the
    // bin-queue depth): the default (24, or 16 when a fragment shader
    // samples) and one shallower and one deeper
    if (base.schedule == 2u) {
        const uint32_t d = base.samples ? 16u : 24u;
        for (uint32_t depth : {d - 8u, d + 8u}) {
            ModuleConfig q = base;
            q.tile_shift = 4;
            q.warps = 8;
            q.depth = depth;
            out.push_back(q);
        }
    }
    return out;
}

// Compiles (NVRTC, one thread per candidate) and loads the candidates'
// modules; null where a candidate failed.
std::vector<rt::Module*> candidate_modules(Device* dev, const std::vector<Pipeline*>& pipelines, const std::vector<ModuleConfig>& cands) {
    std::vector<rt::Module*> out(cands.size(), nullptr);
    std::vector<std::thread> workers;
    for (size_t i = 0; i < cands.size(); i++)
        workers.emplace_back([&, i]() { out[i] = batch_module(dev, pipelines, cands[i]); });
    for (auto& w : workers) w.join();
    return out;
}

std::string batch_signature(const std::vector<Pipeline*>& pipelines, const rt::BatchDraws& in) {
    uint64_t prims = 0;
    for (const CpvDrawParams& P : in.draws) prims += P.total_prims;
    std::string sig = std::to_string(in.draws.size()) + "/" + std::to_string(prims) + "/" + std::to_string(in.fb_width) + "x" +
                      std::to_string(in.fb_height);
    for (const Pipeline* p : pipelines)
        for (uint8_t b : p->key) sig += static_cast<char>('a' + (b & 15)), sig += static_cast<char>('a' + (b >> 4));
    return sig;
}

// Times every candidate on the pass and returns the fastest module and plan.
// The attachments are saved first and restored before each run and at the
// end, so the pass still renders once from its initial contents.
bool tune_batch(Queue* q, Device* dev, const std::vector<Pipeline*>& pipelines, const rt::BatchDraws& in, uint64_t color_bytes,
                uint64_t depth_bytes, ModuleConfig& chosen, rt::Module*& best_m, std::unique_ptr<rt::BatchPlan>& best_plan) {
    const std::vector<ModuleConfig> cands = tune_candidates(batch_config(pipelines));
    const std::vector<rt::Module*> mods = candidate_modules(dev, pipelines, cands);
    uint8_t* saved = nullptr;
    if (cudaMalloc(&saved, color_bytes + depth_bytes) != cudaSuccess) return false;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    bool ok = cudaEventCreate(&e0) == cudaSuccess && cudaEventCreate(&e1) == cudaSuccess;
    auto copy = [&](bool restore) {
        bool good = true;
        if (color_bytes)
            good = cudaMemcpyAsync(restore ? in.color : saved, restore ? saved : in.color, color_bytes, cudaMemcpyDeviceToDevice, q->stream) == cudaSuccess;
        if (depth_bytes)
            good = good && cudaMemcpyAsync(restore ? in.depth : saved + color_bytes, restore ? saved + color_bytes : in.depth, depth_bytes,
                                           cudaMemcpyDeviceToDevice, q->stream) == cudaSuccess;
        return good;
    };
    ok = ok && copy(false);
    float best_ms = 0.0f;
    std::string report;
    for (size_t i = 0; ok && i < cands.size(); i++) {
        if (!mods[i]) continue;
        auto plan = std::make_unique<rt::BatchPlan>();
        if (plan->build(*mods[i], in, q->stream) != rt::kOk) continue;
        // One warm run (graph capture, pair-buffer growth), one timed run.
        if (!copy(true) || plan->launch(*mods[i], q->stream) != rt::kOk || !copy(true)) continue;
        if (cudaEventRecord(e0, q->stream) != cudaSuccess || plan->launch(*mods[i], q->stream) != rt::kOk ||
            cudaEventRecord(e1, q->stream) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess)
            continue;
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        char line[96];
        std::snprintf(line, sizeof(line), "%stile %u warps %u schedule %u batch %u depth %u: %.3f ms", report.empty() ? "" : "; ",
                      1u << cands[i].tile_shift, cands[i].warps, cands[i].schedule, cands[i].batch, cands[i].depth, ms);
        report += line;
        if (!best_plan || ms < best_ms) {
            best_ms = ms;
            chosen = cands[i];
            best_m = mods[i];
            best_plan = std::move(plan);
        }
    }
    ok = copy(true) && ok;
    cudaStreamSynchronize(q->stream);
    cudaFree(saved);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (best_plan) {
        char line[96];
        std::snprintf(line, sizeof(line), "; chosen tile %u warps %u schedule %u batch %u depth %u", 1u << chosen.tile_shift, chosen.warps,
                      chosen.schedule, chosen.batch, chosen.depth);
        g_last_tuning = report + line;
    }
    return ok && best_plan != nullptr;
}

// Builds the batch of the render pass whose commands are (begin, end): the
// draws' parameters, the pipeline set, the batched module and the plan.
// Leaves state->plain set when the pass does not batch.
void build_batch(Queue* q, const CommandBuffer* cb, size_t begin, size_t end, const State& entry, const PassIndirect& indirect, BatchState& state) {
    state.plain = true;
    State s = entry;
    rt::BatchDraws in;
    std::vector<Pipeline*> pipelines;
    float vw = 0.0f, vh = 0.0f;
    // false when the draw cannot join the batch
    auto add = [&](uint32_t count, uint32_t instances, uint32_t first, int32_t vertex_offset, uint32_t first_instance, bool indexed) {
        CpvDrawParams P;
        bool empty = true;
        if (build_draw(s, count, instances, first, vertex_offset, first_instance, indexed, P, empty) != VK_SUCCESS) return false;
        if (empty) return true;
        auto it = std::find(pipelines.begin(), pipelines.end(), s.pipeline);
        if (it == pipelines.end()) {
            if (pipelines.size() == 16) return false;  // 4-bit pipeline index
            pipelines.push_back(s.pipeline);
            it = pipelines.end() - 1;
        }
        if (in.draws.empty()) {
            vw = P.viewport[2];
            vh = P.viewport[3];
            in.color = P.color;
            in.depth = P.depth;
            for (int k = 0; k < CPV_MAX_CA - 1; k++) in.color_extra[k] = P.color_extra[k];
            in.fb_width = P.fb_width;
            in.fb_height = P.fb_height;
        } else if (P.viewport[2] != vw || P.viewport[3] != vh) {
            return false;  // pixel centres depend on the viewport extent
        }
        in.draws.push_back(P);
        in.pipeline.push_back(static_cast<uint32_t>(it - pipelines.begin()));
        const VkPrimitiveTopology topo = s.pipeline->topology;
        in.triangles.push_back(topo == VK_PRIMITIVE_TOPOLOGY_TRIANGLE_LIST || topo == VK_PRIMITIVE_TOPOLOGY_TRIANGLE_STRIP ||
                               topo == VK_PRIMITIVE_TOPOLOGY_TRIANGLE_FAN);
        return true;
    };
    size_t next_indirect = 0;
    for (size_t i = begin + 1; i < end; i++) {
        const Cmd& c = cb->cmds[i];
        if (apply_state(s, c)) continue;
        if (is_indirect(c)) {
            if (next_indirect >= indirect.size() || indirect[next_indirect].first != i) return;
            const bool indexed = c.type == CmdType::DrawIndexedIndirect;
            for (const IndirectDraw& d : indirect[next_indirect].second)
                if (!add(d.count, d.instances, d.first, d.vertex_offset, d.first_instance, indexed)) return;
            next_indirect++;
            continue;
        }
        if (c.type != CmdType::Draw && c.type != CmdType::DrawIndexed) return;
        const bool indexed = c.type == CmdType::DrawIndexed;
        if (!add(c.u[0], c.u[1], c.u[2], indexed ? c.i0 : 0, c.u[3], indexed)) return;
    }
    if (in.draws.empty()) return;
    in.vw = vw;
    in.vh = vh;
    Device* dev = cb->device;
    ModuleConfig mc = batch_config(pipelines);
    if (tuning_enabled(in.draws.size())) {
        const std::string sig = batch_signature(pipelines, in);
        bool known = false;
        {
            std::lock_guard<std::mutex> lock(dev->batch_mutex);
            auto it = dev->tuned.find(sig);
            if (it != dev->tuned.end()) {
                mc = it->second;
                known = true;
            }
        }
        if (!known) {
            const uint32_t w = in.fb_width, h = in.fb_height;
            const uint64_t color_bytes = in.color ? static_cast<uint64_t>(w) * h * 4u : 0u;
            uint64_t depth_bytes = 0;
            if (s.sub().depth != VK_ATTACHMENT_UNUSED) {
                const ImageView* dv = s.fb->attachments[s.sub().depth];
                depth_bytes = static_cast<uint64_t>(w) * h * dv->image->texel;
            }
            rt::Module* m = nullptr;
            std::unique_ptr<rt::BatchPlan> plan;
            if (tune_batch(q, dev, pipelines, in, color_bytes, depth_bytes, mc, m, plan)) {
                std::lock_guard<std::mutex> lock(dev->batch_mutex);
                dev->tuned[sig] = mc;
                state.module = m;
                state.plan = std::move(plan);
                state.plain = false;
                return;
            }
            mc = batch_config(pipelines);
        }
    }
    rt::Module* m = batch_module(dev, pipelines, mc);
    if (!m) return;
    auto plan = std::make_unique<rt::BatchPlan>();
    if (plan->build(*m, in, q->stream) != rt::kOk) return;
    state.module = m;
    state.plan = std::move(plan);
    state.plain = false;
}

// Runs the render pass (begin, end) batched when it batches: returns true
// after enqueuing it, with `s` advanced past its commands; false leaves the
// pass to the per-draw path.
// A pass with indirect draws reads their records at every submission; its
// batch is rebuilt when they differ from the records it was built from.
bool run_batched(Queue* q, CommandBuffer* cb, size_t begin, size_t end, State& s, const std::vector<DeviceMemory*>& written, VkResult& result) {
    PassIndirect indirect;
    for (size_t i = begin + 1; i < end; i++) {
        if (!is_indirect(cb->cmds[i])) continue;
        indirect.emplace_back(i, std::vector<IndirectDraw>());
        if (read_indirect(q, cb->cmds[i], written, indirect.back().second) != VK_SUCCESS) return false;  // the per-draw path reports it
    }
    PassCensus census;
    census.bound = s.pipeline;
    size_t next_indirect = 0;
    for (size_t i = begin + 1; i < end; i++) {
        const Cmd& c = cb->cmds[i];
        census.add(c, is_indirect(c) ? &indirect[next_indirect++].second : nullptr);
    }
    if (!census.batches()) return false;
    auto& slot = cb->batches[begin];
    if (slot && slot->indirect != indirect) {
        // the old plan's buffers may still be in use by this queue's work
        if (cudaStreamSynchronize(q->stream) != cudaSuccess) {
            cudaGetLastError();
            result = VK_ERROR_DEVICE_LOST;
            return true;
        }
        slot.reset();
    }
    if (!slot) {
        slot = std::make_unique<BatchState>();
        slot->indirect = indirect;
        build_batch(q, cb, begin, end, s, indirect, *slot);
    }
    if (slot->plain) return false;
    for (size_t i = begin + 1; i < end; i++) apply_state(s, cb->cmds[i]);
    rt::profile_begin(q->stream, "cpv_batch");
    result = slot->plan->launch(*slot->module, q->stream) == rt::kOk ? VK_SUCCESS : VK_ERROR_DEVICE_LOST;
    rt::profile_end(q->stream);
    return true;
}

}  // namespace

VkResult execute(Queue* q, CommandBuffer* cb, std::vector<DeviceMemory*>& written, bool no_alloc) {
    State s;
    for (size_t idx = 0; idx < cb->cmds.size(); idx++) {
        const Cmd& c = cb->cmds[idx];
        if (apply_state(s, c)) continue;
        VkResult r = VK_SUCCESS;
        switch (c.type) {
        case CmdType::BeginRenderPass: {
            r = begin_render_pass(q, s, c, written);
            if (r != VK_SUCCESS || no_alloc) break;
            size_t end = idx + 1;
            while (end < cb->cmds.size() && cb->cmds[end].type != CmdType::EndRenderPass) end++;
            if (end < cb->cmds.size() && run_batched(q, cb, idx, end, s, written, r)) idx = end - 1;  // continue at EndRenderPass
            break;
        }
        case CmdType::EndRenderPass: s.pass = nullptr; s.fb = nullptr; break;
        case CmdType::Draw: r = draw(q, s, c.u[0], c.u[1], c.u[2], 0, c.u[3], false, no_alloc); break;
        case CmdType::DrawIndexed: r = draw(q, s, c.u[0], c.u[1], c.u[2], c.i0, c.u[3], true, no_alloc); break;
        case CmdType::CopyBuffer: {
            Buffer* src = static_cast<Buffer*>(c.p[0]);
            Buffer* dst = static_cast<Buffer*>(c.p[1]);
            for (const auto& reg : c.buffer_regions) {
                if (reg.srcOffset + reg.size > src->size || reg.dstOffset + reg.size > dst->size) return VK_ERROR_DEVICE_LOST;
                if (cudaMemcpyAsync(dst->device_ptr(reg.dstOffset), src->device_ptr(reg.srcOffset), reg.size, cudaMemcpyDeviceToDevice, q->stream) != cudaSuccess)
                    return VK_ERROR_DEVICE_LOST;
            }
            written.push_back(dst->memory);
            break;
        }
        case CmdType::CopyBufferToImage:
        case CmdType::CopyImageToBuffer: {
            const bool to_image = c.type == CmdType::CopyBufferToImage;
            Buffer* buf = static_cast<Buffer*>(c.p[0]);
            Image* img = static_cast<Image*>(c.p[1]);
            for (const auto& reg : c.image_regions) {
                const uint32_t level = reg.imageSubresource.mipLevel;
                if (level >= img->levels) return VK_ERROR_DEVICE_LOST;
                const ImageLevel& L = img->level[level];
                const uint32_t texel = img->texel;
                const uint32_t row_len = reg.bufferRowLength ? reg.bufferRowLength : reg.imageExtent.width;
                const uint32_t img_h = reg.bufferImageHeight ? reg.bufferImageHeight : reg.imageExtent.height;
                for (uint32_t layer = 0; layer < reg.imageSubresource.layerCount; layer++) {
                    for (uint32_t z = 0; z < reg.imageExtent.depth; z++) {
                        const uint64_t img_off = static_cast<uint64_t>(reg.imageSubresource.baseArrayLayer + layer) * img->layer_size + L.offset +
                                                 static_cast<uint64_t>(reg.imageOffset.z + z) * L.plane + static_cast<uint64_t>(reg.imageOffset.y) * L.stride +
                                                 static_cast<uint64_t>(reg.imageOffset.x) * texel;
                        const uint64_t buf_off = reg.bufferOffset + (static_cast<uint64_t>(layer) * reg.imageExtent.depth + z) * row_len * img_h * texel;
                        const uint64_t width_bytes = static_cast<uint64_t>(reg.imageExtent.width) * texel;
                        if (buf_off + static_cast<uint64_t>(row_len) * texel * (reg.imageExtent.height - 1) + width_bytes > buf->size) return VK_ERROR_DEVICE_LOST;
                        if (img_off + L.stride * (reg.imageExtent.height - 1) + width_bytes > img->total_size) return VK_ERROR_DEVICE_LOST;
                        uint8_t* ip = img->device_ptr() + img_off;
                        uint8_t* bp = buf->device_ptr(buf_off);
                        cudaError_t e;
                        if (to_image)
                            e = cudaMemcpy2DAsync(ip, L.stride, bp, static_cast<size_t>(row_len) * texel, width_bytes, reg.imageExtent.height, cudaMemcpyDeviceToDevice, q->stream);
                        else
                            e = cudaMemcpy2DAsync(bp, static_cast<size_t>(row_len) * texel, ip, L.stride, width_bytes, reg.imageExtent.height, cudaMemcpyDeviceToDevice, q->stream);
                        if (e != cudaSuccess) return VK_ERROR_DEVICE_LOST;
                    }
                }
            }
            written.push_back(to_image ? img->memory : buf->memory);
            break;
        }
        case CmdType::BlitImage: {
            // Colour regions between RGBA8/BGRA8 2D images (depth/stencil
            // blits, other formats and 3D regions are not implemented).
            Image* src = static_cast<Image*>(c.p[0]);
            Image* dst = static_cast<Image*>(c.p[1]);
            auto colour8 = [](VkFormat f) { return f == VK_FORMAT_R8G8B8A8_UNORM || f == VK_FORMAT_B8G8R8A8_UNORM; };
            if (!src || !dst || !src->memory || !dst->memory || !colour8(src->format) || !colour8(dst->format)) return VK_ERROR_DEVICE_LOST;
            for (const VkImageBlit& b : c.blit_regions) {
                const auto& ss = b.srcSubresource;
                const auto& ds = b.dstSubresource;
                if (ss.aspectMask != VK_IMAGE_ASPECT_COLOR_BIT || ss.mipLevel >= src->levels || ds.mipLevel >= dst->levels ||
                    ss.layerCount != ds.layerCount || b.srcOffsets[1].z - b.srcOffsets[0].z != 1 || b.dstOffsets[1].z - b.dstOffsets[0].z != 1)
                    return VK_ERROR_DEVICE_LOST;
                const ImageLevel& sl = src->level[ss.mipLevel];
                const ImageLevel& dl = dst->level[ds.mipLevel];
                for (uint32_t layer = 0; layer < ss.layerCount; layer++) {
                    if (ss.baseArrayLayer + layer >= src->layers || ds.baseArrayLayer + layer >= dst->layers) return VK_ERROR_DEVICE_LOST;
                    CpvTexture t;
                    std::memset(&t, 0, sizeof(t));
                    t.data = src->device_ptr() + static_cast<uint64_t>(ss.baseArrayLayer + layer) * src->layer_size + sl.offset;
                    t.bytes = sl.size;
                    t.levels = 1;
                    t.level_w[0] = sl.width;
                    t.level_h[0] = sl.height;
                    t.format = static_cast<uint32_t>(src->format);
                    t.address_u = t.address_v = VK_SAMPLER_ADDRESS_MODE_CLAMP_TO_EDGE;
                    uint8_t* out = dst->device_ptr() + static_cast<uint64_t>(ds.baseArrayLayer + layer) * dst->layer_size + dl.offset;
                    const int32_t sr[4] = {b.srcOffsets[0].x, b.srcOffsets[0].y, b.srcOffsets[1].x, b.srcOffsets[1].y};
                    const int32_t dr[4] = {b.dstOffsets[0].x, b.dstOffsets[0].y, b.dstOffsets[1].x, b.dstOffsets[1].y};
                    if (rt::blit(q->stream, t, out, dl.width, dl.height, static_cast<uint32_t>(dst->format), sr, dr, c.u[0]) != rt::kOk)
                        return VK_ERROR_DEVICE_LOST;
                }
            }
            written.push_back(dst->memory);
            break;
        }
        case CmdType::CopyImage: {
            // Regions between images of one texel size, row by row
            // (CPVulkan/CommandBuffer.Copy.cpp:1091-1095).
            Image* src = static_cast<Image*>(c.p[0]);
            Image* dst = static_cast<Image*>(c.p[1]);
            if (!src || !dst || !src->memory || !dst->memory || src->texel != dst->texel) return VK_ERROR_DEVICE_LOST;
            const uint32_t texel = src->texel;
            for (const VkImageCopy& rg : c.image_copies) {
                const auto& ss = rg.srcSubresource;
                const auto& ds = rg.dstSubresource;
                if (ss.mipLevel >= src->levels || ds.mipLevel >= dst->levels || ss.layerCount != ds.layerCount) return VK_ERROR_DEVICE_LOST;
                const ImageLevel& sl = src->level[ss.mipLevel];
                const ImageLevel& dl = dst->level[ds.mipLevel];
                auto inside = [](const ImageLevel& L, const VkOffset3D& o, const VkExtent3D& e) {
                    return o.x >= 0 && o.y >= 0 && o.z >= 0 && static_cast<uint64_t>(o.x) + e.width <= L.width && static_cast<uint64_t>(o.y) + e.height <= L.height &&
                           static_cast<uint64_t>(o.z) + e.depth <= std::max(1u, L.depth);
                };
                if (!inside(sl, rg.srcOffset, rg.extent) || !inside(dl, rg.dstOffset, rg.extent)) return VK_ERROR_DEVICE_LOST;
                if (ss.baseArrayLayer + ss.layerCount > src->layers || ds.baseArrayLayer + ds.layerCount > dst->layers) return VK_ERROR_DEVICE_LOST;
                if (rg.extent.width == 0 || rg.extent.height == 0) continue;
                for (uint32_t layer = 0; layer < ss.layerCount; layer++) {
                    for (uint32_t z = 0; z < std::max(1u, rg.extent.depth); z++) {
                        const uint8_t* sp = src->device_ptr() + static_cast<uint64_t>(ss.baseArrayLayer + layer) * src->layer_size + sl.offset +
                                            static_cast<uint64_t>(rg.srcOffset.z + z) * sl.plane + static_cast<uint64_t>(rg.srcOffset.y) * sl.stride +
                                            static_cast<uint64_t>(rg.srcOffset.x) * texel;
                        uint8_t* dp = dst->device_ptr() + static_cast<uint64_t>(ds.baseArrayLayer + layer) * dst->layer_size + dl.offset +
                                      static_cast<uint64_t>(rg.dstOffset.z + z) * dl.plane + static_cast<uint64_t>(rg.dstOffset.y) * dl.stride +
                                      static_cast<uint64_t>(rg.dstOffset.x) * texel;
                        if (cudaMemcpy2DAsync(dp, dl.stride, sp, sl.stride, static_cast<size_t>(rg.extent.width) * texel, rg.extent.height, cudaMemcpyDeviceToDevice,
                                              q->stream) != cudaSuccess)
                            return VK_ERROR_DEVICE_LOST;
                    }
                }
            }
            written.push_back(dst->memory);
            break;
        }
        case CmdType::ClearImage: {
            Image* img = static_cast<Image*>(c.p[0]);
            if (!img || !img->memory || c.clears.empty()) return VK_ERROR_DEVICE_LOST;
            for (const VkImageSubresourceRange& rg : c.ranges) {
                const uint32_t levels = rg.levelCount == VK_REMAINING_MIP_LEVELS ? img->levels - std::min(rg.baseMipLevel, img->levels) : rg.levelCount;
                const uint32_t layers = rg.layerCount == VK_REMAINING_ARRAY_LAYERS ? img->layers - std::min(rg.baseArrayLayer, img->layers) : rg.layerCount;
                if (static_cast<uint64_t>(rg.baseMipLevel) + levels > img->levels || static_cast<uint64_t>(rg.baseArrayLayer) + layers > img->layers)
                    return VK_ERROR_DEVICE_LOST;
                for (uint32_t layer = 0; layer < layers; layer++)
                    for (uint32_t level = 0; level < levels; level++) {
                        const ImageLevel& L = img->level[rg.baseMipLevel + level];
                        const VkResult r = clear_rect(q, img, rg.baseArrayLayer + layer, rg.baseMipLevel + level, rg.aspectMask, c.clears[0], 0, 0, L.width,
                                                      L.height * std::max(1u, L.depth));
                        if (r != VK_SUCCESS) return r;
                    }
            }
            written.push_back(img->memory);
            break;
        }
        case CmdType::ClearAttachments: {
            // Rectangles of the current subpass's attachments
            // (CPVulkan/CommandBuffer.Draw.cpp:2142-2224); a colour index or
            // depth attachment the subpass does not use is not cleared.
            if (!s.pass || !s.fb) return VK_ERROR_DEVICE_LOST;
            for (const VkClearAttachment& a : c.clear_attachments) {
                uint32_t index = VK_ATTACHMENT_UNUSED;
                if (a.aspectMask & VK_IMAGE_ASPECT_COLOR_BIT) {
                    if (a.colorAttachment < s.sub().colour.size()) index = s.sub().colour[a.colorAttachment];
                } else {
                    index = s.sub().depth;
                }
                if (index == VK_ATTACHMENT_UNUSED || index >= s.fb->attachments.size() || !s.fb->attachments[index]) continue;
                const ImageView* v = s.fb->attachments[index];
                for (const VkClearRect& rect : c.clear_rects)
                    for (uint32_t layer = 0; layer < rect.layerCount; layer++) {
                        const VkResult r = clear_rect(q, v->image, v->range.baseArrayLayer + rect.baseArrayLayer + layer, v->range.baseMipLevel, a.aspectMask,
                                                      a.clearValue, rect.rect.offset.x, rect.rect.offset.y, rect.rect.extent.width, rect.rect.extent.height);
                        if (r != VK_SUCCESS) return r;
                    }
                written.push_back(v->image->memory);
            }
            break;
        }
        case CmdType::FillBuffer: {
            Buffer* dst = static_cast<Buffer*>(c.p[0]);
            uint64_t off = c.q[0], size = c.q[1];
            if (size == VK_WHOLE_SIZE) size = (dst->size - off) & ~3ull;
            if (off + size > dst->size) return VK_ERROR_DEVICE_LOST;
            if (rt::fill(q->stream, dst->device_ptr(off), size / 4, 4, c.u[0], 0) != rt::kOk) return VK_ERROR_DEVICE_LOST;
            written.push_back(dst->memory);
            break;
        }
        case CmdType::UpdateBuffer: {
            Buffer* dst = static_cast<Buffer*>(c.p[0]);
            if (c.q[0] + c.bytes.size() > dst->size) return VK_ERROR_DEVICE_LOST;
            // The command owns its bytes until the command buffer is reset;
            // the copy is ordered on the stream.
            if (cudaMemcpyAsync(dst->device_ptr(c.q[0]), c.bytes.data(), c.bytes.size(), cudaMemcpyHostToDevice, q->stream) != cudaSuccess)
                return VK_ERROR_DEVICE_LOST;
            written.push_back(dst->memory);
            break;
        }
        case CmdType::DrawIndirect:
        case CmdType::DrawIndexedIndirect: r = draw_indirect(q, s, c, written, no_alloc); break;
        case CmdType::Barrier:
        default:
            break;
        }
        if (r != VK_SUCCESS) return r;
    }
    return VK_SUCCESS;
}

void CommandBuffer::reset() {
    for (auto& kv : graphs)
        if (kv.second.exec) cudaGraphExecDestroy(kv.second.exec);
    graphs.clear();
    cmds.clear();
    batches.clear();
    written.clear();
    graphable = -1;
}

VkResult run_command_buffer(Queue* q, CommandBuffer* cb, std::vector<DeviceMemory*>& written, bool no_alloc) {
    if (no_alloc || rt::profile_enabled() || env_u32("CPV_CB_GRAPH", 1u) == 0u || cb->graphable == 0) return execute(q, cb, written, no_alloc);
    if (cb->graphable < 0) {
        // First execution: eager. It decides whether the buffer can be a graph
        // (its commands read no host memory and no pass runs batched, whose
        // plans keep graphs of their own) and records what it writes.
        const size_t before = written.size();
        const VkResult r = execute(q, cb, written, false);
        if (r != VK_SUCCESS) return r;
        bool ok = true;  // indirect draws read their arguments on the host at every replay
        for (const Cmd& c : cb->cmds)
            ok = ok && c.type != CmdType::UpdateBuffer && c.type != CmdType::DrawIndirect && c.type != CmdType::DrawIndexedIndirect;
        for (const auto& kv : cb->batches) ok = ok && kv.second->plain;
        cb->graphable = ok ? 1 : 0;
        cb->written.assign(written.begin() + static_cast<std::ptrdiff_t>(before), written.end());
        cb->graphs[q].warm = true;
        return VK_SUCCESS;
    }
    QueueGraph& g = cb->graphs[q];
    if (g.exec && g.generation != q->scratch.generation()) {
        cudaGraphExecDestroy(g.exec);  // the queue's scratch moved since the capture
        g.exec = nullptr;
    }
    if (!g.exec) {
        if (!g.warm) {
            // First run on this queue sizes its scratch; capture on the next.
            g.warm = true;
            return execute(q, cb, written, false);
        }
        cudaGraph_t graph = nullptr;
        std::vector<DeviceMemory*> w;
        const uint64_t before = rt::launches();
        if (cudaStreamBeginCapture(q->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
            cudaGetLastError();
            cb->graphable = 0;
            return execute(q, cb, written, false);
        }
        const VkResult r = execute(q, cb, w, false);
        const cudaError_t e = cudaStreamEndCapture(q->stream, &graph);
        g.kernels = rt::launches() - before;
        rt::count_launch(0 - g.kernels);  // captured, not launched yet
        if (r != VK_SUCCESS || e != cudaSuccess || cudaGraphInstantiate(&g.exec, graph, 0) != cudaSuccess) {
            if (graph) cudaGraphDestroy(graph);
            cudaGetLastError();
            g.exec = nullptr;
            cb->graphable = 0;  // fall back to eager execution for good
            return execute(q, cb, written, false);
        }
        cudaGraphDestroy(graph);
        g.generation = q->scratch.generation();
    }
    if (cudaGraphLaunch(g.exec, q->stream) != cudaSuccess) {
        cudaGetLastError();
        return VK_ERROR_DEVICE_LOST;
    }
    rt::count_launch(g.kernels);
    written.insert(written.end(), cb->written.begin(), cb->written.end());
    return VK_SUCCESS;
}

void precompile_batches(CommandBuffer* cb) {
    if (env_u32("CPV_BATCH", 1u) == 0u) return;
    Pipeline* bound = nullptr;
    std::vector<Pipeline*> pipelines;
    PassCensus census;
    bool in_pass = false;
    for (const Cmd& c : cb->cmds) {
        if (c.type == CmdType::BindPipeline) bound = static_cast<Pipeline*>(c.p[0]);
        switch (c.type) {
        case CmdType::BeginRenderPass:
            in_pass = true;
            pipelines.clear();
            census = PassCensus{};
            census.bound = bound;
            break;
        case CmdType::BindPipeline:
        case CmdType::NextSubpass:
            if (in_pass) census.add(c);
            break;
        case CmdType::Draw:
        case CmdType::DrawIndexed:
        case CmdType::DrawIndirect:
        case CmdType::DrawIndexedIndirect:
            if (!in_pass || !bound) break;
            census.add(c);
            if (std::find(pipelines.begin(), pipelines.end(), bound) == pipelines.end()) pipelines.push_back(bound);
            break;
        case CmdType::EndRenderPass:
            // Compiled and cached; errors surface at submit. A pass the tuner
            // will time gets every candidate compiled now, in parallel.
            if (in_pass && census.batches() && !pipelines.empty() && pipelines.size() <= 16) {
                if (tuning_enabled(census.draws))
                    candidate_modules(cb->device, pipelines, tune_candidates(batch_config(pipelines)));
                else
                    batch_module(cb->device, pipelines, batch_config(pipelines));
            }
            in_pass = false;
            break;
        default: break;
        }
    }
}

const char* last_tuning() { return g_last_tuning.c_str(); }

VkResult check_no_alloc(Queue* q, CommandBuffer* cb) {
    Pipeline* pipeline = nullptr;
    RenderPass* pass = nullptr;
    Framebuffer* fb = nullptr;
    uint32_t subpass = 0;
    // The attachment that sizes a draw of the current subpass: colour, else
    // depth. False when there is none (execute() reports that).
    auto target = [&](uint32_t& w, uint32_t& h) {
        if (!pipeline || !pass || !fb || subpass >= pass->subpasses.size()) return false;
        const Subpass& sub = pass->subpasses[subpass];
        const uint32_t index = !sub.colour.empty() && sub.colour[0] != VK_ATTACHMENT_UNUSED ? sub.colour[0] : sub.depth;
        if (index == VK_ATTACHMENT_UNUSED || index >= fb->attachments.size()) return false;
        const ImageView* cv = fb->attachments[index];
        if (!cv || !cv->image) return false;
        view_base(cv, w, h);
        return true;
    };
    auto fits = [&](uint32_t count, uint32_t instances, uint32_t w, uint32_t h) {
        const uint32_t ppi = primitives_per_instance(pipeline->topology, count);
        std::string err;
        if (rt::static_scratch_check(static_cast<uint64_t>(ppi) * instances, pipeline->module.tile_shift, w, h, err) != rt::kOk) {
            rt::set_last_error("cpv_queue_submit_no_alloc: " + err);
            return false;
        }
        return true;
    };
    const std::vector<DeviceMemory*> none;
    for (const Cmd& c : cb->cmds) {
        switch (c.type) {
        case CmdType::BeginRenderPass:
            pass = static_cast<RenderPass*>(c.p[0]);
            fb = static_cast<Framebuffer*>(c.p[1]);
            subpass = 0;
            break;
        case CmdType::NextSubpass: subpass++; break;
        case CmdType::EndRenderPass: pass = nullptr; fb = nullptr; break;
        case CmdType::BindPipeline: pipeline = static_cast<Pipeline*>(c.p[0]); break;
        case CmdType::Draw:
        case CmdType::DrawIndexed: {
            uint32_t w = 0, h = 0;
            if (target(w, h) && !fits(c.u[0], c.u[1], w, h)) return VK_ERROR_OUT_OF_DEVICE_MEMORY;
            break;
        }
        case CmdType::DrawIndirect:
        case CmdType::DrawIndexedIndirect: {
            // The records as they stand at submission (the host mirror, or
            // HBM after the queue's earlier work). Records that commands of
            // this same submission rewrite are checked again at replay.
            uint32_t w = 0, h = 0;
            if (!target(w, h)) break;
            std::vector<IndirectDraw> records;
            if (read_indirect(q, c, none, records) != VK_SUCCESS) break;  // execute() reports it
            for (const IndirectDraw& d : records)
                if (!fits(d.count, d.instances, w, h)) return VK_ERROR_OUT_OF_DEVICE_MEMORY;
            break;
        }
        default: break;
        }
    }
    return VK_SUCCESS;
}

}  // namespace cpv::icd
