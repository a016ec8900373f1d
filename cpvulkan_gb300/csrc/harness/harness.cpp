// harness.cpp — headless Vulkan application over an ICD shared object.
//
// Loads the ICD as the Khronos loader would (dlopen, interface negotiation,
// vk_icdGetInstanceProcAddr, dispatch-word check and overwrite) and renders
// cpv_scene descriptions through Vulkan calls only: the role the LunarG
// samples play for the reference (Samples/15-draw_cube,
// Samples/utils/util_init.cpp), without a window system.
#include <dlfcn.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <thread>
#include <string>
#include <vector>

#include "../../../include/cpv/vk_subset.h"
#include "../../../include/cpv_harness.h"

extern "C" const uint32_t* cpvh_spirv(uint32_t program, uint32_t stage, size_t* bytes);

namespace {

thread_local std::string g_err;

#define CPVH_FN(name) PFN_##name name = nullptr;
struct Fns {
    CPVH_FN(vkGetInstanceProcAddr)
    CPVH_FN(vkGetDeviceProcAddr)
    CPVH_FN(vkCreateInstance)
    CPVH_FN(vkDestroyInstance)
    CPVH_FN(vkEnumeratePhysicalDevices)
    CPVH_FN(vkGetPhysicalDeviceMemoryProperties)
    CPVH_FN(vkGetPhysicalDeviceQueueFamilyProperties)
    CPVH_FN(vkCreateDevice)
    CPVH_FN(vkDestroyDevice)
    CPVH_FN(vkGetDeviceQueue)
    CPVH_FN(vkDeviceWaitIdle)
    CPVH_FN(vkAllocateMemory)
    CPVH_FN(vkFreeMemory)
    CPVH_FN(vkMapMemory)
    CPVH_FN(vkUnmapMemory)
    CPVH_FN(vkCreateBuffer)
    CPVH_FN(vkDestroyBuffer)
    CPVH_FN(vkGetBufferMemoryRequirements)
    CPVH_FN(vkBindBufferMemory)
    CPVH_FN(vkCreateImage)
    CPVH_FN(vkDestroyImage)
    CPVH_FN(vkGetImageMemoryRequirements)
    CPVH_FN(vkBindImageMemory)
    CPVH_FN(vkCreateImageView)
    CPVH_FN(vkDestroyImageView)
    CPVH_FN(vkCreateSampler)
    CPVH_FN(vkDestroySampler)
    CPVH_FN(vkCreateShaderModule)
    CPVH_FN(vkDestroyShaderModule)
    CPVH_FN(vkCreatePipelineCache)
    CPVH_FN(vkDestroyPipelineCache)
    CPVH_FN(vkCreateGraphicsPipelines)
    CPVH_FN(vkDestroyPipeline)
    CPVH_FN(vkCreatePipelineLayout)
    CPVH_FN(vkDestroyPipelineLayout)
    CPVH_FN(vkCreateDescriptorSetLayout)
    CPVH_FN(vkDestroyDescriptorSetLayout)
    CPVH_FN(vkCreateDescriptorPool)
    CPVH_FN(vkDestroyDescriptorPool)
    CPVH_FN(vkAllocateDescriptorSets)
    CPVH_FN(vkUpdateDescriptorSets)
    CPVH_FN(vkCreateRenderPass)
    CPVH_FN(vkDestroyRenderPass)
    CPVH_FN(vkCreateFramebuffer)
    CPVH_FN(vkDestroyFramebuffer)
    CPVH_FN(vkCreateCommandPool)
    CPVH_FN(vkDestroyCommandPool)
    CPVH_FN(vkAllocateCommandBuffers)
    CPVH_FN(vkBeginCommandBuffer)
    CPVH_FN(vkEndCommandBuffer)
    CPVH_FN(vkCmdBindPipeline)
    CPVH_FN(vkCmdBindDescriptorSets)
    CPVH_FN(vkCmdBindIndexBuffer)
    CPVH_FN(vkCmdBindVertexBuffers)
    CPVH_FN(vkCmdDraw)
    CPVH_FN(vkCmdDrawIndexed)
    CPVH_FN(vkCmdDrawIndirect)
    CPVH_FN(vkCmdDrawIndexedIndirect)
    CPVH_FN(vkCmdDrawIndirectCountKHR)
    CPVH_FN(vkCmdDrawIndexedIndirectCountKHR)
    CPVH_FN(vkCmdCopyBuffer)
    CPVH_FN(vkCmdCopyBufferToImage)
    CPVH_FN(vkCmdCopyImageToBuffer)
    CPVH_FN(vkCmdBlitImage)
    CPVH_FN(vkCmdCopyImage)
    CPVH_FN(vkCmdClearColorImage)
    CPVH_FN(vkCmdClearDepthStencilImage)
    CPVH_FN(vkCmdClearAttachments)
    CPVH_FN(vkCmdPipelineBarrier)
    CPVH_FN(vkCmdPushConstants)
    CPVH_FN(vkCmdBeginRenderPass)
    CPVH_FN(vkCmdNextSubpass)
    CPVH_FN(vkCmdEndRenderPass)
    CPVH_FN(vkCmdExecuteCommands)
    CPVH_FN(vkQueueSubmit)
    CPVH_FN(vkQueueWaitIdle)
    CPVH_FN(vkCreateFence)
    CPVH_FN(vkDestroyFence)
    CPVH_FN(vkResetFences)
    CPVH_FN(vkWaitForFences)
    CPVH_FN(vkGetFenceStatus)
};
#undef CPVH_FN

typedef int (*PFN_cpv_queue_record)(VkQueue, uint32_t);
typedef double (*PFN_cpv_queue_elapsed_ms)(VkQueue, uint32_t, uint32_t);
typedef const char* (*PFN_cpv_last_error)(void);

// What a loader keeps in the first word of dispatchable objects.
struct LoaderDispatch {
    const void* table;
} g_loader_dispatch{&g_loader_dispatch};

}  // namespace

struct cpvh_context {
    void* lib = nullptr;
    Fns f;
    VkInstance instance = nullptr;
    VkPhysicalDevice physical = nullptr;
    VkDevice device = nullptr;
    VkQueue queue = nullptr;          // queues[0]
    std::vector<VkQueue> queues;      // every queue of the device's queue family
    VkPhysicalDeviceMemoryProperties mem{};
    VkPipelineCache cache = nullptr;
    PFN_cpv_queue_record record = nullptr;
    PFN_cpv_queue_elapsed_ms elapsed = nullptr;
    PFN_cpv_last_error icd_error = nullptr;
};

namespace {

std::string icd_error(cpvh_context* c) { return c && c->icd_error ? c->icd_error() : ""; }

bool check_dispatch(void* handle) {
    // Loader contract: the ICD's dispatchable object begins with
    // ICD_LOADER_MAGIC; the loader then stores its dispatch table there.
    uintptr_t* word = reinterpret_cast<uintptr_t*>(handle);
    if (*word != ICD_LOADER_MAGIC) return false;
    *word = reinterpret_cast<uintptr_t>(&g_loader_dispatch);
    return true;
}

uint32_t find_memory_type(const cpvh_context* c, uint32_t bits, bool host_visible) {
    for (uint32_t i = 0; i < c->mem.memoryTypeCount; i++) {
        if (!(bits & (1u << i))) continue;
        const bool hv = (c->mem.memoryTypes[i].propertyFlags & VK_MEMORY_PROPERTY_HOST_VISIBLE_BIT) != 0;
        if (hv == host_visible) return i;
    }
    for (uint32_t i = 0; i < c->mem.memoryTypeCount; i++)
        if (bits & (1u << i)) return i;
    return 0;
}

struct BufferAlloc {
    VkBuffer buffer = nullptr;
    VkDeviceMemory memory = nullptr;
    VkDeviceSize size = 0;
};

struct ImageAlloc {
    VkImage image = nullptr;
    VkDeviceMemory memory = nullptr;
    VkImageView view = nullptr;
};

}  // namespace

struct cpvh_renderer {
    cpvh_context* ctx = nullptr;
    const cpv_scene* scene = nullptr;
    BufferAlloc vertex, index, uniform, staging, readback, indirect, indirect_count;
    uint32_t subpass = 0;  // the subpass the frame draws in (CPVH_SUBPASSES=2: 1)
    bool use_secondary = false;  // CPVH_SECONDARY=1: draws through secondary command buffers
    ImageAlloc colour, depth, texture;
    std::vector<ImageAlloc> extra;  // colour attachments after the first (an unused reference: no image)
    VkSampler sampler = nullptr;
    VkRenderPass pass = nullptr;
    VkFramebuffer fb = nullptr;
    VkDescriptorSetLayout set_layout = nullptr;
    VkDescriptorPool pool = nullptr;
    VkDescriptorSet set = nullptr;
    VkPipelineLayout layout = nullptr;
    std::vector<VkShaderModule> modules;
    std::vector<VkPipeline> pipelines;
    VkCommandPool cmd_pool = nullptr;
    VkCommandBuffer frame_cmd = nullptr, e2e_cmd = nullptr, copy_cmd = nullptr;
    VkFence fence = nullptr;
    uint32_t depth_texel = 0;
    uint32_t colour_texel = 4;
    uint64_t upload_bytes = 0;
};

namespace {

VkResult make_buffer(cpvh_context* c, VkDeviceSize size, VkBufferUsageFlags usage, bool host_visible, BufferAlloc& out) {
    VkBufferCreateInfo bi{};
    bi.sType = VK_STRUCTURE_TYPE_BUFFER_CREATE_INFO;
    bi.size = size ? size : 16;
    bi.usage = usage;
    VkResult r = c->f.vkCreateBuffer(c->device, &bi, nullptr, &out.buffer);
    if (r != VK_SUCCESS) return r;
    VkMemoryRequirements req;
    c->f.vkGetBufferMemoryRequirements(c->device, out.buffer, &req);
    VkMemoryAllocateInfo ai{};
    ai.sType = VK_STRUCTURE_TYPE_MEMORY_ALLOCATE_INFO;
    ai.allocationSize = req.size;
    ai.memoryTypeIndex = find_memory_type(c, req.memoryTypeBits, host_visible);
    r = c->f.vkAllocateMemory(c->device, &ai, nullptr, &out.memory);
    if (r != VK_SUCCESS) return r;
    out.size = bi.size;
    return c->f.vkBindBufferMemory(c->device, out.buffer, out.memory, 0);
}

VkResult make_image(cpvh_context* c, VkFormat fmt, uint32_t w, uint32_t h, uint32_t levels, VkImageUsageFlags usage, VkImageAspectFlags aspect,
                    ImageAlloc& out) {
    VkImageCreateInfo ii{};
    ii.sType = VK_STRUCTURE_TYPE_IMAGE_CREATE_INFO;
    ii.imageType = VK_IMAGE_TYPE_2D;
    ii.format = fmt;
    ii.extent = {w, h, 1};
    ii.mipLevels = levels;
    ii.arrayLayers = 1;
    ii.samples = VK_SAMPLE_COUNT_1_BIT;
    ii.tiling = VK_IMAGE_TILING_OPTIMAL;
    ii.usage = usage;
    VkResult r = c->f.vkCreateImage(c->device, &ii, nullptr, &out.image);
    if (r != VK_SUCCESS) return r;
    VkMemoryRequirements req;
    c->f.vkGetImageMemoryRequirements(c->device, out.image, &req);
    VkMemoryAllocateInfo ai{};
    ai.sType = VK_STRUCTURE_TYPE_MEMORY_ALLOCATE_INFO;
    ai.allocationSize = req.size;
    ai.memoryTypeIndex = find_memory_type(c, req.memoryTypeBits, false);
    r = c->f.vkAllocateMemory(c->device, &ai, nullptr, &out.memory);
    if (r != VK_SUCCESS) return r;
    r = c->f.vkBindImageMemory(c->device, out.image, out.memory, 0);
    if (r != VK_SUCCESS) return r;
    VkImageViewCreateInfo vi{};
    vi.sType = VK_STRUCTURE_TYPE_IMAGE_VIEW_CREATE_INFO;
    vi.image = out.image;
    vi.viewType = VK_IMAGE_VIEW_TYPE_2D;
    vi.format = fmt;
    vi.subresourceRange = {aspect, 0, levels, 0, 1};
    return c->f.vkCreateImageView(c->device, &vi, nullptr, &out.view);
}

void destroy_buffer(cpvh_context* c, BufferAlloc& b) {
    if (b.buffer) c->f.vkDestroyBuffer(c->device, b.buffer, nullptr);
    if (b.memory) c->f.vkFreeMemory(c->device, b.memory, nullptr);
    b = BufferAlloc{};
}

void destroy_image(cpvh_context* c, ImageAlloc& i) {
    if (i.view) c->f.vkDestroyImageView(c->device, i.view, nullptr);
    if (i.image) c->f.vkDestroyImage(c->device, i.image, nullptr);
    if (i.memory) c->f.vkFreeMemory(c->device, i.memory, nullptr);
    i = ImageAlloc{};
}

// Bytes per texel of a colour attachment format; 4 for a depth-only pass,
// whose readback holds zeros in the RGBA8 layout.
uint32_t colour_texel_size(uint32_t f) {
    switch (f) {
    case VK_FORMAT_R8_UNORM: case VK_FORMAT_R8_UINT: case VK_FORMAT_R8_SINT: return 1;
    case VK_FORMAT_R8G8_UNORM: case VK_FORMAT_R16_UNORM: case VK_FORMAT_R8G8_UINT: case VK_FORMAT_R8G8_SINT: case VK_FORMAT_R16_UINT:
    case VK_FORMAT_R16_SINT: return 2;
    case VK_FORMAT_R16G16B16A16_UNORM: case VK_FORMAT_R16G16B16A16_UINT: case VK_FORMAT_R16G16B16A16_SINT: case VK_FORMAT_R16G16B16A16_SFLOAT:
    case VK_FORMAT_R32G32_SFLOAT: case VK_FORMAT_R32G32_UINT: case VK_FORMAT_R32G32_SINT: return 8;
    case VK_FORMAT_R32G32B32A32_SFLOAT: case VK_FORMAT_R32G32B32A32_UINT: case VK_FORMAT_R32G32B32A32_SINT: return 16;
    default: return 4;
    }
}
// Integer colour formats: cleared with the integers round(clear_color * 100).
bool integer_colour(uint32_t f) {
    switch (f) {
    case VK_FORMAT_R8_UINT: case VK_FORMAT_R8_SINT: case VK_FORMAT_R8G8_UINT: case VK_FORMAT_R8G8_SINT: case VK_FORMAT_R8G8B8A8_UINT:
    case VK_FORMAT_R8G8B8A8_SINT: case VK_FORMAT_R16_UINT: case VK_FORMAT_R16_SINT: case VK_FORMAT_R16G16_UINT: case VK_FORMAT_R16G16_SINT:
    case VK_FORMAT_R32_UINT: case VK_FORMAT_R32_SINT: case VK_FORMAT_R16G16B16A16_UINT: case VK_FORMAT_R16G16B16A16_SINT: case VK_FORMAT_R32G32_UINT:
    case VK_FORMAT_R32G32_SINT: case VK_FORMAT_R32G32B32A32_UINT: case VK_FORMAT_R32G32B32A32_SINT: return true;
    default: return false;
    }
}
void clear_value_for(uint32_t fmt, const float c[4], VkClearValue& v) {
    for (int i = 0; i < 4; i++) {
        if (integer_colour(fmt)) v.color.int32[i] = static_cast<int32_t>(std::lround(c[i] * 100.0f));
        else v.color.float32[i] = c[i];
    }
}
uint32_t depth_texel_size(uint32_t f) { return f == VK_FORMAT_D16_UNORM ? 2 : (f == VK_FORMAT_D32_SFLOAT ? 4 : (f == VK_FORMAT_D32_SFLOAT_S8_UINT ? 8 : 0)); }

VkResult submit_and_wait(cpvh_renderer* r, VkCommandBuffer cmd) {
    cpvh_context* c = r->ctx;
    VkSubmitInfo si{};
    si.sType = VK_STRUCTURE_TYPE_SUBMIT_INFO;
    si.commandBufferCount = 1;
    si.pCommandBuffers = &cmd;
    VkResult res = c->f.vkQueueSubmit(c->queue, 1, &si, r->fence);
    if (res != VK_SUCCESS) return res;
    res = c->f.vkWaitForFences(c->device, 1, &r->fence, VK_TRUE, ~0ull);
    c->f.vkResetFences(c->device, 1, &r->fence);
    return res;
}

// Copies the staging buffer's regions into the device-local buffers (the
// layout staging = [vertex | index | uniform]).
void record_upload(cpvh_renderer* r, VkCommandBuffer cmd) {
    cpvh_context* c = r->ctx;
    const cpv_scene* s = r->scene;
    VkDeviceSize off = 0;
    auto copy = [&](BufferAlloc& dst, uint64_t bytes) {
        if (!bytes) return;
        VkBufferCopy bc{off, 0, bytes};
        c->f.vkCmdCopyBuffer(cmd, r->staging.buffer, dst.buffer, 1, &bc);
        off += (bytes + 255) & ~255ull;
    };
    copy(r->vertex, s->vertex_bytes);
    copy(r->index, s->index_bytes);
    copy(r->uniform, s->uniform_bytes);
}

void fill_staging(cpvh_renderer* r, void* map) {
    const cpv_scene* s = r->scene;
    uint8_t* p = static_cast<uint8_t*>(map);
    VkDeviceSize off = 0;
    auto put = [&](const uint8_t* src, uint64_t bytes) {
        if (!bytes) return;
        std::memcpy(p + off, src, bytes);
        off += (bytes + 255) & ~255ull;
    };
    put(s->vertex_data, s->vertex_bytes);
    put(s->index_data, s->index_bytes);
    put(s->uniform_data, s->uniform_bytes);
}

// Binds and draws scene draws [begin, end) into `cmd` (inside a render pass).
void record_draws(cpvh_renderer* r, VkCommandBuffer cmd, uint32_t begin, uint32_t end) {
    cpvh_context* c = r->ctx;
    const cpv_scene* s = r->scene;
    uint32_t bound = ~0u;
    for (uint32_t i = begin; i < end; i++) {
        const cpv_scene_draw& d = s->draws[i];
        const cpv_scene_pipeline& p = s->pipelines[d.pipeline];
        if (bound != d.pipeline) {
            c->f.vkCmdBindPipeline(cmd, VK_PIPELINE_BIND_POINT_GRAPHICS, r->pipelines[d.pipeline]);
            if (r->set) c->f.vkCmdBindDescriptorSets(cmd, VK_PIPELINE_BIND_POINT_GRAPHICS, r->layout, 0, 1, &r->set, 0, nullptr);
            bound = d.pipeline;
        }
        for (uint32_t b = 0; b < p.num_bindings; b++) {
            const VkDeviceSize off = d.vertex_offsets[b];
            c->f.vkCmdBindVertexBuffers(cmd, p.bindings[b].binding, 1, &r->vertex.buffer, &off);
        }
        if (d.push_size) c->f.vkCmdPushConstants(cmd, r->layout, VK_SHADER_STAGE_VERTEX_BIT | VK_SHADER_STAGE_FRAGMENT_BIT, 0, d.push_size, d.push);
        if (d.indexed) c->f.vkCmdBindIndexBuffer(cmd, r->index.buffer, d.index_offset, static_cast<VkIndexType>(s->index_type));
        if (r->indirect_count.buffer) {
            const VkDeviceSize at = static_cast<VkDeviceSize>(i) * 20, count_at = static_cast<VkDeviceSize>(i) * 4;
            if (d.indexed) c->f.vkCmdDrawIndexedIndirectCountKHR(cmd, r->indirect.buffer, at, r->indirect_count.buffer, count_at, 1, 20);
            else c->f.vkCmdDrawIndirectCountKHR(cmd, r->indirect.buffer, at, r->indirect_count.buffer, count_at, 1, 20);
        } else if (r->indirect.buffer) {
            const VkDeviceSize at = static_cast<VkDeviceSize>(i) * 20;
            if (d.indexed) c->f.vkCmdDrawIndexedIndirect(cmd, r->indirect.buffer, at, 1, 20);
            else c->f.vkCmdDrawIndirect(cmd, r->indirect.buffer, at, 1, 20);
        } else if (d.indexed) {
            c->f.vkCmdDrawIndexed(cmd, d.count, d.instance_count, d.first, d.vertex_offset, d.first_instance);
        } else {
            c->f.vkCmdDraw(cmd, d.count, d.instance_count, d.first, d.first_instance);
        }
    }
}

void record_frame(cpvh_renderer* r, VkCommandBuffer cmd) {
    cpvh_context* c = r->ctx;
    const cpv_scene* s = r->scene;
    VkClearValue clears[2 + CPV_SCENE_MAX_EXTRA_COLOR];
    std::memset(clears, 0, sizeof(clears));
    // in attachment order: colour (absent in a depth-only pass), the further
    // colour attachments (the same clear colour), depth
    uint32_t nclears = 0;
    if (s->color_format) {
        clear_value_for(s->color_format, s->clear_color, clears[nclears++]);
        for (uint32_t k = 0; k < s->extra_color_count; k++)
            if (s->extra_color_formats[k]) clear_value_for(s->extra_color_formats[k], s->clear_color, clears[nclears++]);
    }
    if (s->depth_format) {
        clears[nclears].depthStencil.depth = s->clear_depth;
        clears[nclears].depthStencil.stencil = s->clear_stencil;
        nclears++;
    }
    VkRenderPassBeginInfo rb{};
    rb.sType = VK_STRUCTURE_TYPE_RENDER_PASS_BEGIN_INFO;
    rb.renderPass = r->pass;
    rb.framebuffer = r->fb;
    rb.renderArea = {{0, 0}, {s->width, s->height}};
    rb.clearValueCount = nclears;
    rb.pClearValues = clears;
    // CPVH_SECONDARY=1: the draws are recorded into two secondary command
    // buffers (the first and second half), executed in the render pass
    if (r->use_secondary && r->subpass == 0) {
        c->f.vkCmdBeginRenderPass(cmd, &rb, VK_SUBPASS_CONTENTS_SECONDARY_COMMAND_BUFFERS);
        VkCommandBuffer secs[2] = {nullptr, nullptr};
        VkCommandBufferAllocateInfo cai{};
        cai.sType = VK_STRUCTURE_TYPE_COMMAND_BUFFER_ALLOCATE_INFO;
        cai.commandPool = r->cmd_pool;
        cai.level = VK_COMMAND_BUFFER_LEVEL_SECONDARY;
        cai.commandBufferCount = 2;
        if (c->f.vkAllocateCommandBuffers(c->device, &cai, secs) != VK_SUCCESS) return;
        VkCommandBufferInheritanceInfo inh{};
        inh.sType = VK_STRUCTURE_TYPE_COMMAND_BUFFER_INHERITANCE_INFO;
        inh.renderPass = r->pass;
        inh.subpass = 0;
        inh.framebuffer = r->fb;
        VkCommandBufferBeginInfo bi{};
        bi.sType = VK_STRUCTURE_TYPE_COMMAND_BUFFER_BEGIN_INFO;
        bi.flags = VK_COMMAND_BUFFER_USAGE_RENDER_PASS_CONTINUE_BIT | VK_COMMAND_BUFFER_USAGE_SIMULTANEOUS_USE_BIT;
        bi.pInheritanceInfo = &inh;
        const uint32_t half = s->num_draws / 2;
        for (uint32_t k = 0; k < 2; k++) {
            c->f.vkBeginCommandBuffer(secs[k], &bi);
            record_draws(r, secs[k], k == 0 ? 0 : half, k == 0 ? half : s->num_draws);
            c->f.vkEndCommandBuffer(secs[k]);
        }
        c->f.vkCmdExecuteCommands(cmd, 2, secs);
    } else {
        c->f.vkCmdBeginRenderPass(cmd, &rb, VK_SUBPASS_CONTENTS_INLINE);
        if (r->subpass == 1) c->f.vkCmdNextSubpass(cmd, VK_SUBPASS_CONTENTS_INLINE);
        record_draws(r, cmd, 0, s->num_draws);
    }
    c->f.vkCmdEndRenderPass(cmd);
}

void record_readback(cpvh_renderer* r, VkCommandBuffer cmd) {
    cpvh_context* c = r->ctx;
    const cpv_scene* s = r->scene;
    VkBufferImageCopy bc{};
    bc.imageSubresource = {VK_IMAGE_ASPECT_COLOR_BIT, 0, 0, 1};
    bc.imageExtent = {s->width, s->height, 1};
    if (s->color_format) c->f.vkCmdCopyImageToBuffer(cmd, r->colour.image, VK_IMAGE_LAYOUT_TRANSFER_SRC_OPTIMAL, r->readback.buffer, 1, &bc);
    if (s->depth_format) {
        bc.bufferOffset = static_cast<VkDeviceSize>(s->width) * s->height * r->colour_texel;
        bc.imageSubresource.aspectMask = VK_IMAGE_ASPECT_DEPTH_BIT;
        c->f.vkCmdCopyImageToBuffer(cmd, r->depth.image, VK_IMAGE_LAYOUT_TRANSFER_SRC_OPTIMAL, r->readback.buffer, 1, &bc);
    }
}

VkResult record_all(cpvh_renderer* r) {
    cpvh_context* c = r->ctx;
    VkCommandBufferBeginInfo bi{};
    bi.sType = VK_STRUCTURE_TYPE_COMMAND_BUFFER_BEGIN_INFO;
    bi.flags = VK_COMMAND_BUFFER_USAGE_SIMULTANEOUS_USE_BIT;
    c->f.vkBeginCommandBuffer(r->frame_cmd, &bi);
    record_frame(r, r->frame_cmd);
    c->f.vkEndCommandBuffer(r->frame_cmd);
    c->f.vkBeginCommandBuffer(r->e2e_cmd, &bi);
    record_upload(r, r->e2e_cmd);
    record_frame(r, r->e2e_cmd);
    record_readback(r, r->e2e_cmd);
    c->f.vkEndCommandBuffer(r->e2e_cmd);
    return VK_SUCCESS;
}

bool build_pipelines(cpvh_context* c, const cpv_scene* s, VkRenderPass pass, VkPipelineLayout layout, std::vector<VkShaderModule>& modules,
                     std::vector<VkPipeline>& pipelines, std::string& err, uint32_t subpass = 0) {
    const Fns& f = c->f;
    for (uint32_t i = 0; i < s->num_pipelines; i++) {
        const cpv_scene_pipeline& sp = s->pipelines[i];
        VkShaderModule mods[2];
        for (uint32_t st = 0; st < 2; st++) {
            size_t bytes = 0;
            const uint32_t* code = cpvh_spirv(sp.program, st, &bytes);
            if (!code) { err = "no SPIR-V for program " + std::to_string(sp.program); return false; }
            VkShaderModuleCreateInfo smi{};
            smi.sType = VK_STRUCTURE_TYPE_SHADER_MODULE_CREATE_INFO;
            smi.codeSize = bytes;
            smi.pCode = code;
            if (f.vkCreateShaderModule(c->device, &smi, nullptr, &mods[st]) != VK_SUCCESS) { err = "shader module"; return false; }
            modules.push_back(mods[st]);
        }
        VkPipelineShaderStageCreateInfo stages[2]{};
        stages[0].sType = stages[1].sType = VK_STRUCTURE_TYPE_PIPELINE_SHADER_STAGE_CREATE_INFO;
        stages[0].stage = VK_SHADER_STAGE_VERTEX_BIT;
        stages[0].module = mods[0];
        stages[0].pName = "main";
        stages[1].stage = VK_SHADER_STAGE_FRAGMENT_BIT;
        stages[1].module = mods[1];
        stages[1].pName = "main";
        // the fragment shader's specialisation constant 0, when the scene sets one
        const VkSpecializationMapEntry spec_entry{0, 0, 4};
        VkSpecializationInfo spec{};
        if (sp.spec_k) {
            spec.mapEntryCount = 1;
            spec.pMapEntries = &spec_entry;
            spec.dataSize = 4;
            spec.pData = &sp.spec_k;
            stages[1].pSpecializationInfo = &spec;
        }
        VkVertexInputBindingDescription vbd[CPV_SCENE_MAX_BINDINGS];
        VkVertexInputAttributeDescription vad[CPV_SCENE_MAX_ATTRIBUTES];
        for (uint32_t b = 0; b < sp.num_bindings; b++) vbd[b] = {sp.bindings[b].binding, sp.bindings[b].stride, static_cast<VkVertexInputRate>(sp.bindings[b].input_rate)};
        for (uint32_t a = 0; a < sp.num_attributes; a++)
            vad[a] = {sp.attributes[a].location, sp.attributes[a].binding, static_cast<VkFormat>(sp.attributes[a].format), sp.attributes[a].offset};
        VkPipelineVertexInputStateCreateInfo vis{};
        vis.sType = VK_STRUCTURE_TYPE_PIPELINE_VERTEX_INPUT_STATE_CREATE_INFO;
        vis.vertexBindingDescriptionCount = sp.num_bindings;
        vis.pVertexBindingDescriptions = vbd;
        vis.vertexAttributeDescriptionCount = sp.num_attributes;
        vis.pVertexAttributeDescriptions = vad;
        VkPipelineInputAssemblyStateCreateInfo ias{};
        ias.sType = VK_STRUCTURE_TYPE_PIPELINE_INPUT_ASSEMBLY_STATE_CREATE_INFO;
        ias.topology = static_cast<VkPrimitiveTopology>(sp.topology);
        VkViewport vp{s->viewport[0], s->viewport[1], s->viewport[2], s->viewport[3], s->viewport[4], s->viewport[5]};
        VkRect2D sc{{0, 0}, {s->width, s->height}};
        VkPipelineViewportStateCreateInfo vps{};
        vps.sType = VK_STRUCTURE_TYPE_PIPELINE_VIEWPORT_STATE_CREATE_INFO;
        vps.viewportCount = 1;
        vps.pViewports = &vp;
        vps.scissorCount = 1;
        vps.pScissors = &sc;
        VkPipelineRasterizationStateCreateInfo rs{};
        rs.sType = VK_STRUCTURE_TYPE_PIPELINE_RASTERIZATION_STATE_CREATE_INFO;
        rs.polygonMode = VK_POLYGON_MODE_FILL;
        rs.cullMode = sp.cull_mode;
        rs.frontFace = static_cast<VkFrontFace>(sp.front_face);
        rs.lineWidth = sp.line_width;
        VkPipelineMultisampleStateCreateInfo ms{};
        ms.sType = VK_STRUCTURE_TYPE_PIPELINE_MULTISAMPLE_STATE_CREATE_INFO;
        ms.rasterizationSamples = VK_SAMPLE_COUNT_1_BIT;
        VkPipelineDepthStencilStateCreateInfo ds{};
        ds.sType = VK_STRUCTURE_TYPE_PIPELINE_DEPTH_STENCIL_STATE_CREATE_INFO;
        ds.depthTestEnable = sp.depth_test;
        ds.depthWriteEnable = sp.depth_write;
        ds.depthCompareOp = static_cast<VkCompareOp>(sp.depth_compare);
        ds.stencilTestEnable = sp.stencil_test;
        ds.depthBoundsTestEnable = sp.depth_bounds_test;
        ds.minDepthBounds = sp.min_depth_bounds;
        ds.maxDepthBounds = sp.max_depth_bounds;
        const cpv_scene_stencil* so[2] = {&sp.stencil_front, &sp.stencil_back};
        VkStencilOpState* dso[2] = {&ds.front, &ds.back};
        for (int k = 0; k < 2; k++)
            *dso[k] = {static_cast<VkStencilOp>(so[k]->fail_op), static_cast<VkStencilOp>(so[k]->pass_op), static_cast<VkStencilOp>(so[k]->depth_fail_op),
                       static_cast<VkCompareOp>(so[k]->compare_op), so[k]->compare_mask, so[k]->write_mask, so[k]->reference};
        VkPipelineColorBlendAttachmentState cba{};
        cba.blendEnable = sp.blend_enable;
        cba.srcColorBlendFactor = static_cast<VkBlendFactor>(sp.src_color);
        cba.dstColorBlendFactor = static_cast<VkBlendFactor>(sp.dst_color);
        cba.colorBlendOp = static_cast<VkBlendOp>(sp.color_op);
        cba.srcAlphaBlendFactor = static_cast<VkBlendFactor>(sp.src_alpha);
        cba.dstAlphaBlendFactor = static_cast<VkBlendFactor>(sp.dst_alpha);
        cba.alphaBlendOp = static_cast<VkBlendOp>(sp.alpha_op);
        cba.colorWriteMask = sp.color_write_mask;
        // one state per colour reference of the subpass
        VkPipelineColorBlendAttachmentState cbas[1 + CPV_SCENE_MAX_EXTRA_COLOR];
        cbas[0] = cba;
        for (uint32_t k = 0; k < s->extra_color_count; k++) {
            const cpv_scene_attachment_blend& eb = sp.extra_blend[k];
            VkPipelineColorBlendAttachmentState& e = cbas[k + 1];
            e = VkPipelineColorBlendAttachmentState{};
            e.blendEnable = eb.blend_enable;
            e.srcColorBlendFactor = static_cast<VkBlendFactor>(eb.src_color);
            e.dstColorBlendFactor = static_cast<VkBlendFactor>(eb.dst_color);
            e.colorBlendOp = static_cast<VkBlendOp>(eb.color_op);
            e.srcAlphaBlendFactor = static_cast<VkBlendFactor>(eb.src_alpha);
            e.dstAlphaBlendFactor = static_cast<VkBlendFactor>(eb.dst_alpha);
            e.alphaBlendOp = static_cast<VkBlendOp>(eb.alpha_op);
            e.colorWriteMask = eb.color_write_mask;
        }
        VkPipelineColorBlendStateCreateInfo cbs{};
        cbs.sType = VK_STRUCTURE_TYPE_PIPELINE_COLOR_BLEND_STATE_CREATE_INFO;
        cbs.logicOpEnable = sp.logic_op_enable;
        cbs.logicOp = static_cast<VkLogicOp>(sp.logic_op);
        cbs.attachmentCount = s->color_format ? 1 + s->extra_color_count : 0;
        cbs.pAttachments = cbas;
        for (int k = 0; k < 4; k++) cbs.blendConstants[k] = sp.blend_constants[k];
        VkGraphicsPipelineCreateInfo gpi{};
        gpi.sType = VK_STRUCTURE_TYPE_GRAPHICS_PIPELINE_CREATE_INFO;
        gpi.stageCount = 2;
        gpi.pStages = stages;
        gpi.pVertexInputState = &vis;
        gpi.pInputAssemblyState = &ias;
        gpi.pViewportState = &vps;
        gpi.pRasterizationState = &rs;
        gpi.pMultisampleState = &ms;
        gpi.pDepthStencilState = &ds;
        gpi.pColorBlendState = &cbs;
        gpi.layout = layout;
        gpi.renderPass = pass;
        gpi.subpass = subpass;
        VkPipeline pipe = nullptr;
        if (f.vkCreateGraphicsPipelines(c->device, c->cache, 1, &gpi, nullptr, &pipe) != VK_SUCCESS) { err = "vkCreateGraphicsPipelines:"; return false; }
        pipelines.push_back(pipe);
    }
    return true;
}

// The scene's render pass: a cleared colour attachment (none in a
// depth-only pass) then a cleared depth/stencil attachment (when the scene
// has a depth format), both stored. With two_subpasses the scene draws in
// subpass 1 (these attachments), after a subpass 0 that references only the
// depth attachment (only the colour one when there is no depth).
VkResult create_scene_pass(cpvh_context* c, const cpv_scene* s, VkRenderPass* out, bool two_subpasses = false) {
    VkAttachmentDescription att[2 + CPV_SCENE_MAX_EXTRA_COLOR]{};
    VkAttachmentReference crefs[1 + CPV_SCENE_MAX_EXTRA_COLOR], dref{0, VK_IMAGE_LAYOUT_DEPTH_STENCIL_ATTACHMENT_OPTIMAL};
    uint32_t n = 0;
    VkSubpassDescription sub{};
    auto describe = [&](uint32_t fmt, bool depth) {
        VkAttachmentDescription& a = att[n];
        a.format = static_cast<VkFormat>(fmt);
        a.samples = VK_SAMPLE_COUNT_1_BIT;
        a.loadOp = VK_ATTACHMENT_LOAD_OP_CLEAR;
        a.storeOp = VK_ATTACHMENT_STORE_OP_STORE;
        a.stencilLoadOp = depth ? VK_ATTACHMENT_LOAD_OP_CLEAR : VK_ATTACHMENT_LOAD_OP_DONT_CARE;
        a.finalLayout = VK_IMAGE_LAYOUT_TRANSFER_SRC_OPTIMAL;
        return n++;
    };
    // colour references in order (an unused one keeps its position), then depth
    if (s->color_format) {
        crefs[0] = {describe(s->color_format, false), VK_IMAGE_LAYOUT_COLOR_ATTACHMENT_OPTIMAL};
        for (uint32_t k = 0; k < s->extra_color_count; k++) {
            const uint32_t f = s->extra_color_formats[k];
            crefs[k + 1] = {f ? describe(f, false) : VK_ATTACHMENT_UNUSED, VK_IMAGE_LAYOUT_COLOR_ATTACHMENT_OPTIMAL};
        }
        sub.colorAttachmentCount = 1 + s->extra_color_count;
        sub.pColorAttachments = crefs;
    }
    if (s->depth_format) {
        dref.attachment = describe(s->depth_format, true);
        sub.pDepthStencilAttachment = &dref;
    }
    VkSubpassDescription subs[2] = {sub, sub};
    if (two_subpasses) {
        if (sub.pDepthStencilAttachment) {
            subs[0].colorAttachmentCount = 0;
            subs[0].pColorAttachments = nullptr;
        } else {
            subs[0].pDepthStencilAttachment = nullptr;
        }
    }
    VkRenderPassCreateInfo rpi{};
    rpi.sType = VK_STRUCTURE_TYPE_RENDER_PASS_CREATE_INFO;
    rpi.attachmentCount = n;
    rpi.pAttachments = att;
    rpi.subpassCount = two_subpasses ? 2 : 1;
    rpi.pSubpasses = subs;
    return c->f.vkCreateRenderPass(c->device, &rpi, nullptr, out);
}

// A scene's descriptor set layout: binding 0 its uniform buffer; its
// texture at binding 1 as a combined image sampler, a storage image, or a
// sampled image with its sampler at binding 2 (cpv_scene::texture_binding).
std::vector<VkDescriptorSetLayoutBinding> scene_bindings(const cpv_scene* s) {
    std::vector<VkDescriptorSetLayoutBinding> lb;
    if (s->uniform_bytes) lb.push_back({0, VK_DESCRIPTOR_TYPE_UNIFORM_BUFFER, 1, VK_SHADER_STAGE_VERTEX_BIT | VK_SHADER_STAGE_FRAGMENT_BIT, nullptr});
    if (s->uniform_bytes && s->uniform_as_storage) lb.push_back({3, VK_DESCRIPTOR_TYPE_STORAGE_BUFFER, 1, VK_SHADER_STAGE_FRAGMENT_BIT, nullptr});
    if (s->texture_data) {
        switch (s->texture_binding) {
        case CPV_TEXTURE_STORAGE: lb.push_back({1, VK_DESCRIPTOR_TYPE_STORAGE_IMAGE, 1, VK_SHADER_STAGE_FRAGMENT_BIT, nullptr}); break;
        case CPV_TEXTURE_SEPARATE:
            lb.push_back({1, VK_DESCRIPTOR_TYPE_SAMPLED_IMAGE, 1, VK_SHADER_STAGE_FRAGMENT_BIT, nullptr});
            lb.push_back({2, VK_DESCRIPTOR_TYPE_SAMPLER, 1, VK_SHADER_STAGE_FRAGMENT_BIT, nullptr});
            break;
        default: lb.push_back({1, VK_DESCRIPTOR_TYPE_COMBINED_IMAGE_SAMPLER, 1, VK_SHADER_STAGE_FRAGMENT_BIT, nullptr}); break;
        }
    }
    return lb;
}

VkResult make_pass_and_layout(cpvh_context* c, const cpv_scene* s, bool with_sets, VkRenderPass& pass, VkDescriptorSetLayout& set_layout,
                              VkPipelineLayout& layout, bool two_subpasses = false) {
    const Fns& f = c->f;
    VkResult res = create_scene_pass(c, s, &pass, two_subpasses);
    if (res != VK_SUCCESS) return res;
    std::vector<VkDescriptorSetLayoutBinding> lb;
    if (with_sets) lb = scene_bindings(s);
    VkDescriptorSetLayoutCreateInfo dli{};
    dli.sType = VK_STRUCTURE_TYPE_DESCRIPTOR_SET_LAYOUT_CREATE_INFO;
    dli.bindingCount = static_cast<uint32_t>(lb.size());
    dli.pBindings = lb.data();
    res = f.vkCreateDescriptorSetLayout(c->device, &dli, nullptr, &set_layout);
    if (res != VK_SUCCESS) return res;
    VkPushConstantRange pcr{VK_SHADER_STAGE_VERTEX_BIT | VK_SHADER_STAGE_FRAGMENT_BIT, 0, 128};
    VkPipelineLayoutCreateInfo pli{};
    pli.sType = VK_STRUCTURE_TYPE_PIPELINE_LAYOUT_CREATE_INFO;
    pli.setLayoutCount = 1;
    pli.pSetLayouts = &set_layout;
    pli.pushConstantRangeCount = 1;
    pli.pPushConstantRanges = &pcr;
    return f.vkCreatePipelineLayout(c->device, &pli, nullptr, &layout);
}

}  // namespace

extern "C" {

const char* cpvh_last_error(void) { return g_err.c_str(); }

cpvh_context* cpvh_open(const char* icd_path, char* err, uint32_t err_len) {
    auto fail = [&](const std::string& e, cpvh_context* c) -> cpvh_context* {
        g_err = e + (c ? " " + icd_error(c) : "");
        if (err && err_len) std::snprintf(err, err_len, "%s", g_err.c_str());
        if (c) cpvh_close(c);
        return nullptr;
    };
    auto* c = new cpvh_context();
    c->lib = dlopen(icd_path, RTLD_NOW | RTLD_LOCAL);
    if (!c->lib) return fail(std::string("dlopen failed: ") + dlerror(), c);
    auto negotiate = reinterpret_cast<PFN_vk_icdNegotiateLoaderICDInterfaceVersion>(dlsym(c->lib, "vk_icdNegotiateLoaderICDInterfaceVersion"));
    auto gipa = reinterpret_cast<PFN_vk_icdGetInstanceProcAddr>(dlsym(c->lib, "vk_icdGetInstanceProcAddr"));
    c->record = reinterpret_cast<PFN_cpv_queue_record>(dlsym(c->lib, "cpv_queue_record"));
    c->elapsed = reinterpret_cast<PFN_cpv_queue_elapsed_ms>(dlsym(c->lib, "cpv_queue_elapsed_ms"));
    c->icd_error = reinterpret_cast<PFN_cpv_last_error>(dlsym(c->lib, "cpv_last_error"));
    if (!negotiate || !gipa) return fail("not a Vulkan ICD (missing vk_icd* exports)", c);
    uint32_t version = 5;
    if (negotiate(&version) != VK_SUCCESS || version < 1) return fail("interface negotiation failed", c);
    Fns& f = c->f;
    f.vkGetInstanceProcAddr = reinterpret_cast<PFN_vkGetInstanceProcAddr>(gipa(nullptr, "vkGetInstanceProcAddr"));
    f.vkCreateInstance = reinterpret_cast<PFN_vkCreateInstance>(gipa(nullptr, "vkCreateInstance"));
    if (!f.vkGetInstanceProcAddr || !f.vkCreateInstance) return fail("ICD lacks global entry points", c);
    VkApplicationInfo app{};
    app.sType = VK_STRUCTURE_TYPE_APPLICATION_INFO;
    app.pApplicationName = "cpvh";
    app.apiVersion = VK_API_VERSION_1_1;
    VkInstanceCreateInfo ici{};
    ici.sType = VK_STRUCTURE_TYPE_INSTANCE_CREATE_INFO;
    ici.pApplicationInfo = &app;
    if (f.vkCreateInstance(&ici, nullptr, &c->instance) != VK_SUCCESS) return fail("vkCreateInstance failed", c);
    if (!check_dispatch(c->instance)) return fail("VkInstance lacks the loader magic", c);
#define LOAD_I(name) f.name = reinterpret_cast<PFN_##name>(f.vkGetInstanceProcAddr(c->instance, #name))
    LOAD_I(vkDestroyInstance);
    LOAD_I(vkEnumeratePhysicalDevices);
    LOAD_I(vkGetPhysicalDeviceMemoryProperties);
    LOAD_I(vkGetPhysicalDeviceQueueFamilyProperties);
    LOAD_I(vkCreateDevice);
    LOAD_I(vkGetDeviceProcAddr);
#undef LOAD_I
    uint32_t n = 1;
    if (f.vkEnumeratePhysicalDevices(c->instance, &n, &c->physical) != VK_SUCCESS || n < 1) return fail("no physical device", c);
    if (!check_dispatch(c->physical)) return fail("VkPhysicalDevice lacks the loader magic", c);
    f.vkGetPhysicalDeviceMemoryProperties(c->physical, &c->mem);
    // All queues of family 0: the serving loop runs requests on several.
    VkQueueFamilyProperties family{};
    uint32_t families = 1;
    f.vkGetPhysicalDeviceQueueFamilyProperties(c->physical, &families, &family);
    const uint32_t nqueues = families >= 1 && family.queueCount >= 1 ? family.queueCount : 1;
    const std::vector<float> prio(nqueues, 1.0f);
    VkDeviceQueueCreateInfo qci{};
    qci.sType = VK_STRUCTURE_TYPE_DEVICE_QUEUE_CREATE_INFO;
    qci.queueCount = nqueues;
    qci.pQueuePriorities = prio.data();
    VkDeviceCreateInfo dci{};
    dci.sType = VK_STRUCTURE_TYPE_DEVICE_CREATE_INFO;
    dci.queueCreateInfoCount = 1;
    dci.pQueueCreateInfos = &qci;
    const char* const device_extensions[] = {"VK_KHR_draw_indirect_count"};
    dci.enabledExtensionCount = 1;
    dci.ppEnabledExtensionNames = device_extensions;
    if (f.vkCreateDevice(c->physical, &dci, nullptr, &c->device) != VK_SUCCESS) return fail("vkCreateDevice failed:", c);
    if (!check_dispatch(c->device)) return fail("VkDevice lacks the loader magic", c);
#define LOAD_D(name)                                                                     \
    f.name = reinterpret_cast<PFN_##name>(f.vkGetDeviceProcAddr(c->device, #name));      \
    if (!f.name) return fail("ICD lacks " #name, c)
    LOAD_D(vkDestroyDevice); LOAD_D(vkGetDeviceQueue); LOAD_D(vkDeviceWaitIdle); LOAD_D(vkAllocateMemory); LOAD_D(vkFreeMemory);
    LOAD_D(vkMapMemory); LOAD_D(vkUnmapMemory); LOAD_D(vkCreateBuffer); LOAD_D(vkDestroyBuffer); LOAD_D(vkGetBufferMemoryRequirements);
    LOAD_D(vkBindBufferMemory); LOAD_D(vkCreateImage); LOAD_D(vkDestroyImage); LOAD_D(vkGetImageMemoryRequirements); LOAD_D(vkBindImageMemory);
    LOAD_D(vkCreateImageView); LOAD_D(vkDestroyImageView); LOAD_D(vkCreateSampler); LOAD_D(vkDestroySampler); LOAD_D(vkCreateShaderModule);
    LOAD_D(vkDestroyShaderModule); LOAD_D(vkCreatePipelineCache); LOAD_D(vkDestroyPipelineCache); LOAD_D(vkCreateGraphicsPipelines);
    LOAD_D(vkDestroyPipeline); LOAD_D(vkCreatePipelineLayout); LOAD_D(vkDestroyPipelineLayout); LOAD_D(vkCreateDescriptorSetLayout);
    LOAD_D(vkDestroyDescriptorSetLayout); LOAD_D(vkCreateDescriptorPool); LOAD_D(vkDestroyDescriptorPool); LOAD_D(vkAllocateDescriptorSets);
    LOAD_D(vkUpdateDescriptorSets); LOAD_D(vkCreateRenderPass); LOAD_D(vkDestroyRenderPass); LOAD_D(vkCreateFramebuffer);
    LOAD_D(vkDestroyFramebuffer); LOAD_D(vkCreateCommandPool); LOAD_D(vkDestroyCommandPool); LOAD_D(vkAllocateCommandBuffers);
    LOAD_D(vkBeginCommandBuffer); LOAD_D(vkEndCommandBuffer); LOAD_D(vkCmdBindPipeline); LOAD_D(vkCmdBindDescriptorSets);
    LOAD_D(vkCmdBindIndexBuffer); LOAD_D(vkCmdBindVertexBuffers); LOAD_D(vkCmdDraw); LOAD_D(vkCmdDrawIndexed); LOAD_D(vkCmdCopyBuffer);
    LOAD_D(vkCmdDrawIndirect); LOAD_D(vkCmdDrawIndexedIndirect); LOAD_D(vkCmdDrawIndirectCountKHR); LOAD_D(vkCmdDrawIndexedIndirectCountKHR);
    LOAD_D(vkCmdCopyBufferToImage); LOAD_D(vkCmdCopyImageToBuffer); LOAD_D(vkCmdPipelineBarrier); LOAD_D(vkCmdPushConstants);
    LOAD_D(vkCmdBlitImage); LOAD_D(vkCmdCopyImage); LOAD_D(vkCmdClearColorImage); LOAD_D(vkCmdClearDepthStencilImage); LOAD_D(vkCmdClearAttachments);
    LOAD_D(vkCmdBeginRenderPass); LOAD_D(vkCmdNextSubpass); LOAD_D(vkCmdEndRenderPass); LOAD_D(vkCmdExecuteCommands); LOAD_D(vkQueueSubmit); LOAD_D(vkQueueWaitIdle); LOAD_D(vkCreateFence);
    LOAD_D(vkDestroyFence); LOAD_D(vkResetFences); LOAD_D(vkWaitForFences); LOAD_D(vkGetFenceStatus);
#undef LOAD_D
    // CPVH_SUBMIT=no_alloc: every submission of this context goes through the
    // ICD's allocation-free submit export (same signature as vkQueueSubmit).
    if (const char* mode = std::getenv("CPVH_SUBMIT"); mode && std::strcmp(mode, "no_alloc") == 0) {
        auto fn = reinterpret_cast<PFN_vkQueueSubmit>(dlsym(c->lib, "cpv_queue_submit_no_alloc"));
        if (!fn) return fail("CPVH_SUBMIT=no_alloc but the ICD lacks cpv_queue_submit_no_alloc", c);
        f.vkQueueSubmit = fn;
    }
    for (uint32_t i = 0; i < nqueues; i++) {
        VkQueue q = nullptr;
        f.vkGetDeviceQueue(c->device, 0, i, &q);
        if (!q || !check_dispatch(q)) return fail("VkQueue lacks the loader magic", c);
        c->queues.push_back(q);
    }
    c->queue = c->queues[0];
    VkPipelineCacheCreateInfo pci{};
    pci.sType = VK_STRUCTURE_TYPE_PIPELINE_CACHE_CREATE_INFO;
    f.vkCreatePipelineCache(c->device, &pci, nullptr, &c->cache);
    return c;
}

void cpvh_close(cpvh_context* c) {
    if (!c) return;
    if (c->device) {
        c->f.vkDeviceWaitIdle(c->device);
        if (c->cache) c->f.vkDestroyPipelineCache(c->device, c->cache, nullptr);
        c->f.vkDestroyDevice(c->device, nullptr);
    }
    if (c->instance && c->f.vkDestroyInstance) c->f.vkDestroyInstance(c->instance, nullptr);
    // The ICD stays loaded: CUDA state it created lives until process exit.
    delete c;
}

void* cpvh_queue(cpvh_context* c) { return c ? c->queue : nullptr; }

cpvh_renderer* cpvh_renderer_create(cpvh_context* c, const cpv_scene* s, char* err, uint32_t err_len) {
    auto* r = new cpvh_renderer();
    r->ctx = c;
    r->scene = s;
    auto fail = [&](const std::string& e) -> cpvh_renderer* {
        g_err = e + " " + icd_error(c);
        if (err && err_len) std::snprintf(err, err_len, "%s", g_err.c_str());
        cpvh_renderer_destroy(r);
        return nullptr;
    };
    const Fns& f = c->f;
    const VkBufferUsageFlags vb_usage = VK_BUFFER_USAGE_VERTEX_BUFFER_BIT | VK_BUFFER_USAGE_TRANSFER_DST_BIT;
    if (make_buffer(c, s->vertex_bytes, vb_usage, false, r->vertex) != VK_SUCCESS) return fail("vertex buffer");
    if (make_buffer(c, s->index_bytes, VK_BUFFER_USAGE_INDEX_BUFFER_BIT | VK_BUFFER_USAGE_TRANSFER_DST_BIT, false, r->index) != VK_SUCCESS)
        return fail("index buffer");
    if (s->uniform_bytes && make_buffer(c, s->uniform_bytes, VK_BUFFER_USAGE_UNIFORM_BUFFER_BIT | VK_BUFFER_USAGE_TRANSFER_DST_BIT, false, r->uniform) != VK_SUCCESS)
        return fail("uniform buffer");
    const uint64_t staging = ((s->vertex_bytes + 255) & ~255ull) + ((s->index_bytes + 255) & ~255ull) + ((s->uniform_bytes + 255) & ~255ull) +
                             ((s->texture_bytes + 255) & ~255ull);
    r->upload_bytes = s->vertex_bytes + s->index_bytes + s->uniform_bytes;
    if (make_buffer(c, staging, VK_BUFFER_USAGE_TRANSFER_SRC_BIT, true, r->staging) != VK_SUCCESS) return fail("staging buffer");
    r->depth_texel = depth_texel_size(s->depth_format);
    r->colour_texel = colour_texel_size(s->color_format);
    const uint64_t rb_bytes = static_cast<uint64_t>(s->width) * s->height * (std::max<uint32_t>(r->colour_texel, 4u) + r->depth_texel);
    if (make_buffer(c, rb_bytes, VK_BUFFER_USAGE_TRANSFER_DST_BIT, true, r->readback) != VK_SUCCESS) return fail("readback buffer");
    // CPVH_INDIRECT=1: the frame issues every draw as an indirect draw whose
    // record (VkDrawIndexedIndirectCommand / VkDrawIndirectCommand, 20-byte
    // stride) lives in a host-visible buffer. CPVH_INDIRECT=2: as an
    // indirect-count draw of at most one record, whose count word (one per
    // draw, initially 1) lives in a second host-visible buffer.
    if (const char* sec = std::getenv("CPVH_SECONDARY")) r->use_secondary = sec[0] == '1';
    const char* ind = std::getenv("CPVH_INDIRECT");
    if (ind && ind[0] == '2' && s->num_draws) {
        if (make_buffer(c, static_cast<VkDeviceSize>(s->num_draws) * 4, VK_BUFFER_USAGE_INDIRECT_BUFFER_BIT, true, r->indirect_count) != VK_SUCCESS)
            return fail("indirect count buffer");
        void* map = nullptr;
        if (c->f.vkMapMemory(c->device, r->indirect_count.memory, 0, VK_WHOLE_SIZE, 0, &map) != VK_SUCCESS) return fail("indirect count map");
        for (uint32_t i = 0; i < s->num_draws; i++) static_cast<uint32_t*>(map)[i] = 1u;
        c->f.vkUnmapMemory(c->device, r->indirect_count.memory);
    }
    if (ind && (ind[0] == '1' || ind[0] == '2') && s->num_draws) {
        if (make_buffer(c, static_cast<VkDeviceSize>(s->num_draws) * 20, VK_BUFFER_USAGE_INDIRECT_BUFFER_BIT, true, r->indirect) != VK_SUCCESS)
            return fail("indirect buffer");
        void* map = nullptr;
        if (c->f.vkMapMemory(c->device, r->indirect.memory, 0, VK_WHOLE_SIZE, 0, &map) != VK_SUCCESS) return fail("indirect map");
        for (uint32_t i = 0; i < s->num_draws; i++) {
            const cpv_scene_draw& d = s->draws[i];
            uint32_t rec[5];
            if (d.indexed) {
                rec[0] = d.count, rec[1] = d.instance_count, rec[2] = d.first, rec[3] = static_cast<uint32_t>(d.vertex_offset), rec[4] = d.first_instance;
            } else {
                rec[0] = d.count, rec[1] = d.instance_count, rec[2] = d.first, rec[3] = d.first_instance, rec[4] = 0;
            }
            std::memcpy(static_cast<uint8_t*>(map) + static_cast<size_t>(i) * 20, rec, 20);
        }
        c->f.vkUnmapMemory(c->device, r->indirect.memory);
    }
    if (s->color_format &&
        make_image(c, static_cast<VkFormat>(s->color_format), s->width, s->height, 1, VK_IMAGE_USAGE_COLOR_ATTACHMENT_BIT | VK_IMAGE_USAGE_TRANSFER_SRC_BIT,
                   VK_IMAGE_ASPECT_COLOR_BIT, r->colour) != VK_SUCCESS)
        return fail("colour image");
    if (s->depth_format &&
        make_image(c, static_cast<VkFormat>(s->depth_format), s->width, s->height, 1, VK_IMAGE_USAGE_DEPTH_STENCIL_ATTACHMENT_BIT | VK_IMAGE_USAGE_TRANSFER_SRC_BIT,
                   VK_IMAGE_ASPECT_DEPTH_BIT, r->depth) != VK_SUCCESS)
        return fail("depth image");
    r->extra.resize(s->color_format ? s->extra_color_count : 0);
    for (uint32_t k = 0; k < r->extra.size(); k++)
        if (s->extra_color_formats[k] &&
            make_image(c, static_cast<VkFormat>(s->extra_color_formats[k]), s->width, s->height, 1,
                       VK_IMAGE_USAGE_COLOR_ATTACHMENT_BIT | VK_IMAGE_USAGE_TRANSFER_SRC_BIT, VK_IMAGE_ASPECT_COLOR_BIT, r->extra[k]) != VK_SUCCESS)
            return fail("colour image " + std::to_string(k + 1));
    if (s->texture_data) {
        const VkImageUsageFlags tex_usage = s->texture_binding == CPV_TEXTURE_STORAGE ? VK_IMAGE_USAGE_STORAGE_BIT : VK_IMAGE_USAGE_SAMPLED_BIT;
        if (make_image(c, static_cast<VkFormat>(s->texture_format), s->texture_width, s->texture_height, s->texture_levels,
                       tex_usage | VK_IMAGE_USAGE_TRANSFER_DST_BIT, VK_IMAGE_ASPECT_COLOR_BIT, r->texture) != VK_SUCCESS)
            return fail("texture image");
        VkSamplerCreateInfo sci{};
        sci.sType = VK_STRUCTURE_TYPE_SAMPLER_CREATE_INFO;
        sci.magFilter = static_cast<VkFilter>(s->sampler.mag_filter);
        sci.minFilter = static_cast<VkFilter>(s->sampler.min_filter);
        sci.mipmapMode = static_cast<VkSamplerMipmapMode>(s->sampler.mipmap_mode);
        sci.addressModeU = static_cast<VkSamplerAddressMode>(s->sampler.address_u);
        sci.addressModeV = static_cast<VkSamplerAddressMode>(s->sampler.address_v);
        sci.addressModeW = static_cast<VkSamplerAddressMode>(s->sampler.address_w);
        sci.mipLodBias = s->sampler.mip_lod_bias;
        sci.minLod = s->sampler.min_lod;
        sci.maxLod = s->sampler.max_lod;
        sci.borderColor = static_cast<VkBorderColor>(s->sampler.border_color);
        if (f.vkCreateSampler(c->device, &sci, nullptr, &r->sampler) != VK_SUCCESS) return fail("sampler");
    }
    // Render pass + framebuffer.
    // CPVH_SUBPASSES=2: the frame draws in subpass 1 of a two-subpass render
    // pass (its pipelines are created for subpass 1)
    const char* subpasses = std::getenv("CPVH_SUBPASSES");
    r->subpass = subpasses && subpasses[0] == '2' ? 1u : 0u;
    if (create_scene_pass(c, s, &r->pass, r->subpass == 1) != VK_SUCCESS) return fail("render pass");
    // attachments in order: colour (absent in a depth-only pass), the
    // further colour attachments, depth
    VkImageView views[2 + CPV_SCENE_MAX_EXTRA_COLOR];
    uint32_t nviews = 0;
    if (s->color_format) {
        views[nviews++] = r->colour.view;
        for (const ImageAlloc& e : r->extra)
            if (e.view) views[nviews++] = e.view;
    }
    if (s->depth_format) views[nviews++] = r->depth.view;
    VkFramebufferCreateInfo fbi{};
    fbi.sType = VK_STRUCTURE_TYPE_FRAMEBUFFER_CREATE_INFO;
    fbi.renderPass = r->pass;
    fbi.attachmentCount = nviews;
    fbi.pAttachments = views;
    fbi.width = s->width;
    fbi.height = s->height;
    fbi.layers = 1;
    if (f.vkCreateFramebuffer(c->device, &fbi, nullptr, &r->fb) != VK_SUCCESS) return fail("framebuffer");
    // Descriptors: binding 0 uniform buffer, the texture at binding 1 (and
    // its sampler at binding 2 when they are separate).
    const std::vector<VkDescriptorSetLayoutBinding> lb = scene_bindings(s);
    VkDescriptorSetLayoutCreateInfo dli{};
    dli.sType = VK_STRUCTURE_TYPE_DESCRIPTOR_SET_LAYOUT_CREATE_INFO;
    dli.bindingCount = static_cast<uint32_t>(lb.size());
    dli.pBindings = lb.data();
    if (f.vkCreateDescriptorSetLayout(c->device, &dli, nullptr, &r->set_layout) != VK_SUCCESS) return fail("set layout");
    VkDescriptorPoolSize ps[6] = {{VK_DESCRIPTOR_TYPE_UNIFORM_BUFFER, 1}, {VK_DESCRIPTOR_TYPE_COMBINED_IMAGE_SAMPLER, 1}, {VK_DESCRIPTOR_TYPE_STORAGE_IMAGE, 1},
                                  {VK_DESCRIPTOR_TYPE_SAMPLED_IMAGE, 1}, {VK_DESCRIPTOR_TYPE_SAMPLER, 1}, {VK_DESCRIPTOR_TYPE_STORAGE_BUFFER, 1}};
    VkDescriptorPoolCreateInfo dpi{};
    dpi.sType = VK_STRUCTURE_TYPE_DESCRIPTOR_POOL_CREATE_INFO;
    dpi.maxSets = 1;
    dpi.poolSizeCount = 6;
    dpi.pPoolSizes = ps;
    if (f.vkCreateDescriptorPool(c->device, &dpi, nullptr, &r->pool) != VK_SUCCESS) return fail("descriptor pool");
    if (!lb.empty()) {
        VkDescriptorSetAllocateInfo dai{};
        dai.sType = VK_STRUCTURE_TYPE_DESCRIPTOR_SET_ALLOCATE_INFO;
        dai.descriptorPool = r->pool;
        dai.descriptorSetCount = 1;
        dai.pSetLayouts = &r->set_layout;
        if (f.vkAllocateDescriptorSets(c->device, &dai, &r->set) != VK_SUCCESS) return fail("descriptor set");
        VkDescriptorBufferInfo dbi{r->uniform.buffer, 0, VK_WHOLE_SIZE};
        VkDescriptorImageInfo dii{r->sampler, r->texture.view, VK_IMAGE_LAYOUT_SHADER_READ_ONLY_OPTIMAL};
        if (s->texture_binding == CPV_TEXTURE_STORAGE) dii = {VK_NULL_HANDLE, r->texture.view, VK_IMAGE_LAYOUT_GENERAL};
        if (s->texture_binding == CPV_TEXTURE_SEPARATE) dii.sampler = VK_NULL_HANDLE;
        const VkDescriptorImageInfo sampler_info{r->sampler, VK_NULL_HANDLE, VK_IMAGE_LAYOUT_UNDEFINED};
        VkWriteDescriptorSet w[4]{};
        uint32_t nw = 0;
        if (s->uniform_bytes) {
            w[nw].sType = VK_STRUCTURE_TYPE_WRITE_DESCRIPTOR_SET;
            w[nw].dstSet = r->set;
            w[nw].dstBinding = 0;
            w[nw].descriptorCount = 1;
            w[nw].descriptorType = VK_DESCRIPTOR_TYPE_UNIFORM_BUFFER;
            w[nw].pBufferInfo = &dbi;
            nw++;
            if (s->uniform_as_storage) {
                w[nw].sType = VK_STRUCTURE_TYPE_WRITE_DESCRIPTOR_SET;
                w[nw].dstSet = r->set;
                w[nw].dstBinding = 3;
                w[nw].descriptorCount = 1;
                w[nw].descriptorType = VK_DESCRIPTOR_TYPE_STORAGE_BUFFER;
                w[nw].pBufferInfo = &dbi;
                nw++;
            }
        }
        if (s->texture_data) {
            w[nw].sType = VK_STRUCTURE_TYPE_WRITE_DESCRIPTOR_SET;
            w[nw].dstSet = r->set;
            w[nw].dstBinding = 1;
            w[nw].descriptorCount = 1;
            w[nw].descriptorType = s->texture_binding == CPV_TEXTURE_STORAGE    ? VK_DESCRIPTOR_TYPE_STORAGE_IMAGE
                                   : s->texture_binding == CPV_TEXTURE_SEPARATE ? VK_DESCRIPTOR_TYPE_SAMPLED_IMAGE
                                                                                : VK_DESCRIPTOR_TYPE_COMBINED_IMAGE_SAMPLER;
            w[nw].pImageInfo = &dii;
            nw++;
            if (s->texture_binding == CPV_TEXTURE_SEPARATE) {
                w[nw].sType = VK_STRUCTURE_TYPE_WRITE_DESCRIPTOR_SET;
                w[nw].dstSet = r->set;
                w[nw].dstBinding = 2;
                w[nw].descriptorCount = 1;
                w[nw].descriptorType = VK_DESCRIPTOR_TYPE_SAMPLER;
                w[nw].pImageInfo = &sampler_info;
                nw++;
            }
        }
        f.vkUpdateDescriptorSets(c->device, nw, w, 0, nullptr);
    }
    VkPushConstantRange pcr{VK_SHADER_STAGE_VERTEX_BIT | VK_SHADER_STAGE_FRAGMENT_BIT, 0, 128};
    VkPipelineLayoutCreateInfo pli{};
    pli.sType = VK_STRUCTURE_TYPE_PIPELINE_LAYOUT_CREATE_INFO;
    pli.setLayoutCount = 1;
    pli.pSetLayouts = &r->set_layout;
    pli.pushConstantRangeCount = 1;
    pli.pPushConstantRanges = &pcr;
    if (f.vkCreatePipelineLayout(c->device, &pli, nullptr, &r->layout) != VK_SUCCESS) return fail("pipeline layout");
    {
        std::string perr;
        if (!build_pipelines(c, s, r->pass, r->layout, r->modules, r->pipelines, perr, r->subpass)) return fail(perr);
    }
    // Command buffers and fence.
    VkCommandPoolCreateInfo cpi{};
    cpi.sType = VK_STRUCTURE_TYPE_COMMAND_POOL_CREATE_INFO;
    cpi.flags = VK_COMMAND_POOL_CREATE_RESET_COMMAND_BUFFER_BIT;
    if (f.vkCreateCommandPool(c->device, &cpi, nullptr, &r->cmd_pool) != VK_SUCCESS) return fail("command pool");
    VkCommandBuffer cbs3[3];
    VkCommandBufferAllocateInfo cai{};
    cai.sType = VK_STRUCTURE_TYPE_COMMAND_BUFFER_ALLOCATE_INFO;
    cai.commandPool = r->cmd_pool;
    cai.level = VK_COMMAND_BUFFER_LEVEL_PRIMARY;
    cai.commandBufferCount = 3;
    if (f.vkAllocateCommandBuffers(c->device, &cai, cbs3) != VK_SUCCESS) return fail("command buffers");
    for (auto cb : cbs3)
        if (!check_dispatch(cb)) return fail("VkCommandBuffer lacks the loader magic");
    r->frame_cmd = cbs3[0];
    r->e2e_cmd = cbs3[1];
    r->copy_cmd = cbs3[2];
    VkFenceCreateInfo fci{};
    fci.sType = VK_STRUCTURE_TYPE_FENCE_CREATE_INFO;
    if (f.vkCreateFence(c->device, &fci, nullptr, &r->fence) != VK_SUCCESS) return fail("fence");
    // Upload vertex/index/uniform/texture once through the staging buffer.
    void* map = nullptr;
    if (f.vkMapMemory(c->device, r->staging.memory, 0, VK_WHOLE_SIZE, 0, &map) != VK_SUCCESS) return fail("map staging");
    fill_staging(r, map);
    const uint64_t tex_off = ((s->vertex_bytes + 255) & ~255ull) + ((s->index_bytes + 255) & ~255ull) + ((s->uniform_bytes + 255) & ~255ull);
    if (s->texture_data) std::memcpy(static_cast<uint8_t*>(map) + tex_off, s->texture_data, s->texture_bytes);
    f.vkUnmapMemory(c->device, r->staging.memory);
    VkCommandBufferBeginInfo bi{};
    bi.sType = VK_STRUCTURE_TYPE_COMMAND_BUFFER_BEGIN_INFO;
    f.vkBeginCommandBuffer(r->copy_cmd, &bi);
    record_upload(r, r->copy_cmd);
    if (s->texture_data) {
        uint64_t off = tex_off;
        uint32_t w = s->texture_width, h = s->texture_height;
        for (uint32_t l = 0; l < s->texture_levels; l++) {
            VkBufferImageCopy bc{};
            bc.bufferOffset = off;
            bc.imageSubresource = {VK_IMAGE_ASPECT_COLOR_BIT, l, 0, 1};
            bc.imageExtent = {w, h, 1};
            f.vkCmdCopyBufferToImage(r->copy_cmd, r->staging.buffer, r->texture.image, VK_IMAGE_LAYOUT_TRANSFER_DST_OPTIMAL, 1, &bc);
            off += static_cast<uint64_t>(w) * h * 4;
            w = w > 1 ? w / 2 : 1;
            h = h > 1 ? h / 2 : 1;
        }
    }
    f.vkEndCommandBuffer(r->copy_cmd);
    // CPVH_RECORD_ONLY=1: record the frame without uploading (on a device
    // that compiles but cannot execute, recording still compiles the
    // batched modules at vkEndCommandBuffer)
    const char* record_only = std::getenv("CPVH_RECORD_ONLY");
    if (!(record_only && record_only[0] == '1') && submit_and_wait(r, r->copy_cmd) != VK_SUCCESS) return fail("upload submit");
    record_all(r);
    return r;
}

int cpvh_compile_pipelines(cpvh_context* c, const cpv_scene* s, char* err, uint32_t err_len) {
    VkRenderPass pass = nullptr;
    VkDescriptorSetLayout set_layout = nullptr;
    VkPipelineLayout layout = nullptr;
    std::vector<VkShaderModule> modules;
    std::vector<VkPipeline> pipelines;
    std::string perr;
    // CPVH_SUBPASSES=2: pipelines for subpass 1 of the two-subpass pass the
    // renderer uses; "2:0": for its subpass 0 (depth attachment only)
    const char* sp = std::getenv("CPVH_SUBPASSES");
    const bool two = sp && sp[0] == '2';
    const uint32_t subpass = two && std::strcmp(sp, "2:0") != 0 ? 1u : 0u;
    int result = make_pass_and_layout(c, s, true, pass, set_layout, layout, two);
    if (result == VK_SUCCESS && !build_pipelines(c, s, pass, layout, modules, pipelines, perr, subpass)) result = VK_ERROR_INITIALIZATION_FAILED;
    if (result != VK_SUCCESS) {
        g_err = perr + " " + icd_error(c);
        if (err && err_len) std::snprintf(err, err_len, "%s", g_err.c_str());
    }
    for (auto p : pipelines) c->f.vkDestroyPipeline(c->device, p, nullptr);
    for (auto m : modules) c->f.vkDestroyShaderModule(c->device, m, nullptr);
    if (layout) c->f.vkDestroyPipelineLayout(c->device, layout, nullptr);
    if (set_layout) c->f.vkDestroyDescriptorSetLayout(c->device, set_layout, nullptr);
    if (pass) c->f.vkDestroyRenderPass(c->device, pass, nullptr);
    return result;
}

}  // extern "C"

namespace {

// Destroys a renderer's objects. wait_idle: after the device has gone idle
// (any queue may still use them); without it the caller knows that all of
// the renderer's submissions have finished (their fences signalled).
void renderer_destroy(cpvh_renderer* r, bool wait_idle) {
    if (!r) return;
    cpvh_context* c = r->ctx;
    const Fns& f = c->f;
    if (wait_idle) f.vkDeviceWaitIdle(c->device);
    if (r->fence) f.vkDestroyFence(c->device, r->fence, nullptr);
    if (r->cmd_pool) f.vkDestroyCommandPool(c->device, r->cmd_pool, nullptr);
    for (auto p : r->pipelines) f.vkDestroyPipeline(c->device, p, nullptr);
    for (auto m : r->modules) f.vkDestroyShaderModule(c->device, m, nullptr);
    if (r->layout) f.vkDestroyPipelineLayout(c->device, r->layout, nullptr);
    if (r->pool) f.vkDestroyDescriptorPool(c->device, r->pool, nullptr);
    if (r->set_layout) f.vkDestroyDescriptorSetLayout(c->device, r->set_layout, nullptr);
    if (r->fb) f.vkDestroyFramebuffer(c->device, r->fb, nullptr);
    if (r->pass) f.vkDestroyRenderPass(c->device, r->pass, nullptr);
    if (r->sampler) f.vkDestroySampler(c->device, r->sampler, nullptr);
    destroy_image(c, r->colour);
    for (ImageAlloc& e : r->extra) destroy_image(c, e);
    destroy_image(c, r->depth);
    destroy_image(c, r->texture);
    destroy_buffer(c, r->vertex);
    destroy_buffer(c, r->index);
    destroy_buffer(c, r->uniform);
    destroy_buffer(c, r->staging);
    destroy_buffer(c, r->readback);
    destroy_buffer(c, r->indirect);
    destroy_buffer(c, r->indirect_count);
    delete r;
}

}  // namespace

extern "C" {

void cpvh_renderer_destroy(cpvh_renderer* r) { renderer_destroy(r, true); }

int cpvh_renderer_update(cpvh_renderer* r) {
    cpvh_context* c = r->ctx;
    void* map = nullptr;
    if (c->f.vkMapMemory(c->device, r->staging.memory, 0, VK_WHOLE_SIZE, 0, &map) != VK_SUCCESS) return VK_ERROR_MEMORY_MAP_FAILED;
    fill_staging(r, map);
    c->f.vkUnmapMemory(c->device, r->staging.memory);
    VkCommandBufferBeginInfo bi{};
    bi.sType = VK_STRUCTURE_TYPE_COMMAND_BUFFER_BEGIN_INFO;
    c->f.vkBeginCommandBuffer(r->copy_cmd, &bi);
    record_upload(r, r->copy_cmd);
    c->f.vkEndCommandBuffer(r->copy_cmd);
    const VkResult res = submit_and_wait(r, r->copy_cmd);
    record_all(r);
    return res;
}

int cpvh_renderer_set_indirect(cpvh_renderer* r, uint32_t draw, const uint32_t record[5]) {
    cpvh_context* c = r->ctx;
    if (!r->indirect.buffer || draw >= r->scene->num_draws) return VK_ERROR_INITIALIZATION_FAILED;
    void* map = nullptr;
    if (c->f.vkMapMemory(c->device, r->indirect.memory, static_cast<VkDeviceSize>(draw) * 20, 20, 0, &map) != VK_SUCCESS) return VK_ERROR_MEMORY_MAP_FAILED;
    std::memcpy(map, record, 20);
    c->f.vkUnmapMemory(c->device, r->indirect.memory);
    return VK_SUCCESS;
}

int cpvh_renderer_set_indirect_count(cpvh_renderer* r, uint32_t draw, uint32_t count) {
    cpvh_context* c = r->ctx;
    if (!r->indirect_count.buffer || draw >= r->scene->num_draws) return VK_ERROR_INITIALIZATION_FAILED;
    void* map = nullptr;
    if (c->f.vkMapMemory(c->device, r->indirect_count.memory, static_cast<VkDeviceSize>(draw) * 4, 4, 0, &map) != VK_SUCCESS) return VK_ERROR_MEMORY_MAP_FAILED;
    std::memcpy(map, &count, 4);
    c->f.vkUnmapMemory(c->device, r->indirect_count.memory);
    return VK_SUCCESS;
}

int cpvh_render(cpvh_renderer* r, uint32_t frames, double* device_ms, double* latency_ms) {
    cpvh_context* c = r->ctx;
    VkSubmitInfo si{};
    si.sType = VK_STRUCTURE_TYPE_SUBMIT_INFO;
    si.commandBufferCount = 1;
    si.pCommandBuffers = &r->frame_cmd;
    if (c->record) c->record(c->queue, 0);
    for (uint32_t i = 0; i < frames; i++) {
        const bool wait = latency_ms != nullptr || i + 1 == frames;
        const auto t0 = std::chrono::steady_clock::now();
        VkResult res = c->f.vkQueueSubmit(c->queue, 1, &si, wait ? r->fence : nullptr);
        if (res != VK_SUCCESS) return res;
        if (wait) {
            res = c->f.vkWaitForFences(c->device, 1, &r->fence, VK_TRUE, ~0ull);
            c->f.vkResetFences(c->device, 1, &r->fence);
            if (res != VK_SUCCESS) return res;
        }
        if (latency_ms) latency_ms[i] = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    }
    if (c->record) c->record(c->queue, 1);
    if (device_ms) *device_ms = c->elapsed ? c->elapsed(c->queue, 0, 1) : -1.0;
    return VK_SUCCESS;
}

int cpvh_render_timed(cpvh_renderer* r, uint32_t frames, uint64_t flush_bytes, double* frame_ms) {
    cpvh_context* c = r->ctx;
    if (!c->record || !c->elapsed) return VK_ERROR_FEATURE_NOT_PRESENT;
    BufferAlloc flush;
    VkCommandBuffer flush_cmd = nullptr;
    if (flush_bytes) {
        if (make_buffer(c, flush_bytes, VK_BUFFER_USAGE_TRANSFER_DST_BIT, false, flush) != VK_SUCCESS) return VK_ERROR_OUT_OF_DEVICE_MEMORY;
        VkCommandBufferAllocateInfo cai{};
        cai.sType = VK_STRUCTURE_TYPE_COMMAND_BUFFER_ALLOCATE_INFO;
        cai.commandPool = r->cmd_pool;
        cai.level = VK_COMMAND_BUFFER_LEVEL_PRIMARY;
        cai.commandBufferCount = 1;
        c->f.vkAllocateCommandBuffers(c->device, &cai, &flush_cmd);
        auto fill = reinterpret_cast<PFN_vkCmdFillBuffer>(c->f.vkGetDeviceProcAddr(c->device, "vkCmdFillBuffer"));
        VkCommandBufferBeginInfo bi{};
        bi.sType = VK_STRUCTURE_TYPE_COMMAND_BUFFER_BEGIN_INFO;
        c->f.vkBeginCommandBuffer(flush_cmd, &bi);
        fill(flush_cmd, flush.buffer, 0, VK_WHOLE_SIZE, 0x5A5A5A5Au);
        c->f.vkEndCommandBuffer(flush_cmd);
    }
    VkSubmitInfo si{};
    si.sType = VK_STRUCTURE_TYPE_SUBMIT_INFO;
    si.commandBufferCount = 1;
    VkResult res = VK_SUCCESS;
    for (uint32_t i = 0; i < frames && res == VK_SUCCESS; i++) {
        if (flush_cmd) {
            si.pCommandBuffers = &flush_cmd;
            res = c->f.vkQueueSubmit(c->queue, 1, &si, nullptr);
            if (res != VK_SUCCESS) break;
        }
        c->record(c->queue, 2);
        si.pCommandBuffers = &r->frame_cmd;
        res = c->f.vkQueueSubmit(c->queue, 1, &si, r->fence);
        if (res != VK_SUCCESS) break;
        c->record(c->queue, 3);
        res = c->f.vkWaitForFences(c->device, 1, &r->fence, VK_TRUE, ~0ull);
        c->f.vkResetFences(c->device, 1, &r->fence);
        if (frame_ms) frame_ms[i] = c->elapsed(c->queue, 2, 3);
    }
    c->f.vkDeviceWaitIdle(c->device);
    destroy_buffer(c, flush);
    return res;
}

int cpvh_render_e2e(cpvh_renderer* r, uint32_t frames, double* total_ms, uint64_t* h2d, uint64_t* d2h) {
    cpvh_context* c = r->ctx;
    const cpv_scene* s = r->scene;
    const auto t0 = std::chrono::steady_clock::now();
    const uint64_t out_bytes = static_cast<uint64_t>(s->width) * s->height * r->colour_texel;
    std::vector<uint8_t> host_out(out_bytes);
    for (uint32_t i = 0; i < frames; i++) {
        // The inputs live in the staging buffer's host-visible (pinned)
        // memory, written there at creation; mapping and unmapping it hands
        // them to the ICD again, which copies the whole allocation to HBM.
        void* map = nullptr;
        if (c->f.vkMapMemory(c->device, r->staging.memory, 0, VK_WHOLE_SIZE, 0, &map) != VK_SUCCESS) return VK_ERROR_MEMORY_MAP_FAILED;
        c->f.vkUnmapMemory(c->device, r->staging.memory);
        const VkResult res = submit_and_wait(r, r->e2e_cmd);
        if (res != VK_SUCCESS) return res;
        if (c->f.vkMapMemory(c->device, r->readback.memory, 0, VK_WHOLE_SIZE, 0, &map) != VK_SUCCESS) return VK_ERROR_MEMORY_MAP_FAILED;
        std::memcpy(host_out.data(), map, out_bytes);
        c->f.vkUnmapMemory(c->device, r->readback.memory);
    }
    if (total_ms) *total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    if (h2d) *h2d = r->staging.size;
    if (d2h) *d2h = out_bytes;
    return VK_SUCCESS;
}

int cpvh_readback(cpvh_renderer* r, uint8_t* color, uint8_t* depth) {
    cpvh_context* c = r->ctx;
    const cpv_scene* s = r->scene;
    VkCommandBufferBeginInfo bi{};
    bi.sType = VK_STRUCTURE_TYPE_COMMAND_BUFFER_BEGIN_INFO;
    c->f.vkBeginCommandBuffer(r->copy_cmd, &bi);
    record_readback(r, r->copy_cmd);
    c->f.vkEndCommandBuffer(r->copy_cmd);
    VkResult res = submit_and_wait(r, r->copy_cmd);
    if (res != VK_SUCCESS) return res;
    void* map = nullptr;
    res = c->f.vkMapMemory(c->device, r->readback.memory, 0, VK_WHOLE_SIZE, 0, &map);
    if (res != VK_SUCCESS) return res;
    const uint64_t cb = static_cast<uint64_t>(s->width) * s->height * r->colour_texel;
    if (color && s->color_format) std::memcpy(color, map, cb);
    else if (color) std::memset(color, 0, cb);  // a depth-only pass
    if (depth && s->depth_format) std::memcpy(depth, static_cast<uint8_t*>(map) + cb, static_cast<uint64_t>(s->width) * s->height * r->depth_texel);
    c->f.vkUnmapMemory(c->device, r->readback.memory);
    return VK_SUCCESS;
}

int cpvh_readback_extra(cpvh_renderer* r, uint32_t k, uint8_t* out) {
    cpvh_context* c = r->ctx;
    const cpv_scene* s = r->scene;
    if (k < 1 || k > r->extra.size() || !out) return VK_ERROR_INITIALIZATION_FAILED;
    const uint32_t fmt = s->extra_color_formats[k - 1];
    const uint64_t bytes = static_cast<uint64_t>(s->width) * s->height * colour_texel_size(fmt);
    if (!fmt) {  // an unused reference has no image
        std::memset(out, 0, bytes);
        return VK_SUCCESS;
    }
    // the readback buffer holds a 4-byte colour texel per pixel at least
    VkCommandBufferBeginInfo bi{};
    bi.sType = VK_STRUCTURE_TYPE_COMMAND_BUFFER_BEGIN_INFO;
    c->f.vkBeginCommandBuffer(r->copy_cmd, &bi);
    VkBufferImageCopy bc{};
    bc.imageSubresource = {VK_IMAGE_ASPECT_COLOR_BIT, 0, 0, 1};
    bc.imageExtent = {s->width, s->height, 1};
    c->f.vkCmdCopyImageToBuffer(r->copy_cmd, r->extra[k - 1].image, VK_IMAGE_LAYOUT_TRANSFER_SRC_OPTIMAL, r->readback.buffer, 1, &bc);
    c->f.vkEndCommandBuffer(r->copy_cmd);
    VkResult res = submit_and_wait(r, r->copy_cmd);
    if (res != VK_SUCCESS) return res;
    void* map = nullptr;
    res = c->f.vkMapMemory(c->device, r->readback.memory, 0, VK_WHOLE_SIZE, 0, &map);
    if (res != VK_SUCCESS) return res;
    std::memcpy(out, map, bytes);
    c->f.vkUnmapMemory(c->device, r->readback.memory);
    return VK_SUCCESS;
}

int cpvh_blit(cpvh_context* c, uint8_t* src, uint32_t src_w, uint32_t src_h, uint32_t src_levels, uint32_t src_format, uint8_t* dst,
              uint32_t dst_w, uint32_t dst_h, uint32_t dst_levels, uint32_t dst_format, const int32_t* regions, uint32_t region_count,
              uint32_t filter, char* err, uint32_t err_len) {
    const Fns& f = c->f;
    struct Packed {
        uint64_t offset[16] = {};
        uint32_t w[16] = {}, h[16] = {};
        uint64_t bytes = 0;
    };
    auto pack = [](uint32_t w, uint32_t h, uint32_t levels, Packed& p) {
        for (uint32_t l = 0; l < levels; l++) {
            p.offset[l] = p.bytes;
            p.w[l] = w;
            p.h[l] = h;
            p.bytes += static_cast<uint64_t>(w) * h * 4;
            w = w > 1 ? w / 2 : 1;
            h = h > 1 ? h / 2 : 1;
        }
    };
    ImageAlloc src_img, dst_img;
    BufferAlloc staging;
    VkCommandPool pool = nullptr;
    VkFence fence = nullptr;
    int rc = VK_SUCCESS;
    auto cleanup = [&]() {
        if (fence) f.vkDestroyFence(c->device, fence, nullptr);
        if (pool) f.vkDestroyCommandPool(c->device, pool, nullptr);
        destroy_buffer(c, staging);
        destroy_image(c, dst_img);
        destroy_image(c, src_img);
    };
    auto fail = [&](const std::string& e, int code) {
        g_err = e + " " + icd_error(c);
        if (err && err_len) std::snprintf(err, err_len, "%s", g_err.c_str());
        cleanup();
        return code;
    };
    if (!src || src_levels == 0 || src_levels > 16 || (dst && (dst_levels == 0 || dst_levels > 16)))
        return fail("blit: bad image description", VK_ERROR_INITIALIZATION_FAILED);
    Packed sp, dp;
    pack(src_w, src_h, src_levels, sp);
    if (dst) pack(dst_w, dst_h, dst_levels, dp);
    const VkImageUsageFlags usage = VK_IMAGE_USAGE_TRANSFER_SRC_BIT | VK_IMAGE_USAGE_TRANSFER_DST_BIT | VK_IMAGE_USAGE_SAMPLED_BIT;
    if (make_image(c, static_cast<VkFormat>(src_format), src_w, src_h, src_levels, usage, VK_IMAGE_ASPECT_COLOR_BIT, src_img) != VK_SUCCESS)
        return fail("blit: source image", VK_ERROR_OUT_OF_DEVICE_MEMORY);
    if (dst && make_image(c, static_cast<VkFormat>(dst_format), dst_w, dst_h, dst_levels, usage, VK_IMAGE_ASPECT_COLOR_BIT, dst_img) != VK_SUCCESS)
        return fail("blit: destination image", VK_ERROR_OUT_OF_DEVICE_MEMORY);
    if (make_buffer(c, sp.bytes + dp.bytes, VK_BUFFER_USAGE_TRANSFER_SRC_BIT | VK_BUFFER_USAGE_TRANSFER_DST_BIT, true, staging) != VK_SUCCESS)
        return fail("blit: staging buffer", VK_ERROR_OUT_OF_DEVICE_MEMORY);
    void* map = nullptr;
    if (f.vkMapMemory(c->device, staging.memory, 0, VK_WHOLE_SIZE, 0, &map) != VK_SUCCESS) return fail("blit: map", VK_ERROR_MEMORY_MAP_FAILED);
    std::memcpy(map, src, sp.bytes);
    if (dst) std::memcpy(static_cast<uint8_t*>(map) + sp.bytes, dst, dp.bytes);
    f.vkUnmapMemory(c->device, staging.memory);

    VkCommandPoolCreateInfo cpi{};
    cpi.sType = VK_STRUCTURE_TYPE_COMMAND_POOL_CREATE_INFO;
    if (f.vkCreateCommandPool(c->device, &cpi, nullptr, &pool) != VK_SUCCESS) return fail("blit: command pool", VK_ERROR_INITIALIZATION_FAILED);
    VkCommandBufferAllocateInfo cai{};
    cai.sType = VK_STRUCTURE_TYPE_COMMAND_BUFFER_ALLOCATE_INFO;
    cai.commandPool = pool;
    cai.level = VK_COMMAND_BUFFER_LEVEL_PRIMARY;
    cai.commandBufferCount = 1;
    VkCommandBuffer cmd = nullptr;
    if (f.vkAllocateCommandBuffers(c->device, &cai, &cmd) != VK_SUCCESS || !check_dispatch(cmd))
        return fail("blit: command buffer", VK_ERROR_INITIALIZATION_FAILED);
    VkFenceCreateInfo fci{};
    fci.sType = VK_STRUCTURE_TYPE_FENCE_CREATE_INFO;
    if (f.vkCreateFence(c->device, &fci, nullptr, &fence) != VK_SUCCESS) return fail("blit: fence", VK_ERROR_INITIALIZATION_FAILED);

    VkImage target = dst ? dst_img.image : src_img.image;
    const Packed& tp = dst ? dp : sp;
    const uint32_t target_levels = dst ? dst_levels : src_levels;
    auto level_copy = [](const Packed& p, uint64_t base, uint32_t l) {
        VkBufferImageCopy bc{};
        bc.bufferOffset = base + p.offset[l];
        bc.imageSubresource = {VK_IMAGE_ASPECT_COLOR_BIT, l, 0, 1};
        bc.imageExtent = {p.w[l], p.h[l], 1};
        return bc;
    };
    VkMemoryBarrier mb{};
    mb.sType = VK_STRUCTURE_TYPE_MEMORY_BARRIER;
    mb.srcAccessMask = VK_ACCESS_TRANSFER_WRITE_BIT;
    mb.dstAccessMask = VK_ACCESS_TRANSFER_READ_BIT | VK_ACCESS_TRANSFER_WRITE_BIT;
    auto barrier = [&]() {
        f.vkCmdPipelineBarrier(cmd, VK_PIPELINE_STAGE_TRANSFER_BIT, VK_PIPELINE_STAGE_TRANSFER_BIT, 0, 1, &mb, 0, nullptr, 0, nullptr);
    };
    VkCommandBufferBeginInfo bi{};
    bi.sType = VK_STRUCTURE_TYPE_COMMAND_BUFFER_BEGIN_INFO;
    f.vkBeginCommandBuffer(cmd, &bi);
    for (uint32_t l = 0; l < src_levels; l++) {
        const VkBufferImageCopy bc = level_copy(sp, 0, l);
        f.vkCmdCopyBufferToImage(cmd, staging.buffer, src_img.image, VK_IMAGE_LAYOUT_TRANSFER_DST_OPTIMAL, 1, &bc);
    }
    if (dst)
        for (uint32_t l = 0; l < dst_levels; l++) {
            const VkBufferImageCopy bc = level_copy(dp, sp.bytes, l);
            f.vkCmdCopyBufferToImage(cmd, staging.buffer, dst_img.image, VK_IMAGE_LAYOUT_TRANSFER_DST_OPTIMAL, 1, &bc);
        }
    barrier();
    for (uint32_t i = 0; i < region_count; i++) {
        const int32_t* g = regions + i * 10;
        VkImageBlit b{};
        b.srcSubresource = {VK_IMAGE_ASPECT_COLOR_BIT, static_cast<uint32_t>(g[0]), 0, 1};
        b.srcOffsets[0] = {g[1], g[2], 0};
        b.srcOffsets[1] = {g[3], g[4], 1};
        b.dstSubresource = {VK_IMAGE_ASPECT_COLOR_BIT, static_cast<uint32_t>(g[5]), 0, 1};
        b.dstOffsets[0] = {g[6], g[7], 0};
        b.dstOffsets[1] = {g[8], g[9], 1};
        f.vkCmdBlitImage(cmd, src_img.image, VK_IMAGE_LAYOUT_TRANSFER_SRC_OPTIMAL, target, VK_IMAGE_LAYOUT_TRANSFER_DST_OPTIMAL, 1, &b,
                         filter ? VK_FILTER_LINEAR : VK_FILTER_NEAREST);
        barrier();
    }
    const uint64_t out_base = dst ? sp.bytes : 0;
    for (uint32_t l = 0; l < target_levels; l++) {
        const VkBufferImageCopy bc = level_copy(tp, out_base, l);
        f.vkCmdCopyImageToBuffer(cmd, target, VK_IMAGE_LAYOUT_TRANSFER_SRC_OPTIMAL, staging.buffer, 1, &bc);
    }
    f.vkEndCommandBuffer(cmd);
    VkSubmitInfo si{};
    si.sType = VK_STRUCTURE_TYPE_SUBMIT_INFO;
    si.commandBufferCount = 1;
    si.pCommandBuffers = &cmd;
    VkResult res = f.vkQueueSubmit(c->queue, 1, &si, fence);
    if (res == VK_SUCCESS) res = f.vkWaitForFences(c->device, 1, &fence, VK_TRUE, ~0ull);
    if (res != VK_SUCCESS) return fail("blit: submit", res);
    if (f.vkMapMemory(c->device, staging.memory, 0, VK_WHOLE_SIZE, 0, &map) != VK_SUCCESS) return fail("blit: map", VK_ERROR_MEMORY_MAP_FAILED);
    std::memcpy(dst ? dst : src, static_cast<uint8_t*>(map) + out_base, tp.bytes);
    f.vkUnmapMemory(c->device, staging.memory);
    cleanup();
    return rc;
}

namespace {
// Counting allocator for cpvh_allocator_check: every block carries a
// 16-byte header so that frees can be matched to allocations.
struct CountingAllocator {
    uint64_t allocations = 0, frees = 0, live = 0;
};
void* VKAPI_CALL counting_alloc(void* user, size_t size, size_t align, int) {
    if (align > 16) return nullptr;
    auto* c = static_cast<CountingAllocator*>(user);
    auto* p = static_cast<uint8_t*>(std::malloc(size + 16));
    if (!p) return nullptr;
    std::memcpy(p, &size, sizeof(size));
    c->allocations++;
    c->live++;
    return p + 16;
}
void VKAPI_CALL counting_free(void* user, void* mem) {
    if (!mem) return;
    auto* c = static_cast<CountingAllocator*>(user);
    c->frees++;
    c->live--;
    std::free(static_cast<uint8_t*>(mem) - 16);
}
}  // namespace

int cpvh_allocator_check(cpvh_context* c, uint64_t* objects, uint64_t* allocations, uint64_t* frees) {
    const Fns& f = c->f;
    CountingAllocator counts;
    VkAllocationCallbacks cb{};
    cb.pUserData = &counts;
    cb.pfnAllocation = counting_alloc;
    cb.pfnFree = counting_free;
    const VkAllocationCallbacks* a = &cb;
    uint64_t n = 0;
    VkResult r = VK_SUCCESS;
    auto ok = [&](VkResult x) {
        if (x != VK_SUCCESS && r == VK_SUCCESS) r = x;
        if (x == VK_SUCCESS) n++;
        return x == VK_SUCCESS;
    };
    VkBufferCreateInfo bi{};
    bi.sType = VK_STRUCTURE_TYPE_BUFFER_CREATE_INFO;
    bi.size = 4096;
    bi.usage = VK_BUFFER_USAGE_TRANSFER_SRC_BIT;
    VkBuffer buffer = nullptr;
    if (ok(f.vkCreateBuffer(c->device, &bi, a, &buffer))) f.vkDestroyBuffer(c->device, buffer, a);
    VkMemoryAllocateInfo ai{};
    ai.sType = VK_STRUCTURE_TYPE_MEMORY_ALLOCATE_INFO;
    ai.allocationSize = 4096;
    ai.memoryTypeIndex = find_memory_type(c, ~0u, true);
    VkDeviceMemory memory = nullptr;
    if (ok(f.vkAllocateMemory(c->device, &ai, a, &memory))) f.vkFreeMemory(c->device, memory, a);
    VkImageCreateInfo ii{};
    ii.sType = VK_STRUCTURE_TYPE_IMAGE_CREATE_INFO;
    ii.imageType = VK_IMAGE_TYPE_2D;
    ii.format = VK_FORMAT_R8G8B8A8_UNORM;
    ii.extent = {16, 16, 1};
    ii.mipLevels = 1;
    ii.arrayLayers = 1;
    ii.samples = VK_SAMPLE_COUNT_1_BIT;
    ii.usage = VK_IMAGE_USAGE_COLOR_ATTACHMENT_BIT;
    VkImage image = nullptr;
    if (ok(f.vkCreateImage(c->device, &ii, a, &image))) {
        VkImageViewCreateInfo vi{};
        vi.sType = VK_STRUCTURE_TYPE_IMAGE_VIEW_CREATE_INFO;
        vi.image = image;
        vi.viewType = VK_IMAGE_VIEW_TYPE_2D;
        vi.format = ii.format;
        vi.subresourceRange = {VK_IMAGE_ASPECT_COLOR_BIT, 0, 1, 0, 1};
        VkImageView view = nullptr;
        if (ok(f.vkCreateImageView(c->device, &vi, a, &view))) {
            VkAttachmentDescription att{};
            att.format = ii.format;
            att.samples = VK_SAMPLE_COUNT_1_BIT;
            VkAttachmentReference ref{0, VK_IMAGE_LAYOUT_COLOR_ATTACHMENT_OPTIMAL};
            VkSubpassDescription sub{};
            sub.colorAttachmentCount = 1;
            sub.pColorAttachments = &ref;
            VkRenderPassCreateInfo rpi{};
            rpi.sType = VK_STRUCTURE_TYPE_RENDER_PASS_CREATE_INFO;
            rpi.attachmentCount = 1;
            rpi.pAttachments = &att;
            rpi.subpassCount = 1;
            rpi.pSubpasses = &sub;
            VkRenderPass pass = nullptr;
            if (ok(f.vkCreateRenderPass(c->device, &rpi, a, &pass))) {
                VkFramebufferCreateInfo fbi{};
                fbi.sType = VK_STRUCTURE_TYPE_FRAMEBUFFER_CREATE_INFO;
                fbi.renderPass = pass;
                fbi.attachmentCount = 1;
                fbi.pAttachments = &view;
                fbi.width = fbi.height = 16;
                fbi.layers = 1;
                VkFramebuffer fb = nullptr;
                if (ok(f.vkCreateFramebuffer(c->device, &fbi, a, &fb))) f.vkDestroyFramebuffer(c->device, fb, a);
                f.vkDestroyRenderPass(c->device, pass, a);
            }
            f.vkDestroyImageView(c->device, view, a);
        }
        f.vkDestroyImage(c->device, image, a);
    }
    VkSamplerCreateInfo si{};
    si.sType = VK_STRUCTURE_TYPE_SAMPLER_CREATE_INFO;
    VkSampler sampler = nullptr;
    if (ok(f.vkCreateSampler(c->device, &si, a, &sampler))) f.vkDestroySampler(c->device, sampler, a);
    VkPipelineCacheCreateInfo pci{};
    pci.sType = VK_STRUCTURE_TYPE_PIPELINE_CACHE_CREATE_INFO;
    VkPipelineCache cache = nullptr;
    if (ok(f.vkCreatePipelineCache(c->device, &pci, a, &cache))) f.vkDestroyPipelineCache(c->device, cache, a);
    VkDescriptorSetLayoutCreateInfo dli{};
    dli.sType = VK_STRUCTURE_TYPE_DESCRIPTOR_SET_LAYOUT_CREATE_INFO;
    VkDescriptorSetLayout dsl = nullptr;
    if (ok(f.vkCreateDescriptorSetLayout(c->device, &dli, a, &dsl))) {
        VkPipelineLayoutCreateInfo pli{};
        pli.sType = VK_STRUCTURE_TYPE_PIPELINE_LAYOUT_CREATE_INFO;
        pli.setLayoutCount = 1;
        pli.pSetLayouts = &dsl;
        VkPipelineLayout layout = nullptr;
        if (ok(f.vkCreatePipelineLayout(c->device, &pli, a, &layout))) f.vkDestroyPipelineLayout(c->device, layout, a);
        f.vkDestroyDescriptorSetLayout(c->device, dsl, a);
    }
    VkDescriptorPoolCreateInfo dpi{};
    dpi.sType = VK_STRUCTURE_TYPE_DESCRIPTOR_POOL_CREATE_INFO;
    dpi.maxSets = 1;
    VkDescriptorPool dpool = nullptr;
    if (ok(f.vkCreateDescriptorPool(c->device, &dpi, a, &dpool))) f.vkDestroyDescriptorPool(c->device, dpool, a);
    VkCommandPoolCreateInfo cpi{};
    cpi.sType = VK_STRUCTURE_TYPE_COMMAND_POOL_CREATE_INFO;
    VkCommandPool cpool = nullptr;
    if (ok(f.vkCreateCommandPool(c->device, &cpi, a, &cpool))) f.vkDestroyCommandPool(c->device, cpool, a);
    VkFenceCreateInfo fci{};
    fci.sType = VK_STRUCTURE_TYPE_FENCE_CREATE_INFO;
    VkFence fence = nullptr;
    if (ok(f.vkCreateFence(c->device, &fci, a, &fence))) f.vkDestroyFence(c->device, fence, a);
    *objects = n;
    *allocations = counts.allocations;
    *frees = counts.frees;
    return r;
}

int cpvh_image_ops(cpvh_context* c, uint32_t format, uint32_t width, uint32_t height, uint32_t levels, const uint8_t* init0, const uint8_t* init1,
                   const cpvh_image_op* ops, uint32_t op_count, uint8_t* out, char* err, uint32_t err_len) {
    const Fns& f = c->f;
    const bool depth = depth_texel_size(format) != 0;
    const uint32_t texel = depth ? depth_texel_size(format) : colour_texel_size(format);
    const VkImageAspectFlags view_aspect = depth ? (format == VK_FORMAT_D32_SFLOAT_S8_UINT ? VK_IMAGE_ASPECT_DEPTH_BIT | VK_IMAGE_ASPECT_STENCIL_BIT
                                                                                             : VK_IMAGE_ASPECT_DEPTH_BIT)
                                                 : VK_IMAGE_ASPECT_COLOR_BIT;
    uint64_t offset[16] = {}, bytes = 0;
    uint32_t lw[16] = {}, lh[16] = {};
    ImageAlloc img[2];
    BufferAlloc staging;
    std::vector<VkImageView> views;
    std::vector<VkFramebuffer> fbs;
    VkRenderPass pass = nullptr;
    VkCommandPool pool = nullptr;
    VkFence fence = nullptr;
    auto cleanup = [&]() {
        if (fence) f.vkDestroyFence(c->device, fence, nullptr);
        if (pool) f.vkDestroyCommandPool(c->device, pool, nullptr);
        for (VkFramebuffer fb : fbs) f.vkDestroyFramebuffer(c->device, fb, nullptr);
        for (VkImageView v : views) f.vkDestroyImageView(c->device, v, nullptr);
        if (pass) f.vkDestroyRenderPass(c->device, pass, nullptr);
        destroy_buffer(c, staging);
        destroy_image(c, img[1]);
        destroy_image(c, img[0]);
    };
    auto fail = [&](const std::string& e, int code) {
        g_err = e + " " + icd_error(c);
        if (err && err_len) std::snprintf(err, err_len, "%s", g_err.c_str());
        cleanup();
        return code;
    };
    if (!init0 || !out || levels == 0 || levels > 16 || width == 0 || height == 0) return fail("image_ops: bad image description", VK_ERROR_INITIALIZATION_FAILED);
    for (uint32_t l = 0, w = width, h = height; l < levels; l++) {
        offset[l] = bytes;
        lw[l] = w;
        lh[l] = h;
        bytes += static_cast<uint64_t>(w) * h * texel;
        w = w > 1 ? w / 2 : 1;
        h = h > 1 ? h / 2 : 1;
    }
    const VkImageUsageFlags usage = VK_IMAGE_USAGE_TRANSFER_SRC_BIT | VK_IMAGE_USAGE_TRANSFER_DST_BIT |
                                    (depth ? VK_IMAGE_USAGE_DEPTH_STENCIL_ATTACHMENT_BIT : VK_IMAGE_USAGE_COLOR_ATTACHMENT_BIT);
    for (int k = 0; k < 2; k++)
        if (make_image(c, static_cast<VkFormat>(format), width, height, levels, usage, view_aspect, img[k]) != VK_SUCCESS)
            return fail("image_ops: image", VK_ERROR_OUT_OF_DEVICE_MEMORY);
    if (make_buffer(c, 2 * bytes, VK_BUFFER_USAGE_TRANSFER_SRC_BIT | VK_BUFFER_USAGE_TRANSFER_DST_BIT, true, staging) != VK_SUCCESS)
        return fail("image_ops: staging buffer", VK_ERROR_OUT_OF_DEVICE_MEMORY);
    void* map = nullptr;
    if (f.vkMapMemory(c->device, staging.memory, 0, VK_WHOLE_SIZE, 0, &map) != VK_SUCCESS) return fail("image_ops: map", VK_ERROR_MEMORY_MAP_FAILED);
    std::memcpy(map, init0, bytes);
    if (init1) std::memcpy(static_cast<uint8_t*>(map) + bytes, init1, bytes);
    else std::memset(static_cast<uint8_t*>(map) + bytes, 0, bytes);
    f.vkUnmapMemory(c->device, staging.memory);

    // a LOAD / STORE render pass over one attachment, for vkCmdClearAttachments
    VkAttachmentDescription att{};
    att.format = static_cast<VkFormat>(format);
    att.samples = VK_SAMPLE_COUNT_1_BIT;
    att.loadOp = VK_ATTACHMENT_LOAD_OP_LOAD;
    att.storeOp = VK_ATTACHMENT_STORE_OP_STORE;
    att.stencilLoadOp = VK_ATTACHMENT_LOAD_OP_LOAD;
    att.stencilStoreOp = VK_ATTACHMENT_STORE_OP_STORE;
    att.finalLayout = VK_IMAGE_LAYOUT_TRANSFER_SRC_OPTIMAL;
    VkAttachmentReference ref{0, depth ? VK_IMAGE_LAYOUT_DEPTH_STENCIL_ATTACHMENT_OPTIMAL : VK_IMAGE_LAYOUT_COLOR_ATTACHMENT_OPTIMAL};
    VkSubpassDescription sub{};
    sub.colorAttachmentCount = depth ? 0 : 1;
    sub.pColorAttachments = depth ? nullptr : &ref;
    sub.pDepthStencilAttachment = depth ? &ref : nullptr;
    VkRenderPassCreateInfo rpi{};
    rpi.sType = VK_STRUCTURE_TYPE_RENDER_PASS_CREATE_INFO;
    rpi.attachmentCount = 1;
    rpi.pAttachments = &att;
    rpi.subpassCount = 1;
    rpi.pSubpasses = &sub;
    if (f.vkCreateRenderPass(c->device, &rpi, nullptr, &pass) != VK_SUCCESS) return fail("image_ops: render pass", VK_ERROR_INITIALIZATION_FAILED);

    VkCommandPoolCreateInfo cpi{};
    cpi.sType = VK_STRUCTURE_TYPE_COMMAND_POOL_CREATE_INFO;
    if (f.vkCreateCommandPool(c->device, &cpi, nullptr, &pool) != VK_SUCCESS) return fail("image_ops: command pool", VK_ERROR_INITIALIZATION_FAILED);
    VkCommandBufferAllocateInfo cai{};
    cai.sType = VK_STRUCTURE_TYPE_COMMAND_BUFFER_ALLOCATE_INFO;
    cai.commandPool = pool;
    cai.level = VK_COMMAND_BUFFER_LEVEL_PRIMARY;
    cai.commandBufferCount = 1;
    VkCommandBuffer cmd = nullptr;
    if (f.vkAllocateCommandBuffers(c->device, &cai, &cmd) != VK_SUCCESS || !check_dispatch(cmd))
        return fail("image_ops: command buffer", VK_ERROR_INITIALIZATION_FAILED);
    VkFenceCreateInfo fci{};
    fci.sType = VK_STRUCTURE_TYPE_FENCE_CREATE_INFO;
    if (f.vkCreateFence(c->device, &fci, nullptr, &fence) != VK_SUCCESS) return fail("image_ops: fence", VK_ERROR_INITIALIZATION_FAILED);

    VkMemoryBarrier mb{};
    mb.sType = VK_STRUCTURE_TYPE_MEMORY_BARRIER;
    mb.srcAccessMask = VK_ACCESS_TRANSFER_WRITE_BIT;
    mb.dstAccessMask = VK_ACCESS_TRANSFER_READ_BIT | VK_ACCESS_TRANSFER_WRITE_BIT;
    auto barrier = [&]() { f.vkCmdPipelineBarrier(cmd, VK_PIPELINE_STAGE_ALL_COMMANDS_BIT, VK_PIPELINE_STAGE_ALL_COMMANDS_BIT, 0, 1, &mb, 0, nullptr, 0, nullptr); };
    auto level_copy = [&](uint64_t base, uint32_t l) {
        VkBufferImageCopy bc{};
        bc.bufferOffset = base + offset[l];
        bc.imageSubresource = {view_aspect, l, 0, 1};
        bc.imageExtent = {lw[l], lh[l], 1};
        return bc;
    };
    VkCommandBufferBeginInfo bi{};
    bi.sType = VK_STRUCTURE_TYPE_COMMAND_BUFFER_BEGIN_INFO;
    f.vkBeginCommandBuffer(cmd, &bi);
    for (int k = 0; k < 2; k++)
        for (uint32_t l = 0; l < levels; l++) {
            const VkBufferImageCopy bc = level_copy(k * bytes, l);
            f.vkCmdCopyBufferToImage(cmd, staging.buffer, img[k].image, VK_IMAGE_LAYOUT_TRANSFER_DST_OPTIMAL, 1, &bc);
        }
    barrier();
    for (uint32_t i = 0; i < op_count; i++) {
        const cpvh_image_op& op = ops[i];
        const VkImageSubresourceRange range{op.aspect, op.level, op.level_count, 0, 1};
        switch (op.kind) {
        case CPVH_OP_CLEAR_COLOR_IMAGE: {
            VkClearColorValue v;
            std::memcpy(v.float32, op.colour, sizeof(v.float32));
            f.vkCmdClearColorImage(cmd, img[0].image, VK_IMAGE_LAYOUT_TRANSFER_DST_OPTIMAL, &v, 1, &range);
            break;
        }
        case CPVH_OP_CLEAR_DEPTH_STENCIL_IMAGE: {
            const VkClearDepthStencilValue v{op.depth, op.stencil};
            f.vkCmdClearDepthStencilImage(cmd, img[0].image, VK_IMAGE_LAYOUT_TRANSFER_DST_OPTIMAL, &v, 1, &range);
            break;
        }
        case CPVH_OP_COPY_IMAGE: {
            VkImageCopy rc{};
            rc.srcSubresource = {view_aspect, op.src_level, 0, 1};
            rc.srcOffset = {op.src_x, op.src_y, 0};
            rc.dstSubresource = {view_aspect, op.level, 0, 1};
            rc.dstOffset = {op.x, op.y, 0};
            rc.extent = {op.w, op.h, 1};
            f.vkCmdCopyImage(cmd, img[1].image, VK_IMAGE_LAYOUT_TRANSFER_SRC_OPTIMAL, img[0].image, VK_IMAGE_LAYOUT_TRANSFER_DST_OPTIMAL, 1, &rc);
            break;
        }
        case CPVH_OP_CLEAR_ATTACHMENTS: {
            if (op.level >= levels) return fail("image_ops: level", VK_ERROR_INITIALIZATION_FAILED);
            VkImageViewCreateInfo vi{};
            vi.sType = VK_STRUCTURE_TYPE_IMAGE_VIEW_CREATE_INFO;
            vi.image = img[0].image;
            vi.viewType = VK_IMAGE_VIEW_TYPE_2D;
            vi.format = static_cast<VkFormat>(format);
            vi.subresourceRange = {view_aspect, op.level, 1, 0, 1};
            VkImageView view = nullptr;
            if (f.vkCreateImageView(c->device, &vi, nullptr, &view) != VK_SUCCESS) return fail("image_ops: view", VK_ERROR_INITIALIZATION_FAILED);
            views.push_back(view);
            VkFramebufferCreateInfo fbi{};
            fbi.sType = VK_STRUCTURE_TYPE_FRAMEBUFFER_CREATE_INFO;
            fbi.renderPass = pass;
            fbi.attachmentCount = 1;
            fbi.pAttachments = &view;
            fbi.width = lw[op.level];
            fbi.height = lh[op.level];
            fbi.layers = 1;
            VkFramebuffer fb = nullptr;
            if (f.vkCreateFramebuffer(c->device, &fbi, nullptr, &fb) != VK_SUCCESS) return fail("image_ops: framebuffer", VK_ERROR_INITIALIZATION_FAILED);
            fbs.push_back(fb);
            VkRenderPassBeginInfo rb{};
            rb.sType = VK_STRUCTURE_TYPE_RENDER_PASS_BEGIN_INFO;
            rb.renderPass = pass;
            rb.framebuffer = fb;
            rb.renderArea = {{0, 0}, {lw[op.level], lh[op.level]}};
            f.vkCmdBeginRenderPass(cmd, &rb, VK_SUBPASS_CONTENTS_INLINE);
            VkClearAttachment ca{};
            ca.aspectMask = op.aspect;
            ca.colorAttachment = 0;
            if (depth) ca.clearValue.depthStencil = {op.depth, op.stencil};
            else std::memcpy(ca.clearValue.color.float32, op.colour, sizeof(op.colour));
            const VkClearRect rect{{{op.x, op.y}, {op.w, op.h}}, 0, 1};
            f.vkCmdClearAttachments(cmd, 1, &ca, 1, &rect);
            f.vkCmdEndRenderPass(cmd);
            break;
        }
        default: return fail("image_ops: unknown operation", VK_ERROR_INITIALIZATION_FAILED);
        }
        barrier();
    }
    for (uint32_t l = 0; l < levels; l++) {
        const VkBufferImageCopy bc = level_copy(0, l);
        f.vkCmdCopyImageToBuffer(cmd, img[0].image, VK_IMAGE_LAYOUT_TRANSFER_SRC_OPTIMAL, staging.buffer, 1, &bc);
    }
    f.vkEndCommandBuffer(cmd);
    VkSubmitInfo si{};
    si.sType = VK_STRUCTURE_TYPE_SUBMIT_INFO;
    si.commandBufferCount = 1;
    si.pCommandBuffers = &cmd;
    VkResult res = f.vkQueueSubmit(c->queue, 1, &si, fence);
    if (res == VK_SUCCESS) res = f.vkWaitForFences(c->device, 1, &fence, VK_TRUE, ~0ull);
    if (res != VK_SUCCESS) return fail("image_ops: submit", res);
    if (f.vkMapMemory(c->device, staging.memory, 0, VK_WHOLE_SIZE, 0, &map) != VK_SUCCESS) return fail("image_ops: map", VK_ERROR_MEMORY_MAP_FAILED);
    std::memcpy(out, map, bytes);
    f.vkUnmapMemory(c->device, staging.memory);
    cleanup();
    return VK_SUCCESS;
}

}  // extern "C"

// ------------------------------------------------------------ serving loop --
//
// Continuous batching of offscreen clients: every client owns a scene, its
// pipelines, buffers and attachments; requests arrive with Poisson
// inter-arrival times per client; the loop admits a waiting request whenever
// a slot (a queue) is free and its client has no request in flight, and
// retires requests as their fences signal. Work on different queues overlaps
// on the device. Residency is by HBM footprint: clients are made resident at
// creation while they fit the budget; a request of a client that is not
// resident is admitted by making it resident, evicting idle resident clients
// (least recently used first) until it fits.

struct cpvh_server {
    cpvh_context* ctx = nullptr;
    cpvh_serve_config cfg{};
    std::vector<cpv_scene*> scenes;
    std::vector<cpvh_renderer*> clients;  // null: not resident
    std::vector<uint64_t> footprint;
    std::vector<uint64_t> triangles;
    std::vector<uint64_t> last_use;       // admission counter value of the client's last request
    uint64_t resident_bytes = 0;
};

namespace {

uint64_t splitmix(uint64_t& s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

double uniform01(uint64_t& s) { return static_cast<double>(splitmix(s) >> 11) * (1.0 / 9007199254740992.0); }

double percentile(std::vector<double> v, double p) {
    if (v.empty()) return 0.0;
    std::sort(v.begin(), v.end());
    const double pos = p * static_cast<double>(v.size() - 1);
    const size_t i = static_cast<size_t>(pos);
    const double f = pos - static_cast<double>(i);
    return i + 1 < v.size() ? v[i] * (1.0 - f) + v[i + 1] * f : v[i];
}

}  // namespace

extern "C" {

cpvh_server* cpvh_server_create(cpvh_context* ctx, const cpvh_serve_config* cfg, char* err, uint32_t err_len) {
    auto fail = [&](const std::string& why, cpvh_server* s) -> cpvh_server* {
        g_err = why;
        if (err && err_len) std::snprintf(err, err_len, "%s", why.c_str());
        cpvh_server_destroy(s);
        return nullptr;
    };
    if (!ctx || !cfg || cfg->clients == 0 || cfg->min_tris == 0 || cfg->max_tris < cfg->min_tris) return fail("bad serving configuration", nullptr);
    auto* s = new cpvh_server();
    s->ctx = ctx;
    s->cfg = *cfg;
    if (s->cfg.slots == 0) s->cfg.slots = 1;
    uint64_t rng = cfg->seed * 0x2545F4914F6CDD1Dull + 7;
    static const uint64_t sides[4] = {256, 512, 1024, 2048};
    for (uint32_t i = 0; i < cfg->clients; i++) {
        // Image side uniform over {256, 512, 1024, 2048}; triangles
        // log-uniform in [min_tris, max_tris].
        const uint64_t side = cfg->max_side ? std::min<uint64_t>(sides[splitmix(rng) & 3u], cfg->max_side) : sides[splitmix(rng) & 3u];
        const double lt = std::log(static_cast<double>(cfg->min_tris)) +
                          uniform01(rng) * (std::log(static_cast<double>(cfg->max_tris)) - std::log(static_cast<double>(cfg->min_tris)));
        const uint64_t params[3] = {side, static_cast<uint64_t>(std::llround(std::exp(lt))), i};
        cpv_scene* scene = cpvh_scene_create(CPVH_SERVE, cfg->seed + i, params, 3);
        if (!scene) return fail("client scene creation failed", s);
        s->scenes.push_back(scene);
        const uint64_t px = static_cast<uint64_t>(scene->width) * scene->height;
        const uint64_t bytes = px * (4 + depth_texel_size(scene->depth_format)) * 2 /* attachments + readback */ +
                               2 * (scene->vertex_bytes + scene->index_bytes + scene->uniform_bytes) /* buffers + staging */ + scene->texture_bytes;
        s->footprint.push_back(bytes);
        s->triangles.push_back(cpvh_scene_triangles(scene));
        s->last_use.push_back(0);
        cpvh_renderer* r = nullptr;
        if (s->resident_bytes + bytes <= cfg->hbm_budget_bytes) {
            char e[512] = {0};
            r = cpvh_renderer_create(ctx, scene, e, sizeof(e));
            if (!r) return fail(std::string("client renderer creation failed: ") + e, s);
            s->resident_bytes += bytes;
        }
        s->clients.push_back(r);
    }
    return s;
}

void cpvh_server_set_load(cpvh_server* s, double mean_interarrival_ms, double duration_s) {
    if (!s) return;
    s->cfg.mean_interarrival_ms = mean_interarrival_ms;
    s->cfg.duration_s = duration_s;
}

int cpvh_server_run(cpvh_server* s, cpvh_serve_result* out) {
    cpvh_context* c = s->ctx;
    const cpvh_serve_config& cfg = s->cfg;
    struct Request {
        double arrival_ms;
        uint32_t client;
    };
    // Poisson arrivals per client over the window, merged in time order.
    // Without admission on demand, clients that are not resident send none.
    std::vector<Request> arrivals;
    uint64_t rng = cfg.seed * 0x9E3779B97F4A7C15ull + 11;
    for (uint32_t i = 0; i < cfg.clients; i++) {
        if (!s->clients[i] && !cfg.admit_on_demand) continue;
        if (s->footprint[i] > cfg.hbm_budget_bytes) continue;  // can never be resident
        double t = 0.0;
        for (;;) {
            t += -std::log(1.0 - uniform01(rng)) * cfg.mean_interarrival_ms;
            if (t >= cfg.duration_s * 1000.0) break;
            arrivals.push_back({t, i});
        }
    }
    std::sort(arrivals.begin(), arrivals.end(), [](const Request& a, const Request& b) { return a.arrival_ms < b.arrival_ms; });
    const uint32_t slots = std::min<uint32_t>(cfg.slots, static_cast<uint32_t>(c->queues.size()));
    // Warm-up (untimed): the largest resident client once on every queue,
    // so that each queue's binning scratch has grown before the clock starts.
    {
        int big = -1;
        for (uint32_t i = 0; i < cfg.clients; i++)
            if (s->clients[i] && (big < 0 || s->triangles[i] > s->triangles[static_cast<uint32_t>(big)])) big = static_cast<int>(i);
        if (big >= 0) {
            cpvh_renderer* r = s->clients[static_cast<uint32_t>(big)];
            VkSubmitInfo si{};
            si.sType = VK_STRUCTURE_TYPE_SUBMIT_INFO;
            si.commandBufferCount = 1;
            si.pCommandBuffers = &r->frame_cmd;
            for (uint32_t k = 0; k < slots; k++) {
                VkResult res = c->f.vkQueueSubmit(c->queues[k], 1, &si, r->fence);
                if (res == VK_SUCCESS) res = c->f.vkWaitForFences(c->device, 1, &r->fence, VK_TRUE, ~0ull);
                c->f.vkResetFences(c->device, 1, &r->fence);
                if (res != VK_SUCCESS) return res;
            }
        }
    }
    struct Slot {
        bool busy = false;
        uint32_t client = 0;
        double arrival_ms = 0.0, submit_ms = 0.0;
    };
    std::vector<Slot> slot(slots);
    std::vector<std::deque<double>> waiting(cfg.clients);  // arrival times per client
    std::vector<bool> in_flight(cfg.clients, false);
    std::vector<double> latency, submit_latency, queue_delay, residency_ms;
    latency.reserve(arrivals.size());
    uint64_t triangles = 0, uses = 0, evictions = 0;
    uint32_t max_in_flight = 0, busy = 0;
    size_t next = 0, done = 0;
    const auto t0 = std::chrono::steady_clock::now();
    auto now_ms = [&]() { return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count(); };
    double last_done = 0.0;
    // Makes client i resident: evicts idle resident clients, least recently
    // used first, until it fits the budget. False when the clients holding
    // the budget are all busy (the request waits for one to retire).
    auto make_resident = [&](uint32_t i, VkResult& res) {
        res = VK_SUCCESS;
        if (s->clients[i]) return true;
        uint64_t idle_bytes = 0;
        for (uint32_t j = 0; j < cfg.clients; j++)
            if (s->clients[j] && !in_flight[j]) idle_bytes += s->footprint[j];
        if (s->resident_bytes - idle_bytes + s->footprint[i] > cfg.hbm_budget_bytes) return false;
        while (s->resident_bytes + s->footprint[i] > cfg.hbm_budget_bytes) {
            int victim = -1;
            for (uint32_t j = 0; j < cfg.clients; j++)
                if (s->clients[j] && !in_flight[j] && (victim < 0 || s->last_use[j] < s->last_use[static_cast<uint32_t>(victim)])) victim = static_cast<int>(j);
            if (victim < 0) return false;
            renderer_destroy(s->clients[static_cast<uint32_t>(victim)], false);  // idle: its last fence has signalled
            s->clients[static_cast<uint32_t>(victim)] = nullptr;
            s->resident_bytes -= s->footprint[static_cast<uint32_t>(victim)];
            evictions++;
        }
        const double t = now_ms();
        char e[512] = {0};
        s->clients[i] = cpvh_renderer_create(c, s->scenes[i], e, sizeof(e));
        if (!s->clients[i]) {
            g_err = std::string("client residency: ") + e;
            res = VK_ERROR_OUT_OF_DEVICE_MEMORY;
            return false;
        }
        s->resident_bytes += s->footprint[i];
        residency_ms.push_back(now_ms() - t);
        return true;
    };
    std::vector<VkFence> pending;
    while (done < arrivals.size()) {
        const double now = now_ms();
        while (next < arrivals.size() && arrivals[next].arrival_ms <= now) {
            waiting[arrivals[next].client].push_back(arrivals[next].arrival_ms);
            next++;
        }
        // Retire finished requests.
        for (uint32_t k = 0; k < slots; k++) {
            if (!slot[k].busy) continue;
            cpvh_renderer* r = s->clients[slot[k].client];
            const VkResult st = c->f.vkGetFenceStatus(c->device, r->fence);
            if (st == VK_NOT_READY) continue;
            if (st != VK_SUCCESS) return st;
            const double t = now_ms();
            c->f.vkResetFences(c->device, 1, &r->fence);
            latency.push_back(t - slot[k].arrival_ms);
            submit_latency.push_back(t - slot[k].submit_ms);
            triangles += s->triangles[slot[k].client];
            in_flight[slot[k].client] = false;
            slot[k].busy = false;
            busy--;
            done++;
            last_done = t;
        }
        // Admit: the oldest waiting request whose client is idle (and
        // resident, or can be made resident), while a slot is free.
        bool admitted = false;
        for (uint32_t k = 0; k < slots; k++) {
            if (slot[k].busy) continue;
            int best = -1;
            for (uint32_t i = 0; i < cfg.clients; i++) {
                if (waiting[i].empty() || in_flight[i]) continue;
                if (best < 0 || waiting[i].front() < waiting[static_cast<uint32_t>(best)].front()) best = static_cast<int>(i);
            }
            if (best < 0) break;
            const uint32_t i = static_cast<uint32_t>(best);
            VkResult res;
            if (!make_resident(i, res)) {
                if (res != VK_SUCCESS) return res;
                break;  // the budget is held by busy clients: wait for a retirement
            }
            cpvh_renderer* r = s->clients[i];
            VkSubmitInfo si{};
            si.sType = VK_STRUCTURE_TYPE_SUBMIT_INFO;
            si.commandBufferCount = 1;
            si.pCommandBuffers = &r->frame_cmd;
            slot[k].submit_ms = now_ms();
            res = c->f.vkQueueSubmit(c->queues[k], 1, &si, r->fence);
            if (res != VK_SUCCESS) return res;
            slot[k].busy = true;
            slot[k].client = i;
            slot[k].arrival_ms = waiting[i].front();
            queue_delay.push_back(slot[k].submit_ms - slot[k].arrival_ms);
            waiting[i].pop_front();
            in_flight[i] = true;
            s->last_use[i] = ++uses;
            busy++;
            max_in_flight = std::max(max_in_flight, busy);
            admitted = true;
        }
        if (admitted) continue;
        // Nothing to admit: wait for a retirement or the next arrival,
        // whichever comes first, instead of polling.
        const double until = next < arrivals.size() ? arrivals[next].arrival_ms - now_ms() : 1.0;
        if (until <= 0.0) continue;
        const uint64_t timeout_ns = static_cast<uint64_t>(std::min(until, 1.0) * 1e6);
        pending.clear();
        for (uint32_t k = 0; k < slots; k++)
            if (slot[k].busy) pending.push_back(s->clients[slot[k].client]->fence);
        if (!pending.empty()) {
            const VkResult w = c->f.vkWaitForFences(c->device, static_cast<uint32_t>(pending.size()), pending.data(), VK_FALSE, timeout_ns);
            if (w != VK_SUCCESS && w != VK_TIMEOUT) return w;
        } else {
            std::this_thread::sleep_for(std::chrono::nanoseconds(timeout_ns));
        }
    }
    c->f.vkDeviceWaitIdle(c->device);
    if (out) {
        std::memset(out, 0, sizeof(*out));
        out->requests = arrivals.size();
        out->completed = done;
        out->triangles = triangles;
        out->wall_s = last_done / 1000.0;
        out->mtri_s = last_done > 0.0 ? static_cast<double>(triangles) / (last_done / 1000.0) / 1e6 : 0.0;
        out->latency_p50_ms = percentile(latency, 0.50);
        out->latency_p99_ms = percentile(latency, 0.99);
        out->submit_p50_ms = percentile(submit_latency, 0.50);
        out->submit_p99_ms = percentile(submit_latency, 0.99);
        out->queue_p50_ms = percentile(queue_delay, 0.50);
        out->queue_p99_ms = percentile(queue_delay, 0.99);
        out->max_in_flight = max_in_flight;
        out->resident_bytes = s->resident_bytes;
        uint32_t resident = 0;
        for (auto* r : s->clients) resident += r ? 1u : 0u;
        out->resident_clients = resident;
        out->residencies = residency_ms.size();
        out->evictions = evictions;
        out->residency_p50_ms = percentile(residency_ms, 0.50);
        out->residency_p99_ms = percentile(residency_ms, 0.99);
    }
    return VK_SUCCESS;
}

uint32_t cpvh_server_clients(const cpvh_server* s) { return s ? static_cast<uint32_t>(s->clients.size()) : 0u; }

cpvh_renderer* cpvh_server_client(cpvh_server* s, uint32_t i) { return s && i < s->clients.size() ? s->clients[i] : nullptr; }

const cpv_scene* cpvh_server_scene(cpvh_server* s, uint32_t i) { return s && i < s->scenes.size() ? s->scenes[i] : nullptr; }

void cpvh_server_destroy(cpvh_server* s) {
    if (!s) return;
    for (auto* r : s->clients)
        if (r) cpvh_renderer_destroy(r);
    for (auto* sc : s->scenes) cpvh_scene_destroy(sc);
    delete s;
}

}  // extern "C"
