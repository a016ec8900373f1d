// icd.h — object model of the cpvulkan_gb300 Vulkan ICD.
//
// Mirrors the reference ICD's objects (CPVulkan/Instance.h, Device.h,
// Buffer.h, Image.h, Pipeline.h, CommandBuffer.h, Queue.h ...) with GB300
// storage: VkDeviceMemory is a cudaMalloc allocation in HBM (plus a pinned
// host mirror for host-visible memory types), buffers and images are
// sub-ranges of it, and a queue is a CUDA stream.
#pragma once

#include <cuda_runtime.h>

#include <array>
#include <atomic>
#include <cstdint>
#include <map>
#include <memory>
#include <mutex>
#include <set>
#include <string>
#include <vector>

#include "../../../include/cpv/vk_subset.h"
#include "../runtime/runtime.h"
#include "../spirv/spirv.h"

namespace cpv::icd {

// Dispatchable objects start with the loader's word (ICD_LOADER_MAGIC until
// the loader stores its dispatch table there).
struct Dispatchable {
    uintptr_t loader_data = ICD_LOADER_MAGIC;
};

struct PhysicalDevice;
struct Device;
struct Queue;

struct Instance : Dispatchable {
    PhysicalDevice* physical = nullptr;
    uint32_t api_version = VK_API_VERSION_1_1;
};

struct PhysicalDevice : Dispatchable {
    Instance* instance = nullptr;
};

struct DeviceMemory {
    uint8_t* device = nullptr;     // HBM
    uint8_t* host = nullptr;       // pinned mirror (host-visible types)
    VkDeviceSize size = 0;
    uint32_t type = 0;
    bool mapped = false;
    bool device_dirty = false;     // HBM newer than the mirror
};

struct Buffer {
    VkDeviceSize size = 0;
    VkBufferUsageFlags usage = 0;
    DeviceMemory* memory = nullptr;
    VkDeviceSize offset = 0;
    uint8_t* device_ptr(VkDeviceSize at = 0) const { return memory ? memory->device + offset + at : nullptr; }
};

// Linear image layout of the reference (CPVulkanBase/Formats.cpp:453-484):
// levels concatenated inside each layer, tightly packed rows.
struct ImageLevel {
    uint64_t offset = 0;
    uint32_t width = 0, height = 0, depth = 0;
    uint64_t stride = 0, plane = 0, size = 0;
};

struct Image {
    VkFormat format = VK_FORMAT_UNDEFINED;
    uint32_t texel = 0;
    VkExtent3D extent{};
    uint32_t levels = 1, layers = 1;
    std::vector<ImageLevel> level;
    uint64_t layer_size = 0, total_size = 0;
    DeviceMemory* memory = nullptr;
    VkDeviceSize offset = 0;
    uint8_t* device_ptr() const { return memory ? memory->device + offset : nullptr; }
};

struct ImageView {
    Image* image = nullptr;
    VkFormat format = VK_FORMAT_UNDEFINED;
    VkImageSubresourceRange range{};
    VkComponentMapping components{};
};

struct Sampler {
    VkSamplerCreateInfo info{};
};

struct ShaderModule {
    std::vector<uint32_t> words;
    spirv::Module module;
};

struct DescriptorSetLayout {
    std::vector<VkDescriptorSetLayoutBinding> bindings;
    std::vector<std::vector<Sampler*>> immutable;
};

struct Descriptor {
    VkDescriptorType type = VK_DESCRIPTOR_TYPE_MAX_ENUM;
    Buffer* buffer = nullptr;
    VkDeviceSize offset = 0, range = 0;
    ImageView* view = nullptr;
    Sampler* sampler = nullptr;
};

struct DescriptorSet {
    DescriptorSetLayout* layout = nullptr;
    std::map<uint32_t, std::vector<Descriptor>> bindings;
};

struct DescriptorPool {
    std::set<DescriptorSet*> sets;
};

struct PipelineLayout {
    std::vector<DescriptorSetLayout*> sets;
    std::vector<VkPushConstantRange> push;
};

// The attachments one subpass draws to.
struct Subpass {
    std::vector<uint32_t> colour;     // colour attachment indices by position (VK_ATTACHMENT_UNUSED kept, none trailing)
    uint32_t depth = VK_ATTACHMENT_UNUSED;
};

struct RenderPass {
    std::vector<VkAttachmentDescription> attachments;
    std::vector<Subpass> subpasses;   // at least one
};

struct Framebuffer {
    RenderPass* pass = nullptr;
    std::vector<ImageView*> attachments;
    uint32_t width = 0, height = 0, layers = 1;
};

struct PipelineCache {
    std::mutex mutex;
    std::map<std::array<uint8_t, 32>, std::vector<uint8_t>> entries;  // key → cubin
};

struct Pipeline {
    rt::Module module;
    std::array<uint8_t, 32> key{};
    std::vector<spirv::ResourceSlot> slots;
    VkPrimitiveTopology topology = VK_PRIMITIVE_TOPOLOGY_TRIANGLE_LIST;
    VkViewport viewport{};
    bool dynamic_viewport = false;
    bool dynamic_blend_constants = false;
    float blend_constants[4] = {0, 0, 0, 0};
    PipelineLayout* layout = nullptr;
    uint32_t colour_format = 0, depth_format = 0;
    bool blend = false;
    std::string stage;   // stage block: fixed-function macros + translated shaders (see compose_module)
    std::string stage_after;  // after the stage functions: the colour attachments after the first
    uint32_t nv = 0;     // varying floats
    bool prefers_deferred = false;  // fragment shader samples images or is long
    uint32_t tile_shift = 4;        // screen tile of the pipeline's modules
    bool blend_table = false;       // per-primitive blend tables (constant colour, per-channel blend)
    bool fs_constant = false;       // fragment shader shaded once per primitive
    bool samples = false;           // fragment shader samples images
    std::string source;  // generated CUDA translation unit of the per-draw module
};

// Tunables of a raster module, fixed at NVRTC time.
struct ModuleConfig {
    uint32_t tile_shift = 4;  // 8, 16 or 32 px tiles
    uint32_t schedule = 0;    // fragment schedule: 0 immediate, 1 deferred, 2 sparse
    uint32_t warps = 8;       // warps per tile CTA (capped by the tile's pixels)
    uint32_t batch = 256;     // primitives set up per shared-memory batch (set per schedule by module_config)
    uint32_t depth = 0;       // sparse schedule: fragments a pixel lists per batch (0: 24, or 16 when sampling)
    bool samples = false;     // a fragment shader samples images (register budget of the batched raster)
};

// Fragment schedule of a module whose pipelines prefer (or not) dense
// shading; CPV_SCHEDULE=0/1/2 overrides.
uint32_t schedule_for(bool prefers_deferred, bool fs_constant);
// Module configuration for a tile size and shading preference, with the
// environment's tunables applied.
ModuleConfig module_config(uint32_t tile_shift, bool prefers_deferred, bool fs_constant, bool samples);

// The CUDA translation unit of a module over one pipeline's stage block
// (per-draw kernels) or several (batched kernels, pipeline i in namespace
// cpv_p<i>).
std::string compose_module(const std::vector<std::string>& stages, const std::vector<uint32_t>& nvs, const ModuleConfig& mc, bool batched,
                           const std::vector<std::string>& afters = {});

// ---- command recording ----
enum class CmdType : uint8_t {
    BeginRenderPass, EndRenderPass, BindPipeline, BindVertexBuffers, BindIndexBuffer, BindDescriptorSets, PushConstants,
    SetViewport, SetScissor, SetBlendConstants, Draw, DrawIndexed, DrawIndirect, DrawIndexedIndirect, CopyBuffer,
    CopyBufferToImage, CopyImageToBuffer, FillBuffer, UpdateBuffer, Barrier, BlitImage, CopyImage, ClearImage, ClearAttachments, NextSubpass,
};

struct Cmd {
    CmdType type;
    // generic fields (meaning depends on type)
    uint32_t u[8] = {};
    int32_t i0 = 0;
    uint64_t q[4] = {};
    void* p[4] = {};
    std::vector<uint8_t> bytes;
    std::vector<uint64_t> list;
    std::vector<VkBufferImageCopy> image_regions;
    std::vector<VkBufferCopy> buffer_regions;
    std::vector<VkImageBlit> blit_regions;
    std::vector<VkImageCopy> image_copies;
    std::vector<VkImageSubresourceRange> ranges;
    std::vector<VkClearAttachment> clear_attachments;
    std::vector<VkClearRect> clear_rects;
    std::vector<VkClearValue> clears;
    VkViewport viewport{};
};

// Batched execution state of one render pass of a recorded command buffer
// (built on its first execution, reused until the command buffer is reset).
// One VkDrawIndirectCommand / VkDrawIndexedIndirectCommand as a direct
// draw's arguments.
struct IndirectDraw {
    uint32_t count, instances, first;
    int32_t vertex_offset;
    uint32_t first_instance;
    bool operator==(const IndirectDraw& o) const {
        return count == o.count && instances == o.instances && first == o.first && vertex_offset == o.vertex_offset && first_instance == o.first_instance;
    }
};

// The records of a render pass's indirect draws, by command index.
using PassIndirect = std::vector<std::pair<size_t, std::vector<IndirectDraw>>>;

struct BatchState {
    rt::Module* module = nullptr;  // owned by Device::batch_modules
    std::unique_ptr<rt::BatchPlan> plan;
    bool plain = false;            // not batchable: the per-draw path runs
    PassIndirect indirect;         // the indirect draws' records the batch was built from
};

// A command buffer's work captured as a CUDA graph for one queue (its
// binning scratch is per queue).
struct QueueGraph {
    bool warm = false;               // ran once eagerly on this queue (scratch sized)
    cudaGraphExec_t exec = nullptr;
    uint64_t generation = 0;         // the queue's scratch generation at capture
    uint64_t kernels = 0;
};

struct CommandBuffer : Dispatchable {
    Device* device = nullptr;
    std::vector<Cmd> cmds;
    bool recording = false;
    bool secondary = false;  // VK_COMMAND_BUFFER_LEVEL_SECONDARY: executed through vkCmdExecuteCommands
    std::map<size_t, std::unique_ptr<BatchState>> batches;  // by BeginRenderPass command index
    // Replay as a CUDA graph per queue: decided after the first execution
    // (no host-memory sources, no batched pass).
    int graphable = -1;  // -1 unknown, 0 no, 1 yes
    std::vector<DeviceMemory*> written;  // memories its execution writes
    std::map<Queue*, QueueGraph> graphs;
    void reset();
    ~CommandBuffer() { reset(); }
};

struct CommandPool {
    std::set<CommandBuffer*> buffers;
};

struct Fence {
    cudaEvent_t event = nullptr;
    bool signalled = false;   // created signalled or completed and observed
    bool pending = false;     // a submission will record the event
    std::vector<DeviceMemory*> readback;  // host-visible memories written by the submission
};

struct Semaphore {
    cudaEvent_t event = nullptr;
    bool signalled = false;
};

struct Queue : Dispatchable {
    Device* device = nullptr;
    cudaStream_t stream = nullptr;
    cudaEvent_t timing[16] = {};
    rt::Scratch scratch;
    std::vector<DeviceMemory*> pending_readback;
    std::mutex mutex;
};

// Queues a device may create in its one queue family.
constexpr uint32_t kMaxQueues = 16;

struct Device : Dispatchable {
    PhysicalDevice* physical = nullptr;
    // No CUDA device and CPV_COMPILE_ONLY=1: pipelines are translated and
    // compiled with NVRTC but not loaded; memory is host memory; submissions
    // fail with VK_ERROR_DEVICE_LOST. Used to check pipeline compilation on
    // machines without a GPU.
    bool compile_only = false;
    std::vector<Queue*> queues;  // the queues of the one queue family
    Queue* queue = nullptr;      // queues[0]
    std::mutex cache_mutex;
    std::map<std::array<uint8_t, 32>, std::vector<uint8_t>> module_cache;  // in-process NVRTC cubin cache
    std::set<DeviceMemory*> memories;
    std::mutex memory_mutex;
    // Batched modules by (pipeline keys, module configuration).
    std::mutex batch_mutex;
    std::map<std::string, std::unique_ptr<rt::Module>> batch_modules;
    // Module configuration the tuner chose, by batch signature (pipeline
    // keys, draw and primitive counts, target size); guarded by batch_mutex.
    std::map<std::string, ModuleConfig> tuned;
};

// The batched module over `pipelines` (module pipeline i = pipelines[i]),
// compiled with NVRTC on first use and cached on the device. Null on error
// (message in rt::last_error()).
rt::Module* batch_module(Device* dev, const std::vector<Pipeline*>& pipelines, const ModuleConfig& mc);

// Runs a command buffer on a queue: replays its CUDA graph for that queue
// when it has one, captures one on its second run there, else executes
// eagerly (command.cpp). CPV_CB_GRAPH=0 always executes eagerly.
VkResult run_command_buffer(Queue* q, CommandBuffer* cb, std::vector<DeviceMemory*>& written, bool no_alloc);
// Execution of a recorded command buffer on a queue (command.cpp).
// no_alloc: draws bin through the fixed scratch array (rt::draw_plain_static)
// instead of the queue's grow-only scratch.
VkResult execute(Queue* q, CommandBuffer* cb, std::vector<DeviceMemory*>& written, bool no_alloc = false);
// At vkEndCommandBuffer: compiles (NVRTC) and caches the batched module of
// every render pass that will run batched, so its first submission does not.
void precompile_batches(CommandBuffer* cb);
// Report of the calling thread's last batch tuning: each candidate's
// configuration and time, then the choice ("" when none ran).
const char* last_tuning();
// Checks, before any work is enqueued, that every draw of `cb` fits the fixed
// scratch array (VK_ERROR_OUT_OF_DEVICE_MEMORY and a message otherwise).
VkResult check_no_alloc(Queue* q, CommandBuffer* cb);

// Pipeline creation (pipeline.cpp).
VkResult create_graphics_pipeline(Device* dev, PipelineCache* cache, const VkGraphicsPipelineCreateInfo& info, Pipeline** out);

// SHA3-256 (sha3.cpp), FIPS 202.
std::array<uint8_t, 32> sha3_256(const void* data, size_t size);

// Format helpers.
uint32_t format_texel_size(VkFormat f);
// Layout of a colour attachment format the draw path writes: bytes per
// texel, channels, bits per channel, kind (0 UNORM, 1 SNORM, 2 SFLOAT) and
// red in byte 2 (B8G8R8A8) — from the reference's format table
// (CPVulkanBase/Formats.cpp). False for any other format.
struct ColourLayout {
    uint32_t bytes = 0, channels = 0, bits = 0, kind = 0;
    bool bgra = false;
};
bool colour_layout(VkFormat f, ColourLayout& out);
bool format_is_depth(VkFormat f);
bool format_has_stencil(VkFormat f);
void image_layout(Image& img);

// Host-side encode of clear values with the reference's codecs
// (LLVMRuntime/ImageCompiler.cpp:869-947, 1081-1095).
uint32_t encode_unorm_host(float x, float maxv);

}  // namespace cpv::icd
