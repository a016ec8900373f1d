// pipeline.cpp — vkCreateGraphicsPipelines: state validation, SPIR-V → CUDA
// translation of both stages, the pipeline translation unit, the SHA3 cache
// key, NVRTC compilation for sm_103a and module loading.
//
// Reference counterpart: GraphicsPipeline::Create / Parse
// (CPVulkan/Pipeline.cpp:43-714), CompileBaseShaderModule / CalculateHash
// (:540-597, :735-763), and the pipeline wrappers of
// LLVMRuntime/PipelineCompiler.cpp, which bake the fixed-function state into
// the JIT module exactly as the CPV_* constants below bake it into the
// NVRTC module. Unsupported state is rejected with a VkResult instead of the
// reference's abort.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>

#include "icd.h"

namespace cpv::icd {

namespace {

const char* kTranslationVersion = "cpvulkan_gb300 pipeline v1";

uint32_t tile_shift_for_pipeline() {
    const char* v = std::getenv("CPV_TILE");
    if (!v) return 4;
    const int t = std::atoi(v);
    if (t == 8) return 3;
    if (t == 32) return 5;
    return 4;
}

std::string cache_dir() {
    const char* v = std::getenv("CPV_CACHE_DIR");
    return v ? std::string(v) : std::string();
}

std::string hex(const std::array<uint8_t, 32>& k) {
    static const char* d = "0123456789abcdef";
    std::string s;
    for (uint8_t b : k) {
        s.push_back(d[b >> 4]);
        s.push_back(d[b & 15]);
    }
    return s;
}

bool supported_colour(VkFormat f) {
    ColourLayout cl;
    return colour_layout(f, cl);
}
bool supported_depth(VkFormat f) { return f == VK_FORMAT_D16_UNORM || f == VK_FORMAT_D32_SFLOAT || f == VK_FORMAT_D32_SFLOAT_S8_UINT; }

// Per-pipeline macros of a stage block, undefined after its namespace so the
// next pipeline of a module can define its own.
const char* const kStageMacros[] = {
    "CPV_NV", "CPV_TOPOLOGY", "CPV_CULL_MODE", "CPV_FRONT_CW", "CPV_DEPTH_TEST", "CPV_DEPTH_WRITE", "CPV_DEPTH_OP", "CPV_STENCIL_TEST",
    "CPV_ST_F_FAIL", "CPV_ST_F_PASS", "CPV_ST_F_DFAIL", "CPV_ST_F_OP", "CPV_ST_F_CMASK", "CPV_ST_F_WMASK", "CPV_ST_F_REF",
    "CPV_ST_B_FAIL", "CPV_ST_B_PASS", "CPV_ST_B_DFAIL", "CPV_ST_B_OP", "CPV_ST_B_CMASK", "CPV_ST_B_WMASK", "CPV_ST_B_REF",
    "CPV_BLEND", "CPV_SRC_COLOR", "CPV_DST_COLOR", "CPV_COLOR_OP", "CPV_SRC_ALPHA", "CPV_DST_ALPHA", "CPV_ALPHA_OP", "CPV_WRITE_MASK", "CPV_LOGIC", "CPV_LOGIC_OP",
    "CPV_DEPTH_BOUNDS", "CPV_MIN_DEPTH_BOUNDS", "CPV_MAX_DEPTH_BOUNDS",
    "CPV_COLOR_FORMAT", "CPV_DEPTH_FORMAT", "CPV_ORIGIN_UPPER", "CPV_FS_CONSTANT", "CPV_BLEND_TABLE", "CPV_LINE_WIDTH", "CPV_PRIM_KIND",
    "CPV_CF_BYTES", "CPV_CF_CHANNELS", "CPV_CF_BITS", "CPV_CF_KIND", "CPV_CF_BGRA", "CPV_FS_KILL", "CPV_EARLY_DEPTH", "CPV_VS_SAMPLES", "CPV_EXTRA_CA",
    "CPV_LOD_SITES",
};

}  // namespace

ModuleConfig module_config(uint32_t tile_shift, bool prefers_deferred, bool fs_constant, bool samples) {
    ModuleConfig mc;
    mc.tile_shift = tile_shift;
    mc.samples = samples;
    mc.schedule = schedule_for(prefers_deferred, fs_constant);
    // Measured on GB300: the immediate schedule runs best with batches of 128
    // primitives (C3: 2.64 against 2.87 ms; the smaller batch leaves room
    // for a sixth CTA per SM), the sparse one with 256 (C2: 0.39 against
    // 0.54 ms).
    mc.batch = mc.schedule == 0 ? 128u : 256u;
    // Tunables (CPV_RT_WARPS 1-32 warps per tile CTA, CPV_BATCH_PRIMS 32-256
    // primitives per shared-memory batch).
    if (const char* v = std::getenv("CPV_RT_WARPS")) {
        const int w = std::atoi(v);
        if (w >= 1 && w <= 32) mc.warps = static_cast<uint32_t>(w);
    }
    if (const char* v = std::getenv("CPV_BATCH_PRIMS")) {
        const int b = std::atoi(v);
        if (b >= 32 && b <= 256) mc.batch = static_cast<uint32_t>(b);
    }
    return mc;
}

uint32_t schedule_for(bool prefers_deferred, bool fs_constant) {
    if (const char* v = std::getenv("CPV_SCHEDULE")) {
        const int s = std::atoi(v);
        if (s >= 0 && s <= 2) return static_cast<uint32_t>(s);
    }
    // Shading once per primitive (flat-shaded geometry: overlays, quads)
    // goes with the immediate schedule and its per-warp primitive lists.
    // Otherwise the sparse schedule, which falls back to the immediate one
    // batch by batch where primitives are large; dense shading (deferred)
    // stays available through CPV_SCHEDULE=1.
    (void)prefers_deferred;
    return fs_constant ? 0u : 2u;
}

std::string compose_module(const std::vector<std::string>& stages, const std::vector<uint32_t>& nvs, const ModuleConfig& mc, bool batched,
                           const std::vector<std::string>& afters) {
    uint32_t nv_max = 0;
    for (uint32_t nv : nvs) nv_max = nv > nv_max ? nv : nv_max;
    // colour attachments of the pipelines' subpass (the pipelines of one
    // module share it)
    uint32_t num_ca = 1;
    for (const std::string& st : stages) {
        const size_t at = st.find("#define CPV_EXTRA_CA ");
        if (at != std::string::npos) num_ca = std::max<uint32_t>(num_ca, 1u + static_cast<uint32_t>(std::atoi(st.c_str() + at + 21)));
    }
    // the widest first-attachment texel in 32-bit words
    uint32_t colour_words = 1;
    for (const std::string& st : stages) {
        const size_t at = st.find("#define CPV_CF_BYTES ");
        if (at != std::string::npos) colour_words = std::max<uint32_t>(colour_words, (static_cast<uint32_t>(std::atoi(st.c_str() + at + 21)) + 3u) / 4u);
    }
    // the deferred schedule records one colour per fragment
    const uint32_t schedule = num_ca > 1 && mc.schedule == 1 ? 2u : mc.schedule;
    std::ostringstream src;
    src << "// " << kTranslationVersion << (batched ? " (batched)" : "") << "\n";
    src << "#define CPV_PIPELINE_MODULE 1\n";
    src << "#define CPV_TILE_SHIFT " << mc.tile_shift << "\n";
    src << "#define CPV_SCHEDULE " << schedule << "\n";
    src << "#define CPV_NUM_CA " << num_ca << "\n";
    src << "#define CPV_COLOUR_WORDS " << colour_words << "\n";
    src << "#define CPV_RT_WARPS " << mc.warps << "\n";
    src << "#define CPV_BATCH " << mc.batch << "\n";
    // Sparse schedule: fragments a pixel lists per batch before its
    // fallback. Measured on GB300: 24 for flat or lit shading (C4 raster
    // 34.0 ms, against 39.4 at 16 and 36.5 at 32), 16 when a fragment shader
    // samples images (the heightfield raster 0.41 ms, against 0.44 at 32).
    // CPV_SLOT_DEPTH overrides; CPV_SMALL_PX sets the largest in-tile box one
    // thread rasterises (default 32).
    {
        int depth = mc.depth ? static_cast<int>(mc.depth) : (mc.samples ? 16 : 24);
        if (const char* v = std::getenv("CPV_SLOT_DEPTH")) depth = std::atoi(v);
        if (depth >= 1 && depth <= 255) src << "#define CPV_SLOT_DEPTH " << depth << "\n";
        if (const char* v = std::getenv("CPV_SMALL_PX")) {
            const int k = std::atoi(v);
            if (k >= 1 && k <= 1024) src << "#define CPV_SMALL_PX " << k << "\n";
        }
    }
    // Register budget of the per-draw raster: the immediate schedule gains
    // from a seventh resident CTA (C3: 2.53 against 2.64 ms), the others
    // keep the compiler's choice. CPV_PLAIN_MIN_BLOCKS overrides.
    int min_blocks = mc.schedule == 0 ? 7 : 0;
    if (const char* v = std::getenv("CPV_PLAIN_MIN_BLOCKS")) min_blocks = std::atoi(v);
    if (min_blocks >= 1 && min_blocks <= 32) src << "#define CPV_PLAIN_MIN_BLOCKS " << min_blocks << "\n";
    // Register budget of the persistent batched raster, in resident CTAs of
    // 256 threads: 5 (48 registers a thread) for flat or lit shading, 4 (64)
    // when a fragment shader samples images (C4: 39.4 ms at 5 against 40.2
    // at 4; the textured heightfield: 0.41 ms at 4 against 0.43 at 5).
    // CPV_BATCH_MIN_BLOCKS overrides.
    {
        const uint32_t threads = std::min(1u << (2 * mc.tile_shift), 32u * mc.warps);
        int b = static_cast<int>((mc.samples ? 1024u : 1280u) / threads);
        if (b < 1) b = 1;
        if (const char* v = std::getenv("CPV_BATCH_MIN_BLOCKS")) b = std::atoi(v);
        if (b >= 1 && b <= 32) src << "#define CPV_RT_MIN_BLOCKS " << b << "\n";
    }
    // Register budget of the batched set-up in resident CTAs of 256
    // threads (CPV_SETUP_MIN_BLOCKS overrides the kernel's default).
    if (const char* v = std::getenv("CPV_SETUP_MIN_BLOCKS")) {
        const int k = std::atoi(v);
        if (k >= 1 && k <= 8) src << "#define CPV_SETUP_MIN_BLOCKS " << k << "\n";
    }
    src << "#define CPV_NV_MAX " << nv_max << "\n";
    bool any_constant = false;
    for (const std::string& st : stages) any_constant = any_constant || st.find("#define CPV_FS_CONSTANT 1\n") != std::string::npos;
    src << "#define CPV_ANY_FS_CONSTANT " << (any_constant ? 1 : 0) << "\n";
    bool any_lines = false;
    for (const std::string& st : stages)
        any_lines = any_lines || st.find("#define CPV_TOPOLOGY 1\n") != std::string::npos || st.find("#define CPV_TOPOLOGY 2\n") != std::string::npos;
    src << "#define CPV_ANY_LINES " << (any_lines ? 1 : 0) << "\n";
    // Vertex-side kernels fill the UNORM8 decode table only when a vertex
    // shader samples an image.
    bool any_vs_samples = false;
    for (const std::string& st : stages) any_vs_samples = any_vs_samples || st.find("#define CPV_VS_SAMPLES 1\n") != std::string::npos;
    src << "#define CPV_ANY_VS_SAMPLES " << (any_vs_samples ? 1 : 0) << "\n";
    src << "#include \"cpv_device.cuh\"\n#include \"cpv_raster.cuh\"\n";
    for (size_t i = 0; i < stages.size(); i++) {
        src << "namespace cpv_p" << i << " {\n" << stages[i] << "#include \"cpv_stage.cuh\"\n";
        if (i < afters.size()) src << afters[i];
        for (const char* m : kStageMacros) src << "#undef " << m << "\n";
        src << "}  // namespace cpv_p" << i << "\n";
    }
    if (!batched) {
        src << "#include \"cpv_pipeline.cuh\"\n";
    } else {
        // Routes a primitive to its pipeline's stage functions.
        src << "#define CPV_NUM_PIPELINES " << stages.size() << "\n";
        src << "template <typename F> __device__ __forceinline__ void cpv_dispatch(uint32_t pid, F&& f) {\n  switch (pid) {\n";
        for (size_t i = 1; i < stages.size(); i++) src << "  case " << i << ": f(cpv_p" << i << "::Stage()); break;\n";
        src << "  default: f(cpv_p0::Stage()); break;\n  }\n}\n";
        src << "#include \"cpv_batch.cuh\"\n";
    }
    return src.str();
}

namespace {

// Cubin for a module source: device cache → disk cache (CPV_CACHE_DIR) →
// NVRTC. The key hashes the source and the kernel headers it includes.
bool module_cubin(Device* dev, const std::string& source, std::array<uint8_t, 32>& key, std::vector<uint8_t>& cubin) {
    std::string keyed = source;
    for (int i = 0; i < rt::kKernelHeaderCount; i++) keyed += rt::kKernelHeaderSources[i];
    key = sha3_256(keyed.data(), keyed.size());
    {
        std::lock_guard<std::mutex> lock(dev->cache_mutex);
        auto it = dev->module_cache.find(key);
        if (it != dev->module_cache.end()) {
            cubin = it->second;
            return true;
        }
    }
    const std::string dir = cache_dir();
    bool found = false;
    if (!dir.empty()) {
        std::ifstream f(dir + "/" + hex(key) + ".cubin", std::ios::binary);
        if (f) {
            cubin.assign(std::istreambuf_iterator<char>(f), std::istreambuf_iterator<char>());
            found = !cubin.empty();
        }
    }
    if (!found) {
        std::string log;
        if (rt::compile(source, "module_" + hex(key).substr(0, 12) + ".cu", cubin, log) != rt::kOk) {
            rt::set_last_error("NVRTC failed: " + log);
            return false;
        }
        if (!dir.empty()) {
            std::ofstream f(dir + "/" + hex(key) + ".cubin", std::ios::binary);
            f.write(reinterpret_cast<const char*>(cubin.data()), static_cast<std::streamsize>(cubin.size()));
        }
    }
    std::lock_guard<std::mutex> lock(dev->cache_mutex);
    dev->module_cache[key] = cubin;
    return true;
}

}  // namespace

rt::Module* batch_module(Device* dev, const std::vector<Pipeline*>& pipelines, const ModuleConfig& mc) {
    std::string id = std::to_string(mc.tile_shift) + "/" + std::to_string(mc.schedule) + "/" + std::to_string(mc.warps) + "/" + std::to_string(mc.batch) +
                     "/" + std::to_string(mc.depth);
    for (const Pipeline* p : pipelines) id += "/" + hex(p->key);
    {
        std::lock_guard<std::mutex> lock(dev->batch_mutex);
        auto it = dev->batch_modules.find(id);
        if (it != dev->batch_modules.end()) return it->second.get();
    }
    // Compiled and loaded outside the lock, so that several configurations
    // (the tuner's candidates) compile at once; the first one stored wins.
    std::vector<std::string> stages, afters;
    std::vector<uint32_t> nvs;
    for (const Pipeline* p : pipelines) {
        stages.push_back(p->stage);
        afters.push_back(p->stage_after);
        nvs.push_back(p->nv);
    }
    const std::string source = compose_module(stages, nvs, mc, true, afters);
    if (const char* dump = std::getenv("CPV_DUMP_DIR")) {
        std::ofstream f(std::string(dump) + "/batch_" + std::to_string(pipelines.size()) + "_" + std::to_string(mc.tile_shift) + ".cu");
        f << source;
    }
    std::array<uint8_t, 32> key{};
    std::vector<uint8_t> cubin;
    if (!module_cubin(dev, source, key, cubin)) return nullptr;
    auto m = std::make_unique<rt::Module>();
    std::string err;
    if (dev->compile_only) {
        rt::set_last_error("batched module compiled; no device to load it on");
        return nullptr;
    }
    if (rt::load(cubin, mc.tile_shift, true, *m, err) != rt::kOk) {
        rt::set_last_error("batched module load failed: " + err);
        return nullptr;
    }
    std::lock_guard<std::mutex> lock(dev->batch_mutex);
    auto it = dev->batch_modules.find(id);
    if (it != dev->batch_modules.end()) {
        rt::unload(*m);
        return it->second.get();
    }
    rt::Module* out = m.get();
    dev->batch_modules[id] = std::move(m);
    return out;
}

VkResult create_graphics_pipeline(Device* dev, PipelineCache* cache, const VkGraphicsPipelineCreateInfo& ci, Pipeline** out) {
    auto reject = [&](const std::string& why) {
        rt::set_last_error("vkCreateGraphicsPipelines: " + why);
        return VK_ERROR_FEATURE_NOT_PRESENT;
    };
    const ShaderModule* vs = nullptr;
    const ShaderModule* fs = nullptr;
    std::string vs_entry, fs_entry;
    std::vector<spirv::SpecConstant> vs_spec, fs_spec;
    for (uint32_t i = 0; i < ci.stageCount; i++) {
        const auto& st = ci.pStages[i];
        std::vector<spirv::SpecConstant> spec;
        if (st.pSpecializationInfo) {
            const auto* si = st.pSpecializationInfo;
            for (uint32_t k = 0; k < si->mapEntryCount; k++) {
                spirv::SpecConstant sc;
                sc.id = si->pMapEntries[k].constantID;
                const uint8_t* b = static_cast<const uint8_t*>(si->pData) + si->pMapEntries[k].offset;
                sc.bytes.assign(b, b + si->pMapEntries[k].size);
                spec.push_back(sc);
            }
        }
        if (st.stage == VK_SHADER_STAGE_VERTEX_BIT) {
            vs = reinterpret_cast<const ShaderModule*>(st.module);
            vs_entry = st.pName ? st.pName : "main";
            vs_spec = spec;
        } else if (st.stage == VK_SHADER_STAGE_FRAGMENT_BIT) {
            fs = reinterpret_cast<const ShaderModule*>(st.module);
            fs_entry = st.pName ? st.pName : "main";
            fs_spec = spec;
        } else {
            return reject("only vertex and fragment stages are supported");
        }
    }
    if (!vs || !fs) return reject("a vertex and a fragment stage are required");
    if (!ci.pInputAssemblyState || !ci.pRasterizationState || !ci.pVertexInputState) return reject("missing fixed-function state");
    const auto topo = ci.pInputAssemblyState->topology;
    if (topo > VK_PRIMITIVE_TOPOLOGY_TRIANGLE_FAN) return reject("topologies with adjacency and patch lists are not implemented");
    if (ci.pInputAssemblyState->primitiveRestartEnable) return reject("primitive restart");
    const auto& rs = *ci.pRasterizationState;
    if (rs.rasterizerDiscardEnable) return reject("rasterizer discard");
    if (rs.polygonMode != VK_POLYGON_MODE_FILL) return reject("non-fill polygon mode");
    if (rs.depthClampEnable) return reject("depth clamp");
    if (ci.pMultisampleState && ci.pMultisampleState->rasterizationSamples > 1) return reject("multisampling");

    const RenderPass* pass = reinterpret_cast<const RenderPass*>(ci.renderPass);
    if (!pass) return reject("no render pass");
    // up to eight colour attachments (the reference's
    // MAX_FRAGMENT_OUTPUT_ATTACHMENTS), or none (a depth-only pass); with
    // several, the first must be used
    if (ci.subpass >= pass->subpasses.size()) return reject("subpass " + std::to_string(ci.subpass) + " of the render pass");
    const Subpass& sub = pass->subpasses[ci.subpass];
    const uint32_t nca = static_cast<uint32_t>(sub.colour.size());
    if (nca > CPV_MAX_CA) return reject("more than 8 colour attachments");
    if (nca > 1 && sub.colour[0] == VK_ATTACHMENT_UNUSED) return reject("an unused first colour attachment with others after it");
    const VkFormat cfmt = sub.colour.empty() ? VK_FORMAT_UNDEFINED : pass->attachments[sub.colour[0]].format;
    if (!sub.colour.empty() && !supported_colour(cfmt)) return reject("colour attachment format " + std::to_string(cfmt));
    std::vector<VkFormat> extra_fmt;  // attachments 1 .. nca - 1 (UNDEFINED: unused)
    for (uint32_t k = 1; k < nca; k++) {
        const VkFormat f = sub.colour[k] == VK_ATTACHMENT_UNUSED ? VK_FORMAT_UNDEFINED : pass->attachments[sub.colour[k]].format;
        if (f != VK_FORMAT_UNDEFINED && !supported_colour(f)) return reject("colour attachment format " + std::to_string(f));
        ColourLayout ecl;
        if (f != VK_FORMAT_UNDEFINED && colour_layout(f, ecl) && ecl.bytes > 4)
            return reject("an 8- or 16-byte colour format after the first attachment");
        extra_fmt.push_back(f);
    }
    if (sub.colour.empty() && sub.depth == VK_ATTACHMENT_UNUSED) return reject("a colour or a depth attachment is required");
    VkFormat dfmt = VK_FORMAT_UNDEFINED;
    if (sub.depth != VK_ATTACHMENT_UNUSED) {
        dfmt = pass->attachments[sub.depth].format;
        if (!supported_depth(dfmt)) return reject("depth attachment format " + std::to_string(dfmt));
    }

    VkPipelineDepthStencilStateCreateInfo ds{};
    if (ci.pDepthStencilState) ds = *ci.pDepthStencilState;
    const bool stencil = ds.stencilTestEnable && dfmt == VK_FORMAT_D32_SFLOAT_S8_UINT;

    VkPipelineColorBlendAttachmentState blend{};
    blend.colorWriteMask = 0xF;
    float blend_constants[4] = {0, 0, 0, 0};
    bool logic = false;
    uint32_t logic_op = VK_LOGIC_OP_COPY;
    if (ci.pColorBlendState && cfmt != VK_FORMAT_UNDEFINED) {
        if (ci.pColorBlendState->attachmentCount >= 1) blend = ci.pColorBlendState->pAttachments[0];
        for (int i = 0; i < 4; i++) blend_constants[i] = ci.pColorBlendState->blendConstants[i];
        if (ci.pColorBlendState->logicOpEnable) {
            // A logic op applies to the encoded bits of a normalised 8-bit
            // format; blending of the attachment is then treated as disabled
            // (Vulkan 1.1, "Logical Operations"). The reference aborts here
            // (LLVMRuntime/PipelineCompiler.cpp:1687-1690); formats of other
            // widths and float formats are rejected.
            ColourLayout cl;
            if (!colour_layout(cfmt, cl) || cl.bits != 8 || cl.kind >= 2) return reject("logic op on colour format " + std::to_string(cfmt));
            for (VkFormat f : extra_fmt)
                if (f != VK_FORMAT_UNDEFINED && (!colour_layout(f, cl) || cl.bits != 8 || cl.kind >= 2))
                    return reject("logic op on colour format " + std::to_string(f));
            if (static_cast<uint32_t>(ci.pColorBlendState->logicOp) > VK_LOGIC_OP_SET) return reject("logic op " + std::to_string(ci.pColorBlendState->logicOp));
            logic = true;
            logic_op = static_cast<uint32_t>(ci.pColorBlendState->logicOp);
            blend.blendEnable = VK_FALSE;
        }
    }
    // each further attachment's own blend state (independent blending)
    std::vector<VkPipelineColorBlendAttachmentState> extra_blend;
    for (uint32_t k = 1; k < nca; k++) {
        VkPipelineColorBlendAttachmentState b{};
        b.colorWriteMask = 0xF;
        if (ci.pColorBlendState && k < ci.pColorBlendState->attachmentCount) b = ci.pColorBlendState->pAttachments[k];
        if (logic) b.blendEnable = VK_FALSE;
        extra_blend.push_back(b);
    }
    // integer attachments are not blended (Vulkan 1.1, "Blending": blending
    // applies to floating-point and normalised formats only)
    auto integer_format = [](VkFormat f) {
        ColourLayout cl;
        return f != VK_FORMAT_UNDEFINED && colour_layout(f, cl) && cl.kind >= 3;
    };
    if (integer_format(cfmt)) blend.blendEnable = VK_FALSE;
    for (uint32_t k = 1; k < nca; k++)
        if (integer_format(extra_fmt[k - 1])) extra_blend[k - 1].blendEnable = VK_FALSE;
    auto check_blend = [](const VkPipelineColorBlendAttachmentState& b) -> const char* {
        if (!b.blendEnable) return nullptr;
        auto bad = [](VkBlendFactor f) { return f > VK_BLEND_FACTOR_SRC_ALPHA_SATURATE; };
        if (bad(b.srcColorBlendFactor) || bad(b.dstColorBlendFactor) || bad(b.srcAlphaBlendFactor) || bad(b.dstAlphaBlendFactor))
            return "dual-source blend factors";
        if (b.colorBlendOp > VK_BLEND_OP_MAX || b.alphaBlendOp > VK_BLEND_OP_MAX) return "advanced blend ops";
        return nullptr;
    };
    if (const char* why = check_blend(blend)) return reject(why);
    for (const auto& b : extra_blend)
        if (const char* why = check_blend(b)) return reject(why);

    bool dyn_viewport = false, dyn_blend = false;
    if (ci.pDynamicState) {
        for (uint32_t i = 0; i < ci.pDynamicState->dynamicStateCount; i++) {
            const auto d = ci.pDynamicState->pDynamicStates[i];
            if (d == VK_DYNAMIC_STATE_VIEWPORT) dyn_viewport = true;
            else if (d == VK_DYNAMIC_STATE_BLEND_CONSTANTS) dyn_blend = true;
            else if (d == VK_DYNAMIC_STATE_LINE_WIDTH && (topo == VK_PRIMITIVE_TOPOLOGY_LINE_LIST || topo == VK_PRIMITIVE_TOPOLOGY_LINE_STRIP))
                return reject("dynamic line width on a line topology");
            else if (d == VK_DYNAMIC_STATE_SCISSOR || d == VK_DYNAMIC_STATE_LINE_WIDTH || d == VK_DYNAMIC_STATE_DEPTH_BIAS) continue;
            else return reject("dynamic state " + std::to_string(d));
        }
    }
    VkViewport viewport{};
    if (!dyn_viewport) {
        if (!ci.pViewportState || ci.pViewportState->viewportCount != 1 || !ci.pViewportState->pViewports)
            return reject("exactly one static viewport is required");
        viewport = ci.pViewportState->pViewports[0];
    }

    // Vertex input state → translator view.
    std::vector<spirv::VertexBinding> bindings;
    std::vector<spirv::VertexAttribute> attributes;
    for (uint32_t i = 0; i < ci.pVertexInputState->vertexBindingDescriptionCount; i++) {
        const auto& b = ci.pVertexInputState->pVertexBindingDescriptions[i];
        bindings.push_back({b.binding, b.stride, static_cast<uint32_t>(b.inputRate)});
    }
    for (uint32_t i = 0; i < ci.pVertexInputState->vertexAttributeDescriptionCount; i++) {
        const auto& a = ci.pVertexInputState->pVertexAttributeDescriptions[i];
        attributes.push_back({a.location, a.binding, static_cast<uint32_t>(a.format), a.offset});
    }

    // Translate both stages.
    std::vector<spirv::ResourceSlot> slots;
    spirv::StageResult vr, fr;
    std::string err;
    if (!spirv::translate_stage(vs->module, 0, vs_entry, vs_spec, bindings, attributes, slots, vr, err)) return reject("vertex shader: " + err);
    // CPV_SPEC_LOD=1: the labelled quad-derivative LOD mode for implicit-LOD
    // sampling in fragment shaders (Vulkan's λ from screen-space
    // derivatives); otherwise λ is 0, as the reference computes it
    // (CPVulkan/GlslFunctions.cpp:657-672).
    const char* spec_lod_env = std::getenv("CPV_SPEC_LOD");
    const bool spec_lod = spec_lod_env != nullptr && std::atoi(spec_lod_env) == 1;
    if (!spirv::translate_stage(fs->module, 4, fs_entry, fs_spec, {}, {}, slots, fr, err, spec_lod)) return reject("fragment shader: " + err);
    if (fr.lod_sites > 8) return reject("more than 8 implicit-LOD sampling instructions in a fragment shader under CPV_SPEC_LOD");

    const uint32_t nv = vr.num_floats > fr.num_floats ? vr.num_floats : fr.num_floats;
    const uint32_t tile_shift = tile_shift_for_pipeline();
    // Dense shading pays off when the fragment shader samples images or is long.
    const bool prefers_deferred = fr.samples > 0 || fr.instructions > 48;
    // The pipeline's stage block: fixed-function macros, translated shaders
    // and the interpolation table. compose_module() wraps it in a namespace.
    std::ostringstream src;
    src << "#define CPV_NV " << nv << "\n";
    src << "#define CPV_TOPOLOGY " << static_cast<uint32_t>(topo) << "\n";
    src << "#define CPV_CULL_MODE " << rs.cullMode << "\n";
    {
        // The pipeline's (static) line width, bit-exact; the reference reads
        // it from the pipeline even when the width is dynamic state.
        uint32_t bits;
        std::memcpy(&bits, &rs.lineWidth, 4);
        src << "#define CPV_LINE_WIDTH __uint_as_float(" << bits << "u)\n";
    }
    src << "#define CPV_FRONT_CW " << (rs.frontFace == VK_FRONT_FACE_CLOCKWISE ? 1 : 0) << "\n";
    src << "#define CPV_DEPTH_TEST " << (ds.depthTestEnable ? 1 : 0) << "\n";
    src << "#define CPV_DEPTH_WRITE " << (ds.depthWriteEnable ? 1 : 0) << "\n";
    src << "#define CPV_DEPTH_OP " << static_cast<uint32_t>(ds.depthCompareOp) << "\n";
    // Depth bounds test (LLVMRuntime/PipelineCompiler.cpp:1128-1166): static
    // bounds only (the reference aborts on dynamic ones, and so
    // VK_DYNAMIC_STATE_DEPTH_BOUNDS is rejected above); without a depth
    // attachment there is no test.
    const bool depth_bounds = ds.depthBoundsTestEnable && dfmt != VK_FORMAT_UNDEFINED;
    uint32_t min_bits, max_bits;
    std::memcpy(&min_bits, &ds.minDepthBounds, 4);
    std::memcpy(&max_bits, &ds.maxDepthBounds, 4);
    src << "#define CPV_DEPTH_BOUNDS " << (depth_bounds ? 1 : 0) << "\n";
    src << "#define CPV_MIN_DEPTH_BOUNDS __uint_as_float(" << min_bits << "u)\n";
    src << "#define CPV_MAX_DEPTH_BOUNDS __uint_as_float(" << max_bits << "u)\n";
    src << "#define CPV_STENCIL_TEST " << (stencil ? 1 : 0) << "\n";
    const VkStencilOpState* so[2] = {&ds.front, &ds.back};
    const char* sn[2] = {"F", "B"};
    for (int k = 0; k < 2; k++) {
        src << "#define CPV_ST_" << sn[k] << "_FAIL " << static_cast<uint32_t>(so[k]->failOp) << "\n";
        src << "#define CPV_ST_" << sn[k] << "_PASS " << static_cast<uint32_t>(so[k]->passOp) << "\n";
        src << "#define CPV_ST_" << sn[k] << "_DFAIL " << static_cast<uint32_t>(so[k]->depthFailOp) << "\n";
        src << "#define CPV_ST_" << sn[k] << "_OP " << static_cast<uint32_t>(so[k]->compareOp) << "\n";
        src << "#define CPV_ST_" << sn[k] << "_CMASK " << so[k]->compareMask << "u\n";
        src << "#define CPV_ST_" << sn[k] << "_WMASK " << so[k]->writeMask << "u\n";
        src << "#define CPV_ST_" << sn[k] << "_REF " << so[k]->reference << "u\n";
    }
    // One colour attachment's macros: blend state, write mask, format and
    // its layout (texel bytes, channels, bits per channel, kind 0 UNORM /
    // 1 SNORM / 2 SFLOAT, red in byte 2).
    auto colour_block = [](VkFormat f, const VkPipelineColorBlendAttachmentState& b) {
        std::ostringstream o;
        o << "#define CPV_BLEND " << (b.blendEnable ? 1 : 0) << "\n";
        o << "#define CPV_SRC_COLOR " << static_cast<uint32_t>(b.srcColorBlendFactor) << "\n";
        o << "#define CPV_DST_COLOR " << static_cast<uint32_t>(b.dstColorBlendFactor) << "\n";
        o << "#define CPV_COLOR_OP " << static_cast<uint32_t>(b.colorBlendOp) << "\n";
        o << "#define CPV_SRC_ALPHA " << static_cast<uint32_t>(b.srcAlphaBlendFactor) << "\n";
        o << "#define CPV_DST_ALPHA " << static_cast<uint32_t>(b.dstAlphaBlendFactor) << "\n";
        o << "#define CPV_ALPHA_OP " << static_cast<uint32_t>(b.alphaBlendOp) << "\n";
        o << "#define CPV_WRITE_MASK " << (b.colorWriteMask & 0xF) << "u\n";
        o << "#define CPV_COLOR_FORMAT " << static_cast<uint32_t>(f) << "\n";
        ColourLayout cl;
        if (f != VK_FORMAT_UNDEFINED) colour_layout(f, cl);
        o << "#define CPV_CF_BYTES " << cl.bytes << "\n#define CPV_CF_CHANNELS " << cl.channels << "\n#define CPV_CF_BITS " << cl.bits
          << "\n#define CPV_CF_KIND " << cl.kind << "\n#define CPV_CF_BGRA " << (cl.bgra ? 1 : 0) << "\n";
        return o.str();
    };
    src << colour_block(cfmt, blend);
    src << "#define CPV_LOGIC " << (logic ? 1 : 0) << "\n";
    src << "#define CPV_LOGIC_OP " << logic_op << "\n";
    src << "#define CPV_EXTRA_CA " << (nca > 1 ? nca - 1 : 0) << "\n";
    src << "#define CPV_DEPTH_FORMAT " << static_cast<uint32_t>(dfmt) << "\n";
    src << "#define CPV_ORIGIN_UPPER " << (fr.origin_upper_left ? 1 : 0) << "\n";
    // A fragment shader that reads neither FragCoord nor FrontFacing and only
    // flat inputs computes the same result for every fragment of a primitive:
    // it runs once per primitive at set-up.
    // (With several colour attachments the fragment shader runs per
    // fragment: a primitive record holds one colour.)
    bool fs_constant = !fr.reads_frag_coord && !fr.reads_front_facing && nca <= 1;
    for (int k : fr.interp) fs_constant = fs_constant && k == 2;
    src << "#define CPV_FS_CONSTANT " << (fs_constant ? 1 : 0) << "\n";
    src << "#define CPV_FS_KILL " << (fr.has_kill ? 1 : 0) << "\n";
    src << "#define CPV_VS_SAMPLES " << (vr.samples > 0 ? 1 : 0) << "\n";
    src << "#define CPV_LOD_SITES " << fr.lod_sites << "\n";
    // Blending a per-primitive constant colour where each channel's result
    // depends only on that channel of the destination (no DST_ALPHA,
    // ONE_MINUS_DST_ALPHA or SRC_ALPHA_SATURATE colour factors): the result
    // is a byte → byte table per channel, built once per primitive.
    auto dst_alpha_factor = [](VkBlendFactor f) {
        return f == VK_BLEND_FACTOR_DST_ALPHA || f == VK_BLEND_FACTOR_ONE_MINUS_DST_ALPHA || f == VK_BLEND_FACTOR_SRC_ALPHA_SATURATE;
    };
    const bool blend_table = fs_constant && blend.blendEnable && !dst_alpha_factor(blend.srcColorBlendFactor) &&
                             !dst_alpha_factor(blend.dstColorBlendFactor) &&
                             (cfmt == VK_FORMAT_R8G8B8A8_UNORM || cfmt == VK_FORMAT_B8G8R8A8_UNORM);  // tables map RGBA8 bytes
    src << "#define CPV_BLEND_TABLE " << (blend_table ? 1 : 0) << "\n";
    src << vr.code << fr.code;
    src << "__device__ __forceinline__ int cpv_interp(int c) {\n  switch (c) {\n";
    for (size_t i = 0; i < fr.interp.size(); i++)
        if (fr.interp[i] != 0) src << "  case " << i << ": return " << fr.interp[i] << ";\n";
    src << "  default: return 0;\n  }\n}\n";

    // Attachments 1 .. nca - 1: the fragment shader must declare an output
    // for each used one (the reference looks the location up with
    // std::map::at, LLVMRuntime/PipelineCompiler.cpp:1655-1659). Each is
    // compiled from cpv_stage.cuh again in a nested namespace with its own
    // colour macros, after the pipeline's own functions; the pipeline's
    // cpv_load_extra / cpv_store_extra / cpv_write_extra call them.
    std::ostringstream after;
    if (nca > 1) {
        static const char* const colour_macros[] = {"CPV_BLEND", "CPV_SRC_COLOR", "CPV_DST_COLOR", "CPV_COLOR_OP", "CPV_SRC_ALPHA", "CPV_DST_ALPHA",
                                                    "CPV_ALPHA_OP", "CPV_WRITE_MASK", "CPV_COLOR_FORMAT", "CPV_CF_BYTES", "CPV_CF_CHANNELS",
                                                    "CPV_CF_BITS", "CPV_CF_KIND", "CPV_CF_BGRA", "CPV_BLEND_TABLE", "CPV_EXTRA_CA"};
        for (uint32_t k = 1; k < nca; k++) {
            if (extra_fmt[k - 1] != VK_FORMAT_UNDEFINED && !((fr.outputs >> k) & 1u))
                return reject("the fragment shader has no output for colour attachment " + std::to_string(k));
            after << "namespace cpv_ca" << k << " {\n";
            for (const char* m : colour_macros) after << "#undef " << m << "\n";
            after << colour_block(extra_fmt[k - 1], extra_blend[k - 1]) << "#define CPV_BLEND_TABLE 0\n#define CPV_EXTRA_CA 0\n";
            after << "#include \"cpv_stage.cuh\"\n}  // namespace cpv_ca" << k << "\n";
        }
        after << "__device__ __forceinline__ void cpv_load_extra(const uint8_t* const* c, uint64_t pix, CpvPixel& s) {\n";
        for (uint32_t k = 1; k < nca; k++) after << "  cpv_ca" << k << "::cpv_load_colour(c[" << k - 1 << "], pix, &s.extra[" << k - 1 << "]);\n";
        after << "}\n__device__ __forceinline__ void cpv_store_extra(uint8_t* const* c, uint64_t pix, const CpvPixel& s) {\n";
        for (uint32_t k = 1; k < nca; k++) after << "  cpv_ca" << k << "::cpv_store_colour(c[" << k - 1 << "], pix, &s.extra[" << k - 1 << "]);\n";
        after << "}\n__device__ __forceinline__ void cpv_write_extra(const float bc[4], const float* colour, CpvPixel& s) {\n";
        for (uint32_t k = 1; k < nca; k++)
            after << "  cpv_ca" << k << "::cpv_write_colour(bc, colour + " << 4 * k << ", &s.extra[" << k - 1 << "]);\n";
        after << "}\n";
    }

    auto p = std::make_unique<Pipeline>();
    p->stage = src.str();
    p->stage_after = after.str();
    p->nv = nv;
    p->prefers_deferred = prefers_deferred;
    p->samples = fr.samples > 0;
    p->tile_shift = tile_shift;
    p->blend_table = blend_table;
    p->fs_constant = fs_constant;
    p->source = compose_module({p->stage}, {nv}, module_config(tile_shift, prefers_deferred, fs_constant, fr.samples > 0), false, {p->stage_after});
    // The key covers the generated source and the embedded kernel headers it
    // includes, so an on-disk cache never returns a cubin of older kernels.
    {
        std::string keyed = p->source;
        for (int i = 0; i < rt::kKernelHeaderCount; i++) keyed += rt::kKernelHeaderSources[i];
        p->key = sha3_256(keyed.data(), keyed.size());
    }
    if (const char* dump = std::getenv("CPV_DUMP_DIR")) {
        std::ofstream f(std::string(dump) + "/pipeline_" + hex(p->key).substr(0, 12) + ".cu");
        f << p->source;
    }
    p->slots = slots;
    p->topology = topo;
    p->viewport = viewport;
    p->dynamic_viewport = dyn_viewport;
    p->dynamic_blend_constants = dyn_blend;
    for (int i = 0; i < 4; i++) p->blend_constants[i] = blend_constants[i];
    p->layout = reinterpret_cast<PipelineLayout*>(ci.layout);
    p->colour_format = cfmt;
    p->depth_format = dfmt;
    p->blend = blend.blendEnable != 0;

    // Cubin: pipeline cache object → in-process cache → disk cache → NVRTC.
    std::vector<uint8_t> cubin;
    bool found = false;
    if (cache) {
        std::lock_guard<std::mutex> lock(cache->mutex);
        auto it = cache->entries.find(p->key);
        if (it != cache->entries.end()) {
            cubin = it->second;
            found = true;
        }
    }
    if (!found) {
        std::lock_guard<std::mutex> lock(dev->cache_mutex);
        auto it = dev->module_cache.find(p->key);
        if (it != dev->module_cache.end()) {
            cubin = it->second;
            found = true;
        }
    }
    const std::string dir = cache_dir();
    if (!found && !dir.empty()) {
        std::ifstream f(dir + "/" + hex(p->key) + ".cubin", std::ios::binary);
        if (f) {
            cubin.assign(std::istreambuf_iterator<char>(f), std::istreambuf_iterator<char>());
            found = !cubin.empty();
        }
    }
    if (!found) {
        std::string log;
        if (rt::compile(p->source, "pipeline_" + hex(p->key).substr(0, 12) + ".cu", cubin, log) != rt::kOk) {
            rt::set_last_error("NVRTC failed: " + log);
            if (std::getenv("CPV_DUMP_FAILED")) std::fprintf(stderr, "%s\n----\n%s\n", p->source.c_str(), log.c_str());
            return VK_ERROR_INITIALIZATION_FAILED;
        }
        if (!dir.empty()) {
            std::ofstream f(dir + "/" + hex(p->key) + ".cubin", std::ios::binary);
            f.write(reinterpret_cast<const char*>(cubin.data()), static_cast<std::streamsize>(cubin.size()));
        }
    }
    {
        std::lock_guard<std::mutex> lock(dev->cache_mutex);
        dev->module_cache[p->key] = cubin;
    }
    if (cache) {
        std::lock_guard<std::mutex> lock(cache->mutex);
        cache->entries[p->key] = cubin;
    }
    if (dev->compile_only) {
        *out = p.release();
        return VK_SUCCESS;
    }
    if (rt::load(cubin, tile_shift, false, p->module, err) != rt::kOk) {
        rt::set_last_error("module load failed: " + err);
        return VK_ERROR_INITIALIZATION_FAILED;
    }
    p->module.blend_table = blend_table;
    *out = p.release();
    return VK_SUCCESS;
}

}  // namespace cpv::icd
