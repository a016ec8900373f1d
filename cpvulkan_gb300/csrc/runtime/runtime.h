// runtime.h — the CUDA side of the ICD: pipeline module compilation (NVRTC,
// sm_103a), module loading, per-queue scratch memory and the launch
// sequences of one draw (plain path) and of one submission (batched path).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>
#include <string>
#include <vector>

#include "../kernels/cpv_params.h"

namespace cpv::rt {

// Error codes returned across the C ABI (never exceptions).
enum Status : int {
    kOk = 0,
    kErrCuda = -1,
    kErrCompile = -2,
    kErrOutOfMemory = -3,
    kErrInvalid = -4,
    kErrTimeout = -5,
    kErrDeviceLost = -6,
};

// Embedded kernel headers for NVRTC (generated at build time from
// csrc/kernels/: names and sources, in a fixed order).
extern const int kKernelHeaderCount;
extern const char* const kKernelHeaderNames[];
extern const char* const kKernelHeaderSources[];

// A loaded raster module: the per-draw kernels of one pipeline
// (cpv_setup_rects, cpv_raster) or the batched kernels of a set of pipelines
// (cpv_batch_setup, cpv_batch_raster).
struct Module {
    cudaLibrary_t library = nullptr;
    cudaKernel_t setup_rects = nullptr;
    cudaKernel_t raster = nullptr;
    cudaKernel_t blend_tables = nullptr;  // per-draw modules
    cudaKernel_t vertex = nullptr;        // batched modules: the vertex stage
    uint32_t vs_stride = 0;               // batched modules: output floats per vertex slot
    bool blend_table = false;             // the pipeline blends a per-primitive constant colour
    bool batched = false;
    uint32_t tile_shift = 4;
    uint32_t raster_threads = 256;
    uint32_t raster_smem = 0;  // dynamic shared memory of the raster kernel (bytes)
};

// Initialises the CUDA context on device 0 (once per process).
int init(std::string& error);
bool available();

// Compiles a pipeline translation unit with NVRTC for sm_103a.
int compile(const std::string& source, const std::string& name, std::vector<uint8_t>& cubin, std::string& log);
// Loads a cubin and resolves the pipeline kernels.
int load(const std::vector<uint8_t>& cubin, uint32_t tile_shift, bool batched, Module& out, std::string& error);
void unload(Module& m);

// Device words of a queue's per-draw binning: [0] pair total, [1] status,
// [4..7] the union of the draw's tile rectangles, [9] the scan's CTA
// counter, [kSumsWord ..] one scanned sum per binning CTA (at most 2048).
constexpr uint32_t kSumsWord = 16;
constexpr uint64_t kWordsBytes = 4ull * (kSumsWord + 2048u);

// Grow-only device scratch owned by one queue. Draws on that queue's stream
// reuse it in stream order.
class Scratch {
public:
    ~Scratch();
    int reserve_rects(uint64_t prims);
    int reserve_bins(uint64_t entries);  // tiles * spans
    int reserve_list(uint64_t entries);
    int reserve_scan(uint64_t n);
    int reserve_tables(uint64_t bytes);
    uint8_t* tables() const { return tables_; }
    uint16_t* rects() const { return rects_; }
    uint32_t* counts() const { return counts_; }
    uint64_t counts_capacity() const { return counts_cap_; }
    uint32_t* cursor() const { return cursor_; }
    uint32_t* list() const { return list_; }
    uint32_t list_capacity() const { return static_cast<uint32_t>(list_cap_); }
    uint32_t* words() const { return words_; }  // kWordsBytes: see kSumsWord
    uint32_t* scan_level(int level) const { return scan_[level]; }
    int ensure_words();
    // Incremented whenever a buffer is (re)allocated: work captured in a CUDA
    // graph against older pointers must be captured again.
    uint64_t generation() const { return generation_; }

private:
    template <typename T>
    int grow_tracked(T*& ptr, uint64_t& cap, uint64_t need);
    uint64_t generation_ = 0;
    uint16_t* rects_ = nullptr;
    uint64_t rects_cap_ = 0;
    uint32_t* counts_ = nullptr;
    uint64_t counts_cap_ = 0;
    uint32_t* cursor_ = nullptr;
    uint64_t cursor_cap_ = 0;
    uint32_t* list_ = nullptr;
    uint64_t list_cap_ = 0;
    uint32_t* scan_[8] = {};
    uint64_t scan_cap_[8] = {};
    uint32_t* words_ = nullptr;
    uint8_t* tables_ = nullptr;
    uint64_t tables_cap_ = 0;
};

// Launch-count accounting (kernels this library launched), for benchmarks.
uint64_t launches();
void count_launch(uint64_t n = 1);

// Optional per-kernel device timing: when enabled, every kernel of the draw
// path is bracketed by CUDA events on its launching stream; totals are
// summed (after synchronising) per kernel name.
void profile_enable(bool on);
bool profile_enabled();
void profile_begin(cudaStream_t s, const char* name);
void profile_end(cudaStream_t s);
int profile_get(const char* name, uint64_t* count, double* ms);
void profile_reset();

// Plain per-draw path: the full kernel sequence of one draw on `stream`.
// `P` must have geometry, resources and attachments filled; tiling and
// binning fields are filled here.
int draw_plain(cudaStream_t stream, const Module& m, CpvDrawParams P, Scratch& scratch);

// ---- batched path: every draw of a render pass in one kernel sequence ----

// Host description of one batch: the draws' parameters (as the per-draw path
// builds them) and each draw's pipeline index in the batched module. All
// draws share the render pass's attachments and viewport extent.
struct BatchDraws {
    std::vector<CpvDrawParams> draws;
    std::vector<uint32_t> pipeline;
    std::vector<uint8_t> triangles;  // per draw: the pipeline assembles triangles (the vertex stage applies)
    uint8_t* color = nullptr;
    uint8_t* depth = nullptr;
    uint8_t* color_extra[CPV_MAX_CA - 1] = {};
    uint32_t fb_width = 0, fb_height = 0;
    float vw = 0.0f, vh = 0.0f;
};

// Device state of one batched render pass of a recorded command buffer:
// the uploaded draw tables, the binning buffers (sized on the first run) and,
// after the first launch, a CUDA graph of the whole kernel sequence.
class BatchPlan {
public:
    BatchPlan() = default;
    BatchPlan(const BatchPlan&) = delete;
    BatchPlan& operator=(const BatchPlan&) = delete;
    ~BatchPlan();
    // Uploads the tables, allocates every buffer and measures the pair count
    // of the batch with one synchronous set-up run.
    int build(const Module& m, const BatchDraws& in, cudaStream_t stream);
    // Enqueues the batch on `stream`: the captured graph when there is one
    // (captured on the first call), else the kernel sequence. Grows the pair
    // buffers first when an earlier launch needed more than they hold.
    int launch(const Module& m, cudaStream_t stream);
    uint64_t primitives() const { return prims_; }
    uint32_t kernels_per_launch() const { return kernels_; }
    // Vertex slots of the vertex stage (0 when no draw has any).
    uint64_t vertex_slots() const { return vs_slots_; }

private:
    int enqueue(const Module& m, cudaStream_t stream);
    int alloc_pairs(uint32_t capacity);
    void free_pairs();
    int build_vertex_stage(const Module& m, const BatchDraws& in, cudaStream_t stream);

    CpvBatchParams P_{};
    Scratch scan_;
    CpvDrawParams* draws_ = nullptr;
    uint32_t* pipeline_ = nullptr;
    uint32_t* draw_block_ = nullptr;
    uint32_t* block_draw_ = nullptr;
    uint2* rects_ = nullptr;
    uint32_t* block_pairs_ = nullptr;
    uint32_t* block_offsets_ = nullptr;
    uint32_t* keys_[2] = {};
    uint32_t* vals_[2] = {};
    uint32_t cap_ = 0;
    uint32_t* hist_ = nullptr;
    uint32_t* hist_offsets_ = nullptr;
    uint32_t* tile_begin_ = nullptr;
    uint32_t* tile_end_ = nullptr;
    uint32_t* words_ = nullptr;         // [0] pair total, [1] status, [2] tile counter
    float* ndc_ = nullptr;              // pixel-centre NDC of the columns, then the rows
    float* vs_pos_ = nullptr;           // vertex stage: NDC position and clip w per slot
    float* vs_var_ = nullptr;           // vertex stage: outputs per slot
    uint32_t* vs_draw_block_ = nullptr;
    uint32_t* vs_block_draw_ = nullptr;
    uint64_t vs_slots_ = 0;
    uint32_t* pinned_pairs_ = nullptr;  // pair total of the last launch (host)
    cudaEvent_t done_ = nullptr;
    uint64_t prims_ = 0;
    uint32_t tiles_ = 0, radix_ctas_ = 0, raster_ctas_ = 0, passes_ = 1, kernels_ = 0;
    cudaGraphExec_t exec_ = nullptr;
};

// Primitives, vertex slots and (primitive, tile) pairs of the most recent
// batched launch that had completed when the next one was enqueued.
void batch_stats(uint64_t out[3]);

// Fixed binning scratch for submissions that may not allocate: one
// 32 MiB file-scope device array per device. A draw needs 8 bytes per
// primitive for its tile rectangles plus its bins; one that does not fit even
// with one span per tile is rejected (kErrOutOfMemory, message in
// last_error()). The array is shared by every queue of the process on that
// device, so draw_plain_static calls whose work overlaps on the GPU race.
#define CPV_STATIC_SCRATCH_BYTES (32ull << 20)
// Resolves the array's device address for the current device
// (cudaGetSymbolAddress, once per device). Call outside any stream capture.
int static_scratch_setup(std::string& error);
// kOk when a draw of `prims` primitives on a width × height attachment fits.
int static_scratch_check(uint64_t prims, uint32_t tile_shift, uint32_t width, uint32_t height, std::string& error);
// draw_plain with every scratch buffer carved from the fixed array: launches
// the same kernels, allocates nothing, creates no CUDA objects.
int draw_plain_static(cudaStream_t stream, const Module& m, CpvDrawParams P);

// vkCmdBlitImage of one 2D colour region between RGBA8/BGRA8 levels: `src`
// describes the source level (as level 0), `dst` points at the destination
// level's first texel. Regions are {x0, y0, x1, y1} (end exclusive, may be
// reversed); filter 0 NEAREST, 1 LINEAR.
int blit(cudaStream_t stream, const CpvTexture& src, uint8_t* dst, uint32_t dst_w, uint32_t dst_h, uint32_t dst_format, const int32_t src_region[4],
         const int32_t dst_region[4], uint32_t filter);

// Attachment fill with an encoded texel (1, 2, 4 or 8 bytes).
int fill(cudaStream_t stream, void* dst, uint64_t texels, uint32_t texel_bytes, uint32_t lo, uint32_t hi, uint32_t w2 = 0, uint32_t w3 = 0);
// Fill of a w x h rectangle of 2-, 4- or 8-byte texels whose rows start
// `pitch` bytes apart (texel-aligned base and pitch); for 8-byte depth /
// stencil texels write_lo / write_hi pick the depth and stencil words.
int fill_rect(cudaStream_t stream, uint8_t* base, uint64_t pitch, uint32_t w, uint32_t h, uint32_t texel_bytes, uint32_t lo, uint32_t hi, bool write_lo,
              bool write_hi, uint32_t w2 = 0, uint32_t w3 = 0);
// Copies `bytes` from pinned host memory to HBM on `stream`: a kernel whose
// SMs read the host memory directly (16-byte words, both pointers 16-byte
// aligned), the unaligned remainder by cudaMemcpyAsync. CPV_H2D_KERNEL=0
// uses cudaMemcpyAsync for everything.
int copy_host_to_device(cudaStream_t stream, uint8_t* dst, const uint8_t* host, uint64_t bytes);

// Exclusive scan helper (exposed for tests through the C ABI).
int scan_u32(cudaStream_t stream, const uint32_t* in, uint32_t* out, uint64_t n, uint32_t* total, Scratch& scratch);

const char* last_error();
void set_last_error(const std::string& e);

}  // namespace cpv::rt
