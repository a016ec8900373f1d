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

// Embedded device sources (generated at build time from csrc/kernels/*.cuh).
extern const char* const kDeviceHeaderName;
extern const char* const kDeviceHeaderSource;
extern const char* const kPipelineHeaderName;
extern const char* const kPipelineHeaderSource;
extern const char* const kParamsHeaderName;
extern const char* const kParamsHeaderSource;

struct Module {
    cudaLibrary_t library = nullptr;
    cudaKernel_t setup_rects = nullptr;
    cudaKernel_t raster = nullptr;
    uint32_t tile_shift = 4;
    uint32_t raster_threads = 256;
    uint32_t raster_smem = 0;  // dynamic shared memory of cpv_raster (bytes)
};

// Initialises the CUDA context on device 0 (once per process).
int init(std::string& error);
bool available();

// Compiles a pipeline translation unit with NVRTC for sm_103a.
int compile(const std::string& source, const std::string& name, std::vector<uint8_t>& cubin, std::string& log);
// Loads a cubin and resolves the pipeline kernels.
int load(const std::vector<uint8_t>& cubin, uint32_t tile_shift, Module& out, std::string& error);
void unload(Module& m);

// Grow-only device scratch owned by one queue. Draws on that queue's stream
// reuse it in stream order.
class Scratch {
public:
    ~Scratch();
    int reserve_rects(uint64_t prims);
    int reserve_bins(uint64_t entries);  // tiles * spans
    int reserve_list(uint64_t entries);
    int reserve_scan(uint64_t n);
    uint16_t* rects() const { return rects_; }
    uint32_t* counts() const { return counts_; }
    uint32_t* cursor() const { return cursor_; }
    uint32_t* list() const { return list_; }
    uint32_t list_capacity() const { return static_cast<uint32_t>(list_cap_); }
    uint32_t* words() const { return words_; }  // [0] pair total, [1] status
    uint32_t* scan_level(int level) const { return scan_[level]; }
    int ensure_words();

private:
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

// Attachment fill with an encoded texel (1, 2, 4 or 8 bytes).
int fill(cudaStream_t stream, void* dst, uint64_t texels, uint32_t texel_bytes, uint32_t lo, uint32_t hi);

// Exclusive scan helper (exposed for tests through the C ABI).
int scan_u32(cudaStream_t stream, const uint32_t* in, uint32_t* out, uint64_t n, uint32_t* total, Scratch& scratch);

const char* last_error();
void set_last_error(const std::string& e);

}  // namespace cpv::rt
