// runtime.cu — see runtime.h. Compiled by nvcc for sm_103a; the generic
// binning/scan/fill kernels come from cpv_bin.cuh, the pipeline-specific
// kernels from NVRTC modules built at pipeline creation.
#include "runtime.h"

#include <nvrtc.h>

#include <atomic>
#include <cstdlib>
#include <cstring>

#include "../kernels/cpv_bin.cuh"

namespace cpv::rt {

namespace {

std::mutex g_init_mutex;
bool g_initialised = false;
bool g_available = false;
std::atomic<uint64_t> g_launches{0};
thread_local std::string g_last_error;

int cuda_fail(cudaError_t e, const char* what) {
    set_last_error(std::string(what) + ": " + cudaGetErrorString(e));
    return kErrCuda;
}

#define CPV_CUDA(call)                                              \
    do {                                                            \
        cudaError_t e_ = (call);                                    \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call);         \
    } while (0)

template <typename T>
int grow(T*& ptr, uint64_t& cap, uint64_t need) {
    if (need <= cap && ptr) return kOk;
    uint64_t n = cap ? cap : 1024;
    while (n < need) n *= 2;
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    cap = 0;
    if (cudaMalloc(reinterpret_cast<void**>(&ptr), n * sizeof(T)) != cudaSuccess) {
        cudaGetLastError();
        set_last_error("cudaMalloc of binning scratch failed");
        return kErrOutOfMemory;
    }
    cap = n;
    return kOk;
}

uint32_t env_u32(const char* name, uint32_t dflt) {
    const char* v = std::getenv(name);
    if (!v || !*v) return dflt;
    return static_cast<uint32_t>(std::strtoul(v, nullptr, 0));
}

}  // namespace

const char* last_error() { return g_last_error.c_str(); }
void set_last_error(const std::string& e) { g_last_error = e; }

uint64_t launches() { return g_launches.load(); }
void count_launch(uint64_t n) { g_launches += n; }

namespace {
struct ProfileRecord {
    std::string name;
    cudaEvent_t start = nullptr, end = nullptr;
};
std::mutex g_prof_mutex;
bool g_prof_on = false;
std::vector<ProfileRecord> g_prof_records;
std::vector<cudaEvent_t> g_prof_free;
size_t g_prof_open = 0;  // markers begun and not yet ended
struct ProfileTotal {
    uint64_t count = 0;
    double ms = 0.0;
};
std::vector<std::pair<std::string, ProfileTotal>> g_prof_totals;

cudaEvent_t prof_event() {
    if (!g_prof_free.empty()) {
        cudaEvent_t e = g_prof_free.back();
        g_prof_free.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

void prof_drain() {
    for (auto& r : g_prof_records) {
        if (!r.end) continue;
        cudaEventSynchronize(r.end);
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, r.start, r.end);
        bool found = false;
        for (auto& t : g_prof_totals)
            if (t.first == r.name) {
                t.second.count++;
                t.second.ms += ms;
                found = true;
            }
        if (!found) g_prof_totals.push_back({r.name, ProfileTotal{1, ms}});
        g_prof_free.push_back(r.start);
        g_prof_free.push_back(r.end);
    }
    g_prof_records.clear();
}
}  // namespace

void profile_enable(bool on) {
    std::lock_guard<std::mutex> lock(g_prof_mutex);
    g_prof_on = on;
}
bool profile_enabled() { return g_prof_on; }

void profile_begin(cudaStream_t s, const char* name) {
    if (!g_prof_on) return;
    std::lock_guard<std::mutex> lock(g_prof_mutex);
    ProfileRecord r;
    r.name = name;
    r.start = prof_event();
    cudaEventRecord(r.start, s);
    g_prof_records.push_back(r);
    g_prof_open++;
}

void profile_end(cudaStream_t s) {
    if (!g_prof_on) return;
    std::lock_guard<std::mutex> lock(g_prof_mutex);
    // Close the innermost open marker (markers nest).
    for (size_t i = g_prof_records.size(); i-- > 0;) {
        if (g_prof_records[i].end) continue;
        g_prof_records[i].end = prof_event();
        cudaEventRecord(g_prof_records[i].end, s);
        g_prof_open--;
        break;
    }
    if (g_prof_open == 0 && g_prof_records.size() > 4096) prof_drain();
}

int profile_get(const char* name, uint64_t* count, double* ms) {
    std::lock_guard<std::mutex> lock(g_prof_mutex);
    prof_drain();
    for (auto& t : g_prof_totals)
        if (t.first == name) {
            *count = t.second.count;
            *ms = t.second.ms;
            return kOk;
        }
    *count = 0;
    *ms = 0.0;
    return kOk;
}

void profile_reset() {
    std::lock_guard<std::mutex> lock(g_prof_mutex);
    prof_drain();
    g_prof_totals.clear();
}

int init(std::string& error) {
    std::lock_guard<std::mutex> lock(g_init_mutex);
    if (g_initialised) {
        if (!g_available) error = "no CUDA device";
        return g_available ? kOk : kErrCuda;
    }
    g_initialised = true;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
        cudaGetLastError();
        error = "no CUDA device";
        return kErrCuda;
    }
    if (cudaSetDevice(0) != cudaSuccess || cudaFree(nullptr) != cudaSuccess) {
        cudaGetLastError();
        error = "cannot create a CUDA context on device 0";
        return kErrCuda;
    }
    g_available = true;
    return kOk;
}

bool available() { return g_available; }

int compile(const std::string& source, const std::string& name, std::vector<uint8_t>& cubin, std::string& log) {
    nvrtcProgram prog;
    if (nvrtcCreateProgram(&prog, source.c_str(), name.c_str(), kKernelHeaderCount, kKernelHeaderSources, kKernelHeaderNames) != NVRTC_SUCCESS) {
        log = "nvrtcCreateProgram failed";
        return kErrCompile;
    }
    // Exact binary32 semantics: no contraction, IEEE divide and square root,
    // denormals preserved.
    const char* opts[] = {"--gpu-architecture=sm_103a", "-std=c++17", "-fmad=false", "-prec-div=true", "-prec-sqrt=true",
                          "-ftz=false", "-default-device", "-lineinfo", "-diag-suppress=177", "-diag-suppress=550"};
    const nvrtcResult r = nvrtcCompileProgram(prog, static_cast<int>(sizeof(opts) / sizeof(opts[0])), opts);
    size_t log_size = 0;
    nvrtcGetProgramLogSize(prog, &log_size);
    log.assign(log_size, '\0');
    if (log_size) nvrtcGetProgramLog(prog, &log[0]);
    if (r != NVRTC_SUCCESS) {
        nvrtcDestroyProgram(&prog);
        return kErrCompile;
    }
    size_t size = 0;
    if (nvrtcGetCUBINSize(prog, &size) != NVRTC_SUCCESS || size == 0) {
        nvrtcDestroyProgram(&prog);
        log += "\nno cubin produced";
        return kErrCompile;
    }
    cubin.resize(size);
    nvrtcGetCUBIN(prog, reinterpret_cast<char*>(cubin.data()));
    nvrtcDestroyProgram(&prog);
    return kOk;
}

namespace {

bool module_u32(cudaLibrary_t lib, const char* name, uint32_t& value) {
    void* dptr = nullptr;
    size_t bytes = 0;
    if (cudaLibraryGetGlobal(&dptr, &bytes, lib, name) != cudaSuccess || bytes != 4 || cudaMemcpy(&value, dptr, 4, cudaMemcpyDeviceToHost) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return true;
}

}  // namespace

int load(const std::vector<uint8_t>& cubin, uint32_t tile_shift, bool batched, Module& out, std::string& error) {
    if (!g_available) {
        error = "no CUDA device: pipeline modules cannot be loaded";
        return kErrCuda;
    }
    cudaLibrary_t lib = nullptr;
    cudaError_t e = cudaLibraryLoadData(&lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0);
    if (e != cudaSuccess) {
        error = std::string("cudaLibraryLoadData: ") + cudaGetErrorString(e);
        cudaGetLastError();
        return kErrCuda;
    }
    out.library = lib;
    auto fail = [&](const std::string& why) {
        cudaGetLastError();
        cudaLibraryUnload(lib);
        out.library = nullptr;
        error = why;
        return kErrCuda;
    };
    bool ok;
    if (batched)
        ok = cudaLibraryGetKernel(&out.setup_rects, lib, "cpv_batch_setup") == cudaSuccess &&
             cudaLibraryGetKernel(&out.raster, lib, "cpv_batch_raster") == cudaSuccess &&
             cudaLibraryGetKernel(&out.vertex, lib, "cpv_batch_vs") == cudaSuccess && module_u32(lib, "cpv_vs_stride", out.vs_stride);
    else
        ok = cudaLibraryGetKernel(&out.setup_rects, lib, "cpv_setup_rects") == cudaSuccess &&
             cudaLibraryGetKernel(&out.raster, lib, "cpv_raster") == cudaSuccess &&
             cudaLibraryGetKernel(&out.blend_tables, lib, "cpv_blend_tables") == cudaSuccess;
    if (!ok) return fail("pipeline module lacks its kernels");
    out.batched = batched;
    out.tile_shift = tile_shift;
    if (!module_u32(lib, "cpv_raster_smem_bytes", out.raster_smem) || !module_u32(lib, "cpv_raster_threads", out.raster_threads))
        return fail("pipeline module lacks its launch-shape globals");
    // Opt in to the dynamic shared memory even below 48 KB: the kernel's
    // static shared memory counts against the same default limit.
    if (out.raster_smem > 0 &&
        cudaFuncSetAttribute(reinterpret_cast<const void*>(out.raster), cudaFuncAttributeMaxDynamicSharedMemorySize,
                             static_cast<int>(out.raster_smem)) != cudaSuccess)
        return fail("raster kernel needs more shared memory than the device allows");
    return kOk;
}

void unload(Module& m) {
    if (m.library) cudaLibraryUnload(m.library);
    m.library = nullptr;
}

Scratch::~Scratch() {
    if (!available()) return;
    cudaFree(rects_);
    cudaFree(counts_);
    cudaFree(cursor_);
    cudaFree(list_);
    for (auto* p : scan_) cudaFree(p);
    cudaFree(words_);
    cudaFree(tables_);
}

template <typename T>
int Scratch::grow_tracked(T*& ptr, uint64_t& cap, uint64_t need) {
    const T* before = ptr;
    const int r = grow(ptr, cap, need);
    if (ptr != before) generation_++;
    return r;
}

int Scratch::reserve_rects(uint64_t prims) { return grow_tracked(rects_, rects_cap_, prims * 4); }

int Scratch::reserve_bins(uint64_t entries) {
    const int r = grow_tracked(counts_, counts_cap_, entries);
    if (r != kOk) return r;
    return grow_tracked(cursor_, cursor_cap_, entries);
}

int Scratch::reserve_list(uint64_t entries) { return grow_tracked(list_, list_cap_, entries); }

int Scratch::reserve_tables(uint64_t bytes) { return grow_tracked(tables_, tables_cap_, bytes); }

int Scratch::reserve_scan(uint64_t n) {
    int level = 0;
    while (n > CPV_SCAN_BLOCK && level < 8) {
        n = (n + CPV_SCAN_BLOCK - 1) / CPV_SCAN_BLOCK;
        // two arrays per level (sums and scanned sums) share one allocation
        const int r = grow_tracked(scan_[level], scan_cap_[level], 2 * n);
        if (r != kOk) return r;
        level++;
    }
    return kOk;
}

int Scratch::ensure_words() {
    if (words_) return kOk;
    if (cudaMalloc(reinterpret_cast<void**>(&words_), kWordsBytes) != cudaSuccess) {
        cudaGetLastError();
        return kErrOutOfMemory;
    }
    cudaMemset(words_, 0, kWordsBytes);
    generation_++;
    return kOk;
}

namespace {

int scan_level(cudaStream_t stream, const uint32_t* in, uint32_t* out, uint64_t n, uint32_t* total, Scratch& sc, int level) {
    const uint64_t blocks = (n + CPV_SCAN_BLOCK - 1) / CPV_SCAN_BLOCK;
    if (blocks <= 1) {
        cpv_scan_blocks<<<1, CPV_SCAN_THREADS, 0, stream>>>(in, out, n, nullptr);
        count_launch();
    } else {
        uint32_t* sums = sc.scan_level(level);
        uint32_t* sums_scanned = sums + blocks;
        cpv_scan_blocks<<<static_cast<unsigned>(blocks), CPV_SCAN_THREADS, 0, stream>>>(in, out, n, sums);
        count_launch();
        const int r = scan_level(stream, sums, sums_scanned, blocks, nullptr, sc, level + 1);
        if (r != kOk) return r;
        cpv_scan_add<<<static_cast<unsigned>(blocks), CPV_SCAN_THREADS, 0, stream>>>(out, n, sums_scanned);
        count_launch();
    }
    if (total) {
        cpv_scan_total<<<1, 32, 0, stream>>>(in, out, n, total);
        count_launch();
    }
    return kOk;
}

}  // namespace

int scan_u32(cudaStream_t stream, const uint32_t* in, uint32_t* out, uint64_t n, uint32_t* total, Scratch& sc) {
    int r = sc.reserve_scan(n);
    if (r != kOk) return r;
    r = scan_level(stream, in, out, n, total, sc, 0);
    if (r != kOk) return r;
    CPV_CUDA(cudaGetLastError());
    return kOk;
}

int fill(cudaStream_t stream, void* dst, uint64_t texels, uint32_t texel_bytes, uint32_t lo, uint32_t hi, uint32_t w2, uint32_t w3) {
    if (!dst || texels == 0) return kOk;
    const unsigned grid = static_cast<unsigned>(texels / 256 + 1 < 152 * 16 ? texels / 256 + 1 : 152 * 16);
    switch (texel_bytes) {
    case 1:
        CPV_CUDA(cudaMemsetAsync(dst, static_cast<int>(lo & 0xFF), texels, stream));
        return kOk;
    case 2:
        cpv_fill_u16<<<grid, 256, 0, stream>>>(static_cast<uint16_t*>(dst), texels, lo);
        break;
    case 4:
        cpv_fill_u32<<<grid, 256, 0, stream>>>(static_cast<uint32_t*>(dst), texels, lo);
        break;
    case 8:
        cpv_fill_u64<<<grid, 256, 0, stream>>>(static_cast<uint2*>(dst), texels, lo, hi);
        break;
    case 16:
        cpv_fill_u128<<<grid, 256, 0, stream>>>(static_cast<uint4*>(dst), texels, make_uint4(lo, hi, w2, w3));
        break;
    default:
        return kErrInvalid;
    }
    count_launch();
    CPV_CUDA(cudaGetLastError());
    return kOk;
}

int fill_rect(cudaStream_t stream, uint8_t* base, uint64_t pitch, uint32_t w, uint32_t h, uint32_t texel_bytes, uint32_t lo, uint32_t hi, bool write_lo,
              bool write_hi, uint32_t w2, uint32_t w3) {
    if (!base || w == 0 || h == 0) return kOk;
    if (texel_bytes != 1 && texel_bytes != 2 && texel_bytes != 4 && texel_bytes != 8 && texel_bytes != 16) return kErrInvalid;
    if (reinterpret_cast<uintptr_t>(base) % texel_bytes != 0 || pitch % texel_bytes != 0 || pitch < static_cast<uint64_t>(w) * texel_bytes) return kErrInvalid;
    if (!write_lo && !(texel_bytes == 8 && write_hi)) return kOk;
    if (pitch == static_cast<uint64_t>(w) * texel_bytes && write_lo && (texel_bytes != 8 || write_hi))
        return fill(stream, base, static_cast<uint64_t>(w) * h, texel_bytes, lo, hi, w2, w3);  // contiguous: one span
    const dim3 grid((w + 255) / 256 < 8 ? (w + 255) / 256 : 8, h < 2048 ? h : 2048);
    cpv_fill_rect<<<grid, 256, 0, stream>>>(base, pitch, w, h, texel_bytes, make_uint4(lo, hi, w2, w3), write_lo ? 1u : 0u, write_hi ? 1u : 0u);
    count_launch();
    CPV_CUDA(cudaGetLastError());
    return kOk;
}

int copy_host_to_device(cudaStream_t stream, uint8_t* dst, const uint8_t* host, uint64_t bytes) {
    if (bytes == 0) return kOk;
    // The kernel reads the host memory through its device mapping: only
    // page-locked host memory the device can address qualifies.
    const uint8_t* mapped = nullptr;
    cudaPointerAttributes attr{};
    if (cudaPointerGetAttributes(&attr, host) == cudaSuccess && attr.type == cudaMemoryTypeHost && attr.devicePointer)
        mapped = static_cast<const uint8_t*>(attr.devicePointer);
    cudaGetLastError();
    const bool aligned = (reinterpret_cast<uintptr_t>(dst) % 16u) == 0 && (reinterpret_cast<uintptr_t>(mapped) % 16u) == 0;
    uint64_t words = mapped && aligned && env_u32("CPV_H2D_KERNEL", 1u) ? bytes / 16u : 0;
    if (words) {
        int sms = 0;
        CPV_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0));
        // 2 to 32 CTAs per SM measured alike (C4's 2.05 GB in 11.6 ms): the
        // link, not the SMs, sets the rate.
        uint64_t grid = static_cast<uint64_t>(sms) * 8u;
        if (grid > (words + 255) / 256) grid = (words + 255) / 256;
        cpv_copy_words<<<static_cast<unsigned>(grid), 256, 0, stream>>>(reinterpret_cast<uint4*>(dst), reinterpret_cast<const uint4*>(mapped), words);
        count_launch();
        CPV_CUDA(cudaGetLastError());
    }
    const uint64_t done = words * 16u;
    if (done < bytes) CPV_CUDA(cudaMemcpyAsync(dst + done, host + done, bytes - done, cudaMemcpyHostToDevice, stream));
    return kOk;
}

int blit(cudaStream_t stream, const CpvTexture& src, uint8_t* dst, uint32_t dst_w, uint32_t dst_h, uint32_t dst_format, const int32_t src_region[4],
         const int32_t dst_region[4], uint32_t filter) {
    CpvBlitRegion r;
    for (int i = 0; i < 4; i++) {
        r.src[i] = src_region[i];
        r.dst[i] = dst_region[i];
    }
    const uint64_t texels = static_cast<uint64_t>(std::abs(r.dst[2] - r.dst[0])) * static_cast<uint64_t>(std::abs(r.dst[3] - r.dst[1]));
    if (texels == 0) return kOk;
    if (texels > (1ull << 38)) return kErrInvalid;  // keeps the grid within 2^30 blocks
    cpv_blit<<<static_cast<unsigned>((texels + 255) / 256), 256, 0, stream>>>(src, dst, dst_w, dst_h, dst_format, r, filter);
    count_launch();
    CPV_CUDA(cudaGetLastError());
    return kOk;
}

static_assert(kWordsBytes >= 4ull * (kSumsWord + CPV_SCAN_BLOCK), "binning words hold a sum per scan element of a CTA");

namespace {

// CTAs of the per-draw binning kernels whose work is sized on the device,
// for a count matrix of at most `bins` entries: one per CPV_SCAN_BLOCK
// entries, at most one scanned CTA sum per scan element of a CTA (2048:
// about 13 per SM, enough loads in flight for an image-sized matrix). Small
// draws keep small grids, so draws of other queues run beside them.
uint32_t bin_ctas(uint64_t bins) {
    const uint64_t want = (bins + CPV_SCAN_BLOCK - 1) / CPV_SCAN_BLOCK;
    return static_cast<uint32_t>(std::max<uint64_t>(1u, std::min<uint64_t>(CPV_SCAN_BLOCK, want)));
}

// The per-draw binning after cpv_setup_rects has written the rectangles and
// their union (tile_box): count into the (union tiles x spans) matrix, scan
// it (reduce-then-scan over bin_ctas() CTAs; its size is read on the device;
// the scan leaves the counts zero again), write the lists. zero_first: the
// counts' memory is not known to be zero (the fixed scratch moves it with
// the draw's size). words: [0] pair total, [9] the reduce's CTA counter,
// [kSumsWord ..] the CTA sums.
void bin_draw(cudaStream_t stream, const uint16_t* rects, uint64_t G, uint64_t spans, uint64_t bins, const uint32_t* tile_box, uint32_t* counts,
              uint32_t* cursor, uint32_t* list, uint32_t capacity, uint32_t* words, bool zero_first) {
    const uint32_t ctas = bin_ctas(bins);
    uint32_t* sums = words + kSumsWord;
    const uint32_t sp = static_cast<uint32_t>(spans);
    if (zero_first) {
        const unsigned zero_grid = static_cast<unsigned>(std::min<uint64_t>(ctas, (bins + 255) / 256));
        profile_begin(stream, "cpv_bins_zero");
        cpv_bins_zero<<<zero_grid, 256, 0, stream>>>(counts, tile_box, sp);
        profile_end(stream);
        count_launch();
    }
    const unsigned warp_blocks = static_cast<unsigned>((spans * 32 + 255) / 256);
    profile_begin(stream, "cpv_span_count");
    cpv_span_count<<<warp_blocks, 256, 0, stream>>>(rects, G, sp, tile_box, counts);
    profile_end(stream);
    count_launch();
    profile_begin(stream, "cpv_scan");
    cpv_scan_dyn_reduce<<<ctas, CPV_SCAN_THREADS, 0, stream>>>(counts, tile_box, sp, sums, words + 9, words);
    cpv_scan_dyn_apply<<<ctas, CPV_SCAN_THREADS, 0, stream>>>(counts, cursor, tile_box, sp, sums);
    profile_end(stream);
    count_launch();
    count_launch();
    profile_begin(stream, "cpv_span_write");
    cpv_span_write<<<warp_blocks, 256, 0, stream>>>(rects, G, sp, tile_box, cursor, list, capacity, words);
    profile_end(stream);
    count_launch();
}

}  // namespace

int draw_plain(cudaStream_t stream, const Module& m, CpvDrawParams P, Scratch& sc) {
    if (P.total_prims == 0 || P.fb_width == 0 || P.fb_height == 0) return kOk;
    const uint32_t shift = m.tile_shift;
    const uint32_t tile = 1u << shift;
    P.tile_shift = shift;
    P.tiles_x = (P.fb_width + tile - 1) / tile;
    P.tiles_y = (P.fb_height + tile - 1) / tile;
    const uint64_t tiles = static_cast<uint64_t>(P.tiles_x) * P.tiles_y;
    const uint64_t G = P.total_prims;
    int r = sc.ensure_words();
    if (r != kOk) return r;
    P.status = sc.words() + 1;
    const uint32_t direct_limit = env_u32("CPV_DIRECT_LIMIT", 1u << 18);
    uint32_t direct = (G * tiles <= direct_limit) ? 1u : 0u;
    if (G > 0xFFFFFFFFull) return kErrInvalid;
    if (!direct) {
        // Spans: one warp per ~CPV_SPAN_PRIMS primitives (default 256), at
        // most 4096 spans; the (tiles x spans) count matrix grows with them.
        static const uint32_t span_prims = std::max<uint32_t>(32u, env_u32("CPV_SPAN_PRIMS", 256u));
        uint64_t spans = (G + span_prims - 1) / span_prims;
        if (spans > 4096) spans = 4096;
        if (spans < 1) spans = 1;
        // the binning kernels index the (tiles x spans) matrix in 32 bits
        while (spans > 1 && tiles * spans > 0x7FFFFFFFull) spans = (spans + 1) / 2;
        if (tiles * spans > 0x7FFFFFFFull) return kErrInvalid;
        const uint64_t bins = tiles * spans;
        const uint32_t cap = env_u32("CPV_LIST_CAPACITY", 1u << 26);
        if ((r = sc.reserve_rects(G)) != kOk) return r;
        const uint32_t* counts_before = sc.counts();
        if ((r = sc.reserve_bins(bins)) != kOk) return r;
        // the count matrix is all zero between draws (each scan zeroes what
        // it read); a new allocation starts it so
        if (sc.counts() != counts_before) CPV_CUDA(cudaMemsetAsync(sc.counts(), 0, sc.counts_capacity() * sizeof(uint32_t), stream));
        if ((r = sc.reserve_list(cap)) != kOk) return r;
        P.rects = sc.rects();
        P.spans = static_cast<uint32_t>(spans);
        P.list_capacity = sc.list_capacity();
        P.pair_total = sc.words();
        P.tile_end = sc.cursor();
        P.bin_list = sc.list();
        P.tile_box = sc.words() + 4;
        CPV_CUDA(cudaMemsetAsync(P.tile_box, 0, 4 * sizeof(uint32_t), stream));
        {
            void* args[] = {&P};
            profile_begin(stream, "cpv_setup_rects");
            CPV_CUDA(cudaLaunchKernel(reinterpret_cast<const void*>(m.setup_rects), dim3(static_cast<unsigned>((G + 255) / 256)), dim3(256), args, 0, stream));
            profile_end(stream);
            count_launch();
        }
        bin_draw(stream, sc.rects(), G, spans, bins, P.tile_box, sc.counts(), sc.cursor(), sc.list(), sc.list_capacity(), sc.words(), false);
        CPV_CUDA(cudaGetLastError());
    }
    // Blend tables: 1 KiB per primitive, built once per draw, when the
    // pipeline blends a per-primitive constant colour (up to 4 GiB of them;
    // beyond, or with CPV_BLEND_TABLES=0, the raster computes the blend).
    if (m.blend_table && m.blend_tables && env_u32("CPV_BLEND_TABLES", 1u) != 0u && G * 1024u <= (4ull << 30)) {
        if ((r = sc.reserve_tables(G * 1024u)) != kOk) return r;
        P.tables = sc.tables();
        void* args[] = {&P};
        profile_begin(stream, "cpv_blend_tables");
        CPV_CUDA(cudaLaunchKernel(reinterpret_cast<const void*>(m.blend_tables), dim3(static_cast<unsigned>((G + 255) / 256)), dim3(256), args, 0,
                                  stream));
        profile_end(stream);
        count_launch();
    }
    {
        void* args[] = {&P, &direct};
        profile_begin(stream, "cpv_raster");
        CPV_CUDA(cudaLaunchKernel(reinterpret_cast<const void*>(m.raster), dim3(static_cast<unsigned>(tiles)), dim3(m.raster_threads), args, m.raster_smem,
                                  stream));
        profile_end(stream);
        count_launch();
    }
    return kOk;
}

// ---------------------------------------------------------------------------
// Batched path.
// ---------------------------------------------------------------------------

namespace {

template <typename T>
int dev_alloc(T*& ptr, uint64_t count) {
    ptr = nullptr;
    if (count == 0) count = 1;
    if (cudaMalloc(reinterpret_cast<void**>(&ptr), count * sizeof(T)) != cudaSuccess) {
        cudaGetLastError();
        ptr = nullptr;
        set_last_error("cudaMalloc of batch buffers failed (" + std::to_string(count * sizeof(T)) + " bytes)");
        return kErrOutOfMemory;
    }
    return kOk;
}

template <typename T>
void dev_free(T*& ptr) {
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
}

}  // namespace

BatchPlan::~BatchPlan() {
    if (!available()) return;
    if (exec_) cudaGraphExecDestroy(exec_);
    if (done_) cudaEventDestroy(done_);
    dev_free(draws_);
    dev_free(pipeline_);
    dev_free(draw_block_);
    dev_free(block_draw_);
    dev_free(rects_);
    dev_free(block_pairs_);
    dev_free(block_offsets_);
    free_pairs();
    dev_free(hist_);
    dev_free(hist_offsets_);
    dev_free(tile_begin_);
    dev_free(tile_end_);
    dev_free(words_);
    dev_free(ndc_);
    dev_free(vs_pos_);
    dev_free(vs_var_);
    dev_free(vs_draw_block_);
    dev_free(vs_block_draw_);
    if (pinned_pairs_) cudaFreeHost(pinned_pairs_);
}

void BatchPlan::free_pairs() {
    for (int i = 0; i < 2; i++) {
        dev_free(keys_[i]);
        dev_free(vals_[i]);
    }
    cap_ = 0;
}

int BatchPlan::alloc_pairs(uint32_t capacity) {
    free_pairs();
    for (int i = 0; i < 2; i++) {
        int r;
        if ((r = dev_alloc(keys_[i], capacity)) != kOk || (r = dev_alloc(vals_[i], capacity)) != kOk) {
            free_pairs();
            return r;
        }
    }
    cap_ = capacity;
    P_.pair_capacity = capacity;
    return kOk;
}

int BatchPlan::build(const Module& m, const BatchDraws& in, cudaStream_t stream) {
    const uint32_t n = static_cast<uint32_t>(in.draws.size());
    if (n == 0 || in.pipeline.size() != n || !m.batched) {
        set_last_error("batch plan: empty batch or module without batched kernels");
        return kErrInvalid;
    }
    // Block layout: draw d owns blocks [draw_block[d], draw_block[d+1]).
    std::vector<uint32_t> draw_block(n + 1);
    uint64_t blocks = 0;
    prims_ = 0;
    for (uint32_t d = 0; d < n; d++) {
        draw_block[d] = static_cast<uint32_t>(blocks);
        blocks += (in.draws[d].total_prims + CPV_BATCH_BLOCK - 1) / CPV_BATCH_BLOCK;
        prims_ += in.draws[d].total_prims;
        if (blocks * CPV_BATCH_BLOCK >= (1ull << 32)) {
            set_last_error("batch plan: more than 2^32 primitives in one batch");
            return kErrInvalid;
        }
    }
    draw_block[n] = static_cast<uint32_t>(blocks);
    std::vector<uint32_t> block_draw(blocks ? blocks : 1, 0);
    for (uint32_t d = 0; d < n; d++)
        for (uint32_t b = draw_block[d]; b < draw_block[d + 1]; b++) block_draw[b] = d;
    const uint32_t tile = 1u << m.tile_shift;
    const uint32_t tiles_x = (in.fb_width + tile - 1) / tile, tiles_y = (in.fb_height + tile - 1) / tile;
    tiles_ = tiles_x * tiles_y;
    if (tiles_ == 0 || tiles_ > 65536u) {
        set_last_error("batch plan: attachment needs more than 65536 tiles");
        return kErrInvalid;
    }
    passes_ = tiles_ > 256u ? 2u : 1u;
    int r;
    if ((r = dev_alloc(draws_, n)) != kOk || (r = dev_alloc(pipeline_, n)) != kOk || (r = dev_alloc(draw_block_, n + 1)) != kOk ||
        (r = dev_alloc(block_draw_, block_draw.size())) != kOk || (r = dev_alloc(rects_, blocks * CPV_BATCH_BLOCK)) != kOk ||
        (r = dev_alloc(block_pairs_, blocks)) != kOk || (r = dev_alloc(block_offsets_, blocks)) != kOk ||
        (r = dev_alloc(tile_begin_, tiles_)) != kOk || (r = dev_alloc(tile_end_, tiles_)) != kOk || (r = dev_alloc(words_, 64)) != kOk)
        return r;
    if (cudaMallocHost(reinterpret_cast<void**>(&pinned_pairs_), 64) != cudaSuccess) {
        cudaGetLastError();
        set_last_error("batch plan: pinned word allocation failed");
        return kErrOutOfMemory;
    }
    CPV_CUDA(cudaEventCreateWithFlags(&done_, cudaEventDisableTiming));
    CPV_CUDA(cudaMemcpy(draws_, in.draws.data(), n * sizeof(CpvDrawParams), cudaMemcpyHostToDevice));
    CPV_CUDA(cudaMemcpy(pipeline_, in.pipeline.data(), n * sizeof(uint32_t), cudaMemcpyHostToDevice));
    CPV_CUDA(cudaMemcpy(draw_block_, draw_block.data(), (n + 1) * sizeof(uint32_t), cudaMemcpyHostToDevice));
    CPV_CUDA(cudaMemcpy(block_draw_, block_draw.data(), block_draw.size() * sizeof(uint32_t), cudaMemcpyHostToDevice));
    CPV_CUDA(cudaMemset(words_, 0, 64 * sizeof(uint32_t)));
    // Pixel-centre tables for the set-up's coverage pretest, with the same
    // rounded operations as cpv_pixel_ndc (IEEE binary32; the product by 2
    // is exact, so contraction cannot change a value).
    {
        std::vector<float> ndc(static_cast<size_t>(in.fb_width) + in.fb_height);
        auto centre = [](uint32_t i, float extent) {
            const float half = (1.0f / extent) * 0.5f;
            const float q = static_cast<float>(i) / extent;
            const float s = q + half;
            return s * 2.0f - 1.0f;
        };
        for (uint32_t x = 0; x < in.fb_width; x++) ndc[x] = centre(x, in.vw);
        for (uint32_t y = 0; y < in.fb_height; y++) ndc[in.fb_width + y] = centre(y, in.vh);
        if ((r = dev_alloc(ndc_, ndc.size())) != kOk) return r;
        CPV_CUDA(cudaMemcpy(ndc_, ndc.data(), ndc.size() * sizeof(float), cudaMemcpyHostToDevice));
    }

    int sms = 0, per_sm = 0;
    CPV_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0));
    CPV_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, reinterpret_cast<const void*>(m.raster), static_cast<int>(m.raster_threads),
                                                           m.raster_smem));
    if (per_sm < 1) per_sm = 1;
    raster_ctas_ = static_cast<uint32_t>(sms * per_sm);
    if (raster_ctas_ > tiles_) raster_ctas_ = tiles_;
    radix_ctas_ = static_cast<uint32_t>(sms * 4);
    if ((r = dev_alloc(hist_, static_cast<uint64_t>(CPV_RADIX_DIGITS) * radix_ctas_)) != kOk ||
        (r = dev_alloc(hist_offsets_, static_cast<uint64_t>(CPV_RADIX_DIGITS) * radix_ctas_)) != kOk)
        return r;
    // Scan levels for both scans, reserved now so that no launch allocates.
    if ((r = scan_.reserve_scan(blocks)) != kOk || (r = scan_.reserve_scan(static_cast<uint64_t>(CPV_RADIX_DIGITS) * radix_ctas_)) != kOk) return r;

    P_ = CpvBatchParams{};
    P_.draws = draws_;
    P_.draw_pipeline = pipeline_;
    P_.draw_block = draw_block_;
    P_.block_draw = block_draw_;
    P_.num_draws = n;
    P_.total_blocks = static_cast<uint32_t>(blocks);
    P_.color = in.color;
    P_.depth = in.depth;
    for (int k = 0; k < CPV_MAX_CA - 1; k++) P_.color_extra[k] = in.color_extra[k];
    P_.fb_width = in.fb_width;
    P_.fb_height = in.fb_height;
    P_.vw = in.vw;
    P_.vh = in.vh;
    P_.tiles_x = tiles_x;
    P_.tiles_y = tiles_y;
    P_.rects = rects_;
    P_.block_pairs = block_pairs_;
    P_.block_offsets = block_offsets_;
    P_.pair_total = words_;
    P_.tile_begin = tile_begin_;
    P_.tile_end = tile_end_;
    P_.tile_counter = words_ + 2;
    P_.status = words_ + 1;
    P_.ndc_x = ndc_;
    P_.ndc_y = ndc_ + in.fb_width;

    if ((r = build_vertex_stage(m, in, stream)) != kOk) return r;

    // One set-up run (after the vertex stage it reads) to size the pair buffers.
    if (blocks) {
        void* args[] = {&P_};
        if (P_.vs_blocks) {
            CPV_CUDA(cudaLaunchKernel(reinterpret_cast<const void*>(m.vertex), dim3(P_.vs_blocks), dim3(CPV_BATCH_BLOCK), args, 0, stream));
            count_launch();
        }
        CPV_CUDA(cudaLaunchKernel(reinterpret_cast<const void*>(m.setup_rects), dim3(static_cast<unsigned>(blocks)), dim3(CPV_BATCH_BLOCK), args, 0, stream));
        count_launch();
        if ((r = scan_u32(stream, block_pairs_, block_offsets_, blocks, words_, scan_)) != kOk) return r;
    }
    CPV_CUDA(cudaMemcpyAsync(pinned_pairs_, words_, 4, cudaMemcpyDeviceToHost, stream));
    CPV_CUDA(cudaStreamSynchronize(stream));
    const uint64_t pairs = *pinned_pairs_;
    uint64_t cap = pairs + pairs / 4 + (1u << 20);
    if (cap > 0xFFFFFFFFull) cap = 0xFFFFFFFFull;
    // CPV_BATCH_PAIR_CAPACITY forces a capacity (tests of the overflow path).
    if (const uint32_t forced = env_u32("CPV_BATCH_PAIR_CAPACITY", 0u)) cap = forced;
    return alloc_pairs(static_cast<uint32_t>(cap));
}

// The vertex stage: every vertex id of a triangle draw's range, of every
// instance, is shaded once per frame into a slot (NDC position and clip w,
// then the outputs), which the set-up and raster kernels read instead of
// shading the vertex for each triangle and each tile that uses it. A draw
// gets slots when its pipeline assembles triangles and its vertex ids form a
// range no wider than twice its primitives per instance plus 2 (an icosphere
// or a grid uses each vertex in about six triangles; a non-indexed triangle
// list uses each once and is left to the set-up). For an indexed draw the
// range is that of the index values it reads now; a vertex outside it (the
// indices rewritten later) is shaded by the set-up itself, so slots change
// no result. CPV_VERTEX_STAGE=0 turns the stage off.
int BatchPlan::build_vertex_stage(const Module& m, const BatchDraws& in, cudaStream_t stream) {
    const uint32_t n = static_cast<uint32_t>(in.draws.size());
    vs_slots_ = 0;
    P_.vs_blocks = 0;
    if (!m.vertex || !env_u32("CPV_VERTEX_STAGE", 1u) || in.triangles.size() != n) return kOk;
    std::vector<uint8_t> want(n, 0);
    bool any_indexed = false;
    for (uint32_t d = 0; d < n; d++) {
        if (in.triangles[d] && in.draws[d].total_prims && in.draws[d].index_size) {
            want[d] = 1;
            any_indexed = true;
        }
    }
    std::vector<uint2> range(n, make_uint2(0xFFFFFFFFu, 0u));
    if (any_indexed) {
        uint8_t* want_d = nullptr;
        uint2* range_d = nullptr;
        int r;
        if ((r = dev_alloc(want_d, n)) != kOk) return r;
        if ((r = dev_alloc(range_d, n)) != kOk) {
            dev_free(want_d);
            return r;
        }
        bool ok = cudaMemcpyAsync(want_d, want.data(), n, cudaMemcpyHostToDevice, stream) == cudaSuccess;
        if (ok) {
            cpv_index_range<<<n, 256, 0, stream>>>(draws_, want_d, range_d);
            count_launch();
            ok = cudaGetLastError() == cudaSuccess &&
                 cudaMemcpyAsync(range.data(), range_d, n * sizeof(uint2), cudaMemcpyDeviceToHost, stream) == cudaSuccess &&
                 cudaStreamSynchronize(stream) == cudaSuccess;
        }
        dev_free(want_d);
        dev_free(range_d);
        if (!ok) {
            cudaGetLastError();
            set_last_error("batch plan: index range pass failed");
            return kErrCuda;
        }
    }
    const uint32_t trim = env_u32("CPV_VS_TRIM", 0u);
    std::vector<uint32_t> lo(n, 0), count(n, 0);
    std::vector<uint64_t> base(n, 0);
    uint64_t total = 0, blocks = 0;
    std::vector<uint32_t> draw_block(n + 1, 0);
    for (uint32_t d = 0; d < n; d++) {
        const CpvDrawParams& P = in.draws[d];
        uint64_t c = 0;
        uint32_t l = 0;
        if (in.triangles[d] && P.total_prims) {
            if (P.index_size == 0u) {
                l = P.first;
                c = P.count;
            } else if (range[d].x <= range[d].y) {
                l = static_cast<uint32_t>(P.vertex_offset) + range[d].x;
                c = static_cast<uint64_t>(range[d].y) - range[d].x + 1u;
            }
        }
        // CPV_VS_TRIM narrows every range by that many ids at each end
        // (tests of the set-up shading the vertices outside a range).
        if (trim) {
            if (c > 2ull * trim) {
                l += trim;
                c -= 2ull * trim;
            } else {
                c = 0;
            }
        }
        const uint64_t inst = P.instance_count > 1u ? P.instance_count : 1u;
        if (c > 2ull * P.prims_per_instance + 2u || c * inst >= (1ull << 32)) c = 0;
        lo[d] = l;
        count[d] = static_cast<uint32_t>(c);
        base[d] = total;
        total += c * inst;
        draw_block[d] = static_cast<uint32_t>(blocks);
        blocks += (c * inst + CPV_BATCH_BLOCK - 1) / CPV_BATCH_BLOCK;
    }
    draw_block[n] = static_cast<uint32_t>(blocks);
    const uint64_t stride = m.vs_stride;
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
        cudaGetLastError();
        return kOk;
    }
    if (total == 0 || blocks >= (1ull << 31) || total * (16u + 4u * stride) > free_b / 2) return kOk;  // no slots: the set-up shades
    std::vector<uint32_t> block_draw(blocks);
    for (uint32_t d = 0; d < n; d++)
        for (uint32_t b = draw_block[d]; b < draw_block[d + 1]; b++) block_draw[b] = d;
    if (dev_alloc(vs_pos_, total * 4u) != kOk || (stride && dev_alloc(vs_var_, total * stride) != kOk) ||
        dev_alloc(vs_draw_block_, n + 1) != kOk || dev_alloc(vs_block_draw_, blocks) != kOk) {
        dev_free(vs_pos_);
        dev_free(vs_var_);
        dev_free(vs_draw_block_);
        dev_free(vs_block_draw_);
        return kOk;  // no slots: the set-up shades
    }
    std::vector<CpvDrawParams> draws = in.draws;
    for (uint32_t d = 0; d < n; d++) {
        if (!count[d]) continue;
        draws[d].vs_pos = vs_pos_ + 4u * base[d];
        draws[d].vs_var = stride ? vs_var_ + stride * base[d] : nullptr;
        draws[d].vs_lo = lo[d];
        draws[d].vs_count = count[d];
        draws[d].vs_stride = static_cast<uint32_t>(stride);
    }
    CPV_CUDA(cudaMemcpy(draws_, draws.data(), n * sizeof(CpvDrawParams), cudaMemcpyHostToDevice));
    CPV_CUDA(cudaMemcpy(vs_draw_block_, draw_block.data(), (n + 1) * sizeof(uint32_t), cudaMemcpyHostToDevice));
    CPV_CUDA(cudaMemcpy(vs_block_draw_, block_draw.data(), blocks * sizeof(uint32_t), cudaMemcpyHostToDevice));
    P_.vs_draw_block = vs_draw_block_;
    P_.vs_block_draw = vs_block_draw_;
    P_.vs_blocks = static_cast<uint32_t>(blocks);
    vs_slots_ = total;
    return kOk;
}

int BatchPlan::enqueue(const Module& m, cudaStream_t stream) {
    const uint32_t blocks = P_.total_blocks;
    const uint64_t before = launches();
    if (blocks == 0) {
        kernels_ = 0;
        return kOk;  // no primitive: nothing to draw
    }
    // Profile markers (only when profiling, which also bypasses the graph).
    {
        void* args[] = {&P_};
        if (P_.vs_blocks) {
            profile_begin(stream, "cpv_batch_vs");
            CPV_CUDA(cudaLaunchKernel(reinterpret_cast<const void*>(m.vertex), dim3(P_.vs_blocks), dim3(CPV_BATCH_BLOCK), args, 0, stream));
            profile_end(stream);
            count_launch();
        }
        profile_begin(stream, "cpv_batch_setup");
        CPV_CUDA(cudaLaunchKernel(reinterpret_cast<const void*>(m.setup_rects), dim3(blocks), dim3(CPV_BATCH_BLOCK), args, 0, stream));
        profile_end(stream);
        count_launch();
    }
    profile_begin(stream, "cpv_batch_bin");
    int r = scan_u32(stream, block_pairs_, block_offsets_, blocks, words_, scan_);
    if (r != kOk) return r;
    cpv_batch_emit<<<blocks, 256, 0, stream>>>(rects_, block_pairs_, block_offsets_, P_.tiles_x, keys_[0], vals_[0], cap_, words_);
    count_launch();
    for (uint32_t pass = 0; pass < passes_; pass++) {
        const uint32_t src = pass & 1u, dst = src ^ 1u;
        cpv_radix_hist<<<radix_ctas_, CPV_RADIX_THREADS, 0, stream>>>(keys_[src], words_, cap_, 8u * pass, hist_);
        count_launch();
        r = scan_u32(stream, hist_, hist_offsets_, static_cast<uint64_t>(CPV_RADIX_DIGITS) * radix_ctas_, nullptr, scan_);
        if (r != kOk) return r;
        cpv_radix_scatter<<<radix_ctas_, CPV_RADIX_THREADS, 0, stream>>>(keys_[src], vals_[src], keys_[dst], vals_[dst], words_, cap_, 8u * pass,
                                                                       hist_offsets_);
        count_launch();
    }
    const uint32_t fin = passes_ & 1u;
    P_.sorted_prims = vals_[fin];
    CPV_CUDA(cudaMemsetAsync(tile_begin_, 0, tiles_ * sizeof(uint32_t), stream));
    CPV_CUDA(cudaMemsetAsync(tile_end_, 0, tiles_ * sizeof(uint32_t), stream));
    cpv_tile_ranges<<<radix_ctas_, 256, 0, stream>>>(keys_[fin], words_, cap_, tile_begin_, tile_end_);
    count_launch();
    CPV_CUDA(cudaMemsetAsync(words_ + 2, 0, sizeof(uint32_t), stream));
    profile_end(stream);
    {
        void* args[] = {&P_};
        profile_begin(stream, "cpv_batch_raster");
        CPV_CUDA(cudaLaunchKernel(reinterpret_cast<const void*>(m.raster), dim3(raster_ctas_), dim3(m.raster_threads), args, m.raster_smem, stream));
        profile_end(stream);
        count_launch();
    }
    CPV_CUDA(cudaMemcpyAsync(pinned_pairs_, words_, 4, cudaMemcpyDeviceToHost, stream));
    CPV_CUDA(cudaGetLastError());
    kernels_ = static_cast<uint32_t>(launches() - before);
    return kOk;
}

namespace {
std::atomic<uint64_t> g_stat_prims{0}, g_stat_slots{0}, g_stat_pairs{0};
}

void batch_stats(uint64_t out[3]) {
    out[0] = g_stat_prims.load();
    out[1] = g_stat_slots.load();
    out[2] = g_stat_pairs.load();
}

int BatchPlan::launch(const Module& m, cudaStream_t stream) {
    // Statistics of the last completed launch (cpv_batch_stats).
    if (cudaEventQuery(done_) == cudaSuccess) {
        g_stat_prims = prims_;
        g_stat_slots = vs_slots_;
        g_stat_pairs = *pinned_pairs_;
    }
    cudaGetLastError();
    // An earlier launch that needed more pairs than the buffers hold rendered
    // correctly through the rectangle scan; grow the buffers for the next.
    if (exec_ && cudaEventQuery(done_) == cudaSuccess && *pinned_pairs_ > cap_) {
        const uint64_t pairs = *pinned_pairs_;
        uint64_t cap = pairs + pairs / 4 + (1u << 20);
        if (cap > 0xFFFFFFFFull) cap = 0xFFFFFFFFull;
        cudaGraphExecDestroy(exec_);
        exec_ = nullptr;
        const int r = alloc_pairs(static_cast<uint32_t>(cap));
        if (r != kOk) return r;
    }
    cudaGetLastError();
    if (profile_enabled()) {
        // Per-kernel timing needs the events between the kernels: run eagerly.
        const int r = enqueue(m, stream);
        if (r != kOk) return r;
        CPV_CUDA(cudaEventRecord(done_, stream));
        return kOk;
    }
    if (!exec_ && env_u32("CPV_BATCH_GRAPH", 1u)) {
        // Capture the sequence once; later launches replay the graph.
        cudaGraph_t graph = nullptr;
        const uint64_t before = launches();
        CPV_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
        const int r = enqueue(m, stream);
        const cudaError_t e = cudaStreamEndCapture(stream, &graph);
        g_launches -= launches() - before;  // captured, not launched yet
        if (r != kOk || e != cudaSuccess) {
            if (graph) cudaGraphDestroy(graph);
            cudaGetLastError();
            if (r != kOk) return r;
            return cuda_fail(e, "cudaStreamEndCapture");
        }
        const cudaError_t ie = cudaGraphInstantiate(&exec_, graph, 0);
        cudaGraphDestroy(graph);
        if (ie != cudaSuccess) {
            exec_ = nullptr;
            return cuda_fail(ie, "cudaGraphInstantiate");
        }
    }
    if (exec_) {
        CPV_CUDA(cudaGraphLaunch(exec_, stream));
        count_launch(kernels_);
    } else {
        const int r = enqueue(m, stream);
        if (r != kOk) return r;
    }
    CPV_CUDA(cudaEventRecord(done_, stream));
    return kOk;
}

// ---------------------------------------------------------------------------
// Fixed binning scratch for submissions that may not allocate.
//
// One file-scope device array per device holds every per-draw scratch buffer
// of the binning path. It is carved per draw, 256-byte aligned:
//   words  (256 B)            [0] pair total (written by the scan before the
//                             raster reads it), [1] status word
//   rects  (8 B / primitive)  tile rectangles, written by cpv_setup_rects
//   counts (4 B / tile·span)  bin counters: MUST start at zero; zeroed on
//                             the stream at the start of every draw
//   cursor (4 B / tile·span)  scanned counts, then write cursors
//   scan   (per level)        block sums of the multi-level scan
//   list   (the rest)         bin list; when the draw produces more
//                             (primitive, tile) pairs than fit, the raster
//                             walks the tile rectangles instead (same
//                             image, slower)
// Nothing else in the array needs an initial value.
// ---------------------------------------------------------------------------

static __device__ __align__(256) uint8_t cpv_static_scratch[CPV_STATIC_SCRATCH_BYTES];

namespace {

constexpr int kMaxStaticDevices = 64;
std::mutex g_static_mutex;
uint8_t* g_static_addr[kMaxStaticDevices] = {};

uint64_t align256(uint64_t b) { return (b + 255u) & ~255ull; }

struct StaticCarve {
    uint64_t words = 0, rects = 0, counts = 0, cursor = 0, list = 0, end = 0;
};

// Offsets of the binning buffers for `prims` primitives over `bins` tile·span
// bins; end = first byte of the bin list.
StaticCarve static_carve(uint64_t prims, uint64_t bins) {
    StaticCarve c;
    uint64_t o = 0;
    c.words = o;
    o += kWordsBytes;
    c.rects = o;
    o += align256(prims * 8);
    c.counts = o;
    o += align256(bins * 4);
    c.cursor = o;
    o += align256(bins * 4);
    c.list = o;
    c.end = o;
    return c;
}

// The binning decision of draw_plain: direct (no bins) or spans per tile.
// CPV_DIRECT_LIMIT is read once per process, so the pre-check and the draw
// always take the same path.
bool static_direct(uint64_t prims, uint64_t tiles) {
    static const uint32_t limit = env_u32("CPV_DIRECT_LIMIT", 1u << 18);
    return prims * tiles <= limit;
}

// Spans for a draw in the fixed array: draw_plain's choice, halved until the
// buffers leave at least a quarter of the array for the bin list (or one
// span remains).
uint64_t static_spans(uint64_t prims, uint64_t tiles) {
    uint64_t spans = (prims + 255) / 256;
    if (spans > 4096) spans = 4096;
    if (spans < 1) spans = 1;
    while (spans > 1 && static_carve(prims, tiles * spans).end + CPV_STATIC_SCRATCH_BYTES / 4 > CPV_STATIC_SCRATCH_BYTES) spans = (spans + 1) / 2;
    return spans;
}


}  // namespace

int static_scratch_setup(std::string& error) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= kMaxStaticDevices) {
        cudaGetLastError();
        error = "static scratch set-up: no current CUDA device";
        return kErrCuda;
    }
    std::lock_guard<std::mutex> lock(g_static_mutex);
    if (g_static_addr[dev]) return kOk;
    uint8_t* ptr = nullptr;
    e = cudaGetSymbolAddress((void**)&ptr, cpv_static_scratch);
    if (e != cudaSuccess || !ptr) {
        cudaGetLastError();
        error = std::string("cudaGetSymbolAddress(cpv_static_scratch) failed: ") + cudaGetErrorString(e);
        return kErrCuda;
    }
    g_static_addr[dev] = ptr;
    return kOk;
}

int static_scratch_check(uint64_t prims, uint32_t tile_shift, uint32_t width, uint32_t height, std::string& error) {
    if (prims == 0 || width == 0 || height == 0) return kOk;
    const uint64_t tile = 1ull << tile_shift;
    const uint64_t tiles = ((width + tile - 1) / tile) * ((height + tile - 1) / tile);
    if (prims > 0xFFFFFFFFull) {
        error = "draw of " + std::to_string(prims) + " primitives exceeds 2^32 - 1";
        return kErrInvalid;
    }
    if (static_direct(prims, tiles)) return kOk;
    const uint64_t need = static_carve(prims, tiles * static_spans(prims, tiles)).end;
    if (need > CPV_STATIC_SCRATCH_BYTES) {
        error = "draw of " + std::to_string(prims) + " primitives over " + std::to_string(tiles) + " tiles needs " + std::to_string(need) +
                " bytes of binning scratch; the fixed scratch holds " + std::to_string(static_cast<uint64_t>(CPV_STATIC_SCRATCH_BYTES));
        return kErrOutOfMemory;
    }
    return kOk;
}

int draw_plain_static(cudaStream_t stream, const Module& m, CpvDrawParams P) {
    if (P.total_prims == 0 || P.fb_width == 0 || P.fb_height == 0) return kOk;
    int dev = -1;
    CPV_CUDA(cudaGetDevice(&dev));
    uint8_t* base = (dev >= 0 && dev < kMaxStaticDevices) ? g_static_addr[dev] : nullptr;
    if (!base) {
        set_last_error("static scratch used before its set-up on this device");
        return kErrInvalid;
    }
    const uint32_t shift = m.tile_shift;
    const uint32_t tile = 1u << shift;
    P.tile_shift = shift;
    P.tiles_x = (P.fb_width + tile - 1) / tile;
    P.tiles_y = (P.fb_height + tile - 1) / tile;
    const uint64_t tiles = static_cast<uint64_t>(P.tiles_x) * P.tiles_y;
    const uint64_t G = P.total_prims;
    std::string err;
    int r = static_scratch_check(G, shift, P.fb_width, P.fb_height, err);
    if (r != kOk) {
        set_last_error(err);
        return r;
    }
    uint32_t* words = reinterpret_cast<uint32_t*>(base);
    P.status = words + 1;
    uint32_t direct = static_direct(G, tiles) ? 1u : 0u;
    if (!direct) {
        const uint64_t spans = static_spans(G, tiles);
        const uint64_t bins = tiles * spans;
        const StaticCarve c = static_carve(G, bins);
        uint64_t cap = (CPV_STATIC_SCRATCH_BYTES - c.end) / 4;
        if (cap > 0xFFFFFFFFull) cap = 0xFFFFFFFFull;
        uint16_t* rects = reinterpret_cast<uint16_t*>(base + c.rects);
        uint32_t* counts = reinterpret_cast<uint32_t*>(base + c.counts);
        uint32_t* cursor = reinterpret_cast<uint32_t*>(base + c.cursor);
        uint32_t* list = reinterpret_cast<uint32_t*>(base + c.list);
        P.rects = rects;
        P.spans = static_cast<uint32_t>(spans);
        P.list_capacity = static_cast<uint32_t>(cap);
        P.pair_total = words;
        P.tile_end = cursor;
        P.bin_list = list;
        P.tile_box = words + 4;
        CPV_CUDA(cudaMemsetAsync(P.tile_box, 0, 4 * sizeof(uint32_t), stream));
        {
            void* args[] = {&P};
            CPV_CUDA(cudaLaunchKernel(reinterpret_cast<const void*>(m.setup_rects), dim3(static_cast<unsigned>((G + 255) / 256)), dim3(256), args, 0, stream));
            count_launch();
        }
        bin_draw(stream, rects, G, spans, bins, P.tile_box, counts, cursor, list, P.list_capacity, words, true);
    }
    {
        void* args[] = {&P, &direct};
        CPV_CUDA(cudaLaunchKernel(reinterpret_cast<const void*>(m.raster), dim3(static_cast<unsigned>(tiles)), dim3(m.raster_threads), args, m.raster_smem,
                                  stream));
        count_launch();
    }
    CPV_CUDA(cudaGetLastError());
    return kOk;
}

}  // namespace cpv::rt
