/*
 * cpv_bin.cuh — order-preserving sort-middle binning and the other generic
 * device kernels (scan, fills).
 *
 * Binning builds, for every screen tile, the list of primitive ids that
 * touch it, in API order — the per-pixel order the reference's serial loop
 * (CPVulkan/CommandBuffer.Draw.cpp:1526-1593) produces. Primitives are split
 * into S contiguous spans, one warp per span, and the tiles are those of the
 * union of the draw's tile rectangles (reduced by cpv_setup_rects into
 * CpvDrawParams::tile_box), numbered row-major within it:
 *
 *   1. cpv_span_count: each warp counts, per tile, the primitives of its span
 *      that touch the tile → counts[tile * S + span] (counts start zero).
 *   2. exclusive scan of counts in tile-major order (cpv_scan_dyn_reduce,
 *      cpv_scan_dyn_apply, which zeroes the counts again) → the write cursor
 *      of every (tile, span) pair; tile t's list is the contiguous range
 *      [cursor(t, 0), cursor(t + 1, 0)).
 *   3. cpv_span_write: each warp walks its span again in order and appends
 *      primitive ids at its cursors; within a warp, 32 (primitive, tile) pairs
 *      are placed per step with a match-any rank, so the order inside a span
 *      is the primitive order, and spans are laid out in span order.
 *
 * Grids are sized from host-known bounds (primitives, screen tiles, spans)
 * and the union's size is read on the device, so a draw needs no host round
 * trip and the whole sequence can be captured in a CUDA graph. The list has
 * a fixed capacity; a draw that would exceed it records the overflow and
 * the raster kernel falls back to scanning the per-primitive rectangles
 * (slower, same result).
 */
#ifndef CPV_BIN_CUH
#define CPV_BIN_CUH

#include "cpv_device.cuh"

__device__ __forceinline__ void cpv_rect_unpack(const uint16_t* rects, uint64_t g, uint32_t& x0, uint32_t& y0, uint32_t& x1, uint32_t& y1) {
    const uint2 r = reinterpret_cast<const uint2*>(rects)[g];
    x0 = r.x & 0xFFFFu;
    y0 = r.x >> 16;
    x1 = r.y & 0xFFFFu;
    y1 = r.y >> 16;
}

__device__ __forceinline__ void cpv_span_range(uint64_t total, uint32_t spans, uint32_t span, uint64_t& begin, uint64_t& end) {
    const uint64_t per = (total + spans - 1u) / spans;
    begin = per * span;
    end = begin + per;
    if (begin > total) begin = total;
    if (end > total) end = total;
}

/* Zeroes the (union tiles x spans) count matrix (grid-stride over a fixed
 * grid): for a matrix whose memory other buffers used since its last scan. */
extern "C" __global__ void __launch_bounds__(256) cpv_bins_zero(uint32_t* __restrict__ counts, const uint32_t* __restrict__ box, uint32_t spans) {
    const CpvTileBox b = cpv_tile_box(box);
    const uint64_t n = static_cast<uint64_t>(b.w) * b.h * spans;
    const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
    for (uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) counts[i] = 0u;
}

/* counts[tile * spans + span] += primitives of the span touching the tile,
 * tile numbered row-major within the union. */
extern "C" __global__ void __launch_bounds__(256) cpv_span_count(const uint16_t* __restrict__ rects, uint64_t total, uint32_t spans,
                                                                 const uint32_t* __restrict__ box, uint32_t* __restrict__ counts) {
    const uint32_t span = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t lane = threadIdx.x & 31u;
    if (span >= spans) return;
    const CpvTileBox b = cpv_tile_box(box);
    uint64_t begin, end;
    cpv_span_range(total, spans, span, begin, end);
    for (uint64_t g = begin + lane; g < end; g += 32u) {
        uint32_t x0, y0, x1, y1;
        cpv_rect_unpack(rects, g, x0, y0, x1, y1);
        for (uint32_t y = y0; y < y1; y++)
            for (uint32_t x = x0; x < x1; x++) atomicAdd(&counts[(static_cast<uint64_t>(y - b.y0) * b.w + (x - b.x0)) * spans + span], 1u);
    }
}

/* Appends primitive ids in order. cursor = scanned counts (modified in place:
 * afterwards cursor[t * spans + s] is the end of (t, s)). */
extern "C" __global__ void __launch_bounds__(256) cpv_span_write(const uint16_t* __restrict__ rects, uint64_t total, uint32_t spans,
                                                                 const uint32_t* __restrict__ box, uint32_t* __restrict__ cursor,
                                                                 uint32_t* __restrict__ list, uint32_t capacity,
                                                                 const uint32_t* __restrict__ pair_total) {
    const uint32_t span = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t lane = threadIdx.x & 31u;
    if (span >= spans) return;
    const bool overflow = *pair_total > capacity;
    const CpvTileBox b = cpv_tile_box(box);
    uint64_t begin, end;
    cpv_span_range(total, spans, span, begin, end);
    const uint32_t lt_mask = (1u << lane) - 1u;
    for (uint64_t base = begin; base < end; base += 32u) {
        const uint64_t g = base + lane;
        uint32_t x0 = 0, y0 = 0, x1 = 0, y1 = 0;
        if (g < end) cpv_rect_unpack(rects, g, x0, y0, x1, y1);
        const uint32_t w = x1 - x0;
        const uint32_t n = w * (y1 - y0);
        /* inclusive warp scan of pair counts → this lane's first pair */
        uint32_t incl = n;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t v = __shfl_up_sync(0xFFFFFFFFu, incl, o);
            if (lane >= static_cast<uint32_t>(o)) incl += v;
        }
        const uint32_t total_pairs = __shfl_sync(0xFFFFFFFFu, incl, 31);
        const uint32_t excl = incl - n;
        /* place the chunk's pairs 32 at a time, in (primitive, tile) order */
        for (uint32_t p0 = 0; p0 < total_pairs; p0 += 32u) {
            const uint32_t p = p0 + lane;
            const bool valid = p < total_pairs;
            /* owner lane: last lane whose exclusive start <= p */
            uint32_t owner = 0;
#pragma unroll
            for (int step = 16; step >= 1; step >>= 1) {
                const uint32_t cand = owner + static_cast<uint32_t>(step);
                const uint32_t cand_excl = __shfl_sync(0xFFFFFFFFu, excl, cand);
                if (cand_excl <= p) owner = cand;
            }
            /* excl is non-decreasing, so the last lane with excl <= p owns pair p
             * (lanes with no pairs share the next lane's excl and are skipped) */
            const uint32_t o_excl = __shfl_sync(0xFFFFFFFFu, excl, owner);
            const uint32_t o_x0 = __shfl_sync(0xFFFFFFFFu, x0, owner);
            const uint32_t o_y0 = __shfl_sync(0xFFFFFFFFu, y0, owner);
            const uint32_t o_w = __shfl_sync(0xFFFFFFFFu, w, owner);
            uint32_t tile = 0xFFFFFFFFu;
            if (valid) {
                const uint32_t local = p - o_excl;
                tile = (o_y0 - b.y0 + local / o_w) * b.w + (o_x0 - b.x0 + local % o_w);
            }
            const uint32_t key = valid ? tile : (0x80000000u | lane);
            const uint32_t peers = __match_any_sync(0xFFFFFFFFu, key);
            const uint32_t rank = __popc(peers & lt_mask);
            const uint32_t leader = __ffs(peers) - 1u;
            uint32_t pos = 0;
            volatile uint32_t* cur = nullptr;
            if (valid) {
                cur = &cursor[static_cast<uint64_t>(tile) * spans + span];
                pos = *cur + rank;
                if (!overflow && pos < capacity) list[pos] = static_cast<uint32_t>(base + owner);
            }
            __syncwarp();
            if (valid && lane == leader) *cur = *cur + __popc(peers);
            __syncwarp();
        }
    }
}

/* ---- exclusive scan of u32 (three-level, 2048 elements per block) ---- */

#define CPV_SCAN_THREADS 256
#define CPV_SCAN_ITEMS 8
#define CPV_SCAN_BLOCK (CPV_SCAN_THREADS * CPV_SCAN_ITEMS)

__device__ __forceinline__ uint32_t cpv_block_exclusive_scan(uint32_t v, uint32_t& block_total) {
    __shared__ uint32_t warp_sums[CPV_SCAN_THREADS / 32];
    __shared__ uint32_t total_sh;
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    uint32_t incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= static_cast<uint32_t>(o)) incl += t;
    }
    if (lane == 31u) warp_sums[warp] = incl;
    __syncthreads();
    if (warp == 0u) {
        const uint32_t s = lane < CPV_SCAN_THREADS / 32 ? warp_sums[lane] : 0u;
        uint32_t si = s;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, si, o);
            if (lane >= static_cast<uint32_t>(o)) si += t;
        }
        if (lane < CPV_SCAN_THREADS / 32) warp_sums[lane] = si - s;
        if (lane == CPV_SCAN_THREADS / 32 - 1) total_sh = si;
    }
    __syncthreads();
    const uint32_t r = warp_sums[warp] + incl - v;
    block_total = total_sh;
    __syncthreads();
    return r;
}

/* Level scan: out[i] = exclusive prefix within the block; block_sums[b] = block total. */
extern "C" __global__ void __launch_bounds__(CPV_SCAN_THREADS) cpv_scan_blocks(const uint32_t* __restrict__ in, uint32_t* __restrict__ out,
                                                                              uint64_t n, uint32_t* __restrict__ block_sums) {
    const uint64_t base = static_cast<uint64_t>(blockIdx.x) * CPV_SCAN_BLOCK + static_cast<uint64_t>(threadIdx.x) * CPV_SCAN_ITEMS;
    uint32_t v[CPV_SCAN_ITEMS];
    uint32_t sum = 0;
#pragma unroll
    for (int i = 0; i < CPV_SCAN_ITEMS; i++) {
        v[i] = (base + i < n) ? in[base + i] : 0u;
        sum += v[i];
    }
    uint32_t total = 0;
    uint32_t run = cpv_block_exclusive_scan(sum, total);
#pragma unroll
    for (int i = 0; i < CPV_SCAN_ITEMS; i++) {
        if (base + i < n) out[base + i] = run;
        run += v[i];
    }
    if (threadIdx.x == 0 && block_sums) block_sums[blockIdx.x] = total;
}

/* out[i] += add[block(i)]; optionally writes the grand total. */
extern "C" __global__ void __launch_bounds__(CPV_SCAN_THREADS) cpv_scan_add(uint32_t* __restrict__ out, uint64_t n, const uint32_t* __restrict__ add) {
    const uint64_t base = static_cast<uint64_t>(blockIdx.x) * CPV_SCAN_BLOCK;
    const uint32_t a = add[blockIdx.x];
    for (uint32_t i = threadIdx.x; i < CPV_SCAN_BLOCK; i += CPV_SCAN_THREADS) {
        if (base + i < n) out[base + i] += a;
    }
}

/* total = last exclusive prefix + last input. */
extern "C" __global__ void cpv_scan_total(const uint32_t* __restrict__ in, const uint32_t* __restrict__ out, uint64_t n, uint32_t* __restrict__ total) {
    if (threadIdx.x == 0 && blockIdx.x == 0) *total = n ? out[n - 1] + in[n - 1] : 0u;
}

/* ---- exclusive scan of the (union tiles x spans) count matrix ----
 * Its size n = union tiles x spans is known on the device only. Two
 * launches over a fixed grid of G CTAs, CTA b owning the contiguous chunk
 * [b * C, (b + 1) * C), C = ceil(n / G): (1) each CTA sums its chunk and the
 * last CTA to finish scans the G sums (the counter at *done is reset for
 * the next draw; no CTA waits on another), (2) each CTA scans its chunk
 * from its scanned sum and zeroes the counts it read, so the matrix is
 * zero again for the next draw. */

__device__ __forceinline__ void cpv_dyn_chunk(uint32_t n, uint32_t& begin, uint32_t& end) {
    const uint32_t per = (n + gridDim.x - 1u) / gridDim.x;
    begin = per * blockIdx.x;
    end = begin + per;
    if (begin > n) begin = n;
    if (end > n) end = n;
}

__device__ __forceinline__ uint32_t cpv_box_bins(const uint32_t* box, uint32_t spans) {
    const CpvTileBox b = cpv_tile_box(box);
    return b.w * b.h * spans;
}

/* 1: sums[b] = the total of CTA b's chunk; the last CTA replaces sums[0 ..
 * G) by their exclusive scan and stores the pair total (G <= CPV_SCAN_BLOCK). */
extern "C" __global__ void __launch_bounds__(CPV_SCAN_THREADS) cpv_scan_dyn_reduce(const uint32_t* __restrict__ in, const uint32_t* __restrict__ box,
                                                                                  uint32_t spans, uint32_t* sums, uint32_t* done,
                                                                                  uint32_t* __restrict__ total) {
    uint32_t begin, end;
    cpv_dyn_chunk(cpv_box_bins(box, spans), begin, end);
    uint32_t s = 0;
    /* CPV_SCAN_ITEMS independent loads in flight per thread and step */
    for (uint32_t step = begin; step < end; step += CPV_SCAN_BLOCK) {
#pragma unroll
        for (int i = 0; i < CPV_SCAN_ITEMS; i++) {
            const uint32_t k = step + static_cast<uint32_t>(i) * CPV_SCAN_THREADS + threadIdx.x;
            s += k < end ? in[k] : 0u;
        }
    }
    s = __reduce_add_sync(0xFFFFFFFFu, s);
    __shared__ uint32_t warp_sums[CPV_SCAN_THREADS / 32];
    __shared__ uint32_t last;
    if ((threadIdx.x & 31u) == 0u) warp_sums[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0u) {
        uint32_t t = 0;
        for (int w = 0; w < CPV_SCAN_THREADS / 32; w++) t += warp_sums[w];
        sums[blockIdx.x] = t;
        __threadfence();
        last = atomicAdd(done, 1u) == gridDim.x - 1u ? 1u : 0u;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    const uint32_t count = gridDim.x;
    const uint32_t base = threadIdx.x * CPV_SCAN_ITEMS;
    uint32_t v[CPV_SCAN_ITEMS];
    uint32_t sum = 0;
#pragma unroll
    for (int i = 0; i < CPV_SCAN_ITEMS; i++) {
        v[i] = base + i < count ? __ldcg(&sums[base + i]) : 0u;
        sum += v[i];
    }
    uint32_t all;
    uint32_t run = cpv_block_exclusive_scan(sum, all);
#pragma unroll
    for (int i = 0; i < CPV_SCAN_ITEMS; i++) {
        if (base + i < count) sums[base + i] = run;
        run += v[i];
    }
    if (threadIdx.x == 0u) {
        *total = all;
        *done = 0u;
    }
}

/* 2: cursor = exclusive scan of counts, CTA b's chunk offset by sums[b]
 * (CPV_SCAN_BLOCK elements per step, carried along the chunk); the counts
 * read are zeroed. */
extern "C" __global__ void __launch_bounds__(CPV_SCAN_THREADS) cpv_scan_dyn_apply(uint32_t* __restrict__ counts, uint32_t* __restrict__ cursor,
                                                                                 const uint32_t* __restrict__ box, uint32_t spans,
                                                                                 const uint32_t* __restrict__ sums) {
    uint32_t begin, end;
    cpv_dyn_chunk(cpv_box_bins(box, spans), begin, end);
    uint32_t carry = sums[blockIdx.x];
    for (uint32_t step = begin; step < end; step += CPV_SCAN_BLOCK) {
        const uint32_t base = step + threadIdx.x * CPV_SCAN_ITEMS;
        uint32_t v[CPV_SCAN_ITEMS];
        uint32_t sum = 0;
#pragma unroll
        for (int i = 0; i < CPV_SCAN_ITEMS; i++) {
            v[i] = base + i < end ? counts[base + i] : 0u;
            sum += v[i];
        }
        uint32_t all;
        uint32_t run = carry + cpv_block_exclusive_scan(sum, all);
#pragma unroll
        for (int i = 0; i < CPV_SCAN_ITEMS; i++) {
            if (base + i < end) {
                cursor[base + i] = run;
                counts[base + i] = 0u;
            }
            run += v[i];
        }
        carry += all;
    }
}

/* ---- batched binning: pairs, stable radix sort by tile, tile ranges ----
 *
 * The batched path bins every draw of a render pass at once. Set-up writes
 * one tile rectangle per primitive and the pair count of each 256-primitive
 * block; after an exclusive scan of the block counts, cpv_batch_emit writes
 * the (tile, primitive) pairs in primitive order; a stable LSD radix sort by
 * tile (8-bit digits, one or two passes) groups them by tile while keeping
 * primitive (API) order inside each tile; cpv_tile_ranges records where each
 * tile's run starts and ends. Sizes that depend on the data (the pair count)
 * are read on the device, so the sequence has fixed launch shapes and can be
 * captured in a CUDA graph. Pairs beyond the capacity are not written; the
 * raster then scans the rectangles instead (same image). */

#define CPV_RADIX_THREADS 256
#define CPV_RADIX_DIGITS 256

__device__ __forceinline__ uint32_t cpv_pairs_in_bounds(const uint32_t* pair_total, uint32_t capacity) {
    const uint32_t p = *pair_total;
    return p <= capacity ? p : 0u;
}

/* Block-wide exclusive sum over 256 threads. */
__device__ __forceinline__ uint32_t cpv_block256_exclusive(uint32_t v, uint32_t* warp_sums /* [8] */) {
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    uint32_t incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= static_cast<uint32_t>(o)) incl += t;
    }
    if (lane == 31u) warp_sums[warp] = incl;
    __syncthreads();
    uint32_t base = 0;
    for (uint32_t k = 0; k < warp; k++) base += warp_sums[k];
    return base + incl - v;
}

/* One block per 256-primitive set-up block: the block's pairs at
 * block_offsets[block] + (pairs of the block's earlier primitives). A block
 * without pairs has no rectangles written this frame and emits nothing. */
extern "C" __global__ void __launch_bounds__(256) cpv_batch_emit(const uint2* __restrict__ rects, const uint32_t* __restrict__ block_pairs,
                                                                 const uint32_t* __restrict__ block_offsets, uint32_t tiles_x,
                                                                 uint32_t* __restrict__ keys, uint32_t* __restrict__ vals, uint32_t capacity,
                                                                 const uint32_t* __restrict__ pair_total) {
    __shared__ uint32_t warp_sums[8];
    if (block_pairs[blockIdx.x] == 0u) return;
    const uint64_t g = static_cast<uint64_t>(blockIdx.x) * 256u + threadIdx.x;
    const uint2 r = rects[g];
    const uint32_t x0 = r.x & 0xFFFFu, y0 = r.x >> 16, x1 = r.y & 0xFFFFu, y1 = r.y >> 16;
    const uint32_t w = x1 - x0;
    const uint32_t n = w * (y1 - y0);
    const uint32_t excl = cpv_block256_exclusive(n, warp_sums);
    if (*pair_total > capacity) return;
    const uint32_t base = block_offsets[blockIdx.x] + excl;
    for (uint32_t k = 0; k < n; k++) {
        const uint64_t pos = static_cast<uint64_t>(base) + k;
        if (pos >= capacity) break;  /* only reachable if the pair total wrapped 32 bits */
        const uint32_t ty = y0 + k / w, tx = x0 + k % w;
        keys[pos] = ty * tiles_x + tx;
        vals[pos] = static_cast<uint32_t>(g);
    }
}

/* Vertex-stage sizing: one CTA per draw d with want[d] set finds the
 * smallest and largest index value the draw reads inside its bound index
 * buffer (indices outside the buffer read as 0 and are not counted; the
 * set-up shades any vertex outside the found range itself). Writes
 * range[d] = (min, max), or (0xFFFFFFFF, 0) when there is none. */
extern "C" __global__ void __launch_bounds__(256) cpv_index_range(const CpvDrawParams* __restrict__ draws, const uint8_t* __restrict__ want,
                                                                  uint2* __restrict__ range) {
    __shared__ uint32_t smin[8], smax[8];
    const uint32_t d = blockIdx.x;
    uint32_t lo = 0xFFFFFFFFu, hi = 0u;
    if (want[d]) {
        const CpvDrawParams& P = draws[d];
        const uint32_t size = P.index_size;
        for (uint32_t i = threadIdx.x; i < P.count; i += 256u) {
            const uint64_t off = (static_cast<uint64_t>(P.first) + i) * size;
            if (size == 0u || off + size > P.ib_bytes) continue;
            const uint32_t v = size == 2u ? static_cast<uint32_t>(__ldg(reinterpret_cast<const uint16_t*>(P.ib + off)))
                                          : __ldg(reinterpret_cast<const uint32_t*>(P.ib + off));
            lo = v < lo ? v : lo;
            hi = v > hi ? v : hi;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const uint32_t a = __shfl_xor_sync(0xFFFFFFFFu, lo, o), b = __shfl_xor_sync(0xFFFFFFFFu, hi, o);
        lo = a < lo ? a : lo;
        hi = b > hi ? b : hi;
    }
    if ((threadIdx.x & 31u) == 0u) {
        smin[threadIdx.x >> 5] = lo;
        smax[threadIdx.x >> 5] = hi;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < 8; w++) {
            lo = smin[w] < lo ? smin[w] : lo;
            hi = smax[w] > hi ? smax[w] : hi;
        }
        range[d] = make_uint2(lo, hi);
    }
}

/* Contiguous item range of CTA c of `ctas` over n items. */
__device__ __forceinline__ void cpv_cta_range(uint32_t n, uint32_t c, uint32_t ctas, uint32_t& begin, uint32_t& end) {
    const uint32_t per = (n + ctas - 1u) / ctas;
    const uint64_t b = static_cast<uint64_t>(per) * c, e = b + per;
    begin = static_cast<uint32_t>(b < n ? b : n);
    end = static_cast<uint32_t>(e < n ? e : n);
}

/* hist[digit * gridDim.x + cta] = items of the CTA's range with that digit. */
extern "C" __global__ void __launch_bounds__(CPV_RADIX_THREADS) cpv_radix_hist(const uint32_t* __restrict__ keys, const uint32_t* __restrict__ pair_total,
                                                                               uint32_t capacity, uint32_t shift, uint32_t* __restrict__ hist) {
    __shared__ uint32_t counts[CPV_RADIX_DIGITS];
    counts[threadIdx.x] = 0u;
    __syncthreads();
    uint32_t begin, end;
    cpv_cta_range(cpv_pairs_in_bounds(pair_total, capacity), blockIdx.x, gridDim.x, begin, end);
    for (uint32_t i = begin + threadIdx.x; i < end; i += CPV_RADIX_THREADS) atomicAdd(&counts[(keys[i] >> shift) & 0xFFu], 1u);
    __syncthreads();
    hist[threadIdx.x * gridDim.x + blockIdx.x] = counts[threadIdx.x];
}

/* Stable scatter: offsets = exclusive scan of hist (digit-major). Each CTA
 * walks its range in order, 256 items at a time; an item's position is its
 * digit's running offset plus the number of earlier items of the sub-chunk
 * with the same digit (earlier warps, then earlier lanes). */
extern "C" __global__ void __launch_bounds__(CPV_RADIX_THREADS) cpv_radix_scatter(const uint32_t* __restrict__ keys_in, const uint32_t* __restrict__ vals_in,
                                                                                  uint32_t* __restrict__ keys_out, uint32_t* __restrict__ vals_out,
                                                                                  const uint32_t* __restrict__ pair_total, uint32_t capacity, uint32_t shift,
                                                                                  const uint32_t* __restrict__ offsets) {
    __shared__ uint32_t running[CPV_RADIX_DIGITS];
    __shared__ uint32_t warp_count[CPV_RADIX_THREADS / 32][CPV_RADIX_DIGITS];
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    running[threadIdx.x] = offsets[threadIdx.x * gridDim.x + blockIdx.x];
    uint32_t begin, end;
    cpv_cta_range(cpv_pairs_in_bounds(pair_total, capacity), blockIdx.x, gridDim.x, begin, end);
    for (uint32_t base = begin; base < end; base += CPV_RADIX_THREADS) {
#pragma unroll
        for (uint32_t w = 0; w < CPV_RADIX_THREADS / 32; w++) warp_count[w][threadIdx.x] = 0u;
        __syncthreads();
        const uint32_t i = base + threadIdx.x;
        const bool valid = i < end;
        uint32_t key = 0, val = 0, digit = CPV_RADIX_DIGITS + lane;  /* invalid lanes never match a digit */
        if (valid) {
            key = keys_in[i];
            val = vals_in[i];
            digit = (key >> shift) & 0xFFu;
        }
        const uint32_t peers = __match_any_sync(0xFFFFFFFFu, digit);
        const uint32_t rank = __popc(peers & ((1u << lane) - 1u));
        if (valid && rank == 0u) warp_count[warp][digit] = __popc(peers);
        __syncthreads();
        if (valid) {
            uint32_t pos = running[digit] + rank;
            for (uint32_t w = 0; w < warp; w++) pos += warp_count[w][digit];
            keys_out[pos] = key;
            vals_out[pos] = val;
        }
        __syncthreads();
        uint32_t add = 0;
#pragma unroll
        for (uint32_t w = 0; w < CPV_RADIX_THREADS / 32; w++) add += warp_count[w][threadIdx.x];
        running[threadIdx.x] += add;
        __syncthreads();
    }
}

/* tile_begin / tile_end (zeroed beforehand) from the sorted keys. */
extern "C" __global__ void __launch_bounds__(256) cpv_tile_ranges(const uint32_t* __restrict__ keys, const uint32_t* __restrict__ pair_total,
                                                                  uint32_t capacity, uint32_t* __restrict__ tile_begin, uint32_t* __restrict__ tile_end) {
    const uint32_t n = cpv_pairs_in_bounds(pair_total, capacity);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t k = keys[i];
        if (i == 0u || keys[i - 1u] != k) tile_begin[k] = i;
        if (i + 1u == n || keys[i + 1u] != k) tile_end[k] = i + 1u;
    }
}

/* ---- vkCmdBlitImage (CPVulkan/CommandBuffer.cpp:32-240), colour aspect ----
 *
 * One thread per destination texel of a region (2D; the reference's third
 * axis has depth 1 and contributes an exact lerp by 0). Its source position
 * is the reference's: u = (dstX + 0.5 - dst0.x) * ((src1.x - src0.x) / (dst1.x
 * - dst0.x)) + src0.x in binary32, normalised by the source level's width,
 * and the source level is sampled as SampleImage samples it for a blit
 * (level 0 of a one-level image, the blit's filter, CLAMP_TO_EDGE). The
 * result is written through the UNORM8 encoder. `src` describes the source
 * level as level 0. */
struct CpvBlitRegion {
    int32_t src[4]; /* x0, y0, x1, y1 */
    int32_t dst[4];
};

extern "C" __global__ void __launch_bounds__(256) cpv_blit(CpvTexture src, uint8_t* __restrict__ dst, uint32_t dst_w, uint32_t dst_h,
                                                           uint32_t dst_format, CpvBlitRegion r, uint32_t filter) {
    const int32_t dw = abs(r.dst[2] - r.dst[0]), dh = abs(r.dst[3] - r.dst[1]);
    const uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (dw == 0 || dh == 0 || i >= static_cast<uint64_t>(dw) * dh) return;
    const int32_t x = static_cast<int32_t>(i % static_cast<uint64_t>(dw)), y = static_cast<int32_t>(i / static_cast<uint64_t>(dw));
    const int32_t dst_x = r.dst[2] < r.dst[0] ? x + r.dst[2] : x + r.dst[0];
    const int32_t dst_y = r.dst[3] < r.dst[1] ? y + r.dst[3] : y + r.dst[1];
    if (dst_x < 0 || dst_y < 0 || dst_x >= static_cast<int32_t>(dst_w) || dst_y >= static_cast<int32_t>(dst_h)) return;
    const float sx = __fdiv_rn(static_cast<float>(r.src[2] - r.src[0]), static_cast<float>(r.dst[2] - r.dst[0]));
    const float sy = __fdiv_rn(static_cast<float>(r.src[3] - r.src[1]), static_cast<float>(r.dst[3] - r.dst[1]));
    const float u = __fadd_rn(__fmul_rn(__fsub_rn(__fadd_rn(static_cast<float>(dst_x), 0.5f), static_cast<float>(r.dst[0])), sx),
                              static_cast<float>(r.src[0]));
    const float v = __fadd_rn(__fmul_rn(__fsub_rn(__fadd_rn(static_cast<float>(dst_y), 0.5f), static_cast<float>(r.dst[1])), sy),
                              static_cast<float>(r.src[1]));
    float value[4];
    cpv_sample_level(src, 0u, __fdiv_rn(u, __uint2float_rn(src.level_w[0])), __fdiv_rn(v, __uint2float_rn(src.level_h[0])), filter, value);
    uint32_t packed = 0u;
    const bool bgra = dst_format == CPV_FMT_B8G8R8A8_UNORM;
#pragma unroll
    for (int c = 0; c < 4; c++) {
        const int byte = (bgra && c < 3) ? 2 - c : c;
        packed |= cpv_encode_unorm(value[c], 255.0f) << (8 * byte);
    }
    reinterpret_cast<uint32_t*>(dst)[static_cast<uint64_t>(dst_y) * dst_w + dst_x] = packed;
}

/* ---- fills ---- */

extern "C" __global__ void __launch_bounds__(256) cpv_fill_u32(uint32_t* __restrict__ dst, uint64_t count, uint32_t value) {
    for (uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < count; i += static_cast<uint64_t>(gridDim.x) * blockDim.x)
        dst[i] = value;
}

extern "C" __global__ void __launch_bounds__(256) cpv_fill_u16(uint16_t* __restrict__ dst, uint64_t count, uint32_t value) {
    for (uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < count; i += static_cast<uint64_t>(gridDim.x) * blockDim.x)
        dst[i] = static_cast<uint16_t>(value);
}

extern "C" __global__ void __launch_bounds__(256) cpv_fill_u64(uint2* __restrict__ dst, uint64_t count, uint32_t lo, uint32_t hi) {
    for (uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < count; i += static_cast<uint64_t>(gridDim.x) * blockDim.x)
        dst[i] = make_uint2(lo, hi);
}

extern "C" __global__ void __launch_bounds__(256) cpv_fill_u128(uint4* __restrict__ dst, uint64_t count, uint4 value) {
    for (uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < count; i += static_cast<uint64_t>(gridDim.x) * blockDim.x)
        dst[i] = value;
}

/* Fill of a w x h texel rectangle whose rows start `pitch` bytes apart with
 * the texel v (words x, y, z, w): a 2-byte texel takes the low half of v.x;
 * 4- and 8-byte texels take v.x in their first word when write_lo, an
 * 8-byte texel v.y in its second word when write_hi (a D32 + stencil
 * texel's stencil, or an 8-byte colour texel's upper half), a 16-byte
 * texel all four words. */
extern "C" __global__ void __launch_bounds__(256) cpv_fill_rect(uint8_t* __restrict__ base, uint64_t pitch, uint32_t w, uint32_t h, uint32_t texel_bytes,
                                                                uint4 v, uint32_t write_lo, uint32_t write_hi) {
    const uint32_t lo = v.x, hi = v.y;
    /* rows over blockIdx.y, texels of a row over x */
    for (uint32_t y = blockIdx.y; y < h; y += gridDim.y) {
        uint8_t* row = base + static_cast<uint64_t>(y) * pitch;
        for (uint32_t x = blockIdx.x * blockDim.x + threadIdx.x; x < w; x += gridDim.x * blockDim.x) {
            uint8_t* p = row + static_cast<uint64_t>(x) * texel_bytes;
            if (texel_bytes == 1) {
                *p = static_cast<uint8_t>(lo);
            } else if (texel_bytes == 2) {
                *reinterpret_cast<uint16_t*>(p) = static_cast<uint16_t>(lo);
            } else if (texel_bytes == 16) {
                *reinterpret_cast<uint4*>(p) = v;
            } else {
                if (write_lo) *reinterpret_cast<uint32_t*>(p) = lo;
                if (texel_bytes == 8 && write_hi) *reinterpret_cast<uint32_t*>(p + 4) = hi;
            }
        }
    }
}

/* ---- host → HBM copy read by the SMs ----
 * Copies `words` 16-byte words from pinned host memory (device-accessible)
 * to HBM with every SM issuing loads across the chip-to-chip link. Both
 * pointers are 16-byte aligned; the caller copies any tail. */
extern "C" __global__ void __launch_bounds__(256) cpv_copy_words(uint4* __restrict__ dst, const uint4* __restrict__ src, uint64_t words) {
    const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
    uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    /* four independent loads in flight per thread */
    for (; i + 3 * stride < words; i += 4 * stride) {
        const uint4 a = src[i], b = src[i + stride], c = src[i + 2 * stride], d = src[i + 3 * stride];
        dst[i] = a;
        dst[i + stride] = b;
        dst[i + 2 * stride] = c;
        dst[i + 3 * stride] = d;
    }
    for (; i < words; i += stride) dst[i] = src[i];
}

#endif /* CPV_BIN_CUH */
