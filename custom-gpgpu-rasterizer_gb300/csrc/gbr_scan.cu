// gbr_scan.cu -- bin scan: per-bin sizes -> bin-list offsets, fill cursors
// and raster work items.
//
// Three launches over blocks of 1024 bins: block totals, one CTA that scans
// the block totals, block-local scans that write the results.  Every load
// and store of a per-bin array is coalesced whatever the number of bins
// (8,160 bins at 1080p with 16x16 bins, 129,600 at 4K with 8x8 bins, the
// bins of every scene of a batch), and the totals are 64-bit, so a frame
// whose entries exceed the bin storage (or 2^32) is flagged, never wrapped.
//
// Replaces the reference's fixed-capacity queues: bin sizes are known before
// any entry is written (CUDAAtomicQueue.cuh:8-26 drops entries when a
// queue is full).
#include "gbr_device.cuh"
#include "gbr_kernels.h"
#include "gbr_predict.h"

namespace gbr {

namespace {

// Does this scan run at all this frame?  Exact binning behind a predicted
// pass runs only after a predicted overflow.
__device__ __forceinline__ bool scan_runs(const ScanDev& S) {
    return S.mode != kScanExactAfterPredicted || S.ctl->pred_overflow != 0u;
}

__device__ __forceinline__ uint32_t bin_size(const ScanDev& S, uint32_t b) {
    switch (S.mode) {
        case kScanCapacity: return S.capacity[b];
        case kScanPredictedItems: return min(S.cursors[b] - S.offsets[b], S.capacity[b]);
        default: return S.counts[b];
    }
}

__device__ __forceinline__ uint32_t bin_items(uint32_t c, uint32_t chunk) {
    return c == 0u ? 1u : (c + chunk - 1u) / chunk;
}

// Inclusive block scan of two values over 1024 threads (warp scans + one
// warp over the 32 warp totals).  Returns the block totals through t0/t1.
template <typename T>
__device__ __forceinline__ void block_scan2(T& a, T& b, T* s_a, T* s_b, T& t0, T& t1) {
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
#pragma unroll
    for (uint32_t d = 1; d < 32; d <<= 1) {
        const T x = __shfl_up_sync(0xFFFFFFFFu, a, d);
        const T y = __shfl_up_sync(0xFFFFFFFFu, b, d);
        if (lane >= d) { a += x; b += y; }
    }
    if (lane == 31u) { s_a[warp] = a; s_b[warp] = b; }
    __syncthreads();
    if (warp == 0) {
        T x = s_a[lane], y = s_b[lane];
#pragma unroll
        for (uint32_t d = 1; d < 32; d <<= 1) {
            const T u = __shfl_up_sync(0xFFFFFFFFu, x, d);
            const T v = __shfl_up_sync(0xFFFFFFFFu, y, d);
            if (lane >= d) { x += u; y += v; }
        }
        s_a[lane] = x;
        s_b[lane] = y;
    }
    __syncthreads();
    if (warp > 0) { a += s_a[warp - 1]; b += s_b[warp - 1]; }
    t0 = s_a[31];
    t1 = s_b[31];
}

}  // namespace

// 1. Per block of 1024 bins: total size and total work items.
__global__ void __launch_bounds__(1024) scan_partial_kernel(ScanDev S) {
    __shared__ unsigned long long s_a[32], s_b[32];
    if (!scan_runs(S) || (S.mode == kScanPredictedItems && S.ctl->pred_overflow)) return;
    const uint32_t b = blockIdx.x * 1024u + threadIdx.x;
    unsigned long long c = 0, it = 0;
    if (b < S.n) {
        c = bin_size(S, b);
        it = bin_items((uint32_t)c, S.chunk);
    }
    unsigned long long ta, tb;
    block_scan2(c, it, s_a, s_b, ta, tb);
    if (threadIdx.x == 0) {
        S.partial[2u * blockIdx.x] = ta;
        S.partial[2u * blockIdx.x + 1u] = tb;
    }
}

// 2. One CTA: exclusive prefixes of the block totals (in place), the frame's
// totals, and whether they fit the storage.
__global__ void __launch_bounds__(1024) scan_top_kernel(ScanDev S, uint32_t nblk) {
    __shared__ unsigned long long s_a[32], s_b[32];
    if (!scan_runs(S) || (S.mode == kScanPredictedItems && S.ctl->pred_overflow)) return;
    const uint32_t per = (nblk + 1023u) / 1024u;
    const uint32_t k0 = threadIdx.x * per, k1 = min(k0 + per, nblk);
    unsigned long long a = 0, b = 0;
    for (uint32_t k = k0; k < k1; ++k) { a += S.partial[2u * k]; b += S.partial[2u * k + 1u]; }
    const unsigned long long own_a = a, own_b = b;
    unsigned long long total, total_items;
    block_scan2(a, b, s_a, s_b, total, total_items);
    unsigned long long run_a = a - own_a, run_b = b - own_b;
    for (uint32_t k = k0; k < k1; ++k) {
        const unsigned long long pa = S.partial[2u * k], pb = S.partial[2u * k + 1u];
        S.partial[2u * k] = run_a;
        S.partial[2u * k + 1u] = run_b;
        run_a += pa;
        run_b += pb;
    }
    if (threadIdx.x != 0) return;
    Ctl* c = S.ctl;
    if (S.mode == kScanCapacity) {
        const bool fits = total <= S.list_cap;
        c->pred_capacity = total;
        if (fits) S.offsets[S.n] = (uint32_t)total;
        else c->pred_overflow = 1u;
        return;
    }
    // list_cap < 2^31: the offsets of a fitting frame fit 32 bits
    const bool fits = (S.mode == kScanPredictedItems || total <= S.list_cap) && total_items <= S.items_cap;
    c->num_pairs = total;
    c->num_items = fits ? (uint32_t)total_items : 0u;
    c->items_alloc = total_items;
    c->item_next = 0u;
    if (S.mode == kScanPredictedItems) {
        if (!fits) c->pred_overflow = 1u;   // the exact kernels that follow take over
    } else {
        if (fits) S.offsets[S.n] = (uint32_t)total;
        else c->overflow = 1u;
    }
}

// 3. Block-local scans: offsets, cursors and work items of each bin; exact
// counts are zeroed for the next frame, pre-pass accumulators reset.
__global__ void __launch_bounds__(1024) scan_down_kernel(ScanDev S) {
    __shared__ uint32_t s_a[32], s_b[32];
    if (!scan_runs(S)) return;
    const uint32_t b = blockIdx.x * 1024u + threadIdx.x;
    if (S.mode == kScanPredictedItems) {
        if (b < S.n && S.feat) {
            const uint32_t n = S.n;
#pragma unroll
            for (uint32_t k = 0; k < (uint32_t)kFeatSlots; ++k) S.feat[k * n + b] = k == 4u ? 0xFFFFFFFFu : 0u;
        }
        if (S.ctl->pred_overflow) {   // the exact pass counts again
            if (b == 0) { S.ctl->num_visible = 0u; S.ctl->num_float_path = 0u; }
            return;
        }
    }
    const bool fits = S.mode == kScanCapacity ? S.ctl->pred_overflow == 0u
                                              : (S.mode == kScanPredictedItems || S.ctl->overflow == 0u);
    const bool exact = S.mode == kScanExact || S.mode == kScanExactAfterPredicted;
    uint32_t c = 0, it = 0;
    if (b < S.n) {
        c = bin_size(S, b);
        it = bin_items(c, S.chunk);
        if (exact) S.counts[b] = 0u;
    }
    if (!fits) return;   // uniform: the flag was settled by the previous launch
    uint32_t ic = c, iit = it, t0, t1;
    block_scan2(ic, iit, s_a, s_b, t0, t1);
    if (b >= S.n) return;
    const uint32_t run = (uint32_t)S.partial[2u * blockIdx.x] + (ic - c);
    if (S.mode == kScanCapacity) {
        S.offsets[b] = run;
        S.cursors[b] = run;
        return;
    }
    const uint32_t start = S.mode == kScanPredictedItems ? S.offsets[b] : run;
    if (exact) {
        S.offsets[b] = run;
        S.cursors[b] = run;
    }
    uint32_t item = (uint32_t)S.partial[2u * blockIdx.x + 1u] + (iit - it);
    const uint32_t chunk = S.chunk;
    for (uint32_t k = 0; k < it; ++k)
        S.items[item + k] = make_uint4(b, start + k * chunk, min(chunk, c - min(c, k * chunk)), it);
}

ScanDev scan_of(const FrameDev& F, uint32_t mode) {
    ScanDev S;
    S.counts = F.counts;
    S.capacity = F.capacity;
    S.offsets = F.offsets;
    S.cursors = F.cursors;
    S.items = F.items;
    S.partial = F.scan_partial;
    S.ctl = F.ctl;
    S.feat = F.feat;
    S.list_cap = F.list_cap;
    S.items_cap = F.items_cap;
    S.n = F.num_bins;
    S.chunk = F.chunk;
    S.mode = mode;
    return S;
}

uint32_t scan_blocks(uint32_t n) { return n == 0 ? 1u : (n + 1023u) / 1024u; }

cudaError_t launch_scan(const ScanDev& S, cudaStream_t s) {
    const uint32_t nblk = scan_blocks(S.n);
    scan_partial_kernel<<<nblk, 1024, 0, s>>>(S);
    scan_top_kernel<<<1, 1024, 0, s>>>(S, nblk);
    scan_down_kernel<<<nblk, 1024, 0, s>>>(S);
    return cudaGetLastError();
}

}  // namespace gbr
