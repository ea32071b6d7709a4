// gbr_scan.cu -- bin scan: per-bin sizes -> bin-list offsets, fill cursors
// and raster work items, in one launch.
//
// Tiles of 1024 bins (one bin per thread, coalesced loads and stores of every
// per-bin array) scan locally, then chain through a decoupled look-back: a
// tile publishes its totals, sums its predecessors' totals back to the
// nearest tile that has published its inclusive prefix, and publishes its
// own.  Tiles take tickets in the order they start, so a tile only ever waits
// on tiles that are already running, and every wait is bounded (Ctl::error
// records one that gave up).  Totals are 64-bit, so a frame whose entries
// exceed the bin storage (or 2^32) is flagged, never wrapped.
//
// Replaces the reference's fixed-capacity queues: bin sizes are known before
// any entry is written (CUDAAtomicQueue.cuh:8-26 drops entries when a
// queue is full).
#include "gbr_device.cuh"
#include "gbr_kernels.h"
#include "gbr_predict.h"

namespace gbr {

namespace {

constexpr uint32_t kScanSpinLimit = 1u << 22;   // polls of one flag before a wait gives up

// Does this scan run at all this frame?  Not after an earlier scan of the
// frame gave up (Ctl::overflow is set then); exact binning behind a
// predicted pass runs only after a predicted overflow.
__device__ __forceinline__ bool scan_runs(const ScanDev& S) {
    if (S.ctl->overflow) return false;
    return S.mode != kScanExactAfterPredicted || S.ctl->pred_overflow != 0u;
}

// A wait that gave up, or a tile that found the state of an unfinished scan:
// the frame's offsets cannot be trusted.  Ctl::error reports it to the host
// (GBR_ERR_TIMEOUT); Ctl::overflow makes every later kernel of the frame
// (fused predicted pass, guarded exact passes, fill, raster, shade) return
// before it reads an offset, so nothing is written past the bin storage.
__device__ __forceinline__ void give_up(Ctl* ctl) {
    atomicOr(&ctl->error, 1u);
    atomicExch(&ctl->overflow, 1u);
}

// Entries of bin b in the predicted modes (capacity, or filled within it).
__device__ __forceinline__ uint32_t predicted_size(const ScanDev& S, uint32_t b) {
    return S.mode == kScanCapacity ? S.capacity[b] : min(S.cursors[b] - S.offsets[b], S.capacity[b]);
}

// Raster work items of a bin of c entries (an empty bin has none: its pixels
// stay empty in the merge buffer and shade to the clear colour).
__device__ __forceinline__ uint32_t bin_items(uint32_t c, uint32_t chunk) { return (c + chunk - 1u) / chunk; }

__device__ __forceinline__ void st_release(uint32_t* p, uint32_t v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ uint32_t ld_acquire(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ unsigned long long ld_relaxed(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

// Flag tag of scan number `seq`: never 0, so zeroed state never matches.
__device__ __forceinline__ uint32_t scan_tag(uint32_t seq) { return 1u + seq % 0x3FFFFFFFu; }

// Aggregates and inclusive prefixes live apart: a reader that saw the
// aggregate flag reads values the tile never changes afterwards.
__device__ __forceinline__ void publish_aggregate(ScanTile* t, unsigned long long a, unsigned long long b,
                                                  uint32_t tag) {
    t->agg_a = a;
    t->agg_b = b;
    st_release(&t->flag, (tag << 2) | kTileAggregate);   // orders the totals before the flag
}
__device__ __forceinline__ void publish_prefix(ScanTile* t, unsigned long long a, unsigned long long b, uint32_t tag) {
    t->inc_a = a;
    t->inc_b = b;
    st_release(&t->flag, (tag << 2) | kTilePrefix);
}

// Inclusive block scan of two 64-bit values over 1024 threads (warp scans +
// one warp over the 32 warp totals).  Returns the block totals.
__device__ __forceinline__ void block_scan2(unsigned long long& a, unsigned long long& b, unsigned long long* s_a,
                                            unsigned long long* s_b, unsigned long long& t0,
                                            unsigned long long& t1) {
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
#pragma unroll
    for (uint32_t d = 1; d < 32; d <<= 1) {
        const unsigned long long x = __shfl_up_sync(0xFFFFFFFFu, a, d);
        const unsigned long long y = __shfl_up_sync(0xFFFFFFFFu, b, d);
        if (lane >= d) { a += x; b += y; }
    }
    if (lane == 31u) { s_a[warp] = a; s_b[warp] = b; }
    __syncthreads();
    if (warp == 0) {
        unsigned long long x = s_a[lane], y = s_b[lane];
#pragma unroll
        for (uint32_t d = 1; d < 32; d <<= 1) {
            const unsigned long long u = __shfl_up_sync(0xFFFFFFFFu, x, d);
            const unsigned long long v = __shfl_up_sync(0xFFFFFFFFu, y, d);
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

// Exclusive prefix of tile `tile` (called by warp 0): 32 predecessors per
// round, each lane waiting for one flag; the round ends at the nearest
// published prefix (tiles before the first count as a prefix of 0).
__device__ __forceinline__ void look_back(ScanTile* tiles, uint32_t tile, uint32_t tag, Ctl* ctl, uint32_t limit,
                                          unsigned long long& ea, unsigned long long& eb) {
    const uint32_t lane = threadIdx.x & 31u;
    ea = 0;
    eb = 0;
    for (int base = (int)tile - 1;; base -= 32) {
        const int j = base - (int)lane;
        uint32_t state = kTilePrefix;
        unsigned long long va = 0, vb = 0;
        if (j >= 0) {
            uint32_t f = 0;
            for (uint32_t it = 0;; ++it) {
                f = ld_acquire(&tiles[j].flag);
                if ((f >> 2) == tag) break;
                if (it >= limit) {
                    give_up(ctl);
                    f = (tag << 2) | kTilePrefix;   // give up: the frame is flagged
                    break;
                }
                if (it >= 32u) __nanosleep(64);
            }
            state = f & 3u;
            if (state == kTilePrefix) {
                va = ld_relaxed(&tiles[j].inc_a);
                vb = ld_relaxed(&tiles[j].inc_b);
            } else {
                va = ld_relaxed(&tiles[j].agg_a);
                vb = ld_relaxed(&tiles[j].agg_b);
            }
        }
        const uint32_t pmask = __ballot_sync(0xFFFFFFFFu, state == kTilePrefix);
        const uint32_t stop = pmask ? (uint32_t)(__ffs(pmask) - 1) : 31u;
        if (lane > stop) { va = 0; vb = 0; }
#pragma unroll
        for (uint32_t d = 16; d > 0; d >>= 1) {
            va += __shfl_xor_sync(0xFFFFFFFFu, va, d);
            vb += __shfl_xor_sync(0xFFFFFFFFu, vb, d);
        }
        ea += va;
        eb += vb;
        if (pmask) return;
    }
}

}  // namespace

__global__ void __launch_bounds__(1024) scan_kernel(ScanDev S, uint32_t ntiles) {
    __shared__ unsigned long long s_a[32], s_b[32];
    __shared__ unsigned long long s_excl[2];
    __shared__ uint32_t s_tile, s_tag;
    pdl_wait();
    if (S.dirty)   // before any wait: a scan that gives up has still cleared them
        for (uint32_t b = blockIdx.x * 1024u + threadIdx.x; b < S.n; b += gridDim.x * 1024u) S.dirty[b] = 0u;
    if (S.mode == kScanPredictedItems && S.feat) {
        // the pre-pass accumulators start the next frame empty (also when
        // this frame was flagged)
        const uint32_t n = S.n;
        for (uint32_t b = blockIdx.x * 1024u + threadIdx.x; b < n; b += gridDim.x * 1024u)
#pragma unroll
            for (uint32_t k = 0; k < (uint32_t)kFeatSlots; ++k) S.feat[k * n + b] = k == 4u ? 0xFFFFFFFFu : 0u;
    }
    if (!scan_runs(S)) return;
    if (S.mode == kScanPredictedItems) {
        if (S.ctl->pred_overflow) {   // the exact pass that follows counts again
            if (blockIdx.x == 0 && threadIdx.x == 0) { S.ctl->num_visible = 0u; S.ctl->num_float_path = 0u; }
            return;
        }
    }
    ScanTile* tiles = reinterpret_cast<ScanTile*>(S.state + 1);
    if (threadIdx.x == 0) {
        s_tag = scan_tag(ld_acquire(&S.state->seq));   // read before the ticket: the last tile bumps it
        const uint32_t t = atomicAdd(&S.state->ticket, 1u);
        if (t == ntiles - 1u) atomicExch(&S.state->ticket, 0u);   // every tile holds its ticket
        if (t >= ntiles) give_up(S.ctl);   // state left by a scan that did not finish
        s_tile = t;
    }
    __syncthreads();
    const uint32_t tile = s_tile, tag = s_tag;
    if (tile >= ntiles) return;
    const uint32_t b = tile * 1024u + threadIdx.x;
    const bool exact = S.mode == kScanExact || S.mode == kScanExactAfterPredicted;
    uint32_t c = 0, it = 0;
    uint32_t sub[kCountSplit];   // exact modes: the bin's sub-counts (zeroed for the next frame)
    if (b < S.n) {
        if (exact) {
#pragma unroll
            for (uint32_t k = 0; k < kCountSplit; ++k) {
                sub[k] = 0u;
                if (k < S.split) {
                    sub[k] = S.counts[k * S.n + b];
                    S.counts[k * S.n + b] = 0u;
                    c += sub[k];
                }
            }
        } else {
            c = predicted_size(S, b);
        }
        it = bin_items(c, S.chunk);
    }
    unsigned long long ia = c, ib = it, ta, tb;
    block_scan2(ia, ib, s_a, s_b, ta, tb);
    if (threadIdx.x < 32u) {
        unsigned long long ea = 0, eb = 0;
        const bool silent = tile + 1u == S.silent_tile1;   // test hook: this tile never publishes
        if (tile == 0) {
            if (threadIdx.x == 0 && !silent) publish_prefix(&tiles[0], ta, tb, tag);
        } else {
            if (threadIdx.x == 0 && !silent) publish_aggregate(&tiles[tile], ta, tb, tag);
            look_back(tiles, tile, tag, S.ctl, S.spin_limit ? S.spin_limit : kScanSpinLimit, ea, eb);
            if (threadIdx.x == 0 && !silent) publish_prefix(&tiles[tile], ea + ta, eb + tb, tag);
        }
        if (threadIdx.x == 0) { s_excl[0] = ea; s_excl[1] = eb; }
    }
    __syncthreads();
    const unsigned long long run = s_excl[0] + ia - c;     // first entry of bin b
    const unsigned long long item = s_excl[1] + ib - it;   // first work item of bin b
    const unsigned long long total = s_excl[0] + ta, total_items = s_excl[1] + tb;
    Ctl* ctl = S.ctl;
    // offsets past the storage are written but never used: the frame is
    // flagged below and the kernels after the scan skip it
    if (b < S.n) {
        if (S.mode == kScanCapacity) {
            S.offsets[b] = (uint32_t)run;
            S.cursors[b] = (uint32_t)run;
            S.ends[b] = (uint32_t)(run + c);
        } else {
            if (exact) {
                S.offsets[b] = (uint32_t)run;
                uint32_t at = (uint32_t)run;   // each sub-counter's pairs follow the previous one's
#pragma unroll
                for (uint32_t k = 0; k < kCountSplit; ++k) {
                    if (k < S.split) S.sub_base[k * S.n + b] = at;
                    at += sub[k];
                }
            }
            if (item + it <= S.items_cap) {
                const uint32_t start = exact ? (uint32_t)run : S.offsets[b];
                const uint32_t chunk = S.chunk;
                for (uint32_t k = 0; k < it; ++k)
                    S.items[item + k] = make_uint4(b, start + k * chunk, min(chunk, c - min(c, k * chunk)), it);
            }
        }
    }
    if (tile != ntiles - 1u || threadIdx.x != 0) return;
    // the last tile holds the frame's totals
    if (S.mode == kScanCapacity) {
        ctl->pred_capacity = total;
        if (total <= S.list_cap) S.offsets[S.n] = (uint32_t)total;
        else ctl->pred_overflow = 1u;
    } else {
        // list_cap < 2^31: the offsets of a fitting frame fit 32 bits
        const bool fits = (S.mode == kScanPredictedItems || total <= S.list_cap) && total_items <= S.items_cap;
        ctl->num_pairs = total;
        ctl->num_items = fits ? (uint32_t)total_items : 0u;
        ctl->items_alloc = total_items;
        ctl->item_next = 0u;
        if (S.mode == kScanPredictedItems) {
            if (!fits) ctl->pred_overflow = 1u;   // the exact kernels that follow take over
        } else {
            if (fits) S.offsets[S.n] = (uint32_t)total;
            else ctl->overflow = 1u;
        }
    }
    atomicAdd(&S.state->seq, 1u);   // the next scan tags its flags anew
}

ScanDev scan_of(const FrameDev& F, uint32_t mode) {
    ScanDev S;
    S.counts = F.counts;
    S.sub_base = F.sub_base;
    S.split = F.count_split;
    S.capacity = F.capacity;
    S.offsets = F.offsets;
    S.cursors = F.cursors;
    S.ends = F.bin_end;
    S.items = F.items;
    S.state = F.scan_state;
    S.ctl = F.ctl;
    S.feat = F.feat;
    S.list_cap = F.list_cap;
    S.items_cap = F.items_cap;
    S.n = F.num_bins;
    S.chunk = F.chunk;
    S.mode = mode;
    S.spin_limit = F.scan_spin_limit;
    S.silent_tile1 = F.scan_silent_tile1;
    // the frame's first scan (exact, or the predicted capacities) clears
    // the drawn flags the raster sets
    S.dirty = mode == kScanExact || mode == kScanCapacity ? F.dirty_wr : nullptr;
    return S;
}

uint32_t scan_blocks(uint32_t n) { return n == 0 ? 1u : (n + 1023u) / 1024u; }

cudaError_t launch_scan(const ScanDev& S, cudaStream_t s) {
    const uint32_t ntiles = scan_blocks(S.n);
    return launch_pdl(scan_kernel, dim3(ntiles), dim3(1024), 0, s, S, ntiles);
}

}  // namespace gbr
