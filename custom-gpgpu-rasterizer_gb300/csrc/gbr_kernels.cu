// gbr_kernels.cu -- the frame hot path on sm_103a.
//
//   setup_kernel : vertex stage (positions) + triangle assembly + cull +
//                  frustum reject + raster setup + depth-key bound + bin
//                  rectangle, and the count pass of exact binning (one
//                  atomic per (triangle, bin) pair, whose return -- the pair's
//                  rank in its bin -- is kept).
//   setup_rows_kernel: the same with block-private counter rows (dense
//                  frames): pairs counted per bin in shared memory, one
//                  global atomic per (block, bin) reserves the block's run.
//   scan_kernel  : (gbr_scan.cu) bin counts -> list offsets and raster work
//                  items (bin, chunk of <= queue_chunk ids).
//   list_touch_kernel: zeros the frame's list entries in whole words so the
//                  fill's scattered stores merge in L2 (frames of >= 2^20
//                  pairs).
//   fill_kernel  : second pass: each pair's id goes to its bin's offset +
//                  rank, no atomics (fill_rows_kernel: to the block's run,
//                  slots from shared-memory cursors).
//   raster_kernel: persistent CTAs pull work items; a CTA depth-sorts its
//                  chunk by the key bounds, rasterises front to back into a
//                  shared-memory tile of packed (depth key, prim id) with
//                  64-bit atomicMin (hierarchical-z rejection between phases),
//                  and publishes the tile to the merge buffer.
//   shade_kernel : each pixel's winner shaded once: colour, depth and id.
//
// Reference stages replaced: VS_Kernel, TA_Kernel, TB_Kernel,
// RA_PerTileKernel, PS_Kernel and the CLEAR_* kernels
// (CustomCUDARasterizer/CUDARenderer.cu:598-1129, launchers :1625-1966).
#include <algorithm>
#include <cstring>

#include "gbr_device.cuh"
#include "gbr_kernels.h"
#include "gbr_shade.cuh"

namespace gbr {

static int sm_count() {
    static int sms = 0;
    if (sms <= 0) {
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
            cudaGetLastError();
            sms = 152;
        }
    }
    return sms;
}

__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31u; }

__device__ __forceinline__ uint32_t find_mesh(const FrameDev& F, uint32_t prim) {
    uint32_t lo = 0, hi = F.num_meshes - 1u;
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1u) >> 1;
        if (__ldg(&F.meshes[mid].prim_base) <= prim) lo = mid; else hi = mid - 1u;
    }
    return lo;
}

// Lower bound of the depth keys any fragment of the triangle can produce.
// A pixel covered under the 16.16 rule is at most the snapping distance
// outside the float triangle, so each float edge value there is at least
// -beta with beta <= 3*2^-17*D + 2^-32 + 2^-20*D^2 (D = the triangle's
// x + y extent; snapping moves vertices <= 2^-17 px; the float evaluation
// errs by <= 4 ulp of its product terms), and the three edge values sum to
// the float area within 2^-20*D^2 each.  With g = (2^-15*D + 2^-32 +
// 2^-18*D^2)/area, every weight is >= -g and the weights sum to 1 +- g, so
// z >= zmin*(1-g) - (3g + 2^-22)*max|z_i| when zmin >= 0 (2^-22 covers the
// rounding of the fused z chain).  The key of that bound never exceeds the
// key of a fragment of the triangle, so the triangle cannot win a pixel whose
// stored key is below it.  0: no bound (float path, vertices behind z = 0);
// 0x7FFFFFFF: every fragment has z >= 1 and loses everywhere.
__device__ __forceinline__ uint32_t hiz_key(const TriSetup& t) {
    if (t.flags & kFlagFloat) return 0u;
    const float zmin = fminf(t.z0, fminf(t.z1, t.z2));
    if (!(zmin >= 0.f)) return 0u;
    const float zabs = fmaxf(fabsf(t.z0), fmaxf(fabsf(t.z1), fabsf(t.z2)));
    const float D = (max3f(t.x0, t.x1, t.x2) - min3f(t.x0, t.x1, t.x2)) + (max3f(t.y0, t.y1, t.y2) - min3f(t.y0, t.y1, t.y2)) + 1.f;
    const float g = (D * 3.0517578125e-05f + 2.3283064365386963e-10f + D * D * 3.814697265625e-06f) * t.inv_area;
    const float zb = zmin * (1.f - g) - (3.f * g + 2.384185791015625e-07f) * zabs;
    if (!(zb > 0.f)) return 0u;
    if (zb >= 1.f) return 0x7FFFFFFFu;
    return (uint32_t)__float2int_rz(__fmul_rn(zb, 2147483648.0f));
}

// Vertex stage (positions), triangle assembly, cull, frustum reject, raster
// setup record, depth-key bound and bin rectangle of triangle `prim`, then the count pass
// (MODE 0), the predicted-capacity fill (MODE 1) or the count into the
// block's shared-memory row `s_row` (MODE 2).  Called by whole warps.
// Returns the warp's visible and float-path triangle counts (bits 0-15 and
// 16-31), for the block's statistics.
template <int MODE>
__device__ __forceinline__ uint32_t setup_tri(const FrameDev& F, uint32_t prim, uint32_t walk,
                                              uint32_t* s_row = nullptr) {
    const bool in_range = prim < F.num_tris;
    uint2 rect = empty_rect();
    bool visible = false, fpath = false, no_raster = true;
    if (in_range) {
        const uint32_t mi = find_mesh(F, prim);
        const MeshDev& m = F.meshes[mi];
        uint32_t vid[3];
        tri_vertex_ids(m, prim - m.prim_base, vid);
        float nx[3], ny[3], nz[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const F3 p = fetch_position(m, vid[k]);
            const float4 c = xform_point(m.wvp, p.x, p.y, p.z);
            nx[k] = __fdiv_rn(c.x, c.w);
            ny[k] = __fdiv_rn(c.y, c.w);
            nz[k] = __fdiv_rn(c.z, c.w);
        }
        // culling (TA_Kernel, CUDARenderer.cu:759-777): BackFace and
        // FrontFace run the same test in the reference
        bool culled = false;
        if (F.cull != 2u) {
            const F3 a = f3(__fsub_rn(nx[1], nx[0]), __fsub_rn(ny[1], ny[0]), __fsub_rn(nz[1], nz[0]));
            const F3 b = f3(__fsub_rn(nx[2], nx[0]), __fsub_rn(ny[2], ny[0]), __fsub_rn(nz[2], nz[0]));
            const F3 n = normalize3(cross3(a, b));
            culled = dot3(f3(F.cam_fwd[0], F.cam_fwd[1], F.cam_fwd[2]), n) <= 0.0f;
        }
        // IsTriangleVisible (CUDAROPs.cu:168-178)
        const bool ax = (nx[0] < -1.f && nx[1] < -1.f && nx[2] < -1.f) || (nx[0] > 1.f && nx[1] > 1.f && nx[2] > 1.f);
        const bool ay = (ny[0] < -1.f && ny[1] < -1.f && ny[2] < -1.f) || (ny[0] > 1.f && ny[1] > 1.f && ny[2] > 1.f);
        const bool az = (nz[0] < 0.f && nz[1] < 0.f && nz[2] < 0.f) || (nz[0] > 1.f && nz[1] > 1.f && nz[2] > 1.f);
        visible = !culled && !ax && !ay && !az;
        if (visible) {
            const float2 s0 = to_screen(nx[0], ny[0], F.width, F.height);
            const float2 s1 = to_screen(nx[1], ny[1], F.width, F.height);
            const float2 s2 = to_screen(nx[2], ny[2], F.width, F.height);
            const int4 r = bin_rect(s0, s1, s2, F);
            const bool inside = fabsf(s0.x) < kGuardPx && fabsf(s0.y) < kGuardPx && fabsf(s1.x) < kGuardPx &&
                                fabsf(s1.y) < kGuardPx && fabsf(s2.x) < kGuardPx && fabsf(s2.y) < kGuardPx;
            float inv_area = 0.f;
            uint32_t flags;
            if (inside) {
                const int X0 = snap_fx(s0.x), Y0 = snap_fx(s0.y), X1 = snap_fx(s1.x);
                const int Y1 = snap_fx(s1.y), X2 = snap_fx(s2.x), Y2 = snap_fx(s2.y);
                // S = cross(v0 - v1, v2 - v1) of the snapped triangle: > 0 for the
                // covered winding (the three edge functions sum to S)
                const long long S = (long long)(X0 - X1) * (long long)(Y2 - Y1) -
                                    (long long)(Y0 - Y1) * (long long)(X2 - X1);
                // the float area the reference divides its weights by (CUDAROPs.cu:336)
                const float area = fabsf(__fmaf_rn(__fsub_rn(s0.x, s1.x), __fsub_rn(s0.y, s2.y),
                                                   -__fmul_rn(__fsub_rn(s0.y, s1.y), __fsub_rn(s0.x, s2.x))));
                no_raster = !(S > 0 && area > 0.f);
                inv_area = no_raster ? 0.f : __fdiv_rn(1.0f, area);
                flags = no_raster ? 0u : kFlagRaster;
            } else {
                fpath = true;
                no_raster = false;
                flags = kFlagFloat;
            }
            uint4* rec = reinterpret_cast<uint4*>(F.setup) + 3u * prim;
            rec[0] = make_uint4(__float_as_uint(s0.x), __float_as_uint(s0.y), __float_as_uint(s1.x), __float_as_uint(s1.y));
            rec[1] = make_uint4(__float_as_uint(s2.x), __float_as_uint(s2.y), __float_as_uint(nz[0]), __float_as_uint(nz[1]));
            rec[2] = make_uint4(__float_as_uint(nz[2]), __float_as_uint(inv_area), flags, mi);
            rect = pack_rect(r, no_raster);
            // the raster depth-sorts a bin's triangles by this bound before it
            // reads their records
            TriSetup t;
            t.x0 = s0.x; t.y0 = s0.y; t.x1 = s1.x; t.y1 = s1.y; t.x2 = s2.x; t.y2 = s2.y;
            t.z0 = nz[0]; t.z1 = nz[1]; t.z2 = nz[2]; t.inv_area = inv_area; t.flags = flags; t.mesh = mi;
            F.keys[prim] = hiz_key(t);
        }
        F.rects[prim] = rect;
    }
    const uint32_t counts = (uint32_t)__popc(__ballot_sync(0xFFFFFFFFu, visible)) |
                            ((uint32_t)__popc(__ballot_sync(0xFFFFFFFFu, fpath)) << 16);
    if (MODE == 0) bin_walk<0>(F, rect, 0u, visible, walk);
    else if (MODE == 2) bin_walk<4>(F, rect, 0u, visible, walk, s_row);
    else bin_walk<2>(F, rect, prim | (no_raster ? kNoRasterBit : 0u), visible, walk);
    return counts;
}

// Frame statistics of a block: its warps' counts, summed in shared memory,
// then one atomic per counter and block (not per warp: every warp of the
// grid adding to the same two words serialises at one L2 slice).
__device__ __forceinline__ void add_block_stats(Ctl* ctl, uint32_t warp_vis, uint32_t warp_fp) {
    __shared__ uint32_t s_vis, s_fp;
    if (threadIdx.x == 0) { s_vis = 0u; s_fp = 0u; }
    __syncthreads();
    if ((threadIdx.x & 31u) == 0u) {
        if (warp_vis) atomicAdd(&s_vis, warp_vis);
        if (warp_fp) atomicAdd(&s_fp, warp_fp);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        if (s_vis) atomicAdd(&ctl->num_visible, s_vis);
        if (s_fp) atomicAdd(&ctl->num_float_path, s_fp);
    }
}

template <int MODE>
__global__ void __launch_bounds__(256) setup_kernel(FrameDev F) {
    pdl_wait();
    // predicted binning: the exact pass only runs after an overflow, and the
    // predicted pass stops once an overflow is known; neither runs after a
    // scan of the frame gave up (Ctl::overflow)
    if (F.ctl->overflow) return;
    if (MODE == 0 ? (F.exact_guard && !F.ctl->pred_overflow) : (F.ctl->pred_overflow != 0u)) return;
    // a resident grid strides over the triangles, so that a guarded launch
    // that does not run costs one wave of early exits
    uint32_t vis = 0, fp = 0;
    for (uint32_t base = blockIdx.x * blockDim.x; base < F.num_tris; base += gridDim.x * blockDim.x) {
        const uint32_t c = setup_tri<MODE>(F, base + threadIdx.x, (base + threadIdx.x) >> 5);
        vis += c & 0xFFFFu;
        fp += c >> 16;
    }
    add_block_stats(F.ctl, vis, fp);
    pdl_release();
}

// Second pass of exact binning for triangle `prim`.  Called by whole warps.
__device__ __forceinline__ void fill_tri(const FrameDev& F, uint32_t prim, uint32_t walk) {
    const bool in_range = prim < F.num_tris;
    const uint2 rect = in_range ? F.rects[prim] : empty_rect();
    const uint32_t entry = prim | ((rect.y & 0x80000000u) ? kNoRasterBit : 0u);
    bin_walk<1>(F, rect, entry, in_range, walk);
}

__global__ void __launch_bounds__(256) fill_kernel(FrameDev F) {
    pdl_wait();
    if (F.ctl->overflow || (F.exact_guard && !F.ctl->pred_overflow)) return;
    for (uint32_t base = blockIdx.x * blockDim.x; base < F.num_tris; base += gridDim.x * blockDim.x)
        fill_tri(F, base + threadIdx.x, (base + threadIdx.x) >> 5);
    pdl_release();
}

// Exact binning with block-private counter rows (num_bins <= kMaxRowBins,
// one kRowThreads block per SM, F.row_blocks blocks).  The count pass counts
// the block's pairs per bin in shared memory, then takes the block's run of
// each bin it touched with one global atomic per bin (blocks start their
// sweep at different bins, so the blocks' atomics on one bin do not arrive
// together); the run's start, relative to the bin, goes to the block's row
// of F.row_base.
__global__ void __launch_bounds__(kRowThreads, 1) setup_rows_kernel(FrameDev F) {
    extern __shared__ uint32_t s_row[];
    pdl_wait();
    if (F.ctl->overflow) return;
    const uint32_t nb = F.num_bins;
    for (uint32_t b = threadIdx.x; b < nb; b += blockDim.x) s_row[b] = 0u;
    __syncthreads();
    uint32_t vis = 0, fp = 0;
    for (uint32_t base = blockIdx.x * blockDim.x; base < F.num_tris; base += gridDim.x * blockDim.x) {
        const uint32_t c = setup_tri<2>(F, base + threadIdx.x, (base + threadIdx.x) >> 5, s_row);
        vis += c & 0xFFFFu;
        fp += c >> 16;
    }
    // the list's first touch_words words (the last frame's entries), zeroed
    // for the fill as list_touch_kernel does, by a pass whose memory
    // pipeline is otherwise idle
    uint4* const zero_to = reinterpret_cast<uint4*>(F.list);
    for (uint32_t w = blockIdx.x * blockDim.x + threadIdx.x; w < F.touch_words; w += gridDim.x * blockDim.x)
        zero_to[w] = make_uint4(0u, 0u, 0u, 0u);
    __syncthreads();
    uint32_t* const row = F.row_base + (size_t)blockIdx.x * nb;
    const uint32_t shift = (uint32_t)(((unsigned long long)blockIdx.x * nb) / gridDim.x);
    for (uint32_t i = threadIdx.x; i < nb; i += blockDim.x) {
        uint32_t b = i + shift;
        if (b >= nb) b -= nb;
        const uint32_t c = s_row[b];
        if (c) row[b] = atomicAdd(&F.counts[b], c);
    }
    add_block_stats(F.ctl, vis, fp);
    pdl_release();
}

// The fill pass of block-private rows: the same blocks walk the same
// triangles; each bin's cursor starts at the bin's offset plus the block's
// run start, and every pair takes the next slot with a shared-memory atomic.
// Cursors of bins the block never touched hold unused values.
__global__ void __launch_bounds__(kRowThreads, 1) fill_rows_kernel(FrameDev F) {
    extern __shared__ uint32_t s_row[];
    pdl_wait();
    if (F.ctl->overflow) return;
    const uint32_t nb = F.num_bins;
    const uint32_t* const row = F.row_base + (size_t)blockIdx.x * nb;
    for (uint32_t b = threadIdx.x; b < nb; b += blockDim.x) s_row[b] = __ldg(F.offsets + b) + __ldg(row + b);
    __syncthreads();
    for (uint32_t base = blockIdx.x * blockDim.x; base < F.num_tris; base += gridDim.x * blockDim.x) {
        const uint32_t prim = base + threadIdx.x;
        const bool in_range = prim < F.num_tris;
        const uint2 rect = in_range ? F.rects[prim] : empty_rect();
        const uint32_t entry = prim | ((rect.y & 0x80000000u) ? kNoRasterBit : 0u);
        bin_walk<5>(F, rect, entry, in_range, prim >> 5, s_row);
    }
    pdl_release();
}

// Predicted-capacity binning on block-private counter rows, in one launch:
// the count pass of setup_rows_kernel (setup + each pair counted in the
// block's shared-memory row), then one run per bin the block touched,
// reserved with a global atomic on the bin's cursor (which the capacity
// scan set to the bin's offset) and checked against the bin's end (offset +
// predicted capacity), then the fill pass of fill_rows_kernel over the same
// triangles, slots handed out from shared-memory cursors.  Against exact
// binning it saves the scan between count and fill and the second launch;
// against one returning global atomic per pair (setup_kernel<1>) it needs
// one per (block, bin).  A block whose run does not fit raises
// Ctl::pred_overflow and writes nothing (the exact kernels queued behind
// re-bin the frame); the other blocks' runs lie inside their capacities.
__global__ void __launch_bounds__(kRowThreads, 1) predicted_rows_kernel(FrameDev F) {
    extern __shared__ uint32_t s_row[];
    __shared__ uint32_t s_ovf;
    pdl_wait();
    if (F.ctl->overflow || F.ctl->pred_overflow) return;   // block-uniform
    const uint32_t nb = F.num_bins, tid = threadIdx.x;
    for (uint32_t b = tid; b < nb; b += kRowThreads) s_row[b] = 0u;
    if (tid == 0) s_ovf = 0u;
    __syncthreads();
    uint32_t vis = 0, fp = 0;
    for (uint32_t base = blockIdx.x * kRowThreads; base < F.num_tris; base += gridDim.x * kRowThreads) {
        const uint32_t c = setup_tri<2>(F, base + tid, (base + tid) >> 5, s_row);
        vis += c & 0xFFFFu;
        fp += c >> 16;
    }
    __syncthreads();
    // one run per bin the block touched (blocks start their sweep at
    // different bins); a thread's atomics are issued back to back
    const uint32_t shift = (uint32_t)(((unsigned long long)blockIdx.x * nb) / gridDim.x);
    for (uint32_t i0 = 0; i0 < nb; i0 += 8u * kRowThreads) {
        uint32_t bb[8], cc[8], rr[8];
#pragma unroll
        for (uint32_t u = 0; u < 8u; ++u) {
            const uint32_t i = i0 + u * kRowThreads + tid;
            uint32_t b = i + shift;
            if (b >= nb) b -= nb;
            bb[u] = b;
            cc[u] = i < nb ? s_row[b] : 0u;
        }
#pragma unroll
        for (uint32_t u = 0; u < 8u; ++u)
            if (cc[u]) rr[u] = atomicAdd(&F.cursors[bb[u]], cc[u]);
#pragma unroll
        for (uint32_t u = 0; u < 8u; ++u) {
            if (!cc[u]) continue;
            if ((unsigned long long)rr[u] + cc[u] > __ldg(&F.bin_end[bb[u]])) {
                s_ovf = 1u;
                atomicOr(&F.ctl->pred_overflow, 1u);
            }
            s_row[bb[u]] = rr[u];
        }
    }
    __syncthreads();
    if (!s_ovf) {
        for (uint32_t base = blockIdx.x * kRowThreads; base < F.num_tris; base += gridDim.x * kRowThreads) {
            const uint32_t prim = base + tid;
            const bool in_range = prim < F.num_tris;
            const uint2 rect = in_range ? F.rects[prim] : empty_rect();
            const uint32_t entry = prim | ((rect.y & 0x80000000u) ? kNoRasterBit : 0u);
            bin_walk<5>(F, rect, entry, in_range, prim >> 5, s_row);
        }
    }
    add_block_stats(F.ctl, vis, fp);
    pdl_release();
}

// Zeros over the frame's bin-list entries [0, num_pairs) in whole 16-byte
// words, before the exact fill pass scatters its 4-byte stores there.  The
// list's sectors are then fully written in L2, and the scattered stores
// merge into them instead of each partly written sector being completed
// from DRAM (1M soup: scan + fill 84 -> 64 us with this pass).  The
// predicted fused pass, bound by its returning atomics, measured no gain.
__global__ void __launch_bounds__(256) list_touch_kernel(FrameDev F) {
    pdl_wait();
    if (!F.ctl->overflow) {
        const unsigned long long n = min((unsigned long long)F.ctl->num_pairs, F.list_cap);
        uint4* const p = reinterpret_cast<uint4*>(F.list);
        const unsigned long long words = (n + 3u) / 4u;   // list storage is 2 x list_cap entries
        for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < words;
             i += (unsigned long long)gridDim.x * blockDim.x)
            p[i] = make_uint4(0u, 0u, 0u, 0u);
    }
    pdl_release();
}

cudaError_t launch_list_touch(const FrameDev& F, cudaStream_t s) {
    return launch_pdl(list_touch_kernel, dim3(4u * (uint32_t)sm_count()), dim3(256), 0, s, F);
}

// ---------------------------------------------------------------------------
// Raster + ROP + shade
// ---------------------------------------------------------------------------
// A raster CTA of THREADS threads stages 8 entries per thread at once and
// sorts them into THREADS depth buckets (one per thread): the top
// log2(THREADS) bits of the 31-bit depth key.
template <int THREADS>
struct RasterGeom {
    static_assert(THREADS == 128 || THREADS == 256, "raster CTAs of 128 or 256 threads");
    static constexpr uint32_t kEntries = 8u * THREADS;             // entries depth-sorted at once
    static constexpr uint32_t kKeyShift = THREADS == 256 ? 23u : 24u;   // depth key -> bucket
};
static_assert(RasterGeom<kRasterThreads>::kEntries == (uint32_t)kBatch, "the 256-thread raster sorts kBatch entries");

template <int THREADS>
struct RasterSharedT {
    TriSetup rec[kMaxPhase];     // setup records of the running phase
    uint32_t prim[RasterGeom<THREADS>::kEntries];   // staged bin entries (rasterisable triangles)
    uint32_t key[RasterGeom<THREADS>::kEntries];    // their depth-key lower bounds
    uint16_t order[RasterGeom<THREADS>::kEntries];  // staged triangles, front to back by depth bucket
    uint32_t bucket[THREADS];    // counts -> starts -> (after the scatter) ends
    uint32_t warp_count[THREADS / 32];
    uint32_t warp_max[THREADS / 32];
    uint32_t item[4];
    __align__(16) uint4 item_next;   // the next work item, copied ahead by thread 0
    int next;
    uint32_t scene_next;         // batch: scene of the fetched work item
    uint32_t scene_loaded;       // batch: scene whose descriptor `frame` holds
    __align__(8) unsigned long long rec_bar[2];   // mbarriers: a phase's setup records have landed (phases alternate)
    __align__(16) FrameDev frame;
};
using RasterShared = RasterSharedT<kRasterThreads>;

// Setup records reach shared memory by bulk asynchronous copies (the TMA
// engine's cp.async.bulk, one 48-byte copy per record), each completing
// its bytes on one of the CTA's two mbarriers (phases alternate); readers
// wait for that barrier's parity.  Warp 0 issues a phase's copies while the
// phase before it rasterises, so they land in time.
constexpr uint32_t kRecWaitLimit = 1u << 22;   // polls before a wait gives up (the frame is flagged)

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Warp 0 arms `bar` for `pn` records and copies the records of sorted
// entries [p0, p0 + pn) into their ring slots (entry k -> slot k mod
// kMaxPhase).
__device__ __forceinline__ void issue_records(TriSetup* rec, const TriSetup* setup, const uint32_t* prim,
                                              const uint16_t* order, uint32_t p0, uint32_t pn, uint32_t bar,
                                              uint32_t lane);

__device__ __forceinline__ void rec_copy(TriSetup* dst, const TriSetup* src, uint32_t bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], 48, [%2];"
                 ::"r"(smem_addr(dst)), "l"(src), "r"(bar) : "memory");
}

__device__ __forceinline__ void issue_records(TriSetup* rec, const TriSetup* setup, const uint32_t* prim,
                                              const uint16_t* order, uint32_t p0, uint32_t pn, uint32_t bar,
                                              uint32_t lane) {
    if (lane == 0)
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(pn * 48u) : "memory");
    __syncwarp();
    for (uint32_t q = lane; q < pn; q += 32u) {
        const uint32_t k = p0 + q;
        rec_copy(&rec[k & (kMaxPhase - 1u)], setup + prim[order[k]], bar);
    }
}

// Waits for phase `parity` of the mbarrier; false when the bound ran out.
__device__ __forceinline__ bool rec_wait(uint32_t bar, uint32_t parity) {
    for (uint32_t it = 0; it < kRecWaitLimit; ++it) {
        uint32_t done = 0;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(bar), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// `key_bound` = hiz_key(t): a covered pixel whose stored key is already
// below it cannot be won by this triangle, and skips the weights and depth.
__device__ __forceinline__ void raster_fixed(const TriSetup& t, uint32_t prim, unsigned long long* tile, int tx0,
                                             int ty0, int tw, int th, uint32_t lane, uint32_t key_bound) {
    const int X0 = snap_fx(t.x0), Y0 = snap_fx(t.y0), X1 = snap_fx(t.x1);
    const int Y1 = snap_fx(t.y1), X2 = snap_fx(t.x2), Y2 = snap_fx(t.y2);
    const int minx = min(X0, min(X1, X2)), maxx = max(X0, max(X1, X2));
    const int miny = min(Y0, min(Y1, Y2)), maxy = max(Y0, max(Y1, Y2));
    // covered pixels lie in [ceil(min), floor(max)] of the snapped triangle
    const int px0 = max((minx + 0xFFFF) >> kFxBits, tx0), px1 = min(maxx >> kFxBits, tx0 + tw - 1);
    const int py0 = max((miny + 0xFFFF) >> kFxBits, ty0), py1 = min(maxy >> kFxBits, ty0 + th - 1);
    if (px0 > px1 || py0 > py1) return;
    const int bwid = px1 - px0 + 1;
    const int lsw = bwid <= 1 ? 0 : bwid <= 2 ? 1 : bwid <= 4 ? 2 : bwid <= 8 ? 3 : bwid <= 16 ? 4 : 5;
    const int sw = 1 << lsw, sh = 32 >> lsw;
    const int lx = (int)lane & (sw - 1), ly = (int)lane >> lsw;
    const int dxa = X1 - X0, dya = Y1 - Y0;
    const int dxb = X2 - X1, dyb = Y2 - Y1;
    const int dxc = X0 - X2, dyc = Y0 - Y2;
    // exact edge values at the lane's first pixel, then stepped by whole
    // stamps: E(x + sw, y) = E + sw * 2^16 * dy, E(x, y + sh) = E - sh * 2^16 * dx
    const int fx0 = (px0 + lx) << kFxBits, fy0 = (py0 + ly) << kFxBits;
    long long r2 = edge_fx(fx0, fy0, X0, Y0, dxa, dya);
    long long r0 = edge_fx(fx0, fy0, X1, Y1, dxb, dyb);
    long long r1 = edge_fx(fx0, fy0, X2, Y2, dxc, dyc);
    const long long stx = (long long)sw << kFxBits, sty = (long long)sh << kFxBits;
    const long long ix2 = stx * dya, ix0 = stx * dyb, ix1 = stx * dyc;
    const long long iy2 = -sty * dxa, iy0 = -sty * dxb, iy1 = -sty * dxc;
    for (int sy = py0; sy <= py1; sy += sh, r2 += iy2, r0 += iy0, r1 += iy1) {
        const int y = sy + ly;
        long long e2 = r2, e0 = r0, e1 = r1;
        for (int sx = px0; sx <= px1; sx += sw, e2 += ix2, e0 += ix0, e1 += ix1) {
            const int x = sx + lx;
            if (x > px1 || y > py1 || (e0 | e1 | e2) < 0) continue;
            unsigned long long* slot = tile + (y - ty0) * tw + (x - tx0);
            const unsigned long long cur = *((volatile unsigned long long*)slot);
            if ((uint32_t)(cur >> 32) < key_bound) continue;   // occluded: every fragment key is >= the bound
            float w[3];
            weights_fixed(t, x, y, w);
            const float z = interp_z(w[0], w[1], w[2], t.z0, t.z1, t.z2);
            // the reference rejects z < 0 or z > 1; z == 1 saturates the key to
            // INT_MAX and can never win the depth test (CUDAROPs.cu:343-345, 386)
            if (!(z >= 0.f && z < 1.f)) continue;
            const uint32_t key = (uint32_t)__float2int_rz(__fmul_rn(z, 2147483648.0f));
            const unsigned long long packed = ((unsigned long long)key << 32) | prim;
            if (packed < cur) atomicMin(slot, packed);   // a later, lower value only makes atomicMin a no-op
        }
    }
}

// One lane's raster of a small triangle: raster_fixed's snapped box,
// coverage, occlusion test, weights, depth and (key, id) minimum, pixel by
// pixel (the edge functions evaluated exactly at each pixel equal the
// stepped ones).  Returns false, having done nothing, for a triangle on the
// float path or with a box of more than kLanePixels pixels.
__device__ __forceinline__ bool raster_fixed_lane(const TriSetup& t, uint32_t prim, unsigned long long* tile, int tx0,
                                                  int ty0, int tw, int th, uint32_t key_bound) {
    if (t.flags & kFlagFloat) return false;
    const int X0 = snap_fx(t.x0), Y0 = snap_fx(t.y0), X1 = snap_fx(t.x1);
    const int Y1 = snap_fx(t.y1), X2 = snap_fx(t.x2), Y2 = snap_fx(t.y2);
    const int minx = min(X0, min(X1, X2)), maxx = max(X0, max(X1, X2));
    const int miny = min(Y0, min(Y1, Y2)), maxy = max(Y0, max(Y1, Y2));
    const int px0 = max((minx + 0xFFFF) >> kFxBits, tx0), px1 = min(maxx >> kFxBits, tx0 + tw - 1);
    const int py0 = max((miny + 0xFFFF) >> kFxBits, ty0), py1 = min(maxy >> kFxBits, ty0 + th - 1);
    if (px0 > px1 || py0 > py1) return true;
    if ((px1 - px0 + 1) * (py1 - py0 + 1) > kLanePixels) return false;
    for (int y = py0; y <= py1; ++y)
        for (int x = px0; x <= px1; ++x) {
            const int fx = x << kFxBits, fy = y << kFxBits;
            if (edge_fx(fx, fy, X0, Y0, X1 - X0, Y1 - Y0) < 0 || edge_fx(fx, fy, X1, Y1, X2 - X1, Y2 - Y1) < 0 ||
                edge_fx(fx, fy, X2, Y2, X0 - X2, Y0 - Y2) < 0)
                continue;
            unsigned long long* slot = tile + (y - ty0) * tw + (x - tx0);
            const unsigned long long cur = *((volatile unsigned long long*)slot);
            if ((uint32_t)(cur >> 32) < key_bound) continue;   // occluded
            float w[3];
            weights_fixed(t, x, y, w);
            const float z = interp_z(w[0], w[1], w[2], t.z0, t.z1, t.z2);
            if (!(z >= 0.f && z < 1.f)) continue;
            const uint32_t key = (uint32_t)__float2int_rz(__fmul_rn(z, 2147483648.0f));
            const unsigned long long packed = ((unsigned long long)key << 32) | prim;
            if (packed < cur) atomicMin(slot, packed);
        }
    return true;
}

// Triangles outside the guard band: the reference's float edge functions.
__device__ __noinline__ void raster_float(const TriSetup& t, uint32_t prim, unsigned long long* tile, int tx0,
                                             int ty0, int tw, int th, uint32_t lane) {
    const float x0 = t.x0, y0 = t.y0, x1 = t.x1, y1 = t.y1, x2 = t.x2, y2 = t.y2;
    if (x0 != x0 || y0 != y0 || x1 != x1 || y1 != y1 || x2 != x2 || y2 != y2) return;
    int px0 = tx0, px1 = tx0 + tw - 1, py0 = ty0, py1 = ty0 + th - 1;
    const float fx0 = floorf(min3f(x0, x1, x2)) - 1.f, fx1 = ceilf(max3f(x0, x1, x2)) + 1.f;
    const float fy0 = floorf(min3f(y0, y1, y2)) - 1.f, fy1 = ceilf(max3f(y0, y1, y2)) + 1.f;
    if (fx0 > (float)px0) px0 = fx0 > (float)px1 ? px1 + 1 : (int)fx0;
    if (fx1 < (float)px1) px1 = fx1 < (float)px0 ? px0 - 1 : (int)fx1;
    if (fy0 > (float)py0) py0 = fy0 > (float)py1 ? py1 + 1 : (int)fy0;
    if (fy1 < (float)py1) py1 = fy1 < (float)py0 ? py0 - 1 : (int)fy1;
    if (px0 > px1 || py0 > py1) return;
    const int n = (px1 - px0 + 1) * (py1 - py0 + 1);
    const int wdt = px1 - px0 + 1;
    for (int i = (int)lane; i < n; i += 32) {
        const int x = px0 + i % wdt, y = py0 + i / wdt;
        float w[3];
        if (!weights_float(t, (float)x, (float)y, w)) continue;
        const float z = interp_z(w[0], w[1], w[2], t.z0, t.z1, t.z2);
        if (z < 0.f || z > 1.f) continue;  // NaN passes as in the reference
        const int k = cvt_s32(__fmul_rn(z, 2147483648.0f));
        if (k == 2147483647) continue;
        const unsigned long long packed = ((unsigned long long)(uint32_t)k << 32) | prim;
        unsigned long long* slot = tile + (y - ty0) * tw + (x - tx0);
        if (packed < *((volatile unsigned long long*)slot)) atomicMin(slot, packed);
    }
}

__device__ __forceinline__ void clear_pixel(const FrameDev& F, size_t gi) {
    F.colour[gi] = F.vis == 0u ? F.clear_colour32 : 0u;
    F.depth[gi] = 0.f;
    F.ids[gi] = kInvalidPrim;
}

template <bool FLAT>
__device__ __forceinline__ void resolve_pixel(const FrameDev& F, int x, int y, unsigned long long v) {
    const size_t gi = (size_t)y * F.width + (size_t)x;
    if (v == kEmptyVis) {
        clear_pixel(F, gi);
        return;
    }
    const uint32_t prim = (uint32_t)(v & 0xFFFFFFFFull);
    const uint4* rp = reinterpret_cast<const uint4*>(F.setup) + 3u * prim;
    const uint4 a = __ldg(rp), b = __ldg(rp + 1), c = __ldg(rp + 2);
    TriSetup t;
    t.x0 = __uint_as_float(a.x); t.y0 = __uint_as_float(a.y); t.x1 = __uint_as_float(a.z); t.y1 = __uint_as_float(a.w);
    t.x2 = __uint_as_float(b.x); t.y2 = __uint_as_float(b.y); t.z0 = __uint_as_float(b.z); t.z1 = __uint_as_float(b.w);
    t.z2 = __uint_as_float(c.x); t.inv_area = __uint_as_float(c.y); t.flags = c.z; t.mesh = c.w;
    float w[3] = {0.f, 0.f, 0.f};
    if (t.flags & kFlagFloat) weights_float(t, (float)x, (float)y, w);
    else weights_fixed(t, x, y, w);
    const float z = interp_z(w[0], w[1], w[2], t.z0, t.z1, t.z2);
    const MeshDev& m = F.meshes[t.mesh];
    F.colour[gi] = shade_fragment<FLAT>(F, m, prim, w, z);
    F.depth[gi] = z;
    F.ids[gi] = prim;
}

__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// Work item `idx` into shared memory by an asynchronous 16-byte copy (the
// end marker when the queue is drained); cp_async_wait_all() completes it.
__device__ __forceinline__ void fetch_item(uint4* dst, const uint4* items, uint32_t idx, uint32_t num_items) {
    if (idx >= num_items) {
        *dst = make_uint4(0xFFFFFFFFu, 0u, 0u, 0u);
        return;
    }
    const uint32_t s = (uint32_t)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(s), "l"(items + idx) : "memory");
}

// Persistent raster.  Single frame (BATCH false): work items of F.  Batch
// (BATCH true): work items of all scenes of B; the scene of an item is
// found from its global bin, and its frame descriptor is copied to shared
// memory when it differs from the previous item's.
// MIN_CTAS counts CTAs of 256 threads: a 128-thread variant keeps twice as
// many resident (the same registers per thread).
// LANES: the small-triangle variant (kLanePhase), a kernel of its own so
// that the one-triangle-per-warp path keeps its registers.
template <int MIN_CTAS, bool BATCH, bool TMA = false, int THREADS = kRasterThreads, bool LANES = false>
__global__ void __launch_bounds__(THREADS, MIN_CTAS * (kRasterThreads / THREADS)) raster_kernel(FrameDev F, BatchDev B) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    using Shared = RasterSharedT<THREADS>;
    constexpr uint32_t kEntries = RasterGeom<THREADS>::kEntries, kKeyShift = RasterGeom<THREADS>::kKeyShift;
    Shared& S = *reinterpret_cast<Shared*>(smem_raw);
    unsigned long long* tile = reinterpret_cast<unsigned long long*>(smem_raw + sizeof(Shared));
    pdl_wait();
    Ctl* const Q = BATCH ? B.ctl : F.ctl;
    const uint4* const items = BATCH ? B.items : F.items;
    if (Q->overflow) return;
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    const uint32_t num_items = Q->num_items;
    const uint32_t phase_req = BATCH ? B.phase : F.phase;
    const uint32_t phase = phase_req == 0u ? kPhase : min(phase_req, kMaxPhase);
    const uint32_t stage_req = BATCH ? B.stage : F.stage;
    const uint32_t pass = stage_req == 0u ? kEntries : min(stage_req, kEntries);   // entries per raster pass
    if (BATCH && tid == 0) S.scene_loaded = 0xFFFFFFFFu;
    // thread 0 runs one item ahead: the next item's queue slot is taken when
    // an item starts and its descriptor copied to shared memory
    // (asynchronously) while the item is staged
    uint32_t next_idx = 0;
    constexpr bool tma = TMA;   // setup records staged by bulk copies (a variant for single frames)
    const uint32_t rec_bar0 = smem_addr(&S.rec_bar[0]);
    uint32_t rec_parity = 0;   // bit b: completions of record barrier b seen so far, mod 2
    if (tid == 0) {
        if (TMA) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(rec_bar0) : "memory");
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(rec_bar0 + 8u) : "memory");
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        }
        next_idx = atomicAdd(&Q->item_next, 1u);
        fetch_item(&S.item_next, items, next_idx, num_items);
    }
    for (;;) {
        if (tid == 0) {
            cp_async_wait_all();
            uint4 it = S.item_next;
            if (BATCH && it.x != 0xFFFFFFFFu) {
                const uint32_t sc = __ldg(B.bin_scene + it.x);
                S.scene_next = sc;
                it.x -= __ldg(B.bin_base + sc);
            }
            S.item[0] = it.x; S.item[1] = it.y; S.item[2] = it.z; S.item[3] = it.w;
            if (it.x != 0xFFFFFFFFu) next_idx = atomicAdd(&Q->item_next, 1u);
        }
        __syncthreads();
        const uint32_t bin = S.item[0];
        if (bin == 0xFFFFFFFFu) break;
        if (!BATCH && tid == 0 && F.dirty_wr) F.dirty_wr[bin] = 1u;   // the bin's pixels may now be drawn
        if (BATCH) {
            const uint32_t sc = S.scene_next;
            if (sc != S.scene_loaded) {   // uniform across the CTA
                const uint4* src = reinterpret_cast<const uint4*>(B.scenes + sc);
                uint4* dst = reinterpret_cast<uint4*>(&S.frame);
                for (uint32_t i = tid; i < sizeof(FrameDev) / 16u; i += THREADS) dst[i] = __ldg(src + i);
                __syncthreads();
                if (tid == 0) S.scene_loaded = sc;
            }
        }
        const FrameDev& G = BATCH ? S.frame : F;
        const uint32_t start = S.item[1], count = S.item[2], nchunks = S.item[3];
        const int tx0 = (int)((bin % G.nbx) * G.bw), ty0 = (int)((bin / G.nbx) * G.bh);
        const int tw = min((int)G.bw, (int)G.width - tx0), th = min((int)G.bh, (int)G.height - ty0);
        const int npx = (tw > 0 && th > 0) ? tw * th : 0;
        const uint32_t* const list = G.list;
        const TriSetup* const setup = G.setup;
        unsigned long long* const gvis = G.gvis;
        const uint32_t width = G.width;
        for (int i = (int)tid; i < npx; i += THREADS) tile[i] = kEmptyVis;
        if (tid == 0) fetch_item(&S.item_next, items, next_idx, num_items);
        const uint32_t* const keys = G.keys;
        for (uint32_t b0 = 0; b0 < count && npx > 0; b0 += pass) {
            // stage the entries with their depth-key bounds (no setup record
            // is read before a triangle's phase comes) and count the
            // rasterisable ones per depth bucket
            constexpr uint32_t kPer = kEntries / THREADS;
            const uint32_t n = min(pass, count - b0);
            __syncthreads();   // the previous batch is done with the shared arrays
            S.bucket[tid] = 0u;
            __syncthreads();
            // rows of THREADS entries up to the pass's n (uniform); entries at
            // or past n are never read
            const uint32_t rows = (n + THREADS - 1u) / THREADS;
#pragma unroll 4
            for (uint32_t j = 0; j < kPer; ++j) {
                if (j >= rows) break;
                const uint32_t idx = j * THREADS + tid;
                const uint32_t e = idx < n ? __ldg(list + start + b0 + idx) : kNoRasterBit;
                const bool keep = !(e & kNoRasterBit);
                const uint32_t k = keep ? __ldg(keys + e) : 0u;
                S.prim[idx] = e;
                S.key[idx] = k;
                if (keep) atomicAdd(&S.bucket[k >> kKeyShift], 1u);
            }
            __syncthreads();
            // bucket starts: exclusive scan of the 256 counts; their sum is the
            // number of staged triangles
            uint32_t total = 0;
            {
                const uint32_t c = S.bucket[tid];
                uint32_t x = c;
#pragma unroll
                for (uint32_t d = 1; d < 32; d <<= 1) {
                    const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, x, d);
                    if (lane >= d) x += t;
                }
                if (lane == 31u) S.warp_count[warp] = x;
                __syncthreads();
                uint32_t before = 0;
#pragma unroll
                for (uint32_t w = 0; w < THREADS / 32; ++w) {
                    const uint32_t wc = S.warp_count[w];
                    before += w < warp ? wc : 0u;
                    total += wc;
                }
                S.bucket[tid] = before + x - c;
            }
            __syncthreads();
#pragma unroll
            for (uint32_t j = 0; j < kPer; ++j) {
                if (j >= rows) break;
                const uint32_t idx = j * THREADS + tid;
                if (idx < n && !(S.prim[idx] & kNoRasterBit))
                    S.order[atomicAdd(&S.bucket[S.key[idx] >> kKeyShift], 1u)] = (uint16_t)idx;
            }
            // now S.bucket[b] = end of bucket b
            // phases of `phase` triangles; the tile's max depth key is refreshed
            // between phases.  A triangle whose key bound exceeds it cannot win
            // a pixel; once a whole bucket's lower bound does, the rest of the
            // batch is skipped.
            // TMA staging: phases of at most kMaxPhase / 2 triangles prefetch
            // the next phase's records into the other half of the ring
            const bool ahead = tma && phase <= kMaxPhase / 2u;
            for (uint32_t p0 = 0, ph = 0; p0 < total; p0 += phase, ph ^= 1u) {
                __syncthreads();   // the order, or the previous phase's records and tile
                const uint32_t pn = min(phase, total - p0);
                const uint32_t bar = rec_bar0 + 8u * ph, bar_next = rec_bar0 + 8u * (ph ^ 1u);
                const bool next = ahead && p0 + phase < total;   // this phase prefetches the next one's records
                if (tma) {
                    if (warp == 0) {
                        if (p0 == 0u || !ahead)   // this phase's records were not prefetched
                            issue_records(S.rec, setup, S.prim, S.order, p0, pn, bar, lane);
                        if (next)
                            issue_records(S.rec, setup, S.prim, S.order, p0 + phase, min(phase, total - p0 - phase),
                                          bar_next, lane);
                    }
                } else {
                    // 16 bytes per thread (triangle k's record goes to slot k
                    // mod kMaxPhase: phase <= kMaxPhase)
                    for (uint32_t r = tid; r < 3u * pn; r += THREADS) {
                        const uint32_t q = r / 3u, k = p0 + q;
                        const uint4* rp = reinterpret_cast<const uint4*>(setup) + 3u * S.prim[S.order[k]];
                        reinterpret_cast<uint4*>(&S.rec[k & (kMaxPhase - 1u)])[r - 3u * q] = __ldg(rp + (r - 3u * q));
                    }
                }
                if (b0 > 0 || p0 > 0) {
                    uint32_t m = 0;
                    for (int i = (int)tid; i < npx; i += THREADS)
                        m = max(m, (uint32_t)(tile[i] >> 32));
                    m = __reduce_max_sync(0xFFFFFFFFu, m);
                    if (lane == 0) S.warp_max[warp] = m;
                }
                if (tid == 0) S.next = (int)p0;
                __syncthreads();
                // every thread sees this phase's records land before any phase
                // decision; a phase that ends the batch early also waits for
                // the records it prefetched, so no copy is ever left in flight
                if (tma) {
                    if (!rec_wait(bar, (rec_parity >> ph) & 1u) && tid == 0) atomicOr(&Q->error, 8u);
                    rec_parity ^= 1u << ph;
                }
                uint32_t tile_max = 0xFFFFFFFFu;
                if (b0 > 0 || p0 > 0) {
                    tile_max = 0;
#pragma unroll
                    for (uint32_t w = 0; w < THREADS / 32; ++w) tile_max = max(tile_max, S.warp_max[w]);
                }
                // buckets [0, tile_max >> kKeyShift] can still hold a winner
                const uint32_t limit = tile_max >= 0x80000000u ? total : S.bucket[tile_max >> kKeyShift];
                if (p0 >= limit) {   // uniform: every thread sees the same tile_max
                    if (next) {
                        if (!rec_wait(bar_next, (rec_parity >> (ph ^ 1u)) & 1u) && tid == 0) atomicOr(&Q->error, 8u);
                        rec_parity ^= 1u << (ph ^ 1u);
                    }
                    break;
                }
                const uint32_t p1 = min(limit, p0 + phase);
                // a warp takes one sorted triangle at a time; the
                // small-triangle variant takes kLaneGrab in phases of at least
                // kLanePhase triangles, each lane rasterises its own when its
                // pixel box holds at most kLanePixels pixels, and the warp the
                // others
                const bool lanes = LANES && phase >= kLanePhase;
                for (;;) {
                    int kb = 0;
                    if (lane == 0) kb = atomicAdd(&S.next, lanes ? (int)kLaneGrab : 1);
                    kb = __shfl_sync(0xFFFFFFFFu, kb, 0);
                    if (kb >= (int)p1) break;
                    uint32_t m;   // bit l: triangle kb + l goes to the whole warp
                    if (lanes) {
                        const uint32_t k = (uint32_t)kb + lane;
                        bool big = false;
                        if (lane < kLaneGrab && k < p1) {
                            const uint32_t i = S.order[k];
                            const uint32_t key = S.key[i];
                            if (key <= tile_max)
                                big = !raster_fixed_lane(S.rec[k & (kMaxPhase - 1u)], S.prim[i], tile, tx0, ty0, tw, th,
                                                         key);
                        }
                        m = __ballot_sync(0xFFFFFFFFu, big);
                    } else {
                        m = S.key[S.order[kb]] <= tile_max ? 1u : 0u;
                    }
                    for (; m; m &= m - 1u) {
                        const uint32_t k = (uint32_t)kb + (uint32_t)(__ffs(m) - 1), i = S.order[k];
                        const TriSetup& t = S.rec[k & (kMaxPhase - 1u)];
                        if (t.flags & kFlagFloat) raster_float(t, S.prim[i], tile, tx0, ty0, tw, th, lane);
                        else raster_fixed(t, S.prim[i], tile, tx0, ty0, tw, th, lane, S.key[i]);
                    }
                }
            }
        }
        __syncthreads();
        // publish the tile: one chunk owns its pixels (plain stores); the
        // chunks of a longer bin merge with 64-bit atomicMin
        if (npx > 0 && count > 0) {
            for (int i = (int)tid; i < npx; i += THREADS) {
                const unsigned long long v = tile[i];
                unsigned long long* g = &gvis[(size_t)(ty0 + i / tw) * width + (size_t)(tx0 + i % tw)];
                if (nchunks == 1u) *g = v;
                else if (v != kEmptyVis) atomicMin(g, v);
            }
        }
        __syncthreads();
    }
}

// Shades pixel i of the frame: the winner the raster left in the merge
// buffer (or the clear colour), and leaves the buffer empty for the next
// frame.
template <bool FLAT>
__device__ __forceinline__ void shade_px(const FrameDev& F, uint32_t i) {
    const unsigned long long v = F.gvis[i];
    if (v != kEmptyVis) F.gvis[i] = kEmptyVis;
    resolve_pixel<FLAT>(F, (int)(i % F.width), (int)(i / F.width), v);
}

// One thread per pixel.
template <bool FLAT>
__global__ void __launch_bounds__(256) shade_kernel(FrameDev F) {
    pdl_wait();
    const uint32_t i = F.px_begin + blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (F.px_end ? F.px_end : F.width * F.height) || F.ctl->overflow) return;
    shade_px<FLAT>(F, i);
}

// Two-pass shading, for frames that shade through the full vertex stage
// (textured or lit meshes, the normal view).  The light pass clears the
// pixels no triangle won and queues the covered ones; the heavy pass shades
// the queue, 32 covered pixels to a warp, over the whole GPU.  In one pass
// a covered region's pixels sit a few to a warp inside blocks that keep
// their SM slot for the whole shading chain (4K icosphere: 140K covered
// pixels of 8.3M).
//
// Light pass: one thread per 4 consecutive pixels: their merge words come in with two
// 16-byte loads, an all-empty quad (most of a frame whose geometry covers a
// small part of the screen) is cleared with 16-byte stores, and a warp
// queues its covered pixels with one atomic.  Buffers not 16-byte aligned
// take per-pixel accesses.
__global__ void __launch_bounds__(256) shade_queue_kernel(FrameDev F) {
    pdl_wait();
    if (F.ctl->overflow) {
        // not rasterised: the buffers keep the last frame's pixels, and the
        // next frame must find those bins as they were
        if (F.dirty_rd)
            for (uint32_t b = blockIdx.x * blockDim.x + threadIdx.x; b < F.num_bins; b += gridDim.x * blockDim.x)
                F.dirty_wr[b] |= F.dirty_rd[b];
        return;
    }
    // pixels [px_begin, px_end) (px_begin a multiple of 4)
    const uint32_t n = F.px_end ? F.px_end : F.width * F.height, lane = threadIdx.x & 31u;
    const uint32_t i0 = F.px_begin + (blockIdx.x * blockDim.x + threadIdx.x) * 4u;
    const bool aligned = ((reinterpret_cast<uintptr_t>(F.gvis) | reinterpret_cast<uintptr_t>(F.colour) |
                           reinterpret_cast<uintptr_t>(F.depth) | reinterpret_cast<uintptr_t>(F.ids)) & 15u) == 0u;
    // a quad whose pixels all lie in bins clean after the last frame and not
    // drawn in this one already holds the clear values (pixels outside the
    // bin grid are always written)
    bool live = i0 < n;
    if (F.dirty_rd) {
        // the quad's row and column: one division per warp (its 32 quads
        // are consecutive), then at most one row wrap per lane on frames at
        // least 128 pixels wide
        uint32_t y = 0, x = 0;
        if (lane == 0u) {
            y = i0 / F.width;
            x = i0 - y * F.width;
        }
        y = __shfl_sync(0xFFFFFFFFu, y, 0);
        x = __shfl_sync(0xFFFFFFFFu, x, 0) + 4u * lane;
        if (F.width < 128u) {
            y = i0 / F.width;
            x = i0 - y * F.width;
        } else if (x >= F.width) {
            x -= F.width;
            ++y;
        }
        if (!live) {
        } else if (x + 3u < F.width && i0 + 3u < n) {   // one row: bins [x / bw, (x + 3) / bw] of bin row y / bh
            const bool p2 = ((F.bw & (F.bw - 1u)) | (F.bh & (F.bh - 1u))) == 0u;
            const uint32_t sx = (uint32_t)__ffs((int)F.bw) - 1u, sy = (uint32_t)__ffs((int)F.bh) - 1u;
            const uint32_t by = p2 ? y >> sy : y / F.bh;
            const uint32_t bx0 = p2 ? x >> sx : x / F.bw, bx1 = p2 ? (x + 3u) >> sx : (x + 3u) / F.bw;
            live = by >= F.nby || bx1 >= F.nbx;
            for (uint32_t bx = bx0; !live && bx <= bx1; ++bx)
                live = (F.dirty_rd[by * F.nbx + bx] | F.dirty_wr[by * F.nbx + bx]) != 0u;
        } else {   // a quad that wraps a row, or the frame's last pixels
            live = false;
            const uint32_t last = min(i0 + 3u, n - 1u);
            for (uint32_t i = i0; i <= last; ++i) {
                const uint32_t yi = i / F.width, xi = i - yi * F.width;
                const uint32_t bx = xi / F.bw, by = yi / F.bh;
                live |= bx >= F.nbx || by >= F.nby || (F.dirty_rd[by * F.nbx + bx] | F.dirty_wr[by * F.nbx + bx]) != 0u;
            }
        }
        if (!__any_sync(0xFFFFFFFFu, live)) return;   // the warp's 128 pixels already hold the clear values
    }
    uint32_t covered = 0;   // bit k: pixel i0 + k has a winner
    if (!live) {
    } else if (aligned && i0 + 4u <= n) {
        const ulonglong2* g = reinterpret_cast<const ulonglong2*>(F.gvis + i0);
        const ulonglong2 a = g[0], b = g[1];
        covered = (a.x != kEmptyVis ? 1u : 0u) | (a.y != kEmptyVis ? 2u : 0u) | (b.x != kEmptyVis ? 4u : 0u) |
                  (b.y != kEmptyVis ? 8u : 0u);
        if (covered == 0u) {
            const uint32_t c = F.vis == 0u ? F.clear_colour32 : 0u;
            *reinterpret_cast<uint4*>(F.colour + i0) = make_uint4(c, c, c, c);
            *reinterpret_cast<float4*>(F.depth + i0) = make_float4(0.f, 0.f, 0.f, 0.f);
            *reinterpret_cast<uint4*>(F.ids + i0) = make_uint4(kInvalidPrim, kInvalidPrim, kInvalidPrim, kInvalidPrim);
        } else {
            for (uint32_t k = 0; k < 4u; ++k)
                if (!((covered >> k) & 1u)) clear_pixel(F, i0 + k);
        }
    } else {
        for (uint32_t k = 0; k < 4u && i0 + k < n; ++k) {
            if (F.gvis[i0 + k] != kEmptyVis) covered |= 1u << k;
            else clear_pixel(F, i0 + k);
        }
    }
    // the warp's covered pixels go to the queue in one run
    const uint32_t c = (uint32_t)__popc(covered);
    uint32_t incl = c;
#pragma unroll
    for (uint32_t d = 1; d < 32; d <<= 1) {
        const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, incl, d);
        if (lane >= d) incl += t;
    }
    const uint32_t total = __shfl_sync(0xFFFFFFFFu, incl, 31);
    if (total) {
        uint32_t base = 0;
        if (lane == 31u) base = atomicAdd(&F.ctl->shade_count, total);
        base = __shfl_sync(0xFFFFFFFFu, base, 31);
        uint32_t at = base + incl - c;
        for (uint32_t k = 0; k < 4u; ++k)
            if ((covered >> k) & 1u) F.shade_list[at++] = i0 + k;
    }
    pdl_release();
}

// 4 blocks per SM (<= 64 registers): the heavy pass is bound by the latency
// of its dependent loads, and a 4K frame's covered pixels then fit in one
// resident wave (3 blocks per SM at 80 registers: 71.7 -> 63.5 us with 4).
__global__ void __launch_bounds__(256, 4) shade_list_kernel(FrameDev F) {
    pdl_wait();
    if (F.ctl->overflow) return;
    const uint32_t count = F.ctl->shade_count;
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < count; j += gridDim.x * blockDim.x) {
        const uint32_t i = __ldg(F.shade_list + j);
        const unsigned long long v = F.gvis[i];
        F.gvis[i] = kEmptyVis;
        resolve_pixel<false>(F, (int)(i % F.width), (int)(i / F.width), v);
    }
}

// Pixels no bin covers (num_bins * bin_dim smaller than the screen).
__global__ void clear_kernel(FrameDev F) {
    const size_t n = (size_t)F.width * F.height;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        F.colour[i] = F.vis == 0u ? F.clear_colour32 : 0u;
        F.depth[i] = 0.f;
        F.ids[i] = kInvalidPrim;
    }
}

// ---------------------------------------------------------------------------
// Batched frames: every stage of all scenes of a batch in one launch
// ---------------------------------------------------------------------------
static_assert(sizeof(Ctl) % 16 == 0, "control blocks are cleared as 16-byte words");

// Copies scene sc's frame descriptor into shared memory (whole block).
__device__ __forceinline__ void load_scene(const BatchDev& B, uint32_t sc, FrameDev& dst) {
    const uint4* src = reinterpret_cast<const uint4*>(B.scenes + sc);
    uint4* d = reinterpret_cast<uint4*>(&dst);
    for (uint32_t i = threadIdx.x; i < sizeof(FrameDev) / 16u; i += blockDim.x) d[i] = __ldg(src + i);
    __syncthreads();
}

__device__ __forceinline__ void clear_ctl(Ctl* c) {
    uint4* w = reinterpret_cast<uint4*>(c);
#pragma unroll
    for (uint32_t k = 0; k < sizeof(Ctl) / 16u; ++k) w[k] = make_uint4(0u, 0u, 0u, 0u);
}

// Clears the batch's control block and every scene's statistics block.
__global__ void batch_reset_kernel(BatchDev B) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) clear_ctl(B.ctl);
    if (i < B.num_scenes) clear_ctl(B.scenes[i].ctl);
}

// Block -> scene, then the scene's descriptor into shared memory.
// The batch's triangle and pixel passes are cut into chunks of 256 items,
// each belonging to one scene (B.tri_scene / B.px_scene).  A block walks a
// contiguous range of `per` chunks and reloads its shared-memory frame
// descriptor only when the scene changes (a scene's chunks are
// consecutive), so the descriptor copy and its barrier are paid per scene
// rather than per 256 items.  Walk ids stay those of the chunk (chunk * 8 +
// warp), so the count and fill passes meet the same rank slots whatever
// their ranges.
__device__ __forceinline__ bool enter_scene(const BatchDev& B, uint32_t sc, uint32_t& loaded, FrameDev& sF) {
    if (sc == loaded) return false;   // block-uniform
    __syncthreads();                  // every thread is done with the previous descriptor
    load_scene(B, sc, sF);
    loaded = sc;
    return true;
}

__global__ void __launch_bounds__(256) batch_setup_kernel(BatchDev B, uint32_t chunks, uint32_t per) {
    __shared__ __align__(16) FrameDev sF;
    const uint32_t c0 = blockIdx.x * per, c1 = min(c0 + per, chunks);
    uint32_t loaded = 0xFFFFFFFFu, vis = 0, fp = 0;
    for (uint32_t v = c0; v < c1; ++v) {
        const uint32_t sc = __ldg(B.tri_scene + v);
        if (sc != loaded && loaded != 0xFFFFFFFFu) {   // the previous scene's statistics
            add_block_stats(sF.ctl, vis, fp);
            vis = fp = 0;
        }
        enter_scene(B, sc, loaded, sF);
        const uint32_t c = setup_tri<0>(sF, (v - __ldg(B.tri_blocks + sc)) * 256u + threadIdx.x,
                                        (v * 256u + threadIdx.x) >> 5);
        vis += c & 0xFFFFu;
        fp += c >> 16;
    }
    if (loaded != 0xFFFFFFFFu) add_block_stats(sF.ctl, vis, fp);
}

// The fill pass keeps one block per chunk (a range loop measured slower
// here: 489 -> 653 us for the 256-soup batch, more registers per thread).
__global__ void __launch_bounds__(256) batch_fill_kernel(BatchDev B) {
    if (B.ctl->overflow) return;
    __shared__ __align__(16) FrameDev sF;
    const uint32_t sc = __ldg(B.tri_scene + blockIdx.x);
    load_scene(B, sc, sF);
    fill_tri(sF, (blockIdx.x - __ldg(B.tri_blocks + sc)) * 256u + threadIdx.x, (blockIdx.x * 256u + threadIdx.x) >> 5);
}

// ALL_FLAT: every scene of the batch shades flat (B.all_flat), and the
// kernel holds only the flat path's registers (40 against 80: twice the
// resident warps for a batch of vertex-coloured soups).
template <bool ALL_FLAT>
__global__ void __launch_bounds__(256) batch_shade_kernel(BatchDev B, uint32_t chunks, uint32_t per) {
    if (B.ctl->overflow) return;
    __shared__ __align__(16) FrameDev sF;
    const uint32_t c0 = blockIdx.x * per, c1 = min(c0 + per, chunks);
    uint32_t loaded = 0xFFFFFFFFu;
    for (uint32_t v = c0; v < c1; ++v) {
        const uint32_t sc = __ldg(B.px_scene + v);
        enter_scene(B, sc, loaded, sF);
        const uint32_t i = (v - __ldg(B.px_blocks + sc)) * 256u + threadIdx.x;
        if (i >= sF.width * sF.height) continue;
        if (ALL_FLAT) shade_px<true>(sF, i);
        else if (sF.flat_shade) shade_px<true>(sF, i);
        else shade_px<false>(sF, i);
    }
}

// ---------------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------------
size_t raster_smem_bytes(uint32_t bw, uint32_t bh, uint32_t threads) {
    const size_t shared = threads == 128u ? sizeof(RasterSharedT<128>) : sizeof(RasterSharedT<256>);
    return shared + (size_t)bw * bh * sizeof(unsigned long long);
}

// Blocks of 256 threads for a triangle pass: one per 256 triangles, at most
// 8 per SM.  The blocks stride over the triangles, so a guarded launch that
// does not run costs one grid of early exits; more blocks than are resident
// at once (the setup pass holds 5 per SM) balance uneven triangles better
// than exactly one wave (measured ~9% faster for the 1M soup).

static uint32_t triangle_blocks(uint32_t num_tris) {
    return std::min<uint32_t>((num_tris + 255u) / 256u, 8u * (uint32_t)sm_count());
}

// Dynamic shared memory of the block-row kernels: one counter per bin (the
// opt-in above the default 48 KB is made once per device).
static cudaError_t row_smem(const FrameDev& F, size_t* bytes) {
    static uint64_t opted = 0;   // bit d: done on device d (devices 0..63)
    *bytes = (size_t)F.num_bins * sizeof(uint32_t);
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const uint64_t bit = dev < 64 ? (1ull << dev) : 0ull;
    if (!(opted & bit)) {
        const int most = (int)(kMaxRowBins * sizeof(uint32_t));
        e = cudaFuncSetAttribute(setup_rows_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, most);
        if (e == cudaSuccess) e = cudaFuncSetAttribute(fill_rows_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, most);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(predicted_rows_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, most);
        if (e != cudaSuccess) return e;
        opted |= bit;
    }
    return cudaSuccess;
}

cudaError_t launch_setup(const FrameDev& F, bool predicted, cudaStream_t s) {
    if (predicted && F.row_blocks) {
        size_t smem = 0;
        const cudaError_t e = row_smem(F, &smem);
        if (e != cudaSuccess) return e;
        return launch_pdl(predicted_rows_kernel, dim3(F.row_blocks), dim3(kRowThreads), smem, s, F);
    }
    if (!predicted && F.row_blocks) {
        size_t smem = 0;
        const cudaError_t e = row_smem(F, &smem);
        if (e != cudaSuccess) return e;
        return launch_pdl(setup_rows_kernel, dim3(F.row_blocks), dim3(kRowThreads), smem, s, F);
    }
    const uint32_t blocks = triangle_blocks(F.num_tris);
    if (blocks == 0) return cudaSuccess;
    return predicted ? launch_pdl(setup_kernel<1>, dim3(blocks), dim3(256), 0, s, F)
                     : launch_pdl(setup_kernel<0>, dim3(blocks), dim3(256), 0, s, F);
}

cudaError_t launch_fill(const FrameDev& F, cudaStream_t s) {
    if (F.row_blocks) {
        size_t smem = 0;
        const cudaError_t e = row_smem(F, &smem);
        if (e != cudaSuccess) return e;
        return launch_pdl(fill_rows_kernel, dim3(F.row_blocks), dim3(kRowThreads), smem, s, F);
    }
    const uint32_t blocks = triangle_blocks(F.num_tris);
    if (blocks == 0) return cudaSuccess;
    return launch_pdl(fill_kernel, dim3(blocks), dim3(256), 0, s, F);
}

template <bool BATCH, bool TMA = false, int THREADS = kRasterThreads, bool LANES = false>
static cudaError_t launch_raster_variant(const FrameDev& F, const BatchDev& B, uint32_t ctas, uint32_t grid, size_t smem,
                                         cudaStream_t s) {
    const dim3 g(grid), b(THREADS);
    switch (ctas ? ctas : kDefaultRasterCtas) {
        case 2: return launch_pdl(raster_kernel<2, BATCH, TMA, THREADS, LANES>, g, b, smem, s, F, B);
        case 3: return launch_pdl(raster_kernel<3, BATCH, TMA, THREADS, LANES>, g, b, smem, s, F, B);
        case 5: return launch_pdl(raster_kernel<5, BATCH, TMA, THREADS, LANES>, g, b, smem, s, F, B);
        case 6: return launch_pdl(raster_kernel<6, BATCH, TMA, THREADS, LANES>, g, b, smem, s, F, B);
        default: return launch_pdl(raster_kernel<4, BATCH, TMA, THREADS, LANES>, g, b, smem, s, F, B);
    }
}

cudaError_t launch_raster(const FrameDev& F, uint32_t grid, cudaStream_t s) {
    BatchDev none;
    memset(&none, 0, sizeof none);
    const size_t smem = raster_smem_bytes(F.bw, F.bh);
    if (F.rec_tma) return launch_raster_variant<false, true>(F, none, F.raster_ctas, grid, smem, s);
    if (F.raster_lanes) return launch_raster_variant<false, false, kRasterThreads, true>(F, none, F.raster_ctas, grid, smem, s);
    return launch_raster_variant<false>(F, none, F.raster_ctas, grid, smem, s);
}

cudaError_t launch_shade(const FrameDev& F, cudaStream_t s) {
    const uint32_t npx = (F.px_end ? F.px_end : F.width * F.height) - F.px_begin;
    const dim3 g((npx + 255u) / 256u), b(256);
    if (!F.flat_shade && F.shade_list) {
        const cudaError_t e = launch_pdl(shade_queue_kernel, dim3((npx + 1023u) / 1024u), b, 0, s, F);
        if (e != cudaSuccess) return e;
        // one resident wave: the queue is a few pixels per thread at most
        static int per_sm = 0;
        if (per_sm <= 0 &&
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, shade_list_kernel, 256, 0) != cudaSuccess) {
            cudaGetLastError();
            per_sm = 2;
        }
        return launch_pdl(shade_list_kernel, dim3((uint32_t)std::max(per_sm, 1) * (uint32_t)sm_count()), b, 0, s, F);
    }
    return F.flat_shade ? launch_pdl(shade_kernel<true>, g, b, 0, s, F) : launch_pdl(shade_kernel<false>, g, b, 0, s, F);
}

cudaError_t launch_batch(const BatchDev& B, const BatchLaunch& L, cudaStream_t s) {
    if (B.num_scenes == 0) return cudaSuccess;
    batch_reset_kernel<<<(B.num_scenes + 255u) / 256u, 256, 0, s>>>(B);
    // chunk ranges: about 16 blocks per SM, so the ranges balance over two
    // or more resident waves
    const uint32_t target = 16u * (uint32_t)sm_count();
    const uint32_t tri_per = std::max<uint32_t>(1u, (L.tri_blocks + target - 1u) / target);
    const uint32_t px_per = std::max<uint32_t>(1u, (L.px_blocks + target - 1u) / target);
    const uint32_t tri_grid = (L.tri_blocks + tri_per - 1u) / tri_per, px_grid = (L.px_blocks + px_per - 1u) / px_per;
    if (L.tri_blocks) batch_setup_kernel<<<tri_grid, 256, 0, s>>>(B, L.tri_blocks, tri_per);
    cudaError_t e = launch_scan(L.scan, s);
    if (e != cudaSuccess) return e;
    if (L.tri_blocks) batch_fill_kernel<<<L.tri_blocks, 256, 0, s>>>(B);
    FrameDev none;
    memset(&none, 0, sizeof none);
    const size_t smem = raster_smem_bytes(L.bin_w, L.bin_h, L.raster_threads);
    e = L.raster_threads == 128u ? launch_raster_variant<true, false, 128>(none, B, L.raster_ctas, L.raster_grid, smem, s)
                                 : launch_raster_variant<true>(none, B, L.raster_ctas, L.raster_grid, smem, s);
    if (e != cudaSuccess) return e;
    if (L.px_blocks) {
        if (B.all_flat) batch_shade_kernel<true><<<px_grid, 256, 0, s>>>(B, L.px_blocks, px_per);
        else batch_shade_kernel<false><<<px_grid, 256, 0, s>>>(B, L.px_blocks, px_per);
    }
    return cudaGetLastError();
}

cudaError_t launch_clear(const FrameDev& F, cudaStream_t s) {
    clear_kernel<<<1024, 256, 0, s>>>(F);
    return cudaGetLastError();
}

template <int MIN_CTAS, bool BATCH, int THREADS>
static cudaError_t configure_variant(size_t smem, int* blocks_per_sm) {
    cudaError_t e = cudaFuncSetAttribute(raster_kernel<MIN_CTAS, BATCH, false, THREADS>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    if (!BATCH) {   // the bulk-copy staging and small-triangle variants of a single frame
        e = cudaFuncSetAttribute(raster_kernel<MIN_CTAS, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        e = cudaFuncSetAttribute(raster_kernel<MIN_CTAS, false, false, kRasterThreads, true>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, raster_kernel<MIN_CTAS, BATCH, false, THREADS>,
                                                         THREADS, smem);
}

template <bool BATCH, int THREADS = kRasterThreads>
static cudaError_t configure(uint32_t bw, uint32_t bh, uint32_t ctas, int* blocks_per_sm) {
    const size_t smem = raster_smem_bytes(bw, bh, THREADS);
    switch (ctas ? ctas : kDefaultRasterCtas) {
        case 2: return configure_variant<2, BATCH, THREADS>(smem, blocks_per_sm);
        case 3: return configure_variant<3, BATCH, THREADS>(smem, blocks_per_sm);
        case 5: return configure_variant<5, BATCH, THREADS>(smem, blocks_per_sm);
        case 6: return configure_variant<6, BATCH, THREADS>(smem, blocks_per_sm);
        default: return configure_variant<4, BATCH, THREADS>(smem, blocks_per_sm);
    }
}

cudaError_t raster_configure(uint32_t bw, uint32_t bh, uint32_t ctas, int* blocks_per_sm) {
    return configure<false>(bw, bh, ctas, blocks_per_sm);
}

cudaError_t raster_configure_batch(uint32_t bw, uint32_t bh, uint32_t ctas, uint32_t threads, int* blocks_per_sm) {
    return threads == 128u ? configure<true, 128>(bw, bh, ctas, blocks_per_sm) : configure<true>(bw, bh, ctas, blocks_per_sm);
}

cudaError_t raster_configure(uint32_t bw, uint32_t bh, int* blocks_per_sm) {
    return raster_configure(bw, bh, 0u, blocks_per_sm);
}

}  // namespace gbr
