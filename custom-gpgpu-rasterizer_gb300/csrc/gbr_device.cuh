// gbr_device.cuh -- device-side data layout and per-primitive math of the
// GB300 frame hot path.
//
// Float discipline: the library is compiled with -fmad=false, and every fused
// multiply-add is written as __fmaf_rn.  The fusions follow the ones nvcc
// forms in the reference (CustomCUDARasterizer/CUDAROPs.cu,
// CUDATextureSampler.cuh, Matrix4.h, Vector3.h): a*b + c*d -> fma(a, b, c*d),
// s + a*b -> fma(a, b, s), a*b - c*d -> fma(a, b, -(c*d)).  Culling, bin
// rectangles and texel addresses then round exactly as the reference does.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace gbr {

constexpr uint32_t kInvalidPrim = 0xFFFFFFFFu;
constexpr uint32_t kNoRasterBit = 0x80000000u;   // bin-list entry that cannot cover a pixel
constexpr unsigned long long kEmptyVis = 0xFFFFFFFFFFFFFFFFull;
constexpr int kFxBits = 16;                       // 16.16 fixed-point screen coordinates
constexpr float kGuardPx = 8192.0f;               // |coord| below this: exact int64 edge functions
constexpr uint32_t kFlagRaster = 1u;              // fixed path, covered winding, area > 0
constexpr uint32_t kFlagFloat = 2u;               // outside the guard band: float edge functions
constexpr int kMaxBinDim = 64;
constexpr int kRasterThreads = 256;
constexpr int kBatch = 2048;                      // bin entries the raster depth-sorts at once
constexpr int kDepthBuckets = 256;                // front-to-back buckets: top 8 bits of the depth key
constexpr uint32_t kPhase = 16;                   // triangles between hierarchical-z refreshes
constexpr uint32_t kMaxPhase = 128;               // setup records staged per phase (the record ring)
constexpr uint32_t kSparsePhase = 64;             // the library's phase for frames of small triangles
constexpr uint32_t kMinChunk = 64;                // smallest raster work item the library picks
constexpr uint32_t kMaxChunk = 4096;              // largest raster work item the library picks
constexpr uint32_t kBatchChunk = 2048;            // raster work items of a batch frame
// Exact binning counts each bin in `count_split` sub-counters (at most
// kCountSplit), walk w using sub-counter w mod count_split: the crowded
// bins' atomics (a thousand per bin across the 1M soup, several thousand at
// its centre) queue on several addresses instead of one.  More sub-counters
// cost the scan a read and a write each per bin, so sparse frames use one.
constexpr uint32_t kCountSplit = 8;
__host__ __device__ inline uint32_t count_split_for(unsigned long long pairs, uint32_t bins) {
    const unsigned long long per_bin = pairs / (bins ? bins : 1u);
    return per_bin >= 256u ? 8u : per_bin >= 64u ? 4u : per_bin >= 16u ? 2u : 1u;
}
constexpr uint32_t kDefaultRasterCtas = 6;
// The raster's small-triangle variant: in phases of at least kLanePhase
// triangles a warp takes kLaneGrab sorted triangles at once and each lane
// rasterises its own when its pixel box holds at most kLanePixels pixels.
// The library picks it for sparse frames whose triangles span less than
// kLaneExtentPx (width + height, estimated from the last frame's
// (triangle, bin) pairs per visible triangle).
constexpr uint32_t kLanePhase = 32;
constexpr uint32_t kLaneGrab = 16;
constexpr int kLanePixels = 16;
constexpr double kLaneExtentPx = 16.0;        // raster_kernel variant (CTAs per SM) used by default
// Exact binning with block-private counter rows: one block of kRowThreads
// per SM counts its pairs per bin in shared memory (num_bins <=
// kMaxRowBins), then takes its run of every bin it touched with one global
// atomic per bin; the fill pass, the same blocks over the same triangles,
// hands out the runs' slots from shared memory.  Used once a frame has shown
// at least one pair per (block, bin) on average; sparser frames keep the
// global sub-counters.
constexpr uint32_t kRowThreads = 1024;
constexpr uint32_t kMaxRowBins = 32768;
__host__ __device__ inline bool use_count_rows(unsigned long long pairs, uint32_t bins, uint32_t blocks) {
    return bins > 0u && bins <= kMaxRowBins && blocks > 0u && pairs >= (unsigned long long)bins * blocks;
}

enum : uint32_t { kVertexIVertex56 = 0, kVertexPos3Rgba8 = 1 };

struct TexDev {
    const uint32_t* px;
    uint32_t w, h;
};

// One mesh of the frame (CUDAMesh, CustomCUDARasterizer/CUDAMesh.h:27-65)
// with the matrices Render() uploads to constant memory
// (CUDARenderer.cu:237-247): WVP = Proj * View * World, World.
struct MeshDev {
    const void* vertices;
    const uint32_t* indices;   // null: non-indexed list
    uint32_t vertex_format;
    uint32_t topology;
    uint32_t num_vertices;
    uint32_t num_tris;
    uint32_t prim_base;
    uint32_t pad[3];
    float wvp[16];
    float world[16];
    TexDev tex[4];
};

// A scene light (the build's shading extension; gbr_light in gbr.h).
constexpr uint32_t kMaxLights = 8;
struct LightDev {
    uint32_t type;        // 0 directional (vec = travel direction), 1 point (vec = position)
    float colour[3];
    float intensity;
    float vec[3];
};
static_assert(sizeof(LightDev) == 32, "light record is 32 bytes");

// Raster setup record, 48 B: the triangle's float screen vertices (the
// raster snaps them to 16.16 for coverage), NDC z per vertex, 1 / the float
// area the reference divides its weights by, flags, mesh index.
struct __align__(16) TriSetup {
    float x0, y0, x1, y1;
    float x2, y2;
    float z0, z1;
    float z2, inv_area;
    uint32_t flags;
    uint32_t mesh;
};
static_assert(sizeof(TriSetup) == 48, "setup record is 48 bytes");

// Device-side control block of one frame.
struct Ctl {
    unsigned long long num_pairs;
    uint32_t num_visible;
    uint32_t num_float_path;
    uint32_t num_items;
    uint32_t item_next;
    uint32_t overflow;         // bin storage too small: the frame was not rasterised
    uint32_t pred_overflow;    // a predicted per-bin capacity was exceeded
    unsigned long long pred_capacity;
    uint32_t error;            // non-zero: a bounded wait gave up
    uint32_t num_sampled;      // visible triangles seen by the coarse pre-pass
    unsigned long long items_alloc;   // batch: work items requested by all scenes
    uint32_t rank_next;        // exact binning: rank slots reserved by the count pass
    uint32_t shade_count;      // two-pass shading: covered pixels queued by the light pass
};
static_assert(sizeof(Ctl) == 64, "control block is 64 bytes");

// Everything a kernel of the frame needs, passed by value.
struct FrameDev {
    uint32_t width, height;
    uint32_t nbx, nby, bw, bh, num_bins;
    uint32_t cull, sample, vis, clear_colour32;
    uint32_t num_meshes, num_tris;
    uint32_t chunk;
    uint32_t phase;           // triangles between hierarchical-z refreshes (0: kPhase)
    uint32_t raster_ctas;     // raster_kernel variant: CTAs per SM it is compiled for (0: default)
    float cam_pos[3];
    float cam_fwd[3];
    const MeshDev* meshes;
    TriSetup* setup;
    uint2* rects;
    uint32_t* keys;            // per triangle: lower bound of its fragments' depth keys (hiz_key)
    uint32_t* counts;          // kCountSplit sub-counters per bin: counts[k * count_stride + bin]
    uint32_t* sub_base;        // first list entry of each sub-counter's pairs (same layout)
    uint32_t* offsets;        // num_bins + 1
    uint32_t* cursors;
    uint32_t* capacity;       // predicted per-bin capacity (predicted binning)
    uint32_t* bin_end;        // predicted binning: offset + capacity of each bin (the capacity scan writes it)
    uint4* items;
    uint32_t items_cap;
    uint32_t* list;
    unsigned long long list_cap;
    uint32_t* colour;
    float* depth;
    uint32_t* ids;
    unsigned long long* gvis;
    Ctl* ctl;
    // predicted-capacity binning
    uint32_t* feat;            // coarse pre-pass accumulators, kFeatSlots x num_bins (slot-major)
    const uint16_t* mlp_w;     // capacity model parameters, BF16
    float* features_out;       // optional: kFeatures features per bin (training data)
    float cap_alpha, cap_beta, cap_gamma;  // capacity = ceil(l*(1+alpha) + beta*sqrt(l+1) + gamma)
    uint32_t sample_stride;    // the pre-pass samples one triangle per group of sample_stride
    uint32_t exact_guard;      // exact-binning kernels run only after a predicted overflow
    const LightDev* lights;    // scene lights (num_lights == 0: the reference shader's constant light)
    uint32_t num_lights;
    uint32_t flat_shade;      // PBR view and no mesh with a diffuse map: pixels shade from vertex colours
    struct ScanState* scan_state;   // bin scan scratch (scan_state_bytes)
    // exact binning: the count pass keeps each (triangle, bin) pair's rank
    // within its bin, so the fill pass stores every entry without atomics
    uint32_t* ranks;           // rank_cap slots; a warp's walk owns a contiguous run
    uint32_t* walk_base;       // first slot of each walk (walk = triangle slot / 32)
    uint32_t* rank_next;       // slot reservation counter (a Ctl's rank_next)
    unsigned long long rank_cap;
    uint32_t count_stride;     // bins between sub-counter rows (the scan's bin count)
    uint32_t count_split;      // sub-counters per bin in use: 1, 2, 4 or 8
    // exact binning with block-private counter rows (row_blocks > 0)
    uint32_t* row_base;        // row_blocks x num_bins: a block's first entry in each bin it touched, bin-relative
    uint32_t row_blocks;       // blocks of the count and fill passes (0: sub-counters)
    uint32_t touch_words;      // block rows: 16-byte words of the list the count pass zeroes (list_touch_kernel)
    uint32_t* shade_list;      // two-pass shading: covered pixels' indices, width x height slots (null: one pass)
    // bin-scan waits: polls of one flag before a wait gives up (0: the
    // library's bound), and 1 + the index of a tile that publishes nothing
    // (0: none) -- the test hook that makes a bounded wait run out
    uint32_t scan_spin_limit;
    uint32_t scan_silent_tile1;
    // raster pass size (the reference's queue size, SetupBins'
    // queueMaxSize): a work item's entries are depth-sorted and rasterised
    // into the tile this many at a time (0 or above kBatch: kBatch)
    uint32_t stage;
    // a frame split across GPUs by bin rows: this frame bins and
    // rasterises bin rows [row0, row1) and shades pixels [px_begin, px_end)
    // (row1 = 0: every row; px_end = 0: every pixel)
    uint32_t row0, row1;
    uint32_t px_begin, px_end;
    uint32_t rec_tma;          // raster: setup records staged by bulk asynchronous copies (1) or loads (0)
    uint32_t raster_lanes;     // raster: the small-triangle variant (a lane per triangle; phases >= kLanePhase)
    uint32_t rows_pad;
    // two-pass shading of a sparse frame: one byte per bin, "may hold drawn
    // pixels".  dirty_rd: after the last frame; dirty_wr: this frame's, zeroed
    // by its first scan and set by the raster for every bin it draws.  The
    // light pass leaves the quads of bins clean in both untouched: their
    // pixels already hold the clear values.  (null: every pixel is written)
    uint8_t* dirty_rd;
    uint8_t* dirty_wr;
};
static_assert(sizeof(FrameDev) % 16 == 0, "frame descriptors are copied as 16-byte words");

// The bin scan (gbr_scan.cu) over n per-bin sizes.
enum : uint32_t {
    kScanExact = 0,                // exact counts -> offsets, cursors, work items
    kScanCapacity = 1,             // predicted capacities -> offsets, cursors
    kScanExactAfterPredicted = 2,  // as kScanExact, run only after a predicted overflow
    kScanPredictedItems = 3        // filled sizes within the capacities -> work items
};
// Single-pass bin scan (decoupled look-back): tiles of 1024 bins take
// tickets in launch order, publish their totals, then their inclusive
// prefixes; a tile sums its predecessors' totals back to the nearest
// published prefix.  Flags carry the scan's sequence tag, so the state needs
// zeroing once when allocated and never between scans.
struct ScanTile {
    uint32_t flag;                  // tag << 2 | kTileAggregate / kTilePrefix
    uint32_t pad;
    unsigned long long agg_a, agg_b;   // the tile's bin entries and work items
    unsigned long long inc_a, inc_b;   // inclusive prefixes (valid with kTilePrefix)
    unsigned long long pad2;
};
struct ScanState {
    uint32_t ticket;                // next tile of the running scan
    uint32_t seq;                   // scans completed (tags the flags)
    uint32_t pad[6];
};
static_assert(sizeof(ScanTile) == 48 && sizeof(ScanState) == 32, "scan state layout");
enum : uint32_t { kTileAggregate = 1, kTilePrefix = 2 };
__host__ __device__ constexpr size_t scan_state_bytes(uint32_t num_bins) {
    return sizeof(ScanState) + sizeof(ScanTile) * (size_t)(num_bins == 0 ? 1u : (num_bins + 1023u) / 1024u);
}

struct ScanDev {
    uint32_t* counts;              // exact sub-counts (kCountSplit rows of stride n), zeroed for the next frame
    uint32_t* sub_base;            // exact modes: list start of each sub-count (same layout)
    uint32_t split;                // sub-counters per bin in use
    const uint32_t* capacity;      // predicted capacities
    uint32_t* offsets;             // n + 1
    uint32_t* cursors;
    uint32_t* ends;                // kScanCapacity: offset + capacity of each bin
    uint4* items;
    ScanState* state;
    Ctl* ctl;
    uint32_t* feat;                // kScanPredictedItems: pre-pass accumulators to reset (or null)
    unsigned long long list_cap;
    uint32_t items_cap;
    uint32_t n;
    uint32_t chunk;
    uint32_t mode;
    uint32_t spin_limit;           // polls of one flag before a look-back wait gives up (0: kScanSpinLimit)
    uint32_t silent_tile1;         // 1 + a tile that publishes nothing (0: none; test hook)
    uint8_t* dirty;                // the frame's per-bin drawn flags to zero (FrameDev::dirty_wr; null: none)
};

// Many scenes rendered as one batch frame.  Each scene keeps its own frame
// descriptor (its resolution, bins, meshes, frame buffers, statistics
// block); bin counters, setup records and the bin list are slices of
// batch-wide arrays, and the raster work items of all scenes share one
// queue.  The block tables map a grid's blocks to scenes: scene s owns
// blocks [tri_blocks[s], tri_blocks[s+1]) of the setup and fill grids and
// [px_blocks[s], px_blocks[s+1]) of the shade grid; its bins are global
// bins [bin_base[s], bin_base[s+1]).
struct BatchDev {
    const FrameDev* scenes;
    const uint32_t* tri_blocks;   // num_scenes + 1
    const uint32_t* px_blocks;    // num_scenes + 1
    const uint32_t* bin_base;     // num_scenes + 1
    const uint32_t* tri_scene;    // per triangle-pass block: its scene
    const uint32_t* px_scene;     // per pixel-pass block: its scene
    const uint32_t* bin_scene;    // per global bin: its scene
    uint4* items;                 // (global bin, list start, count, chunks of the bin)
    Ctl* ctl;                     // the batch's list/item allocation, work queue and overflow flag
    unsigned long long list_cap;
    uint32_t items_cap;
    uint32_t num_scenes;
    uint32_t phase;               // raster: triangles between hierarchical-z refreshes (0: kPhase)
    uint32_t all_flat;            // every scene shades flat: the shade pass runs its flat variant
    uint32_t stage;               // raster pass size (FrameDev::stage)
};

// ---------------------------------------------------------------------------
// Conversions with the semantics of nvcc's cvt.rzi (saturating, NaN -> 0),
// written out so that the result does not depend on how a cast is lowered.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int cvt_s32(float x) {
    if (x != x) return 0;
    if (x >= 2147483648.0f) return 2147483647;
    if (x <= -2147483648.0f) return (int)0x80000000u;
    return __float2int_rz(x);
}

__device__ __forceinline__ int cvt_s16(float x) {
    if (x != x) return 0;
    if (x >= 32767.0f) return 32767;
    if (x <= -32768.0f) return -32768;
    return __float2int_rz(x);
}

__device__ __forceinline__ uint32_t cvt_u8(float x) {
    if (!(x > 0.0f)) return 0u;
    if (x >= 255.0f) return 255u;
    return (uint32_t)__float2int_rz(x);
}

__device__ __forceinline__ float M4(const float* m, int r, int c) { return m[c * 4 + r]; }

struct F3 { float x, y, z; };

__device__ __forceinline__ F3 f3(float x, float y, float z) { F3 o; o.x = x; o.y = y; o.z = z; return o; }
__device__ __forceinline__ F3 sub3(F3 a, F3 b) { return f3(__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z)); }
__device__ __forceinline__ float dot3(F3 a, F3 b) { return __fmaf_rn(a.z, b.z, __fmaf_rn(a.x, b.x, __fmul_rn(a.y, b.y))); }
__device__ __forceinline__ F3 cross3(F3 a, F3 b) {
    return f3(__fmaf_rn(a.y, b.z, -__fmul_rn(a.z, b.y)),
              __fmaf_rn(a.z, b.x, -__fmul_rn(a.x, b.z)),
              __fmaf_rn(a.x, b.y, -__fmul_rn(a.y, b.x)));
}
// Normalize (Vector.h:41-56): zero vector for zero magnitude.
__device__ __forceinline__ F3 normalize3(F3 v) {
    const float m = __fsqrt_rn(dot3(v, v));
    if (m == 0.0f) return f3(0.f, 0.f, 0.f);
    const float inv = __fdiv_rn(1.0f, m);
    return f3(__fmul_rn(v.x, inv), __fmul_rn(v.y, inv), __fmul_rn(v.z, inv));
}

// Matrix<4,4> * Point4(p, 1) (Matrix4.h:158-166) as fused in GetNDCVertex.
__device__ __forceinline__ float4 xform_point(const float* m, float px, float py, float pz) {
    float4 o;
    o.x = __fadd_rn(__fmaf_rn(M4(m, 0, 2), pz, __fmaf_rn(M4(m, 0, 0), px, __fmul_rn(M4(m, 0, 1), py))), M4(m, 0, 3));
    o.y = __fadd_rn(__fmaf_rn(M4(m, 1, 2), pz, __fmaf_rn(M4(m, 1, 0), px, __fmul_rn(M4(m, 1, 1), py))), M4(m, 1, 3));
    o.z = __fadd_rn(__fmaf_rn(M4(m, 2, 2), pz, __fmaf_rn(M4(m, 2, 0), px, __fmul_rn(M4(m, 2, 1), py))), M4(m, 2, 3));
    o.w = __fadd_rn(__fmaf_rn(M4(m, 3, 2), pz, __fmaf_rn(M4(m, 3, 0), px, __fmul_rn(M4(m, 3, 1), py))), M4(m, 3, 3));
    return o;
}

// Matrix<3,3> * Vector3 (Matrix3.h:126-133) on the upper 3x3 of a 4x4.
__device__ __forceinline__ F3 rot3(const float* m, F3 v) {
    return f3(__fmaf_rn(M4(m, 0, 2), v.z, __fmaf_rn(M4(m, 0, 0), v.x, __fmul_rn(M4(m, 0, 1), v.y))),
              __fmaf_rn(M4(m, 1, 2), v.z, __fmaf_rn(M4(m, 1, 0), v.x, __fmul_rn(M4(m, 1, 1), v.y))),
              __fmaf_rn(M4(m, 2, 2), v.z, __fmaf_rn(M4(m, 2, 0), v.x, __fmul_rn(M4(m, 2, 1), v.y))));
}

// Position of vertex vi (object space).
__device__ __forceinline__ F3 fetch_position(const MeshDev& m, uint32_t vi) {
    if (m.vertex_format == kVertexPos3Rgba8) {
        const float4 v = __ldg(reinterpret_cast<const float4*>(m.vertices) + vi);
        return f3(v.x, v.y, v.z);
    }
    const float* b = reinterpret_cast<const float*>(m.vertices) + 14u * (size_t)vi;
    const float2 xy = __ldg(reinterpret_cast<const float2*>(b));
    return f3(xy.x, xy.y, __ldg(b + 2));
}

// Triangle assembly (TA_Kernel, CUDARenderer.cu:716-753); strips use the
// intended order (the reference's strip branch reads an uninitialised
// triangle).
__device__ __forceinline__ void tri_vertex_ids(const MeshDev& m, uint32_t local, uint32_t v[3]) {
    if (!m.indices) {
        v[0] = 3u * local; v[1] = 3u * local + 1u; v[2] = 3u * local + 2u;
    } else if (m.topology == 0u) {
        v[0] = __ldg(m.indices + 3u * local); v[1] = __ldg(m.indices + 3u * local + 1u);
        v[2] = __ldg(m.indices + 3u * local + 2u);
    } else {
        v[0] = __ldg(m.indices + local); v[1] = __ldg(m.indices + local + 1u); v[2] = __ldg(m.indices + local + 2u);
        if (local & 1u) { const uint32_t s = v[1]; v[1] = v[2]; v[2] = s; }
    }
}

// NDC -> screen (NDCToScreenSpace, CUDAROPs.cu:88-97).
__device__ __forceinline__ float2 to_screen(float x, float y, uint32_t w, uint32_t h) {
    float2 s;
    s.x = __fmul_rn(__fdiv_rn(__fadd_rn(x, 1.f), 2.f), (float)w);
    s.y = __fmul_rn(__fdiv_rn(__fsub_rn(1.f, y), 2.f), (float)h);
    return s;
}

__device__ __forceinline__ float min3f(float a, float b, float c) {
    float m = a;
    if (b < m) m = b;
    if (c < m) m = c;
    return m;
}
__device__ __forceinline__ float max3f(float a, float b, float c) {
    float m = a;
    if (b > m) m = b;
    if (c > m) m = c;
    return m;
}
__device__ __forceinline__ int clampi(int v, int lo, int hi) {
    const int c = v < lo ? lo : v;
    return c > hi ? hi : c;
}

// GetBoundingBox (CUDAROPs.cu:180-200) with short arithmetic, then the
// TB_Kernel bin range (CUDARenderer.cu:935-942).  Returns x0,y0,x1,y1.
__device__ __forceinline__ int4 bin_rect(float2 s0, float2 s1, float2 s2, const FrameDev& F) {
    int xmin = (int)(short)(cvt_s16(min3f(s0.x, s1.x, s2.x)) - 1);
    int ymin = (int)(short)(cvt_s16(min3f(s0.y, s1.y, s2.y)) - 1);
    int xmax = (int)(short)(cvt_s16(max3f(s0.x, s1.x, s2.x)) + 1);
    int ymax = (int)(short)(cvt_s16(max3f(s0.y, s1.y, s2.y)) + 1);
    xmin = clampi(xmin, 0, (int)(short)F.width);
    ymin = clampi(ymin, 0, (int)(short)F.height);
    xmax = clampi(xmax, 0, (int)(short)F.width);
    ymax = clampi(ymax, 0, (int)(short)F.height);
    int4 r;
    r.x = clampi(xmin / (int)F.bw, 0, (int)F.nbx);
    r.y = clampi(ymin / (int)F.bh, 0, (int)F.nby);
    r.z = clampi(xmax / (int)F.bw, 0, (int)F.nbx - 1);
    r.w = clampi(ymax / (int)F.bh, 0, (int)F.nby - 1);
    if (F.row1) {   // a frame split by bin rows keeps this GPU's rows (empty if none)
        r.y = max(r.y, (int)F.row0);
        r.w = min(r.w, (int)F.row1 - 1);
    }
    return r;
}

// Packed bin rectangle: x = bx0 | bx1 << 16, y = by0 | by1 << 16 | noRaster << 31.
__device__ __forceinline__ uint2 pack_rect(int4 r, bool no_raster) {
    uint2 p;
    p.x = (uint32_t)r.x | ((uint32_t)r.z << 16);
    p.y = (uint32_t)r.y | ((uint32_t)r.w << 16) | (no_raster ? 0x80000000u : 0u);
    return p;
}
__device__ __forceinline__ uint2 empty_rect() { return make_uint2(1u, 0u); }

// Exact 16.16 edge function E(P; A, B) = (P - A) x (B - A), units 2^-32 px^2.
__device__ __forceinline__ long long edge_fx(int px_fx, int py_fx, int ax, int ay, int dx, int dy) {
    return (long long)(px_fx - ax) * (long long)dy - (long long)(py_fx - ay) * (long long)dx;
}

// z = w2*z2 + w0*z0 + w1*z1 in the reference's fused order (CUDAROPs.cu:341).
__device__ __forceinline__ float interp_z(float w0, float w1, float w2, float z0, float z1, float z2) {
    return __fmaf_rn(w2, z2, __fmaf_rn(w0, z0, __fmul_rn(w1, z1)));
}

__device__ __forceinline__ int snap_fx(float v) { return __float2int_rn(__fmul_rn(v, 65536.f)); }

// The reference's float edge functions at a pixel (IsPixelInTriangle,
// CUDAROPs.cu:120-142): w[2] from edge v0->v1, w[0] from v1->v2, w[1] from
// v2->v0.
__device__ __forceinline__ void edges_ref(const TriSetup& t, float px, float py, float w[3]) {
    const float eax = __fsub_rn(t.x1, t.x0), eay = __fsub_rn(t.y1, t.y0);
    const float ebx = __fsub_rn(t.x2, t.x1), eby = __fsub_rn(t.y2, t.y1);
    const float ecx = __fsub_rn(t.x0, t.x2), ecy = __fsub_rn(t.y0, t.y2);
    w[2] = __fmaf_rn(__fsub_rn(px, t.x0), eay, -__fmul_rn(__fsub_rn(py, t.y0), eax));
    w[0] = __fmaf_rn(__fsub_rn(px, t.x1), eby, -__fmul_rn(__fsub_rn(py, t.y1), ebx));
    w[1] = __fmaf_rn(__fsub_rn(px, t.x2), ecy, -__fmul_rn(__fsub_rn(py, t.y2), ecx));
}

// Interpolation weights of a pixel covered under the fixed-point rule: the
// reference's float edge values times 1/area (coverage itself is decided on
// the snapped triangle by the raster).
__device__ __forceinline__ void weights_fixed(const TriSetup& t, int x, int y, float w[3]) {
    edges_ref(t, (float)x, (float)y, w);
    w[0] = __fmul_rn(w[0], t.inv_area);
    w[1] = __fmul_rn(w[1], t.inv_area);
    w[2] = __fmul_rn(w[2], t.inv_area);
}

// Float coverage and weights as IsPixelInTriangle + normalisation
// (CUDAROPs.cu:120-145, 334-339), for triangles outside the guard band.
__device__ __forceinline__ bool weights_float(const TriSetup& t, float px, float py, float w[3]) {
    edges_ref(t, px, py, w);
    if (!(w[0] >= 0.f && w[1] >= 0.f && w[2] >= 0.f)) return false;
    const float ax = __fsub_rn(t.x0, t.x1), ay = __fsub_rn(t.y0, t.y1);
    const float bx = __fsub_rn(t.x0, t.x2), by = __fsub_rn(t.y0, t.y2);
    const float area = fabsf(__fmaf_rn(ax, by, -__fmul_rn(ay, bx)));
    w[0] = __fdiv_rn(w[0], area);
    w[1] = __fdiv_rn(w[1], area);
    w[2] = __fdiv_rn(w[2], area);
    return true;
}

// Position of the n-th lowest set bit of m (1 <= n <= popc(m)).
__device__ __forceinline__ uint32_t nth_set_bit(uint32_t m, uint32_t n) {
    uint32_t pos = 0;
#pragma unroll
    for (uint32_t s = 16; s >= 1; s >>= 1) {
        const uint32_t c = __popc(m & ((1u << s) - 1u));
        if (c < n) { n -= c; m >>= s; pos += s; }
    }
    return pos;
}

// Walks the bins of the warp's packed rectangles; called by whole warps of
// 256-thread blocks (kRowThreads blocks in modes 4 and 5).  The warp's (triangle, bin) pairs are expanded
// load-balanced, 32 consecutive pairs per round: the lane whose pair range
// covers the round's first pair is found with a ballot, the starts of the
// other ranges inside the round with one OR-reduction, and a lane's pair
// belongs to the r-th non-empty range after the first, r = the starts at or
// before it -- integer-pipe work, with one shared-memory load for the
// owner's rectangle.  A lane takes up to kPairsPerLane pairs per pass and
// issues their atomics back to back: atomics with return are bound by their
// latency, so several must be in flight per lane.
// Mode 0: count (atomicAdd on the walk's sub-counter of the bin; its return,
// the pair's rank there, is kept in the walk's rank slots), 1: fill (entry
// at the sub-counter's list start + rank: no atomics), 2: predicted fill (append within the bin's predicted
// capacity), 3: pre-pass count (atomicAdd on the first feature slot),
// 4: count into the block's shared-memory row `s_row` (no return), 5: fill
// from the block's shared-memory cursors `s_row` (kRowThreads blocks).  A
// walk is identified by `walk` (its first triangle slot / 32), so the count
// and fill passes of the same triangles meet the same slots.  One atomic per
// pair: merging the atomics of same-bin lanes -- every such lane of the warp
// (__match_any_sync) or runs of neighbouring lanes -- measured 8-10% slower
// on GB300 for both the 1M soup and the 4K icosphere.
#ifndef GBR_PAIRS_PER_LANE
#define GBR_PAIRS_PER_LANE 4
#endif
constexpr uint32_t kPairsPerLane = GBR_PAIRS_PER_LANE;

template <int MODE>
__device__ __forceinline__ void bin_walk(const FrameDev& F, uint2 rect, uint32_t entry, bool valid, uint32_t walk,
                                         uint32_t* s_row = nullptr) {
    constexpr uint32_t kWarps = MODE >= 4 ? kRowThreads / 32u : 8u;
    __shared__ uint4 s_tab[kWarps][32];   // per warp: (first pair, width, bx0 | by0 << 16, entry) of each lane
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint32_t bx0 = rect.x & 0xFFFFu, bx1 = rect.x >> 16;
    const uint32_t by0 = rect.y & 0xFFFFu, by1 = (rect.y >> 16) & 0x7FFFu;
    uint32_t w = 0, n = 0;
    if (valid && bx0 <= bx1 && by0 <= by1) {
        w = bx1 - bx0 + 1u;
        n = w * (by1 - by0 + 1u);
    }
    uint32_t incl = n;   // inclusive prefix of pair counts over the warp
#pragma unroll
    for (uint32_t d = 1; d < 32; d <<= 1) {
        const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, incl, d);
        if (lane >= d) incl += t;
    }
    const uint32_t total = __shfl_sync(0xFFFFFFFFu, incl, 31);
    if (total == 0u) return;   // warp-uniform
    const uint32_t excl = incl - n;
    // exact binning: the walk's rank slots, reserved by the count pass and
    // found again by the fill pass (same triangles, same enumeration)
    uint32_t wb = 0;
    const uint32_t krow = (walk & (F.count_split - 1u)) * F.count_stride;   // the walk's sub-counter row
    if (MODE == 0) {
        if (lane == 0) {
            wb = atomicAdd(F.rank_next, total);
            F.walk_base[walk] = wb;
        }
        wb = __shfl_sync(0xFFFFFFFFu, wb, 0);
    } else if (MODE == 1) {
        wb = __ldg(&F.walk_base[walk]);
    }
    s_tab[warp][lane] = make_uint4(excl, w, bx0 | (by0 << 16), entry);
    __syncwarp();
    const uint32_t nonempty = __ballot_sync(0xFFFFFFFFu, n != 0u);
    const uint32_t upto = lane == 31u ? 0xFFFFFFFFu : ((2u << lane) - 1u);   // bits 0..lane
    for (uint32_t base = 0; base < total; base += 32u * kPairsPerLane) {   // warp-uniform
        uint32_t bin[kPairsPerLane], ent[kPairsPerLane];
        bool act[kPairsPerLane];
#pragma unroll
        for (uint32_t u = 0; u < kPairsPerLane; ++u) {
            act[u] = false;
            bin[u] = 0u;
            ent[u] = 0u;
            const uint32_t b = base + u * 32u;
            if (b >= total) continue;   // warp-uniform
            const uint32_t start = (n != 0u && excl > b && excl - b < 32u) ? (1u << (excl - b)) : 0u;
            const uint32_t starts = __reduce_or_sync(0xFFFFFFFFu, start);
            const uint32_t first = (uint32_t)(__ffs(__ballot_sync(0xFFFFFFFFu, n != 0u && excl <= b && b < incl)) - 1);
            const uint32_t r = (uint32_t)__popc(starts & upto);
            const uint32_t after = first == 31u ? 0u : nonempty & ~((2u << first) - 1u);
            const uint32_t o = r == 0u ? first : nth_set_bit(after, r);
            const uint4 d = s_tab[warp][o & 31u];
            const uint32_t k = b + lane;
            act[u] = k < total;
            const uint32_t j = k - d.x;
            const uint32_t q = act[u] ? j / d.y : 0u;
            bin[u] = ((d.z & 0xFFFFu) + (j - q * d.y)) + ((d.z >> 16) + q) * F.nbx;
            ent[u] = d.w;
        }
        if (MODE == 3) {
#pragma unroll
            for (uint32_t u = 0; u < kPairsPerLane; ++u)
                if (act[u]) atomicAdd(&F.feat[bin[u]], 1u);
        } else if (MODE == 4) {
#pragma unroll
            for (uint32_t u = 0; u < kPairsPerLane; ++u)
                if (act[u]) atomicAdd(&s_row[bin[u]], 1u);
        } else if (MODE == 5) {
            uint32_t pos[kPairsPerLane];
#pragma unroll
            for (uint32_t u = 0; u < kPairsPerLane; ++u) pos[u] = act[u] ? atomicAdd(&s_row[bin[u]], 1u) : 0u;
#pragma unroll
            for (uint32_t u = 0; u < kPairsPerLane; ++u)
                if (act[u]) F.list[pos[u]] = ent[u];
        } else if (MODE == 0) {
            // count, keeping the pair's rank within its bin (slots past the
            // storage are dropped: that frame overflows and is not filled)
            uint32_t rank[kPairsPerLane];
#pragma unroll
            for (uint32_t u = 0; u < kPairsPerLane; ++u) rank[u] = act[u] ? atomicAdd(&F.counts[krow + bin[u]], 1u) : 0u;
#pragma unroll
            for (uint32_t u = 0; u < kPairsPerLane; ++u) {
                const unsigned long long slot = (unsigned long long)wb + base + u * 32u + lane;
                if (act[u] && slot < F.rank_cap) F.ranks[slot] = rank[u];
            }
        } else if (MODE == 1) {
            // fill: the sub-counter's list start plus the rank the count pass kept
            uint32_t rank[kPairsPerLane];
#pragma unroll
            for (uint32_t u = 0; u < kPairsPerLane; ++u) rank[u] = act[u] ? __ldg(&F.ranks[wb + base + u * 32u + lane]) : 0u;
#pragma unroll
            for (uint32_t u = 0; u < kPairsPerLane; ++u)
                if (act[u]) F.list[__ldg(&F.sub_base[krow + bin[u]]) + rank[u]] = ent[u];
        } else {
            uint32_t pos[kPairsPerLane];
#pragma unroll
            for (uint32_t u = 0; u < kPairsPerLane; ++u) pos[u] = act[u] ? atomicAdd(&F.cursors[bin[u]], 1u) : 0u;
#pragma unroll
            for (uint32_t u = 0; u < kPairsPerLane; ++u) {
                if (!act[u]) continue;
                // cursors start at the bin's offset; the bin owns capacity[bin] slots
                if (pos[u] < __ldg(&F.offsets[bin[u]]) + __ldg(&F.capacity[bin[u]])) F.list[pos[u]] = ent[u];
                else atomicOr(&F.ctl->pred_overflow, 1u);
            }
        }
    }
    __syncwarp();   // the warp's table row is rewritten by its next walk
}

}  // namespace gbr
