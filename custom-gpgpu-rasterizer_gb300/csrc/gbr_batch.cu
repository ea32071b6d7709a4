// gbr_batch.cu -- batched frames: many scenes rendered by one persistent
// launch chain, replayed from a CUDA graph, with an autotuner for the bin
// size, queue chunk and raster variant.
//
// The reference renders one scene per Render() call, with a launch chain
// per mesh and a binner launch per 256 triangles, each followed by a device
// synchronisation (CustomCUDARasterizer/CUDARenderer.cu:249-339).  Here a
// batch frame is six kernels whatever the number of scenes, meshes or
// triangles: reset, setup + count over the triangles of every scene, one
// scan CTA per scene, fill, one persistent raster over the work items
// (scene, bin, chunk) of every scene, and shade over every scene's pixels.
//
// Host-side state per batch frame:
//   layout   -- per-scene bin grids, triangle and pixel block ranges, and the
//               slices of the batch-wide bin and setup arrays; rebuilt when a
//               scene's resolution or triangle count or the configuration
//               changes (the CUDA graph is then captured again).
//   table    -- per-scene frame descriptors and per-mesh descriptors (camera
//               matrices, textures), uploaded through a double-buffered
//               pinned staging area before the graph launch when it changed.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/gbr.h"
#include "gbr_internal.h"
#include "gbr_kernels.h"

using namespace gbr;

namespace {

struct Member {
    gbr_renderer* r = nullptr;
    gbr_camera cam{};
    uint32_t cull = 0, sample = 0, vis = 0;
};

struct SceneLayout {
    uint32_t W = 0, H = 0, nbx = 0, nby = 0, num_meshes = 0;
    uint64_t tris = 0;
    uint32_t bin_base = 0, mesh_base = 0;
    uint64_t tri_base = 0;
};

}  // namespace

struct gbr_batch {
    int device = 0;
    int num_sms = 0;
    std::vector<Member> members;
    gbr_batch_config cfg{16u, 64u, 0u, 0u, 0u};
    bool timing = false;

    // layout
    bool layout_valid = false;
    std::vector<SceneLayout> layout;
    uint32_t total_bins = 0, total_meshes = 0;
    uint64_t total_tris = 0;
    uint32_t tri_blocks = 0, px_blocks = 0;
    int raster_bps = 1;

    // device storage
    uint32_t* d_tables = nullptr;        // tri_blocks | px_blocks | bin_base (num_scenes + 1 each) | tri_scene | px_scene | bin_scene
    uint32_t* d_counts = nullptr;     // kCountSplit x bins
    uint32_t* d_sub_base = nullptr;   // kCountSplit x bins
    uint32_t count_split = 1;         // sub-counters per bin in use
    uint32_t all_flat = 0;            // every scene shades flat (the captured shade variant)
    uint32_t* d_offsets = nullptr;
    uint32_t* d_cursors = nullptr;
    ScanState* d_scan = nullptr;   // bin scan state (zeroed once)
    TriSetup* d_setup = nullptr;
    uint2* d_rects = nullptr;
    uint32_t* d_walk = nullptr;     // first rank slot of each 32-triangle walk (8 per block)
    uint32_t* d_keys = nullptr;     // per-triangle depth-key bounds
    uint32_t* d_list = nullptr;
    uint64_t list_cap = 0;
    uint4* d_items = nullptr;
    uint32_t items_cap = 0;
    Ctl* d_ctl = nullptr;
    Ctl* h_ctl = nullptr;
    unsigned char* d_table = nullptr;    // FrameDev[num_scenes] then MeshDev[total_meshes]
    unsigned char* h_staging[2] = {nullptr, nullptr};
    cudaEvent_t staging_evt[2] = {nullptr, nullptr};
    size_t table_cap = 0;
    int staging_next = 0;
    std::vector<unsigned char> last_table;

    // graph
    cudaStream_t cap_stream = nullptr;
    cudaGraphExec_t graph = nullptr;
    uint32_t graph_captures = 0;

    // frame state
    bool have_frame = false;
    bool frame_checked = false;   // finish_batch has waited for and checked the last frame
    cudaStream_t last_stream = nullptr;
    uint32_t overflow_reruns = 0;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    bool ev_recorded = false;
};

namespace {

uint32_t ceil_div(uint64_t a, uint64_t b) { return (uint32_t)((a + b - 1u) / b); }

// raster CTA width of a configuration (0: 256)
uint32_t raster_threads(const gbr_batch_config& c) { return c.raster_threads == 128u ? 128u : 256u; }

void drop_graph(gbr_batch* b) {
    if (b->graph) cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
}

void free_layout_storage(gbr_batch* b) {
    cudaFree(b->d_tables); cudaFree(b->d_counts); cudaFree(b->d_sub_base); cudaFree(b->d_offsets); cudaFree(b->d_cursors);
    cudaFree(b->d_setup); cudaFree(b->d_rects); cudaFree(b->d_scan); cudaFree(b->d_walk); cudaFree(b->d_keys);
    b->d_tables = b->d_counts = b->d_offsets = b->d_cursors = nullptr;
    b->d_sub_base = nullptr;
    b->d_scan = nullptr;
    b->d_setup = nullptr;
    b->d_rects = nullptr;
    b->d_walk = nullptr;
    b->d_keys = nullptr;
}

gbr_status ensure_list(gbr_batch* b, uint64_t pairs, uint64_t items) {
    if (pairs <= b->list_cap && items <= b->items_cap && b->d_list && b->d_items) return GBR_OK;
    uint64_t cap = std::max<uint64_t>(std::max<uint64_t>(pairs + pairs / 4u, b->list_cap), 1u << 20);
    if (cap > 0x7FFFFFFFull) cap = 0x7FFFFFFFull;
    if (pairs > cap) return fail(GBR_ERR_OUT_OF_MEMORY, "batch needs %llu bin entries (max 2^31-1)", (unsigned long long)pairs);
    uint64_t icap = std::max<uint64_t>(items + items / 4u, (uint64_t)b->total_bins + cap / kBatchChunk + 1u);
    icap = std::max<uint64_t>(icap, b->items_cap);
    if (icap > 0xFFFFFFFFull) icap = 0xFFFFFFFFull;
    drop_graph(b);
    cudaFree(b->d_list);
    cudaFree(b->d_items);
    b->d_list = nullptr;
    b->d_items = nullptr;
    // the bin list, then as many rank slots (exact binning's count pass)
    if (cudaMalloc(&b->d_list, 2u * cap * sizeof(uint32_t)) != cudaSuccess ||
        cudaMalloc(&b->d_items, icap * sizeof(uint4)) != cudaSuccess) {
        cudaGetLastError();
        b->list_cap = 0;
        b->items_cap = 0;
        return fail(GBR_ERR_OUT_OF_MEMORY, "cannot allocate %llu bin entries", (unsigned long long)cap);
    }
    b->list_cap = cap;
    b->items_cap = (uint32_t)icap;
    return GBR_OK;
}

// Rebuilds the layout if a scene's resolution, mesh count or triangle count
// or the configuration changed since the last frame.
gbr_status ensure_layout(gbr_batch* b) {
    const uint32_t n = (uint32_t)b->members.size();
    const uint32_t bs = b->cfg.bin_size;
    bool same = b->layout_valid && b->layout.size() == n;
    for (uint32_t i = 0; same && i < n; ++i) {
        const gbr_renderer* r = b->members[i].r;
        const SceneLayout& L = b->layout[i];
        same = L.W == r->W && L.H == r->H && L.num_meshes == r->meshes.size() && L.tris == scene_triangles(r);
    }
    if (same) return GBR_OK;

    drop_graph(b);
    free_layout_storage(b);
    b->layout.assign(n, SceneLayout());
    uint64_t bins = 0, tris = 0, tri_blocks = 0, px_blocks = 0;
    uint32_t meshes = 0;
    std::vector<uint32_t> tables(3u * (n + 1u));
    for (uint32_t i = 0; i < n; ++i) {
        const gbr_renderer* r = b->members[i].r;
        SceneLayout& L = b->layout[i];
        L.W = r->W;
        L.H = r->H;
        L.nbx = ceil_div(r->W, bs);
        L.nby = ceil_div(r->H, bs);
        L.num_meshes = (uint32_t)r->meshes.size();
        L.tris = scene_triangles(r);
        if (L.tris >= 0x7FFFFFFFull) return fail(GBR_ERR_INVALID_ARG, "scene %u has too many triangles", i);
        L.bin_base = (uint32_t)bins;
        L.mesh_base = meshes;
        L.tri_base = tris;
        tables[i] = (uint32_t)tri_blocks;
        tables[(n + 1u) + i] = (uint32_t)px_blocks;
        tables[2u * (n + 1u) + i] = (uint32_t)bins;
        bins += (uint64_t)L.nbx * L.nby;
        tris += L.tris;
        meshes += L.num_meshes;
        tri_blocks += ceil_div(L.tris, 256u);
        px_blocks += ceil_div((uint64_t)L.W * L.H, 256u);
    }
    tables[n] = (uint32_t)tri_blocks;
    tables[(n + 1u) + n] = (uint32_t)px_blocks;
    tables[2u * (n + 1u) + n] = (uint32_t)bins;
    if (bins >= 0xFFFFFFFFull || tri_blocks >= 0x7FFFFFFFull || px_blocks >= 0x7FFFFFFFull || tris >= (1ull << 40))
        return fail(GBR_ERR_INVALID_ARG, "batch too large (%llu bins, %llu triangles)", (unsigned long long)bins,
                    (unsigned long long)tris);
    b->total_bins = (uint32_t)bins;
    b->total_tris = tris;
    b->total_meshes = meshes;
    b->tri_blocks = (uint32_t)tri_blocks;
    b->px_blocks = (uint32_t)px_blocks;
    // then each triangle-pass and pixel-pass block's scene
    tables.reserve(tables.size() + tri_blocks + px_blocks + bins);
    for (uint32_t i = 0; i < n; ++i)
        tables.insert(tables.end(), tables[i + 1u] - tables[i], i);
    for (uint32_t i = 0; i < n; ++i)
        tables.insert(tables.end(), tables[(n + 1u) + i + 1u] - tables[(n + 1u) + i], i);
    for (uint32_t i = 0; i < n; ++i)   // and each global bin's scene
        tables.insert(tables.end(), tables[2u * (n + 1u) + i + 1u] - tables[2u * (n + 1u) + i], i);

    GBR_CUDA(cudaMalloc(&b->d_tables, tables.size() * sizeof(uint32_t)));
    GBR_CUDA(cudaMemcpy(b->d_tables, tables.data(), tables.size() * sizeof(uint32_t), cudaMemcpyHostToDevice));
    GBR_CUDA(cudaMalloc(&b->d_counts, kCountSplit * std::max<uint64_t>(bins, 1u) * sizeof(uint32_t)));
    GBR_CUDA(cudaMemset(b->d_counts, 0, kCountSplit * std::max<uint64_t>(bins, 1u) * sizeof(uint32_t)));
    GBR_CUDA(cudaMalloc(&b->d_sub_base, kCountSplit * std::max<uint64_t>(bins, 1u) * sizeof(uint32_t)));
    // one scan over the bins of every scene: scene s's offsets are entries
    // [bin_base[s], bin_base[s+1]] of the batch-wide array
    GBR_CUDA(cudaMalloc(&b->d_offsets, (bins + 1u) * sizeof(uint32_t)));
    GBR_CUDA(cudaMalloc(&b->d_scan, scan_state_bytes((uint32_t)bins)));
    GBR_CUDA(cudaMemset(b->d_scan, 0, scan_state_bytes((uint32_t)bins)));
    GBR_CUDA(cudaMalloc(&b->d_cursors, std::max<uint64_t>(bins, 1u) * sizeof(uint32_t)));
    GBR_CUDA(cudaMalloc(&b->d_setup, std::max<uint64_t>(tris, 1u) * sizeof(TriSetup)));
    GBR_CUDA(cudaMalloc(&b->d_rects, std::max<uint64_t>(tris, 1u) * sizeof(uint2)));
    GBR_CUDA(cudaMalloc(&b->d_walk, std::max<uint64_t>(tri_blocks, 1u) * 8u * sizeof(uint32_t)));
    GBR_CUDA(cudaMalloc(&b->d_keys, std::max<uint64_t>(tris, 1u) * sizeof(uint32_t)));
    gbr_status st = ensure_list(b, std::max<uint64_t>(b->list_cap, 4u * tris), b->items_cap);
    if (st != GBR_OK) return st;

    const size_t table_bytes = (size_t)n * sizeof(FrameDev) + (size_t)meshes * sizeof(MeshDev);
    if (table_bytes > b->table_cap) {
        for (int k = 0; k < 2; ++k)
            if (b->staging_evt[k]) GBR_CUDA(cudaEventSynchronize(b->staging_evt[k]));
        cudaFree(b->d_table);
        cudaFreeHost(b->h_staging[0]);
        cudaFreeHost(b->h_staging[1]);
        b->d_table = nullptr;
        b->h_staging[0] = b->h_staging[1] = nullptr;
        b->table_cap = 0;
        const size_t cap = std::max<size_t>(table_bytes, 4096u);
        GBR_CUDA(cudaMalloc(&b->d_table, cap));
        GBR_CUDA(cudaMallocHost(&b->h_staging[0], cap));
        GBR_CUDA(cudaMallocHost(&b->h_staging[1], cap));
        b->table_cap = cap;
    }
    b->last_table.clear();

    int bps = 0;
    GBR_CUDA(raster_configure_batch(bs, bs, b->cfg.raster_ctas, raster_threads(b->cfg), &bps));
    b->raster_bps = std::max(bps, 1);
    b->layout_valid = true;
    return GBR_OK;
}

// Frame and mesh descriptors of every scene for this frame.
void build_table(gbr_batch* b, std::vector<unsigned char>& out) {
    const uint32_t n = (uint32_t)b->members.size();
    out.assign((size_t)n * sizeof(FrameDev) + (size_t)b->total_meshes * sizeof(MeshDev), 0);
    FrameDev* frames = reinterpret_cast<FrameDev*>(out.data());
    MeshDev* meshes = reinterpret_cast<MeshDev*>(out.data() + (size_t)n * sizeof(FrameDev));
    const MeshDev* d_meshes = reinterpret_cast<const MeshDev*>(b->d_table + (size_t)n * sizeof(FrameDev));
    for (uint32_t i = 0; i < n; ++i) {
        const Member& m = b->members[i];
        const SceneLayout& L = b->layout[i];
        if (L.num_meshes) build_mesh_table(m.r, &m.cam, meshes + L.mesh_base);
        FrameDev F;
        frame_basics(m.r, &m.cam, m.cull, m.sample, m.vis, F);
        F.nbx = L.nbx; F.nby = L.nby; F.bw = b->cfg.bin_size; F.bh = b->cfg.bin_size; F.num_bins = L.nbx * L.nby;
        F.chunk = kBatchChunk;
        F.stage = b->cfg.queue_chunk;
        F.phase = b->cfg.raster_phase;
        F.raster_ctas = b->cfg.raster_ctas;
        F.meshes = d_meshes + L.mesh_base;
        F.setup = b->d_setup + L.tri_base;
        F.rects = b->d_rects + L.tri_base;
        F.keys = b->d_keys + L.tri_base;
        F.counts = b->d_counts + L.bin_base;
        F.sub_base = b->d_sub_base + L.bin_base;
        F.count_stride = b->total_bins;   // sub-counter rows span every scene's bins
        F.count_split = b->count_split;
        F.offsets = b->d_offsets + L.bin_base;
        F.cursors = b->d_cursors + L.bin_base;
        F.list = b->d_list;
        F.list_cap = b->list_cap;
        F.ranks = b->d_list + b->list_cap;
        F.rank_cap = b->list_cap;
        F.walk_base = b->d_walk;          // walks are numbered over the whole batch grid
        F.rank_next = &b->d_ctl->rank_next;
        F.ctl = m.r->d_ctl;
        memcpy(frames + i, &F, sizeof F);
    }
}

BatchDev batch_dev(const gbr_batch* b) {
    const uint32_t n = (uint32_t)b->members.size();
    BatchDev B;
    memset(&B, 0, sizeof B);
    B.scenes = reinterpret_cast<const FrameDev*>(b->d_table);
    B.tri_blocks = b->d_tables;
    B.px_blocks = b->d_tables + (n + 1u);
    B.bin_base = b->d_tables + 2u * (n + 1u);
    B.tri_scene = b->d_tables + 3u * (n + 1u);
    B.px_scene = B.tri_scene + b->tri_blocks;
    B.bin_scene = B.px_scene + b->px_blocks;
    B.items = b->d_items;
    B.ctl = b->d_ctl;
    B.list_cap = b->list_cap;
    B.items_cap = b->items_cap;
    B.num_scenes = n;
    B.phase = b->cfg.raster_phase;
    B.all_flat = b->all_flat;
    B.stage = b->cfg.queue_chunk;
    return B;
}

gbr_status capture_graph(gbr_batch* b) {
    drop_graph(b);
    BatchLaunch L;
    L.tri_blocks = b->tri_blocks;
    L.px_blocks = b->px_blocks;
    L.raster_grid = (uint32_t)(b->num_sms * b->raster_bps);
    L.raster_ctas = b->cfg.raster_ctas;
    L.raster_threads = raster_threads(b->cfg);
    L.bin_w = L.bin_h = b->cfg.bin_size;
    const BatchDev B = batch_dev(b);
    memset(&L.scan, 0, sizeof L.scan);
    L.scan.counts = b->d_counts;
    L.scan.sub_base = b->d_sub_base;
    L.scan.split = b->count_split;
    L.scan.offsets = b->d_offsets;
    L.scan.cursors = b->d_cursors;
    L.scan.items = b->d_items;
    L.scan.state = b->d_scan;
    L.scan.ctl = b->d_ctl;
    L.scan.list_cap = b->list_cap;
    L.scan.items_cap = b->items_cap;
    L.scan.n = b->total_bins;
    L.scan.chunk = kBatchChunk;
    L.scan.mode = kScanExact;
    GBR_CUDA(cudaStreamBeginCapture(b->cap_stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = launch_batch(B, L, b->cap_stream);
    cudaGraph_t g = nullptr;
    cudaError_t e2 = cudaStreamEndCapture(b->cap_stream, &g);
    if (e != cudaSuccess || e2 != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return fail(GBR_ERR_CUDA, "batch graph capture: %s", cudaGetErrorString(e != cudaSuccess ? e : e2));
    }
    e = cudaGraphInstantiate(&b->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        b->graph = nullptr;
        return fail(GBR_ERR_CUDA, "batch graph instantiation: %s", cudaGetErrorString(e));
    }
    ++b->graph_captures;
    return GBR_OK;
}

gbr_status render_batch(gbr_batch* b, cudaStream_t s) {
    if (b->members.empty()) return fail(GBR_ERR_INVALID_ARG, "the batch has no scenes");
    gbr_status st = ensure_layout(b);
    if (st != GBR_OK) return st;
    std::vector<unsigned char> table;
    build_table(b, table);
    // the shade pass's variant lives in the graph: a change is captured anew
    uint32_t all_flat = 1u;
    for (size_t i = 0; i < b->members.size(); ++i)
        all_flat &= reinterpret_cast<const FrameDev*>(table.data())[i].flat_shade;
    if (all_flat != b->all_flat) {
        b->all_flat = all_flat;
        drop_graph(b);
    }
    if (table != b->last_table) {
        const int k = b->staging_next;
        GBR_CUDA(cudaEventSynchronize(b->staging_evt[k]));   // this staging buffer's last copy is done
        memcpy(b->h_staging[k], table.data(), table.size());
        GBR_CUDA(cudaMemcpyAsync(b->d_table, b->h_staging[k], table.size(), cudaMemcpyHostToDevice, s));
        GBR_CUDA(cudaEventRecord(b->staging_evt[k], s));
        b->staging_next = 1 - k;
        b->last_table.swap(table);
    }
    if (!b->graph) {
        st = capture_graph(b);
        if (st != GBR_OK) return st;
    }
    if (b->timing) GBR_CUDA(cudaEventRecord(b->ev[0], s));
    GBR_CUDA(cudaGraphLaunch(b->graph, s));
    if (b->timing) {
        GBR_CUDA(cudaEventRecord(b->ev[1], s));
        b->ev_recorded = true;
    }
    b->have_frame = true;
    b->frame_checked = false;
    for (Member& m : b->members) m.r->dirty_valid = false;   // the batch rewrote their frame buffers
    b->last_stream = s;
    return GBR_OK;
}

// Waits for the stream; re-renders with larger bin storage if the batch
// outgrew it.
gbr_status finish_batch(gbr_batch* b, cudaStream_t s) {
    // the readbacks of a frame's scenes after the first find it complete
    if (b->frame_checked) return GBR_OK;
    GBR_CUDA(cudaMemcpyAsync(b->h_ctl, b->d_ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, s));   // pinned: one wait
    GBR_CUDA(cudaStreamSynchronize(s));
    if (b->h_ctl->error) {   // a bounded wait of the bin scan gave up: restart its state
        GBR_CUDA(cudaMemset(b->d_scan, 0, scan_state_bytes(b->total_bins)));
        return fail(GBR_ERR_TIMEOUT, "bin scan wait timed out; the batch frame is invalid");
    }
    for (int attempt = 0; b->h_ctl->overflow && attempt < 3; ++attempt) {
        gbr_status st = ensure_list(b, b->h_ctl->num_pairs, b->h_ctl->items_alloc);
        if (st != GBR_OK) return st;
        ++b->overflow_reruns;
        st = render_batch(b, s);
        if (st != GBR_OK) return st;
        GBR_CUDA(cudaMemcpyAsync(b->h_ctl, b->d_ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, s));   // pinned: one wait
        GBR_CUDA(cudaStreamSynchronize(s));
    }
    if (b->h_ctl->overflow) return fail(GBR_ERR_OUT_OF_MEMORY, "batch bin storage overflow persists");
    // sub-counters per bin for the next frames, from this frame's density
    // (a change is captured anew: the scan's parameters live in the graph)
    const uint32_t split = count_split_for(b->h_ctl->num_pairs, b->total_bins);
    if (split != b->count_split) {
        b->count_split = split;
        drop_graph(b);
    }
    if (b->h_ctl->error) {   // a bounded wait of the bin scan gave up: restart its state
        GBR_CUDA(cudaMemset(b->d_scan, 0, scan_state_bytes(b->total_bins)));
        return fail(GBR_ERR_TIMEOUT, "bin scan wait timed out; the batch frame is invalid");
    }
    b->frame_checked = true;
    return GBR_OK;
}

gbr_status check_state(uint32_t cull, uint32_t sample, uint32_t vis) {
    if (cull > GBR_CULL_NONE || sample > GBR_SAMPLE_BILINEAR || vis > GBR_VIS_NORMAL)
        return fail(GBR_ERR_INVALID_ARG, "bad cull/sample/vis (%u/%u/%u)", cull, sample, vis);
    return GBR_OK;
}

gbr_status check_config(const gbr_batch_config& c) {
    if (c.bin_size == 0 || c.bin_size > (uint32_t)kMaxBinDim || c.queue_chunk == 0 || c.raster_phase > kMaxPhase ||
        (c.raster_ctas != 0 && (c.raster_ctas < 2 || c.raster_ctas > 6)) ||
        (c.raster_threads != 0 && c.raster_threads != 128 && c.raster_threads != 256))
        return fail(GBR_ERR_INVALID_ARG,
                    "batch config: bin %u (1..%d), chunk %u (>= 1), ctas %u (0, 2..6), phase %u, threads %u (0, 128, 256)",
                    c.bin_size, kMaxBinDim, c.queue_chunk, c.raster_ctas, c.raster_phase, c.raster_threads);
    return GBR_OK;
}

}  // namespace

extern "C" {

gbr_status gbr_batch_create(gbr_batch** out) {
    if (!out) return fail(GBR_ERR_INVALID_ARG, "out is null");
    *out = nullptr;
    gbr_batch* b = new (std::nothrow) gbr_batch();
    if (!b) return fail(GBR_ERR_OUT_OF_MEMORY, "host allocation failed");
    cudaError_t e = cudaGetDevice(&b->device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&b->num_sms, cudaDevAttrMultiProcessorCount, b->device);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_ctl, sizeof(Ctl));
    if (e == cudaSuccess) e = cudaMemset(b->d_ctl, 0, sizeof(Ctl));
    if (e == cudaSuccess) e = cudaMallocHost(&b->h_ctl, sizeof(Ctl));
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->cap_stream, cudaStreamNonBlocking);
    for (int k = 0; k < 2 && e == cudaSuccess; ++k) e = cudaEventCreateWithFlags(&b->staging_evt[k], cudaEventDisableTiming);
    for (int k = 0; k < 2 && e == cudaSuccess; ++k) e = cudaEventCreate(&b->ev[k]);
    if (e != cudaSuccess) {
        gbr_batch_destroy(b);
        return fail(GBR_ERR_CUDA, "gbr_batch_create: %s", cudaGetErrorString(e));
    }
    *out = b;
    return GBR_OK;
}

gbr_status gbr_batch_destroy(gbr_batch* b) {
    if (!b) return GBR_OK;
    cudaDeviceSynchronize();
    drop_graph(b);
    free_layout_storage(b);
    cudaFree(b->d_list); cudaFree(b->d_items); cudaFree(b->d_ctl); cudaFree(b->d_table);
    cudaFreeHost(b->h_ctl); cudaFreeHost(b->h_staging[0]); cudaFreeHost(b->h_staging[1]);
    for (int k = 0; k < 2; ++k) {
        if (b->staging_evt[k]) cudaEventDestroy(b->staging_evt[k]);
        if (b->ev[k]) cudaEventDestroy(b->ev[k]);
    }
    if (b->cap_stream) cudaStreamDestroy(b->cap_stream);
    for (Member& m : b->members) --m.r->in_batches;
    delete b;
    return GBR_OK;
}

gbr_status gbr_batch_add(gbr_batch* b, gbr_renderer* r, const gbr_camera* cam, uint32_t cull, uint32_t sample,
                         uint32_t vis, uint32_t* index) {
    if (!b || !r || !cam) return fail(GBR_ERR_INVALID_ARG, "null batch, renderer or camera");
    gbr_status st = check_state(cull, sample, vis);
    if (st != GBR_OK) return st;
    for (const Member& m : b->members)
        if (m.r == r) return fail(GBR_ERR_INVALID_ARG, "the renderer is already in the batch");
    Member m;
    m.r = r;
    m.cam = *cam;
    m.cull = cull; m.sample = sample; m.vis = vis;
    b->members.push_back(m);
    ++r->in_batches;
    b->layout_valid = false;
    if (index) *index = (uint32_t)b->members.size() - 1u;
    return GBR_OK;
}

gbr_status gbr_batch_set_view(gbr_batch* b, uint32_t index, const gbr_camera* cam, uint32_t cull, uint32_t sample,
                              uint32_t vis) {
    if (!b || !cam || index >= b->members.size()) return fail(GBR_ERR_INVALID_ARG, "bad batch, index or camera");
    gbr_status st = check_state(cull, sample, vis);
    if (st != GBR_OK) return st;
    Member& m = b->members[index];
    m.cam = *cam;
    m.cull = cull; m.sample = sample; m.vis = vis;
    return GBR_OK;
}

gbr_status gbr_batch_set_config(gbr_batch* b, const gbr_batch_config* cfg) {
    if (!b || !cfg) return fail(GBR_ERR_INVALID_ARG, "null argument");
    gbr_status st = check_config(*cfg);
    if (st != GBR_OK) return st;
    if (memcmp(cfg, &b->cfg, sizeof *cfg) != 0) {
        b->cfg = *cfg;
        b->layout_valid = false;
    }
    return GBR_OK;
}

gbr_status gbr_batch_get_config(const gbr_batch* b, gbr_batch_config* cfg) {
    if (!b || !cfg) return fail(GBR_ERR_INVALID_ARG, "null argument");
    *cfg = b->cfg;
    return GBR_OK;
}

gbr_status gbr_batch_set_timing(gbr_batch* b, int enabled) {
    if (!b) return fail(GBR_ERR_INVALID_ARG, "batch is null");
    b->timing = enabled != 0;
    return GBR_OK;
}

gbr_status gbr_batch_render(gbr_batch* b, void* stream) {
    if (!b) return fail(GBR_ERR_INVALID_ARG, "batch is null");
    return render_batch(b, (cudaStream_t)stream);
}

gbr_status gbr_batch_autotune(gbr_batch* b, const uint32_t* bin_sizes, uint32_t num_bin_sizes, const uint32_t* chunks,
                              uint32_t num_chunks, const uint32_t* raster_ctas, uint32_t num_raster_ctas,
                              const uint32_t* raster_threads, uint32_t num_raster_threads, uint32_t frames, void* stream,
                              gbr_batch_config* best) {
    if (!b) return fail(GBR_ERR_INVALID_ARG, "batch is null");
    if (b->members.empty()) return fail(GBR_ERR_INVALID_ARG, "the batch has no scenes");
    cudaStream_t s = (cudaStream_t)stream;
    const gbr_batch_config base = b->cfg;
    std::vector<uint32_t> bl = bin_sizes && num_bin_sizes ? std::vector<uint32_t>(bin_sizes, bin_sizes + num_bin_sizes)
                                                          : std::vector<uint32_t>{base.bin_size};
    std::vector<uint32_t> cl = chunks && num_chunks ? std::vector<uint32_t>(chunks, chunks + num_chunks)
                                                    : std::vector<uint32_t>{base.queue_chunk};
    std::vector<uint32_t> rl = raster_ctas && num_raster_ctas
                                   ? std::vector<uint32_t>(raster_ctas, raster_ctas + num_raster_ctas)
                                   : std::vector<uint32_t>{base.raster_ctas};
    std::vector<uint32_t> tl = raster_threads && num_raster_threads
                                   ? std::vector<uint32_t>(raster_threads, raster_threads + num_raster_threads)
                                   : std::vector<uint32_t>{base.raster_threads};
    if (frames == 0) frames = 1;
    const bool timing = b->timing;
    b->timing = true;
    gbr_batch_config winner = base;
    float best_ms = -1.f;
    gbr_status st = GBR_OK;
    for (uint32_t bs : bl)
        for (uint32_t ch : cl)
            for (uint32_t rc : rl)
            for (uint32_t rt : tl) {
                gbr_batch_config c = base;
                c.bin_size = bs;
                c.queue_chunk = ch;
                c.raster_ctas = rc;
                c.raster_threads = rt;
                st = gbr_batch_set_config(b, &c);
                if (st != GBR_OK) goto done;
                // warm-up frame: sizes the storage (overflow re-render) and captures the graph
                st = render_batch(b, s);
                if (st == GBR_OK) st = finish_batch(b, s);
                if (st != GBR_OK) goto done;
                float total = 0.f;
                for (uint32_t f = 0; f < frames; ++f) {
                    st = render_batch(b, s);
                    if (st == GBR_OK) st = finish_batch(b, s);
                    if (st != GBR_OK) goto done;
                    float ms = 0.f;
                    cudaEventElapsedTime(&ms, b->ev[0], b->ev[1]);
                    total += ms;
                }
                const float ms = total / (float)frames;
                if (best_ms < 0.f || ms < best_ms) {
                    best_ms = ms;
                    winner = c;
                }
            }
done:
    b->timing = timing;
    if (st != GBR_OK) {
        gbr_batch_set_config(b, &base);
        return st;
    }
    st = gbr_batch_set_config(b, &winner);
    if (st != GBR_OK) return st;
    if (best) *best = winner;
    return GBR_OK;
}

gbr_status gbr_batch_get_stats(gbr_batch* b, gbr_batch_stats* out, void* stream) {
    if (!b || !out) return fail(GBR_ERR_INVALID_ARG, "null argument");
    memset(out, 0, sizeof *out);
    out->num_scenes = (uint32_t)b->members.size();
    out->graph_captures = b->graph_captures;
    for (const Member& m : b->members) out->num_triangles += scene_triangles(m.r);
    if (!b->have_frame) return GBR_OK;
    gbr_status st = finish_batch(b, (cudaStream_t)stream);
    if (st != GBR_OK) return st;
    out->overflow_reruns = b->overflow_reruns;
    out->graph_captures = b->graph_captures;
    out->num_pairs = b->h_ctl->num_pairs;
    out->num_work_items = b->h_ctl->items_alloc;
    Ctl c;
    for (const Member& m : b->members) {
        GBR_CUDA(cudaMemcpy(&c, m.r->d_ctl, sizeof c, cudaMemcpyDeviceToHost));
        out->num_visible += c.num_visible;
    }
    if (b->timing && b->ev_recorded) cudaEventElapsedTime(&out->ms_frame, b->ev[0], b->ev[1]);
    return GBR_OK;
}

gbr_status gbr_batch_scene_bins(const gbr_batch* b, uint32_t index, uint32_t* num_bins_x, uint32_t* num_bins_y) {
    if (!b || index >= b->members.size()) return fail(GBR_ERR_INVALID_ARG, "bad batch or index");
    const gbr_renderer* r = b->members[index].r;
    if (num_bins_x) *num_bins_x = ceil_div(r->W, b->cfg.bin_size);
    if (num_bins_y) *num_bins_y = ceil_div(r->H, b->cfg.bin_size);
    return GBR_OK;
}

gbr_status gbr_batch_readback(gbr_batch* b, uint32_t index, uint32_t* colour, float* depth, uint32_t* ids,
                              void* stream) {
    if (!b || index >= b->members.size()) return fail(GBR_ERR_INVALID_ARG, "bad batch or index");
    if (!b->have_frame) return fail(GBR_ERR_INVALID_ARG, "no batch frame rendered");
    cudaStream_t s = (cudaStream_t)stream;
    gbr_status st = finish_batch(b, s);
    if (st != GBR_OK) return st;
    const gbr_renderer* r = b->members[index].r;
    const size_t npx = (size_t)r->W * r->H;
    if (colour) GBR_CUDA(cudaMemcpyAsync(colour, r->d_colour, npx * 4u, cudaMemcpyDeviceToHost, s));
    if (depth) GBR_CUDA(cudaMemcpyAsync(depth, r->d_depth, npx * 4u, cudaMemcpyDeviceToHost, s));
    if (ids) GBR_CUDA(cudaMemcpyAsync(ids, r->d_ids, npx * 4u, cudaMemcpyDeviceToHost, s));
    GBR_CUDA(cudaStreamSynchronize(s));
    return GBR_OK;
}

gbr_status gbr_batch_readback_all(gbr_batch* b, uint32_t* const* colours, void* stream) {
    if (!b || !colours) return fail(GBR_ERR_INVALID_ARG, "null argument");
    if (!b->have_frame) return fail(GBR_ERR_INVALID_ARG, "no batch frame rendered");
    cudaStream_t s = (cudaStream_t)stream;
    gbr_status st = finish_batch(b, s);
    if (st != GBR_OK) return st;
    for (size_t i = 0; i < b->members.size(); ++i) {
        if (!colours[i]) continue;
        const gbr_renderer* r = b->members[i].r;
        GBR_CUDA(cudaMemcpyAsync(colours[i], r->d_colour, (size_t)r->W * r->H * 4u, cudaMemcpyDeviceToHost, s));
    }
    GBR_CUDA(cudaStreamSynchronize(s));
    return GBR_OK;
}

gbr_status gbr_batch_get_bins(gbr_batch* b, uint32_t index, uint32_t* offsets, uint32_t* ids, uint64_t capacity,
                              uint64_t* num_pairs, void* stream) {
    if (!b || index >= b->members.size()) return fail(GBR_ERR_INVALID_ARG, "bad batch or index");
    if (!b->have_frame) return fail(GBR_ERR_INVALID_ARG, "no batch frame rendered");
    gbr_status st = finish_batch(b, (cudaStream_t)stream);
    if (st != GBR_OK) return st;
    const SceneLayout& L = b->layout[index];
    const uint32_t nb = L.nbx * L.nby;
    std::vector<uint32_t> off(nb + 1u);
    GBR_CUDA(cudaMemcpy(off.data(), b->d_offsets + L.bin_base, (nb + 1u) * sizeof(uint32_t), cudaMemcpyDeviceToHost));
    const uint64_t total = (uint64_t)off[nb] - off[0];
    if (num_pairs) *num_pairs = total;
    if (offsets)
        for (uint32_t k = 0; k <= nb; ++k) offsets[k] = off[k] - off[0];
    if (ids) {
        if (capacity < total) return fail(GBR_ERR_INVALID_ARG, "ids capacity %llu < %llu pairs",
                                          (unsigned long long)capacity, (unsigned long long)total);
        if (total) GBR_CUDA(cudaMemcpy(ids, b->d_list + off[0], total * sizeof(uint32_t), cudaMemcpyDeviceToHost));
        for (uint64_t i = 0; i < total; ++i) ids[i] &= ~kNoRasterBit;
    }
    return GBR_OK;
}

}  // extern "C"
