// gbr_api.cu -- C ABI (include/gbr.h) over the frame kernels.
//
// Host orchestration of one frame, replacing CUDARenderer::Render's
// per-mesh loop, its per-256-triangle chunk loop and the device-wide
// synchronisation after every stage (CustomCUDARasterizer/CUDARenderer.cu:
// 206-354): a frame is four kernel launches on the caller's stream with no
// host synchronisation, whatever the number of meshes or triangles.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/gbr.h"
#include "gbr_internal.h"
#include "gbr_kernels.h"
#include "gbr_predict.h"

using namespace gbr;

namespace {
thread_local std::string g_last_error;
}  // namespace

gbr_status gbr::fail(gbr_status st, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return st;
}

// Lets other translation units of the library report through
// gbr_last_error_string().
void gbr::set_last_error(const char* msg) { g_last_error = msg; }

void gbr::mat4_mul(const float* lm, const float* rm, float* out) {
    float t[16];
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) {
            float s = lm[0 * 4 + r] * rm[c * 4 + 0];
            s = s + lm[1 * 4 + r] * rm[c * 4 + 1];
            s = s + lm[2 * 4 + r] * rm[c * 4 + 2];
            s = s + lm[3 * 4 + r] * rm[c * 4 + 3];
            t[c * 4 + r] = s;
        }
    memcpy(out, t, sizeof t);
}

namespace {

TexDev tex_dev(const gbr_renderer* r, int32_t id) {
    TexDev t{nullptr, 0u, 0u};
    if (id >= 0 && (size_t)id < r->textures.size() && r->textures[id].d_px) {
        t.px = r->textures[id].d_px;
        t.w = r->textures[id].w;
        t.h = r->textures[id].h;
    }
    return t;
}

}  // namespace

uint64_t gbr::scene_triangles(const gbr_renderer* r) {
    uint64_t n = 0;
    for (const MeshHost& m : r->meshes) n += m.num_tris;
    return n;
}

void gbr::build_mesh_table(const gbr_renderer* r, const gbr_camera* cam, MeshDev* out) {
    float vp[16];
    mat4_mul(cam->proj, cam->view, vp);
    uint32_t base = 0;
    for (size_t i = 0; i < r->meshes.size(); ++i) {
        const MeshHost& m = r->meshes[i];
        MeshDev& d = out[i];
        memset(&d, 0, sizeof d);
        d.vertices = m.d_vertices;
        d.indices = m.d_indices;
        d.vertex_format = m.vertex_format;
        d.topology = m.topology;
        d.num_vertices = m.num_vertices;
        d.num_tris = (uint32_t)m.num_tris;
        d.prim_base = base;
        base += (uint32_t)m.num_tris;
        mat4_mul(vp, m.world, d.wvp);
        memcpy(d.world, m.world, sizeof d.world);
        // UpdateCUDAMeshTextures (CUDARenderer.cu:549-573): normal needs
        // diffuse; specular and gloss need normal
        const TexDev diff = tex_dev(r, m.tex_ids[0]);
        if (diff.px) {
            d.tex[0] = diff;
            const TexDev norm = tex_dev(r, m.tex_ids[1]);
            if (norm.px) {
                d.tex[1] = norm;
                d.tex[2] = tex_dev(r, m.tex_ids[2]);
                d.tex[3] = tex_dev(r, m.tex_ids[3]);
            }
        }
    }
}

void gbr::frame_basics(const gbr_renderer* r, const gbr_camera* cam, uint32_t cull, uint32_t sample, uint32_t vis,
                       FrameDev& F) {
    memset(&F, 0, sizeof F);
    F.width = r->W; F.height = r->H;
    F.cull = cull; F.sample = sample; F.vis = vis; F.clear_colour32 = 0x003F3F3Fu;
    F.num_meshes = (uint32_t)r->meshes.size();
    F.num_tris = (uint32_t)scene_triangles(r);
    for (int k = 0; k < 3; ++k) { F.cam_pos[k] = cam->pos[k]; F.cam_fwd[k] = cam->fwd[k]; }
    F.colour = r->d_colour; F.depth = r->d_depth; F.ids = r->d_ids; F.gvis = r->d_gvis;
    F.lights = r->d_lights;
    F.num_lights = r->num_lights;
    bool textured = false;
    for (const MeshHost& m : r->meshes) textured |= m.tex_ids[0] >= 0 && (size_t)m.tex_ids[0] < r->textures.size() &&
                                                   r->textures[m.tex_ids[0]].d_px;
    F.flat_shade = vis == GBR_VIS_PBR && !textured ? 1u : 0u;
}

namespace {

uint64_t tri_count(uint32_t num_vertices, const uint32_t* indices, uint32_t num_indices, uint32_t topology) {
    if (!indices) return num_vertices / 3u;
    if (topology == GBR_TOPOLOGY_TRIANGLE_LIST) return num_indices / 3u;
    return num_indices >= 2u ? num_indices - 2u : 0u;
}

void free_bins(gbr_renderer* r) {
    cudaFree(r->d_counts); cudaFree(r->d_sub_base); cudaFree(r->d_offsets); cudaFree(r->d_cursors); cudaFree(r->d_capacity);
    cudaFree(r->d_row_base);
    r->d_row_base = nullptr;
    cudaFree(r->d_bin_end); cudaFree(r->d_items); cudaFree(r->d_list); cudaFree(r->d_scan);
    r->d_scan = nullptr;
    cudaFree(r->d_feat); cudaFree(r->d_features_out);
    r->d_feat = nullptr;
    r->d_features_out = nullptr;
    r->d_sub_base = nullptr;
    r->d_counts = r->d_offsets = r->d_cursors = r->d_capacity = r->d_bin_end = r->d_list = nullptr;
    r->d_items = nullptr;
    r->items_cap = 0;
    r->list_cap = 0;
    r->seen_pairs = r->seen_visible = 0;
    cudaFree(r->d_dirty);
    r->d_dirty = nullptr;
    r->dirty_valid = false;
}

gbr_status ensure_list(gbr_renderer* r, uint64_t pairs) {
    const uint32_t nb = r->nbx * r->nby;
    if (pairs <= r->list_cap && r->d_list) return GBR_OK;
    uint64_t cap = std::max<uint64_t>(pairs + pairs / 4u, 1u << 20);
    if (cap > 0x7FFFFFFFull) cap = 0x7FFFFFFFull;
    if (pairs > cap) return fail(GBR_ERR_OUT_OF_MEMORY, "frame needs %llu bin entries (max 2^31-1)", (unsigned long long)pairs);
    cudaFree(r->d_list);
    cudaFree(r->d_items);
    r->d_list = nullptr;
    r->d_items = nullptr;
    // work items of kMinChunk..kMaxChunk entries
    const uint64_t items = (uint64_t)nb + cap / kMinChunk + 1u;
    // the bin list, then as many rank slots (exact binning's count pass)
    if (cudaMalloc(&r->d_list, 2u * cap * sizeof(uint32_t)) != cudaSuccess ||
        cudaMalloc(&r->d_items, items * sizeof(uint4)) != cudaSuccess) {
        cudaGetLastError();
        r->list_cap = 0;
        r->items_cap = 0;
        return fail(GBR_ERR_OUT_OF_MEMORY, "cannot allocate %llu bin entries", (unsigned long long)cap);
    }
    r->list_cap = cap;
    r->items_cap = (uint32_t)std::min<uint64_t>(items, 0xFFFFFFFFull);
    return GBR_OK;
}

gbr_status ensure_tris(gbr_renderer* r, uint64_t tris) {
    if (tris <= r->tri_cap && r->d_setup) return GBR_OK;
    cudaFree(r->d_setup);
    cudaFree(r->d_rects);
    cudaFree(r->d_walk);
    cudaFree(r->d_keys);
    r->d_setup = nullptr;
    r->d_rects = nullptr;
    r->d_walk = nullptr;
    r->d_keys = nullptr;
    const uint64_t cap = std::max<uint64_t>(tris, 1024u);
    if (cudaMalloc(&r->d_setup, cap * sizeof(TriSetup)) != cudaSuccess ||
        cudaMalloc(&r->d_rects, cap * sizeof(uint2)) != cudaSuccess ||
        cudaMalloc(&r->d_walk, (cap / 32u + 8u) * sizeof(uint32_t)) != cudaSuccess ||
        cudaMalloc(&r->d_keys, cap * sizeof(uint32_t)) != cudaSuccess) {
        cudaGetLastError();
        r->tri_cap = 0;
        return fail(GBR_ERR_OUT_OF_MEMORY, "cannot allocate setup records for %llu triangles", (unsigned long long)tris);
    }
    r->tri_cap = cap;
    return GBR_OK;
}

gbr_status ensure_meshes(gbr_renderer* r, uint32_t n) {
    if (n <= r->meshes_cap && r->d_meshes) return GBR_OK;
    if (r->meshes_evt) cudaEventSynchronize(r->meshes_evt);
    cudaFree(r->d_meshes);
    cudaFreeHost(r->h_meshes);
    r->d_meshes = nullptr;
    r->h_meshes = nullptr;
    const uint32_t cap = std::max<uint32_t>(n, 16u);
    GBR_CUDA(cudaMalloc(&r->d_meshes, cap * sizeof(MeshDev)));
    GBR_CUDA(cudaMallocHost(&r->h_meshes, cap * sizeof(MeshDev)));
    r->meshes_cap = cap;
    r->last_uploaded.clear();
    return GBR_OK;
}

gbr_status validate_mesh_args(const void* vertices, uint32_t num_vertices, uint32_t vertex_format,
                              const uint32_t* indices, uint32_t num_indices, uint32_t topology, const float* world) {
    if (!vertices && num_vertices) return fail(GBR_ERR_INVALID_ARG, "vertices is null");
    if (vertex_format > GBR_VERTEX_POS3_RGBA8) return fail(GBR_ERR_INVALID_ARG, "unknown vertex format %u", vertex_format);
    if (topology > GBR_TOPOLOGY_TRIANGLE_STRIP) return fail(GBR_ERR_INVALID_ARG, "unknown topology %u", topology);
    if (!indices && topology != GBR_TOPOLOGY_TRIANGLE_LIST)
        return fail(GBR_ERR_INVALID_ARG, "a triangle strip needs an index buffer");
    if (!world) return fail(GBR_ERR_INVALID_ARG, "world matrix is null");
    (void)num_indices;
    return GBR_OK;
}

// Renders one frame on `s` (no host synchronisation).
gbr_status render_frame(gbr_renderer* r, const gbr_camera* cam, uint32_t cull, uint32_t sample, uint32_t vis,
                        cudaStream_t s) {
    const uint32_t nb = r->nbx * r->nby;
    uint64_t ntris = 0;
    for (const MeshHost& m : r->meshes) ntris += m.num_tris;
    if (ntris >= 0x7FFFFFFFull) return fail(GBR_ERR_INVALID_ARG, "too many triangles (%llu)", (unsigned long long)ntris);
    gbr_status st = ensure_tris(r, ntris);
    if (st != GBR_OK) return st;
    st = ensure_list(r, std::max<uint64_t>(r->list_cap, 8u * ntris));
    if (st != GBR_OK) return st;
    st = ensure_meshes(r, (uint32_t)r->meshes.size());
    if (st != GBR_OK) return st;

    // per-mesh descriptors with the matrices of this frame
    std::vector<MeshDev> md(r->meshes.size());
    if (!md.empty()) build_mesh_table(r, cam, md.data());
    const bool same = md.size() == r->last_uploaded.size() &&
                      (md.empty() || memcmp(md.data(), r->last_uploaded.data(), md.size() * sizeof(MeshDev)) == 0);
    if (!same && !md.empty()) {
        GBR_CUDA(cudaEventSynchronize(r->meshes_evt));  // previous copy out of the staging buffer is done
        memcpy(r->h_meshes, md.data(), md.size() * sizeof(MeshDev));
        GBR_CUDA(cudaMemcpyAsync(r->d_meshes, r->h_meshes, md.size() * sizeof(MeshDev), cudaMemcpyHostToDevice, s));
        GBR_CUDA(cudaEventRecord(r->meshes_evt, s));
        r->last_uploaded = md;
    }

    FrameDev F;
    frame_basics(r, cam, cull, sample, vis, F);
    F.nbx = r->nbx; F.nby = r->nby; F.bw = r->bw; F.bh = r->bh; F.num_bins = nb;
    // raster work: once a frame has been seen, items hold about half of a
    // raster CTA's share of the pairs (so a few crowded bins do not
    // serialise the frame), within [kMinChunk, kMaxChunk]; queue_chunk is
    // the pass size (entries depth-sorted and rasterised at a time); with the
    // library's phase, triangles spanning under 4 bins on average (little
    // overdraw per bin) refresh the tile's depth bound every kSparsePhase
    // triangles rather than every kPhase (every kMaxPhase with the
    // small-triangle variant, below)
    F.chunk = kMaxChunk;
    F.stage = r->chunk;   // queue_chunk: entries per raster pass
    F.phase = r->raster_phase;
    if (r->seen_pairs) {
        const uint64_t grid = (uint64_t)r->num_sms * (uint64_t)std::max(r->raster_blocks_per_sm, 1);
        const uint64_t share = r->seen_pairs / (2u * grid);
        F.chunk = (uint32_t)std::max<uint64_t>(std::min<uint64_t>(share, kMaxChunk), kMinChunk);
        if (F.phase == 0u) F.phase = r->seen_pairs < 4u * r->seen_visible ? kSparsePhase : kPhase;
        // small triangles: about (pairs per visible triangle - 1) x the bin
        // side of width + height each; with the library's phase the
        // small-triangle variant runs phases of the whole record ring, so
        // that every warp of the CTA takes a share of each phase
        if (F.phase >= kLanePhase && r->seen_visible) {
            const double extent = ((double)r->seen_pairs / (double)r->seen_visible - 1.0) * 0.5 * (r->bw + r->bh);
            F.raster_lanes = extent < kLaneExtentPx ? 1u : 0u;
            if (F.raster_lanes && r->raster_phase == 0u) F.phase = kMaxPhase;
        }
    }
    F.raster_ctas = r->raster_ctas;
    F.meshes = r->d_meshes;
    F.setup = r->d_setup; F.rects = r->d_rects; F.keys = r->d_keys;
    F.counts = r->d_counts; F.sub_base = r->d_sub_base; F.count_stride = nb; F.offsets = r->d_offsets;
    F.cursors = r->d_cursors; F.capacity = r->d_capacity;
    F.count_split = count_split_for(r->seen_pairs, nb);   // 1 until a frame has been seen
    F.bin_end = r->d_bin_end;
    F.items = r->d_items; F.items_cap = r->items_cap;
    F.list = r->d_list; F.list_cap = r->list_cap;
    F.ranks = r->d_list + r->list_cap; F.rank_cap = r->list_cap;
    F.walk_base = r->d_walk; F.rank_next = &r->d_ctl->rank_next;
    F.ctl = r->d_ctl;
    F.scan_state = r->d_scan;
    F.rec_tma = r->rec_tma;
    F.scan_spin_limit = r->scan_spin_limit;
    if (r->row1) {   // this renderer's share of a frame split by bin rows
        F.row0 = r->row0;
        F.row1 = std::min(r->row1, r->nby);
        F.px_begin = (F.row0 * r->bh * r->W) & ~3u;   // a multiple of 4: the quad-wide shade pass
        F.px_end = std::min(F.row1 * r->bh, r->H) * r->W;
    }
    F.scan_silent_tile1 = r->scan_silent_tile1;
    const bool predicted = r->binning == GBR_BINNING_PREDICTED && r->predictor_ready && !r->collect;
    F.feat = r->d_feat;
    F.mlp_w = r->sampled_rule ? nullptr : r->d_mlp_w;   // null: capacities from the sampled counts alone
    F.features_out = r->collect ? r->d_features_out : nullptr;
    F.cap_alpha = r->cap_alpha; F.cap_beta = r->cap_beta; F.cap_gamma = r->cap_gamma;
    F.sample_stride = kSampleStride;
    F.exact_guard = predicted ? 1u : 0u;
    // exact binning of a dense frame: block-private counter rows
    const uint32_t rows = std::min<uint32_t>((F.num_tris + kRowThreads - 1u) / kRowThreads, (uint32_t)r->num_sms);
    if (!predicted && r->d_row_base && use_count_rows(r->seen_pairs, nb, rows)) {
        F.row_base = r->d_row_base;
        F.row_blocks = rows;
        F.count_split = 1u;
    }
    r->last_row_blocks = F.row_blocks;
    r->last_raster_lanes = F.raster_lanes;
    // frames shaded through the full vertex stage shade their covered
    // pixels in a second, densely packed pass
    if (!F.flat_shade && vis != GBR_VIS_DEPTH) {
        if (!r->d_shade_list) GBR_CUDA(cudaMalloc(&r->d_shade_list, (size_t)r->W * r->H * sizeof(uint32_t)));
        F.shade_list = r->d_shade_list;
        // the light pass leaves bins that stay clean untouched
        if (r->d_dirty) {
            uint8_t* rd = r->d_dirty + (size_t)r->dirty_parity * nb;
            uint8_t* wr = r->d_dirty + (size_t)(r->dirty_parity ^ 1u) * nb;
            if (!r->dirty_valid || r->dirty_vis != vis) GBR_CUDA(cudaMemsetAsync(rd, 1, nb, s));
            F.dirty_rd = rd;
            F.dirty_wr = wr;
            r->dirty_parity ^= 1u;
            r->dirty_valid = true;
            r->dirty_vis = vis;
        }
    } else {
        r->dirty_valid = false;   // one-pass shading writes every pixel
    }

    const bool stages = r->timing == GBR_TIMING_STAGES;
    const bool touch = r->seen_pairs >= kListTouchMinPairs;
    if (touch && F.row_blocks)   // the block-row count pass zeroes the last frame's entries (and 1/16 more)
        F.touch_words = (uint32_t)((std::min<uint64_t>(r->list_cap, r->seen_pairs + r->seen_pairs / 16u) + 3u) / 4u);
    if (r->timing) GBR_CUDA(cudaEventRecord(r->ev[0], s));
    GBR_CUDA(cudaMemsetAsync(r->d_ctl, 0, sizeof(Ctl), s));
    if (predicted) {
        // coarse pre-pass -> capacities -> one fused setup + fill pass; the
        // exact kernels behind it only run if a bin overflowed.  The fused
        // pass counts in block-private rows where the bins fit shared memory
        // (its own descriptor: the guarded exact kernels behind it keep
        // global counters).  The list is not zeroed ahead of it: the pass's
        // own setup writes evict a zeroed region from L2 before its fill
        // (measured: 10 us of zeroing, no gain in the fill)
        FrameDev P = F;
        P.touch_words = 0u;
        if (nb <= kMaxRowBins && rows > 0u) P.row_blocks = rows;
        GBR_CUDA(launch_prepass(F, s));
        GBR_CUDA(launch_capacity(F, true, s));
        GBR_CUDA(launch_scan(scan_of(F, kScanCapacity), s));
        GBR_CUDA(launch_setup(P, true, s));
        if (stages) GBR_CUDA(cudaEventRecord(r->ev[1], s));
        GBR_CUDA(launch_scan(scan_of(F, kScanPredictedItems), s));
        GBR_CUDA(launch_setup(F, false, s));
        GBR_CUDA(launch_scan(scan_of(F, kScanExactAfterPredicted), s));
        GBR_CUDA(launch_fill(F, s));
    } else {
        if (r->collect) {
            GBR_CUDA(launch_prepass(F, s));
            GBR_CUDA(launch_capacity(F, false, s));
            GBR_CUDA(launch_feat_reset(F, s));
        }
        GBR_CUDA(launch_setup(F, false, s));
        if (stages) GBR_CUDA(cudaEventRecord(r->ev[1], s));
        GBR_CUDA(launch_scan(scan_of(F, kScanExact), s));
        if (touch && !F.row_blocks) GBR_CUDA(launch_list_touch(F, s));
        GBR_CUDA(launch_fill(F, s));
    }
    r->last_predicted = predicted;
    if (stages) GBR_CUDA(cudaEventRecord(r->ev[2], s));
    GBR_CUDA(launch_raster(F, (uint32_t)(r->num_sms * r->raster_blocks_per_sm), s));
    if (stages) GBR_CUDA(cudaEventRecord(r->ev[4], s));
    GBR_CUDA(launch_shade(F, s));
    if (r->timing) {
        GBR_CUDA(cudaEventRecord(r->ev[3], s));
        r->ev_recorded = true;
    }
    r->have_frame = true;
    r->last_cam = *cam;
    r->last_cull = cull; r->last_sample = sample; r->last_vis = vis;
    return GBR_OK;
}

// A bounded wait of the bin scan gave up: the frame's kernels after the scan
// returned without touching the frame buffers.  The scan state restarts
// from zero.
gbr_status scan_timed_out(gbr_renderer* r) {
    GBR_CUDA(cudaMemset(r->d_scan, 0, scan_state_bytes(r->nbx * r->nby)));
    return fail(GBR_ERR_TIMEOUT, "bin scan wait timed out; the frame is invalid");
}

// Waits for the stream; re-renders with larger bin storage if the frame
// overflowed it.
gbr_status finish_frame(gbr_renderer* r, cudaStream_t s) {
    GBR_CUDA(cudaMemcpyAsync(r->h_ctl, r->d_ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, s));   // pinned: one wait
    GBR_CUDA(cudaStreamSynchronize(s));
    // a bounded wait that gave up flags the frame before any storage check
    // (its overflow flag only stopped the kernels after the scan)
    if (r->h_ctl->error) return scan_timed_out(r);
    for (int attempt = 0; r->h_ctl->overflow && attempt < 3; ++attempt) {
        const uint64_t need = r->h_ctl->num_pairs;
        gbr_status st = ensure_list(r, need);
        if (st != GBR_OK) return st;
        ++r->overflow_reruns;
        st = render_frame(r, &r->last_cam, r->last_cull, r->last_sample, r->last_vis, s);
        if (st != GBR_OK) return st;
        GBR_CUDA(cudaMemcpyAsync(r->h_ctl, r->d_ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, s));   // pinned: one wait
        GBR_CUDA(cudaStreamSynchronize(s));
        if (r->h_ctl->error) return scan_timed_out(r);
    }
    if (r->h_ctl->overflow) return fail(GBR_ERR_OUT_OF_MEMORY, "bin storage overflow persists");
    r->seen_pairs = r->h_ctl->num_pairs;
    r->seen_visible = r->h_ctl->num_visible;
    // predicted capacities that did not fit the list: grow it for the next
    // frames, within reason (the frame itself was re-binned exactly)
    const uint64_t want = r->h_ctl->pred_capacity;
    if (r->last_predicted && want > r->list_cap && want <= 0x7FFFFFFFull &&
        want <= 16u * r->h_ctl->num_pairs + (1u << 22)) {
        if (ensure_list(r, want) != GBR_OK) ensure_list(r, r->h_ctl->num_pairs);
    }
    return GBR_OK;
}

}  // namespace

extern "C" {

const char* gbr_last_error_string(void) { return g_last_error.c_str(); }

uint32_t gbr_version(void) { return 0x000100u; }

gbr_status gbr_create(uint32_t width, uint32_t height, gbr_renderer** out) {
    if (!out) return fail(GBR_ERR_INVALID_ARG, "out is null");
    *out = nullptr;
    if (width == 0 || height == 0 || width > 8192u || height > 8192u)
        return fail(GBR_ERR_INVALID_ARG, "resolution %ux%u outside 1..8192", width, height);
    gbr_renderer* r = new (std::nothrow) gbr_renderer();
    if (!r) return fail(GBR_ERR_OUT_OF_MEMORY, "host allocation failed");
    r->W = width;
    r->H = height;
    cudaError_t e = cudaGetDevice(&r->device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&r->num_sms, cudaDevAttrMultiProcessorCount, r->device);
    const size_t npx = (size_t)width * height;
    if (e == cudaSuccess) e = cudaMalloc(&r->d_colour, npx * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMalloc(&r->d_depth, npx * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&r->d_ids, npx * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMalloc(&r->d_gvis, npx * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMemset(r->d_gvis, 0xFF, npx * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMemset(r->d_colour, 0, npx * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMemset(r->d_depth, 0, npx * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(r->d_ids, 0xFF, npx * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMalloc(&r->d_ctl, sizeof(Ctl));
    if (e == cudaSuccess) e = cudaMemset(r->d_ctl, 0, sizeof(Ctl));
    if (e == cudaSuccess) e = cudaMallocHost(&r->h_ctl, sizeof(Ctl));
    if (e == cudaSuccess) e = cudaMalloc(&r->d_lights, kMaxLights * sizeof(LightDev));
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&r->meshes_evt, cudaEventDisableTiming);
    for (int i = 0; i < 5 && e == cudaSuccess; ++i) e = cudaEventCreate(&r->ev[i]);
    if (e != cudaSuccess) {
        gbr_destroy(r);
        return fail(GBR_ERR_CUDA, "gbr_create: %s", cudaGetErrorString(e));
    }
    *out = r;
    return GBR_OK;
}

gbr_status gbr_destroy(gbr_renderer* r) {
    if (!r) return GBR_OK;
    if (r->in_batches) return fail(GBR_ERR_INVALID_ARG, "the renderer is in %u batch(es): destroy them first", r->in_batches);
    cudaDeviceSynchronize();
    gbr_scene_clear(r);
    for (TexHost& t : r->textures) free_texture(t);
    free_bins(r);
    cudaFree(r->d_colour); cudaFree(r->d_depth); cudaFree(r->d_ids); cudaFree(r->d_gvis); cudaFree(r->d_shade_list);
    cudaFree(r->d_setup); cudaFree(r->d_rects); cudaFree(r->d_walk); cudaFree(r->d_keys); cudaFree(r->d_meshes); cudaFree(r->d_ctl); cudaFree(r->d_mlp_w);
    cudaFree(r->d_lights);
    cudaFreeHost(r->h_meshes); cudaFreeHost(r->h_ctl);
    if (r->meshes_evt) cudaEventDestroy(r->meshes_evt);
    for (int i = 0; i < 5; ++i)
        if (r->ev[i]) cudaEventDestroy(r->ev[i]);
    delete r;
    return GBR_OK;
}

gbr_status gbr_setup_bins(gbr_renderer* r, uint32_t num_bins_x, uint32_t num_bins_y, uint32_t bin_w, uint32_t bin_h,
                          uint32_t queue_chunk) {
    if (!r) return fail(GBR_ERR_INVALID_ARG, "renderer is null");
    if (num_bins_x == 0 || num_bins_y == 0 || bin_w == 0 || bin_h == 0 || bin_w > (uint32_t)kMaxBinDim ||
        bin_h > (uint32_t)kMaxBinDim)
        return fail(GBR_ERR_INVALID_ARG, "bins %ux%u of %ux%u px: need >= 1 bin of 1..%d px", num_bins_x, num_bins_y,
                    bin_w, bin_h, kMaxBinDim);
    if (num_bins_x > 32767u || num_bins_y > 32767u) return fail(GBR_ERR_INVALID_ARG, "too many bins");
    if (queue_chunk == 0) queue_chunk = 4096;
    cudaDeviceSynchronize();
    free_bins(r);
    r->nbx = num_bins_x; r->nby = num_bins_y; r->bw = bin_w; r->bh = bin_h; r->chunk = queue_chunk;
    r->row0 = r->row1 = 0u;   // a new bin grid: every row
    const uint32_t nb = num_bins_x * num_bins_y;
    GBR_CUDA(cudaMalloc(&r->d_counts, (size_t)kCountSplit * nb * sizeof(uint32_t)));
    GBR_CUDA(cudaMemset(r->d_counts, 0, (size_t)kCountSplit * nb * sizeof(uint32_t)));
    GBR_CUDA(cudaMalloc(&r->d_sub_base, (size_t)kCountSplit * nb * sizeof(uint32_t)));
    if (nb <= kMaxRowBins && r->num_sms > 0)
        GBR_CUDA(cudaMalloc(&r->d_row_base, (size_t)r->num_sms * nb * sizeof(uint32_t)));
    GBR_CUDA(cudaMalloc(&r->d_offsets, (nb + 1u) * sizeof(uint32_t)));
    GBR_CUDA(cudaMemset(r->d_offsets, 0, (nb + 1u) * sizeof(uint32_t)));
    GBR_CUDA(cudaMalloc(&r->d_cursors, nb * sizeof(uint32_t)));
    GBR_CUDA(cudaMalloc(&r->d_capacity, nb * sizeof(uint32_t)));
    GBR_CUDA(cudaMemset(r->d_capacity, 0, nb * sizeof(uint32_t)));
    GBR_CUDA(cudaMalloc(&r->d_bin_end, nb * sizeof(uint32_t)));
    GBR_CUDA(cudaMalloc(&r->d_dirty, 2u * (size_t)nb));
    GBR_CUDA(cudaMalloc(&r->d_scan, scan_state_bytes(nb)));
    GBR_CUDA(cudaMemset(r->d_scan, 0, scan_state_bytes(nb)));
    GBR_CUDA(cudaMemset(r->d_bin_end, 0, nb * sizeof(uint32_t)));
    // pre-pass accumulators: slot 4 (depth min) starts at all ones, the rest at 0
    GBR_CUDA(cudaMalloc(&r->d_feat, (size_t)kFeatSlots * nb * sizeof(uint32_t)));
    GBR_CUDA(cudaMemset(r->d_feat, 0, (size_t)kFeatSlots * nb * sizeof(uint32_t)));
    GBR_CUDA(cudaMemset(r->d_feat + 4u * nb, 0xFF, nb * sizeof(uint32_t)));
    GBR_CUDA(cudaMalloc(&r->d_features_out, (size_t)kFeatures * nb * sizeof(float)));
    int bps = 0;
    GBR_CUDA(raster_configure(bin_w, bin_h, r->raster_ctas, &bps));
    r->raster_blocks_per_sm = std::max(bps, 1);
    r->bins_ready = true;
    r->have_frame = false;
    return GBR_OK;
}

static gbr_status add_mesh(gbr_renderer* r, MeshHost&& m, uint32_t* mesh_id) {
    r->meshes.push_back(std::move(m));
    if (mesh_id) *mesh_id = (uint32_t)r->meshes.size() - 1u;
    return GBR_OK;
}

gbr_status gbr_mesh_upload(gbr_renderer* r, const void* vertices, uint32_t num_vertices, uint32_t vertex_format,
                           const uint32_t* indices, uint32_t num_indices, uint32_t topology, const float world[16],
                           const int32_t tex_ids[4], uint32_t* mesh_id) {
    if (!r) return fail(GBR_ERR_INVALID_ARG, "renderer is null");
    gbr_status st = validate_mesh_args(vertices, num_vertices, vertex_format, indices, num_indices, topology, world);
    if (st != GBR_OK) return st;
    MeshHost m;
    m.owned = true;
    m.num_vertices = num_vertices;
    m.num_indices = indices ? num_indices : 0u;
    m.vertex_format = vertex_format;
    m.topology = topology;
    m.num_tris = tri_count(num_vertices, indices, num_indices, topology);
    memcpy(m.world, world, sizeof m.world);
    if (tex_ids) memcpy(m.tex_ids, tex_ids, sizeof m.tex_ids);
    if (indices) {
        for (uint32_t i = 0; i < num_indices; ++i)
            if (indices[i] >= num_vertices)
                return fail(GBR_ERR_INVALID_ARG, "index %u at position %u is out of range (%u vertices)", indices[i], i,
                            num_vertices);
    }
    const size_t vbytes = (size_t)num_vertices * (vertex_format == GBR_VERTEX_IVERTEX56 ? 56u : 16u);
    if (vbytes) {
        GBR_CUDA(cudaMalloc(&m.d_vertices, vbytes));
        GBR_CUDA(cudaMemcpy(m.d_vertices, vertices, vbytes, cudaMemcpyHostToDevice));
    }
    if (indices && num_indices) {
        cudaError_t e = cudaMalloc(&m.d_indices, (size_t)num_indices * sizeof(uint32_t));
        if (e == cudaSuccess) e = cudaMemcpy(m.d_indices, indices, (size_t)num_indices * 4u, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            cudaFree(m.d_vertices);
            return fail(GBR_ERR_CUDA, "index upload: %s", cudaGetErrorString(e));
        }
    }
    return add_mesh(r, std::move(m), mesh_id);
}

gbr_status gbr_mesh_update_vertices(gbr_renderer* r, uint32_t mesh_id, const void* vertices, uint32_t num_vertices,
                                    void* stream) {
    if (!r || mesh_id >= r->meshes.size()) return fail(GBR_ERR_INVALID_ARG, "bad renderer or mesh id");
    MeshHost& m = r->meshes[mesh_id];
    if (!m.owned) return fail(GBR_ERR_INVALID_ARG, "mesh %u is bound to caller memory", mesh_id);
    if (num_vertices != m.num_vertices || !vertices)
        return fail(GBR_ERR_INVALID_ARG, "vertex count %u differs from the mesh's %u", num_vertices, m.num_vertices);
    const size_t vbytes = (size_t)num_vertices * (m.vertex_format == GBR_VERTEX_IVERTEX56 ? 56u : 16u);
    GBR_CUDA(cudaMemcpyAsync(m.d_vertices, vertices, vbytes, cudaMemcpyHostToDevice, (cudaStream_t)stream));
    return GBR_OK;
}

gbr_status gbr_mesh_bind_device(gbr_renderer* r, const void* d_vertices, uint32_t num_vertices, uint32_t vertex_format,
                                const uint32_t* d_indices, uint32_t num_indices, uint32_t topology,
                                const float world[16], const int32_t tex_ids[4], uint32_t* mesh_id) {
    if (!r) return fail(GBR_ERR_INVALID_ARG, "renderer is null");
    gbr_status st = validate_mesh_args(d_vertices, num_vertices, vertex_format, d_indices, num_indices, topology, world);
    if (st != GBR_OK) return st;
    if (vertex_format == GBR_VERTEX_POS3_RGBA8 && ((uintptr_t)d_vertices & 15u))
        return fail(GBR_ERR_INVALID_ARG, "compact vertices must be 16-byte aligned");
    MeshHost m;
    m.owned = false;
    m.d_vertices = const_cast<void*>(d_vertices);
    m.d_indices = const_cast<uint32_t*>(d_indices);
    m.num_vertices = num_vertices;
    m.num_indices = d_indices ? num_indices : 0u;
    m.vertex_format = vertex_format;
    m.topology = topology;
    m.num_tris = tri_count(num_vertices, d_indices, num_indices, topology);
    memcpy(m.world, world, sizeof m.world);
    if (tex_ids) memcpy(m.tex_ids, tex_ids, sizeof m.tex_ids);
    return add_mesh(r, std::move(m), mesh_id);
}

gbr_status gbr_mesh_set_world(gbr_renderer* r, uint32_t mesh_id, const float world[16]) {
    if (!r || mesh_id >= r->meshes.size() || !world) return fail(GBR_ERR_INVALID_ARG, "bad renderer, mesh id or matrix");
    memcpy(r->meshes[mesh_id].world, world, 16 * sizeof(float));
    return GBR_OK;
}

gbr_status gbr_mesh_set_textures(gbr_renderer* r, uint32_t mesh_id, const int32_t tex_ids[4]) {
    if (!r || mesh_id >= r->meshes.size() || !tex_ids) return fail(GBR_ERR_INVALID_ARG, "bad renderer, mesh id or ids");
    memcpy(r->meshes[mesh_id].tex_ids, tex_ids, 4 * sizeof(int32_t));
    return GBR_OK;
}

gbr_status gbr_scene_clear(gbr_renderer* r) {
    if (!r) return fail(GBR_ERR_INVALID_ARG, "renderer is null");
    cudaDeviceSynchronize();
    for (MeshHost& m : r->meshes)
        if (m.owned) {
            cudaFree(m.d_vertices);
            cudaFree(m.d_indices);
        }
    r->meshes.clear();
    r->last_uploaded.clear();
    r->have_frame = false;
    return GBR_OK;
}

gbr_status gbr_texture_upload(gbr_renderer* r, const uint32_t* rgba8, uint32_t w, uint32_t h, int32_t* tex_id) {
    if (!r || !rgba8 || !tex_id) return fail(GBR_ERR_INVALID_ARG, "null argument");
    if (w == 0 || h == 0 || (uint64_t)w * h > 0x7FFFFFFFull) return fail(GBR_ERR_INVALID_ARG, "texture %ux%u", w, h);
    TexHost t;
    t.w = w;
    t.h = h;
    GBR_CUDA(cudaMalloc(&t.d_px, (size_t)w * h * 4u));
    cudaError_t e = cudaMemcpy(t.d_px, rgba8, (size_t)w * h * 4u, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaFree(t.d_px);
        return fail(GBR_ERR_CUDA, "texture upload: %s", cudaGetErrorString(e));
    }
    r->textures.push_back(t);
    *tex_id = (int32_t)r->textures.size() - 1;
    r->last_uploaded.clear();
    return GBR_OK;
}

gbr_status gbr_texture_remove(gbr_renderer* r, int32_t tex_id) {
    if (!r || tex_id < 0 || (size_t)tex_id >= r->textures.size() || !r->textures[tex_id].d_px)
        return fail(GBR_ERR_NOT_FOUND, "texture %d does not exist", tex_id);
    cudaDeviceSynchronize();
    free_texture(r->textures[tex_id]);
    r->last_uploaded.clear();
    return GBR_OK;
}

gbr_status gbr_set_lights(gbr_renderer* r, const gbr_light* lights, uint32_t n) {
    if (!r || (n && !lights) || n > kMaxLights) return fail(GBR_ERR_INVALID_ARG, "bad renderer or lights (n %u, max %u)", n, kMaxLights);
    static_assert(sizeof(gbr_light) == sizeof(LightDev), "gbr_light mirrors the device record");
    for (uint32_t k = 0; k < n; ++k)
        if (lights[k].type > GBR_LIGHT_POINT) return fail(GBR_ERR_INVALID_ARG, "light %u: unknown type %u", k, lights[k].type);
    if (n) {
        cudaDeviceSynchronize();   // frames in flight read the previous lights
        GBR_CUDA(cudaMemcpy(r->d_lights, lights, n * sizeof(LightDev), cudaMemcpyHostToDevice));
    }
    r->num_lights = n;
    return GBR_OK;
}

gbr_status gbr_set_binning(gbr_renderer* r, uint32_t method) {
    if (!r || method > GBR_BINNING_PREDICTED) return fail(GBR_ERR_INVALID_ARG, "bad renderer or binning method");
    r->binning = method;
    return GBR_OK;
}

gbr_status gbr_set_raster_params(gbr_renderer* r, uint32_t phase, uint32_t ctas_per_sm) {
    if (!r || phase > kMaxPhase || (ctas_per_sm != 0 && (ctas_per_sm < 2 || ctas_per_sm > 6)))
        return fail(GBR_ERR_INVALID_ARG, "phase %u (0..%u) / ctas_per_sm %u (0, 2..6)", phase, kMaxPhase, ctas_per_sm);
    r->raster_phase = phase;
    r->raster_ctas = ctas_per_sm;
    if (r->bins_ready) {
        int bps = 0;
        GBR_CUDA(raster_configure(r->bw, r->bh, ctas_per_sm, &bps));
        r->raster_blocks_per_sm = std::max(bps, 1);
    }
    return GBR_OK;
}

gbr_status gbr_set_raster_staging(gbr_renderer* r, uint32_t mode) {
    if (!r || mode > GBR_STAGING_TMA) return fail(GBR_ERR_INVALID_ARG, "bad renderer or staging mode %u", mode);
    r->rec_tma = mode == GBR_STAGING_TMA ? 1u : 0u;
    return GBR_OK;
}

gbr_status gbr_set_bin_rows(gbr_renderer* r, uint32_t row0, uint32_t row1) {
    if (!r) return fail(GBR_ERR_INVALID_ARG, "renderer is null");
    if (!r->bins_ready) return fail(GBR_ERR_INVALID_ARG, "gbr_setup_bins was not called");
    if (!(row0 == 0u && row1 == 0u) && !(row0 < row1 && row1 <= r->nby))
        return fail(GBR_ERR_INVALID_ARG, "bin rows [%u, %u) outside [0, %u)", row0, row1, r->nby);
    r->row0 = row0;
    r->row1 = row1;
    r->dirty_valid = false;
    return GBR_OK;
}

gbr_status gbr_set_scan_wait(gbr_renderer* r, uint32_t spin_limit, int32_t silent_tile) {
    if (!r || silent_tile < -1) return fail(GBR_ERR_INVALID_ARG, "bad renderer or silent tile %d", silent_tile);
    r->scan_spin_limit = spin_limit;
    r->scan_silent_tile1 = (uint32_t)(silent_tile + 1);
    return GBR_OK;
}

gbr_status gbr_set_timing(gbr_renderer* r, int mode) {
    if (!r) return fail(GBR_ERR_INVALID_ARG, "renderer is null");
    if (mode < GBR_TIMING_OFF || mode > GBR_TIMING_TOTAL) return fail(GBR_ERR_INVALID_ARG, "unknown timing mode");
    r->timing = mode;
    return GBR_OK;
}

gbr_status gbr_render(gbr_renderer* r, const gbr_camera* cam, uint32_t cull, uint32_t sample, uint32_t vis,
                      void* stream) {
    if (!r || !cam) return fail(GBR_ERR_INVALID_ARG, "null renderer or camera");
    if (!r->bins_ready) return fail(GBR_ERR_INVALID_ARG, "gbr_setup_bins was not called");
    if (cull > GBR_CULL_NONE || sample > GBR_SAMPLE_BILINEAR || vis > GBR_VIS_NORMAL)
        return fail(GBR_ERR_INVALID_ARG, "bad cull/sample/vis (%u/%u/%u)", cull, sample, vis);
    return render_frame(r, cam, cull, sample, vis, (cudaStream_t)stream);
}

gbr_status gbr_readback(gbr_renderer* r, uint32_t* colour, float* depth, void* stream) {
    if (!r) return fail(GBR_ERR_INVALID_ARG, "renderer is null");
    if (!r->have_frame && !r->drawn) return fail(GBR_ERR_INVALID_ARG, "no frame rendered");
    cudaStream_t s = (cudaStream_t)stream;
    if (r->have_frame) {
        gbr_status st = finish_frame(r, s);
        if (st != GBR_OK) return st;
    }
    const size_t npx = (size_t)r->W * r->H;
    if (colour) GBR_CUDA(cudaMemcpyAsync(colour, r->d_colour, npx * 4u, cudaMemcpyDeviceToHost, s));
    if (depth) GBR_CUDA(cudaMemcpyAsync(depth, r->d_depth, npx * 4u, cudaMemcpyDeviceToHost, s));
    GBR_CUDA(cudaStreamSynchronize(s));
    return GBR_OK;
}

gbr_status gbr_predicted_capacities(gbr_renderer* r, uint32_t* capacities, void* stream) {
    if (!r || !capacities) return fail(GBR_ERR_INVALID_ARG, "null argument");
    if (!r->have_frame || !r->last_predicted) return fail(GBR_ERR_INVALID_ARG, "no predicted-binning frame rendered");
    cudaStream_t s = (cudaStream_t)stream;
    gbr_status st = finish_frame(r, s);
    if (st != GBR_OK) return st;
    GBR_CUDA(cudaMemcpyAsync(capacities, r->d_capacity, (size_t)r->nbx * r->nby * 4u, cudaMemcpyDeviceToHost, s));
    GBR_CUDA(cudaStreamSynchronize(s));
    return GBR_OK;
}

gbr_status gbr_readback_ids(gbr_renderer* r, uint32_t* ids, void* stream) {
    if (!r || !ids) return fail(GBR_ERR_INVALID_ARG, "null argument");
    if (!r->have_frame) return fail(GBR_ERR_INVALID_ARG, "no frame rendered");
    cudaStream_t s = (cudaStream_t)stream;
    gbr_status st = finish_frame(r, s);
    if (st != GBR_OK) return st;
    GBR_CUDA(cudaMemcpyAsync(ids, r->d_ids, (size_t)r->W * r->H * 4u, cudaMemcpyDeviceToHost, s));
    GBR_CUDA(cudaStreamSynchronize(s));
    return GBR_OK;
}

gbr_status gbr_device_buffers(gbr_renderer* r, void** d_colour, void** d_depth) {
    if (!r) return fail(GBR_ERR_INVALID_ARG, "renderer is null");
    if (d_colour) *d_colour = r->d_colour;
    if (d_depth) *d_depth = r->d_depth;
    return GBR_OK;
}

gbr_status gbr_get_bins(gbr_renderer* r, uint32_t* offsets, uint32_t* ids, uint64_t capacity, uint64_t* num_pairs,
                        void* stream) {
    if (!r) return fail(GBR_ERR_INVALID_ARG, "renderer is null");
    if (!r->have_frame) return fail(GBR_ERR_INVALID_ARG, "no frame rendered");
    cudaStream_t s = (cudaStream_t)stream;
    gbr_status st = finish_frame(r, s);
    if (st != GBR_OK) return st;
    const uint32_t nb = r->nbx * r->nby;
    std::vector<uint32_t> off(nb + 1u);
    GBR_CUDA(cudaMemcpy(off.data(), r->d_offsets, (nb + 1u) * sizeof(uint32_t), cudaMemcpyDeviceToHost));
    if (r->last_predicted && !r->h_ctl->pred_overflow) {
        // predicted capacities: bin b holds min(cursor - offset, capacity) entries
        // from its offset; the tail of each bin's capacity is unused
        std::vector<uint32_t> cur(nb), cap(nb), out_off(nb + 1u, 0u);
        GBR_CUDA(cudaMemcpy(cur.data(), r->d_cursors, nb * sizeof(uint32_t), cudaMemcpyDeviceToHost));
        GBR_CUDA(cudaMemcpy(cap.data(), r->d_capacity, nb * sizeof(uint32_t), cudaMemcpyDeviceToHost));
        for (uint32_t b = 0; b < nb; ++b) out_off[b + 1] = out_off[b] + std::min(cur[b] - off[b], cap[b]);
        const uint64_t total = out_off[nb];
        if (num_pairs) *num_pairs = total;
        if (offsets) memcpy(offsets, out_off.data(), (nb + 1u) * sizeof(uint32_t));
        if (ids) {
            if (capacity < total) return fail(GBR_ERR_INVALID_ARG, "ids capacity %llu < %llu pairs",
                                              (unsigned long long)capacity, (unsigned long long)total);
            std::vector<uint32_t> all(off[nb]);
            if (!all.empty())
                GBR_CUDA(cudaMemcpy(all.data(), r->d_list, all.size() * sizeof(uint32_t), cudaMemcpyDeviceToHost));
            for (uint32_t b = 0; b < nb; ++b)
                for (uint32_t k = 0; k < out_off[b + 1] - out_off[b]; ++k) ids[out_off[b] + k] = all[off[b] + k] & ~kNoRasterBit;
        }
        return GBR_OK;
    }
    const uint64_t total = off[nb];
    if (num_pairs) *num_pairs = total;
    if (offsets) memcpy(offsets, off.data(), (nb + 1u) * sizeof(uint32_t));
    if (ids) {
        if (capacity < total) return fail(GBR_ERR_INVALID_ARG, "ids capacity %llu < %llu pairs",
                                          (unsigned long long)capacity, (unsigned long long)total);
        if (total) GBR_CUDA(cudaMemcpy(ids, r->d_list, total * sizeof(uint32_t), cudaMemcpyDeviceToHost));
        for (uint64_t i = 0; i < total; ++i) ids[i] &= ~kNoRasterBit;
    }
    return GBR_OK;
}

gbr_status gbr_set_predictor(gbr_renderer* r, const uint16_t* weights_bf16, uint32_t num_params, float alpha,
                             float beta, float gamma) {
    if (!r) return fail(GBR_ERR_INVALID_ARG, "renderer is null");
    if (!weights_bf16 && num_params == 0u) {
        // the plain method: l = the pre-pass's sampled pair count x the sampling stride
        r->sampled_rule = true;
    } else {
        if (!weights_bf16 || num_params != (uint32_t)kMlpParams)
            return fail(GBR_ERR_INVALID_ARG, "predictor needs %d BF16 parameters (or none)", kMlpParams);
        if (!r->d_mlp_w) GBR_CUDA(cudaMalloc(&r->d_mlp_w, kMlpParamsPadded * sizeof(uint16_t)));
        GBR_CUDA(cudaMemcpy(r->d_mlp_w, weights_bf16, kMlpParams * sizeof(uint16_t), cudaMemcpyHostToDevice));
        r->sampled_rule = false;
    }
    r->cap_alpha = alpha;
    r->cap_beta = beta;
    r->cap_gamma = gamma;
    r->predictor_ready = true;
    return GBR_OK;
}

gbr_status gbr_collect_bin_features(gbr_renderer* r, const gbr_camera* cam, uint32_t cull, uint32_t sample,
                                    uint32_t vis, float* features, uint32_t* counts, void* stream) {
    if (!r || !cam || !features || !counts) return fail(GBR_ERR_INVALID_ARG, "null argument");
    if (!r->bins_ready) return fail(GBR_ERR_INVALID_ARG, "gbr_setup_bins was not called");
    cudaStream_t s = (cudaStream_t)stream;
    r->collect = true;
    gbr_status st = render_frame(r, cam, cull, sample, vis, s);
    if (st == GBR_OK) st = finish_frame(r, s);
    r->collect = false;
    if (st != GBR_OK) return st;
    const uint32_t nb = r->nbx * r->nby;
    std::vector<uint32_t> off(nb + 1u);
    GBR_CUDA(cudaMemcpy(off.data(), r->d_offsets, (nb + 1u) * sizeof(uint32_t), cudaMemcpyDeviceToHost));
    for (uint32_t b = 0; b < nb; ++b) counts[b] = off[b + 1] - off[b];
    GBR_CUDA(cudaMemcpy(features, r->d_features_out, (size_t)nb * kFeatures * sizeof(float), cudaMemcpyDeviceToHost));
    return GBR_OK;
}

uint32_t gbr_mlp_num_params(void) { return (uint32_t)kMlpParams; }

gbr_status gbr_mlp_predict(const uint16_t* d_w, const float* d_x, uint32_t n, float* d_out, void* stream) {
    if (!d_w || (!d_x && n) || (!d_out && n)) return fail(GBR_ERR_INVALID_ARG, "null argument");
    GBR_CUDA(launch_mlp_predict(d_w, d_x, n, d_out, (cudaStream_t)stream));
    return GBR_OK;
}

gbr_status gbr_mlp_loss_grad(const uint16_t* d_w, const float* d_x, const float* d_y, uint32_t n, float* d_grad,
                             float* d_loss, void* stream) {
    if (!d_w || !d_grad || !d_loss || ((!d_x || !d_y) && n)) return fail(GBR_ERR_INVALID_ARG, "null argument");
    GBR_CUDA(launch_mlp_grad(d_w, d_x, d_y, n, d_grad, d_loss, (cudaStream_t)stream));
    return GBR_OK;
}

gbr_status gbr_mlp_adam(float* d_master, uint16_t* d_w, const float* d_grad, float* d_m, float* d_v, uint32_t step,
                        float lr, float grad_scale, void* stream) {
    if (!d_master || !d_w || !d_grad || !d_m || !d_v || step == 0) return fail(GBR_ERR_INVALID_ARG, "bad argument");
    GBR_CUDA(launch_mlp_adam(d_master, d_w, d_grad, d_m, d_v, step, lr, grad_scale, (cudaStream_t)stream));
    return GBR_OK;
}

gbr_status gbr_get_stats(gbr_renderer* r, gbr_stats* out, void* stream) {
    if (!r || !out) return fail(GBR_ERR_INVALID_ARG, "null argument");
    memset(out, 0, sizeof *out);
    for (const MeshHost& m : r->meshes) out->num_triangles += m.num_tris;
    out->overflow_reruns = r->overflow_reruns;
    if (!r->have_frame) return GBR_OK;
    gbr_status st = finish_frame(r, (cudaStream_t)stream);
    if (st != GBR_OK) return st;
    out->num_visible = r->h_ctl->num_visible;
    out->num_pairs = r->h_ctl->num_pairs;
    out->num_work_items = r->h_ctl->num_items;
    out->num_float_path = r->h_ctl->num_float_path;
    out->predicted_overflow = r->h_ctl->pred_overflow;
    out->predicted_capacity = r->h_ctl->pred_capacity;
    out->count_blocks = r->last_row_blocks;
    out->raster_lanes = r->last_raster_lanes;
    out->ms_setup = out->ms_bin = out->ms_raster = out->ms_shade = out->ms_total = 0.f;
    if (r->timing == GBR_TIMING_TOTAL && r->ev_recorded) {
        cudaEventElapsedTime(&out->ms_total, r->ev[0], r->ev[3]);
    } else if (r->timing && r->ev_recorded) {
        cudaEventElapsedTime(&out->ms_setup, r->ev[0], r->ev[1]);
        cudaEventElapsedTime(&out->ms_bin, r->ev[1], r->ev[2]);
        cudaEventElapsedTime(&out->ms_raster, r->ev[2], r->ev[4]);
        cudaEventElapsedTime(&out->ms_shade, r->ev[4], r->ev[3]);
        cudaEventElapsedTime(&out->ms_total, r->ev[0], r->ev[3]);
    }
    return GBR_OK;
}

}  // extern "C"
