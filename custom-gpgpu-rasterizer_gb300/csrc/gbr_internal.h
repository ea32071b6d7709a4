// gbr_internal.h -- host-side state shared by the library's translation
// units: the renderer object behind the C ABI's gbr_renderer handle, and
// the per-frame descriptor builders used by the single-frame path
// (gbr_api.cu) and the batched path (gbr_batch.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "../../include/gbr.h"
#include "gbr_device.cuh"

namespace gbr {

// Records the message for gbr_last_error_string() and returns st.
gbr_status fail(gbr_status st, const char* fmt, ...);

#define GBR_CUDA(call)                                                                                        \
    do {                                                                                                      \
        cudaError_t e_ = (call);                                                                              \
        if (e_ != cudaSuccess) return ::gbr::fail(GBR_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

struct MeshHost {
    bool owned = false;
    void* d_vertices = nullptr;
    uint32_t* d_indices = nullptr;
    uint32_t num_vertices = 0, num_indices = 0, vertex_format = 0, topology = 0;
    uint64_t num_tris = 0;
    float world[16];
    int32_t tex_ids[4] = {-1, -1, -1, -1};
};

struct TexHost {
    uint32_t* d_px = nullptr;
    uint32_t w = 0, h = 0;
    // hardware texture object for gbr_draw_texture (made on first use, over
    // a pitched copy when the rows are not aligned for a pitch-2D texture)
    unsigned long long tex_obj = 0;
    uint32_t* d_pitched = nullptr;
};
// Releases a texture's device memory and texture object (the device is idle).
void free_texture(TexHost& t);

// Matrix<4,4>::operator*(Matrix<4,4>) (Matrix4.h:120-143) on the host, left
// to right with no fused multiply-add (built with -ffp-contract=off), as the
// reference computes WVP.
void mat4_mul(const float* lm, const float* rm, float* out);

}  // namespace gbr

struct gbr_renderer {
    int device = 0;
    int num_sms = 0;
    uint32_t W = 0, H = 0;
    uint32_t nbx = 0, nby = 0, bw = 0, bh = 0, chunk = 256;
    bool bins_ready = false;
    uint32_t binning = GBR_BINNING_EXACT;
    int timing = 0;           // GBR_TIMING_*
    int raster_blocks_per_sm = 1;
    uint32_t raster_phase = 0;   // 0: library default
    uint32_t raster_ctas = 0;    // 0: library default
    uint32_t row0 = 0, row1 = 0;      // gbr_set_bin_rows: this renderer's bin rows (row1 0: all)
    uint32_t rec_tma = 0;             // gbr_set_raster_staging: 1 = bulk asynchronous copies
    uint32_t scan_spin_limit = 0;     // gbr_set_scan_wait (0: the library's bound)
    uint32_t scan_silent_tile1 = 0;   // gbr_set_scan_wait: 1 + the silent tile (0: none)
    // the last finished frame's pair and visible-triangle counts: they size
    // the next frames' raster work items and phases (0: none seen yet)
    uint64_t seen_pairs = 0, seen_visible = 0;

    // predicted-capacity binning
    uint32_t* d_feat = nullptr;
    uint16_t* d_mlp_w = nullptr;
    bool predictor_ready = false;
    bool sampled_rule = false;   // capacities from the sampled pair counts, no network
    float cap_alpha = 0.f, cap_beta = 0.f, cap_gamma = 0.f;
    float* d_features_out = nullptr;
    bool collect = false;
    bool last_predicted = false;

    std::vector<gbr::MeshHost> meshes;
    std::vector<gbr::TexHost> textures;

    uint32_t* d_colour = nullptr;
    float* d_depth = nullptr;
    uint32_t* d_ids = nullptr;
    unsigned long long* d_gvis = nullptr;
    uint32_t* d_shade_list = nullptr;   // two-pass shading queue, W x H (allocated on first use)

    uint32_t* d_counts = nullptr;     // kCountSplit x bins
    uint32_t* d_sub_base = nullptr;   // kCountSplit x bins
    uint32_t* d_row_base = nullptr;   // num_sms x bins (block-row exact binning; bins <= kMaxRowBins)
    uint32_t last_row_blocks = 0;     // blocks of the last frame's block-row count pass (0: sub-counters)
    uint32_t last_raster_lanes = 0;   // the last frame's raster took the small-triangle variant
    uint32_t* d_offsets = nullptr;
    uint32_t* d_cursors = nullptr;
    uint32_t* d_capacity = nullptr;
    uint32_t* d_bin_end = nullptr;
    gbr::ScanState* d_scan = nullptr;   // bin scan state (zeroed once)
    uint4* d_items = nullptr;
    uint32_t items_cap = 0;
    uint32_t* d_list = nullptr;
    uint64_t list_cap = 0;

    gbr::TriSetup* d_setup = nullptr;
    uint2* d_rects = nullptr;
    uint32_t* d_walk = nullptr;     // first rank slot of each 32-triangle walk
    uint32_t* d_keys = nullptr;     // per-triangle depth-key bounds
    uint64_t tri_cap = 0;

    gbr::MeshDev* d_meshes = nullptr;
    gbr::MeshDev* h_meshes = nullptr;
    uint32_t meshes_cap = 0;
    std::vector<gbr::MeshDev> last_uploaded;
    cudaEvent_t meshes_evt = nullptr;

    gbr::Ctl* d_ctl = nullptr;
    gbr::Ctl* h_ctl = nullptr;

    gbr::LightDev* d_lights = nullptr;   // kMaxLights records
    uint32_t num_lights = 0;

    bool have_frame = false;
    bool drawn = false;   // a texture was drawn into the colour buffer (gbr_draw_texture*)
    gbr_camera last_cam{};
    uint32_t last_cull = 0, last_sample = 0, last_vis = 0;
    uint32_t overflow_reruns = 0;
    cudaEvent_t ev[5] = {};
    bool ev_recorded = false;
    uint32_t in_batches = 0;     // gbr_batch objects this renderer is a member of
    // two-pass frames: per-bin "may hold drawn pixels" flags, two buffers of
    // num_bins bytes alternating by frame (FrameDev::dirty_rd / dirty_wr).
    // dirty_valid: they describe the frame buffers as the last frame left
    // them, cleared for visualisation dirty_vis; any other writer of the
    // buffers (one-pass frames, texture blits, batch frames, a new bin
    // band) clears it, and the next two-pass frame marks every bin first.
    uint8_t* d_dirty = nullptr;
    uint32_t dirty_parity = 0;
    bool dirty_valid = false;
    uint32_t dirty_vis = 0;
};

namespace gbr {

// Number of triangles of the renderer's scene.
uint64_t scene_triangles(const gbr_renderer* r);

// The per-mesh descriptors of one frame seen through `cam`: WVP = Proj *
// View * World per mesh, the texture slots bound as UpdateCUDAMeshTextures
// binds them, and prim_base numbering the scene's triangles from 0.
void build_mesh_table(const gbr_renderer* r, const gbr_camera* cam, MeshDev* out);

// The frame descriptor fields that depend only on the renderer's resolution
// and the render state (no binning storage).
void frame_basics(const gbr_renderer* r, const gbr_camera* cam, uint32_t cull, uint32_t sample, uint32_t vis,
                  FrameDev& F);

}  // namespace gbr
