/*
 * gbr.h -- C ABI of the GB300 frame-hot-path renderer.
 *
 * Drop-in for the per-frame path of Custom-CUDA-Rasterizer's CUDARenderer
 * (CustomCUDARasterizer/CUDARenderer.h:31-141): mesh and texture upload
 * (CUDAMesh, CUDATextureManager), bin setup, the per-frame render call with
 * CullingMode / SampleState / VisualisationState, and the framebuffer
 * readback that Present() performs.  Plain C types only; a CUDA stream is
 * passed as void* (cudaStream_t), NULL meaning the legacy default stream.
 *
 * Every entry point returns a gbr_status; none exits or throws.  The message
 * of the last failure on the calling thread is gbr_last_error_string().
 *
 * Enum values are the reference's integer values (CullingMode.h,
 * VisualisationState.h, SampleState.h, PrimitiveTopology.h).
 */
#ifndef GBR_H
#define GBR_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    GBR_OK = 0,
    GBR_ERR_INVALID_ARG = 1,
    GBR_ERR_CUDA = 2,
    GBR_ERR_OVERFLOW_RERUN = 3, /* informational: a frame was re-binned after a capacity overflow */
    GBR_ERR_TIMEOUT = 4,
    GBR_ERR_OUT_OF_MEMORY = 5,
    GBR_ERR_NOT_FOUND = 6
} gbr_status;

/* CullingMode (CullingMode.h:3-7) */
enum { GBR_CULL_BACKFACE = 0, GBR_CULL_FRONTFACE = 1, GBR_CULL_NONE = 2 };
/* SampleState (SampleState.h:3-7); GBR_SAMPLE_BILINEAR is the build's
 * extension (the reference's "Linear" is a 5-tap filter,
 * CUDATextureSampler.cuh:112-190): true bilinear filtering, texel centres at
 * (i + 1/2) / size, addresses clamped to the texture. */
enum { GBR_SAMPLE_POINT = 0, GBR_SAMPLE_LINEAR = 1, GBR_SAMPLE_BILINEAR = 2 };
/* VisualisationState (VisualisationState.h:3-7) */
enum { GBR_VIS_PBR = 0, GBR_VIS_DEPTH = 1, GBR_VIS_NORMAL = 2 };
/* PrimitiveTopology (PrimitiveTopology.h:3-7) */
enum { GBR_TOPOLOGY_TRIANGLE_LIST = 0, GBR_TOPOLOGY_TRIANGLE_STRIP = 1 };
/* Vertex layouts accepted by gbr_mesh_upload */
enum {
    GBR_VERTEX_IVERTEX56 = 0,  /* IVertex (Vertex.h:113-145): p3 uv2 n3 tan3 c3 floats, 56 B */
    GBR_VERTEX_POS3_RGBA8 = 1  /* p3 floats + RGBA8 colour (byte0 = R), 16 B */
};
/* Texture slots (Mesh::TextureID, Mesh.h:9-15) */
enum { GBR_TEX_DIFFUSE = 0, GBR_TEX_NORMAL = 1, GBR_TEX_SPECULAR = 2, GBR_TEX_GLOSSINESS = 3 };
/* Binning method */
enum { GBR_BINNING_EXACT = 0, GBR_BINNING_PREDICTED = 1 };

typedef struct gbr_renderer gbr_renderer;

/* Camera state Render() reads (CUDARenderer.cu:215-219): position, forward
 * (the look-at matrix's third column), view and projection matrices, column
 * major with element (r, c) at [c*4 + r] (Matrix.h:9-21). */
typedef struct {
    float pos[3];
    float fwd[3];
    float view[16];
    float proj[16];
} gbr_camera;

typedef struct {
    uint64_t num_triangles;      /* GetTotalNumTriangles (CUDARenderer.h:64) */
    uint64_t num_visible;        /* GetTotalNumVisibleTriangles (CUDARenderer.h:63) */
    uint64_t num_pairs;          /* (triangle, bin) pairs of the last frame */
    uint64_t num_work_items;     /* raster work items (bin chunks) */
    uint64_t num_float_path;     /* visible triangles outside the fixed-point guard band */
    uint32_t overflow_reruns;    /* frames re-binned exactly after a capacity overflow */
    uint32_t predicted_overflow; /* last predicted-capacity frame overflowed a bin */
    uint64_t predicted_capacity; /* sum of predicted per-bin capacities, last frame */
    float ms_setup, ms_bin, ms_raster, ms_total; /* per-stage times of the last frame with timing on */
    float ms_shade;              /* the shade pass (included in ms_total, not in ms_raster) */
    uint32_t count_blocks;       /* blocks with private counter rows in the last frame's exact
                                    count pass (0: per-bin counters in global memory) */
    uint32_t raster_lanes;       /* 1: the last frame's raster took its small-triangle variant (a lane
                                    per triangle; picked for sparse frames of small triangles) */
    uint32_t reserved;
} gbr_stats;

/* CUDARenderer(const WindowHelper&) (CUDARenderer.cu:33-46): headless, the
 * frame buffers live on the current CUDA device. */
gbr_status gbr_create(uint32_t width, uint32_t height, gbr_renderer **out);
/* ~CUDARenderer (CUDARenderer.cu:48-53) */
gbr_status gbr_destroy(gbr_renderer *r);

/* SetupBins(numBins, binDim, queueMaxSize) (CUDARenderer.cu:199-204).
 * Bins are exact-sized (no capacity, no dropped triangles); queue_chunk
 * keeps the queue size's role in the raster: a bin's triangles are
 * depth-sorted and rasterised into its tile queue_chunk at a time (at most
 * 2048; 0 = 4096, i.e. 2048).  Long bins are split across raster CTAs by the
 * library, in work items of 64..4096 entries sized from the last frame. */
gbr_status gbr_setup_bins(gbr_renderer *r, uint32_t num_bins_x, uint32_t num_bins_y,
                          uint32_t bin_w, uint32_t bin_h, uint32_t queue_chunk);

/* LoadScene -> new CUDAMesh(Mesh*) (CUDARenderer.cu:177-197, CUDAMesh.cpp:4-20,
 * 42-59): copies the host vertex and index buffers to the device.
 * indices may be NULL for a non-indexed triangle list (vertex 3t+k of
 * triangle t).  world: the mesh's world matrix.  tex_ids: texture ids
 * (-1 = none) resolved as UpdateCUDAMeshTextures (CUDARenderer.cu:542-573). */
gbr_status gbr_mesh_upload(gbr_renderer *r, const void *vertices, uint32_t num_vertices,
                           uint32_t vertex_format, const uint32_t *indices, uint32_t num_indices,
                           uint32_t topology, const float world[16], const int32_t tex_ids[4],
                           uint32_t *mesh_id);
/* Replace a mesh's vertices (same count and layout) with an asynchronous
 * host-to-device copy on `stream`; host memory should be pinned. */
gbr_status gbr_mesh_update_vertices(gbr_renderer *r, uint32_t mesh_id, const void *vertices,
                                    uint32_t num_vertices, void *stream);
/* Bind device-resident vertices (and optional indices) that the caller owns
 * and keeps alive; no copy is made. */
gbr_status gbr_mesh_bind_device(gbr_renderer *r, const void *d_vertices, uint32_t num_vertices,
                                uint32_t vertex_format, const uint32_t *d_indices, uint32_t num_indices,
                                uint32_t topology, const float world[16], const int32_t tex_ids[4],
                                uint32_t *mesh_id);
/* CUDAMesh::GetWorld() assignment (CUDAMesh.h:17-18) */
gbr_status gbr_mesh_set_world(gbr_renderer *r, uint32_t mesh_id, const float world[16]);
gbr_status gbr_mesh_set_textures(gbr_renderer *r, uint32_t mesh_id, const int32_t tex_ids[4]);
/* FreeAllCUDAMeshBuffers (CUDARenderer.cu:488-496) */
gbr_status gbr_scene_clear(gbr_renderer *r);

/* CUDATexture::Create + CUDATextureManager::AddCUDATexture
 * (CUDATexture.cpp:24-72, CUDATextureManager.cpp:29-37): RGBA8 texels,
 * byte0 = R as the sampler reads them (RGBRaw.h:34-38), rows of w texels. */
gbr_status gbr_texture_upload(gbr_renderer *r, const uint32_t *rgba8, uint32_t w, uint32_t h, int32_t *tex_id);
/* CUDATextureManager::RemoveCUDATexture (CUDATextureManager.cpp:39-54) */
gbr_status gbr_texture_remove(gbr_renderer *r, int32_t tex_id);

/* DrawTexture (CUDARenderer.cu:1968-1988, TextureTestKernel :1565-1588):
 * texture `tex_id` (gbr_texture_upload) stretched over the colour buffer
 * through the texture hardware (normalised coordinates, point filtering,
 * wrap addressing, as CUDATexture::Create sets it up), red and blue bytes
 * swapped.  Asynchronous on `stream`; gbr_readback returns the image. */
gbr_status gbr_draw_texture(gbr_renderer *r, int32_t tex_id, void *stream);
/* DrawTextureGlobal (CUDARenderer.cu:1990-2012, DrawTextureGlobalKernel
 * :1590-1615): uv = pixel / window size (stretch_to_window) or / texture
 * size, the shader's sampler `sample` (GBR_SAMPLE_*), colour32 as the pixel
 * shader writes it. */
gbr_status gbr_draw_texture_global(gbr_renderer *r, int32_t tex_id, int stretch_to_window, uint32_t sample,
                                   void *stream);

/* ObjParser (ObjParser.h:8-48, ObjParser.cpp): Wavefront OBJ text ->
 * IVertex vertices (GBR_VERTEX_IVERTEX56) + triangle-list indices, with the
 * reference's line grammar, vertex de-duplication and tangent generation
 * (gbr_obj.cpp states where it sets what the reference leaves unset).  A
 * host-side reader: no device work. */
typedef struct gbr_ivertex {
    float p[3], uv[2], n[3], tan[3], c[3]; /* IVertex (Vertex.h:113-145), 56 B */
} gbr_ivertex;
/* VertexType (VertexType.h:3-11) flags of a read mesh */
enum { GBR_VT_POS = 0, GBR_VT_UV = 1, GBR_VT_COL = 2, GBR_VT_NORM = 4, GBR_VT_TAN = 8, GBR_VT_VD = 16 };
typedef struct gbr_obj_mesh {
    gbr_ivertex *vertices;  /* num_vertices, malloc'd: release with gbr_obj_free */
    uint32_t *indices;      /* num_indices (3 per face) */
    uint32_t num_vertices, num_indices;
    uint32_t num_faces;     /* "f" lines read */
    int32_t vertex_type;    /* GBR_VT_* */
} gbr_obj_mesh;
/* ReadFromObjFile after OpenFile + SetInvertYAxis: `path` must end in the
 * reference's ".obj" (from its first '.'); GBR_ERR_NOT_FOUND if it cannot be
 * opened, GBR_ERR_INVALID_ARG (with the line) where the reference would throw
 * or index out of range. */
gbr_status gbr_obj_read_file(const char *path, int invert_y, gbr_obj_mesh *out);
/* The same from text in memory. */
gbr_status gbr_obj_read_text(const char *text, size_t length, int invert_y, gbr_obj_mesh *out);
void gbr_obj_free(gbr_obj_mesh *mesh);

/* Learned bin capacity (no counterpart in the reference, whose queues have a
 * fixed size and drop triangles when full, CUDAAtomicQueue.cuh:8-26).
 * gbr_set_predictor installs the capacity model: num_params BF16 parameters
 * of the 12-64-64-1 MLP (gbr_mlp_num_params()) and the capacity rule
 * ceil(l*(1+alpha) + beta*sqrt(l+1) + gamma) for a predicted count l,
 * clamped to the scene's triangle count.  With
 * GBR_BINNING_PREDICTED a frame bins in one pass into the predicted
 * capacities; if any bin overflows, the frame is re-binned exactly on the
 * device, so bin lists and images never depend on the prediction.
 * gbr_collect_bin_features renders one exact frame and returns, per bin, the
 * model's 12 input features and the exact triangle count (training data).
 * gbr_mlp_* are the model's GPU kernels on caller device buffers: forward
 * predictions, loss + gradient (added into d_grad and d_loss; loss =
 * (log1p(l) - log1p(count))^2 summed), and one Adam step on FP32 master
 * parameters that also refreshes their BF16 copy. */
gbr_status gbr_set_predictor(gbr_renderer *r, const uint16_t *weights_bf16, uint32_t num_params, float alpha,
                             float beta, float gamma);
/* The per-bin capacities the model predicted for the last frame rendered
 * with predicted binning (num_bins_x * num_bins_y values). */
gbr_status gbr_predicted_capacities(gbr_renderer *r, uint32_t *capacities, void *stream);
gbr_status gbr_collect_bin_features(gbr_renderer *r, const gbr_camera *cam, uint32_t cull, uint32_t sample,
                                    uint32_t vis, float *features, uint32_t *counts, void *stream);
uint32_t gbr_mlp_num_params(void);
gbr_status gbr_mlp_predict(const uint16_t *d_w, const float *d_x, uint32_t n, float *d_out, void *stream);
gbr_status gbr_mlp_loss_grad(const uint16_t *d_w, const float *d_x, const float *d_y, uint32_t n, float *d_grad,
                             float *d_loss, void *stream);
gbr_status gbr_mlp_adam(float *d_master, uint16_t *d_w, const float *d_grad, float *d_m, float *d_v, uint32_t step,
                        float lr, float grad_scale, void *stream);

/* Scene lights (SceneGraph::AddLight with DirectionalLight / PointLight,
 * SceneGraph.h, DirectionalLight.cpp, PointLight.cpp).  The reference's GPU
 * shader ignores the scene's lights and uses one constant light
 * (CUDAROPs.cu:417-420); that stays the behaviour with no lights set.  With
 * n > 0 lights the normal-mapped shading sums, per light, the shader's
 * Lambert (and, with specular and gloss maps, Phong) terms with L = the
 * direction the light travels at the shaded world point and irradiance =
 * colour x intensity (/ squared distance for a point light), plus the
 * shader's ambient and MaxToOne.  Up to 8 lights; n = 0 restores the
 * constant light. */
enum { GBR_LIGHT_DIRECTIONAL = 0, GBR_LIGHT_POINT = 1 };
typedef struct {
    uint32_t type;     /* GBR_LIGHT_* */
    float colour[3];
    float intensity;
    float vec[3];      /* directional: direction the light travels; point: world position */
} gbr_light;
gbr_status gbr_set_lights(gbr_renderer *r, const gbr_light *lights, uint32_t n);

/* Binning method for the following frames. */
gbr_status gbr_set_binning(gbr_renderer *r, uint32_t method);
/* Raster tuning (no counterpart in the reference; used by the autotuner):
 * phase = triangles rasterised between hierarchical-z refreshes, 0..128 (0: the library's choice: 16,
 * 64 for frames of small triangles, 128 with the raster's small-triangle variant),
 * ctas_per_sm = occupancy variant of the raster kernel, 2..6 (0: 6). */
gbr_status gbr_set_raster_params(gbr_renderer *r, uint32_t phase, uint32_t ctas_per_sm);
/* How the raster stages triangle-setup records into shared memory (no
 * counterpart in the reference, whose RA_PerTileKernel reads them from global
 * memory per pixel, CUDARenderer.cu:1039-1129): GBR_STAGING_LOADS (default),
 * 16-byte loads by the CTA's threads; GBR_STAGING_TMA, one 48-byte bulk
 * asynchronous copy (cp.async.bulk) per record completing on an mbarrier,
 * the next phase's records copied while the current one rasterises.  Both
 * give identical frames. */
enum { GBR_STAGING_LOADS = 0, GBR_STAGING_TMA = 1 };
gbr_status gbr_set_raster_staging(gbr_renderer *r, uint32_t mode);
/* A frame split across GPUs by bin rows (no counterpart in the reference,
 * which renders on one GPU, main.cpp:397-399): the following frames of this
 * renderer bin and rasterise only bin rows [row0, row1) -- triangles are set
 * up and binned as usual, their bin rectangles cut to those rows -- and shade
 * only the pixels of those rows; pixels of other rows are left as they were.
 * Each GPU renders its rows of the same scene and the rows are composited
 * (the bands are disjoint, so the composite equals the one-GPU frame).
 * (0, 0) restores every row; gbr_setup_bins also does. */
gbr_status gbr_set_bin_rows(gbr_renderer *r, uint32_t row0, uint32_t row1);
/* Test hook (no counterpart in the reference, whose spin locks wait without
 * a bound, CUDAAtomicQueue.cuh:8-26).  Every wait of the bin scan on another
 * tile is bounded; a wait that gives up flags the frame: the kernels after
 * the scan return without writing, and gbr_readback / gbr_get_stats /
 * gbr_get_bins return GBR_ERR_TIMEOUT for it.  spin_limit = polls of one flag
 * before a wait gives up (0: the library's bound, 2^22); silent_tile >= 0
 * makes that tile of 1024 bins publish nothing, so the tiles after it wait
 * until their bound runs out (-1: none).  Applies to the following frames. */
gbr_status gbr_set_scan_wait(gbr_renderer *r, uint32_t spin_limit, int32_t silent_tile);
/* Record CUDA-event times into gbr_stats (off by default).
 * GBR_TIMING_STAGES records an event between every stage, which also keeps
 * consecutive kernels from overlapping their launch; GBR_TIMING_TOTAL times
 * only the whole frame (ms_total; the stage times read 0). */
enum { GBR_TIMING_OFF = 0, GBR_TIMING_STAGES = 1, GBR_TIMING_TOTAL = 2 };
gbr_status gbr_set_timing(gbr_renderer *r, int mode);

/* EnterValidRenderingState + Render (CUDARenderer.cu:206-381): clears, runs
 * the whole frame on `stream` and returns without synchronising.  The
 * framebuffer holds RGBA::GetRGBAFromColour words (bytes B, G, R, 0). */
gbr_status gbr_render(gbr_renderer *r, const gbr_camera *cam, uint32_t cull, uint32_t sample,
                      uint32_t vis, void *stream);

/* Present (CUDARenderer.cu:383-395) without a window: waits for `stream`
 * and copies the framebuffer (and optionally the per-pixel interpolated
 * depth, 0 where no fragment landed) to host memory.  If the frame's bin
 * storage overflowed, the frame is re-rendered with exact storage first. */
gbr_status gbr_readback(gbr_renderer *r, uint32_t *colour, float *depth, void *stream);
/* Winning primitive id per pixel (0xFFFFFFFF where empty). */
gbr_status gbr_readback_ids(gbr_renderer *r, uint32_t *ids, void *stream);
/* Device addresses of the colour (uint32) and depth (float) buffers. */
gbr_status gbr_device_buffers(gbr_renderer *r, void **d_colour, void **d_depth);
/* Per-bin triangle lists of the last frame: offsets[num_bins+1] and
 * ids[capacity] (global primitive ids; order inside a bin unspecified).
 * *num_pairs gets the total; GBR_ERR_INVALID_ARG when capacity is short. */
gbr_status gbr_get_bins(gbr_renderer *r, uint32_t *offsets, uint32_t *ids, uint64_t capacity,
                        uint64_t *num_pairs, void *stream);
/* GetTotalNumVisibleTriangles / GetTotalNumTriangles and per-stage timers
 * (CUDARenderer.h:63-73); synchronises with `stream`. */
gbr_status gbr_get_stats(gbr_renderer *r, gbr_stats *out, void *stream);

/* Batched frames (no counterpart in the reference, whose Render() draws one
 * scene with one launch chain per mesh and per 256-triangle chunk,
 * CUDARenderer.cu:249-339).  A batch renders many renderers' scenes -- each
 * with its own resolution, meshes, textures, camera and render state -- as
 * one frame: six launches in total (reset, setup + count, per-scene scan,
 * fill, one persistent raster over the (scene, bin) work queue of every
 * scene, shade), replayed from a CUDA graph.  All scenes of a batch use the
 * batch's square bin size and queue chunk; each scene's output lands in its
 * renderer's frame buffers.  A renderer in a batch cannot be destroyed
 * until the batch is; its scene may change between batch frames. */
typedef struct gbr_batch gbr_batch;
typedef struct {
    uint32_t bin_size;     /* bins of bin_size x bin_size pixels, 1..64 */
    uint32_t queue_chunk;  /* entries depth-sorted and rasterised per pass over a tile, >= 1 (at most 2048
                              used); work items hold 2048 entries */
    uint32_t raster_ctas;  /* raster variant: CTAs per SM, 2..6 (0: 6), counted in CTAs of 256 threads */
    uint32_t raster_phase; /* triangles between hierarchical-z refreshes, 0..128 (0: 16) */
    uint32_t raster_threads; /* threads per bin: raster CTAs of 128 or 256 threads (0: 256); a 128-thread CTA
                                depth-sorts 1024 entries at a time into 128 buckets, and twice raster_ctas
                                of them are resident per SM */
} gbr_batch_config;
typedef struct {
    uint32_t num_scenes;
    uint32_t graph_captures;  /* CUDA graphs captured so far (layout or storage changes) */
    uint32_t overflow_reruns; /* batch frames re-rendered after outgrowing the bin storage */
    uint32_t pad;
    uint64_t num_triangles, num_visible, num_pairs, num_work_items;
    float ms_frame;           /* device time of the last batch frame (timing on) */
    float pad2;
} gbr_batch_stats;

gbr_status gbr_batch_create(gbr_batch **out);
gbr_status gbr_batch_destroy(gbr_batch *b);
/* Adds renderer r with the camera and render state it is drawn with;
 * *index numbers it in the batch. */
gbr_status gbr_batch_add(gbr_batch *b, gbr_renderer *r, const gbr_camera *cam, uint32_t cull, uint32_t sample,
                         uint32_t vis, uint32_t *index);
gbr_status gbr_batch_set_view(gbr_batch *b, uint32_t index, const gbr_camera *cam, uint32_t cull, uint32_t sample,
                              uint32_t vis);
gbr_status gbr_batch_set_config(gbr_batch *b, const gbr_batch_config *cfg);
gbr_status gbr_batch_get_config(const gbr_batch *b, gbr_batch_config *cfg);
/* Times `frames` batch frames (after one warm-up frame) for every
 * combination of the candidate bin sizes, queue chunks, raster variants
 * (CTAs per SM) and threads per bin (a NULL list keeps the current value)
 * and keeps the fastest; *best gets it.  Synchronises `stream`. */
gbr_status gbr_batch_autotune(gbr_batch *b, const uint32_t *bin_sizes, uint32_t num_bin_sizes, const uint32_t *chunks,
                              uint32_t num_chunks, const uint32_t *raster_ctas, uint32_t num_raster_ctas,
                              const uint32_t *raster_threads, uint32_t num_raster_threads, uint32_t frames,
                              void *stream, gbr_batch_config *best);
gbr_status gbr_batch_set_timing(gbr_batch *b, int enabled);
/* One batch frame on `stream`, without host synchronisation. */
gbr_status gbr_batch_render(gbr_batch *b, void *stream);
/* Synchronise `stream` (re-rendering the batch if it outgrew its bin
 * storage) and report the last batch frame. */
gbr_status gbr_batch_get_stats(gbr_batch *b, gbr_batch_stats *out, void *stream);
/* Bin grid of scene `index` under the current configuration. */
gbr_status gbr_batch_scene_bins(const gbr_batch *b, uint32_t index, uint32_t *num_bins_x, uint32_t *num_bins_y);
/* As gbr_readback / gbr_readback_ids / gbr_get_bins for scene `index` of the
 * last batch frame (any output pointer may be NULL). */
gbr_status gbr_batch_readback(gbr_batch *b, uint32_t index, uint32_t *colour, float *depth, uint32_t *ids,
                              void *stream);
/* The colour buffers of every scene of the last batch frame: colours[i]
 * (NULL: skipped) gets scene i's framebuffer; the copies are queued on
 * `stream` together and waited for once. */
gbr_status gbr_batch_readback_all(gbr_batch *b, uint32_t *const *colours, void *stream);
gbr_status gbr_batch_get_bins(gbr_batch *b, uint32_t index, uint32_t *offsets, uint32_t *ids, uint64_t capacity,
                              uint64_t *num_pairs, void *stream);

/* No counterpart in the reference.  Renders one frame of one mesh (vertex
 * colours; no textures) from device-resident vertices into caller-owned
 * device buffers (width*height colour words and depths, and the winning
 * primitive ids when d_ids is not NULL) without allocating any device
 * memory, for callers that may not allocate while they render:
 * hosts with a fixed device-memory budget that forbid library allocations,
 * real-time loops that cannot take cudaMalloc's implicit synchronisation,
 * processes under a hard memory cap.  Its scratch is one static device
 * array of about 20 MiB that every GPU loading the library holds until
 * exit.  Limits: <= 65536 triangles, <= 2^20 pixels, <= 4096 bins of
 * <= 64x64 px, queue_chunk >= 64, <= 2^20 (triangle, bin) entries; larger
 * inputs return GBR_ERR_INVALID_ARG (or GBR_ERR_OUT_OF_MEMORY for the
 * entry count, found after the frame).  The first call on a device sets up
 * its scratch address and should come before any stream capture.  Calls
 * share the scratch: calls whose GPU work overlaps race.  Returns after
 * synchronising `stream`.  d_indices (NULL for a non-indexed list) stays on
 * the device and is not range-checked: every index must be below
 * num_vertices. */
gbr_status gbr_render_noalloc(const void *d_vertices, uint32_t num_vertices, uint32_t vertex_format,
                              const uint32_t *d_indices, uint32_t num_indices, uint32_t topology,
                              const float world[16], const gbr_camera *cam, uint32_t width, uint32_t height,
                              uint32_t num_bins_x, uint32_t num_bins_y, uint32_t bin_w, uint32_t bin_h,
                              uint32_t queue_chunk, uint32_t cull, uint32_t sample, uint32_t vis,
                              uint32_t *d_colour, float *d_depth, uint32_t *d_ids, void *stream);

const char *gbr_last_error_string(void);
/* Library version, e.g. 0x000100 for 0.1.0. */
uint32_t gbr_version(void);

#ifdef __cplusplus
}
#endif
#endif
