/*
 * gbr_oracle.h -- CPU oracle for the frame hot path of Custom-CUDA-Rasterizer.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a sequential (optionally multi-threaded
 * over bins) plain-C restatement of the reference's GPU pipeline:
 *   VS_Kernel -> TA_Kernel -> TB_Kernel -> RA_PerTileKernel -> PS_Kernel
 * (CustomCUDARasterizer/CUDARenderer.cu, CUDAROPs.cu, CUDATextureSampler.cuh).
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline may load
 * it, and only as the checker.  The product path never calls it.
 *
 * Float semantics: compile with -ffp-contract=off.  Every place where the
 * reference's nvcc build contracts a*b+c into one fused multiply-add is
 * written as an explicit fmaf() here, so that the oracle reproduces the
 * GPU's roundings instead of the host compiler's.
 */
#ifndef GBR_ORACLE_H
#define GBR_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* vertex formats */
#define ORC_VERTEX_IVERTEX56   0u  /* reference IVertex: p3 uv2 n3 tan3 c3 (floats), 56 B */
#define ORC_VERTEX_POS3_RGBA8  1u  /* compact soup vertex: p3 (floats) + RGBA8, 16 B */

/* raster modes */
#define ORC_RASTER_REFERENCE   0u  /* float edge functions at integer pixels (CUDAROPs.cu:128-145) */
#define ORC_RASTER_FIXED       1u  /* the GB300 build's 16.16 fixed-point edge functions */

/* Scene lights (the build's extension; the reference's GPU shader has one
 * constant light, CUDAROPs.cu:417-420).  Light colour x intensity as
 * DirectionalLight::GetBiradiance, / squared distance for a point light as
 * PointLight::GetBiradiance (DirectionalLight.cpp, PointLight.cpp). */
#define ORC_MAX_LIGHTS         8u
#define ORC_LIGHT_DIRECTIONAL  0u  /* vec = direction the light travels */
#define ORC_LIGHT_POINT        1u  /* vec = world position */
typedef struct {
    uint32_t type;
    float colour[3];
    float intensity;
    float vec[3];
} orc_light;

typedef struct {
    uint32_t width, height;
    uint32_t num_bins_x, num_bins_y, bin_w, bin_h;
    uint32_t cull;          /* 0 BackFace, 1 FrontFace, 2 NoCulling */
    uint32_t sample;        /* 0 Point, 1 Linear, 2 Bilinear (the build's extension) */
    uint32_t vis;           /* 0 PBR, 1 Depth, 2 Normal */
    uint32_t raster_mode;   /* ORC_RASTER_* */
    uint32_t clear_colour32;
    uint32_t num_threads;   /* 0 or 1: single thread */
    uint32_t bin_stride;    /* rasterise only bins b with b % bin_stride == bin_phase (0: all) */
    uint32_t bin_phase;
    float cam_pos[3];
    float cam_fwd[3];
    float view[16];         /* column-major, element (r,c) at [c*4+r] */
    float proj[16];
    uint32_t num_lights;    /* 0: the reference shader's constant light */
    orc_light lights[ORC_MAX_LIGHTS];
    uint32_t bin_row0;      /* rasterise only bin rows [bin_row0, bin_row1) (bin_row1 0: all): one */
    uint32_t bin_row1;      /* GPU's band of a frame split across GPUs by bin rows */
} orc_frame;

typedef struct {
    const void *vertices;
    uint32_t num_vertices;
    uint32_t vertex_format;
    const uint32_t *indices;   /* NULL: non-indexed, vertex i of triangle t is 3t+i */
    uint32_t num_indices;
    uint32_t topology;         /* 0 TriangleList, 1 TriangleStrip */
    float world[16];
    const uint32_t *tex[4];    /* Diffuse, Normal, Specular, Glossiness; NULL = unbound */
    uint32_t tex_w[4];
    uint32_t tex_h[4];
} orc_mesh;

typedef struct {
    uint64_t num_triangles;
    uint64_t num_visible;      /* survived cull + frustum reject */
    uint64_t num_pairs;        /* (triangle, bin) pairs */
    uint64_t num_float_path;   /* visible triangles outside the fixed-point guard band */
    uint64_t fragments;        /* covered pixels that passed the z range test */
    uint64_t covered_pixels;   /* pixels with a winning fragment */
} orc_stats;

typedef struct {
    int32_t covered_ref;       /* float edge test (reference) */
    int32_t covered_fixed;     /* 16.16 fixed-point edge test */
    float e_ref[3];            /* reference float edge values (weights before /area) */
    float e_bound[3];          /* bound on |e_ref - e_exact| from snapping + float rounding */
    float z_ref;               /* interpolated z, reference weights */
    float z_fixed;             /* interpolated z, fixed-point weights */
    int32_t visible;           /* triangle survived cull + frustum */
    int32_t float_path;
} orc_probe_out;

/* Render one frame.  Output buffers are W*H; any may be NULL.  ids gets the
 * winning global primitive id per pixel (0xFFFFFFFF where empty).  depth gets
 * the winning fragment's interpolated z (0 where empty, as the reference's
 * cleared PixelShade buffer).  Bin lists: bin_offsets[numBins+1] and
 * bin_ids[bin_capacity], each bin ascending by primitive id.  Returns 0 on
 * success, 1 bad argument, 2 bin_capacity too small (offsets still written),
 * 3 out of memory. */
int orc_render(const orc_frame *f, const orc_mesh *meshes, uint32_t num_meshes,
               uint32_t *colour, float *depth, uint32_t *ids,
               uint32_t *bin_offsets, uint32_t *bin_ids, uint64_t bin_capacity,
               orc_stats *stats);

/* Coverage and depth of one primitive at one pixel, in both raster modes. */
int orc_probe(const orc_frame *f, const orc_mesh *meshes, uint32_t num_meshes,
              uint32_t prim, uint32_t px, uint32_t py, orc_probe_out *out);

/* Single-function entry points for known-answer tests. */
void orc_vs_position(const float *wvp, const float *p, float *out_clip);
void orc_mat4_mul(const float *lm, const float *rm, float *out);
int  orc_cull(const float *p0, const float *p1, const float *p2, const float *cam_fwd, uint32_t cull);
int  orc_frustum_visible(const float *p0, const float *p1, const float *p2);
void orc_bin_rect(const float *ndc_xy, uint32_t width, uint32_t height,
                  uint32_t nbx, uint32_t nby, uint32_t bw, uint32_t bh, int32_t *out_rect);
void orc_sample(const uint32_t *pixels, uint32_t w, uint32_t h, float u, float v,
                uint32_t sample, float *out_rgb);
uint32_t orc_rgba_from_colour(const float *rgb);
void orc_camera(const float *pos, float fov_deg, float aspect_w, float aspect_h,
                float near_z, float far_z, float *out_view, float *out_proj,
                float *out_fwd);

#ifdef __cplusplus
}
#endif
#endif
