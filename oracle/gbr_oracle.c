/*
 * gbr_oracle.c -- CPU oracle (test infrastructure) for the frame hot path of
 * Custom-CUDA-Rasterizer.  See gbr_oracle.h.  Each function names the
 * reference file:line it restates (paths inside CustomCUDARasterizer/).
 *
 * Build: gcc -O2 -std=c11 -ffp-contract=off -fPIC -shared -pthread -lm
 * (oracle/build_oracle.py).  -ffp-contract=off is required: the fused
 * multiply-adds the reference's nvcc build forms are spelled out as fmaf().
 *
 * Contraction model.  nvcc fuses `a*b + c*d` into fma(a, b, c*d) (the left
 * product is fused), `s + a*b` into fma(a, b, s), and `a*b - c*d` into
 * fma(a, b, -(c*d)).  A chain `a*b + c*d + e*f + g` becomes
 * fma(e, f, fma(a, b, c*d)) + g.  The oracle follows that model everywhere a
 * rounding can change a discrete decision (cull, bins, coverage, texel).
 */
#define _GNU_SOURCE
#include "gbr_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#define INV_PRIM 0xFFFFFFFFu
#define FX_BITS 16
#define FX_ONE (1 << FX_BITS)
#define GUARD_PX 8192.0f

typedef struct { float x, y, z; } v3;
typedef struct { float x, y; } v2;

/* ------------------------------------------------------------------ */
/* Conversions with PTX semantics: float->int saturates, NaN -> 0.     */
/* (the reference relies on nvcc's cvt.rzi.* for (int), (short), u8)   */
/* ------------------------------------------------------------------ */
static int32_t cvt_s32(float x)
{
    if (x != x) return 0;
    if (x >= 2147483648.0f) return 2147483647;
    if (x <= -2147483648.0f) return (int32_t)0x80000000u;
    return (int32_t)x;
}

static int16_t cvt_s16(float x)
{
    if (x != x) return 0;
    if (x >= 32767.0f) return 32767;
    if (x <= -32768.0f) return -32768;
    return (int16_t)(int32_t)x;
}

static uint8_t cvt_u8(float x)
{
    if (!(x > 0.0f)) return 0;     /* negative and NaN */
    if (x >= 255.0f) return 255;
    return (uint8_t)(int32_t)x;
}

/* Matrix element (r, c) of a column-major matrix stored data[c][r]
 * (Matrix.h:9-21). */
#define M4(m, r, c) ((m)[(c) * 4 + (r)])

/* Matrix<4,4>::operator*(Matrix) on the host (Matrix4.h:120-143); the
 * reference computes WVP on the CPU (CUDARenderer.cu:219,242), no fusion. */
void orc_mat4_mul(const float *lm, const float *rm, float *out)
{
    float t[16];
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) {
            float s = M4(lm, r, 0) * M4(rm, 0, c);
            s = s + M4(lm, r, 1) * M4(rm, 1, c);
            s = s + M4(lm, r, 2) * M4(rm, 2, c);
            s = s + M4(lm, r, 3) * M4(rm, 3, c);
            M4(t, r, c) = s;
        }
    memcpy(out, t, sizeof t);
}

/* Matrix<4,4>::operator*(Point4) with w=1 (Matrix4.h:158-166), as fused by
 * nvcc in VS_Kernel -> GetNDCVertex (CUDAROPs.cu:103). */
void orc_vs_position(const float *m, const float *p, float *out)
{
    for (int r = 0; r < 4; ++r)
        out[r] = fmaf(M4(m, r, 2), p[2], fmaf(M4(m, r, 0), p[0], M4(m, r, 1) * p[1])) + M4(m, r, 3);
}

/* Matrix<3,3> * Vector3 (Matrix3.h:126-133) for the upper 3x3 of a 4x4. */
static v3 rot3(const float *m, v3 v)
{
    v3 o;
    o.x = fmaf(M4(m, 0, 2), v.z, fmaf(M4(m, 0, 0), v.x, M4(m, 0, 1) * v.y));
    o.y = fmaf(M4(m, 1, 2), v.z, fmaf(M4(m, 1, 0), v.x, M4(m, 1, 1) * v.y));
    o.z = fmaf(M4(m, 2, 2), v.z, fmaf(M4(m, 2, 0), v.x, M4(m, 2, 1) * v.y));
    return o;
}

static float dot3(v3 a, v3 b) { return fmaf(a.z, b.z, fmaf(a.x, b.x, a.y * b.y)); }

static v3 cross3(v3 a, v3 b)
{
    v3 o;
    o.x = fmaf(a.y, b.z, -(a.z * b.y));
    o.y = fmaf(a.z, b.x, -(a.x * b.z));
    o.z = fmaf(a.x, b.y, -(a.y * b.x));
    return o;
}

/* Normalize (Vector.h:41-56): zero vector when the magnitude is 0. */
static v3 normalize3(v3 v)
{
    const float m = sqrtf(dot3(v, v));
    if (m == 0.0f) { v3 z = {0.f, 0.f, 0.f}; return z; }
    const float inv = 1.0f / m;
    v3 o = {v.x * inv, v.y * inv, v.z * inv};
    return o;
}

static v3 sub3(v3 a, v3 b) { v3 o = {a.x - b.x, a.y - b.y, a.z - b.z}; return o; }

/* ------------------------------------------------------------------ */
/* Camera (Camera.cpp:6-36, 97-108; Camera.h:26; Matrix4.h:329-361)    */
/* ------------------------------------------------------------------ */
static void inverse4(const float *m, float *out)
{
    /* FGED1 inverse as in Matrix4.h:329-361, host arithmetic */
    const v3 a = {M4(m, 0, 0), M4(m, 1, 0), M4(m, 2, 0)};
    const v3 b = {M4(m, 0, 1), M4(m, 1, 1), M4(m, 2, 1)};
    const v3 c = {M4(m, 0, 2), M4(m, 1, 2), M4(m, 2, 2)};
    const v3 d = {M4(m, 0, 3), M4(m, 1, 3), M4(m, 2, 3)};
    const float x = M4(m, 3, 0), y = M4(m, 3, 1), z = M4(m, 3, 2), w = M4(m, 3, 3);
#define HCROSS(p, q) ((v3){(p).y * (q).z - (p).z * (q).y, (p).z * (q).x - (p).x * (q).z, (p).x * (q).y - (p).y * (q).x})
#define HDOT(p, q) ((p).x * (q).x + (p).y * (q).y + (p).z * (q).z)
    v3 s = HCROSS(a, b), t = HCROSS(c, d);
    v3 u = {a.x * y - b.x * x, a.y * y - b.y * x, a.z * y - b.z * x};
    v3 v = {c.x * w - d.x * z, c.y * w - d.y * z, c.z * w - d.z * z};
    const float det = HDOT(s, v) + HDOT(t, u);
    const float inv = 1.0f / det;
    s.x *= inv; s.y *= inv; s.z *= inv;
    t.x *= inv; t.y *= inv; t.z *= inv;
    u.x *= inv; u.y *= inv; u.z *= inv;
    v.x *= inv; v.y *= inv; v.z *= inv;
    v3 bv = HCROSS(b, v), va = HCROSS(v, a), du = HCROSS(d, u), uc = HCROSS(u, c);
    v3 r0 = {bv.x + t.x * y, bv.y + t.y * y, bv.z + t.z * y};
    v3 r1 = {va.x - t.x * x, va.y - t.y * x, va.z - t.z * x};
    v3 r2 = {du.x + s.x * w, du.y + s.y * w, du.z + s.z * w};
    v3 r3 = {uc.x - s.x * z, uc.y - s.y * z, uc.z - s.z * z};
    /* constructor takes rows (Matrix4.h:23-32) */
    const float rows[4][4] = {
        {r0.x, r0.y, r0.z, -HDOT(b, t)},
        {r1.x, r1.y, r1.z, HDOT(a, t)},
        {r2.x, r2.y, r2.z, -HDOT(d, s)},
        {r3.x, r3.y, r3.z, HDOT(c, s)}};
#undef HCROSS
#undef HDOT
    for (int r = 0; r < 4; ++r)
        for (int cc = 0; cc < 4; ++cc) M4(out, r, cc) = rows[r][cc];
}

void orc_camera(const float *pos, float fov_deg, float aspect_w, float aspect_h,
                float near_z, float far_z, float *view, float *proj, float *fwd)
{
    float look[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
    look[12] = pos[0]; look[13] = pos[1]; look[14] = pos[2];
    inverse4(look, view);
    const float radians = fov_deg * ((float)3.14159265358979323846 / 180.f);
    const float fov = tanf(radians / 2.f);
    const float aspect = aspect_w / aspect_h;
    const float A = far_z / (near_z - far_z);
    const float B = (far_z * near_z) / (near_z - far_z);
    for (int i = 0; i < 16; ++i) proj[i] = (i % 5 == 0) ? 1.f : 0.f;
    proj[0 * 4 + 0] = 1.f / (aspect * fov);
    proj[1 * 4 + 1] = 1.f / fov;
    proj[2 * 4 + 2] = A;
    proj[2 * 4 + 3] = -1.f;
    proj[3 * 4 + 2] = B;
    proj[3 * 4 + 3] = 1.f;  /* identity start (Camera.cpp:23) leaves data[3][3] = 1 */
    fwd[0] = look[8]; fwd[1] = look[9]; fwd[2] = look[10];
}

/* ------------------------------------------------------------------ */
/* Vertex fetch and VS (VS_Kernel CUDARenderer.cu:673-700,              */
/* GetNDCVertex CUDAROPs.cu:99-118)                                     */
/* ------------------------------------------------------------------ */
typedef struct {
    float p[4];        /* NDC xyz, clip w */
    v2 uv;
    v3 n, tan, vd, c;
    v3 wp;             /* world position (scene lights) */
} overtex;

typedef struct {
    const orc_mesh *m;
    float wvp[16];
    uint64_t prim_base;
    uint64_t num_tris;
} mesh_state;

static void fetch_ivertex(const orc_mesh *m, uint32_t i, float *out14)
{
    if (m->vertex_format == ORC_VERTEX_IVERTEX56) {
        memcpy(out14, (const char *)m->vertices + (size_t)i * 56u, 56);
    } else {
        const char *base = (const char *)m->vertices + (size_t)i * 16u;
        float p[3];
        uint32_t rgba;
        memcpy(p, base, 12);
        memcpy(&rgba, base + 12, 4);
        out14[0] = p[0]; out14[1] = p[1]; out14[2] = p[2];
        for (int k = 3; k < 11; ++k) out14[k] = 0.f;
        /* RGBA8 -> RGBColor as GetRGBColor (RGBRaw.h:34-38): r = byte0/255 */
        out14[11] = (float)(rgba & 0xFFu) / 255.f;
        out14[12] = (float)((rgba >> 8) & 0xFFu) / 255.f;
        out14[13] = (float)((rgba >> 16) & 0xFFu) / 255.f;
    }
}

static void vs_full(const mesh_state *ms, const orc_frame *f, uint32_t vi, overtex *o)
{
    float iv[14];
    fetch_ivertex(ms->m, vi, iv);
    float clip[4];
    orc_vs_position(ms->wvp, iv, clip);
    o->p[0] = clip[0] / clip[3];
    o->p[1] = clip[1] / clip[3];
    o->p[2] = clip[2] / clip[3];
    o->p[3] = clip[3];
    const v3 n = {iv[5], iv[6], iv[7]}, t = {iv[8], iv[9], iv[10]};
    o->n = rot3(ms->m->world, n);
    o->tan = rot3(ms->m->world, t);
    float wp[4];
    orc_vs_position(ms->m->world, iv, wp);
    const v3 wpos = {wp[0], wp[1], wp[2]}, cp = {f->cam_pos[0], f->cam_pos[1], f->cam_pos[2]};
    o->vd = normalize3(sub3(wpos, cp));
    o->wp = wpos;
    o->uv.x = iv[3]; o->uv.y = iv[4];
    o->c.x = iv[11]; o->c.y = iv[12]; o->c.z = iv[13];
}

static void vs_ndc(const mesh_state *ms, uint32_t vi, float out[4])
{
    float iv[14];
    fetch_ivertex(ms->m, vi, iv);
    float clip[4];
    orc_vs_position(ms->wvp, iv, clip);
    out[0] = clip[0] / clip[3];
    out[1] = clip[1] / clip[3];
    out[2] = clip[2] / clip[3];
    out[3] = clip[3];
}

/* Triangle assembly (TA_Kernel CUDARenderer.cu:716-753).  The strip path of
 * the reference reads an uninitialised triangle (the inner declaration at
 * :737 shadows :716); the oracle implements the intended strip order. */
static void tri_indices(const orc_mesh *m, uint64_t t, uint32_t idx[3])
{
    if (!m->indices) {
        idx[0] = (uint32_t)(3 * t); idx[1] = (uint32_t)(3 * t + 1); idx[2] = (uint32_t)(3 * t + 2);
        return;
    }
    if (m->topology == 0) {
        idx[0] = m->indices[3 * t]; idx[1] = m->indices[3 * t + 1]; idx[2] = m->indices[3 * t + 2];
    } else {
        idx[0] = m->indices[t]; idx[1] = m->indices[t + 1]; idx[2] = m->indices[t + 2];
        if (t & 1) { uint32_t s = idx[1]; idx[1] = idx[2]; idx[2] = s; }
    }
}

static uint64_t mesh_num_tris(const orc_mesh *m)
{
    if (!m->indices) return m->num_vertices / 3u;
    if (m->topology == 0) return m->num_indices / 3u;
    return m->num_indices >= 2 ? m->num_indices - 2u : 0u;
}

/* Culling (TA_Kernel CUDARenderer.cu:759-777).  BackFace and FrontFace run
 * the same test in the reference. */
int orc_cull(const float *p0, const float *p1, const float *p2, const float *fwd, uint32_t cull)
{
    if (cull == 2u) return 0;
    const v3 a = {p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2]};
    const v3 b = {p2[0] - p0[0], p2[1] - p0[1], p2[2] - p0[2]};
    const v3 n = normalize3(cross3(a, b));
    const v3 cf = {fwd[0], fwd[1], fwd[2]};
    return dot3(cf, n) <= 0.0f;
}

/* IsTriangleVisible (CUDAROPs.cu:147-178). */
int orc_frustum_visible(const float *v0, const float *v1, const float *v2)
{
    const int ax = (v0[0] < -1.f && v1[0] < -1.f && v2[0] < -1.f) || (v0[0] > 1.f && v1[0] > 1.f && v2[0] > 1.f);
    const int ay = (v0[1] < -1.f && v1[1] < -1.f && v2[1] < -1.f) || (v0[1] > 1.f && v1[1] > 1.f && v2[1] > 1.f);
    const int az = (v0[2] < 0.f && v1[2] < 0.f && v2[2] < 0.f) || (v0[2] > 1.f && v1[2] > 1.f && v2[2] > 1.f);
    return !ax && !ay && !az;
}

/* NDCToScreenSpace (CUDAROPs.cu:88-97). */
static v2 to_screen(float x, float y, uint32_t w, uint32_t h)
{
    v2 s;
    s.x = ((x + 1.f) / 2.f) * (float)w;
    s.y = ((1.f - y) / 2.f) * (float)h;
    return s;
}

static float min3f(float a, float b, float c)
{
    float m = a;
    if (b < m) m = b;
    if (c < m) m = c;
    return m;
}

static float max3f(float a, float b, float c)
{
    float m = a;
    if (b > m) m = b;
    if (c > m) m = c;
    return m;
}

static int16_t clamp_s16(int16_t v, int16_t lo, int16_t hi)
{
    const int16_t c = v < lo ? lo : v;
    return c > hi ? hi : c;
}

static int32_t clamp_i32(int32_t v, int32_t lo, int32_t hi)
{
    const int32_t c = v < lo ? lo : v;
    return c > hi ? hi : c;
}

/* GetBoundingBox (CUDAROPs.cu:180-200) + TB_Kernel bin range
 * (CUDARenderer.cu:932-942).  rect = {binMinX, binMinY, binMaxX, binMaxY};
 * empty when min > max. */
static void bin_rect_screen(v2 s0, v2 s1, v2 s2, uint32_t width, uint32_t height,
                            uint32_t nbx, uint32_t nby, uint32_t bw, uint32_t bh, int32_t *rect)
{
    int16_t xmin = (int16_t)(cvt_s16(min3f(s0.x, s1.x, s2.x)) - 1);
    int16_t ymin = (int16_t)(cvt_s16(min3f(s0.y, s1.y, s2.y)) - 1);
    int16_t xmax = (int16_t)(cvt_s16(max3f(s0.x, s1.x, s2.x)) + 1);
    int16_t ymax = (int16_t)(cvt_s16(max3f(s0.y, s1.y, s2.y)) + 1);
    xmin = clamp_s16(xmin, 0, (int16_t)width);
    ymin = clamp_s16(ymin, 0, (int16_t)height);
    xmax = clamp_s16(xmax, 0, (int16_t)width);
    ymax = clamp_s16(ymax, 0, (int16_t)height);
    rect[0] = clamp_i32((int32_t)xmin / (int32_t)bw, 0, (int32_t)nbx);
    rect[1] = clamp_i32((int32_t)ymin / (int32_t)bh, 0, (int32_t)nby);
    rect[2] = clamp_i32((int32_t)xmax / (int32_t)bw, 0, (int32_t)nbx - 1);
    rect[3] = clamp_i32((int32_t)ymax / (int32_t)bh, 0, (int32_t)nby - 1);
}

void orc_bin_rect(const float *ndc_xy, uint32_t width, uint32_t height,
                  uint32_t nbx, uint32_t nby, uint32_t bw, uint32_t bh, int32_t *rect)
{
    bin_rect_screen(to_screen(ndc_xy[0], ndc_xy[1], width, height),
                    to_screen(ndc_xy[2], ndc_xy[3], width, height),
                    to_screen(ndc_xy[4], ndc_xy[5], width, height),
                    width, height, nbx, nby, bw, bh, rect);
}

/* ------------------------------------------------------------------ */
/* Per-triangle raster setup                                           */
/* ------------------------------------------------------------------ */
typedef struct {
    v2 s[3];            /* float screen coords */
    float z[3];         /* NDC z */
    int32_t X[3], Y[3]; /* 16.16 snapped */
    int64_t area_fx;    /* exact double area of the snapped triangle, 2^-32 px^2 */
    float inv_area_ref; /* 1 / |cross(v0-v1, v0-v2)| of the float screen triangle */
    int visible;
    int float_path;
    int coverable_fx;
    uint32_t mesh;
    uint32_t vidx[3];
} tri_setup;

static int in_guard(v2 s)
{
    return s.x > -GUARD_PX && s.x < GUARD_PX && s.y > -GUARD_PX && s.y < GUARD_PX;
}

static int32_t snap(float v) { return (int32_t)lrintf(v * (float)FX_ONE); }

static void setup_fixed(tri_setup *t)
{
    t->float_path = !(in_guard(t->s[0]) && in_guard(t->s[1]) && in_guard(t->s[2]));
    t->coverable_fx = 0;
    t->area_fx = 0;
    t->inv_area_ref = 0.f;
    if (t->float_path) return;
    for (int i = 0; i < 3; ++i) { t->X[i] = snap(t->s[i].x); t->Y[i] = snap(t->s[i].y); }
    /* S = E(v0; v1, v2) = cross(v0 - v1, v2 - v1); equals |cross(v0-v1, v0-v2)|
     * when the triangle has the covered winding */
    const int64_t S = (int64_t)(t->X[0] - t->X[1]) * (int64_t)(t->Y[2] - t->Y[1]) -
                      (int64_t)(t->Y[0] - t->Y[1]) * (int64_t)(t->X[2] - t->X[1]);
    t->area_fx = S;
    /* the float area the reference divides by (CUDAROPs.cu:336); a triangle
     * whose float area is 0 would give NaN weights and is not rasterised */
    const v2 a = {t->s[0].x - t->s[1].x, t->s[0].y - t->s[1].y};
    const v2 b = {t->s[0].x - t->s[2].x, t->s[0].y - t->s[2].y};
    const float area = fabsf(fmaf(a.x, b.y, -(a.y * b.x)));
    if (S > 0 && area > 0.f) {
        t->coverable_fx = 1;
        t->inv_area_ref = 1.0f / area;
    }
}

/* Exact 16.16 edge function E(P; A, B) = (P-A) x (B-A) in 2^-32 px^2. */
static int64_t edge_fx(int32_t px, int32_t py, int32_t ax, int32_t ay, int32_t bx, int32_t by)
{
    const int64_t dx = (int64_t)(px * FX_ONE) - ax;
    const int64_t dy = (int64_t)(py * FX_ONE) - ay;
    return dx * (int64_t)(by - ay) - dy * (int64_t)(bx - ax);
}

/* The reference's float edge functions at a pixel, weights order as
 * IsPixelInTriangle (CUDAROPs.cu:120-142): w[2] from edge v0->v1, w[0] from
 * v1->v2, w[1] from v2->v0. */
static void edges_ref(const tri_setup *t, float px, float py, float w[3])
{
    const v2 v0 = t->s[0], v1 = t->s[1], v2_ = t->s[2];
    const v2 ea = {v1.x - v0.x, v1.y - v0.y};
    const v2 eb = {v2_.x - v1.x, v2_.y - v1.y};
    const v2 ec = {v0.x - v2_.x, v0.y - v2_.y};
    w[2] = fmaf(px - v0.x, ea.y, -((py - v0.y) * ea.x));
    w[0] = fmaf(px - v1.x, eb.y, -((py - v1.y) * eb.x));
    w[1] = fmaf(px - v2_.x, ec.y, -((py - v2_.y) * ec.x));
}

/* Fixed-point coverage (exact int64 edge functions of the 16.16 snapped
 * triangle, inclusive); the interpolation weights are the reference's float
 * edge values times 1/area, so depth and attributes follow the unsnapped
 * triangle. */
static int cover_fixed(const tri_setup *t, int32_t px, int32_t py, float w[3])
{
    const int64_t e2 = edge_fx(px, py, t->X[0], t->Y[0], t->X[1], t->Y[1]);
    const int64_t e0 = edge_fx(px, py, t->X[1], t->Y[1], t->X[2], t->Y[2]);
    const int64_t e1 = edge_fx(px, py, t->X[2], t->Y[2], t->X[0], t->Y[0]);
    if (e0 < 0 || e1 < 0 || e2 < 0) return 0;
    edges_ref(t, (float)px, (float)py, w);
    w[0] = w[0] * t->inv_area_ref;
    w[1] = w[1] * t->inv_area_ref;
    w[2] = w[2] * t->inv_area_ref;
    return 1;
}

/* Float coverage, IsPixelInTriangle + weight normalisation
 * (CUDAROPs.cu:120-145, 334-339). */
static int cover_ref(const tri_setup *t, float px, float py, float w[3], float eraw[3])
{
    const v2 v0 = t->s[0], v1 = t->s[1], v2_ = t->s[2];
    edges_ref(t, px, py, w);
    if (eraw) { eraw[0] = w[0]; eraw[1] = w[1]; eraw[2] = w[2]; }
    if (!(w[0] >= 0.f && w[1] >= 0.f && w[2] >= 0.f)) return 0;
    const v2 a = {v0.x - v1.x, v0.y - v1.y}, b = {v0.x - v2_.x, v0.y - v2_.y};
    const float area = fabsf(fmaf(a.x, b.y, -(a.y * b.x)));
    w[0] /= area; w[1] /= area; w[2] /= area;
    return 1;
}

/* z = sum w_i z_i (CUDAROPs.cu:341), shared by both modes. */
static float interp_z(const float w[3], const float z[3])
{
    return fmaf(w[2], z[2], fmaf(w[0], z[0], w[1] * z[1]));
}

/* Coverage + z for one pixel in the frame's raster mode.  Returns 1 and the
 * depth key when the fragment passes the early z test (CUDAROPs.cu:343-345,
 * 385-386). */
static int fragment(const tri_setup *t, uint32_t mode, int32_t px, int32_t py, float w[3],
                    float *z_out, int32_t *key)
{
    int cov;
    if (mode == ORC_RASTER_FIXED && !t->float_path) {
        if (!t->coverable_fx) return 0;
        cov = cover_fixed(t, px, py, w);
    } else {
        cov = cover_ref(t, (float)px, (float)py, w, NULL);
    }
    if (!cov) return 0;
    const float z = interp_z(w, t->z);
    if (z < 0.f || z > 1.f) return 0;
    *z_out = z;
    *key = cvt_s32(z * 2147483648.0f);  /* (int)(z * INT_MAX), INT_MAX -> 2^31 as float */
    return 1;
}

/* ------------------------------------------------------------------ */
/* Sampling (CUDATextureSampler.cuh:87-190) and shading                */
/* (CUDAROPs.cu:411-470, CUDARenderer.cu:833-897)                       */
/* ------------------------------------------------------------------ */
static v3 rgb_of(uint32_t c)
{
    v3 o = {(float)(c & 0xFFu) / 255.f, (float)((c >> 8) & 0xFFu) / 255.f, (float)((c >> 16) & 0xFFu) / 255.f};
    return o;
}

static v3 sample_point(const uint32_t *px, uint32_t w, uint32_t h, v2 uv)
{
    const int u = cvt_s32(fmaf(uv.x, (float)w, 0.5f));
    const int v = cvt_s32(fmaf(uv.y, (float)h, 0.5f));
    if (u < 0 || v < 0 || (uint32_t)u >= w || (uint32_t)v >= h) { v3 m = {1.f, 0.f, 1.f}; return m; }
    return rgb_of(px[(uint32_t)u + (uint32_t)v * w]);
}

static v3 sample_linear(const uint32_t *px, uint32_t w, uint32_t h, v2 uv)
{
    const int x = cvt_s32(fmaf(uv.x, (float)w, 0.5f));
    const int y = cvt_s32(fmaf(uv.y, (float)h, 0.5f));
    if (x < 0 || y < 0 || (uint32_t)x >= w || (uint32_t)y >= h) { v3 m = {1.f, 0.f, 1.f}; return m; }
    const int size = (int)(w * h);
    const int o = x + y * (int)w;
    int nb[4];
    nb[0] = o - 1; if (nb[0] < 0) nb[0] = o;
    nb[1] = o + 1; if (nb[1] >= size) nb[1] = o;
    nb[2] = o + (int)w; if (nb[2] >= size) nb[2] = o;
    nb[3] = o - (int)w; if (nb[3] < 0) nb[3] = o;
    const float wt = 1.f / 8.f;
    float r = 0.f, g = 0.f, b = 0.f;
    for (int i = 0; i < 4; ++i) {
        const uint32_t c = px[nb[i]];
        r = fmaf((float)(c & 0xFFu), wt, r);
        g = fmaf((float)((c >> 8) & 0xFFu), wt, g);
        b = fmaf((float)((c >> 16) & 0xFFu), wt, b);
    }
    const uint32_t c = px[o];
    r = r + (float)(c & 0xFFu) / 2.f;
    g = g + (float)((c >> 8) & 0xFFu) / 2.f;
    b = b + (float)((c >> 16) & 0xFFu) / 2.f;
    const float rev = 1.0f / 255.f;
    v3 out = {r * rev, g * rev, b * rev};
    return out;
}

/* Bilinear filtering (the build's extension; the reference's "linear"
 * sampler is the 5-tap filter above): texel centres at (i + 1/2) / size,
 * the four nearest texels weighted by the fractional offsets, addresses
 * clamped to the texture. */
static v3 sample_bilinear(const uint32_t *px, uint32_t w, uint32_t h, v2 uv)
{
    const float x = fmaf(uv.x, (float)w, -0.5f), y = fmaf(uv.y, (float)h, -0.5f);
    const float fx = floorf(x), fy = floorf(y);
    const float ax = x - fx, ay = y - fy;
    int xi = cvt_s32(fx), yi = cvt_s32(fy);
    xi = xi < -1 ? -1 : (xi > (int)w - 1 ? (int)w - 1 : xi);
    yi = yi < -1 ? -1 : (yi > (int)h - 1 ? (int)h - 1 : yi);
    const uint32_t x0 = (uint32_t)(xi < 0 ? 0 : xi), x1 = (uint32_t)(xi + 1 > (int)w - 1 ? (int)w - 1 : xi + 1);
    const uint32_t y0 = (uint32_t)(yi < 0 ? 0 : yi), y1 = (uint32_t)(yi + 1 > (int)h - 1 ? (int)h - 1 : yi + 1);
    const uint32_t c00 = px[x0 + y0 * w], c10 = px[x1 + y0 * w], c01 = px[x0 + y1 * w], c11 = px[x1 + y1 * w];
    float out[3];
    for (int k = 0; k < 3; ++k) {
        const float a = (float)((c00 >> (8 * k)) & 0xFFu), b = (float)((c10 >> (8 * k)) & 0xFFu);
        const float c = (float)((c01 >> (8 * k)) & 0xFFu), d = (float)((c11 >> (8 * k)) & 0xFFu);
        const float top = fmaf(ax, b - a, a), bottom = fmaf(ax, d - c, c);
        out[k] = fmaf(ay, bottom - top, top) * (1.0f / 255.f);
    }
    v3 o = {out[0], out[1], out[2]};
    return o;
}

static v3 sample_tex(const uint32_t *px, uint32_t w, uint32_t h, v2 uv, uint32_t ss)
{
    if (ss == 2u) return sample_bilinear(px, w, h, uv);
    return ss == 1u ? sample_linear(px, w, h, uv) : sample_point(px, w, h, uv);
}

void orc_sample(const uint32_t *pixels, uint32_t w, uint32_t h, float u, float v, uint32_t ss, float *out)
{
    const v2 uv = {u, v};
    const v3 c = sample_tex(pixels, w, h, uv, ss);
    out[0] = c.x; out[1] = c.y; out[2] = c.z;
}

/* RGBA::GetRGBAFromColour (RGBRaw.h:24-32): R and B swapped, A = 0. */
uint32_t orc_rgba_from_colour(const float *rgb)
{
    const uint32_t r8 = cvt_u8(rgb[2] * 255.f);
    const uint32_t g8 = cvt_u8(rgb[1] * 255.f);
    const uint32_t b8 = cvt_u8(rgb[0] * 255.f);
    return r8 | (g8 << 8) | (b8 << 16);
}

/* Lambert + Phong over the scene lights (the build's extension, used when
 * lights are set): per light the reference shader's terms with its constant
 * light replaced -- L = the direction the light travels at P (a point
 * light's from its position to P), irradiance E = intensity (/ squared
 * distance for a point light), diffuse += diffuse * colour * max(0,
 * dot(-N, L)) / pi * E, specular += specular * colour * clamp(dot(vd,
 * reflect(L, N)), 0, 1)^(gloss * 25); then ambient + diffuse + specular and
 * MaxToOne as CUDAROPs.cu:452-455, or the diffuse term alone without the
 * specular and gloss maps (:459-462). */
static v3 shade_lit(const orc_frame *f, v3 diffuse, v3 fn, v3 vd, v3 P, int has_spec, v3 spec, v3 gloss)
{
    v3 dacc = {0.f, 0.f, 0.f}, sacc = {0.f, 0.f, 0.f};
    const v3 nfn = {-fn.x, -fn.y, -fn.z};
    for (uint32_t k = 0; k < f->num_lights && k < ORC_MAX_LIGHTS; ++k) {
        const orc_light *lt = &f->lights[k];
        v3 L;
        float E;
        if (lt->type == ORC_LIGHT_POINT) {
            const v3 d = {P.x - lt->vec[0], P.y - lt->vec[1], P.z - lt->vec[2]};
            E = lt->intensity / dot3(d, d);
            L = normalize3(d);
        } else {
            L.x = lt->vec[0]; L.y = lt->vec[1]; L.z = lt->vec[2];
            E = lt->intensity;
        }
        float obs = dot3(nfn, L);
        obs = obs > 0.f ? obs : 0.f;
        obs = obs / (float)3.14159265358979323846;
        obs = obs * E;
        dacc.x = fmaf(diffuse.x * lt->colour[0], obs, dacc.x);
        dacc.y = fmaf(diffuse.y * lt->colour[1], obs, dacc.y);
        dacc.z = fmaf(diffuse.z * lt->colour[2], obs, dacc.z);
        if (has_spec) {
            const float s2 = 2.f * dot3(L, fn);
            const v3 refl = {fmaf(fn.x, s2, -L.x), fmaf(fn.y, s2, -L.y), fmaf(fn.z, s2, -L.z)};
            float ang = dot3(vd, refl);
            ang = ang < 0.f ? 0.f : (ang > 1.f ? 1.f : ang);
            ang = powf(ang, gloss.x * 25.f);
            sacc.x = fmaf(spec.x * lt->colour[0], ang, sacc.x);
            sacc.y = fmaf(spec.y * lt->colour[1], ang, sacc.y);
            sacc.z = fmaf(spec.z * lt->colour[2], ang, sacc.z);
        }
    }
    if (!has_spec) return dacc;
    v3 fc = {0.05f + dacc.x, 0.05f + dacc.y, 0.05f + dacc.z};
    fc.x = fc.x + sacc.x; fc.y = fc.y + sacc.y; fc.z = fc.z + sacc.z;
    float mx = fc.y < fc.z ? fc.z : fc.y;
    mx = fc.x < mx ? mx : fc.x;
    if (mx > 1.f) {
        const float rev = 1.0f / mx;
        fc.x *= rev; fc.y *= rev; fc.z *= rev;
    }
    return fc;
}

static v3 shade_pixel_safe(const orc_frame *f, const orc_mesh *m, v2 uv, v3 n, v3 tan, v3 vd, v3 P, uint32_t ss)
{
    const v3 amb = {0.05f, 0.05f, 0.05f};
    const v3 L = {0.577f, -0.577f, -0.577f};
    const float intensity = 7.0f, shininess = 25.f;
    const v3 diffuse = sample_tex(m->tex[0], m->tex_w[0], m->tex_h[0], uv, ss);
    if (!m->tex[1]) return diffuse;
    const v3 ns = sample_tex(m->tex[1], m->tex_w[1], m->tex_h[1], uv, ss);
    const v3 cr = cross3(tan, n);
    const v3 bin = {-cr.x, -cr.y, -cr.z};
    const v3 fn0 = {fmaf(2.f, ns.x, -1.f), fmaf(2.f, ns.y, -1.f), fmaf(2.f, ns.z, -1.f)};
    v3 fn;  /* FMatrix3{tan, binormal, n} * fn0, columns tan|binormal|n */
    fn.x = fmaf(n.x, fn0.z, fmaf(tan.x, fn0.x, bin.x * fn0.y));
    fn.y = fmaf(n.y, fn0.z, fmaf(tan.y, fn0.x, bin.y * fn0.y));
    fn.z = fmaf(n.z, fn0.z, fmaf(tan.z, fn0.x, bin.z * fn0.y));
    if (f->num_lights) {
        const int has_spec = m->tex[2] && m->tex[3];
        const v3 zero = {0.f, 0.f, 0.f};
        const v3 spec = has_spec ? sample_tex(m->tex[2], m->tex_w[2], m->tex_h[2], uv, ss) : zero;
        const v3 gloss = has_spec ? sample_tex(m->tex[3], m->tex_w[3], m->tex_h[3], uv, ss) : zero;
        return shade_lit(f, diffuse, fn, vd, P, has_spec, spec, gloss);
    }
    const v3 nfn = {-fn.x, -fn.y, -fn.z};
    float obs = dot3(nfn, L);
    {   /* ClampFast(obs, 0, obs) (CUDAROPs.cu:439): a no-op for obs < 0 */
        const float c = obs < 0.f ? 0.f : obs;
        obs = c > obs ? obs : c;
    }
    obs = obs / (float)3.14159265358979323846;
    obs = obs * intensity;
    const v3 dcol = {diffuse.x * obs, diffuse.y * obs, diffuse.z * obs};
    if (!(m->tex[2] && m->tex[3])) return dcol;
    const v3 spec = sample_tex(m->tex[2], m->tex_w[2], m->tex_h[2], uv, ss);
    const v3 gloss = sample_tex(m->tex[3], m->tex_w[3], m->tex_h[3], uv, ss);
    const float dl = dot3(L, fn);
    const float s2 = 2.f * dl;
    const v3 refl = {fmaf(fn.x, s2, -L.x), fmaf(fn.y, s2, -L.y), fmaf(fn.z, s2, -L.z)};
    float ang = dot3(vd, refl);
    ang = ang < 0.f ? 0.f : (ang > 1.f ? 1.f : ang);
    ang = powf(ang, gloss.x * shininess);
    const v3 scol = {spec.x * ang, spec.y * ang, spec.z * ang};
    v3 fc = {amb.x + dcol.x, amb.y + dcol.y, amb.z + dcol.z};
    fc.x = fc.x + scol.x; fc.y = fc.y + scol.y; fc.z = fc.z + scol.z;
    /* MaxToOne (RGBColor.h:74-79) */
    float mx = fc.y < fc.z ? fc.z : fc.y;
    mx = fc.x < mx ? mx : fc.x;
    if (mx > 1.f) {
        const float rev = 1.0f / mx;
        fc.x *= rev; fc.y *= rev; fc.z *= rev;
    }
    return fc;
}

/* Fragment attributes (RasterizePixelAtomic, CUDAROPs.cu:347-380) and the
 * pixel shader for the selected visualisation (CUDARenderer.cu:833-897). */
static uint32_t shade_fragment(const orc_frame *f, const mesh_state *ms, const tri_setup *t,
                               const float w[3], float z)
{
    overtex v[3];
    for (int k = 0; k < 3; ++k) vs_full(ms, f, t->vidx[k], &v[k]);
    const float i0 = 1.f / v[0].p[3], i1 = 1.f / v[1].p[3], i2 = 1.f / v[2].p[3];
    const float winterp = 1.f / fmaf(i2, w[2], fmaf(i0, w[0], i1 * w[1]));
#define INTERP(a0, a1, a2) fmaf(w[2], (a2) * i2, fmaf(w[0], (a0) * i0, w[1] * ((a1) * i1)))
    if (f->vis == 1u) {
        /* PS_VisualiseDepthColourKernel: b8 = Remap(z, 0.985, 1) * 255 */
        const float rz = (z - 0.985f) / (1.f - 0.985f);
        return (uint32_t)cvt_u8(rz * 255.f) << 16;
    }
    v3 n = {INTERP(v[0].n.x, v[1].n.x, v[2].n.x), INTERP(v[0].n.y, v[1].n.y, v[2].n.y),
            INTERP(v[0].n.z, v[1].n.z, v[2].n.z)};
    n.x *= winterp; n.y *= winterp; n.z *= winterp;
    if (f->vis == 2u) {
        const float rgb[3] = {n.x, n.y, n.z};
        return orc_rgba_from_colour(rgb);
    }
    const orc_mesh *m = ms->m;
    if (!m->tex[0]) {
        const float rgb[3] = {INTERP(v[0].c.x, v[1].c.x, v[2].c.x), INTERP(v[0].c.y, v[1].c.y, v[2].c.y),
                              INTERP(v[0].c.z, v[1].c.z, v[2].c.z)};
        return orc_rgba_from_colour(rgb);
    }
    v2 uv = {INTERP(v[0].uv.x, v[1].uv.x, v[2].uv.x), INTERP(v[0].uv.y, v[1].uv.y, v[2].uv.y)};
    uv.x *= winterp; uv.y *= winterp;
    const v3 tan = {INTERP(v[0].tan.x, v[1].tan.x, v[2].tan.x), INTERP(v[0].tan.y, v[1].tan.y, v[2].tan.y),
                    INTERP(v[0].tan.z, v[1].tan.z, v[2].tan.z)};
    const v3 vd = normalize3((v3){INTERP(v[0].vd.x, v[1].vd.x, v[2].vd.x), INTERP(v[0].vd.y, v[1].vd.y, v[2].vd.y),
                                  INTERP(v[0].vd.z, v[1].vd.z, v[2].vd.z)});
    v3 P = {0.f, 0.f, 0.f};
    if (f->num_lights) {   /* world position, perspective-correct like uv */
        P.x = INTERP(v[0].wp.x, v[1].wp.x, v[2].wp.x) * winterp;
        P.y = INTERP(v[0].wp.y, v[1].wp.y, v[2].wp.y) * winterp;
        P.z = INTERP(v[0].wp.z, v[1].wp.z, v[2].wp.z) * winterp;
    }
#undef INTERP
    const v3 col = shade_pixel_safe(f, m, uv, n, tan, vd, P, f->sample);
    const float rgb[3] = {col.x, col.y, col.z};
    return orc_rgba_from_colour(rgb);
}

/* ------------------------------------------------------------------ */
/* Frame                                                                */
/* ------------------------------------------------------------------ */
typedef struct {
    const orc_frame *f;
    mesh_state *ms;
    uint32_t num_meshes;
    tri_setup *tris;
    const uint32_t *offsets;
    const uint32_t *list;
    uint32_t *colour, *ids;
    float *depth;
    uint32_t nbins;
    volatile int next;
    pthread_mutex_t lock;
    uint64_t fragments, covered;
} raster_job;

static void raster_bin(raster_job *job, uint32_t bin, uint64_t *frag_count, uint64_t *cov_count)
{
    const orc_frame *f = job->f;
    const uint32_t bx = bin % f->num_bins_x, by = bin / f->num_bins_x;
    const int32_t x0 = (int32_t)(bx * f->bin_w), y0 = (int32_t)(by * f->bin_h);
    int32_t x1 = x0 + (int32_t)f->bin_w, y1 = y0 + (int32_t)f->bin_h;
    if (x1 > (int32_t)f->width) x1 = (int32_t)f->width;
    if (y1 > (int32_t)f->height) y1 = (int32_t)f->height;
    if (x0 >= x1 || y0 >= y1) return;
    const int32_t tw = x1 - x0, th = y1 - y0;
    int32_t *best_key = (int32_t *)malloc(sizeof(int32_t) * (size_t)(tw * th));
    uint32_t *best_id = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)(tw * th));
    float *best_z = (float *)malloc(sizeof(float) * (size_t)(tw * th));
    float *best_w = (float *)malloc(sizeof(float) * 3u * (size_t)(tw * th));
    for (int32_t i = 0; i < tw * th; ++i) { best_key[i] = 2147483647; best_id[i] = INV_PRIM; }
    uint64_t frags = 0;
    for (uint32_t k = job->offsets[bin]; k < job->offsets[bin + 1]; ++k) {
        const uint32_t prim = job->list[k];
        const tri_setup *t = &job->tris[prim];
        /* pixels outside [floor(min)-1, ceil(max)+1] cannot be covered */
        const float fx0 = floorf(min3f(t->s[0].x, t->s[1].x, t->s[2].x)) - 1.f;
        const float fx1 = ceilf(max3f(t->s[0].x, t->s[1].x, t->s[2].x)) + 1.f;
        const float fy0 = floorf(min3f(t->s[0].y, t->s[1].y, t->s[2].y)) - 1.f;
        const float fy1 = ceilf(max3f(t->s[0].y, t->s[1].y, t->s[2].y)) + 1.f;
        int32_t px0 = x0, px1 = x1 - 1, py0 = y0, py1 = y1 - 1;
        if (fx0 == fx0 && fx0 > (float)px0) px0 = (int32_t)fx0;
        if (fx1 == fx1 && fx1 < (float)px1) px1 = (int32_t)fx1;
        if (fy0 == fy0 && fy0 > (float)py0) py0 = (int32_t)fy0;
        if (fy1 == fy1 && fy1 < (float)py1) py1 = (int32_t)fy1;
        for (int32_t py = py0; py <= py1; ++py)
            for (int32_t px = px0; px <= px1; ++px) {
                float w[3], z;
                int32_t key;
                if (!fragment(t, f->raster_mode, px, py, w, &z, &key)) continue;
                ++frags;
                const int32_t li = (py - y0) * tw + (px - x0);
                /* PerformDepthTestAtomic (CUDAROPs.cu:231-251): strict < on the
                 * integer key; bins are walked in ascending primitive id, so the
                 * lowest id wins a tie */
                if (key < best_key[li]) {
                    best_key[li] = key;
                    best_id[li] = prim;
                    best_z[li] = z;
                    best_w[3 * li] = w[0]; best_w[3 * li + 1] = w[1]; best_w[3 * li + 2] = w[2];
                }
            }
    }
    uint64_t cov = 0;
    for (int32_t py = y0; py < y1; ++py)
        for (int32_t px = x0; px < x1; ++px) {
            const int32_t li = (py - y0) * tw + (px - x0);
            const size_t gi = (size_t)py * f->width + (size_t)px;
            uint32_t c32;
            float zz = 0.f;
            if (best_id[li] == INV_PRIM) {
                c32 = f->vis == 0u ? f->clear_colour32 : 0u;
            } else {
                const tri_setup *t = &job->tris[best_id[li]];
                c32 = shade_fragment(f, &job->ms[t->mesh], t, &best_w[3 * li], best_z[li]);
                zz = best_z[li];
                ++cov;
            }
            if (job->colour) job->colour[gi] = c32;
            if (job->depth) job->depth[gi] = zz;
            if (job->ids) job->ids[gi] = best_id[li];
        }
    free(best_key); free(best_id); free(best_z); free(best_w);
    *frag_count += frags;
    *cov_count += cov;
}

static void *raster_worker(void *arg)
{
    raster_job *job = (raster_job *)arg;
    uint64_t frags = 0, cov = 0;
    const uint32_t stride = job->f->bin_stride > 1u ? job->f->bin_stride : 1u;
    const uint32_t phase = stride > 1u ? job->f->bin_phase % stride : 0u;
    for (;;) {
        const int b = __sync_fetch_and_add(&job->next, 1);
        if ((uint32_t)b >= job->nbins) break;
        if ((uint32_t)b % stride != phase) continue;
        if (job->f->bin_row1) {   /* a band of bin rows */
            const uint32_t row = (uint32_t)b / job->f->num_bins_x;
            if (row < job->f->bin_row0 || row >= job->f->bin_row1) continue;
        }
        raster_bin(job, (uint32_t)b, &frags, &cov);
    }
    pthread_mutex_lock(&job->lock);
    job->fragments += frags;
    job->covered += cov;
    pthread_mutex_unlock(&job->lock);
    return NULL;
}

static int prepare(const orc_frame *f, const orc_mesh *meshes, uint32_t num_meshes,
                   mesh_state **ms_out, uint64_t *ntris_out)
{
    if (!f || (!meshes && num_meshes) || f->width == 0 || f->height == 0 || f->bin_w == 0 ||
        f->bin_h == 0 || f->num_bins_x == 0 || f->num_bins_y == 0 || f->width > 32767u || f->height > 32767u)
        return 1;
    mesh_state *ms = (mesh_state *)calloc(num_meshes ? num_meshes : 1u, sizeof(mesh_state));
    if (!ms) return 3;
    float vp[16];
    orc_mat4_mul(f->proj, f->view, vp);
    uint64_t base = 0;
    for (uint32_t i = 0; i < num_meshes; ++i) {
        ms[i].m = &meshes[i];
        orc_mat4_mul(vp, meshes[i].world, ms[i].wvp);
        ms[i].prim_base = base;
        ms[i].num_tris = mesh_num_tris(&meshes[i]);
        base += ms[i].num_tris;
    }
    *ms_out = ms;
    *ntris_out = base;
    return 0;
}

static void setup_triangle(const orc_frame *f, const mesh_state *ms, uint32_t mesh, uint64_t local,
                           tri_setup *t)
{
    uint32_t idx[3];
    tri_indices(ms->m, local, idx);
    float p[3][4];
    for (int k = 0; k < 3; ++k) vs_ndc(ms, idx[k], p[k]);
    t->mesh = mesh;
    t->vidx[0] = idx[0]; t->vidx[1] = idx[1]; t->vidx[2] = idx[2];
    t->visible = !orc_cull(p[0], p[1], p[2], f->cam_fwd, f->cull) && orc_frustum_visible(p[0], p[1], p[2]);
    for (int k = 0; k < 3; ++k) {
        t->s[k] = to_screen(p[k][0], p[k][1], f->width, f->height);
        t->z[k] = p[k][2];
    }
    setup_fixed(t);
}

int orc_render(const orc_frame *f, const orc_mesh *meshes, uint32_t num_meshes,
               uint32_t *colour, float *depth, uint32_t *ids,
               uint32_t *bin_offsets, uint32_t *bin_ids, uint64_t bin_capacity, orc_stats *stats)
{
    mesh_state *ms = NULL;
    uint64_t ntris = 0;
    int rc = prepare(f, meshes, num_meshes, &ms, &ntris);
    if (rc) return rc;
    const uint32_t nbins = f->num_bins_x * f->num_bins_y;
    tri_setup *tris = (tri_setup *)calloc(ntris ? ntris : 1u, sizeof(tri_setup));
    int32_t *rects = (int32_t *)calloc(4u * (ntris ? ntris : 1u), sizeof(int32_t));
    uint32_t *offsets = (uint32_t *)calloc((size_t)nbins + 1u, sizeof(uint32_t));
    if (!tris || !rects || !offsets) { free(ms); free(tris); free(rects); free(offsets); return 3; }

    /* VS + TA + bin counting, one triangle at a time in primitive order */
    uint64_t visible = 0, fpath = 0;
    for (uint32_t mi = 0; mi < num_meshes; ++mi)
        for (uint64_t lt = 0; lt < ms[mi].num_tris; ++lt) {
            const uint64_t prim = ms[mi].prim_base + lt;
            tri_setup *t = &tris[prim];
            setup_triangle(f, &ms[mi], mi, lt, t);
            int32_t *r = &rects[4 * prim];
            r[0] = 1; r[1] = 1; r[2] = 0; r[3] = 0;
            if (!t->visible) continue;
            ++visible;
            fpath += (uint64_t)t->float_path;
            bin_rect_screen(t->s[0], t->s[1], t->s[2], f->width, f->height, f->num_bins_x, f->num_bins_y,
                            f->bin_w, f->bin_h, r);
            for (int32_t x = r[0]; x <= r[2]; ++x)
                for (int32_t y = r[1]; y <= r[3]; ++y) offsets[(uint32_t)x + (uint32_t)y * f->num_bins_x + 1u]++;
        }
    for (uint32_t b = 0; b < nbins; ++b) offsets[b + 1] += offsets[b];
    const uint64_t pairs = offsets[nbins];
    uint32_t *list = (uint32_t *)malloc(sizeof(uint32_t) * (pairs ? pairs : 1u));
    uint32_t *cursor = (uint32_t *)calloc(nbins, sizeof(uint32_t));
    if (!list || !cursor) { free(ms); free(tris); free(rects); free(offsets); free(list); free(cursor); return 3; }
    for (uint64_t prim = 0; prim < ntris; ++prim) {
        const int32_t *r = &rects[4 * prim];
        for (int32_t x = r[0]; x <= r[2]; ++x)
            for (int32_t y = r[1]; y <= r[3]; ++y) {
                const uint32_t b = (uint32_t)x + (uint32_t)y * f->num_bins_x;
                list[offsets[b] + cursor[b]++] = (uint32_t)prim;
            }
    }
    free(cursor);
    free(rects);

    /* RA + PS: pixels outside every bin tile keep the clear colour */
    if (colour || depth || ids) {
        const size_t npx = (size_t)f->width * f->height;
        for (size_t i = 0; i < npx; ++i) {
            if (colour) colour[i] = f->vis == 0u ? f->clear_colour32 : 0u;
            if (depth) depth[i] = 0.f;
            if (ids) ids[i] = INV_PRIM;
        }
    }
    raster_job job;
    memset(&job, 0, sizeof job);
    job.f = f; job.ms = ms; job.num_meshes = num_meshes; job.tris = tris;
    job.offsets = offsets; job.list = list; job.colour = colour; job.depth = depth; job.ids = ids;
    job.nbins = nbins; job.next = 0;
    pthread_mutex_init(&job.lock, NULL);
    uint32_t nth = f->num_threads > 1u ? f->num_threads : 1u;
    if (nth > 256u) nth = 256u;
    if (!colour && !depth && !ids) {
        /* binning only */
    } else if (nth == 1u) {
        raster_worker(&job);
    } else {
        pthread_t th[256];
        uint32_t started = 0;
        for (uint32_t i = 0; i < nth; ++i)
            if (pthread_create(&th[i], NULL, raster_worker, &job) == 0) ++started;
        if (started == 0) raster_worker(&job);
        for (uint32_t i = 0; i < started; ++i) pthread_join(th[i], NULL);
    }
    pthread_mutex_destroy(&job.lock);

    rc = 0;
    if (bin_offsets) memcpy(bin_offsets, offsets, sizeof(uint32_t) * ((size_t)nbins + 1u));
    if (bin_ids) {
        if (pairs > bin_capacity) rc = 2;
        else memcpy(bin_ids, list, sizeof(uint32_t) * pairs);
    }
    if (stats) {
        stats->num_triangles = ntris;
        stats->num_visible = visible;
        stats->num_pairs = pairs;
        stats->num_float_path = fpath;
        stats->fragments = job.fragments;
        stats->covered_pixels = job.covered;
    }
    free(list); free(offsets); free(tris); free(ms);
    return rc;
}

int orc_probe(const orc_frame *f, const orc_mesh *meshes, uint32_t num_meshes,
              uint32_t prim, uint32_t px, uint32_t py, orc_probe_out *out)
{
    mesh_state *ms = NULL;
    uint64_t ntris = 0;
    int rc = prepare(f, meshes, num_meshes, &ms, &ntris);
    if (rc) return rc;
    if (prim >= ntris || !out) { free(ms); return 1; }
    uint32_t mi = 0;
    while (mi + 1 < num_meshes && ms[mi + 1].prim_base <= prim) ++mi;
    tri_setup t;
    setup_triangle(f, &ms[mi], mi, prim - ms[mi].prim_base, &t);
    memset(out, 0, sizeof *out);
    out->visible = t.visible;
    out->float_path = t.float_path;
    float w[3], e[3];
    out->covered_ref = cover_ref(&t, (float)px, (float)py, w, e);
    out->z_ref = out->covered_ref ? interp_z(w, t.z) : 0.f;
    out->e_ref[0] = e[0]; out->e_ref[1] = e[1]; out->e_ref[2] = e[2];
    if (!t.float_path) {
        out->covered_fixed = t.coverable_fx && cover_fixed(&t, (int32_t)px, (int32_t)py, w);
        out->z_fixed = out->covered_fixed ? interp_z(w, t.z) : 0.f;
    } else {
        out->covered_fixed = out->covered_ref;
        out->z_fixed = out->z_ref;
    }
    /* |e_ref - e_exact(snapped)| <= snapping (vertices move <= 2^-17 px per
     * axis) + float rounding of the reference's subtraction/product chain;
     * edge i: w[2] = v0->v1, w[0] = v1->v2, w[1] = v2->v0 */
    const int ea[3] = {1, 2, 0}, eb[3] = {2, 0, 1};
    for (int i = 0; i < 3; ++i) {
        const v2 A = t.s[ea[i]], B = t.s[eb[i]];
        const float dpx = fabsf((float)px - A.x) + fabsf((float)py - A.y);
        const float dab = fabsf(B.x - A.x) + fabsf(B.y - A.y);
        const float snapb = ldexpf(dpx, -FX_BITS) + ldexpf(dab, -(FX_BITS + 1)) + ldexpf(1.f, -2 * FX_BITS);
        const float rnd = ldexpf(16.f * (fabsf((float)px - A.x) * fabsf(B.y - A.y) +
                                         fabsf((float)py - A.y) * fabsf(B.x - A.x)), -24);
        out->e_bound[i] = 2.f * (snapb + rnd);
    }
    free(ms);
    return 0;
}
