// gbr_shade.cuh -- deferred per-pixel shading of the winning fragment.
//
// After visibility is resolved for a tile, each pixel's winning primitive is
// re-fetched, its three vertices go through the full vertex stage
// (GetNDCVertex, CustomCUDARasterizer/CUDAROPs.cu:99-118), the fragment
// attributes are interpolated as RasterizePixelAtomic does
// (CUDAROPs.cu:347-380) and the pixel shader of the selected
// VisualisationState runs (PS_Kernel / PS_VisualiseDepthColourKernel /
// PS_VisualiseNormalKernel, CUDARenderer.cu:833-897).  Only one fragment per
// pixel is shaded, instead of every fragment that wins a depth test.
#pragma once
#include "gbr_device.cuh"

namespace gbr {

// b / 255 for every byte value b, each the correctly rounded quotient
// (evaluated at compile time in single precision): the RGBA8 vertex colours
// read as GetRGBColor (RGBRaw.h:34-38) divides, without a division per use
// (a product with 1/255 differs in 126 of the 256 values).
struct ByteOver255 {
    float v[256];
    constexpr ByteOver255() : v() {
        for (int b = 0; b < 256; ++b) v[b] = (float)b / 255.0f;
    }
};
__device__ constexpr ByteOver255 kByteOver255{};

struct OVtx {
    float px, py, pz, pw;  // NDC xyz, clip w
    float u, v;
    F3 n, tan, vd, c;
    F3 wp;                 // world position (scene lights)
};

__device__ __forceinline__ void fetch_full(const MeshDev& m, uint32_t vi, float iv[14]) {
    if (m.vertex_format == kVertexPos3Rgba8) {
        const float4 v = __ldg(reinterpret_cast<const float4*>(m.vertices) + vi);
        const uint32_t rgba = __float_as_uint(v.w);
        iv[0] = v.x; iv[1] = v.y; iv[2] = v.z;
#pragma unroll
        for (int k = 3; k < 11; ++k) iv[k] = 0.f;
        // GetRGBColor (RGBRaw.h:34-38): r = byte0 / 255
        iv[11] = kByteOver255.v[rgba & 0xFFu];
        iv[12] = kByteOver255.v[(rgba >> 8) & 0xFFu];
        iv[13] = kByteOver255.v[(rgba >> 16) & 0xFFu];
    } else {
        const float2* b = reinterpret_cast<const float2*>(reinterpret_cast<const float*>(m.vertices) + 14u * (size_t)vi);
#pragma unroll
        for (int k = 0; k < 7; ++k) {
            const float2 t = __ldg(b + k);
            iv[2 * k] = t.x;
            iv[2 * k + 1] = t.y;
        }
    }
}

__device__ __forceinline__ OVtx vertex_stage(const MeshDev& m, const FrameDev& F, uint32_t vi) {
    float iv[14];
    fetch_full(m, vi, iv);
    OVtx o;
    const float4 clip = xform_point(m.wvp, iv[0], iv[1], iv[2]);
    o.px = __fdiv_rn(clip.x, clip.w);
    o.py = __fdiv_rn(clip.y, clip.w);
    o.pz = __fdiv_rn(clip.z, clip.w);
    o.pw = clip.w;
    o.n = rot3(m.world, f3(iv[5], iv[6], iv[7]));
    o.tan = rot3(m.world, f3(iv[8], iv[9], iv[10]));
    const float4 wp = xform_point(m.world, iv[0], iv[1], iv[2]);
    o.vd = normalize3(sub3(f3(wp.x, wp.y, wp.z), f3(F.cam_pos[0], F.cam_pos[1], F.cam_pos[2])));
    o.wp = f3(wp.x, wp.y, wp.z);
    o.u = iv[3];
    o.v = iv[4];
    o.c = f3(iv[11], iv[12], iv[13]);
    return o;
}

__device__ __forceinline__ F3 rgb_of(uint32_t c) {   // byte / 255 per channel
    return f3(kByteOver255.v[c & 0xFFu], kByteOver255.v[(c >> 8) & 0xFFu], kByteOver255.v[(c >> 16) & 0xFFu]);
}

// SamplePoint (CUDATextureSampler.cuh:87-104): u = int(uv.x*w + 0.5);
// out of range samples magenta.
__device__ __forceinline__ F3 sample_point(const TexDev& t, float u, float v) {
    const int x = cvt_s32(__fmaf_rn(u, (float)t.w, 0.5f));
    const int y = cvt_s32(__fmaf_rn(v, (float)t.h, 0.5f));
    if (x < 0 || y < 0 || (uint32_t)x >= t.w || (uint32_t)y >= t.h) return f3(1.f, 0.f, 1.f);
    return rgb_of(__ldg(t.px + (uint32_t)x + (uint32_t)y * t.w));
}

// SampleLinear (CUDATextureSampler.cuh:112-190): centre at 1/2 plus the four
// row-major neighbours at 1/8 each (wrapping across rows, clamped at the
// buffer ends).
__device__ __forceinline__ F3 sample_linear(const TexDev& t, float u, float v) {
    const int x = cvt_s32(__fmaf_rn(u, (float)t.w, 0.5f));
    const int y = cvt_s32(__fmaf_rn(v, (float)t.h, 0.5f));
    if (x < 0 || y < 0 || (uint32_t)x >= t.w || (uint32_t)y >= t.h) return f3(1.f, 0.f, 1.f);
    const int size = (int)(t.w * t.h);
    const int o = x + y * (int)t.w;
    int nb[4];
    nb[0] = o - 1; if (nb[0] < 0) nb[0] = o;
    nb[1] = o + 1; if (nb[1] >= size) nb[1] = o;
    nb[2] = o + (int)t.w; if (nb[2] >= size) nb[2] = o;
    nb[3] = o - (int)t.w; if (nb[3] < 0) nb[3] = o;
    const float wt = __fdiv_rn(1.f, 8.f);
    float r = 0.f, g = 0.f, b = 0.f;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const uint32_t c = __ldg(t.px + nb[i]);
        r = __fmaf_rn((float)(c & 0xFFu), wt, r);
        g = __fmaf_rn((float)((c >> 8) & 0xFFu), wt, g);
        b = __fmaf_rn((float)((c >> 16) & 0xFFu), wt, b);
    }
    const uint32_t c = __ldg(t.px + o);
    r = __fadd_rn(r, __fdiv_rn((float)(c & 0xFFu), 2.f));
    g = __fadd_rn(g, __fdiv_rn((float)((c >> 8) & 0xFFu), 2.f));
    b = __fadd_rn(b, __fdiv_rn((float)((c >> 16) & 0xFFu), 2.f));
    const float rev = __fdiv_rn(1.0f, 255.f);
    return f3(__fmul_rn(r, rev), __fmul_rn(g, rev), __fmul_rn(b, rev));
}

// Bilinear filtering (the build's extension, GBR_SAMPLE_BILINEAR): texel
// centres at (i + 1/2) / size, the four nearest texels weighted by the
// fractional offsets, addresses clamped to the texture.
__device__ __forceinline__ F3 sample_bilinear(const TexDev& t, float u, float v) {
    const float x = __fmaf_rn(u, (float)t.w, -0.5f), y = __fmaf_rn(v, (float)t.h, -0.5f);
    const float fx = floorf(x), fy = floorf(y);
    const float ax = __fsub_rn(x, fx), ay = __fsub_rn(y, fy);
    const int w = (int)t.w, h = (int)t.h;
    int xi = cvt_s32(fx), yi = cvt_s32(fy);
    xi = xi < -1 ? -1 : (xi > w - 1 ? w - 1 : xi);
    yi = yi < -1 ? -1 : (yi > h - 1 ? h - 1 : yi);
    const uint32_t x0 = (uint32_t)(xi < 0 ? 0 : xi), x1 = (uint32_t)(xi + 1 > w - 1 ? w - 1 : xi + 1);
    const uint32_t y0 = (uint32_t)(yi < 0 ? 0 : yi), y1 = (uint32_t)(yi + 1 > h - 1 ? h - 1 : yi + 1);
    const uint32_t c00 = __ldg(t.px + x0 + y0 * t.w), c10 = __ldg(t.px + x1 + y0 * t.w);
    const uint32_t c01 = __ldg(t.px + x0 + y1 * t.w), c11 = __ldg(t.px + x1 + y1 * t.w);
    float out[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float a = (float)((c00 >> (8 * k)) & 0xFFu), b = (float)((c10 >> (8 * k)) & 0xFFu);
        const float c = (float)((c01 >> (8 * k)) & 0xFFu), d = (float)((c11 >> (8 * k)) & 0xFFu);
        const float top = __fmaf_rn(ax, __fsub_rn(b, a), a), bottom = __fmaf_rn(ax, __fsub_rn(d, c), c);
        out[k] = __fmul_rn(__fmaf_rn(ay, __fsub_rn(bottom, top), top), __fdiv_rn(1.0f, 255.f));
    }
    return f3(out[0], out[1], out[2]);
}

__device__ __forceinline__ F3 sample_tex(const TexDev& t, float u, float v, uint32_t ss) {
    if (ss == 2u) return sample_bilinear(t, u, v);
    return ss == 1u ? sample_linear(t, u, v) : sample_point(t, u, v);
}

// Lambert + Phong over the scene lights (the build's extension, used when
// lights are set): per light the reference shader's terms with its constant
// light replaced -- L = the direction the light travels at P (a point
// light's from its position to P), irradiance E = intensity (/ squared
// distance for a point light, PointLight::GetBiradiance), diffuse +=
// diffuse * colour * max(0, dot(-N, L)) / pi * E, specular += specular *
// colour * clamp(dot(vd, reflect(L, N)), 0, 1)^(gloss * 25); then ambient +
// diffuse + specular and MaxToOne (CUDAROPs.cu:452-455), or the diffuse
// term alone without the specular and gloss maps (:459-462).
__device__ __forceinline__ F3 shade_lit(const FrameDev& F, F3 diffuse, F3 fn, F3 vd, F3 P, bool has_spec, F3 spec,
                                        F3 gloss) {
    F3 dacc = f3(0.f, 0.f, 0.f), sacc = f3(0.f, 0.f, 0.f);
    const F3 nfn = f3(-fn.x, -fn.y, -fn.z);
    const uint32_t nl = F.num_lights < kMaxLights ? F.num_lights : kMaxLights;
    for (uint32_t k = 0; k < nl; ++k) {
        const LightDev lt = F.lights[k];
        F3 L;
        float E;
        if (lt.type == 1u) {
            const F3 d = f3(__fsub_rn(P.x, lt.vec[0]), __fsub_rn(P.y, lt.vec[1]), __fsub_rn(P.z, lt.vec[2]));
            E = __fdiv_rn(lt.intensity, dot3(d, d));
            L = normalize3(d);
        } else {
            L = f3(lt.vec[0], lt.vec[1], lt.vec[2]);
            E = lt.intensity;
        }
        float obs = dot3(nfn, L);
        obs = obs > 0.f ? obs : 0.f;
        obs = __fdiv_rn(obs, 3.14159265358979323846f);
        obs = __fmul_rn(obs, E);
        dacc = f3(__fmaf_rn(__fmul_rn(diffuse.x, lt.colour[0]), obs, dacc.x),
                  __fmaf_rn(__fmul_rn(diffuse.y, lt.colour[1]), obs, dacc.y),
                  __fmaf_rn(__fmul_rn(diffuse.z, lt.colour[2]), obs, dacc.z));
        if (has_spec) {
            const float s2 = __fmul_rn(2.f, dot3(L, fn));
            const F3 refl = f3(__fmaf_rn(fn.x, s2, -L.x), __fmaf_rn(fn.y, s2, -L.y), __fmaf_rn(fn.z, s2, -L.z));
            float ang = dot3(vd, refl);
            ang = ang < 0.f ? 0.f : (ang > 1.f ? 1.f : ang);
            ang = powf(ang, __fmul_rn(gloss.x, 25.f));
            sacc = f3(__fmaf_rn(__fmul_rn(spec.x, lt.colour[0]), ang, sacc.x),
                      __fmaf_rn(__fmul_rn(spec.y, lt.colour[1]), ang, sacc.y),
                      __fmaf_rn(__fmul_rn(spec.z, lt.colour[2]), ang, sacc.z));
        }
    }
    if (!has_spec) return dacc;
    F3 fc = f3(__fadd_rn(0.05f, dacc.x), __fadd_rn(0.05f, dacc.y), __fadd_rn(0.05f, dacc.z));
    fc = f3(__fadd_rn(fc.x, sacc.x), __fadd_rn(fc.y, sacc.y), __fadd_rn(fc.z, sacc.z));
    float mx = fc.y < fc.z ? fc.z : fc.y;
    mx = fc.x < mx ? mx : fc.x;
    if (mx > 1.f) {
        const float rev = __fdiv_rn(1.0f, mx);
        fc = f3(__fmul_rn(fc.x, rev), __fmul_rn(fc.y, rev), __fmul_rn(fc.z, rev));
    }
    return fc;
}

// RGBA::GetRGBAFromColour (RGBRaw.h:24-32): bytes B, G, R, 0.
__device__ __forceinline__ uint32_t rgba_from_colour(F3 c) {
    return cvt_u8(__fmul_rn(c.z, 255.f)) | (cvt_u8(__fmul_rn(c.y, 255.f)) << 8) | (cvt_u8(__fmul_rn(c.x, 255.f)) << 16);
}

// ShadePixelSafe (CUDAROPs.cu:411-470).
__device__ __forceinline__ F3 shade_pixel_safe(const FrameDev& F, const MeshDev& m, float u, float v, F3 n, F3 tan,
                                               F3 vd, F3 P, uint32_t ss) {
    const F3 L = f3(0.577f, -0.577f, -0.577f);
    const F3 diffuse = sample_tex(m.tex[0], u, v, ss);
    if (!m.tex[1].px) return diffuse;
    const F3 ns = sample_tex(m.tex[1], u, v, ss);
    const F3 cr = cross3(tan, n);
    const F3 bin = f3(-cr.x, -cr.y, -cr.z);
    const F3 fn0 = f3(__fmaf_rn(2.f, ns.x, -1.f), __fmaf_rn(2.f, ns.y, -1.f), __fmaf_rn(2.f, ns.z, -1.f));
    const F3 fn = f3(__fmaf_rn(n.x, fn0.z, __fmaf_rn(tan.x, fn0.x, __fmul_rn(bin.x, fn0.y))),
                     __fmaf_rn(n.y, fn0.z, __fmaf_rn(tan.y, fn0.x, __fmul_rn(bin.y, fn0.y))),
                     __fmaf_rn(n.z, fn0.z, __fmaf_rn(tan.z, fn0.x, __fmul_rn(bin.z, fn0.y))));
    if (F.num_lights) {
        const bool has_spec = m.tex[2].px && m.tex[3].px;
        const F3 zero = f3(0.f, 0.f, 0.f);
        const F3 spec = has_spec ? sample_tex(m.tex[2], u, v, ss) : zero;
        const F3 gloss = has_spec ? sample_tex(m.tex[3], u, v, ss) : zero;
        return shade_lit(F, diffuse, fn, vd, P, has_spec, spec, gloss);
    }
    float obs = dot3(f3(-fn.x, -fn.y, -fn.z), L);
    {   // ClampFast(obs, 0, obs) (CUDAROPs.cu:439) leaves negative values as they are
        const float c = obs < 0.f ? 0.f : obs;
        obs = c > obs ? obs : c;
    }
    obs = __fdiv_rn(obs, 3.14159265358979323846f);
    obs = __fmul_rn(obs, 7.0f);
    const F3 dcol = f3(__fmul_rn(diffuse.x, obs), __fmul_rn(diffuse.y, obs), __fmul_rn(diffuse.z, obs));
    if (!(m.tex[2].px && m.tex[3].px)) return dcol;
    const F3 spec = sample_tex(m.tex[2], u, v, ss);
    const F3 gloss = sample_tex(m.tex[3], u, v, ss);
    const float s2 = __fmul_rn(2.f, dot3(L, fn));
    const F3 refl = f3(__fmaf_rn(fn.x, s2, -L.x), __fmaf_rn(fn.y, s2, -L.y), __fmaf_rn(fn.z, s2, -L.z));
    float ang = dot3(vd, refl);
    ang = ang < 0.f ? 0.f : (ang > 1.f ? 1.f : ang);
    ang = powf(ang, __fmul_rn(gloss.x, 25.f));
    F3 fc = f3(__fadd_rn(0.05f, dcol.x), __fadd_rn(0.05f, dcol.y), __fadd_rn(0.05f, dcol.z));
    fc = f3(__fadd_rn(fc.x, __fmul_rn(spec.x, ang)), __fadd_rn(fc.y, __fmul_rn(spec.y, ang)),
            __fadd_rn(fc.z, __fmul_rn(spec.z, ang)));
    float mx = fc.y < fc.z ? fc.z : fc.y;   // MaxToOne (RGBColor.h:74-79)
    mx = fc.x < mx ? mx : fc.x;
    if (mx > 1.f) {
        const float rev = __fdiv_rn(1.0f, mx);
        fc = f3(__fmul_rn(fc.x, rev), __fmul_rn(fc.y, rev), __fmul_rn(fc.z, rev));
    }
    return fc;
}

// Colour of the fragment of primitive `prim` at pixel (x, y) with weights w.
// FLAT: the frame is known to shade every pixel from vertex colours (PBR
// view, no mesh with a diffuse map), which keeps the kernel's registers to
// what that path needs.
template <bool FLAT>
__device__ __forceinline__ uint32_t shade_fragment(const FrameDev& F, const MeshDev& m, uint32_t prim,
                                                   const float w[3], float z) {
    if (!FLAT && F.vis == 1u) {  // Remap(z, 0.985, 1) * 255 into the blue byte
        const float rz = __fdiv_rn(__fsub_rn(z, 0.985f), __fsub_rn(1.f, 0.985f));
        return cvt_u8(__fmul_rn(rz, 255.f)) << 16;
    }
    uint32_t vid[3];
    tri_vertex_ids(m, prim - m.prim_base, vid);
    if (FLAT || (F.vis == 0u && !m.tex[0].px)) {
        // untextured: the vertex colours weighted by w / w_clip, not
        // multiplied by the interpolated w (CUDAROPs.cu:379-380); of the
        // vertex stage only each vertex's clip w and colour are needed, the
        // same operations as in vertex_stage
        float ic[3];
        F3 col[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            float iv[14];
            fetch_full(m, vid[k], iv);
            const float* M = m.wvp;
            const float cw = __fadd_rn(__fmaf_rn(M4(M, 3, 2), iv[2], __fmaf_rn(M4(M, 3, 0), iv[0], __fmul_rn(M4(M, 3, 1), iv[1]))),
                                       M4(M, 3, 3));
            ic[k] = __fdiv_rn(1.f, cw);
            col[k] = f3(iv[11], iv[12], iv[13]);
        }
#define GBR_CINTERP(a0, a1, a2) \
    __fmaf_rn(w[2], __fmul_rn((a2), ic[2]), __fmaf_rn(w[0], __fmul_rn((a0), ic[0]), __fmul_rn(w[1], __fmul_rn((a1), ic[1]))))
        const F3 c = f3(GBR_CINTERP(col[0].x, col[1].x, col[2].x), GBR_CINTERP(col[0].y, col[1].y, col[2].y),
                        GBR_CINTERP(col[0].z, col[1].z, col[2].z));
#undef GBR_CINTERP
        return rgba_from_colour(c);
    }
    const OVtx v0 = vertex_stage(m, F, vid[0]);
    const OVtx v1 = vertex_stage(m, F, vid[1]);
    const OVtx v2 = vertex_stage(m, F, vid[2]);
    const float i0 = __fdiv_rn(1.f, v0.pw), i1 = __fdiv_rn(1.f, v1.pw), i2 = __fdiv_rn(1.f, v2.pw);
    const float winterp = __fdiv_rn(1.f, __fmaf_rn(i2, w[2], __fmaf_rn(i0, w[0], __fmul_rn(i1, w[1]))));
#define GBR_INTERP(a0, a1, a2) \
    __fmaf_rn(w[2], __fmul_rn((a2), i2), __fmaf_rn(w[0], __fmul_rn((a0), i0), __fmul_rn(w[1], __fmul_rn((a1), i1))))
    F3 n = f3(GBR_INTERP(v0.n.x, v1.n.x, v2.n.x), GBR_INTERP(v0.n.y, v1.n.y, v2.n.y), GBR_INTERP(v0.n.z, v1.n.z, v2.n.z));
    n = f3(__fmul_rn(n.x, winterp), __fmul_rn(n.y, winterp), __fmul_rn(n.z, winterp));
    if (F.vis == 2u) return rgba_from_colour(n);
    if (!m.tex[0].px) {
        // colour is not multiplied by the interpolated w (CUDAROPs.cu:379-380)
        const F3 c = f3(GBR_INTERP(v0.c.x, v1.c.x, v2.c.x), GBR_INTERP(v0.c.y, v1.c.y, v2.c.y),
                        GBR_INTERP(v0.c.z, v1.c.z, v2.c.z));
        return rgba_from_colour(c);
    }
    const float u = __fmul_rn(GBR_INTERP(v0.u, v1.u, v2.u), winterp);
    const float vv = __fmul_rn(GBR_INTERP(v0.v, v1.v, v2.v), winterp);
    // tangent is not multiplied by the interpolated w (CUDAROPs.cu:371-372)
    const F3 tan = f3(GBR_INTERP(v0.tan.x, v1.tan.x, v2.tan.x), GBR_INTERP(v0.tan.y, v1.tan.y, v2.tan.y),
                      GBR_INTERP(v0.tan.z, v1.tan.z, v2.tan.z));
    const F3 vd = normalize3(f3(GBR_INTERP(v0.vd.x, v1.vd.x, v2.vd.x), GBR_INTERP(v0.vd.y, v1.vd.y, v2.vd.y),
                                GBR_INTERP(v0.vd.z, v1.vd.z, v2.vd.z)));
    F3 P = f3(0.f, 0.f, 0.f);
    if (F.num_lights)   // world position, perspective-correct like uv
        P = f3(__fmul_rn(GBR_INTERP(v0.wp.x, v1.wp.x, v2.wp.x), winterp),
               __fmul_rn(GBR_INTERP(v0.wp.y, v1.wp.y, v2.wp.y), winterp),
               __fmul_rn(GBR_INTERP(v0.wp.z, v1.wp.z, v2.wp.z), winterp));
#undef GBR_INTERP
    return rgba_from_colour(shade_pixel_safe(F, m, u, vv, n, tan, vd, P, F.sample));
}

}  // namespace gbr
