// gbr_kernels.cu -- the frame hot path on sm_103a.
//
//   setup_count : vertex stage (positions) + triangle assembly + cull +
//                 frustum reject + raster setup + bin rectangle, and the
//                 count pass of exact binning (warp-aggregated atomics).
//   bin_scan    : exclusive scan of bin counts -> list offsets, fill cursors
//                 and raster work items (bin, chunk of <= queue_chunk ids).
//   bin_fill    : second pass: each triangle appends its id to every bin of
//                 its rectangle (warp-aggregated, one atomic per distinct bin).
//   raster      : persistent CTAs pull work items; a CTA rasterises its chunk
//                 into a shared-memory tile of packed (depth key, prim id)
//                 with 64-bit atomicMin, merges multi-chunk bins through a
//                 global tile, then shades each pixel once and writes colour,
//                 depth and id.
//
// Reference stages replaced: VS_Kernel, TA_Kernel, TB_Kernel,
// RA_PerTileKernel, PS_Kernel and the CLEAR_* kernels
// (CustomCUDARasterizer/CUDARenderer.cu:598-1129, launchers :1625-1966).
#include "gbr_device.cuh"
#include "gbr_kernels.h"
#include "gbr_shade.cuh"

namespace gbr {

__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31u; }

__device__ __forceinline__ uint32_t find_mesh(const FrameDev& F, uint32_t prim) {
    uint32_t lo = 0, hi = F.num_meshes - 1u;
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1u) >> 1;
        if (__ldg(&F.meshes[mid].prim_base) <= prim) lo = mid; else hi = mid - 1u;
    }
    return lo;
}

// Walks the bins of a packed rectangle; warp-aggregates equal bins.
// Mode 0: count (atomicAdd on counts), mode 1: fill (append entry),
// mode 2: predicted fill (append within a predicted capacity).
template <int MODE>
__device__ __forceinline__ void bin_walk(const FrameDev& F, uint2 rect, uint32_t entry, bool valid) {
    int bx0 = (int)(rect.x & 0xFFFFu), bx1 = (int)(rect.x >> 16);
    int by0 = (int)(rect.y & 0xFFFFu), by1 = (int)((rect.y >> 16) & 0x7FFFu);
    bool more = valid && bx0 <= bx1 && by0 <= by1;
    int bx = bx0, by = by0;
    const uint32_t lane = lane_id();
    for (;;) {
        const unsigned act = __ballot_sync(0xFFFFFFFFu, more);
        if (!act) break;
        if (more) {
            const uint32_t bin = (uint32_t)bx + (uint32_t)by * F.nbx;
            const unsigned peers = __match_any_sync(act, bin);
            const uint32_t leader = (uint32_t)(__ffs(peers) - 1);
            const uint32_t n = (uint32_t)__popc(peers);
            if (MODE == 0) {
                if (lane == leader) atomicAdd(&F.counts[bin], n);
            } else {
                uint32_t base = 0;
                if (lane == leader) base = atomicAdd(&F.cursors[bin], n);
                base = __shfl_sync(peers, base, (int)leader);
                const uint32_t pos = base + (uint32_t)__popc(peers & ((1u << lane) - 1u));
                if (MODE == 1) {
                    F.list[pos] = entry;
                } else {
                    // cursors start at the bin's offset; the bin owns capacity[bin] slots
                    if (pos < __ldg(&F.offsets[bin]) + __ldg(&F.capacity[bin])) F.list[pos] = entry;
                    else if (lane == leader) atomicOr(&F.ctl->pred_overflow, 1u);
                }
            }
            if (++bx > bx1) { bx = bx0; if (++by > by1) more = false; }
        }
    }
}

template <int MODE>
__global__ void __launch_bounds__(256) setup_kernel(FrameDev F) {
    const uint32_t prim = blockIdx.x * blockDim.x + threadIdx.x;
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
        }
        F.rects[prim] = rect;
    }
    // frame statistics, one atomic per warp
    const unsigned vis_mask = __ballot_sync(0xFFFFFFFFu, visible);
    const unsigned fp_mask = __ballot_sync(0xFFFFFFFFu, fpath);
    if (lane_id() == 0) {
        if (vis_mask) atomicAdd(&F.ctl->num_visible, (uint32_t)__popc(vis_mask));
        if (fp_mask) atomicAdd(&F.ctl->num_float_path, (uint32_t)__popc(fp_mask));
    }
    if (MODE == 0) bin_walk<0>(F, rect, 0u, visible);
    else bin_walk<2>(F, rect, prim | (no_raster ? kNoRasterBit : 0u), visible);
}

// Single CTA.  counts -> offsets (exclusive, num_bins + 1), cursors, work
// items; zeroes counts for the next frame.  predicted: capacities replace
// counts for the offsets, and items are built later by pred_items.
template <bool PREDICTED>
__global__ void __launch_bounds__(1024) scan_kernel(FrameDev F) {
    __shared__ uint32_t s_a[1024];
    __shared__ uint32_t s_b[1024];
    const uint32_t nb = F.num_bins;
    const uint32_t per = (nb + blockDim.x - 1u) / blockDim.x;
    const uint32_t b0 = threadIdx.x * per;
    const uint32_t b1 = min(b0 + per, nb);
    const uint32_t chunk = F.chunk;
    uint32_t sum = 0, items = 0;
    for (uint32_t b = b0; b < b1; ++b) {
        const uint32_t c = PREDICTED ? F.capacity[b] : F.counts[b];
        sum += c;
        items += c == 0u ? 1u : (c + chunk - 1u) / chunk;
    }
    s_a[threadIdx.x] = sum;
    s_b[threadIdx.x] = items;
    __syncthreads();
    // Hillis-Steele inclusive scan over 1024 partials (counts < 2^32 total)
    for (uint32_t off = 1; off < blockDim.x; off <<= 1) {
        const uint32_t a = threadIdx.x >= off ? s_a[threadIdx.x - off] : 0u;
        const uint32_t c = threadIdx.x >= off ? s_b[threadIdx.x - off] : 0u;
        __syncthreads();
        s_a[threadIdx.x] += a;
        s_b[threadIdx.x] += c;
        __syncthreads();
    }
    uint32_t run = s_a[threadIdx.x] - sum;
    uint32_t item = s_b[threadIdx.x] - items;
    const uint32_t total = s_a[blockDim.x - 1u];
    const uint32_t total_items = s_b[blockDim.x - 1u];
    const bool fits = (unsigned long long)total <= F.list_cap && total_items <= F.items_cap;
    for (uint32_t b = b0; b < b1; ++b) {
        const uint32_t c = PREDICTED ? F.capacity[b] : F.counts[b];
        F.offsets[b] = run;
        F.cursors[b] = run;
        if (!PREDICTED) {
            F.counts[b] = 0u;
            const uint32_t n = c == 0u ? 1u : (c + chunk - 1u) / chunk;
            if (fits)
                for (uint32_t k = 0; k < n; ++k)
                    F.items[item + k] = make_uint4(b, run + k * chunk, min(chunk, c - min(c, k * chunk)), n);
            item += n;
        }
        run += c;
    }
    if (threadIdx.x == 0) {
        F.offsets[nb] = total;
        if (PREDICTED) {
            F.ctl->pred_capacity = total;
            if ((unsigned long long)total > F.list_cap) F.ctl->pred_overflow = 1u;
        } else {
            F.ctl->num_pairs = total;
            F.ctl->num_items = fits ? total_items : 0u;
            F.ctl->item_next = 0u;
            if (!fits) F.ctl->overflow = 1u;
        }
    }
}

__global__ void __launch_bounds__(256) fill_kernel(FrameDev F) {
    if (F.ctl->overflow) return;
    const uint32_t prim = blockIdx.x * blockDim.x + threadIdx.x;
    const bool in_range = prim < F.num_tris;
    const uint2 rect = in_range ? F.rects[prim] : empty_rect();
    const uint32_t entry = prim | ((rect.y & 0x80000000u) ? kNoRasterBit : 0u);
    bin_walk<1>(F, rect, entry, in_range);
}

// ---------------------------------------------------------------------------
// Raster + ROP + shade
// ---------------------------------------------------------------------------
struct RasterShared {
    TriSetup rec[kBatch];
    uint32_t prim[kBatch];
    uint32_t warp_count[kRasterThreads / 32];
    uint32_t warp_max[kRasterThreads / 32];
    uint32_t item[4];
    int next;
    int nv;
    int last;
    uint32_t tile_max;   // max depth key over the tile's pixels (0xFFFFFFFF while any pixel is empty)
};

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
// key of a fragment of the triangle.
__device__ __forceinline__ bool hiz_reject(const TriSetup& t, int minx, int maxx, int miny, int maxy,
                                           uint32_t tile_max) {
    if (tile_max == 0xFFFFFFFFu) return false;
    const float zmin = fminf(t.z0, fminf(t.z1, t.z2));
    if (!(zmin >= 0.f)) return false;
    const float zabs = fmaxf(fabsf(t.z0), fmaxf(fabsf(t.z1), fabsf(t.z2)));
    const float D = (float)((maxx - minx) + (maxy - miny)) * (1.0f / 65536.f) + 1.f;
    const float g = (D * 3.0517578125e-05f + 2.3283064365386963e-10f + D * D * 3.814697265625e-06f) * t.inv_area;
    const float zb = zmin * (1.f - g) - (3.f * g + 2.384185791015625e-07f) * zabs;
    if (!(zb > 0.f)) return false;
    if (zb >= 1.f) return true;
    return (uint32_t)__float2int_rz(__fmul_rn(zb, 2147483648.0f)) > tile_max;
}

__device__ __forceinline__ void raster_fixed(const TriSetup& t, uint32_t prim, unsigned long long* tile, int tx0,
                                             int ty0, int tw, int th, uint32_t lane, uint32_t tile_max) {
    const int X0 = snap_fx(t.x0), Y0 = snap_fx(t.y0), X1 = snap_fx(t.x1);
    const int Y1 = snap_fx(t.y1), X2 = snap_fx(t.x2), Y2 = snap_fx(t.y2);
    const int minx = min(X0, min(X1, X2)), maxx = max(X0, max(X1, X2));
    const int miny = min(Y0, min(Y1, Y2)), maxy = max(Y0, max(Y1, Y2));
    // covered pixels lie in [ceil(min), floor(max)] of the snapped triangle
    const int px0 = max((minx + 0xFFFF) >> kFxBits, tx0), px1 = min(maxx >> kFxBits, tx0 + tw - 1);
    const int py0 = max((miny + 0xFFFF) >> kFxBits, ty0), py1 = min(maxy >> kFxBits, ty0 + th - 1);
    if (px0 > px1 || py0 > py1) return;
    if (hiz_reject(t, minx, maxx, miny, maxy, tile_max)) return;
    const int bwid = px1 - px0 + 1;
    const int lsw = bwid <= 1 ? 0 : bwid <= 2 ? 1 : bwid <= 4 ? 2 : bwid <= 8 ? 3 : bwid <= 16 ? 4 : 5;
    const int sw = 1 << lsw, sh = 32 >> lsw;
    const int lx = (int)lane & (sw - 1), ly = (int)lane >> lsw;
    const int dxa = X1 - X0, dya = Y1 - Y0;
    const int dxb = X2 - X1, dyb = Y2 - Y1;
    const int dxc = X0 - X2, dyc = Y0 - Y2;
    for (int sy = py0; sy <= py1; sy += sh) {
        const int y = sy + ly;
        for (int sx = px0; sx <= px1; sx += sw) {
            const int x = sx + lx;
            if (x > px1 || y > py1) continue;
            const int Px = x << kFxBits, Py = y << kFxBits;
            const long long e2 = edge_fx(Px, Py, X0, Y0, dxa, dya);
            const long long e0 = edge_fx(Px, Py, X1, Y1, dxb, dyb);
            const long long e1 = edge_fx(Px, Py, X2, Y2, dxc, dyc);
            if ((e0 | e1 | e2) < 0) continue;
            float w[3];
            weights_fixed(t, x, y, w);
            const float z = interp_z(w[0], w[1], w[2], t.z0, t.z1, t.z2);
            // the reference rejects z < 0 or z > 1; z == 1 saturates the key to
            // INT_MAX and can never win the depth test (CUDAROPs.cu:343-345, 386)
            if (!(z >= 0.f && z < 1.f)) continue;
            const uint32_t key = (uint32_t)__float2int_rz(__fmul_rn(z, 2147483648.0f));
            const unsigned long long packed = ((unsigned long long)key << 32) | prim;
            unsigned long long* slot = tile + (y - ty0) * tw + (x - tx0);
            if (packed < *((volatile unsigned long long*)slot)) atomicMin(slot, packed);
        }
    }
}

// Triangles outside the guard band: the reference's float edge functions.
__device__ __forceinline__ void raster_float(const TriSetup& t, uint32_t prim, unsigned long long* tile, int tx0,
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

__device__ __forceinline__ void resolve_pixel(const FrameDev& F, int x, int y, unsigned long long v) {
    const size_t gi = (size_t)y * F.width + (size_t)x;
    if (v == kEmptyVis) {
        F.colour[gi] = F.vis == 0u ? F.clear_colour32 : 0u;
        F.depth[gi] = 0.f;
        F.ids[gi] = kInvalidPrim;
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
    F.colour[gi] = shade_fragment(F, m, prim, w, z);
    F.depth[gi] = z;
    F.ids[gi] = prim;
}

__global__ void __launch_bounds__(kRasterThreads, 2) raster_kernel(FrameDev F) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    RasterShared& S = *reinterpret_cast<RasterShared*>(smem_raw);
    unsigned long long* tile = reinterpret_cast<unsigned long long*>(smem_raw + sizeof(RasterShared));
    if (F.ctl->overflow) return;
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    const uint32_t num_items = F.ctl->num_items;
    for (;;) {
        if (tid == 0) {
            const uint32_t idx = atomicAdd(&F.ctl->item_next, 1u);
            const uint4 it = idx < num_items ? F.items[idx] : make_uint4(0xFFFFFFFFu, 0u, 0u, 0u);
            S.item[0] = it.x; S.item[1] = it.y; S.item[2] = it.z; S.item[3] = it.w;
        }
        __syncthreads();
        const uint32_t bin = S.item[0];
        if (bin == 0xFFFFFFFFu) break;
        const uint32_t start = S.item[1], count = S.item[2], nchunks = S.item[3];
        const int tx0 = (int)((bin % F.nbx) * F.bw), ty0 = (int)((bin / F.nbx) * F.bh);
        const int tw = min((int)F.bw, (int)F.width - tx0), th = min((int)F.bh, (int)F.height - ty0);
        const int npx = (tw > 0 && th > 0) ? tw * th : 0;
        for (int i = (int)tid; i < npx; i += kRasterThreads) tile[i] = kEmptyVis;
        for (uint32_t b0 = 0; b0 < count && npx > 0; b0 += kBatch) {
            __syncthreads();
            const uint32_t n = min((uint32_t)kBatch, count - b0);
            const uint32_t e = tid < n ? __ldg(F.list + start + b0 + tid) : kNoRasterBit;
            const bool keep = !(e & kNoRasterBit);
            const unsigned bal = __ballot_sync(0xFFFFFFFFu, keep);
            if (lane == 0) S.warp_count[warp] = (uint32_t)__popc(bal);
            if (tid == 0) S.next = 0;
            __syncthreads();
            uint32_t base = 0, total = 0;
#pragma unroll
            for (uint32_t w = 0; w < kRasterThreads / 32; ++w) {
                const uint32_t c = S.warp_count[w];
                base += w < warp ? c : 0u;
                total += c;
            }
            if (keep) {
                const uint32_t pos = base + (uint32_t)__popc(bal & ((1u << lane) - 1u));
                const uint4* rp = reinterpret_cast<const uint4*>(F.setup) + 3u * e;
                uint4* dst = reinterpret_cast<uint4*>(&S.rec[pos]);
                dst[0] = __ldg(rp);
                dst[1] = __ldg(rp + 1);
                dst[2] = __ldg(rp + 2);
                S.prim[pos] = e;
            }
            __syncthreads();
            // phases of kPhase triangles; the tile's max depth key is refreshed
            // between phases for the hierarchical-z test
            for (uint32_t p0 = 0; p0 < total; p0 += kPhase) {
                const uint32_t p1 = min(total, p0 + kPhase);
                if (b0 > 0 || p0 > 0) {
                    uint32_t m = 0;
                    for (int i = (int)tid; i < npx; i += kRasterThreads)
                        m = max(m, (uint32_t)(tile[i] >> 32));
                    m = __reduce_max_sync(0xFFFFFFFFu, m);
                    if (lane == 0) S.warp_max[warp] = m;
                }
                if (tid == 0) S.next = (int)p0;
                __syncthreads();
                uint32_t tile_max = 0xFFFFFFFFu;
                if (b0 > 0 || p0 > 0) {
                    tile_max = 0;
#pragma unroll
                    for (uint32_t w = 0; w < kRasterThreads / 32; ++w) tile_max = max(tile_max, S.warp_max[w]);
                }
                for (;;) {
                    int i = 0;
                    if (lane == 0) i = atomicAdd(&S.next, 1);
                    i = __shfl_sync(0xFFFFFFFFu, i, 0);
                    if (i >= (int)p1) break;
                    const TriSetup& t = S.rec[i];
                    if (t.flags & kFlagFloat) raster_float(t, S.prim[i], tile, tx0, ty0, tw, th, lane);
                    else raster_fixed(t, S.prim[i], tile, tx0, ty0, tw, th, lane, tile_max);
                }
                __syncthreads();
            }
        }
        __syncthreads();
        if (npx > 0) {
            if (nchunks == 1u) {
                for (int i = (int)tid; i < npx; i += kRasterThreads)
                    resolve_pixel(F, tx0 + i % tw, ty0 + i / tw, tile[i]);
            } else {
                for (int i = (int)tid; i < npx; i += kRasterThreads) {
                    const unsigned long long v = tile[i];
                    if (v != kEmptyVis)
                        atomicMin(&F.gvis[(size_t)(ty0 + i / tw) * F.width + (size_t)(tx0 + i % tw)], v);
                }
                __threadfence();
                __syncthreads();
                if (tid == 0) S.last = atomicAdd(&F.bin_done[bin], 1u) == nchunks - 1u;
                __syncthreads();
                if (S.last) {
                    __threadfence();
                    for (int i = (int)tid; i < npx; i += kRasterThreads) {
                        const int x = tx0 + i % tw, y = ty0 + i / tw;
                        const unsigned long long v = atomicExch(&F.gvis[(size_t)y * F.width + (size_t)x], kEmptyVis);
                        resolve_pixel(F, x, y, v);
                    }
                    if (tid == 0) F.bin_done[bin] = 0u;
                }
            }
        }
        __syncthreads();
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
// Launchers
// ---------------------------------------------------------------------------
size_t raster_smem_bytes(uint32_t bw, uint32_t bh) {
    return sizeof(RasterShared) + (size_t)bw * bh * sizeof(unsigned long long);
}

cudaError_t launch_setup(const FrameDev& F, bool predicted, cudaStream_t s) {
    const uint32_t blocks = (F.num_tris + 255u) / 256u;
    if (blocks == 0) return cudaSuccess;
    if (predicted) setup_kernel<1><<<blocks, 256, 0, s>>>(F);
    else setup_kernel<0><<<blocks, 256, 0, s>>>(F);
    return cudaGetLastError();
}

cudaError_t launch_scan(const FrameDev& F, bool predicted, cudaStream_t s) {
    if (predicted) scan_kernel<true><<<1, 1024, 0, s>>>(F);
    else scan_kernel<false><<<1, 1024, 0, s>>>(F);
    return cudaGetLastError();
}

cudaError_t launch_fill(const FrameDev& F, cudaStream_t s) {
    const uint32_t blocks = (F.num_tris + 255u) / 256u;
    if (blocks == 0) return cudaSuccess;
    fill_kernel<<<blocks, 256, 0, s>>>(F);
    return cudaGetLastError();
}

cudaError_t launch_raster(const FrameDev& F, uint32_t grid, cudaStream_t s) {
    raster_kernel<<<grid, kRasterThreads, raster_smem_bytes(F.bw, F.bh), s>>>(F);
    return cudaGetLastError();
}

cudaError_t launch_clear(const FrameDev& F, cudaStream_t s) {
    clear_kernel<<<1024, 256, 0, s>>>(F);
    return cudaGetLastError();
}

cudaError_t raster_configure(uint32_t bw, uint32_t bh, int* blocks_per_sm) {
    const size_t smem = raster_smem_bytes(bw, bh);
    cudaError_t e = cudaFuncSetAttribute(raster_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, raster_kernel, kRasterThreads, smem);
}

}  // namespace gbr
