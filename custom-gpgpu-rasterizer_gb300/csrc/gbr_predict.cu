// gbr_predict.cu -- learned per-bin capacity for single-pass binning.
//
// Exact binning reads every triangle twice (count pass, then fill pass) with
// one global atomic per (triangle, bin) pair in each.  Predicted binning
// replaces the count pass:
//   prepass_kernel   one triangle from each group of sample_stride
//                    consecutive triangles (drawn by a hash of the group)
//                    goes through the vertex stage and binning rule; per
//                    bin it accumulates the
//                    sampled pair count, and per centroid bin the count,
//                    bounding-box area (sum, max) and depth range;
//   capacity_kernel  12 features per bin from those accumulators -> MLP
//                    12-64-64-1 (ReLU, softplus out; parameters BF16, math
//                    FP32) -> predicted count l -> capacity
//                    ceil(l*(1+alpha) + beta*sqrt(l+1) + gamma), at most
//                    the triangle count;
//   scan (capacities) -> one fused setup + fill pass appending inside each
//                    bin's capacity -> a scan of the filled sizes builds the
//                    raster work items (gbr_scan.cu, kScanPredictedItems).
// Any append beyond a bin's capacity raises ctl->pred_overflow; the exact
// count / scan / fill kernels are always launched behind it and run only
// then, so an overflowing frame is re-binned exactly on the device with no
// host round trip and its bin lists are identical to exact binning's.
//
// Training kernels (predict, loss + gradient, Adam) work on (features,
// exact count) pairs produced by exact binning; the loss is
// (log1p(l) - log1p(count))^2.
#include <cuda_bf16.h>

#include <algorithm>

#include "gbr_device.cuh"
#include "gbr_kernels.h"
#include "gbr_predict.h"

namespace gbr {

namespace {

__device__ __forceinline__ uint32_t ordered(float f) {
    const uint32_t b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float unordered(uint32_t u) {
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u);
}

__device__ __forceinline__ float bf16_to_f32(uint16_t h) { return __uint_as_float((uint32_t)h << 16); }

__device__ __forceinline__ uint32_t mesh_of(const FrameDev& F, uint32_t prim) {
    uint32_t lo = 0, hi = F.num_meshes - 1u;
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1u) >> 1;
        if (__ldg(&F.meshes[mid].prim_base) <= prim) lo = mid; else hi = mid - 1u;
    }
    return lo;
}

// Loads the BF16 parameters into shared memory as floats.
__device__ __forceinline__ void load_params(const uint16_t* w, float* s) {
    for (int i = threadIdx.x; i < kMlpParams; i += blockDim.x) s[i] = bf16_to_f32(w[i]);
    __syncthreads();
}

// Hidden layer 1 and the pre-softplus output; h1 is kept for the backward pass.
__device__ __forceinline__ float mlp_forward(const float* w, const float* x, float* h1) {
#pragma unroll 4
    for (int j = 0; j < kMlpHidden; ++j) {
        float a = w[kOffB1 + j];
#pragma unroll
        for (int k = 0; k < kFeatures; ++k) a = __fmaf_rn(x[k], w[kOffW1 + k * kMlpHidden + j], a);
        h1[j] = fmaxf(a, 0.f);
    }
    float y = w[kOffB3];
    for (int j = 0; j < kMlpHidden; ++j) {
        float a = w[kOffB2 + j];
#pragma unroll 8
        for (int i = 0; i < kMlpHidden; ++i) a = __fmaf_rn(h1[i], w[kOffW2 + i * kMlpHidden + j], a);
        y = __fmaf_rn(fmaxf(a, 0.f), w[kOffW3 + j], y);
    }
    return y;
}

__device__ __forceinline__ float softplus(float y) { return y > 20.f ? y : log1pf(expf(y)); }

}  // namespace

// ---------------------------------------------------------------------------
// Frame kernels
// ---------------------------------------------------------------------------
// Integer hash (a 32-bit finaliser: xor-shift / multiply rounds).
__device__ __forceinline__ uint32_t hash32(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7FEB352Du;
    x ^= x >> 15;
    x *= 0x846CA68Bu;
    x ^= x >> 16;
    return x;
}

__global__ void __launch_bounds__(256) prepass_kernel(FrameDev F) {
    // one triangle drawn from each group of sample_stride consecutive
    // triangles: a fixed stride would alias with structured index orders
    // (a subdivided mesh numbers its children level by level, so every 8th
    // triangle falls on a few of the base faces only)
    pdl_wait();
    const uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t first = idx * F.sample_stride;
    uint32_t prim = first + hash32(idx) % F.sample_stride;
    if (prim >= F.num_tris) prim = first;
    const uint32_t lane = threadIdx.x & 31u;
    bool visible = false;
    int4 r = make_int4(1, 1, 0, 0);
    uint32_t cbin = 0;
    float area = 0.f, zc = 0.f;
    if (prim < F.num_tris) {
        const MeshDev& m = F.meshes[mesh_of(F, prim)];
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
        bool culled = false;
        if (F.cull != 2u) {
            const F3 a = f3(__fsub_rn(nx[1], nx[0]), __fsub_rn(ny[1], ny[0]), __fsub_rn(nz[1], nz[0]));
            const F3 b = f3(__fsub_rn(nx[2], nx[0]), __fsub_rn(ny[2], ny[0]), __fsub_rn(nz[2], nz[0]));
            culled = dot3(f3(F.cam_fwd[0], F.cam_fwd[1], F.cam_fwd[2]), normalize3(cross3(a, b))) <= 0.0f;
        }
        const bool ax = (nx[0] < -1.f && nx[1] < -1.f && nx[2] < -1.f) || (nx[0] > 1.f && nx[1] > 1.f && nx[2] > 1.f);
        const bool ay = (ny[0] < -1.f && ny[1] < -1.f && ny[2] < -1.f) || (ny[0] > 1.f && ny[1] > 1.f && ny[2] > 1.f);
        const bool az = (nz[0] < 0.f && nz[1] < 0.f && nz[2] < 0.f) || (nz[0] > 1.f && nz[1] > 1.f && nz[2] > 1.f);
        visible = !culled && !ax && !ay && !az;
        if (visible) {
            const float2 s0 = to_screen(nx[0], ny[0], F.width, F.height);
            const float2 s1 = to_screen(nx[1], ny[1], F.width, F.height);
            const float2 s2 = to_screen(nx[2], ny[2], F.width, F.height);
            r = bin_rect(s0, s1, s2, F);
            const float cx = (s0.x + s1.x + s2.x) * (1.f / 3.f), cy = (s0.y + s1.y + s2.y) * (1.f / 3.f);
            const int bx = clampi((int)floorf(cx / (float)F.bw), 0, (int)F.nbx - 1);
            const int by = clampi((int)floorf(cy / (float)F.bh), 0, (int)F.nby - 1);
            cbin = (uint32_t)bx + (uint32_t)by * F.nbx;
            area = (max3f(s0.x, s1.x, s2.x) - min3f(s0.x, s1.x, s2.x)) * (max3f(s0.y, s1.y, s2.y) - min3f(s0.y, s1.y, s2.y));
            zc = (nz[0] + nz[1] + nz[2]) * (1.f / 3.f);
            if (!(area == area) || area > 1e12f) area = 1e12f;
            if (!(zc == zc)) zc = 0.f;
        }
    }
    // sampled visible triangles: one atomic per block
    __shared__ uint32_t s_sampled;
    if (threadIdx.x == 0) s_sampled = 0u;
    __syncthreads();
    const unsigned vis = __ballot_sync(0xFFFFFFFFu, visible);
    if (lane == 0 && vis) atomicAdd(&s_sampled, (uint32_t)__popc(vis));
    __syncthreads();
    if (threadIdx.x == 0 && s_sampled) atomicAdd(&F.ctl->num_sampled, s_sampled);
    const uint32_t nb = F.num_bins;
    if (visible) {
        atomicAdd(&F.feat[1u * nb + cbin], 1u);
        atomicAdd(reinterpret_cast<float*>(&F.feat[2u * nb + cbin]), area);
        atomicMax(&F.feat[3u * nb + cbin], __float_as_uint(area));
        atomicMin(&F.feat[4u * nb + cbin], ordered(zc));
        atomicMax(&F.feat[5u * nb + cbin], ordered(zc));
    }
    // sampled (triangle, bin) pairs
    bin_walk<3>(F, visible ? pack_rect(r, false) : empty_rect(), 0u, visible, 0u);
}

// The kFeatures features of bin b (shared by inference and training data).
__device__ __forceinline__ void bin_features(const FrameDev& F, uint32_t b, float* x) {
    const uint32_t nb = F.num_bins;
    const float s = (float)F.sample_stride;
    const int bx = (int)(b % F.nbx), by = (int)(b / F.nbx);
    auto sc = [&](int x_, int y_) -> float {
        if (x_ < 0 || y_ < 0 || x_ >= (int)F.nbx || y_ >= (int)F.nby) return 0.f;
        return (float)__ldg(&F.feat[(uint32_t)x_ + (uint32_t)y_ * F.nbx]) * s;
    };
    float n9 = 0.f;
    for (int dy = -1; dy <= 1; ++dy)
        for (int dx = -1; dx <= 1; ++dx) n9 += sc(bx + dx, by + dy);
    const uint32_t cc = __ldg(&F.feat[1u * nb + b]);
    const float area_sum = __uint_as_float(__ldg(&F.feat[2u * nb + b]));
    const float area_max = __uint_as_float(__ldg(&F.feat[3u * nb + b]));
    const int tw = min((int)F.bw, (int)F.width - bx * (int)F.bw), th = min((int)F.bh, (int)F.height - by * (int)F.bh);
    // sampled pair estimates on a linear scale (a ReLU network passes them
    // through to the softplus output unchanged where they are right),
    // sizes and densities on a log scale
    const float lin = 1.f / 256.f;
    x[0] = sc(bx, by) * lin;
    x[1] = n9 * (1.f / 9.f) * lin;
    x[2] = log1pf((float)cc * s);
    x[3] = cc ? log1pf(area_sum / (float)cc) : 0.f;
    x[4] = cc ? log1pf(area_max) : 0.f;
    x[5] = cc ? unordered(__ldg(&F.feat[5u * nb + b])) - unordered(__ldg(&F.feat[4u * nb + b])) : 0.f;
    x[6] = sc(bx - 1, by) * lin;
    x[7] = sc(bx + 1, by) * lin;
    x[8] = sc(bx, by - 1) * lin;
    x[9] = sc(bx, by + 1) * lin;
    x[10] = (tw > 0 && th > 0) ? (float)(tw * th) / (float)(F.bw * F.bh) : 0.f;
    x[11] = log1pf((float)F.ctl->num_sampled * s / (float)nb);
    // degenerate geometry (w near 0) can make the area or depth terms
    // infinite: keep every feature finite
#pragma unroll
    for (int k = 0; k < kFeatures; ++k) x[k] = x[k] == x[k] ? fminf(fmaxf(x[k], -1.0e4f), 1.0e4f) : 0.f;
}

// One warp per bin: lane j holds hidden units j and j + 32 of both layers;
// the parameters stay BF16 in shared memory (widened to FP32 on use, FP32
// accumulation), layer-2 inputs come from a per-warp copy of h1 in shared
// memory, the output is a warp reduction.  Every lane returns the
// pre-softplus output.
__device__ __forceinline__ float wbf(const uint16_t* w, int i) { return __uint_as_float((uint32_t)w[i] << 16); }

__device__ __forceinline__ float mlp_forward_warp(const uint16_t* w, const float* x, float* h1s) {
    const int lane = (int)(threadIdx.x & 31u);
    float a = wbf(w, kOffB1 + lane), c = wbf(w, kOffB1 + lane + 32);
#pragma unroll
    for (int k = 0; k < kFeatures; ++k) {
        a = __fmaf_rn(x[k], wbf(w, kOffW1 + k * kMlpHidden + lane), a);
        c = __fmaf_rn(x[k], wbf(w, kOffW1 + k * kMlpHidden + lane + 32), c);
    }
    h1s[lane] = fmaxf(a, 0.f);
    h1s[lane + 32] = fmaxf(c, 0.f);
    __syncwarp();
    float p = wbf(w, kOffB2 + lane), q = wbf(w, kOffB2 + lane + 32);
#pragma unroll 16
    for (int i = 0; i < kMlpHidden; ++i) {
        const float h = h1s[i];
        p = __fmaf_rn(h, wbf(w, kOffW2 + i * kMlpHidden + lane), p);
        q = __fmaf_rn(h, wbf(w, kOffW2 + i * kMlpHidden + lane + 32), q);
    }
    __syncwarp();   // h1s is reused by the warp's next bin
    float y = __fmaf_rn(fmaxf(p, 0.f), wbf(w, kOffW3 + lane), __fmul_rn(fmaxf(q, 0.f), wbf(w, kOffW3 + lane + 32)));
#pragma unroll
    for (int d = 16; d >= 1; d >>= 1) y += __shfl_xor_sync(0xFFFFFFFFu, y, d);
    return y + wbf(w, kOffB3);
}

// Features of every bin (and, with `predict`, the model's capacity), one
// bin per warp, the BF16 parameters copied to shared memory once per block
// with 16-byte loads.
__global__ void __launch_bounds__(256) capacity_kernel(FrameDev F, int predict) {
    __shared__ __align__(16) uint16_t w[kMlpParamsPadded];
    __shared__ float h1s[8][kMlpHidden];
    pdl_wait();
    if (predict) {
        const uint4* src = reinterpret_cast<const uint4*>(F.mlp_w);
        uint4* dst = reinterpret_cast<uint4*>(w);
        for (int i = (int)threadIdx.x; i < kMlpParamsPadded / 8; i += (int)blockDim.x) dst[i] = __ldg(src + i);
        __syncthreads();
    }
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint32_t nwarps = gridDim.x * (blockDim.x >> 5);
    for (uint32_t b = blockIdx.x * (blockDim.x >> 5) + warp; b < F.num_bins; b += nwarps) {   // warp-uniform
        float x[kFeatures];
        bin_features(F, b, x);
        if (F.features_out && lane == 0)
            for (int k = 0; k < kFeatures; ++k) F.features_out[(size_t)b * kFeatures + k] = x[k];
        if (!predict) continue;
        const float l = softplus(mlp_forward_warp(w, x, h1s[warp]));
        if (lane != 0) continue;
        const float cap = ceilf(l * (1.f + F.cap_alpha) + F.cap_beta * sqrtf(l + 1.f) + F.cap_gamma);
        // a bin never holds more than every triangle; an undefined prediction
        // gets that bound too
        const float most = (float)F.num_tris;
        F.capacity[b] = (uint32_t)(cap == cap ? fminf(fmaxf(cap, 0.f), most) : most);
    }
}

// ---------------------------------------------------------------------------
// Training kernels
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) mlp_predict_kernel(const uint16_t* wq, const float* x, uint32_t n, float* out) {
    __shared__ float w[kMlpParams];
    load_params(wq, w);
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float h1[kMlpHidden];
    out[i] = softplus(mlp_forward(w, x + (size_t)i * kFeatures, h1));
}

// One sample per thread, kGradSamples samples per block; weight gradients
// are sums over the block's samples, added to `grad` with atomics.
__global__ void __launch_bounds__(kGradSamples) mlp_grad_kernel(const uint16_t* wq, const float* x, const float* y,
                                                              uint32_t n, float* grad, float* loss) {
    extern __shared__ float sm[];
    float* w = sm;                                   // kMlpParams
    float* H1 = w + kMlpParamsPadded;                // [kGradSamples][kMlpHidden]: h1, later dh1
    float* D2 = H1 + kGradSamples * kMlpHidden;      // [kGradSamples][kMlpHidden]: h2, later dh2
    float* X = D2 + kGradSamples * kMlpHidden;       // [kGradSamples][kFeatures]
    float* G = X + kGradSamples * kFeatures;         // [kGradSamples]: dL/d(output pre-softplus)
    load_params(wq, w);
    const uint32_t t = threadIdx.x;
    const uint32_t i = blockIdx.x * kGradSamples + t;
    const bool valid = i < n;
    float* h1 = H1 + t * kMlpHidden;
    float* h2 = D2 + t * kMlpHidden;
    float* xs = X + t * kFeatures;
    float g = 0.f, l = 0.f;
    if (valid) {
        for (int k = 0; k < kFeatures; ++k) xs[k] = x[(size_t)i * kFeatures + k];
        for (int j = 0; j < kMlpHidden; ++j) {
            float a = w[kOffB1 + j];
            for (int k = 0; k < kFeatures; ++k) a = __fmaf_rn(xs[k], w[kOffW1 + k * kMlpHidden + j], a);
            h1[j] = fmaxf(a, 0.f);
        }
        float out = w[kOffB3];
        for (int j = 0; j < kMlpHidden; ++j) {
            float a = w[kOffB2 + j];
            for (int k = 0; k < kMlpHidden; ++k) a = __fmaf_rn(h1[k], w[kOffW2 + k * kMlpHidden + j], a);
            h2[j] = fmaxf(a, 0.f);
            out = __fmaf_rn(h2[j], w[kOffW3 + j], out);
        }
        const float lam = softplus(out);
        const float d = log1pf(lam) - log1pf(y[i]);
        l = d * d;
        const float sig = 1.f / (1.f + expf(-out));   // d softplus / d out
        g = 2.f * d / (1.f + lam) * sig;
    } else {
        for (int k = 0; k < kFeatures; ++k) xs[k] = 0.f;
        for (int j = 0; j < kMlpHidden; ++j) { h1[j] = 0.f; h2[j] = 0.f; }
    }
    G[t] = g;
    // loss sum
    float ls = l;
    for (int o = 16; o > 0; o >>= 1) ls += __shfl_xor_sync(0xFFFFFFFFu, ls, o);
    if ((t & 31u) == 0) atomicAdd(loss, ls);
    __syncthreads();
    // output layer: dW3[j] = sum_s g_s h2_s[j], db3 = sum_s g_s
    for (int j = t; j < kMlpHidden; j += kGradSamples) {
        float a = 0.f;
        for (int s = 0; s < kGradSamples; ++s) a = __fmaf_rn(G[s], D2[s * kMlpHidden + j], a);
        atomicAdd(&grad[kOffW3 + j], a);
    }
    if (t == 0) {
        float a = 0.f;
        for (int s = 0; s < kGradSamples; ++s) a += G[s];
        atomicAdd(&grad[kOffB3], a);
    }
    __syncthreads();
    // dh2 = g * W3 * [h2 > 0] (in place)
    for (int j = 0; j < kMlpHidden; ++j) h2[j] = h2[j] > 0.f ? g * w[kOffW3 + j] : 0.f;
    __syncthreads();
    // dW2[k][j] = sum_s h1_s[k] dh2_s[j]; db2[j] = sum_s dh2_s[j]
    for (int e = t; e < kMlpHidden * kMlpHidden; e += kGradSamples) {
        const int k = e / kMlpHidden, j = e % kMlpHidden;
        float a = 0.f;
        for (int s = 0; s < kGradSamples; ++s) a = __fmaf_rn(H1[s * kMlpHidden + k], D2[s * kMlpHidden + j], a);
        atomicAdd(&grad[kOffW2 + e], a);
    }
    for (int j = t; j < kMlpHidden; j += kGradSamples) {
        float a = 0.f;
        for (int s = 0; s < kGradSamples; ++s) a += D2[s * kMlpHidden + j];
        atomicAdd(&grad[kOffB2 + j], a);
    }
    __syncthreads();
    // dh1 = (W2 dh2) * [h1 > 0] (in place)
    for (int k = 0; k < kMlpHidden; ++k) {
        float a = 0.f;
        for (int j = 0; j < kMlpHidden; ++j) a = __fmaf_rn(w[kOffW2 + k * kMlpHidden + j], h2[j], a);
        h1[k] = h1[k] > 0.f ? a : 0.f;
    }
    __syncthreads();
    // dW1[k][j] = sum_s x_s[k] dh1_s[j]; db1[j] = sum_s dh1_s[j]
    for (int e = t; e < kFeatures * kMlpHidden; e += kGradSamples) {
        const int k = e / kMlpHidden, j = e % kMlpHidden;
        float a = 0.f;
        for (int s = 0; s < kGradSamples; ++s) a = __fmaf_rn(X[s * kFeatures + k], H1[s * kMlpHidden + j], a);
        atomicAdd(&grad[kOffW1 + e], a);
    }
    for (int j = t; j < kMlpHidden; j += kGradSamples) {
        float a = 0.f;
        for (int s = 0; s < kGradSamples; ++s) a += H1[s * kMlpHidden + j];
        atomicAdd(&grad[kOffB1 + j], a);
    }
}

// Adam on FP32 master parameters; the BF16 copy the kernels read is
// refreshed from them (round to nearest even).
__global__ void mlp_adam_kernel(float* master, uint16_t* wq, const float* grad, float* m, float* v, uint32_t step,
                                float lr, float grad_scale) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (uint32_t)kMlpParams) return;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    const float g = grad[i] * grad_scale;
    const float mi = b1 * m[i] + (1.f - b1) * g;
    const float vi = b2 * v[i] + (1.f - b2) * g * g;
    m[i] = mi;
    v[i] = vi;
    const float mh = mi / (1.f - powf(b1, (float)step));
    const float vh = vi / (1.f - powf(b2, (float)step));
    const float p = master[i] - lr * mh / (sqrtf(vh) + eps);
    master[i] = p;
    wq[i] = __bfloat16_as_ushort(__float2bfloat16_rn(p));
}

// ---------------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------------
cudaError_t launch_prepass(const FrameDev& F, cudaStream_t s) {
    const uint32_t n = (F.num_tris + F.sample_stride - 1u) / F.sample_stride;
    if (n) return launch_pdl(prepass_kernel, dim3((n + 255u) / 256u), dim3(256), 0, s, F);
    return cudaGetLastError();
}

cudaError_t launch_capacity(const FrameDev& F, bool predict, cudaStream_t s) {
    // 8 warps per block, one bin per warp up to 4096 blocks (then a few)
    const uint32_t blocks = std::min<uint32_t>((F.num_bins + 7u) / 8u, 4096u);
    return launch_pdl(capacity_kernel, dim3(blocks ? blocks : 1u), dim3(256), 0, s, F, predict ? 1 : 0);
    return cudaGetLastError();
}


__global__ void feat_reset_kernel(FrameDev F) {
    const uint32_t nb = F.num_bins;
    for (uint32_t b = blockIdx.x * blockDim.x + threadIdx.x; b < nb; b += gridDim.x * blockDim.x) {
        F.feat[b] = 0u;
        F.feat[1u * nb + b] = 0u;
        F.feat[2u * nb + b] = 0u;
        F.feat[3u * nb + b] = 0u;
        F.feat[4u * nb + b] = 0xFFFFFFFFu;
        F.feat[5u * nb + b] = 0u;
    }
}

cudaError_t launch_feat_reset(const FrameDev& F, cudaStream_t s) {
    feat_reset_kernel<<<(F.num_bins + 255u) / 256u, 256, 0, s>>>(F);
    return cudaGetLastError();
}

cudaError_t launch_mlp_predict(const uint16_t* w, const float* x, uint32_t n, float* out, cudaStream_t s) {
    if (n) mlp_predict_kernel<<<(n + 255u) / 256u, 256, 0, s>>>(w, x, n, out);
    return cudaGetLastError();
}

cudaError_t launch_mlp_grad(const uint16_t* w, const float* x, const float* y, uint32_t n, float* grad, float* loss,
                            cudaStream_t s) {
    const size_t smem = ((size_t)kMlpParamsPadded + 2u * kGradSamples * kMlpHidden + kGradSamples * kFeatures +
                         kGradSamples) * sizeof(float);
    cudaError_t e = cudaFuncSetAttribute(mlp_grad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    if (n) mlp_grad_kernel<<<(n + kGradSamples - 1u) / kGradSamples, kGradSamples, smem, s>>>(w, x, y, n, grad, loss);
    return cudaGetLastError();
}

cudaError_t launch_mlp_adam(float* master, uint16_t* wq, const float* grad, float* m, float* v, uint32_t step, float lr,
                            float grad_scale, cudaStream_t s) {
    mlp_adam_kernel<<<(kMlpParams + 255) / 256, 256, 0, s>>>(master, wq, grad, m, v, step, lr, grad_scale);
    return cudaGetLastError();
}

}  // namespace gbr
