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
//   capacity_tc_kernel  12 features per bin from those accumulators -> MLP
//                    12-64-64-1 (ReLU, softplus out) on the tensor cores:
//                    tcgen05.mma with BF16 operands in shared memory and
//                    FP32 accumulators in tensor memory, 128 bins per CTA
//                    -> predicted count l -> capacity
//                    ceil(l*(1+alpha) + beta*sqrt(l+1) + gamma), at most
//                    the triangle count (capacity_kernel, one warp per bin
//                    with FP32 math, only collects the features);
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

// Features of every bin (and, with `predict`, its capacity), one bin per
// warp.  predict 1: the model, its BF16 parameters copied to shared memory
// once per block with 16-byte loads; predict 2: no model, the predicted
// count is the plain estimate from the pre-pass (sampled pairs x the
// sampling stride, feature 0 x 256).
__global__ void __launch_bounds__(256) capacity_kernel(FrameDev F, int predict) {
    __shared__ __align__(16) uint16_t w[kMlpParamsPadded];
    __shared__ float h1s[8][kMlpHidden];
    pdl_wait();
    if (predict == 1) {
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
        const float l = predict == 1 ? softplus(mlp_forward_warp(w, x, h1s[warp])) : x[0] * 256.f;
        if (lane != 0) continue;
        const float cap = ceilf(l * (1.f + F.cap_alpha) + F.cap_beta * sqrtf(l + 1.f) + F.cap_gamma);
        // a bin never holds more than every triangle; an undefined prediction
        // gets that bound too
        const float most = (float)F.num_tris;
        F.capacity[b] = (uint32_t)(cap == cap ? fminf(fmaxf(cap, 0.f), most) : most);
    }
}

// ---------------------------------------------------------------------------
// Capacity inference on the tensor cores (tcgen05, accumulators in TMEM)
// ---------------------------------------------------------------------------
// One CTA of 128 threads takes 128 bins: thread t computes bin t's
// features into row t of the layer-1 operand.  Layer 1 is one
// tcgen05.mma (M 128, N 64, K 16: the 12 features padded with zeros),
// layer 2 four (K 64), each BF16 x BF16 with FP32 accumulation into tensor
// memory (columns 0-63 and 64-127 of a 128-column allocation).  Thread t
// reads row t back (TMEM lane t: warp w owns lanes 32w..32w+31), adds the
// bias and applies ReLU in FP32; the hidden layer is rounded to BF16 as the
// next MMA's operand; the 64 -> 1 output layer, softplus and the capacity
// rule run in FP32 registers.  Operands sit in shared memory in the
// canonical no-swizzle K-major layout: 8 x 8 core matrices of 16-byte rows,
// consecutive in K (leading offset 128 B), then in M / N (stride offset
// K / 8 x 128 B).  The two waits on the MMAs' mbarrier are bounded: one
// that gives up flags Ctl::error and leaves the CTA's bins at the triangle
// count.
namespace tc {

constexpr uint32_t kM = 128, kN = 64, kK1 = 16, kK2 = 64;
constexpr uint32_t kWaitLimit = 1u << 22;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// byte offset of element (row, k) of a K-major tile with `kdim` columns
__device__ __forceinline__ uint32_t kmajor_offset(uint32_t row, uint32_t k, uint32_t kdim) {
    return (row >> 3) * (kdim / 8u) * 128u + (k >> 3) * 128u + (row & 7u) * 16u + (k & 7u) * 2u;
}

// shared-memory matrix descriptor: start, leading and stride byte offsets
// (all >> 4), descriptor version 1, no swizzle
__device__ __forceinline__ unsigned long long smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (unsigned long long)((addr >> 4) & 0x3FFFu) | ((unsigned long long)((lbo >> 4) & 0x3FFFu) << 16) |
           ((unsigned long long)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// kind::f16 instruction descriptor: FP32 accumulator, BF16 A and B, both
// K-major, N and M
__host__ __device__ constexpr uint32_t instr_desc(uint32_t m, uint32_t n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((n >> 3) << 17) | ((m >> 4) << 24);
}

__device__ __forceinline__ void mma(uint32_t d_tmem, unsigned long long a, unsigned long long b, uint32_t idesc,
                                    uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void commit(uint32_t mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar) : "memory");
}

// waits for phase `parity` of the mbarrier; false when the bound ran out
__device__ __forceinline__ bool wait(uint32_t mbar, uint32_t parity) {
    for (uint32_t it = 0; it < kWaitLimit; ++it) {
        uint32_t done = 0;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(mbar), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ void ld16(uint32_t taddr, uint32_t* r) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                 : "r"(taddr)
                 : "memory");
}

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ uint16_t bf16_bits(float f) { return __bfloat16_as_ushort(__float2bfloat16_rn(f)); }

}  // namespace tc

__global__ void __launch_bounds__(128) capacity_tc_kernel(FrameDev F) {
    using namespace tc;
    __shared__ __align__(128) unsigned char sA1[kM * kK1 * 2];   // features (bf16)
    __shared__ __align__(128) unsigned char sB1[kN * kK1 * 2];   // W1^T
    __shared__ __align__(128) unsigned char sA2[kM * kK2 * 2];   // hidden layer (bf16)
    __shared__ __align__(128) unsigned char sB2[kN * kK2 * 2];   // W2^T
    __shared__ float sb1[kN], sb2[kN], sw3[kN];
    __shared__ __align__(8) unsigned long long s_mbar;
    __shared__ uint32_t s_tmem;
    pdl_wait();
    const uint32_t tid = threadIdx.x, warp = tid >> 5;
    const uint16_t* w = F.mlp_w;
    // W1^T (n = hidden unit, k = feature, zero past feature 11) and W2^T
    for (uint32_t i = tid; i < kN * kK1; i += blockDim.x) {
        const uint32_t n = i / kK1, k = i % kK1;
        const uint16_t v = k < (uint32_t)kFeatures ? w[kOffW1 + k * kMlpHidden + n] : (uint16_t)0;
        *reinterpret_cast<uint16_t*>(sB1 + kmajor_offset(n, k, kK1)) = v;
    }
    for (uint32_t i = tid; i < kN * kK2; i += blockDim.x) {
        const uint32_t n = i / kK2, k = i % kK2;
        *reinterpret_cast<uint16_t*>(sB2 + kmajor_offset(n, k, kK2)) = w[kOffW2 + k * kMlpHidden + n];
    }
    if (tid < kN) {
        sb1[tid] = bf16_to_f32(w[kOffB1 + tid]);
        sb2[tid] = bf16_to_f32(w[kOffB2 + tid]);
        sw3[tid] = bf16_to_f32(w[kOffW3 + tid]);
    }
    // this thread's bin: its features as row `tid` of the layer-1 operand
    const uint32_t b = blockIdx.x * kM + tid;
    float x[kFeatures];
#pragma unroll
    for (int k = 0; k < kFeatures; ++k) x[k] = 0.f;
    if (b < F.num_bins) bin_features(F, b, x);
#pragma unroll
    for (uint32_t k = 0; k < kK1; ++k)
        *reinterpret_cast<uint16_t*>(sA1 + kmajor_offset(tid, k, kK1)) = k < (uint32_t)kFeatures ? bf16_bits(x[k]) : 0;
    const uint32_t mbar = smem_u32(&s_mbar);
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 128;" ::"r"(smem_u32(&s_tmem))
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_async_smem();   // the operands written above, to the tensor cores' (async) proxy
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = s_tmem;
    constexpr uint32_t idesc = instr_desc(kM, kN);
    if (tid == 0) {
        mma(tmem, smem_desc(smem_u32(sA1), 128u, (kK1 / 8u) * 128u), smem_desc(smem_u32(sB1), 128u, (kK1 / 8u) * 128u),
            idesc, 0u);
        commit(mbar);
    }
    bool ok = wait(mbar, 0u);
    fence_after();
    const uint32_t lane_base = (warp * 32u) << 16;   // TMEM lane field
    uint32_t r[16];
    if (ok) {
#pragma unroll
        for (uint32_t c = 0; c < kN; c += 16) {
            ld16(tmem + lane_base + c, r);
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
            for (uint32_t j = 0; j < 16; ++j) {
                const float h = fmaxf(__uint_as_float(r[j]) + sb1[c + j], 0.f);
                *reinterpret_cast<uint16_t*>(sA2 + kmajor_offset(tid, c + j, kK2)) = bf16_bits(h);
            }
        }
    }
    fence_async_smem();
    fence_before();
    __syncthreads();
    fence_after();
    ok = __syncthreads_and(ok ? 1 : 0) != 0;   // every thread saw layer 1 arrive
    if (ok && tid == 0) {
#pragma unroll
        for (uint32_t s = 0; s < kK2 / 16u; ++s)
            mma(tmem + kN, smem_desc(smem_u32(sA2) + s * 256u, 128u, (kK2 / 8u) * 128u),
                smem_desc(smem_u32(sB2) + s * 256u, 128u, (kK2 / 8u) * 128u), idesc, s > 0 ? 1u : 0u);
        commit(mbar);
    }
    if (ok) ok = wait(mbar, 1u);
    fence_after();
    float y = bf16_to_f32(w[kOffB3]);
    if (ok) {
#pragma unroll
        for (uint32_t c = 0; c < kN; c += 16) {
            ld16(tmem + lane_base + kN + c, r);
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
            for (uint32_t j = 0; j < 16; ++j) y = __fmaf_rn(fmaxf(__uint_as_float(r[j]) + sb2[c + j], 0.f), sw3[c + j], y);
        }
    }
    if (b < F.num_bins) {
        const float most = (float)F.num_tris;
        float cap = most;   // a bin the model could not score gets the bound
        if (ok) {
            const float l = softplus(y);
            const float c = ceilf(l * (1.f + F.cap_alpha) + F.cap_beta * sqrtf(l + 1.f) + F.cap_gamma);
            cap = c == c ? fminf(fmaxf(c, 0.f), most) : most;
        }
        F.capacity[b] = (uint32_t)cap;
    }
    if (!ok && tid == 0) atomicOr(&F.ctl->error, 2u);
    fence_before();
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 128;" ::"r"(tmem) : "memory");
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
    if (predict && F.mlp_w)   // the model on the tensor cores, 128 bins per CTA
        return launch_pdl(capacity_tc_kernel, dim3(std::max<uint32_t>((F.num_bins + 127u) / 128u, 1u)), dim3(128), 0, s, F);
    // features only (training data), or capacities from the sampled counts:
    // 8 warps per block, one bin per warp
    const uint32_t blocks = std::min<uint32_t>((F.num_bins + 7u) / 8u, 4096u);
    return launch_pdl(capacity_kernel, dim3(blocks ? blocks : 1u), dim3(256), 0, s, F, predict ? 2 : 0);
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
