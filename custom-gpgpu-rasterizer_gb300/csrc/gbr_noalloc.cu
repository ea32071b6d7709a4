// gbr_noalloc.cu -- gbr_render_noalloc: one frame rendered into caller
// buffers without any device allocation.
//
// Who needs it: callers that may not allocate device memory while they
// render -- an engine or media pipeline that owns a fixed device-memory
// budget and forbids library allocations, a real-time loop that cannot
// afford cudaMalloc's implicit device synchronisation and latency spikes,
// or a process running under a hard memory cap where an allocation could
// fail in the middle of a frame.  gbr_create/gbr_setup_bins allocate their
// frame storage; this entry point instead uses one file-scope device array
// (g_scratch below) that the CUDA runtime reserves when the library is
// loaded, on every GPU that loads it, until the process exits.
//
// Limits (the scratch array is sized for them, about 20 MiB): at most
// kNaMaxTris triangles, kNaMaxBins bins, kNaMaxPixels pixels, kNaMaxPairs
// (triangle, bin) entries, bins of at most 64x64 pixels and a queue chunk of
// at least kNaMinChunk.  Larger inputs are rejected before any GPU work.
//
// Set-up: the first call on a device, with that device current, looks up
// the device address of g_scratch (cudaGetSymbolAddress); make that first
// call before any stream capture.  Every call shares g_scratch and leaves
// its last contents there: each call first clears the parts that must start
// empty (bin counters, the merge tile, the control block), and calls whose
// work overlaps on the GPU (different streams, or different host threads on
// the same device) race on it and must be serialised by the caller.
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>

#include "../../include/gbr.h"
#include "gbr_internal.h"
#include "gbr_kernels.h"

using namespace gbr;

namespace {

constexpr uint32_t kNaMaxTris = 65536u;
constexpr uint32_t kNaMaxBins = 4096u;
constexpr uint32_t kNaMaxPixels = 1u << 20;
constexpr uint32_t kNaMaxPairs = 1u << 20;
constexpr uint32_t kNaMinChunk = 64u;
constexpr uint32_t kNaMaxItems = kNaMaxBins + kNaMaxPairs / kNaMinChunk + 1u;
constexpr int kNaMaxDevices = 64;

constexpr size_t align256(size_t x) { return (x + 255u) & ~size_t(255u); }
constexpr size_t kOffSetup = 0;
constexpr size_t kOffRects = kOffSetup + align256(size_t(kNaMaxTris) * sizeof(TriSetup));
constexpr size_t kOffCounts = kOffRects + align256(size_t(kNaMaxTris) * sizeof(uint2));
constexpr size_t kOffSubBase = kOffCounts + align256(size_t(kCountSplit) * kNaMaxBins * 4u);
constexpr size_t kOffOffsets = kOffSubBase + align256(size_t(kCountSplit) * kNaMaxBins * 4u);
constexpr size_t kOffCursors = kOffOffsets + align256(size_t(kNaMaxBins + 1u) * 4u);
constexpr size_t kOffCapacity = kOffCursors + align256(size_t(kNaMaxBins) * 4u);
constexpr size_t kOffBinDone = kOffCapacity + align256(size_t(kNaMaxBins) * 4u);
constexpr size_t kOffItems = kOffBinDone + align256(size_t(kNaMaxBins) * 4u);
constexpr size_t kOffList = kOffItems + align256(size_t(kNaMaxItems) * sizeof(uint4));
constexpr size_t kOffGvis = kOffList + align256(size_t(kNaMaxPairs) * 4u);
constexpr size_t kOffIds = kOffGvis + align256(size_t(kNaMaxPixels) * 8u);
constexpr size_t kOffCtl = kOffIds + align256(size_t(kNaMaxPixels) * 4u);
constexpr size_t kOffMesh = kOffCtl + align256(sizeof(Ctl));
constexpr size_t kOffScan = kOffMesh + align256(sizeof(MeshDev));
constexpr size_t kOffRanks = kOffScan + align256(scan_state_bytes(kNaMaxBins));
constexpr size_t kOffWalk = kOffRanks + align256(size_t(kNaMaxPairs) * 4u);
constexpr size_t kOffKeys = kOffWalk + align256(size_t(kNaMaxTris / 32u + 8u) * 4u);
constexpr size_t kScratchBytes = kOffKeys + align256(size_t(kNaMaxTris) * 4u);

// The only device memory this entry point uses besides the caller's.
static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

struct DeviceSlot {
    bool ready = false;
    unsigned char* base = nullptr;
    int num_sms = 0;
};
std::mutex g_mu;
DeviceSlot g_slots[kNaMaxDevices];

gbr_status na_fail(gbr_status st, const char* msg) {
    set_last_error(msg);  // read back through gbr_last_error_string()
    return st;
}

// Clears what must start empty and stores the mesh descriptor.
__global__ void noalloc_prepare_kernel(FrameDev F, MeshDev desc, uint32_t npx) {
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < npx; i += stride) F.gvis[i] = kEmptyVis;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < F.num_bins; i += stride) {
#pragma unroll
        for (uint32_t k = 0; k < kCountSplit; ++k) F.counts[k * F.num_bins + i] = 0u;
        F.bin_end[i] = 0u;
    }
    // the caller's scratch: the bin scan state starts zeroed every frame
    uint32_t* scan = reinterpret_cast<uint32_t*>(F.scan_state);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < scan_state_bytes(F.num_bins) / 4u; i += stride)
        scan[i] = 0u;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        *const_cast<MeshDev*>(F.meshes) = desc;
        memset(F.ctl, 0, sizeof(Ctl));
    }
}

}  // namespace

extern "C" gbr_status gbr_render_noalloc(const void* d_vertices, uint32_t num_vertices, uint32_t vertex_format,
                                         const uint32_t* d_indices, uint32_t num_indices, uint32_t topology,
                                         const float world[16], const gbr_camera* cam, uint32_t width,
                                         uint32_t height, uint32_t num_bins_x, uint32_t num_bins_y, uint32_t bin_w,
                                         uint32_t bin_h, uint32_t queue_chunk, uint32_t cull, uint32_t sample,
                                         uint32_t vis, uint32_t* d_colour, float* d_depth, uint32_t* d_ids,
                                         void* stream) {
    if (!d_vertices || !world || !cam || !d_colour || !d_depth) return na_fail(GBR_ERR_INVALID_ARG, "null argument");
    if (vertex_format > GBR_VERTEX_POS3_RGBA8 || topology > GBR_TOPOLOGY_TRIANGLE_STRIP ||
        (!d_indices && topology != GBR_TOPOLOGY_TRIANGLE_LIST) || cull > GBR_CULL_NONE || sample > GBR_SAMPLE_BILINEAR ||
        vis > GBR_VIS_NORMAL)
        return na_fail(GBR_ERR_INVALID_ARG, "bad vertex format, topology or render state");
    const uint64_t tris = !d_indices ? num_vertices / 3u
                          : topology == GBR_TOPOLOGY_TRIANGLE_LIST ? num_indices / 3u
                          : (num_indices >= 2u ? num_indices - 2u : 0u);
    const uint64_t npx = (uint64_t)width * height, nb = (uint64_t)num_bins_x * num_bins_y;
    if (tris > kNaMaxTris) return na_fail(GBR_ERR_INVALID_ARG, "more than 65536 triangles");
    if (width == 0 || height == 0 || width > 8192u || height > 8192u || npx > kNaMaxPixels)
        return na_fail(GBR_ERR_INVALID_ARG, "resolution above 2^20 pixels");
    if (nb == 0 || nb > kNaMaxBins || bin_w == 0 || bin_h == 0 || bin_w > (uint32_t)kMaxBinDim ||
        bin_h > (uint32_t)kMaxBinDim)
        return na_fail(GBR_ERR_INVALID_ARG, "bins: 1..4096 bins of 1..64 pixels");
    if (queue_chunk < kNaMinChunk) return na_fail(GBR_ERR_INVALID_ARG, "queue_chunk below 64");
    if (vertex_format == GBR_VERTEX_POS3_RGBA8 && ((uintptr_t)d_vertices & 15u))
        return na_fail(GBR_ERR_INVALID_ARG, "compact vertices must be 16-byte aligned");

    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return na_fail(GBR_ERR_CUDA, cudaGetErrorString(e));
    if (dev < 0 || dev >= kNaMaxDevices) return na_fail(GBR_ERR_INVALID_ARG, "device ordinal above 63");
    DeviceSlot slot;
    {
        std::lock_guard<std::mutex> lock(g_mu);
        DeviceSlot& s = g_slots[dev];
        if (!s.ready) {
            void* base = nullptr;
            e = cudaGetSymbolAddress(&base, g_scratch);
            if (e != cudaSuccess) return na_fail(GBR_ERR_CUDA, cudaGetErrorString(e));
            e = cudaDeviceGetAttribute(&s.num_sms, cudaDevAttrMultiProcessorCount, dev);
            if (e != cudaSuccess) return na_fail(GBR_ERR_CUDA, cudaGetErrorString(e));
            s.base = static_cast<unsigned char*>(base);
            s.ready = true;
        }
        slot = s;
    }
    int blocks_per_sm = 0;
    e = raster_configure(bin_w, bin_h, &blocks_per_sm);
    if (e != cudaSuccess) return na_fail(GBR_ERR_CUDA, cudaGetErrorString(e));

    unsigned char* b = slot.base;
    FrameDev F;
    memset(&F, 0, sizeof F);
    F.width = width; F.height = height;
    F.nbx = num_bins_x; F.nby = num_bins_y; F.bw = bin_w; F.bh = bin_h; F.num_bins = (uint32_t)nb;
    F.cull = cull; F.sample = sample; F.vis = vis; F.clear_colour32 = 0x003F3F3Fu;
    // an untextured mesh in the PBR view shades from its vertex colours, as
    // the regular entry point does (frame_basics)
    F.flat_shade = vis == GBR_VIS_PBR ? 1u : 0u;
    F.num_meshes = 1u;
    F.num_tris = (uint32_t)tris;
    F.chunk = kMaxChunk;      // work items: the library's split
    F.stage = queue_chunk;    // entries per raster pass
    for (int k = 0; k < 3; ++k) { F.cam_pos[k] = cam->pos[k]; F.cam_fwd[k] = cam->fwd[k]; }
    F.meshes = reinterpret_cast<const MeshDev*>(b + kOffMesh);
    F.setup = reinterpret_cast<TriSetup*>(b + kOffSetup);
    F.rects = reinterpret_cast<uint2*>(b + kOffRects);
    F.keys = reinterpret_cast<uint32_t*>(b + kOffKeys);
    F.counts = reinterpret_cast<uint32_t*>(b + kOffCounts);
    F.sub_base = reinterpret_cast<uint32_t*>(b + kOffSubBase);
    F.count_stride = F.num_bins;
    F.count_split = 1u;   // no frame history: one counter per bin
    F.offsets = reinterpret_cast<uint32_t*>(b + kOffOffsets);
    F.cursors = reinterpret_cast<uint32_t*>(b + kOffCursors);
    F.capacity = reinterpret_cast<uint32_t*>(b + kOffCapacity);
    F.bin_end = reinterpret_cast<uint32_t*>(b + kOffBinDone);
    F.items = reinterpret_cast<uint4*>(b + kOffItems);
    F.items_cap = kNaMaxItems;
    F.list = reinterpret_cast<uint32_t*>(b + kOffList);
    F.list_cap = kNaMaxPairs;
    F.gvis = reinterpret_cast<unsigned long long*>(b + kOffGvis);
    F.ids = d_ids ? d_ids : reinterpret_cast<uint32_t*>(b + kOffIds);
    F.ctl = reinterpret_cast<Ctl*>(b + kOffCtl);
    F.scan_state = reinterpret_cast<ScanState*>(b + kOffScan);
    F.ranks = reinterpret_cast<uint32_t*>(b + kOffRanks);
    F.rank_cap = kNaMaxPairs;
    F.walk_base = reinterpret_cast<uint32_t*>(b + kOffWalk);
    F.rank_next = &reinterpret_cast<Ctl*>(b + kOffCtl)->rank_next;
    F.colour = d_colour;
    F.depth = d_depth;

    MeshDev desc;
    memset(&desc, 0, sizeof desc);
    desc.vertices = d_vertices;
    desc.indices = d_indices;
    desc.vertex_format = vertex_format;
    desc.topology = topology;
    desc.num_vertices = num_vertices;
    desc.num_tris = (uint32_t)tris;
    float vp[16];
    // WVP exactly as the regular entry point builds it (culling and bin
    // rectangles depend on its rounding)
    mat4_mul(cam->proj, cam->view, vp);
    mat4_mul(vp, world, desc.wvp);
    memcpy(desc.world, world, sizeof desc.world);

    cudaStream_t s = (cudaStream_t)stream;
    noalloc_prepare_kernel<<<256, 256, 0, s>>>(F, desc, (uint32_t)npx);
    e = cudaGetLastError();
    if (e == cudaSuccess && ((uint64_t)num_bins_x * bin_w < width || (uint64_t)num_bins_y * bin_h < height))
        e = launch_clear(F, s);
    if (e == cudaSuccess) e = launch_setup(F, false, s);
    if (e == cudaSuccess) e = launch_scan(scan_of(F, kScanExact), s);
    if (e == cudaSuccess) e = launch_fill(F, s);
    if (e == cudaSuccess) e = launch_raster(F, (uint32_t)(slot.num_sms * (blocks_per_sm > 0 ? blocks_per_sm : 1)), s);
    if (e == cudaSuccess) e = launch_shade(F, s);
    if (e != cudaSuccess) return na_fail(GBR_ERR_CUDA, cudaGetErrorString(e));
    // the frame is only valid if its bin entries fitted the static storage
    e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return na_fail(GBR_ERR_CUDA, cudaGetErrorString(e));
    Ctl ctl;
    e = cudaMemcpy(&ctl, b + kOffCtl, sizeof ctl, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return na_fail(GBR_ERR_CUDA, cudaGetErrorString(e));
    if (ctl.overflow) return na_fail(GBR_ERR_OUT_OF_MEMORY, "frame needs more than 2^20 bin entries");
    if (ctl.error) return na_fail(GBR_ERR_TIMEOUT, "bin scan wait timed out; the frame is invalid");
    return GBR_OK;
}
