// gbr_kernels.h -- host-side launchers of the frame kernels (gbr_kernels.cu).
#pragma once
#include <cuda_runtime.h>

#include "gbr_device.cuh"

namespace gbr {

// Programmatic dependent launch (sm_90+): a kernel started with launch_pdl
// may be scheduled while the kernel before it in the stream is finishing;
// it calls pdl_wait() before it touches anything, which returns once that
// kernel has completed and its writes are visible.  A kernel calls
// pdl_release() when its own work is issued, letting the next one launch.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_release() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                              Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr;
    attr.id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr.val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = &attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, args...);
}

// threads: raster CTA width (128 or 256)
size_t raster_smem_bytes(uint32_t bw, uint32_t bh, uint32_t threads = 256);
cudaError_t raster_configure(uint32_t bw, uint32_t bh, int* blocks_per_sm);
// ctas: the raster_kernel variant compiled for 2..6 CTAs per SM (0: default)
cudaError_t raster_configure(uint32_t bw, uint32_t bh, uint32_t ctas, int* blocks_per_sm);
cudaError_t launch_setup(const FrameDev& F, bool predicted, cudaStream_t s);
// The bin scan of a frame (mode: kScanExact, ...), one launch.
ScanDev scan_of(const FrameDev& F, uint32_t mode);
uint32_t scan_blocks(uint32_t num_bins);   // tiles of 1024 bins
cudaError_t launch_scan(const ScanDev& S, cudaStream_t s);
cudaError_t launch_fill(const FrameDev& F, cudaStream_t s);
// Zeros the frame's list entries ahead of a scattering fill pass (see
// list_touch_kernel); worth its launch once a frame holds ~1M entries.
constexpr unsigned long long kListTouchMinPairs = 1ull << 20;
cudaError_t launch_list_touch(const FrameDev& F, cudaStream_t s);
cudaError_t launch_raster(const FrameDev& F, uint32_t grid, cudaStream_t s);
cudaError_t launch_shade(const FrameDev& F, cudaStream_t s);
cudaError_t launch_clear(const FrameDev& F, cudaStream_t s);

// Grid sizes of a batch frame (see BatchDev).
struct BatchLaunch {
    uint32_t tri_blocks;    // setup / fill blocks of all scenes
    uint32_t px_blocks;     // shade blocks of all scenes
    uint32_t raster_grid;   // persistent raster CTAs
    uint32_t raster_ctas;   // raster variant (CTAs per SM it is compiled for; 0: default)
    uint32_t raster_threads;   // raster CTA width: 128 or 256
    uint32_t bin_w, bin_h;  // the largest bin of the batch (shared-memory tile)
    ScanDev scan;           // the scan over the bins of every scene
};
// reset, setup + count, bin scan (three launches), fill, raster, shade
cudaError_t launch_batch(const BatchDev& B, const BatchLaunch& L, cudaStream_t s);
cudaError_t raster_configure_batch(uint32_t bw, uint32_t bh, uint32_t ctas, uint32_t threads, int* blocks_per_sm);

// Message returned by gbr_last_error_string() on the calling thread.
void set_last_error(const char* msg);

}  // namespace gbr
