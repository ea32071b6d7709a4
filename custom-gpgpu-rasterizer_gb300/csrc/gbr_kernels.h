// gbr_kernels.h -- host-side launchers of the frame kernels (gbr_kernels.cu).
#pragma once
#include <cuda_runtime.h>

#include "gbr_device.cuh"

namespace gbr {

size_t raster_smem_bytes(uint32_t bw, uint32_t bh);
cudaError_t raster_configure(uint32_t bw, uint32_t bh, int* blocks_per_sm);
// ctas: the raster_kernel variant compiled for 2..6 CTAs per SM (0: default)
cudaError_t raster_configure(uint32_t bw, uint32_t bh, uint32_t ctas, int* blocks_per_sm);
cudaError_t launch_setup(const FrameDev& F, bool predicted, cudaStream_t s);
// The bin scan of a frame (mode: kScanExact, ...) and its three launches.
ScanDev scan_of(const FrameDev& F, uint32_t mode);
uint32_t scan_blocks(uint32_t num_bins);   // blocks of 1024 bins; FrameDev::scan_partial holds 2 per block
cudaError_t launch_scan(const ScanDev& S, cudaStream_t s);
cudaError_t launch_fill(const FrameDev& F, cudaStream_t s);
cudaError_t launch_raster(const FrameDev& F, uint32_t grid, cudaStream_t s);
cudaError_t launch_clear(const FrameDev& F, cudaStream_t s);

// Grid sizes of a batch frame (see BatchDev).
struct BatchLaunch {
    uint32_t tri_blocks;    // setup / fill blocks of all scenes
    uint32_t px_blocks;     // shade blocks of all scenes
    uint32_t raster_grid;   // persistent raster CTAs
    uint32_t raster_ctas;   // raster variant (CTAs per SM it is compiled for; 0: default)
    uint32_t bin_w, bin_h;  // the largest bin of the batch (shared-memory tile)
    ScanDev scan;           // the scan over the bins of every scene
};
// reset, setup + count, bin scan (three launches), fill, raster, shade
cudaError_t launch_batch(const BatchDev& B, const BatchLaunch& L, cudaStream_t s);
cudaError_t raster_configure_batch(uint32_t bw, uint32_t bh, uint32_t ctas, int* blocks_per_sm);

// Message returned by gbr_last_error_string() on the calling thread.
void set_last_error(const char* msg);

}  // namespace gbr
