// gbr_kernels.h -- host-side launchers of the frame kernels (gbr_kernels.cu).
#pragma once
#include <cuda_runtime.h>

#include "gbr_device.cuh"

namespace gbr {

size_t raster_smem_bytes(uint32_t bw, uint32_t bh);
cudaError_t raster_configure(uint32_t bw, uint32_t bh, int* blocks_per_sm);
cudaError_t launch_setup(const FrameDev& F, bool predicted, cudaStream_t s);
cudaError_t launch_scan(const FrameDev& F, bool predicted, cudaStream_t s);
cudaError_t launch_fill(const FrameDev& F, cudaStream_t s);
cudaError_t launch_raster(const FrameDev& F, uint32_t grid, cudaStream_t s);
cudaError_t launch_clear(const FrameDev& F, cudaStream_t s);

// Message returned by gbr_last_error_string() on the calling thread.
void set_last_error(const char* msg);

}  // namespace gbr
