// gbr_predict.h -- layout of the bin-capacity model and the launchers of
// gbr_predict.cu.
#pragma once
#include <cuda_runtime.h>

#include "gbr_device.cuh"

namespace gbr {

constexpr int kFeatures = 12;   // per-bin features (gbr_predict.cu: bin_features)
constexpr int kMlpHidden = 64;
// parameter offsets: W1[12][64], b1[64], W2[64][64], b2[64], W3[64], b3
constexpr int kOffW1 = 0;
constexpr int kOffB1 = kOffW1 + kFeatures * kMlpHidden;
constexpr int kOffW2 = kOffB1 + kMlpHidden;
constexpr int kOffB2 = kOffW2 + kMlpHidden * kMlpHidden;
constexpr int kOffW3 = kOffB2 + kMlpHidden;
constexpr int kOffB3 = kOffW3 + kMlpHidden;
constexpr int kMlpParams = kOffB3 + 1;                       // 5057
constexpr int kMlpParamsPadded = (kMlpParams + 7) / 8 * 8;   // 5064
constexpr int kGradSamples = 64;                             // samples per gradient block
constexpr int kFeatSlots = 6;   // pre-pass accumulators per bin: sampled pairs, centroid count,
                                // bbox area sum, bbox area max, depth min, depth max
constexpr uint32_t kSampleStride = 8;

cudaError_t launch_prepass(const FrameDev& F, cudaStream_t s);
cudaError_t launch_capacity(const FrameDev& F, bool predict, cudaStream_t s);
cudaError_t launch_feat_reset(const FrameDev& F, cudaStream_t s);
cudaError_t launch_mlp_predict(const uint16_t* w, const float* x, uint32_t n, float* out, cudaStream_t s);
cudaError_t launch_mlp_grad(const uint16_t* w, const float* x, const float* y, uint32_t n, float* grad, float* loss,
                            cudaStream_t s);
cudaError_t launch_mlp_adam(float* master, uint16_t* wq, const float* grad, float* m, float* v, uint32_t step, float lr,
                            float grad_scale, cudaStream_t s);

}  // namespace gbr
