// cov_learn.h -- alignment summary features for the learned null (internal).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace covgpu {

constexpr int kNFeat = 64;        // features per alignment
constexpr int kIdentPairs = 4096; // sequence pairs sampled for the identity features

// doubles of scratch launch_features needs for L columns
size_t feat_scratch_doubles(int L);

// the 64 features of the alignment ax [N][Lp] (first L columns) with weights
// w[N]; tree_len is the caller's tree-length summary
cudaError_t launch_features(const uint8_t* ax, int N, int L, int Lp, const double* w, double tree_len,
                            double* scratch, float* feat, cudaStream_t st);

}  // namespace covgpu
