// cov_prep.h -- sequence weights and the gap filter on the device (internal).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace covgpu {

// unnormalised position-based weights w[N] of the alignment ax [N][Lp]
// (inv is scratch [L][4])
cudaError_t launch_weights_pb(const uint8_t* ax, int N, int L, int Lp, double* inv, double* w, cudaStream_t st);
// unnormalised GSC weights w[N] (scratch of gsc_scratch_bytes(N, L) bytes,
// 16-byte aligned)
size_t      gsc_scratch_bytes(int N, int L);
cudaError_t launch_weights_gsc(const uint8_t* ax, int N, int L, int Lp, void* scratch, double* w, cudaStream_t st);
// after launch_weights_gsc: nonzero when a grid barrier of the UPGMA timed out
int         gsc_error(const void* scratch, cudaStream_t st);
// useme[L]: 1 where the weighted residue fraction is at least 1 - gapthresh
// (wgt null: unit weights)
cudaError_t launch_gapfilter(const uint8_t* ax, const double* wgt, int N, int L, int Lp, double gapthresh, int* useme,
                             cudaStream_t st);

}  // namespace covgpu
