// cov_umma.h -- tensor-core (tcgen05) counting of the pair count tensor.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "cov_dev.cuh"

namespace covgpu {

struct UmmaPlan;

// nullptr when the shape cannot be served by the tensor path
// a plan for alignments of N x L, with buffers for up to capN sequences,
// capLp padded columns and capntiles tiles
UmmaPlan*   umma_plan_create(int N, int L, int Lp, int nT, const TileRC* d_tiles, int ntiles, int maxslots, int capN,
                             int capLp, int capntiles);
// the plan for other dimensions within its capacity; false if they do not fit
bool        umma_plan_resize(UmmaPlan* p, int N, int L, int Lp, int nT, int ntiles);
void        umma_plan_destroy(UmmaPlan* p);
void        umma_set_weights(UmmaPlan* p, const double* wgt, int N, cudaStream_t st);
// counts of nslots alignments (slot stride in bytes of the code buffer) into
// cnt [slot][tile][16][TPP]; unit = unit weights (RAF), counted on FP8 E4M3
// one-hot operands; ev0/ev1 (optional) are recorded around the weighted
// count kernel itself
// (unit counts: only the cells of cellmask, bit 4x + y, are stored)
cudaError_t umma_count(UmmaPlan* p, const uint8_t* ax, int64_t slot_stride, int nslots, bool unit, float* cnt,
                       cudaStream_t st, cudaEvent_t ev0 = nullptr, cudaEvent_t ev1 = nullptr,
                       unsigned cellmask = 0xFFFFu);
// error code recorded by the kernel (0 = none; 101-105 = a barrier wait
// timed out); reading it resets it
int         umma_error(UmmaPlan* p);
// times the weighted count for each raster super-block size in cand and
// keeps the fastest (0 ok, 11 bad candidate, 90 CUDA error)
int         umma_autotune(UmmaPlan* p, const uint8_t* ax, int64_t slot_stride, int nslots, float* cnt,
                          cudaStream_t st, const int* cand, int ncand, int reps, float* ms, int* best_sb);

}  // namespace covgpu
