// cov_sim.h -- the P(t) alignment simulator (internal).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace covgpu {

// per-branch conditionals P4 [nbranch][4][4], P16 [nbranch][16][16] of the
// rate matrices Q4, Q16 at the branch times, their inverse-CDF thresholds
// C4, C16, and the thresholds R4, R16 of the backgrounds pi4, pi16; status
// gets 41 (negative time) or 42 (P needed regularisation beyond -1e-3)
cudaError_t launch_sim_tables(const double* Q4, const double* Q16, const double* pi4, const double* pi16,
                              const double* times, int nbranch, double* P4, double* P16, unsigned long long* C4,
                              unsigned long long* C16, unsigned long long* R4, unsigned long long* R16, int* status,
                              cudaStream_t st);

// nrep alignments: units (column, partner or -1) evolved down the tree from
// root (or the background when root is null), depth by depth (device list of
// internal nodes by depth, host offsets level_off[nlevels + 1]), leaves into
// out (slot stride out_slot_stride, rows Lp), then gap runs; state is
// scratch [nrep][N-1][nunits]
cudaError_t launch_sim_evolve(const int* left, const int* right, const int* level_nodes, const int* level_off,
                              int nlevels, int N, int L, int Lp, const int2* units, int nunits,
                              const unsigned long long* C4, const unsigned long long* C16,
                              const unsigned long long* R4, const unsigned long long* R16, const uint8_t* root,
                              double gap_rate, double gap_mean, uint64_t seed, uint32_t first_rep, int nrep,
                              uint8_t* state, uint8_t* out, int64_t out_slot_stride, cudaStream_t st);

}  // namespace covgpu
