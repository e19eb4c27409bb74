// cov_subst.h -- substitutions on the tree and pair power (internal).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace covgpu {

// ax: the alignment [N][Lp] (leaf rows), F: internal states [N-1][Lp];
// Sb, Ub scratch [L][Wb] (Wb = words of 32 branches); nsubs [L]; ndouble,
// njoin [L][L], upper triangle (i < j), the rest zero
cudaError_t launch_substitutions(const uint8_t* ax, const uint8_t* F, const int* left, const int* right, int N, int L,
                                 int Lp, int includegaps, uint32_t* Sb, uint32_t* Ub, int* nsubs, int* ndouble,
                                 int* njoin, cudaStream_t st);
// per pair i < j (row-major upper triangle): tab = [subs, prob] x (single,
// join, double), ns points each
cudaError_t launch_power(const int* nsubs, const int* ndouble, const int* njoin, int L, int ns, const double* tab,
                         int have_single, int have_join, int have_double, double* power, double* power_join,
                         double* power_double, cudaStream_t st);

}  // namespace covgpu
