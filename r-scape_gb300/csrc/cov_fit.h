// cov_fit.h -- GPU pieces of the null-tail fit (internal).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace covgpu {

struct FitWork;
FitWork* fitwork_create();
void     fitwork_destroy(FitWork* fw);

// binned ML gamma fit of the tail bins [cmin, imax] of the histogram with
// counts h_obs, location mu = phi, likelihood evaluated on the device, in
// two steps: the launch (inputs copied, search launched, result copied back
// asynchronously; 0, 1 empty tail or 90 CUDA error) and, once the caller has
// synchronised the stream, the result (0, 2 barrier timeout, or the
// search's status)
int gamma_fit_launch(FitWork* fw, const uint64_t* h_obs, int cmin, int imax, double bmin, double w, double phi,
                     cudaStream_t st);
int gamma_fit_collect(FitWork* fw, double* ret_lambda, double* ret_tau, int* ret_evals);

// survfit table [2 nb] of a gamma (doexp = 0) or exponential tail
cudaError_t launch_survfit(int cmin, int nb, double bmin, double w, double mass, int doexp, double mu, double lambda,
                           double tau, double* d_sf, cudaStream_t st);

// aggregated p-value of each helix (pairs d_off[h] .. d_off[h+1]-1 of
// d_pval): method 0 Fisher, 1 Lancaster (d_aux: substitutions per pair),
// 2 weighted Fisher (d_aux: power per pair), 3 Sidak; d_term scratch [2 nbp]
cudaError_t launch_aggregate(int method, int nh, const int* d_off, const double* d_pval, const double* d_aux,
                             double* d_term, double* d_pagg, cudaStream_t st);

}  // namespace covgpu
