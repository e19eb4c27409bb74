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

// a batch of gamma fits, one block each, launched together (the same search
// as gamma_fit_launch on a grid of one block): launch, then, once the
// caller has synchronised the stream, collect fit k (0, 1 empty tail, 2
// barrier timeout, or the search's status)
struct FitReq { const uint64_t* obs; int cmin, imax; double bmin, w, phi; };
struct FitBatch;
FitBatch* fitbatch_create();
void      fitbatch_destroy(FitBatch* fb);
int gamma_fit_batch_launch(FitBatch* fb, int nfit, const FitReq* req, cudaStream_t st);
int gamma_fit_batch_collect(FitBatch* fb, int k, double* ret_lambda, double* ret_tau, int* ret_evals);

// survival tables of a batch of tails (entry e: 2 nb values into sf; pre:
// device prefix of the entries' blocks of 256 values)
struct SurvReq { int cmin, nb, doexp; double bmin, w, mass, mu, lambda, tau, lga; double* sf; };
cudaError_t grp_survfit(const SurvReq* d_req, const int* pre, int nr, int nb, cudaStream_t st);

// survfit table [2 nb] of a gamma (doexp = 0) or exponential tail
cudaError_t launch_survfit(int cmin, int nb, double bmin, double w, double mass, int doexp, double mu, double lambda,
                           double tau, double* d_sf, cudaStream_t st);

// aggregated p-value of each helix (pairs d_off[h] .. d_off[h+1]-1 of
// d_pval): method 0 Fisher, 1 Lancaster (d_aux: substitutions per pair),
// 2 weighted Fisher (d_aux: power per pair), 3 Sidak; d_term scratch [2 nbp]
cudaError_t launch_aggregate(int method, int nh, const int* d_off, const double* d_pval, const double* d_aux,
                             double* d_term, double* d_pagg, cudaStream_t st);

}  // namespace covgpu
