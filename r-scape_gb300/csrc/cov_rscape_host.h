// cov_rscape_host.h -- the host steps of the E-valued path for one
// statistic of one alignment (internal), shared by covgpu_rscape and the
// family batch (covgpu_rscape_families):
//   rs_nshuffle    R-scape's null count rule (src/R-scape.c:2449-2459)
//   rs_width       calculate_width_histo on the first null and the bins of
//                  the cumulative null (src/R-scape.c:1353-1360,
//                  src/covariation.c:348-374)
//   rs_histogram   the cumulative null histogram from the device's bin
//                  counts, the tail mass and the tail by mass; the
//                  exponential fit when it is asked for
//                  (src/covariation.c:414-466, 1914-1973)
//   rs_tables      the result fields, the score at the E-value threshold
//                  and the cov2evalue tail table
#pragma once
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <vector>

#include "cov_kernels.h"
#include "covgpu.h"
#include "rscape_cov.h"

struct RsStat {
  bool active = false;
  double w = 0.0, xmin = INFINITY, xmax = -INFINITY;
  int nbcum = 0, nb_real = 0, wbase = 0;
  int64_t obs_off = 0, sf_off = 0, tail_off = 0;
  ESL_HISTOGRAM* h = nullptr;   // owned by the caller (covh_Destroy)
  double pmass = 0.0, newmass = 0.0, mu = 0.0, lambda = 0.0, tau = 0.0;
  int evals = 0;
  bool have_sf = false;
};

int rs_nshuffle(const covgpu_params* p, int N, int L, double* fracfit);
// mm: [slot][ntypes][2] (min, max) of the corrected scores; 0 or 30 (err set)
int rs_width(const covgpu_params* p, int N, int ns, const double* mm, int ntypes, int q, covgpu_result& R,
             RsStat& X, char* err, size_t errlen);
// ob: the nbcum bin counts of the nulls; 0, 5, 31 or 32 (err set)
int rs_histogram(const covgpu_params* p, double fracfit, int ns, int64_t P, const uint64_t* ob, RsStat& X, char* err,
                 size_t errlen);
// sf: the host copy of the survival table (read when X.have_sf); tq: nb
// entries of the tail table; Nb of the P pairs are the structure's (the
// two-set test), the other P - Nb the tests of the remaining pairs
void rs_tables(const covgpu_params* p, int64_t P, int64_t Nb, RsStat& X, const double* sf, covgpu_result& R,
               double* tq);
covgpu::EvalTables rs_evaltables(const covgpu_params* p, int64_t Nt, const RsStat& X, const double* d_sf,
                                 const double* d_tail);
// the two-set test's pairs from p's contacts over the L(L-1)/2 pairs in
// scan order: bpmask, pairs whose first contact is a base pair for the
// sample (the hit list's rule); *nsel, pairs with any such contact (the
// ranking's classes, Nb).  Empty without contacts or with samplesize 3.
// 0, or 11 (err set).
int rs_pair_sets(const covgpu_params* p, int L, std::vector<uint32_t>& bpmask, int64_t* nsel, char* err,
                 size_t errlen);
