// cov_fit.cu -- binned maximum-likelihood gamma fit of the null tail with
// the likelihood evaluated on the GPU (FP64).
//
// esl_gam_FitCompleteBinned (called at src/covariation.c:1956) is restated
// as: location mu = phi (the tail's lower bound, fixed), rate lambda and
// shape tau maximising sum_b obs_b log(S(lo_b) - S(hi_b)) over the tail bins
// [cmin, imax], S(x) = Q(tau, lambda (x - mu)); Nelder-Mead (1965) on
// (log lambda, log tau) from moment estimates.  The whole search (Newton
// rounds, Nelder-Mead if they do not converge; see k_gam_fit) is one
// cooperative launch: each round evaluates all its likelihood points
// together, each block summing a fixed chunk of the non-empty tail bins;
// after a grid barrier every block adds the block sums in the same fixed
// order, so all blocks hold bit-identical likelihoods and take the same
// decisions without a second barrier.  Results do not depend on timing.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "cov_dev.cuh"
#include "cov_fit.h"

namespace covgpu {

// regularised upper incomplete gamma Q(a, x): series for x < a + 1, Lentz's
// continued fraction otherwise (Abramowitz & Stegun 6.5.29, 6.5.31)
__device__ double gamma_q_dev(double a, double x, double lga) {
  if (x <= 0.0) return 1.0;
  if (x < a + 1.0) {
    double sum = 1.0 / a, del = sum, ap = a;
    for (int n = 0; n < 10000; n++) {
      ap += 1.0; del *= x / ap; sum += del;
      if (fabs(del) < fabs(sum) * 1e-16) break;
    }
    return 1.0 - sum * exp(-x + a * log(x) - lga);
  }
  double b = x + 1.0 - a, c = 1.0 / 1e-300, d = 1.0 / b, h = d;
  for (int i = 1; i < 10000; i++) {
    const double an = -i * (i - a);
    b += 2.0;
    d = an * d + b; if (fabs(d) < 1e-300) d = 1e-300;
    c = b + an / c; if (fabs(c) < 1e-300) c = 1e-300;
    d = 1.0 / d;
    const double del = d * c;
    h *= del;
    if (fabs(del - 1.0) < 1e-16) break;
  }
  return exp(-x + a * log(x) - lga) * h;
}

struct FitPoint { double lambda, tau, lga, lconst; };   // lconst = tau log lambda - lgamma(tau)

// log of the gamma probability of the bin [lo, lo + h), location mu, with
// logx = log(lo - mu) when lo > mu.
// Far enough above mu (h <= (lo - mu) / 16, lambda h <= 1/2) the probability
// is computed as f(x) * integral_0^h exp(g(t)) dt,  x = lo - mu,
//   g(t) = (tau - 1) log(1 + t/x) - lambda t,
// with exp(g) = sum_k c_k t^k from (x + t) E' = (tau - 1 - lambda (x + t)) E:
//   c_{k+1} = ((tau - 1 - lambda x - k) c_k - lambda c_{k-1}) / (x (k + 1)),
// summed as d_k = c_k h^k, which needs one log and avoids the cancellation
// of Q(lo) - Q(hi); closer to mu the difference of Q is used.
__constant__ double c_inv[64];   // c_inv[k] = 1 / (k + 1)

__device__ double gam_logp_bin(double lo, double h, double mu, double logx, const FitPoint& P) {
  const double x = lo - mu;
  if (x > 0.0 && h <= 0.0625 * x && P.lambda * h <= 0.5) {
    const double r = h / x, s = P.lambda * h;
    double dkm1 = 0.0, dk = 1.0, sum = 1.0;
    for (int k = 0; k < 60; k++) {
      const double dk1 = (((P.tau - 1.0 - k) * r - s) * dk - s * r * dkm1) * c_inv[k];
      const double term = dk1 * c_inv[k + 1];
      sum += term;
      dkm1 = dk; dk = dk1;
      if (fabs(term) <= 1e-17 * fabs(sum)) break;
    }
    return P.lconst + (P.tau - 1.0) * logx - P.lambda * x + log(h * sum);
  }
  const double l = (lo < mu) ? mu : lo, hi = lo + h;
  const double slo = (l <= mu) ? 1.0 : gamma_q_dev(P.tau, P.lambda * (l - mu), P.lga);
  const double shi = (hi <= mu) ? 1.0 : gamma_q_dev(P.tau, P.lambda * (hi - mu), P.lga);
  const double p = slo - shi;
  return log(p > 0.0 ? p : 1e-300);
}

__device__ __forceinline__ uint64_t fit_clock() {
  uint64_t t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

constexpr uint64_t kFitWaitNs = 2000000000ull;   // grid barrier gives up after 2 s
constexpr int kFitMaxPts = 6;                      // likelihood points per evaluation round

struct FitOut { double lambda, tau; int evals, status; };

struct FitGrid {
  const int* bins;       // non-empty tail bins, in bin order
  const double* cnts;    // their counts
  double* logx;          // scratch: log(lower bound - mu) per bin
  int nnz;
  double bmin, w, mu;
  double* part;          // [2][6][gridDim.x] block sums
  unsigned* bar;         // arrival counter, zero at launch
  FitOut* out;
};

// evaluates the npts points in pts (shared) over the tail.  The work items
// (point q, bin k), point-major, are spread over all threads of the grid:
// FP64 throughput is per SM, so the grid is sized to use every SM's FP64
// unit before it stacks warps on one.  Each block sums its items per point,
// arrives at the grid barrier, then adds all block sums in block order into
// F (shared).  False when the barrier timed out.
__device__ bool fit_eval(const FitGrid& g, const FitPoint* pts, int npts, unsigned& phase, double* F, double* red,
                         int* flag, int G, int bid) {
  const int T = G * blockDim.x, nw = blockDim.x >> 5;
  const int nitems = npts * g.nnz;
  double* part = g.part + (size_t)(phase & 1u) * kFitMaxPts * G;
  double acc[kFitMaxPts];
#pragma unroll
  for (int q = 0; q < kFitMaxPts; q++) acc[q] = 0.0;
  for (int it = bid * blockDim.x + threadIdx.x; it < nitems; it += T) {
    const int q = it / g.nnz, k = it - q * g.nnz;
    const int b = g.bins[k];
    const double lo = g.w * b + g.bmin, hi = g.w * (b + 1) + g.bmin;
    const double v = g.cnts[k] * gam_logp_bin(lo, hi - lo, g.mu, g.logx[k], pts[q]);
#pragma unroll
    for (int r = 0; r < kFitMaxPts; r++)
      if (q == r) acc[r] -= v;
  }
  const int warp = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < kFitMaxPts; q++) {
    double a = acc[q];
    for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
    if ((threadIdx.x & 31) == 0) red[warp * kFitMaxPts + q] = a;
  }
  __syncthreads();
  if (threadIdx.x < npts) {
    double t = 0.0;
    for (int i = 0; i < nw; i++) t += red[i * kFitMaxPts + threadIdx.x];
    part[threadIdx.x * G + bid] = t;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    atomicAdd(g.bar, 1u);
    const unsigned target = (phase + 1u) * (unsigned)G;
    uint64_t t0 = 0;
    int ok = 1;
    while (ld_acquire(g.bar) < target) {
      const uint64_t now = fit_clock();
      if (t0 == 0) t0 = now;
      else if (now - t0 > kFitWaitNs) { ok = 0; break; }
    }
    *flag = ok;
  }
  __syncthreads();
  if (!*flag) return false;
  if (threadIdx.x < 32) {
    for (int q = 0; q < npts; q++) {
      double t = 0.0;
      for (int i = threadIdx.x; i < G; i += 32) t += __ldcg(part + q * G + i);
      for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
      if (threadIdx.x == 0) F[q] = t;
    }
  }
  __syncthreads();
  phase++;
  return true;
}

__device__ void fit_set_point(FitPoint* P, double l0, double l1) {
  P->lambda = exp(l0);
  P->tau = exp(l1);
  P->lga = lgamma(P->tau);
  P->lconst = P->tau * log(P->lambda) - P->lga;
}

// thread 0 has written the n simplex coordinates pc; lanes 0..n-1 turn them
// into likelihood points in parallel
__device__ __forceinline__ void fit_set_points(FitPoint* pts, const double (*pc)[2], int n) {
  __syncthreads();
  if ((int)threadIdx.x < n) fit_set_point(&pts[threadIdx.x], pc[threadIdx.x][0], pc[threadIdx.x][1]);
  __syncthreads();
}

// The search.  Phase 1, Newton on theta = (log lambda, log tau): every round
// evaluates the 6-point stencil theta, theta +- h e1, theta +- h e2,
// theta + h (e1 + e2) (h = 1e-5) for the gradient and Hessian by central
// differences, steps -H^-1 g (a scaled gradient step where H is not
// positive definite, steps capped at 1 in log space), and halves a step that
// raised the likelihood's negative; it stops when the step is below 1e-10.
// Phase 2, only when phase 1 did not converge in 40 rounds: Nelder-Mead from
// the best point of phase 1, the same points a sequential Nelder-Mead
// visits, to 1e-12 in F and 1e-9 in theta.
// (G, bid): the blocks of the search and this block's index; a grouped
// launch runs one search per block (G = 1)
__device__ __forceinline__ void gam_fit_body(const FitGrid& g, double s00, double s01, int G, int bid) {
  __shared__ FitPoint pts[kFitMaxPts];
  __shared__ double F[kFitMaxPts], red[8 * kFitMaxPts], pc[kFitMaxPts][2];
  __shared__ int flag, ctl;
  {
    const int T = G * blockDim.x;
    for (int k = bid * blockDim.x + threadIdx.x; k < g.nnz; k += T) {
      const double x = (g.w * g.bins[k] + g.bmin) - g.mu;
      g.logx[k] = (x > 0.0) ? log(x) : 0.0;
    }
  }
  // the bins' log x are read by other blocks' threads: a barrier round with
  // no points publishes them grid-wide
  unsigned phase = 0;
  int evals = 0, status = 0;
  if (!fit_eval(g, pts, 0, phase, F, red, &flag, G, bid)) status = 2;

  // ---- phase 1: Newton ----
  // Steps below kNewtonTol in (log lambda, log tau) end the search: the
  // 6-point stencil's gradient carries the FP64 rounding of -log L (~1e-16
  // |F|) divided by H, which for tails of ~1e5 scores puts the smallest
  // reachable step near 1e-11-1e-10; the oracle's Nelder-Mead stops at ~1e-8.
  constexpr double H = 1e-5, kNewtonTol = 1e-9;
  double th0 = s00, th1 = s01;               // thread 0's state
  double bth0 = s00, bth1 = s01, bF = INFINITY;
  double d0 = 0.0, d1 = 0.0;                 // last step
  int converged = 0;
  for (int r = 0; r < 40 && !status; r++) {
    if (threadIdx.x == 0) {
      pc[0][0] = th0;     pc[0][1] = th1;
      pc[1][0] = th0 + H; pc[1][1] = th1;
      pc[2][0] = th0 - H; pc[2][1] = th1;
      pc[3][0] = th0;     pc[3][1] = th1 + H;
      pc[4][0] = th0;     pc[4][1] = th1 - H;
      pc[5][0] = th0 + H; pc[5][1] = th1 + H;
    }
    fit_set_points(pts, pc, 6);
    if (!fit_eval(g, pts, 6, phase, F, red, &flag, G, bid)) { status = 2; break; }
    evals += 6;
    if (threadIdx.x == 0) {
      ctl = 1;
      const double F0 = F[0];
      if (!(F0 <= bF) && r > 0) {
        // the step raised -log L (or gave NaN): back off towards the best point
        d0 *= 0.5; d1 *= 0.5;
        th0 = bth0 + d0; th1 = bth1 + d1;
        if (fabs(d0) < kNewtonTol && fabs(d1) < kNewtonTol) { th0 = bth0; th1 = bth1; converged = 1; ctl = 0; }
      } else {
        bth0 = th0; bth1 = th1; bF = F0;
        const double g0 = (F[1] - F[2]) / (2.0 * H), g1 = (F[3] - F[4]) / (2.0 * H);
        const double h00 = (F[1] - 2.0 * F0 + F[2]) / (H * H), h11 = (F[3] - 2.0 * F0 + F[4]) / (H * H);
        const double h01 = (F[5] - F[1] - F[3] + F0) / (H * H);
        const double det = h00 * h11 - h01 * h01;
        if (h00 > 0.0 && h11 > 0.0 && det > 0.0) {
          d0 = -(h11 * g0 - h01 * g1) / det;
          d1 = -(h00 * g1 - h01 * g0) / det;
        } else {
          const double sc = fmax(fmax(fabs(h00), fabs(h11)), 1.0);
          d0 = -g0 / sc; d1 = -g1 / sc;
        }
        const double m = fmax(fabs(d0), fabs(d1));
        if (m > 1.0) { d0 /= m; d1 /= m; }
        if (m < kNewtonTol) { converged = 1; ctl = 0; }
        else { th0 = bth0 + d0; th1 = bth1 + d1; }
      }
    }
    __syncthreads();
    if (!ctl) break;
    __syncthreads();
  }

  // ---- phase 2: Nelder-Mead when Newton did not converge ----
  double S[3][2], SF[3];   // the simplex, kept by thread 0
  if (threadIdx.x == 0) {
    flag = converged;
    const double c0 = isfinite(bF) ? bth0 : s00, c1 = isfinite(bF) ? bth1 : s01;
    S[0][0] = c0;       S[0][1] = c1;
    S[1][0] = c0 + 0.5; S[1][1] = c1;
    S[2][0] = c0;       S[2][1] = c1 + 0.5;
    for (int k = 0; k < 3; k++) { pc[k][0] = S[k][0]; pc[k][1] = S[k][1]; }
  }
  __syncthreads();
  const bool need_nm = !flag;
  __syncthreads();
  if (need_nm && !status) {
    fit_set_points(pts, pc, 3);
    if (!fit_eval(g, pts, 3, phase, F, red, &flag, G, bid)) status = 2;
    evals += 3;
    if (threadIdx.x == 0) for (int k = 0; k < 3; k++) SF[k] = F[k];
    for (int it = 0; it < 4000 && !status; it++) {
      int lo = 0, hi = 0, md = 0;
      if (threadIdx.x == 0) {
        for (int k = 1; k < 3; k++) { if (SF[k] < SF[lo]) lo = k; if (SF[k] > SF[hi]) hi = k; }
        md = 3 - lo - hi;
        if (md == lo || md == hi || md < 0 || md > 2)
          md = (hi == 0) ? ((lo == 1) ? 2 : 1) : ((hi == 1) ? ((lo == 0) ? 2 : 0) : ((lo == 0) ? 1 : 0));
        if (fabs(SF[hi] - SF[lo]) <= 1e-12 * (fabs(SF[lo]) + 1e-30) && fabs(S[hi][0] - S[lo][0]) < 1e-9 &&
            fabs(S[hi][1] - S[lo][1]) < 1e-9) {
          ctl = 0;
        } else {
          const double c0 = 0.5 * (S[lo][0] + S[md][0]), c1 = 0.5 * (S[lo][1] + S[md][1]);
          pc[0][0] = c0 + (c0 - S[hi][0]);       pc[0][1] = c1 + (c1 - S[hi][1]);         // reflection
          pc[1][0] = c0 + 2.0 * (c0 - S[hi][0]); pc[1][1] = c1 + 2.0 * (c1 - S[hi][1]);   // expansion
          pc[2][0] = c0 + 0.5 * (S[hi][0] - c0); pc[2][1] = c1 + 0.5 * (S[hi][1] - c1);   // contraction
          ctl = 1;
        }
      }
      __syncthreads();
      if (!ctl) break;
      fit_set_points(pts, pc, 3);
      if (!fit_eval(g, pts, 3, phase, F, red, &flag, G, bid)) { status = 2; break; }
      evals += 3;
      if (threadIdx.x == 0) {
        const double fr = F[0];
        ctl = 1;
        if (fr < SF[lo]) {
          if (F[1] < fr) { S[hi][0] = pc[1][0]; S[hi][1] = pc[1][1]; SF[hi] = F[1]; }
          else           { S[hi][0] = pc[0][0]; S[hi][1] = pc[0][1]; SF[hi] = fr; }
        } else if (fr < SF[md]) {
          S[hi][0] = pc[0][0]; S[hi][1] = pc[0][1]; SF[hi] = fr;
        } else if (F[2] < SF[hi]) {
          S[hi][0] = pc[2][0]; S[hi][1] = pc[2][1]; SF[hi] = F[2];
        } else {   // shrink towards the best vertex
          int nq = 0;
          for (int k = 0; k < 3; k++)
            if (k != lo) {
              pc[nq][0] = S[lo][0] + 0.5 * (S[k][0] - S[lo][0]);
              pc[nq][1] = S[lo][1] + 0.5 * (S[k][1] - S[lo][1]);
              nq++;
            }
          ctl = 2;
        }
      }
      __syncthreads();
      if (ctl == 2) {
        fit_set_points(pts, pc, 2);
        if (!fit_eval(g, pts, 2, phase, F, red, &flag, G, bid)) { status = 2; break; }
        evals += 2;
        if (threadIdx.x == 0) {
          int nq = 0;
          for (int k = 0; k < 3; k++)
            if (k != lo) { S[k][0] = pc[nq][0]; S[k][1] = pc[nq][1]; SF[k] = F[nq]; nq++; }
        }
      }
      __syncthreads();
    }
  }
  if (bid == 0 && threadIdx.x == 0) {
    double l0 = bth0, l1 = bth1;
    if (need_nm) {
      int lo = 0;
      for (int k = 1; k < 3; k++) if (SF[k] < SF[lo]) lo = k;
      l0 = S[lo][0]; l1 = S[lo][1];
    }
    g.out->lambda = exp(l0);
    g.out->tau = exp(l1);
    g.out->evals = evals;
    g.out->status = status;
  }
}

__global__ void __launch_bounds__(256)
k_gam_fit(FitGrid g, double s00, double s01) {
  gam_fit_body(g, s00, s01, (int)gridDim.x, (int)blockIdx.x);
}

// one search per block: fit e of the batch's fits
__global__ void __launch_bounds__(256)
k_gam_fit_grp(const FitGrid* __restrict__ gs, const double2* __restrict__ start) {
  const FitGrid g = gs[blockIdx.x];
  const double2 s0 = start[blockIdx.x];
  gam_fit_body(g, s0.x, s0.y, 1, 0);
}

struct FitWork {
  int* d_bins = nullptr;
  double* d_cnts = nullptr;
  double* d_logx = nullptr;
  int cap_bins = 0;
  double* d_part = nullptr;
  unsigned* d_bar = nullptr;
  FitOut* d_out = nullptr;
  FitOut* h_out = nullptr;   // pinned
  int max_grid = 0;
};

FitWork* fitwork_create() { return new FitWork(); }
void fitwork_destroy(FitWork* fw) {
  if (!fw) return;
  if (fw->d_bins) cudaFree(fw->d_bins);
  if (fw->d_cnts) cudaFree(fw->d_cnts);
  if (fw->d_logx) cudaFree(fw->d_logx);
  if (fw->d_part) cudaFree(fw->d_part);
  if (fw->d_bar) cudaFree(fw->d_bar);
  if (fw->d_out) cudaFree(fw->d_out);
  if (fw->h_out) cudaFreeHost(fw->h_out);
  delete fw;
}

// survfit[b] = mass * S(upper bound of bin b) for b in [cmin, 2 nb), 0 below
// (cov_histogram_SetSurvFitTail, src/covariation.c:1676-1699)
__global__ void k_survfit(int cmin, int nb, double bmin, double w, double mass, int doexp, double mu, double lambda,
                          double tau, double lga, double* __restrict__ sf) {
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < 2 * nb; b += gridDim.x * blockDim.x) {
    double v = 0.0;
    if (b >= cmin) {
      const double x = w * (b + 1) + bmin;
      double S;
      if (x <= mu) S = 1.0;
      else if (doexp) S = exp(-lambda * (x - mu));
      else S = gamma_q_dev(tau, lambda * (x - mu), lga);
      v = mass * S;
    }
    sf[b] = v;
  }
}

cudaError_t launch_survfit(int cmin, int nb, double bmin, double w, double mass, int doexp, double mu, double lambda,
                           double tau, double* d_sf, cudaStream_t st) {
  const int n = 2 * nb;
  k_survfit<<<std::max(1, std::min(1024, (n + 255) / 256)), 256, 0, st>>>(cmin, nb, bmin, w, mass, doexp, mu, lambda,
                                                                          tau, doexp ? 0.0 : std::lgamma(tau), d_sf);
  return cudaGetLastError();
}

// the start of a gamma fit (moment estimates, log lambda and log tau) and
// the non-empty tail bins; 1 when the tail is empty
static int fit_prepare(const uint64_t* h_obs, int cmin, int imax, double bmin, double w, double mu,
                       std::vector<int>& bins, std::vector<double>& cnts, double* s00, double* s01) {
  double m = 0.0, v = 0.0, n = 0.0;
  bins.clear();
  cnts.clear();
  for (int b = cmin; b <= imax; b++) {
    const double mid = (w * b + bmin) + 0.5 * w - mu;
    n += (double)h_obs[b]; m += (double)h_obs[b] * mid;
    if (h_obs[b]) { bins.push_back(b); cnts.push_back((double)h_obs[b]); }
  }
  if (n <= 0) return 1;
  m /= n;
  for (int b = cmin; b <= imax; b++) {
    const double mid = (w * b + bmin) + 0.5 * w - mu;
    v += (double)h_obs[b] * (mid - m) * (mid - m);
  }
  v /= n;
  if (!(v > 0.0) || !(m > 0.0)) { v = w * w; if (!(m > 0.0)) m = w; }
  *s00 = std::log(m / v);
  *s01 = std::log(m * m / v);
  return 0;
}

// 0 ok, 1 empty tail, 90 CUDA error; the result is read by gamma_fit_collect
// once the stream has passed the launch
int gamma_fit_launch(FitWork* fwp, const uint64_t* h_obs, int cmin, int imax, double bmin, double w, double phi,
                     cudaStream_t st) {
  FitWork& fw = *fwp;
  const double mu = phi;
  std::vector<int> bins;
  std::vector<double> cnts;
  double s00 = 0.0, s01 = 0.0;
  if (fit_prepare(h_obs, cmin, imax, bmin, w, mu, bins, cnts, &s00, &s01)) return 1;

  if (!fw.max_grid) {
    int dev = 0, nsm = 0, occ = 0, coop = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 90;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_gam_fit, 256, 0) != cudaSuccess || !coop || occ < 1)
      return 90;
    fw.max_grid = nsm;   // one block per SM is co-resident
    double inv[64];
    for (int k = 0; k < 64; k++) inv[k] = 1.0 / (k + 1);
    if (cudaMemcpyToSymbol(c_inv, inv, sizeof(inv)) != cudaSuccess) return 90;
    if (cudaMalloc(&fw.d_part, sizeof(double) * 2 * kFitMaxPts * fw.max_grid) != cudaSuccess) return 90;
    if (cudaMalloc(&fw.d_bar, sizeof(unsigned)) != cudaSuccess) return 90;
    if (cudaMalloc(&fw.d_out, sizeof(FitOut)) != cudaSuccess) return 90;
    if (cudaMallocHost(&fw.h_out, sizeof(FitOut)) != cudaSuccess) return 90;
  }
  const int nnz = (int)bins.size();
  if (fw.cap_bins < nnz) {
    if (fw.d_bins) cudaFree(fw.d_bins);
    if (fw.d_cnts) cudaFree(fw.d_cnts);
    if (fw.d_logx) cudaFree(fw.d_logx);
    fw.d_bins = nullptr; fw.d_cnts = nullptr; fw.d_logx = nullptr; fw.cap_bins = 0;
    if (cudaMalloc(&fw.d_bins, sizeof(int) * nnz) != cudaSuccess) return 90;
    if (cudaMalloc(&fw.d_cnts, sizeof(double) * nnz) != cudaSuccess) return 90;
    if (cudaMalloc(&fw.d_logx, sizeof(double) * nnz) != cudaSuccess) return 90;
    fw.cap_bins = nnz;
  }
  if (cudaMemcpyAsync(fw.d_bins, bins.data(), sizeof(int) * nnz, cudaMemcpyHostToDevice, st) != cudaSuccess) return 90;
  if (cudaMemcpyAsync(fw.d_cnts, cnts.data(), sizeof(double) * nnz, cudaMemcpyHostToDevice, st) != cudaSuccess) return 90;
  if (cudaMemsetAsync(fw.d_bar, 0, sizeof(unsigned), st) != cudaSuccess) return 90;

  FitGrid g;
  g.bins = fw.d_bins; g.cnts = fw.d_cnts; g.logx = fw.d_logx; g.nnz = nnz;
  g.bmin = bmin; g.w = w; g.mu = mu;
  g.part = fw.d_part; g.bar = fw.d_bar; g.out = fw.d_out;
  void* args[] = {&g, &s00, &s01};
  // one warp per SM until every SM has one, then up to 8 warps per block
  const int nitems = kFitMaxPts * nnz;
  const int W = std::max(1, std::min(8, (nitems + 32 * fw.max_grid - 1) / (32 * fw.max_grid)));
  const int G = std::max(1, std::min(fw.max_grid, (nitems + 32 * W - 1) / (32 * W)));
  if (cudaLaunchCooperativeKernel((const void*)k_gam_fit, dim3(G), dim3(32 * W), args, 0, st) != cudaSuccess)
    return 90;
  if (cudaMemcpyAsync(fw.h_out, fw.d_out, sizeof(FitOut), cudaMemcpyDeviceToHost, st) != cudaSuccess) return 90;
  return 0;
}

// 0 ok, 2 barrier timeout, else the search's status
int gamma_fit_collect(FitWork* fwp, double* ret_lambda, double* ret_tau, int* ret_evals) {
  const FitWork& fw = *fwp;
  if (fw.h_out->status) return fw.h_out->status;
  *ret_lambda = fw.h_out->lambda;
  *ret_tau = fw.h_out->tau;
  if (ret_evals) *ret_evals = fw.h_out->evals;
  return 0;
}




// ------------------------------------------------------------------------
// a batch of gamma fits (one block per fit, every search launched at once)
// and the survival tables of a batch of tails
// ------------------------------------------------------------------------
struct FitBatch {
  int cap_fit = 0, cap_bins = 0;
  FitGrid* d_grid = nullptr;
  double2* d_start = nullptr;
  int* d_bins = nullptr;
  double* d_cnts = nullptr;
  double* d_logx = nullptr;
  double* d_part = nullptr;
  unsigned* d_bar = nullptr;
  FitOut* d_out = nullptr;
  FitOut* h_out = nullptr;   // pinned
  std::vector<int> status;   // per fit: 1 empty tail (not launched)
  std::vector<int> slot;     // per fit: its block, or -1
  bool inv_set = false;
};

FitBatch* fitbatch_create() { return new FitBatch(); }
void fitbatch_destroy(FitBatch* fb) {
  if (!fb) return;
  void* p[] = {fb->d_grid, fb->d_start, fb->d_bins, fb->d_cnts, fb->d_logx, fb->d_part, fb->d_bar, fb->d_out};
  for (void* x : p) if (x) cudaFree(x);
  if (fb->h_out) cudaFreeHost(fb->h_out);
  delete fb;
}

int gamma_fit_batch_launch(FitBatch* fb, int nfit, const FitReq* req, cudaStream_t st) {
  fb->status.assign(nfit, 0);
  fb->slot.assign(nfit, -1);
  if (!fb->inv_set) {
    double inv[64];
    for (int k = 0; k < 64; k++) inv[k] = 1.0 / (k + 1);
    if (cudaMemcpyToSymbol(c_inv, inv, sizeof(inv)) != cudaSuccess) return 90;
    fb->inv_set = true;
  }
  std::vector<int> bins_all, bins;
  std::vector<double> cnts_all, cnts;
  std::vector<int> boff;
  std::vector<double2> start;
  int nl = 0;
  for (int k = 0; k < nfit; k++) {
    double s00, s01;
    if (fit_prepare(req[k].obs, req[k].cmin, req[k].imax, req[k].bmin, req[k].w, req[k].phi, bins, cnts, &s00,
                    &s01)) {
      fb->status[k] = 1;
      continue;
    }
    fb->slot[k] = nl++;
    boff.push_back((int)bins_all.size());
    bins_all.insert(bins_all.end(), bins.begin(), bins.end());
    cnts_all.insert(cnts_all.end(), cnts.begin(), cnts.end());
    start.push_back(make_double2(s00, s01));
  }
  boff.push_back((int)bins_all.size());
  if (nl == 0) return 0;
  const int nb = (int)bins_all.size();
  if (fb->cap_fit < nl) {
    void* p[] = {fb->d_grid, fb->d_start, fb->d_part, fb->d_bar, fb->d_out};
    for (void* x : p) if (x) cudaFree(x);
    if (fb->h_out) cudaFreeHost(fb->h_out);
    fb->d_grid = nullptr; fb->d_start = nullptr; fb->d_part = nullptr; fb->d_bar = nullptr; fb->d_out = nullptr;
    fb->h_out = nullptr; fb->cap_fit = 0;
    const int cap = std::max(nl, 64);
    if (cudaMalloc(&fb->d_grid, sizeof(FitGrid) * cap) != cudaSuccess ||
        cudaMalloc(&fb->d_start, sizeof(double2) * cap) != cudaSuccess ||
        cudaMalloc(&fb->d_part, sizeof(double) * 2 * kFitMaxPts * cap) != cudaSuccess ||
        cudaMalloc(&fb->d_bar, sizeof(unsigned) * cap) != cudaSuccess ||
        cudaMalloc(&fb->d_out, sizeof(FitOut) * cap) != cudaSuccess ||
        cudaMallocHost(&fb->h_out, sizeof(FitOut) * cap) != cudaSuccess)
      return 90;
    fb->cap_fit = cap;
  }
  if (fb->cap_bins < nb) {
    if (fb->d_bins) cudaFree(fb->d_bins);
    if (fb->d_cnts) cudaFree(fb->d_cnts);
    if (fb->d_logx) cudaFree(fb->d_logx);
    fb->d_bins = nullptr; fb->d_cnts = nullptr; fb->d_logx = nullptr; fb->cap_bins = 0;
    const int cap = std::max(nb, 4096);
    if (cudaMalloc(&fb->d_bins, sizeof(int) * cap) != cudaSuccess ||
        cudaMalloc(&fb->d_cnts, sizeof(double) * cap) != cudaSuccess ||
        cudaMalloc(&fb->d_logx, sizeof(double) * cap) != cudaSuccess)
      return 90;
    fb->cap_bins = cap;
  }
  std::vector<FitGrid> grid(nl);
  for (int k = 0; k < nfit; k++) {
    const int e = fb->slot[k];
    if (e < 0) continue;
    FitGrid& g = grid[e];
    g.bins = fb->d_bins + boff[e]; g.cnts = fb->d_cnts + boff[e]; g.logx = fb->d_logx + boff[e];
    g.nnz = boff[e + 1] - boff[e];
    g.bmin = req[k].bmin; g.w = req[k].w; g.mu = req[k].phi;
    g.part = fb->d_part + (size_t)e * 2 * kFitMaxPts;
    g.bar = fb->d_bar + e;
    g.out = fb->d_out + e;
  }
  if (cudaMemcpyAsync(fb->d_bins, bins_all.data(), sizeof(int) * nb, cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaMemcpyAsync(fb->d_cnts, cnts_all.data(), sizeof(double) * nb, cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaMemcpyAsync(fb->d_grid, grid.data(), sizeof(FitGrid) * nl, cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaMemcpyAsync(fb->d_start, start.data(), sizeof(double2) * nl, cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaMemsetAsync(fb->d_bar, 0, sizeof(unsigned) * nl, st) != cudaSuccess)
    return 90;
  k_gam_fit_grp<<<nl, 256, 0, st>>>(fb->d_grid, fb->d_start);
  if (cudaGetLastError() != cudaSuccess) return 90;
  if (cudaMemcpyAsync(fb->h_out, fb->d_out, sizeof(FitOut) * nl, cudaMemcpyDeviceToHost, st) != cudaSuccess) return 90;
  return 0;
}

int gamma_fit_batch_collect(FitBatch* fb, int k, double* ret_lambda, double* ret_tau, int* ret_evals) {
  if (fb->status[k]) return fb->status[k];
  const FitOut& o = fb->h_out[fb->slot[k]];
  if (o.status) return o.status;
  *ret_lambda = o.lambda;
  *ret_tau = o.tau;
  if (ret_evals) *ret_evals = o.evals;
  return 0;
}

__global__ void k_survfit_grp(const SurvReq* __restrict__ r, const int* __restrict__ pre, int nr) {
  const int e = grp_find(pre, nr, (int)blockIdx.x);
  const SurvReq& q = r[e];
  const int b = ((int)blockIdx.x - __ldg(pre + e)) * blockDim.x + threadIdx.x;
  if (b >= 2 * q.nb) return;
  double v = 0.0;
  if (b >= q.cmin) {
    const double x = q.w * (b + 1) + q.bmin;
    double S;
    if (x <= q.mu) S = 1.0;
    else if (q.doexp) S = exp(-q.lambda * (x - q.mu));
    else S = gamma_q_dev(q.tau, q.lambda * (x - q.mu), q.lga);
    v = q.mass * S;
  }
  q.sf[b] = v;
}

cudaError_t grp_survfit(const SurvReq* d_req, const int* pre, int nr, int nb, cudaStream_t st) {
  if (nb > 0) k_survfit_grp<<<nb, 256, 0, st>>>(d_req, pre, nr);
  return cudaGetLastError();
}

// ------------------------------------------------------------------------
// helix aggregation of pair p-values (agg_FISHER, agg_LANCASTER,
// agg_WFISHER, agg_SIDAK of src/aggregate.c:141-322): one warp per helix
// ------------------------------------------------------------------------
// y >= 0 with Q(a, y) = p, by doubling then bisection on the upper tail (the
// chi-square quantile of the complement of p, formed without 1 - p)
__device__ double gamma_q_inv(double a, double p) {
  if (!(p > 0.0)) return INFINITY;
  if (p >= 1.0) return 0.0;
  const double lga = lgamma(a);
  double lo = 0.0, hi = fmax(1.0, a);
  for (int k = 0; k < 1000 && gamma_q_dev(a, hi, lga) > p; k++) { lo = hi; hi *= 2.0; }
  for (int k = 0; k < 200 && hi - lo > 1e-15 * hi; k++) {
    const double mid = 0.5 * (lo + hi);
    if (gamma_q_dev(a, mid, lga) > p) lo = mid; else hi = mid;
  }
  return 0.5 * (lo + hi);
}

__global__ void k_aggregate(int method, int nh, const int* __restrict__ off, const double* __restrict__ pval,
                            const double* __restrict__ aux, double* __restrict__ term, double* __restrict__ pagg) {
  const int h = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (h >= nh) return;
  const int a = off[h], n = off[h + 1] - a;
  if (n <= 0) { if (lane == 0) pagg[h] = -1.0; return; }
  if (n == 1) { if (lane == 0) pagg[h] = pval[a]; return; }
  if (method == 1 || method == 2) {
    // weights: Lancaster 1 + substitutions; weighted Fisher (0.01 + power)
    // scaled to sum 2n (extract_rm_weights_*, src/aggregate.c:375-482)
    double wsum = 0.0;
    if (method == 2)
      for (int k = 0; k < n; k++) wsum += 0.01 + aux[a + k];
    const double f = (method == 2 && wsum > 0.0) ? 2.0 * n / wsum : 1.0;
    for (int k = lane; k < n; k += 32) {
      const double w = (method == 1) ? 1.0 + aux[a + k] : (0.01 + aux[a + k]) * f;
      term[2 * (a + k)] = w;
      term[2 * (a + k) + 1] = 2.0 * gamma_q_inv(0.5 * w, pval[a + k]);   // chi-square(w) quantile at 1 - p
    }
  }
  __syncwarp();
  if (lane != 0) return;
  double r;
  if (method == 0) {           // Fisher: chi-square with 2n degrees of freedom
    double chi = 0.0;
    for (int k = 0; k < n; k++) chi += -2.0 * log(pval[a + k]);
    r = isnan(chi) ? NAN : gamma_q_dev((double)n, 0.5 * chi, lgamma((double)n));
  } else if (method == 3) {    // Sidak
    double pmin = pval[a];
    for (int k = 1; k < n; k++) pmin = fmin(pmin, pval[a + k]);
    r = 1.0 - exp((double)n * log(1.0 - pmin));
  } else {                     // Lancaster / weighted Fisher
    double df = 0.0, chi = 0.0;
    for (int k = 0; k < n; k++) df += term[2 * (a + k)];
    for (int k = 0; k < n; k++) chi += term[2 * (a + k) + 1];
    r = isnan(chi) ? NAN : gamma_q_dev(0.5 * df, 0.5 * chi, lgamma(0.5 * df));
  }
  pagg[h] = r;
}

cudaError_t launch_aggregate(int method, int nh, const int* d_off, const double* d_pval, const double* d_aux,
                             double* d_term, double* d_pagg, cudaStream_t st) {
  if (nh <= 0) return cudaSuccess;
  k_aggregate<<<(nh + 7) / 8, 256, 0, st>>>(method, nh, d_off, d_pval, d_aux, d_term, d_pagg);
  return cudaGetLastError();
}

}  // namespace covgpu
