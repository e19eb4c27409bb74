// cov_kernels.h -- launchers of the covariation kernels (internal).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "cov_dev.cuh"

namespace covgpu {

constexpr int MAXOUT = 4;   // score matrices produced by one k_stats launch

struct StatsArgs {
  const float*  cnt;        // weighted counts [slot][tile][16][2][TPP] (double-float planes)
  const float*  ucnt;       // unit-weight counts (RAF) [slot][tile][16][TPP] or nullptr
  const double* pm;         // [slot][Lp][4]
  const float2* pmdf;       // [slot][Lp][4] pm as double-float (hi, lo)
  const float4* lpi;        // [slot][Lp][4] {ln pm, 1/pm} as double-floats
  const float4* logtab;     // df_log's table (LOGTAB_TOT entries)
  const double* meanp;      // [slot][4]
  float2*       cov;        // [slot][nout][tile][TPP] scores as double-float (hi, lo)
  double*       part1;      // [slot][nout][nT][nT][TP]
  const TileRC* tiles;
  int           ntiles, nT, L, Lp, N;
  float2        wtot;       // sum of the quantised weights as double-float (ngap = wtot - nseff)
  float2        invD, invN; // 1/(N(N-1)) and 1/N for RAF, as double-float
  unsigned      stats;      // StatBit mask of what pair_stats must compute
  int           cls;        // 0 = C16, 1 = C2, 2 = CWC (GT)
  int           nout;       // number of output matrices (<= MAXOUT)
  int           outstat[MAXOUT];  // index into PairOut.v for output q
  float         allow[16];
};

// constants of the histogram's bin function, split on the host
struct BinC {
  float2 nbmin;    // -bmin
  float2 invw;     // 1/w
  float2 lo;       // bmin + w (scores are clamped up to it)
  float  mconst;   // absolute part of the fast-path margin
  float  absb;     // |bmin|
  float  mscale;   // 4e-7 / w: the FP32 estimate's error per unit of |x| + |bmin|
  int    bin_lo;   // bin of the clamp value bmin + w, from its FP64 value
  double bmin, w;
};

// tables of cov2evalue for one null histogram
struct EvalTables {
  const double* sf;         // survival fit [2*nb] or nullptr
  const double* ptail;      // ptail[b] = tail[b] / Nc, tail[b] = sum_{i>=b}^{imax} obs[i]
  double        bmin, w, phi, xmax, Nc, Nt, thresh;
  double        pNc;        // 1 / Nc
  int           nb, imin, imax;
  // the two-set test and --structured (src/covariation.c:846-854): pair
  // n = i (2L - i - 1)/2 + j - i - 1 takes Nb tests when bit n of bpmask is
  // set, else Nx tests when n <= kstar, else Nt
  const uint32_t* bpmask = nullptr;
  double        Nb = 0.0, Nx = 0.0;
  long long     kstar = -1;
};

// the E-value pass's comparison bounds (made on the host from EvalTables)
struct EvalCmp {
  float phi_dn, phi_up, xmax_dn, xmax_up;   // x.hi < dn: x < y; x.hi > up: x > y
  long long thresh_bits;
  int all;                                   // thresh > 1000: every pair is listed
};

// weights of the counting kernels: nl = 1 (all weights equal: count times
// s_hi + s_lo) or 3 limbs of b bits (count = limb_count(d0, d1, d2, B = 2^b,
// s_hi = 2^-E)); d_limbf = the limbs as floats, [3][N], for the SIMT path
struct CountWeights {
  int          nl = 1, bits = 0;
  float        B = 1.f, s_hi = 1.f, s_lo = 0.f;
  const float* d_limbf = nullptr;
};
// quantises the weights (host): limbs lim[3][stride] (uint16, zero-padded),
// the scale 2^-E, and the total of the quantised weights
void make_limbs(const double* w, int N, int stride, uint16_t* lim, CountWeights* W, double* wtot_q);

cudaError_t launch_count_simt(const uint8_t* ax, int64_t slot_stride, const CountWeights& W, bool unit, int N, int Lp,
                              const TileRC* tiles, int ntiles, int nslots, float* cnt, cudaStream_t st);
// pp [L][L][16], nseff [L][L], ngap [L][L] (each may be null) of the tiles'
// double-float counts in the reference's host layout
cudaError_t launch_probs_host_layout(const float* cnt, const TileRC* tiles, int ntiles, int L, double wt, double* pp,
                                     double* nseff, double* ngap, cudaStream_t st);
cudaError_t launch_pair_marg(const float* cnt, int L, const TileRC* tiles, int ntiles, int nT, int nslots,
                             double* part4, double* partR, cudaStream_t st);
cudaError_t launch_pm_final(const double* part4, const double* partR, int L, int Lp, int nT, int nslots, double* pm,
                            float2* pmdf, float4* lpi, double* mpc, double* meanp, int* status, cudaStream_t st);
cudaError_t launch_ps(const uint8_t* ax, int64_t slot_stride, const double* w, int N, int L, int Lp, int nslots,
                      double* ps, cudaStream_t st);
cudaError_t launch_stats(const StatsArgs& A, int nslots, cudaStream_t st);
// power_SPAIR_AddMI's pair classes of one alignment's double-float counts:
// [L(L-1)/2] each, row-major over i < j
cudaError_t launch_pair_classes(const float* cnt, const TileRC* tiles, int ntiles, int L, double* wcf, double* wob,
                                double* non, cudaStream_t st);
// pair-probability validation of one alignment's double-float counts; *bad set on failure
cudaError_t launch_validate_pp(const float* cnt, const TileRC* tiles, int ntiles, int L, double tol, int* bad,
                               cudaStream_t st);
cudaError_t launch_rafs(const float2* raf, float2* out, int64_t sin, int64_t sout, const TileRC* tiles,
                        const int* tile_index, int ntiles, int nT, int L, int nslots, double* part1, int64_t pstride,
                        cudaStream_t st);
// actype per output q (sq = slot * nout + q): 0 = APC, 1 = ASC, -1 = none
struct CorrTypes { int act[MAXOUT]; int nout; };
// colx [nsq][Lp] (FP64) with its double-float copy colxf; avg [nsq] (FP64)
// with apcf [nsq] = (avg, 1/avg) as double-float pairs
cudaError_t launch_apc(float2* cov, const double* part1, double* colx, float2* colxf, double* avg, float4* apcf,
                       CorrTypes ct, const TileRC* tiles, int ntiles, int nT, int L, int Lp, int nsq, double* tmin,
                       double* tmax, double* mm, int* status, cudaStream_t st);
cudaError_t launch_tile(const double* full, const TileRC* tiles, int ntiles, int L, float2* tilev, cudaStream_t st);
cudaError_t launch_tile_rowsums(const float2* tilev, const TileRC* tiles, int ntiles, int nT, int L, double* part1,
                                cudaStream_t st);
cudaError_t launch_minmax(const float2* cov, const TileRC* tiles, int ntiles, int L, int nsq, double* tmin,
                          double* tmax, double* mm, cudaStream_t st);
// histogram of nslots score planes into obs[nbcap]; wbase = a bin at or below
// the smallest score's bin (the shared-memory window starts there)
cudaError_t launch_hist(const float2* cov, int64_t slot_stride, const TileRC* tiles, int ntiles, int L, int nslots,
                        double bmin, double w, int nbcap, int wbase, unsigned long long* obs, int* status,
                        cudaStream_t st);
cudaError_t launch_evalue(const float2* cov, const TileRC* tiles, int ntiles, int L, const EvalTables& T, double* evt,
                          int* nhits, int hitcap, int* hi, int* hj, double* hsc, double* hE, double* hp,
                          cudaStream_t st);
cudaError_t launch_untile(const float2* tilev, const TileRC* tiles, int ntiles, int L, double diag, double* full,
                          cudaStream_t st);
cudaError_t launch_untile(const double* tilev, const TileRC* tiles, int ntiles, int L, double diag, double* full,
                          cudaStream_t st);

// null alignments (cov_null.cu)
struct NullTree {
  int        N;
  const int* left;    // [N-1] device, Easel convention (<= 0: leaf -value)
  const int* right;   // [N-1] device
};
// level_nodes: device list of internal nodes ordered by depth; level_off:
// host offsets of each depth in that list (nlevels + 1 entries)
// the Fitch reconstruction of one alignment (random tie-breaks from stream
// nid): F [N-1][Lp] states of the internal nodes, S [N-1][Lp] scratch sets
cudaError_t launch_fitch_recon(const uint8_t* ax, int N, int L, int Lp, const NullTree& T, const int* level_nodes,
                               const int* level_off, int nlevels, uint64_t seed, uint32_t nid, uint8_t* F, uint8_t* S,
                               cudaStream_t st);
cudaError_t launch_nullgen(const uint8_t* ax, int N, int L, int Lp, const NullTree& T, const int* level_nodes,
                           const int* level_off, int nlevels, uint64_t seed, uint32_t first_null, int nnull,
                           uint8_t* fitch, uint8_t* scratch, uint8_t* out_ax, int64_t out_slot_stride,
                           cudaStream_t st);

}  // namespace covgpu
