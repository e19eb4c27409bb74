// cov_batch.h -- grouped launches over a batch of alignment families
// (internal).
//
// A family is one input alignment (slot 0) and its null alignments (slots
// 1..ns), all N x L; families of a batch differ in N, L and ns.  Every
// buffer of a family lies inside the batch's device arena, in the layout the
// single-family kernels use (cov_dev.cuh), so a grouped launch runs the same
// kernel body on every family: its blocks are the concatenation of each
// family's own grid, and a block finds its family by a binary search over the
// prefix of the families' block counts (grp_find), then works on that
// family's pointers and sizes.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "cov_kernels.h"

namespace covgpu {

struct FamDev {
  int N, L, Lp, nT, ntiles, nslots, Lw;   // Lw: columns / 4 rounded up (GSC codes)
  uint8_t* ax;                 // [nslots][N][Lp]
  const TileRC* tiles;         // [ntiles]
  const int* tile_index;       // [nT][nT]
  const int* order;            // [ntiles] tile order of the tensor count kernel
  double* w;                   // [N] weights (device rule output, then the weights counted)
  float* limbf;                // [3][N] weight limbs as floats (SIMT counting)
  uint16_t* limbs;             // [3][Npad] weight limbs (tensor operand preparation)
  int nl, Npad;                // limbs in use; sequences padded to the tensor K block
  int oprow0;                  // first row of the family in the packed tensor operand buffer
  float B, s_hi, s_lo;         // limb base and scale (CountWeights)
  double* pbinv;               // [L][4] position-based weights scratch
  double* gD;                  // [N][N] GSC distances
  uint32_t* gra;               // [N][Lw] GSC codes, row role
  uint32_t* grb;               // [N][Lw] GSC codes, column role
  int* glen;                   // [N] residues per sequence
  const int* left;             // [N-1] tree (Easel convention)
  const int* right;            // [N-1]
  const int* lnodes;           // [N-1] internal nodes by depth
  uint8_t* fitch;              // [ns][N-1][Lp]
  uint8_t* scratch;            // [ns][N-1][Lp]
  float* cnt;                  // [nslots][ntiles][32][TPP] weighted counts (double-float planes)
  float* ucnt;                 // [nslots][ntiles][16][TPP] unit counts (RAF) or nullptr
  double* part4;               // [nslots][nT][nT][TP][4]
  double* partR;               // [nslots][nT][nT][TP]
  double* pm;                  // [nslots][Lp][4]
  float2* pmdf;                // [nslots][Lp][4]
  float4* lpi;                 // [nslots][Lp][4]
  double* mpc;                 // [nslots][Lp][4] (ps buffer of the single path)
  double* meanp;               // [nslots][4]
  float2* cov;                 // [nslots][nout][ntiles][TPP]
  float2* cov2;                // [nslots][ntiles][TPP] RAFS input copy, or nullptr
  double* part1;               // [nslots][nout][nT][nT][TP]
  double* colx;                // [nslots * nout][Lp]
  float2* colxf;               // [nslots * nout][Lp]
  double* avg;                 // [nslots * nout]
  float4* apcf;                // [nslots * nout]
  double* tmin;                // [nslots * nout][nblk]
  double* tmax;                // [nslots * nout][nblk]
  double* mm;                  // [nslots * nout][2]
  int* status;                 // this family's status word
  StatsArgs sa;                // the statistics pass's arguments for this family
};

// per (family, statistic) tables of the histogram and E-value passes
struct StatDev {
  int fam, q, active;
  // histogram of the nulls' scores
  BinC hb;
  int nbcap, wbase, nwin;
  unsigned long long* obs;
  // E-values and hits of the input alignment
  EvalTables T;
  EvalCmp K;
  int* nhits;
  int hitcap;
  int* hi;
  int* hj;
  double* hsc;
  double* hE;
  double* hp;
};

// the tensor count kernel's view of a family
struct UmmaFam {
  int row0;                    // first operand row of the family in the packed operand buffer
  int rows_per_buf;            // nslots * 4 Lp (rows of one of the four operand buffers)
  int Lp, ntiles, nkb;         // nkb: K blocks of 64 sequences
  int64_t orow0;               // first row (of 32 counts) of the family's counts in the output map
  const int* order;            // [ntiles] tile order
  const TileRC* tiles;
  float B, s_hi, s_lo;
};

// ---- grouped launchers (pre: device prefix [nf + 1] of each family's blocks
// for that kernel, nblocks = pre[nf]) ----
// weights (cov_prep.cu)
cudaError_t grp_weights_pb(const FamDev* F, int nf, const int* pre_col, int nb_col, const int* pre_row, int nb_row,
                           cudaStream_t st);
cudaError_t grp_weights_gsc(const FamDev* F, int nf, const int* pre_codes, int nb_codes, const int* pre_ident,
                            int nb_ident, const int* pre_upgma, int nb_upgma, int maxN, cudaStream_t st);
// normalisation and limbs of the device weights (one block per family of pre)
cudaError_t grp_weights_limbs(FamDev* F, int nf, const int* pre, int nb, UmmaFam* U, cudaStream_t st);
int         grp_weights_gsc_prepare();
// nulls (cov_null.cu): one depth d of every family; lv[f] = {offset of depth d
// in lnodes, nodes at depth d} (nn = 0: nothing at this depth)
cudaError_t grp_fitch_up(const FamDev* F, int nf, const int2* lv, const int* pre, int nb, uint64_t seed,
                         cudaStream_t st);
cudaError_t grp_root(const FamDev* F, int nf, const int* pre_state, int nb_state, const int* pre_row, int nb_row,
                     uint64_t seed, cudaStream_t st);
cudaError_t grp_replay(const FamDev* F, int nf, const int2* lv, const int* pre, int nb, bool cta, bool srow,
                       int maxLp, uint64_t seed, cudaStream_t st);
bool        replay_uses_cta(int nn, int nnull);
int         replay_smem_max();
// counting (cov_kernels.cu SIMT, cov_umma.cu tensor)
cudaError_t grp_count_simt(const FamDev* F, int nf, const int* pre, int nb, bool unit, bool limbs,
                           cudaStream_t st);
cudaError_t grp_umma_prep(const FamDev* F, int nf, const int* pre, int nb, int pitch, uint16_t* ops,
                          cudaStream_t st);
// the weighted tensor count of every family of fams (NL = 3 or 1 limbs),
// tasks (family, slot, tile) in the order of the prefix tpre; ops: packed
// operand buffer of pitch sequences per row, rows in total; cnt_base: the
// arena base the families' orow0 are counted from, cnt_rows rows of 32
int         grp_umma_count(const UmmaFam* fams, int nf, const int* tpre, int64_t ntask, int nl, const uint16_t* ops,
                           int pitch, int64_t rows, float* cnt_base, int64_t cnt_rows, int* err, cudaStream_t st);
// marginals, statistics, corrections (cov_kernels.cu)
cudaError_t grp_marginals(const FamDev* F, int nf, const int* pre_marg, int nb_marg, const int* pre_pm, int nb_pm,
                          const int* pre_mp, int nb_mp, cudaStream_t st);
cudaError_t grp_stats(const FamDev* F, int nf, const int* pre, int nb, unsigned cf, cudaStream_t st);
cudaError_t grp_rafs(const FamDev* F, int nf, const int* pre, int nb, int q, cudaStream_t st);
cudaError_t grp_apc(const FamDev* F, int nf, const int* pre_colx, int nb_colx, const int* pre_sq, int nb_sq,
                    const int* pre_apply, int nb_apply, CorrTypes ct, cudaStream_t st);
// histograms and E-values, one entry per active (family, statistic)
cudaError_t grp_hist(const FamDev* F, const StatDev* S, int ns, const int* pre, int nb, int maxwin, cudaStream_t st);
cudaError_t grp_evalue(const FamDev* F, const StatDev* S, int ns, const int* pre, int nb, cudaStream_t st);
unsigned    stats_cf(unsigned mask);
int         apc_blocks(int ntiles);
int         hist_threads();
// host-side bin constants and E-value comparison bounds
BinC        binc_host(double bmin, double w);
EvalCmp     evalcmp_host(const EvalTables& T);

}  // namespace covgpu
