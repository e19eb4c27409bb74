// cov_engine.cu -- host orchestration of the GB300 covariation engine and
// its C-ABI (include/covgpu.h).  One context = one device stream and the
// device buffers for up to `maxslots` alignments of N x L.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "cov_dev.cuh"
#include "cov_df.cuh"
#include "cov_kernels.h"
#include "cov_fit.h"
#include "cov_learn.h"
#include "cov_prep.h"
#include "cov_sim.h"
#include "cov_subst.h"
#include "cov_umma.h"
#include "covgpu.h"
#include "cov_rscape_host.h"
#include "rscape_cov.h"

using namespace covgpu;

struct covgpu_ctx {
  int dev = 0;
  cudaStream_t st = nullptr;
  int N = 0, L = 0, Lp = 0, nT = 0, ntiles = 0, maxslots = 0, maxnull = 0;
  // the dimensions the buffers were made for (covgpu_resize stays within them)
  int capN = 0, capL = 0, capLp = 0, capnT = 0, capntiles = 0;
  char err[512] = {0};
  TileRC* d_tiles = nullptr;
  int* d_tile_index = nullptr;
  uint8_t* d_ax = nullptr;
  double* d_wd = nullptr;
  std::vector<double> h_w;
  CountWeights cw;                  // quantised weights of the SIMT counting kernel
  float* d_limbf = nullptr;         // their limbs as floats [3][N]
  double wtot_q = 0.0;              // total of the quantised weights
  float4* d_logtab = nullptr;       // df_log's table
  // host staging of covgpu_rscape (null histograms, survival tables, tail
  // tables), kept across calls so same-sized calls neither allocate nor clear
  std::vector<uint64_t> h_obs;
  std::vector<double> h_sf, h_tail;
  double wtot = 0.0;
  bool have_w = false;
  float* d_cnt = nullptr;
  float* d_ucnt = nullptr;
  double *d_part4 = nullptr, *d_partR = nullptr, *d_pm = nullptr, *d_meanp = nullptr, *d_ps = nullptr;
  float2* d_pmdf = nullptr;
  float4* d_lpi = nullptr;          // {ln pm, 1/pm} as double-floats
  float2 *d_cov = nullptr, *d_cov2 = nullptr;   // score planes as double-float pairs
  float2* d_colxf = nullptr;
  float4* d_apcf = nullptr;
  double* d_evt = nullptr;                      // E-value planes for the host
  double *d_part1 = nullptr, *d_colx = nullptr, *d_avg = nullptr;
  double *d_tmin = nullptr, *d_tmax = nullptr, *d_mm = nullptr;
  int* d_status = nullptr;
  int last_nout = 0, last_first = 0, last_nslots = 0;
  int* d_left = nullptr;
  int* d_right = nullptr;
  int* d_lnodes = nullptr;
  std::vector<int> loff;
  bool have_tree = false;
  uint8_t *d_fitch = nullptr, *d_scratch = nullptr;
  unsigned long long* d_obs = nullptr;
  int nbcap = 0;
  double *d_sf = nullptr, *d_tail = nullptr;
  int sfcap = 0;
  int* d_nhits = nullptr;
  int *d_hi = nullptr, *d_hj = nullptr;
  double *d_hsc = nullptr, *d_hE = nullptr, *d_hp = nullptr;
  int hitcap = 0;
  double* d_full = nullptr;
  double* d_pcls = nullptr;         // covgpu_pair_classes outputs [3][capL(capL-1)/2]
  uint32_t* d_bpmask = nullptr;     // the two-set test's base-pair bitmap [capL(capL-1)/2 bits]
  int *d_ci = nullptr, *d_cj = nullptr;   // --structured: the hits under the first hits' rule
  double* d_cd = nullptr;                 // their scores, E-values and p-values [3][ccap]
  int ccap = 0;
  double* d_pphost = nullptr;       // covgpu_get_probs: pp, nseff, ngap in the host layout [capL^2 (16 + 2)]
  UmmaPlan* umma = nullptr;
  FitWork* fitw[MAXOUT] = {};
  // simulator
  double *d_simQ = nullptr, *d_simT = nullptr, *d_P4 = nullptr, *d_P16 = nullptr;
  unsigned long long *d_C4 = nullptr, *d_C16 = nullptr, *d_R = nullptr;
  int2* d_units = nullptr;
  uint8_t *d_simroot = nullptr, *d_simstate = nullptr;
  size_t simstate_cap = 0;
  int sim_branches = 0;
  std::vector<double> sim_key;   // times and model of the tables on the device
  // substitutions of the last covgpu_substitutions
  int *d_nsubs = nullptr, *d_ndouble = nullptr, *d_njoin = nullptr;
  // learned-null features
  double* d_featscr = nullptr;
  float* d_feat = nullptr;
  void* d_gsc = nullptr;       // GSC scratch, kept across calls
  size_t gsc_cap = 0;
  double* d_pbscr = nullptr;   // position-based weights scratch
  bool want_qsum = false;     // covgpu_rscape keeps the null-score summary of type 0
  double qsum[17] = {0};
  bool have_qsum = false;
  unsigned char* d_flush = nullptr;
  bool counted = false;
  // the weighted counts in d_cnt are those of slots [cnt_first, cnt_first +
  // cnt_nslots) as they are now (invalidated by anything that changes those
  // alignments or the weights), so a later covgpu_score of the same slots
  // reuses them
  bool cnt_valid = false;
  int cnt_first = 0, cnt_nslots = 0, cnt_counter = -1;
  cudaEvent_t ev[6] = {};
  // the statistics' tail fits run side by side, one stream each (a fit is a
  // cooperative launch of a few dozen small blocks)
  cudaStream_t fst[MAXOUT] = {};
  cudaEvent_t fev[MAXOUT + 1] = {};
  double tms[5] = {0, 0, 0, 0, 0};
  double fit_ms = 0.0;
  int nlaunch = 0;
};

static int fail(covgpu_ctx* c, int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(c->err, sizeof(c->err), fmt, ap);
  va_end(ap);
  return code;
}

#define CK(call)                                                                         \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess) return fail(ctx, 90, "%s: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

template <class T>
static cudaError_t dalloc(T** p, size_t n) {
  return cudaMalloc((void**)p, std::max<size_t>(n, 1) * sizeof(T));
}

extern "C" void covgpu_params_default(covgpu_params* p) {
  memset(p, 0, sizeof(*p));
  p->covclass = 3; p->nseqthresh = 8; p->alenthresh = 50; p->nshuffle = -1;
  p->thresh = 0.05; p->bmin = -10.0; p->w0 = 0.05; p->hpts = 400; p->pmass = 0.0005; p->fracfit = 1.0;
  p->doexpfit = 0; p->tol = 1e-6; p->seed = 42; p->counter = COVGPU_COUNT_SIMT;
  p->samplesize = 3; p->expBP = -1.0;
  p->allow[0 * 4 + 3] = p->allow[3 * 4 + 0] = 1.0;   // src/R-scape.c:883-887
  p->allow[1 * 4 + 2] = p->allow[2 * 4 + 1] = 1.0;
  p->allow[2 * 4 + 3] = p->allow[3 * 4 + 2] = 1.0;
}

extern "C" const char* covgpu_errmsg(const covgpu_ctx* ctx) { return ctx ? ctx->err : "no context"; }

extern "C" int covgpu_create(covgpu_ctx** ret, int device, int N, int L, int maxslots, int maxnull) {
  *ret = nullptr;
  if (N < 1 || L < 1 || maxslots < 1 || maxnull < 0) return 11;
  covgpu_ctx* ctx = new covgpu_ctx();
  ctx->dev = device; ctx->N = N; ctx->L = L; ctx->maxslots = maxslots; ctx->maxnull = maxnull;
  ctx->nT = (L + TP - 1) / TP;
  ctx->Lp = ctx->nT * TP;
  ctx->ntiles = ctx->nT * (ctx->nT + 1) / 2;
  ctx->capN = N; ctx->capL = L; ctx->capLp = ctx->Lp; ctx->capnT = ctx->nT; ctx->capntiles = ctx->ntiles;
  *ret = ctx;
  CK(cudaSetDevice(device));
  CK(cudaStreamCreateWithFlags(&ctx->st, cudaStreamNonBlocking));
  for (auto& e : ctx->ev) CK(cudaEventCreate(&e));
  for (auto& f : ctx->fst) CK(cudaStreamCreateWithFlags(&f, cudaStreamNonBlocking));
  for (auto& e : ctx->fev) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  std::vector<TileRC> tiles;
  std::vector<int> tindex((size_t)ctx->nT * ctx->nT, -1);
  for (int I = 0; I < ctx->nT; I++)
    for (int J = I; J < ctx->nT; J++) { tindex[(size_t)I * ctx->nT + J] = (int)tiles.size(); tiles.push_back({I, J}); }
  const size_t nT2 = (size_t)ctx->nT * ctx->nT, ntl = ctx->ntiles, S = maxslots;
  CK(dalloc(&ctx->d_tiles, ntl));
  CK(dalloc(&ctx->d_tile_index, nT2));
  CK(cudaMemcpy(ctx->d_tiles, tiles.data(), ntl * sizeof(TileRC), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(ctx->d_tile_index, tindex.data(), nT2 * sizeof(int), cudaMemcpyHostToDevice));
  CK(dalloc(&ctx->d_ax, S * N * ctx->Lp));
  CK(cudaMemset(ctx->d_ax, 4, S * N * ctx->Lp));
  CK(dalloc(&ctx->d_limbf, (size_t)3 * N));
  CK(dalloc(&ctx->d_wd, N));
  CK(dalloc(&ctx->d_cnt, S * ntl * 32 * TPP));
  CK(dalloc(&ctx->d_logtab, LOGTAB_TOT));
  {
    float4 tab[LOGTAB_TOT];
    logtab_host(tab);
    CK(cudaMemcpy(ctx->d_logtab, tab, sizeof(tab), cudaMemcpyHostToDevice));
  }
  CK(dalloc(&ctx->d_part4, S * nT2 * TP * 4));
  CK(dalloc(&ctx->d_partR, S * nT2 * TP));
  CK(dalloc(&ctx->d_pm, S * ctx->Lp * 4));
  CK(dalloc(&ctx->d_pmdf, S * ctx->Lp * 4));
  CK(dalloc(&ctx->d_lpi, S * ctx->Lp * 4));
  CK(dalloc(&ctx->d_meanp, S * 4));
  CK(dalloc(&ctx->d_ps, S * ctx->Lp * 5));
  CK(dalloc(&ctx->d_cov, S * MAXOUT * ntl * TPP));
  CK(dalloc(&ctx->d_part1, S * MAXOUT * nT2 * TP));
  CK(dalloc(&ctx->d_colx, S * MAXOUT * ctx->Lp));
  CK(dalloc(&ctx->d_colxf, S * MAXOUT * ctx->Lp));
  CK(dalloc(&ctx->d_avg, S * MAXOUT));
  CK(dalloc(&ctx->d_apcf, S * MAXOUT));
  CK(dalloc(&ctx->d_tmin, S * MAXOUT * ntl));
  CK(dalloc(&ctx->d_tmax, S * MAXOUT * ntl));
  CK(dalloc(&ctx->d_mm, S * MAXOUT * 2));
  CK(dalloc(&ctx->d_status, 1));
  CK(cudaMemset(ctx->d_status, 0, sizeof(int)));
  CK(dalloc(&ctx->d_nhits, MAXOUT + 1));   // per statistic, and the --structured pass's
  if (maxnull > 0 && N > 1) {
    CK(dalloc(&ctx->d_fitch, (size_t)maxnull * (N - 1) * ctx->Lp));
    CK(dalloc(&ctx->d_scratch, (size_t)maxnull * (N - 1) * ctx->Lp));
  }
  ctx->err[0] = 0;
  return 0;
}

extern "C" void covgpu_destroy(covgpu_ctx* ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->dev);
  if (ctx->st) cudaStreamSynchronize(ctx->st);
  void* ptrs[] = {ctx->d_tiles, ctx->d_tile_index, ctx->d_ax, ctx->d_limbf, ctx->d_logtab, ctx->d_lpi, ctx->d_wd, ctx->d_cnt, ctx->d_ucnt,
                  ctx->d_part4, ctx->d_partR, ctx->d_pm, ctx->d_meanp, ctx->d_ps, ctx->d_cov, ctx->d_cov2,
                  ctx->d_part1, ctx->d_colx, ctx->d_avg, ctx->d_tmin, ctx->d_tmax, ctx->d_mm, ctx->d_status,
                  ctx->d_left, ctx->d_right, ctx->d_lnodes, ctx->d_fitch, ctx->d_scratch, ctx->d_obs, ctx->d_sf,
                  ctx->d_tail, ctx->d_nhits, ctx->d_hi, ctx->d_hj, ctx->d_hsc, ctx->d_hE, ctx->d_hp, ctx->d_full,
                  ctx->d_flush, ctx->d_pmdf, ctx->d_colxf, ctx->d_apcf, ctx->d_evt, ctx->d_pcls,
                  ctx->d_bpmask, ctx->d_pphost, ctx->d_ci, ctx->d_cj, ctx->d_cd};
  for (void* p : ptrs) if (p) cudaFree(p);
  if (ctx->umma) umma_plan_destroy(ctx->umma);
  for (FitWork* f : ctx->fitw) if (f) fitwork_destroy(f);
  void* sims[] = {ctx->d_simQ, ctx->d_simT, ctx->d_P4, ctx->d_P16, ctx->d_C4, ctx->d_C16, ctx->d_R, ctx->d_units,
                  ctx->d_simroot, ctx->d_simstate, ctx->d_nsubs, ctx->d_ndouble, ctx->d_njoin, ctx->d_featscr,
                  ctx->d_feat, ctx->d_gsc, ctx->d_pbscr};
  for (void* p : sims) if (p) cudaFree(p);
  for (auto& e : ctx->ev) if (e) cudaEventDestroy(e);
  for (auto& e : ctx->fev) if (e) cudaEventDestroy(e);
  for (auto& f : ctx->fst) if (f) { cudaStreamSynchronize(f); cudaStreamDestroy(f); }
  if (ctx->st) cudaStreamDestroy(ctx->st);
  delete ctx;
}

// tile lists of the current nT
static int build_tiles(covgpu_ctx* ctx) {
  const int nT = ctx->nT;
  std::vector<TileRC> tiles;
  std::vector<int> tindex((size_t)nT * nT, -1);
  for (int I = 0; I < nT; I++)
    for (int J = I; J < nT; J++) { tindex[(size_t)I * nT + J] = (int)tiles.size(); tiles.push_back({I, J}); }
  CK(cudaMemcpy(ctx->d_tiles, tiles.data(), tiles.size() * sizeof(TileRC), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(ctx->d_tile_index, tindex.data(), tindex.size() * sizeof(int), cudaMemcpyHostToDevice));
  return 0;
}

extern "C" int covgpu_resize(covgpu_ctx* ctx, int N, int L) {
  if (!ctx) return 11;
  CK(cudaSetDevice(ctx->dev));
  ctx->cnt_valid = false;
  if (N < 1 || L < 1 || N > ctx->capN || L > ctx->capL)
    return fail(ctx, 11, "%d x %d is outside the context's %d x %d", N, L, ctx->capN, ctx->capL);
  CK(cudaStreamSynchronize(ctx->st));
  ctx->N = N; ctx->L = L;
  ctx->nT = (L + TP - 1) / TP;
  ctx->Lp = ctx->nT * TP;
  ctx->ntiles = ctx->nT * (ctx->nT + 1) / 2;
  int s;
  if ((s = build_tiles(ctx))) return s;
  // gap codes in every slot's rows (columns past L are never scored)
  CK(cudaMemset(ctx->d_ax, 4, (size_t)ctx->maxslots * N * ctx->Lp));
  ctx->have_w = false;
  ctx->have_tree = false;
  ctx->counted = false;
  ctx->cnt_valid = false;
  ctx->last_nout = ctx->last_first = ctx->last_nslots = 0;
  ctx->sim_key.clear();
  if (ctx->umma && !umma_plan_resize(ctx->umma, N, L, ctx->Lp, ctx->nT, ctx->ntiles)) {
    umma_plan_destroy(ctx->umma);
    ctx->umma = nullptr;
  }
  return 0;
}

extern "C" int covgpu_set_weights(covgpu_ctx* ctx, const double* wgt) {
  if (!ctx) return 11;
  CK(cudaSetDevice(ctx->dev));
  const int N = ctx->N;
  ctx->cnt_valid = false;
  double s = 0.0;
  for (int i = 0; i < N; i++) {
    if (!(wgt[i] >= 0.0) || !std::isfinite(wgt[i])) return fail(ctx, 11, "weight %d is negative or not finite", i);
    s += wgt[i];
  }
  ctx->h_w.assign(wgt, wgt + N);
  ctx->wtot = s;
  // the counting kernels count quantised weights (make_limbs); the SIMT path
  // takes the limbs as floats, the tensor path as FP16 operands
  std::vector<uint16_t> lim((size_t)3 * N);
  make_limbs(wgt, N, N, lim.data(), &ctx->cw, &ctx->wtot_q);
  std::vector<float> lf(lim.begin(), lim.end());
  CK(cudaMemcpyAsync(ctx->d_wd, wgt, N * sizeof(double), cudaMemcpyHostToDevice, ctx->st));
  CK(cudaMemcpyAsync(ctx->d_limbf, lf.data(), lf.size() * sizeof(float), cudaMemcpyHostToDevice, ctx->st));
  CK(cudaStreamSynchronize(ctx->st));
  ctx->cw.d_limbf = ctx->d_limbf;
  if (ctx->umma) umma_set_weights(ctx->umma, wgt, N, ctx->st);
  ctx->have_w = true;
  return 0;
}

extern "C" int covgpu_set_alignment(covgpu_ctx* ctx, int slot, const uint8_t* ax) {
  if (!ctx) return 11;
  if (slot < 0 || slot >= ctx->maxslots) return fail(ctx, 11, "slot %d out of range", slot);
  CK(cudaSetDevice(ctx->dev));
  ctx->cnt_valid = false;
  // the largest code first (a reduction over the host threads); the
  // position of a bad code is looked up only when there is one
  const int64_t n = (int64_t)ctx->N * ctx->L;
  uint8_t mx = 0;
#pragma omp parallel for reduction(max : mx) schedule(static) if (n > (1 << 20))
  for (int64_t k = 0; k < n; k++) mx = std::max(mx, ax[k]);
  if (mx > 17)
    for (int64_t k = 0; k < n; k++)
      if (ax[k] > 17) return fail(ctx, 11, "code %d at %lld is not an RNA digital code", ax[k], (long long)k);
  uint8_t* dst = ctx->d_ax + (size_t)slot * ctx->N * ctx->Lp;
  CK(cudaMemcpy2DAsync(dst, ctx->Lp, ax, ctx->L, ctx->L, ctx->N, cudaMemcpyHostToDevice, ctx->st));
  CK(cudaStreamSynchronize(ctx->st));
  return 0;
}

extern "C" int covgpu_get_alignment(covgpu_ctx* ctx, int slot, uint8_t* ax) {
  if (!ctx) return 11;
  if (slot < 0 || slot >= ctx->maxslots) return fail(ctx, 11, "slot %d out of range", slot);
  CK(cudaSetDevice(ctx->dev));
  const uint8_t* src = ctx->d_ax + (size_t)slot * ctx->N * ctx->Lp;
  CK(cudaMemcpy2DAsync(ax, ctx->L, src, ctx->Lp, ctx->L, ctx->N, cudaMemcpyDeviceToHost, ctx->st));
  CK(cudaStreamSynchronize(ctx->st));
  return 0;
}

extern "C" int covgpu_set_tree(covgpu_ctx* ctx, const int* parent, const int* left, const int* right) {
  if (!ctx) return 11;
  const int N = ctx->N;
  CK(cudaSetDevice(ctx->dev));
  if (N < 2) { ctx->have_tree = false; return 0; }
  // validate: Easel convention, parent[v] < v, every leaf and node reached once
  std::vector<int> seen_leaf(N, 0), seen_node(N - 1, 0), depth(N - 1, 0);
  for (int v = 0; v < N - 1; v++) {
    const int ch[2] = {left[v], right[v]};
    for (int k = 0; k < 2; k++) {
      const int c = ch[k];
      if (c <= 0) {
        if (-c >= N || seen_leaf[-c]++) return fail(ctx, 11, "tree: leaf %d repeated or out of range", -c);
      } else {
        if (c >= N - 1 || c <= v || seen_node[c]++) return fail(ctx, 11, "tree: node %d has bad child %d", v, c);
        if (parent && parent[c] != v) return fail(ctx, 11, "tree: parent[%d] != %d", c, v);
        depth[c] = depth[v] + 1;
      }
    }
  }
  int maxd = 0;
  for (int v = 0; v < N - 1; v++) maxd = std::max(maxd, depth[v]);
  std::vector<int> order;
  ctx->loff.assign(maxd + 2, 0);
  for (int d = 0; d <= maxd; d++) {
    ctx->loff[d] = (int)order.size();
    for (int v = 0; v < N - 1; v++) if (depth[v] == d) order.push_back(v);
  }
  ctx->loff[maxd + 1] = (int)order.size();
  if (!ctx->d_left) {
    CK(dalloc(&ctx->d_left, ctx->capN - 1));
    CK(dalloc(&ctx->d_right, ctx->capN - 1));
    CK(dalloc(&ctx->d_lnodes, ctx->capN - 1));
  }
  CK(cudaMemcpy(ctx->d_left, left, (N - 1) * sizeof(int), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(ctx->d_right, right, (N - 1) * sizeof(int), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(ctx->d_lnodes, order.data(), (N - 1) * sizeof(int), cudaMemcpyHostToDevice));
  ctx->have_tree = true;
  return 0;
}

static int make_nulls_async(covgpu_ctx* ctx, uint64_t seed, int first_null, int nnull, int first_slot) {
  if (nnull <= 0) return 0;
  ctx->cnt_valid = false;
  if (!ctx->have_tree) return fail(ctx, 11, "no tree set");
  if (nnull > ctx->maxnull) return fail(ctx, 11, "%d nulls > capacity %d", nnull, ctx->maxnull);
  if (first_slot < 1 || first_slot + nnull > ctx->maxslots) return fail(ctx, 11, "null slots out of range");
  if (ctx->L > 48 * 1024) return fail(ctx, 11, "alignment longer than 49152 columns");
  NullTree T{ctx->N, ctx->d_left, ctx->d_right};
  const int64_t sstride = (int64_t)ctx->N * ctx->Lp;
  CK(launch_nullgen(ctx->d_ax, ctx->N, ctx->L, ctx->Lp, T, ctx->d_lnodes, ctx->loff.data(),
                    (int)ctx->loff.size() - 1, seed, (uint32_t)first_null, nnull, ctx->d_fitch, ctx->d_scratch,
                    ctx->d_ax + first_slot * sstride, sstride, ctx->st));
  ctx->nlaunch += 2 + 2 * ((int)ctx->loff.size() - 1);
  return 0;
}

static int check_status(covgpu_ctx* ctx);

extern "C" int covgpu_weights_pb_dev(covgpu_ctx* ctx, int slot, int set, double* wgt) {
  if (!ctx) return 11;
  CK(cudaSetDevice(ctx->dev));
  ctx->cnt_valid = false;
  const int N = ctx->N, L = ctx->L, Lp = ctx->Lp;
  if (slot < 0 || slot >= ctx->maxslots || !wgt) return fail(ctx, 11, "bad slot or output");
  // scratch kept across calls (a cudaFree per call would synchronise the device)
  if (!ctx->d_pbscr) CK(dalloc(&ctx->d_pbscr, (size_t)ctx->capL * 4 + ctx->capN));
  double* d_inv = ctx->d_pbscr;
  double* d_w = ctx->d_pbscr + (size_t)ctx->capL * 4;
  cudaError_t e = launch_weights_pb(ctx->d_ax + (size_t)slot * N * Lp, N, L, Lp, d_inv, d_w, ctx->st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(wgt, d_w, N * sizeof(double), cudaMemcpyDeviceToHost, ctx->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->st);
  if (e != cudaSuccess) return fail(ctx, 90, "CUDA error %s", cudaGetErrorString(e));
  // renormalised to sum to N (the sum in sequence order, as the reference)
  double sum = 0.0;
  for (int s = 0; s < N; s++) sum += wgt[s];
  for (int s = 0; s < N; s++) wgt[s] = (sum > 0.0) ? wgt[s] * (double)N / sum : 1.0;
  return set ? covgpu_set_weights(ctx, wgt) : 0;
}

extern "C" int covgpu_weights_gsc_dev(covgpu_ctx* ctx, int slot, int set, double* wgt) {
  if (!ctx) return 11;
  CK(cudaSetDevice(ctx->dev));
  ctx->cnt_valid = false;
  const int N = ctx->N, L = ctx->L, Lp = ctx->Lp;
  if (slot < 0 || slot >= ctx->maxslots || !wgt) return fail(ctx, 11, "bad slot or output");
  if (N > 16384) return fail(ctx, 11, "GSC weights are for up to 16384 sequences (N^2 distances)");
  if (N == 1) { wgt[0] = 1.0; return set ? covgpu_set_weights(ctx, wgt) : 0; }
  // scratch kept across calls (families of a resized context reuse it)
  const size_t need = gsc_scratch_bytes(N, L) + ((size_t)N * sizeof(double) + 256);
  if (ctx->gsc_cap < need) {
    if (ctx->d_gsc) cudaFree(ctx->d_gsc);
    ctx->d_gsc = nullptr;
    ctx->gsc_cap = 0;
    const size_t cap = std::max(need, gsc_scratch_bytes(ctx->capN, ctx->capL) + (size_t)ctx->capN * sizeof(double) + 256);
    CK(cudaMalloc(&ctx->d_gsc, cap));
    ctx->gsc_cap = cap;
  }
  uint8_t* scratch = (uint8_t*)ctx->d_gsc;
  double* d_w = (double*)(scratch + ((gsc_scratch_bytes(N, L) + 255) & ~(size_t)255));
  cudaError_t e = launch_weights_gsc(ctx->d_ax + (size_t)slot * N * Lp, N, L, Lp, scratch, d_w, ctx->st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(wgt, d_w, N * sizeof(double), cudaMemcpyDeviceToHost, ctx->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->st);
  if (e != cudaSuccess) return fail(ctx, 90, "CUDA error %s", cudaGetErrorString(e));
  if (gsc_error(scratch, ctx->st)) return fail(ctx, 24, "GSC weights: a grid barrier timed out");
  double sum = 0.0;
  for (int s = 0; s < N; s++) sum += wgt[s];
  for (int s = 0; s < N; s++) wgt[s] = (sum > 0.0) ? wgt[s] * (double)N / sum : 1.0;
  return set ? covgpu_set_weights(ctx, wgt) : 0;
}

// random stream of the reconstruction's tie-breaks (null alignments use
// stream ids 0 .. nshuffle-1)
constexpr uint32_t kReconStream = 0xFFFFFFFFu;

extern "C" int covgpu_substitutions(covgpu_ctx* ctx, int slot, uint64_t seed, int includegaps, int* nsubs,
                                    int* ndouble, int* njoin) {
  if (!ctx) return 11;
  CK(cudaSetDevice(ctx->dev));
  const int N = ctx->N, L = ctx->L, Lp = ctx->Lp;
  if (!ctx->have_tree) return fail(ctx, 11, "no tree set");
  if (N < 2) return fail(ctx, 11, "substitutions need a tree of at least two leaves");
  if (slot < 0 || slot >= ctx->maxslots) return fail(ctx, 11, "bad slot");
  const size_t rows = (size_t)(N - 1) * Lp;
  uint8_t *F = ctx->d_fitch, *S = ctx->d_scratch, *tmp = nullptr;
  if (!F || !S) {
    CK(cudaMalloc(&tmp, 2 * rows));
    F = tmp; S = tmp + rows;
  }
  const int Wb = (2 * (N - 1) + 31) / 32;
  uint32_t* bits = nullptr;
  cudaError_t e = cudaMalloc(&bits, 2 * (size_t)L * Wb * sizeof(uint32_t));
  if (e == cudaSuccess && !ctx->d_nsubs) {
    e = dalloc(&ctx->d_nsubs, (size_t)ctx->capL);
    if (e == cudaSuccess) e = dalloc(&ctx->d_ndouble, (size_t)ctx->capL * ctx->capL);
    if (e == cudaSuccess) e = dalloc(&ctx->d_njoin, (size_t)ctx->capL * ctx->capL);
  }
  const uint8_t* ax = ctx->d_ax + (size_t)slot * N * Lp;
  NullTree T{N, ctx->d_left, ctx->d_right};
  if (e == cudaSuccess)
    e = launch_fitch_recon(ax, N, L, Lp, T, ctx->d_lnodes, ctx->loff.data(), (int)ctx->loff.size() - 1, seed,
                           kReconStream, F, S, ctx->st);
  if (e == cudaSuccess)
    e = launch_substitutions(ax, F, ctx->d_left, ctx->d_right, N, L, Lp, includegaps ? 1 : 0, bits,
                             bits + (size_t)L * Wb, ctx->d_nsubs, ctx->d_ndouble, ctx->d_njoin, ctx->st);
  if (e == cudaSuccess && nsubs) e = cudaMemcpyAsync(nsubs, ctx->d_nsubs, L * sizeof(int), cudaMemcpyDeviceToHost, ctx->st);
  if (e == cudaSuccess && ndouble)
    e = cudaMemcpyAsync(ndouble, ctx->d_ndouble, (size_t)L * L * sizeof(int), cudaMemcpyDeviceToHost, ctx->st);
  if (e == cudaSuccess && njoin)
    e = cudaMemcpyAsync(njoin, ctx->d_njoin, (size_t)L * L * sizeof(int), cudaMemcpyDeviceToHost, ctx->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->st);
  if (bits) cudaFree(bits);
  if (tmp) cudaFree(tmp);
  if (e != cudaSuccess) return fail(ctx, 90, "CUDA error %s", cudaGetErrorString(e));
  ctx->nlaunch += 4 + 2 * ((int)ctx->loff.size() - 1);
  return 0;
}

extern "C" int covgpu_power(covgpu_ctx* ctx, int ns, const double* subs, const double* prob, const double* subs_join,
                            const double* prob_join, const double* subs_double, const double* prob_double,
                            double* power, double* power_join, double* power_double) {
  if (!ctx) return 11;
  CK(cudaSetDevice(ctx->dev));
  const int L = ctx->L;
  if (!ctx->d_nsubs) return fail(ctx, 11, "no substitutions yet");
  if (ns < 0 || ns > 100000) return fail(ctx, 11, "bad number of power curve points");
  std::vector<double> tab(6 * (size_t)std::max(ns, 1), 0.0);
  const double* src[6] = {subs, prob, subs_join, prob_join, subs_double, prob_double};
  for (int k = 0; k < 6; k++)
    if (src[k]) for (int s = 0; s < ns; s++) tab[(size_t)k * ns + s] = src[k][s];
  const int64_t P = (int64_t)L * (L - 1) / 2;
  double *d_tab = nullptr, *d_out = nullptr;
  CK(dalloc(&d_tab, tab.size()));
  cudaError_t e = dalloc(&d_out, (size_t)3 * std::max<int64_t>(P, 1));
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_tab, tab.data(), tab.size() * sizeof(double), cudaMemcpyHostToDevice, ctx->st);
  if (e == cudaSuccess)
    e = launch_power(ctx->d_nsubs, ctx->d_ndouble, ctx->d_njoin, L, ns, d_tab, subs && prob, subs_join && prob_join,
                     subs_double && prob_double, d_out, d_out + P, d_out + 2 * P, ctx->st);
  double* outs[3] = {power, power_join, power_double};
  for (int k = 0; k < 3 && e == cudaSuccess; k++)
    if (outs[k] && P > 0)
      e = cudaMemcpyAsync(outs[k], d_out + k * P, P * sizeof(double), cudaMemcpyDeviceToHost, ctx->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->st);
  cudaFree(d_tab);
  if (d_out) cudaFree(d_out);
  if (e != cudaSuccess) return fail(ctx, 90, "CUDA error %s", cudaGetErrorString(e));
  return 0;
}

extern "C" int covgpu_gapfilter_dev(covgpu_ctx* ctx, int slot, const double* wgt, double gapthresh, int* useme) {
  if (!ctx) return 11;
  CK(cudaSetDevice(ctx->dev));
  const int N = ctx->N, L = ctx->L, Lp = ctx->Lp;
  if (slot < 0 || slot >= ctx->maxslots || !useme) return fail(ctx, 11, "bad slot or output");
  double* d_w = nullptr;
  int* d_use = nullptr;
  CK(dalloc(&d_use, (size_t)L));
  cudaError_t e = cudaSuccess;
  if (wgt) {
    e = dalloc(&d_w, (size_t)N);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_w, wgt, N * sizeof(double), cudaMemcpyHostToDevice, ctx->st);
  }
  if (e == cudaSuccess) e = launch_gapfilter(ctx->d_ax + (size_t)slot * N * Lp, d_w, N, L, Lp, gapthresh, d_use, ctx->st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(useme, d_use, L * sizeof(int), cudaMemcpyDeviceToHost, ctx->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->st);
  cudaFree(d_use);
  if (d_w) cudaFree(d_w);
  if (e != cudaSuccess) return fail(ctx, 90, "CUDA error %s", cudaGetErrorString(e));
  return 0;
}

extern "C" int covgpu_simulate(covgpu_ctx* ctx, const double* ld, const double* rd, const double* Q4,
                               const double* pi4, const double* Q16, const double* pi16, const int* ct,
                               const uint8_t* root, double gap_rate, double gap_mean, uint64_t seed, uint32_t rep0,
                               int first_slot, int nrep) {
  if (!ctx) return 11;
  CK(cudaSetDevice(ctx->dev));
  ctx->cnt_valid = false;
  const int N = ctx->N, L = ctx->L, Lp = ctx->Lp;
  if (!ctx->have_tree) return fail(ctx, 11, "no tree set");
  if (N < 2) return fail(ctx, 11, "the simulator needs a tree of at least two leaves");
  if (!ld || !rd || !Q4 || !pi4 || !Q16 || !pi16 || !ct) return fail(ctx, 11, "missing simulator argument");
  if (nrep < 1 || first_slot < 0 || first_slot + nrep > ctx->maxslots) return fail(ctx, 11, "slots out of range");
  if (gap_rate < 0.0 || gap_rate > 1.0 || (gap_rate > 0.0 && !(gap_mean >= 1.0)))
    return fail(ctx, 11, "gap_rate in [0,1] and gap_mean >= 1");
  double s4 = 0.0, s16 = 0.0;
  for (int k = 0; k < 4; k++) { if (!(pi4[k] >= 0.0)) return fail(ctx, 11, "bad background"); s4 += pi4[k]; }
  for (int k = 0; k < 16; k++) { if (!(pi16[k] >= 0.0)) return fail(ctx, 11, "bad background"); s16 += pi16[k]; }
  if (fabs(s4 - 1.0) > 1e-6 || fabs(s16 - 1.0) > 1e-6) return fail(ctx, 11, "backgrounds must sum to 1");
  // units: unpaired columns and base pairs (c < partner), in column order
  std::vector<int2> units;
  for (int c = 0; c < L; c++) {
    const int p = ct[c];
    if (p < -1 || p >= L || p == c || (p >= 0 && ct[p] != c)) return fail(ctx, 11, "ct: bad partner of column %d", c);
    if (p >= 0 && p < c) continue;
    units.push_back(make_int2(c, p));
    if (root && (root[c] > 3 || (p >= 0 && root[p] > 3))) return fail(ctx, 11, "root: non-canonical residue");
  }
  const int nunits = (int)units.size();
  const int nb = 2 * (N - 1);
  std::vector<double> times(nb), Q(16 + 256 + 4 + 16);
  for (int v = 0; v < N - 1; v++) { times[2 * v] = ld[v]; times[2 * v + 1] = rd[v]; }
  for (int k = 0; k < 16; k++) Q[k] = Q4[k];
  for (int k = 0; k < 256; k++) Q[16 + k] = Q16[k];
  for (int k = 0; k < 4; k++) Q[272 + k] = pi4[k];
  for (int k = 0; k < 16; k++) Q[276 + k] = pi16[k];
  if (ctx->sim_branches != nb) {
    void* old[] = {ctx->d_simT, ctx->d_P4, ctx->d_P16, ctx->d_C4, ctx->d_C16};
    for (void* p : old) if (p) cudaFree(p);
    CK(dalloc(&ctx->d_simT, nb));
    CK(dalloc(&ctx->d_P4, (size_t)nb * 16));
    CK(dalloc(&ctx->d_P16, (size_t)nb * 256));
    CK(dalloc(&ctx->d_C4, (size_t)nb * 16));
    CK(dalloc(&ctx->d_C16, (size_t)nb * 256));
    ctx->sim_branches = nb;
  }
  if (!ctx->d_simQ) {
    CK(dalloc(&ctx->d_simQ, 16 + 256 + 4 + 16));
    CK(dalloc(&ctx->d_R, 4 + 16));
    CK(dalloc(&ctx->d_units, ctx->capL));
    CK(dalloc(&ctx->d_simroot, ctx->capLp));
  }
  const size_t need = (size_t)nrep * (N - 1) * nunits;
  if (ctx->simstate_cap < need) {
    if (ctx->d_simstate) cudaFree(ctx->d_simstate);
    CK(dalloc(&ctx->d_simstate, need));
    ctx->simstate_cap = need;
  }
  CK(cudaMemcpyAsync(ctx->d_units, units.data(), nunits * sizeof(int2), cudaMemcpyHostToDevice, ctx->st));
  if (root) CK(cudaMemcpyAsync(ctx->d_simroot, root, L, cudaMemcpyHostToDevice, ctx->st));
  // the tables depend on the branch times and the model only: keep them
  // across calls on the same tree and model
  std::vector<double> key(times);
  key.insert(key.end(), Q.begin(), Q.end());
  if (key != ctx->sim_key) {
    CK(cudaMemcpyAsync(ctx->d_simT, times.data(), nb * sizeof(double), cudaMemcpyHostToDevice, ctx->st));
    CK(cudaMemcpyAsync(ctx->d_simQ, Q.data(), Q.size() * sizeof(double), cudaMemcpyHostToDevice, ctx->st));
    CK(launch_sim_tables(ctx->d_simQ, ctx->d_simQ + 16, ctx->d_simQ + 272, ctx->d_simQ + 276, ctx->d_simT, nb,
                         ctx->d_P4, ctx->d_P16, ctx->d_C4, ctx->d_C16, ctx->d_R, ctx->d_R + 4, ctx->d_status,
                         ctx->st));
    ctx->sim_key.swap(key);
  }
  const int64_t sstride = (int64_t)N * Lp;
  CK(launch_sim_evolve(ctx->d_left, ctx->d_right, ctx->d_lnodes, ctx->loff.data(), (int)ctx->loff.size() - 1, N, L,
                       Lp, ctx->d_units, nunits, ctx->d_C4, ctx->d_C16, ctx->d_R,
                       ctx->d_R + 4, root ? ctx->d_simroot : nullptr, gap_rate, gap_mean, seed, rep0, nrep,
                       ctx->d_simstate, ctx->d_ax + first_slot * sstride, sstride, ctx->st));
  ctx->nlaunch += 6;
  int s = 0;
  CK(cudaMemcpyAsync(&s, ctx->d_status, sizeof(int), cudaMemcpyDeviceToHost, ctx->st));
  CK(cudaStreamSynchronize(ctx->st));
  if (s == 41 || s == 42) {
    cudaMemset(ctx->d_status, 0, sizeof(int));
    return fail(ctx, s, s == 41 ? "negative branch length" : "P(t) needed regularisation beyond -1e-3");
  }
  return check_status(ctx);
}

extern "C" int covgpu_sim_tables(covgpu_ctx* ctx, double* P4, double* P16) {
  if (!ctx) return 11;
  CK(cudaSetDevice(ctx->dev));
  if (!ctx->sim_branches) return fail(ctx, 11, "no simulation yet");
  if (P4) CK(cudaMemcpy(P4, ctx->d_P4, (size_t)ctx->sim_branches * 16 * sizeof(double), cudaMemcpyDeviceToHost));
  if (P16) CK(cudaMemcpy(P16, ctx->d_P16, (size_t)ctx->sim_branches * 256 * sizeof(double), cudaMemcpyDeviceToHost));
  return 0;
}

extern "C" int covgpu_make_nulls(covgpu_ctx* ctx, uint64_t seed, int first_null, int nnull, int first_slot) {
  if (!ctx) return 11;
  CK(cudaSetDevice(ctx->dev));
  int s = make_nulls_async(ctx, seed, first_null, nnull, first_slot);
  if (s) return s;
  CK(cudaStreamSynchronize(ctx->st));
  return 0;
}

// ------------------------------------------------------------------------
// scoring
// ------------------------------------------------------------------------
static int stat_index(int base) {
  switch (base) {
    case 0: return 0;    // CHI
    case 3: return 1;    // GT
    case 6: return 2;    // MI
    case 9: return 3;    // MIr
    case 12: return 4;   // MIg
    case 15: return 5;   // OMES
    case 18: return 6;   // RAF
    case 21: return 6;   // RAFS (RAF, then the stencil)
    case 24: return 8;   // CCF
  }
  return -1;
}

static int score_async(covgpu_ctx* ctx, int first, int nslots, int ntypes, const int* types, int covclass,
                       int nseqthresh, int alenthresh, const double* allow, int counter, bool reuse = false) {
  if (ntypes < 1 || ntypes > MAXOUT) return fail(ctx, 11, "1..%d covariation types per call", MAXOUT);
  if (first < 0 || nslots < 1 || first + nslots > ctx->maxslots) return fail(ctx, 11, "slots out of range");
  if (!ctx->have_w) return fail(ctx, 11, "weights not set");
  const int N = ctx->N, L = ctx->L, Lp = ctx->Lp, nT = ctx->nT, ntiles = ctx->ntiles;
  bool need_w = false, need_u = false;
  unsigned mask = 0;
  StatsArgs A;
  memset(&A, 0, sizeof(A));
  CorrTypes ct;
  ct.nout = ntypes;
  int rafs_q[MAXOUT], nrafs = 0;
  int cls = covclass;
  if (cls == 3) cls = (N <= nseqthresh || L <= alenthresh) ? 1 : 0;
  for (int q = 0; q < ntypes; q++) {
    if (types[q] < 0 || types[q] >= 27) return fail(ctx, 11, "covariation type %d not supported", types[q]);
    const int base = (types[q] / 3) * 3, corr = types[q] % 3;
    const int si = stat_index(base);
    A.outstat[q] = si;
    ct.act[q] = (corr == 0) ? -1 : corr - 1;
    if (base == 18 || base == 21) { need_u = true; mask |= S_RAF; }
    else { need_w = true; mask |= (1u << si); }
    if (base == 24) mask |= S_CCF;
    if (base == 21) rafs_q[nrafs++] = q;
    if (cls == 2 && base != 3 && base != 18 && base != 21 && base != 24)
      return fail(ctx, 11, "class CWC is only defined for GT");
  }
  for (int q = ntypes; q < MAXOUT; q++) { A.outstat[q] = 0; ct.act[q] = -1; }
  const int64_t sstride = (int64_t)N * Lp;
  const uint8_t* ax = ctx->d_ax + first * sstride;
  const int64_t cstride = (int64_t)ntiles * 16 * TPP;
  const bool have = reuse && ctx->cnt_valid && ctx->cnt_first == first && ctx->cnt_nslots == nslots &&
                    ctx->cnt_counter == counter;
  if (need_w && !have) {
    if (counter == COVGPU_COUNT_TENSOR) {
      if (!ctx->umma) {
        ctx->umma = umma_plan_create(N, L, Lp, ctx->nT, ctx->d_tiles, ntiles, ctx->maxslots, ctx->capN, ctx->capLp,
                                     ctx->capntiles);
        if (!ctx->umma) return fail(ctx, 12, "tensor counting not available for this shape");
        umma_set_weights(ctx->umma, ctx->h_w.data(), N, ctx->st);
      }
      CK(umma_count(ctx->umma, ax, sstride, nslots, false, ctx->d_cnt, ctx->st, ctx->ev[4], ctx->ev[5]));
    } else {
      cudaEventRecord(ctx->ev[4], ctx->st);
      CK(launch_count_simt(ax, sstride, ctx->cw, false, N, Lp, ctx->d_tiles, ntiles, nslots, ctx->d_cnt, ctx->st));
      cudaEventRecord(ctx->ev[5], ctx->st);
    }
    ctx->counted = true;
    CK(launch_pair_marg(ctx->d_cnt, L, ctx->d_tiles, ntiles, nT, nslots, ctx->d_part4, ctx->d_partR, ctx->st));
    CK(launch_pm_final(ctx->d_part4, ctx->d_partR, L, Lp, nT, nslots, ctx->d_pm, ctx->d_pmdf, ctx->d_lpi, ctx->d_ps,
                       ctx->d_meanp, ctx->d_status, ctx->st));
    // operand preparation + count (tensor) or count; marginals, pm, mean p
    ctx->nlaunch += (counter == COVGPU_COUNT_TENSOR ? 2 : 1) + 3;
    ctx->cnt_valid = true;
    ctx->cnt_first = first; ctx->cnt_nslots = nslots; ctx->cnt_counter = counter;
  }
  if (need_u) {
    if (!ctx->d_ucnt) CK(dalloc(&ctx->d_ucnt, (size_t)ctx->maxslots * ctx->capntiles * 16 * TPP));
    if (counter == COVGPU_COUNT_TENSOR && ctx->umma) {
      // RAF reads the unit counts of the allowed cells only
      unsigned mask = 0;
      for (int k = 0; k < 16; k++) if (allow[k] > 0.0) mask |= 1u << k;
      CK(umma_count(ctx->umma, ax, sstride, nslots, true, ctx->d_ucnt, ctx->st, nullptr, nullptr, mask));
    } else {
      CK(launch_count_simt(ax, sstride, ctx->cw, true, N, Lp, ctx->d_tiles, ntiles, nslots, ctx->d_ucnt, ctx->st));
    }
    ctx->nlaunch += (counter == COVGPU_COUNT_TENSOR && ctx->umma) ? 2 : 1;   // FP8 preparation + count
  }
  A.cnt = need_w ? ctx->d_cnt : nullptr;
  A.ucnt = need_u ? ctx->d_ucnt : nullptr;
  A.pm = ctx->d_pm;
  A.pmdf = ctx->d_pmdf;
  A.lpi = ctx->d_lpi;
  A.logtab = ctx->d_logtab;
  A.meanp = ctx->d_meanp;
  A.cov = ctx->d_cov;
  A.part1 = ctx->d_part1;
  A.tiles = ctx->d_tiles;
  A.ntiles = ntiles; A.nT = nT; A.L = L; A.Lp = Lp; A.N = N;
  {
    const float hi = (float)ctx->wtot_q;
    A.wtot = make_float2(hi, (float)(ctx->wtot_q - (double)hi));
  }
  A.stats = mask;
  A.cls = cls;
  {
    auto split = [](double x) { const float h = (float)x; return make_float2(h, (float)(x - (double)h)); };
    A.invD = split(1.0 / ((N > 1) ? (double)N * ((double)N - 1.0) : 1.0));
    A.invN = split(1.0 / (double)N);
  }
  A.nout = ntypes;
  for (int k = 0; k < 16; k++) A.allow[k] = (float)allow[k];
  if (!need_w) {
    // RAF only: pm is never read, but keep the pointers valid
    CK(cudaMemsetAsync(ctx->d_pm, 0, (size_t)nslots * Lp * 4 * sizeof(double), ctx->st));
    CK(cudaMemsetAsync(ctx->d_pmdf, 0, (size_t)nslots * Lp * 4 * sizeof(float2), ctx->st));
    CK(cudaMemsetAsync(ctx->d_lpi, 0, (size_t)nslots * Lp * 4 * sizeof(float4), ctx->st));
  }
  CK(launch_stats(A, nslots, ctx->st));
  ctx->nlaunch += 1;
  const int64_t plane = (int64_t)ntiles * TPP;
  const int64_t pplane = (int64_t)nT * nT * TP;
  for (int r = 0; r < nrafs; r++) {
    const int q = rafs_q[r];
    if (!ctx->d_cov2) CK(dalloc(&ctx->d_cov2, (size_t)ctx->maxslots * ctx->capntiles * TPP));
    CK(cudaMemcpy2DAsync(ctx->d_cov2, plane * sizeof(float2), ctx->d_cov + q * plane, ntypes * plane * sizeof(float2),
                         plane * sizeof(float2), nslots, cudaMemcpyDeviceToDevice, ctx->st));
    CK(launch_rafs(ctx->d_cov2, ctx->d_cov + q * plane, plane, ntypes * plane, ctx->d_tiles, ctx->d_tile_index, ntiles,
                   nT, L, nslots, ctx->d_part1 + q * pplane, ntypes * pplane, ctx->st));
    ctx->nlaunch += 1;
  }
  CK(launch_apc(ctx->d_cov, ctx->d_part1, ctx->d_colx, ctx->d_colxf, ctx->d_avg, ctx->d_apcf, ct, ctx->d_tiles,
                ntiles, nT, L, Lp, nslots * ntypes, ctx->d_tmin, ctx->d_tmax, ctx->d_mm, ctx->d_status, ctx->st));
  ctx->nlaunch += 4;
  ctx->last_nout = ntypes; ctx->last_first = first; ctx->last_nslots = nslots;
  return 0;
}

static int check_status(covgpu_ctx* ctx) {
  int s = 0;
  CK(cudaMemcpyAsync(&s, ctx->d_status, sizeof(int), cudaMemcpyDeviceToHost, ctx->st));
  CK(cudaStreamSynchronize(ctx->st));
  if (ctx->umma) {
    const int ue = umma_error(ctx->umma);
    if (ue) return fail(ctx, 24, "tensor counting kernel: barrier wait timed out (code %d)", ue);
  }
  if (s) {
    cudaMemsetAsync(ctx->d_status, 0, sizeof(int), ctx->st);
    if (s == 2) return fail(ctx, 20, "marginal probabilities failed validation");
    if (s == 3) return fail(ctx, 21, "bad covariation: NaN after correction");
    if (s == 4) return fail(ctx, 22, "histogram bin out of range");
    return fail(ctx, 23, "device status %d", s);
  }
  return 0;
}

static int score_sync(covgpu_ctx* ctx, int first_slot, int nslots, int ntypes, const int* covtypes, int covclass,
                      int nseqthresh, int alenthresh, const double* allow, int counter, double* minmax, bool reuse) {
  CK(cudaSetDevice(ctx->dev));
  int s = score_async(ctx, first_slot, nslots, ntypes, covtypes, covclass, nseqthresh, alenthresh, allow, counter,
                      reuse);
  if (s) return s;
  if (minmax)
    CK(cudaMemcpyAsync(minmax, ctx->d_mm, (size_t)nslots * ntypes * 2 * sizeof(double), cudaMemcpyDeviceToHost,
                       ctx->st));
  CK(cudaStreamSynchronize(ctx->st));
  return check_status(ctx);
}

extern "C" int covgpu_score(covgpu_ctx* ctx, int first_slot, int nslots, int ntypes, const int* covtypes,
                            int covclass, int nseqthresh, int alenthresh, const double* allow, int counter,
                            double* minmax) {
  if (!ctx) return 11;
  return score_sync(ctx, first_slot, nslots, ntypes, covtypes, covclass, nseqthresh, alenthresh, allow, counter,
                    minmax, false);
}

extern "C" int covgpu_score_reuse(covgpu_ctx* ctx, int first_slot, int nslots, int ntypes, const int* covtypes,
                                  int covclass, int nseqthresh, int alenthresh, const double* allow, int counter,
                                  double* minmax) {
  if (!ctx) return 11;
  return score_sync(ctx, first_slot, nslots, ntypes, covtypes, covclass, nseqthresh, alenthresh, allow, counter,
                    minmax, true);
}

extern "C" int covgpu_get_cov(covgpu_ctx* ctx, int slot, int which, double* COV) {
  if (!ctx) return 11;
  CK(cudaSetDevice(ctx->dev));
  const int rel = slot - ctx->last_first;
  if (rel < 0 || rel >= ctx->last_nslots || which < 0 || which >= ctx->last_nout)
    return fail(ctx, 11, "no scores for slot %d / type %d", slot, which);
  if (!ctx->d_full) CK(dalloc(&ctx->d_full, (size_t)ctx->capL * ctx->capL));
  const int64_t plane = (int64_t)ctx->ntiles * TPP;
  CK(launch_untile(ctx->d_cov + ((int64_t)rel * ctx->last_nout + which) * plane, ctx->d_tiles, ctx->ntiles, ctx->L,
                   -INFINITY, ctx->d_full, ctx->st));
  CK(cudaMemcpyAsync(COV, ctx->d_full, (size_t)ctx->L * ctx->L * sizeof(double), cudaMemcpyDeviceToHost, ctx->st));
  CK(cudaStreamSynchronize(ctx->st));
  return 0;
}

extern "C" int covgpu_get_probs(covgpu_ctx* ctx, int slot, const double* wgt, double* pp, double* nseff,
                                double* ngap, double* pm, double* ps) {
  if (!ctx) return 11;
  CK(cudaSetDevice(ctx->dev));
  const int rel = slot - ctx->last_first;
  if (rel < 0 || rel >= ctx->last_nslots) return fail(ctx, 11, "slot %d was not scored", slot);
  const int L = ctx->L, Lp = ctx->Lp, N = ctx->N;
  if (pm) {
    std::vector<double> t((size_t)Lp * 4);
    CK(cudaMemcpyAsync(t.data(), ctx->d_pm + (size_t)rel * Lp * 4, t.size() * sizeof(double), cudaMemcpyDeviceToHost,
                       ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    memcpy(pm, t.data(), (size_t)L * 4 * sizeof(double));
  }
  if (ps) {
    CK(launch_ps(ctx->d_ax + (size_t)slot * N * Lp, (int64_t)N * Lp, ctx->d_wd, N, L, Lp, 1, ctx->d_ps, ctx->st));
    std::vector<double> t((size_t)Lp * 5);
    CK(cudaMemcpyAsync(t.data(), ctx->d_ps, t.size() * sizeof(double), cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    memcpy(ps, t.data(), (size_t)L * 5 * sizeof(double));
  }
  if (pp || nseff || ngap) {
    // ngap = (sum of the weights) - nseff, both of the quantised weights the
    // counts were made from (wgt, when given, for the exact total)
    double wt = ctx->wtot_q;
    if (wgt) { wt = 0.0; for (int s = 0; s < N; s++) wt += wgt[s]; }
    // the reference's host layout, made on the device and copied in one
    // transfer per array (the diagonal and ngap's lower triangle stay zero)
    const size_t LL = (size_t)L * L;
    if (!ctx->d_pphost) CK(dalloc(&ctx->d_pphost, (size_t)ctx->capL * ctx->capL * 18));
    double* dpp = ctx->d_pphost;
    double* dns = dpp + LL * 16;
    double* dng = dns + LL;
    CK(cudaMemsetAsync(dpp, 0, LL * 18 * sizeof(double), ctx->st));
    CK(launch_probs_host_layout(ctx->d_cnt + (size_t)rel * ctx->ntiles * 32 * TPP, ctx->d_tiles, ctx->ntiles, L, wt,
                                pp ? dpp : nullptr, nseff ? dns : nullptr, ngap ? dng : nullptr, ctx->st));
    if (pp) CK(cudaMemcpyAsync(pp, dpp, LL * 16 * sizeof(double), cudaMemcpyDeviceToHost, ctx->st));
    if (nseff) CK(cudaMemcpyAsync(nseff, dns, LL * sizeof(double), cudaMemcpyDeviceToHost, ctx->st));
    if (ngap) CK(cudaMemcpyAsync(ngap, dng, LL * sizeof(double), cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
  }
  return 0;
}

// ------------------------------------------------------------------------
// the whole per-alignment path
// ------------------------------------------------------------------------
static double elapsed(cudaEvent_t a, cudaEvent_t b) {
  float ms = 0.f;
  cudaEventElapsedTime(&ms, a, b);
  return (double)ms;
}

static int bins_for(double bmin, double bmax, double w) {
  int nb = (int)((bmax - bmin) / w);
  return nb < 1 ? 1 : nb;
}

// Summary of a null histogram (features 47-63 of the learned null): log of
// the number of scores; the tail fit mu_q, log m_q (m_q = tau/lambda, the
// mean excess), log tau_q (from the quantiles when the fit failed); and,
// as offsets from mu_q in units of m_q, the mean of the scores (bin
// midpoints), their deviation, the upper quantiles at survival 0.5 ...
// 0.0005 (linear within a bin) and the largest null score.
static void null_summary(const ESL_HISTOGRAM* h, double xmax, double mu, double lambda, double tau, double* out) {
  static const double lev[10] = {0.5, 0.3, 0.1, 0.05, 0.03, 0.01, 0.005, 0.003, 0.001, 0.0005};
  double tot = 0.0, s1 = 0.0, s2 = 0.0;
  for (int b = 0; b < h->nb; b++) {
    const double c = (double)h->obs[b];
    tot += c;
    s1 += c * (h->bmin + (b + 0.5) * h->w);
  }
  const double mean = tot > 0.0 ? s1 / tot : 0.0;
  for (int b = 0; b < h->nb; b++) {
    const double d = h->bmin + (b + 0.5) * h->w - mean;
    s2 += (double)h->obs[b] * d * d;
  }
  out[0] = tot > 0.0 ? log(tot) : 0.0;
  out[1] = mean;
  out[2] = tot > 0.0 ? sqrt(s2 / tot) : 0.0;
  for (int k = 0; k < 10; k++) {
    const double target = lev[k] * tot;
    double above = 0.0, qv = h->bmin;
    for (int b = h->nb - 1; b >= 0; b--) {
      const double c = (double)h->obs[b];
      if (c > 0.0 && above + c >= target) {
        qv = h->bmin + (b + 1) * h->w - (target - above) / c * h->w;
        break;
      }
      above += c;
    }
    out[3 + k] = qv;
  }
  if (std::isfinite(mu) && lambda > 0.0 && std::isfinite(lambda) && tau > 0.0 && std::isfinite(tau)) {
    out[13] = mu; out[14] = log(tau / lambda); out[15] = log(tau);
  } else {
    out[13] = out[12];
    out[14] = log(std::max(h->w, (out[12] - out[9]) / log(10.0)));
    out[15] = 0.0;
  }
  out[16] = xmax;
  // the location features relative to the tail fit, in its own scale
  const double m = exp(out[14]);
  out[1] = (out[1] - out[13]) / m;
  out[2] = out[2] / m;
  for (int k = 0; k < 10; k++) out[3 + k] = (out[3 + k] - out[13]) / m;
  out[16] = (out[16] - out[13]) / m;
}

// ------------------------------------------------------------------------
// the host steps of the E-valued path per statistic, shared by
// covgpu_rscape and the family batch (cov_rscape_host.h)
// ------------------------------------------------------------------------
int rs_nshuffle(const covgpu_params* p, int N, int L, double* fracfit) {
  int ns = p->nshuffle;
  *fracfit = p->fracfit;
  if (ns < 0) {   // src/R-scape.c:2449-2456
    ns = 20;
    if ((double)N * L < 1e3) ns = 200;
    if (L < 50) ns = 200;
    if (L < 40) ns = 300;
    if (N < 4) ns = 300;
  }
  if ((double)N * L < 1e3) *fracfit = 0.3;   // :2458-2459
  if (N == 1) ns = 0;
  return ns;
}

int rs_width(const covgpu_params* p, int N, int ns, const double* mm, int ntypes, int q, covgpu_result& R,
             RsStat& X, char* err, size_t errlen) {
  auto MMn = [&](int slot, int k) { return mm[((size_t)slot * ntypes + q) * 2 + k]; };
  R.nshuffle = ns;
  R.minCOV = MMn(0, 0); R.maxCOV = MMn(0, 1);
  if (N == 1) { R.status = 2; return 0; }
  // calculate_width_histo (src/R-scape.c:1353-1360) on the first null
  double w = p->w0;
  const double nmin = MMn(1, 0), nmax = MMn(1, 1);
  R.null_minCOV = nmin; R.null_maxCOV = nmax;
  if (nmax <= p->bmin) {
    snprintf(err, errlen, "bmin %f should be larger than maxCOV %f", p->bmin, nmax);
    return 30;
  }
  const double wn = (nmax - std::max(p->bmin, nmin)) / (double)p->hpts;
  w = std::min(w, wn);
  if (w < p->tol) w = 0.0;
  R.w = w;
  if (w < 1e-20) { R.status = 1; return 0; }   // src/covariation.c:348-374
  // null histograms share bmin and w: their sum is the cumulative null
  int nbcum = 0;
  double xmin = INFINITY, xmax = -INFINITY;
  for (int k = 1; k <= ns; k++) {
    double bmax = MMn(k, 1) + 5 * w;
    while (fabs(bmax - p->bmin) < p->tol) bmax += w;
    nbcum = std::max(nbcum, bins_for(p->bmin, bmax, w));
    xmin = std::min(xmin, std::max(MMn(k, 0), p->bmin + w));
    xmax = std::max(xmax, std::max(MMn(k, 1), p->bmin + w));
  }
  double bmax_r = R.maxCOV + 5 * w;
  while (fabs(bmax_r - p->bmin) < p->tol) bmax_r += w;
  X.active = true;
  X.w = w; X.xmin = xmin; X.xmax = xmax; X.nbcum = nbcum;
  X.nb_real = bins_for(p->bmin, bmax_r, w);
  // the window starts one bin below the smallest null score's bin
  X.wbase = std::isfinite(xmin) ? std::max(0, (int)std::floor((xmin - p->bmin) / w) - 2) : 0;
  return 0;
}

int rs_histogram(const covgpu_params* p, double fracfit, int ns, int64_t P, const uint64_t* ob, RsStat& X, char* err,
                 size_t errlen) {
  const int nbcum = X.nbcum;
  double bmax_c = p->bmin + nbcum * X.w;
  ESL_HISTOGRAM* h = covh_Create(p->bmin, bmax_c, X.w);
  if (!h) { snprintf(err, errlen, "out of host memory"); return 5; }
  X.h = h;
  if (h->nb != nbcum) {   // guard the rounding of (bmax - bmin)/w
    free(h->obs); h->nb = nbcum; h->obs = (uint64_t*)calloc(nbcum, sizeof(uint64_t));
  }
  uint64_t tot = 0;
  int imin = nbcum, imax = -1;
  for (int b = 0; b < nbcum; b++) {
    h->obs[b] = ob[b]; tot += ob[b];
    if (ob[b]) { imin = std::min(imin, b); imax = std::max(imax, b); }
  }
  h->n = (uint64_t)ns * (uint64_t)P; h->Nc = tot; h->No = tot;
  h->xmin = X.xmin; h->xmax = X.xmax; h->imin = imin; h->imax = imax; h->cmin = imin;
  if (h->nb < X.nb_real) {   // src/covariation.c:462-466
    h->obs = (uint64_t*)realloc(h->obs, sizeof(uint64_t) * X.nb_real);
    for (int b = h->nb; b < X.nb_real; b++) h->obs[b] = 0;
    h->nb = X.nb_real;
  }
  X.pmass = covh_pmass(h, p->pmass, fracfit);
  if (std::isnan(X.pmass)) { snprintf(err, errlen, "bad null histogram fit, pmass is nan"); return 31; }
  // tail by mass, then the tail fit and the survival table on the device
  // (src/covariation.c:1914-1973)
  X.newmass = covh_SetTailByMass(h, X.pmass);
  X.mu = h->phi;
  if (p->doexpfit) {
    double n = 0.0, sk = 0.0;
    for (int b = h->cmin; b <= h->imax; b++) { n += (double)h->obs[b]; sk += (double)(b - h->cmin) * (double)h->obs[b]; }
    if (n <= 0) { snprintf(err, errlen, "could not do exponential fit"); return 32; }
    X.lambda = (sk > 0.0) ? log(1.0 + n / sk) / h->w : INFINITY;
  }
  return 0;
}

void rs_tables(const covgpu_params* p, int64_t P, int64_t Nb, RsStat& X, const double* sf, covgpu_result& R,
               double* tq) {
  const ESL_HISTOGRAM* h = X.h;
  R.pmass = X.pmass; R.newmass = X.newmass; R.mu = X.mu; R.lambda = X.lambda; R.tau = X.tau;
  // the pairs outside the structure are Nt = P - Nb tests; the thresholds of
  // base pairs and of the others (src/covariation.c:490-500)
  R.Nt = (uint64_t)(P - Nb);
  R.Nb = (uint64_t)Nb;
  R.sc_thresh = covh_evalue2cov(p->thresh, (double)(Nb > 0 ? Nb : P), X.h, X.have_sf ? sf : nullptr);
  R.sc_nbp = covh_evalue2cov(p->thresh, (double)(Nb > 0 ? P - Nb : P), X.h, X.have_sf ? sf : nullptr);
  R.h_bmin = h->bmin; R.h_w = h->w; R.h_nb = h->nb; R.h_imin = h->imin; R.h_imax = h->imax; R.h_cmin = h->cmin;
  R.h_n = h->n; R.h_Nc = h->Nc; R.h_No = h->No; R.h_xmin = h->xmin; R.h_xmax = h->xmax; R.h_phi = h->phi;
  // cov2evalue tables: the tail branch's p-values tail[b] / Nc
  double c = 0.0;
  for (int b = h->nb - 1; b >= 0; b--) { if (b <= h->imax) c += (double)h->obs[b]; tq[b] = c; }
  for (int b = 0; b < h->nb; b++) tq[b] /= (double)h->Nc;
}

EvalTables rs_evaltables(const covgpu_params* p, int64_t Nt, const RsStat& X, const double* d_sf,
                         const double* d_tail) {
  const ESL_HISTOGRAM* h = X.h;
  EvalTables T;
  T.sf = X.have_sf ? d_sf : nullptr;
  T.ptail = d_tail;
  T.bmin = h->bmin; T.w = h->w; T.phi = h->phi; T.xmax = h->xmax; T.Nc = (double)h->Nc; T.Nt = (double)Nt;
  T.pNc = 1.0 / T.Nc;
  T.thresh = p->thresh; T.nb = h->nb; T.imin = h->imin; T.imax = h->imax;
  return T;
}

int rs_pair_sets(const covgpu_params* p, int L, std::vector<uint32_t>& bpmask, int64_t* nsel, char* err,
                 size_t errlen) {
  const int64_t P = (int64_t)L * (L - 1) / 2;
  bpmask.clear();
  *nsel = 0;
  if (p->ncnt <= 0 || p->samplesize == 3) return 0;
  if (p->samplesize < 0 || p->samplesize > 3) { snprintf(err, errlen, "samplesize %d", p->samplesize); return 11; }
  if (!p->cnt_i || !p->cnt_j || !p->cnt_type) { snprintf(err, errlen, "%d contacts without arrays", p->ncnt); return 11; }
  auto takes = [&](int t) {
    return p->samplesize == 0 ? t < 34 : (p->samplesize == 1 ? t < 32 : t == 0);
  };
  std::vector<uint32_t> sel((size_t)(P + 31) / 32 + 1, 0u), seen((size_t)(P + 31) / 32 + 1, 0u);
  bpmask.assign((size_t)(P + 31) / 32 + 1, 0u);
  for (int h = 0; h < p->ncnt; h++) {
    const int64_t i = p->cnt_i[h], j = p->cnt_j[h];
    if (i < 1 || j > L || i >= j) continue;   // the reference matches cnt.i == i + 1 < cnt.j == j + 1 only
    const int64_t n = (i - 1) * (2LL * L - (i - 1) - 1) / 2 + (j - i - 1);
    const uint32_t bit = 1u << (n & 31);
    if (!(seen[n >> 5] & bit)) {   // the first contact's type (CMAP_GetBPTYPE)
      seen[n >> 5] |= bit;
      if (takes(p->cnt_type[h])) bpmask[n >> 5] |= bit;
    }
    if (takes(p->cnt_type[h])) sel[n >> 5] |= bit;   // any contact (CMAP_Is*Local)
  }
  for (uint32_t w : sel) *nsel += __builtin_popcount(w);
  return 0;
}

// --structured (src/covariation.c:850-854): a pair outside the structure
// takes expBP tests while fewer than expBP hits precede it in scan order.
// Up to the hit that brings the count to m = ceil(expBP) every pair follows
// that rule (Nb tests for the structure's base pairs), so that hit is the
// m-th of the pairs that are hits under it: one compaction pass of the
// statistic's scores with the rule, its scan index into *kstar (LLONG_MAX
// when fewer than m pairs are such hits).
static int structured_kstar(covgpu_ctx* ctx, const float2* cov, EvalTables T, double expBP, long long* kstar) {
  const int L = ctx->L;
  T.Nx = expBP;
  T.kstar = LLONG_MAX;
  const long long m = (long long)std::ceil(expBP);
  for (int round = 0; round < 2; round++) {
    if (ctx->ccap < 1024) {
      cudaFree(ctx->d_ci); cudaFree(ctx->d_cj); cudaFree(ctx->d_cd);
      ctx->d_ci = ctx->d_cj = nullptr; ctx->d_cd = nullptr; ctx->ccap = 0;
      CK(dalloc(&ctx->d_ci, 1024)); CK(dalloc(&ctx->d_cj, 1024)); CK(dalloc(&ctx->d_cd, 3 * 1024));
      ctx->ccap = 1024;
    }
    const int cap = ctx->ccap;
    CK(cudaMemsetAsync(ctx->d_nhits + MAXOUT, 0, sizeof(int), ctx->st));
    CK(launch_evalue(cov, ctx->d_tiles, ctx->ntiles, L, T, nullptr, ctx->d_nhits + MAXOUT, cap, ctx->d_ci, ctx->d_cj,
                     ctx->d_cd, ctx->d_cd + cap, ctx->d_cd + 2 * cap, ctx->st));
    int nc = 0;
    CK(cudaMemcpyAsync(&nc, ctx->d_nhits + MAXOUT, sizeof(int), cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    ctx->nlaunch += 1;
    if (nc > cap) {   // room for all of them, then once more
      cudaFree(ctx->d_ci); cudaFree(ctx->d_cj); cudaFree(ctx->d_cd);
      ctx->d_ci = ctx->d_cj = nullptr; ctx->d_cd = nullptr; ctx->ccap = 0;
      CK(dalloc(&ctx->d_ci, nc)); CK(dalloc(&ctx->d_cj, nc)); CK(dalloc(&ctx->d_cd, 3 * (size_t)nc));
      ctx->ccap = nc;
      continue;
    }
    std::vector<int> ci(nc), cj(nc);
    if (nc > 0) {
      CK(cudaMemcpy(ci.data(), ctx->d_ci, nc * sizeof(int), cudaMemcpyDeviceToHost));
      CK(cudaMemcpy(cj.data(), ctx->d_cj, nc * sizeof(int), cudaMemcpyDeviceToHost));
    }
    std::vector<long long> n(nc);
    for (int k = 0; k < nc; k++) n[k] = (long long)ci[k] * (2LL * L - ci[k] - 1) / 2 + (cj[k] - ci[k] - 1);
    if ((long long)nc < m) { *kstar = LLONG_MAX; return 0; }
    std::nth_element(n.begin(), n.begin() + (m - 1), n.end());
    *kstar = n[m - 1];
    return 0;
  }
  return fail(ctx, 90, "--structured: the hit count changed between two passes");
}

extern "C" int covgpu_rscape(covgpu_ctx* ctx, const covgpu_params* p, const uint8_t* ax, const double* wgt,
                             int ntypes, const int* covtypes, covgpu_result* results, covgpu_hit* hits, int hitcap) {
  if (!ctx) return 11;
  CK(cudaSetDevice(ctx->dev));
  const int N = ctx->N, L = ctx->L;
  const int64_t P = (int64_t)L * (L - 1) / 2;
  if (ntypes < 1 || ntypes > MAXOUT) return fail(ctx, 11, "1..%d covariation types per call", MAXOUT);
  for (int q = 0; q < ntypes; q++) {
    memset(&results[q], 0, sizeof(covgpu_result));
    results[q].covtype = covtypes[q];
  }
  ctx->nlaunch = 0;
  ctx->counted = false;
  ctx->cnt_valid = false;
  ctx->fit_ms = 0.0;
  int s;
  // ax / wgt == NULL: use the alignment and weights already on the device
  if (wgt && (s = covgpu_set_weights(ctx, wgt))) return s;
  if (ax && (s = covgpu_set_alignment(ctx, 0, ax))) return s;
  if (!ctx->have_w) return fail(ctx, 11, "weights not set");
  // the two-set test's pairs (none in the one-set test)
  std::vector<uint32_t> bpmask;
  int64_t Nb = 0;
  if ((s = rs_pair_sets(p, L, bpmask, &Nb, ctx->err, sizeof(ctx->err)))) return s;
  double fracfit = p->fracfit;
  const int ns = rs_nshuffle(p, N, L, &fracfit);
  if (ns > ctx->maxnull || ns + 1 > ctx->maxslots)
    return fail(ctx, 11, "%d null alignments need maxnull >= %d and maxslots >= %d", ns, ns, ns + 1);
  CK(cudaEventRecord(ctx->ev[0], ctx->st));
  if ((s = make_nulls_async(ctx, p->seed, 0, ns, 1))) return s;
  CK(cudaEventRecord(ctx->ev[1], ctx->st));
  if ((s = score_async(ctx, 0, ns + 1, ntypes, covtypes, p->covclass, p->nseqthresh, p->alenthresh, p->allow,
                       p->counter)))
    return s;
  CK(cudaEventRecord(ctx->ev[2], ctx->st));
  std::vector<double> mm((size_t)(ns + 1) * ntypes * 2);
  CK(cudaMemcpyAsync(mm.data(), ctx->d_mm, mm.size() * sizeof(double), cudaMemcpyDeviceToHost, ctx->st));
  CK(cudaStreamSynchronize(ctx->st));
  if ((s = check_status(ctx))) return s;
  const int64_t plane = (int64_t)ctx->ntiles * TPP;
  // hit buffers: hitcap per statistic
  if (hitcap > 0 && ctx->hitcap < hitcap * ntypes) {
    cudaFree(ctx->d_hi); cudaFree(ctx->d_hj); cudaFree(ctx->d_hsc); cudaFree(ctx->d_hE); cudaFree(ctx->d_hp);
    const size_t n = (size_t)hitcap * ntypes;
    CK(dalloc(&ctx->d_hi, n)); CK(dalloc(&ctx->d_hj, n));
    CK(dalloc(&ctx->d_hsc, n)); CK(dalloc(&ctx->d_hE, n)); CK(dalloc(&ctx->d_hp, n));
    ctx->hitcap = hitcap * ntypes;
  }
  // The statistics go through the null histogram, the tail fit, the
  // survival table and the E-values phase by phase, all statistics in each
  // phase, so each phase costs one host round trip instead of one per
  // statistic.
  struct Stats {
    RsStat q[MAXOUT];
    ~Stats() { for (auto& x : q) if (x.h) covh_Destroy(x.h); }
  } S;

  // phase 1: width and bins from the nulls' ranges, the histograms
  int64_t obs_tot = 0;
  for (int q = 0; q < ntypes; q++) {
    RsStat& X = S.q[q];
    if ((s = rs_width(p, N, ns, mm.data(), ntypes, q, results[q], X, ctx->err, sizeof(ctx->err)))) return s;
    if (!X.active) continue;
    X.obs_off = obs_tot;
    obs_tot += X.nbcum;
  }
  if (ctx->nbcap < obs_tot) {
    if (ctx->d_obs) cudaFree(ctx->d_obs);
    ctx->d_obs = nullptr;
    CK(dalloc(&ctx->d_obs, obs_tot));
    ctx->nbcap = (int)obs_tot;
  }
  std::vector<uint64_t>& obs = ctx->h_obs;   // every entry is written by the copy below
  obs.resize(std::max<int64_t>(obs_tot, 1));
  if (obs_tot > 0) {
    CK(cudaMemsetAsync(ctx->d_obs, 0, (size_t)obs_tot * sizeof(unsigned long long), ctx->st));
    for (int q = 0; q < ntypes; q++) {
      const RsStat& X = S.q[q];
      if (!X.active) continue;
      CK(launch_hist(ctx->d_cov + ((int64_t)1 * ntypes + q) * plane, ntypes * plane, ctx->d_tiles, ctx->ntiles, L, ns,
                     p->bmin, X.w, X.nbcum, X.wbase, ctx->d_obs + X.obs_off, ctx->d_status, ctx->st));
      ctx->nlaunch += 1;
    }
    CK(cudaMemcpyAsync(obs.data(), ctx->d_obs, (size_t)obs_tot * sizeof(uint64_t), cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    if ((s = check_status(ctx))) return s;
  }

  // phase 2: the histograms on the host, tail by mass, the tail fits
  // (gamma: likelihood on the device, the statistics' searches side by side
  // on their own streams, forked from and joined back into the main one)
  auto tf0 = std::chrono::steady_clock::now();
  bool any_fit = false;
  CK(cudaEventRecord(ctx->fev[MAXOUT], ctx->st));
  for (int q = 0; q < ntypes; q++) {
    RsStat& X = S.q[q];
    if (!X.active) continue;
    if ((s = rs_histogram(p, fracfit, ns, P, obs.data() + X.obs_off, X, ctx->err, sizeof(ctx->err)))) return s;
    if (!p->doexpfit) {
      const ESL_HISTOGRAM* h = X.h;
      if (!ctx->fitw[q]) ctx->fitw[q] = fitwork_create();
      CK(cudaStreamWaitEvent(ctx->fst[q], ctx->fev[MAXOUT], 0));
      const int fs = gamma_fit_launch(ctx->fitw[q], h->obs, h->cmin, h->imax, h->bmin, h->w, h->phi, ctx->fst[q]);
      if (fs) {
        cudaStreamSynchronize(ctx->fst[q]);
        return fail(ctx, 32, "could not do a Gamma fit (%d)", fs);
      }
      CK(cudaEventRecord(ctx->fev[q], ctx->fst[q]));
      CK(cudaStreamWaitEvent(ctx->st, ctx->fev[q], 0));
      ctx->nlaunch += 1;
      any_fit = true;
    }
  }
  if (any_fit) {
    CK(cudaStreamSynchronize(ctx->st));
    for (int q = 0; q < ntypes; q++) {
      RsStat& X = S.q[q];
      if (!X.active || p->doexpfit) continue;
      const int fs = gamma_fit_collect(ctx->fitw[q], &X.lambda, &X.tau, &X.evals);
      if (fs) return fail(ctx, 32, "could not do a Gamma fit (%d)", fs);
    }
  }

  // phase 3: the survival tables on the device
  int64_t sf_tot = 0, tail_tot = 0;
  for (int q = 0; q < ntypes; q++) {
    RsStat& X = S.q[q];
    if (!X.active) continue;
    X.tail_off = tail_tot;
    tail_tot += X.h->nb;
    if (!std::isinf(X.lambda)) { X.have_sf = true; X.sf_off = sf_tot; sf_tot += 2 * (int64_t)X.h->nb; }
  }
  if ((int64_t)ctx->sfcap < std::max(sf_tot, tail_tot)) {
    if (ctx->d_sf) cudaFree(ctx->d_sf);
    if (ctx->d_tail) cudaFree(ctx->d_tail);
    ctx->d_sf = nullptr; ctx->d_tail = nullptr; ctx->sfcap = 0;
    const int64_t cap = std::max(sf_tot, tail_tot);
    CK(dalloc(&ctx->d_sf, cap));
    CK(dalloc(&ctx->d_tail, cap));
    ctx->sfcap = (int)cap;
  }
  std::vector<double>& sfh = ctx->h_sf;      // every entry is written by the copy below
  sfh.resize(std::max<int64_t>(sf_tot, 1));
  if (sf_tot > 0) {
    // the survival tables side by side, as the fits
    CK(cudaEventRecord(ctx->fev[MAXOUT], ctx->st));
    for (int q = 0; q < ntypes; q++) {
      const RsStat& X = S.q[q];
      if (!X.have_sf) continue;
      CK(cudaStreamWaitEvent(ctx->fst[q], ctx->fev[MAXOUT], 0));
      CK(launch_survfit(X.h->cmin, X.h->nb, X.h->bmin, X.h->w, X.newmass, p->doexpfit, X.mu, X.lambda, X.tau,
                        ctx->d_sf + X.sf_off, ctx->fst[q]));
      CK(cudaEventRecord(ctx->fev[q], ctx->fst[q]));
      CK(cudaStreamWaitEvent(ctx->st, ctx->fev[q], 0));
      ctx->nlaunch += 1;
    }
    CK(cudaMemcpyAsync(sfh.data(), ctx->d_sf, (size_t)sf_tot * sizeof(double), cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
  }
  ctx->fit_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - tf0).count();

  // phase 4: thresholds and E-value tables on the host, the E-values and
  // hit lists on the device
  std::vector<double>& tail = ctx->h_tail;   // every entry of each statistic is written below
  tail.resize(std::max<int64_t>(tail_tot, 1));
  for (int q = 0; q < ntypes; q++) {
    RsStat& X = S.q[q];
    if (!X.active) continue;
    if (getenv("COVGPU_DEBUG"))
      fprintf(stderr, "covgpu: type %d nb %d tail bins %d fit %.2f ms (%d evaluations) mu %g lambda %g tau %g\n",
              covtypes[q], X.h->nb, X.h->imax - X.h->cmin + 1, ctx->fit_ms, X.evals, X.mu, X.lambda, X.tau);
    rs_tables(p, P, Nb, X, sfh.data() + X.sf_off, results[q], tail.data() + X.tail_off);
  }
  int nhit[MAXOUT] = {0, 0, 0, 0};
  if (tail_tot > 0) {
    CK(cudaMemcpyAsync(ctx->d_tail, tail.data(), (size_t)tail_tot * sizeof(double), cudaMemcpyHostToDevice, ctx->st));
    if (!bpmask.empty()) {
      const size_t capw = (size_t)(((int64_t)ctx->capL * (ctx->capL - 1) / 2 + 31) / 32) + 1;
      if (!ctx->d_bpmask) CK(dalloc(&ctx->d_bpmask, capw));
      CK(cudaMemcpyAsync(ctx->d_bpmask, bpmask.data(), (size_t)((P + 31) / 32) * sizeof(uint32_t),
                         cudaMemcpyHostToDevice, ctx->st));
    }
    // --structured: where the first hits' rule ends, per statistic
    long long kstar[MAXOUT] = {-1, -1, -1, -1};
    for (int q = 0; q < ntypes && p->expBP > 0.0; q++) {
      const RsStat& X = S.q[q];
      if (!X.active) continue;
      if (p->thresh > 1000.0) { kstar[q] = (long long)std::ceil(p->expBP) - 1; continue; }   // every pair a hit
      EvalTables T = rs_evaltables(p, P - Nb, X, ctx->d_sf + X.sf_off, ctx->d_tail + X.tail_off);
      if (!bpmask.empty()) { T.bpmask = ctx->d_bpmask; T.Nb = (double)Nb; }
      if ((s = structured_kstar(ctx, ctx->d_cov + (int64_t)q * plane, T, p->expBP, &kstar[q]))) return s;
    }
    CK(cudaMemsetAsync(ctx->d_nhits, 0, MAXOUT * sizeof(int), ctx->st));
    for (int q = 0; q < ntypes; q++) {
      const RsStat& X = S.q[q];
      if (!X.active) continue;
      EvalTables T = rs_evaltables(p, P - Nb, X, ctx->d_sf + X.sf_off, ctx->d_tail + X.tail_off);
      if (!bpmask.empty()) { T.bpmask = ctx->d_bpmask; T.Nb = (double)Nb; }
      if (p->expBP > 0.0) { T.Nx = p->expBP; T.kstar = kstar[q]; }
      const size_t ho = (size_t)q * hitcap;
      CK(launch_evalue(ctx->d_cov + (int64_t)q * plane, ctx->d_tiles, ctx->ntiles, L, T, nullptr, ctx->d_nhits + q,
                       hitcap, ctx->d_hi + ho, ctx->d_hj + ho, ctx->d_hsc + ho, ctx->d_hE + ho, ctx->d_hp + ho,
                       ctx->st));
      ctx->nlaunch += 1;
    }
    CK(cudaMemcpyAsync(nhit, ctx->d_nhits, MAXOUT * sizeof(int), cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
  }
  // the hit lists of all statistics, read back together into one host
  // staging area sized by the hits found (statistic q's at hoff[q])
  size_t hoff[MAXOUT + 1] = {0, 0, 0, 0, 0};
  for (int q = 0; q < ntypes; q++) {
    size_t n = 0;
    if (S.q[q].active) {
      results[q].nhit = nhit[q];
      if (hits) n = (size_t)std::max(0, std::min(nhit[q], hitcap));
    }
    hoff[q + 1] = hoff[q] + n;
  }
  const size_t nall = hoff[ntypes];
  std::vector<int> hi_(nall), hj_(nall);
  std::vector<double> hs_(nall), hE_(nall), hp_(nall);
  for (int q = 0; q < ntypes; q++) {
    const size_t n = hoff[q + 1] - hoff[q], o = hoff[q], ho = (size_t)q * hitcap;
    if (n == 0) continue;
    CK(cudaMemcpyAsync(hi_.data() + o, ctx->d_hi + ho, n * sizeof(int), cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaMemcpyAsync(hj_.data() + o, ctx->d_hj + ho, n * sizeof(int), cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaMemcpyAsync(hs_.data() + o, ctx->d_hsc + ho, n * sizeof(double), cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaMemcpyAsync(hE_.data() + o, ctx->d_hE + ho, n * sizeof(double), cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaMemcpyAsync(hp_.data() + o, ctx->d_hp + ho, n * sizeof(double), cudaMemcpyDeviceToHost, ctx->st));
  }
  if (nall > 0) CK(cudaStreamSynchronize(ctx->st));
  for (int q = 0; q < ntypes; q++) {
    const RsStat& X = S.q[q];
    if (!X.active) continue;
    const size_t n = hoff[q + 1] - hoff[q], o = hoff[q];
    if (n > 0) {
      covgpu_hit* H = hits + (size_t)q * hitcap;
      for (size_t k = 0; k < n; k++) H[k] = covgpu_hit{hi_[o + k], hj_[o + k], hs_[o + k], hE_[o + k], hp_[o + k]};
      // the reference lists hits in row-major pair order (src/covariation.c:827-893)
      std::sort(H, H + n, [](const covgpu_hit& a, const covgpu_hit& b) {
        return (a.i != b.i) ? a.i < b.i : a.j < b.j;
      });
    }
    if (q == 0 && ctx->want_qsum) {
      null_summary(X.h, X.xmax, X.mu, X.lambda, X.tau, ctx->qsum);
      ctx->have_qsum = true;
    }
  }
  CK(cudaEventRecord(ctx->ev[3], ctx->st));
  CK(cudaEventSynchronize(ctx->ev[3]));
  ctx->tms[0] = elapsed(ctx->ev[0], ctx->ev[1]);
  ctx->tms[1] = ctx->counted ? elapsed(ctx->ev[4], ctx->ev[5]) : 0.0;
  ctx->tms[2] = elapsed(ctx->ev[1], ctx->ev[2]);
  ctx->tms[3] = elapsed(ctx->ev[2], ctx->ev[3]);
  ctx->tms[4] = elapsed(ctx->ev[0], ctx->ev[3]);
  return 0;
}

// ------------------------------------------------------------------------
// learned null
// ------------------------------------------------------------------------
extern "C" int covgpu_features(covgpu_ctx* ctx, int slot, double tree_len, float* feat) {
  if (!ctx) return 11;
  CK(cudaSetDevice(ctx->dev));
  if (slot < 0 || slot >= ctx->maxslots || !feat) return fail(ctx, 11, "bad slot or output");
  if (!ctx->have_w) return fail(ctx, 11, "weights not set");
  if (!std::isfinite(tree_len)) return fail(ctx, 11, "tree length is not finite");
  if (!ctx->d_featscr) {
    CK(dalloc(&ctx->d_featscr, feat_scratch_doubles(ctx->capL)));
    CK(dalloc(&ctx->d_feat, kNFeat));
  }
  CK(launch_features(ctx->d_ax + (size_t)slot * ctx->N * ctx->Lp, ctx->N, ctx->L, ctx->Lp, ctx->d_wd, tree_len,
                     ctx->d_featscr, ctx->d_feat, ctx->st));
  ctx->nlaunch += 4;
  CK(cudaMemcpyAsync(feat, ctx->d_feat, kNFeat * sizeof(float), cudaMemcpyDeviceToHost, ctx->st));
  CK(cudaStreamSynchronize(ctx->st));
  return 0;
}

static int learned_features(covgpu_ctx* ctx, const covgpu_params* p, double tree_len, int covtype, int nquick,
                            float* feat, covgpu_result* quick) {
  int s;
  if (nquick < 1) return fail(ctx, 11, "the learned null needs at least one quick null");
  if ((s = covgpu_features(ctx, 0, tree_len, feat))) return s;
  covgpu_params pq = *p;
  pq.nshuffle = nquick;
  ctx->want_qsum = true;
  ctx->have_qsum = false;
  s = covgpu_rscape(ctx, &pq, nullptr, nullptr, 1, &covtype, quick, nullptr, 0);
  ctx->want_qsum = false;
  if (s) return s;
  for (int k = 0; k < 17; k++) feat[47 + k] = ctx->have_qsum ? (float)ctx->qsum[k] : NAN;
  return 0;
}

extern "C" int covgpu_learned_features(covgpu_ctx* ctx, const covgpu_params* p, double tree_len, int covtype,
                                       int nquick, float* feat) {
  if (!ctx) return 11;
  CK(cudaSetDevice(ctx->dev));
  covgpu_result quick;
  return learned_features(ctx, p, tree_len, covtype, nquick, feat, &quick);
}

extern "C" int covgpu_rscape_learned(covgpu_ctx* ctx, const covgpu_params* p, const uint8_t* ax, const double* wgt,
                                     covgpu_mlp* net, double tree_len, int covtype, int nquick,
                                     covgpu_result* result, covgpu_hit* hits, int hitcap, int* used_net) {
  if (!ctx) return 11;
  CK(cudaSetDevice(ctx->dev));
  const int L = ctx->L;
  const int64_t P = (int64_t)L * (L - 1) / 2;
  if (!net) return fail(ctx, 11, "no network");
  if ((p->ncnt > 0 && p->samplesize != 3) || p->expBP > 0.0)
    return fail(ctx, 11, "the learned null computes one-set E-values (no two-set test, no --structured)");
  *used_net = 0;
  int s;
  if (wgt && (s = covgpu_set_weights(ctx, wgt))) return s;
  if (ax && (s = covgpu_set_alignment(ctx, 0, ax))) return s;
  float feat[kNFeat], out[COVGPU_NOUT];
  covgpu_result quick;
  memset(&quick, 0, sizeof(quick));
  if (ctx->N < 2 || L < 2 || (s = learned_features(ctx, p, tree_len, covtype, nquick, feat, &quick)) ||
      quick.status != 0 || !covgpu_mlp_in_range(net, feat))
    return covgpu_rscape(ctx, p, nullptr, nullptr, 1, &covtype, result, hits, hitcap);
  if (covgpu_mlp_forward(net, feat, 1, out)) return fail(ctx, 25, "network: %s", covgpu_mlp_errmsg(net));
  // the outputs correct the quick nulls' tail (features 60-62: mu, log mean
  // excess, log shape): mu + out0 * excess, log excess + out1, log shape + out2
  const double mq = std::exp((double)feat[61]);
  const double mu = (double)feat[60] + (double)out[0] * mq;
  const double tau = std::exp((double)feat[62] + (double)out[2]);
  const double lambda = tau / std::exp((double)feat[61] + (double)out[1]);
  if (!std::isfinite(mu) || !(tau > 0.0) || !std::isfinite(tau) || !(lambda > 0.0) || !std::isfinite(lambda))
    return covgpu_rscape(ctx, p, nullptr, nullptr, 1, &covtype, result, hits, hitcap);
  *used_net = 1;
  // the quick run scored the alignment (slot 0, type 0) and fixed the width
  // from its first null, as the full run would
  covgpu_result& R = *result;
  R = quick;
  R.nhit = 0;
  R.mu = mu; R.lambda = lambda; R.tau = tau; R.pmass = p->pmass; R.newmass = p->pmass;
  R.Nt = (uint64_t)P;
  const double w = R.w;
  CK(cudaEventRecord(ctx->ev[2], ctx->st));
  double bmax = R.maxCOV + 5 * w;
  while (fabs(bmax - p->bmin) < p->tol) bmax += w;
  const int nb = bins_for(p->bmin, bmax, w);
  if (ctx->sfcap < 2 * nb) {
    if (ctx->d_sf) cudaFree(ctx->d_sf);
    if (ctx->d_tail) cudaFree(ctx->d_tail);
    CK(dalloc(&ctx->d_sf, 2 * nb));
    CK(dalloc(&ctx->d_tail, 2 * nb));
    ctx->sfcap = 2 * nb;
  }
  // survival at every bin's upper bound, mass pmass above mu
  CK(launch_survfit(0, nb, p->bmin, w, p->pmass, 0, mu, lambda, tau, ctx->d_sf, ctx->st));
  if (hitcap > 0 && ctx->hitcap < hitcap) {
    cudaFree(ctx->d_hi); cudaFree(ctx->d_hj); cudaFree(ctx->d_hsc); cudaFree(ctx->d_hE); cudaFree(ctx->d_hp);
    CK(dalloc(&ctx->d_hi, hitcap)); CK(dalloc(&ctx->d_hj, hitcap));
    CK(dalloc(&ctx->d_hsc, hitcap)); CK(dalloc(&ctx->d_hE, hitcap)); CK(dalloc(&ctx->d_hp, hitcap));
    ctx->hitcap = hitcap;
  }
  EvalTables T;
  T.sf = ctx->d_sf;
  T.ptail = ctx->d_tail;   // not read: every score takes the fitted branch
  T.bmin = p->bmin; T.w = w; T.phi = -INFINITY; T.xmax = INFINITY; T.Nc = 1.0; T.Nt = (double)P;
  T.pNc = 1.0;
  T.thresh = p->thresh; T.nb = nb; T.imin = 0; T.imax = nb - 1;
  CK(cudaMemsetAsync(ctx->d_nhits, 0, sizeof(int), ctx->st));
  CK(launch_evalue(ctx->d_cov, ctx->d_tiles, ctx->ntiles, L, T, nullptr, ctx->d_nhits, ctx->hitcap, ctx->d_hi,
                   ctx->d_hj, ctx->d_hsc, ctx->d_hE, ctx->d_hp, ctx->st));
  ctx->nlaunch += 2;
  std::vector<double> sf(2 * (size_t)nb);
  int nh = 0;
  CK(cudaMemcpyAsync(sf.data(), ctx->d_sf, sf.size() * sizeof(double), cudaMemcpyDeviceToHost, ctx->st));
  CK(cudaMemcpyAsync(&nh, ctx->d_nhits, sizeof(int), cudaMemcpyDeviceToHost, ctx->st));
  CK(cudaStreamSynchronize(ctx->st));
  // score at the threshold: the lower bound of the first bin whose E-value
  // falls below it
  R.sc_thresh = INFINITY;
  for (int b = 0; b < 2 * nb; b++)
    if (sf[b] * (double)P < p->thresh) { R.sc_thresh = p->bmin + b * w; break; }
  R.nhit = nh;
  const int nget = std::min(nh, hitcap);
  if (nget > 0 && hits) {
    std::vector<int> hi(nget), hj(nget);
    std::vector<double> hs(nget), hE(nget), hp(nget);
    CK(cudaMemcpyAsync(hi.data(), ctx->d_hi, nget * sizeof(int), cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaMemcpyAsync(hj.data(), ctx->d_hj, nget * sizeof(int), cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaMemcpyAsync(hs.data(), ctx->d_hsc, nget * sizeof(double), cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaMemcpyAsync(hE.data(), ctx->d_hE, nget * sizeof(double), cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaMemcpyAsync(hp.data(), ctx->d_hp, nget * sizeof(double), cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    for (int k = 0; k < nget; k++) hits[k] = covgpu_hit{hi[k], hj[k], hs[k], hE[k], hp[k]};
    std::sort(hits, hits + nget, [](const covgpu_hit& a, const covgpu_hit& b) {
      return (a.i != b.i) ? a.i < b.i : a.j < b.j;
    });
  }
  CK(cudaEventRecord(ctx->ev[3], ctx->st));
  CK(cudaEventSynchronize(ctx->ev[3]));
  ctx->tms[3] += elapsed(ctx->ev[2], ctx->ev[3]);
  ctx->tms[4] += elapsed(ctx->ev[2], ctx->ev[3]);
  return 0;
}

// ------------------------------------------------------------------------
// helix aggregation (agg_CalculatePvalues, src/aggregate.c:41-128)
// ------------------------------------------------------------------------
extern "C" int covgpu_aggregate(covgpu_ctx* ctx, int method, int nh, const int* helix_off, const double* pval,
                                const double* aux, double* pagg, double* Eagg) {
  if (!ctx) return 11;
  CK(cudaSetDevice(ctx->dev));
  if (method < COVGPU_AGG_FISHER || method > COVGPU_AGG_SIDAK) return fail(ctx, 11, "unknown aggregation method");
  if (nh < 0 || (nh > 0 && (!helix_off || !pval || !pagg))) return fail(ctx, 11, "bad helix arguments");
  if (nh == 0) return 0;
  if (helix_off[0] != 0) return fail(ctx, 11, "helix offsets must start at 0");
  for (int h = 0; h < nh; h++)
    if (helix_off[h + 1] < helix_off[h]) return fail(ctx, 11, "helix offsets decrease at %d", h);
  const int nbp = helix_off[nh];
  const bool need_aux = (method == COVGPU_AGG_LANCASTER || method == COVGPU_AGG_WFISHER);
  if (need_aux && !aux) return fail(ctx, 11, "this method needs per-pair weights");
  for (int k = 0; k < nbp; k++) {
    if (!(pval[k] >= 0.0 && pval[k] <= 1.0)) return fail(ctx, 11, "p-value %d outside [0, 1]", k);
    if (need_aux && !(aux[k] >= 0.0 && std::isfinite(aux[k]))) return fail(ctx, 11, "weight %d is negative", k);
  }
  const size_t nd = (size_t)nbp * 4 + nh + 1;   // pval, aux, term[2], pagg
  double* d = nullptr;
  int* d_off = nullptr;
  CK(dalloc(&d, nd));
  cudaError_t e = dalloc(&d_off, (size_t)nh + 1);
  double *d_pval = d, *d_aux = d + nbp, *d_term = d + 2 * (size_t)nbp, *d_pagg = d + 4 * (size_t)nbp;
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_off, helix_off, ((size_t)nh + 1) * sizeof(int), cudaMemcpyHostToDevice, ctx->st);
  if (e == cudaSuccess && nbp)
    e = cudaMemcpyAsync(d_pval, pval, (size_t)nbp * sizeof(double), cudaMemcpyHostToDevice, ctx->st);
  if (e == cudaSuccess && need_aux && nbp)
    e = cudaMemcpyAsync(d_aux, aux, (size_t)nbp * sizeof(double), cudaMemcpyHostToDevice, ctx->st);
  if (e == cudaSuccess) e = launch_aggregate(method, nh, d_off, d_pval, d_aux, d_term, d_pagg, ctx->st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(pagg, d_pagg, (size_t)nh * sizeof(double), cudaMemcpyDeviceToHost, ctx->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->st);
  cudaFree(d);
  if (d_off) cudaFree(d_off);
  if (e != cudaSuccess) return fail(ctx, 90, "CUDA error %s", cudaGetErrorString(e));
  // E-value: times the number of helices tested (rm->Eval, src/aggregate.c:114)
  if (Eagg)
    for (int h = 0; h < nh; h++) Eagg[h] = (pagg[h] < 0.0) ? -1.0 : (double)nh * pagg[h];
  return 0;
}

// ------------------------------------------------------------------------
// schedule autotuner for the tensor count kernel
// ------------------------------------------------------------------------
extern "C" int covgpu_autotune(covgpu_ctx* ctx, int first_slot, int nslots, int ncand, const int* cand, float* ms,
                               int* best) {
  if (!ctx) return 11;
  CK(cudaSetDevice(ctx->dev));
  ctx->cnt_valid = false;
  static const int defaults[] = {4, 6, 8, 10, 12, 16, 24, 32004, 48004, 48008, 96004};
  if (!cand || ncand <= 0) { cand = defaults; ncand = (int)(sizeof(defaults) / sizeof(defaults[0])); }
  if (first_slot < 0 || nslots < 1 || first_slot + nslots > ctx->maxslots) return fail(ctx, 11, "slots out of range");
  if (!ctx->have_w) return fail(ctx, 11, "weights not set");
  if (!ctx->umma) {
    ctx->umma = umma_plan_create(ctx->N, ctx->L, ctx->Lp, ctx->nT, ctx->d_tiles, ctx->ntiles, ctx->maxslots,
                                 ctx->capN, ctx->capLp, ctx->capntiles);
    if (!ctx->umma) return fail(ctx, 12, "tensor counting not available for this shape");
    umma_set_weights(ctx->umma, ctx->h_w.data(), ctx->N, ctx->st);
  }
  const int64_t sstride = (int64_t)ctx->N * ctx->Lp;
  std::vector<float> t(ncand, 0.f);
  int b = 0;
  const int s = umma_autotune(ctx->umma, ctx->d_ax + first_slot * sstride, sstride, nslots, ctx->d_cnt, ctx->st, cand,
                              ncand, 3, t.data(), &b);
  if (s) return fail(ctx, s, "autotune failed (%d)", s);
  if (ms) for (int k = 0; k < ncand; k++) ms[k] = t[k];
  if (best) *best = b;
  ctx->counted = false;
  ctx->cnt_valid = false;
  return check_status(ctx);
}

extern "C" int covgpu_last_timing(const covgpu_ctx* ctx, double* ms5, int* nlaunch) {
  if (!ctx) return 11;
  for (int k = 0; k < 5; k++) ms5[k] = ctx->tms[k];
  if (nlaunch) *nlaunch = ctx->nlaunch;
  return 0;
}

// overwrite a buffer larger than L2 (129 MB) so that the next call starts
// from a cold cache
extern "C" int covgpu_flush_l2(covgpu_ctx* ctx) {
  if (!ctx) return 11;
  CK(cudaSetDevice(ctx->dev));
  const size_t n = (size_t)256 << 20;
  if (!ctx->d_flush) CK(dalloc(&ctx->d_flush, n));
  CK(cudaMemsetAsync(ctx->d_flush, ctx->nlaunch & 0xff, n, ctx->st));
  CK(cudaStreamSynchronize(ctx->st));
  return 0;
}

extern "C" int covgpu_validate_probs(covgpu_ctx* ctx, double tol) {
  if (!ctx) return 11;
  CK(cudaSetDevice(ctx->dev));
  if (!ctx->counted || ctx->last_first != 0) return fail(ctx, 11, "no weighted counts of slot 0 on the device");
  CK(cudaMemsetAsync(ctx->d_nhits, 0, sizeof(int), ctx->st));
  CK(launch_validate_pp(ctx->d_cnt, ctx->d_tiles, ctx->ntiles, ctx->L, tol, ctx->d_nhits, ctx->st));
  int bad = 0;
  CK(cudaMemcpyAsync(&bad, ctx->d_nhits, sizeof(int), cudaMemcpyDeviceToHost, ctx->st));
  CK(cudaStreamSynchronize(ctx->st));
  if (bad) return fail(ctx, 20, "pair probabilities failed validation");
  return 0;
}

extern "C" int covgpu_pair_classes(covgpu_ctx* ctx, int slot, double* wcf, double* wobble, double* noncan) {
  if (!ctx) return 11;
  CK(cudaSetDevice(ctx->dev));
  if (!ctx->cnt_valid || slot < ctx->cnt_first || slot >= ctx->cnt_first + ctx->cnt_nslots)
    return fail(ctx, 11, "no weighted counts of slot %d on the device", slot);
  const int L = ctx->L;
  const int64_t P = (int64_t)L * (L - 1) / 2;
  if (P < 1) return 0;
  // three outputs of P values each, for the largest L of the context
  if (!ctx->d_pcls) CK(dalloc(&ctx->d_pcls, 3 * ((size_t)ctx->capL * (ctx->capL - 1) / 2)));
  double* d = ctx->d_pcls;
  const float* cnt = ctx->d_cnt + (size_t)(slot - ctx->cnt_first) * ctx->ntiles * 32 * TPP;
  CK(launch_pair_classes(cnt, ctx->d_tiles, ctx->ntiles, L, d, d + P, d + 2 * P, ctx->st));
  if (wcf) CK(cudaMemcpyAsync(wcf, d, P * sizeof(double), cudaMemcpyDeviceToHost, ctx->st));
  if (wobble) CK(cudaMemcpyAsync(wobble, d + P, P * sizeof(double), cudaMemcpyDeviceToHost, ctx->st));
  if (noncan) CK(cudaMemcpyAsync(noncan, d + 2 * P, P * sizeof(double), cudaMemcpyDeviceToHost, ctx->st));
  CK(cudaStreamSynchronize(ctx->st));
  return 0;
}

// ------------------------------------------------------------------------
// single-matrix operations for the reference-named entry points: the score
// matrix comes from the host (full L x L, both triangles) or, when NULL, is
// the device's latest score of slot 0 / type 0.
// ------------------------------------------------------------------------
static int upload_full(covgpu_ctx* ctx, const double* COV) {
  if (!COV) {
    if (ctx->last_nout < 1 || ctx->last_first != 0) return fail(ctx, 11, "no device score matrix for slot 0");
    return 0;
  }
  if (!ctx->d_full) CK(dalloc(&ctx->d_full, (size_t)ctx->capL * ctx->capL));
  CK(cudaMemcpyAsync(ctx->d_full, COV, (size_t)ctx->L * ctx->L * sizeof(double), cudaMemcpyHostToDevice, ctx->st));
  CK(launch_tile(ctx->d_full, ctx->d_tiles, ctx->ntiles, ctx->L, ctx->d_cov, ctx->st));
  ctx->last_nout = 1; ctx->last_first = 0; ctx->last_nslots = 1;
  return 0;
}

extern "C" int covgpu_correct(covgpu_ctx* ctx, const double* COV, int actype, double* out, double* minmax) {
  if (!ctx) return 11;
  CK(cudaSetDevice(ctx->dev));
  if (actype != 0 && actype != 1) return fail(ctx, 11, "wrong correction type");
  int s = upload_full(ctx, COV);
  if (s) return s;
  const int nout = ctx->last_nout;
  // the corrected plane is slot 0 / type 0 of the tile layout
  CK(launch_tile_rowsums(ctx->d_cov, ctx->d_tiles, ctx->ntiles, ctx->nT, ctx->L, ctx->d_part1, ctx->st));
  CorrTypes ct;
  ct.nout = 1; ct.act[0] = actype; ct.act[1] = ct.act[2] = ct.act[3] = -1;
  CK(launch_apc(ctx->d_cov, ctx->d_part1, ctx->d_colx, ctx->d_colxf, ctx->d_avg, ctx->d_apcf, ct, ctx->d_tiles,
                ctx->ntiles, ctx->nT, ctx->L, ctx->Lp, 1, ctx->d_tmin, ctx->d_tmax, ctx->d_mm, ctx->d_status,
                ctx->st));
  ctx->last_nout = 1;
  (void)nout;
  if (minmax) CK(cudaMemcpyAsync(minmax, ctx->d_mm, 2 * sizeof(double), cudaMemcpyDeviceToHost, ctx->st));
  CK(cudaStreamSynchronize(ctx->st));
  if ((s = check_status(ctx))) return s;
  if (out) return covgpu_get_cov(ctx, 0, 0, out);
  return 0;
}

extern "C" int covgpu_hist_full(covgpu_ctx* ctx, const double* COV, double bmin, double w, int nb, uint64_t* obs) {
  if (!ctx) return 11;
  CK(cudaSetDevice(ctx->dev));
  int s = upload_full(ctx, COV);
  if (s) return s;
  if (nb < 1 || !(w > 0.0)) return fail(ctx, 11, "bad histogram shape");
  if (ctx->nbcap < nb) {
    if (ctx->d_obs) cudaFree(ctx->d_obs);
    CK(dalloc(&ctx->d_obs, nb));
    ctx->nbcap = nb;
  }
  CK(cudaMemsetAsync(ctx->d_obs, 0, (size_t)nb * sizeof(unsigned long long), ctx->st));
  CK(launch_hist(ctx->d_cov, 0, ctx->d_tiles, ctx->ntiles, ctx->L, 1, bmin, w, nb, 0, ctx->d_obs, ctx->d_status,
                 ctx->st));
  CK(cudaMemcpyAsync(obs, ctx->d_obs, (size_t)nb * sizeof(uint64_t), cudaMemcpyDeviceToHost, ctx->st));
  CK(cudaStreamSynchronize(ctx->st));
  return check_status(ctx);
}

// the hit buffers hold at least cap hits
static int hits_reserve(covgpu_ctx* ctx, int cap) {
  if (cap > 0 && ctx->hitcap < cap) {
    cudaFree(ctx->d_hi); cudaFree(ctx->d_hj); cudaFree(ctx->d_hsc); cudaFree(ctx->d_hE); cudaFree(ctx->d_hp);
    ctx->d_hi = ctx->d_hj = nullptr;
    ctx->d_hsc = ctx->d_hE = ctx->d_hp = nullptr;
    ctx->hitcap = 0;
    CK(dalloc(&ctx->d_hi, cap)); CK(dalloc(&ctx->d_hj, cap));
    CK(dalloc(&ctx->d_hsc, cap)); CK(dalloc(&ctx->d_hE, cap)); CK(dalloc(&ctx->d_hp, cap));
    ctx->hitcap = cap;
  }
  return 0;
}

// one E-value pass over the uploaded scores: the number of pairs with
// E < thresh into *nh (the first hitcap of them in the hit buffers), the
// tile-packed E-values into evt when given
static int evalue_pass(covgpu_ctx* ctx, const EvalTables& T, double* evt, int* nh) {
  CK(cudaMemsetAsync(ctx->d_nhits, 0, sizeof(int), ctx->st));
  CK(launch_evalue(ctx->d_cov, ctx->d_tiles, ctx->ntiles, ctx->L, T, evt, ctx->d_nhits, ctx->hitcap, ctx->d_hi,
                   ctx->d_hj, ctx->d_hsc, ctx->d_hE, ctx->d_hp, ctx->st));
  CK(cudaMemcpyAsync(nh, ctx->d_nhits, sizeof(int), cudaMemcpyDeviceToHost, ctx->st));
  CK(cudaStreamSynchronize(ctx->st));
  return 0;
}

// the first n hits of the hit buffers, in scan order (i, then j)
static int hits_fetch(covgpu_ctx* ctx, int n, std::vector<covgpu_hit>& out) {
  out.resize(n);
  if (n == 0) return 0;
  std::vector<int> hi(n), hj(n);
  std::vector<double> hs(n), hE(n), hp(n);
  CK(cudaMemcpy(hi.data(), ctx->d_hi, n * sizeof(int), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(hj.data(), ctx->d_hj, n * sizeof(int), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(hs.data(), ctx->d_hsc, n * sizeof(double), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(hE.data(), ctx->d_hE, n * sizeof(double), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(hp.data(), ctx->d_hp, n * sizeof(double), cudaMemcpyDeviceToHost));
  for (int k = 0; k < n; k++) out[k] = covgpu_hit{hi[k], hj[k], hs[k], hE[k], hp[k]};
  std::sort(out.begin(), out.end(), [](const covgpu_hit& a, const covgpu_hit& b) {
    return (a.i != b.i) ? a.i < b.i : a.j < b.j;
  });
  return 0;
}

extern "C" int covgpu_evalue_sets(covgpu_ctx* ctx, const double* COV, const void* hv, const double* survfit,
                                  double Nt, double Nb, double expBP, const uint32_t* bpmask, double thresh,
                                  double* Eval, covgpu_hit* hits, int hitcap, int* nhit) {
  if (!ctx) return 11;
  CK(cudaSetDevice(ctx->dev));
  const ESL_HISTOGRAM* h = (const ESL_HISTOGRAM*)hv;
  int s = upload_full(ctx, COV);
  if (s) return s;
  const int L = ctx->L;
  const int64_t P = (int64_t)L * (L - 1) / 2;
  std::vector<double> tail(h->nb, 0.0);
  double c = 0.0;
  for (int b = h->nb - 1; b >= 0; b--) { if (b <= h->imax) c += (double)h->obs[b]; tail[b] = c; }
  for (int b = 0; b < h->nb; b++) tail[b] /= (double)h->Nc;   // the tail branch's p-values
  if (ctx->sfcap < 2 * h->nb) {
    if (ctx->d_sf) cudaFree(ctx->d_sf);
    if (ctx->d_tail) cudaFree(ctx->d_tail);
    CK(dalloc(&ctx->d_sf, 2 * h->nb));
    CK(dalloc(&ctx->d_tail, 2 * h->nb));
    ctx->sfcap = 2 * h->nb;
  }
  CK(cudaMemcpyAsync(ctx->d_tail, tail.data(), h->nb * sizeof(double), cudaMemcpyHostToDevice, ctx->st));
  if (survfit) CK(cudaMemcpyAsync(ctx->d_sf, survfit, 2 * h->nb * sizeof(double), cudaMemcpyHostToDevice, ctx->st));
  if ((s = hits_reserve(ctx, hitcap))) return s;
  EvalTables T;
  T.sf = survfit ? ctx->d_sf : nullptr;
  T.ptail = ctx->d_tail;
  T.bmin = h->bmin; T.w = h->w; T.phi = h->phi; T.xmax = h->xmax; T.Nc = (double)h->Nc; T.Nt = Nt;
  T.pNc = 1.0 / T.Nc;
  T.thresh = thresh; T.nb = h->nb; T.imin = h->imin; T.imax = h->imax;
  if (bpmask) {
    const size_t nw = (size_t)((P + 31) / 32), capw = (size_t)(((int64_t)ctx->capL * (ctx->capL - 1) / 2 + 31) / 32);
    if (!ctx->d_bpmask) CK(dalloc(&ctx->d_bpmask, std::max<size_t>(capw, 1)));
    CK(cudaMemcpyAsync(ctx->d_bpmask, bpmask, nw * sizeof(uint32_t), cudaMemcpyHostToDevice, ctx->st));
    T.bpmask = ctx->d_bpmask;
    T.Nb = Nb;
  }
  // --structured (src/covariation.c:850-854): a pair outside the structure
  // takes expBP tests while fewer than expBP hits precede it in scan order.
  // kstar is the scan index of the hit that brings the count to expBP: a
  // first pass lists every pair that is a hit under the smaller of expBP and
  // Nt (a superset of the hits), the host replays the rule over them in scan
  // order, and the second pass applies it to every pair.
  if (expBP > 0.0) {
    T.Nx = expBP;
    if (thresh > 1000.0) {
      T.kstar = (long long)std::ceil(expBP) - 1;   // every pair is a hit: h = n
    } else {
      EvalTables T1 = T;
      T1.Nx = std::min(expBP, Nt);
      T1.kstar = LLONG_MAX;
      int nc = 0;
      if ((s = evalue_pass(ctx, T1, nullptr, &nc))) return s;
      if (nc > ctx->hitcap) {
        if ((s = hits_reserve(ctx, nc))) return s;
        if ((s = evalue_pass(ctx, T1, nullptr, &nc))) return s;
      }
      std::vector<covgpu_hit> cand;
      if ((s = hits_fetch(ctx, nc, cand))) return s;
      long long kstar = LLONG_MAX;
      int64_t nh = 0;
      for (const covgpu_hit& x : cand) {
        const long long n = (long long)x.i * (2LL * L - x.i - 1) / 2 + (x.j - x.i - 1);
        const bool isbp = bpmask && ((bpmask[n >> 5] >> (n & 31)) & 1u);
        const double E = isbp ? x.pval * Nb : ((double)nh < expBP ? x.pval * expBP : x.pval * Nt);
        if (E < thresh && ++nh >= expBP) { kstar = n; break; }
      }
      T.kstar = kstar;
    }
  }
  double* evt = nullptr;
  if (Eval) {
    if (!ctx->d_evt) CK(dalloc(&ctx->d_evt, (size_t)ctx->capntiles * TPP));
    evt = ctx->d_evt;
  }
  int nh = 0;
  if ((s = evalue_pass(ctx, T, evt, &nh))) return s;
  if (Eval) {
    if (!ctx->d_full) CK(dalloc(&ctx->d_full, (size_t)ctx->capL * ctx->capL));
    CK(launch_untile(evt, ctx->d_tiles, ctx->ntiles, L, INFINITY, ctx->d_full, ctx->st));
    CK(cudaMemcpyAsync(Eval, ctx->d_full, (size_t)L * L * sizeof(double), cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
  }
  *nhit = nh;
  const int nget = std::min(nh, hitcap);
  if (nget > 0 && hits) {
    std::vector<covgpu_hit> got;
    if ((s = hits_fetch(ctx, std::min(nh, ctx->hitcap), got))) return s;
    std::copy(got.begin(), got.begin() + nget, hits);
  }
  return 0;
}

// page-locks a host array for the copies to and from the device (the
// drop-in's pp, nseff, ngap, COV and Eval); 0, or 90 when the driver refuses
extern "C" int covgpu_host_pin(void* p, size_t bytes) {
  if (!p || bytes == 0) return 0;
  return cudaHostRegister(p, bytes, cudaHostRegisterDefault) == cudaSuccess ? 0 : (cudaGetLastError(), 90);
}

extern "C" void covgpu_host_unpin(void* p) {
  if (p) cudaHostUnregister(p);
}

extern "C" int covgpu_evalue_full(covgpu_ctx* ctx, const double* COV, const void* hv, const double* survfit,
                                  double Nt, double thresh, double* Eval, covgpu_hit* hits, int hitcap, int* nhit) {
  if (!ctx) return 11;
  return covgpu_evalue_sets(ctx, COV, hv, survfit, Nt, 0.0, -1.0, nullptr, thresh, Eval, hits, hitcap, nhit);
}
