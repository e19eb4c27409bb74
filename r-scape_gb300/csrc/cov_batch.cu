// cov_batch.cu -- the E-valued path over a batch of alignment families
// (covgpu_rscape_families, include/covgpu.h): per family what
// covgpu_rscape does for one alignment (R-scape's rscape_for_msa covariation
// part, src/R-scape.c:1080-1276 per input alignment, with the null loop of
// null_rscape, :1614-1724), for many families of different N, L and null
// counts at once.
//
// Families are processed in chunks that fit the batch's device budget (the
// families sorted by padded N, so a chunk's tensor operands share a row
// pitch close to each family's own).  A chunk's buffers sit in one arena,
// buffer kind by buffer kind (every family's codes, then every family's
// weights, ...), in the single-family layouts, and every device pass is one
// grouped launch over the chunk's families (cov_batch.h): weights (GSC with
// one CTA per family for the merges, or position-based), the nulls (one
// launch per tree depth over every family), the tensor count (one
// persistent launch over every (family, alignment, tile) task), marginals,
// statistics, APC/ASC, histograms, the tail fits (one block per fit),
// survival tables and E-values.  The host steps between the passes
// (cov_rscape_host.h) run for every family and statistic, with one host
// round trip per phase for the whole chunk.  The device passes from the
// nulls to the corrected scores are captured once per chunk layout into a
// CUDA graph and replayed while the layout repeats.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <vector>

#include "cov_batch.h"
#include "cov_dev.cuh"
#include "cov_df.cuh"
#include "cov_fit.h"
#include "cov_kernels.h"
#include "cov_rscape_host.h"
#include "cov_umma.h"
#include "covgpu.h"
#include "rscape_cov.h"

using namespace covgpu;

namespace {

constexpr size_t kAlign = 256;
size_t align_up(size_t x) { return (x + kAlign - 1) & ~(kAlign - 1); }

// a family as the host plans it
struct FamHost {
  int idx = 0;                 // position in the caller's arrays
  int N = 0, L = 0, Lp = 0, nT = 0, ntiles = 0, ns = 0, nslots = 0, Npad = 0, Lw = 0;
  double fracfit = 1.0;
  bool gsc = false, pb = false;
  bool tens = false;           // weighted counts on the tensor cores (else on the SIMT kernel)
  std::vector<int> order;      // internal nodes by depth (lnodes)
  std::vector<int> loff;       // depth offsets into order
  int depth() const { return (int)loff.size() - 1; }
};

// a bump layout over one arena: the same sequence of take() calls sizes the
// arena (base == nullptr) and places the buffers
struct Bump {
  uint8_t* base = nullptr;
  size_t off = 0;
  template <class T>
  T* take(size_t n) {
    const size_t o = off;
    off += align_up(std::max<size_t>(n, 1) * sizeof(T));
    return base ? reinterpret_cast<T*>(base + o) : nullptr;
  }
};

// the chunk's device buffers, every kind over all of its families
struct Layout {
  std::vector<FamDev> F;
  uint8_t* ax = nullptr; size_t ax_bytes = 0;
  double* w = nullptr;                       // weights region start (w, limbf, limbs)
  size_t wreg_bytes = 0;
  std::vector<size_t> w_off, lf_off, lb_off; // byte offsets inside the weights region
  int* tree = nullptr; size_t tree_n = 0;    // left, right, lnodes of every family
  uint8_t* tiles = nullptr; size_t tiles_bytes = 0;
  uint16_t* ops = nullptr; int pitch = 0; int64_t op_rows = 0;
  float* cnt = nullptr; int64_t cnt_floats = 0;
  double* pm = nullptr; size_t pm_bytes = 0; // pm, pmdf, lpi regions (RAF only: zeroed)
  double* mm = nullptr; size_t mm_n = 0;
  int* status = nullptr;
  size_t total = 0;
};

// the state of one chunk between its device passes and its host phases
struct Pending {
  std::vector<FamHost> fams;
  Layout Lo;
  size_t tab_used = 0, oF = 0;
};

// one of the batch's two pipeline slots: while the host phases of one chunk
// run on one slot, the device passes of the next run on the other
struct Slot {
  cudaStream_t st = nullptr;
  cudaStream_t st2 = nullptr;  // the weights, alongside the nulls
  cudaEvent_t fork = nullptr, join = nullptr;
  cudaEvent_t ev[3] = {};
  uint8_t* arena = nullptr;
  size_t arena_cap = 0;
  uint8_t* tab = nullptr;      // descriptor tables
  size_t tab_cap = 0;
  int* d_uerr = nullptr;       // the tensor count kernel's error word
  // the captured device passes of the slot's recent chunk layouts, keyed by
  // the descriptor tables and launch parameters (least recently used first out)
  struct Graph { std::vector<uint8_t> key; cudaGraphExec_t exec = nullptr; int launches = 0; uint64_t used = 0; };
  std::vector<Graph> graphs;
  uint64_t tick = 0;
  Pending pc;
};

}  // namespace

struct covgpu_batch {
  int dev = 0;
  char err[512] = {0};
  size_t budget = 0;           // device bytes of one chunk (half of the batch's budget)
  uint8_t* stat = nullptr;     // per (family, statistic) buffers of the chunk in its host phases
  size_t stat_cap = 0;
  float4* d_logtab = nullptr;
  FitBatch* fits = nullptr;
  double ms[3] = {0, 0, 0};
  int nlaunch = 0, nchunks = 0, graph_replays = 0;
  int simt_below = 64;         // families of fewer sequences count on the SIMT kernel (tensor counter)
  int sb = 10;                 // raster super-block of the tensor count's tile order
  Slot slot[2];
};

static int bfail(covgpu_batch* b, int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(b->err, sizeof(b->err), fmt, ap);
  va_end(ap);
  return code;
}

#define BK(call)                                                                         \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess) return bfail(b, 90, "%s: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

static int grow(covgpu_batch* b, uint8_t** p, size_t* cap, size_t need) {
  if (*cap >= need) return 0;
  if (*p) cudaFree(*p);
  *p = nullptr;
  *cap = 0;
  const size_t n = std::max(need, (size_t)1 << 20);
  BK(cudaMalloc((void**)p, n));
  *cap = n;
  return 0;
}

extern "C" int covgpu_batch_create(covgpu_batch** ret, int device, double mem_gb) {
  *ret = nullptr;
  covgpu_batch* b = new covgpu_batch();
  b->dev = device;
  *ret = b;
  BK(cudaSetDevice(device));
  for (Slot& S : b->slot) {
    BK(cudaStreamCreateWithFlags(&S.st, cudaStreamNonBlocking));
    BK(cudaStreamCreateWithFlags(&S.st2, cudaStreamNonBlocking));
    BK(cudaEventCreateWithFlags(&S.fork, cudaEventDisableTiming));
    BK(cudaEventCreateWithFlags(&S.join, cudaEventDisableTiming));
    for (auto& e : S.ev) BK(cudaEventCreate(&e));
    BK(cudaMalloc(&S.d_uerr, sizeof(int)));
    BK(cudaMemset(S.d_uerr, 0, sizeof(int)));
  }
  size_t fr = 0, tot = 0;
  BK(cudaMemGetInfo(&fr, &tot));
  const double want = mem_gb > 0.0 ? mem_gb * 1e9 : 0.25 * (double)fr;
  b->budget = (size_t)std::max(1.6e7, std::min(want, 0.8 * (double)fr)) / 2;
  BK(cudaMalloc(&b->d_logtab, LOGTAB_TOT * sizeof(float4)));
  {
    float4 tab[LOGTAB_TOT];
    logtab_host(tab);
    BK(cudaMemcpy(b->d_logtab, tab, sizeof(tab), cudaMemcpyHostToDevice));
  }
  b->fits = fitbatch_create();
  return 0;
}

extern "C" void covgpu_batch_destroy(covgpu_batch* b) {
  if (!b) return;
  cudaSetDevice(b->dev);
  for (Slot& S : b->slot) {
    if (S.st) cudaStreamSynchronize(S.st);
    if (S.st2) cudaStreamSynchronize(S.st2);
  }
  for (Slot& S : b->slot) {
    for (auto& g : S.graphs) if (g.exec) cudaGraphExecDestroy(g.exec);
    void* q[] = {S.arena, S.tab, S.d_uerr};
    for (void* x : q) if (x) cudaFree(x);
    for (auto& e : S.ev) if (e) cudaEventDestroy(e);
    if (S.fork) cudaEventDestroy(S.fork);
    if (S.join) cudaEventDestroy(S.join);
    if (S.st2) cudaStreamDestroy(S.st2);
    if (S.st) cudaStreamDestroy(S.st);
  }
  void* p[] = {b->stat, b->d_logtab};
  for (void* x : p) if (x) cudaFree(x);
  if (b->fits) fitbatch_destroy(b->fits);
  delete b;
}

extern "C" const char* covgpu_batch_errmsg(const covgpu_batch* b) { return b ? b->err : "no batch"; }

extern "C" int covgpu_batch_timing(const covgpu_batch* b, double* ms3, int* nlaunch, int* nchunks) {
  if (!b) return 11;
  if (ms3) for (int k = 0; k < 3; k++) ms3[k] = b->ms[k];
  if (nlaunch) *nlaunch = b->nlaunch;
  if (nchunks) *nchunks = b->nchunks;
  return 0;
}

namespace {

// statistic index of a covariation type's base (cov_engine.cu)
int stat_of(int base) {
  switch (base) {
    case 0: return 0; case 3: return 1; case 6: return 2; case 9: return 3; case 12: return 4;
    case 15: return 5; case 18: return 6; case 21: return 6; case 24: return 8;
  }
  return -1;
}

struct Types {
  int ntypes = 0;
  bool need_w = false, need_u = false;
  unsigned mask = 0;
  CorrTypes ct;
  int outstat[MAXOUT];
  std::vector<int> rafs_q;
};

// tree depths of a family: internal nodes by depth (Easel convention)
int plan_tree(covgpu_batch* b, const covgpu_family& fam, FamHost& f) {
  const int N = f.N;
  f.order.clear();
  f.loff.assign(1, 0);
  if (N < 2) return 0;
  if (!fam.left || !fam.right) return bfail(b, 11, "family %d: no tree", f.idx);
  std::vector<int> seen_leaf(N, 0), seen_node(N - 1, 0), depth(N - 1, 0);
  for (int v = 0; v < N - 1; v++) {
    const int ch[2] = {fam.left[v], fam.right[v]};
    for (int k = 0; k < 2; k++) {
      const int c = ch[k];
      if (c <= 0) {
        if (-c >= N || seen_leaf[-c]++) return bfail(b, 11, "family %d: tree leaf %d repeated or out of range", f.idx, -c);
      } else {
        if (c >= N - 1 || c <= v || seen_node[c]++)
          return bfail(b, 11, "family %d: tree node %d has bad child %d", f.idx, v, c);
        if (fam.parent && fam.parent[c] != v) return bfail(b, 11, "family %d: tree parent[%d] != %d", f.idx, c, v);
        depth[c] = depth[v] + 1;
      }
    }
  }
  int maxd = 0;
  for (int v = 0; v < N - 1; v++) maxd = std::max(maxd, depth[v]);
  f.loff.assign(maxd + 2, 0);
  std::vector<int> cnt(maxd + 1, 0);
  for (int v = 0; v < N - 1; v++) cnt[depth[v]]++;
  for (int d = 0; d <= maxd; d++) f.loff[d + 1] = f.loff[d] + cnt[d];
  f.order.assign(N - 1, 0);
  std::vector<int> pos(f.loff.begin(), f.loff.end() - 1);
  for (int v = 0; v < N - 1; v++) f.order[pos[depth[v]]++] = v;
  return 0;
}

// the blocked raster order of the tensor count kernel's tiles (as
// umma_plan's, super-blocks of SB x SB tiles)
// the grouped count's task order of one family: the single-alignment
// count's rasters (covgpu_tile_order: squares, or bands of a x b tiles for
// a schedule value 1000 a + b); the schedule is checked when it is set
void tile_order(int nT, int SB, std::vector<int>& order) {
  order.assign((size_t)nT * (nT + 1) / 2, 0);
  int nj = 0;
  if (covgpu_tile_order(nT, SB, order.data(), nullptr, 0, &nj) != 0)
    covgpu_tile_order(nT, 10, order.data(), nullptr, 0, &nj);
}


size_t fam_bytes_hint(const FamHost& f, int nout, bool need_u, bool rafs, int pitch) {
  const size_t S = f.nslots, nT2 = (size_t)f.nT * f.nT, ntl = f.ntiles;
  size_t b = S * f.N * f.Lp + 3 * (size_t)f.N * 16 + ntl * 16 + nT2 * 4;
  b += (f.gsc ? (size_t)f.N * f.N * 8 + 2 * (size_t)f.N * f.Lw * 4 : 0) + (f.pb ? (size_t)f.L * 32 : 0);
  b += 2 * (size_t)f.ns * std::max(f.N - 1, 0) * f.Lp;
  b += (size_t)4 * S * 4 * f.Lp * pitch * 2;           // tensor operands
  b += S * ntl * 32 * TPP * 4 + (need_u ? S * ntl * 16 * TPP * 4 : 0);
  b += S * nT2 * TP * 40 + S * f.Lp * 4 * 40;
  b += S * nout * ntl * TPP * 8 + (rafs ? S * ntl * TPP * 8 : 0) + S * nout * nT2 * TP * 8;
  b += S * nout * (f.Lp * 16 + 64 + (size_t)apc_blocks(f.ntiles) * 16);
  return b + 40 * kAlign;
}

void place(Layout& Lo, std::vector<FamHost>& fams, const Types& T, int counter, uint8_t* base, bool rafs) {
  Bump m;
  m.base = base;
  const int nf = (int)fams.size();
  Lo.F.assign(nf, FamDev());
  // codes
  const size_t ax0 = m.off;
  for (int k = 0; k < nf; k++) Lo.F[k].ax = m.take<uint8_t>((size_t)fams[k].nslots * fams[k].N * fams[k].Lp);
  Lo.ax = base ? base + ax0 : nullptr;
  Lo.ax_bytes = m.off - ax0;
  // weights region: w, limbs as floats, limbs
  const size_t w0 = m.off;
  Lo.w_off.assign(nf, 0); Lo.lf_off.assign(nf, 0); Lo.lb_off.assign(nf, 0);
  for (int k = 0; k < nf; k++) { Lo.w_off[k] = m.off - w0; Lo.F[k].w = m.take<double>(fams[k].N); }
  for (int k = 0; k < nf; k++) { Lo.lf_off[k] = m.off - w0; Lo.F[k].limbf = m.take<float>(3 * (size_t)fams[k].N); }
  for (int k = 0; k < nf; k++) {
    Lo.lb_off[k] = m.off - w0;
    Lo.F[k].limbs = m.take<uint16_t>(3 * (size_t)fams[k].Npad);
  }
  Lo.w = base ? reinterpret_cast<double*>(base + w0) : nullptr;
  Lo.wreg_bytes = m.off - w0;
  // tree: left, right, lnodes per family, one int array
  const size_t t0 = m.off;
  size_t tn = 0;
  for (int k = 0; k < nf; k++) tn += 3 * (size_t)std::max(fams[k].N - 1, 1);
  int* tree = m.take<int>(tn);
  Lo.tree = tree; Lo.tree_n = tn;
  {
    size_t o = 0;
    for (int k = 0; k < nf; k++) {
      const size_t n = std::max(fams[k].N - 1, 1);
      Lo.F[k].left = tree ? tree + o : nullptr;
      Lo.F[k].right = tree ? tree + o + n : nullptr;
      Lo.F[k].lnodes = tree ? tree + o + 2 * n : nullptr;
      o += 3 * n;
    }
  }
  (void)t0;
  // tiles: TileRC, tile index, order
  const size_t ti0 = m.off;
  for (int k = 0; k < nf; k++) {
    Lo.F[k].tiles = m.take<TileRC>(fams[k].ntiles);
    Lo.F[k].tile_index = m.take<int>((size_t)fams[k].nT * fams[k].nT);
    Lo.F[k].order = m.take<int>(fams[k].ntiles);
  }
  Lo.tiles = base ? base + ti0 : nullptr;
  Lo.tiles_bytes = m.off - ti0;
  // weights scratch
  for (int k = 0; k < nf; k++) {
    const FamHost& f = fams[k];
    FamDev& d = Lo.F[k];
    d.pbinv = f.pb ? m.take<double>((size_t)f.L * 4) : nullptr;
    if (f.gsc) {
      d.gD = m.take<double>((size_t)f.N * f.N);
      d.gra = m.take<uint32_t>((size_t)f.N * f.Lw);
      d.grb = m.take<uint32_t>((size_t)f.N * f.Lw);
      d.glen = m.take<int>(f.N);
    }
  }
  // nulls
  for (int k = 0; k < nf; k++) {
    const FamHost& f = fams[k];
    const size_t rows = (size_t)f.ns * std::max(f.N - 1, 0) * f.Lp;
    Lo.F[k].fitch = rows ? m.take<uint8_t>(rows) : nullptr;
    Lo.F[k].scratch = rows ? m.take<uint8_t>(rows) : nullptr;
  }
  // tensor operands of the families counted on the tensor cores:
  // [family][4 buffers][nslots][4 Lp] rows of pitch
  Lo.pitch = 64;
  for (auto& f : fams) if (f.tens) Lo.pitch = std::max(Lo.pitch, f.Npad);
  Lo.op_rows = 0;
  for (int k = 0; k < nf; k++) {
    Lo.F[k].oprow0 = (int)Lo.op_rows;
    if (fams[k].tens) Lo.op_rows += (int64_t)4 * fams[k].nslots * 4 * fams[k].Lp;
  }
  Lo.ops = (Lo.op_rows > 0 && T.need_w) ? m.take<uint16_t>((size_t)Lo.op_rows * Lo.pitch) : nullptr;
  (void)counter;
  // counts
  const size_t c0 = m.off;
  for (int k = 0; k < nf; k++)
    Lo.F[k].cnt = T.need_w ? m.take<float>((size_t)fams[k].nslots * fams[k].ntiles * 32 * TPP) : nullptr;
  Lo.cnt = base ? reinterpret_cast<float*>(base + c0) : nullptr;
  Lo.cnt_floats = (int64_t)((m.off - c0) / sizeof(float));
  for (int k = 0; k < nf; k++)
    Lo.F[k].ucnt = T.need_u ? m.take<float>((size_t)fams[k].nslots * fams[k].ntiles * 16 * TPP) : nullptr;
  // marginals
  for (int k = 0; k < nf; k++) {
    const FamHost& f = fams[k];
    const size_t S = f.nslots, nT2 = (size_t)f.nT * f.nT;
    Lo.F[k].part4 = m.take<double>(S * nT2 * TP * 4);
    Lo.F[k].partR = m.take<double>(S * nT2 * TP);
    Lo.F[k].mpc = m.take<double>(S * f.Lp * 4);
    Lo.F[k].meanp = m.take<double>(S * 4);
  }
  const size_t pm0 = m.off;
  for (int k = 0; k < nf; k++) Lo.F[k].pm = m.take<double>((size_t)fams[k].nslots * fams[k].Lp * 4);
  for (int k = 0; k < nf; k++) Lo.F[k].pmdf = m.take<float2>((size_t)fams[k].nslots * fams[k].Lp * 4);
  for (int k = 0; k < nf; k++) Lo.F[k].lpi = m.take<float4>((size_t)fams[k].nslots * fams[k].Lp * 4);
  Lo.pm = base ? reinterpret_cast<double*>(base + pm0) : nullptr;
  Lo.pm_bytes = m.off - pm0;
  // scores and corrections
  const int nout = T.ntypes;
  for (int k = 0; k < nf; k++) {
    const FamHost& f = fams[k];
    const size_t S = f.nslots, nT2 = (size_t)f.nT * f.nT, nsq = S * nout;
    FamDev& d = Lo.F[k];
    d.cov = m.take<float2>(S * nout * f.ntiles * TPP);
    d.cov2 = rafs ? m.take<float2>(S * f.ntiles * TPP) : nullptr;
    d.part1 = m.take<double>(S * nout * nT2 * TP);
    d.colx = m.take<double>(nsq * f.Lp);
    d.colxf = m.take<float2>(nsq * f.Lp);
    d.avg = m.take<double>(nsq);
    d.apcf = m.take<float4>(nsq);
    d.tmin = m.take<double>(nsq * apc_blocks(f.ntiles));
    d.tmax = m.take<double>(nsq * apc_blocks(f.ntiles));
  }
  // every family's (min, max) pairs in one region (read back in one copy;
  // a family's pairs start at F[k].mm - mm)
  const size_t mm0 = m.off;
  for (int k = 0; k < nf; k++) Lo.F[k].mm = m.take<double>((size_t)fams[k].nslots * nout * 2);
  Lo.mm = base ? reinterpret_cast<double*>(base + mm0) : nullptr;
  Lo.mm_n = (m.off - mm0) / sizeof(double);
  Lo.status = m.take<int>(nf);
  for (int k = 0; k < nf; k++) Lo.F[k].status = Lo.status ? Lo.status + k : nullptr;
  Lo.total = m.off;
}

// prefix of per-family block counts (appended to the descriptor table)
struct Tab {
  std::vector<uint8_t> h;
  size_t put(const void* p, size_t bytes) {
    const size_t o = align_up(h.size());
    h.resize(o + align_up(std::max<size_t>(bytes, 1)));
    if (bytes) memcpy(h.data() + o, p, bytes);
    return o;
  }
};

struct Pre {
  std::vector<int> v;
  int total() const { return v.back(); }
};
template <class F>
Pre prefix(int n, F blocks) {
  Pre p;
  p.v.assign(n + 1, 0);
  for (int k = 0; k < n; k++) p.v[k + 1] = p.v[k] + blocks(k);
  return p;
}

}  // namespace

// the device passes of one chunk on slot S, from the uploads to the
// corrected scores, launched and left running; the chunk's state is kept in
// S.pc for chunk_finish
static int chunk_launch(covgpu_batch* b, Slot& S, const covgpu_params* p, const covgpu_family* fam_in,
                        std::vector<FamHost>& fams, const Types& T) {
  const int nf = (int)fams.size(), nout = T.ntypes;
  const int counter = p->counter;
  const bool rafs = !T.rafs_q.empty();
  // ---- layout ----
  Layout Lo;
  place(Lo, fams, T, counter, nullptr, rafs);
  int s;
  if ((s = grow(b, &S.arena, &S.arena_cap, Lo.total))) return s;
  place(Lo, fams, T, counter, S.arena, rafs);
  // ---- host tables: tiles, trees, weights given by the caller ----
  std::vector<uint8_t> tiles_h(Lo.tiles_bytes, 0);
  for (int k = 0; k < nf; k++) {
    const FamHost& f = fams[k];
    const size_t base = (const uint8_t*)Lo.F[k].tiles - Lo.tiles;
    TileRC* tl = reinterpret_cast<TileRC*>(tiles_h.data() + base);
    int* ti = reinterpret_cast<int*>(tiles_h.data() + ((const uint8_t*)Lo.F[k].tile_index - Lo.tiles));
    int* od = reinterpret_cast<int*>(tiles_h.data() + ((const uint8_t*)Lo.F[k].order - Lo.tiles));
    int n = 0;
    for (int I = 0; I < f.nT; I++)
      for (int J = 0; J < f.nT; J++) ti[I * f.nT + J] = -1;
    for (int I = 0; I < f.nT; I++)
      for (int J = I; J < f.nT; J++) { ti[I * f.nT + J] = n; tl[n++] = TileRC{I, J}; }
    std::vector<int> order;
    tile_order(f.nT, b->sb, order);
    memcpy(od, order.data(), order.size() * sizeof(int));
  }
  std::vector<int> tree_h(Lo.tree_n, 0);
  {
    size_t o = 0;
    for (int k = 0; k < nf; k++) {
      const FamHost& f = fams[k];
      const size_t n = std::max(f.N - 1, 1);
      if (f.N >= 2) {
        memcpy(&tree_h[o], fam_in[f.idx].left, (f.N - 1) * sizeof(int));
        memcpy(&tree_h[o + n], fam_in[f.idx].right, (f.N - 1) * sizeof(int));
        memcpy(&tree_h[o + 2 * n], f.order.data(), (f.N - 1) * sizeof(int));
      }
      o += 3 * n;
    }
  }
  for (int k = 0; k < nf; k++) {
    FamDev& d = Lo.F[k];
    const FamHost& f = fams[k];
    d.N = f.N; d.L = f.L; d.Lp = f.Lp; d.nT = f.nT; d.ntiles = f.ntiles; d.nslots = f.nslots; d.Lw = f.Lw;
    d.Npad = f.Npad;
    d.sa.nout = nout;
  }
  // ---- uploads ----
  BK(cudaMemsetAsync(Lo.ax, 4, Lo.ax_bytes, S.st));
  BK(cudaMemsetAsync(Lo.status, 0, nf * sizeof(int), S.st));
  for (int k = 0; k < nf; k++) {
    const FamHost& f = fams[k];
    BK(cudaMemcpy2DAsync(Lo.F[k].ax, f.Lp, fam_in[f.idx].ax, f.L, f.L, f.N, cudaMemcpyHostToDevice, S.st));
  }
  BK(cudaMemcpyAsync(Lo.tiles, tiles_h.data(), Lo.tiles_bytes, cudaMemcpyHostToDevice, S.st));
  BK(cudaMemcpyAsync(Lo.tree, tree_h.data(), tree_h.size() * sizeof(int), cudaMemcpyHostToDevice, S.st));

  // ---- weights: the caller's, normalised and quantised here; R-scape's
  // rule (GSC or position-based), normalised and quantised on the device
  // inside the graph below, alongside the nulls ----
  std::vector<uint8_t> wreg(Lo.wreg_bytes, 0);
  std::vector<double> wtot_q(nf, 0.0);
  for (int k = 0; k < nf; k++) {
    const FamHost& f = fams[k];
    FamDev& d = Lo.F[k];
    if (f.gsc || f.pb) {   // made on the device: three limbs
      d.nl = 3; d.B = 0.f; d.s_hi = 0.f; d.s_lo = 0.f;
      continue;
    }
    double* w = reinterpret_cast<double*>(wreg.data() + Lo.w_off[k]);
    const double* src = fam_in[f.idx].wgt;
    if (!src) {   // one sequence
      for (int i = 0; i < f.N; i++) w[i] = 1.0;
    } else {
      for (int i = 0; i < f.N; i++) {
        if (!(src[i] >= 0.0) || !std::isfinite(src[i]))
          return bfail(b, 11, "family %d: weight %d is negative or not finite", f.idx, i);
        w[i] = src[i];
      }
    }
    std::vector<uint16_t> lim((size_t)3 * f.Npad, 0);
    CountWeights cw;
    make_limbs(w, f.N, f.Npad, lim.data(), &cw, &wtot_q[k]);
    memcpy(wreg.data() + Lo.lb_off[k], lim.data(), lim.size() * sizeof(uint16_t));
    float* lf = reinterpret_cast<float*>(wreg.data() + Lo.lf_off[k]);
    for (int l = 0; l < 3; l++)
      for (int i = 0; i < f.N; i++) lf[(size_t)l * f.N + i] = (float)lim[(size_t)l * f.Npad + i];
    d.nl = cw.nl; d.B = cw.B; d.s_hi = cw.s_hi; d.s_lo = cw.s_lo;
  }
  BK(cudaMemcpyAsync(Lo.w, wreg.data(), Lo.wreg_bytes, cudaMemcpyHostToDevice, S.st));
  // the statistics pass's arguments
  for (int k = 0; k < nf; k++) {
    const FamHost& f = fams[k];
    FamDev& d = Lo.F[k];
    StatsArgs& A = d.sa;
    memset(&A, 0, sizeof(A));
    A.cnt = T.need_w ? d.cnt : nullptr;
    A.ucnt = T.need_u ? d.ucnt : nullptr;
    A.pm = d.pm; A.pmdf = d.pmdf; A.lpi = d.lpi; A.logtab = b->d_logtab; A.meanp = d.meanp;
    A.cov = d.cov; A.part1 = d.part1; A.tiles = d.tiles;
    A.ntiles = f.ntiles; A.nT = f.nT; A.L = f.L; A.Lp = f.Lp; A.N = f.N;
    const float hi = (float)wtot_q[k];   // made on the device for R-scape's weights
    A.wtot = make_float2(hi, (float)(wtot_q[k] - (double)hi));
    A.stats = T.mask;
    int cls = p->covclass;
    if (cls == 3) cls = (f.N <= p->nseqthresh || f.L <= p->alenthresh) ? 1 : 0;
    A.cls = cls;
    auto split = [](double x) { const float h = (float)x; return make_float2(h, (float)(x - (double)h)); };
    A.invD = split(1.0 / ((f.N > 1) ? (double)f.N * ((double)f.N - 1.0) : 1.0));
    A.invN = split(1.0 / (double)f.N);
    A.nout = nout;
    for (int q = 0; q < MAXOUT; q++) A.outstat[q] = (q < nout) ? T.outstat[q] : 0;
    for (int c = 0; c < 16; c++) A.allow[c] = (float)p->allow[c];
  }

  // ---- the device passes from the nulls to the corrected scores ----
  Tab tb;
  const size_t oF = tb.put(Lo.F.data(), nf * sizeof(FamDev));
  int maxdepth = 0, maxLp = 32;
  for (auto& f : fams) { maxdepth = std::max(maxdepth, f.depth()); maxLp = std::max(maxLp, f.Lp); }
  const bool srow_cta = maxLp <= replay_smem_max(), srow_warp = 8 * maxLp <= replay_smem_max();
  struct Lvl { size_t lv, up, cta, warp; int nup, ncta, nwarp; };
  std::vector<Lvl> lvl(maxdepth);
  for (int dd = 0; dd < maxdepth; dd++) {
    std::vector<int2> lv(nf);
    for (int k = 0; k < nf; k++) {
      const FamHost& f = fams[k];
      const bool has = f.ns > 0 && dd < f.depth();
      lv[k] = has ? make_int2(f.loff[dd], f.loff[dd + 1] - f.loff[dd]) : make_int2(0, 0);
    }
    Pre pu = prefix(nf, [&](int k) { return lv[k].y ? (lv[k].y * (fams[k].Lp >> 4) + 255) / 256 * fams[k].ns : 0; });
    Pre pc = prefix(nf, [&](int k) {
      return (lv[k].y && replay_uses_cta(lv[k].y, fams[k].ns)) ? 2 * lv[k].y * fams[k].ns : 0;
    });
    Pre pw = prefix(nf, [&](int k) {
      return (lv[k].y && !replay_uses_cta(lv[k].y, fams[k].ns)) ? (2 * lv[k].y + 7) / 8 * fams[k].ns : 0;
    });
    lvl[dd].lv = tb.put(lv.data(), nf * sizeof(int2));
    lvl[dd].up = tb.put(pu.v.data(), pu.v.size() * 4); lvl[dd].nup = pu.total();
    lvl[dd].cta = tb.put(pc.v.data(), pc.v.size() * 4); lvl[dd].ncta = pc.total();
    lvl[dd].warp = tb.put(pw.v.data(), pw.v.size() * 4); lvl[dd].nwarp = pw.total();
  }
  Pre pcol = prefix(nf, [&](int k) { return fams[k].pb ? (fams[k].L + 255) / 256 : 0; });
  Pre prow = prefix(nf, [&](int k) { return fams[k].pb ? fams[k].N : 0; });
  Pre pcod = prefix(nf, [&](int k) { return fams[k].gsc ? fams[k].N : 0; });
  Pre pid = prefix(nf, [&](int k) { const int nt = (fams[k].N + 31) / 32; return fams[k].gsc ? nt * nt : 0; });
  Pre pup = prefix(nf, [&](int k) { return fams[k].gsc ? 1 : 0; });
  Pre plb = prefix(nf, [&](int k) { return (fams[k].gsc || fams[k].pb) ? 1 : 0; });
  int maxN = 1;
  for (auto& f : fams) if (f.gsc) maxN = std::max(maxN, f.N);
  const size_t o_col = tb.put(pcol.v.data(), pcol.v.size() * 4), o_row = tb.put(prow.v.data(), prow.v.size() * 4);
  const size_t o_cod = tb.put(pcod.v.data(), pcod.v.size() * 4), o_id = tb.put(pid.v.data(), pid.v.size() * 4);
  const size_t o_up = tb.put(pup.v.data(), pup.v.size() * 4), o_lb = tb.put(plb.v.data(), plb.v.size() * 4);
  Pre prs = prefix(nf, [&](int k) { return fams[k].ns > 0 ? (fams[k].L + 255) / 256 * fams[k].ns : 0; });
  Pre prr = prefix(nf, [&](int k) { return fams[k].ns > 0 ? (fams[k].Lp + 255) / 256 * fams[k].ns : 0; });
  Pre pprep = prefix(nf, [&](int k) {
    return fams[k].tens ? fams[k].Npad / 64 * (fams[k].Lp / 32) * fams[k].nslots : 0;
  });
  Pre ptile = prefix(nf, [&](int k) { return fams[k].ntiles * fams[k].nslots; });
  Pre pt3 = prefix(nf, [&](int k) { return (fams[k].tens && Lo.F[k].nl == 3) ? fams[k].ntiles * fams[k].nslots : 0; });
  Pre pt1 = prefix(nf, [&](int k) { return (fams[k].tens && Lo.F[k].nl == 1) ? fams[k].ntiles * fams[k].nslots : 0; });
  Pre psimt = prefix(nf, [&](int k) { return fams[k].tens ? 0 : fams[k].ntiles * fams[k].nslots; });
  Pre ppm = prefix(nf, [&](int k) { return (fams[k].L + 127) / 128 * fams[k].nslots; });
  Pre pmp = prefix(nf, [&](int k) { return fams[k].nslots; });
  Pre pcx = prefix(nf, [&](int k) { return (fams[k].L + 255) / 256 * fams[k].nslots * nout; });
  Pre psq = prefix(nf, [&](int k) { return fams[k].nslots * nout; });
  Pre pap = prefix(nf, [&](int k) { return apc_blocks(fams[k].ntiles) * fams[k].nslots * nout; });
  const size_t o_rs = tb.put(prs.v.data(), prs.v.size() * 4), o_rr = tb.put(prr.v.data(), prr.v.size() * 4);
  const size_t o_prep = tb.put(pprep.v.data(), pprep.v.size() * 4), o_tile = tb.put(ptile.v.data(), ptile.v.size() * 4);
  const size_t o_t3 = tb.put(pt3.v.data(), pt3.v.size() * 4), o_t1 = tb.put(pt1.v.data(), pt1.v.size() * 4);
  const size_t o_simt = tb.put(psimt.v.data(), psimt.v.size() * 4);
  const size_t o_pm = tb.put(ppm.v.data(), ppm.v.size() * 4), o_mp = tb.put(pmp.v.data(), pmp.v.size() * 4);
  const size_t o_cx = tb.put(pcx.v.data(), pcx.v.size() * 4), o_sq = tb.put(psq.v.data(), psq.v.size() * 4);
  const size_t o_ap = tb.put(pap.v.data(), pap.v.size() * 4);
  std::vector<UmmaFam> uf(nf);
  for (int k = 0; k < nf; k++) {
    const FamHost& f = fams[k];
    const FamDev& d = Lo.F[k];
    UmmaFam& u = uf[k];
    u.row0 = d.oprow0;
    u.rows_per_buf = f.nslots * 4 * f.Lp;
    u.Lp = f.Lp; u.ntiles = f.ntiles; u.nkb = f.Npad / 64;
    u.orow0 = d.cnt ? (int64_t)(d.cnt - Lo.cnt) / 32 : 0;
    u.order = d.order; u.tiles = d.tiles;
    u.B = d.B; u.s_hi = d.s_hi; u.s_lo = d.s_lo;
  }
  const size_t o_uf = tb.put(uf.data(), nf * sizeof(UmmaFam));
  // with room after the tables for the histogram pass's tables (chunk_finish)
  const size_t stat_room = align_up((size_t)nf * nout * sizeof(StatDev)) + align_up(((size_t)nf * nout + 1) * 4) +
                           2 * kAlign;
  if ((s = grow(b, &S.tab, &S.tab_cap, align_up(tb.h.size()) + stat_room))) return s;
  BK(cudaMemcpyAsync(S.tab, tb.h.data(), tb.h.size(), cudaMemcpyHostToDevice, S.st));
  const FamDev* dF = reinterpret_cast<const FamDev*>(S.tab + oF);
  auto P = [&](size_t o) { return reinterpret_cast<const int*>(S.tab + o); };
  if (pup.total() && !grp_weights_gsc_prepare()) return bfail(b, 90, "GSC kernel attributes");

  // the key of this chunk's device passes: the descriptor tables (they hold
  // every pointer and size the launches read) and the launch parameters
  std::vector<uint8_t> key(tb.h);
  {
    const int64_t extra[] = {nf, counter, (int64_t)T.mask, T.need_w, T.need_u, (int64_t)(uintptr_t)S.arena,
                             (int64_t)(uintptr_t)S.tab, maxLp, (int64_t)p->seed};
    key.insert(key.end(), (const uint8_t*)extra, (const uint8_t*)extra + sizeof(extra));
    for (int q : T.rafs_q) key.push_back((uint8_t)q);
    key.insert(key.end(), (const uint8_t*)&T.ct, (const uint8_t*)&T.ct + sizeof(T.ct));
  }
  int launches = 0;
  auto passes = [&]() -> int {
    // R-scape's weights on the second stream, alongside the nulls
    const bool wdev = plb.total() > 0;
    if (wdev) {
      BK(cudaEventRecord(S.fork, S.st));
      BK(cudaStreamWaitEvent(S.st2, S.fork, 0));
      FamDev* dFw = reinterpret_cast<FamDev*>(S.tab + oF);
      UmmaFam* dUw = reinterpret_cast<UmmaFam*>(S.tab + o_uf);
      BK(grp_weights_pb(dF, nf, P(o_col), pcol.total(), P(o_row), prow.total(), S.st2));
      BK(grp_weights_gsc(dF, nf, P(o_cod), pcod.total(), P(o_id), pid.total(), P(o_up), pup.total(), maxN, S.st2));
      BK(grp_weights_limbs(dFw, nf, P(o_lb), plb.total(), dUw, S.st2));
      BK(cudaEventRecord(S.join, S.st2));
      launches += (pcol.total() ? 2 : 0) + (pup.total() ? 3 : 0) + 1;
    }
    // nulls: Fitch up the tree, the roots, the replay down it
    for (int dd = maxdepth - 1; dd >= 0; dd--)
      if (lvl[dd].nup) {
        BK(grp_fitch_up(dF, nf, reinterpret_cast<const int2*>(S.tab + lvl[dd].lv), P(lvl[dd].up), lvl[dd].nup,
                        p->seed, S.st));
        launches++;
      }
    if (prs.total()) {
      BK(grp_root(dF, nf, P(o_rs), prs.total(), P(o_rr), prr.total(), p->seed, S.st));
      launches += 2;
    }
    for (int dd = 0; dd < maxdepth; dd++) {
      const int2* lv = reinterpret_cast<const int2*>(S.tab + lvl[dd].lv);
      if (lvl[dd].ncta) {
        BK(grp_replay(dF, nf, lv, P(lvl[dd].cta), lvl[dd].ncta, true, srow_cta, maxLp, p->seed, S.st));
        launches++;
      }
      if (lvl[dd].nwarp) {
        BK(grp_replay(dF, nf, lv, P(lvl[dd].warp), lvl[dd].nwarp, false, srow_warp, maxLp, p->seed, S.st));
        launches++;
      }
    }
    if (wdev) BK(cudaStreamWaitEvent(S.st, S.join, 0));
    // counts and marginals
    if (T.need_w) {
      // the tensor cores count the families at or above the batch's SIMT
      // threshold, the SIMT kernel the others: the two give the same counts
      if (pprep.total()) {
        BK(grp_umma_prep(dF, nf, P(o_prep), pprep.total(), Lo.pitch, Lo.ops, S.st));
        const UmmaFam* dU = reinterpret_cast<const UmmaFam*>(S.tab + o_uf);
        for (int nl : {3, 1}) {
          const Pre& pt = (nl == 3) ? pt3 : pt1;
          if (!pt.total()) continue;
          const int us = grp_umma_count(dU, nf, P(nl == 3 ? o_t3 : o_t1), pt.total(), nl, Lo.ops, Lo.pitch,
                                        Lo.op_rows, Lo.cnt, Lo.cnt_floats / 32, S.d_uerr, S.st);
          if (us) return bfail(b, us == 11 ? 12 : 90, "tensor counting not available for this batch (%d)", us);
          launches++;
        }
        launches++;
      }
      if (psimt.total()) {
        BK(grp_count_simt(dF, nf, P(o_simt), psimt.total(), false, true, S.st));
        launches++;
      }
      BK(grp_marginals(dF, nf, P(o_tile), ptile.total(), P(o_pm), ppm.total(), P(o_mp), pmp.total(), S.st));
      launches += 3;
    } else {
      BK(cudaMemsetAsync(Lo.pm, 0, Lo.pm_bytes, S.st));
    }
    if (T.need_u) {
      BK(grp_count_simt(dF, nf, P(o_tile), ptile.total(), true, false, S.st));
      launches++;
    }
    BK(grp_stats(dF, nf, P(o_tile), ptile.total(), stats_cf(T.mask), S.st));
    launches++;
    for (int q : T.rafs_q) {
      for (int k = 0; k < nf; k++) {
        const FamDev& d = Lo.F[k];
        const int64_t plane = (int64_t)d.ntiles * TPP;
        BK(cudaMemcpy2DAsync(d.cov2, plane * sizeof(float2), d.cov + q * plane, nout * plane * sizeof(float2),
                             plane * sizeof(float2), d.nslots, cudaMemcpyDeviceToDevice, S.st));
      }
      BK(grp_rafs(dF, nf, P(o_tile), ptile.total(), q, S.st));
      launches++;
    }
    BK(grp_apc(dF, nf, P(o_cx), pcx.total(), P(o_sq), psq.total(), P(o_ap), pap.total(), T.ct, S.st));
    launches += 4;
    return 0;
  };
  BK(cudaEventRecord(S.ev[0], S.st));
  Slot::Graph* hit = nullptr;
  for (auto& g : S.graphs)
    if (g.key == key) { hit = &g; break; }
  if (hit) {
    BK(cudaGraphLaunch(hit->exec, S.st));
    b->graph_replays++;
    launches = hit->launches;
    hit->used = ++S.tick;
  } else {
    cudaGraph_t g = nullptr;
    BK(cudaStreamBeginCapture(S.st, cudaStreamCaptureModeThreadLocal));
    const int ps = passes();
    cudaError_t ce = cudaStreamEndCapture(S.st, &g);
    if (ps) { if (g) cudaGraphDestroy(g); return ps; }
    if (ce != cudaSuccess) return bfail(b, 90, "graph capture: %s", cudaGetErrorString(ce));
    cudaGraphExec_t exec = nullptr;
    ce = cudaGraphInstantiate(&exec, g, 0);
    cudaGraphDestroy(g);
    if (ce != cudaSuccess) return bfail(b, 90, "graph instantiate: %s", cudaGetErrorString(ce));
    constexpr size_t kGraphs = 24;
    if (S.graphs.size() >= kGraphs) {   // out goes the least recently used
      auto old = std::min_element(S.graphs.begin(), S.graphs.end(),
                                  [](const Slot::Graph& x, const Slot::Graph& y) { return x.used < y.used; });
      cudaGraphExecDestroy(old->exec);
      S.graphs.erase(old);
    }
    S.graphs.push_back(Slot::Graph{std::move(key), exec, launches, ++S.tick});
    BK(cudaGraphLaunch(exec, S.st));
  }
  b->nlaunch += launches;
  BK(cudaEventRecord(S.ev[1], S.st));
  S.pc.fams = std::move(fams);
  S.pc.Lo = std::move(Lo);
  S.pc.tab_used = tb.h.size();
  S.pc.oF = oF;
  return 0;
}

// the host phases of the chunk whose device passes chunk_launch started on
// slot S: ranges, histograms, fits, survival tables, E-values and hits,
// written at each family's position
static int chunk_finish(covgpu_batch* b, Slot& S, const covgpu_params* p, const Types& T, const int* covtypes,
                        covgpu_result* results, covgpu_hit* hits, int hitcap) {
  std::vector<FamHost>& fams = S.pc.fams;
  Layout& Lo = S.pc.Lo;
  const int nf = (int)fams.size(), nout = T.ntypes;
  const FamDev* dF = reinterpret_cast<const FamDev*>(S.tab + S.pc.oF);
  int s;
  std::vector<double> mm(Lo.mm_n);
  std::vector<int> stat(nf);
  BK(cudaMemcpyAsync(mm.data(), Lo.mm, mm.size() * sizeof(double), cudaMemcpyDeviceToHost, S.st));
  BK(cudaMemcpyAsync(stat.data(), Lo.status, nf * sizeof(int), cudaMemcpyDeviceToHost, S.st));
  int uerr = 0;
  BK(cudaMemcpyAsync(&uerr, S.d_uerr, sizeof(int), cudaMemcpyDeviceToHost, S.st));
  BK(cudaStreamSynchronize(S.st));
  if (uerr) {
    cudaMemset(S.d_uerr, 0, sizeof(int));
    return bfail(b, 24, "tensor counting kernel: barrier wait timed out (code %d)", uerr);
  }
  auto status_fail = [&](int k, int st) {
    const int fi = fams[k].idx;
    if (st == 2) return bfail(b, 20, "family %d: marginal probabilities failed validation", fi);
    if (st == 3) return bfail(b, 21, "family %d: bad covariation: NaN after correction", fi);
    if (st == 4) return bfail(b, 22, "family %d: histogram bin out of range", fi);
    return bfail(b, 23, "family %d: device status %d", fi, st);
  };
  for (int k = 0; k < nf; k++)
    if (stat[k]) return status_fail(k, stat[k]);

  // ---- phase 1: widths and bins; the null histograms ----
  struct Entry { int k, q; RsStat X; };
  std::vector<Entry> E;
  std::vector<std::vector<RsStat>> XS(nf, std::vector<RsStat>(nout));
  struct HistGuard {
    std::vector<std::vector<RsStat>>* x;
    ~HistGuard() { for (auto& v : *x) for (auto& r : v) if (r.h) covh_Destroy(r.h); }
  } guard{&XS};
  std::vector<size_t> mm_off(nf);
  for (int k = 0; k < nf; k++) mm_off[k] = (size_t)(Lo.F[k].mm - Lo.mm);
  int64_t obs_tot = 0;
  std::vector<std::pair<int, int>> act;   // active (family, statistic)
  for (int k = 0; k < nf; k++) {
    const FamHost& f = fams[k];
    for (int q = 0; q < nout; q++) {
      covgpu_result& R = results[(size_t)f.idx * nout + q];
      memset(&R, 0, sizeof(R));
      R.covtype = covtypes[q];
      RsStat& X = XS[k][q];
      char em[256];
      if ((s = rs_width(p, f.N, f.ns, mm.data() + mm_off[k], nout, q, R, X, em, sizeof(em))))
        return bfail(b, s, "family %d: %s", f.idx, em);
      if (!X.active) continue;
      X.obs_off = obs_tot;
      obs_tot += X.nbcum;
      act.push_back({k, q});
    }
  }
  const int na = (int)act.size();
  std::vector<StatDev> SD(na);
  std::vector<uint64_t> obs(std::max<int64_t>(obs_tot, 1));
  Bump sm;
  unsigned long long* d_obs = nullptr;
  if (na > 0) {
    // the stat area: obs, then (phase 3) sf and tail tables, hits
    size_t hits_per = 0;
    for (auto& a : act) {
      const FamHost& f = fams[a.first];
      hits_per += (size_t)std::min<int64_t>(hitcap, (int64_t)f.L * (f.L - 1) / 2 + 1);
    }
    int64_t nbtot = 0;
    for (auto& a : act) nbtot += XS[a.first][a.second].nb_real + XS[a.first][a.second].nbcum;
    const size_t need = align_up(obs_tot * 8) + 4 * align_up((size_t)nbtot * 8 * 2) + align_up(na * 4) +
                        5 * align_up(hits_per * 8) + 2 * align_up((size_t)na * 1024 + 4096) + 16 * kAlign;
    if ((s = grow(b, &b->stat, &b->stat_cap, need))) return s;
    sm.base = b->stat;
    d_obs = sm.take<unsigned long long>(obs_tot);
    int maxwin = 1;
    std::vector<int> hb(na);
    for (int e = 0; e < na; e++) {
      const int k = act[e].first, q = act[e].second;
      const FamHost& f = fams[k];
      const RsStat& X = XS[k][q];
      StatDev& x = SD[e];
      memset(&x, 0, sizeof(x));
      x.fam = k; x.q = q; x.active = 1;
      x.hb = binc_host(p->bmin, X.w);
      x.nbcap = X.nbcum;
      x.wbase = std::max(0, std::min(X.wbase, X.nbcum - 1));
      x.nwin = std::min(48 * 1024, X.nbcum - x.wbase);
      x.obs = d_obs + X.obs_off;
      maxwin = std::max(maxwin, x.nwin);
      const int64_t items = (int64_t)f.ntiles * f.ns;
      hb[e] = (int)std::max<int64_t>(1, std::min<int64_t>(items / 16, 304));
    }
    Pre ph = prefix(na, [&](int e) { return hb[e]; });
    Tab t2;
    const size_t o_sd = t2.put(SD.data(), na * sizeof(StatDev)), o_ph = t2.put(ph.v.data(), ph.v.size() * 4);
    // the room after the descriptor tables was reserved by chunk_launch
    uint8_t* tab2 = S.tab + align_up(S.pc.tab_used);
    if (align_up(S.pc.tab_used) + t2.h.size() > S.tab_cap) return bfail(b, 90, "batch table area overflow");
    BK(cudaMemcpyAsync(tab2, t2.h.data(), t2.h.size(), cudaMemcpyHostToDevice, S.st));
    BK(cudaMemsetAsync(d_obs, 0, std::max<int64_t>(obs_tot, 1) * 8, S.st));
    BK(grp_hist(dF, reinterpret_cast<const StatDev*>(tab2 + o_sd), na, reinterpret_cast<const int*>(tab2 + o_ph),
                ph.total(), maxwin, S.st));
    b->nlaunch += 1;
    BK(cudaMemcpyAsync(obs.data(), d_obs, obs_tot * 8, cudaMemcpyDeviceToHost, S.st));
    BK(cudaMemcpyAsync(stat.data(), Lo.status, nf * sizeof(int), cudaMemcpyDeviceToHost, S.st));
    BK(cudaStreamSynchronize(S.st));
    for (int k = 0; k < nf; k++)
      if (stat[k]) return status_fail(k, stat[k]);

    // ---- phase 2: histograms, tails, the tail fits ----
    std::vector<FitReq> fr;
    std::vector<int> fe;
    for (int e = 0; e < na; e++) {
      const int k = act[e].first, q = act[e].second;
      const FamHost& f = fams[k];
      RsStat& X = XS[k][q];
      const int64_t P = (int64_t)f.L * (f.L - 1) / 2;
      char em[256];
      if ((s = rs_histogram(p, f.fracfit, f.ns, P, obs.data() + X.obs_off, X, em, sizeof(em))))
        return bfail(b, s, "family %d: %s", f.idx, em);
      if (!p->doexpfit) {
        const ESL_HISTOGRAM* h = X.h;
        fr.push_back(FitReq{h->obs, h->cmin, h->imax, h->bmin, h->w, h->phi});
        fe.push_back(e);
      }
    }
    if (!fr.empty()) {
      const int fs = gamma_fit_batch_launch(b->fits, (int)fr.size(), fr.data(), S.st);
      if (fs) return bfail(b, 32, "could not do the Gamma fits (%d)", fs);
      b->nlaunch += 1;
      BK(cudaStreamSynchronize(S.st));
      for (size_t k = 0; k < fr.size(); k++) {
        const int e = fe[k];
        RsStat& X = XS[act[e].first][act[e].second];
        const int st2 = gamma_fit_batch_collect(b->fits, (int)k, &X.lambda, &X.tau, &X.evals);
        if (st2) return bfail(b, 32, "family %d: could not do a Gamma fit (%d)", fams[act[e].first].idx, st2);
      }
    }

    // ---- phase 3: survival tables ----
    int64_t sf_tot = 0, tail_tot = 0;
    for (int e = 0; e < na; e++) {
      RsStat& X = XS[act[e].first][act[e].second];
      X.tail_off = tail_tot;
      tail_tot += X.h->nb;
      if (!std::isinf(X.lambda)) { X.have_sf = true; X.sf_off = sf_tot; sf_tot += 2 * (int64_t)X.h->nb; }
    }
    double* d_sf = sm.take<double>(sf_tot);
    double* d_tail = sm.take<double>(tail_tot);
    int* d_nh = sm.take<int>(na);
    std::vector<double> sfh(std::max<int64_t>(sf_tot, 1));
    if (sf_tot > 0) {
      std::vector<SurvReq> sr;
      std::vector<int> sb;
      for (int e = 0; e < na; e++) {
        const RsStat& X = XS[act[e].first][act[e].second];
        if (!X.have_sf) continue;
        const ESL_HISTOGRAM* h = X.h;
        SurvReq r;
        r.cmin = h->cmin; r.nb = h->nb; r.doexp = p->doexpfit;
        r.bmin = h->bmin; r.w = h->w; r.mass = X.newmass; r.mu = X.mu; r.lambda = X.lambda; r.tau = X.tau;
        r.lga = p->doexpfit ? 0.0 : std::lgamma(X.tau);
        r.sf = d_sf + X.sf_off;
        sr.push_back(r);
        sb.push_back((2 * h->nb + 255) / 256);
      }
      Pre psf = prefix((int)sr.size(), [&](int e) { return sb[e]; });
      Tab t3;
      const size_t o_sr = t3.put(sr.data(), sr.size() * sizeof(SurvReq)), o_ps = t3.put(psf.v.data(), psf.v.size() * 4);
      uint8_t* tab3 = sm.take<uint8_t>(t3.h.size());
      BK(cudaMemcpyAsync(tab3, t3.h.data(), t3.h.size(), cudaMemcpyHostToDevice, S.st));
      BK(grp_survfit(reinterpret_cast<const SurvReq*>(tab3 + o_sr), reinterpret_cast<const int*>(tab3 + o_ps),
                     (int)sr.size(), psf.total(), S.st));
      b->nlaunch += 1;
      BK(cudaMemcpyAsync(sfh.data(), d_sf, sf_tot * 8, cudaMemcpyDeviceToHost, S.st));
      BK(cudaStreamSynchronize(S.st));
    }

    // ---- phase 4: thresholds, tail tables, E-values and hits ----
    std::vector<double> tail(std::max<int64_t>(tail_tot, 1));
    std::vector<int> dcap(na);
    for (int e = 0; e < na; e++) {
      const int k = act[e].first, q = act[e].second;
      const FamHost& f = fams[k];
      RsStat& X = XS[k][q];
      const int64_t P = (int64_t)f.L * (f.L - 1) / 2;
      covgpu_result& R = results[(size_t)f.idx * nout + q];
      rs_tables(p, P, 0, X, sfh.data() + X.sf_off, R, tail.data() + X.tail_off);
      StatDev& x = SD[e];
      x.T = rs_evaltables(p, P, X, d_sf + X.sf_off, d_tail + X.tail_off);
      x.K = evalcmp_host(x.T);
      x.hb = binc_host(x.T.bmin, x.T.w);
      dcap[e] = (int)std::min<int64_t>(hitcap, P + 1);
      x.hitcap = dcap[e];
      x.nhits = d_nh + e;
    }
    for (int e = 0; e < na; e++) SD[e].hi = sm.take<int>(dcap[e]);
    for (int e = 0; e < na; e++) SD[e].hj = sm.take<int>(dcap[e]);
    for (int e = 0; e < na; e++) SD[e].hsc = sm.take<double>(dcap[e]);
    for (int e = 0; e < na; e++) SD[e].hE = sm.take<double>(dcap[e]);
    for (int e = 0; e < na; e++) SD[e].hp = sm.take<double>(dcap[e]);
    if (sm.off > b->stat_cap) return bfail(b, 90, "batch statistics area overflow");
    Pre pe = prefix(na, [&](int e) { return fams[act[e].first].ntiles; });
    Tab t4;
    const size_t o_sd4 = t4.put(SD.data(), na * sizeof(StatDev)), o_pe = t4.put(pe.v.data(), pe.v.size() * 4);
    uint8_t* tab4 = sm.take<uint8_t>(t4.h.size());
    if (sm.off > b->stat_cap) return bfail(b, 90, "batch statistics area overflow");
    BK(cudaMemcpyAsync(d_tail, tail.data(), std::max<int64_t>(tail_tot, 1) * 8, cudaMemcpyHostToDevice, S.st));
    BK(cudaMemcpyAsync(tab4, t4.h.data(), t4.h.size(), cudaMemcpyHostToDevice, S.st));
    BK(cudaMemsetAsync(d_nh, 0, na * sizeof(int), S.st));
    BK(grp_evalue(dF, reinterpret_cast<const StatDev*>(tab4 + o_sd4), na, reinterpret_cast<const int*>(tab4 + o_pe),
                  pe.total(), S.st));
    b->nlaunch += 1;
    std::vector<int> nh(na);
    BK(cudaMemcpyAsync(nh.data(), d_nh, na * sizeof(int), cudaMemcpyDeviceToHost, S.st));
    BK(cudaStreamSynchronize(S.st));
    // the hit lists, read back together
    std::vector<size_t> ho(na + 1, 0);
    for (int e = 0; e < na; e++) ho[e + 1] = ho[e] + (hits ? (size_t)std::max(0, std::min(nh[e], dcap[e])) : 0);
    const size_t nall = ho[na];
    std::vector<int> hi_(nall), hj_(nall);
    std::vector<double> hs_(nall), hE_(nall), hp_(nall);
    for (int e = 0; e < na; e++) {
      const size_t n = ho[e + 1] - ho[e], o = ho[e];
      if (!n) continue;
      BK(cudaMemcpyAsync(hi_.data() + o, SD[e].hi, n * sizeof(int), cudaMemcpyDeviceToHost, S.st));
      BK(cudaMemcpyAsync(hj_.data() + o, SD[e].hj, n * sizeof(int), cudaMemcpyDeviceToHost, S.st));
      BK(cudaMemcpyAsync(hs_.data() + o, SD[e].hsc, n * sizeof(double), cudaMemcpyDeviceToHost, S.st));
      BK(cudaMemcpyAsync(hE_.data() + o, SD[e].hE, n * sizeof(double), cudaMemcpyDeviceToHost, S.st));
      BK(cudaMemcpyAsync(hp_.data() + o, SD[e].hp, n * sizeof(double), cudaMemcpyDeviceToHost, S.st));
    }
    if (nall) BK(cudaStreamSynchronize(S.st));
    for (int e = 0; e < na; e++) {
      const int k = act[e].first, q = act[e].second;
      covgpu_result& R = results[(size_t)fams[k].idx * nout + q];
      R.nhit = nh[e];
      const size_t n = ho[e + 1] - ho[e], o = ho[e];
      if (!n) continue;
      covgpu_hit* H = hits + ((size_t)fams[k].idx * nout + q) * hitcap;
      for (size_t i = 0; i < n; i++) H[i] = covgpu_hit{hi_[o + i], hj_[o + i], hs_[o + i], hE_[o + i], hp_[o + i]};
      // the reference lists hits in row-major pair order (src/covariation.c:827-893)
      std::sort(H, H + n, [](const covgpu_hit& a, const covgpu_hit& c) { return (a.i != c.i) ? a.i < c.i : a.j < c.j; });
    }
  }
  BK(cudaEventRecord(S.ev[2], S.st));
  BK(cudaEventSynchronize(S.ev[2]));
  float a = 0.f, c = 0.f;
  cudaEventElapsedTime(&a, S.ev[0], S.ev[1]);
  cudaEventElapsedTime(&c, S.ev[1], S.ev[2]);
  b->ms[0] += a; b->ms[1] += c;
  return 0;
}

extern "C" int covgpu_rscape_families(covgpu_batch* b, const covgpu_params* p, int nfam, const covgpu_family* fams_in,
                                      int ntypes, const int* covtypes, covgpu_result* results, covgpu_hit* hits,
                                      int hitcap) {
  if (!b) return 11;
  BK(cudaSetDevice(b->dev));
  b->err[0] = 0;
  b->ms[0] = b->ms[1] = b->ms[2] = 0.0;
  b->nlaunch = 0;
  b->nchunks = 0;
  if (nfam < 0 || !fams_in || !results || (nfam > 0 && (!covtypes || hitcap < 0)))
    return bfail(b, 11, "bad arguments");
  if (ntypes < 1 || ntypes > MAXOUT) return bfail(b, 11, "1..%d covariation types per call", MAXOUT);
  if (p->counter != COVGPU_COUNT_SIMT && p->counter != COVGPU_COUNT_TENSOR) return bfail(b, 11, "bad counter");
  if ((p->ncnt > 0 && p->samplesize != 3) || p->expBP > 0.0)
    return bfail(b, 11, "a structure belongs to one alignment: the two-set test and --structured run in covgpu_rscape");
  // the statistics, as score_async reads them
  Types T;
  T.ntypes = ntypes;
  T.ct.nout = ntypes;
  for (int q = 0; q < ntypes; q++) {
    if (covtypes[q] < 0 || covtypes[q] >= 27) return bfail(b, 11, "covariation type %d not supported", covtypes[q]);
    const int base = (covtypes[q] / 3) * 3, corr = covtypes[q] % 3;
    const int si = stat_of(base);
    T.outstat[q] = si;
    T.ct.act[q] = (corr == 0) ? -1 : corr - 1;
    if (base == 18 || base == 21) { T.need_u = true; T.mask |= S_RAF; }
    else { T.need_w = true; T.mask |= (1u << si); }
    if (base == 24) T.mask |= S_CCF;
    if (base == 21) T.rafs_q.push_back(q);
    if (p->covclass == 2 && base != 3 && base != 18 && base != 21 && base != 24)
      return bfail(b, 11, "class CWC is only defined for GT");
  }
  for (int q = ntypes; q < MAXOUT; q++) { T.outstat[q] = 0; T.ct.act[q] = -1; }
  const auto t0 = std::chrono::steady_clock::now();
  // plan every family
  std::vector<FamHost> all(nfam);
  for (int k = 0; k < nfam; k++) {
    const covgpu_family& f = fams_in[k];
    FamHost& h = all[k];
    h.idx = k;
    if (f.N < 1 || f.L < 2 || !f.ax) return bfail(b, 11, "family %d: bad sizes or no alignment", k);
    if (f.L > 48 * 1024) return bfail(b, 11, "family %d: alignment longer than 49152 columns", k);
    const int64_t n = (int64_t)f.N * f.L;
    uint8_t mx = 0;
    for (int64_t i = 0; i < n; i++) mx = std::max(mx, f.ax[i]);
    if (mx > 17) return bfail(b, 11, "family %d: a code is not an RNA digital code", k);
    h.N = f.N; h.L = f.L;
    h.nT = (f.L + TP - 1) / TP; h.Lp = h.nT * TP; h.ntiles = h.nT * (h.nT + 1) / 2;
    h.ns = rs_nshuffle(p, f.N, f.L, &h.fracfit);
    if (f.N > 1 && h.ns < 1) return bfail(b, 11, "family %d: at least one null alignment is needed", k);
    h.nslots = h.ns + 1;
    h.Npad = (f.N + 63) / 64 * 64;
    h.Lw = (f.L + 3) / 4;
    h.tens = p->counter == COVGPU_COUNT_TENSOR && f.N >= b->simt_below;
    h.gsc = !f.wgt && f.N <= 1000 && f.N > 1;
    h.pb = !f.wgt && f.N > 1000;
    if (h.gsc && f.N > 4096) return bfail(b, 11, "family %d: GSC weights in a batch are for up to 4096 sequences", k);
    int s;
    if ((s = plan_tree(b, f, h))) return s;
  }
  // chunks: families sorted by padded N, cut at the device budget; chunk
  // k + 1's device passes are launched on the other slot before chunk k's
  // host phases run
  std::vector<int> ord(nfam);
  std::iota(ord.begin(), ord.end(), 0);
  std::stable_sort(ord.begin(), ord.end(), [&](int a, int c) { return all[a].Npad < all[c].Npad; });
  const bool rafs = !T.rafs_q.empty();
  int cur = 0, prev = -1;
  auto drain = [&]() {
    for (Slot& S : b->slot) { cudaStreamSynchronize(S.st); cudaStreamSynchronize(S.st2); }
  };
  size_t k = 0;
  while (k < ord.size()) {
    std::vector<FamHost> chunk;
    size_t bytes = 0;
    int pitch = 0;
    while (k < ord.size()) {
      const FamHost& f = all[ord[k]];
      const int pn = std::max(pitch, f.Npad);
      // operands of the families already in the chunk grow with the pitch
      size_t grown = bytes;
      const int pn2 = f.tens ? pn : pitch;
      if (pn2 != pitch)
        for (const auto& c : chunk) if (c.tens) grown += (size_t)4 * c.nslots * 4 * c.Lp * (pn2 - pitch) * 2;
      const size_t add = fam_bytes_hint(f, ntypes, T.need_u, rafs, f.tens ? pn2 : 0);
      if (!chunk.empty() && grown + add > b->budget) break;
      chunk.push_back(f);
      bytes = grown + add;
      pitch = pn2;
      k++;
    }
    int s = chunk_launch(b, b->slot[cur], p, fams_in, chunk, T);
    if (!s && prev >= 0) s = chunk_finish(b, b->slot[prev], p, T, covtypes, results, hits, hitcap);
    if (s) { drain(); return s; }
    b->nchunks++;
    prev = cur;
    cur ^= 1;
  }
  if (prev >= 0) {
    const int s = chunk_finish(b, b->slot[prev], p, T, covtypes, results, hits, hitcap);
    if (s) { drain(); return s; }
  }
  b->ms[2] = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return 0;
}

// the batch's count schedule: families of fewer than simt_below sequences
// are counted on the SIMT kernel when the tensor counter is asked for (the
// two give the same counts), and sb is the raster super-block of the tensor
// count's tile order
extern "C" int covgpu_batch_set_schedule(covgpu_batch* b, int simt_below, int sb) {
  int probe[1], nj = 0;
  if (!b || simt_below < 0 || covgpu_tile_order(1, sb, probe, nullptr, 0, &nj) != 0) return 11;
  b->simt_below = simt_below;
  b->sb = sb;
  return 0;
}

// Schedule autotuner of the batch: runs the caller's families once per
// (threshold, super-block) pair, each timed as the best of two calls after a
// warm-up call (host wall clock of the whole call), and keeps the fastest.
// ms[i * nsb + j] gets each time.
extern "C" int covgpu_batch_autotune(covgpu_batch* b, const covgpu_params* p, int nfam, const covgpu_family* fams,
                                     int ntypes, const int* covtypes, int nthr, const int* thr, int nsb,
                                     const int* sbs, double* ms, int* best_thr, int* best_sb) {
  if (!b) return 11;
  if (nthr < 1 || nsb < 1 || !thr || !sbs || nfam < 1) return bfail(b, 11, "bad autotune candidates");
  std::vector<covgpu_result> res((size_t)nfam * std::max(ntypes, 1));
  const int keep_thr = b->simt_below, keep_sb = b->sb;
  double best = INFINITY;
  int bt = keep_thr, bs = keep_sb;
  for (int i = 0; i < nthr; i++)
    for (int j = 0; j < nsb; j++) {
      int probe[1], nj = 0;
      if (thr[i] < 0 || covgpu_tile_order(1, sbs[j], probe, nullptr, 0, &nj) != 0) {
        b->simt_below = keep_thr; b->sb = keep_sb;
        return bfail(b, 11, "bad autotune candidate (%d, %d)", thr[i], sbs[j]);
      }
      b->simt_below = thr[i];
      b->sb = sbs[j];
      double t = INFINITY;
      for (int r = 0; r < 3; r++) {
        const int s = covgpu_rscape_families(b, p, nfam, fams, ntypes, covtypes, res.data(), nullptr, 0);
        if (s) { b->simt_below = keep_thr; b->sb = keep_sb; return s; }
        if (r) t = std::min(t, b->ms[2]);
      }
      if (ms) ms[(size_t)i * nsb + j] = t;
      if (t < best) { best = t; bt = thr[i]; bs = sbs[j]; }
    }
  b->simt_below = bt;
  b->sb = bs;
  if (best_thr) *best_thr = bt;
  if (best_sb) *best_sb = bs;
  return 0;
}
