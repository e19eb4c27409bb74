// cov_prep.cu -- alignment preparation on the device: sequence weights and
// the gap-column filter of an alignment already resident in a context slot.
//
//   k_pb_colinv   one thread per column: counts of the canonical residues
//                 and of the residue types; inv[c][x] = 1/(types * count_x)
//   k_pb_rows     one CTA per sequence: w_s = sum_c inv[c][a_sc] over its
//                 canonical residues (fixed-order block reduction)
//                 -- position-based weights, Henikoff & Henikoff 1994
//                 (esl_msaweight_PB, called at src/R-scape.c:1556 for
//                 nseq > 1000), renormalised to sum to N on the host
//   k_gapfilter   one thread per column: the weighted fraction of residues
//                 (ACGU and degenerate codes) among residues and gaps ('-',
//                 '*'; '~' is skipped) against 1 - gapthresh
//                 (msamanip_RemoveGapColumns, src/msamanip.c:461-501)
//   GSC weights   (Gerstein, Sonnhammer & Chothia 1994; esl_msaweight_GSC,
//                 called at src/R-scape.c:1555 for nseq <= 1000):
//     k_gsc_codes  residue codes with non-residues masked to values that
//                  match nothing (0xFE in the row role, 0xFF in the column
//                  role), and the residue count of every sequence
//     k_gsc_ident  32 x 32 tiles of sequence pairs: identities counted four
//                  columns at a time (__vcmpeq4) from shared-memory tiles;
//                  D = 1 - identities / min(len_a, len_b)
//     k_gsc_scan   UPGMA step 1: the closest pair of live clusters, ties to
//                  the first pair in row-major order (a < b), per block
//     k_gsc_merge  UPGMA step 2 (one CTA): the pair; each side's new branch
//                  shared among its leaves in proportion to their weights
//                  (equally while those are 0); size-weighted average
//                  distances of the merged cluster (FP64 without
//                  contraction, the operations of the definition)
//     k_gsc_upgma_grid  all merges in one cooperative launch over the SMs,
//                  one grid barrier per merge (bounded wait), cached row
//                  minima, FP64 work spread over every SM
//     k_gsc_upgma  all merges in one CTA with cached row minima (where a
//                  cooperative launch is not available); the two kernels
//                  above for sizes beyond shared memory
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "cov_dev.cuh"
#include "cov_prep.h"
#include "cov_batch.h"

namespace covgpu {

__device__ __forceinline__ void pb_colinv_body(
    const GridIdx g, const uint8_t* __restrict__ ax, int N, int L, int Lp, double* __restrict__ inv) {
  const int c = g.x * blockDim.x + threadIdx.x;
  if (c >= L) return;
  int cnt[4] = {0, 0, 0, 0};
  for (int s = 0; s < N; s++) {
    const int x = ax[(int64_t)s * Lp + c];
    if (x < 4) cnt[x]++;
  }
  const int types = (cnt[0] > 0) + (cnt[1] > 0) + (cnt[2] > 0) + (cnt[3] > 0);
#pragma unroll
  for (int x = 0; x < 4; x++)
    inv[(int64_t)c * 4 + x] = (types > 0 && cnt[x] > 0) ? 1.0 / ((double)types * (double)cnt[x]) : 0.0;
}
__global__ void __launch_bounds__(256)
k_pb_colinv(const uint8_t* __restrict__ ax, int N, int L, int Lp, double* __restrict__ inv) {
  pb_colinv_body(native_grid(), ax, N, L, Lp, inv);
}

__device__ __forceinline__ void pb_rows_body(
    const GridIdx g, const uint8_t* __restrict__ ax, int L, int Lp, const double* __restrict__ inv,
    double* __restrict__ w) {
  __shared__ double red[8];
  const int s = g.x;
  const uint8_t* row = ax + (int64_t)s * Lp;
  double acc = 0.0;
  for (int c = threadIdx.x; c < L; c += blockDim.x) {
    const int x = row[c];
    if (x < 4) acc += inv[(int64_t)c * 4 + x];
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int i = 0; i < (int)(blockDim.x >> 5); i++) t += red[i];
    w[s] = t;
  }
}
__global__ void __launch_bounds__(256)
k_pb_rows(const uint8_t* __restrict__ ax, int L, int Lp, const double* __restrict__ inv, double* __restrict__ w) {
  pb_rows_body(native_grid(), ax, L, Lp, inv, w);
}

__global__ void __launch_bounds__(256)
k_gapfilter(const uint8_t* __restrict__ ax, const double* __restrict__ wgt, int N, int L, int Lp, double idthresh,
            int* __restrict__ useme) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= L) return;
  double r = 0.0, tot = 0.0;
  for (int s = 0; s < N; s++) {
    const int x = ax[(int64_t)s * Lp + c];
    const double w = wgt ? wgt[s] : 1.0;
    if (x < 4 || (x > 4 && x <= 15)) { r += w; tot += w; }
    else if (x == 4 || x == 16) tot += w;
  }
  useme[c] = (r > 0.0 && r / tot >= idthresh) ? 1 : 0;
}

__device__ __forceinline__ void gsc_codes_body(
    const GridIdx g, const uint8_t* __restrict__ ax, int N, int L, int Lp, int Lw, uint32_t* __restrict__ ra,
            uint32_t* __restrict__ rb, int* __restrict__ len) {
  __shared__ int red[8];
  const int s = g.x;
  int n = 0;
  for (int w = threadIdx.x; w < Lw; w += blockDim.x) {
    uint32_t va = 0, vb = 0;
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const int c = 4 * w + k;
      const int x = (c < L) ? ax[(int64_t)s * Lp + c] : 4;
      const bool res = (x < 4) || (x > 4 && x <= 15);
      n += res;
      va |= (uint32_t)(res ? x : 0xFE) << (8 * k);
      vb |= (uint32_t)(res ? x : 0xFF) << (8 * k);
    }
    ra[(int64_t)s * Lw + w] = va;
    rb[(int64_t)s * Lw + w] = vb;
  }
  for (int o = 16; o > 0; o >>= 1) n += __shfl_xor_sync(0xffffffffu, n, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = n;
  __syncthreads();
  if (threadIdx.x == 0) {
    int t = 0;
    for (int i = 0; i < (int)(blockDim.x >> 5); i++) t += red[i];
    len[s] = t;
  }
}
__global__ void __launch_bounds__(256)
k_gsc_codes(const uint8_t* __restrict__ ax, int N, int L, int Lp, int Lw, uint32_t* __restrict__ ra,
            uint32_t* __restrict__ rb, int* __restrict__ len) {
  gsc_codes_body(native_grid(), ax, N, L, Lp, Lw, ra, rb, len);
}

// D[a][b] for the 32 x 32 tile (g.y, g.x), a < b
__device__ __forceinline__ void gsc_ident_body(
    const GridIdx g, const uint32_t* __restrict__ ra, const uint32_t* __restrict__ rb, const int* __restrict__ len,
    int N, int Lw, double* __restrict__ D) {
  __shared__ uint32_t sa[32][33], sb[32][33];
  const int A0 = g.y * 32, B0 = g.x * 32;
  if (B0 + 31 < A0) return;   // tile entirely below the diagonal
  const int tid = threadIdx.x, ty = tid >> 5, tx = tid & 31;
  int cnt[4] = {0, 0, 0, 0};
  for (int w0 = 0; w0 < Lw; w0 += 32) {
    for (int e = tid; e < 32 * 32; e += 256) {
      const int r = e >> 5, k = e & 31;
      const int a = A0 + r, b = B0 + r, w = w0 + k;
      sa[r][k] = (a < N && w < Lw) ? ra[(int64_t)a * Lw + w] : 0xFEFEFEFEu;
      sb[r][k] = (b < N && w < Lw) ? rb[(int64_t)b * Lw + w] : 0xFFFFFFFFu;
    }
    __syncthreads();
#pragma unroll 4
    for (int k = 0; k < 32; k++) {
      const uint32_t y = sb[tx][k];
#pragma unroll
      for (int q = 0; q < 4; q++) cnt[q] += __popc(__vcmpeq4(sa[ty + 8 * q][k], y)) >> 3;
    }
    __syncthreads();
  }
#pragma unroll
  for (int q = 0; q < 4; q++) {
    const int a = A0 + ty + 8 * q, b = B0 + tx;
    if (a < N && b < N && a < b) {
      const int mn = min(len[a], len[b]);
      const double d = (mn == 0) ? 1.0 : 1.0 - (double)cnt[q] / (double)mn;
      D[(int64_t)a * N + b] = d;
      D[(int64_t)b * N + a] = d;
    }
  }
}
__global__ void __launch_bounds__(256)
k_gsc_ident(const uint32_t* __restrict__ ra, const uint32_t* __restrict__ rb, const int* __restrict__ len, int N,
            int Lw, double* __restrict__ D) {
  gsc_ident_body(native_grid(), ra, rb, len, N, Lw, D);
}

struct GscBest { double d; int a, b; };

__device__ __forceinline__ bool gsc_better(double d, int a, int b, double d2, int a2, int b2) {
  return d < d2 || (d == d2 && (a < a2 || (a == a2 && b < b2)));
}

// per block: the best live pair (a < b) among rows a = warp id, strided
__global__ void __launch_bounds__(256)
k_gsc_scan(const double* __restrict__ D, const int* __restrict__ alive, int N, GscBest* __restrict__ part) {
  __shared__ GscBest wb[8];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int gw = blockIdx.x * 8 + warp, nw = gridDim.x * 8;
  double bd = INFINITY;
  int ba = N, bb = N;
  for (int a = gw; a < N; a += nw) {
    if (!alive[a]) continue;
    for (int b = a + 1 + lane; b < N; b += 32) {
      if (!alive[b]) continue;
      const double d = D[(int64_t)a * N + b];
      if (gsc_better(d, a, b, bd, ba, bb)) { bd = d; ba = a; bb = b; }
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    const double d2 = __shfl_xor_sync(0xffffffffu, bd, o);
    const int a2 = __shfl_xor_sync(0xffffffffu, ba, o), b2 = __shfl_xor_sync(0xffffffffu, bb, o);
    if (gsc_better(d2, a2, b2, bd, ba, bb)) { bd = d2; ba = a2; bb = b2; }
  }
  if (lane == 0) wb[warp] = GscBest{bd, ba, bb};
  __syncthreads();
  if (threadIdx.x == 0) {
    GscBest r = wb[0];
    for (int w = 1; w < 8; w++)
      if (gsc_better(wb[w].d, wb[w].a, wb[w].b, r.d, r.a, r.b)) r = wb[w];
    part[blockIdx.x] = r;
  }
}

// one CTA of 1024 threads: the merge of the closest pair
__global__ void __launch_bounds__(1024)
k_gsc_merge(double* __restrict__ D, int* __restrict__ alive, int* __restrict__ size, double* __restrict__ height,
            int* __restrict__ cl, double* __restrict__ w, int N, const GscBest* __restrict__ part, int nparts) {
  __shared__ GscBest best;
  __shared__ double rtot[2][32];
  __shared__ int rcnt[2][32];
  __shared__ double tot[2];
  __shared__ int cnt[2];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) {
    GscBest r = part[0];
    for (int i = 1; i < nparts; i++)
      if (gsc_better(part[i].d, part[i].a, part[i].b, r.d, r.a, r.b)) r = part[i];
    best = r;
  }
  __syncthreads();
  const int ba = best.a, bb = best.b;
  if (ba >= N || bb >= N) return;   // one cluster left
  const double h = best.d / 2.0;
  // the leaves of each side: their weight sums and counts
  double ta = 0.0, tb = 0.0;
  int ca = 0, cb = 0;
  for (int l = tid; l < N; l += blockDim.x) {
    if (cl[l] == ba) { ta += w[l]; ca++; }
    else if (cl[l] == bb) { tb += w[l]; cb++; }
  }
  for (int o = 16; o > 0; o >>= 1) {
    ta += __shfl_xor_sync(0xffffffffu, ta, o); tb += __shfl_xor_sync(0xffffffffu, tb, o);
    ca += __shfl_xor_sync(0xffffffffu, ca, o); cb += __shfl_xor_sync(0xffffffffu, cb, o);
  }
  if (lane == 0) { rtot[0][warp] = ta; rtot[1][warp] = tb; rcnt[0][warp] = ca; rcnt[1][warp] = cb; }
  __syncthreads();
  if (tid == 0) {
    double x = 0.0, y = 0.0;
    int m = 0, n = 0;
    for (int i = 0; i < (int)(blockDim.x >> 5); i++) { x += rtot[0][i]; y += rtot[1][i]; m += rcnt[0][i]; n += rcnt[1][i]; }
    tot[0] = x; tot[1] = y; cnt[0] = m; cnt[1] = n;
  }
  __syncthreads();
  double bla = h - height[ba], blb = h - height[bb];
  if (bla < 0.0) bla = 0.0;
  if (blb < 0.0) blb = 0.0;
  const int sa = size[ba], sb = size[bb];
  for (int l = tid; l < N; l += blockDim.x) {
    if (cl[l] == ba) w[l] += (tot[0] > 0.0) ? __ddiv_rn(__dmul_rn(bla, w[l]), tot[0]) : bla / (double)cnt[0];
    else if (cl[l] == bb) w[l] += (tot[1] > 0.0) ? __ddiv_rn(__dmul_rn(blb, w[l]), tot[1]) : blb / (double)cnt[1];
  }
  for (int c = tid; c < N; c += blockDim.x) {
    if (alive[c] && c != ba && c != bb) {
      const double d = __ddiv_rn(__dadd_rn(__dmul_rn(D[(int64_t)ba * N + c], (double)sa),
                                           __dmul_rn(D[(int64_t)bb * N + c], (double)sb)),
                                 (double)(sa + sb));
      D[(int64_t)ba * N + c] = d;
      D[(int64_t)c * N + ba] = d;
    }
  }
  __syncthreads();
  for (int l = tid; l < N; l += blockDim.x)
    if (cl[l] == bb) cl[l] = ba;
  if (tid == 0) { size[ba] = sa + sb; height[ba] = h; alive[bb] = 0; }
}

// Order key of a distance: distances lie in [0, 1] (or +inf), and for
// non-negative doubles the IEEE bit patterns order as the values, so the
// searches compare 64-bit integers (GB300's FP64 pipe is 1/64 of FP32, its
// compares included); NaN and negative values map past every distance.
__device__ __forceinline__ unsigned long long dkey(double d) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(d);
  return (u <= 0x7FF0000000000000ull) ? u : ~0ull;
}
struct GscKey { unsigned long long k; int a, b; };
__device__ __forceinline__ bool key_better(unsigned long long k, int a, int b, unsigned long long k2, int a2,
                                           int b2) {
  return k < k2 || (k == k2 && (a < a2 || (a == a2 && b < b2)));
}

// all N-1 UPGMA merges in one CTA of 1024 threads.  The clusters' state
// (liveness, sizes, heights, weight sums, leaf labels, weights) sits in
// shared memory,
// the distances in global memory (L2-resident).  Each live row a keeps its
// closest live column b > a (ties to the smaller b), so the closest pair is
// the best row minimum in (d, a, b) order -- the same pair as a full scan.
// A merge of (ba, bb) changes row ba, column ba of the rows above it and
// kills column bb; only rows whose cached minimum pointed at ba or bb, and
// row ba, are rescanned (one warp per row).  The weight split and the
// distance update are the FP64 operations of k_gsc_upgma_grid, and each
// cluster's weight sum is kept as that kernel keeps it ((ta + bla) + (tb +
// blb) at a merge), so both kernels give the same weights.
__device__ __forceinline__ void gsc_upgma_body(double* __restrict__ D, int N, double* __restrict__ w_out) {
  extern __shared__ __align__(16) unsigned char gsm[];
  unsigned long long* rkey = reinterpret_cast<unsigned long long*>(gsm);
  double* height = reinterpret_cast<double*>(rkey + N);
  double* w = height + N;
  double* cw = w + N;
  int* rarg = reinterpret_cast<int*>(cw + N);
  int* size = rarg + N;
  int* cl = size + N;
  int* resc = cl + N;
  unsigned char* alive = reinterpret_cast<unsigned char*>(resc + N);
  __shared__ GscKey wb[32];
  __shared__ GscKey best;
  __shared__ int nresc;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = blockDim.x >> 5;
  const unsigned long long NONE = ~0ull;
  for (int s = tid; s < N; s += blockDim.x) {
    alive[s] = 1; size[s] = 1; height[s] = 0.0; cl[s] = s; w[s] = 0.0; cw[s] = 0.0;
  }
  __syncthreads();
  // the best live column b > a of row a (warp-wide; 8 loads in flight per
  // lane, the row comes from L2), into rkey/rarg
  auto scan_row = [&](int a) {
    unsigned long long bk = NONE;
    int bb2 = N;
    const double* row = D + (int64_t)a * N;
    for (int b0 = a + 1 + lane; b0 < N; b0 += 32 * 8) {
      unsigned long long v[8];
#pragma unroll
      for (int u = 0; u < 8; u++) {
        const int b = b0 + 32 * u;
        v[u] = (b < N && alive[b]) ? dkey(row[b]) : NONE;
      }
#pragma unroll
      for (int u = 0; u < 8; u++) {
        const int b = b0 + 32 * u;
        if (v[u] < bk || (v[u] == bk && v[u] != NONE && b < bb2)) { bk = v[u]; bb2 = b; }
      }
    }
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long k2 = __shfl_xor_sync(0xffffffffu, bk, o);
      const int b2 = __shfl_xor_sync(0xffffffffu, bb2, o);
      if (k2 < bk || (k2 == bk && b2 < bb2)) { bk = k2; bb2 = b2; }
    }
    if (lane == 0) { rkey[a] = bk; rarg[a] = (bk == NONE) ? N : bb2; }
  };
  for (int a = warp; a < N; a += nwarps) scan_row(a);
  __syncthreads();
  for (int m = 0; m < N - 1; m++) {
    // the closest pair
    GscKey r{NONE, N, N};
    for (int a = tid; a < N; a += blockDim.x)
      if (alive[a] && rkey[a] != NONE && key_better(rkey[a], a, rarg[a], r.k, r.a, r.b)) r = GscKey{rkey[a], a, rarg[a]};
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long k2 = __shfl_xor_sync(0xffffffffu, r.k, o);
      const int a2 = __shfl_xor_sync(0xffffffffu, r.a, o), b2 = __shfl_xor_sync(0xffffffffu, r.b, o);
      if (key_better(k2, a2, b2, r.k, r.a, r.b)) { r.k = k2; r.a = a2; r.b = b2; }
    }
    if (lane == 0) wb[warp] = r;
    __syncthreads();
    if (tid == 0) {
      GscKey q = wb[0];
      for (int i = 1; i < nwarps; i++)
        if (key_better(wb[i].k, wb[i].a, wb[i].b, q.k, q.a, q.b)) q = wb[i];
      best = q;
      nresc = 0;
    }
    __syncthreads();
    const int ba = best.a, bb = best.b;
    if (best.k == NONE || ba >= N || bb >= N) break;   // no pair left with a distance
    const double h = __longlong_as_double((long long)best.k) / 2.0;
    // the leaves of each side share the side's new branch in proportion to
    // their weights (equally while the side's weight sum is 0)
    const double ta = cw[ba], tb = cw[bb];
    double bla = h - height[ba], blb = h - height[bb];
    if (bla < 0.0) bla = 0.0;
    if (blb < 0.0) blb = 0.0;
    const int sa = size[ba], sb = size[bb];
    for (int l = tid; l < N; l += blockDim.x) {
      if (cl[l] == ba) w[l] += (ta > 0.0) ? __ddiv_rn(__dmul_rn(bla, w[l]), ta) : bla / (double)sa;
      else if (cl[l] == bb) w[l] += (tb > 0.0) ? __ddiv_rn(__dmul_rn(blb, w[l]), tb) : blb / (double)sb;
    }
    for (int c = tid; c < N; c += blockDim.x) {
      if (alive[c] && c != ba && c != bb) {
        const double d = __ddiv_rn(__dadd_rn(__dmul_rn(D[(int64_t)ba * N + c], (double)sa),
                                             __dmul_rn(D[(int64_t)bb * N + c], (double)sb)),
                                   (double)(sa + sb));
        D[(int64_t)ba * N + c] = d;
        D[(int64_t)c * N + ba] = d;
        if (c < ba) {            // column ba of row c changed, column bb dies
          const unsigned long long kd = dkey(d);
          if (kd != NONE && (kd < rkey[c] || (kd == rkey[c] && ba < rarg[c]))) { rkey[c] = kd; rarg[c] = ba; }
          else if (rarg[c] == ba || rarg[c] == bb) resc[atomicAdd(&nresc, 1)] = c;
        } else if (c < bb && rarg[c] == bb) {
          resc[atomicAdd(&nresc, 1)] = c;
        }
      }
    }
    __syncthreads();
    for (int l = tid; l < N; l += blockDim.x)
      if (cl[l] == bb) cl[l] = ba;
    if (tid == 0) {
      size[ba] = sa + sb; height[ba] = h; cw[ba] = (ta + bla) + (tb + blb); alive[bb] = 0;
      resc[atomicAdd(&nresc, 1)] = ba;
    }
    __syncthreads();
    for (int k = warp; k < nresc; k += nwarps) scan_row(resc[k]);
    __syncthreads();
  }
  for (int s = tid; s < N; s += blockDim.x) w_out[s] = w[s];
}
__global__ void __launch_bounds__(1024)
k_gsc_upgma(double* __restrict__ D, int N, double* __restrict__ w_out) {
  gsc_upgma_body(D, N, w_out);
}

// ------------------------------------------------------------------------
// UPGMA across the grid: one cooperative launch, one grid barrier per merge.
// Index i (row, column, leaf) belongs to block i % G.  Every block keeps a
// private copy of the clusters' state (liveness, size, height, weight sum)
// and updates it identically; each block caches the minima of its own rows
// and rescans the ones a merge invalidated (their entries were written by the
// block itself or before the last barrier).  The merged row's new minimum is
// not rescanned: every block offers its best new entry of that row with its
// next partial, and the reduction after the barrier yields both the row's
// minimum and the next closest pair.  FP64 work (the size-weighted distances
// and the weight split) is spread over every SM.
// ------------------------------------------------------------------------
struct __align__(16) GscPart { unsigned long long k; int a, b; unsigned long long ck; int cb, pad; };

__device__ __forceinline__ unsigned gsc_ld_acquire(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ uint64_t gsc_clock() {
  uint64_t t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}
constexpr uint64_t kGscWaitNs = 2000000000ull;   // a grid barrier gives up after 2 s

__global__ void __launch_bounds__(256)
k_gsc_upgma_grid(double* __restrict__ D, int N, double* __restrict__ w, int* __restrict__ cl,
                 GscPart* __restrict__ part, unsigned* __restrict__ bar, int* __restrict__ err) {
  extern __shared__ __align__(16) unsigned char gsm2[];
  const int G = gridDim.x, bid = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nwarps = blockDim.x >> 5;
  const int nown = (N - bid + G - 1) / G;           // rows/columns/leaves bid, bid + G, ...
  double* height = reinterpret_cast<double*>(gsm2);
  double* cw = height + N;
  unsigned long long* rkey = reinterpret_cast<unsigned long long*>(cw + N);   // own rows
  int* size = reinterpret_cast<int*>(rkey + nown);
  int* rarg = size + N;                              // own rows
  int* resc = rarg + nown;                           // own rows to rescan
  unsigned char* alive = reinterpret_cast<unsigned char*>(resc + nown);
  __shared__ GscPart wpart[8];
  __shared__ unsigned long long sk[2];
  __shared__ int si[4];
  __shared__ int nresc, ok;
  const unsigned long long NONE = ~0ull;
  for (int s = tid; s < N; s += blockDim.x) { alive[s] = 1; size[s] = 1; height[s] = 0.0; cw[s] = 0.0; }
  for (int r = tid; r < nown; r += blockDim.x) { const int l = bid + r * G; cl[l] = l; w[l] = 0.0; }
  __syncthreads();
  // the best live column b > a of row a, warp-wide
  auto scan_row = [&](int a, int r) {
    unsigned long long bk = NONE;
    int bb2 = N;
    const double* row = D + (int64_t)a * N;
    for (int b0 = a + 1 + lane; b0 < N; b0 += 32 * 8) {
      unsigned long long v[8];
#pragma unroll
      for (int u = 0; u < 8; u++) {
        const int b = b0 + 32 * u;
        v[u] = (b < N && alive[b]) ? dkey(__ldcg(row + b)) : NONE;
      }
#pragma unroll
      for (int u = 0; u < 8; u++) {
        const int b = b0 + 32 * u;
        if (v[u] < bk || (v[u] == bk && v[u] != NONE && b < bb2)) { bk = v[u]; bb2 = b; }
      }
    }
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long k2 = __shfl_xor_sync(0xffffffffu, bk, o);
      const int b2 = __shfl_xor_sync(0xffffffffu, bb2, o);
      if (k2 < bk || (k2 == bk && b2 < bb2)) { bk = k2; bb2 = b2; }
    }
    if (lane == 0) { rkey[r] = bk; rarg[r] = (bk == NONE) ? N : bb2; }
  };
  for (int r = warp; r < nown; r += nwarps) scan_row(bid + r * G, r);
  __syncthreads();
  int prev = -1;                          // merged row whose minimum comes from the partials
  unsigned long long ck = NONE;           // this block's best new entry of row prev
  int cb = N;
  for (int m = 0; m < N - 1; m++) {
    // phase 1: the best cached minimum over own live rows (row prev excluded)
    GscPart q{NONE, N, N, ck, cb, 0};
    for (int r = tid; r < nown; r += blockDim.x) {
      const int a = bid + r * G;
      if (a != prev && alive[a] && rkey[r] != NONE && key_better(rkey[r], a, rarg[r], q.k, q.a, q.b)) {
        q.k = rkey[r]; q.a = a; q.b = rarg[r];
      }
    }
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long k2 = __shfl_xor_sync(0xffffffffu, q.k, o);
      const int a2 = __shfl_xor_sync(0xffffffffu, q.a, o), b2 = __shfl_xor_sync(0xffffffffu, q.b, o);
      if (key_better(k2, a2, b2, q.k, q.a, q.b)) { q.k = k2; q.a = a2; q.b = b2; }
    }
    if (lane == 0) wpart[warp] = q;
    __syncthreads();
    GscPart* pp = part + (size_t)(m & 1) * G;
    if (tid == 0) {
      GscPart r0 = wpart[0];
      for (int i = 1; i < nwarps; i++)
        if (key_better(wpart[i].k, wpart[i].a, wpart[i].b, r0.k, r0.a, r0.b)) {
          r0.k = wpart[i].k; r0.a = wpart[i].a; r0.b = wpart[i].b;
        }
      r0.ck = ck; r0.cb = cb;
      pp[bid] = r0;
      __threadfence();
      atomicAdd(bar, 1u);
      const unsigned target = (unsigned)(m + 1) * (unsigned)G;
      uint64_t t0 = 0;
      int good = 1;
      while (gsc_ld_acquire(bar) < target) {
        const uint64_t now = gsc_clock();
        if (t0 == 0) t0 = now;
        else if (now - t0 > kGscWaitNs) { good = 0; break; }
      }
      ok = good;
    }
    __syncthreads();
    if (!ok) { if (tid == 0) atomicExch(err, 1); return; }
    // phase 2: every block reduces all partials in block order
    if (warp == 0) {
      unsigned long long bk = NONE, pk = NONE;
      int ba = N, bb = N, pb = N;
      for (int i = lane; i < G; i += 32) {   // written by other SMs: read past L1, 32 bytes in two loads
        const int4 x = __ldcg(reinterpret_cast<const int4*>(pp + i));
        const int4 y = __ldcg(reinterpret_cast<const int4*>(pp + i) + 1);
        const unsigned long long vk = ((unsigned long long)(unsigned)x.y << 32) | (unsigned)x.x;
        const unsigned long long vck = ((unsigned long long)(unsigned)y.y << 32) | (unsigned)y.x;
        const int va = x.z, vb = x.w, vcb = y.z;
        if (key_better(vk, va, vb, bk, ba, bb)) { bk = vk; ba = va; bb = vb; }
        if (vck < pk || (vck == pk && vck != NONE && vcb < pb)) { pk = vck; pb = vcb; }
      }
      for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long k2 = __shfl_xor_sync(0xffffffffu, bk, o);
        const int a2 = __shfl_xor_sync(0xffffffffu, ba, o), b2 = __shfl_xor_sync(0xffffffffu, bb, o);
        if (key_better(k2, a2, b2, bk, ba, bb)) { bk = k2; ba = a2; bb = b2; }
        const unsigned long long p2 = __shfl_xor_sync(0xffffffffu, pk, o);
        const int c2 = __shfl_xor_sync(0xffffffffu, pb, o);
        if (p2 < pk || (p2 == pk && c2 < pb)) { pk = p2; pb = c2; }
      }
      if (lane == 0) {
        if (prev >= 0 && pk != NONE && key_better(pk, prev, pb, bk, ba, bb)) { bk = pk; ba = prev; bb = pb; }
        sk[0] = bk; sk[1] = pk; si[0] = ba; si[1] = bb; si[2] = pb;
      }
    }
    __syncthreads();
    if (prev >= 0 && prev % G == bid && tid == 0) {
      const int r = prev / G;
      rkey[r] = sk[1]; rarg[r] = (sk[1] == NONE) ? N : si[2];
    }
    const unsigned long long bk = sk[0];
    const int ba = si[0], bb = si[1];
    if (bk == NONE || ba >= N || bb >= N) break;   // uniform: no pair left
    const double h = __longlong_as_double((long long)bk) / 2.0;
    const int sa = size[ba], sb = size[bb];
    const double ta = cw[ba], tb = cw[bb];
    double bla = h - height[ba], blb = h - height[bb];
    if (bla < 0.0) bla = 0.0;
    if (blb < 0.0) blb = 0.0;
    if (tid == 0) nresc = 0;
    __syncthreads();
    // own leaves: the branch shares, then the new label
    for (int r = tid; r < nown; r += blockDim.x) {
      const int l = bid + r * G;
      const int c = cl[l];
      if (c == ba) {
        w[l] += (ta > 0.0) ? __ddiv_rn(__dmul_rn(bla, w[l]), ta) : bla / (double)sa;
      } else if (c == bb) {
        w[l] += (tb > 0.0) ? __ddiv_rn(__dmul_rn(blb, w[l]), tb) : blb / (double)sb;
        cl[l] = ba;
      }
    }
    // own columns: the merged cluster's distances, the cached minima of own
    // rows, and this block's best new entry of row ba
    unsigned long long myk = NONE;
    int myb = N;
    for (int r = tid; r < nown; r += blockDim.x) {
      const int c = bid + r * G;
      if (!alive[c] || c == ba || c == bb) continue;
      const double d = __ddiv_rn(__dadd_rn(__dmul_rn(__ldcg(D + (int64_t)ba * N + c), (double)sa),
                                           __dmul_rn(__ldcg(D + (int64_t)bb * N + c), (double)sb)),
                                 (double)(sa + sb));
      D[(int64_t)ba * N + c] = d;
      D[(int64_t)c * N + ba] = d;
      const unsigned long long kd = dkey(d);
      if (c > ba) {
        if (kd < myk || (kd == myk && kd != NONE && c < myb)) { myk = kd; myb = c; }
      } else {            // row c, column ba changed, column bb dies
        if (kd != NONE && (kd < rkey[r] || (kd == rkey[r] && ba < rarg[r]))) { rkey[r] = kd; rarg[r] = ba; }
        else if (rarg[r] == ba || rarg[r] == bb) resc[atomicAdd(&nresc, 1)] = r;
      }
      if (c > ba && c < bb && rarg[r] == bb) resc[atomicAdd(&nresc, 1)] = r;
    }
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long k2 = __shfl_xor_sync(0xffffffffu, myk, o);
      const int b2 = __shfl_xor_sync(0xffffffffu, myb, o);
      if (k2 < myk || (k2 == myk && b2 < myb)) { myk = k2; myb = b2; }
    }
    if (lane == 0) { wpart[warp].ck = myk; wpart[warp].cb = myb; }
    __syncthreads();
    // the private cluster state, identical in every block
    if (tid == 0) {
      size[ba] = sa + sb; height[ba] = h; cw[ba] = (ta + bla) + (tb + blb); alive[bb] = 0;
      ck = NONE; cb = N;
      for (int i = 0; i < nwarps; i++)
        if (wpart[i].ck < ck || (wpart[i].ck == ck && wpart[i].ck != NONE && wpart[i].cb < cb)) {
          ck = wpart[i].ck; cb = wpart[i].cb;
        }
      si[3] = cb; sk[1] = ck;
    }
    __syncthreads();
    ck = sk[1]; cb = si[3];
    // rescans of own rows whose minimum was lost (their entries are this
    // block's own writes or older than the last barrier)
    for (int k = warp; k < nresc; k += nwarps) { const int r = resc[k]; scan_row(bid + r * G, r); }
    prev = ba;
    __syncthreads();
  }
}

static size_t gsc_grid_smem(int N, int G) {
  const int nown = (N + G - 1) / G;
  return (size_t)N * (2 * sizeof(double) + sizeof(int) + 1) + (size_t)nown * (sizeof(unsigned long long) +
         2 * sizeof(int)) + 16;
}

// shared memory of k_gsc_upgma for N sequences
static size_t gsc_upgma_smem(int N) { return (size_t)N * (4 * sizeof(double) + 4 * sizeof(int) + 1) + 16; }

__global__ void k_gsc_init(int N, int* __restrict__ alive, int* __restrict__ size, double* __restrict__ height,
                           int* __restrict__ cl, double* __restrict__ w) {
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < N; s += gridDim.x * blockDim.x) {
    alive[s] = 1; size[s] = 1; height[s] = 0.0; cl[s] = s; w[s] = 0.0;
  }
}

constexpr int kGscMaxGrid = 256;
constexpr size_t kGscHead = 16 + 2 * kGscMaxGrid * sizeof(GscPart);   // barrier, error flag, partials

size_t gsc_scratch_bytes(int N, int L) {
  const size_t Lw = ((size_t)L + 3) / 4;
  return kGscHead + (size_t)N * N * sizeof(double) + 2 * (size_t)N * Lw * sizeof(uint32_t) +
         (size_t)N * (4 * sizeof(int) + 2 * sizeof(double)) + 64 * sizeof(GscBest) + 256;
}

cudaError_t launch_weights_gsc(const uint8_t* ax, int N, int L, int Lp, void* scratch, double* w, cudaStream_t st) {
  const int Lw = (L + 3) / 4;
  uint8_t* p = (uint8_t*)scratch;
  unsigned* bar = (unsigned*)p;
  int* err = (int*)(p + 4);
  GscPart* gpart = (GscPart*)(p + 16);
  p += kGscHead;
  double* D = (double*)p;                 p += (size_t)N * N * sizeof(double);
  double* height = (double*)p;            p += (size_t)N * sizeof(double);
  uint32_t* ra = (uint32_t*)p;            p += (size_t)N * Lw * sizeof(uint32_t);
  uint32_t* rb = (uint32_t*)p;            p += (size_t)N * Lw * sizeof(uint32_t);
  int* len = (int*)p;                     p += (size_t)N * sizeof(int);
  int* alive = (int*)p;                   p += (size_t)N * sizeof(int);
  int* size = (int*)p;                    p += (size_t)N * sizeof(int);
  int* cl = (int*)p;                      p += (size_t)N * sizeof(int);
  p = (uint8_t*)(((uintptr_t)p + 15) & ~(uintptr_t)15);
  GscBest* part = (GscBest*)p;
  cudaError_t e = cudaMemsetAsync(scratch, 0, 16, st);
  if (e != cudaSuccess) return e;
  k_gsc_codes<<<N, 256, 0, st>>>(ax, N, L, Lp, Lw, ra, rb, len);
  const int nt = (N + 31) / 32;
  k_gsc_ident<<<dim3(nt, nt), 256, 0, st>>>(ra, rb, len, N, Lw, D);
  // all merges in one cooperative launch over the SMs (FP64 work spread out)
  int dev = 0, nsm = 1, coop = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
  // about 64 rows per block: the FP64 work of a merge stays small per SM and
  // the barrier and the reduction of the partials stay short
  const int G = std::max(1, std::min(std::min(nsm, 32), (N + 63) / 64));
  const size_t smg = gsc_grid_smem(N, G);
  // the launch limit of both merge kernels is raised once, to the 200 KB
  // that either may take: a limit set per call to that call's size would
  // race with other host threads' calls for other N (a launch above the
  // limit another thread just set fails with an invalid argument)
  static const cudaError_t attr = [] {
    cudaError_t r = cudaFuncSetAttribute(k_gsc_upgma_grid, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    if (r == cudaSuccess) r = cudaFuncSetAttribute(k_gsc_upgma, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    return r;
  }();
  if (attr != cudaSuccess) return attr;
  if (coop && N >= 2 && smg <= 200 * 1024) {
    int occ = 0;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_gsc_upgma_grid, 256, smg)) != cudaSuccess) return e;
    if (occ >= 1 && G <= occ * nsm) {
      int n = N;
      void* args[] = {(void*)&D, (void*)&n, (void*)&w, (void*)&cl, (void*)&gpart, (void*)&bar, (void*)&err};
      return cudaLaunchCooperativeKernel((const void*)k_gsc_upgma_grid, dim3(G), dim3(256), args, smg, st);
    }
  }
  // one CTA while the cluster state fits in its shared memory
  const size_t sm = gsc_upgma_smem(N);
  if (sm <= 200 * 1024) {
    k_gsc_upgma<<<1, 1024, sm, st>>>(D, N, w);
    return cudaGetLastError();
  }
  k_gsc_init<<<(N + 255) / 256, 256, 0, st>>>(N, alive, size, height, cl, w);
  const int Gs = std::min(48, std::max(1, (N + 7) / 8));
  for (int m = 0; m < N - 1; m++) {
    k_gsc_scan<<<Gs, 256, 0, st>>>(D, alive, N, part);
    k_gsc_merge<<<1, 1024, 0, st>>>(D, alive, size, height, cl, w, N, part, Gs);
  }
  return cudaGetLastError();
}

int gsc_error(const void* scratch, cudaStream_t st) {
  int err = 0;
  if (cudaMemcpyAsync(&err, (const uint8_t*)scratch + 4, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return 90;
  return err;
}

cudaError_t launch_weights_pb(const uint8_t* ax, int N, int L, int Lp, double* inv, double* w, cudaStream_t st) {
  k_pb_colinv<<<(L + 255) / 256, 256, 0, st>>>(ax, N, L, Lp, inv);
  k_pb_rows<<<N, 256, 0, st>>>(ax, L, Lp, inv, w);
  return cudaGetLastError();
}

cudaError_t launch_gapfilter(const uint8_t* ax, const double* wgt, int N, int L, int Lp, double gapthresh, int* useme,
                             cudaStream_t st) {
  k_gapfilter<<<(L + 255) / 256, 256, 0, st>>>(ax, wgt, N, L, Lp, 1.0 - gapthresh, useme);
  return cudaGetLastError();
}

// ------------------------------------------------------------------------
// grouped launches over a batch of families: position-based weights of the
// families with pb set, GSC weights (one CTA per family for the merges) of
// those with gsc set
// ------------------------------------------------------------------------
__global__ void __launch_bounds__(256)
k_pb_colinv_grp(const FamDev* __restrict__ F, int nf, const int* __restrict__ pre) {
  const int f = grp_find(pre, nf, (int)blockIdx.x);
  const FamDev& d = F[f];
  pb_colinv_body(GridIdx{(int)blockIdx.x - __ldg(pre + f), 0, (d.L + 255) / 256}, d.ax, d.N, d.L, d.Lp, d.pbinv);
}

__global__ void __launch_bounds__(256)
k_pb_rows_grp(const FamDev* __restrict__ F, int nf, const int* __restrict__ pre) {
  const int f = grp_find(pre, nf, (int)blockIdx.x);
  const FamDev& d = F[f];
  pb_rows_body(GridIdx{(int)blockIdx.x - __ldg(pre + f), 0, d.N}, d.ax, d.L, d.Lp, d.pbinv, d.w);
}

__global__ void __launch_bounds__(256)
k_gsc_codes_grp(const FamDev* __restrict__ F, int nf, const int* __restrict__ pre) {
  const int f = grp_find(pre, nf, (int)blockIdx.x);
  const FamDev& d = F[f];
  gsc_codes_body(GridIdx{(int)blockIdx.x - __ldg(pre + f), 0, d.N}, d.ax, d.N, d.L, d.Lp, d.Lw, d.gra, d.grb, d.glen);
}

__global__ void __launch_bounds__(256)
k_gsc_ident_grp(const FamDev* __restrict__ F, int nf, const int* __restrict__ pre) {
  const int f = grp_find(pre, nf, (int)blockIdx.x);
  const FamDev& d = F[f];
  const int nt = (d.N + 31) / 32, loc = (int)blockIdx.x - __ldg(pre + f);
  gsc_ident_body(GridIdx{loc % nt, loc / nt, nt}, d.gra, d.grb, d.glen, d.N, d.Lw, d.gD);
}

__global__ void __launch_bounds__(1024)
k_gsc_upgma_grp(const FamDev* __restrict__ F, int nf, const int* __restrict__ pre) {
  const int f = grp_find(pre, nf, (int)blockIdx.x);
  const FamDev& d = F[f];
  gsc_upgma_body(d.gD, d.N, d.w);
}

cudaError_t grp_weights_pb(const FamDev* F, int nf, const int* pre_col, int nb_col, const int* pre_row, int nb_row,
                           cudaStream_t st) {
  if (nb_col > 0) k_pb_colinv_grp<<<nb_col, 256, 0, st>>>(F, nf, pre_col);
  if (nb_row > 0) k_pb_rows_grp<<<nb_row, 256, 0, st>>>(F, nf, pre_row);
  return cudaGetLastError();
}

// maxN: the largest N among the GSC families (the merges' shared memory)
cudaError_t grp_weights_gsc(const FamDev* F, int nf, const int* pre_codes, int nb_codes, const int* pre_ident,
                            int nb_ident, const int* pre_upgma, int nb_upgma, int maxN, cudaStream_t st) {
  if (nb_upgma <= 0) return cudaSuccess;
  const size_t sm = gsc_upgma_smem(maxN);
  if (sm > 200 * 1024 || !grp_weights_gsc_prepare()) return cudaErrorInvalidValue;
  if (nb_codes > 0) k_gsc_codes_grp<<<nb_codes, 256, 0, st>>>(F, nf, pre_codes);
  if (nb_ident > 0) k_gsc_ident_grp<<<nb_ident, 256, 0, st>>>(F, nf, pre_ident);
  k_gsc_upgma_grp<<<nb_upgma, 1024, sm, st>>>(F, nf, pre_upgma);
  return cudaGetLastError();
}

// the device weights of each family of pre (one block each), made as the
// host makes a caller's weights: normalised to sum to N (the sum in sequence
// order), then quantised to three b-bit limbs as make_limbs does
// (cov_kernels.cu) in its general form -- normalised weights that are all
// equal are all 1.0, whose limbs give the same counts as the one-limb form.
// Writes the limbs (uint16 [3][Npad], zero-padded, and as floats [3][N]) and
// the family's limb base, scale and quantised total into F and U.
__global__ void __launch_bounds__(256)
k_weights_limbs_grp(FamDev* __restrict__ F, int nf, const int* __restrict__ pre, UmmaFam* __restrict__ U) {
  const int f = grp_find(pre, nf, (int)blockIdx.x);
  FamDev& d = F[f];
  const int N = d.N, tid = threadIdx.x;
  __shared__ double ssum, red[256];
  __shared__ unsigned long long tot;
  __shared__ int sE, sb;
  if (tid == 0) {
    double sum = 0.0;
    for (int i = 0; i < N; i++) sum = __dadd_rn(sum, d.w[i]);
    ssum = sum;
    tot = 0ull;
  }
  __syncthreads();
  const double sum = ssum;
  double wmax = 0.0;
  for (int i = tid; i < N; i += blockDim.x) {
    const double w = (sum > 0.0) ? __ddiv_rn(__dmul_rn(d.w[i], (double)N), sum) : 1.0;
    d.w[i] = w;
    wmax = fmax(wmax, w);
  }
  red[tid] = wmax;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (tid < o) red[tid] = fmax(red[tid], red[tid + o]);
    __syncthreads();
  }
  if (tid == 0) {
    int b = 11;
    while (b > 1 && (double)N * (double)((1 << b) - 1) >= 16777216.0) b--;
    int e2;
    frexp(red[0], &e2);
    sb = b;
    sE = 3 * b - e2;
  }
  __syncthreads();
  const int b = sb, E = sE;
  const double qmax = ldexp(1.0, 3 * b) - 1.0;
  const unsigned long long mask = (1ull << b) - 1ull;
  unsigned long long t = 0;
  for (int i = tid; i < d.Npad; i += blockDim.x) {
    unsigned long long q = 0;
    if (i < N) {
      double qd = rint(ldexp(d.w[i], E));
      if (qd > qmax) qd = qmax;
      q = (unsigned long long)qd;
    }
    const uint16_t l0 = (uint16_t)(q & mask), l1 = (uint16_t)((q >> b) & mask), l2 = (uint16_t)(q >> (2 * b));
    d.limbs[i] = l0;
    d.limbs[d.Npad + i] = l1;
    d.limbs[2 * d.Npad + i] = l2;
    if (i < N) {
      d.limbf[i] = (float)l0;
      d.limbf[N + i] = (float)l1;
      d.limbf[2 * N + i] = (float)l2;
    }
    t += q;
  }
  atomicAdd(&tot, t);
  __syncthreads();
  if (tid == 0) {
    const float B = (float)(1 << b), s_hi = (float)ldexp(1.0, -E);
    const double wq = ldexp((double)tot, -E);
    const float whi = (float)wq;
    d.nl = 3; d.B = B; d.s_hi = s_hi; d.s_lo = 0.f;
    d.sa.wtot = make_float2(whi, (float)(wq - (double)whi));
    U[f].B = B; U[f].s_hi = s_hi; U[f].s_lo = 0.f;
  }
}

cudaError_t grp_weights_limbs(FamDev* F, int nf, const int* pre, int nb, UmmaFam* U, cudaStream_t st) {
  if (nb > 0) k_weights_limbs_grp<<<nb, 256, 0, st>>>(F, nf, pre, U);
  return cudaGetLastError();
}

// the merges' shared-memory limit, raised once, outside any stream capture
int grp_weights_gsc_prepare() {
  static const int ok = [] {
    return cudaFuncSetAttribute(k_gsc_upgma_grp, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024) ==
                   cudaSuccess ? 1 : 0;
  }();
  return ok;
}

}  // namespace covgpu
