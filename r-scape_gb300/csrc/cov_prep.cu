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
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "cov_prep.h"

namespace covgpu {

__global__ void __launch_bounds__(256)
k_pb_colinv(const uint8_t* __restrict__ ax, int N, int L, int Lp, double* __restrict__ inv) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
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
k_pb_rows(const uint8_t* __restrict__ ax, int L, int Lp, const double* __restrict__ inv, double* __restrict__ w) {
  __shared__ double red[8];
  const int s = blockIdx.x;
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

__global__ void __launch_bounds__(256)
k_gsc_codes(const uint8_t* __restrict__ ax, int N, int L, int Lp, int Lw, uint32_t* __restrict__ ra,
            uint32_t* __restrict__ rb, int* __restrict__ len) {
  __shared__ int red[8];
  const int s = blockIdx.x;
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

// D[a][b] for the 32 x 32 tile (blockIdx.y, blockIdx.x), a < b
__global__ void __launch_bounds__(256)
k_gsc_ident(const uint32_t* __restrict__ ra, const uint32_t* __restrict__ rb, const int* __restrict__ len, int N,
            int Lw, double* __restrict__ D) {
  __shared__ uint32_t sa[32][33], sb[32][33];
  const int A0 = blockIdx.y * 32, B0 = blockIdx.x * 32;
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

__global__ void k_gsc_init(int N, int* __restrict__ alive, int* __restrict__ size, double* __restrict__ height,
                           int* __restrict__ cl, double* __restrict__ w) {
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < N; s += gridDim.x * blockDim.x) {
    alive[s] = 1; size[s] = 1; height[s] = 0.0; cl[s] = s; w[s] = 0.0;
  }
}

size_t gsc_scratch_bytes(int N, int L) {
  const size_t Lw = ((size_t)L + 3) / 4;
  return (size_t)N * N * sizeof(double) + 2 * (size_t)N * Lw * sizeof(uint32_t) + (size_t)N * (4 * sizeof(int) +
         2 * sizeof(double)) + 64 * sizeof(GscBest) + 256;
}

cudaError_t launch_weights_gsc(const uint8_t* ax, int N, int L, int Lp, void* scratch, double* w, cudaStream_t st) {
  const int Lw = (L + 3) / 4;
  uint8_t* p = (uint8_t*)scratch;
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
  k_gsc_codes<<<N, 256, 0, st>>>(ax, N, L, Lp, Lw, ra, rb, len);
  const int nt = (N + 31) / 32;
  k_gsc_ident<<<dim3(nt, nt), 256, 0, st>>>(ra, rb, len, N, Lw, D);
  k_gsc_init<<<(N + 255) / 256, 256, 0, st>>>(N, alive, size, height, cl, w);
  const int G = std::min(48, std::max(1, (N + 7) / 8));
  for (int m = 0; m < N - 1; m++) {
    k_gsc_scan<<<G, 256, 0, st>>>(D, alive, N, part);
    k_gsc_merge<<<1, 1024, 0, st>>>(D, alive, size, height, cl, w, N, part, G);
  }
  return cudaGetLastError();
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

}  // namespace covgpu
