// cov_kernels.cu -- SIMT kernels of the covariation path (sm_103a).
//
//   k_count_simt    weighted (or unit-weight) 4x4 joint counts of every
//                   column pair: mutual_naive_ppij, src/correlators.c:1695-1780
//   k_pair_marg     per-tile partial sums of the pair-normalised marginals:
//                   corr_Marginals, src/correlators.c:1337-1375
//   k_pm_final      marginals pm and the CCF column means (:1030-1036)
//   k_ps            single-column frequencies: mutual_naive_psi, :1782-1817
//   k_stats         CHI/GT/MI/MIr/MIg/OMES (C16, C2, GT-CWC), RAF, CCF per
//                   pair from the counts (:92-1061) + row/column sums for APC
//   k_rafs          RAFS stencil on RAF (:935-982)
//   k_apc_*         corr_CalculateCOVCorrected APC/ASC (:1063-1157)
//   k_hist          histogram of pair scores (src/covariation.c:414-457)
//   k_evalue        per-pair E-values and the hit list (:2369-2400, :778-1006)
//   k_untile        tile-packed scores -> full L x L matrix for the host
//
// Score matrices live on the device as double-float pairs (float2: hi + lo,
// ~48-bit significand): GB300 issues FP64 at 1/64 of its FP32 rate, so the
// per-pair passes (APC/ASC, min/max, histogram bins) run on the FP32 pipes;
// FP64 is kept for the row/column means, a bin next to a bin boundary, and
// the E-value tables.
#include "cov_dev.cuh"
#include "cov_kernels.h"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>

namespace covgpu {

// Easel's bin of x: ceil((x - bmin)/w - 1).  The quotient is first formed
// with the reciprocal; only when it lies within 1e-9 of an integer (where
// the last ulp could move the ceiling) is the IEEE division redone, so the
// bin always equals the one the division gives.
__host__ __device__ __forceinline__ int exact_bin(double x, double bmin, double w, double invw) {
  // fp32 estimate first: three roundings put it within 1.8e-7 |q| of the
  // exact quotient, so away from integers it has the same ceiling
  const float qf = (float)(x - bmin) * (float)invw;
  const float fr = qf - rintf(qf);
  if (fabsf(qf) < 4194304.f && fabsf(fr) > 4e-7f * fabsf(qf) + 1e-6f) return (int)ceilf(qf - 1.0f);
  double q = (x - bmin) * invw;
  if (fabs(q - rint(q)) < 1e-9) q = (x - bmin) / w;
  return (int)ceil(q - 1.0);
}

// ------------------------------------------------------------------------
// Counting (plain SIMT path): one CTA per (tile, alignment); 256 threads,
// each owning a 2x2 block of pairs and 4x16 fp32 accumulators.  Sequences
// are staged 32 at a time in shared memory as float4 one-hot (i side) and
// weight-scaled one-hot (j side) vectors; every pair then takes 16 FMAs per
// sequence.  With unit weights the counts are exact integers (< 2^24).
// ------------------------------------------------------------------------
template <bool UNIT>
__global__ void __launch_bounds__(256, 2)
k_count_simt(const uint8_t* __restrict__ ax, int64_t slot_stride, const float* __restrict__ w,
             int N, int Lp, const TileRC* __restrict__ tiles, int ntiles, float* __restrict__ cnt) {
  __shared__ float4 ohi[32][TP];
  __shared__ float4 whj[32][TP];
  const int t = blockIdx.x, slot = blockIdx.y, tid = threadIdx.x;
  const TileRC tr = tiles[t];
  const uint8_t* A = ax + (int64_t)slot * slot_stride;
  const int ty = tid >> 4, tx = tid & 15;
  float acc[4][16];
#pragma unroll
  for (int p = 0; p < 4; p++)
#pragma unroll
    for (int c = 0; c < 16; c++) acc[p][c] = 0.f;

  for (int s0 = 0; s0 < N; s0 += 32) {
#pragma unroll
    for (int k = 0; k < 8; k++) {
      const int e = tid + 256 * k;          // 0..2047
      const int half = e >> 10, s = (e >> 5) & 31, c = e & 31;
      const int seq = s0 + s;
      int code = 4;
      float val = 0.f;
      if (seq < N) {
        code = A[(int64_t)seq * Lp + (half ? tr.J : tr.I) * TP + c];
        val = half ? (UNIT ? 1.f : w[seq]) : 1.f;
      }
      float4 v;
      v.x = (code == 0) ? val : 0.f;
      v.y = (code == 1) ? val : 0.f;
      v.z = (code == 2) ? val : 0.f;
      v.w = (code == 3) ? val : 0.f;
      if (half) whj[s][c] = v; else ohi[s][c] = v;
    }
    __syncthreads();
    const int smax = min(32, N - s0);
    for (int s = 0; s < smax; s++) {
      const float4 i0 = ohi[s][2 * ty], i1 = ohi[s][2 * ty + 1];
      const float4 j0 = whj[s][2 * tx], j1 = whj[s][2 * tx + 1];
      const float iv[2][4] = {{i0.x, i0.y, i0.z, i0.w}, {i1.x, i1.y, i1.z, i1.w}};
      const float jv[2][4] = {{j0.x, j0.y, j0.z, j0.w}, {j1.x, j1.y, j1.z, j1.w}};
#pragma unroll
      for (int a = 0; a < 2; a++)
#pragma unroll
        for (int b = 0; b < 2; b++)
#pragma unroll
          for (int x = 0; x < 4; x++)
#pragma unroll
            for (int y = 0; y < 4; y++) acc[a * 2 + b][x * 4 + y] = fmaf(iv[a][x], jv[b][y], acc[a * 2 + b][x * 4 + y]);
    }
    __syncthreads();
  }
  float* out = cnt + ((int64_t)slot * ntiles + t) * 16 * TPP;
#pragma unroll
  for (int a = 0; a < 2; a++)
#pragma unroll
    for (int c = 0; c < 16; c++) {
      float2 v = make_float2(acc[a * 2 + 0][c], acc[a * 2 + 1][c]);
      *reinterpret_cast<float2*>(out + c * TPP + (2 * ty + a) * TP + 2 * tx) = v;
    }
}

// double-float arithmetic (pairs of fp32 values, ~48-bit significand)
struct df { float hi, lo; };

__device__ __forceinline__ df two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  return {s, (a - (s - bb)) + (b - bb)};
}
__device__ __forceinline__ df fast_two_sum(float a, float b) {   // |a| >= |b|
  const float s = a + b;
  return {s, b - (s - a)};
}
__device__ __forceinline__ df df_add_f(df a, float b) {
  const df s = two_sum(a.hi, b);
  return fast_two_sum(s.hi, s.lo + a.lo);
}
__device__ __forceinline__ df df_add(df a, df b) {
  const df s = two_sum(a.hi, b.hi);
  return fast_two_sum(s.hi, s.lo + (a.lo + b.lo));
}
__device__ __forceinline__ df df_mul(df a, df b) {
  const float p = a.hi * b.hi;
  const float e = fmaf(a.hi, b.hi, -p);
  return fast_two_sum(p, fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, e)));
}
__device__ __forceinline__ df df_of(double x) {
  const float hi = (float)x;
  return {hi, (float)(x - (double)hi)};
}
__device__ __forceinline__ double df_to_d(df a) { return (double)a.hi + (double)a.lo; }
__device__ __forceinline__ df df_neg(df a) { return {-a.hi, -a.lo}; }
// a * b exactly as a double-float (FMA residual)
__device__ __forceinline__ df two_prod(float a, float b) {
  const float p = a * b;
  return {p, fmaf(a, b, -p)};
}
__device__ __forceinline__ df ld_df(const float2* p) { const float2 v = *p; return {v.x, v.y}; }
__device__ __forceinline__ void st_df(float2* p, df v) { *p = make_float2(v.hi, v.lo); }
// order of normalised double-float values (|lo| <= ulp(hi)/2)
__device__ __forceinline__ bool df_lt(df a, df b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
__device__ __forceinline__ df df_min(df a, df b) { return df_lt(b, a) ? b : a; }
__device__ __forceinline__ df df_max(df a, df b) { return df_lt(a, b) ? b : a; }

// constants of the bin function, split on the host
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

static BinC make_binc(double bmin, double w) {
  auto split = [](double x) { const float h = (float)x; return make_float2(h, (float)(x - (double)h)); };
  BinC B;
  B.nbmin = split(-bmin);
  B.invw = split(1.0 / w);
  B.lo = split(bmin + w);
  B.mconst = (float)(1e-11 * (std::fabs(bmin) / w + 1.0));
  B.absb = (float)std::fabs(bmin);
  B.mscale = (float)(4e-7 / w);
  B.bin_lo = exact_bin(bmin + w, bmin, w, 1.0 / w);
  B.bmin = bmin; B.w = w;
  return B;
}

// Easel's bin of x = hi + lo: ceil((x - bmin)/w - 1).  The quotient is
// formed in double-float (error < 1e-12 (|q| + |bmin|/w + 1) against the FP64
// expression); when it lies closer than that to an integer the FP64
// expression of exact_bin decides, so the bin is the one FP64 gives.
//
// First an FP32 estimate: the dropped low parts of x and -bmin, the rounding
// of 1/w and three roundings keep it within 2^-22 (|x| + |bmin|)/w (< the
// 4e-7 scale of mscale) of the exact quotient, so away from integers it has
// the same ceiling; most scores are decided there in a few instructions.
__device__ __forceinline__ int bin_df(df x, const BinC& B) {
  {
    const float q = (x.hi + B.nbmin.x) * B.invw.x;
    const float n = rintf(q);
    const float marg = fmaf(fabsf(x.hi) + B.absb, B.mscale, 1e-6f);
    if (fabsf(q) < 4194304.f && fabsf(q - n) > marg) return (q > n) ? (int)n : (int)n - 1;
  }
  const df q = df_mul(df_add(x, {B.nbmin.x, B.nbmin.y}), {B.invw.x, B.invw.y});
  const float n = rintf(q.hi);
  const float f = (q.hi - n) + q.lo;
  if (fabsf(q.hi) < 4194304.f && fabsf(f) > 1e-11f * fabsf(q.hi) + B.mconst) return (f > 0.f) ? (int)n : (int)n - 1;
  return exact_bin(df_to_d(x), B.bmin, B.w, 1.0 / B.w);
}

// bin of max(x, bmin + w) (src/covariation.c:431-432); NaN goes to the
// clamp, whose bin comes from the FP64 value of bmin + w
__device__ __forceinline__ int bin_clamped(df x, const BinC& B) {
  return df_lt({B.lo.x, B.lo.y}, x) ? bin_df(x, B) : B.bin_lo;
}

// block min/max of double-float values (256 threads) -> FP64 per block
__device__ __forceinline__ void block_minmax_store(df lo, df hi, double* tmin, double* tmax) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const df l2 = {__shfl_xor_sync(0xffffffffu, lo.hi, o), __shfl_xor_sync(0xffffffffu, lo.lo, o)};
    const df h2 = {__shfl_xor_sync(0xffffffffu, hi.hi, o), __shfl_xor_sync(0xffffffffu, hi.lo, o)};
    lo = df_min(lo, l2); hi = df_max(hi, h2);
  }
  __shared__ float4 sm[8];
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = make_float4(lo.hi, lo.lo, hi.hi, hi.lo);
  __syncthreads();
  if (threadIdx.x == 0) {
    df l = {sm[0].x, sm[0].y}, h = {sm[0].z, sm[0].w};
    for (int w = 1; w < (int)(blockDim.x >> 5); w++) {
      l = df_min(l, {sm[w].x, sm[w].y});
      h = df_max(h, {sm[w].z, sm[w].w});
    }
    *tmin = (l.hi == INFINITY) ? DBL_MAX : df_to_d(l);
    *tmax = (h.hi == -INFINITY) ? -DBL_MAX : df_to_d(h);
  }
}


// ------------------------------------------------------------------------
// Block helper for the per-tile kernels: 256 threads, thread tid owns the
// pairs p = tid + 256k (k = 0..3): row a = (tid >> 5) + 8k, column b = lane.
// Reduces NV channels of per-pair values into per-row sums (of rv) and
// per-column sums (of cv) in double-float arithmetic and stores them as FP64
// in the partial layout part[I][J][a][c] (rows of tile (I,J)) and
// part[J][I][b][c] (columns); a diagonal tile adds both roles into
// part[I][I].
// ------------------------------------------------------------------------
__device__ __forceinline__ df warp_sum_df(df v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const df w = {__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o)};
    v = df_add(v, w);
  }
  return v;
}

template <int NV>
__device__ __forceinline__ void tile_rowcol_store2(const df (&rv)[4][NV], const df (&cv)[4][NV],
                                                   double* __restrict__ part, int nT, int I, int J) {
  __shared__ df colbuf[8][TP][NV];
  __shared__ df rowbuf[TP][NV];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
#pragma unroll
  for (int k = 0; k < 4; k++)
#pragma unroll
    for (int c = 0; c < NV; c++) {
      const df r = warp_sum_df(rv[k][c]);
      if (lane == 0) rowbuf[warp + 8 * k][c] = r;
    }
#pragma unroll
  for (int c = 0; c < NV; c++) colbuf[warp][lane][c] = df_add(df_add(cv[0][c], cv[1][c]), df_add(cv[2][c], cv[3][c]));
  __syncthreads();
  if (tid < TP * NV) {
    const int col = tid / NV, c = tid % NV;
    df cs = {0.f, 0.f};
    for (int wv = 0; wv < 8; wv++) cs = df_add(cs, colbuf[wv][col][c]);
    if (I == J) {
      part[(((int64_t)I * nT + J) * TP + col) * NV + c] = df_to_d(df_add(rowbuf[col][c], cs));
    } else {
      part[(((int64_t)I * nT + J) * TP + col) * NV + c] = df_to_d(rowbuf[col][c]);
      part[(((int64_t)J * nT + I) * TP + col) * NV + c] = df_to_d(cs);
    }
  }
  __syncthreads();
}

template <int NV>
__device__ __forceinline__ void tile_rowcol_store(const df (&v)[4][NV], double* __restrict__ part, int nT, int I,
                                                  int J) {
  tile_rowcol_store2<NV>(v, v, part, nT, I, J);
}

// Pair-normalised marginal contributions: for every pair with nseff > 0,
// row i gains (4e-10 + sum_y C(x,y)) / S and column j gains
// (4e-10 + sum_x C(x,y)) / S, S = 16e-10 + nseff (the prior of
// src/correlators.c:1713 and the normalisation of :1758).  Each pair's
// contribution is formed in fp32 (relative error ~1e-7, independent from pair
// to pair) and summed over partners in FP64, so the marginals keep ~1e-9.
// Also the upper-triangle row sums of nseff for the CCF column means.
__global__ void __launch_bounds__(256)
k_pair_marg(const float* __restrict__ cnt, int L, const TileRC* __restrict__ tiles, int ntiles, int nT,
            double* __restrict__ part4, double* __restrict__ partR) {
  const int t = blockIdx.x, slot = blockIdx.y, tid = threadIdx.x;
  const TileRC tr = tiles[t];
  const float* C = cnt + ((int64_t)slot * ntiles + t) * 16 * TPP;
  // every pair's row contributions, column contributions and nseff go to
  // shared tiles as they are formed (FP32: the double-float sums below take
  // them with a zero low part), so nothing is held in registers across pairs
  __shared__ float sr[4][TP][TP + 1];
  __shared__ float sc[4][TP][TP + 1];
  __shared__ float sn[TP][TP + 1];
  __shared__ float2 srow[4][TP];   // diagonal tiles: row sums, added to the column sums
#pragma unroll
  for (int k = 0; k < 4; k++) {
    const int p = tid + 256 * k, a = p >> 5, b = p & 31;
    const int i = tr.I * TP + a, j = tr.J * TP + b;
    float c[16];
#pragma unroll
    for (int q = 0; q < 16; q++) c[q] = C[q * TPP + p];
    float row[4], col[4];
#pragma unroll
    for (int x = 0; x < 4; x++) {
      row[x] = (c[x * 4 + 0] + c[x * 4 + 1]) + (c[x * 4 + 2] + c[x * 4 + 3]);
      col[x] = (c[0 * 4 + x] + c[1 * 4 + x]) + (c[2 * 4 + x] + c[3 * 4 + x]);
    }
    const float ne = (row[0] + row[1]) + (row[2] + row[3]);
    const bool pair = (i < j) && (j < L);
    const bool ok = pair && (ne > 0.f);
    const float invS = ok ? 1.0f / (16e-10f + ne) : 0.f;
#pragma unroll
    for (int x = 0; x < 4; x++) {
      sr[x][a][b] = ok ? (4e-10f + row[x]) * invS : 0.f;
      sc[x][a][b] = ok ? (4e-10f + col[x]) * invS : 0.f;
    }
    sn[a][b] = pair ? ne : 0.f;
  }
  __syncthreads();
  // row sums over b (threads 0-127) and column sums over a (128-255), one
  // thread per (value, line) adding its 32 entries in order; rows into
  // part[I][J], columns into part[J][I], both into part[I][I] on a diagonal
  // tile
  double* P4 = part4 + (int64_t)slot * nT * nT * TP * 4;
  double* PR = partR + (int64_t)slot * nT * nT * TP;
  const bool diag = (tr.I == tr.J);
  const int c4 = (tid >> 5) & 3, line = tid & 31;
  df sum = {0.f, 0.f};
  if (tid < 128) {
    for (int b = 0; b < TP; b++) sum = df_add_f(sum, sr[c4][line][b]);
    if (!diag) P4[(((int64_t)tr.I * nT + tr.J) * TP + line) * 4 + c4] = df_to_d(sum);
    else       srow[c4][line] = make_float2(sum.hi, sum.lo);
  } else {
    for (int a = 0; a < TP; a++) sum = df_add_f(sum, sc[c4][a][line]);
    if (!diag) P4[(((int64_t)tr.J * nT + tr.I) * TP + line) * 4 + c4] = df_to_d(sum);
  }
  if (diag) {
    __syncthreads();
    if (tid >= 128)
      P4[(((int64_t)tr.I * nT + tr.I) * TP + line) * 4 + c4] =
          df_to_d(df_add({srow[c4][line].x, srow[c4][line].y}, sum));
  }
  if (tid < TP) {
    df ns = {0.f, 0.f};
    for (int b = 0; b < TP; b++) ns = df_add_f(ns, sn[tid][b]);
    PR[((int64_t)tr.I * nT + tr.J) * TP + tid] = df_to_d(ns);
    if (!diag) PR[((int64_t)tr.J * nT + tr.I) * TP + tid] = 0.0;   // the column sums of nseff are not used
  }
}

// pm[c][x] = normalise(sum over every tile touching column c); one thread
// per column.  mpc[c][x] = pm[c][x] * (sum_{j>c} nseff[c][j]) feeds the CCF
// column means (src/correlators.c:1030-1036).
__global__ void k_pm_final(const double* __restrict__ part4, const double* __restrict__ partR, int L, int Lp, int nT,
                           double* __restrict__ pm, float2* __restrict__ pmdf, double* __restrict__ mpc,
                           int* __restrict__ status) {
  const int slot = blockIdx.y;
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= L) return;
  const double* P = part4 + (int64_t)slot * nT * nT * TP * 4;
  const double* R = partR + (int64_t)slot * nT * nT * TP;
  const int I = c / TP, a = c % TP;
  double m[4] = {0, 0, 0, 0}, rs = 0.0;
  for (int K = 0; K < nT; K++) {
    const double4 v = *reinterpret_cast<const double4*>(P + (((int64_t)I * nT + K) * TP + a) * 4);
    m[0] += v.x; m[1] += v.y; m[2] += v.z; m[3] += v.w;
    rs += R[((int64_t)I * nT + K) * TP + a];
  }
  const double sum = m[0] + m[1] + m[2] + m[3];
#pragma unroll
  for (int x = 0; x < 4; x++) m[x] = (sum != 0.0) ? m[x] / sum : 0.25;
  if (fabs(m[0] + m[1] + m[2] + m[3] - 1.0) > 1e-6) atomicExch(status, 2);
#pragma unroll
  for (int x = 0; x < 4; x++) {
    pm[((int64_t)slot * Lp + c) * 4 + x] = m[x];
    const float hi = (float)m[x];
    pmdf[((int64_t)slot * Lp + c) * 4 + x] = make_float2(hi, (float)(m[x] - (double)hi));
    mpc[((int64_t)slot * Lp + c) * 4 + x] = rs * m[x];
  }
}

__global__ void k_meanp(const double* __restrict__ mpc, int L, int Lp, double* __restrict__ meanp) {
  const int slot = blockIdx.x;
  __shared__ double buf[4][256];
  double acc[4] = {0, 0, 0, 0};
  for (int c = threadIdx.x; c < L; c += blockDim.x)
#pragma unroll
    for (int x = 0; x < 4; x++) acc[x] += mpc[((int64_t)slot * Lp + c) * 4 + x];
#pragma unroll
  for (int x = 0; x < 4; x++) buf[x][threadIdx.x] = acc[x];
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o)
#pragma unroll
      for (int x = 0; x < 4; x++) buf[x][threadIdx.x] += buf[x][threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double s = buf[0][0] + buf[1][0] + buf[2][0] + buf[3][0];
    for (int x = 0; x < 4; x++) meanp[slot * 4 + x] = (s != 0.0) ? buf[x][0] / s : 0.25;
  }
}

// ps[c][x], x over the five codes 0..4 (gap included), prior 1e-5.
__global__ void k_ps(const uint8_t* __restrict__ ax, int64_t slot_stride, const double* __restrict__ w, int N, int L,
                     int Lp, double* __restrict__ ps) {
  const int slot = blockIdx.y;
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= L) return;
  const uint8_t* A = ax + (int64_t)slot * slot_stride;
  double q[5] = {1e-5, 1e-5, 1e-5, 1e-5, 1e-5};
  for (int s = 0; s < N; s++) {
    const int r = A[(int64_t)s * Lp + c];
    if (r < 5) q[r] += w[s];
  }
  double sum = q[0] + q[1] + q[2] + q[3] + q[4];
  for (int x = 0; x < 5; x++) ps[((int64_t)slot * Lp + c) * 5 + x] = q[x] / sum;
}

// ------------------------------------------------------------------------
// Statistics.  Per cell, o = nseff*pp and e = nseff*pm_i(x)*pm_j(y) are
// formed in double-float arithmetic (pairs of fp32 values, ~48-bit
// significand; GB300 runs fp32 at 64x its FP64 rate) and their difference
// u = o - e is rounded once to fp32; the rest is fp32.  The G-test is summed
// as 2*sum_e e*g(u/e) (each term >= 0), which equals the reference's
// 2*sum o*ln(o/e) because sum u = 0 to rounding when every cell enters (pp
// and pm are normalised); the CWC form, which sums a subset of cells, adds
// its sum u explicitly.
//
// o = (1e-10 + C) ne / (16e-10 + ne) is written as C + do with
// do = 1e-10 - 16e-10 C / ne (to 1e-18 absolute), the prior of
// src/correlators.c:1713 and the normalisation of :1758.
// ------------------------------------------------------------------------
// u = o - e with o = c + dc (c >= 0 exact fp32, |dc| tiny), e in double-float
__device__ __forceinline__ float diff_oe(float c, float dc, df e) {
  const df s = two_sum(c, -e.hi);
  return s.hi + (s.lo + (dc - e.lo));
}

// G-test term e*g(d), d = u/e, o = c + dc: for |d| < 1/4 the polynomial
// gfun_poly, elsewhere r ln r - (r - 1) with r = 1 + d, as
// r log1p(d) - d.  Below zero r is the quotient o/e (relative error 2^-22,
// so r ln r is off by at most 2.4e-7 r |ln r| <= 9e-8), not 1 + d: for
// empty cells (r ~ 1e-10) 1 + d rounds to a multiple of 2^-24 and, times
// log1p(d) ~ -20, would add ~1e-6 e per cell.  Both forms are evaluated and
// one is selected: a warp holds pairs whose cells fall on both sides, and a
// branch would make every warp run every path.  ie = 1/e (approximate
// reciprocal, shared with the caller's CHI term).
__device__ __forceinline__ float gterm_f(float u, float e, float ie, float o) {
  const float d = u * ie;
  const float dn = fminf(fmaxf(d, -0.25f), 0.25f);     // the polynomial only where it is used
  const float near = gfun_poly(dn);
  const float dp = fmaxf(d, -1.f);
  const float r = (d < 0.f) ? o * ie : 1.f + dp;
  const float l = log1pf(fmaxf(dp, -0.99999994f));     // finite where 1 + d rounds to 0
  const float far = r * l - dp;
  return e * ((fabsf(d) < 0.25f) ? near : far);
}

struct PairOut { float chi, gt, mi, mir, mig, omes; df raf, ccf; };

__device__ __forceinline__ df pick_df(const PairOut& o, int k) {
  switch (k) {
    case 0: return {o.chi, 0.f};
    case 1: return {o.gt, 0.f};
    case 2: return {o.mi, 0.f};
    case 3: return {o.mir, 0.f};
    case 4: return {o.mig, 0.f};
    case 5: return {o.omes, 0.f};
    case 6: return o.raf;
    case 8: return o.ccf;
  }
  return {0.f, 0.f};
}

// per-cell terms a k_stats variant computes (the C16/CWC cell loop is the
// hot part; a variant carries only what its statistics read)
enum CellF : unsigned { CF_G = 1u, CF_CHI = 2u, CF_OMES = 4u, CF_H = 8u, CF_ALL = 15u };


template <unsigned CF>
__device__ __forceinline__ void pair_stats(const StatsArgs& A, const float (&c)[16], const float (&uc)[16],
                                           bool have_uc, const float2* pmi, const float2* pmj, const double* pmid,
                                           const double* pmjd, const double* meanp, df ne, PairOut& out) {
  const unsigned S = A.stats;
  // ---- RAF from unit-weight counts (src/correlators.c:897-925 reduced):
  // the sums are exact integers in fp32 (< 2^24); c_ij = nA^2 - (sum r_x^2
  // + sum c_y^2)/2 is an integer below 2^48, formed exactly in double-float
  // from exact FP32 products; the two ratios are double-float products ----
  if ((S & (S_RAF | S_RAFS)) && have_uc) {
    float nAf = 0.f, r[4] = {0.f, 0.f, 0.f, 0.f}, cc[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int x = 0; x < 4; x++)
#pragma unroll
      for (int y = 0; y < 4; y++)
        if (A.allow[x * 4 + y] > 0.f) {
          const float n = uc[x * 4 + y];
          nAf += n; r[x] += n; cc[y] += n;
        }
    // c_ij = nA^2 - (sum r_x^2 + sum c_y^2)/2 in 64-bit integers (the
    // counts are integers below 2^24, c_ij below 2^48), then split exactly
    // into a double-float
    // (sum r_x^2 + sum c_y^2 is even: each sum has the parity of nA)
    int64_t sq = 0;
#pragma unroll
    for (int x = 0; x < 4; x++) {
      const int a = (int)r[x], b = (int)cc[x];
      sq += (int64_t)a * a + (int64_t)b * b;
    }
    const int nA = (int)nAf;
    const int64_t ci = (int64_t)nA * nA - sq / 2;
    const float ci_hi = (float)ci;
    const df cnum = {ci_hi, (float)(ci - (int64_t)ci_hi)};   // exact: the rest is an integer below 2^24
    const df q1 = df_mul(cnum, {A.invD.x, A.invD.y});
    const df q2 = df_mul({(float)A.N - nAf, 0.f}, {A.invN.x, A.invN.y});
    out.raf = df_add({2.f * q1.hi, 2.f * q1.lo}, df_neg(q2));
  }
  // ---- CCF (src/correlators.c:1038-1053), FP64 ----
  if (S & S_CCF) {
    const double ned = df_to_d(ne);
    double ccf = 0.0;
#pragma unroll
    for (int x = 0; x < 4; x++)
#pragma unroll
      for (int y = 0; y < 4; y++) {
        const double cc = (ned * pmid[x] - meanp[x]) * (ned * pmjd[y] - meanp[y]);
        ccf += cc * cc;
      }
    out.ccf = df_of(sqrt(ccf));
  }
  const unsigned SP = S & (S_CHI | S_GT | S_MI | S_MIr | S_MIg | S_OMES);
  if (!SP) return;

  if (ne.hi <= 0.f) {
    // no sequence with both residues canonical: pp = 1/16 (prior only)
    double mi = 0.0, hh = 0.0;
    if (A.cls != 1) {
      for (int x = 0; x < 4; x++)
        for (int y = 0; y < 4; y++) {
          const double p = 0.0625;
          if (pmid[x] > 0.0 && pmjd[y] > 0.0) mi += p * (log(p) - log(pmid[x]) - log(pmjd[y]));
          hh -= p * log(p);
        }
    } else {
      double pw = 0, pn = 0, qw = 0, qn = 0;
      for (int x = 0; x < 4; x++)
        for (int y = 0; y < 4; y++) {
          if (A.allow[x * 4 + y] > 0.f) { pw += 0.0625; qw += pmid[x] * pmjd[y]; }
          else                          { pn += 0.0625; qn += pmid[x] * pmjd[y]; }
        }
      if (pw > 0.0) { mi += pw * (log(pw) - log(qw)); hh -= pw * log(pw); }
      if (pn > 0.0) { mi += pn * (log(pn) - log(qn)); hh -= pn * log(pn); }
    }
    out.chi = 0.f; out.gt = 0.f; out.omes = 0.f;
    out.mi = (float)mi; out.mir = (float)((hh > 1e-2) ? mi / hh : 0.0); out.mig = (float)mi;
    return;
  }

  const float inv_ne = 1.0f / ne.hi;
  const df ng = df_add({A.wtot.x, A.wtot.y}, {-ne.hi, -ne.lo});   // ngap = sum w - nseff
  if (A.cls == 0 || A.cls == 2) {
    float gsum = 0.f, chi = 0.f, omes = 0.f, hh = 0.f, usum = 0.f;
#pragma unroll
    for (int x = 0; x < 4; x++) {
      const df ax = df_mul(ne, {pmi[x].x, pmi[x].y});
#pragma unroll
      for (int y = 0; y < 4; y++) {
        if (A.cls == 2 && !(A.allow[x * 4 + y] > 0.f)) continue;
        const float C = c[x * 4 + y];
        const float dc = 1e-10f - 16e-10f * C * inv_ne;
        const float o = C + dc;
        if (CF & (CF_G | CF_CHI | CF_OMES)) {
          const df e = df_mul(ax, {pmj[y].x, pmj[y].y});
          const float u = diff_oe(C, dc, e);
          if (e.hi > 0.f) {
            const float ie = __fdividef(1.f, e.hi);
            if (CF & CF_G) { gsum += gterm_f(u, e.hi, ie, o); usum += u; }
            if (CF & CF_CHI) chi += u * u * ie;
            if (CF & CF_OMES) omes += u * u;
          }
        }
        if (CF & CF_H) {
          const float p = o * inv_ne;
          hh -= (p > 0.f) ? p * __logf(p) : 0.f;
        }
      }
    }
    const float gt = (A.cls == 2) ? 2.f * (gsum + usum) : 2.f * gsum;
    const float mi = gsum * inv_ne;
    out.chi = chi;
    out.gt = gt;
    out.mi = mi;
    out.mir = (hh > 1e-2f) ? mi / hh : 0.f;
    out.mig = mi - (ng.hi + ng.lo) * inv_ne;
    out.omes = omes * inv_ne;
  } else {
    // C2: allowed / not-allowed merged cells (e.g. src/correlators.c:426-458)
    df Cw = {0.f, 0.f}, Cn = {0.f, 0.f}, qw = {0.f, 0.f}, qn = {0.f, 0.f};
    int nal = 0;
#pragma unroll
    for (int x = 0; x < 4; x++)
#pragma unroll
      for (int y = 0; y < 4; y++) {
        const df pq = df_mul({pmi[x].x, pmi[x].y}, {pmj[y].x, pmj[y].y});
        if (A.allow[x * 4 + y] > 0.f) { Cw = df_add_f(Cw, c[x * 4 + y]); qw = df_add(qw, pq); nal++; }
        else                          { Cn = df_add_f(Cn, c[x * 4 + y]); qn = df_add(qn, pq); }
      }
    const float dw = nal * 1e-10f - 16e-10f * Cw.hi * inv_ne;
    const float dn = (16 - nal) * 1e-10f - 16e-10f * Cn.hi * inv_ne;
    const df ew = df_mul(ne, qw), en = df_mul(ne, qn);
    // u = (Cw.hi + Cw.lo + dw) - ew
    const float uw = diff_oe(Cw.hi, Cw.lo + dw, ew);
    const float un = diff_oe(Cn.hi, Cn.lo + dn, en);
    const float ow = Cw.hi + (Cw.lo + dw), on = Cn.hi + (Cn.lo + dn);
    float g = 0.f, chi = 0.f, om = 0.f;
    if (ew.hi > 0.f) {
      const float ie = __fdividef(1.f, ew.hi);
      g += gterm_f(uw, ew.hi, ie, ow); chi += uw * uw * ie; om += uw * uw;
    }
    if (en.hi > 0.f) {
      const float ie = __fdividef(1.f, en.hi);
      g += gterm_f(un, en.hi, ie, on); chi += un * un * ie; om += un * un;
    }
    const float pw = ow * inv_ne, pn = on * inv_ne;
    float hh = 0.f;
    hh -= (pw > 0.f) ? pw * __logf(pw) : 0.f;
    hh -= (pn > 0.f) ? pn * __logf(pn) : 0.f;
    const float mi = g * inv_ne;
    out.chi = chi;
    out.gt = 2.f * g;
    out.mi = mi;
    out.mir = (hh > 1e-2f) ? mi / hh : 0.f;
    out.mig = mi - (ng.hi + ng.lo) * inv_ne;
    out.omes = om * inv_ne;
  }
}

// One CTA per (tile, alignment), 256 threads, thread tid owns the pairs
// p = tid + 256k (row a = warp + 8k, column b = lane).  Each pair's scores
// go straight to the score planes and into a shared-memory copy of the
// tile; after the tile, one thread per (row, output) adds its row and one
// per (column, output) its column in double-float, in a fixed order, for the
// APC/ASC partials.
template <unsigned CF>
__global__ void __launch_bounds__(256)
k_stats(StatsArgs A) {
  const int t = blockIdx.x, slot = blockIdx.y, tid = threadIdx.x;
  const TileRC tr = A.tiles[t];
  const float* C = A.cnt ? A.cnt + ((int64_t)slot * A.ntiles + t) * 16 * TPP : nullptr;
  const float* U = A.ucnt ? A.ucnt + ((int64_t)slot * A.ntiles + t) * 16 * TPP : nullptr;
  const double* pm = A.pm + (int64_t)slot * A.Lp * 4;
  const float2* pmdf = A.pmdf + (int64_t)slot * A.Lp * 4;
  const double* meanp = A.meanp + slot * 4;
  __shared__ float2 vs[MAXOUT][TP][TP + 1];   // the tile's scores, [q][a][b]
#pragma unroll 1
  for (int k = 0; k < 4; k++) {
    const int p = tid + 256 * k, a = p >> 5, b = p & 31;
    const int i = tr.I * TP + a, j = tr.J * TP + b;
    const bool valid = (i < j) && (j < A.L);
    float c[16], uc[16];
#pragma unroll
    for (int q = 0; q < 16; q++) {
      c[q] = C ? C[q * TPP + p] : 0.f;
      uc[q] = (U && A.allow[q] > 0.f) ? U[q * TPP + p] : 0.f;   // RAF reads the allowed cells only
    }
    df ne = {0.f, 0.f};
#pragma unroll
    for (int q = 0; q < 16; q++) ne = df_add_f(ne, c[q]);
    PairOut o;
    o.chi = o.gt = o.mi = o.mir = o.mig = o.omes = 0.f;
    o.raf = o.ccf = df{0.f, 0.f};
    if (valid) {
      const int ii = i < A.L ? i : 0, jj = j < A.L ? j : 0;
      pair_stats<CF>(A, c, uc, U != nullptr, pmdf + ii * 4, pmdf + jj * 4, pm + ii * 4, pm + jj * 4, meanp, ne, o);
    }
#pragma unroll
    for (int q = 0; q < MAXOUT; q++) {
      if (q < A.nout) {
        const df v = valid ? pick_df(o, A.outstat[q]) : df{0.f, 0.f};
        st_df(A.cov + (((int64_t)slot * A.nout + q) * A.ntiles + t) * TPP + p, v);
        vs[q][a][b] = make_float2(v.hi, v.lo);
      }
    }
  }
  __syncthreads();
  // rows of tile (I,J) at part[I][J], columns at part[J][I]; a diagonal tile
  // adds both roles into part[I][I]
  double* base = A.part1 + (int64_t)slot * A.nout * A.nT * A.nT * TP;
  const int64_t qstride = (int64_t)A.nT * A.nT * TP;
  if (tr.I != tr.J) {
    if (tid < 2 * TP * A.nout) {
      const int role = tid / (TP * A.nout), rem = tid % (TP * A.nout);
      const int line = rem / A.nout, q = rem % A.nout;
      df sum = {0.f, 0.f};
      if (role == 0) { for (int b = 0; b < TP; b++) sum = df_add(sum, {vs[q][line][b].x, vs[q][line][b].y}); }
      else           { for (int a = 0; a < TP; a++) sum = df_add(sum, {vs[q][a][line].x, vs[q][a][line].y}); }
      const int64_t cell = (role == 0) ? ((int64_t)tr.I * A.nT + tr.J) : ((int64_t)tr.J * A.nT + tr.I);
      base[q * qstride + cell * TP + line] = df_to_d(sum);
    }
  } else if (tid < TP * A.nout) {
    const int line = tid / A.nout, q = tid % A.nout;
    df r = {0.f, 0.f}, c = {0.f, 0.f};
    for (int b = 0; b < TP; b++) r = df_add(r, {vs[q][line][b].x, vs[q][line][b].y});
    for (int a = 0; a < TP; a++) c = df_add(c, {vs[q][a][line].x, vs[q][a][line].y});
    base[q * qstride + ((int64_t)tr.I * A.nT + tr.I) * TP + line] = df_to_d(df_add(r, c));
  }
}

// RAFS from the RAF scores (both in tile layout); b_{i-1,j+1}, b_{i+1,j-1}
__device__ __forceinline__ df tile_get(const float2* cov, const int* tile_index, int nT, int i, int j) {
  const int I = i / TP, J = j / TP;
  const int t = tile_index[I * nT + J];
  return ld_df(cov + (int64_t)t * TPP + (i % TP) * TP + (j % TP));
}

__global__ void __launch_bounds__(256)
k_rafs(const float2* __restrict__ raf, float2* __restrict__ out, int64_t slot_stride_in, int64_t slot_stride_out,
       const TileRC* __restrict__ tiles, const int* __restrict__ tile_index, int ntiles, int nT, int L,
       double* __restrict__ part1, int64_t part_stride) {
  const int t = blockIdx.x, slot = blockIdx.y, tid = threadIdx.x;
  const TileRC tr = tiles[t];
  const float2* B = raf + slot * slot_stride_in;
  df v[4][1];
#pragma unroll
  for (int k = 0; k < 4; k++) {
    const int p = tid + 256 * k, a = p >> 5, b = p & 31;
    const int i = tr.I * TP + a, j = tr.J * TP + b;
    df r = {0.f, 0.f};
    if (i < j && j < L) {
      const df c = ld_df(B + (int64_t)t * TPP + p);
      r = {2.f * c.hi, 2.f * c.lo};
      if (i > 0 && j < L - 1) r = df_add(r, tile_get(B, tile_index, nT, i - 1, j + 1));
      if (j > 0 && i < L - 1 && i < j - 2) r = df_add(r, tile_get(B, tile_index, nT, i + 1, j - 1));
      r = {0.25f * r.hi, 0.25f * r.lo};
    }
    st_df(out + slot * slot_stride_out + (int64_t)t * TPP + p, r);
    v[k][0] = r;
  }
  tile_rowcol_store<1>(v, part1 + slot * part_stride, nT, tr.I, tr.J);
}

// COVx[c] = sum_{j != c} COV[c][j] / (L-1), from the tile partials
__global__ void k_apc_colx(const double* __restrict__ part1, int nT, int L, int Lp, double* __restrict__ colx,
                           float2* __restrict__ colxf) {
  const int sq = blockIdx.y;   // (slot, stat) flattened
  const double* P = part1 + (int64_t)sq * nT * nT * TP;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < L; c += gridDim.x * blockDim.x) {
    const int I = c / TP, a = c % TP;
    double s = 0.0;
    for (int K = 0; K < nT; K++) s += P[((int64_t)I * nT + K) * TP + a];
    const double x = (L > 1) ? s / ((double)L - 1.0) : s;
    colx[(int64_t)sq * Lp + c] = x;
    st_df(colxf + (int64_t)sq * Lp + c, df_of(x));
  }
}

// avg = 2/(L(L-1)) * sum_{i<j} COV = sum_c COVx[c] / L
__global__ void k_apc_avg(const double* __restrict__ colx, int L, int Lp, double* __restrict__ avg,
                          float4* __restrict__ apcf) {
  const int sq = blockIdx.x;
  __shared__ double buf[256];
  double s = 0.0;
  for (int c = threadIdx.x; c < L; c += blockDim.x) s += colx[(int64_t)sq * Lp + c];
  buf[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) buf[threadIdx.x] += buf[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double A = (L > 1) ? buf[0] * ((double)L - 1.0) / ((double)L * ((double)L - 1.0)) : 0.0;
    avg[sq] = A;
    const df a = df_of(A), ia = df_of(A != 0.0 ? 1.0 / A : 0.0);
    apcf[sq] = make_float4(a.hi, a.lo, ia.hi, ia.lo);
  }
}

// COV <- COV - COVx_i COVx_j / avg (APC) or COV - (COVx_i + COVx_j - avg) (ASC);
// per-tile min/max of the corrected scores.  Double-float arithmetic.
// APC/ASC applied in place, APC_TILES tiles per block (the block's min/max
// reduction amortised over them), two pairs per 16-byte access
constexpr int APC_TILES = 4;

__global__ void __launch_bounds__(256)
k_apc_apply(float2* __restrict__ cov, const float2* __restrict__ colxf, const double* __restrict__ avg,
            const float4* __restrict__ apcf, CorrTypes ct, const TileRC* __restrict__ tiles, int ntiles, int L, int Lp,
            double* __restrict__ tmin, double* __restrict__ tmax, int* __restrict__ status) {
  const int sq = blockIdx.y, tid = threadIdx.x;
  const int actype = ct.act[sq % ct.nout];
  const bool Anz = (avg[sq] != 0.0);
  const float4 af = apcf[sq];
  const df A = {af.x, af.y}, invA = {af.z, af.w};
  const float2* X = colxf + (int64_t)sq * Lp;
  df lo = {INFINITY, 0.f}, hi = {-INFINITY, 0.f};
  auto corrected = [&](df v, int i, int j) -> df {
    if (actype == 0) return Anz ? df_add(v, df_neg(df_mul(df_mul(ld_df(X + i), ld_df(X + j)), invA))) : df{0.f, 0.f};
    if (actype == 1) return df_add(v, df_neg(df_add(df_add(ld_df(X + i), ld_df(X + j)), df_neg(A))));
    return v;
  };
  for (int tt = 0; tt < APC_TILES; tt++) {
    const int t = blockIdx.x * APC_TILES + tt;
    if (t >= ntiles) break;
    const TileRC tr = tiles[t];
    float4* V = reinterpret_cast<float4*>(cov + ((int64_t)sq * ntiles + t) * TPP);
#pragma unroll
    for (int k = 0; k < 2; k++) {
      const int q = tid + 256 * k;           // pairs 2q, 2q + 1: one row, adjacent columns
      const int p = 2 * q, a = p >> 5, b = p & 31;
      const int i = tr.I * TP + a, j = tr.J * TP + b;
      const float4 w = V[q];
      df v0 = {w.x, w.y}, v1 = {w.z, w.w};
      const bool ok0 = (i < j && j < L), ok1 = (i < j + 1 && j + 1 < L);
      if (ok0) {
        v0 = corrected(v0, i, j);
        if (isnan(v0.hi)) atomicExch(status, 3);
        lo = df_min(lo, v0); hi = df_max(hi, v0);
      }
      if (ok1) {
        v1 = corrected(v1, i, j + 1);
        if (isnan(v1.hi)) atomicExch(status, 3);
        lo = df_min(lo, v1); hi = df_max(hi, v1);
      }
      if (actype >= 0 && (ok0 || ok1)) V[q] = make_float4(v0.hi, v0.lo, v1.hi, v1.lo);
    }
  }
  const int nblk = gridDim.x;
  block_minmax_store(lo, hi, tmin + (int64_t)sq * nblk + blockIdx.x, tmax + (int64_t)sq * nblk + blockIdx.x);
}

// min/max of the scores of every valid pair (before any correction)
__global__ void __launch_bounds__(256)
k_tile_minmax(const float2* __restrict__ cov, const TileRC* __restrict__ tiles, int ntiles, int L,
              double* __restrict__ tmin, double* __restrict__ tmax) {
  const int t = blockIdx.x, sq = blockIdx.y, tid = threadIdx.x;
  const TileRC tr = tiles[t];
  const float2* V = cov + ((int64_t)sq * ntiles + t) * TPP;
  df lo = {INFINITY, 0.f}, hi = {-INFINITY, 0.f};
  for (int k = 0; k < 4; k++) {
    const int p = tid + 256 * k, a = p >> 5, b = p & 31;
    const int i = tr.I * TP + a, j = tr.J * TP + b;
    if (i < j && j < L) { const df v = ld_df(V + p); lo = df_min(lo, v); hi = df_max(hi, v); }
  }
  block_minmax_store(lo, hi, tmin + (int64_t)sq * ntiles + t, tmax + (int64_t)sq * ntiles + t);
}

__global__ void k_reduce_minmax(const double* __restrict__ tmin, const double* __restrict__ tmax, int ntiles,
                                double* __restrict__ mm) {
  const int sq = blockIdx.x;
  __shared__ double smin[256], smax[256];
  double lo = DBL_MAX, hi = -DBL_MAX;
  for (int t = threadIdx.x; t < ntiles; t += blockDim.x) {
    lo = fmin(lo, tmin[(int64_t)sq * ntiles + t]);
    hi = fmax(hi, tmax[(int64_t)sq * ntiles + t]);
  }
  smin[threadIdx.x] = lo; smax[threadIdx.x] = hi;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) {
      smin[threadIdx.x] = fmin(smin[threadIdx.x], smin[threadIdx.x + o]);
      smax[threadIdx.x] = fmax(smax[threadIdx.x], smax[threadIdx.x + o]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) { mm[sq * 2 + 0] = (smin[0] == DBL_MAX) ? INFINITY : smin[0]; mm[sq * 2 + 1] = (smax[0] == -DBL_MAX) ? -INFINITY : smax[0]; }
}

// Histogram of max(COV, bmin + w) over the valid pairs of several alignments
// (src/covariation.c:431-432), bins b = ceil((x - bmin)/w - 1).  One pass:
// each CTA keeps a private window of up to 48K 32-bit counters in shared
// memory starting at bin wbase (the bin of the smallest score), counts its
// (tile, alignment) items there with one shared-memory atomic per score, and
// sends the sparse bins above the window straight to the global histogram.
// A CTA is R groups of 256 threads (R = 4 when the window leaves room for one
// CTA per SM, else 1), each group walking its own items; a thread reads four
// scores of a tile with two 16-byte loads, and the items advance by the
// number of groups without divisions, two items' loads issued before either
// is binned.
constexpr int HIST_WIN = 48 * 1024;

__device__ __forceinline__ void hist_add(df x, int i, int j, int L, const BinC& B, int nbcap, int wbase, int nwin,
                                         unsigned int* sh, unsigned long long* obs, int* status) {
  if (!(i < j && j < L)) return;
  int bin = bin_clamped(x, B);
  if (bin < 0 || bin >= nbcap) { atomicExch(status, 4); return; }
  const int rel = bin - wbase;
  if (rel >= 0 && rel < nwin) atomicAdd(sh + rel, 1u);
  else                        atomicAdd(obs + bin, 1ull);
}

__global__ void __launch_bounds__(1024)
k_hist(const float2* __restrict__ cov, int64_t slot_stride, const TileRC* __restrict__ tiles, int ntiles, int nslots,
       int L, BinC B, int nbcap, int wbase, int nwin, unsigned long long* __restrict__ obs, int* __restrict__ status) {
  extern __shared__ unsigned int sh[];
  for (int k = threadIdx.x; k < nwin; k += blockDim.x) sh[k] = 0u;
  __syncthreads();
  // group vb of G = gridDim.x * R groups; its item (slot, t) advances by
  // G = gs ntiles + gt
  const int R = blockDim.x >> 8, tid = threadIdx.x & 255;
  const int vb = blockIdx.x * R + (threadIdx.x >> 8);
  const int G = gridDim.x * R, gs = G / ntiles, gt = G - gs * ntiles;
  int slot = vb / ntiles, t = vb - slot * ntiles;
  auto advance = [&](int& sl, int& tt) { tt += gt; sl += gs; if (tt >= ntiles) { tt -= ntiles; sl++; } };
  // this thread's scores of a tile: p = 2 (tid + 256 k) + h, k, h in {0, 1}
  while (slot < nslots) {
    int slot2 = slot, t2 = t;
    advance(slot2, t2);
    const bool two = slot2 < nslots;
    float4 v[2][2];
    const float4* V0 = reinterpret_cast<const float4*>(cov + slot * slot_stride + (int64_t)t * TPP);
#pragma unroll
    for (int k = 0; k < 2; k++) v[0][k] = V0[tid + 256 * k];
    if (two) {
      const float4* V1 = reinterpret_cast<const float4*>(cov + slot2 * slot_stride + (int64_t)t2 * TPP);
#pragma unroll
      for (int k = 0; k < 2; k++) v[1][k] = V1[tid + 256 * k];
    }
#pragma unroll
    for (int u = 0; u < 2; u++) {
      if (u == 1 && !two) break;
      const TileRC tr = tiles[u ? t2 : t];
#pragma unroll
      for (int k = 0; k < 2; k++) {
        const int p = 2 * (tid + 256 * k), a = p >> 5, b = p & 31;
        const int i = tr.I * TP + a, j = tr.J * TP + b;
        hist_add({v[u][k].x, v[u][k].y}, i, j, L, B, nbcap, wbase, nwin, sh, obs, status);
        hist_add({v[u][k].z, v[u][k].w}, i, j + 1, L, B, nbcap, wbase, nwin, sh, obs, status);
      }
    }
    slot = slot2; t = t2;
    advance(slot, t);
  }
  __syncthreads();
  for (int k = threadIdx.x; k < nwin; k += blockDim.x)
    if (sh[k]) atomicAdd(obs + wbase + k, (unsigned long long)sh[k]);
}

// E-value of every pair (cov2evalue at src/covariation.c:2369-2400 with
// Nc = 1, times the number of tests) and the compacted hit list.  The FP64
// work per pair is one multiply: the quotients of the tail branch are a
// table (ptail = tail / Nc, divided on the host), the comparisons of x with
// phi and xmax are decided on x.hi against float brackets two ulps either
// side (FP64 only inside them), and E < thresh is compared on the bit
// patterns (non-negative doubles order as their bits).
struct EvalCmp {
  float phi_dn, phi_up, xmax_dn, xmax_up;   // x.hi < dn: x < y; x.hi > up: x > y
  long long thresh_bits;
  int all;                                   // thresh > 1000: every pair is listed
};

__device__ __forceinline__ bool ge_df(df x, float dn, float up, double y) {
  if (x.hi > up) return true;
  if (x.hi < dn) return false;
  return df_to_d(x) >= y;
}

__global__ void __launch_bounds__(256)
k_evalue(const float2* __restrict__ cov, const TileRC* __restrict__ tiles, int ntiles, int L, EvalTables T, BinC B,
         EvalCmp K, double* __restrict__ evt, int* __restrict__ nhits, int hitcap, int* __restrict__ hi,
         int* __restrict__ hj, double* __restrict__ hsc, double* __restrict__ hE, double* __restrict__ hp) {
  const int t = blockIdx.x, tid = threadIdx.x;
  const TileRC tr = tiles[t];
  const float2* V = cov + (int64_t)t * TPP;
  for (int k = 0; k < 4; k++) {
    const int p = tid + 256 * k, a = p >> 5, b = p & 31;
    const int i = tr.I * TP + a, j = tr.J * TP + b;
    double E = INFINITY;
    if (i < j && j < L) {
      const df xv = ld_df(V + p);
      const int icov = bin_df(xv, B);
      double pv;
      if (T.sf && icov >= 2 * T.nb - 1)                     pv = T.sf[2 * T.nb - 1];
      else if (T.sf && ge_df(xv, K.phi_dn, K.phi_up, T.phi)) pv = T.sf[max(icov + 1, 0)];
      else if (ge_df(xv, K.xmax_dn, K.xmax_up, T.xmax))      pv = T.pNc;
      else if (icov <= T.imax) {
        const int ic = (icov < T.imin) ? T.imin : icov;
        pv = (ic >= T.imax - 1) ? T.pNc : T.ptail[ic];
      } else pv = INFINITY;
      E = pv * T.Nt;
      const long long eb = __double_as_longlong(E);
      const bool below = (eb >= 0) ? (eb < K.thresh_bits) : (E < T.thresh);
      if (below || K.all) {
        const int h = atomicAdd(nhits, 1);
        if (h < hitcap) { hi[h] = i; hj[h] = j; hsc[h] = df_to_d(xv); hE[h] = E; hp[h] = pv; }
      }
    }
    if (evt) evt[(int64_t)t * TPP + p] = E;
  }
}

// tile-packed -> full symmetric L x L (diagonal = diag)
__device__ __forceinline__ double to_d(double v) { return v; }
__device__ __forceinline__ double to_d(float2 v) { return (double)v.x + (double)v.y; }

template <typename T>
__global__ void __launch_bounds__(256)
k_untile(const T* __restrict__ tilev, const TileRC* __restrict__ tiles, int L, double diag, double* __restrict__ full) {
  const int t = blockIdx.x, tid = threadIdx.x;
  const TileRC tr = tiles[t];
  __shared__ double s[TP][TP + 1];
  for (int k = 0; k < 4; k++) {
    const int p = tid + 256 * k, a = p >> 5, b = p & 31;
    s[a][b] = to_d(tilev[(int64_t)t * TPP + p]);
  }
  __syncthreads();
  for (int k = 0; k < 4; k++) {
    const int p = tid + 256 * k, a = p >> 5, b = p & 31;
    // upper: row i = I*TP + a, col j = J*TP + b
    int i = tr.I * TP + a, j = tr.J * TP + b;
    if (i < L && j < L) {
      if (i < j) full[(int64_t)i * L + j] = s[a][b];
      else if (i == j) full[(int64_t)i * L + j] = diag;
    }
    // lower: row J*TP + a, col I*TP + b holds s[b][a]
    i = tr.J * TP + a; j = tr.I * TP + b;
    if (i < L && j < L && j < i) full[(int64_t)i * L + j] = s[b][a];
  }
}

// full symmetric L x L (host layout) -> tile-packed upper triangle
__global__ void __launch_bounds__(256)
k_tile(const double* __restrict__ full, const TileRC* __restrict__ tiles, int L, float2* __restrict__ tilev) {
  const int t = blockIdx.x, tid = threadIdx.x;
  const TileRC tr = tiles[t];
  for (int k = 0; k < 4; k++) {
    const int p = tid + 256 * k, a = p >> 5, b = p & 31;
    const int i = tr.I * TP + a, j = tr.J * TP + b;
    st_df(tilev + (int64_t)t * TPP + p, df_of((i < j && j < L) ? full[(int64_t)i * L + j] : 0.0));
  }
}

// per-tile row/column sums of a tile-packed score matrix (for APC/ASC of a
// matrix handed in by the caller)
__global__ void __launch_bounds__(256)
k_tile_rowsums(const float2* __restrict__ tilev, const TileRC* __restrict__ tiles, int nT, int L,
               double* __restrict__ part1) {
  const int t = blockIdx.x, tid = threadIdx.x;
  const TileRC tr = tiles[t];
  df v[4][1];
#pragma unroll
  for (int k = 0; k < 4; k++) {
    const int p = tid + 256 * k, a = p >> 5, b = p & 31;
    const int i = tr.I * TP + a, j = tr.J * TP + b;
    v[k][0] = (i < j && j < L) ? ld_df(tilev + (int64_t)t * TPP + p) : df{0.f, 0.f};
  }
  tile_rowcol_store<1>(v, part1, nT, tr.I, tr.J);
}

// ------------------------------------------------------------------------
// launchers
// ------------------------------------------------------------------------
cudaError_t launch_count_simt(const uint8_t* ax, int64_t slot_stride, const float* w, bool unit, int N, int Lp,
                              const TileRC* tiles, int ntiles, int nslots, float* cnt, cudaStream_t st) {
  dim3 grid(ntiles, nslots);
  if (unit) k_count_simt<true><<<grid, 256, 0, st>>>(ax, slot_stride, w, N, Lp, tiles, ntiles, cnt);
  else      k_count_simt<false><<<grid, 256, 0, st>>>(ax, slot_stride, w, N, Lp, tiles, ntiles, cnt);
  return cudaGetLastError();
}

cudaError_t launch_pair_marg(const float* cnt, int L, const TileRC* tiles, int ntiles, int nT, int nslots,
                             double* part4, double* partR, cudaStream_t st) {
  k_pair_marg<<<dim3(ntiles, nslots), 256, 0, st>>>(cnt, L, tiles, ntiles, nT, part4, partR);
  return cudaGetLastError();
}

cudaError_t launch_pm_final(const double* part4, const double* partR, int L, int Lp, int nT, int nslots, double* pm,
                            float2* pmdf, double* mpc, double* meanp, int* status, cudaStream_t st) {
  k_pm_final<<<dim3((L + 127) / 128, nslots), 128, 0, st>>>(part4, partR, L, Lp, nT, pm, pmdf, mpc, status);
  k_meanp<<<nslots, 256, 0, st>>>(mpc, L, Lp, meanp);
  return cudaGetLastError();
}

cudaError_t launch_ps(const uint8_t* ax, int64_t slot_stride, const double* w, int N, int L, int Lp, int nslots,
                      double* ps, cudaStream_t st) {
  k_ps<<<dim3((L + 127) / 128, nslots), 128, 0, st>>>(ax, slot_stride, w, N, L, Lp, ps);
  return cudaGetLastError();
}

cudaError_t launch_stats(const StatsArgs& A, int nslots, cudaStream_t st) {
  // the smallest cell-loop variant covering the requested statistics
  unsigned cf = 0;
  if (A.stats & (S_GT | S_MI | S_MIr | S_MIg)) cf |= CF_G;
  if (A.stats & S_CHI) cf |= CF_CHI;
  if (A.stats & S_OMES) cf |= CF_OMES;
  if (A.stats & S_MIr) cf |= CF_H;
  const dim3 grid(A.ntiles, nslots);
  if (cf == 0 || cf == CF_G)          k_stats<CF_G><<<grid, 256, 0, st>>>(A);
  else if (cf == CF_CHI)              k_stats<CF_CHI><<<grid, 256, 0, st>>>(A);
  else if (cf == (CF_G | CF_CHI))     k_stats<CF_G | CF_CHI><<<grid, 256, 0, st>>>(A);
  else                                k_stats<CF_ALL><<<grid, 256, 0, st>>>(A);
  return cudaGetLastError();
}

cudaError_t launch_rafs(const float2* raf, float2* out, int64_t sin, int64_t sout, const TileRC* tiles,
                        const int* tile_index, int ntiles, int nT, int L, int nslots, double* part1, int64_t pstride,
                        cudaStream_t st) {
  k_rafs<<<dim3(ntiles, nslots), 256, 0, st>>>(raf, out, sin, sout, tiles, tile_index, ntiles, nT, L, part1, pstride);
  return cudaGetLastError();
}

cudaError_t launch_apc(float2* cov, const double* part1, double* colx, float2* colxf, double* avg, float4* apcf,
                       CorrTypes ct, const TileRC* tiles, int ntiles, int nT, int L, int Lp, int nsq, double* tmin,
                       double* tmax, double* mm, int* status, cudaStream_t st) {
  k_apc_colx<<<dim3((L + 255) / 256, nsq), 256, 0, st>>>(part1, nT, L, Lp, colx, colxf);
  k_apc_avg<<<nsq, 256, 0, st>>>(colx, L, Lp, avg, apcf);
  const int nblk = (ntiles + APC_TILES - 1) / APC_TILES;
  k_apc_apply<<<dim3(nblk, nsq), 256, 0, st>>>(cov, colxf, avg, apcf, ct, tiles, ntiles, L, Lp, tmin, tmax, status);
  k_reduce_minmax<<<nsq, 256, 0, st>>>(tmin, tmax, nblk, mm);
  return cudaGetLastError();
}

cudaError_t launch_minmax(const float2* cov, const TileRC* tiles, int ntiles, int L, int nsq, double* tmin,
                          double* tmax, double* mm, cudaStream_t st) {
  k_tile_minmax<<<dim3(ntiles, nsq), 256, 0, st>>>(cov, tiles, ntiles, L, tmin, tmax);
  k_reduce_minmax<<<nsq, 256, 0, st>>>(tmin, tmax, ntiles, mm);
  return cudaGetLastError();
}

cudaError_t launch_hist(const float2* cov, int64_t slot_stride, const TileRC* tiles, int ntiles, int L, int nslots,
                        double bmin, double w, int nbcap, int wbase, unsigned long long* obs, int* status,
                        cudaStream_t st) {
  const BinC B = make_binc(bmin, w);
  wbase = std::max(0, std::min(wbase, nbcap - 1));
  const int nwin = std::min(HIST_WIN, nbcap - wbase);
  // once per process (thread-safe static initialisation)
  static const bool attr = [] {
    cudaFuncSetAttribute(k_hist, cudaFuncAttributeMaxDynamicSharedMemorySize, HIST_WIN * 4);
    return true;
  }();
  (void)attr;
  int dev = 0, nsm = 152, occ = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  // 256-thread CTAs while four or more fit on an SM, else 1024-thread ones
  int threads = 256;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_hist, 256, (size_t)nwin * 4) != cudaSuccess || occ < 4) {
    threads = 1024;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_hist, 1024, (size_t)nwin * 4) != cudaSuccess || occ < 1)
      occ = 1;
  }
  const int R = threads / 256;
  const int64_t items = (int64_t)ntiles * nslots;
  if (items >= ((int64_t)1 << 30)) return cudaErrorInvalidValue;   // the kernel indexes items in 32 bits
  // whole CTAs, every group with at least one item
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(items / R, (int64_t)nsm * occ));
  k_hist<<<grid, threads, (size_t)nwin * 4, st>>>(cov, slot_stride, tiles, ntiles, nslots, L, B, nbcap, wbase, nwin,
                                                  obs, status);
  return cudaGetLastError();
}

cudaError_t launch_evalue(const float2* cov, const TileRC* tiles, int ntiles, int L, const EvalTables& T, double* evt,
                          int* nhits, int hitcap, int* hi, int* hj, double* hsc, double* hE, double* hp,
                          cudaStream_t st) {
  auto bracket = [](double y, float& dn, float& up) {
    const float f = (float)y;
    up = std::nextafter(std::nextafter(f, INFINITY), INFINITY);
    dn = std::nextafter(std::nextafter(f, -INFINITY), -INFINITY);
  };
  EvalCmp K;
  bracket(T.phi, K.phi_dn, K.phi_up);
  bracket(T.xmax, K.xmax_dn, K.xmax_up);
  // non-negative E < thresh as bit patterns; a negative thresh admits none
  K.thresh_bits = 0;
  if (T.thresh > 0.0) std::memcpy(&K.thresh_bits, &T.thresh, sizeof(double));
  K.all = (T.thresh > 1000.0) ? 1 : 0;
  k_evalue<<<ntiles, 256, 0, st>>>(cov, tiles, ntiles, L, T, make_binc(T.bmin, T.w), K, evt, nhits, hitcap, hi, hj,
                                   hsc, hE, hp);
  return cudaGetLastError();
}

cudaError_t launch_tile(const double* full, const TileRC* tiles, int ntiles, int L, float2* tilev, cudaStream_t st) {
  k_tile<<<ntiles, 256, 0, st>>>(full, tiles, L, tilev);
  return cudaGetLastError();
}

cudaError_t launch_tile_rowsums(const float2* tilev, const TileRC* tiles, int ntiles, int nT, int L, double* part1,
                                cudaStream_t st) {
  k_tile_rowsums<<<ntiles, 256, 0, st>>>(tilev, tiles, nT, L, part1);
  return cudaGetLastError();
}

cudaError_t launch_untile(const float2* tilev, const TileRC* tiles, int ntiles, int L, double diag, double* full,
                          cudaStream_t st) {
  k_untile<float2><<<ntiles, 256, 0, st>>>(tilev, tiles, L, diag, full);
  return cudaGetLastError();
}

cudaError_t launch_untile(const double* tilev, const TileRC* tiles, int ntiles, int L, double diag, double* full,
                          cudaStream_t st) {
  k_untile<double><<<ntiles, 256, 0, st>>>(tilev, tiles, L, diag, full);
  return cudaGetLastError();
}

}  // namespace covgpu
