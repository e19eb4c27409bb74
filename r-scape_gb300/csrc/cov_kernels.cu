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
#include "cov_df.cuh"
#include "cov_kernels.h"
#include "cov_batch.h"

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
// value-scaled one-hot (j side) vectors; every pair then takes 16 FMAs per
// sequence.  The j-side values are integers (1, or one weight limb of at
// most 2^b - 1 with N (2^b - 1) < 2^24), so every accumulator holds an exact
// integer.
//   MODE_UNIT   unit weights (RAF): FP32 counts, one plane
//   MODE_EQUAL  all weights equal to w: the unit count times w as a
//               double-float (unit_count)
//   MODE_LIMBS  three weight limbs, counted one after the other (limb 2,
//               then 1, then 0) and combined exactly as limb_count does: the
//               partial result of the previous limb is kept in the output
//               planes, which only this thread touches
// Double-float counts go to two planes per cell, [slot][tile][16][hi|lo][TPP].
// ------------------------------------------------------------------------
enum CountMode { MODE_UNIT = 0, MODE_EQUAL = 1, MODE_LIMBS = 3 };

template <int MODE>
__device__ __forceinline__ void count_simt_body(
    const GridIdx g, const uint8_t* __restrict__ ax, int64_t slot_stride, const float* __restrict__ limbs, int N,
    int Lp,
             const TileRC* __restrict__ tiles, int ntiles, float* __restrict__ cnt, float B, float s_hi, float s_lo) {
  __shared__ float4 ohi[32][TP];
  __shared__ float4 whj[32][TP];
  const int t = g.x, slot = g.y, tid = threadIdx.x;
  const TileRC tr = tiles[t];
  const uint8_t* A = ax + (int64_t)slot * slot_stride;
  const int ty = tid >> 4, tx = tid & 15;
  constexpr int NPASS = (MODE == MODE_LIMBS) ? 3 : 1;
  const int64_t tbase = (int64_t)slot * ntiles + t;
#pragma unroll 1
  for (int pass = 0; pass < NPASS; pass++) {
    const int limb = NPASS - 1 - pass;     // limbs 2, 1, 0
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
          val = (half && MODE == MODE_LIMBS) ? limbs[(int64_t)limb * N + seq] : 1.f;
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
              for (int y = 0; y < 4; y++)
                acc[a * 2 + b][x * 4 + y] = fmaf(iv[a][x], jv[b][y], acc[a * 2 + b][x * 4 + y]);
      }
      __syncthreads();
    }
    if (MODE == MODE_UNIT) {
      float* out = cnt + tbase * 16 * TPP;
#pragma unroll
      for (int a = 0; a < 2; a++)
#pragma unroll
        for (int c = 0; c < 16; c++)
          *reinterpret_cast<float2*>(out + c * TPP + (2 * ty + a) * TP + 2 * tx) =
              make_float2(acc[a * 2 + 0][c], acc[a * 2 + 1][c]);
      continue;
    }
    float* out = cnt + tbase * 32 * TPP;
#pragma unroll
    for (int a = 0; a < 2; a++)
#pragma unroll
      for (int c = 0; c < 16; c++) {
        float2* hp = reinterpret_cast<float2*>(out + (2 * c) * TPP + (2 * ty + a) * TP + 2 * tx);
        float2* lp = reinterpret_cast<float2*>(out + (2 * c + 1) * TPP + (2 * ty + a) * TP + 2 * tx);
        df r[2];
#pragma unroll
        for (int b = 0; b < 2; b++) {
          const float d = acc[a * 2 + b][c];
          if (MODE == MODE_EQUAL) {
            r[b] = unit_count(d, s_hi, s_lo);
          } else if (limb == 2) {
            r[b] = {d * (B * B), 0.f};                       // c2
          } else if (limb == 1) {
            const float2 h = *hp;
            r[b] = two_sum(b ? h.y : h.x, d * B);           // s1 = c2 + c1
          } else {
            const float2 h = *hp, l = *lp;
            const df s2 = two_sum(b ? h.y : h.x, d);        // s1.hi + c0
            const df q = fast_two_sum(s2.hi, (b ? l.y : l.x) + s2.lo);
            r[b] = {q.hi * s_hi, q.lo * s_hi};               // times 2^-E
          }
        }
        *hp = make_float2(r[0].hi, r[1].hi);
        *lp = make_float2(r[0].lo, r[1].lo);
      }
  }
}
template <int MODE>
__global__ void __launch_bounds__(256, 2)
k_count_simt(const uint8_t* __restrict__ ax, int64_t slot_stride, const float* __restrict__ limbs, int N, int Lp,
             const TileRC* __restrict__ tiles, int ntiles, float* __restrict__ cnt, float B, float s_hi, float s_lo) {
  count_simt_body<MODE>(native_grid(), ax, slot_stride, limbs, N, Lp, tiles, ntiles, cnt, B, s_hi, s_lo);
}

// constants of the bin function, split on the host
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
// row i gains (4e-10 + sum_y C(x,y)) / Z and column j gains
// (4e-10 + sum_x C(x,y)) / Z, Z = 16e-10 + nseff (the prior of
// src/correlators.c:1713 and the normalisation of :1758).  The counts are
// double-float; each contribution is a double-float quotient and the sums
// over partners are double-float (stored as FP64), so pm keeps ~1e-13.  Also
// the upper-triangle row sums of nseff for the CCF column means.
__device__ __forceinline__ df cnt_df(const float* __restrict__ C, int q, int p) {
  return {C[(2 * q) * TPP + p], C[(2 * q + 1) * TPP + p]};
}

__device__ __forceinline__ void pair_marg_body(
    const GridIdx g, const float* __restrict__ cnt, int L, const TileRC* __restrict__ tiles, int ntiles, int nT,
            double* __restrict__ part4, double* __restrict__ partR) {
  const int t = g.x, slot = g.y, tid = threadIdx.x;
  const TileRC tr = tiles[t];
  const float* C = cnt + ((int64_t)slot * ntiles + t) * 32 * TPP;
  // one buffer for the row contributions, then for the column ones
  __shared__ float2 sb[4][TP][TP + 1];
  __shared__ float2 sn[TP][TP + 1];
  df colc[4][4];
#pragma unroll
  for (int k = 0; k < 4; k++) {
    const int p = tid + 256 * k, a = p >> 5, b = p & 31;
    const int i = tr.I * TP + a, j = tr.J * TP + b;
    df row[4], col[4];
#pragma unroll
    for (int x = 0; x < 4; x++) { row[x] = {0.f, 0.f}; col[x] = {0.f, 0.f}; }
#pragma unroll
    for (int q = 0; q < 16; q++) {
      const df c = cnt_df(C, q, p);
      df_acc(row[q >> 2], c);
      df_acc(col[q & 3], c);
    }
    df ne = {0.f, 0.f};
#pragma unroll
    for (int x = 0; x < 4; x++) { row[x] = df_norm(row[x]); col[x] = df_norm(col[x]); df_acc(ne, row[x]); }
    ne = df_norm(ne);
    const bool pair = (i < j) && (j < L);
    const bool ok = pair && (ne.hi > 0.f);
    const df iZ = df_recip(df_add_f(ne, 1.6e-9f));
#pragma unroll
    for (int x = 0; x < 4; x++) {
      const df r = ok ? df_mul(df_add_f(row[x], 4e-10f), iZ) : df{0.f, 0.f};
      colc[k][x] = ok ? df_mul(df_add_f(col[x], 4e-10f), iZ) : df{0.f, 0.f};
      sb[x][a][b] = make_float2(r.hi, r.lo);
    }
    sn[a][b] = pair ? make_float2(ne.hi, ne.lo) : make_float2(0.f, 0.f);
  }
  __syncthreads();
  // threads 0-127: row sums over b, then column sums over a, one thread per
  // (state, line) adding its 32 entries in order; rows go to part[I][J],
  // columns to part[J][I], both to part[I][I] on a diagonal tile.
  // threads 128-159: the nseff row sums.
  double* P4 = part4 + (int64_t)slot * nT * nT * TP * 4;
  double* PR = partR + (int64_t)slot * nT * nT * TP;
  const bool diag = (tr.I == tr.J);
  const int c4 = (tid >> 5) & 3, line = tid & 31;
  df rsum = {0.f, 0.f};
  if (tid < 128) {
    for (int b = 0; b < TP; b++) df_acc(rsum, {sb[c4][line][b].x, sb[c4][line][b].y});
    rsum = df_norm(rsum);
    if (!diag) P4[(((int64_t)tr.I * nT + tr.J) * TP + line) * 4 + c4] = df_to_d(rsum);
  } else if (tid < 128 + TP) {
    df ns = {0.f, 0.f};
    for (int b = 0; b < TP; b++) df_acc(ns, {sn[line][b].x, sn[line][b].y});
    PR[((int64_t)tr.I * nT + tr.J) * TP + line] = df_to_d(df_norm(ns));
    if (!diag) PR[((int64_t)tr.J * nT + tr.I) * TP + line] = 0.0;   // the column sums of nseff are not used
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < 4; k++) {
    const int p = tid + 256 * k, a = p >> 5, b = p & 31;
#pragma unroll
    for (int x = 0; x < 4; x++) sb[x][a][b] = make_float2(colc[k][x].hi, colc[k][x].lo);
  }
  __syncthreads();
  if (tid < 128) {
    df csum = {0.f, 0.f};
    for (int a = 0; a < TP; a++) df_acc(csum, {sb[c4][a][line].x, sb[c4][a][line].y});
    csum = df_norm(csum);
    if (!diag) P4[(((int64_t)tr.J * nT + tr.I) * TP + line) * 4 + c4] = df_to_d(csum);
    else       P4[(((int64_t)tr.I * nT + tr.I) * TP + line) * 4 + c4] = df_to_d(df_add(rsum, csum));
  }
}
__global__ void __launch_bounds__(256)
k_pair_marg(const float* __restrict__ cnt, int L, const TileRC* __restrict__ tiles, int ntiles, int nT,
            double* __restrict__ part4, double* __restrict__ partR) {
  pair_marg_body(native_grid(), cnt, L, tiles, ntiles, nT, part4, partR);
}

// pm[c][x] = normalise(sum over every tile touching column c); one thread
// per column.  pmdf is pm as a double-float; lpi[c][x] = {ln pm, 1/pm} as
// double-floats (FP64 log and division, 0 where pm = 0) for the pair
// statistics.  mpc[c][x] = pm[c][x] * (sum_{j>c} nseff[c][j]) feeds the CCF
// column means (src/correlators.c:1030-1036).
__device__ __forceinline__ void pm_final_body(
    const GridIdx g, const double* __restrict__ part4, const double* __restrict__ partR, int L, int Lp, int nT,
                           double* __restrict__ pm, float2* __restrict__ pmdf, float4* __restrict__ lpi,
                           double* __restrict__ mpc, int* __restrict__ status) {
  const int slot = g.y;
  const int c = g.x * blockDim.x + threadIdx.x;
  if (c >= L) return;
  const double* P = part4 + (int64_t)slot * nT * nT * TP * 4;
  const double* R = partR + (int64_t)slot * nT * nT * TP;
  const int I = c / TP, a = c % TP;
  double m[4] = {0, 0, 0, 0}, rs = 0.0;
  for (int K = 0; K < nT; K++) {
    const double2* v = reinterpret_cast<const double2*>(P + (((int64_t)I * nT + K) * TP + a) * 4);
    const double2 v0 = v[0], v1 = v[1];
    m[0] += v0.x; m[1] += v0.y; m[2] += v1.x; m[3] += v1.y;
    rs += R[((int64_t)I * nT + K) * TP + a];
  }
  const double sum = m[0] + m[1] + m[2] + m[3];
#pragma unroll
  for (int x = 0; x < 4; x++) m[x] = (sum != 0.0) ? m[x] / sum : 0.25;
  if (fabs(m[0] + m[1] + m[2] + m[3] - 1.0) > 1e-6) atomicExch(status, 2);
#pragma unroll
  for (int x = 0; x < 4; x++) {
    const int64_t o = ((int64_t)slot * Lp + c) * 4 + x;
    pm[o] = m[x];
    st_df(pmdf + o, df_of(m[x]));
    const df l = df_of(m[x] > 0.0 ? log(m[x]) : 0.0), r = df_of(m[x] > 0.0 ? 1.0 / m[x] : 0.0);
    lpi[o] = make_float4(l.hi, l.lo, r.hi, r.lo);
    mpc[o] = rs * m[x];
  }
}
__global__ void k_pm_final(const double* __restrict__ part4, const double* __restrict__ partR, int L, int Lp, int nT,
                           double* __restrict__ pm, float2* __restrict__ pmdf, float4* __restrict__ lpi,
                           double* __restrict__ mpc, int* __restrict__ status) {
  pm_final_body(native_grid(), part4, partR, L, Lp, nT, pm, pmdf, lpi, mpc, status);
}

__device__ __forceinline__ void meanp_body(
    const GridIdx g, const double* __restrict__ mpc, int L, int Lp, double* __restrict__ meanp) {
  const int slot = g.x;
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
__global__ void k_meanp(const double* __restrict__ mpc, int L, int Lp, double* __restrict__ meanp) {
  meanp_body(native_grid(), mpc, L, Lp, meanp);
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
// Statistics, all per-pair arithmetic in double-float.  With c' = 1e-10 + C
// (the prior of src/correlators.c:1713), Z = sum c' = nseff + 16e-10 and
// pp = c'/Z (:1758), S = sum c' ln c', R_x = sum_y c'_xy, K_y = sum_x c'_xy:
//   MI   = sum pp (ln pp - ln pm_i - ln pm_j)
//        = (S - Z ln Z - sum_x R_x ln pm_i(x) - sum_y K_y ln pm_j(y)) / Z
//   GT   = 2 sum o ln(o/e), o = nseff pp, e = nseff pm_i pm_j  =  2 nseff MI
//   H    = -sum pp ln pp = ln Z - S/Z                       (MIr = MI / H)
//   MIg  = MI - ngap / nseff
//   CHI  = sum (o - e)^2 / e = (nseff / Z^2) sum_x T_x / pm_i(x) - nseff,
//          T_x = sum_y c'_xy^2 / pm_j(y)       (sum o = sum e = nseff)
//   OMES = sum (o - e)^2 / nseff
//        = nseff (sum c'^2 / Z^2 - (2/Z) sum_x pm_i(x) V_x + |pm_i|^2 |pm_j|^2),
//          V_x = sum_y c'_xy pm_j(y)
// These are the reference's C16 sums (src/correlators.c:92-122, 224-252,
// 359-390, 536-561, 659-690, 792-822) regrouped so that a cell costs one
// double-float logarithm and a few products.  Every cell enters: nseff > 0
// makes every pm of both columns positive (the partner contributes at least
// the prior).  The regrouped sums cancel at most log2(Z ln Z / |Z MI|) of
// the 48 bits, which leaves the scores within ~1e-11 relative of FP64 for
// the alignments of this path.  The C2 class (merged allowed / other cells,
// :137-168, 269-301, 426-463, 575-605, 705-736, 838-866) and the GT CWC
// class (:393-423) are formed from the same pieces on their cells; pairs
// with nseff = 0 (prior only, pp = 1/16) are FP64.
// ------------------------------------------------------------------------
struct PairOut { df chi, gt, mi, mir, mig, omes, raf, ccf; };

__device__ __forceinline__ df pick_df(const PairOut& o, int k) {
  switch (k) {
    case 0: return o.chi;
    case 1: return o.gt;
    case 2: return o.mi;
    case 3: return o.mir;
    case 4: return o.mig;
    case 5: return o.omes;
    case 6: return o.raf;
    case 8: return o.ccf;
  }
  return {0.f, 0.f};
}

// per-cell terms a k_stats variant computes: the logarithm family (GT, MI,
// MIr, MIg), CHI, OMES
enum CellF : unsigned { CF_G = 1u, CF_CHI = 2u, CF_OMES = 4u, CF_ALL = 7u };

__device__ __forceinline__ bool above_h(df H) {   // H > 1e-2 as the FP64 value would compare
  return (H.hi > 0.0100001f) || (H.hi > 0.0099999f && df_to_d(H) > 1e-2);
}

template <unsigned CF>
__device__ __forceinline__ void pair_stats(const StatsArgs& A, const df (&c)[16], const float (&uc)[16],
                                           bool have_uc, const float2* pmi, const float2* pmj, const float4* lpi,
                                           const float4* lpj, const double* pmid, const double* pmjd,
                                           const double* meanp, const float4* tab, PairOut& out) {
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
  df ne;
  {
    df z = {0.f, 0.f};
#pragma unroll
    for (int q = 0; q < 16; q++) df_acc(z, c[q]);
    ne = df_norm(z);
  }
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
    out.chi = out.gt = out.omes = df{0.f, 0.f};
    out.mi = df_of(mi); out.mir = df_of((hh > 1e-2) ? mi / hh : 0.0); out.mig = df_of(mi);
    return;
  }

  const df Z = df_add_f(ne, 16.f * 1e-10f);
  const df iZ = df_recip(Z);
  const df wt = {A.wtot.x, A.wtot.y};
  if (A.cls == 0) {
    // ---- C16: one pass over the cells ----
    df R[4], K[4], T[4], V[4], Sx = {0.f, 0.f}, W = {0.f, 0.f};
#pragma unroll
    for (int x = 0; x < 4; x++) R[x] = K[x] = T[x] = V[x] = df{0.f, 0.f};
#pragma unroll
    for (int x = 0; x < 4; x++)
#pragma unroll
      for (int y = 0; y < 4; y++) {
        const df cp = df_add_f(c[x * 4 + y], 1e-10f);
        df_acc(R[x], cp);
        df_acc(K[y], cp);
        if (CF & CF_G) df_acc(Sx, df_mul_u(cp, df_log(cp, tab)));
        if (CF & (CF_CHI | CF_OMES)) {
          const df sq = df_sqr_u(cp);
          if (CF & CF_CHI) df_acc(T[x], df_mul_u(sq, {lpj[y].z, lpj[y].w}));
          if (CF & CF_OMES) { df_acc(W, sq); df_acc(V[x], df_mul_u(cp, {pmj[y].x, pmj[y].y})); }
        }
      }
    if (CF & CF_G) {
      const df Sn = df_norm(Sx);
      const df lnZ = df_log(Z, tab);
      df P = {0.f, 0.f};
#pragma unroll
      for (int x = 0; x < 4; x++) {
        df_acc(P, df_mul_u(df_norm(R[x]), {lpi[x].x, lpi[x].y}));
        df_acc(P, df_mul_u(df_norm(K[x]), {lpj[x].x, lpj[x].y}));
      }
      const df Mn = df_sub(df_sub(Sn, df_mul(Z, lnZ)), df_norm(P));
      const df mi = df_mul(Mn, iZ);
      out.mi = mi;
      out.gt = df_scale(df_mul(ne, mi), 2.f);
      // the mask is the same for every thread: no divergence
      if (S & S_MIr) {
        const df H = df_sub(lnZ, df_mul(Sn, iZ));
        out.mir = above_h(H) ? df_div(mi, H) : df{0.f, 0.f};
      }
      if (S & S_MIg) out.mig = df_sub(mi, df_div(df_sub(wt, ne), ne));
    }
    if (CF & CF_CHI) {
      df Q = {0.f, 0.f};
#pragma unroll
      for (int x = 0; x < 4; x++) df_acc(Q, df_mul_u(df_norm(T[x]), {lpi[x].z, lpi[x].w}));
      out.chi = df_sub(df_mul(df_mul(ne, df_mul(iZ, iZ)), df_norm(Q)), ne);
    }
    if (CF & CF_OMES) {
      df U = {0.f, 0.f}, Ai = {0.f, 0.f}, Aj = {0.f, 0.f};
#pragma unroll
      for (int x = 0; x < 4; x++) {
        df_acc(U, df_mul_u({pmi[x].x, pmi[x].y}, df_norm(V[x])));
        df_acc(Ai, df_sqr_u({pmi[x].x, pmi[x].y}));
        df_acc(Aj, df_sqr_u({pmj[x].x, pmj[x].y}));
      }
      const df t1 = df_mul(df_norm(W), df_mul(iZ, iZ));
      const df t2 = df_scale(df_mul(df_norm(U), iZ), 2.f);
      const df t3 = df_mul(df_norm(Ai), df_norm(Aj));
      out.omes = df_mul(ne, df_add(df_sub(t1, t2), t3));
    }
  } else if (A.cls == 2) {
    // ---- GT, CWC: the allowed cells only ----
    df SA = {0.f, 0.f}, CA = {0.f, 0.f}, PA = {0.f, 0.f};
#pragma unroll
    for (int x = 0; x < 4; x++)
#pragma unroll
      for (int y = 0; y < 4; y++) {
        if (!(A.allow[x * 4 + y] > 0.f)) continue;
        const df cp = df_add_f(c[x * 4 + y], 1e-10f);
        df_acc(SA, df_mul_u(cp, df_log(cp, tab)));
        df_acc(CA, cp);
        df_acc(PA, df_mul_u(cp, df_add({lpi[x].x, lpi[x].y}, {lpj[y].x, lpj[y].y})));
      }
    const df lnZ = df_log(Z, tab);
    const df M = df_sub(df_sub(df_norm(SA), df_mul(lnZ, df_norm(CA))), df_norm(PA));
    out.gt = df_scale(df_mul(df_mul(ne, iZ), M), 2.f);
  } else {
    // ---- C2: allowed / not-allowed merged cells (e.g. src/correlators.c:426-458) ----
    df Cw = {0.f, 0.f}, Cn = {0.f, 0.f}, qw = {0.f, 0.f}, qn = {0.f, 0.f};
#pragma unroll
    for (int x = 0; x < 4; x++)
#pragma unroll
      for (int y = 0; y < 4; y++) {
        const df cp = df_add_f(c[x * 4 + y], 1e-10f);
        const df pq = df_mul_u({pmi[x].x, pmi[x].y}, {pmj[y].x, pmj[y].y});
        if (A.allow[x * 4 + y] > 0.f) { df_acc(Cw, cp); df_acc(qw, pq); }
        else                          { df_acc(Cn, cp); df_acc(qn, pq); }
      }
    Cw = df_norm(Cw); Cn = df_norm(Cn); qw = df_norm(qw); qn = df_norm(qn);
    const df pw = df_mul(Cw, iZ), pn = df_mul(Cn, iZ);
    const df lnZ = df_log(Z, tab);
    const bool hw = Cw.hi > 0.f, hn = Cn.hi > 0.f;   // the prior makes both positive
    const df lCw = hw ? df_sub(df_log(Cw, tab), lnZ) : df{0.f, 0.f};   // ln pw
    const df lCn = hn ? df_sub(df_log(Cn, tab), lnZ) : df{0.f, 0.f};   // ln pn
    const df lqw = (qw.hi > 0.f) ? df_log(qw, tab) : df{0.f, 0.f};
    const df lqn = (qn.hi > 0.f) ? df_log(qn, tab) : df{0.f, 0.f};
    df mi = {0.f, 0.f}, hh = {0.f, 0.f};
    if (hw && qw.hi > 0.f) mi = df_add(mi, df_mul(pw, df_sub(lCw, lqw)));
    if (hn && qn.hi > 0.f) mi = df_add(mi, df_mul(pn, df_sub(lCn, lqn)));
    out.gt = df_scale(df_mul(ne, mi), 2.f);
    out.mi = mi;
    if (S & S_MIr) {
      if (hw) hh = df_sub(hh, df_mul(pw, lCw));
      if (hn) hh = df_sub(hh, df_mul(pn, lCn));
      out.mir = above_h(hh) ? df_div(mi, hh) : df{0.f, 0.f};
    }
    if (S & S_MIg) out.mig = df_sub(mi, df_div(df_sub(wt, ne), ne));
    if (S & (S_CHI | S_OMES)) {
      df chi = {0.f, 0.f}, om = {0.f, 0.f};
      if (qw.hi > 0.f) {
        const df d = df_sub(pw, qw), d2 = df_mul(d, d);
        chi = df_add(chi, df_div(d2, qw)); om = df_add(om, d2);
      }
      if (qn.hi > 0.f) {
        const df d = df_sub(pn, qn), d2 = df_mul(d, d);
        chi = df_add(chi, df_div(d2, qn)); om = df_add(om, d2);
      }
      out.chi = df_mul(ne, chi);
      out.omes = df_mul(ne, om);
    }
  }
}

// One CTA per (tile, alignment), 256 threads, thread tid owns the pairs
// p = tid + 256k (row a = warp + 8k, column b = lane).  Each pair's scores
// go straight to the score planes and into a shared-memory copy of the
// tile; after the tile, one thread per (row, output) adds its row and one
// per (column, output) its column in double-float, in a fixed order, for the
// APC/ASC partials.
template <unsigned CF>
__device__ __forceinline__ void stats_body(
    const GridIdx g, StatsArgs A) {
  const int t = g.x, slot = g.y, tid = threadIdx.x;
  const TileRC tr = A.tiles[t];
  const float* C = A.cnt ? A.cnt + ((int64_t)slot * A.ntiles + t) * 32 * TPP : nullptr;
  const float* U = A.ucnt ? A.ucnt + ((int64_t)slot * A.ntiles + t) * 16 * TPP : nullptr;
  const double* pm = A.pm + (int64_t)slot * A.Lp * 4;
  const float2* pmdf = A.pmdf + (int64_t)slot * A.Lp * 4;
  const float4* lpi = A.lpi + (int64_t)slot * A.Lp * 4;
  const double* meanp = A.meanp + slot * 4;
  __shared__ float2 vs[MAXOUT][TP][TP + 1];   // the tile's scores, [q][a][b]
  __shared__ float4 tab[LOGTAB_TOT];
  static_assert(LOGTAB_TOT <= 256, "one table entry per thread");
  if (tid < LOGTAB_TOT) tab[tid] = A.logtab[tid];
  __syncthreads();
#pragma unroll 1
  for (int k = 0; k < 4; k++) {
    const int p = tid + 256 * k, a = p >> 5, b = p & 31;
    const int i = tr.I * TP + a, j = tr.J * TP + b;
    const bool valid = (i < j) && (j < A.L);
    df c[16];
    float uc[16];
#pragma unroll
    for (int q = 0; q < 16; q++) {
      c[q] = C ? df{C[(2 * q) * TPP + p], C[(2 * q + 1) * TPP + p]} : df{0.f, 0.f};
      uc[q] = (U && A.allow[q] > 0.f) ? U[q * TPP + p] : 0.f;   // RAF reads the allowed cells only
    }
    PairOut o;
    o.chi = o.gt = o.mi = o.mir = o.mig = o.omes = o.raf = o.ccf = df{0.f, 0.f};
    if (valid) {
      const int ii = i < A.L ? i : 0, jj = j < A.L ? j : 0;
      pair_stats<CF>(A, c, uc, U != nullptr, pmdf + ii * 4, pmdf + jj * 4, lpi + ii * 4, lpi + jj * 4, pm + ii * 4,
                     pm + jj * 4, meanp, tab, o);
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
template <unsigned CF>
__global__ void __launch_bounds__(256, 2)
k_stats(StatsArgs A) {
  stats_body<CF>(native_grid(), A);
}

// power_SPAIR_AddMI (src/power.c:201-218) for every pair i < j of one
// alignment, from its double-float counts: the pair probabilities pp =
// (1e-10 + C) / sum (the FP64 operations the host fill of mi->pp makes), then
// the Watson-Crick fraction pp(AU) + pp(UA) + pp(CG) + pp(GC), the wobble
// fraction pp(GU) + pp(UG) and the rest; written at the row-major index of
// (i, j) in the upper triangle
__global__ void __launch_bounds__(256)
k_pair_classes(const float* __restrict__ cnt, const TileRC* __restrict__ tiles, int L, double* __restrict__ wcf,
               double* __restrict__ wob, double* __restrict__ non) {
  const int t = blockIdx.x, tid = threadIdx.x;
  const TileRC tr = tiles[t];
  const float* C = cnt + (int64_t)t * 32 * TPP;
  for (int k = 0; k < 4; k++) {
    const int p = tid + 256 * k, a = p >> 5, b = p & 31;
    const int i = tr.I * TP + a, j = tr.J * TP + b;
    if (!(i < j && j < L)) continue;
    double c[16], sum = 0.0;
#pragma unroll
    for (int q = 0; q < 16; q++) {
      c[q] = __dadd_rn(1e-10, __dadd_rn((double)C[(2 * q) * TPP + p], (double)C[(2 * q + 1) * TPP + p]));
      sum = __dadd_rn(sum, c[q]);
    }
    auto pp = [&](int q) { return __ddiv_rn(c[q], sum); };
    const double w = __dadd_rn(__dadd_rn(__dadd_rn(pp(0 * 4 + 3), pp(3 * 4 + 0)), pp(1 * 4 + 2)), pp(2 * 4 + 1));
    const double g = __dadd_rn(pp(2 * 4 + 3), pp(3 * 4 + 2));
    const int64_t n = (int64_t)i * (2 * (int64_t)L - i - 1) / 2 + (j - i - 1);
    wcf[n] = w;
    wob[n] = g;
    non[n] = __dsub_rn(__dsub_rn(1.0, w), g);
  }
}

// corr_ValidateProbs (src/correlators.c:1499-1545) for the pair
// probabilities pp = (1e-10 + C) / (16e-10 + nseff) of one alignment, from
// its double-float counts: each in [0, 1 + tol], summing to 1 within tol;
// a failing pair sets *bad
__global__ void __launch_bounds__(256)
k_validate_pp(const float* __restrict__ cnt, const TileRC* __restrict__ tiles, int L, double tol,
              int* __restrict__ bad) {
  const int t = blockIdx.x, tid = threadIdx.x;
  const TileRC tr = tiles[t];
  const float* C = cnt + (int64_t)t * 32 * TPP;
  for (int k = 0; k < 4; k++) {
    const int p = tid + 256 * k, a = p >> 5, b = p & 31;
    const int i = tr.I * TP + a, j = tr.J * TP + b;
    if (!(i < j && j < L)) continue;
    double c[16], Z = 0.0;
#pragma unroll
    for (int q = 0; q < 16; q++) {
      c[q] = 1e-10 + ((double)C[(2 * q) * TPP + p] + (double)C[(2 * q + 1) * TPP + p]);
      Z += c[q];
    }
    // one reciprocal per pair (FP64 division is slow on this part): each
    // value within an ulp of c/Z, far inside the checks' tolerance
    double sum = 0.0;
    bool ok = (Z > 0.0);
    const double iZ = 1.0 / Z;
#pragma unroll
    for (int q = 0; q < 16; q++) {
      const double v = c[q] * iZ;
      ok = ok && (v >= 0.0) && (v <= 1.0 + tol);
      sum += v;
    }
    if (!ok || !(fabs(sum - 1.0) <= tol)) atomicExch(bad, 1);
  }
}

// RAFS from the RAF scores (both in tile layout); b_{i-1,j+1}, b_{i+1,j-1}
__device__ __forceinline__ df tile_get(const float2* cov, const int* tile_index, int nT, int i, int j) {
  const int I = i / TP, J = j / TP;
  const int t = tile_index[I * nT + J];
  return ld_df(cov + (int64_t)t * TPP + (i % TP) * TP + (j % TP));
}

__device__ __forceinline__ void rafs_body(
    const GridIdx g, const float2* __restrict__ raf, float2* __restrict__ out, int64_t slot_stride_in,
    int64_t slot_stride_out,
       const TileRC* __restrict__ tiles, const int* __restrict__ tile_index, int ntiles, int nT, int L,
       double* __restrict__ part1, int64_t part_stride) {
  const int t = g.x, slot = g.y, tid = threadIdx.x;
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
__global__ void __launch_bounds__(256)
k_rafs(const float2* __restrict__ raf, float2* __restrict__ out, int64_t slot_stride_in, int64_t slot_stride_out,
       const TileRC* __restrict__ tiles, const int* __restrict__ tile_index, int ntiles, int nT, int L,
       double* __restrict__ part1, int64_t part_stride) {
  rafs_body(native_grid(), raf, out, slot_stride_in, slot_stride_out, tiles, tile_index, ntiles, nT, L, part1,
                           part_stride);
}

// COVx[c] = sum_{j != c} COV[c][j] / (L-1), from the tile partials
__device__ __forceinline__ void apc_colx_body(
    const GridIdx g, const double* __restrict__ part1, int nT, int L, int Lp, double* __restrict__ colx,
                           float2* __restrict__ colxf) {
  const int sq = g.y;   // (slot, stat) flattened
  const double* P = part1 + (int64_t)sq * nT * nT * TP;
  for (int c = g.x * blockDim.x + threadIdx.x; c < L; c += g.gx * blockDim.x) {
    const int I = c / TP, a = c % TP;
    double s = 0.0;
    for (int K = 0; K < nT; K++) s += P[((int64_t)I * nT + K) * TP + a];
    const double x = (L > 1) ? s / ((double)L - 1.0) : s;
    colx[(int64_t)sq * Lp + c] = x;
    st_df(colxf + (int64_t)sq * Lp + c, df_of(x));
  }
}
__global__ void k_apc_colx(const double* __restrict__ part1, int nT, int L, int Lp, double* __restrict__ colx,
                           float2* __restrict__ colxf) {
  apc_colx_body(native_grid(), part1, nT, L, Lp, colx, colxf);
}

// avg = 2/(L(L-1)) * sum_{i<j} COV = sum_c COVx[c] / L
__device__ __forceinline__ void apc_avg_body(
    const GridIdx g, const double* __restrict__ colx, int L, int Lp, double* __restrict__ avg,
                          float4* __restrict__ apcf) {
  const int sq = g.x;
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
__global__ void k_apc_avg(const double* __restrict__ colx, int L, int Lp, double* __restrict__ avg,
                          float4* __restrict__ apcf) {
  apc_avg_body(native_grid(), colx, L, Lp, avg, apcf);
}

// COV <- COV - COVx_i COVx_j / avg (APC) or COV - (COVx_i + COVx_j - avg) (ASC);
// per-tile min/max of the corrected scores.  Double-float arithmetic.
// APC/ASC applied in place, APC_TILES tiles per block (the block's min/max
// reduction amortised over them), two pairs per 16-byte access
constexpr int APC_TILES = 4;

__device__ __forceinline__ void apc_apply_body(
    const GridIdx g, float2* __restrict__ cov, const float2* __restrict__ colxf, const double* __restrict__ avg,
            const float4* __restrict__ apcf, CorrTypes ct, const TileRC* __restrict__ tiles, int ntiles, int L, int Lp,
            double* __restrict__ tmin, double* __restrict__ tmax, int* __restrict__ status) {
  const int sq = g.y, tid = threadIdx.x;
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
    const int t = g.x * APC_TILES + tt;
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
  const int nblk = g.gx;
  block_minmax_store(lo, hi, tmin + (int64_t)sq * nblk + g.x, tmax + (int64_t)sq * nblk + g.x);
}
__global__ void __launch_bounds__(256)
k_apc_apply(float2* __restrict__ cov, const float2* __restrict__ colxf, const double* __restrict__ avg,
            const float4* __restrict__ apcf, CorrTypes ct, const TileRC* __restrict__ tiles, int ntiles, int L, int Lp,
            double* __restrict__ tmin, double* __restrict__ tmax, int* __restrict__ status) {
  apc_apply_body(native_grid(), cov, colxf, avg, apcf, ct, tiles, ntiles, L, Lp, tmin, tmax, status);
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

__device__ __forceinline__ void reduce_minmax_body(
    const GridIdx g, const double* __restrict__ tmin, const double* __restrict__ tmax, int ntiles,
                                double* __restrict__ mm) {
  const int sq = g.x;
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
__global__ void k_reduce_minmax(const double* __restrict__ tmin, const double* __restrict__ tmax, int ntiles,
                                double* __restrict__ mm) {
  reduce_minmax_body(native_grid(), tmin, tmax, ntiles, mm);
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

__device__ __forceinline__ void hist_body(
    const GridIdx g, const float2* __restrict__ cov, int64_t slot_stride, const TileRC* __restrict__ tiles,
    int ntiles, int nslots,
       int L, BinC B, int nbcap, int wbase, int nwin, unsigned long long* __restrict__ obs, int* __restrict__ status) {
  extern __shared__ unsigned int sh[];
  for (int k = threadIdx.x; k < nwin; k += blockDim.x) sh[k] = 0u;
  __syncthreads();
  // group vb of G = g.gx * R groups; its item (slot, t) advances by
  // G = gs ntiles + gt
  const int R = blockDim.x >> 8, tid = threadIdx.x & 255;
  const int vb = g.x * R + (threadIdx.x >> 8);
  const int G = g.gx * R, gs = G / ntiles, gt = G - gs * ntiles;
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
__global__ void __launch_bounds__(1024)
k_hist(const float2* __restrict__ cov, int64_t slot_stride, const TileRC* __restrict__ tiles, int ntiles, int nslots,
       int L, BinC B, int nbcap, int wbase, int nwin, unsigned long long* __restrict__ obs, int* __restrict__ status) {
  hist_body(native_grid(), cov, slot_stride, tiles, ntiles, nslots, L, B, nbcap, wbase, nwin, obs, status);
}

// E-value of every pair (cov2evalue at src/covariation.c:2369-2400 with
// Nc = 1, times the number of tests) and the compacted hit list.  The FP64
// work per pair is one multiply: the quotients of the tail branch are a
// table (ptail = tail / Nc, divided on the host), the comparisons of x with
// phi and xmax are decided on x.hi against float brackets two ulps either
// side (FP64 only inside them), and E < thresh is compared on the bit
// patterns (non-negative doubles order as their bits).

__device__ __forceinline__ bool ge_df(df x, float dn, float up, double y) {
  if (x.hi > up) return true;
  if (x.hi < dn) return false;
  return df_to_d(x) >= y;
}

__device__ __forceinline__ void evalue_body(
    const GridIdx g, const float2* __restrict__ cov, const TileRC* __restrict__ tiles, int ntiles, int L,
    EvalTables T, BinC B,
         EvalCmp K, double* __restrict__ evt, int* __restrict__ nhits, int hitcap, int* __restrict__ hi,
         int* __restrict__ hj, double* __restrict__ hsc, double* __restrict__ hE, double* __restrict__ hp) {
  const int t = g.x, tid = threadIdx.x;
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
      double mult = T.Nt;
      if (T.bpmask || T.kstar >= 0) {
        const long long n = (long long)i * (2LL * L - i - 1) / 2 + (j - i - 1);
        if (T.bpmask && ((__ldg(T.bpmask + (n >> 5)) >> (n & 31)) & 1u)) mult = T.Nb;
        else if (n <= T.kstar)                                             mult = T.Nx;
      }
      E = pv * mult;
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
__global__ void __launch_bounds__(256)
k_evalue(const float2* __restrict__ cov, const TileRC* __restrict__ tiles, int ntiles, int L, EvalTables T, BinC B,
         EvalCmp K, double* __restrict__ evt, int* __restrict__ nhits, int hitcap, int* __restrict__ hi,
         int* __restrict__ hj, double* __restrict__ hsc, double* __restrict__ hE, double* __restrict__ hp) {
  evalue_body(native_grid(), cov, tiles, ntiles, L, T, B, K, evt, nhits, hitcap, hi, hj, hsc, hE, hp);
}

// pp, nseff and ngap of every pair in the reference's host layout
// (mi->pp[i][j][16], nseff[i][j], ngap[i][j]) from the double-float counts:
// C_q = hi + lo, nseff = sum_q C_q, pp = (1e-10 + C_xy) / sum_q (1e-10 + C_q)
// at [i][j][4x + y] and [j][i][4y + x] (src/correlators.c:1300-1317,
// 1695-1780), ngap[i][j] = wt - nseff, all in FP64 in that order
__global__ void __launch_bounds__(256)
k_probs_host_layout(const float* __restrict__ cnt, const TileRC* __restrict__ tiles, int L, double wt,
                    double* __restrict__ pp, double* __restrict__ nseff, double* __restrict__ ngap) {
  const int t = blockIdx.x, tid = threadIdx.x;
  const TileRC tr = tiles[t];
  const float* Cb = cnt + (int64_t)t * 32 * TPP;
  for (int k = 0; k < 4; k++) {
    const int p = tid + 256 * k;
    const int i = tr.I * TP + (p >> 5), j = tr.J * TP + (p & 31);
    if (!(i < j && j < L)) continue;
    double C[16], ne = 0.0, sum = 0.0;
#pragma unroll
    for (int q = 0; q < 16; q++) {
      C[q] = __dadd_rn((double)Cb[(2 * q) * TPP + p], (double)Cb[(2 * q + 1) * TPP + p]);
      ne = __dadd_rn(ne, C[q]);
    }
    const int64_t ij = (int64_t)i * L + j, ji = (int64_t)j * L + i;
    if (nseff) { nseff[ij] = ne; nseff[ji] = ne; }
    if (ngap) ngap[ij] = __dsub_rn(wt, ne);
    if (pp) {
#pragma unroll
      for (int q = 0; q < 16; q++) sum = __dadd_rn(sum, __dadd_rn(1e-10, C[q]));
#pragma unroll
      for (int x = 0; x < 4; x++)
#pragma unroll
        for (int y = 0; y < 4; y++) {
          const double v = __ddiv_rn(__dadd_rn(1e-10, C[x * 4 + y]), sum);
          pp[ij * 16 + x * 4 + y] = v;
          pp[ji * 16 + y * 4 + x] = v;
        }
    }
  }
}

cudaError_t launch_probs_host_layout(const float* cnt, const TileRC* tiles, int ntiles, int L, double wt, double* pp,
                                     double* nseff, double* ngap, cudaStream_t st) {
  if (ntiles > 0) k_probs_host_layout<<<ntiles, 256, 0, st>>>(cnt, tiles, L, wt, pp, nseff, ngap);
  return cudaGetLastError();
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
cudaError_t launch_count_simt(const uint8_t* ax, int64_t slot_stride, const CountWeights& W, bool unit, int N, int Lp,
                              const TileRC* tiles, int ntiles, int nslots, float* cnt, cudaStream_t st) {
  dim3 grid(ntiles, nslots);
  if (unit)
    k_count_simt<MODE_UNIT><<<grid, 256, 0, st>>>(ax, slot_stride, nullptr, N, Lp, tiles, ntiles, cnt, 1.f, 1.f, 0.f);
  else if (W.nl == 1)
    k_count_simt<MODE_EQUAL><<<grid, 256, 0, st>>>(ax, slot_stride, nullptr, N, Lp, tiles, ntiles, cnt, 1.f, W.s_hi,
                                                    W.s_lo);
  else
    k_count_simt<MODE_LIMBS><<<grid, 256, 0, st>>>(ax, slot_stride, W.d_limbf, N, Lp, tiles, ntiles, cnt, W.B, W.s_hi,
                                                    0.f);
  return cudaGetLastError();
}

cudaError_t launch_pair_marg(const float* cnt, int L, const TileRC* tiles, int ntiles, int nT, int nslots,
                             double* part4, double* partR, cudaStream_t st) {
  k_pair_marg<<<dim3(ntiles, nslots), 256, 0, st>>>(cnt, L, tiles, ntiles, nT, part4, partR);
  return cudaGetLastError();
}

cudaError_t launch_pm_final(const double* part4, const double* partR, int L, int Lp, int nT, int nslots, double* pm,
                            float2* pmdf, float4* lpi, double* mpc, double* meanp, int* status, cudaStream_t st) {
  k_pm_final<<<dim3((L + 127) / 128, nslots), 128, 0, st>>>(part4, partR, L, Lp, nT, pm, pmdf, lpi, mpc, status);
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
  const dim3 grid(A.ntiles, nslots);
  if (cf == 0 || cf == CF_G)          k_stats<CF_G><<<grid, 256, 0, st>>>(A);
  else if (cf == CF_CHI)              k_stats<CF_CHI><<<grid, 256, 0, st>>>(A);
  else if (cf == (CF_G | CF_CHI))     k_stats<CF_G | CF_CHI><<<grid, 256, 0, st>>>(A);
  else                                k_stats<CF_ALL><<<grid, 256, 0, st>>>(A);
  return cudaGetLastError();
}

cudaError_t launch_pair_classes(const float* cnt, const TileRC* tiles, int ntiles, int L, double* wcf, double* wob,
                                double* non, cudaStream_t st) {
  k_pair_classes<<<ntiles, 256, 0, st>>>(cnt, tiles, L, wcf, wob, non);
  return cudaGetLastError();
}

cudaError_t launch_validate_pp(const float* cnt, const TileRC* tiles, int ntiles, int L, double tol, int* bad,
                               cudaStream_t st) {
  k_validate_pp<<<ntiles, 256, 0, st>>>(cnt, tiles, L, tol, bad);
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

EvalCmp evalcmp_host(const EvalTables& T) {
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
  return K;
}

cudaError_t launch_evalue(const float2* cov, const TileRC* tiles, int ntiles, int L, const EvalTables& T, double* evt,
                          int* nhits, int hitcap, int* hi, int* hj, double* hsc, double* hE, double* hp,
                          cudaStream_t st) {
  k_evalue<<<ntiles, 256, 0, st>>>(cov, tiles, ntiles, L, T, make_binc(T.bmin, T.w), evalcmp_host(T), evt, nhits,
                                   hitcap, hi, hj, hsc, hE, hp);
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

// ------------------------------------------------------------------------
// host helpers
// ------------------------------------------------------------------------
void logtab_host(float4* tab) {
  for (int j = 0; j < LOGTAB_N; j++) {
    const double cj = 1.0 + (j + 0.5) / LOGTAB_N;
    const float r = (float)(1.0 / cj);
    const double nl = -std::log((double)r);
    const float hi = (float)nl;
    tab[j] = make_float4(r, hi, (float)(nl - (double)hi), 0.f);
  }
  // k ln 2 for the biased exponent e = k + 127, ln 2 as a double pair
  const double ln2_hi = 0.6931471805599453, ln2_lo = 2.3190468138462996e-17;
  float* kl = reinterpret_cast<float*>(tab + LOGTAB_N);
  for (int e = 0; e < 256; e++) {
    const double k = (double)(e - 127);
    const double v = k * ln2_hi;   // |k| < 2^8: error below 2^-52 |v|
    const float hi = (float)v;
    kl[2 * e] = hi;
    kl[2 * e + 1] = (float)((v - (double)hi) + k * ln2_lo);
  }
}

void make_limbs(const double* w, int N, int stride, uint16_t* lim, CountWeights* W, double* wtot_q) {
  double wmax = 0.0;
  bool equal = true;
  for (int s = 0; s < N; s++) { wmax = std::max(wmax, w[s]); if (w[s] != w[0]) equal = false; }
  std::memset(lim, 0, sizeof(uint16_t) * 3 * (size_t)stride);
  W->d_limbf = nullptr;
  if (equal || wmax <= 0.0) {
    const double s0 = (N > 0) ? w[0] : 1.0;
    W->nl = 1; W->bits = 0; W->B = 1.f;
    W->s_hi = (float)s0; W->s_lo = (float)(s0 - (double)W->s_hi);
    for (int s = 0; s < N; s++) lim[s] = 1;
    *wtot_q = (double)N * s0;
    return;
  }
  // b-bit limbs with N (2^b - 1) < 2^24: every limb sum is an exact FP32
  // integer, and b <= 11 keeps a limb exact in FP16
  int b = 11;
  while (b > 1 && (double)N * (double)((1 << b) - 1) >= 16777216.0) b--;
  const int bits = 3 * b;
  int e2;
  std::frexp(wmax, &e2);                     // wmax = f 2^e2, f in [0.5, 1)
  const int E = bits - e2;                   // wmax 2^E < 2^bits
  const double qmax = std::ldexp(1.0, bits) - 1.0;
  const uint64_t mask = (1ull << b) - 1ull;
  uint64_t tot = 0;
  for (int s = 0; s < N; s++) {
    double qd = std::nearbyint(std::ldexp(w[s], E));
    if (qd > qmax) qd = qmax;
    const uint64_t q = (uint64_t)qd;
    lim[s] = (uint16_t)(q & mask);
    lim[stride + s] = (uint16_t)((q >> b) & mask);
    lim[2 * (size_t)stride + s] = (uint16_t)(q >> (2 * b));
    tot += q;
  }
  W->nl = 3; W->bits = b;
  W->B = (float)(1 << b);
  W->s_hi = (float)std::ldexp(1.0, -E);
  W->s_lo = 0.f;
  *wtot_q = std::ldexp((double)tot, -E);
}

// ------------------------------------------------------------------------
// grouped launches over a batch of families (cov_batch.h): block b of a
// grouped launch is block b - pre[f] of family f's own grid, x-major
// ------------------------------------------------------------------------
struct GrpLoc { int f; GridIdx g; };
__device__ __forceinline__ GrpLoc grp_loc(const int* __restrict__ pre, int nf, int gx_of_f(const FamDev&),
                                          const FamDev* __restrict__ F) {
  const int f = grp_find(pre, nf, (int)blockIdx.x);
  const int loc = (int)blockIdx.x - __ldg(pre + f), gx = gx_of_f(F[f]);
  return GrpLoc{f, GridIdx{loc % gx, loc / gx, gx}};
}
__device__ __forceinline__ int gx_tiles(const FamDev& d) { return d.ntiles; }
__device__ __forceinline__ int gx_cols128(const FamDev& d) { return (d.L + 127) / 128; }
__device__ __forceinline__ int gx_cols256(const FamDev& d) { return (d.L + 255) / 256; }
__device__ __forceinline__ int gx_one(const FamDev&) { return 1; }
__device__ __forceinline__ int gx_apc(const FamDev& d) { return (d.ntiles + APC_TILES - 1) / APC_TILES; }

template <bool UNIT>
__global__ void __launch_bounds__(256, 2)
k_count_simt_grp(const FamDev* __restrict__ F, const int* __restrict__ pre, int nf) {
  const GrpLoc l = grp_loc(pre, nf, gx_tiles, F);
  const FamDev& d = F[l.f];
  const int64_t ss = (int64_t)d.N * d.Lp;
  if (UNIT)
    count_simt_body<MODE_UNIT>(l.g, d.ax, ss, nullptr, d.N, d.Lp, d.tiles, d.ntiles, d.ucnt, 1.f, 1.f, 0.f);
  else if (d.nl == 1)
    count_simt_body<MODE_EQUAL>(l.g, d.ax, ss, nullptr, d.N, d.Lp, d.tiles, d.ntiles, d.cnt, 1.f, d.s_hi, d.s_lo);
  else
    count_simt_body<MODE_LIMBS>(l.g, d.ax, ss, d.limbf, d.N, d.Lp, d.tiles, d.ntiles, d.cnt, d.B, d.s_hi, 0.f);
}

__global__ void __launch_bounds__(256)
k_pair_marg_grp(const FamDev* __restrict__ F, const int* __restrict__ pre, int nf) {
  const GrpLoc l = grp_loc(pre, nf, gx_tiles, F);
  const FamDev& d = F[l.f];
  pair_marg_body(l.g, d.cnt, d.L, d.tiles, d.ntiles, d.nT, d.part4, d.partR);
}

__global__ void k_pm_final_grp(const FamDev* __restrict__ F, const int* __restrict__ pre, int nf) {
  const GrpLoc l = grp_loc(pre, nf, gx_cols128, F);
  const FamDev& d = F[l.f];
  pm_final_body(l.g, d.part4, d.partR, d.L, d.Lp, d.nT, d.pm, d.pmdf, d.lpi, d.mpc, d.status);
}

__global__ void k_meanp_grp(const FamDev* __restrict__ F, const int* __restrict__ pre, int nf) {
  const GrpLoc l = grp_loc(pre, nf, gx_one, F);
  const FamDev& d = F[l.f];
  meanp_body(GridIdx{l.g.y, 0, 1}, d.mpc, d.L, d.Lp, d.meanp);
}

template <unsigned CF>
__global__ void __launch_bounds__(256, 2)
k_stats_grp(const FamDev* __restrict__ F, const int* __restrict__ pre, int nf) {
  const GrpLoc l = grp_loc(pre, nf, gx_tiles, F);
  stats_body<CF>(l.g, F[l.f].sa);
}

__global__ void __launch_bounds__(256)
k_rafs_grp(const FamDev* __restrict__ F, const int* __restrict__ pre, int nf, int q) {
  const GrpLoc l = grp_loc(pre, nf, gx_tiles, F);
  const FamDev& d = F[l.f];
  const int nout = d.sa.nout;
  const int64_t plane = (int64_t)d.ntiles * TPP, pplane = (int64_t)d.nT * d.nT * TP;
  rafs_body(l.g, d.cov2, d.cov + q * plane, plane, nout * plane, d.tiles, d.tile_index, d.ntiles, d.nT, d.L,
            d.part1 + q * pplane, nout * pplane);
}

__global__ void k_apc_colx_grp(const FamDev* __restrict__ F, const int* __restrict__ pre, int nf) {
  const GrpLoc l = grp_loc(pre, nf, gx_cols256, F);
  const FamDev& d = F[l.f];
  apc_colx_body(l.g, d.part1, d.nT, d.L, d.Lp, d.colx, d.colxf);
}

__global__ void k_apc_avg_grp(const FamDev* __restrict__ F, const int* __restrict__ pre, int nf) {
  const GrpLoc l = grp_loc(pre, nf, gx_one, F);
  const FamDev& d = F[l.f];
  apc_avg_body(GridIdx{l.g.y, 0, 1}, d.colx, d.L, d.Lp, d.avg, d.apcf);
}

__global__ void __launch_bounds__(256)
k_apc_apply_grp(const FamDev* __restrict__ F, const int* __restrict__ pre, int nf, CorrTypes ct) {
  const GrpLoc l = grp_loc(pre, nf, gx_apc, F);
  const FamDev& d = F[l.f];
  apc_apply_body(l.g, d.cov, d.colxf, d.avg, d.apcf, ct, d.tiles, d.ntiles, d.L, d.Lp, d.tmin, d.tmax, d.status);
}

__global__ void k_reduce_minmax_grp(const FamDev* __restrict__ F, const int* __restrict__ pre, int nf) {
  const GrpLoc l = grp_loc(pre, nf, gx_one, F);
  const FamDev& d = F[l.f];
  reduce_minmax_body(GridIdx{l.g.y, 0, 1}, d.tmin, d.tmax, (d.ntiles + APC_TILES - 1) / APC_TILES, d.mm);
}

// one (family, statistic) per entry of S: the nulls' scores of that
// statistic into its histogram
__global__ void __launch_bounds__(1024)
k_hist_grp(const FamDev* __restrict__ F, const StatDev* __restrict__ S, const int* __restrict__ pre, int ns) {
  const int e = grp_find(pre, ns, (int)blockIdx.x);
  const StatDev& x = S[e];
  const FamDev& d = F[x.fam];
  const int gx = __ldg(pre + e + 1) - __ldg(pre + e);
  const int64_t plane = (int64_t)d.ntiles * TPP;
  const int nout = d.sa.nout;
  hist_body(GridIdx{(int)blockIdx.x - __ldg(pre + e), 0, gx}, d.cov + (int64_t)(nout + x.q) * plane, nout * plane,
            d.tiles, d.ntiles, d.nslots - 1, d.L, x.hb, x.nbcap, x.wbase, x.nwin, x.obs, d.status);
}

__global__ void __launch_bounds__(256)
k_evalue_grp(const FamDev* __restrict__ F, const StatDev* __restrict__ S, const int* __restrict__ pre, int ns) {
  const int e = grp_find(pre, ns, (int)blockIdx.x);
  const StatDev& x = S[e];
  const FamDev& d = F[x.fam];
  const int64_t plane = (int64_t)d.ntiles * TPP;
  evalue_body(GridIdx{(int)blockIdx.x - __ldg(pre + e), 0, d.ntiles}, d.cov + (int64_t)x.q * plane, d.tiles,
              d.ntiles, d.L, x.T, x.hb, x.K, nullptr, x.nhits, x.hitcap, x.hi, x.hj, x.hsc, x.hE, x.hp);
}

unsigned stats_cf(unsigned mask) {
  unsigned cf = 0;
  if (mask & (S_GT | S_MI | S_MIr | S_MIg)) cf |= CF_G;
  if (mask & S_CHI) cf |= CF_CHI;
  if (mask & S_OMES) cf |= CF_OMES;
  return cf;
}
int apc_blocks(int ntiles) { return (ntiles + APC_TILES - 1) / APC_TILES; }
int hist_threads() { return 1024; }
BinC binc_host(double bmin, double w) { return make_binc(bmin, w); }

cudaError_t grp_count_simt(const FamDev* F, int nf, const int* pre, int nb, bool unit, bool limbs, cudaStream_t st) {
  (void)limbs;
  if (nb <= 0) return cudaSuccess;
  if (unit) k_count_simt_grp<true><<<nb, 256, 0, st>>>(F, pre, nf);
  else      k_count_simt_grp<false><<<nb, 256, 0, st>>>(F, pre, nf);
  return cudaGetLastError();
}

cudaError_t grp_marginals(const FamDev* F, int nf, const int* pre_marg, int nb_marg, const int* pre_pm, int nb_pm,
                          const int* pre_mp, int nb_mp, cudaStream_t st) {
  if (nb_marg > 0) k_pair_marg_grp<<<nb_marg, 256, 0, st>>>(F, pre_marg, nf);
  if (nb_pm > 0) k_pm_final_grp<<<nb_pm, 128, 0, st>>>(F, pre_pm, nf);
  if (nb_mp > 0) k_meanp_grp<<<nb_mp, 256, 0, st>>>(F, pre_mp, nf);
  return cudaGetLastError();
}

cudaError_t grp_stats(const FamDev* F, int nf, const int* pre, int nb, unsigned cf, cudaStream_t st) {
  if (nb <= 0) return cudaSuccess;
  if (cf == 0 || cf == CF_G)          k_stats_grp<CF_G><<<nb, 256, 0, st>>>(F, pre, nf);
  else if (cf == CF_CHI)              k_stats_grp<CF_CHI><<<nb, 256, 0, st>>>(F, pre, nf);
  else if (cf == (CF_G | CF_CHI))     k_stats_grp<CF_G | CF_CHI><<<nb, 256, 0, st>>>(F, pre, nf);
  else                                k_stats_grp<CF_ALL><<<nb, 256, 0, st>>>(F, pre, nf);
  return cudaGetLastError();
}

cudaError_t grp_rafs(const FamDev* F, int nf, const int* pre, int nb, int q, cudaStream_t st) {
  if (nb > 0) k_rafs_grp<<<nb, 256, 0, st>>>(F, pre, nf, q);
  return cudaGetLastError();
}

cudaError_t grp_apc(const FamDev* F, int nf, const int* pre_colx, int nb_colx, const int* pre_sq, int nb_sq,
                    const int* pre_apply, int nb_apply, CorrTypes ct, cudaStream_t st) {
  if (nb_colx > 0) k_apc_colx_grp<<<nb_colx, 256, 0, st>>>(F, pre_colx, nf);
  if (nb_sq > 0) k_apc_avg_grp<<<nb_sq, 256, 0, st>>>(F, pre_sq, nf);
  if (nb_apply > 0) k_apc_apply_grp<<<nb_apply, 256, 0, st>>>(F, pre_apply, nf, ct);
  if (nb_sq > 0) k_reduce_minmax_grp<<<nb_sq, 256, 0, st>>>(F, pre_sq, nf);
  return cudaGetLastError();
}

cudaError_t grp_hist(const FamDev* F, const StatDev* S, int ns, const int* pre, int nb, int maxwin, cudaStream_t st) {
  if (nb <= 0) return cudaSuccess;
  static const bool attr = [] {
    cudaFuncSetAttribute(k_hist_grp, cudaFuncAttributeMaxDynamicSharedMemorySize, HIST_WIN * 4);
    return true;
  }();
  (void)attr;
  k_hist_grp<<<nb, 1024, (size_t)std::max(1, maxwin) * 4, st>>>(F, S, pre, ns);
  return cudaGetLastError();
}

cudaError_t grp_evalue(const FamDev* F, const StatDev* S, int ns, const int* pre, int nb, cudaStream_t st) {
  if (nb > 0) k_evalue_grp<<<nb, 256, 0, st>>>(F, S, pre, ns);
  return cudaGetLastError();
}

}  // namespace covgpu
