// cov_dev.cuh -- device-side helpers shared by the covariation kernels.
//
// Layout conventions of the GPU library (all buffers live in HBM):
//   alignment codes  uint8 [slot][N][Lp] row-major, Easel RNA digital codes
//                    (0..3 = ACGU, 4 = gap, 15 = N); Lp = L rounded up to a
//                    multiple of TP, padding columns hold the gap code.
//   column tiles     TP x TP blocks of column pairs (i in tile I, j in tile J,
//                    I <= J), enumerated row by row of the upper triangle.
//   counts           float [slot][tile][16][2][TP*TP]: the 4x4 weighted joint
//                    counts of every pair of the tile, cell-major, each a
//                    double-float (hi plane, then lo plane); unit-weight
//                    counts (RAF) float [slot][tile][16][TP*TP], exact.
//   scores           float2 [slot][stat][tile][TP*TP], double-float (hi, lo)
//                    values of the tile-packed COV.
//   column partials  double [slot][nT][nT][TP][...]: per-tile row sums
//                    (index [I][J]) and column sums (index [J][I]).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#define TP 32             // column tile edge
#define TPP (TP * TP)     // pairs per tile

namespace covgpu {

// statistic bits (one score matrix per requested statistic)
enum StatBit : unsigned {
  S_CHI = 1u << 0, S_GT = 1u << 1, S_MI = 1u << 2, S_MIr = 1u << 3, S_MIg = 1u << 4,
  S_OMES = 1u << 5, S_RAF = 1u << 6, S_RAFS = 1u << 7, S_CCF = 1u << 8
};
constexpr int NSTAT = 9;

struct TileRC { int I, J; };

// the block a kernel body works on: the launch's own blockIdx.x, blockIdx.y
// and gridDim.x, or the coordinates inside one alignment family of a grouped
// launch (one launch over the blocks of many families)
struct GridIdx { int x, y, gx; };
__device__ __forceinline__ GridIdx native_grid() {
  return GridIdx{(int)blockIdx.x, (int)blockIdx.y, (int)gridDim.x};
}
// the entry f of the ascending prefix pre[0..nf] with pre[f] <= b < pre[f + 1]
// (entries of empty families are skipped: their prefix does not advance)
__device__ __forceinline__ int grp_find(const int* __restrict__ pre, int nf, int b) {
  int lo = 0, hi = nf;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (__ldg(pre + mid) <= b) lo = mid; else hi = mid;
  }
  return lo;
}

// ---- Philox4x32-10 (Salmon et al., SC'11) ----
__host__ __device__ __forceinline__ void philox4x32(uint32_t k0, uint32_t k1, uint32_t c[4]) {
#pragma unroll
  for (int r = 0; r < 10; r++) {
    uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
    uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
    uint32_t n0 = (uint32_t)(p1 >> 32) ^ c[1] ^ k0;
    uint32_t n2 = (uint32_t)(p0 >> 32) ^ c[3] ^ k1;
    c[1] = (uint32_t)p1; c[3] = (uint32_t)p0; c[0] = n0; c[2] = n2;
    k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
  }
}

__host__ __device__ __forceinline__ uint32_t rng_u32(uint64_t seed, uint32_t tag, uint32_t null_id,
                                                     uint32_t a, uint32_t b) {
  uint32_t c[4] = {tag, null_id, a, b};
  philox4x32((uint32_t)seed, (uint32_t)(seed >> 32), c);
  return c[0];
}

__host__ __device__ __forceinline__ void round_keys(uint64_t seed, uint32_t tag, uint32_t null_id,
                                                    uint32_t idx, uint32_t rk[6]) {
  uint32_t c[4] = {tag, null_id, idx, 0};
  philox4x32((uint32_t)seed, (uint32_t)(seed >> 32), c);
  rk[0] = c[0]; rk[1] = c[1]; rk[2] = c[2]; rk[3] = c[3];
  uint32_t d[4] = {tag, null_id, idx, 1};
  philox4x32((uint32_t)seed, (uint32_t)(seed >> 32), d);
  rk[4] = d[0]; rk[5] = d[1];
}

__host__ __device__ __forceinline__ uint32_t fmix32(uint32_t h) {
  h ^= h >> 16; h *= 0x85EBCA6Bu; h ^= h >> 13; h *= 0xC2B2AE35u; h ^= h >> 16;
  return h;
}

// random permutation of [0,L): 6-round Feistel network on the smallest
// even-bit domain >= L, cycle-walked into [0,L)
__host__ __device__ __forceinline__ uint32_t feistel_perm(uint32_t t, uint32_t hbits, uint32_t L,
                                                          const uint32_t rk[6]) {
  const uint32_t mask = (1u << hbits) - 1u;
  uint32_t x = t;
  do {
    uint32_t l = x >> hbits, r = x & mask;
#pragma unroll
    for (int k = 0; k < 6; k++) { uint32_t nl = r; r = l ^ (fmix32(r ^ rk[k]) & mask); l = nl; }
    x = (l << hbits) | r;
  } while (x >= L);
  return x;
}

__host__ __device__ __forceinline__ uint32_t feistel_hbits(uint32_t L) {
  uint32_t h = 1;
  while ((1u << (2 * h)) < L) h++;
  return h;
}

constexpr uint32_t TAG_FLEAF = 0x11u, TAG_FCHOOSE = 0x12u, TAG_COLPERM = 0x13u, TAG_SUBST = 0x14u;

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

}  // namespace covgpu
