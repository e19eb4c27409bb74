// cov_null.cu -- null alignments on the GPU: Fitch ancestral states and the
// shuffled-substitution replay of R-scape's default null (--nullphylo).
//
//   k_fitch      one thread per (column, null): Tree_FitchAlgorithmAncenstral
//                / tree_fitch_column (src/msatree.c:173-227, 1700-1838); up
//                pass = intersection over the five states, else the union of
//                residues only (tree_fitch_upwards :1877-1908); down pass
//                keeps the parent's state when the child's set holds it.
//   k_colperm    msamanip_ShuffleColumns (src/msamanip.c:1164-1233) on the
//                internal-node rows of the reconstruction.
//   k_branch     one CTA per (branch, null), tree levels in order:
//                shuffle_tree_substitutions + shuffle_tree_substitute_all
//                (src/msamanip.c:1597-1747).  The child takes a copy of its
//                shuffled parent; the branch's substitution counts (measured
//                on the unshuffled reconstruction) are replayed on positions
//                of the shuffled parent holding the old state, visited in a
//                random order (a Feistel permutation; a block-wide scan gives
//                each position its rank within its state class).
//
// Random draws are counter-based (Philox keyed by the seed, the null index,
// the node and the column), so the result does not depend on scheduling.
//
// Buffers (per null q): fitch[q][v][Lp] and S[q][v][Lp] for internal nodes v,
// shint[q][v][Lp] their shuffled rows; leaf rows go straight to the output
// alignment slot.
#include "cov_dev.cuh"
#include "cov_kernels.h"

namespace covgpu {

__device__ __forceinline__ int choose_member(unsigned S, uint64_t seed, uint32_t null_id, uint32_t node, uint32_t col) {
  const int m = __popc(S);
  int k = 0;
  if (m > 1) k = (int)(((uint64_t)rng_u32(seed, TAG_FCHOOSE, null_id, node, col) * (uint64_t)m) >> 32);
  for (int x = 0; x < 5; x++)
    if (S & (1u << x)) { if (k == 0) return x; k--; }
  return 4;
}

__device__ __forceinline__ unsigned leaf_set(const uint8_t* ax, int Lp, int n, int c, uint64_t seed, uint32_t nid) {
  const int x = ax[(int64_t)n * Lp + c];
  if (x <= 4) return 1u << x;
  return 1u << (int)(((uint64_t)rng_u32(seed, TAG_FLEAF, nid, (uint32_t)n, (uint32_t)c) * 5u) >> 32);
}

__global__ void __launch_bounds__(128)
k_fitch(const uint8_t* __restrict__ ax, int N, int L, int Lp, const int* __restrict__ left,
        const int* __restrict__ right, uint64_t seed, uint32_t first_null, uint8_t* __restrict__ fitch,
        uint8_t* __restrict__ Sbuf) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  const int q = blockIdx.y;
  if (c >= L) return;
  const uint32_t nid = first_null + q;
  const int64_t qoff = (int64_t)q * (N - 1) * Lp;
  uint8_t* S = Sbuf + qoff;
  uint8_t* F = fitch + qoff;
  for (int v = N - 2; v >= 0; v--) {
    const int l = left[v], r = right[v];
    const unsigned Sl = (l <= 0) ? leaf_set(ax, Lp, -l, c, seed, nid) : S[(int64_t)l * Lp + c];
    const unsigned Sr = (r <= 0) ? leaf_set(ax, Lp, -r, c, seed, nid) : S[(int64_t)r * Lp + c];
    const unsigned I = Sl & Sr;
    S[(int64_t)v * Lp + c] = (uint8_t)(I ? I : ((Sl | Sr) & 0xFu));
  }
  F[c] = (uint8_t)choose_member(S[c], seed, nid, 0, (uint32_t)c);
  for (int v = 0; v < N - 1; v++) {
    const int a = F[(int64_t)v * Lp + c];
    const int ch[2] = {left[v], right[v]};
#pragma unroll
    for (int k = 0; k < 2; k++) {
      if (ch[k] > 0) {
        unsigned Sc = S[(int64_t)ch[k] * Lp + c];
        if (Sc & (1u << a)) Sc = 1u << a;
        F[(int64_t)ch[k] * Lp + c] = (uint8_t)choose_member(Sc, seed, nid, (uint32_t)ch[k], (uint32_t)c);
      }
    }
  }
}

// internal rows: shint[q][v][c] = fitch[q][v][perm_q(c)], padding = gap
__global__ void __launch_bounds__(256)
k_colperm(const uint8_t* __restrict__ fitch, int N, int L, int Lp, uint64_t seed, uint32_t first_null,
          uint8_t* __restrict__ shint) {
  const int q = blockIdx.z;
  const int v = blockIdx.y;
  const uint32_t nid = first_null + q;
  uint32_t rk[6];
  round_keys(seed, TAG_COLPERM, nid, 0, rk);
  const uint32_t hb = feistel_hbits((uint32_t)L);
  const int64_t row = ((int64_t)q * (N - 1) + v) * Lp;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < Lp; c += gridDim.x * blockDim.x) {
    uint8_t x = 4;
    if (c < L) x = fitch[row + feistel_perm((uint32_t)c, hb, (uint32_t)L, rk)];
    shint[row + c] = x;
  }
}

// one CTA per (branch, null) for the internal nodes of one tree level
__global__ void __launch_bounds__(1024)
k_branch(const uint8_t* __restrict__ ax, int N, int L, int Lp, const int* __restrict__ left,
         const int* __restrict__ right, const int* __restrict__ nodes, uint64_t seed, uint32_t first_null,
         const uint8_t* __restrict__ fitch, uint8_t* __restrict__ shint, uint8_t* __restrict__ out_ax,
         int64_t out_slot_stride) {
  extern __shared__ uint8_t psh[];         // shuffled parent row, L bytes
  __shared__ int nsub[25];
  __shared__ int cum[5][6];
  __shared__ int wtot[32][5];
  const int q = blockIdx.y;
  const int v = nodes[blockIdx.x >> 1];
  const int side = blockIdx.x & 1;
  const int ch = side ? right[v] : left[v];
  const int cidx = (ch <= 0) ? -ch : N + ch;
  const uint32_t nid = first_null + q;
  const int tid = threadIdx.x, nth = blockDim.x;
  const int64_t qoff = (int64_t)q * (N - 1) * Lp;
  const uint8_t* Fp = fitch + qoff + (int64_t)v * Lp;
  const uint8_t* Fc = (ch <= 0) ? ax + (int64_t)(-ch) * Lp : fitch + qoff + (int64_t)ch * Lp;
  const uint8_t* Pp = shint + qoff + (int64_t)v * Lp;
  uint8_t* Cc = (ch <= 0) ? out_ax + (int64_t)q * out_slot_stride + (int64_t)(-ch) * Lp
                          : shint + qoff + (int64_t)ch * Lp;

  if (tid < 25) nsub[tid] = 0;
  __syncthreads();
  for (int c = tid; c < Lp; c += nth) {
    const uint8_t p = Pp[c];
    if (c < L) {
      psh[c] = p;
      const int a = Fp[c], b = Fc[c];
      if (a != b && a <= 4 && b <= 4) atomicAdd(&nsub[a * 5 + b], 1);
    }
    Cc[c] = (c < L) ? p : (uint8_t)4;
  }
  __syncthreads();
  if (tid < 5) {
    cum[tid][0] = 0;
    for (int d = 0; d < 5; d++) cum[tid][d + 1] = cum[tid][d] + nsub[tid * 5 + d];
  }
  uint32_t rk[6];
  round_keys(seed, TAG_SUBST, nid, (uint32_t)cidx, rk);
  const uint32_t hb = feistel_hbits((uint32_t)L);
  __syncthreads();
  const int total = cum[0][5] + cum[1][5] + cum[2][5] + cum[3][5] + cum[4][5];
  if (total == 0) return;

  // slot t -> position perm(t); each thread takes a contiguous run of slots
  const int per = (L + nth - 1) / nth;
  const int t0 = tid * per, t1 = min(L, t0 + per);
  int cnt[5] = {0, 0, 0, 0, 0};
  for (int t = t0; t < t1; t++) {
    const int o = psh[feistel_perm((uint32_t)t, hb, (uint32_t)L, rk)];
    if (o <= 4) cnt[o]++;
  }
  // exclusive block scan of the five class counters
  const int lane = tid & 31, warp = tid >> 5;
  int inc[5];
#pragma unroll
  for (int k = 0; k < 5; k++) {
    int x = cnt[k];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    inc[k] = x;
  }
  if (lane == 31)
#pragma unroll
    for (int k = 0; k < 5; k++) wtot[warp][k] = inc[k];
  __syncthreads();
  if (warp == 0) {
    const int nw = nth >> 5;
#pragma unroll
    for (int k = 0; k < 5; k++) {
      int x = (lane < nw) ? wtot[lane][k] : 0;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
      }
      if (lane < nw) wtot[lane][k] = x;     // inclusive over warps
    }
  }
  __syncthreads();
  int rank[5];
#pragma unroll
  for (int k = 0; k < 5; k++) rank[k] = inc[k] - cnt[k] + ((warp > 0) ? wtot[warp - 1][k] : 0);
  for (int t = t0; t < t1; t++) {
    const uint32_t p = feistel_perm((uint32_t)t, hb, (uint32_t)L, rk);
    const int o = psh[p];
    if (o > 4) continue;
    const int r = rank[o]++;
    if (r < cum[o][5]) {
      int d = 0;
      while (r >= cum[o][d + 1]) d++;
      Cc[p] = (uint8_t)d;
    }
  }
}

cudaError_t launch_nullgen(const uint8_t* ax, int N, int L, int Lp, const NullTree& T, const int* level_nodes,
                           const int* level_off, int nlevels, uint64_t seed, uint32_t first_null, int nnull,
                           uint8_t* fitch, uint8_t* scratch, uint8_t* out_ax, int64_t out_slot_stride,
                           cudaStream_t st) {
  // scratch holds the Fitch sets first, then the shuffled internal rows
  k_fitch<<<dim3((L + 127) / 128, nnull), 128, 0, st>>>(ax, N, L, Lp, T.left, T.right, seed, first_null, fitch,
                                                        scratch);
  k_colperm<<<dim3((Lp + 255) / 256, N - 1, nnull), 256, 0, st>>>(fitch, N, L, Lp, seed, first_null, scratch);
  for (int d = 0; d < nlevels; d++) {
    const int nn = level_off[d + 1] - level_off[d];
    if (nn <= 0) continue;
    k_branch<<<dim3(2 * nn, nnull), 1024, L, st>>>(ax, N, L, Lp, T.left, T.right, level_nodes + level_off[d], seed,
                                                   first_null, fitch, scratch, out_ax, out_slot_stride);
  }
  return cudaGetLastError();
}

}  // namespace covgpu
