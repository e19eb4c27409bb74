// cov_null.cu -- null alignments on the GPU: Fitch ancestral states and the
// shuffled-substitution replay of R-scape's default null (--nullphylo).
//
// The work goes by tree depth (nodes of one depth are independent):
//   k_fitch_up   deepest depth first, one thread per (internal node, 16
//                columns, null): the up pass of Tree_FitchAlgorithmAncenstral
//                / tree_fitch_column (src/msatree.c:173-227, 1700-1838):
//                intersection of the children's sets over the five states,
//                else the union of residues only (tree_fitch_upwards
//                :1877-1908), as byte-SIMD on 16-column vectors.
//   k_root       the root's state per column, then its row with the columns
//                shuffled (msamanip_ShuffleColumns, src/msamanip.c:1164-1233).
//                Only the root's shuffled row is ever read: every other row
//                is replaced by its parent's row before use.
//   k_replay     top depth first, one warp per (branch, null):
//                shuffle_tree_substitutions + shuffle_tree_substitute_all
//                (src/msamanip.c:1597-1747).  The warp finishes the child's
//                Fitch state (down pass: keep the parent's state when the
//                child's set holds it), counts the branch's substitutions on
//                the unshuffled reconstruction, copies the parent's current
//                row and replays the substitutions on positions of that row
//                holding the old state, visited in a random order (a Feistel
//                permutation); each class's positions are ranked with warp
//                ballots and the pass stops once every substitution is placed.
//
// Random draws are counter-based (Philox keyed by the seed, the null index,
// the node and the column), so the result does not depend on scheduling.
//
// Buffers (per null q): F[q][v][Lp] the Fitch states of internal node v;
// SR[q][v][Lp] first its Fitch set, then (once the set is used) its row of
// the null alignment; leaf rows go straight to the output alignment slot.
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


// set of a leaf residue: one state, a random one for ambiguity codes
__device__ __forceinline__ uint32_t leaf_byte(uint32_t x, int n, int c, uint64_t seed, uint32_t nid) {
  if (x <= 4) return 1u << x;
  return 1u << (int)(((uint64_t)rng_u32(seed, TAG_FLEAF, nid, (uint32_t)n, (uint32_t)c) * 5u) >> 32);
}

// the sets of 16 consecutive columns of child ch (internal row or leaf)
__device__ __forceinline__ uint4 child_sets(int ch, const uint8_t* ax, const uint8_t* S, int Lp, int c0, uint64_t seed,
                                           uint32_t nid) {
  if (ch > 0) return *reinterpret_cast<const uint4*>(S + (int64_t)ch * Lp + c0);
  const uint4 a = *reinterpret_cast<const uint4*>(ax + (int64_t)(-ch) * Lp + c0);
  uint32_t w[4] = {a.x, a.y, a.z, a.w};
#pragma unroll
  for (int k = 0; k < 4; k++) {
    uint32_t o = 0;
#pragma unroll
    for (int b = 0; b < 4; b++) o |= leaf_byte((w[k] >> (8 * b)) & 0xFFu, -ch, c0 + 4 * k + b, seed, nid) << (8 * b);
    w[k] = o;
  }
  return make_uint4(w[0], w[1], w[2], w[3]);
}

// per byte: I = a & b if nonzero, else (a | b) without the gap bit
__device__ __forceinline__ uint32_t fitch_word(uint32_t a, uint32_t b) {
  const uint32_t I = a & b, U = (a | b) & 0x0F0F0F0Fu;
  const uint32_t z = __vcmpeq4(I, 0u);   // 0xFF in the bytes where I == 0
  return (I & ~z) | (U & z);
}

// up pass for the internal nodes of one depth
__global__ void __launch_bounds__(256)
k_fitch_up(const uint8_t* __restrict__ ax, int N, int Lp, const int* __restrict__ left, const int* __restrict__ right,
           const int* __restrict__ nodes, int nn, uint64_t seed, uint32_t first_null, uint8_t* __restrict__ SR) {
  const int chunks = Lp >> 4;
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= nn * chunks) return;
  const int q = blockIdx.y, v = nodes[idx / chunks], c0 = (idx % chunks) << 4;
  const uint32_t nid = first_null + q;
  uint8_t* S = SR + (int64_t)q * (N - 1) * Lp;
  const uint4 a = child_sets(left[v], ax, S, Lp, c0, seed, nid);
  const uint4 b = child_sets(right[v], ax, S, Lp, c0, seed, nid);
  *reinterpret_cast<uint4*>(S + (int64_t)v * Lp + c0) =
      make_uint4(fitch_word(a.x, b.x), fitch_word(a.y, b.y), fitch_word(a.z, b.z), fitch_word(a.w, b.w));
}

// the root's states F[q][0][c] from its sets
__global__ void __launch_bounds__(256)
k_root_state(int N, int L, int Lp, uint64_t seed, uint32_t first_null, const uint8_t* __restrict__ SR,
             uint8_t* __restrict__ F) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x, q = blockIdx.y;
  if (c >= L) return;
  const int64_t off = (int64_t)q * (N - 1) * Lp;
  F[off + c] = (uint8_t)choose_member(SR[off + c], seed, first_null + q, 0u, (uint32_t)c);
}

// the root's row of the null: its states with the columns shuffled
__global__ void __launch_bounds__(256)
k_root_row(int N, int L, int Lp, uint64_t seed, uint32_t first_null, const uint8_t* __restrict__ F,
           uint8_t* __restrict__ SR) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x, q = blockIdx.y;
  if (c >= Lp) return;
  uint32_t rk[6];
  round_keys(seed, TAG_COLPERM, first_null + q, 0, rk);
  const int64_t off = (int64_t)q * (N - 1) * Lp;
  SR[off + c] = (c < L) ? F[off + feistel_perm((uint32_t)c, feistel_hbits((uint32_t)L), (uint32_t)L, rk)] : (uint8_t)4;
}

// one warp per (branch, null) for the internal nodes v of one depth
__global__ void __launch_bounds__(256)
k_replay(const uint8_t* __restrict__ ax, int N, int L, int Lp, const int* __restrict__ left,
         const int* __restrict__ right, const int* __restrict__ nodes, int nn, uint64_t seed, uint32_t first_null,
         uint8_t* __restrict__ F, uint8_t* __restrict__ SR, uint8_t* __restrict__ out_ax, int64_t out_slot_stride) {
  __shared__ int nsub_s[8][25];
  __shared__ int cum_s[8][5][6];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int item = blockIdx.x * 8 + warp;
  if (item >= 2 * nn) return;
  const int q = blockIdx.y;
  const int v = nodes[item >> 1];
  const int ch = (item & 1) ? right[v] : left[v];
  const int cidx = (ch <= 0) ? -ch : N + ch;
  const uint32_t nid = first_null + q;
  const int64_t qoff = (int64_t)q * (N - 1) * Lp;
  const uint8_t* Fp = F + qoff + (int64_t)v * Lp;
  const uint8_t* Rp = SR + qoff + (int64_t)v * Lp;          // parent's current row
  uint8_t* Fc = F + qoff + (int64_t)(ch > 0 ? ch : 0) * Lp;  // written for an internal child only
  const uint8_t* Sc = SR + qoff + (int64_t)(ch > 0 ? ch : 0) * Lp;
  const uint8_t* Lc = ax + (int64_t)(ch <= 0 ? -ch : 0) * Lp;
  uint8_t* Cc = (ch <= 0) ? out_ax + (int64_t)q * out_slot_stride + (int64_t)(-ch) * Lp
                          : SR + qoff + (int64_t)ch * Lp;
  int* nsub = nsub_s[warp];
  if (lane < 25) nsub[lane] = 0;
  __syncwarp();

  // child's states (down pass for an internal child) and the substitution
  // counts parent -> child, 16 columns per lane and step
  for (int c0 = lane * 16; c0 < Lp; c0 += 32 * 16) {
    const uint4 pv = *reinterpret_cast<const uint4*>(Fp + c0);
    uint4 cv;
    if (ch > 0) {
      const uint4 sv = *reinterpret_cast<const uint4*>(Sc + c0);
      uint32_t pw[4] = {pv.x, pv.y, pv.z, pv.w}, sw[4] = {sv.x, sv.y, sv.z, sv.w}, ow[4];
#pragma unroll
      for (int k = 0; k < 4; k++) {
        uint32_t o = 0;
#pragma unroll
        for (int b = 0; b < 4; b++) {
          const int c = c0 + 4 * k + b;
          uint32_t st = 4;
          if (c < L) {
            const uint32_t a = (pw[k] >> (8 * b)) & 0xFFu;
            unsigned set = (sw[k] >> (8 * b)) & 0xFFu;
            if (set & (1u << a)) set = 1u << a;
            st = (uint32_t)choose_member(set, seed, nid, (uint32_t)ch, (uint32_t)c);
          }
          o |= st << (8 * b);
        }
        ow[k] = o;
      }
      cv = make_uint4(ow[0], ow[1], ow[2], ow[3]);
      *reinterpret_cast<uint4*>(Fc + c0) = cv;
    } else {
      cv = *reinterpret_cast<const uint4*>(Lc + c0);
    }
    const uint32_t pw[4] = {pv.x, pv.y, pv.z, pv.w}, cw[4] = {cv.x, cv.y, cv.z, cv.w};
#pragma unroll
    for (int k = 0; k < 4; k++) {
      if (pw[k] == cw[k]) continue;
#pragma unroll
      for (int b = 0; b < 4; b++) {
        const int c = c0 + 4 * k + b;
        const uint32_t a = (pw[k] >> (8 * b)) & 0xFFu, d = (cw[k] >> (8 * b)) & 0xFFu;
        if (c < L && a != d && a <= 4 && d <= 4) atomicAdd(&nsub[a * 5 + d], 1);
      }
    }
  }
  // the child's row starts as a copy of the parent's row
  for (int c0 = lane * 16; c0 < Lp; c0 += 32 * 16)
    *reinterpret_cast<uint4*>(Cc + c0) = *reinterpret_cast<const uint4*>(Rp + c0);
  __syncwarp();
  int (*cum)[6] = cum_s[warp];
  if (lane < 5) {
    cum[lane][0] = 0;
    for (int d = 0; d < 5; d++) cum[lane][d + 1] = cum[lane][d] + nsub[lane * 5 + d];
  }
  __syncwarp();
  int need[5], run[5] = {0, 0, 0, 0, 0}, total = 0;
#pragma unroll
  for (int o = 0; o < 5; o++) { need[o] = cum[o][5]; total += need[o]; }
  if (total == 0) return;

  // slot t -> position perm(t) of the parent's row; the r-th slot holding
  // state o (in slot order) takes substitution r of class o while r < need[o]
  uint32_t rk[6];
  round_keys(seed, TAG_SUBST, nid, (uint32_t)cidx, rk);
  const uint32_t hb = feistel_hbits((uint32_t)L);
  const unsigned lt = (1u << lane) - 1u;
  for (int t0 = 0; t0 < L; t0 += 32) {
    const int t = t0 + lane;
    uint32_t p = 0;
    int o = 5;
    if (t < L) {
      p = feistel_perm((uint32_t)t, hb, (uint32_t)L, rk);
      o = Rp[p];
    }
    bool done = true;
#pragma unroll
    for (int oc = 0; oc < 5; oc++) {
      const unsigned m = __ballot_sync(0xffffffffu, o == oc);
      if (o == oc) {
        const int r = run[oc] + __popc(m & lt);
        if (r < need[oc]) {
          int d = 0;
          while (r >= cum[oc][d + 1]) d++;
          Cc[p] = (uint8_t)d;
        }
      }
      run[oc] += __popc(m);
      done = done && (run[oc] >= need[oc]);
    }
    if (done) break;
  }
}

// down pass of the Fitch reconstruction for the internal children of one
// depth: one thread per (branch, 16 columns); a child keeps its parent's
// state when its set holds it, else a random member of its set
__global__ void __launch_bounds__(256)
k_fitch_down(int N, int L, int Lp, const int* __restrict__ left, const int* __restrict__ right,
             const int* __restrict__ nodes, int nn, uint64_t seed, uint32_t nid, const uint8_t* __restrict__ S,
             uint8_t* __restrict__ F) {
  const int chunks = Lp >> 4;
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= 2 * nn * chunks) return;
  const int kb = idx / chunks, c0 = (idx % chunks) << 4;
  const int v = nodes[kb >> 1];
  const int ch = (kb & 1) ? right[v] : left[v];
  if (ch <= 0) return;
  for (int k = 0; k < 16; k++) {
    const int c = c0 + k;
    uint8_t st = 4;
    if (c < L) {
      const int a = F[(int64_t)v * Lp + c];
      unsigned set = S[(int64_t)ch * Lp + c];
      if (set & (1u << a)) set = 1u << a;
      st = (uint8_t)choose_member(set, seed, nid, (uint32_t)ch, (uint32_t)c);
    }
    F[(int64_t)ch * Lp + c] = st;
  }
}

cudaError_t launch_fitch_recon(const uint8_t* ax, int N, int L, int Lp, const NullTree& T, const int* level_nodes,
                               const int* level_off, int nlevels, uint64_t seed, uint32_t nid, uint8_t* F, uint8_t* S,
                               cudaStream_t st) {
  const int chunks = Lp / 16;
  for (int d = nlevels - 1; d >= 0; d--) {
    const int nn = level_off[d + 1] - level_off[d];
    if (nn <= 0) continue;
    k_fitch_up<<<dim3((nn * chunks + 255) / 256, 1), 256, 0, st>>>(ax, N, Lp, T.left, T.right,
                                                                    level_nodes + level_off[d], nn, seed, nid, S);
  }
  k_root_state<<<dim3((L + 255) / 256, 1), 256, 0, st>>>(N, L, Lp, seed, nid, S, F);
  for (int d = 0; d < nlevels; d++) {
    const int nn = level_off[d + 1] - level_off[d];
    if (nn <= 0) continue;
    k_fitch_down<<<(2 * nn * chunks + 255) / 256, 256, 0, st>>>(N, L, Lp, T.left, T.right, level_nodes + level_off[d],
                                                                 nn, seed, nid, S, F);
  }
  return cudaGetLastError();
}

cudaError_t launch_nullgen(const uint8_t* ax, int N, int L, int Lp, const NullTree& T, const int* level_nodes,
                           const int* level_off, int nlevels, uint64_t seed, uint32_t first_null, int nnull,
                           uint8_t* fitch, uint8_t* scratch, uint8_t* out_ax, int64_t out_slot_stride,
                           cudaStream_t st) {
  // scratch holds the Fitch sets, each row replaced by the null's row once used
  const int chunks = Lp / 16;
  for (int d = nlevels - 1; d >= 0; d--) {
    const int nn = level_off[d + 1] - level_off[d];
    if (nn <= 0) continue;
    k_fitch_up<<<dim3((nn * chunks + 255) / 256, nnull), 256, 0, st>>>(ax, N, Lp, T.left, T.right,
                                                                       level_nodes + level_off[d], nn, seed,
                                                                       first_null, scratch);
  }
  k_root_state<<<dim3((L + 255) / 256, nnull), 256, 0, st>>>(N, L, Lp, seed, first_null, scratch, fitch);
  k_root_row<<<dim3((Lp + 255) / 256, nnull), 256, 0, st>>>(N, L, Lp, seed, first_null, fitch, scratch);
  for (int d = 0; d < nlevels; d++) {
    const int nn = level_off[d + 1] - level_off[d];
    if (nn <= 0) continue;
    k_replay<<<dim3((2 * nn + 7) / 8, nnull), 256, 0, st>>>(ax, N, L, Lp, T.left, T.right, level_nodes + level_off[d],
                                                             nn, seed, first_null, fitch, scratch, out_ax,
                                                             out_slot_stride);
  }
  return cudaGetLastError();
}

}  // namespace covgpu
