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
//   k_replay     top depth first, one CTA per (branch, null):
//                shuffle_tree_substitutions + shuffle_tree_substitute_all
//                (src/msamanip.c:1597-1747).  The CTA finishes the child's
//                Fitch state (down pass: keep the parent's state when the
//                child's set holds it), counts the branch's substitutions on
//                the unshuffled reconstruction, copies the parent's current
//                row and replays the substitutions on positions of that row
//                holding the old state, visited in a random order (a Feistel
//                permutation), 256 slots at a time; each class's positions
//                are ranked with warp ballots and a prefix over the warps,
//                and the pass stops once every substitution is placed.
//
// Random draws are counter-based (Philox keyed by the seed, the null index,
// the node and the column), so the result does not depend on scheduling.
//
// Buffers (per null q): F[q][v][Lp] the Fitch states of internal node v;
// SR[q][v][Lp] first its Fitch set, then (once the set is used) its row of
// the null alignment; leaf rows go straight to the output alignment slot.
#include "cov_dev.cuh"
#include "cov_kernels.h"
#include "cov_batch.h"

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
__device__ __forceinline__ void fitch_up_body(
    const GridIdx g, const uint8_t* __restrict__ ax, int N, int Lp, const int* __restrict__ left,
    const int* __restrict__ right, const int* __restrict__ nodes, int nn, uint64_t seed, uint32_t first_null,
    uint8_t* __restrict__ SR) {
  const int chunks = Lp >> 4;
  const int idx = g.x * blockDim.x + threadIdx.x;
  if (idx >= nn * chunks) return;
  const int q = g.y, v = nodes[idx / chunks], c0 = (idx % chunks) << 4;
  const uint32_t nid = first_null + q;
  uint8_t* S = SR + (int64_t)q * (N - 1) * Lp;
  const uint4 a = child_sets(left[v], ax, S, Lp, c0, seed, nid);
  const uint4 b = child_sets(right[v], ax, S, Lp, c0, seed, nid);
  *reinterpret_cast<uint4*>(S + (int64_t)v * Lp + c0) =
      make_uint4(fitch_word(a.x, b.x), fitch_word(a.y, b.y), fitch_word(a.z, b.z), fitch_word(a.w, b.w));
}
__global__ void __launch_bounds__(256)
k_fitch_up(const uint8_t* __restrict__ ax, int N, int Lp, const int* __restrict__ left, const int* __restrict__ right,
           const int* __restrict__ nodes, int nn, uint64_t seed, uint32_t first_null, uint8_t* __restrict__ SR) {
  fitch_up_body(native_grid(), ax, N, Lp, left, right, nodes, nn, seed, first_null, SR);
}

// the root's states F[q][0][c] from its sets
__device__ __forceinline__ void root_state_body(
    const GridIdx g, int N, int L, int Lp, uint64_t seed, uint32_t first_null, const uint8_t* __restrict__ SR,
             uint8_t* __restrict__ F) {
  const int c = g.x * blockDim.x + threadIdx.x, q = g.y;
  if (c >= L) return;
  const int64_t off = (int64_t)q * (N - 1) * Lp;
  F[off + c] = (uint8_t)choose_member(SR[off + c], seed, first_null + q, 0u, (uint32_t)c);
}
__global__ void __launch_bounds__(256)
k_root_state(int N, int L, int Lp, uint64_t seed, uint32_t first_null, const uint8_t* __restrict__ SR,
             uint8_t* __restrict__ F) {
  root_state_body(native_grid(), N, L, Lp, seed, first_null, SR, F);
}

// the root's row of the null: its states with the columns shuffled
__device__ __forceinline__ void root_row_body(
    const GridIdx g, int N, int L, int Lp, uint64_t seed, uint32_t first_null, const uint8_t* __restrict__ F,
           uint8_t* __restrict__ SR) {
  const int c = g.x * blockDim.x + threadIdx.x, q = g.y;
  if (c >= Lp) return;
  uint32_t rk[6];
  round_keys(seed, TAG_COLPERM, first_null + q, 0, rk);
  const int64_t off = (int64_t)q * (N - 1) * Lp;
  SR[off + c] = (c < L) ? F[off + feistel_perm((uint32_t)c, feistel_hbits((uint32_t)L), (uint32_t)L, rk)] : (uint8_t)4;
}
__global__ void __launch_bounds__(256)
k_root_row(int N, int L, int Lp, uint64_t seed, uint32_t first_null, const uint8_t* __restrict__ F,
           uint8_t* __restrict__ SR) {
  root_row_body(native_grid(), N, L, Lp, seed, first_null, F, SR);
}

// The replay of one (branch, null) item: phase 1, the child's Fitch states
// (down pass) and the branch's substitution counts, 16 columns per thread;
// phase 2, the child's row starts as a copy of the parent's row (staged in
// shared memory too when srow is given, for the random reads of phase 3);
// phase 3 walks the slots t in order, maps each to position perm(t) of the
// parent's row and, for the state o there, ranks the slot among the slots of
// class o so far: the r-th takes substitution r of class o while r <
// need[o].  Once every class has its substitutions the walk stops (later
// slots would place nothing).  Two kernels run phase 3: one warp per item,
// 32 slots a step (levels with many items), and one CTA per item, 256 slots
// a step with a prefix over the warps (levels with few, long items).
struct ReplayItem {
  int ch, cidx;
  uint32_t nid;
  const uint8_t *Fp, *Rp, *Sc, *Lc;
  uint8_t *Fc, *Cc;
};

__device__ __forceinline__ ReplayItem replay_item(const uint8_t* ax, int N, int Lp, const int* left, const int* right,
                                                  const int* nodes, int item, int q, uint32_t first_null,
                                                  uint8_t* F, uint8_t* SR, uint8_t* out_ax, int64_t out_slot_stride) {
  ReplayItem it;
  const int v = nodes[item >> 1];
  it.ch = (item & 1) ? right[v] : left[v];
  it.cidx = (it.ch <= 0) ? -it.ch : N + it.ch;
  it.nid = first_null + q;
  const int64_t qoff = (int64_t)q * (N - 1) * Lp;
  it.Fp = F + qoff + (int64_t)v * Lp;
  it.Rp = SR + qoff + (int64_t)v * Lp;                            // parent's current row
  it.Fc = F + qoff + (int64_t)(it.ch > 0 ? it.ch : 0) * Lp;       // written for an internal child only
  it.Sc = SR + qoff + (int64_t)(it.ch > 0 ? it.ch : 0) * Lp;
  it.Lc = ax + (int64_t)(it.ch <= 0 ? -it.ch : 0) * Lp;
  it.Cc = (it.ch <= 0) ? out_ax + (int64_t)q * out_slot_stride + (int64_t)(-it.ch) * Lp
                       : SR + qoff + (int64_t)it.ch * Lp;
  return it;
}

// phases 1 and 2 by nthr threads (this one: tid); nsub (25 counters, zeroed)
// and srow (nullptr or Lp bytes) in shared memory
__device__ __forceinline__ void replay_prepare(const ReplayItem& it, int L, int Lp, uint64_t seed, int tid, int nthr,
                                               int* nsub, uint8_t* srow) {
  for (int c0 = tid * 16; c0 < Lp; c0 += nthr * 16) {
    const uint4 pv = *reinterpret_cast<const uint4*>(it.Fp + c0);
    uint4 cv;
    if (it.ch > 0) {
      const uint4 sv = *reinterpret_cast<const uint4*>(it.Sc + c0);
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
            st = (uint32_t)choose_member(set, seed, it.nid, (uint32_t)it.ch, (uint32_t)c);
          }
          o |= st << (8 * b);
        }
        ow[k] = o;
      }
      cv = make_uint4(ow[0], ow[1], ow[2], ow[3]);
      *reinterpret_cast<uint4*>(it.Fc + c0) = cv;
    } else {
      cv = *reinterpret_cast<const uint4*>(it.Lc + c0);
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
  for (int c0 = tid * 16; c0 < Lp; c0 += nthr * 16) {   // Lp is a multiple of 32
    const uint4 v4 = *reinterpret_cast<const uint4*>(it.Rp + c0);
    *reinterpret_cast<uint4*>(it.Cc + c0) = v4;
    if (srow) *reinterpret_cast<uint4*>(srow + c0) = v4;
  }
}

__device__ __forceinline__ unsigned pick5(const unsigned (&m)[5], int k) {
  return k == 0 ? m[0] : k == 1 ? m[1] : k == 2 ? m[2] : k == 3 ? m[3] : m[4];
}

// one warp per item, eight items per CTA (SROW: Lp bytes of row per warp)
template <bool SROW>
__device__ __forceinline__ void replay_warp_body(
    const GridIdx g, const uint8_t* __restrict__ ax, int N, int L, int Lp, const int* __restrict__ left,
              const int* __restrict__ right, const int* __restrict__ nodes, int nn, uint64_t seed,
              uint32_t first_null, uint8_t* __restrict__ F, uint8_t* __restrict__ SR, uint8_t* __restrict__ out_ax,
              int64_t out_slot_stride) {
  extern __shared__ __align__(16) uint8_t rowbuf[];
  __shared__ int nsub_s[8][25];
  __shared__ int cum_s[8][5][6];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int item = g.x * 8 + warp;
  if (item >= 2 * nn) return;
  const ReplayItem it = replay_item(ax, N, Lp, left, right, nodes, item, g.y, first_null, F, SR, out_ax,
                                    out_slot_stride);
  int* nsub = nsub_s[warp];
  if (lane < 25) nsub[lane] = 0;
  __syncwarp();
  uint8_t* srow = SROW ? rowbuf + (size_t)warp * Lp : nullptr;
  replay_prepare(it, L, Lp, seed, lane, 32, nsub, srow);
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
  uint32_t rk[6];
  round_keys(seed, TAG_SUBST, it.nid, (uint32_t)it.cidx, rk);
  const uint32_t hb = feistel_hbits((uint32_t)L);
  const unsigned lt = (1u << lane) - 1u;
  const uint8_t* R = SROW ? srow : it.Rp;
  for (int t0 = 0; t0 < L; t0 += 32) {
    const int t = t0 + lane;
    uint32_t p = 0;
    int o = 5;
    if (t < L) {
      p = feistel_perm((uint32_t)t, hb, (uint32_t)L, rk);
      o = R[p];
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
          it.Cc[p] = (uint8_t)d;
        }
      }
      run[oc] += __popc(m);
      done = done && (run[oc] >= need[oc]);
    }
    if (done) break;
  }
}
template <bool SROW>
__global__ void __launch_bounds__(256)
k_replay_warp(const uint8_t* __restrict__ ax, int N, int L, int Lp, const int* __restrict__ left,
              const int* __restrict__ right, const int* __restrict__ nodes, int nn, uint64_t seed,
              uint32_t first_null, uint8_t* __restrict__ F, uint8_t* __restrict__ SR, uint8_t* __restrict__ out_ax,
              int64_t out_slot_stride) {
  replay_warp_body<SROW>(native_grid(), ax, N, L, Lp, left, right, nodes, nn, seed, first_null, F, SR, out_ax,
                                        out_slot_stride);
}

// one CTA per item (SROW: Lp bytes of row)
template <bool SROW>
__device__ __forceinline__ void replay_cta_body(
    const GridIdx g, const uint8_t* __restrict__ ax, int N, int L, int Lp, const int* __restrict__ left,
             const int* __restrict__ right, const int* __restrict__ nodes, int nn, uint64_t seed,
             uint32_t first_null, uint8_t* __restrict__ F, uint8_t* __restrict__ SR, uint8_t* __restrict__ out_ax,
             int64_t out_slot_stride) {
  extern __shared__ __align__(16) uint8_t rowbuf[];
  __shared__ int nsub[25];
  __shared__ int cum[5][6];
  __shared__ int gcnt[8][5];   // slots per class in each warp's group of the chunk
  __shared__ int base[5];      // slots per class before the chunk
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int item = g.x;
  if (item >= 2 * nn) return;
  const ReplayItem it = replay_item(ax, N, Lp, left, right, nodes, item, g.y, first_null, F, SR, out_ax,
                                    out_slot_stride);
  if (tid < 25) nsub[tid] = 0;
  __syncthreads();
  replay_prepare(it, L, Lp, seed, tid, 256, nsub, SROW ? rowbuf : nullptr);
  __syncthreads();
  if (tid < 5) {
    cum[tid][0] = 0;
    for (int d = 0; d < 5; d++) cum[tid][d + 1] = cum[tid][d] + nsub[tid * 5 + d];
    base[tid] = 0;
  }
  __syncthreads();
  int need[5], total = 0;
#pragma unroll
  for (int o = 0; o < 5; o++) { need[o] = cum[o][5]; total += need[o]; }
  if (total == 0) return;   // the same in every thread
  uint32_t rk[6];
  round_keys(seed, TAG_SUBST, it.nid, (uint32_t)it.cidx, rk);
  const uint32_t hb = feistel_hbits((uint32_t)L);
  const unsigned lt = (1u << lane) - 1u;
  const uint8_t* R = SROW ? rowbuf : it.Rp;
  for (int t0 = 0; t0 < L; t0 += 256) {
    const int t = t0 + tid;
    uint32_t p = 0;
    int o = 5;
    if (t < L) {
      p = feistel_perm((uint32_t)t, hb, (uint32_t)L, rk);
      o = R[p];
    }
    unsigned m[5];
#pragma unroll
    for (int oc = 0; oc < 5; oc++) m[oc] = __ballot_sync(0xffffffffu, o == oc);
    if (lane < 5) gcnt[warp][lane] = __popc(pick5(m, lane));
    __syncthreads();
    if (o < 5) {
      int r = base[o] + __popc(pick5(m, o) & lt);
      for (int w = 0; w < warp; w++) r += gcnt[w][o];
      if (r < cum[o][5]) {   // need[o], read from shared memory (o varies by lane)
        int d = 0;
        while (r >= cum[o][d + 1]) d++;
        it.Cc[p] = (uint8_t)d;
      }
    }
    __syncthreads();   // base and gcnt read
    if (tid < 5) {
      int s2 = base[tid];
      for (int w = 0; w < 8; w++) s2 += gcnt[w][tid];
      base[tid] = s2;
    }
    __syncthreads();
    bool all = true;
#pragma unroll
    for (int oc = 0; oc < 5; oc++) all = all && (base[oc] >= need[oc]);
    if (all) break;   // the same in every thread
  }
}
template <bool SROW>
__global__ void __launch_bounds__(256)
k_replay_cta(const uint8_t* __restrict__ ax, int N, int L, int Lp, const int* __restrict__ left,
             const int* __restrict__ right, const int* __restrict__ nodes, int nn, uint64_t seed,
             uint32_t first_null, uint8_t* __restrict__ F, uint8_t* __restrict__ SR, uint8_t* __restrict__ out_ax,
             int64_t out_slot_stride) {
  replay_cta_body<SROW>(native_grid(), ax, N, L, Lp, left, right, nodes, nn, seed, first_null, F, SR, out_ax,
                                       out_slot_stride);
}

// items per level up to which the replay goes one CTA per item: measured on
// N=2000 x L=3000 with 20 nulls, one CTA per item is faster up to about 3,000
// items (long branches near the root), one warp per item beyond
constexpr int64_t kReplayCtaItems = 3000;

// the replay's shared-memory row buffers: the launch limit of both kernels
// is raised once to the device's opt-in maximum; rows that do not fit are
// read from global memory instead
static int replay_smem_limit() {
  static const int lim = [] {
    int dev = 0, optin = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess)
      return 48 * 1024;
    const int dyn = optin - 4096;   // room for the kernels' static arrays
    if (dyn <= 48 * 1024 ||
        cudaFuncSetAttribute(k_replay_warp<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn) != cudaSuccess ||
        cudaFuncSetAttribute(k_replay_cta<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn) != cudaSuccess)
      return 48 * 1024;
    return dyn;
  }();
  return lim;
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
  // levels with few items (near the root and the leaves) go one CTA per
  // item; the others one warp per item
  const int lim = replay_smem_limit();
  const bool srow_cta = (size_t)Lp <= (size_t)lim, srow_warp = (size_t)8 * Lp <= (size_t)lim;
  for (int d = 0; d < nlevels; d++) {
    const int nn = level_off[d + 1] - level_off[d];
    if (nn <= 0) continue;
    const int* lv = level_nodes + level_off[d];
    if ((int64_t)2 * nn * nnull <= kReplayCtaItems) {
      const dim3 g(2 * nn, nnull);
      if (srow_cta)
        k_replay_cta<true><<<g, 256, (size_t)Lp, st>>>(ax, N, L, Lp, T.left, T.right, lv, nn, seed, first_null, fitch,
                                                      scratch, out_ax, out_slot_stride);
      else
        k_replay_cta<false><<<g, 256, 0, st>>>(ax, N, L, Lp, T.left, T.right, lv, nn, seed, first_null, fitch,
                                               scratch, out_ax, out_slot_stride);
    } else {
      const dim3 g((2 * nn + 7) / 8, nnull);
      if (srow_warp)
        k_replay_warp<true><<<g, 256, (size_t)8 * Lp, st>>>(ax, N, L, Lp, T.left, T.right, lv, nn, seed, first_null,
                                                            fitch, scratch, out_ax, out_slot_stride);
      else
        k_replay_warp<false><<<g, 256, 0, st>>>(ax, N, L, Lp, T.left, T.right, lv, nn, seed, first_null, fitch,
                                                scratch, out_ax, out_slot_stride);
    }
  }
  return cudaGetLastError();
}

// ------------------------------------------------------------------------
// grouped launches over a batch of families: one tree depth of every
// family per launch (lv[f] = {offset of the depth in lnodes, nodes at it});
// every family's nulls use the single-family streams (null ids 0..ns-1)
// ------------------------------------------------------------------------
__global__ void __launch_bounds__(256)
k_fitch_up_grp(const FamDev* __restrict__ F, int nf, const int2* __restrict__ lv, const int* __restrict__ pre,
               uint64_t seed) {
  const int f = grp_find(pre, nf, (int)blockIdx.x);
  const FamDev& d = F[f];
  const int2 v = lv[f];
  const int gx = (v.y * (d.Lp >> 4) + 255) / 256, loc = (int)blockIdx.x - __ldg(pre + f);
  fitch_up_body(GridIdx{loc % gx, loc / gx, gx}, d.ax, d.N, d.Lp, d.left, d.right, d.lnodes + v.x, v.y, seed, 0u,
                d.scratch);
}

__global__ void __launch_bounds__(256)
k_root_state_grp(const FamDev* __restrict__ F, int nf, const int* __restrict__ pre, uint64_t seed) {
  const int f = grp_find(pre, nf, (int)blockIdx.x);
  const FamDev& d = F[f];
  const int gx = (d.L + 255) / 256, loc = (int)blockIdx.x - __ldg(pre + f);
  root_state_body(GridIdx{loc % gx, loc / gx, gx}, d.N, d.L, d.Lp, seed, 0u, d.scratch, d.fitch);
}

__global__ void __launch_bounds__(256)
k_root_row_grp(const FamDev* __restrict__ F, int nf, const int* __restrict__ pre, uint64_t seed) {
  const int f = grp_find(pre, nf, (int)blockIdx.x);
  const FamDev& d = F[f];
  const int gx = (d.Lp + 255) / 256, loc = (int)blockIdx.x - __ldg(pre + f);
  root_row_body(GridIdx{loc % gx, loc / gx, gx}, d.N, d.L, d.Lp, seed, 0u, d.fitch, d.scratch);
}

template <bool SROW>
__global__ void __launch_bounds__(256)
k_replay_warp_grp(const FamDev* __restrict__ F, int nf, const int2* __restrict__ lv, const int* __restrict__ pre,
                  uint64_t seed) {
  const int f = grp_find(pre, nf, (int)blockIdx.x);
  const FamDev& d = F[f];
  const int2 v = lv[f];
  const int gx = (2 * v.y + 7) / 8, loc = (int)blockIdx.x - __ldg(pre + f);
  const int64_t ss = (int64_t)d.N * d.Lp;
  replay_warp_body<SROW>(GridIdx{loc % gx, loc / gx, gx}, d.ax, d.N, d.L, d.Lp, d.left, d.right, d.lnodes + v.x, v.y,
                         seed, 0u, d.fitch, d.scratch, d.ax + ss, ss);
}

template <bool SROW>
__global__ void __launch_bounds__(256)
k_replay_cta_grp(const FamDev* __restrict__ F, int nf, const int2* __restrict__ lv, const int* __restrict__ pre,
                 uint64_t seed) {
  const int f = grp_find(pre, nf, (int)blockIdx.x);
  const FamDev& d = F[f];
  const int2 v = lv[f];
  const int gx = 2 * v.y, loc = (int)blockIdx.x - __ldg(pre + f);
  const int64_t ss = (int64_t)d.N * d.Lp;
  replay_cta_body<SROW>(GridIdx{loc % gx, loc / gx, gx}, d.ax, d.N, d.L, d.Lp, d.left, d.right, d.lnodes + v.x, v.y,
                        seed, 0u, d.fitch, d.scratch, d.ax + ss, ss);
}

bool replay_uses_cta(int nn, int nnull) { return (int64_t)2 * nn * nnull <= kReplayCtaItems; }
int replay_smem_max() {
  static const int lim = [] {
    const int l = replay_smem_limit();
    if (l > 48 * 1024 &&
        (cudaFuncSetAttribute(k_replay_warp_grp<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, l) != cudaSuccess ||
         cudaFuncSetAttribute(k_replay_cta_grp<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, l) != cudaSuccess))
      return 48 * 1024;
    return l;
  }();
  return lim;
}

cudaError_t grp_fitch_up(const FamDev* F, int nf, const int2* lv, const int* pre, int nb, uint64_t seed,
                         cudaStream_t st) {
  if (nb > 0) k_fitch_up_grp<<<nb, 256, 0, st>>>(F, nf, lv, pre, seed);
  return cudaGetLastError();
}

cudaError_t grp_root(const FamDev* F, int nf, const int* pre_state, int nb_state, const int* pre_row, int nb_row,
                     uint64_t seed, cudaStream_t st) {
  if (nb_state > 0) k_root_state_grp<<<nb_state, 256, 0, st>>>(F, nf, pre_state, seed);
  if (nb_row > 0) k_root_row_grp<<<nb_row, 256, 0, st>>>(F, nf, pre_row, seed);
  return cudaGetLastError();
}

// srow: every family of the launch has its rows staged in shared memory
// (maxLp bytes per item)
cudaError_t grp_replay(const FamDev* F, int nf, const int2* lv, const int* pre, int nb, bool cta, bool srow,
                       int maxLp, uint64_t seed, cudaStream_t st) {
  if (nb <= 0) return cudaSuccess;
  if (cta) {
    if (srow) k_replay_cta_grp<true><<<nb, 256, (size_t)maxLp, st>>>(F, nf, lv, pre, seed);
    else      k_replay_cta_grp<false><<<nb, 256, 0, st>>>(F, nf, lv, pre, seed);
  } else {
    if (srow) k_replay_warp_grp<true><<<nb, 256, (size_t)8 * maxLp, st>>>(F, nf, lv, pre, seed);
    else      k_replay_warp_grp<false><<<nb, 256, 0, st>>>(F, nf, lv, pre, seed);
  }
  return cudaGetLastError();
}

}  // namespace covgpu
