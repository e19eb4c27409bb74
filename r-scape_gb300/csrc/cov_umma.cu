// cov_umma.cu -- pair counting on the 5th-generation tensor cores (sm_103a).
//
// The 4x4 joint counts of every column pair are the one-hot contraction
//   C = X^T diag(w) X,   X[s, 4i+x] = [a_si == x]  (x = A,C,G,U; gaps and
//                                                    unknown residues: 0)
// of mutual_naive_ppij (src/correlators.c:1695-1780) for all pairs at once.
// Operands, K-major (sequences contiguous):
//   A      = X^T                         (0/1, exact)
//   B_l    = l_l(s) X^T,  l = 0..2        weight limbs: each weight is
//            quantised to q_s = round(w_s 2^E) < 2^(3b) and split into three
//            b-bit limbs q = l0 + 2^b l1 + 2^2b l2, b = min(11,
//            floor(log2((2^24 - 1)/N))): integers exact in FP16, FP16
//            operands (33-bit weights up to N = 8196, 27 bits at N = 20000).
// Each limb accumulates in its own FP32 TMEM accumulator, where the sum
// (<= (2^b - 1) N < 2^24) is an exact integer; the epilogue combines the
// three with error-free FP32 sums into a double-float count (limb_count),
// exact to 2^-46 relative, times the power of two 2^-E, with no FP64 and no
// integer conversion on the path (exact integers under unit weights).  The
// double-float counts go out as two planes (hi, lo).  Equal weights take one
// limb (the unit count times the weight, unit_count).  Three limbs need 384
// TMEM columns, one accumulator set: the epilogue reads a cell row of all
// three limbs, hands the set back after the last row, and stores while the
// next task's MMAs run.
//
// Operand rows are state-major inside each 32-column tile
// (row = 128 tile + 32 x + column), so accumulator row m = 32 x + a and
// column n = 32 y + b: warp x, lane a of the epilogue holds cell (x, y) of
// the pairs (a, b = 0..31), one contiguous 128-byte row of the count tile.
//
// Kernel: persistent, one CTA per SM working through (column tile I <= J,
// alignment) tasks in a blocked raster order; 128-row operand tiles (32
// columns x 4 states), K in blocks of 64 sequences (128 with FP8).  Warp 0
// lane 0 issues TMA loads (128B-swizzled boxes) into a 3-4 stage ring guarded
// by mbarriers, warp 1 lane 0 issues tcgen05.mma into TMEM (kind::f16
// 128x256x16 over limbs 0 and 1, whose B tiles are adjacent; kind::f8f6f4
// 128x256x32 over two column tiles for unit weights) and
// frees stages with tcgen05.commit; four epilogue warps read their 32 TMEM
// lanes each (tcgen05.ld 32x32b.x32), hand the accumulators back, combine
// the limbs, write the 32x32 block of one cell into a 128B-swizzled shared
// buffer (conflict free) and store it with a TMA tensor store,
// double-buffered, while the next task's MMAs run.  The counts land in the
// layout of the SIMT kernel, [slot][tile][cell][32 a][32 b].  Every wait is
// bounded: on timeout the kernel records an error code, drains its copies
// with a bounded wait and frees TMEM before returning.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "cov_df.cuh"
#include "cov_kernels.h"
#include "cov_umma.h"
#include "cov_batch.h"

namespace covgpu {

constexpr int UM = 128;          // rows of A tile (32 columns x 4 states)
constexpr int UN = 128;          // rows of B tile
constexpr int UK = 64;           // sequences per stage (128 bytes of BF16)
constexpr int UK8 = 128;         // sequences per stage of the FP8 operands (128 bytes)
constexpr int TILE_BYTES = UM * UK * 2;   // 16 KB per operand tile
constexpr uint64_t WAIT_NS = 2000000000ull;   // every barrier wait gives up after 2 s

struct UmmaPlan {
  int N = 0, L = 0, Lp = 0, nT = 0, ntiles = 0, maxslots = 0;
  int Npad = 0;                  // sequences padded to UK
  const TileRC* d_tiles = nullptr;
  int* d_order = nullptr;           // launch order of the tiles (blocked raster)
  int4* d_jpairs = nullptr;         // unit-weight tasks: {I, J0, tile (I, J0), tile (I, J0 + 1)}, same raster
  int njpairs = 0;
  __nv_bfloat16* d_ops = nullptr;   // [(1 + 3) * maxslots * 4Lp][Npad] FP16 bits: one-hot, then 3 limb buffers
  uint8_t* d_ops8 = nullptr;        // [maxslots * 4Lp][Npad8] FP8 E4M3 one-hot (unit weights)
  int Npad8 = 0;                    // sequences padded to UK8
  CUtensorMap tmap8;
  uint16_t* d_limbs = nullptr;      // [3][Npad] weight limbs
  CountWeights cw;                  // limbs in use (1 when all weights are equal, else 3) and the scale
  CUtensorMap tmap;
  int* d_err = nullptr;
  int nsm = 152;
  int sb = 10;                      // raster super-block (tiles per side), set by umma_autotune
  // capacity of the buffers (the plan can be resized within it)
  int capN = 0, capLp = 0, order_cap = 0;
  size_t ops_bytes = 0, ops8_bytes = 0;
};

// ---------------------------------------------------------------------------
// device helpers (inline PTX)
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ uint64_t globaltimer() {
  uint64_t t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}

// bounded wait for the phase with the given parity; false after WAIT_NS
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  const uint32_t a = smem_u32(bar);
  uint64_t t0 = 0;
  for (uint32_t it = 0;; it++) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
    if ((it & 255u) == 0) {
      const uint64_t now = globaltimer();
      if (t0 == 0) t0 = now;
      else if (now - t0 > WAIT_NS) return false;
    }
  }
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          smem_u32(dst)),
      "l"(map), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

// shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups
// 1024 bytes apart (start address and offsets in 16-byte units)
__device__ __forceinline__ uint64_t make_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFF) >> 4);          // start address
  d |= (uint64_t)1 << 16;                           // leading byte offset (unused for SW128 K-major)
  d |= (uint64_t)(1024 >> 4) << 32;                 // stride byte offset
  d |= (uint64_t)1 << 46;                           // descriptor version
  d |= (uint64_t)2 << 61;                           // SWIZZLE_128B
  return d;
}

// instruction descriptor, kind::f16: F16 x F16 -> F32, both K-major (A and
// B formats 0 = F16)
__host__ __device__ constexpr uint32_t make_idesc_fp16(int M, int N) {
  return (1u << 4) | (0u << 7) | (0u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// instruction descriptor, kind::f8f6f4: E4M3 x E4M3 -> F32, both K-major
__host__ __device__ constexpr uint32_t make_idesc_e4m3(int M, int N) {
  return (1u << 4) | (0u << 7) | (0u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void umma_e4m3(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                          uint32_t accum) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n}\n" ::"r"(dtmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accum)
      : "memory");
}

__device__ __forceinline__ void umma_f16(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accum) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dtmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accum)
      : "memory");
}

__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
}

__device__ __forceinline__ void tmem_ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

__device__ __forceinline__ void tma_store_2d(const CUtensorMap* map, const void* src, int x, int y) {
  asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%2, %3}], [%1];" ::"l"(map),
               "r"(smem_u32(src)), "r"(x), "r"(y)
               : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void bulk_wait_read() {
  asm volatile("cp.async.bulk.wait_group.read %0;" ::"n"(N) : "memory");
}
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// ---------------------------------------------------------------------------
// operand preparation: codes [slot][N][Lp] -> one-hot rows [4Lp][Npad] (A)
// and limb-scaled rows (B_l), FP16, row 128 t + 32 x + c for column 32 t + c
// and state x; one CTA per (64 sequences, 32 columns, slot)
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint16_t op_bits(float v) { return __half_as_ushort(__float2half_rn(v)); }

// (sb, cb, slot): the block of 64 sequences, of 32 columns, the alignment;
// pitch: sequences per operand row; limbs: [3][lstride]
__device__ __forceinline__ void umma_prep_body(int sb, int cb, int slot, const uint8_t* __restrict__ ax,
                                               int64_t slot_stride, int N, int Lp, int pitch, int nslots, int nl,
                                               const uint16_t* __restrict__ limbs, int lstride, bool unit,
                                               uint16_t* __restrict__ ops) {
  __shared__ uint8_t cs[64][33];
  __shared__ uint16_t lb[3][64];
  const int s0 = sb * 64, c0 = cb * 32, tid = threadIdx.x;
  const uint8_t* A = ax + (int64_t)slot * slot_stride;
  for (int e = tid; e < 64 * 32; e += 256) {
    const int s = e / 32, c = e % 32;
    cs[s][c] = (s0 + s < N) ? A[(int64_t)(s0 + s) * Lp + c0 + c] : (uint8_t)4;
  }
  if (tid < 64)
    for (int l = 0; l < nl; l++) lb[l][tid] = (s0 + tid < N) ? (unit ? 1 : limbs[l * lstride + s0 + tid]) : 0;
  __syncthreads();
  // 128 rows (4 states x 32 columns, state-major) x 64 sequences; each
  // thread writes 8 consecutive sequences (16 bytes) of one row
  const int64_t rows_per_buf = (int64_t)nslots * 4 * Lp;
  const uint16_t one = op_bits(1.f), zero = op_bits(0.f);
  for (int e = tid; e < 128 * 8; e += 256) {
    const int r = e / 8, chunk = e % 8;
    const int x = r / 32, c = r % 32;
    const int64_t row = (int64_t)slot * 4 * Lp + 4 * c0 + r;
    __align__(16) uint16_t va[8];
    __align__(16) uint16_t vb[3][8];
#pragma unroll
    for (int k = 0; k < 8; k++) {
      const int s = chunk * 8 + k;
      const bool on = (cs[s][c] == x);
      va[k] = on ? one : zero;
#pragma unroll
      for (int l = 0; l < 3; l++) vb[l][k] = (on && l < nl) ? op_bits((float)lb[l][s]) : zero;
    }
    *reinterpret_cast<uint4*>(ops + row * pitch + s0 + chunk * 8) = *reinterpret_cast<uint4*>(va);
#pragma unroll
    for (int l = 0; l < 3; l++)   // compile-time limb index: the arrays stay in registers
      if (l < nl)
        *reinterpret_cast<uint4*>(ops + ((1 + l) * rows_per_buf + row) * pitch + s0 + chunk * 8) =
            *reinterpret_cast<uint4*>(vb[l]);
  }
}

__global__ void __launch_bounds__(256)
k_umma_prep(const uint8_t* __restrict__ ax, int64_t slot_stride, int N, int Lp, int Npad, int nslots, int nl,
            const uint16_t* __restrict__ limbs, bool unit, uint16_t* __restrict__ ops) {
  umma_prep_body(blockIdx.x, blockIdx.y, blockIdx.z, ax, slot_stride, N, Lp, Npad, nslots, nl, limbs, Npad, unit,
                 ops);
}

// FP8 E4M3 one-hot rows [4Lp][Npad8] (1.0 = 0x38), state-major as above;
// one CTA per (128 sequences, 32 columns, slot)
__global__ void __launch_bounds__(256)
k_umma_prep8(const uint8_t* __restrict__ ax, int64_t slot_stride, int N, int Lp, int Npad8, int nslots,
             uint8_t* __restrict__ ops8) {
  __shared__ uint8_t cs[128][33];
  const int s0 = blockIdx.x * 128, c0 = blockIdx.y * 32, slot = blockIdx.z, tid = threadIdx.x;
  const uint8_t* A = ax + (int64_t)slot * slot_stride;
  for (int e = tid; e < 128 * 32; e += 256) {
    const int s = e / 32, c = e % 32;
    cs[s][c] = (s0 + s < N) ? A[(int64_t)(s0 + s) * Lp + c0 + c] : (uint8_t)4;
  }
  __syncthreads();
  // 128 rows x 128 sequences; each thread writes 16 sequences of one row
  for (int e = tid; e < 128 * 8; e += 256) {
    const int r = e / 8, chunk = e % 8;
    const int x = r / 32, c = r % 32;
    const int64_t row = (int64_t)slot * 4 * Lp + 4 * c0 + r;
    uint32_t w[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
      uint32_t v = 0;
#pragma unroll
      for (int b = 0; b < 4; b++) v |= (cs[chunk * 16 + 4 * k + b][c] == x ? 0x38u : 0u) << (8 * b);
      w[k] = v;
    }
    *reinterpret_cast<uint4*>(ops8 + row * Npad8 + s0 + chunk * 16) = make_uint4(w[0], w[1], w[2], w[3]);
  }
  (void)nslots;
}

// ---------------------------------------------------------------------------
// the counting kernel: persistent, one CTA (6 warps) per SM
//   warp 0 lane 0   TMA producer over all of the CTA's (tile, alignment)
//                   tasks: the stage ring and its phases run on across tasks
//   warp 1 lane 0   MMA issuer: per task, waits until the epilogue has
//                   drained the accumulator set it will use
//   warps 2..5      epilogue: warp w reads TMEM lanes 32 (w % 4) (cell row
//                   x = w % 4), releases the accumulator set after its last
//                   TMEM load, then combines, stages and stores while the
//                   next task's MMAs run
// The unit-weight (FP8) kernel takes two column tiles per task, J0 and
// J0 + 1 (jpairs: I, J0 and the two tile indices, -1 for a tile outside
// I <= J < nT, which is computed and not stored): one M = 128, N = 256 MMA
// reads the A tile once for both, where the shared-memory bandwidth, A and B
// read per MMA and written by TMA, bounded the one-tile form.
// ---------------------------------------------------------------------------
// GRP: a grouped launch over the families of a batch (fams, tpre, nfam):
// task k is task k - tpre[f] of family f, (slot, tile in fams[f].order); the
// operand rows, K blocks, weight scale and output rows are family f's;
// ntiles is then the number of tasks and nslots 1
template <int NL, int STAGES, int ACC, bool F8, bool GRP = false>
__global__ void __launch_bounds__(192, 1)
k_count_umma(const __grid_constant__ CUtensorMap tmap, const __grid_constant__ CUtensorMap omap,
             const TileRC* __restrict__ tiles, const int* __restrict__ order, int ntiles,
             const int4* __restrict__ jpairs, int npairs, int nslots_buf,
             int nslots, int Lp, int nkb, int bbuf, float B, float s_hi, float s_lo, unsigned cellmask,
             int* __restrict__ err, const UmmaFam* __restrict__ fams = nullptr, const int* __restrict__ tpre = nullptr,
             int nfam = 0) {
  static_assert(!(GRP && F8), "grouped launches count weighted alignments");
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  constexpr int NB = F8 ? 2 : NL;          // B tiles per stage (limbs, or the column tiles J0, J0 + 1)
  constexpr int STAGE_BYTES = TILE_BYTES * (1 + NB);
  constexpr int KE = F8 ? UK8 : UK;        // sequences per stage (one 128-byte row)
  constexpr uint32_t ACC_COLS = NB * UN;   // one accumulator set: NB x 128 columns
  constexpr uint32_t TMEM_COLS = (ACC * ACC_COLS <= 128) ? 128 : (ACC * ACC_COLS <= 256 ? 256 : 512);
  static_assert(ACC * ACC_COLS <= 512, "TMEM holds 512 columns");
  // 1024-byte aligned: the stage ring, then two 4 KB staging buffers per
  // epilogue warp
  uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint8_t* ring = smem;
  uint8_t* stagebuf = smem + (size_t)STAGES * STAGE_BYTES;
  __shared__ __align__(8) uint64_t full_bar[STAGES];
  __shared__ __align__(8) uint64_t empty_bar[STAGES];
  __shared__ __align__(8) uint64_t tfull_bar[ACC];    // MMA -> epilogue: accumulator set ready
  __shared__ __align__(8) uint64_t tempty_bar[ACC];   // epilogue -> MMA: accumulator set drained
  __shared__ uint32_t tmem_base;
  __shared__ int abort_flag;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int64_t nunits = F8 ? npairs : ntiles;   // tasks per alignment
  const int64_t ntask = nunits * nslots;
  const int64_t rows_per_buf = (int64_t)nslots_buf * 4 * Lp;

  if (tid == 0) {
    for (int s = 0; s < STAGES; s++) { mbar_init(&full_bar[s], 1); mbar_init(&empty_bar[s], 1); }
    for (int a = 0; a < ACC; a++) { mbar_init(&tfull_bar[a], 1); mbar_init(&tempty_bar[a], 4); }
    abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(&tmap) : "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(&omap) : "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_base;
  uint32_t issued = 0;   // k-blocks whose loads the producer issued

  if (warp == 0) {
    if (lane == 0) {
      // ---- TMA producer ----
      uint32_t g = 0;
      for (int64_t task = blockIdx.x; task < ntask; task += gridDim.x) {
        int rowA, rowB, tnkb = nkb;
        int64_t rpb = rows_per_buf;
        if (GRP) {
          const int f = grp_find(tpre, nfam, (int)task);
          const UmmaFam& fm = fams[f];
          const int loc = (int)task - tpre[f], slot = loc / fm.ntiles;
          const TileRC tr = fm.tiles[fm.order[loc - slot * fm.ntiles]];
          rowA = fm.row0 + slot * 4 * fm.Lp + tr.I * UM;
          rowB = fm.row0 + slot * 4 * fm.Lp + tr.J * UN;
          tnkb = fm.nkb;
          rpb = fm.rows_per_buf;
        } else {
          const int slot = (int)(task / nunits);
          int I, J0;
          if (F8) { const int4 q = jpairs[task % nunits]; I = q.x; J0 = q.y; }
          else    { const TileRC tr = tiles[order[task % nunits]]; I = tr.I; J0 = tr.J; }
          rowA = (int)((int64_t)slot * 4 * Lp + (int64_t)I * UM);
          rowB = (int)((int64_t)slot * 4 * Lp + (int64_t)J0 * UN);
        }
        for (int kb = 0; kb < tnkb; kb++, g++) {
          const int s = (int)(g % STAGES);
          const uint32_t ph = (g / STAGES) & 1u;
          if (g >= STAGES) {
            if (!mbar_wait(&empty_bar[s], ph ^ 1u)) { atomicExch(err, 101); abort_flag = 1; }
          }
          if (*(volatile int*)&abort_flag) break;
          uint8_t* st = ring + (size_t)s * STAGE_BYTES;
          mbar_expect_tx(&full_bar[s], STAGE_BYTES);
          tma_load_2d(st, &tmap, kb * KE, rowA, &full_bar[s]);
          // F8: the rows of J0 + 1 follow those of J0 (beyond the last
          // alignment of the buffer they lie outside the map: zero fill)
#pragma unroll
          for (int l = 0; l < NB; l++)
            tma_load_2d(st + (size_t)(1 + l) * TILE_BYTES, &tmap, kb * KE,
                        F8 ? rowB + l * UN : (int)((bbuf + l) * rpb) + rowB, &full_bar[s]);
          issued = g + 1;
        }
        if (*(volatile int*)&abort_flag) break;
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // ---- MMA issuer ----
      constexpr uint32_t idesc = F8 ? make_idesc_e4m3(UM, UN) : make_idesc_fp16(UM, UN);
      // limbs 0 and 1 as one M = 128, N = 256 MMA: their B tiles are
      // consecutive in the stage (256 rows, 1024-byte 8-row groups throughout)
      // and their accumulators consecutive in TMEM, so A is read from shared
      // memory once for both (the ring's shared-memory bandwidth, A read per
      // limb, bounded the two-MMA form)
      constexpr bool PAIR = !F8 && NL >= 2;
      constexpr uint32_t idesc2 = F8 ? make_idesc_e4m3(UM, 2 * UN) : make_idesc_fp16(UM, 2 * UN);
      uint32_t g = 0;
      int i = 0;
      for (int64_t task = blockIdx.x; task < ntask; task += gridDim.x, i++) {
        const int a = i % ACC;
        const uint32_t aph = (uint32_t)(i / ACC) & 1u;
        if (i >= ACC && !mbar_wait(&tempty_bar[a], aph ^ 1u)) { atomicExch(err, 105); abort_flag = 1; }
        if (*(volatile int*)&abort_flag) break;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t dacc = tmem + (uint32_t)a * ACC_COLS;
        int tnkb = nkb;
        if (GRP) tnkb = fams[grp_find(tpre, nfam, (int)task)].nkb;
        for (int kb = 0; kb < tnkb; kb++, g++) {
          const int s = (int)(g % STAGES);
          const uint32_t ph = (g / STAGES) & 1u;
          if (!mbar_wait(&full_bar[s], ph)) { atomicExch(err, 102); abort_flag = 1; }
          if (*(volatile int*)&abort_flag) break;
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint32_t sa = smem_u32(ring + (size_t)s * STAGE_BYTES);
#pragma unroll
          // four MMAs of 32 bytes of K each (16 BF16 or 32 FP8 sequences)
          for (int k16 = 0; k16 < 4; k16++) {
            const uint64_t ad = make_desc(sa + k16 * 32);
            const uint32_t acc = (kb > 0 || k16 > 0) ? 1u : 0u;
            const uint64_t bd = make_desc(sa + (uint32_t)TILE_BYTES + k16 * 32);
            if (F8) {              // column tiles J0 and J0 + 1
              umma_e4m3(dacc, ad, bd, idesc2, acc);
            } else if (PAIR) {     // limbs 0 and 1 (and limb 2 on its own)
              umma_f16(dacc, ad, bd, idesc2, acc);
              if (NL == 3) umma_f16(dacc + (uint32_t)(2 * UN), ad, make_desc(sa + 3u * TILE_BYTES + k16 * 32), idesc, acc);
            } else {
              umma_f16(dacc, ad, bd, idesc, acc);
            }
          }
          umma_commit(&empty_bar[s]);
        }
        if (*(volatile int*)&abort_flag) break;
        umma_commit(&tfull_bar[a]);
      }
    }
  } else {
    // ---- epilogue ----
    const int x = warp & 3;                         // TMEM lane quarter = cell row x
    uint8_t* wbuf = stagebuf + (size_t)(warp - 2) * 8192;
    uint32_t nst = 0;                               // TMA stores issued by this warp
    int i = 0;
    for (int64_t task = blockIdx.x; task < ntask; task += gridDim.x, i++) {
      const int a = i % ACC;
      const uint32_t aph = (uint32_t)(i / ACC) & 1u;
      if (!mbar_wait(&tfull_bar[a], aph)) { atomicExch(err, 103); abort_flag = 1; }
      __syncwarp();
      if (*(volatile int*)&abort_flag) break;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      int slot, t0, t1 = -1, tnt = ntiles;
      float tB = B, ts_hi = s_hi, ts_lo = s_lo;
      int64_t orow_f = 0;
      if (GRP) {
        const int f = grp_find(tpre, nfam, (int)task);
        const UmmaFam& fm = fams[f];
        const int loc = (int)task - tpre[f];
        slot = loc / fm.ntiles;
        t0 = fm.order[loc - slot * fm.ntiles];
        tnt = fm.ntiles;
        tB = fm.B; ts_hi = fm.s_hi; ts_lo = fm.s_lo;
        orow_f = fm.orow0;
      } else {
        slot = (int)(task / nunits);
        if (F8) { const int4 q = jpairs[task % nunits]; t0 = q.z; t1 = q.w; }
        else    { t0 = order[task % nunits]; }
      }
      const uint32_t taddr = tmem + ((uint32_t)(x * 32) << 16) + (uint32_t)a * ACC_COLS;
      // F8: cells of tile J0 (h = 0), then of J0 + 1 (h = 1)
      constexpr int NCHUNK = F8 ? 8 : 4;
#pragma unroll 1
      for (int cy = 0; cy < NCHUNK; cy++) {
        const int h = cy >> 2, y = cy & 3;
        uint32_t d[NL][32];
#pragma unroll
        for (int l = 0; l < NL; l++) tmem_ld32(taddr + (uint32_t)((F8 ? h : l) * UN + y * 32), d[l]);
        tmem_ld_wait();
        if (cy == NCHUNK - 1) {
          // this warp's last read of the accumulator set: hand it back
          asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
          __syncwarp();
          if (lane == 0)
            asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&tempty_bar[a])) : "memory");
        }
        // F8 (unit weights): exact FP32 integers, one plane; weighted:
        // double-float counts, a hi and a lo plane
        float vh[32], vl[32];
#pragma unroll
        for (int k = 0; k < 32; k++) {
          if (F8) {
            vh[k] = __uint_as_float(d[0][k]);
            vl[k] = 0.f;
          } else if (NL == 1) {
            const df c = unit_count(__uint_as_float(d[0][k]), ts_hi, ts_lo);
            vh[k] = c.hi; vl[k] = c.lo;
          } else {
            const df c = limb_count(__uint_as_float(d[0][k]), __uint_as_float(d[NL > 1 ? 1 : 0][k]),
                                    __uint_as_float(d[NL > 2 ? 2 : 0][k]), tB, ts_hi);
            vh[k] = c.hi; vl[k] = c.lo;
          }
        }
        const int t = h ? t1 : t0;
        if (t < 0) continue;                                // outside I <= J < nT
        if (!((cellmask >> (x * 4 + y)) & 1u)) continue;   // a cell nobody reads is not stored
        constexpr int NPL = F8 ? 1 : 2;
        // F8: row block of cell (x, y) in [slot][tile][16][32]; weighted: of
        // plane h2 of cell (x, y) in [slot][tile][16][2][32]
        const int orow0 = F8 ? ((slot * ntiles + t) * 16 + x * 4 + y) * 32
                             : (int)(orow_f + ((int64_t)(slot * tnt + t) * 32 + 2 * (x * 4 + y)) * 32);
#pragma unroll
        for (int h2 = 0; h2 < NPL; h2++) {
          uint8_t* buf = wbuf + (nst & 1u) * 4096;
          if (nst >= 2) {
            if (lane == 0) bulk_wait_read<1>();   // the store two back has read this buffer
            __syncwarp();
          }
          const float* v = h2 ? vl : vh;
          // row a = lane, 16-byte chunk c at position c ^ (a & 7) (128B swizzle)
#pragma unroll
          for (int c = 0; c < 8; c++)
            *reinterpret_cast<float4*>(buf + lane * 128 + ((c ^ (lane & 7)) << 4)) =
                make_float4(v[4 * c], v[4 * c + 1], v[4 * c + 2], v[4 * c + 3]);
          fence_proxy_async();
          __syncwarp();
          if (lane == 0) {
            tma_store_2d(&omap, buf, 0, orow0 + h2 * 32);
            bulk_commit();
          }
          nst++;
        }
      }
    }
    if (lane == 0) bulk_wait_all();
    __syncwarp();
  }
  // teardown: after an abort, drain the copies still in flight into the
  // ring before the shared memory is released
  if (warp == 0 && lane == 0 && *(volatile int*)&abort_flag) {
    for (uint32_t g = (issued > (uint32_t)STAGES ? issued - STAGES : 0u); g < issued; g++)
      mbar_wait(&full_bar[g % STAGES], (g / STAGES) & 1u);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    __syncwarp();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
  }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
static PFN_cuTensorMapEncodeTiled_v12000 get_encode() {
  // looked up once per process (thread-safe static initialisation)
  static const PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
    cudaDriverEntryPointQueryResult q;
    void* p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      return (PFN_cuTensorMapEncodeTiled_v12000)p;
    return (PFN_cuTensorMapEncodeTiled_v12000)nullptr;
  }();
  return fn;
}

constexpr int STAGES3 = 3;   // 3 limbs: 64 KB per stage
constexpr int STAGES1 = 4;   // 1 limb : 32 KB per stage (FP8, two column tiles: 48 KB)

constexpr int ACC3 = 1;      // 3 limbs: 384 TMEM columns, one accumulator set
constexpr int ACC1 = 2;      // 1 limb : two 128-column sets, epilogue overlapped

// nb = B tiles per stage (limbs, or the FP8 kernel's two column tiles)
static size_t smem_bytes(int nb, int stages) {
  const size_t ring = (size_t)stages * TILE_BYTES * (1 + nb);
  const size_t stage_out = (size_t)4 * 8192;   // two 4 KB buffers per epilogue warp
  return ring + stage_out + 1024;
}

// blocked raster: super-blocks of SBI x SBJ tiles (I <= J) in turn, band of
// SBI tile rows by band, so the CTAs resident at one time share a few operand
// row blocks in L2.  A schedule value v below 1000 is a square SB = v; v =
// 1000 SBI + SBJ is a band SBI rows high and SBJ columns wide (a tall band
// reads each column block's operands once per band, so fewer bands mean
// fewer re-reads of the B operands from DRAM).
static bool decode_sb(int v, int* sbi, int* sbj) {
  if (v < 1) return false;
  if (v < 1000) { *sbi = *sbj = v; return true; }
  *sbi = v / 1000; *sbj = v % 1000;
  return *sbi >= 1 && *sbj >= 1;
}

// the two task orders of a schedule value on nT x nT tiles (host code)
static bool build_order(int nT, int SB, std::vector<int>& order, std::vector<int4>& jp) {
  int SBI = 0, SBJ = 0;
  if (nT < 1 || !decode_sb(SB, &SBI, &SBJ)) return false;
  const int ntiles = nT * (nT + 1) / 2;
  order.clear();
  order.reserve(ntiles);
  auto tindex = [nT](int I, int J) { return I * nT - I * (I - 1) / 2 + (J - I); };   // I-major tile list
  for (int bI = 0; bI < nT; bI += SBI)
    for (int bJ = bI; bJ < nT; bJ += SBJ)
      for (int I = bI; I < std::min(nT, bI + SBI); I++)
        for (int J = std::max(I, bJ); J < std::min(nT, bJ + SBJ); J++) order.push_back(tindex(I, J));
  if ((int)order.size() != ntiles) return false;
  {   // every tile exactly once
    std::vector<char> seen(ntiles, 0);
    for (int t : order) {
      if (t < 0 || t >= ntiles || seen[t]) return false;
      seen[t] = 1;
    }
  }
  // column-tile pairs (J0, J0 + 1), J0 even, for the unit-weight kernel:
  // super-blocks of SBI rows x SBJ/2 pairs; each tile I <= J lies in exactly
  // one pair, so there are at most ntiles of them
  jp.clear();
  jp.reserve(ntiles);
  const int nP = (nT + 1) / 2, SP = std::max(1, SBJ / 2);
  for (int bI = 0; bI < nT; bI += SBI)
    for (int bP = bI / 2; bP < nP; bP += SP)
      for (int I = bI; I < std::min(nT, bI + SBI); I++)
        for (int q = std::max(I / 2, bP); q < std::min(nP, bP + SP); q++) {
          const int J0 = 2 * q;
          jp.push_back(make_int4(I, J0, J0 >= I ? tindex(I, J0) : -1, J0 + 1 < nT ? tindex(I, J0 + 1) : -1));
        }
  return (int)jp.size() <= ntiles;
}

static bool set_order(UmmaPlan* p, int SB) {
  std::vector<int> order;
  std::vector<int4> jp;
  if (!build_order(p->nT, SB, order, jp) || (int)order.size() != p->ntiles) return false;
  p->sb = SB;
  p->njpairs = (int)jp.size();
  return cudaMemcpy(p->d_order, order.data(), sizeof(int) * p->ntiles, cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemcpy(p->d_jpairs, jp.data(), sizeof(int4) * jp.size(), cudaMemcpyHostToDevice) == cudaSuccess;
}

}  // namespace covgpu

// host code, no device: the tensor count's task orders for a schedule value
// (see covgpu_autotune) on nT column tiles; order[nT (nT + 1) / 2] gets the
// weighted kernel's tiles (indices into the I-major list of tiles I <= J),
// jpairs[4 * capacity] the unit-weight kernel's {I, J0, tile (I, J0), tile
// (I, J0 + 1)} (-1 outside I <= J < nT), *njpairs their number
extern "C" int covgpu_tile_order(int nT, int schedule, int* order, int* jpairs, int jcap, int* njpairs) {
  std::vector<int> o;
  std::vector<int4> jp;
  if (!order || !njpairs || !covgpu::build_order(nT, schedule, o, jp)) return 11;
  if (jpairs && (int)jp.size() > jcap) return 11;
  std::memcpy(order, o.data(), sizeof(int) * o.size());
  if (jpairs) std::memcpy(jpairs, jp.data(), sizeof(int4) * jp.size());
  *njpairs = (int)jp.size();
  return 0;
}

namespace covgpu {

// dimensions of the current alignments within the plan's buffers: tile
// order, operand tensor maps; false when they do not fit
static bool plan_dims(UmmaPlan* p, int N, int L, int Lp, int nT, int ntiles) {
  const int Npad = (N + UK - 1) / UK * UK;
  const int64_t rows = (int64_t)4 * p->maxslots * 4 * Lp;
  if (N < 1 || N > p->capN || Lp > p->capLp || ntiles > p->order_cap || rows >= ((int64_t)1 << 31) ||
      (size_t)rows * Npad * sizeof(__nv_bfloat16) > p->ops_bytes)
    return false;
  p->N = N; p->L = L; p->Lp = Lp; p->nT = nT; p->ntiles = ntiles; p->Npad = Npad;
  if (!set_order(p, p->sb)) return false;
  cuuint64_t gdim[2] = {(cuuint64_t)p->Npad, (cuuint64_t)rows};
  cuuint64_t gstride[1] = {(cuuint64_t)p->Npad * sizeof(__nv_bfloat16)};
  cuuint32_t box[2] = {UK, UM};
  cuuint32_t estride[2] = {1, 1};
  if (get_encode()(&p->tmap, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, p->d_ops, gdim, gstride, box, estride,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
    return false;
  if (p->d_ops8) {   // the FP8 operands are re-encoded on their next use
    p->Npad8 = 0;
  }
  return true;
}

UmmaPlan* umma_plan_create(int N, int L, int Lp, int nT, const TileRC* d_tiles, int ntiles, int maxslots, int capN,
                           int capLp, int capntiles) {
  int dev = 0, major = 0, minor = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
  cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
  if (major != 10) return nullptr;               // tcgen05 needs a Blackwell datacenter part
  if (capN < 1 || capN > 65536) return nullptr;  // limb sums stay exact in FP32 up to here
  if (!get_encode()) return nullptr;
  UmmaPlan* p = new UmmaPlan();
  p->maxslots = maxslots; p->d_tiles = d_tiles;
  p->capN = capN; p->capLp = capLp; p->order_cap = capntiles;
  const int Npad_cap = (capN + UK - 1) / UK * UK;
  const int64_t rows_cap = (int64_t)4 * maxslots * 4 * capLp;
  if (rows_cap >= ((int64_t)1 << 31)) { delete p; return nullptr; }
  p->ops_bytes = (size_t)rows_cap * Npad_cap * sizeof(__nv_bfloat16);
  if (cudaMalloc(&p->d_ops, p->ops_bytes) != cudaSuccess) { p->d_ops = nullptr; umma_plan_destroy(p); return nullptr; }
  if (cudaMemset(p->d_ops, 0, p->ops_bytes) != cudaSuccess ||
      cudaMalloc(&p->d_limbs, (size_t)3 * Npad_cap * sizeof(uint16_t)) != cudaSuccess ||
      cudaMalloc(&p->d_order, sizeof(int) * std::max(1, capntiles)) != cudaSuccess ||
      cudaMalloc(&p->d_jpairs, sizeof(int4) * std::max(1, capntiles)) != cudaSuccess ||
      cudaMalloc(&p->d_err, sizeof(int)) != cudaSuccess) {
    umma_plan_destroy(p);
    return nullptr;
  }
  cudaMemset(p->d_err, 0, sizeof(int));
  if (!plan_dims(p, N, L, Lp, nT, ntiles)) { umma_plan_destroy(p); return nullptr; }
  cudaFuncSetAttribute(k_count_umma<3, STAGES3, ACC3, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)smem_bytes(3, STAGES3));
  cudaFuncSetAttribute(k_count_umma<1, STAGES1, ACC1, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)smem_bytes(1, STAGES1));
  cudaFuncSetAttribute(k_count_umma<1, STAGES1, ACC1, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)smem_bytes(2, STAGES1));   // two B tiles per stage
  cudaDeviceGetAttribute(&p->nsm, cudaDevAttrMultiProcessorCount, dev);
  return p;
}

bool umma_plan_resize(UmmaPlan* p, int N, int L, int Lp, int nT, int ntiles) {
  return plan_dims(p, N, L, Lp, nT, ntiles);
}

void umma_plan_destroy(UmmaPlan* p) {
  if (!p) return;
  if (p->d_ops) cudaFree(p->d_ops);
  if (p->d_ops8) cudaFree(p->d_ops8);
  if (p->d_order) cudaFree(p->d_order);
  if (p->d_jpairs) cudaFree(p->d_jpairs);
  if (p->d_limbs) cudaFree(p->d_limbs);
  if (p->d_err) cudaFree(p->d_err);
  delete p;
}

void umma_set_weights(UmmaPlan* p, const double* wgt, int N, cudaStream_t st) {
  std::vector<uint16_t> lim((size_t)3 * p->Npad, 0);
  double wtot_q = 0.0;
  make_limbs(wgt, N, p->Npad, lim.data(), &p->cw, &wtot_q);
  cudaMemcpyAsync(p->d_limbs, lim.data(), lim.size() * sizeof(uint16_t), cudaMemcpyHostToDevice, st);
  cudaStreamSynchronize(st);
}

// TMA store map over a count buffer viewed as rows of 32 FP32 counts, box
// 32 x 32, 128-byte swizzle: [maxslots][ntiles][16][planes][32][32] (planes
// = 2 for double-float counts, 1 for the FP8 unit counts)
static bool encode_out_map(UmmaPlan* p, float* cnt, int planes, CUtensorMap* m) {
  const uint64_t rows = (uint64_t)p->maxslots * p->ntiles * 16 * planes * 32;
  if (rows >= ((uint64_t)1 << 31)) return false;
  cuuint64_t gdim[2] = {32, (cuuint64_t)rows};
  cuuint64_t gstride[1] = {32 * sizeof(float)};
  cuuint32_t box[2] = {32, 32};
  cuuint32_t estride[2] = {1, 1};
  return get_encode()(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, cnt, gdim, gstride, box, estride,
                      CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_NONE,
                      CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// FP8 operand buffer (allocated once, at capacity) and its tensor map for
// the current dimensions, made on the first unit-weight pass after a resize
static cudaError_t ensure_fp8(UmmaPlan* p) {
  if (p->d_ops8 && p->Npad8) return cudaSuccess;
  cudaError_t e;
  if (!p->d_ops8) {
    const int64_t rows_cap = (int64_t)p->maxslots * 4 * p->capLp;
    const int Npad8_cap = (p->capN + UK8 - 1) / UK8 * UK8;
    p->ops8_bytes = (size_t)rows_cap * Npad8_cap;
    e = cudaMalloc(&p->d_ops8, p->ops8_bytes);
    if (e != cudaSuccess) { p->d_ops8 = nullptr; p->ops8_bytes = 0; return e; }
    if ((e = cudaMemset(p->d_ops8, 0, p->ops8_bytes)) != cudaSuccess) return e;
  }
  const int Npad8 = (p->N + UK8 - 1) / UK8 * UK8;
  const int64_t rows = (int64_t)p->maxslots * 4 * p->Lp;
  if ((size_t)rows * Npad8 > p->ops8_bytes) return cudaErrorInvalidValue;
  cuuint64_t gdim[2] = {(cuuint64_t)Npad8, (cuuint64_t)rows};
  cuuint64_t gstride[1] = {(cuuint64_t)Npad8};
  cuuint32_t box[2] = {UK8, UM};
  cuuint32_t estride[2] = {1, 1};
  if (get_encode()(&p->tmap8, CU_TENSOR_MAP_DATA_TYPE_UINT8, 2, p->d_ops8, gdim, gstride, box, estride,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
    return cudaErrorInvalidValue;
  p->Npad8 = Npad8;
  return cudaSuccess;
}

cudaError_t umma_count(UmmaPlan* p, const uint8_t* ax, int64_t slot_stride, int nslots, bool unit, float* cnt,
                       cudaStream_t st, cudaEvent_t ev0, cudaEvent_t ev1, unsigned cellmask) {
  if (nslots > p->maxslots) return cudaErrorInvalidValue;
  if (((uintptr_t)cnt & 15u) != 0) return cudaErrorInvalidValue;
  CUtensorMap omap;
  if (!encode_out_map(p, cnt, unit ? 1 : 2, &omap)) return cudaErrorInvalidValue;
  // persistent: one CTA per SM, tasks (alignment, tile in raster order)
  const int64_t ntask = (int64_t)p->ntiles * nslots;
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(ntask, p->nsm));
  if (unit) {
    // unit weights: the one-hot itself on both sides, exact in FP8 E4M3
    cudaError_t e = ensure_fp8(p);
    if (e != cudaSuccess) return e;
    k_umma_prep8<<<dim3(p->Npad8 / 128, p->Lp / 32, nslots), 256, 0, st>>>(ax, slot_stride, p->N, p->Lp, p->Npad8,
                                                                            nslots, p->d_ops8);
    const int64_t ntask8 = (int64_t)p->njpairs * nslots;
    const int grid8 = (int)std::max<int64_t>(1, std::min<int64_t>(ntask8, p->nsm));
    k_count_umma<1, STAGES1, ACC1, true><<<grid8, 192, smem_bytes(2, STAGES1), st>>>(
        p->tmap8, omap, p->d_tiles, p->d_order, p->ntiles, p->d_jpairs, p->njpairs, p->maxslots, nslots, p->Lp,
        p->Npad8 / UK8, 0, 1.0f, 1.0f, 0.0f, cellmask, p->d_err);
    return cudaGetLastError();
  }
  const CountWeights& W = p->cw;
  dim3 pg(p->Npad / 64, p->Lp / 32, nslots);
  k_umma_prep<<<pg, 256, 0, st>>>(ax, slot_stride, p->N, p->Lp, p->Npad, p->maxslots, W.nl, p->d_limbs, false,
                                  reinterpret_cast<uint16_t*>(p->d_ops));
  const int nkb = p->Npad / UK;
  if (ev0) cudaEventRecord(ev0, st);
  if (W.nl == 1)
    k_count_umma<1, STAGES1, ACC1, false><<<grid, 192, smem_bytes(1, STAGES1), st>>>(
        p->tmap, omap, p->d_tiles, p->d_order, p->ntiles, nullptr, 0, p->maxslots, nslots, p->Lp, nkb, 1, 1.0f,
        W.s_hi, W.s_lo, 0xFFFFu, p->d_err);
  else
    k_count_umma<3, STAGES3, ACC3, false><<<grid, 192, smem_bytes(3, STAGES3), st>>>(
        p->tmap, omap, p->d_tiles, p->d_order, p->ntiles, nullptr, 0, p->maxslots, nslots, p->Lp, nkb, 1, W.B,
        W.s_hi, W.s_lo, 0xFFFFu, p->d_err);
  if (ev1) cudaEventRecord(ev1, st);
  return cudaGetLastError();
}

// Schedule autotuner: times the weighted count launch on the alignments at
// hand for each raster super-block in cand[] (median of reps launches, CUDA
// events on the stream) and keeps the fastest; ms[k] gets each time.
int umma_autotune(UmmaPlan* p, const uint8_t* ax, int64_t slot_stride, int nslots, float* cnt, cudaStream_t st,
                  const int* cand, int ncand, int reps, float* ms, int* best_sb) {
  cudaEvent_t a, b;
  if (cudaEventCreate(&a) != cudaSuccess) return 90;
  if (cudaEventCreate(&b) != cudaSuccess) { cudaEventDestroy(a); return 90; }
  int best = p->sb;
  float bt = INFINITY;
  int status = 0;
  for (int k = 0; k < ncand && !status; k++) {
    if (cand[k] < 1 || !set_order(p, cand[k])) { status = 11; break; }
    std::vector<float> t;
    for (int r = 0; r < reps + 1 && !status; r++) {   // the first launch warms up
      if (umma_count(p, ax, slot_stride, nslots, false, cnt, st, a, b) != cudaSuccess ||
          cudaEventSynchronize(b) != cudaSuccess) { status = 90; break; }
      float x = 0.f;
      cudaEventElapsedTime(&x, a, b);
      if (r) t.push_back(x);
    }
    if (status) break;
    std::sort(t.begin(), t.end());
    const float med = t[t.size() / 2];
    if (ms) ms[k] = med;
    if (med < bt) { bt = med; best = cand[k]; }
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (!set_order(p, best) && !status) status = 90;
  if (best_sb) *best_sb = best;
  return status;
}

int umma_error(UmmaPlan* p) {
  int e = 0;
  cudaMemcpy(&e, p->d_err, sizeof(int), cudaMemcpyDeviceToHost);
  if (e) cudaMemset(p->d_err, 0, sizeof(int));
  return e;
}

// ------------------------------------------------------------------------
// grouped launches over a batch of families (cov_batch.h)
// ------------------------------------------------------------------------
__global__ void __launch_bounds__(256)
k_umma_prep_grp(const FamDev* __restrict__ F, int nf, const int* __restrict__ pre, int pitch,
                uint16_t* __restrict__ ops) {
  const int f = grp_find(pre, nf, (int)blockIdx.x);
  const FamDev& d = F[f];
  const int nsb = d.Npad / 64, ncb = d.Lp / 32;
  const int loc = (int)blockIdx.x - __ldg(pre + f), sb = loc % nsb, rest = loc / nsb;
  umma_prep_body(sb, rest % ncb, rest / ncb, d.ax, (int64_t)d.N * d.Lp, d.N, d.Lp, pitch, d.nslots, d.nl, d.limbs,
                 d.Npad, false, ops + (int64_t)d.oprow0 * pitch);
}

cudaError_t grp_umma_prep(const FamDev* F, int nf, const int* pre, int nb, int pitch, uint16_t* ops,
                          cudaStream_t st) {
  if (nb > 0) k_umma_prep_grp<<<nb, 256, 0, st>>>(F, nf, pre, pitch, ops);
  return cudaGetLastError();
}

// 0 ok, 11 the buffers exceed a tensor map's 32-bit row coordinates or the
// device has no tensor path, 90 CUDA error
int grp_umma_count(const UmmaFam* fams, int nf, const int* tpre, int64_t ntask, int nl, const uint16_t* ops,
                   int pitch, int64_t rows, float* cnt_base, int64_t cnt_rows, int* err, cudaStream_t st) {
  if (ntask <= 0) return 0;
  if (ntask >= ((int64_t)1 << 31) || rows >= ((int64_t)1 << 31) || cnt_rows >= ((int64_t)1 << 31)) return 11;
  if (!get_encode() || (pitch % UK) != 0 || ((uintptr_t)ops & 15u) || ((uintptr_t)cnt_base & 15u)) return 11;
  CUtensorMap tmap, omap;
  {
    cuuint64_t gdim[2] = {(cuuint64_t)pitch, (cuuint64_t)rows};
    cuuint64_t gstride[1] = {(cuuint64_t)pitch * sizeof(uint16_t)};
    cuuint32_t box[2] = {UK, UM};
    cuuint32_t estride[2] = {1, 1};
    if (get_encode()(&tmap, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, (void*)ops, gdim, gstride, box, estride,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return 11;
  }
  {
    cuuint64_t gdim[2] = {32, (cuuint64_t)cnt_rows};
    cuuint64_t gstride[1] = {32 * sizeof(float)};
    cuuint32_t box[2] = {32, 32};
    cuuint32_t estride[2] = {1, 1};
    if (get_encode()(&omap, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, cnt_base, gdim, gstride, box, estride,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_NONE,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return 11;
  }
  static const int nsm = [] {
    int dev = 0, n = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    cudaFuncSetAttribute(k_count_umma<3, STAGES3, ACC3, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)smem_bytes(3, STAGES3));
    cudaFuncSetAttribute(k_count_umma<1, STAGES1, ACC1, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)smem_bytes(1, STAGES1));
    return n;
  }();
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(ntask, nsm));
  if (nl == 1)
    k_count_umma<1, STAGES1, ACC1, false, true><<<grid, 192, smem_bytes(1, STAGES1), st>>>(
        tmap, omap, nullptr, nullptr, (int)ntask, nullptr, 0, 1, 1, 0, 0, 1, 1.f, 1.f, 0.f, 0xFFFFu, err, fams,
        tpre, nf);
  else
    k_count_umma<3, STAGES3, ACC3, false, true><<<grid, 192, smem_bytes(3, STAGES3), st>>>(
        tmap, omap, nullptr, nullptr, (int)ntask, nullptr, 0, 1, 1, 0, 0, 1, 1.f, 1.f, 0.f, 0xFFFFu, err, fams,
        tpre, nf);
  return cudaGetLastError() == cudaSuccess ? 0 : 90;
}

}  // namespace covgpu
