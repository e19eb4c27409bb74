// cov_sim.cu -- the P(t) alignment simulator on the GPU.
//
// cov_GenerateAlignmentUngapped / cov_evolve_root_ungapped_tree /
// cov_emit_ungapped / cov_substitute (src/cov_simulate.c:288-324,388-451,
// 586-631,725-798) with ratematrix_ConditionalsFromRate
// (src/ratematrix.c:185-233):
//   k_sim_ptable  one CTA per branch and model: P(t) = exp(t Q) by scaling
//                 and squaring of an 18-term Taylor series in FP64 (one
//                 thread per matrix entry), the reference's time rules and
//                 regularisation (small negatives zeroed, rows renormalised),
//                 then per row the inverse-CDF thresholds
//                 C[k] = floor(running sum 2^64) as 64-bit integers.
//   k_sim_root    the root state of every (column unit, replicate): a unit
//                 is an unpaired column (4 states) or a base pair (16
//                 states); given, or drawn from the background.
//   k_sim_level   one launch per tree depth, one thread per (branch of the
//                 depth's internal nodes, unit, replicate): the child draws
//                 its state from its branch's conditional on the parent's
//                 state, the first state whose threshold exceeds a 64-bit
//                 Philox draw (the same draws as visiting the internal nodes
//                 in index order, parents first).  Internal states live in
//                 a node-major buffer (consecutive units in consecutive
//                 threads: coalesced); leaf states go to the output slot.
//   k_sim_gaps    one thread per (leaf, replicate): gap runs along the row
//                 (a gapped column continues the run with probability pext,
//                 any other column opens one with probability popen).
//
// Random streams are counter-based (Philox keyed by the seed; counters are
// the replicate, the child node and the unit), so results do not depend on
// scheduling and the oracle reproduces them draw for draw from the same
// tables.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>

#include "cov_dev.cuh"
#include "cov_sim.h"

namespace covgpu {

constexpr uint32_t TAG_SIMROOT = 0x21u, TAG_SIMSUB = 0x22u, TAG_SIMGAP = 0x23u;

__device__ __forceinline__ uint64_t rng_u64(uint64_t seed, uint32_t tag, uint32_t rep, uint32_t a, uint32_t b) {
  uint32_t c[4] = {tag, rep, a, b};
  philox4x32((uint32_t)seed, (uint32_t)(seed >> 32), c);
  return (uint64_t)c[0] | ((uint64_t)c[1] << 32);
}

// one CTA (n*n threads, n = 4 or 16) per branch: times[b] -> P[b], C[b]
template <int n>
__global__ void __launch_bounds__(n * n)
k_sim_ptable(const double* __restrict__ Q, const double* __restrict__ times, double* __restrict__ Pout,
             unsigned long long* __restrict__ Cout, int* __restrict__ status) {
  __shared__ double A[n * n], T[n * n], P[n * n], X[n * n];
  __shared__ double rown[n];
  __shared__ int ksh, bad;
  const int b = blockIdx.x, tid = threadIdx.x, i = tid / n, j = tid % n;
  double rt = times[b];
  // the reference's time rules: (-1e-5, 0) -> 1e-5, below fails, above 1e4 capped
  if (rt < 0.0) {
    if (rt > -1e-5) rt = 1e-5;
    else { if (tid == 0) atomicExch(status, 41); rt = 0.0; }
  }
  const double t = (rt > 10000.0) ? 10000.0 : rt;
  if (tid == 0) bad = 0;
  if (tid < n) {
    double r = 0.0;
    for (int l = 0; l < n; l++) r += fabs(Q[tid * n + l] * t);
    rown[tid] = r;
  }
  __syncthreads();
  if (tid == 0) {
    double nrm = 0.0;
    for (int l = 0; l < n; l++) nrm = fmax(nrm, rown[l]);
    int k = 0;
    while (nrm > 0.5) { nrm *= 0.5; k++; }
    ksh = k;
  }
  __syncthreads();
  const int k = ksh;
  A[tid] = Q[tid] * t / ldexp(1.0, k);
  P[tid] = (i == j) ? 1.0 : 0.0;
  T[tid] = P[tid];
  __syncthreads();
  for (int m = 1; m <= 18; m++) {
    double s = 0.0;
    for (int l = 0; l < n; l++) s += T[i * n + l] * A[l * n + j];
    __syncthreads();
    T[tid] = s / m;
    P[tid] += T[tid];
    __syncthreads();
  }
  for (int q = 0; q < k; q++) {
    double s = 0.0;
    for (int l = 0; l < n; l++) s += P[i * n + l] * P[l * n + j];
    __syncthreads();
    X[tid] = s;
    __syncthreads();
    P[tid] = X[tid];
    __syncthreads();
  }
  // small negatives zeroed, others fail
  double v = P[tid];
  if (v < 0.0) {
    if (fabs(v) < 0.001) v = 0.0;
    else bad = 1;
  }
  P[tid] = v;
  __syncthreads();
  if (tid < n) {
    double s = 0.0;
    for (int l = 0; l < n; l++) s += P[tid * n + l];
    rown[tid] = s;
    if (!(s > 0.0)) bad = 1;
  }
  __syncthreads();
  P[tid] = P[tid] / rown[i];
  Pout[(size_t)b * n * n + tid] = P[tid];
  __syncthreads();
  if (tid < n) {
    double c = 0.0;
    for (int l = 0; l < n; l++) {
      c += P[tid * n + l];
      Cout[(size_t)b * n * n + tid * n + l] =
          (l == n - 1 || c >= 1.0) ? ~0ull : (unsigned long long)ldexp(c, 64);
    }
  }
  if (tid == 0 && bad) atomicExch(status, 42);
}

__device__ __forceinline__ int sim_draw(const unsigned long long* __restrict__ C, int n, uint64_t U) {
  for (int i = 0; i < n - 1; i++)
    if (U < C[i]) return i;
  return n - 1;
}

// the root's state of every (unit, replicate): given, or drawn from the
// background
__global__ void __launch_bounds__(256)
k_sim_root(int N, const int2* __restrict__ units, int nunits, const unsigned long long* __restrict__ R4,
           const unsigned long long* __restrict__ R16, const uint8_t* __restrict__ root, uint64_t seed,
           uint32_t first_rep, uint8_t* __restrict__ state) {
  const int u = blockIdx.x * blockDim.x + threadIdx.x, rep = blockIdx.y;
  if (u >= nunits) return;
  const int2 un = units[u];
  const bool paired = un.y >= 0;
  int x;
  if (root) {
    x = paired ? root[un.x] * 4 + root[un.y] : root[un.x];
  } else {
    const uint64_t U = rng_u64(seed, TAG_SIMROOT, first_rep + rep, 0u, (uint32_t)u);
    x = paired ? sim_draw(R16, 16, U) : sim_draw(R4, 4, U);
  }
  state[(size_t)rep * (N - 1) * nunits + u] = (uint8_t)x;
}

// the branches of the internal nodes of one tree depth: one thread per
// (branch, unit), consecutive units in consecutive threads
__global__ void __launch_bounds__(256)
k_sim_level(const int* __restrict__ left, const int* __restrict__ right, const int* __restrict__ nodes, int nn, int N,
            int Lp, const int2* __restrict__ units, int nunits, const unsigned long long* __restrict__ C4,
            const unsigned long long* __restrict__ C16, uint64_t seed, uint32_t first_rep,
            uint8_t* __restrict__ state, uint8_t* __restrict__ out, int64_t out_slot_stride) {
  const int64_t item = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int rep = blockIdx.y;
  if (item >= (int64_t)2 * nn * nunits) return;
  const int kb = (int)(item / nunits), u = (int)(item % nunits);
  const int v = nodes[kb >> 1], side = kb & 1;
  const int ch = side ? right[v] : left[v];
  const int b = 2 * v + side;
  const int2 un = units[u];
  const bool paired = un.y >= 0;
  uint8_t* S = state + (size_t)rep * (N - 1) * nunits;
  const int a = S[(size_t)v * nunits + u];
  const uint32_t cid = (uint32_t)((ch <= 0) ? -ch : N + ch);
  const uint64_t U = rng_u64(seed, TAG_SIMSUB, first_rep + rep, cid, (uint32_t)u);
  const int y = paired ? sim_draw(C16 + ((size_t)b * 16 + a) * 16, 16, U) : sim_draw(C4 + ((size_t)b * 4 + a) * 4, 4, U);
  if (ch > 0) {
    S[(size_t)ch * nunits + u] = (uint8_t)y;
  } else {
    uint8_t* O = out + (int64_t)rep * out_slot_stride + (int64_t)(-ch) * Lp;
    if (paired) { O[un.x] = (uint8_t)(y >> 2); O[un.y] = (uint8_t)(y & 3); }
    else        { O[un.x] = (uint8_t)y; }
  }
}

// one thread per (leaf, replicate): gap runs along the row
__global__ void __launch_bounds__(256)
k_sim_gaps(int N, int L, int Lp, double popen, double pext, uint64_t seed, uint32_t first_rep, uint8_t* __restrict__ out,
           int64_t out_slot_stride) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x, rep = blockIdx.y;
  if (n >= N) return;
  uint8_t* row = out + (int64_t)rep * out_slot_stride + (int64_t)n * Lp;
  const uint32_t rid = first_rep + rep;
  int run = 0;
  for (int c = 0; c < L; c++) {
    uint32_t o[4] = {TAG_SIMGAP, rid, (uint32_t)n, (uint32_t)c};
    philox4x32((uint32_t)seed, (uint32_t)(seed >> 32), o);
    const double ue = (double)o[0] * (1.0 / 4294967296.0);
    const double uo = (double)o[1] * (1.0 / 4294967296.0);
    if ((run && ue < pext) || uo < popen) { row[c] = 4; run = 1; }
    else run = 0;
  }
}

// the background's thresholds (one row)
__global__ void k_sim_rootcdf(const double* __restrict__ pi, int n, unsigned long long* __restrict__ C) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double c = 0.0;
  for (int l = 0; l < n; l++) {
    c += pi[l];
    C[l] = (l == n - 1 || c >= 1.0) ? ~0ull : (unsigned long long)ldexp(c, 64);
  }
}

cudaError_t launch_sim_tables(const double* Q4, const double* Q16, const double* pi4, const double* pi16,
                              const double* times, int nbranch, double* P4, double* P16, unsigned long long* C4,
                              unsigned long long* C16, unsigned long long* R4, unsigned long long* R16, int* status,
                              cudaStream_t st) {
  k_sim_ptable<4><<<nbranch, 16, 0, st>>>(Q4, times, P4, C4, status);
  k_sim_ptable<16><<<nbranch, 256, 0, st>>>(Q16, times, P16, C16, status);
  k_sim_rootcdf<<<1, 32, 0, st>>>(pi4, 4, R4);
  k_sim_rootcdf<<<1, 32, 0, st>>>(pi16, 16, R16);
  return cudaGetLastError();
}

cudaError_t launch_sim_evolve(const int* left, const int* right, const int* level_nodes, const int* level_off,
                              int nlevels, int N, int L, int Lp, const int2* units, int nunits,
                              const unsigned long long* C4, const unsigned long long* C16,
                              const unsigned long long* R4, const unsigned long long* R16, const uint8_t* root,
                              double gap_rate, double gap_mean, uint64_t seed, uint32_t first_rep, int nrep,
                              uint8_t* state, uint8_t* out, int64_t out_slot_stride, cudaStream_t st) {
  k_sim_root<<<dim3((nunits + 255) / 256, nrep), 256, 0, st>>>(N, units, nunits, R4, R16, root, seed, first_rep,
                                                                state);
  for (int d = 0; d < nlevels; d++) {
    const int nn = level_off[d + 1] - level_off[d];
    if (nn <= 0) continue;
    const int64_t items = (int64_t)2 * nn * nunits;
    k_sim_level<<<dim3((unsigned)((items + 255) / 256), nrep), 256, 0, st>>>(
        left, right, level_nodes + level_off[d], nn, N, Lp, units, nunits, C4, C16, seed, first_rep, state, out,
        out_slot_stride);
  }
  const double popen = (gap_mean > 0.0) ? gap_rate / gap_mean : 0.0;
  const double pext = (gap_mean > 1.0) ? 1.0 - 1.0 / gap_mean : 0.0;
  if (popen > 0.0)
    k_sim_gaps<<<dim3((N + 255) / 256, nrep), 256, 0, st>>>(N, L, Lp, popen, pext, seed, first_rep, out,
                                                             out_slot_stride);
  return cudaGetLastError();
}

}  // namespace covgpu
