// cov_subst.cu -- substitutions on the tree and the power of every pair.
//
// Tree_Substitutions (src/msatree.c:1423-1554) on the Fitch reconstruction
// of the alignment: for every branch (parent v -> child) and column c, bit
// s = the child's residue differs from the parent's (both canonical unless
// gaps are included) and bit u = both canonical and equal; the bits of 32
// branches pack one word, so per column
//   nsubs[c]     = sum popc(s_c)
// and per pair i < j
//   ndouble[i,j] = sum popc(s_i & s_j)                 (both change)
//   njoin[i,j]   = sum popc((s|u)_i & (s|u)_j) - popc(u_i & u_j)
//                  (both canonical, at least one changes; with gaps
//                  included: sum popc(s_i | s_j))
// computed in 32 x 32 tiles of pairs from shared-memory word tiles.
//
// power_SPAIR_Create (src/power.c:65-218): the power of a pair is the step
// curve's probability at its substitution count (nsubs_i + nsubs_j, njoin,
// ndouble): the last point whose count the pair's exceeds.
#include <cuda_runtime.h>

#include <cstdint>

#include "cov_subst.h"

namespace covgpu {

// one thread per (column, word of 32 branches), columns fastest
__global__ void __launch_bounds__(256)
k_subst_bits(const uint8_t* __restrict__ ax, const uint8_t* __restrict__ F, const int* __restrict__ left,
             const int* __restrict__ right, int N, int L, int Lp, int Wb, int includegaps, uint32_t* __restrict__ Sb,
             uint32_t* __restrict__ Ub) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (int64_t)Wb * L) return;
  const int k = (int)(idx / L), c = (int)(idx % L);
  const int nb = 2 * (N - 1);
  uint32_t s = 0, u = 0;
  for (int t = 0; t < 32; t++) {
    const int e = 32 * k + t;
    if (e >= nb) break;
    const int v = e >> 1;
    const int ch = (e & 1) ? right[v] : left[v];
    const int a = F[(int64_t)v * Lp + c];
    const int b = (ch > 0) ? F[(int64_t)ch * Lp + c] : ax[(int64_t)(-ch) * Lp + c];
    if (includegaps) {
      s |= (uint32_t)(a != b) << t;
      u |= (uint32_t)(a == b) << t;
    } else {
      const bool can = a < 4 && b < 4;
      s |= (uint32_t)(can && a != b) << t;
      u |= (uint32_t)(can && a == b) << t;
    }
  }
  Sb[(int64_t)c * Wb + k] = s;
  Ub[(int64_t)c * Wb + k] = u;
}

__global__ void __launch_bounds__(256)
k_subst_nsubs(const uint32_t* __restrict__ Sb, int L, int Wb, int* __restrict__ nsubs) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= L) return;
  int n = 0;
  for (int k = 0; k < Wb; k++) n += __popc(Sb[(int64_t)c * Wb + k]);
  nsubs[c] = n;
}

// the upper triangle (i < j) of ndouble and njoin, tile (blockIdx.y, blockIdx.x)
__global__ void __launch_bounds__(256)
k_subst_pairs(const uint32_t* __restrict__ Sb, const uint32_t* __restrict__ Ub, int L, int Wb, int includegaps,
              int* __restrict__ ndouble, int* __restrict__ njoin) {
  __shared__ uint32_t si[32][33], ui[32][33], sj[32][33], uj[32][33];
  const int I0 = blockIdx.y * 32, J0 = blockIdx.x * 32;
  if (J0 + 31 <= I0) return;   // no pair i < j in this tile
  const int tid = threadIdx.x, ty = tid >> 5, tx = tid & 31;
  int dbl[4] = {0, 0, 0, 0}, cc[4] = {0, 0, 0, 0}, uu[4] = {0, 0, 0, 0};
  for (int w0 = 0; w0 < Wb; w0 += 32) {
    for (int e = tid; e < 32 * 32; e += 256) {
      const int r = e >> 5, k = e & 31, w = w0 + k;
      const int i = I0 + r, j = J0 + r;
      si[r][k] = (i < L && w < Wb) ? Sb[(int64_t)i * Wb + w] : 0u;
      ui[r][k] = (i < L && w < Wb) ? Ub[(int64_t)i * Wb + w] : 0u;
      sj[r][k] = (j < L && w < Wb) ? Sb[(int64_t)j * Wb + w] : 0u;
      uj[r][k] = (j < L && w < Wb) ? Ub[(int64_t)j * Wb + w] : 0u;
    }
    __syncthreads();
#pragma unroll 4
    for (int k = 0; k < 32; k++) {
      const uint32_t b_s = sj[tx][k], b_u = uj[tx][k];
#pragma unroll
      for (int q = 0; q < 4; q++) {
        const uint32_t a_s = si[ty + 8 * q][k], a_u = ui[ty + 8 * q][k];
        dbl[q] += __popc(a_s & b_s);
        if (includegaps) {
          cc[q] += __popc(a_s | b_s);
        } else {
          cc[q] += __popc((a_s | a_u) & (b_s | b_u));
          uu[q] += __popc(a_u & b_u);
        }
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int q = 0; q < 4; q++) {
    const int i = I0 + ty + 8 * q, j = J0 + tx;
    if (i < j && j < L) {
      ndouble[(int64_t)i * L + j] = dbl[q];
      njoin[(int64_t)i * L + j] = cc[q] - uu[q];
    }
  }
}

__device__ __forceinline__ double step_power(double n, const double* __restrict__ subs, const double* __restrict__ prob,
                                             int ns) {
  double p = 0.0;
  for (int s = 0; s < ns; s++) {
    if (n > subs[s]) p = prob[s];
    else break;
  }
  return p;
}

// pair n = (i, j), i < j, in row-major order of the upper triangle
__global__ void __launch_bounds__(256)
k_power(const int* __restrict__ nsubs, const int* __restrict__ ndouble, const int* __restrict__ njoin, int L,
        int ns, const double* __restrict__ tab, int have_single, int have_join, int have_double,
        double* __restrict__ power, double* __restrict__ power_join, double* __restrict__ power_double) {
  const int i = blockIdx.y;
  const int64_t base = (int64_t)i * L - (int64_t)i * (i + 1) / 2;   // pairs before row i
  for (int j = i + 1 + blockIdx.x * blockDim.x + threadIdx.x; j < L; j += gridDim.x * blockDim.x) {
    const int64_t n = base + (j - i - 1);
    if (power) power[n] = have_single ? step_power((double)(nsubs[i] + nsubs[j]), tab, tab + ns, ns) : 0.0;
    if (power_join) power_join[n] = have_join ? step_power((double)njoin[(int64_t)i * L + j], tab + 2 * ns, tab + 3 * ns, ns) : -1.0;
    if (power_double)
      power_double[n] = have_double ? step_power((double)ndouble[(int64_t)i * L + j], tab + 4 * ns, tab + 5 * ns, ns) : -1.0;
  }
}

cudaError_t launch_substitutions(const uint8_t* ax, const uint8_t* F, const int* left, const int* right, int N, int L,
                                 int Lp, int includegaps, uint32_t* Sb, uint32_t* Ub, int* nsubs, int* ndouble,
                                 int* njoin, cudaStream_t st) {
  const int Wb = (2 * (N - 1) + 31) / 32;
  const int64_t items = (int64_t)Wb * L;
  k_subst_bits<<<(unsigned)((items + 255) / 256), 256, 0, st>>>(ax, F, left, right, N, L, Lp, Wb, includegaps, Sb, Ub);
  k_subst_nsubs<<<(L + 255) / 256, 256, 0, st>>>(Sb, L, Wb, nsubs);
  cudaMemsetAsync(ndouble, 0, (size_t)L * L * sizeof(int), st);
  cudaMemsetAsync(njoin, 0, (size_t)L * L * sizeof(int), st);
  const int nt = (L + 31) / 32;
  k_subst_pairs<<<dim3(nt, nt), 256, 0, st>>>(Sb, Ub, L, Wb, includegaps, ndouble, njoin);
  return cudaGetLastError();
}

cudaError_t launch_power(const int* nsubs, const int* ndouble, const int* njoin, int L, int ns, const double* tab,
                         int have_single, int have_join, int have_double, double* power, double* power_join,
                         double* power_double, cudaStream_t st) {
  k_power<<<dim3((L + 255) / 256, L), 256, 0, st>>>(nsubs, ndouble, njoin, L, ns, tab, have_single, have_join,
                                                     have_double, power, power_join, power_double);
  return cudaGetLastError();
}

}  // namespace covgpu
