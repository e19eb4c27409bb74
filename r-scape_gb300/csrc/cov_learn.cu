// cov_learn.cu -- the learned null: alignment summary features and a small
// multilayer perceptron trained and evaluated on the device.
//
// No counterpart in the reference.  R-scape estimates the null score tail
// of every alignment by simulating null alignments and fitting their
// scores (null_rscape, src/R-scape.c:1614-1724; cov_NullFitGamma,
// src/covariation.c:1943-1973).  This file lets a network trained on those
// fits predict the tail from 64 summary features of the alignment, so that
// alignments inside the training range need no simulated nulls.
//
// Features, per alignment of N sequences x L columns, weights w.  On the
// device (k_feat_*):
//    0 log N            1 log L             2 log Neff, Neff = (sum w)^2 / sum w^2
//    3 mean identity    4 tree-length summary (given by the caller)
//    5-20  16-bin histogram of column entropies (bits, [0, 2]), fractions
//   21-36  16-bin histogram of column gap fractions ([0, 1])
//   37 sd identity     38 mean entropy     39 sd entropy      40 mean gap fraction
//   41 sd gap fraction 42 sd/mean of w     43-46 weighted residue composition (A, C, G, U)
// Column entropy and gap fraction use the weighted residue counts n_x of the
// column: gap fraction (sum w - sum_x n_x)/sum w, entropy -sum p log2 p over
// p = n_x / sum_x n_x.  Identity of two sequences: identical canonical
// residues over columns where both are canonical (0 if none), over all pairs
// when N(N-1)/2 <= 4096, else over 4096 pairs drawn with splitmix64.
// Features 47-63 summarise the scores of a few simulated nulls; the engine
// fills them from their histogram (covgpu_learned_features).
//
// Network: 64 -> 256 -> 256 -> 256 -> 3, SiLU after each hidden layer.
// Weights are BF16 copies of FP32 master parameters (biases stay FP32);
// activations, accumulation and gradients are FP32.  Inputs and targets
// are standardised with the training set's mean and deviation.  Training is
// mean squared error + AdamW; one step (batch gather, forward, loss,
// backward, update) is one CUDA graph, replayed.  The matrix products are
// 256-wide and latency-bound, so they use one tiled SIMT kernel
// (64 x 64 tiles, 4 x 4 per thread, fixed summation order: gradients are
// reproducible run to run).
#include "covgpu.h"
#include "cov_learn.h"

#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <vector>

namespace covgpu {

// ------------------------------------------------------------------------
// features
// ------------------------------------------------------------------------
__host__ __device__ inline uint64_t splitmix64(uint64_t x) {   // Steele, Lea & Flood 2014
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

constexpr uint64_t kIdentSeed = 0x5EED1DE7ull;
constexpr int kColStat = 6;   // entropy, gap fraction, n_A, n_C, n_G, n_U

size_t feat_scratch_doubles(int L) { return (size_t)L * kColStat + kIdentPairs + 64; }

// one warp per 32 columns per row group: 8 warps stride over the rows, the
// 8 partial sums are added in warp order
__global__ void __launch_bounds__(256) k_feat_cols(const uint8_t* __restrict__ ax, int N, int L, int Lp,
                                                   const double* __restrict__ w, const double* __restrict__ pwtot,
                                                   double* __restrict__ col) {
  __shared__ double part[8][4][32];
  const double wtot = *pwtot;
  const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
  const int c = blockIdx.x * 32 + lane;
  double n[4] = {0.0, 0.0, 0.0, 0.0};
  if (c < L)
    for (int s = wp; s < N; s += 8) {
      const int x = ax[(int64_t)s * Lp + c];
      if (x < 4) n[x] += w[s];
    }
  for (int x = 0; x < 4; x++) part[wp][x][lane] = n[x];
  __syncthreads();
  if (wp == 0 && c < L) {
    double t[4];
    for (int x = 0; x < 4; x++) {
      double a = 0.0;
      for (int k = 0; k < 8; k++) a += part[k][x][lane];
      t[x] = a;
    }
    const double r = (t[0] + t[1]) + (t[2] + t[3]);
    double H = 0.0;
    if (r > 0.0)
      for (int x = 0; x < 4; x++)
        if (t[x] > 0.0) {
          const double p = t[x] / r;
          H -= p * log2(p);
        }
    double* o = col + (int64_t)c * kColStat;
    o[0] = H;
    o[1] = wtot > 0.0 ? fmax(0.0, (wtot - r) / wtot) : 0.0;
    for (int x = 0; x < 4; x++) o[2 + x] = t[x];
  }
}

__device__ __forceinline__ void ident_pair(int k, int N, int npair_all, int* pi, int* pj) {
  if (npair_all <= kIdentPairs) {
    int i = 0, rem = k;
    while (rem >= N - 1 - i) { rem -= N - 1 - i; i++; }
    *pi = i; *pj = i + 1 + rem;
  } else {
    const uint64_t h = splitmix64(kIdentSeed + (uint64_t)k);
    const int i = (int)((uint32_t)h % (uint32_t)N);
    int j = (int)((uint32_t)(h >> 32) % (uint32_t)(N - 1));
    if (j >= i) j++;
    *pi = i; *pj = j;
  }
}

// one warp per sequence pair; 4 columns per load
__global__ void __launch_bounds__(256) k_feat_ident(const uint8_t* __restrict__ ax, int N, int L, int Lp, int M,
                                                    int npair_all, double* __restrict__ id) {
  const int lane = threadIdx.x & 31;
  const int k = blockIdx.x * 8 + (threadIdx.x >> 5);
  if (k >= M) return;
  int i, j;
  ident_pair(k, N, npair_all, &i, &j);
  const uint32_t* a = reinterpret_cast<const uint32_t*>(ax + (int64_t)i * Lp);
  const uint32_t* b = reinterpret_cast<const uint32_t*>(ax + (int64_t)j * Lp);
  int both = 0, same = 0;
  for (int q = lane; q * 4 < L; q += 32) {
    const uint32_t u = a[q], v = b[q];
#pragma unroll
    for (int e = 0; e < 4; e++) {
      const int c = q * 4 + e;
      const uint32_t x = (u >> (8 * e)) & 0xFFu, y = (v >> (8 * e)) & 0xFFu;
      if (c < L && x < 4u && y < 4u) { both++; same += (x == y); }
    }
  }
  for (int o = 16; o; o >>= 1) {
    both += __shfl_xor_sync(0xffffffffu, both, o);
    same += __shfl_xor_sync(0xffffffffu, same, o);
  }
  if (lane == 0) id[k] = both ? (double)same / (double)both : 0.0;
}

// bin of v * scale in [0, 16): NaN and negatives go to bin 0
__device__ __forceinline__ int bin16(double v, double scale) {
  const double q = v * scale;
  if (!(q >= 0.0)) return 0;
  return q >= 15.0 ? 15 : (int)q;
}

// sum over the block in a fixed order (strided partials, then a tree)
__device__ double block_sum(double v, double* sh) {
  const int t = threadIdx.x;
  sh[t] = v;
  __syncthreads();
  for (int s = blockDim.x >> 1; s; s >>= 1) {
    if (t < s) sh[t] += sh[t + s];
    __syncthreads();
  }
  const double r = sh[0];
  __syncthreads();
  return r;
}

__global__ void __launch_bounds__(1024) k_feat_final(const double* __restrict__ col, const double* __restrict__ id,
                                                     const double* __restrict__ w, int N, int L, int M,
                                                     double tree_len, float* __restrict__ feat) {
  __shared__ double sh[1024];
  __shared__ int hist[2][16];
  const int t = threadIdx.x, nt = blockDim.x;
  if (t < 32) hist[t / 16][t % 16] = 0;
  __syncthreads();
  // weights
  double a = 0.0, b = 0.0;
  for (int s = t; s < N; s += nt) { a += w[s]; b += w[s] * w[s]; }
  const double sw = block_sum(a, sh), sw2 = block_sum(b, sh);
  const double wmean = sw / N;
  a = 0.0;
  for (int s = t; s < N; s += nt) a += (w[s] - wmean) * (w[s] - wmean);
  const double wvar = block_sum(a, sh) / N;
  // columns
  double sH = 0.0, sg = 0.0, sn[4] = {0.0, 0.0, 0.0, 0.0};
  for (int c = t; c < L; c += nt) {
    const double* o = col + (int64_t)c * kColStat;
    sH += o[0]; sg += o[1];
    for (int x = 0; x < 4; x++) sn[x] += o[2 + x];
    atomicAdd(&hist[0][bin16(o[0], 8.0)], 1);
    atomicAdd(&hist[1][bin16(o[1], 16.0)], 1);
  }
  const double mH = block_sum(sH, sh) / L, mg = block_sum(sg, sh) / L;
  double comp[4];
  for (int x = 0; x < 4; x++) comp[x] = block_sum(sn[x], sh);
  a = 0.0; b = 0.0;
  for (int c = t; c < L; c += nt) {
    const double* o = col + (int64_t)c * kColStat;
    a += (o[0] - mH) * (o[0] - mH);
    b += (o[1] - mg) * (o[1] - mg);
  }
  const double vH = block_sum(a, sh) / L, vg = block_sum(b, sh) / L;
  // identities
  a = 0.0;
  for (int k = t; k < M; k += nt) a += id[k];
  const double mid = M ? block_sum(a, sh) / M : block_sum(0.0, sh);
  a = 0.0;
  for (int k = t; k < M; k += nt) a += (id[k] - mid) * (id[k] - mid);
  const double vid = M ? block_sum(a, sh) / M : block_sum(0.0, sh);
  __syncthreads();
  if (t == 0) {
    const double rtot = (comp[0] + comp[1]) + (comp[2] + comp[3]);
    double f[5], g[10];
    f[0] = log((double)N);
    f[1] = log((double)L);
    f[2] = sw2 > 0.0 ? log(sw * sw / sw2) : 0.0;
    f[3] = mid;
    f[4] = tree_len;
    g[0] = sqrt(vid);
    g[1] = mH;
    g[2] = sqrt(vH);
    g[3] = mg;
    g[4] = sqrt(vg);
    g[5] = wmean > 0.0 ? sqrt(wvar) / wmean : 0.0;
    for (int x = 0; x < 4; x++) g[6 + x] = rtot > 0.0 ? comp[x] / rtot : 0.0;
    for (int k = 0; k < 5; k++) feat[k] = (float)f[k];
    for (int k = 0; k < 10; k++) feat[37 + k] = (float)g[k];
  }
  if (t < 32) feat[5 + t] = (float)((double)hist[t / 16][t % 16] / (double)L);
  if (t >= 47 && t < kNFeat) feat[t] = 0.f;
}

__global__ void __launch_bounds__(1024) k_feat_wtot(const double* __restrict__ w, int N, double* __restrict__ out) {
  __shared__ double sh[1024];
  double a = 0.0;
  for (int s = threadIdx.x; s < N; s += blockDim.x) a += w[s];
  a = block_sum(a, sh);
  if (threadIdx.x == 0) *out = a;
}

cudaError_t launch_features(const uint8_t* ax, int N, int L, int Lp, const double* w, double tree_len,
                            double* scratch, float* feat, cudaStream_t st) {
  double* col = scratch;
  double* id = scratch + (size_t)L * kColStat;
  double* red = id + kIdentPairs;
  const long long npair_all = (long long)N * (N - 1) / 2;
  const int M = (int)std::min<long long>(kIdentPairs, npair_all);
  k_feat_wtot<<<1, 1024, 0, st>>>(w, N, red);
  k_feat_cols<<<(L + 31) / 32, 256, 0, st>>>(ax, N, L, Lp, w, red, col);
  if (M > 0)
    k_feat_ident<<<(M + 7) / 8, 256, 0, st>>>(ax, N, L, Lp, M, (int)std::min<long long>(npair_all, 1 << 30), id);
  k_feat_final<<<1, 1024, 0, st>>>(col, id, w, N, L, M, tree_len, feat);
  return cudaGetLastError();
}

}  // namespace covgpu

// ------------------------------------------------------------------------
// the network
// ------------------------------------------------------------------------
namespace covgpu {

constexpr int kHid = 256, kOut = 3;
constexpr int oW1 = 0, ob1 = oW1 + kHid * kNFeat, oW2 = ob1 + kHid, ob2 = oW2 + kHid * kHid, oW3 = ob2 + kHid,
              ob3 = oW3 + kHid * kHid, oW4 = ob3 + kHid, ob4 = oW4 + kOut * kHid, kNParam = ob4 + kOut;
static_assert(kNParam == COVGPU_MLP_NPARAM, "parameter layout");

__device__ __forceinline__ float ld_f(const float* p) { return *p; }
__device__ __forceinline__ float ld_f(const __nv_bfloat16* p) { return __bfloat162float(*p); }
__device__ __forceinline__ float sigm(float z) { return 1.f / (1.f + expf(-z)); }

enum { EPI_PLAIN = 0, EPI_SILU = 1, EPI_DSILU = 2 };

// C[m][n] (row-major, M x Nc) = sum_k A(m,k) B(k,n), A(m,k) = A[m*sam + k*sak],
// B(k,n) = B[k*sbk + n*sbn].  Epilogues: PLAIN C = acc (+ bias[n]);
// SILU C2 = z = acc + bias[n], C = silu(z); DSILU C = acc * silu'(aux[m][n]).
template <class TA, class TB, int EPI>
__global__ void __launch_bounds__(256) k_gemm(const TA* __restrict__ A, int sam, int sak, const TB* __restrict__ B,
                                              int sbk, int sbn, int M, int Nc, int K,
                                              const float* __restrict__ bias, const float* __restrict__ aux,
                                              float* __restrict__ C, float* __restrict__ C2) {
  __shared__ float As[16][65];
  __shared__ float Bs[16][65];
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const int m0 = blockIdx.y * 64, n0 = blockIdx.x * 64;
  float acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int j = 0; j < 4; j++) acc[i][j] = 0.f;
  for (int k0 = 0; k0 < K; k0 += 16) {
#pragma unroll
    for (int r = 0; r < 4; r++) {
      const int e = tid + 256 * r, kk = e >> 6, mm = e & 63;
      const int k = k0 + kk, m = m0 + mm, n = n0 + mm;
      As[kk][mm] = (m < M && k < K) ? ld_f(A + (int64_t)m * sam + (int64_t)k * sak) : 0.f;
      Bs[kk][mm] = (n < Nc && k < K) ? ld_f(B + (int64_t)k * sbk + (int64_t)n * sbn) : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < 16; kk++) {
      float a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; i++) { a[i] = As[kk][ty + 16 * i]; b[i] = Bs[kk][tx + 16 * i]; }
#pragma unroll
      for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int j = 0; j < 4; j++) {
      const int m = m0 + ty + 16 * i, n = n0 + tx + 16 * j;
      if (m >= M || n >= Nc) continue;
      const int64_t o = (int64_t)m * Nc + n;
      if (EPI == EPI_PLAIN) {
        C[o] = acc[i][j] + (bias ? bias[n] : 0.f);
      } else if (EPI == EPI_SILU) {
        const float z = acc[i][j] + bias[n];
        C2[o] = z;
        C[o] = z * sigm(z);
      } else {
        const float z = aux[o], sg = sigm(z);
        C[o] = acc[i][j] * (sg * (1.f + z * (1.f - sg)));
      }
    }
}

template <class TA, class TB, int EPI>
static void gemm(cudaStream_t st, const TA* A, int sam, int sak, const TB* B, int sbk, int sbn, int M, int Nc, int K,
                 const float* bias, const float* aux, float* C, float* C2 = nullptr) {
  const dim3 grid((Nc + 63) / 64, (M + 63) / 64);
  k_gemm<TA, TB, EPI><<<grid, 256, 0, st>>>(A, sam, sak, B, sbk, sbn, M, Nc, K, bias, aux, C, C2);
}

// out[o] = sum_b G[b][o], b in order
__global__ void k_colsum(const float* __restrict__ G, int B, int O, float* __restrict__ out) {
  const int o = blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= O) return;
  float s = 0.f;
  for (int b = 0; b < B; b++) s += G[(int64_t)b * O + o];
  out[o] = s;
}

// standardised batch rows perm[off .. off+B) of X, T; off from the step counter
__global__ void k_gather(const float* __restrict__ X, const float* __restrict__ T, const int* __restrict__ perm,
                         const int* __restrict__ counter, int spe, int B, const float* __restrict__ nrm,
                         float* __restrict__ Xb, float* __restrict__ Tb) {
  const int off = (counter ? (*counter % spe) : 0) * B;
  const float *xm = nrm, *xs = nrm + kNFeat, *ym = nrm + 2 * kNFeat, *ys = ym + kOut;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < B * kNFeat; e += gridDim.x * blockDim.x) {
    const int b = e / kNFeat, f = e % kNFeat;
    const int r = perm ? perm[off + b] : b;
    Xb[e] = (X[(int64_t)r * kNFeat + f] - xm[f]) / xs[f];
    if (T && f < kOut) Tb[b * kOut + f] = (T[(int64_t)r * kOut + f] - ym[f]) / ys[f];
  }
}

// Y = (Yp scale) ystd + ymean; scale = 1 / members for an ensemble's sum
__global__ void k_denorm(const float* __restrict__ Yp, int n, const float* __restrict__ nrm, float scale,
                         float* __restrict__ Y) {
  const float *ym = nrm + 2 * kNFeat, *ys = ym + kOut;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e < n * kOut) Y[e] = (Yp[e] * scale) * ys[e % kOut] + ym[e % kOut];
}

// the members' standardised outputs summed in member order
__global__ void k_accum(const float* __restrict__ Yp, int n, bool first, float* __restrict__ Yacc) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e < n) Yacc[e] = first ? Yp[e] : Yacc[e] + Yp[e];
}

// dY = 2 (Y - T) / (B * 3); loss = mean squared error.  With a counter:
// lossbuf[step] = loss and the step counter advances (the update reads it)
__global__ void __launch_bounds__(256) k_loss(const float* __restrict__ Yp, const float* __restrict__ Tb, int B,
                                              float* __restrict__ dY, float* __restrict__ lossbuf,
                                              int* __restrict__ counter) {
  __shared__ float sh[256];
  const int t = threadIdx.x;
  const int n = B * kOut;
  const float sc = 2.f / (float)n;
  float a = 0.f;
  for (int e = t; e < n; e += 256) {
    const float d = Yp[e] - Tb[e];
    dY[e] = sc * d;
    a += d * d;
  }
  sh[t] = a;
  __syncthreads();
  for (int s = 128; s; s >>= 1) {
    if (t < s) sh[t] += sh[t + s];
    __syncthreads();
  }
  if (t == 0) {
    const float loss = sh[0] / (float)n;
    if (counter) {
      const int s = *counter;
      lossbuf[s] = loss;
      *counter = s + 1;
    } else {
      lossbuf[0] = loss;
    }
  }
}

// AdamW (Loshchilov & Hutter 2019) on the FP32 master parameters, with the
// BF16 copy refreshed; the step number is the advanced counter
__global__ void k_adam(float* __restrict__ p, float* __restrict__ m, float* __restrict__ v,
                       const float* __restrict__ g, __nv_bfloat16* __restrict__ pb, int n,
                       const int* __restrict__ counter, const float* __restrict__ hyper) {
  const float lr = hyper[0], wd = hyper[1], b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  const float t = (float)*counter;
  const float bc1 = 1.f - powf(b1, t), bc2 = 1.f - powf(b2, t);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float pi = p[i] - lr * ((mi / bc1) / (sqrtf(vi / bc2) + eps) + wd * p[i]);
    p[i] = pi;
    pb[i] = __float2bfloat16_rn(pi);
  }
}

__global__ void k_to_bf16(const float* __restrict__ p, __nv_bfloat16* __restrict__ pb, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) pb[i] = __float2bfloat16_rn(p[i]);
}

}  // namespace covgpu

using namespace covgpu;

struct covgpu_mlp {
  int dev = 0;
  cudaStream_t st = nullptr;
  int cap = 0;
  char err[256] = {0};
  float *p = nullptr, *m = nullptr, *v = nullptr, *g = nullptr;
  __nv_bfloat16* pb = nullptr;
  float* nrm = nullptr;   // xmean[64] xstd[64] ymean[3] ystd[3]
  float* hyper = nullptr; // lr, weight decay
  std::vector<float> h_nrm, xlo, xhi;
  float *Xin = nullptr, *Xb = nullptr, *Tb = nullptr, *Yp = nullptr, *dY = nullptr, *Yout = nullptr;
  float *Z[3] = {}, *H[3] = {}, *D[3] = {};
  int* counter = nullptr;
  // an ensemble: nmem parameter sets (FP32 and BF16) whose outputs the
  // forward pass averages; the primary parameters p stay the trained ones
  int nmem = 0;
  float* mp = nullptr;
  __nv_bfloat16* mpb = nullptr;
  float* Yacc = nullptr;
};

static int mfail(covgpu_mlp* net, int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(net->err, sizeof(net->err), fmt, ap);
  va_end(ap);
  return code;
}

#define MCK(call)                                                                            \
  do {                                                                                       \
    cudaError_t e_ = (call);                                                                 \
    if (e_ != cudaSuccess) return mfail(net, 90, "%s: %s", #call, cudaGetErrorString(e_));   \
  } while (0)

template <class T>
static cudaError_t malloc_n(T** p, size_t n) {
  return cudaMalloc((void**)p, std::max<size_t>(n, 1) * sizeof(T));
}

// the network with parameters p (FP32 biases) and pb (BF16 weights)
static void enqueue_forward(covgpu_mlp* net, int B, const float* p, const __nv_bfloat16* pb) {
  cudaStream_t st = net->st;
  gemm<float, __nv_bfloat16, EPI_SILU>(st, net->Xb, kNFeat, 1, pb + oW1, 1, kNFeat, B, kHid, kNFeat, p + ob1,
                                       nullptr, net->H[0], net->Z[0]);
  gemm<float, __nv_bfloat16, EPI_SILU>(st, net->H[0], kHid, 1, pb + oW2, 1, kHid, B, kHid, kHid, p + ob2, nullptr,
                                       net->H[1], net->Z[1]);
  gemm<float, __nv_bfloat16, EPI_SILU>(st, net->H[1], kHid, 1, pb + oW3, 1, kHid, B, kHid, kHid, p + ob3, nullptr,
                                       net->H[2], net->Z[2]);
  gemm<float, __nv_bfloat16, EPI_PLAIN>(st, net->H[2], kHid, 1, pb + oW4, 1, kHid, B, kOut, kHid, p + ob4, nullptr,
                                        net->Yp);
}
static void enqueue_forward(covgpu_mlp* net, int B) { enqueue_forward(net, B, net->p, net->pb); }

// gradients into net->g, from dY
static void enqueue_backward(covgpu_mlp* net, int B) {
  cudaStream_t st = net->st;
  float* g = net->g;
  // layer 4
  gemm<float, float, EPI_PLAIN>(st, net->dY, 1, kOut, net->H[2], kHid, 1, kOut, kHid, B, nullptr, nullptr, g + oW4);
  k_colsum<<<1, 32, 0, st>>>(net->dY, B, kOut, g + ob4);
  gemm<float, __nv_bfloat16, EPI_DSILU>(st, net->dY, kOut, 1, net->pb + oW4, kHid, 1, B, kHid, kOut, nullptr,
                                        net->Z[2], net->D[2]);
  // layer 3
  gemm<float, float, EPI_PLAIN>(st, net->D[2], 1, kHid, net->H[1], kHid, 1, kHid, kHid, B, nullptr, nullptr, g + oW3);
  k_colsum<<<1, kHid, 0, st>>>(net->D[2], B, kHid, g + ob3);
  gemm<float, __nv_bfloat16, EPI_DSILU>(st, net->D[2], kHid, 1, net->pb + oW3, kHid, 1, B, kHid, kHid, nullptr,
                                        net->Z[1], net->D[1]);
  // layer 2
  gemm<float, float, EPI_PLAIN>(st, net->D[1], 1, kHid, net->H[0], kHid, 1, kHid, kHid, B, nullptr, nullptr, g + oW2);
  k_colsum<<<1, kHid, 0, st>>>(net->D[1], B, kHid, g + ob2);
  gemm<float, __nv_bfloat16, EPI_DSILU>(st, net->D[1], kHid, 1, net->pb + oW2, kHid, 1, B, kHid, kHid, nullptr,
                                        net->Z[0], net->D[0]);
  // layer 1
  gemm<float, float, EPI_PLAIN>(st, net->D[0], 1, kHid, net->Xb, kNFeat, 1, kHid, kNFeat, B, nullptr, nullptr,
                                g + oW1);
  k_colsum<<<1, kHid, 0, st>>>(net->D[0], B, kHid, g + ob1);
}

extern "C" const char* covgpu_mlp_errmsg(const covgpu_mlp* net) { return net ? net->err : "no network"; }

extern "C" void covgpu_mlp_destroy(covgpu_mlp* net) {
  if (!net) return;
  cudaSetDevice(net->dev);
  void* bufs[] = {net->p, net->m, net->v, net->g, net->pb, net->nrm, net->hyper, net->Xin, net->Xb, net->Tb,
                  net->Yp, net->dY, net->Yout, net->Z[0], net->Z[1], net->Z[2], net->H[0], net->H[1], net->H[2],
                  net->D[0], net->D[1], net->D[2], net->counter, net->mp, net->mpb, net->Yacc};
  for (void* b : bufs) if (b) cudaFree(b);
  if (net->st) cudaStreamDestroy(net->st);
  delete net;
}

extern "C" int covgpu_mlp_create(covgpu_mlp** ret, int device, int batch_cap, uint64_t seed) {
  *ret = nullptr;
  if (batch_cap < 1 || batch_cap > (1 << 20)) return 11;
  covgpu_mlp* net = new covgpu_mlp();
  *ret = net;
  net->dev = device;
  net->cap = batch_cap;
  MCK(cudaSetDevice(device));
  MCK(cudaStreamCreateWithFlags(&net->st, cudaStreamNonBlocking));
  const size_t P = kNParam, cap = batch_cap;
  MCK(malloc_n(&net->p, P)); MCK(malloc_n(&net->m, P)); MCK(malloc_n(&net->v, P)); MCK(malloc_n(&net->g, P));
  MCK(malloc_n(&net->pb, P));
  MCK(malloc_n(&net->nrm, 2 * kNFeat + 2 * kOut));
  MCK(malloc_n(&net->hyper, 2));
  MCK(malloc_n(&net->Xin, cap * kNFeat)); MCK(malloc_n(&net->Xb, cap * kNFeat)); MCK(malloc_n(&net->Tb, cap * kOut));
  MCK(malloc_n(&net->Yp, cap * kOut)); MCK(malloc_n(&net->dY, cap * kOut)); MCK(malloc_n(&net->Yout, cap * kOut));
  for (int l = 0; l < 3; l++) {
    MCK(malloc_n(&net->Z[l], cap * kHid)); MCK(malloc_n(&net->H[l], cap * kHid)); MCK(malloc_n(&net->D[l], cap * kHid));
  }
  MCK(malloc_n(&net->counter, 1));
  // LeCun-uniform weights (variance 1/fan_in), zero biases; splitmix64 stream
  std::vector<float> h(P, 0.f);
  uint64_t st = seed;
  auto uni = [&]() { st = splitmix64(st); return (double)(st >> 11) * (1.0 / 9007199254740992.0); };
  auto fill = [&](int off, int fo, int fi) {
    const double a = std::sqrt(3.0 / fi);
    for (int k = 0; k < fo * fi; k++) h[off + k] = (float)((2.0 * uni() - 1.0) * a);
  };
  fill(oW1, kHid, kNFeat); fill(oW2, kHid, kHid); fill(oW3, kHid, kHid); fill(oW4, kOut, kHid);
  net->h_nrm.assign(2 * kNFeat + 2 * kOut, 0.f);
  for (int f = 0; f < kNFeat; f++) net->h_nrm[kNFeat + f] = 1.f;
  for (int k = 0; k < kOut; k++) net->h_nrm[2 * kNFeat + kOut + k] = 1.f;
  net->xlo.assign(kNFeat, -INFINITY);
  net->xhi.assign(kNFeat, INFINITY);
  MCK(cudaMemcpy(net->nrm, net->h_nrm.data(), net->h_nrm.size() * sizeof(float), cudaMemcpyHostToDevice));
  return covgpu_mlp_set_params(net, h.data());
}

extern "C" int covgpu_mlp_set_params(covgpu_mlp* net, const float* params) {
  if (!net) return 11;
  MCK(cudaSetDevice(net->dev));
  for (int k = 0; k < kNParam; k++)
    if (!std::isfinite(params[k])) return mfail(net, 11, "parameter %d is not finite", k);
  MCK(cudaMemcpyAsync(net->p, params, kNParam * sizeof(float), cudaMemcpyHostToDevice, net->st));
  k_to_bf16<<<(kNParam + 255) / 256, 256, 0, net->st>>>(net->p, net->pb, kNParam);
  MCK(cudaGetLastError());
  MCK(cudaStreamSynchronize(net->st));
  return 0;
}

extern "C" int covgpu_mlp_set_members(covgpu_mlp* net, const float* params, int nmem) {
  if (!net) return 11;
  MCK(cudaSetDevice(net->dev));
  if (nmem < 0 || nmem > COVGPU_MLP_MAXMEM) return mfail(net, 11, "%d members outside 0..%d", nmem, COVGPU_MLP_MAXMEM);
  if (nmem > 0 && !params) return mfail(net, 11, "no member parameters");
  for (size_t k = 0; k < (size_t)nmem * kNParam; k++)
    if (!std::isfinite(params[k])) return mfail(net, 11, "member %d parameter %d is not finite", (int)(k / kNParam),
                                                (int)(k % kNParam));
  MCK(cudaStreamSynchronize(net->st));
  if (net->mp) cudaFree(net->mp);
  if (net->mpb) cudaFree(net->mpb);
  if (net->Yacc) cudaFree(net->Yacc);
  net->mp = nullptr; net->mpb = nullptr; net->Yacc = nullptr; net->nmem = 0;
  if (nmem == 0) return 0;
  const size_t n = (size_t)nmem * kNParam;
  MCK(malloc_n(&net->mp, n)); MCK(malloc_n(&net->mpb, n)); MCK(malloc_n(&net->Yacc, (size_t)net->cap * kOut));
  MCK(cudaMemcpyAsync(net->mp, params, n * sizeof(float), cudaMemcpyHostToDevice, net->st));
  k_to_bf16<<<(int)((n + 255) / 256), 256, 0, net->st>>>(net->mp, net->mpb, (int)n);
  MCK(cudaGetLastError());
  MCK(cudaStreamSynchronize(net->st));
  net->nmem = nmem;
  return 0;
}

extern "C" int covgpu_mlp_get_params(covgpu_mlp* net, float* params) {
  if (!net) return 11;
  MCK(cudaSetDevice(net->dev));
  MCK(cudaMemcpyAsync(params, net->p, kNParam * sizeof(float), cudaMemcpyDeviceToHost, net->st));
  MCK(cudaStreamSynchronize(net->st));
  return 0;
}

extern "C" int covgpu_mlp_set_norm(covgpu_mlp* net, const float* xmean, const float* xstd, const float* ymean,
                                   const float* ystd, const float* xlo, const float* xhi) {
  if (!net) return 11;
  MCK(cudaSetDevice(net->dev));
  for (int f = 0; f < kNFeat; f++) {
    if (!(xstd[f] > 0.f) || !std::isfinite(xmean[f])) return mfail(net, 11, "feature %d: bad standardisation", f);
    net->h_nrm[f] = xmean[f];
    net->h_nrm[kNFeat + f] = xstd[f];
    net->xlo[f] = xlo ? xlo[f] : -INFINITY;
    net->xhi[f] = xhi ? xhi[f] : INFINITY;
  }
  for (int k = 0; k < kOut; k++) {
    if (!(ystd[k] > 0.f) || !std::isfinite(ymean[k])) return mfail(net, 11, "output %d: bad standardisation", k);
    net->h_nrm[2 * kNFeat + k] = ymean[k];
    net->h_nrm[2 * kNFeat + kOut + k] = ystd[k];
  }
  MCK(cudaMemcpy(net->nrm, net->h_nrm.data(), net->h_nrm.size() * sizeof(float), cudaMemcpyHostToDevice));
  return 0;
}

extern "C" int covgpu_mlp_get_norm(const covgpu_mlp* net, float* xmean, float* xstd, float* ymean, float* ystd,
                                   float* xlo, float* xhi) {
  if (!net) return 11;
  for (int f = 0; f < kNFeat; f++) {
    if (xmean) xmean[f] = net->h_nrm[f];
    if (xstd) xstd[f] = net->h_nrm[kNFeat + f];
    if (xlo) xlo[f] = net->xlo[f];
    if (xhi) xhi[f] = net->xhi[f];
  }
  for (int k = 0; k < kOut; k++) {
    if (ymean) ymean[k] = net->h_nrm[2 * kNFeat + k];
    if (ystd) ystd[k] = net->h_nrm[2 * kNFeat + kOut + k];
  }
  return 0;
}

extern "C" int covgpu_mlp_in_range(const covgpu_mlp* net, const float* feat) {
  if (!net || !feat) return 0;
  for (int f = 0; f < kNFeat; f++)
    if (!(feat[f] >= net->xlo[f] && feat[f] <= net->xhi[f])) return 0;
  return 1;
}

extern "C" int covgpu_mlp_forward(covgpu_mlp* net, const float* X, int n, float* Y) {
  if (!net) return 11;
  MCK(cudaSetDevice(net->dev));
  if (n < 0) return mfail(net, 11, "negative row count");
  for (int r0 = 0; r0 < n; r0 += net->cap) {
    const int B = std::min(net->cap, n - r0);
    MCK(cudaMemcpyAsync(net->Xin, X + (size_t)r0 * kNFeat, (size_t)B * kNFeat * sizeof(float),
                        cudaMemcpyHostToDevice, net->st));
    k_gather<<<std::min(1024, (B * kNFeat + 255) / 256), 256, 0, net->st>>>(net->Xin, nullptr, nullptr, nullptr, 1,
                                                                            B, net->nrm, net->Xb, nullptr);
    if (net->nmem == 0) {
      enqueue_forward(net, B);
      k_denorm<<<(B * kOut + 255) / 256, 256, 0, net->st>>>(net->Yp, B, net->nrm, 1.f, net->Yout);
    } else {
      for (int k = 0; k < net->nmem; k++) {
        enqueue_forward(net, B, net->mp + (size_t)k * kNParam, net->mpb + (size_t)k * kNParam);
        k_accum<<<(B * kOut + 255) / 256, 256, 0, net->st>>>(net->Yp, B * kOut, k == 0, net->Yacc);
      }
      k_denorm<<<(B * kOut + 255) / 256, 256, 0, net->st>>>(net->Yacc, B, net->nrm, 1.f / (float)net->nmem,
                                                            net->Yout);
    }
    MCK(cudaGetLastError());
    MCK(cudaMemcpyAsync(Y + (size_t)r0 * kOut, net->Yout, (size_t)B * kOut * sizeof(float), cudaMemcpyDeviceToHost,
                        net->st));
  }
  MCK(cudaStreamSynchronize(net->st));
  return 0;
}

extern "C" int covgpu_mlp_grad(covgpu_mlp* net, const float* X, const float* T, int n, float* grad, float* loss) {
  if (!net) return 11;
  MCK(cudaSetDevice(net->dev));
  if (n < 1 || n > net->cap) return mfail(net, 11, "batch of %d rows outside 1..%d", n, net->cap);
  float* dT = nullptr;
  MCK(malloc_n(&dT, (size_t)n * kOut));
  cudaError_t e = cudaMemcpyAsync(net->Xin, X, (size_t)n * kNFeat * sizeof(float), cudaMemcpyHostToDevice, net->st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dT, T, (size_t)n * kOut * sizeof(float), cudaMemcpyHostToDevice, net->st);
  if (e == cudaSuccess) {
    k_gather<<<std::min(1024, (n * kNFeat + 255) / 256), 256, 0, net->st>>>(net->Xin, dT, nullptr, nullptr, 1, n,
                                                                            net->nrm, net->Xb, net->Tb);
    enqueue_forward(net, n);
    k_loss<<<1, 256, 0, net->st>>>(net->Yp, net->Tb, n, net->dY, net->Yout, nullptr);
    enqueue_backward(net, n);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(grad, net->g, kNParam * sizeof(float), cudaMemcpyDeviceToHost, net->st);
  if (e == cudaSuccess && loss) e = cudaMemcpyAsync(loss, net->Yout, sizeof(float), cudaMemcpyDeviceToHost, net->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(net->st);
  cudaFree(dT);
  if (e != cudaSuccess) return mfail(net, 90, "CUDA error %s", cudaGetErrorString(e));
  return 0;
}

extern "C" int covgpu_mlp_train(covgpu_mlp* net, const float* X, const float* T, int n, int epochs, int batch,
                                float lr, float wd, uint64_t seed, float* epoch_loss) {
  if (!net) return 11;
  MCK(cudaSetDevice(net->dev));
  if (batch < 1 || batch > net->cap || n < batch || epochs < 1)
    return mfail(net, 11, "need 1 <= batch <= %d, batch <= n and epochs >= 1", net->cap);
  for (size_t k = 0; k < (size_t)n * kNFeat; k++)
    if (!std::isfinite(X[k])) return mfail(net, 11, "feature row %zu is not finite", k / kNFeat);
  for (size_t k = 0; k < (size_t)n * kOut; k++)
    if (!std::isfinite(T[k])) return mfail(net, 11, "target row %zu is not finite", k / kOut);
  const int spe = n / batch;
  const int nsteps = spe * epochs;
  float *dX = nullptr, *dT = nullptr, *lossbuf = nullptr;
  int* dperm = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaError_t e = malloc_n(&dX, (size_t)n * kNFeat);
  if (e == cudaSuccess) e = malloc_n(&dT, (size_t)n * kOut);
  if (e == cudaSuccess) e = malloc_n(&lossbuf, (size_t)nsteps);
  if (e == cudaSuccess) e = malloc_n(&dperm, (size_t)spe * batch);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dX, X, (size_t)n * kNFeat * sizeof(float), cudaMemcpyHostToDevice, net->st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dT, T, (size_t)n * kOut * sizeof(float), cudaMemcpyHostToDevice, net->st);
  // a fresh AdamW run from the current parameters
  if (e == cudaSuccess) e = cudaMemsetAsync(net->m, 0, kNParam * sizeof(float), net->st);
  if (e == cudaSuccess) e = cudaMemsetAsync(net->v, 0, kNParam * sizeof(float), net->st);
  if (e == cudaSuccess) e = cudaMemsetAsync(net->counter, 0, sizeof(int), net->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(net->st);
  // one training step as a graph
  if (e == cudaSuccess) e = cudaStreamBeginCapture(net->st, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    k_gather<<<std::min(1024, (batch * kNFeat + 255) / 256), 256, 0, net->st>>>(dX, dT, dperm, net->counter, spe,
                                                                                batch, net->nrm, net->Xb, net->Tb);
    enqueue_forward(net, batch);
    k_loss<<<1, 256, 0, net->st>>>(net->Yp, net->Tb, batch, net->dY, lossbuf, net->counter);
    enqueue_backward(net, batch);
    k_adam<<<296, 256, 0, net->st>>>(net->p, net->m, net->v, net->g, net->pb, kNParam, net->counter, net->hyper);
    cudaError_t ec = cudaStreamEndCapture(net->st, &graph);
    e = (ec != cudaSuccess) ? ec : cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
  std::vector<int> perm(n);
  uint64_t rs = splitmix64(seed);
  for (int ep = 0; ep < epochs && e == cudaSuccess; ep++) {
    // Fisher-Yates shuffle of the rows, then a cosine learning-rate decay to 5%
    for (int k = 0; k < n; k++) perm[k] = k;
    for (int k = n - 1; k > 0; k--) {
      rs = splitmix64(rs);
      const int r = (int)(rs % (uint64_t)(k + 1));
      std::swap(perm[k], perm[r]);
    }
    const float hyp[2] = {lr * (0.05f + 0.95f * 0.5f * (1.f + (float)std::cos(3.14159265358979323846 * ep / epochs))), wd};
    e = cudaMemcpyAsync(dperm, perm.data(), (size_t)spe * batch * sizeof(int), cudaMemcpyHostToDevice, net->st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(net->hyper, hyp, sizeof(hyp), cudaMemcpyHostToDevice, net->st);
    // the copies above read host memory that changes next epoch
    if (e == cudaSuccess) e = cudaStreamSynchronize(net->st);
    for (int s = 0; s < spe && e == cudaSuccess; s++) e = cudaGraphLaunch(exec, net->st);
  }
  std::vector<float> lh(nsteps);
  if (e == cudaSuccess) e = cudaMemcpyAsync(lh.data(), lossbuf, nsteps * sizeof(float), cudaMemcpyDeviceToHost, net->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(net->st);
  if (exec) cudaGraphExecDestroy(exec);
  if (graph) cudaGraphDestroy(graph);
  cudaFree(dX); cudaFree(dT); cudaFree(lossbuf); cudaFree(dperm);
  if (e != cudaSuccess) return mfail(net, 90, "CUDA error %s", cudaGetErrorString(e));
  if (epoch_loss)
    for (int ep = 0; ep < epochs; ep++) {
      double a = 0.0;
      for (int s = 0; s < spe; s++) a += lh[(size_t)ep * spe + s];
      epoch_loss[ep] = (float)(a / spe);
    }
  return 0;
}
