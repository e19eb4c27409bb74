// cov_noalloc.cu -- APC/ASC correction of a device-resident score matrix
// that allocates no device memory.
//
// For callers that cannot allocate device memory: code running while a CUDA
// stream is being captured into a graph (cudaMalloc is not permitted then),
// host code whose device memory comes from a fixed pool owned by someone
// else, or a real-time caller that must not block in the allocator.  They
// pass the input score matrix and the output buffers; the per-column sums,
// the average and the min/max partials live in the file-scope array below,
// which every GPU that loads this library keeps until the process exits.
//
// The array is shared by every call: calls that run at the same time on the
// GPU (different streams, or different host threads) race on it and must be
// serialised by the caller.  Each call clears the parts it accumulates into.
//
// A NaN among the corrected scores is an error in the reference
// (src/correlators.c:1124, "bad covariation").  The call is asynchronous, so
// it reports this in the result: d_minmax becomes {NaN, NaN}.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cfloat>
#include <cmath>
#include <cstdint>
#include <mutex>

#include "covgpu.h"

namespace {

// scratch: column sums [COVGPU_NOALLOC_MAX_L] + average + min/max partials
constexpr int MAXL = COVGPU_NOALLOC_MAX_L;
constexpr int MMBLK = 256;   // blocks of the apply kernel (min/max partials)
struct Scratch {
  double colx[MAXL];
  double avg;
  double tmin[MMBLK];
  double tmax[MMBLK];
  int nan;            // set when a corrected score is NaN
};
static __device__ __align__(256) Scratch g_scratch;

// one block per row i: COVx[i] = sum_{j != i} COV[i][j] / (L - 1)
__global__ void k_na_colx(const double* __restrict__ cov, int L, Scratch* sc) {
  const int i = blockIdx.x;
  __shared__ double buf[256];
  double s = 0.0;
  for (int j = threadIdx.x; j < L; j += blockDim.x)
    if (j != i) s += cov[(int64_t)i * L + j];
  buf[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) buf[threadIdx.x] += buf[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    sc->colx[i] = (L > 1) ? buf[0] / ((double)L - 1.0) : buf[0];
    if (i == 0) sc->nan = 0;   // this call's NaN flag (read after k_na_apply)
  }
}

// avg = 2/(L(L-1)) sum_{i<j} COV = sum_i COVx[i] / L
__global__ void k_na_avg(int L, Scratch* sc) {
  __shared__ double buf[256];
  double s = 0.0;
  for (int c = threadIdx.x; c < L; c += blockDim.x) s += sc->colx[c];
  buf[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) buf[threadIdx.x] += buf[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) sc->avg = (L > 1) ? buf[0] * ((double)L - 1.0) / ((double)L * ((double)L - 1.0)) : 0.0;
}

// out[i][j] = corrected score (i != j), diagonal -inf; per-block min/max.
// Each element is read and written by the same thread, so out may be cov.
__global__ void k_na_apply(const double* cov, double* out, int L, int actype, Scratch* sc) {
  __shared__ double smin[256], smax[256];
  const double A = sc->avg;
  double lo = DBL_MAX, hi = -DBL_MAX;
  const int64_t n = (int64_t)L * L;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(k / L), j = (int)(k % L);
    if (i == j) { out[k] = -INFINITY; continue; }
    const double v = cov[k];
    double r;
    if (actype == 0) r = (A != 0.0) ? v - sc->colx[i] * sc->colx[j] / A : 0.0;
    else             r = v - (sc->colx[i] + sc->colx[j] - A);
    out[k] = r;
    if (isnan(r)) sc->nan = 1;
    lo = fmin(lo, r); hi = fmax(hi, r);
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
  if (threadIdx.x == 0) { sc->tmin[blockIdx.x] = smin[0]; sc->tmax[blockIdx.x] = smax[0]; }
}

__global__ void k_na_minmax(Scratch* sc, int nblk, double* __restrict__ minmax) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double lo = DBL_MAX, hi = -DBL_MAX;
    for (int b = 0; b < nblk; b++) { lo = fmin(lo, sc->tmin[b]); hi = fmax(hi, sc->tmax[b]); }
    minmax[0] = (lo == DBL_MAX) ? INFINITY : lo;
    minmax[1] = (hi == -DBL_MAX) ? -INFINITY : hi;
    if (sc->nan) minmax[0] = minmax[1] = NAN;
  }
}

// device address of g_scratch, looked up once per device and context (the
// host-side symbol is only a stand-in and must never be handed to a kernel).
// The context id is part of the key: after a device reset the module is
// loaded again into a new context, possibly at another address.
constexpr int MAXDEV = 64;
struct AddrCache { unsigned long long ctx_id = 0; Scratch* addr = nullptr; };
AddrCache g_addr[MAXDEV];
std::mutex g_addr_mu;

// id of the current context, through the driver entry points the runtime
// exposes (no link against the driver library); 0 if unavailable
unsigned long long current_ctx_id() {
  using GetCurrent = CUresult (*)(CUcontext*);
  using GetId = CUresult (*)(CUcontext, unsigned long long*);
  static GetCurrent get_current = nullptr;
  static GetId get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    cudaDriverEntryPointQueryResult q;
    void* p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = (GetCurrent)p;
    p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = (GetId)p;
  });
  CUcontext c = nullptr;
  unsigned long long id = 0;
  if (!get_current || !get_id || get_current(&c) != CUDA_SUCCESS || !c || get_id(c, &id) != CUDA_SUCCESS) return 0;
  return id;
}

}  // namespace

extern "C" int covgpu_correct_noalloc(const double* d_cov, double* d_out, int L, int actype, double* d_minmax,
                                      void* stream) {
  if (L < 2 || L > MAXL) return 11;
  if (actype != 0 && actype != 1) return 11;
  if (!d_cov || !d_out || !d_minmax) return 11;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAXDEV) return 90;
  Scratch* sc = nullptr;
  {
    std::lock_guard<std::mutex> g(g_addr_mu);
    const unsigned long long id = current_ctx_id();
    if (!g_addr[dev].addr || id != g_addr[dev].ctx_id) {
      void* p = nullptr;
      if (cudaGetSymbolAddress(&p, g_scratch) != cudaSuccess || !p) return 90;
      g_addr[dev].addr = (Scratch*)p;
      g_addr[dev].ctx_id = id;
    }
    sc = g_addr[dev].addr;
  }
  cudaStream_t st = (cudaStream_t)stream;
  k_na_colx<<<L, 256, 0, st>>>(d_cov, L, sc);
  k_na_avg<<<1, 256, 0, st>>>(L, sc);
  k_na_apply<<<MMBLK, 256, 0, st>>>(d_cov, d_out, L, actype, sc);
  k_na_minmax<<<1, 32, 0, st>>>(sc, MMBLK, d_minmax);
  return (cudaGetLastError() == cudaSuccess) ? 0 : 90;
}
