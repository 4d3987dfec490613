// hd_noalloc.cu -- L2 norm / error of a nodal DG vector without any
// allocation by the library (hd_norm_and_error_noalloc).
//
// Who needs it: callers that must not allocate device memory themselves or
// through a library -- plug-ins inside a host application that owns every
// byte of device memory (pre-planned pools, enforced memory budgets), time
// loops whose host framework forbids device allocation after start-up
// because of its latency and fragmentation, and diagnostics run next to a
// memory manager that holds the CUDA allocator.  hd_adv_create() allocates
// its reduction scratch with cudaMalloc, so this entry point takes the mesh
// descriptor instead of a handle and keeps its scratch in a fixed-size array
// in device global memory that is part of the loaded library.
//
// Set-up: the first call on a device (with that device current) looks up the
// array's device address with cudaGetSymbolAddress and caches it; make that
// first call before any stream capture.
//
// The scratch array (kNoAllocPartials pairs of doubles, 256 KiB plus the
// final pair) is held by every GPU that loads the library until the process
// exits.  Every call shares it, so calls whose kernels overlap on the GPU (on
// different streams, or from different host threads) race and give wrong
// results; serialise them.  Each call overwrites every partial it later reads,
// so nothing has to start at zero.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/hyperdeal_gb300.h"
#include "hd_ecl.cuh"
#include "hd_rules.h"

namespace {

constexpr int kNoAllocThreads = 256;
constexpr int kNoAllocPerThread = 32;  // DoFs summed by one thread
constexpr int kNoAllocPartials = 16384;
constexpr long long kNoAllocMaxDofs =
    (long long)kNoAllocPartials * kNoAllocThreads * kNoAllocPerThread;  // 134,217,728

// block partial sums (v^2 JxW, e^2 JxW), then the two final norms
__device__ __align__(256) double g_noalloc_scratch[2 * kNoAllocPartials + 2];

struct Geom {
  int D, dim_x, N, NC;
  long long ncx, n;
  int cells[hd::kMaxDim];
  double lo[hd::kMaxDim], h[hd::kMaxDim];
  double gl[hd::kMaxN], glw[hd::kMaxN];
};

template <typename T>
__global__ void noalloc_partials(Geom g, hd::DevFunction f, double t, const T* __restrict__ src,
                                 double* __restrict__ partials) {
  double s0 = 0.0, s1 = 0.0;
  const long long base = (long long)blockIdx.x * kNoAllocThreads * kNoAllocPerThread + threadIdx.x;
  for (int j = 0; j < kNoAllocPerThread; ++j) {
    const long long i = base + (long long)j * kNoAllocThreads;
    if (i >= g.n) break;
    const long long gid = i / g.NC;
    int node = int(i - gid * g.NC);
    long long gx = gid % g.ncx, gv = gid / g.ncx;
    double x[hd::kMaxDim], jxw = 1.0;
    for (int d = 0; d < g.D; ++d) {
      int c;
      if (d < g.dim_x) { c = int(gx % g.cells[d]); gx /= g.cells[d]; }
      else { c = int(gv % g.cells[d]); gv /= g.cells[d]; }
      const int id = node % g.N;
      node /= g.N;
      x[d] = g.lo[d] + (c + g.gl[id]) * g.h[d];
      jxw *= g.h[d] * g.glw[id];
    }
    const double v = double(src[i]);
    const double e = v - hd::eval_function(f, x, g.D, t);
    s0 += v * v * jxw;
    s1 += e * e * jxw;
  }
  __shared__ double r0[kNoAllocThreads / 32], r1[kNoAllocThreads / 32];
  for (int o = 16; o > 0; o >>= 1) {
    s0 += __shfl_down_sync(0xffffffffu, s0, o);
    s1 += __shfl_down_sync(0xffffffffu, s1, o);
  }
  if ((threadIdx.x & 31) == 0) {
    r0[threadIdx.x / 32] = s0;
    r1[threadIdx.x / 32] = s1;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0;
    for (int k = 0; k < kNoAllocThreads / 32; ++k) {
      a += r0[k];
      b += r1[k];
    }
    partials[2 * blockIdx.x] = a;
    partials[2 * blockIdx.x + 1] = b;
  }
}

__global__ void noalloc_finish(double* __restrict__ scratch, int nblocks) {
  // one warp, fixed order: lane l sums partials l, l+32, ..., then a fixed tree
  double a = 0.0, b = 0.0;
  for (int k = threadIdx.x; k < nblocks; k += 32) {
    a += scratch[2 * k];
    b += scratch[2 * k + 1];
  }
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_down_sync(0xffffffffu, a, o);
    b += __shfl_down_sync(0xffffffffu, b, o);
  }
  if (threadIdx.x == 0) {
    scratch[2 * kNoAllocPartials] = sqrt(a);
    scratch[2 * kNoAllocPartials + 1] = sqrt(b);
  }
}

constexpr const char* kTooLarge =
    "hd_norm_and_error_noalloc: more than 134,217,728 DoFs (its static scratch holds 16384 block partials); "
    "use hd_norm_and_error";

int noalloc_fail(int code, const char* msg) {
  hd::set_last_error(msg);
  return code;
}

// device address of the scratch array, looked up once per device
std::mutex g_addr_mutex;
double* g_addr[64] = {nullptr};

int scratch_address(double** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return noalloc_fail(HD_ERR_CUDA, cudaGetErrorString(e));
  if (dev < 0 || dev >= 64) return noalloc_fail(HD_ERR_UNSUPPORTED, "device index above 63");
  std::lock_guard<std::mutex> lock(g_addr_mutex);
  if (!g_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return noalloc_fail(HD_ERR_CUDA, cudaGetErrorString(e));
    g_addr[dev] = static_cast<double*>(p);
  }
  *out = g_addr[dev];
  return HD_OK;
}

}  // namespace

extern "C" int hd_norm_and_error_noalloc(const hd_adv_desc* desc, const hd_function* f, double time,
                                         const void* src, double* result, void* stream) {
  if (!desc || !f || !src || !result) return noalloc_fail(HD_ERR_INVALID, "hd_norm_and_error_noalloc: null argument");
  const hd_adv_desc& d = *desc;
  if (d.dim_x < 1 || d.dim_x > 3 || d.dim_v < 1 || d.dim_v > 3 || d.degree < 1 || d.degree + 1 > hd::kMaxN ||
      d.n_points != d.degree + 1 || (d.dtype != HD_F64 && d.dtype != HD_F32))
    return noalloc_fail(HD_ERR_INVALID, "hd_norm_and_error_noalloc: unsupported descriptor");
  if (d.quadrature != HD_QUAD_GAUSS_LOBATTO)
    return noalloc_fail(HD_ERR_UNSUPPORTED, "hd_norm_and_error_noalloc: Gauss-Lobatto collocation only");
  if (f->kind < 0 || f->kind > 2)
    return noalloc_fail(HD_ERR_INVALID, "hd_norm_and_error_noalloc: unknown function kind");
  Geom g;
  std::memset(&g, 0, sizeof(g));
  g.D = d.dim_x + d.dim_v;
  g.dim_x = d.dim_x;
  g.N = d.degree + 1;
  g.NC = hd::ipow(g.N, g.D);
  long long ncells = 1;
  g.ncx = 1;
  for (int i = 0; i < g.D; ++i) {
    const bool isx = i < d.dim_x;
    const int c = isx ? d.cells_x[i] : d.cells_v[i - d.dim_x];
    const double lo = isx ? d.lo_x[i] : d.lo_v[i - d.dim_x];
    const double hi = isx ? d.hi_x[i] : d.hi_v[i - d.dim_x];
    if (c < 1 || !(hi > lo)) return noalloc_fail(HD_ERR_INVALID, "hd_norm_and_error_noalloc: bad mesh");
    g.cells[i] = c;
    g.lo[i] = lo;
    g.h[i] = (hi - lo) / c;
    // ncells <= 2^27 and c < 2^31 before the product, so it cannot overflow
    ncells *= c;
    if (ncells > kNoAllocMaxDofs) return noalloc_fail(HD_ERR_INVALID, kTooLarge);
    if (isx) g.ncx *= c;
  }
  // ncells <= 2^27 and NC <= 6^6, so this product fits comfortably in 64 bits
  g.n = ncells * g.NC;
  if (g.n > kNoAllocMaxDofs) return noalloc_fail(HD_ERR_INVALID, kTooLarge);
  hd::rules::gauss_lobatto(g.N, g.gl, g.glw);
  hd::DevFunction df;
  std::memset(&df, 0, sizeof(df));
  df.kind = f->kind;
  df.amp = f->amp;
  for (int i = 0; i < HD_MAX_DIM; ++i) {
    df.omega[i] = f->omega[i];
    df.speed[i] = f->speed[i];
    df.phase[i] = f->phase[i];
    df.cosine[i] = f->cosine[i];
  }
  double* scratch = nullptr;
  int rc = scratch_address(&scratch);
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  const long long per_block = (long long)kNoAllocThreads * kNoAllocPerThread;
  const int nblocks = int((g.n + per_block - 1) / per_block);
  if (d.dtype == HD_F32)
    noalloc_partials<float><<<nblocks, kNoAllocThreads, 0, s>>>(g, df, time, (const float*)src, scratch);
  else
    noalloc_partials<double><<<nblocks, kNoAllocThreads, 0, s>>>(g, df, time, (const double*)src, scratch);
  noalloc_finish<<<1, 32, 0, s>>>(scratch, nblocks);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return noalloc_fail(HD_ERR_CUDA, cudaGetErrorString(e));
  e = cudaMemcpyAsync(result, scratch + 2 * kNoAllocPartials, 2 * sizeof(double), cudaMemcpyDeviceToHost, s);
  if (e != cudaSuccess) return noalloc_fail(HD_ERR_CUDA, cudaGetErrorString(e));
  e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return noalloc_fail(HD_ERR_CUDA, cudaGetErrorString(e));
  return HD_OK;
}

