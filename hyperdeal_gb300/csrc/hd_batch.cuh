// hd_batch.cuh -- many independent advection instances of one class
// (phase-space dimension D, nodes per direction N, storage type T) advanced
// by ONE persistent launch per stage.  The CTAs of the launch walk the
// concatenated cell blocks of all instances of the class; each block is
// computed with its own instance's parameters (mesh, line operators, stage
// factors, vectors), and the next block -- of whichever instance -- is staged
// by cp.async while the current one is computed, as in the single-instance
// generic kernel (hd_ecl.cuh).  FP64 instances switched to FP32x2 arithmetic
// (hd_adv_set_arithmetic) form their own class with the FP32x2 block.
#pragma once

#include <cuda_runtime.h>

#include "hd_ecl.cuh"

namespace hd {

constexpr int kBatchMaxInstances = 256;

// launch of the batch kernel for one class: params[i] are the instances'
// stage parameters (device memory), prefix[i] = first cell block of instance i
// (prefix[n] = total blocks), cpb cells per block, ctas_per_sm (0 = occupancy)
template <typename T>
struct BatchLaunch {
  const EclParams<T>* params;
  const long long* prefix;
  int n;
  int cpb;
  int ctas_per_sm;
};

struct BatchLaunchers {
  cudaError_t (*f64)(const BatchLaunch<double>&, int mode, cudaStream_t);
  cudaError_t (*f32)(const BatchLaunch<float>&, int mode, cudaStream_t);
  int max_cpb_f64, max_cpb_f32;
  int def_cpb_f64, def_cpb_f32;  // default tiles (ecl_default_cpb)
  bool ok;
  cudaError_t (*f64x)(const BatchLaunch<double>&, int mode, cudaStream_t);  // FP64 storage, FP32x2 arithmetic
};

// classes with a batch kernel: D in {4, 5}, N in {3..6} (degree 2..5);
// other classes return ok == false and are advanced per instance
BatchLaunchers batch_launchers(int D, int N);
BatchLaunchers batch_launchers_d4(int N);
BatchLaunchers batch_launchers_d5(int N);

template <int D, int N, typename T, int MODE, typename A = T>
__global__ void __launch_bounds__(EclShape<D, N, T>::THREADS,
                                  std::is_same_v<A, f32x2> ? 2 : EclShape<D, N, T>::MINB)
    ecl_batch_kernel(const EclParams<T>* __restrict__ params, const long long* __restrict__ prefix, int n, int cpb) {
  using S = EclShape<D, N, T>;
  constexpr int NC = S::NC, TPC = S::TPC;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ long long s_prefix[kBatchMaxInstances + 1];
  for (int i = threadIdx.x; i <= n; i += blockDim.x) s_prefix[i] = prefix[i];
  __syncthreads();
  constexpr bool SU = EclStaging<D, N, T, MODE, A>::STAGE_U;
  const long long bufe = ecl_buffer_elems<D, N, T>(cpb);
  T* const s_in0 = reinterpret_cast<T*>(smem_raw);
  T* const s_in1 = s_in0 + bufe;
  T* const s_o = s_in0 + 2 * bufe;
  T* const s_u0 = s_in0 + 3 * bufe;
  T* const s_u1 = s_in0 + 4 * bufe;
  const int tid = threadIdx.x, nthr = blockDim.x;
  const int lc = tid / TPC, tl = tid % TPC;
  const long long total = s_prefix[n];
  // instance of global block gb: the last i with prefix[i] <= gb
  auto locate = [&](long long gb) -> int {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) / 2;
      if (s_prefix[mid] <= gb) lo = mid;
      else hi = mid - 1;
    }
    return lo;
  };
  auto stage = [&](T* dst, T* dstu, int inst, long long lb) {
    const EclParams<T>& P = params[inst];
    const long long c0 = lb * cpb;
    const long long ncell = (P.n_cells - c0) < cpb ? (P.n_cells - c0) : cpb;
    stage_cells<D, N, T>(dst, P.tin + c0 * NC, ncell, tid, nthr);
    if constexpr (SU) {
      stage_cells<D, N, T>(dstu, P.uin + c0 * NC, ncell, tid, nthr);
    } else if constexpr ((MODE == kStageMid || MODE == kStageLast) && (NC * sizeof(T)) % 16 == 0) {
      // the block's RK solution into L2 one block ahead (as in ecl_kernel)
      const long long bytes = ncell * NC * (long long)sizeof(T);
      const long long off = (long long)tid * 16384;
      if (off < bytes)
        prefetch_l2_bulk(reinterpret_cast<const char*>(P.uin + c0 * NC) + off,
                         unsigned(bytes - off < 16384 ? bytes - off : 16384));
    }
  };
  long long b = blockIdx.x;
  int inst = 0;
  if (b < total) {
    inst = locate(b);
    stage(s_in0, s_u0, inst, b - s_prefix[inst]);
  }
  cp_async_commit();
  bool odd = false;
  for (; b < total; b += gridDim.x) {
    T* const cur = odd ? s_in1 : s_in0;
    T* const nxt = odd ? s_in0 : s_in1;
    T* const curu = odd ? s_u1 : s_u0;
    T* const nxtu = odd ? s_u0 : s_u1;
    const long long nb = b + gridDim.x;
    int ninst = inst;
    if (nb < total) {
      ninst = locate(nb);
      stage(nxt, nxtu, ninst, nb - s_prefix[ninst]);
    }
    cp_async_commit();
    cp_async_wait<1>();
    __syncthreads();
    if constexpr (std::is_same_v<A, f32x2>) {
      // FP32x2: the block converts the staged input to double-word FP32 in
      // place as its first direction reads it (as in ecl_kernel)
      ecl_block_x2<D, N, MODE, false, true>(params[inst], (b - s_prefix[inst]) * cpb, lc, tl, cur, s_o,
                                            SU ? curu : nullptr);
    } else {
      ecl_block<D, N, T, MODE, false>(params[inst], (b - s_prefix[inst]) * cpb, lc, tl, cur, s_o, SU ? curu : nullptr);
    }
    __syncthreads();
    odd = !odd;
    inst = ninst;
  }
  cp_async_wait<0>();
}

template <int D, int N, typename T, typename A = T>
cudaError_t launch_batch(const BatchLaunch<T>& L, int mode, cudaStream_t stream) {
  using S = EclShape<D, N, T>;
  if constexpr (!S::SUPPORTED) {
    return cudaErrorNotSupported;
  } else {
    if (L.n < 1 || L.n > kBatchMaxInstances) return cudaErrorInvalidValue;
    if (mode < kApply || mode > kStageLast) return cudaErrorInvalidValue;
    int cpb = (L.cpb < 1 || L.cpb > S::CPB) ? ecl_default_cpb<D, N, T>() : L.cpb;
    const int nbuf = mode == kStageMid ? EclStaging<D, N, T, kStageMid, A>::NBUF
                     : mode == kStageLast ? EclStaging<D, N, T, kStageLast, A>::NBUF : 3;
    // (the static prefix table takes 2 KiB beside the dynamic tiles); the
    // block offsets were made for this cpb, so it must fit as it is
    if (size_t(nbuf * ecl_buffer_elems<D, N, T>(cpb)) * sizeof(T) > 218 * 1024) return cudaErrorInvalidValue;
    const int threads = S::TPC * cpb;
    const size_t smem = size_t(nbuf * ecl_buffer_elems<D, N, T>(cpb)) * sizeof(T);
    static bool attr_done[4] = {false, false, false, false};
    static int sms = 0;
    auto go = [&](auto kern) -> cudaError_t {
      if (!attr_done[mode]) {
        int cmax = S::CPB;
        while (cmax > 1 && size_t(nbuf * ecl_buffer_elems<D, N, T>(cmax)) * sizeof(T) > 218 * 1024) --cmax;
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             int(nbuf * ecl_buffer_elems<D, N, T>(cmax) * sizeof(T)));
        if (e != cudaSuccess) return e;
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        attr_done[mode] = true;
      }
      int per_sm = L.ctas_per_sm;
      if (per_sm < 1) {
        cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem);
        if (e != cudaSuccess) return e;
        if (per_sm < 1) per_sm = 1;
      }
      const unsigned grid = unsigned((long long)sms * per_sm);
      kern<<<grid, threads, smem, stream>>>(L.params, L.prefix, L.n, cpb);
      return cudaGetLastError();
    };
    switch (mode) {
      case kApply: return go(ecl_batch_kernel<D, N, T, kApply, A>);
      case kStageFirst: return go(ecl_batch_kernel<D, N, T, kStageFirst, A>);
      case kStageMid: return go(ecl_batch_kernel<D, N, T, kStageMid, A>);
      case kStageLast: return go(ecl_batch_kernel<D, N, T, kStageLast, A>);
      default: return cudaErrorInvalidValue;
    }
  }
}

// the largest tile whose staging (five buffers in the stage modes) fits
template <int D, int N, typename T>
constexpr int batch_max_cpb() {
  int c = EclShape<D, N, T>::CPB;
  while (c > 1 && size_t(EclStaging<D, N, T, kStageMid>::NBUF * ecl_buffer_elems<D, N, T>(c)) * sizeof(T) > 218 * 1024)
    --c;
  return c;
}

template <int D, int N>
BatchLaunchers make_batch_launchers() {
  constexpr int m64 = batch_max_cpb<D, N, double>(), m32 = batch_max_cpb<D, N, float>();
  constexpr int d64 = ecl_default_cpb<D, N, double>(), d32 = ecl_default_cpb<D, N, float>();
  return BatchLaunchers{&launch_batch<D, N, double>, &launch_batch<D, N, float>, m64, m32, d64 < m64 ? d64 : m64,
                        d32 < m32 ? d32 : m32, EclShape<D, N, double>::SUPPORTED && EclShape<D, N, float>::SUPPORTED,
                        &launch_batch<D, N, double, f32x2>};
}

}  // namespace hd
