// hd_ecl6.cu -- host side of the pipelined degree-3 FP32 kernel (6D cells,
// or 4D x0-rows of 16 cells): tensor-map encoding (through the driver entry
// point, no -lcuda) and launch.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>

#include "hd_ecl6.cuh"

namespace hd {

namespace {

using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  });
  return fn;
}

// rank-3 view [outer][4][inner] of the vector with a box of one face (index 1 fixed)
bool encode_trace(EncodeTiledFn enc, CUtensorMap* m, const float* base, long long n, cuuint64_t inner,
                  cuuint32_t box_outer) {
  cuuint64_t dims[3] = {inner, 4, cuuint64_t(n) / (inner * 4)};
  cuuint64_t strides[2] = {inner * 4, inner * 16};
  cuuint32_t box[3] = {cuuint32_t(inner), 1, box_outer};
  cuuint32_t es[3] = {1, 1, 1};
  return enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(base), dims, strides, box, es,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_NONE,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace

// T (and U) tiles of one cell: [n/32][32] floats, box [128][32], 128-byte swizzle
static bool encode_tile(EncodeTiledFn enc, CUtensorMap* m, const float* base, long long n) {
  cuuint64_t dims[2] = {32, cuuint64_t(n) / 32};
  cuuint64_t strides[1] = {128};
  cuuint32_t box[2] = {32, 128};
  cuuint32_t es[2] = {1, 1};
  return enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(base), dims, strides, box, es,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

cudaError_t encode_ecl6_maps(const float* tin, const float* uin, long long n, Ecl6Maps* m) {
  EncodeTiledFn enc = encode_fn();
  if (!enc) return cudaErrorNotSupported;
  std::memset(m, 0, sizeof(*m));
  if (!encode_tile(enc, &m->tcell, tin, n) || !encode_tile(enc, &m->ucell, uin ? uin : tin, n))
    return cudaErrorInvalidValue;
  // faces: view [n/(4S)][4][S] with S the node stride of the direction; one face of
  // one cell is the box [1024/S][1][S]
  if (!encode_trace(enc, &m->tx2, tin, n, 16, 64) || !encode_trace(enc, &m->tv0, tin, n, 64, 16) ||
      !encode_trace(enc, &m->tv1, tin, n, 256, 4))
    return cudaErrorInvalidValue;
  return cudaSuccess;
}

bool ecl6_eligible(const EclParams<float>& P) {
  if (!((P.D == 6 && P.dim_x == 3) || (P.D == 4 && P.dim_x == 2))) return false;
  for (int d = 0; d < P.D; ++d)
    if (!P.periodic[d]) return false;
  const long long nc = P.D == 6 ? 4096LL : 256LL;
  if (P.n_cells * nc > (1LL << 36)) return false;  // TMA row coordinate range
  if (P.D == 4) {
    // units are whole x0-rows of 16 cells; not for parts (no ghost faces)
    long long total = 1;
    for (int d = 0; d < 4; ++d) total *= P.cells[d];
    if (P.cells[0] != 16 || P.n_cells != total) return false;
  }
  return true;
}

cudaError_t launch_ecl6(const EclParams<float>& P, int* err, int* ticket, int mode, cudaStream_t stream,
                        unsigned wait_limit, int skip_issue) {
  Ecl6Params E;
  E.p = P;
  E.wait_limit = wait_limit ? wait_limit : E6_WAIT_LIMIT;
  E.skip_issue = skip_issue;
  const bool d4 = P.D == 4;
  if (d4) {
    // units of 16 cells (one x0-row each), claimed one at a time
    E.row_len = 1;
    E.row_lo = int(P.c_lo / 16);
    E.row_hi = int(P.c_hi / 16);
    E.row0 = int(P.gid0 / 16);
    E.lay0 = 0;
    E.lay1 = 1 << 30;
    E.n_units = P.n_cells / 16;
  } else {
    E.row_len = P.cells[0];
    // parts hold whole layers of v2, so every boundary below falls on a row
    E.row_lo = int(P.c_lo / P.cells[0]);
    E.row_hi = int(P.c_hi / P.cells[0]);
    E.row0 = int(P.gid0 / P.cells[0]);
    E.lay0 = int(P.gid0 / P.layer);
    E.lay1 = int((P.gid0 + P.n_cells) / P.layer);
    E.n_units = P.n_cells;
  }
  E.err = err;
  E.ticket = ticket;
  const int n_rows = E.row_hi - E.row_lo;
  if (n_rows <= 0) return cudaSuccess;  // an empty cell range launches nothing
  Ecl6Maps maps;
  cudaError_t e = encode_ecl6_maps(P.tin, P.uin, P.n_cells * (d4 ? 256LL : 4096LL), &maps);
  if (e != cudaSuccess) return e;
  static bool attr_done[8] = {false, false, false, false, false, false, false, false};
  const int ki = mode + (d4 ? 4 : 0);
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  int grid = 2 * sms;
  if (grid > n_rows) grid = n_rows;
  auto go = [&](auto kern) -> cudaError_t {
    if (!attr_done[ki]) {
      cudaError_t ee = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, E6_SMEM);
      if (ee != cudaSuccess) return ee;
      attr_done[ki] = true;
    }
    // the row tickets start at 0 for every launch (stream-ordered, also inside a captured graph)
    cudaError_t ee = cudaMemsetAsync(ticket, 0, sizeof(int), stream);
    if (ee != cudaSuccess) return ee;
    kern<<<grid, E6_THREADS, E6_SMEM, stream>>>(E, maps);
    return cudaGetLastError();
  };
  if (d4) {
    switch (mode) {
      case kApply: return go(ecl6_kernel<kApply, 4>);
      case kStageFirst: return go(ecl6_kernel<kStageFirst, 4>);
      case kStageMid: return go(ecl6_kernel<kStageMid, 4>);
      case kStageLast: return go(ecl6_kernel<kStageLast, 4>);
      default: return cudaErrorInvalidValue;
    }
  }
  switch (mode) {
    case kApply: return go(ecl6_kernel<kApply>);
    case kStageFirst: return go(ecl6_kernel<kStageFirst>);
    case kStageMid: return go(ecl6_kernel<kStageMid>);
    case kStageLast: return go(ecl6_kernel<kStageLast>);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace hd
