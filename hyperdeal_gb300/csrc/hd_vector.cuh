// hd_vector.cuh -- declarations of the vector kernels (hd_vector.cu).
#pragma once

#include <cuda_runtime.h>

#include "hd_ecl.cuh"

namespace hd {

constexpr int kNormBlocks = 152 * 4;  // fixed grid -> deterministic reduction order

// geometry of a nodal DG vector on the Cartesian phase-space mesh
struct VecGeom {
  int D, dim_x, N, NC;
  long long ncx, n_dofs;
  long long gid0;  // global id of the vector's first cell (a part of a partitioned operator)
  int cells[kMaxDim];
  double lo[kMaxDim], h[kMaxDim];
  double gl[kMaxN], glw[kMaxN];
  int gauss;                                // Gauss quadrature: norms at the Gauss points
  double gq[kMaxN], gw[kMaxN], S[kMaxN * kMaxN];  // points, weights, nodal -> Gauss-point values
};

// `table` holds sum_d cells_d * (k+1) doubles (the factors of a product function)
cudaError_t launch_interpolate(const VecGeom& g, const DevFunction& f, double t, void* dst, int is_f32,
                               double* table, cudaStream_t s);
cudaError_t launch_norm_error(const VecGeom& g, const DevFunction& f, double t, const void* src, int is_f32,
                              double* table, double* partials, double* out, cudaStream_t s);
// n_faces chunks of face_bytes from src + i * stride_bytes to dst + i * face_bytes
cudaError_t launch_pack_faces(const void* src, long long stride_bytes, long long face_bytes, long long n_faces,
                              void* dst, cudaStream_t s);
cudaError_t launch_lsrk_update(int is_f32, long long n, double bi, double ai, const void* K, void* sol,
                               void* next_T, cudaStream_t s);

}  // namespace hd
