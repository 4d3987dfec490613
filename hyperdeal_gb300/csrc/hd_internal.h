// hd_internal.h -- library-internal definitions shared by the C ABI
// translation units (hd_capi.cu, hd_batch.cu).
#pragma once

#include <cuda_runtime.h>

#include "../../include/hyperdeal_gb300.h"
#include "hd_ecl.cuh"
#include "hd_gauss.cuh"
#include "hd_vector.cuh"

// per-direction line operator in FP64 (see derive_line_op in hd_capi.cu)
struct LineOpD {
  double M[hd::kMaxN * hd::kMaxN];
  double cin;
  int in_node, nb_node, step, active;
};

// one-dimensional tables of the Gauss path: Gauss points/weights, the
// derivative matrix of their Lagrange basis, its end values l0 = l(0),
// l1 = l(1), and S[q][j] = L_j(xi_q) (Gauss-Lobatto basis at Gauss points)
struct GaussTables {
  double x[hd::kMaxN], w[hd::kMaxN], D[hd::kMaxN * hd::kMaxN];
  double l0[hd::kMaxN], l1[hd::kMaxN];
  double S[hd::kMaxN * hd::kMaxN], Si[hd::kMaxN * hd::kMaxN];
};

struct hd_adv {
  hd_adv_desc desc;
  int D, N, NC, dtype;
  long long n_cells, n_dofs, ncx;
  double lo[HD_MAX_DIM], hi[HD_MAX_DIM], h[HD_MAX_DIM];
  int cells[HD_MAX_DIM], periodic[HD_MAX_DIM];
  double gl[hd::kMaxN], glw[hd::kMaxN], Dm[hd::kMaxN * hd::kMaxN];
  LineOpD ops[HD_MAX_DIM];
  hd::EclLaunchers launchers;
  hd::EclParams<double> p64;
  hd::EclParams<float> p32;
  hd::VecGeom geom;
  double* d_partials;  // norm reduction scratch (2*kNormBlocks + 2 doubles) + error flag
  int* d_err;          // device error flag of the pipelined kernel (inside d_partials)
  int* d_tickets;      // kTicketSlots row counters of the pipelined kernel (inside d_partials)
  unsigned ticket_slot;  // next counter: consecutive launches use different ones, so that
                         // launches of one operator on different streams may overlap
  double* d_table;     // factor table of product functions (sum_d cells_d * (k+1) doubles)
  int device;
  int variant;         // HD_KERNEL_AUTO / _GENERIC / _PIPELINED
  int arith;           // HD_ARITH_NATIVE / _FP32X2 (FP64 storage)
  int gauss;           // 1: Gauss quadrature (non-collocation) path
  hd_part_layout part; // v-slab part of a partitioned operator (n_parts = 1: the whole mesh)
  int n_parts, part_index;
  unsigned wait_limit;  // pipelined kernel: try_wait rounds of its bounded waits (0: default)
  int skip_issue;       // pipelined kernel test hook (hd_adv_set_wait_test; -1: off)
  GaussTables gt;
  hd::GaussExtra<double> g64;
  hd::GaussExtra<float> g32;
  hd::GaussLaunchers glaunch;
};

struct hd_lsrk {
  char type[8];
  int ns;
  double ai[16], bi[16], ci[16];
};

namespace hd {
constexpr int kTicketSlots = 64;
// one stage launch of an operator (the kernel hd_adv_kernel reports)
int adv_launch(hd_adv* op, int mode, const void* tin, const void* uin, void* uout, void* tout, double fb, double fa,
               double time, cudaStream_t s);
}  // namespace hd
