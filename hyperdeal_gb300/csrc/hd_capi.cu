// hd_capi.cu -- C ABI of the GB300 advection path (include/hyperdeal_gb300.h).
//
// Host side: validates the descriptor, builds the 1D tables (Gauss-Lobatto
// nodes/weights and the collocation derivative matrix), derives the
// per-direction line operators from the reference's operator formulas, picks
// the (D, k, dtype) kernel and runs the LSRK stage sequence.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>
#include <algorithm>

#include "../../include/hyperdeal_gb300.h"
#include "hd_ecl.cuh"
#include "hd_internal.h"
#include "hd_vector.cuh"
#include "hd_rules.h"

namespace {

using hd::rules::gauss_lobatto;
using hd::rules::gauss_rule;
using hd::rules::lagrange_derivative_matrix;
using hd::rules::lagrange_value;

thread_local std::string g_last_error;

int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

int cuda_fail(cudaError_t e, const char* what) {
  return fail(HD_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

// inverse of an n x n matrix by Gauss-Jordan with partial pivoting
bool invert(int n, const double* A, double* Ai) {
  double a[hd::kMaxN][2 * hd::kMaxN];
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < 2 * n; ++j) a[i][j] = j < n ? A[i * n + j] : (j - n == i ? 1.0 : 0.0);
  for (int c = 0; c < n; ++c) {
    int piv = c;
    for (int r = c + 1; r < n; ++r)
      if (std::fabs(a[r][c]) > std::fabs(a[piv][c])) piv = r;
    if (std::fabs(a[piv][c]) < 1e-300) return false;
    for (int j = 0; j < 2 * n; ++j) std::swap(a[c][j], a[piv][j]);
    const double inv = 1.0 / a[c][c];
    for (int j = 0; j < 2 * n; ++j) a[c][j] *= inv;
    for (int r = 0; r < n; ++r) {
      if (r == c) continue;
      const double f = a[r][c];
      for (int j = 0; j < 2 * n; ++j) a[r][j] -= f * a[c][j];
    }
  }
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) Ai[i * n + j] = a[i][n + j];
  return true;
}

// The same line operator in the Lagrange basis of the Gauss points (weights
// w, derivative matrix D), whose face values are the interpolations
// l0 . v, l1 . v and whose test functions take the values l0[i], l1[i] on
// the faces (advection_operation.h:294-316, :426-449, :459-482 with
// Gauss quadrature); the result is divided by the diagonal Gauss mass.
void line_operator_gauss(int n, const double* w, const double* D, const double* l0, const double* l1, double a,
                         double h, double s, const double* u, double uL, double uR, double* out) {
  for (int i = 0; i < n; ++i) {
    double vol = 0.0, skw = 0.0;
    for (int q = 0; q < n; ++q) vol += D[q * n + i] * w[q] * u[q];
    for (int j = 0; j < n; ++j) skw += D[i * n + j] * u[j];
    out[i] = (1.0 - s) * (a / h) * vol / w[i] - s * (a / h) * skw;
  }
  double um0 = 0.0, um1 = 0.0;
  for (int j = 0; j < n; ++j) {
    um0 += l0[j] * u[j];
    um1 += l1[j] * u[j];
  }
  {
    const double an = -a;
    const double flux = 0.5 * ((um0 + uL) * an + std::fabs(an) * (um0 - uL));
    for (int i = 0; i < n; ++i) out[i] += -(flux - s * um0 * an) * l0[i] / (h * w[i]);
  }
  {
    const double an = a;
    const double flux = 0.5 * ((um1 + uR) * an + std::fabs(an) * (um1 - uR));
    for (int i = 0; i < n; ++i) out[i] += -(flux - s * um1 * an) * l1[i] / (h * w[i]);
  }
}

// M (Gauss basis), the inflow vector cv and the own inflow-face vector le
bool derive_line_op_gauss(int n, const GaussTables& T, double a, double h, double s, LineOpD* op, double* cv,
                          double* le) {
  double u[hd::kMaxN], out[hd::kMaxN];
  bool any = false;
  for (int q = 0; q < n; ++q) {
    for (int j = 0; j < n; ++j) u[j] = (j == q);
    line_operator_gauss(n, T.w, T.D, T.l0, T.l1, a, h, s, u, 0.0, 0.0, out);
    for (int i = 0; i < n; ++i) {
      op->M[i * n + q] = out[i];
      any = any || out[i] != 0.0;
    }
  }
  for (int j = 0; j < n; ++j) u[j] = 0.0;
  double cL[hd::kMaxN], cR[hd::kMaxN];
  line_operator_gauss(n, T.w, T.D, T.l0, T.l1, a, h, s, u, 1.0, 0.0, cL);
  line_operator_gauss(n, T.w, T.D, T.l0, T.l1, a, h, s, u, 0.0, 1.0, cR);
  bool anyL = false, anyR = false;
  for (int i = 0; i < n; ++i) {
    anyL = anyL || cL[i] != 0.0;
    anyR = anyR || cR[i] != 0.0;
  }
  if (anyL && anyR) return false;  // not a one-sided upwind flux
  if (anyR) {
    op->step = +1; op->in_node = n - 1; op->nb_node = 0;
    for (int i = 0; i < n; ++i) { cv[i] = cR[i]; le[i] = T.l1[i]; }
  } else {
    op->step = -1; op->in_node = 0; op->nb_node = n - 1;
    for (int i = 0; i < n; ++i) { cv[i] = cL[i]; le[i] = T.l0[i]; }
  }
  op->cin = 0.0;
  op->active = any || anyL || anyR;
  return true;
}

// The reference's operator restricted to one line of n nodes along direction d
// of a Cartesian cell (constant velocity a, width h, skew factor s), with the
// exterior values uL / uR of the left / right faces; the JxW factors of the
// other directions cancel between integration and inverse mass:
//   volume  (1-s) (a/h) (1/w_i) sum_q D[q][i] w_q u_q  -  s (a/h) sum_j D[i][j] u_j
//           (advection_operation.h:325-404, fe_evaluation_cell.h:278-348)
//   faces   -(flux - s u- a.n) / (h w_i) at i = 0 (n = -e_d) and i = n-1 (n = +e_d),
//           flux = 0.5 ((u- + u+) a.n + |a.n| (u- - u+))  (alpha = 1)
//           (advection_operation.h:459-482, fe_evaluation_face.h:381-399)
//   inverse mass: division by JxW_i (fe_evaluation_cell_inverse.h:131-133)
void line_operator(int n, const double* w, const double* D, double a, double h, double s, const double* u,
                   double uL, double uR, double* out) {
  for (int i = 0; i < n; ++i) {
    double vol = 0.0, skw = 0.0;
    for (int q = 0; q < n; ++q) vol += D[q * n + i] * w[q] * u[q];
    for (int j = 0; j < n; ++j) skw += D[i * n + j] * u[j];
    out[i] = (1.0 - s) * (a / h) * vol / w[i] - s * (a / h) * skw;
  }
  {
    const double an = -a, um = u[0];
    const double flux = 0.5 * ((um + uL) * an + std::fabs(an) * (um - uL));
    out[0] += -(flux - s * um * an) / (h * w[0]);
  }
  {
    const double an = a, um = u[n - 1];
    const double flux = 0.5 * ((um + uR) * an + std::fabs(an) * (um - uR));
    out[n - 1] += -(flux - s * um * an) / (h * w[n - 1]);
  }
}



// linear operator coefficients by probing line_operator with unit inputs
bool derive_line_op(int n, const double* w, const double* D, double a, double h, double s, LineOpD* op) {
  double u[hd::kMaxN], out[hd::kMaxN];
  bool any = false;
  for (int q = 0; q < n; ++q) {
    for (int j = 0; j < n; ++j) u[j] = (j == q);
    line_operator(n, w, D, a, h, s, u, 0.0, 0.0, out);
    for (int i = 0; i < n; ++i) {
      op->M[i * n + q] = out[i];
      any = any || out[i] != 0.0;
    }
  }
  for (int j = 0; j < n; ++j) u[j] = 0.0;
  double cL[hd::kMaxN], cR[hd::kMaxN];
  line_operator(n, w, D, a, h, s, u, 1.0, 0.0, cL);
  line_operator(n, w, D, a, h, s, u, 0.0, 1.0, cR);
  for (int i = 1; i < n; ++i)
    if (cL[i] != 0.0) return false;
  for (int i = 0; i < n - 1; ++i)
    if (cR[i] != 0.0) return false;
  if (cL[0] != 0.0 && cR[n - 1] != 0.0) return false;  // not a one-sided upwind flux
  if (cR[n - 1] != 0.0) {
    op->step = +1; op->in_node = n - 1; op->nb_node = 0; op->cin = cR[n - 1];
  } else {
    op->step = -1; op->in_node = 0; op->nb_node = n - 1; op->cin = cL[0];
  }
  op->active = any || op->cin != 0.0;
  return true;
}

hd::DevFunction to_dev(const hd_function& f) {
  hd::DevFunction d;
  std::memset(&d, 0, sizeof(d));
  d.kind = f.kind;
  d.amp = f.amp;
  for (int i = 0; i < HD_MAX_DIM; ++i) {
    d.omega[i] = f.omega[i];
    d.speed[i] = f.speed[i];
    d.phase[i] = f.phase[i];
    d.cosine[i] = f.cosine[i];
  }
  return d;
}

}  // namespace

namespace hd {
// lets the other translation units report through hd_last_error()
void set_last_error(const char* msg) { g_last_error = msg; }
}  // namespace hd



namespace {

template <typename T>
void fill_params(const hd_adv* op, hd::EclParams<T>* P) {
  std::memset(P, 0, sizeof(*P));
  P->n_cells = op->n_cells;
  P->D = op->D;
  P->dim_x = op->desc.dim_x;
  long long st = 1;
  for (int d = 0; d < op->D; ++d) {
    P->cells[d] = op->cells[d];
    P->cstride[d] = st;
    st *= op->cells[d];
    P->periodic[d] = op->periodic[d];
    P->lo[d] = op->lo[d];
    P->h[d] = op->h[d];
    const LineOpD& L = op->ops[d];
    for (int i = 0; i < op->N * op->N; ++i) P->op[d].M[i] = T(L.M[i]);
    P->op[d].cin = T(L.cin);
    P->op[d].c0 = L.in_node == 0 ? T(L.cin) : T(0);
    P->op[d].cl = L.in_node == op->N - 1 ? T(L.cin) : T(0);
    P->op[d].in_node = L.in_node;
    P->op[d].nb_node = L.nb_node;
    P->op[d].step = L.step;
    P->op[d].active = L.active;
    if constexpr (sizeof(T) == 8) {
      hd::LineOp<hd::f32x2>& X = P->opx[d];
      for (int i = 0; i < op->N * op->N; ++i) X.M[i] = hd::x2_split_host(L.M[i]);
      X.cin = hd::x2_split_host(L.cin);
      X.c0 = L.in_node == 0 ? X.cin : hd::f32x2{0.f, 0.f};
      X.cl = L.in_node == op->N - 1 ? X.cin : hd::f32x2{0.f, 0.f};
      X.in_node = L.in_node;
      X.nb_node = L.nb_node;
      X.step = L.step;
      X.active = L.active;
    }
  }
  if (op->D < hd::kMaxDim) P->cstride[op->D] = st;
  long long nx = 1;
  for (int d = 0; d < op->D; ++d) {
    P->dcell[d] = hd::make_divu64((unsigned long long)op->cells[d]);
    if (d < op->desc.dim_x) nx *= op->cells[d];
  }
  P->dxcells = hd::make_divu64((unsigned long long)nx);
  P->gid0 = op->part.first_cell;
  P->c_lo = 0;
  P->c_hi = op->n_cells;
  P->layer = op->part.layer_cells;
  P->ghost = nullptr;
  P->err = nullptr;
  for (int i = 0; i < op->N; ++i) P->gl[i] = op->gl[i];
  P->bc_inhom = op->desc.bc_kind == HD_BC_FUNCTION;
  P->bc = to_dev(op->desc.bc);
}

hd::EclLaunchers get_launchers(int D, int N) {
  switch (D) {
    case 2: return hd::ecl_launchers_d2(N);
    case 3: return hd::ecl_launchers_d3(N);
    case 4: return hd::ecl_launchers_d4(N);
    case 5: return hd::ecl_launchers_d5(N);
    case 6: return hd::ecl_launchers_d6(N);
    default: return hd::EclLaunchers{nullptr, nullptr, 0, 0, 0, 0, 0, 0, false, false};
  }
}

// kernel that runs for this operator (HD_KERNEL_GENERIC or HD_KERNEL_PIPELINED)
int selected_kernel(const hd_adv* op) {
  const bool pipelined_ok = !op->gauss && op->dtype == HD_F32 && op->N == 4 && hd::ecl6_eligible(op->p32);
  if (op->variant == HD_KERNEL_GENERIC) return HD_KERNEL_GENERIC;
  return pipelined_ok ? HD_KERNEL_PIPELINED : HD_KERNEL_GENERIC;
}

// local cells [lo, hi) of a cell subset (enum hd_cells); the boundary cells of
// a part are one layer at one end of its range, so both subsets are ranges
void cell_range(const hd_adv* op, int which, long long* lo, long long* hi) {
  const hd_part_layout& L = op->part;
  *lo = 0;
  *hi = op->n_cells;
  if (which == HD_CELLS_BOUNDARY) {
    *lo = L.boundary_first;
    *hi = L.boundary_first + L.boundary_cells;
  } else if (which == HD_CELLS_INTERIOR && L.boundary_cells > 0) {
    if (L.boundary_first == 0) *lo = L.boundary_cells;
    else *hi = L.boundary_first;
  }
}

template <typename T>
void set_launch(const hd_adv* op, hd::EclParams<T>* P, const void* tin, const void* uin, void* uout, void* tout,
                double fb, double fa, double time, long long c_lo, long long c_hi) {
  P->tin = (const T*)tin; P->uin = (const T*)uin; P->uout = (T*)uout; P->tout = (T*)tout;
  P->fb = T(fb); P->fa = T(fa); P->time = time;
  P->c_lo = c_lo; P->c_hi = c_hi;
  // the ghost region follows the part's cells in the operator input
  P->ghost = op->part.ghost_values > 0 ? (const T*)tin + op->n_dofs : nullptr;
}

int launch(hd_adv* op, int mode, const void* tin, const void* uin, void* uout, void* tout, double fb,
           double fa, double time, cudaStream_t s, int which = HD_CELLS_ALL) {
  cudaError_t e;
  long long c_lo = 0, c_hi = 0;
  cell_range(op, which, &c_lo, &c_hi);
  if (c_hi <= c_lo) return HD_OK;  // an empty subset: nothing to launch
  if (op->gauss) {
    if (op->dtype == HD_F64) {
      hd::EclParams<double> P = op->p64;
      P.tin = (const double*)tin; P.uin = (const double*)uin; P.uout = (double*)uout; P.tout = (double*)tout;
      P.fb = fb; P.fa = fa; P.time = time;
      e = op->glaunch.f64(P, op->g64, mode, s);
    } else {
      hd::EclParams<float> P = op->p32;
      P.tin = (const float*)tin; P.uin = (const float*)uin; P.uout = (float*)uout; P.tout = (float*)tout;
      P.fb = float(fb); P.fa = float(fa); P.time = time;
      e = op->glaunch.f32(P, op->g32, mode, s);
    }
  } else if (selected_kernel(op) == HD_KERNEL_PIPELINED) {
    hd::EclParams<float> P = op->p32;
    set_launch(op, &P, tin, uin, uout, tout, fb, fa, time, c_lo, c_hi);
    int* ticket = op->d_tickets + (op->ticket_slot++ % hd::kTicketSlots);
    e = hd::launch_ecl6(P, op->d_err, ticket, mode, s, op->wait_limit, op->skip_issue);
  } else if (op->dtype == HD_F64) {
    hd::EclParams<double> P = op->p64;
    set_launch(op, &P, tin, uin, uout, tout, fb, fa, time, c_lo, c_hi);
    e = (op->arith == HD_ARITH_FP32X2 ? op->launchers.f64x : op->launchers.f64)(P, mode, s);
  } else {
    hd::EclParams<float> P = op->p32;
    set_launch(op, &P, tin, uin, uout, tout, fb, fa, time, c_lo, c_hi);
    e = op->launchers.f32(P, mode, s);
  }
  if (e != cudaSuccess) return cuda_fail(e, "ECL kernel launch");
  return HD_OK;
}

bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

// Part `part` of n_parts v-slabs: whole layers of the last direction (D-1).
// `last` is the line operator of that direction: only its upwind side is read,
// so a part receives the faces of one layer of its upwind part and sends one
// layer to its downwind part (with wraps on a periodic direction).
int compute_layout(int D, int N, const int* cells, const LineOpD& last, int periodic_last, int n_parts, int part,
                   hd_part_layout* L) {
  const int lc = cells[D - 1];
  if (n_parts < 1 || n_parts > lc || part < 0 || part >= n_parts)
    return fail(HD_ERR_INVALID, "partition: need 1 <= n_parts <= %d (cells in the last direction), 0 <= part < "
                                "n_parts (got %d, %d)", lc, n_parts, part);
  long long ncells = 1;
  for (int d = 0; d < D; ++d) ncells *= cells[d];
  const long long layer = ncells / lc;
  const long long l0 = (long long)part * lc / n_parts, l1 = (long long)(part + 1) * lc / n_parts;
  std::memset(L, 0, sizeof(*L));
  L->first_cell = l0 * layer;
  L->n_cells = (l1 - l0) * layer;
  L->layer_cells = layer;
  L->face_values = hd::ipow(N, D - 1);
  L->recv_from = -1;
  L->send_to = -1;
  if (n_parts > 1 && last.active) {
    int up, down;
    if (last.step < 0) {  // upwind neighbour at the lower layer
      up = part - 1;
      down = part + 1;
      L->boundary_first = 0;
      L->send_first_cell = L->n_cells - layer;
    } else {
      up = part + 1;
      down = part - 1;
      L->boundary_first = L->n_cells - layer;
      L->send_first_cell = 0;
    }
    if (up < 0 || up >= n_parts) up = periodic_last ? (up + n_parts) % n_parts : -1;
    if (down < 0 || down >= n_parts) down = periodic_last ? (down + n_parts) % n_parts : -1;
    L->recv_from = up;
    L->send_to = down;
    L->send_slab = last.nb_node;
    if (up >= 0) {
      L->ghost_values = layer * L->face_values;
      L->boundary_cells = layer;
    }
  }
  return HD_OK;
}

}  // namespace

namespace hd {
int adv_launch(hd_adv* op, int mode, const void* tin, const void* uin, void* uout, void* tout, double fb, double fa,
               double time, cudaStream_t s) {
  return launch(op, mode, tin, uin, uout, tout, fb, fa, time, s);
}
}  // namespace hd

extern "C" {

int hd_last_error(char* buf, size_t len) {
  const int n = int(g_last_error.size());
  if (buf && len) {
    std::strncpy(buf, g_last_error.c_str(), len - 1);
    buf[len - 1] = 0;
  }
  return n;
}

const char* hd_version(void) { return "hyperdeal_gb300 0.1 (sm_103a)"; }

static int create_impl(const hd_adv_desc* desc, int n_parts, int part, bool layout_only, hd_adv** out,
                       hd_part_layout* layout_out) {
  try {
    if (!desc || (!out && !layout_out)) return fail(HD_ERR_INVALID, "hd_adv_create: null argument");
    if (out) *out = nullptr;
    const hd_adv_desc& d = *desc;
    if (d.dim_x < 1 || d.dim_x > 3 || d.dim_v < 1 || d.dim_v > 3)
      return fail(HD_ERR_INVALID, "dim_x and dim_v must be in 1..3 (got %d, %d)", d.dim_x, d.dim_v);
    if (d.degree < 1 || d.degree + 1 > hd::kMaxN)
      return fail(HD_ERR_UNSUPPORTED, "degree %d not built (1..%d)", d.degree, hd::kMaxN - 1);
    if (d.n_points != d.degree + 1)
      return fail(HD_ERR_UNSUPPORTED, "n_points must equal degree+1, got %d (over-integration is not built)",
                  d.n_points);
    if (d.quadrature != HD_QUAD_GAUSS_LOBATTO && d.quadrature != HD_QUAD_GAUSS)
      return fail(HD_ERR_INVALID, "unknown quadrature %d", d.quadrature);
    if (d.dtype != HD_F64 && d.dtype != HD_F32) return fail(HD_ERR_INVALID, "unknown dtype %d", d.dtype);
    if (d.bc_kind != HD_BC_HOMOGENEOUS && d.bc_kind != HD_BC_FUNCTION)
      return fail(HD_ERR_INVALID, "unknown bc_kind %d", d.bc_kind);
    if (!std::isfinite(d.skew)) return fail(HD_ERR_INVALID, "skew factor is not finite");
    if (n_parts > 1 && d.quadrature != HD_QUAD_GAUSS_LOBATTO)
      return fail(HD_ERR_UNSUPPORTED, "partitioned operators use Gauss-Lobatto collocation");
    hd_adv* op = new (std::nothrow) hd_adv;
    if (!op) return fail(HD_ERR_ALLOC, "out of host memory");
    std::memset(op, 0, sizeof(*op));
    op->desc = d;
    op->D = d.dim_x + d.dim_v;
    op->N = d.degree + 1;
    op->dtype = d.dtype;
    op->NC = hd::ipow(op->N, op->D);
    op->n_cells = 1;
    op->ncx = 1;
    for (int i = 0; i < op->D; ++i) {
      const bool isx = i < d.dim_x;
      const int c = isx ? d.cells_x[i] : d.cells_v[i - d.dim_x];
      const double lo = isx ? d.lo_x[i] : d.lo_v[i - d.dim_x];
      const double hi = isx ? d.hi_x[i] : d.hi_v[i - d.dim_x];
      if (c < 1) { delete op; return fail(HD_ERR_INVALID, "cells in direction %d must be >= 1", i); }
      if (!(hi > lo) || !std::isfinite(lo) || !std::isfinite(hi)) {
        delete op;
        return fail(HD_ERR_INVALID, "box in direction %d must have hi > lo", i);
      }
      if (!std::isfinite(d.velocity[i])) { delete op; return fail(HD_ERR_INVALID, "velocity %d not finite", i); }
      op->cells[i] = c;
      op->lo[i] = lo;
      op->hi[i] = hi;
      op->h[i] = (hi - lo) / c;
      op->periodic[i] = isx ? (d.periodic_x != 0) : (d.periodic_v != 0);
      if (op->n_cells > (1LL << 40) / c) { delete op; return fail(HD_ERR_INVALID, "mesh too large"); }
      op->n_cells *= c;
      if (isx) op->ncx *= c;
    }
    gauss_lobatto(op->N, op->gl, op->glw);
    lagrange_derivative_matrix(op->N, op->gl, op->Dm);
    op->gauss = d.quadrature == HD_QUAD_GAUSS;
    if (op->gauss) {
      GaussTables& T = op->gt;
      const int n = op->N;
      gauss_rule(n, T.x, T.w);
      lagrange_derivative_matrix(n, T.x, T.D);
      for (int i = 0; i < n; ++i) {
        T.l0[i] = lagrange_value(n, T.x, i, 0.0);
        T.l1[i] = lagrange_value(n, T.x, i, 1.0);
        for (int j = 0; j < n; ++j) T.S[i * n + j] = lagrange_value(n, op->gl, j, T.x[i]);
      }
      if (!invert(n, T.S, T.Si)) { delete op; return fail(HD_ERR_INVALID, "basis change is singular"); }
      double cv[hd::kMaxN], le[hd::kMaxN];
      for (int i = 0; i < op->D; ++i) {
        if (!derive_line_op_gauss(n, T, d.velocity[i], op->h[i], d.skew, &op->ops[i], cv, le)) {
          delete op;
          return fail(HD_ERR_UNSUPPORTED, "direction %d: flux is not one-sided upwind", i);
        }
        for (int j = 0; j < n; ++j) {
          op->g64.cv[i][j] = cv[j];
          op->g64.le[i][j] = le[j];
          op->g32.cv[i][j] = float(cv[j]);
          op->g32.le[i][j] = float(le[j]);
        }
      }
      for (int j = 0; j < n * n; ++j) {
        op->g64.S[j] = T.S[j];
        op->g64.Si[j] = T.Si[j];
        op->g32.S[j] = float(T.S[j]);
        op->g32.Si[j] = float(T.Si[j]);
      }
      for (int j = 0; j < n; ++j) op->g64.gq[j] = op->g32.gq[j] = T.x[j];
      op->glaunch = hd::gauss_launchers(op->D, op->N);
      const bool ok = d.dtype == HD_F64 ? op->glaunch.ok_f64 : op->glaunch.ok_f32;
      if (!op->glaunch.f64 || !ok) {
        delete op;
        return fail(HD_ERR_UNSUPPORTED, "no Gauss-quadrature kernel for D=%d, degree=%d, dtype=%s",
                    d.dim_x + d.dim_v, d.degree, d.dtype == HD_F64 ? "f64" : "f32");
      }
    } else {
      for (int i = 0; i < op->D; ++i)
        if (!derive_line_op(op->N, op->glw, op->Dm, d.velocity[i], op->h[i], d.skew, &op->ops[i])) {
          delete op;
          return fail(HD_ERR_UNSUPPORTED, "direction %d: flux is not one-sided upwind", i);
        }
    }
    {
      const int rc = compute_layout(op->D, op->N, op->cells, op->ops[op->D - 1], op->periodic[op->D - 1], n_parts,
                                    part, &op->part);
      if (rc) { delete op; return rc; }
      op->n_parts = n_parts;
      op->part_index = part;
      op->n_cells = op->part.n_cells;  // the cells of this part (all of them for n_parts = 1)
      op->n_dofs = op->n_cells * op->NC;
    }
    if (layout_only) {
      *layout_out = op->part;
      delete op;
      return HD_OK;
    }
    op->launchers = get_launchers(op->D, op->N);
    const bool ok = d.dtype == HD_F64 ? op->launchers.ok_f64 : op->launchers.ok_f32;
    if (!op->launchers.f64 || !ok) {
      delete op;
      return fail(HD_ERR_UNSUPPORTED, "no kernel for D=%d, degree=%d, dtype=%s (cell does not fit in shared memory)",
                  d.dim_x + d.dim_v, d.degree, d.dtype == HD_F64 ? "f64" : "f32");
    }
    fill_params(op, &op->p64);
    fill_params(op, &op->p32);
    hd::VecGeom& g = op->geom;
    std::memset(&g, 0, sizeof(g));
    g.D = op->D; g.dim_x = d.dim_x; g.N = op->N; g.NC = op->NC; g.ncx = op->ncx; g.n_dofs = op->n_dofs;
    g.gid0 = op->part.first_cell;
    for (int i = 0; i < op->D; ++i) { g.cells[i] = op->cells[i]; g.lo[i] = op->lo[i]; g.h[i] = op->h[i]; }
    for (int i = 0; i < op->N; ++i) { g.gl[i] = op->gl[i]; g.glw[i] = op->glw[i]; }
    g.gauss = op->gauss;
    if (op->gauss) {
      for (int i = 0; i < op->N; ++i) { g.gq[i] = op->gt.x[i]; g.gw[i] = op->gt.w[i]; }
      for (int i = 0; i < op->N * op->N; ++i) g.S[i] = op->gt.S[i];
    }
    cudaError_t e = cudaGetDevice(&op->device);
    if (e != cudaSuccess) { delete op; return cuda_fail(e, "cudaGetDevice"); }
    // norm partials (2 * kNormBlocks), result (2), error flag of the pipelined kernel (1),
    // the pipelined kernel's row counters (kTicketSlots ints)
    e = cudaMalloc(&op->d_partials, sizeof(double) * (2 * hd::kNormBlocks + 3 + hd::kTicketSlots / 2));
    if (e != cudaSuccess) { delete op; return cuda_fail(e, "cudaMalloc (norm scratch)"); }
    op->d_err = reinterpret_cast<int*>(op->d_partials + 2 * hd::kNormBlocks + 2);
    op->p64.err = op->d_err;  // (bounds-checked builds record violations here)
    op->p32.err = op->d_err;
    op->d_tickets = reinterpret_cast<int*>(op->d_partials + 2 * hd::kNormBlocks + 3);
    op->ticket_slot = 0;
    e = cudaMemset(op->d_err, 0, sizeof(int));
    if (e != cudaSuccess) { cudaFree(op->d_partials); delete op; return cuda_fail(e, "cudaMemset (error flag)"); }
    op->variant = HD_KERNEL_AUTO;
    op->arith = HD_ARITH_NATIVE;
    op->wait_limit = 0;
    op->skip_issue = -1;
    {
      size_t tsize = 0;
      for (int i = 0; i < op->D; ++i) tsize += size_t(op->cells[i]) * op->N;
      e = cudaMalloc(&op->d_table, sizeof(double) * tsize);
      if (e != cudaSuccess) { cudaFree(op->d_partials); delete op; return cuda_fail(e, "cudaMalloc (function table)"); }
    }
    *out = op;
    return HD_OK;
  } catch (...) {
    return fail(HD_ERR_INVALID, "hd_adv_create: unexpected exception");
  }
}

int hd_adv_create(const hd_adv_desc* desc, hd_adv** out) {
  if (!out) return fail(HD_ERR_INVALID, "hd_adv_create: null argument");
  return create_impl(desc, 1, 0, false, out, nullptr);
}

int hd_adv_create_part(const hd_adv_desc* desc, int n_parts, int part, hd_adv** out) {
  if (!out) return fail(HD_ERR_INVALID, "hd_adv_create_part: null argument");
  return create_impl(desc, n_parts, part, false, out, nullptr);
}

int hd_part_layout_get(const hd_adv_desc* desc, int n_parts, int part, hd_part_layout* out) {
  if (!out) return fail(HD_ERR_INVALID, "hd_part_layout_get: null argument");
  return create_impl(desc, n_parts, part, true, nullptr, out);
}

int hd_adv_part_layout(const hd_adv* op, hd_part_layout* out) {
  if (!op || !out) return fail(HD_ERR_INVALID, "hd_adv_part_layout: null argument");
  *out = op->part;
  return HD_OK;
}

int hd_adv_pack_faces(hd_adv* op, const void* vec, void* sendbuf, void* stream) {
  if (!op || !vec || !sendbuf) return fail(HD_ERR_INVALID, "hd_adv_pack_faces: null argument");
  const hd_part_layout& L = op->part;
  if (L.send_to < 0) return HD_OK;  // nobody reads this part's faces
  const int sz = op->dtype == HD_F64 ? 8 : 4;
  const char* src = (const char*)vec + (L.send_first_cell * op->NC + (long long)L.send_slab * L.face_values) * sz;
  cudaError_t e = hd::launch_pack_faces(src, op->NC * sz, L.face_values * sz, L.layer_cells, sendbuf,
                                        (cudaStream_t)stream);
  return e == cudaSuccess ? HD_OK : cuda_fail(e, "face pack kernel");
}

int hd_adv_apply_cells(hd_adv* op, void* dst, const void* src, double time, int cells, void* stream) {
  if (!op || !dst || !src) return fail(HD_ERR_INVALID, "hd_adv_apply: null argument");
  if (cells != HD_CELLS_ALL && cells != HD_CELLS_INTERIOR && cells != HD_CELLS_BOUNDARY)
    return fail(HD_ERR_INVALID, "hd_adv_apply_cells: unknown cell subset %d", cells);
  if (!aligned16(dst) || !aligned16(src)) return fail(HD_ERR_INVALID, "hd_adv_apply: vectors must be 16-byte aligned");
  const size_t sz = op->dtype == HD_F64 ? 8 : 4;
  const size_t bytes = size_t(op->n_dofs + op->part.ghost_values) * sz;
  const char* a = (const char*)src;
  const char* b = (const char*)dst;
  if (a < b + bytes && b < a + bytes) return fail(HD_ERR_INVALID, "hd_adv_apply: dst and src overlap");
  return launch(op, hd::kApply, src, src, dst, nullptr, 0.0, 0.0, time, (cudaStream_t)stream, cells);
}

int hd_adv_destroy(hd_adv* op) {
  if (!op) return HD_OK;
  if (op->d_partials) cudaFree(op->d_partials);
  if (op->d_table) cudaFree(op->d_table);
  delete op;
  return HD_OK;
}

long long hd_adv_n_dofs(const hd_adv* op) { return op ? op->n_dofs : -1; }

int hd_adv_set_tile(hd_adv* op, int cells_per_cta, int ctas_per_sm) {
  if (!op) return fail(HD_ERR_INVALID, "hd_adv_set_tile: null handle");
  if (cells_per_cta < 0 || ctas_per_sm < 0 || ctas_per_sm > 32)
    return fail(HD_ERR_INVALID, "hd_adv_set_tile: cells_per_cta >= 0, 0 <= ctas_per_sm <= 32");
  op->p64.cpb = op->p32.cpb = cells_per_cta;
  op->p64.ctas_per_sm = op->p32.ctas_per_sm = ctas_per_sm;
  return HD_OK;
}

int hd_adv_autotune(hd_adv* op, const void* src, void* dst, int reps, int* cells_per_cta, int* ctas_per_sm,
                    double* ms, void* stream) {
  if (!op || !src || !dst || src == dst) return fail(HD_ERR_INVALID, "hd_adv_autotune: bad argument");
  if (reps < 1) reps = 3;
  cudaStream_t s = (cudaStream_t)stream;
  const bool f64 = op->desc.dtype == HD_F64;
  const int maxc = f64 ? op->launchers.cells_per_cta_f64 : op->launchers.cells_per_cta_f32;
  std::vector<int> cands;
  for (int v = maxc; v >= 1 && cands.size() < 5; v /= 2) cands.push_back(v);
  if (std::find(cands.begin(), cands.end(), 1) == cands.end()) cands.push_back(1);
  cudaEvent_t e0, e1;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)
    return fail(HD_ERR_CUDA, "hd_adv_autotune: events");
  float best = 1e30f;
  int best_c = 0, best_p = 0, rc = HD_OK;
  for (int c : cands)
    for (int per : {0, 2}) {
      op->p64.cpb = op->p32.cpb = c;
      op->p64.ctas_per_sm = op->p32.ctas_per_sm = per;
      rc = launch(op, hd::kApply, src, src, dst, nullptr, 0.0, 0.0, 0.0, s);  // warm-up
      if (rc) break;
      cudaEventRecord(e0, s);
      for (int r = 0; r < reps && !rc; ++r) rc = launch(op, hd::kApply, src, src, dst, nullptr, 0.0, 0.0, 0.0, s);
      cudaEventRecord(e1, s);
      if (rc) break;
      if (cudaEventSynchronize(e1) != cudaSuccess) { rc = fail(HD_ERR_CUDA, "hd_adv_autotune: timing"); break; }
      float t = 0.f;
      cudaEventElapsedTime(&t, e0, e1);
      if (t < best) { best = t; best_c = c; best_p = per; }
    }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  op->p64.cpb = op->p32.cpb = best_c;
  op->p64.ctas_per_sm = op->p32.ctas_per_sm = best_p;
  if (rc) return rc;
  if (cells_per_cta) *cells_per_cta = best_c;
  if (ctas_per_sm) *ctas_per_sm = best_p;
  if (ms) *ms = best / reps;
  return HD_OK;
}

int hd_adv_tile_limits(const hd_adv* op, int* max_cells_per_cta, int* threads_per_cell) {
  if (!op) return fail(HD_ERR_INVALID, "hd_adv_tile_limits: null handle");
  const bool f64 = op->desc.dtype == HD_F64;
  const int cpb = f64 ? op->launchers.cells_per_cta_f64 : op->launchers.cells_per_cta_f32;
  const int thr = f64 ? op->launchers.threads_f64 : op->launchers.threads_f32;
  if (max_cells_per_cta) *max_cells_per_cta = cpb;
  if (threads_per_cell) *threads_per_cell = cpb > 0 ? thr / cpb : 0;
  return HD_OK;
}

int hd_adv_set_kernel(hd_adv* op, int variant) {
  if (!op) return fail(HD_ERR_INVALID, "hd_adv_set_kernel: null handle");
  if (variant != HD_KERNEL_AUTO && variant != HD_KERNEL_GENERIC && variant != HD_KERNEL_PIPELINED)
    return fail(HD_ERR_INVALID, "unknown kernel variant %d", variant);
  if (variant == HD_KERNEL_PIPELINED && !(!op->gauss && op->dtype == HD_F32 && op->N == 4 && hd::ecl6_eligible(op->p32)))
    return fail(HD_ERR_UNSUPPORTED, "the pipelined kernel needs a fully periodic 3x+3v mesh, degree 3, FP32");
  op->variant = variant;
  return HD_OK;
}

int hd_adv_kernel(const hd_adv* op) { return op ? selected_kernel(op) : -1; }

int hd_adv_set_arithmetic(hd_adv* op, int arithmetic) {
  if (!op) return fail(HD_ERR_INVALID, "hd_adv_set_arithmetic: null handle");
  if (arithmetic != HD_ARITH_NATIVE && arithmetic != HD_ARITH_FP32X2)
    return fail(HD_ERR_INVALID, "unknown arithmetic %d", arithmetic);
  if (arithmetic == HD_ARITH_FP32X2 && (op->dtype != HD_F64 || op->gauss || !op->launchers.f64x))
    return fail(HD_ERR_UNSUPPORTED, "FP32x2 arithmetic needs FP64 storage and Gauss-Lobatto collocation");
  op->arith = arithmetic;
  return HD_OK;
}

int hd_adv_arithmetic(const hd_adv* op) { return op ? op->arith : -1; }

int hd_adv_set_wait_test(hd_adv* op, unsigned wait_limit, int skip_issue) {
  if (!op) return fail(HD_ERR_INVALID, "hd_adv_set_wait_test: null handle");
  if (skip_issue < -1) return fail(HD_ERR_INVALID, "hd_adv_set_wait_test: skip_issue must be >= -1");
  op->wait_limit = wait_limit;
  op->skip_issue = skip_issue;
  return HD_OK;
}

int hd_adv_device_status(hd_adv* op, int* status) {
  if (!op || !status) return fail(HD_ERR_INVALID, "hd_adv_device_status: null argument");
  int v = 0;
  cudaError_t e = cudaMemcpy(&v, op->d_err, sizeof(int), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(e, "read device error flag");
  *status = v;
  if (v) {
    e = cudaMemset(op->d_err, 0, sizeof(int));
    if (e != cudaSuccess) return cuda_fail(e, "clear device error flag");
  }
  return HD_OK;
}

double hd_adv_critical_time_step(const hd_adv* op) {
  if (!op) return -1.0;
  double vx = 0.0, vv = 0.0;
  for (int d = 0; d < op->D; ++d) {
    const double v = std::fabs(op->desc.velocity[d] / op->h[d]);
    if (d < op->desc.dim_x) vx = std::fmax(vx, v);
    else vv = std::fmax(vv, v);
  }
  return std::fmin(1.0 / vx, 1.0 / vv);
}

int hd_adv_apply(hd_adv* op, void* dst, const void* src, double time, void* stream) {
  return hd_adv_apply_cells(op, dst, src, time, HD_CELLS_ALL, stream);
}

int hd_interpolate(hd_adv* op, const hd_function* f, double time, void* dst, void* stream) {
  if (!op || !f || !dst) return fail(HD_ERR_INVALID, "hd_interpolate: null argument");
  if (f->kind < 0 || f->kind > 2) return fail(HD_ERR_INVALID, "hd_interpolate: unknown function kind %d", f->kind);
  cudaError_t e = hd::launch_interpolate(op->geom, to_dev(*f), time, dst, op->dtype == HD_F32, op->d_table,
                                         (cudaStream_t)stream);
  return e == cudaSuccess ? HD_OK : cuda_fail(e, "interpolate kernel");
}

int hd_norm_and_error(hd_adv* op, const hd_function* f, double time, const void* src, double* result,
                      void* stream) {
  if (!op || !f || !src || !result) return fail(HD_ERR_INVALID, "hd_norm_and_error: null argument");
  cudaStream_t s = (cudaStream_t)stream;
  if (f->kind < 0 || f->kind > 2) return fail(HD_ERR_INVALID, "hd_norm_and_error: unknown function kind %d", f->kind);
  cudaError_t e = hd::launch_norm_error(op->geom, to_dev(*f), time, src, op->dtype == HD_F32, op->d_table,
                                        op->d_partials, op->d_partials + 2 * hd::kNormBlocks, s);
  if (e != cudaSuccess) return cuda_fail(e, "norm kernel");
  e = cudaMemcpyAsync(result, op->d_partials + 2 * hd::kNormBlocks, 2 * sizeof(double), cudaMemcpyDeviceToHost, s);
  if (e != cudaSuccess) return cuda_fail(e, "norm copy");
  e = cudaStreamSynchronize(s);
  return e == cudaSuccess ? HD_OK : cuda_fail(e, "norm synchronize");
}

int hd_lsrk_create(const char* type, hd_lsrk** out) {
  if (!type || !out) return fail(HD_ERR_INVALID, "hd_lsrk_create: null argument");
  hd_lsrk rk;
  std::memset(&rk, 0, sizeof(rk));
  // Kennedy, Carpenter, Lewis (2000) coefficients, tabulated as in
  // base/time_integrators.templates.h:33-89
  if (!std::strcmp(type, "rk33")) {
    const double b[] = {0.245170287303492, 0.184896052186740, 0.569933660509768};
    const double a[] = {0.755726351946097, 0.386954477304099};
    rk.ns = 3; std::memcpy(rk.bi, b, sizeof(b)); std::memcpy(rk.ai, a, sizeof(a));
  } else if (!std::strcmp(type, "rk45")) {
    const double b[] = {1153189308089. / 22510343858157., 1772645290293. / 4653164025191.,
                        -1672844663538. / 4480602732383., 2114624349019. / 3568978502595.,
                        5198255086312. / 14908931495163.};
    const double a[] = {970286171893. / 4311952581923., 6584761158862. / 12103376702013.,
                        2251764453980. / 15575788980749., 26877169314380. / 34165994151039.};
    rk.ns = 5; std::memcpy(rk.bi, b, sizeof(b)); std::memcpy(rk.ai, a, sizeof(a));
  } else if (!std::strcmp(type, "rk47")) {
    const double b[] = {0.0941840925477795334, 0.149683694803496998, 0.285204742060440058,
                        -0.122201846148053668, 0.0605151571191401122, 0.345986987898399296,
                        0.186627171718797670};
    const double a0[] = {0.241566650129646868, 0.0423866513027719953, 0.215602732678803776,
                         0.232328007537583987, 0.256223412574146438, 0.0978694102142697230};
    rk.ns = 7; std::memcpy(rk.bi, b, sizeof(b));
    for (int i = 0; i < 6; ++i) rk.ai[i] = a0[i] + b[i];
  } else if (!std::strcmp(type, "rk59")) {
    const double b[] = {2274579626619. / 23610510767302., 693987741272. / 12394497460941.,
                        -347131529483. / 15096185902911., 1144057200723. / 32081666971178.,
                        1562491064753. / 11797114684756., 13113619727965. / 44346030145118.,
                        393957816125. / 7825732611452., 720647959663. / 6565743875477.,
                        3559252274877. / 14424734981077.};
    const double a[] = {1107026461565. / 5417078080134., 38141181049399. / 41724347789894.,
                        493273079041. / 11940823631197., 1851571280403. / 6147804934346.,
                        11782306865191. / 62590030070788., 9452544825720. / 13648368537481.,
                        4435885630781. / 26285702406235., 2357909744247. / 11371140753790.};
    rk.ns = 9; std::memcpy(rk.bi, b, sizeof(b)); std::memcpy(rk.ai, a, sizeof(a));
  } else {
    return fail(HD_ERR_UNSUPPORTED, "unknown LSRK type '%s' (rk33, rk45, rk47, rk59)", type);
  }
  std::strncpy(rk.type, type, sizeof(rk.type) - 1);
  // stage times c_s = sum_{j < s-1} b_j + a_{s-1} (time_integrators.templates.h:172-183)
  double sum_b = 0.0;
  rk.ci[0] = 0.0;
  for (int s = 1; s < rk.ns; ++s) {
    rk.ci[s] = sum_b + rk.ai[s - 1];
    sum_b += rk.bi[s - 1];
  }
  hd_lsrk* p = new (std::nothrow) hd_lsrk(rk);
  if (!p) return fail(HD_ERR_ALLOC, "out of host memory");
  *out = p;
  return HD_OK;
}

int hd_lsrk_destroy(hd_lsrk* rk) {
  delete rk;
  return HD_OK;
}

int hd_lsrk_n_stages(const hd_lsrk* rk) { return rk ? rk->ns : 0; }

int hd_lsrk_coefficients(const hd_lsrk* rk, double* ai, double* bi, double* ci) {
  if (!rk) return fail(HD_ERR_INVALID, "hd_lsrk_coefficients: null handle");
  if (ai) std::memcpy(ai, rk->ai, sizeof(double) * (rk->ns - 1));
  if (bi) std::memcpy(bi, rk->bi, sizeof(double) * rk->ns);
  if (ci) std::memcpy(ci, rk->ci, sizeof(double) * rk->ns);
  return HD_OK;
}

// Buffer rotation of the fused step (X0 = sol, X1 = Ki, X2 = Ti as passed):
// X0 holds U and the first stage input; the new solution accumulates in X1;
// the stage inputs alternate between X0 (even stages) and X2 (odd stages),
// each stage writing the next input into the other one.
int hd_lsrk_stage_input(const hd_lsrk* rk, int stage) {
  if (!rk || stage < 0 || stage >= rk->ns) return -1;
  return (stage % 2) ? 2 : 0;
}

int hd_lsrk_stage(hd_adv* op, const hd_lsrk* rk, int stage, void* const* X, double time, double dt, int cells,
                  void* stream) {
  if (!op || !rk || !X || !X[0] || !X[1] || !X[2]) return fail(HD_ERR_INVALID, "hd_lsrk_stage: null argument");
  if (stage < 0 || stage >= rk->ns) return fail(HD_ERR_INVALID, "hd_lsrk_stage: stage %d of %d", stage, rk->ns);
  if (cells != HD_CELLS_ALL && cells != HD_CELLS_INTERIOR && cells != HD_CELLS_BOUNDARY)
    return fail(HD_ERR_INVALID, "hd_lsrk_stage: unknown cell subset %d", cells);
  if (X[0] == X[1] || X[0] == X[2] || X[1] == X[2]) return fail(HD_ERR_INVALID, "hd_lsrk_stage: vectors must differ");
  if (!aligned16(X[0]) || !aligned16(X[1]) || !aligned16(X[2]))
    return fail(HD_ERR_INVALID, "hd_lsrk_stage: vectors must be 16-byte aligned");
  const bool last = stage == rk->ns - 1;
  const double fb = rk->bi[stage] * dt;
  const double fa = last ? 0.0 : rk->ai[stage] * dt;
  const double t_s = time + rk->ci[stage] * dt;
  int mode = stage == 0 ? hd::kStageFirst : (last ? hd::kStageLast : hd::kStageMid);
  if (stage == 0 && last) mode = hd::kStageFirst;  // single-stage schemes are not built
  void* t_in = X[hd_lsrk_stage_input(rk, stage)];
  void* t_out = last ? nullptr : X[(stage % 2) ? 0 : 2];
  return launch(op, mode, t_in, stage == 0 ? t_in : X[1], X[1], t_out, fb, fa, t_s, (cudaStream_t)stream, cells);
}

int hd_lsrk_step(hd_adv* op, const hd_lsrk* rk, void** sol, void** Ki, void** Ti, double time, double dt,
                 void* stream) {
  if (!op || !rk || !sol || !Ki || !Ti || !*sol || !*Ki || !*Ti)
    return fail(HD_ERR_INVALID, "hd_lsrk_step: null argument");
  if (op->part.ghost_values > 0)
    return fail(HD_ERR_UNSUPPORTED, "hd_lsrk_step: a part with ghost faces steps with hd_lsrk_stage and an "
                                    "exchange of the stage input's faces before every stage");
  void* X[3] = {*sol, *Ki, *Ti};
  for (int st = 0; st < rk->ns; ++st) {
    const int rc = hd_lsrk_stage(op, rk, st, X, time, dt, HD_CELLS_ALL, stream);
    if (rc) return rc;
  }
  *sol = X[1];
  *Ki = X[0];
  *Ti = X[2];
  return HD_OK;
}

int hd_lsrk_stage_update(int dtype, long long n, double factor_bi, double factor_ai, const void* K, void* sol,
                         void* next_T, void* stream) {
  if (!K || !sol || n < 0) return fail(HD_ERR_INVALID, "hd_lsrk_stage_update: bad argument");
  if (dtype != HD_F64 && dtype != HD_F32) return fail(HD_ERR_INVALID, "unknown dtype %d", dtype);
  cudaError_t e = hd::launch_lsrk_update(dtype == HD_F32, n, factor_bi, factor_ai, K, sol,
                                         factor_ai == 0.0 ? nullptr : next_T, (cudaStream_t)stream);
  return e == cudaSuccess ? HD_OK : cuda_fail(e, "lsrk update kernel");
}

int hd_lsrk_step_unfused(hd_adv* op, const hd_lsrk* rk, void* sol, void* Ki, void* Ti, double time, double dt,
                         void* stream) {
  if (!op || !rk || !sol || !Ki || !Ti) return fail(HD_ERR_INVALID, "hd_lsrk_step_unfused: null argument");
  if (op->part.ghost_values > 0)
    return fail(HD_ERR_UNSUPPORTED, "hd_lsrk_step_unfused: a part with ghost faces needs an exchange per stage");
  cudaStream_t s = (cudaStream_t)stream;
  const size_t bytes = size_t(op->n_dofs) * (op->dtype == HD_F64 ? 8 : 4);
  // first stage with only_Ti_is_ghosted = true: Ti = sol (time_integrators.templates.h:142-148)
  cudaError_t e = cudaMemcpyAsync(Ti, sol, bytes, cudaMemcpyDeviceToDevice, s);
  if (e != cudaSuccess) return cuda_fail(e, "copy sol -> Ti");
  for (int st = 0; st < rk->ns; ++st) {
    const bool last = st == rk->ns - 1;
    int rc = hd_adv_apply(op, Ki, Ti, time + rk->ci[st] * dt, stream);
    if (rc) return rc;
    rc = hd_lsrk_stage_update(op->dtype, op->n_dofs, rk->bi[st] * dt, last ? 0.0 : rk->ai[st] * dt, Ki, sol, Ti,
                              stream);
    if (rc) return rc;
  }
  return HD_OK;
}

}  // extern "C"
