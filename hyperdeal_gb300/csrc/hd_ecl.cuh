// hd_ecl.cuh -- element-centric (ECL) upwind-DG advection kernels for sm_103a.
//
// Persistent CTAs walk blocks of whole cells.  Each block's (k+1)^D nodal
// values per cell are staged in shared memory by 16-byte cp.async copies one
// block ahead; the D one-dimensional line operators are applied two
// directions at a time ("plane phases") with the plane's N x N values held
// in registers, and the upwind neighbour's face trace is read from global
// memory (L2) -- there is no face loop and no atomics.  The inverse (diagonal) mass, the upwind flux and the downwind
// self-term are folded into the per-direction line operator M_d and the
// inflow coefficient c_d that the host derives from the reference's formulas,
// so one phase does  acc_line += M_d u_line  and  acc[in_node] += c_d u+.
// The last phase writes the result once: either K = A(u) (apply) or, fused
// with the low-storage Runge-Kutta stage, U' = U + b K and T' = U + a K.
//
// Reference operator: include/hyper.deal/operators/advection/
// advection_operation.h:218-566 (volume :325-404, faces :406-526, inverse
// mass :528-563); stage update: base/time_integrators.templates.h:111-135.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

#include "hd_df.cuh"

namespace hd {

constexpr int kMaxDim = 6;
constexpr int kMaxN = 6;  // nodes per direction (degree <= 5)

__host__ __device__ constexpr int ipow(int b, int e) { return e == 0 ? 1 : b * ipow(b, e - 1); }

// Division of 64-bit unsigned integers by an invariant divisor d >= 1 through
// a multiply-high (Granlund and Montgomery, "Division by invariant integers
// using multiplication", PLDI 1994, Figure 4.1 with N = 64):
//   l = ceil(log2 d), m = floor(2^64 (2^l - d) / d) + 1 (< 2^64),
//   t = mulhi(m, n), q = (t + ((n - t) >> min(l, 1))) >> max(l - 1, 0),
// exact for every 0 <= n < 2^64.  The cell coordinates of the generic kernels
// use it: a 64-bit division by a runtime divisor is a long emulated sequence
// on the GPU, and every thread decomposes its cell's id once per cell.
struct DivU64 {
  unsigned long long d, m;
  int s1, s2;
};

inline DivU64 make_divu64(unsigned long long d) {
  int l = 0;
  while (l < 64 && (1ULL << l) < d) ++l;
  const unsigned __int128 num = (((unsigned __int128)1 << l) - d) << 64;
  DivU64 r;
  r.d = d;
  r.m = (unsigned long long)(num / d) + 1;
  r.s1 = l < 1 ? l : 1;
  r.s2 = l > 1 ? l - 1 : 0;
  return r;
}

__host__ __device__ __forceinline__ unsigned long long divu64(unsigned long long n, const DivU64& v) {
#ifdef __CUDA_ARCH__
  const unsigned long long t = __umul64hi(v.m, n);
#else
  const unsigned long long t = (unsigned long long)(((unsigned __int128)v.m * n) >> 64);
#endif
  return (t + ((n - t) >> v.s1)) >> v.s2;
}

// analytic function  amp * prod_d trig(omega_d (x_d - speed_d t) + phase_d)
struct DevFunction {
  int kind;
  double amp;
  double omega[kMaxDim], speed[kMaxDim], phase[kMaxDim];
  int cosine[kMaxDim];
};

// one-dimensional line operator of one direction (see hd_capi.cu: derived
// from the reference's volume + face + inverse-mass formulas)
template <typename T>
struct LineOp {
  T M[kMaxN * kMaxN];  // out_i += M[i*N + q] * u_q
  T cin;               // out_{in_node} += cin * u+
  T c0, cl;            // the same coefficient split by target: node 0 / node N-1 (the other is 0)
  int in_node;         // node of the line that receives the inflow term
  int nb_node;         // node of the upwind neighbour's line giving u+
  int step;            // -1: upwind neighbour on the left, +1: on the right
  int active;          // 0: nothing to do in this direction
};

template <typename T>
struct EclParams {
  const T* tin;   // operator input (also read at neighbours)
  const T* uin;   // RK solution (own cell only); may equal tin
  T* uout;        // apply: result K; stage: new solution
  T* tout;        // stage: next stage input (unused for the last stage)
  T fb, fa;       // stage factors b_s dt, a_s dt
  long long n_cells;
  int D, dim_x;
  int cells[kMaxDim];
  long long cstride[kMaxDim];
  int periodic[kMaxDim];
  // invariant divisors of the cell-id decomposition: cells[d] and the number of
  // x-cells cstride[dim_x]
  DivU64 dcell[kMaxDim], dxcells;
  LineOp<T> op[kMaxDim];
  // FP64 storage only: the same operators as FP32x2 words (hd_df.cuh) for the
  // FP32x2-arithmetic kernels
  std::conditional_t<sizeof(T) == 8, LineOp<f32x2>, char> opx[kMaxDim];
  int bc_inhom;
  DevFunction bc;
  double time;
  double lo[kMaxDim], h[kMaxDim];
  double gl[kMaxN];  // Gauss-Lobatto nodes on [0,1]
  int cpb;           // generic kernel tile: cells per CTA (0 = the shape's maximum)
  int ctas_per_sm;   //   and CTAs per SM of the persistent grid (0 = occupancy limit)
  // Partitioned operators (hd_adv_create_part): the vectors hold the cells
  // [gid0, gid0 + n_cells) of the global mesh -- whole layers of the last
  // direction -- and cells/cstride above describe the global mesh.  A launch
  // processes the local cells [c_lo, c_hi).  The upwind faces of cells owned
  // by another part (only across the last direction) are read from `ghost`:
  // one face of NC/N values per cell of a layer, in the cells' in-layer order
  // (layer = cells per layer).  Unpartitioned: gid0 = 0, c_lo = 0,
  // c_hi = n_cells, ghost = nullptr.
  long long gid0, c_lo, c_hi, layer;
  const T* ghost;
  int* err;  // the operator's device status (bounds-checked builds record violations there)
};

// Device status code of a failed bounds check (builds with -DHD_CHECK only).
constexpr int kCheckError = 4;

// Bounds-checked build (-DHD_CHECK; hyperdeal_gb300/build.py --check): the
// global loads and stores of the ECL kernels check their element index
// against the buffer they address -- the part's cells (n_cells NC values) or
// the ghost region (layer NC/N values) -- and a violation records kCheckError
// in the device status and skips the access instead of trapping.  In the
// normal build the check is the constant true and costs nothing.
template <int NC, int N, typename T>
__device__ __forceinline__ bool checked(const EclParams<T>& P, const T* base, long long idx) {
#ifdef HD_CHECK
  const long long bound = (base == P.ghost && base != P.tin) ? P.layer * (NC / N) : P.n_cells * NC;
  if (idx >= 0 && idx < bound) return true;
  if (P.err) atomicExch(P.err, kCheckError);
  return false;
#else
  (void)P;
  (void)base;
  (void)idx;
  return true;
#endif
}

// coordinates of global cell g: g = gid_x + n_x gid_v, each part lexicographic
template <int D, typename T>
__device__ __forceinline__ void cell_coords(const EclParams<T>& P, long long g, int* cc) {
  const unsigned long long ug = (unsigned long long)g;
  unsigned long long gv = divu64(ug, P.dxcells);
  unsigned long long gx = ug - gv * P.dxcells.d;
#pragma unroll
  for (int d = 0; d < D; ++d) {
    const bool x = d < P.dim_x;
    const unsigned long long r = x ? gx : gv;
    const unsigned long long q = divu64(r, P.dcell[d]);
    cc[d] = int(r - q * P.dcell[d].d);
    if (x) gx = q;
    else gv = q;
  }
}

enum EclMode { kApply = 0, kStageFirst = 1, kStageMid = 2, kStageLast = 3 };

// (explicitly rounded operations here and in the boundary values below: the
// result must not depend on how the surrounding kernel lets the compiler fuse
// multiplies and adds, so that every kernel evaluating the same boundary data
// gets the same bits)
__device__ __forceinline__ double eval_function(const DevFunction& f, const double* x, int D, double t) {
  if (f.kind == 0) return 0.0;
  if (f.kind == 1) return f.amp;
  double r = f.amp;
  for (int d = 0; d < D; ++d) {
    const double arg = __fma_rn(f.omega[d], __fma_rn(-f.speed[d], t, x[d]), f.phase[d]);
    r = __dmul_rn(r, f.cosine[d] ? cos(arg) : sin(arg));
  }
  return r;
}

// coordinate lo + (c + xi) h of a node (xi: reference coordinate in [0, 1])
__device__ __forceinline__ double node_coord(double lo, int c, double xi, double h) {
  return __fma_rn(__dadd_rn(double(c), xi), h, lo);
}

// exterior value of an inhomogeneous Dirichlet face: u+ = -u- + 2 g
__device__ __forceinline__ double dirichlet_exterior(double um, double g) { return __fma_rn(2.0, g, -um); }

// threads per cell and cells per CTA
template <int D, int N, typename T>
struct EclShape {
  static constexpr int NC = ipow(N, D);                       // nodes per cell
  static constexpr int NPLANE = D >= 2 ? ipow(N, D - 2) : 1;  // planes per phase
  static constexpr int TB = (N <= 4 ? 256 : 128);             // target CTA size
  static constexpr int TPC = NPLANE < TB ? NPLANE : TB;       // threads per cell
  static constexpr int CPB = TB / TPC > 0 ? TB / TPC : 1;     // cells per CTA
  static constexpr int THREADS = TPC * CPB;
  static constexpr size_t SMEM = size_t(3) * CPB * NC * sizeof(T);  // 2 staging buffers + accumulator
  static constexpr int NPH = (D + 1) / 2;                     // phases
  // at least two CTAs of the largest shape per SM (caps registers at 128)
  // for FP32, which is bandwidth-bound and needs the occupancy, and for the
  // FP64 6D shapes up to degree 3, whose FP64-pipe-bound arithmetic needs the
  // warps more than the registers (measured on GB300: 331 vs 359 ms per rk45
  // step at 8^3 x 8^3 cells, k = 3); other FP64 shapes are faster without the cap
  static constexpr int MINB = (sizeof(T) == 4 || (D == 6 && N <= 4)) ? 2 : 1;
  static constexpr bool SUPPORTED = SMEM + 48 <= 220 * 1024;
};

// Per-cell stride of the shared-memory tiles: when cells share a warp (fewer
// than 32 threads per cell) consecutive cells are offset by 64 extra bytes, so
// that the same access of two cells falls into different banks.
template <int D, int N, typename T>
struct EclTile {
  static constexpr int NC = ipow(N, D);
  static constexpr bool PAD = EclShape<D, N, T>::TPC < 32 && (NC * sizeof(T)) % 16 == 0;
  static constexpr int CST = NC + (PAD ? int(64 / sizeof(T)) : 0);
};

// 16-byte vector of T (shared-memory plane loads/stores)
template <typename T>
struct Vec16;
template <>
struct Vec16<float> {
  using type = float4;
  static constexpr int n = 4;
  __device__ static float get(const float4& v, int j) { return j == 0 ? v.x : j == 1 ? v.y : j == 2 ? v.z : v.w; }
  __device__ static float4 make(const float* p) { return make_float4(p[0], p[1], p[2], p[3]); }
};
template <>
struct Vec16<double> {
  using type = double2;
  static constexpr int n = 2;
  __device__ static double get(const double2& v, int j) { return j == 0 ? v.x : v.y; }
  __device__ static double2 make(const double* p) { return make_double2(p[0], p[1]); }
};

// node index of the plane/line base for work item `item` in phase with
// directions (dA, dB) (dB = -1 for a single-direction phase): the digits of
// `item` enumerate the remaining directions in increasing order
template <int D, int N>
__device__ __forceinline__ int item_base(int item, int dA, int dB) {
  int base = 0, stride = 1;
#pragma unroll
  for (int e = 0; e < D; ++e) {
    if (e != dA && e != dB) {
      base += (item % N) * stride;
      item /= N;
    }
    stride *= N;
  }
  return base;
}

// upwind neighbour of cell `gid` with coordinates cc along d (-1: domain boundary)
template <typename T>
__device__ __forceinline__ long long neighbour(const EclParams<T>& P, long long gid, const int* cc, int d) {
  const int step = P.op[d].step;
  const int c = cc[d] + step;
  if (c >= 0 && c < P.cells[d]) return gid + step * P.cstride[d];
  if (!P.periodic[d]) return -1;
  return gid + step * P.cstride[d] - (long long)step * P.cells[d] * P.cstride[d];
}

// Source of the upwind trace of neighbour nb (global id; -1: none): returns
// the base pointer and sets *off so that base[*off + node] is the trace value
// at node `node` of the neighbour's nb_node slab (node numbered inside the
// neighbour's cell).  A neighbour in this part's vector is read in place; a
// neighbour owned by another part -- only across the last direction, whose
// layers the parts split, so its slab nb_node is the contiguous node range
// [nb_node NC/N, (nb_node + 1) NC/N) -- is read from the ghost region, where
// its face is the NC/N values of that range in order.  Every index formed for
// a node of the slab lies inside the buffer it addresses.
// `slot` is the cell's own position in its layer of the last direction, which
// is also its upwind neighbour's across that direction (no division here).
// GH = false: the launch has no ghost region (P.ghost == nullptr), every
// neighbour is a cell of this part's vector; GH = true: the ghost region is
// optional (the kernels of FP64 storage serve both kinds of launch).
template <int NC, int N, bool GH, typename T>
__device__ __forceinline__ const T* trace_src(const EclParams<T>& P, long long nb, int nb_node, long long slot,
                                              long long* off) {
  if constexpr (!GH) {
    (void)nb_node;
    (void)slot;
    *off = nb >= 0 ? (nb - P.gid0) * NC : 0;
    return P.tin;
  }
  const long long l = nb - P.gid0;
  if (nb < 0) {
    *off = 0;
    return P.tin;
  }
  if (P.ghost == nullptr || (l >= 0 && l < P.n_cells)) {
    *off = l * NC;
    return P.tin;
  }
  constexpr int NF = NC / N;
  *off = (slot - (long long)nb_node) * NF;
  return P.ghost;
}

// cell coordinates passed by value (an out-of-line callee gets registers, and
// the caller's array stays in registers too)
struct CellCoords {
  int c[kMaxDim];
};

// exterior value of an inhomogeneous Dirichlet face, u+ = -u- + 2 g(x, t), out
// of line: the coordinate arithmetic (FP64) of an inlined copy was hoisted out
// of the kernels' line loops into every cell and direction, boundary or not
template <int D, int N, typename T>
__device__ __noinline__ double dirichlet_inhom_value(const EclParams<T>& P, CellCoords cc, int d, int node, double um) {
  double x[kMaxDim];
  int t = node;
#pragma unroll
  for (int e = 0; e < D; ++e) {
    const int ie = t % N;
    t /= N;
    x[e] = (e == d) ? node_coord(P.lo[e], cc.c[e], P.op[d].step > 0 ? 1.0 : 0.0, P.h[e])
                    : node_coord(P.lo[e], cc.c[e], P.gl[ie], P.h[e]);
  }
  return dirichlet_exterior(um, eval_function(P.bc, x, D, P.time));
}

// exterior value on a boundary (inflow) face: u+ = -u- (+ 2 g(x, t))
template <int D, int N, typename T>
__device__ __forceinline__ T boundary_value(const EclParams<T>& P, const int* cc, int d, int node, T um) {
  if (!P.bc_inhom) return -um;
  CellCoords c;
#pragma unroll
  for (int e = 0; e < kMaxDim; ++e) c.c[e] = e < D ? cc[e] : 0;
  return T(dirichlet_inhom_value<D, N, T>(P, c, d, node, double(um)));
}

// ---- asynchronous global -> shared copies (cp.async; the copies of a group
// complete in order, so one group per cell block gives a two-stage pipeline)
__device__ __forceinline__ void cp_async_16(void* smem, const void* gmem) {
  const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
template <int BYTES>
__device__ __forceinline__ void cp_async_small(void* smem, const void* gmem) {
  const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
  asm volatile("cp.async.ca.shared.global [%0], [%1], %2;\n" ::"r"(s), "l"(gmem), "n"(BYTES) : "memory");
}
// bulk prefetch of [p, p + bytes) into L2 (16-byte aligned, a multiple of 16 bytes)
__device__ __forceinline__ void prefetch_l2_bulk(const void* p, unsigned bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;\n" ::"l"(p), "r"(bytes) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int PENDING>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(PENDING) : "memory"); }

// copy nval contiguous values to a 16-byte aligned shared buffer: 16-byte
// copies when the global start is 16-byte aligned and the size a multiple
// of 16 bytes, element copies otherwise
template <typename T>
__device__ __forceinline__ void stage_async(T* dst, const T* src, long long nval, int tid, int nthreads) {
  if ((reinterpret_cast<uintptr_t>(src) & 15) == 0 && (nval * sizeof(T)) % 16 == 0) {
    constexpr int VPV = 16 / sizeof(T);
    const long long nvec = nval / VPV;
    for (long long v = tid; v < nvec; v += nthreads) cp_async_16(dst + v * VPV, src + v * VPV);
  } else {
    for (long long i = tid; i < nval; i += nthreads) cp_async_small<sizeof(T)>(dst + i, src + i);
  }
}

// shared-memory elements of one staging buffer (rounded to 16 bytes)
template <int D, int N, typename T>
__host__ __device__ constexpr long long ecl_buffer_elems(int cpb) {
  const long long bytes = (long long)cpb * EclTile<D, N, T>::CST * sizeof(T);
  return ((bytes + 15) / 16) * 16 / (long long)sizeof(T);
}

// stage `ncell` consecutive cells into a shared buffer with the cell stride
// of EclTile (16-byte copies when the source is 16-byte aligned)
template <int D, int N, typename T>
__device__ __forceinline__ void stage_cells(T* dst, const T* src, long long ncell, int tid, int nthreads) {
  using TL = EclTile<D, N, T>;
  if constexpr (!TL::PAD) {
    stage_async(dst, src, ncell * TL::NC, tid, nthreads);
  } else {
    constexpr int VPV = 16 / sizeof(T), CPC = TL::NC / VPV;  // chunks per cell
    if ((reinterpret_cast<uintptr_t>(src) & 15) == 0) {
      for (long long v = tid; v < ncell * CPC; v += nthreads) {
        const long long c = v / CPC;
        cp_async_16(dst + c * TL::CST + (v - c * CPC) * VPV, src + v * VPV);
      }
    } else {
      for (long long i = tid; i < ncell * TL::NC; i += nthreads) {
        const long long c = i / TL::NC;
        cp_async_small<sizeof(T)>(dst + c * TL::CST + (i - c * TL::NC), src + i);
      }
    }
  }
}

// one block of P.cpb cells (the CTA's cells start at cell0) from the staged
// input `su_all`: the D line operators two directions per phase, the last
// phase writing K or the fused stage update
// (stage modes mid/last: `uu_all` is the block's RK solution staged in shared
// memory next to the operator input, or nullptr to read it from global memory)
template <int D, int N, typename T, int MODE, bool GH>
__device__ __forceinline__ void ecl_block(const EclParams<T>& P, long long cell0, int lc, int tl, const T* su_all,
                                          T* so_all, const T* uu_all) {
  using S = EclShape<D, N, T>;
  constexpr int NC = S::NC, TPC = S::TPC;
  const long long gid = cell0 + lc;  // local cell
  const bool valid = gid < P.c_hi;
  // global id (of a valid cell also for the idle threads of a partial block)
  const long long gg = P.gid0 + (valid ? gid : P.c_lo);

  // ---- cell coordinates
  int cc[D];
  cell_coords<D>(P, gg, cc);
  // position in the layer of the last direction (ghost faces of parts)
  const long long slot = gg - (long long)cc[D - 1] * P.cstride[D - 1];
  constexpr int CST = EclTile<D, N, T>::CST;
  const T* su = su_all + lc * CST;
  T* so = so_all + lc * CST;

#pragma unroll
  for (int ph = 0; ph < S::NPH; ++ph) {
    const int dA = 2 * ph;
    const int dB = (2 * ph + 1 < D) ? 2 * ph + 1 : -1;
    const int dBi = dB >= 0 ? dB : dA;  // an index that is valid also where dB = -1 is never used
    const int strideA = ipow(N, dA);
    const int strideB = strideA * N;
    const int nitems = dB >= 0 ? ipow(N, D - 2) : ipow(N, D - 1);
    const bool last = (ph == S::NPH - 1);
    const bool actA = valid && P.op[dA].active;
    const bool actB = dB >= 0 && valid && P.op[dBi].active;
    const long long nbA = actA ? neighbour(P, gg, cc, dA) : -1;
    const long long nbB = actB ? neighbour(P, gg, cc, dBi) : -1;
    // trace sources: the neighbour (here or in the ghost region), or cell 0
    // where there is none, so that every load address is valid even if the
    // compiler issues the guarded loads unconditionally
    long long oA = 0, oB = 0;
    const T* const sA = trace_src<NC, N, GH>(P, nbA, P.op[dA].nb_node, slot, &oA);
    const T* const sB = dB >= 0 ? trace_src<NC, N, GH>(P, nbB, P.op[dBi].nb_node, slot, &oB) : P.tin;

    for (int item = tl; item < nitems; item += TPC) {
      const int base = item_base<D, N>(item, dA, dB);
      if (dB >= 0) {
        const LineOp<T>& LA = P.op[dA];
        const LineOp<T>& LB = P.op[dBi];
        // upwind face values of the N lines of both directions, issued first
        T upA[N], upB[N];
#pragma unroll
        for (int b = 0; b < N; ++b)
        {
          const long long ia = oA + base + LA.nb_node * strideA + b * strideB;
          upA[b] = nbA >= 0 && checked<NC, N>(P, sA, ia) ? __ldg(sA + ia) : T(0);
        }
#pragma unroll
        for (int a = 0; a < N; ++a) {
          const long long ib = oB + base + a * strideA + LB.nb_node * strideB;
          upB[a] = nbB >= 0 && checked<NC, N>(P, sB, ib) ? __ldg(sB + ib) : T(0);
        }
        T uu[N][N], acc[N][N];  // [a][b]: node base + a*strideA + b*strideB
        // phase 0: the plane of directions 0, 1 is N*N contiguous values; when
        // that is a whole number of 16-byte words it is read as such (far
        // fewer shared-memory wavefronts than scalar loads of the strided plane)
        // (not for the register-capped FP64 6D shapes: the extra live values spill)
        constexpr bool kVec = (N * N * sizeof(T)) % 16 == 0 && !(sizeof(T) == 8 && D == 6);
        if (kVec && ph == 0) {
          using V = Vec16<T>;
          T flat[N * N];
#pragma unroll
          for (int k = 0; k < N * N / V::n; ++k) {
            const typename V::type w = *reinterpret_cast<const typename V::type*>(su + base + k * V::n);
#pragma unroll
            for (int j = 0; j < V::n; ++j) flat[k * V::n + j] = V::get(w, j);
          }
#pragma unroll
          for (int a = 0; a < N; ++a)
#pragma unroll
            for (int b = 0; b < N; ++b) {
              uu[a][b] = flat[a + N * b];
              acc[a][b] = T(0);
            }
        } else {
#pragma unroll
          for (int a = 0; a < N; ++a)
#pragma unroll
            for (int b = 0; b < N; ++b) {
              const int node = base + a * strideA + b * strideB;
              uu[a][b] = su[node];
              acc[a][b] = ph == 0 ? T(0) : so[node];
            }
        }
        if (actA) {
#pragma unroll
          for (int b = 0; b < N; ++b) {
#pragma unroll
            for (int i = 0; i < N; ++i) {
              T s = acc[i][b];
#pragma unroll
              for (int q = 0; q < N; ++q) s = fma(LA.M[i * N + q], uu[q][b], s);
              acc[i][b] = s;
            }
            T up = upA[b];
            if (nbA < 0) {
              const T um = LA.in_node == 0 ? uu[0][b] : uu[N - 1][b];
              up = boundary_value<D, N, T>(P, cc, dA, base + LA.in_node * strideA + b * strideB, um);
            }
            acc[0][b] = fma(LA.c0, up, acc[0][b]);
            acc[N - 1][b] = fma(LA.cl, up, acc[N - 1][b]);
          }
        }
        if (actB) {
#pragma unroll
          for (int a = 0; a < N; ++a) {
#pragma unroll
            for (int i = 0; i < N; ++i) {
              T s = acc[a][i];
#pragma unroll
              for (int q = 0; q < N; ++q) s = fma(LB.M[i * N + q], uu[a][q], s);
              acc[a][i] = s;
            }
            T up = upB[a];
            if (nbB < 0) {
              const T um = LB.in_node == 0 ? uu[a][0] : uu[a][N - 1];
              up = boundary_value<D, N, T>(P, cc, dB, base + a * strideA + LB.in_node * strideB, um);
            }
            acc[a][0] = fma(LB.c0, up, acc[a][0]);
            acc[a][N - 1] = fma(LB.cl, up, acc[a][N - 1]);
          }
        }
        if (!last) {
          if (kVec && ph == 0) {
            using V = Vec16<T>;
            T flat[N * N];
#pragma unroll
            for (int a = 0; a < N; ++a)
#pragma unroll
              for (int b = 0; b < N; ++b) flat[a + N * b] = acc[a][b];
#pragma unroll
            for (int k = 0; k < N * N / V::n; ++k)
              *reinterpret_cast<typename V::type*>(so + base + k * V::n) = V::make(flat + k * V::n);
          } else {
#pragma unroll
            for (int a = 0; a < N; ++a)
#pragma unroll
              for (int b = 0; b < N; ++b) so[base + a * strideA + b * strideB] = acc[a][b];
          }
        } else if (valid) {
          const long long g0 = gid * NC;
#pragma unroll
          for (int b = 0; b < N; ++b)
#pragma unroll
            for (int a = 0; a < N; ++a) {
              const long long gi = g0 + base + a * strideA + b * strideB;
              const T k = acc[a][b];
              if (!checked<NC, N>(P, P.tin, gi)) continue;
              if constexpr (MODE == kApply) {
                P.uout[gi] = k;
              } else {
                T u;
                if constexpr (MODE == kStageFirst) u = uu[a][b];
                else u = uu_all ? uu_all[lc * CST + base + a * strideA + b * strideB] : P.uin[gi];
                P.uout[gi] = fma(P.fb, k, u);
                if constexpr (MODE != kStageLast) P.tout[gi] = fma(P.fa, k, u);
              }
            }
        }
      } else {
        // single-direction phase (odd D): lines along dA
        const LineOp<T>& LA = P.op[dA];
        const long long iu = oA + base + LA.nb_node * strideA;
        const T upf = nbA >= 0 && checked<NC, N>(P, sA, iu) ? __ldg(sA + iu) : T(0);
        T uu[N], acc[N];
#pragma unroll
        for (int a = 0; a < N; ++a) {
          const int node = base + a * strideA;
          uu[a] = su[node];
          acc[a] = ph == 0 ? T(0) : so[node];
        }
        if (actA) {
#pragma unroll
          for (int i = 0; i < N; ++i) {
            T s = acc[i];
#pragma unroll
            for (int q = 0; q < N; ++q) s = fma(LA.M[i * N + q], uu[q], s);
            acc[i] = s;
          }
          T up = upf;
          if (nbA < 0) {
            const T um = LA.in_node == 0 ? uu[0] : uu[N - 1];
            up = boundary_value<D, N, T>(P, cc, dA, base + LA.in_node * strideA, um);
          }
          acc[0] = fma(LA.c0, up, acc[0]);
          acc[N - 1] = fma(LA.cl, up, acc[N - 1]);
        }
        if (!last) {
#pragma unroll
          for (int a = 0; a < N; ++a) so[base + a * strideA] = acc[a];
        } else if (valid) {
          const long long g0 = gid * NC;
#pragma unroll
          for (int a = 0; a < N; ++a) {
            const long long gi = g0 + base + a * strideA;
            const T k = acc[a];
            if (!checked<NC, N>(P, P.tin, gi)) continue;
            if constexpr (MODE == kApply) {
              P.uout[gi] = k;
            } else {
              const T u = (MODE == kStageFirst) ? uu[a] : (uu_all ? uu_all[lc * CST + base + a * strideA] : P.uin[gi]);
              P.uout[gi] = fma(P.fb, k, u);
              if constexpr (MODE != kStageLast) P.tout[gi] = fma(P.fa, k, u);
            }
          }
        }
      }
    }
    if (!last) __syncthreads();
  }
}

// upwind value of a boundary line of the FP32x2 kernels, out of line (the
// FP64 conversions and boundary arithmetic stay off the periodic path)
template <int D, int N>
__device__ __noinline__ f32x2 x2_boundary_value(const EclParams<double>& P, CellCoords cc, int d, int node,
                                                const f32x2* sx) {
  const double um = x2_to_double(sx[node]);
  const double v = P.bc_inhom ? dirichlet_inhom_value<D, N, double>(P, cc, d, node, um) : -um;
  return x2_from_double(v);
}

// The block in FP32x2 arithmetic on FP64 storage (hd_df.cuh), organised line
// by line instead of plane by plane: a line's N values and N accumulators are
// read from shared memory, its N x N double-word multiply-adds and inflow
// term applied, and the accumulators written back -- or, after the last
// direction of the last phase, the result written to global memory.  The line
// loop is not unrolled: a double-word multiply-add is about twelve FP32
// instructions, and fully unrolled planes overflow the instruction cache; the
// phase and direction loops are unrolled (one copy of the line code per
// direction, whose coefficients and strides are then constant operands).
// The accumulators are stored between directions as they are, hi + lo not
// renormalised: they are only ever added to (the TwoSum of x2_mac is exact
// for any hi, lo), and the few dozen low parts summed per value stay far
// below hi; the result's conversion adds hi and lo in FP64.
// In the first phase a cell's threads visit their lines in a rotated order
// (its planes lie N*N values apart, a multiple of the bank count), and lines
// along direction 0 (contiguous, 16-byte aligned for even N) are read as
// 16-byte words.
// CVT: the staged tile still holds the FP64 values; the first direction of
// the first phase converts each line it reads to FP32x2 in place (a cell's
// first-phase work items are whole planes of directions 0 and 1, so every
// value is converted once, by the thread that reads it again for direction 1,
// before the barrier after which other threads read it)
template <int D, int N, int MODE, bool GH, bool CVT = false>
__device__ __forceinline__ void ecl_block_x2(const EclParams<double>& P, long long cell0, int lc, int tl,
                                             double* su_all, double* so_all, const double* uu_all) {
  using S = EclShape<D, N, double>;
  constexpr int NC = S::NC, TPC = S::TPC;
  constexpr int CST = EclTile<D, N, double>::CST;
  const long long gid = cell0 + lc;  // local cell
  const bool valid = gid < P.c_hi;
  const long long gg = P.gid0 + (valid ? gid : P.c_lo);  // global id
  int cc[D];
  cell_coords<D>(P, gg, cc);
  // position in the layer of the last direction (ghost faces of parts)
  const long long slot = gg - (long long)cc[D - 1] * P.cstride[D - 1];
  // the staged input was converted to FP32x2 words in place (ecl_kernel)
  f32x2* sx = reinterpret_cast<f32x2*>(su_all + lc * CST);
  f32x2* so = reinterpret_cast<f32x2*>(so_all + lc * CST);
  const double* uu = uu_all ? uu_all + lc * CST : nullptr;
  const long long g0 = gid * NC;

#pragma unroll
  for (int ph = 0; ph < S::NPH; ++ph) {
    const int dA = 2 * ph;
    const int dB = (2 * ph + 1 < D) ? 2 * ph + 1 : -1;
    int strideA = 1;
    for (int e = 0; e < dA; ++e) strideA *= N;
    const int strideB = strideA * N;
    const int nitems = dB >= 0 ? ipow(N, D - 2) : ipow(N, D - 1);
    const int ndir = dB >= 0 ? 2 : 1;
    const int nl = dB >= 0 ? N : 1;      // lines per direction in a work item
    // first line of the thread: rotated in the first phase only (its planes lie
    // N*N values apart); in the later phases the threads of a warp take the same
    // line, whose nodes -- and upwind trace values -- are consecutive across
    // the threads, so that their global loads and stores coalesce
    const int rot = (ph == 0 && nl > 1) ? tl % N : 0;
    const bool lastph = ph == S::NPH - 1;
    for (int item = tl; item < nitems; item += TPC) {
      const int base = item_base<D, N>(item, dA, dB);
#pragma unroll
      for (int dd = 0; dd < ndir; ++dd) {
        // (dB is -1 in the single-direction phase of an odd dimension; d never
        // takes that value, even where a compiler evaluates this ahead of the
        // loop bound, so cc[d] and opx[d] always index inside their arrays)
        const int d = (dd == 0 || dB < 0) ? dA : dB;
        const int st = dd == 0 ? strideA : strideB;   // along the line
        const int lst = dd == 0 ? strideB : strideA;  // between the lines
        const LineOp<f32x2>& L = P.opx[d];
        const bool act = valid && L.active;
        const long long nb = act ? neighbour(P, gg, cc, d) : -1;
        // the direction's coefficients in registers for its lines (d is not a
        // compile-time index here: each use would be a constant-bank load)
        f32x2 Mr[N * N];
#pragma unroll
        for (int k = 0; k < N * N; ++k) Mr[k] = L.M[k];
        const f32x2 cin = L.cin;
        const bool first = ph == 0 && dd == 0;
        const bool fin = lastph && dd == ndir - 1;
        // upwind trace (here or in the ghost region; cell 0 where there is no
        // neighbour: every load address stays valid even if the compiler issues
        // the guarded loads unconditionally)
        long long fo = 0;
        const double* const fs = trace_src<NC, N, GH>(P, nb, L.nb_node, slot, &fo);
        const double* face = fs + (fo + L.nb_node * st);
        int l = rot;
        const long long fbase = fo + L.nb_node * st;  // index of `face` relative to fs
        // the upwind trace values of all the item's lines, in visiting order,
        // issued together before the first line
        double fu[N];
#pragma unroll
        for (int j = 0; j < N; ++j) {
          const int lj = (rot + j) % N;
          fu[j] = j < nl && nb >= 0 && checked<NC, N>(P, fs, fbase + base + lj * lst) ? __ldg(face + base + lj * lst)
                                                                                        : 0.0;
        }
#pragma unroll 1
        for (int j = 0; j < nl; ++j) {
          const int lb = base + l * lst;
          const double upd = fu[0];
#pragma unroll
          for (int k = 0; k + 1 < N; ++k) fu[k] = fu[k + 1];
          l = l + 1 < nl ? l + 1 : 0;
          f32x2 u[N], acc[N];
          if (CVT && first) {
            // (direction 0: contiguous lines; 16-byte words for even N)
            double* const su = su_all + lc * CST;
            if constexpr ((N % 2) == 0) {
#pragma unroll
              for (int q = 0; q < N; q += 2) {
                const double2 w = *reinterpret_cast<const double2*>(su + lb + q);
                u[q] = x2_from_double(w.x);
                u[q + 1] = x2_from_double(w.y);
                *reinterpret_cast<float4*>(sx + lb + q) = make_float4(u[q].hi, u[q].lo, u[q + 1].hi, u[q + 1].lo);
              }
            } else {
#pragma unroll
              for (int q = 0; q < N; ++q) {
                u[q] = x2_from_double(su[lb + q]);
                sx[lb + q] = u[q];
              }
            }
          } else if ((N % 2) == 0 && st == 1) {
#pragma unroll
            for (int q = 0; q < N; q += 2) {
              const float4 w = *reinterpret_cast<const float4*>(sx + lb + q);
              u[q] = f32x2{w.x, w.y};
              u[q + 1] = f32x2{w.z, w.w};
            }
          } else {
#pragma unroll
            for (int q = 0; q < N; ++q) u[q] = sx[lb + q * st];
          }
          if (first) {
#pragma unroll
            for (int i = 0; i < N; ++i) acc[i] = f32x2{0.f, 0.f};
          } else if ((N % 2) == 0 && st == 1) {
#pragma unroll
            for (int i = 0; i < N; i += 2) {
              const float4 w = *reinterpret_cast<const float4*>(so + lb + i);
              acc[i] = f32x2{w.x, w.y};
              acc[i + 1] = f32x2{w.z, w.w};
            }
          } else {
#pragma unroll
            for (int i = 0; i < N; ++i) acc[i] = so[lb + i * st];
          }
          if (act) {
#pragma unroll
            for (int i = 0; i < N; ++i) {
              // (the first direction's accumulators start from its first product)
              if (first) acc[i] = x2_mul(Mr[i * N], u[0]);
              else x2_mac(acc[i], Mr[i * N], u[0]);
#pragma unroll
              for (int q = 1; q < N; ++q) x2_mac(acc[i], Mr[i * N + q], u[q]);
            }
            const int in = L.in_node;
            f32x2 up;
            if (nb >= 0) {
              up = x2_from_double(upd);
            } else {
              CellCoords c;
#pragma unroll
              for (int e = 0; e < kMaxDim; ++e) c.c[e] = e < D ? cc[e] : 0;
              up = x2_boundary_value<D, N>(P, c, d, lb + in * st, sx);
            }
            if (in == 0) x2_mac(acc[0], cin, up);
            else x2_mac(acc[N - 1], cin, up);
          }
          if (!fin) {
            if ((N % 2) == 0 && st == 1) {
#pragma unroll
              for (int i = 0; i < N; i += 2)
                *reinterpret_cast<float4*>(so + lb + i) = make_float4(acc[i].hi, acc[i].lo, acc[i + 1].hi, acc[i + 1].lo);
            } else {
#pragma unroll
              for (int i = 0; i < N; ++i) so[lb + i * st] = acc[i];
            }
          } else if (valid) {
#pragma unroll
            for (int i = 0; i < N; ++i) {
              const int node = lb + i * st;
              const long long gi = g0 + node;
              const double k = x2_to_double(acc[i]);
              if (!checked<NC, N>(P, P.tin, gi)) continue;
              if constexpr (MODE == kApply) {
                P.uout[gi] = k;
              } else {
                // exact U: the RK solution in FP64 (the first stage's is its input, read again from L2)
                const double uv = uu ? uu[node] : P.uin[gi];
                P.uout[gi] = fma(P.fb, k, uv);
                if constexpr (MODE != kStageLast) P.tout[gi] = fma(P.fa, k, uv);
              }
            }
          }
        }
      }
    }
    if (!lastph) __syncthreads();
  }
}

// stage modes mid/last also stage the RK solution of the block (two more
// buffers) when five buffers of one cell fit in shared memory (not for the
// FP64 6D shapes: their 32 KiB+ cell tiles would leave one CTA per SM)
template <int D, int N, typename T, int MODE, typename A = T>
struct EclStaging {
  // (not for FP32x2 arithmetic either: its issue-bound kernels gain more from
  // the CTAs that the two extra buffers would cost than from staging U)
  static constexpr bool STAGE_U = (MODE == kStageMid || MODE == kStageLast) && !(sizeof(T) == 8 && D == 6) &&
                                  !std::is_same_v<A, f32x2> &&
                                  size_t(5) * EclShape<D, N, T>::NC * sizeof(T) + 64 <= 220 * 1024;
  static constexpr int NBUF = STAGE_U ? 5 : 3;
};

// Persistent generic kernel: CTAs walk blocks of P.cpb cells with a stride of
// the grid; the next block's input is staged by cp.async while the current
// one is computed (two staging buffers + one accumulator tile).  The FP32x2
// kernels are capped at 128 registers (two CTAs of the largest shape per SM):
// their issue-bound line loops need the warps.
// GH: the launch may read a ghost region (P.ghost != nullptr; parts of a
// partitioned mesh only) -- the kernels without it keep the plain neighbour
// addressing of an unpartitioned vector
// 6D FP32x2: one staging buffer (the next block's input prefetched into L2
// instead of staged) and three CTAs per SM at 85 registers
template <int D, int N, typename T, typename A>
struct EclX2Single {
  static constexpr bool value = std::is_same_v<A, f32x2> && D == 6;
};

template <int D, int N, typename T, int MODE, typename A = T, bool GH = false>
__global__ void __launch_bounds__(EclShape<D, N, T>::THREADS,
                                  std::is_same_v<A, f32x2> ? (EclX2Single<D, N, T, A>::value ? 3 : 2)
                                                           : EclShape<D, N, T>::MINB)
    ecl_kernel(const __grid_constant__ EclParams<T> P) {
  using S = EclShape<D, N, T>;
  constexpr int NC = S::NC, TPC = S::TPC;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int cpb = P.cpb;
  constexpr bool SU = EclStaging<D, N, T, MODE, A>::STAGE_U;
  constexpr bool SINGLE = EclX2Single<D, N, T, A>::value;
  const long long bufe = ecl_buffer_elems<D, N, T>(cpb);
  T* const s_in0 = reinterpret_cast<T*>(smem_raw);
  T* const s_in1 = s_in0 + bufe;
  T* const s_o = s_in0 + (SINGLE ? 1 : 2) * bufe;
  T* const s_u0 = s_in0 + 3 * bufe;  // (stage modes with STAGE_U only)
  T* const s_u1 = s_in0 + 4 * bufe;
  const int tid = threadIdx.x, nthr = blockDim.x;
  const int lc = tid / TPC, tl = tid % TPC;
  const long long nblk = (P.c_hi - P.c_lo + cpb - 1) / cpb;
  auto stage = [&](T* dst, T* dstu, long long blk) {
    const long long c0 = P.c_lo + blk * cpb;
    long long ncell = (P.c_hi - c0) < cpb ? (P.c_hi - c0) : cpb;
    if (!checked<NC, N>(P, P.tin, (c0 + ncell) * NC - 1)) ncell = 0;
    stage_cells<D, N, T>(dst, P.tin + c0 * NC, ncell, tid, nthr);
    if constexpr (SU) {
      stage_cells<D, N, T>(dstu, P.uin + c0 * NC, ncell, tid, nthr);
    } else if constexpr ((MODE == kStageMid || MODE == kStageLast) && (NC * sizeof(T)) % 16 == 0) {
      // the block's RK solution, read from global memory by the last phase,
      // into L2 one block ahead (bulk prefetches of up to 16 KiB)
      const long long bytes = ncell * NC * (long long)sizeof(T);
      const long long off = (long long)tid * 16384;
      if (off < bytes)
        prefetch_l2_bulk(reinterpret_cast<const char*>(P.uin + c0 * NC) + off,
                         unsigned(bytes - off < 16384 ? bytes - off : 16384));
    }
  };
  if constexpr (SINGLE) {
    for (long long b = blockIdx.x; b < nblk; b += gridDim.x) {
      stage(s_in0, nullptr, b);
      cp_async_commit();
      // the next block's input into L2 meanwhile (bulk prefetches of up to 16 KiB)
      const long long nb = b + gridDim.x;
      if (nb < nblk) {
        const long long c0 = P.c_lo + nb * cpb;
        const long long ncell = (P.c_hi - c0) < cpb ? (P.c_hi - c0) : cpb;
        const long long bytes = ncell * NC * (long long)sizeof(T);
        const long long off = (long long)tid * 16384;
        if (off < bytes)
          prefetch_l2_bulk(reinterpret_cast<const char*>(P.tin + c0 * NC) + off,
                           unsigned(bytes - off < 16384 ? bytes - off : 16384));
      }
      cp_async_wait<0>();
      __syncthreads();
      ecl_block_x2<D, N, MODE, GH, true>(P, P.c_lo + b * cpb, lc, tl, s_in0, s_o, nullptr);
      __syncthreads();  // the buffer and s_o are free for the next block
    }
    return;
  }
  long long b = blockIdx.x;
  if (b < nblk) stage(s_in0, s_u0, b);
  cp_async_commit();
  bool odd = false;
  for (; b < nblk; b += gridDim.x) {
    T* const cur = odd ? s_in1 : s_in0;
    T* const nxt = odd ? s_in0 : s_in1;
    T* const curu = odd ? s_u1 : s_u0;
    T* const nxtu = odd ? s_u0 : s_u1;
    const long long nb = b + gridDim.x;
    if (nb < nblk) stage(nxt, nxtu, nb);
    cp_async_commit();
    cp_async_wait<1>();  // this thread's copies of block b are complete
    __syncthreads();     // ... and everybody's
    // (FP32x2: the block converts the staged input to double-word FP32 in
    // place as its first direction reads it, once per value -- the line loops
    // read each value up to D times)
    if constexpr (std::is_same_v<A, f32x2>)
      ecl_block_x2<D, N, MODE, GH, true>(P, P.c_lo + b * cpb, lc, tl, cur, s_o, SU ? curu : nullptr);
    else
      ecl_block<D, N, T, MODE, GH>(P, P.c_lo + b * cpb, lc, tl, cur, s_o, SU ? curu : nullptr);
    __syncthreads();     // cur and s_o are free for the next blocks
    odd = !odd;
  }
  cp_async_wait<0>();
}

// default tile: CTAs of about 64 threads (measured on GB300 over 2D-5D,
// degrees 2-5, both storage types: small CTAs let more of them share an SM
// and overlap their staging with other CTAs' arithmetic)
template <int D, int N, typename T>
__host__ __device__ constexpr int ecl_default_cpb() {
  constexpr int tpc = EclShape<D, N, T>::TPC, cpb = (64 + tpc / 2) / tpc;
  return cpb < 1 ? 1 : (cpb > EclShape<D, N, T>::CPB ? EclShape<D, N, T>::CPB : cpb);
}

// host launcher of the four kernels (one per mode) of one (D, N, T, A, GH):
// P is the launch's final parameter block, nbuf its staging buffers per cell tile
template <int D, int N, typename T, typename A, bool GH>
cudaError_t launch_ecl_mode(const EclParams<T>& P, int mode, int nbuf, cudaStream_t stream) {
  using S = EclShape<D, N, T>;
  if constexpr (!S::SUPPORTED) {
    return cudaErrorNotSupported;
  } else {
    const int threads = S::TPC * P.cpb;
    const size_t smem = size_t(nbuf * ecl_buffer_elems<D, N, T>(P.cpb)) * sizeof(T);
    // one flag per mode: the four kernels share this lambda's instantiation
    static bool attr_done[4] = {false, false, false, false};
    static int sms = 0;
    auto go = [&](auto kern) -> cudaError_t {
      if (!attr_done[mode]) {
        int cmax = S::CPB;
        while (cmax > 1 && size_t(nbuf * ecl_buffer_elems<D, N, T>(cmax)) * sizeof(T) > 220 * 1024) --cmax;
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             int(nbuf * ecl_buffer_elems<D, N, T>(cmax) * sizeof(T)));
        if (e != cudaSuccess) return e;
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        attr_done[mode] = true;
      }
      int per_sm = P.ctas_per_sm;
      if (per_sm < 1) {
        cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem);
        if (e != cudaSuccess) return e;
        if (per_sm < 1) per_sm = 1;
      }
      const long long nblk = (P.c_hi - P.c_lo + P.cpb - 1) / P.cpb;
      if (nblk <= 0) return cudaSuccess;  // an empty cell range launches nothing
      const long long want = (long long)sms * per_sm;
      const unsigned grid = unsigned(nblk < want ? nblk : want);
      kern<<<grid, threads, smem, stream>>>(P);
      return cudaGetLastError();
    };
    switch (mode) {
      case kApply: return go(ecl_kernel<D, N, T, kApply, A, GH>);
      case kStageFirst: return go(ecl_kernel<D, N, T, kStageFirst, A, GH>);
      case kStageMid: return go(ecl_kernel<D, N, T, kStageMid, A, GH>);
      case kStageLast: return go(ecl_kernel<D, N, T, kStageLast, A, GH>);
      default: return cudaErrorInvalidValue;
    }
  }
}

// host launcher for one (D, N, T, arithmetic A): P.cpb cells per CTA (1..CPB;
// 0 = default) and ctas_per_sm CTAs per SM (0 = as many as fit), persistent
// grid.  FP32 storage, bandwidth-bound with little arithmetic per cell, has
// kernels without the ghost-region addressing for unpartitioned launches
// (measured on GB300, 4D k = 3: 6% per rk45 step) and kernels with it for
// parts, instantiated in units of their own (ecl_gh_<D>_<N>.cu) so that both
// compile in parallel; the FP64 kernels, bound by their arithmetic, serve both.
template <int D, int N, typename T, typename A = T>
cudaError_t launch_ecl(const EclParams<T>& P0, int mode, cudaStream_t stream) {
  using S = EclShape<D, N, T>;
  if constexpr (!S::SUPPORTED) {
    return cudaErrorNotSupported;
  } else {
    EclParams<T> P = P0;
    if (P.cpb < 1 || P.cpb > S::CPB) P.cpb = ecl_default_cpb<D, N, T>();
    if (mode < kApply || mode > kStageLast) return cudaErrorInvalidValue;
    const int nbuf = EclX2Single<D, N, T, A>::value ? 2
                     : mode == kStageMid ? EclStaging<D, N, T, kStageMid, A>::NBUF
                     : mode == kStageLast ? EclStaging<D, N, T, kStageLast, A>::NBUF : 3;
    // the staged tiles of the largest shape may not fit five times: shrink the tile
    while (P.cpb > 1 && size_t(nbuf * ecl_buffer_elems<D, N, T>(P.cpb)) * sizeof(T) > 220 * 1024) --P.cpb;
    if constexpr (std::is_same_v<T, float>)
      return P.ghost ? launch_ecl_mode<D, N, T, A, true>(P, mode, nbuf, stream)
                     : launch_ecl_mode<D, N, T, A, false>(P, mode, nbuf, stream);
    else
      return launch_ecl_mode<D, N, T, A, true>(P, mode, nbuf, stream);
  }
}

// the FP32 ghost-region launcher of one (D, N): explicitly instantiated in
// ecl_gh_<D>_<N>.cu, declared (not instantiated) in ecl_<D>_<N>.cu
#define HD_ECL_GH_INSTANCES(PREFIX, D, N) \
  PREFIX template cudaError_t launch_ecl_mode<D, N, float, float, true>(const EclParams<float>&, int, int, cudaStream_t);

// launcher table entry
struct EclLaunchers {
  cudaError_t (*f64)(const EclParams<double>&, int, cudaStream_t);
  cudaError_t (*f32)(const EclParams<float>&, int, cudaStream_t);
  size_t smem_f64, smem_f32;
  int threads_f64, threads_f32, cells_per_cta_f64, cells_per_cta_f32;
  bool ok_f64, ok_f32;
  cudaError_t (*f64x)(const EclParams<double>&, int, cudaStream_t);  // FP64 storage, FP32x2 arithmetic
};

template <int D, int N>
EclLaunchers make_launchers() {
  using S64 = EclShape<D, N, double>;
  using S32 = EclShape<D, N, float>;
  return EclLaunchers{&launch_ecl<D, N, double>, &launch_ecl<D, N, float>, S64::SMEM, S32::SMEM,
                      S64::THREADS, S32::THREADS, S64::CPB, S32::CPB, S64::SUPPORTED, S32::SUPPORTED,
                      &launch_ecl<D, N, double, f32x2>};
}

// message of the last failure for hd_last_error() (hd_capi.cu)
void set_last_error(const char* msg);

// pipelined 6D degree-3 FP32 kernel (hd_ecl6.cu): eligible for fully periodic
// 3x+3v meshes; err receives a device error code on a bounded-wait time-out;
// ticket is a device int the launch uses as its row counter
bool ecl6_eligible(const EclParams<float>& P);
// wait_limit: try_wait rounds of the bounded waits (0: the default); skip_issue: test
// hook, nothing is issued for cell skip_issue of the launch's first row (-1: off)
cudaError_t launch_ecl6(const EclParams<float>& P, int* err, int* ticket, int mode, cudaStream_t stream,
                        unsigned wait_limit = 0, int skip_issue = -1);

// defined in hd_dispatch.cu (over the generated units ecl_<D>_<N>.cu)
EclLaunchers ecl_launchers_d2(int N);
EclLaunchers ecl_launchers_d3(int N);
EclLaunchers ecl_launchers_d4(int N);
EclLaunchers ecl_launchers_d5(int N);
EclLaunchers ecl_launchers_d6(int N);

}  // namespace hd
