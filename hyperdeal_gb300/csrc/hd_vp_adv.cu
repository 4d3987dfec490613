// hd_vp_adv.cu -- ECL advection with the Vlasov-Poisson phase-space velocity.
//
// Along every line of a cell the velocity component of that line's direction
// is constant: for an x-direction d it is the line's v-coordinate v_d (the
// line moves in x only), for a v-direction it is grad(phi)_d at the line's
// x-node (the line moves in v only).  The operator on a line is therefore
// (a/h) [G u + upwind face terms], with the upwind side chosen per line by
// the sign of a -- the reference's flux 0.5((u-+u+)a.n + |a.n|(u- - u+))
// evaluated at the line's face points (advection_operation.h:325-526 with
// the velocities of velocity_field_view.h:103-209 of the VP example).
//
// The kernel has the structure of the generic advection kernel (hd_ecl.cuh):
// persistent CTAs walk blocks of cells, the next block's input (and, in the
// middle/last RK stages, its RK solution) is staged by cp.async while the
// current block is computed, and the LSRK stage update is fused into the
// last phase.
#include <cuda_runtime.h>

#include "hd_ecl.cuh"
#include "hd_ecl6.cuh"
#include "hd_vp.cuh"
#include "hd_vp_pipe.cuh"

namespace hd {

template <typename T>
struct VpLine {
  T G[kMaxN * kMaxN];  // G[i*N + q]
  T winv0, winvk;      // 1/w_0, 1/w_{N-1}
};

template <int D, int N, typename T, int MODE>
__device__ __forceinline__ void vp_block(const VpAdvParams<T>& P, const VpLine<T>& Lk, long long cell0, int lc,
                                         int tl, const T* su_all, T* so_all, const T* uu_all) {
  using S = EclShape<D, N, T>;
  constexpr int NC = S::NC, TPC = S::TPC, DX = D / 2;
  const VpGeom& g = P.g;
  const long long gid = cell0 + lc;
  const bool valid = gid < g.n_cells;
  int cc[D];
  long long nbL[D], nbR[D];
  long long gx = 0;
  {
    const long long gg = valid ? gid : 0;
    gx = vp_cell_coords<D>(g, gg, cc);
#pragma unroll
    for (int d = 0; d < D; ++d) {
      const long long cs = g.cstride[d];
      nbL[d] = cc[d] > 0 ? gg - cs : gg + (long long)(g.cells[d] - 1) * cs;
      nbR[d] = cc[d] + 1 < g.cells[d] ? gg + cs : gg - (long long)(g.cells[d] - 1) * cs;
    }
  }
  constexpr int CST = EclTile<D, N, T>::CST;
  const T* su = su_all + lc * CST;
  T* so = so_all + lc * CST;

  // velocity / h of the line along d through node `bnode` (any node of the line)
  auto line_scale = [&](int d, int bnode) -> T {
    if (d < DX) {
      const int e = DX + d;
      const int ie = (bnode / ipow(N, e)) % N;
      return __ldg(P.xs + (d * kVpMaxCellsV + cc[e]) * N + ie);
    }
    return __ldg(P.es + (gx * g.NCx + (bnode % ipow(N, DX))) * DX + (d - DX));
  };
  // the result of node `node` (local index) with value k
  auto emit = [&](int node, T k, T uval) {
    const long long gi = gid * NC + node;
    if constexpr (MODE == kApply) {
      P.dst[gi] = k;
    } else {
      const T u = (MODE == kStageFirst) ? uval : (uu_all ? uu_all[lc * CST + node] : P.uin[gi]);
      P.dst[gi] = fma(P.fb, k, u);
      if constexpr (MODE != kStageLast) P.tout[gi] = fma(P.fa, k, u);
    }
  };

  // phases of two directions; each line: out += (a/h) [G u + upwind face terms]
#pragma unroll
  for (int ph = 0; ph < S::NPH; ++ph) {
    const int dA = 2 * ph;
    const int dB = (2 * ph + 1 < D) ? 2 * ph + 1 : -1;
    const int strideA = ipow(N, dA);
    const int strideB = strideA * N;
    const int nitems = dB >= 0 ? ipow(N, D - 2) : ipow(N, D - 1);
    const bool last = (ph == S::NPH - 1);
    for (int item = tl; item < nitems; item += TPC) {
      const int base = item_base<D, N>(item, dA, dB);
      if (dB >= 0) {
        // scales and the upwind values of every line, issued first; both
        // neighbours' face values are loaded (independent of the scale's
        // sign, so no load waits for another) and the upwind one is selected
        T scA[N], scB[N], upA[N], upB[N];
#pragma unroll
        for (int b = 0; b < N; ++b) {
          const int bn = base + b * strideB;
          scA[b] = valid ? line_scale(dA, bn) : T(0);
          const T l = valid ? __ldg(P.src + nbL[dA] * NC + bn + (N - 1) * strideA) : T(0);
          const T r = valid ? __ldg(P.src + nbR[dA] * NC + bn) : T(0);
          upA[b] = scA[b] > T(0) ? l : r;
        }
#pragma unroll
        for (int a = 0; a < N; ++a) {
          const int bn = base + a * strideA;
          scB[a] = valid ? line_scale(dB, bn) : T(0);
          const T l = valid ? __ldg(P.src + nbL[dB] * NC + bn + (N - 1) * strideB) : T(0);
          const T r = valid ? __ldg(P.src + nbR[dB] * NC + bn) : T(0);
          upB[a] = scB[a] > T(0) ? l : r;
        }
        T uu[N][N], acc[N][N];
        constexpr bool kVec = (N * N * sizeof(T)) % 16 == 0;  // phase 0: N*N contiguous values per plane
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
        if (valid) {
#pragma unroll
          for (int b = 0; b < N; ++b) {
            const T sc = scA[b];
#pragma unroll
            for (int i = 0; i < N; ++i) {
              T s = T(0);
#pragma unroll
              for (int q = 0; q < N; ++q) s = fma(Lk.G[i * N + q], uu[q][b], s);
              acc[i][b] = fma(sc, s, acc[i][b]);
            }
            if (sc > T(0)) {
              acc[N - 1][b] = fma(-sc * Lk.winvk, uu[N - 1][b], acc[N - 1][b]);
              acc[0][b] = fma(sc * Lk.winv0, upA[b], acc[0][b]);
            } else if (sc < T(0)) {
              acc[0][b] = fma(sc * Lk.winv0, uu[0][b], acc[0][b]);
              acc[N - 1][b] = fma(-sc * Lk.winvk, upA[b], acc[N - 1][b]);
            }
          }
#pragma unroll
          for (int a = 0; a < N; ++a) {
            const T sc = scB[a];
#pragma unroll
            for (int i = 0; i < N; ++i) {
              T s = T(0);
#pragma unroll
              for (int q = 0; q < N; ++q) s = fma(Lk.G[i * N + q], uu[a][q], s);
              acc[a][i] = fma(sc, s, acc[a][i]);
            }
            if (sc > T(0)) {
              acc[a][N - 1] = fma(-sc * Lk.winvk, uu[a][N - 1], acc[a][N - 1]);
              acc[a][0] = fma(sc * Lk.winv0, upB[a], acc[a][0]);
            } else if (sc < T(0)) {
              acc[a][0] = fma(sc * Lk.winv0, uu[a][0], acc[a][0]);
              acc[a][N - 1] = fma(-sc * Lk.winvk, upB[a], acc[a][N - 1]);
            }
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
#pragma unroll
          for (int a = 0; a < N; ++a)
#pragma unroll
            for (int b = 0; b < N; ++b) emit(base + a * strideA + b * strideB, acc[a][b], uu[a][b]);
        }
      } else {
        T uu[N], acc[N];
#pragma unroll
        for (int a = 0; a < N; ++a) {
          uu[a] = su[base + a * strideA];
          acc[a] = ph == 0 ? T(0) : so[base + a * strideA];
        }
        if (valid) {
          const T sc = line_scale(dA, base);
          const T up = __ldg(P.src + (sc > T(0) ? nbL[dA] * NC + base + (N - 1) * strideA : nbR[dA] * NC + base));
#pragma unroll
          for (int i = 0; i < N; ++i) {
            T s = T(0);
#pragma unroll
            for (int q = 0; q < N; ++q) s = fma(Lk.G[i * N + q], uu[q], s);
            acc[i] = fma(sc, s, acc[i]);
          }
          if (sc > T(0)) {
            acc[N - 1] = fma(-sc * Lk.winvk, uu[N - 1], acc[N - 1]);
            acc[0] = fma(sc * Lk.winv0, up, acc[0]);
          } else if (sc < T(0)) {
            acc[0] = fma(sc * Lk.winv0, uu[0], acc[0]);
            acc[N - 1] = fma(-sc * Lk.winvk, up, acc[N - 1]);
          }
        }
        if (!last) {
#pragma unroll
          for (int a = 0; a < N; ++a) so[base + a * strideA] = acc[a];
        } else if (valid) {
#pragma unroll
          for (int a = 0; a < N; ++a) emit(base + a * strideA, acc[a], uu[a]);
        }
      }
    }
    if (!last) __syncthreads();
  }
}

// The block in FP32x2 arithmetic on FP64 storage (hd_df.cuh), line by line as
// ecl_block_x2 in hd_ecl.cuh: the staged input was converted to double-word
// words in place; per line  t_i = sum_q G_iq u_q  (double-word), acc_i += s t_i
// with the line's scale s, then the upwind face terms; the stage update is
// done in FP64 on the rounded result.
template <int D, int N, int MODE>
__device__ __forceinline__ void vp_block_x2(const VpAdvParams<double>& P, const VpLine<f32x2>& Lk, long long cell0,
                                            int lc, int tl, const double* su_all, double* so_all) {
  using S = EclShape<D, N, double>;
  constexpr int NC = S::NC, TPC = S::TPC, DX = D / 2;
  constexpr int CST = EclTile<D, N, double>::CST;
  const VpGeom& g = P.g;
  const long long gid = cell0 + lc;
  const bool valid = gid < g.n_cells;
  int cc[D];
  long long nbL[D], nbR[D];
  long long gx = 0;
  {
    const long long gg = valid ? gid : 0;
    gx = vp_cell_coords<D>(g, gg, cc);
#pragma unroll
    for (int d = 0; d < D; ++d) {
      const long long cs = g.cstride[d];
      nbL[d] = cc[d] > 0 ? gg - cs : gg + (long long)(g.cells[d] - 1) * cs;
      nbR[d] = cc[d] + 1 < g.cells[d] ? gg + cs : gg - (long long)(g.cells[d] - 1) * cs;
    }
  }
  const f32x2* sx = reinterpret_cast<const f32x2*>(su_all + lc * CST);
  f32x2* so = reinterpret_cast<f32x2*>(so_all + lc * CST);
  const long long g0 = gid * NC;
  auto line_scale = [&](int d, int bnode) -> double {
    if (d < DX) {
      const int e = DX + d;
      int ie = bnode;
      for (int k = 0; k < e; ++k) ie /= N;
      return __ldg(P.xs + (d * kVpMaxCellsV + cc[e]) * N + ie % N);
    }
    return __ldg(P.es + (gx * g.NCx + (bnode % ipow(N, DX))) * DX + (d - DX));
  };

  // phase and direction loops unrolled (each direction's line code compiled
  // once, with its strides constant), the line loop rolled
#pragma unroll
  for (int ph = 0; ph < S::NPH; ++ph) {
    const int dA = 2 * ph;
    const int dB = (2 * ph + 1 < D) ? 2 * ph + 1 : -1;
    int strideA = 1;
    for (int e = 0; e < dA; ++e) strideA *= N;
    const int strideB = strideA * N;
    const int nitems = dB >= 0 ? ipow(N, D - 2) : ipow(N, D - 1);
    const int ndir = dB >= 0 ? 2 : 1;
    const int nl = dB >= 0 ? N : 1;
    const int rot = nl > 1 ? tl % N : 0;
    const bool lastph = ph == S::NPH - 1;
    for (int item = tl; item < nitems; item += TPC) {
      const int base = item_base<D, N>(item, dA, dB);
#pragma unroll
      for (int dd = 0; dd < ndir; ++dd) {
        // (never the -1 of a single-direction phase, even if evaluated ahead of the bound)
        const int d = (dd == 0 || dB < 0) ? dA : dB;
        const int st = dd == 0 ? strideA : strideB;   // along the line
        const int lst = dd == 0 ? strideB : strideA;  // between the lines
        const bool first = ph == 0 && dd == 0;
        const bool fin = lastph && dd == ndir - 1;
        int l = rot;
#pragma unroll 1
        for (int j = 0; j < nl; ++j) {
          const int lb = base + l * lst;
          l = l + 1 < nl ? l + 1 : 0;
          const double sc = valid ? line_scale(d, lb) : 0.0;
          // the scale in double-word form; its sign (that of hi; +-0 only where
          // |sc| < 2^-126, whose terms vanish) picks the upwind side without an
          // FP64 comparison
          const f32x2 s2 = x2_from_double(sc);
          const bool pos = s2.hi > 0.f;
          // upwind trace (the neighbour cells are valid cells even for an invalid gid)
          const double up = __ldg(P.src + (pos ? nbL[d] * NC + lb + (N - 1) * st : nbR[d] * NC + lb));
          f32x2 u[N], acc[N];
          if ((N % 2) == 0 && st == 1) {
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
          } else {
#pragma unroll
            for (int i = 0; i < N; ++i) acc[i] = so[lb + i * st];
          }
          if (s2.hi != 0.f) {
#pragma unroll
            for (int i = 0; i < N; ++i) {
              f32x2 t = x2_mul(Lk.G[i * N], u[0]);
#pragma unroll
              for (int q = 1; q < N; ++q) x2_mac(t, Lk.G[i * N + q], u[q]);
              x2_mac(acc[i], s2, x2_norm(t));
            }
            // upwind face: (s / w_k)(u+ - u-) at the inflow node
            const f32x2 c0 = x2_norm(x2_mul(s2, Lk.winv0));
            const f32x2 ck = x2_norm(x2_mul(s2, Lk.winvk));
            const f32x2 nck{-ck.hi, -ck.lo};
            const f32x2 upx = x2_from_double(up);
            if (pos) {
              x2_mac(acc[N - 1], nck, u[N - 1]);
              x2_mac(acc[0], c0, upx);
            } else {
              x2_mac(acc[0], c0, u[0]);
              x2_mac(acc[N - 1], nck, upx);
            }
          }
          if (!fin) {
            // accumulators stored as they are between directions (only added to)
#pragma unroll
            for (int i = 0; i < N; ++i) so[lb + i * st] = acc[i];
          } else if (valid) {
#pragma unroll
            for (int i = 0; i < N; ++i) {
              const long long gi = g0 + lb + i * st;
              const double k = x2_to_double(acc[i]);
              if constexpr (MODE == kApply) {
                P.dst[gi] = k;
              } else {
                const double uv = P.uin[gi];  // exact U in FP64 (kStageFirst: the stage input)
                P.dst[gi] = fma(P.fb, k, uv);
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

template <int D, int N, typename T, int MODE, typename A = T>
__global__ void __launch_bounds__(EclShape<D, N, T>::THREADS,
                                  std::is_same_v<A, f32x2> ? 2 : EclShape<D, N, T>::MINB)
    vp_adv_kernel(const __grid_constant__ VpAdvParams<T> P, const __grid_constant__ VpLine<A> Lk, int cpb) {
  using S = EclShape<D, N, T>;
  constexpr int NC = S::NC, TPC = S::TPC;
  constexpr bool SU = EclStaging<D, N, T, MODE, A>::STAGE_U;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const long long bufe = ecl_buffer_elems<D, N, T>(cpb);
  T* const s_in0 = reinterpret_cast<T*>(smem_raw);
  T* const s_in1 = s_in0 + bufe;
  T* const s_o = s_in0 + 2 * bufe;
  T* const s_u0 = s_in0 + 3 * bufe;
  T* const s_u1 = s_in0 + 4 * bufe;
  const int tid = threadIdx.x, nthr = blockDim.x;
  const int lc = tid / TPC, tl = tid % TPC;
  const long long n_cells = P.g.n_cells;
  const long long nblk = (n_cells + cpb - 1) / cpb;
  auto stage = [&](T* dst, T* dstu, long long blk) {
    const long long c0 = blk * cpb;
    const long long ncell = (n_cells - c0) < cpb ? (n_cells - c0) : cpb;
    stage_cells<D, N, T>(dst, P.src + c0 * NC, ncell, tid, nthr);
    if constexpr (SU) stage_cells<D, N, T>(dstu, P.uin + c0 * NC, ncell, tid, nthr);
  };
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
    cp_async_wait<1>();
    __syncthreads();
    if constexpr (std::is_same_v<A, f32x2>) {
      // FP32x2: the staged input converted to double-word FP32 in place, once per value
      const int nv = cpb * EclTile<D, N, T>::CST;
      for (int i = tid; i < nv; i += nthr) {
        const double v = cur[i];
        reinterpret_cast<f32x2*>(cur)[i] = x2_from_double(v);
      }
      __syncthreads();
      vp_block_x2<D, N, MODE>(P, Lk, b * cpb, lc, tl, cur, s_o);
    } else {
      vp_block<D, N, T, MODE>(P, Lk, b * cpb, lc, tl, cur, s_o, SU ? curu : nullptr);
    }
    __syncthreads();
    odd = !odd;
  }
  cp_async_wait<0>();
}

template <int D, int N, typename T, typename A>
static cudaError_t launch_vp_kernel(const VpAdvParams<T>& P, const VpLine<A>& Lk, int mode, cudaStream_t s) {
  using S = EclShape<D, N, T>;
  const int nbuf = mode == kStageMid ? EclStaging<D, N, T, kStageMid, A>::NBUF
                   : mode == kStageLast ? EclStaging<D, N, T, kStageLast, A>::NBUF : 3;
  // measured on GB300: FP32 is fastest with the largest tile, FP64 with the default one
  int cpb = sizeof(T) == 4 ? S::CPB : ecl_default_cpb<D, N, T>();
  while (cpb > 1 && size_t(nbuf * ecl_buffer_elems<D, N, T>(cpb)) * sizeof(T) > 220 * 1024) --cpb;
  const int threads = S::TPC * cpb;
  const size_t smem = size_t(nbuf * ecl_buffer_elems<D, N, T>(cpb)) * sizeof(T);
  static bool attr_done[4] = {false, false, false, false};
  static int sms = 0;
  auto go = [&](auto kern) -> cudaError_t {
    if (!attr_done[mode]) {
      cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
      if (e != cudaSuccess) return e;
      int dev = 0;
      cudaGetDevice(&dev);
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
      attr_done[mode] = true;
    }
    int per_sm = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) per_sm = 1;
    const long long nblk = (P.g.n_cells + cpb - 1) / cpb;
    const long long want = (long long)sms * per_sm;
    kern<<<unsigned(nblk < want ? nblk : want), threads, smem, s>>>(P, Lk, cpb);
    return cudaGetLastError();
  };
  switch (mode) {
    case kApply: return go(vp_adv_kernel<D, N, T, kApply, A>);
    case kStageFirst: return go(vp_adv_kernel<D, N, T, kStageFirst, A>);
    case kStageMid: return go(vp_adv_kernel<D, N, T, kStageMid, A>);
    default: return go(vp_adv_kernel<D, N, T, kStageLast, A>);
  }
}

// x2: FP64 storage with FP32x2 arithmetic (built for the 1x1v and 2x2v shapes)
template <int D, int N, typename T>
static cudaError_t launch_vp_dn(const VpAdvParams<T>& P, int mode, cudaStream_t s, bool x2) {
  using S = EclShape<D, N, T>;
  if constexpr (!S::SUPPORTED) {
    return cudaErrorNotSupported;
  } else {
    if (mode < kApply || mode > kStageLast) return cudaErrorInvalidValue;
    if (x2) {
      if constexpr (sizeof(T) == 8 && D <= 4) {
        VpLine<f32x2> Lx;
        for (int i = 0; i < N * N; ++i) Lx.G[i] = x2_split_host(P.g.G[i]);
        Lx.winv0 = x2_split_host(1.0 / P.g.glw[0]);
        Lx.winvk = x2_split_host(1.0 / P.g.glw[N - 1]);
        return launch_vp_kernel<D, N, T, f32x2>(P, Lx, mode, s);
      } else {
        return cudaErrorNotSupported;
      }
    }
    VpLine<T> Lk;
    for (int i = 0; i < N * N; ++i) Lk.G[i] = T(P.g.G[i]);
    Lk.winv0 = T(1.0 / P.g.glw[0]);
    Lk.winvk = T(1.0 / P.g.glw[N - 1]);
    return launch_vp_kernel<D, N, T, T>(P, Lk, mode, s);
  }
}

// ---------------------------------------------------------------------------
// Gauss quadrature.  One CTA per cell (grid-stride): the cell's nodal values
// are transformed to the Gauss points (S along every direction), both
// neighbours' traces of every direction are gathered -- the neighbour's
// Gauss-Lobatto end-node slab, S along the tangential directions -- and every
// line of every direction adds (a/h)(A v + c u_up) with the operator of its
// velocity's sign; S^{-1} along every direction takes the result back to
// nodal values.  Shared memory (T): v and r (NC each), the 2D traces (NC/N
// each).  Runtime D and N; this path serves the reference's Gauss cases, not
// the benchmark's collocation meshes.

template <typename T, int MODE>
__global__ void vp_gauss_kernel(VpAdvParams<T> P) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const VpGeom& g = P.g;
  const int D = g.D, N = g.N, NC = g.NC, DX = g.dx, NF = NC / N;
  T* v = reinterpret_cast<T*>(smem_raw);
  T* r = v + NC;
  T* face = r + NC;  // [2 d + side][NF]: side 0 the left neighbour's trace, 1 the right one's
  const int tid = threadIdx.x, nthr = blockDim.x;
  for (long long gid = blockIdx.x; gid < g.n_cells; gid += gridDim.x) {
    int cc[kMaxDim];
    long long nb[kMaxDim][2];
    const long long gx = gid % g.ncx;
    {
      long long a = gx, b = gid / g.ncx;
      for (int d = 0; d < D; ++d) {
        if (d < DX) { cc[d] = int(a % g.cells[d]); a /= g.cells[d]; }
        else { cc[d] = int(b % g.cells[d]); b /= g.cells[d]; }
        const long long cs = g.cstride[d];
        nb[d][0] = cc[d] > 0 ? gid - cs : gid + (long long)(g.cells[d] - 1) * cs;
        nb[d][1] = cc[d] + 1 < g.cells[d] ? gid + cs : gid - (long long)(g.cells[d] - 1) * cs;
      }
    }
    for (int i = tid; i < NC; i += nthr) v[i] = P.src[gid * NC + i];
    // traces: the left neighbour's slab i_d = N-1, the right one's slab i_d = 0,
    // stored with the digit d removed
    for (int k = tid; k < 2 * D * NF; k += nthr) {
      const int fd = k / (2 * NF), side = (k / NF) % 2, l = k % NF;
      int sd = 1;
      for (int f = 0; f < fd; ++f) sd *= N;
      const int node = (l % sd) + (side ? 0 : N - 1) * sd + (l / sd) * sd * N;
      face[k] = P.src[nb[fd][side] * NC + node];
    }
    __syncthreads();
    for (int e = 0; e < D; ++e) {
      vp_line_pass(v, g.S, N, D, e, tid, nthr);
      __syncthreads();
    }
    // tangential S on every trace: face fd, face-local direction t (rank of e != fd)
    for (int t = 0; t < D - 1; ++t) {
      for (int fs = 0; fs < 2 * D; ++fs) vp_line_pass(face + fs * NF, g.S, N, D - 1, t, tid, nthr);
      __syncthreads();
    }
    for (int i = tid; i < NC; i += nthr) r[i] = T(0);
    __syncthreads();
    for (int d = 0; d < D; ++d) {
      int sd = 1;
      for (int f = 0; f < d; ++f) sd *= N;
      for (int line = tid; line < NF; line += nthr) {
        const int base = (line % sd) + (line / sd) * sd * N;  // node of the line with i_d = 0
        // velocity / h of the line: x-direction d moves with v_d at the line's
        // v-point, v-direction d with d_d phi at the line's x-point
        T a;
        if (d < DX) {
          const int e = DX + d;
          int se = 1;
          for (int f = 0; f < e; ++f) se *= N;
          a = __ldg(P.xs + (d * kVpMaxCellsV + cc[e]) * N + (base / se) % N);
        } else {
          int sx = 1;
          for (int f = 0; f < DX; ++f) sx *= N;
          a = __ldg(P.es + (gx * g.NCx + (base % sx)) * DX + (d - DX));
        }
        const bool pos = a > T(0);
        const double* Am = pos ? g.Ap : g.Am;
        const double* cv = pos ? g.cp : g.cm;
        const T up = face[(2 * d + (pos ? 0 : 1)) * NF + line];
        T u[kMaxN];
        for (int j = 0; j < N; ++j) u[j] = v[base + j * sd];
        for (int i = 0; i < N; ++i) {
          T acc = T(cv[i]) * up;
          for (int j = 0; j < N; ++j) acc = fma(T(Am[i * N + j]), u[j], acc);
          r[base + i * sd] += a * acc;
        }
      }
      __syncthreads();
    }
    for (int e = 0; e < D; ++e) {
      vp_line_pass(r, g.Si, N, D, e, tid, nthr);
      __syncthreads();
    }
    for (int i = tid; i < NC; i += nthr) {
      const long long gi = gid * NC + i;
      const T k = r[i];
      if constexpr (MODE == kApply) {
        P.dst[gi] = k;
      } else {
        const T u = (MODE == kStageFirst) ? P.src[gi] : P.uin[gi];
        P.dst[gi] = fma(P.fb, k, u);
        if constexpr (MODE != kStageLast) P.tout[gi] = fma(P.fa, k, u);
      }
    }
    __syncthreads();  // v, r and the traces are reused by the next cell
  }
}

// shared memory of the Gauss kernel for a geometry (bytes)
template <typename T>
static size_t vp_gauss_smem(const VpGeom& g) {
  return sizeof(T) * (size_t(2) * g.NC + size_t(2) * g.D * (g.NC / g.N));
}

template <typename T>
static cudaError_t launch_vp_gauss(const VpAdvParams<T>& P, int mode, cudaStream_t s) {
  const size_t smem = vp_gauss_smem<T>(P.g);
  if (smem > 220 * 1024) return cudaErrorNotSupported;
  const int threads = 128;
  static int sms = 0;
  auto go = [&](auto kern) -> cudaError_t {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess) return e;
    if (!sms) {
      int dev = 0;
      cudaGetDevice(&dev);
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    }
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) per_sm = 1;
    const long long want = (long long)sms * per_sm;
    kern<<<unsigned(P.g.n_cells < want ? P.g.n_cells : want), threads, smem, s>>>(P);
    return cudaGetLastError();
  };
  switch (mode) {
    case kApply: return go(vp_gauss_kernel<T, kApply>);
    case kStageFirst: return go(vp_gauss_kernel<T, kStageFirst>);
    case kStageMid: return go(vp_gauss_kernel<T, kStageMid>);
    case kStageLast: return go(vp_gauss_kernel<T, kStageLast>);
    default: return cudaErrorInvalidValue;
  }
}

template <typename T>
static cudaError_t launch_vp_any(const VpAdvParams<T>& P, int mode, cudaStream_t s, bool x2) {
  if (P.g.gauss) return x2 ? cudaErrorNotSupported : launch_vp_gauss(P, mode, s);
#define HD_VP_CASE(DD, NN) \
  if (P.g.D == DD && P.g.N == NN) return launch_vp_dn<DD, NN, T>(P, mode, s, x2);
  HD_VP_CASE(2, 2) HD_VP_CASE(2, 3) HD_VP_CASE(2, 4) HD_VP_CASE(2, 5) HD_VP_CASE(2, 6)
  HD_VP_CASE(4, 2) HD_VP_CASE(4, 3) HD_VP_CASE(4, 4) HD_VP_CASE(4, 5) HD_VP_CASE(4, 6)
  HD_VP_CASE(6, 2) HD_VP_CASE(6, 3) HD_VP_CASE(6, 4)
#undef HD_VP_CASE
  return cudaErrorNotSupported;
}

cudaError_t launch_vp_advection(const VpAdvParams<float>& P, int mode, cudaStream_t s) {
  return launch_vp_any(P, mode, s, false);
}

bool vp_pipe_eligible(const VpGeom& g) {
  return !g.gauss && g.D == 4 && g.N == 4 && g.cells[0] == 16 && g.n_cells * 256LL < (1LL << 36);
}

cudaError_t launch_vp_pipelined(const VpAdvParams<float>& P, int mode, cudaStream_t s, int* state,
                                unsigned wait_limit, int skip_issue) {
  if (!vp_pipe_eligible(P.g)) return cudaErrorNotSupported;
  if (mode < kApply || mode > kStageLast) return cudaErrorInvalidValue;
  VpPipeParams Q;
  Q.a = P;
  for (int i = 0; i < 16; ++i) Q.G[i] = float(P.g.G[i]);
  Q.winv0 = float(1.0 / P.g.glw[0]);
  Q.winvk = float(1.0 / P.g.glw[3]);
  Q.n_units = int(P.g.n_cells / 16);
  Q.err = state;
  Q.ticket = state + 1;
  Q.wait_limit = wait_limit ? wait_limit : E6_WAIT_LIMIT;
  Q.skip_issue = skip_issue;
  Ecl6Maps maps;
  cudaError_t e = encode_ecl6_maps(P.src, P.uin ? P.uin : P.src, P.g.n_cells * 256LL, &maps);
  if (e != cudaSuccess) return e;
  static bool attr_done[4] = {false, false, false, false};
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  }
  const int grid = 2 * sms < Q.n_units ? 2 * sms : Q.n_units;
  auto go = [&](auto kern) -> cudaError_t {
    if (!attr_done[mode]) {
      cudaError_t ee = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, E6_SMEM);
      if (ee != cudaSuccess) return ee;
      attr_done[mode] = true;
    }
    cudaError_t ee = cudaMemsetAsync(Q.ticket, 0, sizeof(int), s);
    if (ee != cudaSuccess) return ee;
    kern<<<grid, E6_THREADS, E6_SMEM, s>>>(Q, maps);
    return cudaGetLastError();
  };
  switch (mode) {
    case kApply: return go(vp_pipe_kernel<kApply>);
    case kStageFirst: return go(vp_pipe_kernel<kStageFirst>);
    case kStageMid: return go(vp_pipe_kernel<kStageMid>);
    default: return go(vp_pipe_kernel<kStageLast>);
  }
}
cudaError_t launch_vp_advection(const VpAdvParams<double>& P, int mode, cudaStream_t s, bool x2) {
  return launch_vp_any(P, mode, s, x2);
}

}  // namespace hd
