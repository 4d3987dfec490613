// hd_vp_pipe.cuh -- the TMA-pipelined kernel of hd_ecl6.cuh carried over to the
// Vlasov-Poisson advection: 2x+2v, degree 3, FP32 storage, 16 cells along x0.
//
// The unit is one x0-row of 16 cells (4,096 values, the layout of one 6D
// cell), staged by the producer warp through the same 2-slot mbarrier ring as
// the 2D TMA tile with the 128-byte swizzle, together with the RK solution
// tile and the traces of BOTH neighbours along v0 and v1 (the velocity of a
// v-line is the field at its x-point, whose sign changes inside a unit, so
// each line picks its upwind side): the 6D x2 / v0 face boxes of the left
// neighbour's slab k and the right neighbour's slab 0.  The x0 traces are
// cells of the unit itself (a unit is a whole periodic x0-row), the x1 traces
// of both neighbouring units two 128-bit loads issued one unit ahead.
//
// Every line of direction d adds (a/h) [G u + upwind face terms] as the
// collocation kernel of hd_vp_adv.cu does, with a the line's velocity: v_d at
// the line's v-node for the x-directions (xs), d_d phi at its x-node for the
// v-directions (es).  A thread's plane shares one velocity per direction, so
// each thread reads two scales per phase.  The upwind side is applied without
// a branch: with a+ = max(a, 0), a- = min(a, 0) the terms a+ / w_0 u_left and
// a- / w_0 u_0 at node 0, -a+ / w_k u_k and -a- / w_k u_right at node k,
// one of each pair being an exact zero -- the same rounding as the branchy
// form.  Bounded waits, time-out, abort and drain as hd::ecl6_kernel.
#pragma once

#include "hd_ecl6.cuh"
#include "hd_vp.cuh"

namespace hd {

struct VpPipeParams {
  VpAdvParams<float> a;  // vectors, stage factors, velocity tables, geometry
  float G[16];           // line matrix G[i*4 + q] (hd_vp.cuh VpGeom::G)
  float winv0, winvk;    // 1/w_0, 1/w_3
  int n_units;           // x0-rows of 16 cells
  int* err;              // device error flag (E6_ERR_*)
  int* ticket;           // next unclaimed unit (zeroed before every launch)
  unsigned wait_limit;   // try_wait rounds of every bounded wait
  int skip_issue;        // test hook: 0 = the producer holding unit 0 issues nothing for it; -1 = off
};

// neighbour unit of unit r along direction d (1: x1, 2: v0, 3: v1), periodic
__device__ __forceinline__ int vpp_neighbour(const VpGeom& g, int r, int d, int step) {
  const int c1n = g.cells[1], c2n = g.cells[2], c3n = g.cells[3];
  const int c1 = r % c1n, c2 = (r / c1n) % c2n, c3 = r / (c1n * c2n);
  int c = d == 1 ? c1 : (d == 2 ? c2 : c3);
  const int n = d == 1 ? c1n : (d == 2 ? c2n : c3n);
  const int us = d == 1 ? 1 : (d == 2 ? c1n : c1n * c2n);
  int cn = c + step;
  cn = cn < 0 ? n - 1 : (cn >= n ? 0 : cn);
  return r + (cn - c) * us;
}

template <int MODE>
__global__ void __maxnreg__(104) vp_pipe_kernel(const __grid_constant__ VpPipeParams P,
                                                const __grid_constant__ Ecl6Maps maps) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  constexpr bool READ_U = (MODE == kStageMid || MODE == kStageLast);
  if (smem_u32(smem_raw) & 1023u) {
    if (threadIdx.x == 0) atomicExch(P.err, E6_ERR_SMEM_ALIGN);
    return;
  }
  float* s_stage = reinterpret_cast<float*>(smem_raw);
  float* so = reinterpret_cast<float*>(smem_raw + E6_STAGES * E6_STAGE_BYTES);
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem_raw + E6_STAGES * E6_STAGE_BYTES + E6_OUT_BYTES);
  uint64_t* full = bars;
  uint64_t* empty = bars + E6_STAGES;
  volatile int* s_abort = reinterpret_cast<volatile int*>(bars + 2 * E6_STAGES);
  volatile int* s_rows = reinterpret_cast<volatile int*>(bars + 2 * E6_STAGES) + 2;
  volatile int* s_cont = s_rows + 4;
  const VpGeom& g = P.a.g;

  const int tid = threadIdx.x;
  if (tid == 0) {
    for (int s = 0; s < E6_STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], E6_CTHREADS / 32);
    }
    *s_abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();

  if (tid >= E6_CTHREADS) {
    // ------------------------------------------------------------------ producer
    if (tid == E6_CTHREADS) {
      int issued = 0;
      bool ok = true;
      const uint64_t pol_u = l2_evict_first_policy();
      const uint32_t bytes = 16384u + (READ_U ? 16384u : 0u) + 4u * 4096u;
      auto take = [&]() -> int {
        const int t = atomicAdd(P.ticket, 1);
        return t < P.n_units ? t : -1;
      };
      int q = 0;
      int r = take();
      s_rows[0] = r;
      s_rows[1] = r >= 0 ? take() : -1;
      if (r < 0) mbar_arrive(&full[0]);  // no unit for this CTA: release the compute warps
      for (int it = 0; r >= 0; ++it) {
        const int s = it % E6_STAGES;
        if (it >= E6_STAGES && !mbar_wait(&empty[s], ((it / E6_STAGES) - 1) & 1, P.wait_limit)) {
          atomicExch(P.err, E6_ERR_TIMEOUT_EMPTY);
          *s_abort = 1;
          ok = false;
          break;
        }
        if (*s_abort) { ok = false; break; }
        if (q > 0) {
          r = s_rows[q % 4];
          if (r < 0) break;
          s_rows[(q + 1) % 4] = take();
        }
        float* st = s_stage + s * E6_STAGE_FLOATS;
        if (P.skip_issue == 0 && r == 0) {
          // test hook: nothing arrives on this slot, its consumers' bounded wait runs out
          ++issued;
          ++q;
          continue;
        }
        const int nl2 = vpp_neighbour(g, r, 2, -1), nr2 = vpp_neighbour(g, r, 2, 1);
        const int nl3 = vpp_neighbour(g, r, 3, -1), nr3 = vpp_neighbour(g, r, 3, 1);
        mbar_arrive_expect_tx(&full[s], bytes);
        tma_load_2d(st, &maps.tcell, 0, r * 128, &full[s]);
        if (READ_U) tma_load_2d_hint(st + 4096, &maps.ucell, 0, r * 128, &full[s], pol_u);
        // v0 traces: left neighbour's slab 3, right neighbour's slab 0 (boxes [64][1][16])
        tma_load_3d(st + 8192, &maps.tx2, 0, 3, nl2 * 64, &full[s]);
        tma_load_3d(st + 9216, &maps.tx2, 0, 0, nr2 * 64, &full[s]);
        // v1 traces (boxes [16][1][64])
        tma_load_3d(st + 10240, &maps.tv0, 0, 3, nl3 * 16, &full[s]);
        tma_load_3d(st + 11264, &maps.tv0, 0, 0, nr3 * 16, &full[s]);
        ++issued;
        ++q;
      }
      if (!ok) {
        for (int it = issued - E6_STAGES < 0 ? 0 : issued - E6_STAGES; it < issued; ++it)
          mbar_wait(&full[it % E6_STAGES], (it / E6_STAGES) & 1, P.wait_limit);
      }
    }
    return;
  }

  // -------------------------------------------------------------------- consumers
  const int lane = tid & 31, warp = tid >> 5;
  // phase 0: plane 16*tid + i0 + 4 i1 of cell c = tid >> 4 (item i2 + 4 i3 = tid & 15)
  const int row0 = tid >> 1;
  const int t0_chunk = (4 * (tid & 1)) ^ (row0 & 7);
  const int o0_chunk = (4 * (tid & 1)) ^ (row0 & 7) ^ (((row0 >> 3) & 1) << 2);
  const int c0 = tid >> 4, item = tid & 15;
  // phase 1: nodes (lo + 256 hi) + 16 i2 + 64 i3, lo = i0 + 4 i1, hi = c0
  const int lo = tid & 15, hi = tid >> 4;
  int tb1[4], ob1[4][2];
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    tb1[r] = 256 * hi + (lo & 3) + 4 * ((lo >> 2) ^ r);
    ob1[r][0] = tb1[r] + 16 * (hi & 1);
    ob1[r][1] = tb1[r] + 16 - 16 * (hi & 1);
  }
  const int vnode = 4 * (lane & 7) + 32 * warp + 256 * (lane >> 3);
  const int vt = 32 * warp + 256 * (lane >> 3) + (((lane & 7) ^ warp) << 2);
  const int vo = 32 * warp + 256 * (lane >> 3) + (((lane & 7) ^ warp ^ (4 * ((lane >> 3) & 1))) << 2);
  const float w0 = P.winv0, wk = P.winvk;
  const int C1 = g.cells[1], C2 = g.cells[2];

  float4 x1l = make_float4(0.f, 0.f, 0.f, 0.f), x1r = x1l;  // x1 traces of this thread's plane
  auto fetch_x1 = [&](int r) {
    const int nl = vpp_neighbour(g, r, 1, -1), nr = vpp_neighbour(g, r, 1, 1);
    x1l = __ldg(reinterpret_cast<const float4*>(P.a.src + (long long)nl * 4096 + 16 * tid + 12));
    x1r = __ldg(reinterpret_cast<const float4*>(P.a.src + (long long)nr * 4096 + 16 * tid));
  };

  if (lane == 0 && !mbar_wait(&full[0], 0, P.wait_limit)) {
    *s_abort = 1;
    atomicExch(P.err, E6_ERR_TIMEOUT_FULL);
  }
  __syncwarp();
  if (tid == 0) s_cont[0] = (!*s_abort && s_rows[0] >= 0) ? 1 : 0;
  bar_compute();
  if (!s_cont[0]) return;
  int q = 0;
  int r = s_rows[0];
  fetch_x1(r);
  for (int it = 0;; ++it) {
    const int s = it % E6_STAGES;
    const float* st = s_stage + s * E6_STAGE_FLOATS;
    if (lane == 0 && !*s_abort && !mbar_wait(&full[s], (it / E6_STAGES) & 1, P.wait_limit)) {
      *s_abort = 1;
      atomicExch(P.err, E6_ERR_TIMEOUT_FULL);
    }
    __syncwarp();
    const int next_row = s_rows[(q + 1) % 4];
    const bool has_next = next_row >= 0;
    const int c1 = r % C1, c2 = (r / C1) % C2, c3 = r / (C1 * C2);

    // ---------------- phase 0: x0 (a, along i0) and x1 (b, along i1)
    {
      float uu[4][4], acc[4][4];
#pragma unroll
      for (int b = 0; b < 4; ++b) {
        const float4 v = *reinterpret_cast<const float4*>(st + row0 * 32 + ((t0_chunk ^ b) << 2));
        uu[0][b] = v.x; uu[1][b] = v.y; uu[2][b] = v.z; uu[3][b] = v.w;
      }
      // velocities / h: v_0 at the plane's v0-node i2, v_1 at its v1-node i3
      const float sa = __ldg(P.a.xs + (0 * kVpMaxCellsV + c2) * 4 + (item & 3));
      const float sb = __ldg(P.a.xs + (1 * kVpMaxCellsV + c3) * 4 + (item >> 2));
      const float ap = fmaxf(sa, 0.f), am = fminf(sa, 0.f);
      const int nl = (((c0 + 15) & 15) << 8) + (item << 4) + 3, nr = (((c0 + 1) & 15) << 8) + (item << 4);
#pragma unroll
      for (int b = 0; b < 4; ++b) {
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          float sacc = 0.f;
#pragma unroll
          for (int qq = 0; qq < 4; ++qq) sacc = fmaf(P.G[i * 4 + qq], uu[qq][b], sacc);
          acc[i][b] = fmaf(sa, sacc, 0.f);
        }
        const float fl = st[swz_t(nl + 4 * b)], fr = st[swz_t(nr + 4 * b)];
        acc[3][b] = fmaf(-am * wk, fr, fmaf(-ap * wk, uu[3][b], acc[3][b]));
        acc[0][b] = fmaf(ap * w0, fl, fmaf(am * w0, uu[0][b], acc[0][b]));
      }
      const float bp = fmaxf(sb, 0.f), bm = fminf(sb, 0.f);
      const float xl[4] = {x1l.x, x1l.y, x1l.z, x1l.w}, xr[4] = {x1r.x, x1r.y, x1r.z, x1r.w};
#pragma unroll
      for (int a = 0; a < 4; ++a) {
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          float sacc = 0.f;
#pragma unroll
          for (int qq = 0; qq < 4; ++qq) sacc = fmaf(P.G[i * 4 + qq], uu[a][qq], sacc);
          acc[a][i] = fmaf(sb, sacc, acc[a][i]);
        }
        acc[a][3] = fmaf(-bm * wk, xr[a], fmaf(-bp * wk, uu[a][3], acc[a][3]));
        acc[a][0] = fmaf(bp * w0, xl[a], fmaf(bm * w0, uu[a][0], acc[a][0]));
      }
#pragma unroll
      for (int b = 0; b < 4; ++b)
        *reinterpret_cast<float4*>(so + row0 * 32 + ((o0_chunk ^ b) << 2)) =
            make_float4(acc[0][b], acc[1][b], acc[2][b], acc[3][b]);
    }
    if (has_next) fetch_x1(next_row);
    bar_compute();

    // ---------------- phase 1: v0 (a, along i2) and v1 (b, along i3)
    {
      float uu[4][4], acc[4][4];
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) {
          const int Rr = (a >> 1) + 2 * b;
          const int e = (a & 1) ^ (Rr >> 2);
          uu[a][b] = st[tb1[Rr & 3] + 32 * Rr + 16 * e];
          acc[a][b] = so[ob1[Rr & 3][e] + 32 * Rr];
        }
      // velocities / h: d_d phi at the plane's x-node (x-cell c0 + 16 c1, node lo)
      const float* es = P.a.es + ((long long)(hi + 16 * c1) * 16 + lo) * 2;
      const float sa = __ldg(es), sb = __ldg(es + 1);
      const float ap = fmaxf(sa, 0.f), am = fminf(sa, 0.f);
      const float* tl2 = st + 8192 + 64 * hi + lo;
      const float* tr2 = st + 9216 + 64 * hi + lo;
#pragma unroll
      for (int b = 0; b < 4; ++b) {
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          float sacc = 0.f;
#pragma unroll
          for (int qq = 0; qq < 4; ++qq) sacc = fmaf(P.G[i * 4 + qq], uu[qq][b], sacc);
          acc[i][b] = fmaf(sa, sacc, acc[i][b]);
        }
        acc[3][b] = fmaf(-am * wk, tr2[16 * b], fmaf(-ap * wk, uu[3][b], acc[3][b]));
        acc[0][b] = fmaf(ap * w0, tl2[16 * b], fmaf(am * w0, uu[0][b], acc[0][b]));
      }
      const float bp = fmaxf(sb, 0.f), bm = fminf(sb, 0.f);
      const float* tl3 = st + 10240 + 64 * hi + lo;
      const float* tr3 = st + 11264 + 64 * hi + lo;
#pragma unroll
      for (int a = 0; a < 4; ++a) {
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          float sacc = 0.f;
#pragma unroll
          for (int qq = 0; qq < 4; ++qq) sacc = fmaf(P.G[i * 4 + qq], uu[a][qq], sacc);
          acc[a][i] = fmaf(sb, sacc, acc[a][i]);
        }
        acc[a][3] = fmaf(-bm * wk, tr3[16 * a], fmaf(-bp * wk, uu[a][3], acc[a][3]));
        acc[a][0] = fmaf(bp * w0, tl3[16 * a], fmaf(bm * w0, uu[a][0], acc[a][0]));
      }
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) {
          const int Rr = (a >> 1) + 2 * b;
          const int e = (a & 1) ^ (Rr >> 2);
          so[ob1[Rr & 3][e] + 32 * Rr] = acc[a][b];
        }
    }
    bar_compute();

    // ---------------- epilogue: K or the fused stage update, 128-bit stores
    {
      float4 uv[4];
      if constexpr (MODE != kApply) {
        const float* ut = READ_U ? st + 4096 : st;
#pragma unroll
        for (int j = 0; j < 4; ++j) uv[j] = *reinterpret_cast<const float4*>(ut + vt + 1024 * j);
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(&empty[s]);
      if (!*s_abort) {
        float4* go = reinterpret_cast<float4*>(P.a.dst + (long long)r * 4096 + vnode);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const float4 kv = *reinterpret_cast<const float4*>(so + vo + 1024 * j);
          if constexpr (MODE == kApply) {
            __stcs(go + 256 * j, kv);
          } else {
            const float4 u = uv[j];
            __stcs(go + 256 * j, make_float4(fmaf(P.a.fb, kv.x, u.x), fmaf(P.a.fb, kv.y, u.y),
                                             fmaf(P.a.fb, kv.z, u.z), fmaf(P.a.fb, kv.w, u.w)));
            if constexpr (MODE != kStageLast) {
              float4* gt = reinterpret_cast<float4*>(P.a.tout + (long long)r * 4096 + vnode);
              __stcs(gt + 256 * j, make_float4(fmaf(P.a.fa, kv.x, u.x), fmaf(P.a.fa, kv.y, u.y),
                                               fmaf(P.a.fa, kv.z, u.z), fmaf(P.a.fa, kv.w, u.w)));
            }
          }
        }
      }
    }
    if (tid == 0) s_cont[(it + 1) & 1] = (!*s_abort && has_next) ? 1 : 0;
    bar_compute();
    if (!s_cont[(it + 1) & 1]) break;
    ++q;
    r = next_row;
  }
}

}  // namespace hd
