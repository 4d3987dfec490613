// hd_ecl6.cuh -- persistent, TMA-pipelined ECL kernel for the 6D (3x+3v),
// degree-3 (4 nodes per direction), FP32-storage case, all faces periodic.
//
// Structure (one CTA per SM slot, 8 compute warps + 1 producer warp):
//   * Work item = one x0-row of cells (consecutive cell ids).  A CTA walks the
//     row in the upwind order of direction x0, so the x0 face trace a cell
//     needs is the previous cell's face, which the thread owning that plane
//     still holds in registers ("carry"); only a row's first cell reads it
//     from global memory.
//   * The producer warp streams, per cell, through a 2-stage ring guarded by
//     mbarriers: the cell's 4096 values as one 2D TMA tile with the 128-byte
//     swizzle (conflict-free plane reads), the upwind face traces of x1, x2,
//     v0, v1 as one 3D TMA box each, and the v2 trace (contiguous) as one 1D
//     bulk copy.
//   * The compute warps apply the line operators two directions per phase
//     (x0x1, x2v0, v1v2) with an XOR-swizzled accumulator tile in shared
//     memory; the last phase writes K or the fused LSRK update with coalesced
//     stores.  U (own nodes) is prefetched into registers at the cell start.
//   * Every mbarrier wait is bounded: on time-out the kernel records an
//     error code, drains its own in-flight copies (bounded) and returns.
//
// Reference operator: include/hyper.deal/operators/advection/
// advection_operation.h:218-566; LSRK stage: base/time_integrators.templates.h:111-135.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "hd_ecl.cuh"

namespace hd {

struct Ecl6Maps {
  CUtensorMap tcell;  // vector as [n/32][32] floats, box [128][32], 128B swizzle
  CUtensorMap tr[4];  // traces of x1, x2, v0, v1: [n/S][4][S], box [256/S... ][1][S]
};

constexpr int E6_CTHREADS = 256;  // compute threads
constexpr int E6_THREADS = 288;   // + one producer warp
constexpr int E6_STAGES = 2;
constexpr int E6_STAGE_BYTES = 16384 + 5 * 4096;  // cell tile + 5 traces
constexpr int E6_OUT_BYTES = 2 * 16384;  // double-buffered accumulator tile
constexpr int E6_SMEM = 1024 /*alignment slack*/ + E6_STAGES * E6_STAGE_BYTES + E6_OUT_BYTES + 64;
constexpr unsigned E6_WAIT_LIMIT = 1u << 22;  // try_wait rounds before giving up (~seconds)

enum : int { E6_ERR_TIMEOUT_FULL = 1, E6_ERR_TIMEOUT_EMPTY = 2 };

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(
                   smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

// bounded wait for the phase with the given parity; false on time-out
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  const uint32_t a = smem_u32(bar);
  for (uint32_t it = 0; it < E6_WAIT_LIMIT; ++it) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          smem_u32(dst)),
      "l"(map), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int x, int y, int z, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(
          smem_u32(dst)),
      "l"(map), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void bar_compute() { asm volatile("bar.sync 1, 256;" ::: "memory"); }

// float offset of node i in the TMA 128B-swizzled cell tile ([128 rows][32 floats])
__device__ __forceinline__ int swz_t(int i) {
  const int row = i >> 5;
  return (i & ~28) | ((((i >> 2) & 7) ^ (row & 7)) << 2);
}
// float offset of node i in the accumulator tile: chunk ^= (row & 7) ^ (bit 3 of row) << 2
__device__ __forceinline__ int swz_o(int i) {
  const int row = i >> 5;
  const int x = (row & 7) ^ (((row >> 3) & 1) << 2);
  return (i & ~28) | ((((i >> 2) & 7) ^ x) << 2);
}

struct Ecl6Params {
  EclParams<float> p;  // operator, mesh, vectors, stage factors
  int n_rows;          // x0-rows of cells
  int row_len;         // cells per row (cells in x0)
  int* err;            // device error flag
};

// cell id of the k-th cell of row r in the row's upwind traversal order
__device__ __forceinline__ long long e6_cell(const Ecl6Params& P, int r, int k) {
  const int c = P.p.op[0].step < 0 ? k : (P.row_len - 1 - k);
  return (long long)r * P.row_len + c;
}

// upwind neighbour of `gid` in direction d on the fully periodic mesh
__device__ __forceinline__ long long e6_nb(const Ecl6Params& P, long long gid, int d) {
  const long long cs = P.p.cstride[d];
  const int nc = P.p.cells[d];
  const int c = int((gid / cs) % nc);
  const int step = P.p.op[d].step;
  const int cn = c + step;
  if (cn < 0) return gid + (long long)(nc - 1) * cs;
  if (cn >= nc) return gid - (long long)(nc - 1) * cs;
  return gid + step * cs;
}

template <int MODE>
__global__ void __launch_bounds__(E6_THREADS, 2) ecl6_kernel(const __grid_constant__ Ecl6Params P,
                                                             const __grid_constant__ Ecl6Maps maps) {
  extern __shared__ unsigned char smem_raw[];
  unsigned char* base = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  float* s_stage = reinterpret_cast<float*>(base);
  float* s_out = reinterpret_cast<float*>(base + E6_STAGES * E6_STAGE_BYTES);  // 2 accumulator tiles
  uint64_t* bars = reinterpret_cast<uint64_t*>(base + E6_STAGES * E6_STAGE_BYTES + E6_OUT_BYTES);
  uint64_t* full = bars;               // [E6_STAGES]: TMA bytes landed
  uint64_t* empty = bars + E6_STAGES;  // [E6_STAGES]: all 8 compute warps done with the slot
  volatile int* s_abort = reinterpret_cast<volatile int*>(bars + 2 * E6_STAGES);

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

  const int n_my_rows = P.n_rows > (int)blockIdx.x ? (P.n_rows - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
  const int n_cells_cta = n_my_rows * P.row_len;

  if (tid >= E6_CTHREADS) {
    // ------------------------------------------------------------------ producer
    if (tid == E6_CTHREADS) {
      int issued = 0;
      bool ok = true;
      uint32_t bytes = 16384;
#pragma unroll
      for (int d = 1; d < 6; ++d) bytes += P.p.op[d].active ? 4096u : 0u;
      for (int it = 0; it < n_cells_cta; ++it) {
        const int s = it % E6_STAGES;
        if (it >= E6_STAGES && !mbar_wait(&empty[s], ((it / E6_STAGES) - 1) & 1)) {
          atomicExch(P.err, E6_ERR_TIMEOUT_EMPTY);
          *s_abort = 1;
          ok = false;
          break;
        }
        if (*s_abort) { ok = false; break; }
        const int r = (int)blockIdx.x + (it / P.row_len) * (int)gridDim.x;
        const long long gid = e6_cell(P, r, it % P.row_len);
        float* st = s_stage + s * (E6_STAGE_BYTES / 4);
        mbar_arrive_expect_tx(&full[s], bytes);
        tma_load_2d(st, &maps.tcell, 0, int(gid * 128), &full[s]);
        // upwind traces (face node nb_node of the upwind neighbour)
#pragma unroll
        for (int d = 1; d < 5; ++d)
          if (P.p.op[d].active)
            tma_load_3d(st + 4096 + (d - 1) * 1024, &maps.tr[d - 1], 0, P.p.op[d].nb_node,
                        int(e6_nb(P, gid, d) * (256 >> (2 * (d - 1)))), &full[s]);
        if (P.p.op[5].active)
          bulk_load(st + 4096 + 4 * 1024, P.p.tin + e6_nb(P, gid, 5) * 4096 + P.p.op[5].nb_node * 1024, 4096u,
                    &full[s]);
        ++issued;
      }
      // on an abort, wait (bounded) for the copies still in flight before leaving
      if (!ok) {
        for (int it = issued - E6_STAGES < 0 ? 0 : issued - E6_STAGES; it < issued; ++it)
          mbar_wait(&full[it % E6_STAGES], (it / E6_STAGES) & 1);
      }
    }
    return;
  }

  // -------------------------------------------------------------------- consumers
  const LineOp<float>* L = P.p.op;
  float carry[4] = {0.f, 0.f, 0.f, 0.f};
  constexpr long long NC = 4096;
  const int lane = tid & 31, warp = tid >> 5;

  // per-thread shared-memory offsets (floats); the compile-time parts are added per access
  // phase 0: plane 16*tid + a + 4b, rows tid>>1 of the swizzled tiles
  const int row0 = tid >> 1;
  const int t0_chunk = (4 * (tid & 1)) ^ (row0 & 7);
  const int o0_chunk = (4 * (tid & 1)) ^ (row0 & 7) ^ (((row0 >> 3) & 1) << 2);
  // phase 1: nodes (lo + 256 hi) + 16a + 64b; R = (a>>1) + 2b picks the row, a&1 the chunk bit 2
  const int lo = tid & 15, hi = tid >> 4;
  int tb1[4], ob1[4][2];
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    tb1[r] = 256 * hi + (lo & 3) + 4 * ((lo >> 2) ^ r);
    ob1[r][0] = tb1[r] + 16 * (hi & 1);
    ob1[r][1] = tb1[r] + 16 - 16 * (hi & 1);
  }
  // phase 2: nodes tid + 256a + 1024b; row & 7 = warp
  const int tb2 = (tid & ~28) | ((((tid >> 2) & 7) ^ warp) << 2);
  const int ob2[2] = {tb2, (tid & ~28) | ((((tid >> 2) & 7) ^ warp ^ 4) << 2)};

  for (int it = 0; it < n_cells_cta; ++it) {
    const int s = it % E6_STAGES;
    const int k = it % P.row_len;
    const int r = (int)blockIdx.x + (it / P.row_len) * (int)gridDim.x;
    const long long gid = e6_cell(P, r, k);
    const float* st = s_stage + s * (E6_STAGE_BYTES / 4);
    float* so = s_out + (it & 1) * 4096;

    // row start: x0 face of the upwind neighbour of the row's first cell
    if (k == 0 && L[0].active) {
      const float* src = P.p.tin + e6_nb(P, gid, 0) * NC + 16 * tid + L[0].nb_node;
#pragma unroll
      for (int b = 0; b < 4; ++b) carry[b] = __ldg(src + 4 * b);
    }
    // U at this thread's phase-2 nodes
    float uU[16];
    if constexpr (MODE == kStageMid || MODE == kStageLast) {
      const float* up = P.p.uin + gid * NC + tid;
#pragma unroll
      for (int b = 0; b < 4; ++b)
#pragma unroll
        for (int a = 0; a < 4; ++a) uU[a + 4 * b] = __ldg(up + 256 * a + 1024 * b);
    }

    // every compute thread waits for the slot (bounded); a time-out turns the
    // rest of the CTA's work into no-ops (no stores) without leaving any barrier
    if (!*s_abort && !mbar_wait(&full[s], (it / E6_STAGES) & 1)) {
      *s_abort = 1;
      atomicExch(P.err, E6_ERR_TIMEOUT_FULL);
    }

    // ---------------- phase 0: directions x0 (a) and x1 (b); plane = nodes 16*tid + a + 4b
    {
      float uu[4][4], acc[4][4];
#pragma unroll
      for (int b = 0; b < 4; ++b) {
        const float4 v = *reinterpret_cast<const float4*>(st + row0 * 32 + ((t0_chunk ^ b) << 2));
        uu[0][b] = v.x; uu[1][b] = v.y; uu[2][b] = v.z; uu[3][b] = v.w;
      }
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] = 0.f;
      if (L[0].active) {
#pragma unroll
        for (int b = 0; b < 4; ++b) {
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            float sacc = 0.f;
#pragma unroll
            for (int q = 0; q < 4; ++q) sacc = fmaf(L[0].M[i * 4 + q], uu[q][b], sacc);
            acc[i][b] = sacc;
          }
          const float up = carry[b];
          acc[0][b] = fmaf(L[0].c0, up, acc[0][b]);
          acc[3][b] = fmaf(L[0].cl, up, acc[3][b]);
        }
        // the next cell in traversal order needs this cell's face nb_node
#pragma unroll
        for (int b = 0; b < 4; ++b) carry[b] = L[0].nb_node ? uu[3][b] : uu[0][b];
      }
      if (L[1].active) {
        const float4 t1 = *reinterpret_cast<const float4*>(st + 4096 + 4 * tid);
        const float upv[4] = {t1.x, t1.y, t1.z, t1.w};
#pragma unroll
        for (int a = 0; a < 4; ++a) {
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            float sacc = acc[a][i];
#pragma unroll
            for (int q = 0; q < 4; ++q) sacc = fmaf(L[1].M[i * 4 + q], uu[a][q], sacc);
            acc[a][i] = sacc;
          }
          acc[a][0] = fmaf(L[1].c0, upv[a], acc[a][0]);
          acc[a][3] = fmaf(L[1].cl, upv[a], acc[a][3]);
        }
      }
#pragma unroll
      for (int b = 0; b < 4; ++b)
        *reinterpret_cast<float4*>(so + row0 * 32 + ((o0_chunk ^ b) << 2)) =
            make_float4(acc[0][b], acc[1][b], acc[2][b], acc[3][b]);
    }
    bar_compute();

    // ---------------- phase 1: directions x2 (a, stride 16) and v0 (b, stride 64)
    {
      float uu[4][4], acc[4][4];
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) {
          const int R = (a >> 1) + 2 * b;
          const int e = (a & 1) ^ (R >> 2);
          uu[a][b] = st[tb1[R & 3] + 32 * R + 16 * e];
          acc[a][b] = so[ob1[R & 3][e] + 32 * R];
        }
      if (L[2].active) {
        const float* tr = st + 5120 + 64 * hi + lo;
#pragma unroll
        for (int b = 0; b < 4; ++b) {
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            float sacc = acc[i][b];
#pragma unroll
            for (int q = 0; q < 4; ++q) sacc = fmaf(L[2].M[i * 4 + q], uu[q][b], sacc);
            acc[i][b] = sacc;
          }
          const float up = tr[16 * b];
          acc[0][b] = fmaf(L[2].c0, up, acc[0][b]);
          acc[3][b] = fmaf(L[2].cl, up, acc[3][b]);
        }
      }
      if (L[3].active) {
        const float* tr = st + 6144 + 64 * hi + lo;
#pragma unroll
        for (int a = 0; a < 4; ++a) {
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            float sacc = acc[a][i];
#pragma unroll
            for (int q = 0; q < 4; ++q) sacc = fmaf(L[3].M[i * 4 + q], uu[a][q], sacc);
            acc[a][i] = sacc;
          }
          const float up = tr[16 * a];
          acc[a][0] = fmaf(L[3].c0, up, acc[a][0]);
          acc[a][3] = fmaf(L[3].cl, up, acc[a][3]);
        }
      }
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) {
          const int R = (a >> 1) + 2 * b;
          const int e = (a & 1) ^ (R >> 2);
          so[ob1[R & 3][e] + 32 * R] = acc[a][b];
        }
    }
    bar_compute();

    // ---------------- phase 2: directions v1 (a, stride 256) and v2 (b, stride 1024), epilogue
    {
      float uu[4][4], acc[4][4];
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) {
          uu[a][b] = st[tb2 + 256 * a + 1024 * b];
          acc[a][b] = so[ob2[a & 1] + 256 * a + 1024 * b];
        }
      if (L[4].active) {
        const float* tr = st + 7168 + tid;
#pragma unroll
        for (int b = 0; b < 4; ++b) {
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            float sacc = acc[i][b];
#pragma unroll
            for (int q = 0; q < 4; ++q) sacc = fmaf(L[4].M[i * 4 + q], uu[q][b], sacc);
            acc[i][b] = sacc;
          }
          const float up = tr[256 * b];
          acc[0][b] = fmaf(L[4].c0, up, acc[0][b]);
          acc[3][b] = fmaf(L[4].cl, up, acc[3][b]);
        }
      }
      if (L[5].active) {
        const float* tr = st + 8192 + tid;
#pragma unroll
        for (int a = 0; a < 4; ++a) {
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            float sacc = acc[a][i];
#pragma unroll
            for (int q = 0; q < 4; ++q) sacc = fmaf(L[5].M[i * 4 + q], uu[a][q], sacc);
            acc[a][i] = sacc;
          }
          const float up = tr[256 * a];
          acc[a][0] = fmaf(L[5].c0, up, acc[a][0]);
          acc[a][3] = fmaf(L[5].cl, up, acc[a][3]);
        }
      }
      // this warp is done with the stage slot
      __syncwarp();
      if (lane == 0) mbar_arrive(&empty[s]);
      if (!*s_abort) {
        float* go = P.p.uout + gid * NC + tid;
        float* gt = P.p.tout + gid * NC + tid;
#pragma unroll
        for (int b = 0; b < 4; ++b)
#pragma unroll
          for (int a = 0; a < 4; ++a) {
            const int off = 256 * a + 1024 * b;
            const float kk = acc[a][b];
            if constexpr (MODE == kApply) {
              go[off] = kk;
            } else {
              const float u = (MODE == kStageFirst) ? uu[a][b] : uU[a + 4 * b];
              go[off] = fmaf(P.p.fb, kk, u);
              if constexpr (MODE != kStageLast) gt[off] = fmaf(P.p.fa, kk, u);
            }
          }
      }
    }
  }
}

}  // namespace hd
