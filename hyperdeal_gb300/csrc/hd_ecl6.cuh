// hd_ecl6.cuh -- persistent, TMA-pipelined ECL kernel for the 6D (3x+3v),
// degree-3 (4 nodes per direction), FP32-storage case, all faces periodic.
//
// Structure (one CTA per SM slot, 8 compute warps + 1 producer warp):
//   * Work item = one x0-row of cells (consecutive cell ids), claimed from a
//     global ticket counter (one row ahead), so the rows in flight form a
//     contiguous window.  A CTA walks the
//     row in the upwind order of direction x0, so the x0 face trace a cell
//     needs is the previous cell's face, which the thread owning that plane
//     still holds in registers ("carry"); only a row's first cell reads it
//     from global memory.
//   * The producer warp streams, per cell, through a 2-slot ring guarded by
//     mbarriers: the cell's 4096 stage-input values and its 4096 RK-solution
//     values as two 2D TMA tiles with the 128-byte swizzle (conflict-free
//     plane reads), and the upwind face traces of x2, v0, v1 (3D TMA boxes)
//     and v2 (contiguous, 1D bulk copy).  The x1 trace (4 floats at a 64-byte
//     stride, a poor TMA shape) is loaded one cell ahead by the compute
//     threads with one 128-bit load each.
//   * The compute warps apply the line operators two directions per phase
//     (x0x1, x2v0, v1v2) with an XOR-swizzled accumulator tile in shared
//     memory; the last phase transposes the result through the warp's own
//     slice of that tile and writes K or the fused LSRK update with 128-bit
//     stores.
//   * Every mbarrier wait is bounded: on time-out the kernel records an
//     error code, drains its own in-flight copies (bounded) and returns.
//
// The same kernel serves the 4D (2x+2v) degree-3 case (DIM = 4) when the
// mesh has 16 cells along x0: one x0-row of 16 cells (256 values each) is a
// unit of 4,096 values laid out exactly like one 6D cell, the 4D cell index
// taking the place of the 6D digits (i4, i5).  Phase 0 (x0, x1) and phase 1
// (v0, v1 at node strides 16 and 64, the 6D x2 and v0 strides) are then the
// 6D phases; the x0 upwind trace is a cell of the same unit (the unit is a
// whole periodic x0-row), read from the staged tile; the v0 and v1 traces of
// the 16 cells are the 6D x2 and v0 boxes of the neighbouring unit; there is
// no third phase.  Units are claimed one at a time (rows of length 1).
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
  CUtensorMap tcell;  // stage input T as [n/32][32] floats, box [128][32], 128B swizzle
  CUtensorMap ucell;  // RK solution U, same shape (stage kernels that read U)
  CUtensorMap tx2;    // T as [n/64][4][16], box [64][1][16]: one x2 face
  CUtensorMap tv0;    // T as [n/256][4][64], box [16][1][64]: one v0 face
  CUtensorMap tv1;    // T as [n/1024][4][256], box [4][1][256]: one v1 face
};

constexpr int E6_CTHREADS = 256;  // compute threads
constexpr int E6_THREADS = 288;   // + one producer warp
constexpr int E6_STAGES = 2;
// slot (floats): T tile [0,4096), U tile [4096,8192), faces x2 [8192,9216), v0 [9216,10240),
// v1 [10240,11264), v2 [11264,12288)
constexpr int E6_STAGE_FLOATS = 12288;
constexpr int E6_STAGE_BYTES = 4 * E6_STAGE_FLOATS;
constexpr int E6_OUT_BYTES = 16384;  // accumulator tile
constexpr int E6_SMEM = E6_STAGES * E6_STAGE_BYTES + E6_OUT_BYTES + 64;
constexpr unsigned E6_WAIT_LIMIT = 1u << 22;  // try_wait rounds before giving up (~seconds)

enum : int { E6_ERR_TIMEOUT_FULL = 1, E6_ERR_TIMEOUT_EMPTY = 2, E6_ERR_SMEM_ALIGN = 3 };

// tensor maps of a vector of n floats (hd_ecl6.cu); uin may be null (then tin)
cudaError_t encode_ecl6_maps(const float* tin, const float* uin, long long n, Ecl6Maps* m);


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
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint32_t limit = E6_WAIT_LIMIT) {
  const uint32_t a = smem_u32(bar);
  for (uint32_t it = 0; it < limit; ++it) {
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

// the same with an L2 cache-policy hint (createpolicy)
__device__ __forceinline__ void tma_load_2d_hint(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar,
                                                 uint64_t policy) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1, {%2, "
      "%3}], [%4], %5;" ::"r"(smem_u32(dst)),
      "l"(map), "r"(x), "r"(y), "r"(smem_u32(bar)), "l"(policy)
      : "memory");
}

// L2 policy "evict first" for data read or written once per stage
__device__ __forceinline__ uint64_t l2_evict_first_policy() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
  return p;
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
  EclParams<float> p;  // operator, mesh, vectors, stage factors, part (gid0, ghost, layer)
  int row_lo, row_hi;  // the launch's x0-rows of cells (local rows [row_lo, row_hi))
  int row_len;         // cells per row (cells in x0)
  int row0;            // global row index of local row 0 (parts hold whole layers)
  int lay0, lay1;      // this part's layers [lay0, lay1) of direction v2
  long long n_units;   // cells (6D) or x0-rows of 16 cells (4D) of the launch's vectors
  int* err;            // device error flag
  int* ticket;         // next unclaimed row (zeroed before every launch)
  unsigned wait_limit; // try_wait rounds of every bounded wait (E6_WAIT_LIMIT)
  int skip_issue;      // test hook (hd_adv_set_wait_test): the producer holding the launch's
                       // first row (always some CTA's first claim) issues nothing for cell
                       // skip_issue of that row (-1: off), so that the compute warps' wait
                       // for that slot runs out
};

// Cell index c checked against [0, n) in builds with -DHD_CHECK: outside, the
// violation is recorded (kCheckError) and cell 0 is used instead, so that the
// copy or access stays valid and the barrier accounting intact.
__device__ __forceinline__ long long e6_checked(const Ecl6Params& P, long long c, long long n) {
#ifdef HD_CHECK
  if (c < 0 || c >= n) {
    atomicExch(P.err, kCheckError);
    return 0;
  }
#else
  (void)P;
  (void)n;
#endif
  return c;
}

// first (local) cell id of row r and the upwind-neighbour offsets (in cells)
// of the row's cells in directions 1..5 (inside a row only x0 varies); ghost5:
// the v2 neighbour belongs to another part (its face is in the ghost region).
// DIM = 4: unit r (one x0-row of 16 cells) and its neighbours' offsets in
// units along x1, v0, v1.
struct E6Row {
  long long first;
  int nb[6];
  int ghost5;
};

template <int DIM>
__device__ __forceinline__ E6Row e6_row(const Ecl6Params& P, int r) {
  E6Row R;
  R.first = (long long)r * P.row_len;
  R.nb[0] = 0;
  R.ghost5 = 0;
  int rem = P.row0 + r;  // global row: coordinates of the global mesh
  if constexpr (DIM == 4) {
    int us = 1;  // unit stride of direction d
#pragma unroll
    for (int d = 1; d < 4; ++d) {
      const int nc = P.p.cells[d];
      const int c = rem % nc;
      rem /= nc;
      const int cn = c + P.p.op[d].step;
      const int cw = cn < 0 ? nc - 1 : (cn >= nc ? 0 : cn);  // periodic wrap
      R.nb[d] = (cw - c) * us;
      us *= nc;
    }
    R.nb[4] = R.nb[5] = 0;
  } else {
#pragma unroll
    for (int d = 1; d < 6; ++d) {
      const int nc = P.p.cells[d];
      const int c = rem % nc;
      rem /= nc;
      const int step = P.p.op[d].step;
      const int cs = int(P.p.cstride[d]);
      const int cn = c + step;
      const int cw = cn < 0 ? nc - 1 : (cn >= nc ? 0 : cn);  // periodic wrap
      R.nb[d] = (cw - c) * cs;
      if (d == 5 && (cw < P.lay0 || cw >= P.lay1)) R.ghost5 = 1;
    }
  }
  return R;
}

// cell id of the k-th cell of a row in the upwind traversal order of x0
__device__ __forceinline__ long long e6_cell(const Ecl6Params& P, long long first, int k) {
  return first + (P.p.op[0].step < 0 ? k : (P.row_len - 1 - k));
}

template <int MODE, int DIM = 6>
__global__ void __maxnreg__(104) ecl6_kernel(const __grid_constant__ Ecl6Params P,
                                             const __grid_constant__ Ecl6Maps maps) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  constexpr bool READ_U = (MODE == kStageMid || MODE == kStageLast);
  if (smem_u32(smem_raw) & 1023u) {  // the swizzled tiles need 1024-byte alignment
    if (threadIdx.x == 0) atomicExch(P.err, E6_ERR_SMEM_ALIGN);
    return;
  }
  float* s_stage = reinterpret_cast<float*>(smem_raw);
  float* so = reinterpret_cast<float*>(smem_raw + E6_STAGES * E6_STAGE_BYTES);  // accumulator tile
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem_raw + E6_STAGES * E6_STAGE_BYTES + E6_OUT_BYTES);
  uint64_t* full = bars;               // [E6_STAGES]: TMA bytes landed
  uint64_t* empty = bars + E6_STAGES;  // [E6_STAGES]: all 8 compute warps done with the slot
  volatile int* s_abort = reinterpret_cast<volatile int*>(bars + 2 * E6_STAGES);
  // rows claimed by this CTA: s_rows[q % 4] = row of the CTA's q-th row (-1: none);
  // s_cont[it & 1]: whether the compute warps continue after cell it (one decision
  // for all of them, taken by thread 0 before a barrier)
  volatile int* s_rows = reinterpret_cast<volatile int*>(bars + 2 * E6_STAGES) + 2;
  volatile int* s_cont = s_rows + 4;

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

  // Rows are claimed dynamically from a global ticket counter, one row ahead,
  // so that the rows in flight across the grid stay a contiguous window of the
  // row order (their upwind x1 / x2 / v0 neighbours are then read while still
  // in L2), whatever the CTAs' relative speed.

  if (tid >= E6_CTHREADS) {
    // ------------------------------------------------------------------ producer
    if (tid == E6_CTHREADS) {
      int issued = 0;
      bool ok = true;
      const uint64_t pol_u = l2_evict_first_policy();
      uint32_t bytes = 16384u + (READ_U ? 16384u : 0u);
#pragma unroll
      for (int d = 2; d < 6; ++d) bytes += P.p.op[d].active ? 4096u : 0u;
      auto take = [&]() -> int {
        const int t = atomicAdd(P.ticket, 1);
        return t < P.row_hi - P.row_lo ? P.row_lo + t : -1;
      };
      int q = 0, k = 0;
      int r = take();
      s_rows[0] = r;
      s_rows[1] = r >= 0 ? take() : -1;
      E6Row R = e6_row<DIM>(P, r >= 0 ? r : 0);
      if (r < 0) mbar_arrive(&full[0]);  // no row for this CTA: release the compute warps
      for (int it = 0; r >= 0; ++it) {
        const int s = it % E6_STAGES;
        if (it >= E6_STAGES && !mbar_wait(&empty[s], ((it / E6_STAGES) - 1) & 1, P.wait_limit)) {
          atomicExch(P.err, E6_ERR_TIMEOUT_EMPTY);
          *s_abort = 1;
          ok = false;
          break;
        }
        if (*s_abort) { ok = false; break; }
        if (k == 0 && q > 0) {
          r = s_rows[q % 4];
          if (r < 0) break;  // the compute warps stop at the end of row q - 1 by themselves
          s_rows[(q + 1) % 4] = take();
          R = e6_row<DIM>(P, r);
        }
        const long long gid = e6_cell(P, R.first, k);
        float* st = s_stage + s * E6_STAGE_FLOATS;
        if (k == P.skip_issue && R.first == (long long)P.row_lo * P.row_len) {
          // test hook: nothing arrives on this slot, its consumers' bounded wait runs out
          ++issued;
          if (++k == P.row_len) {
            k = 0;
            ++q;
          }
          continue;
        }
        const long long nc = P.n_units;
        const long long gc = e6_checked(P, gid, nc);
        mbar_arrive_expect_tx(&full[s], bytes);
        tma_load_2d(st, &maps.tcell, 0, int(gc * 128), &full[s]);
        // U is read once per stage: evict it first, so that L2 keeps the stage
        // input T, whose faces the neighbours read again later
        if (READ_U) tma_load_2d_hint(st + 4096, &maps.ucell, 0, int(gc * 128), &full[s], pol_u);
        if (P.p.op[2].active)
          tma_load_3d(st + 8192, &maps.tx2, 0, P.p.op[2].nb_node, int(e6_checked(P, gid + R.nb[2], nc) * 64),
                      &full[s]);
        if (P.p.op[3].active)
          tma_load_3d(st + 9216, &maps.tv0, 0, P.p.op[3].nb_node, int(e6_checked(P, gid + R.nb[3], nc) * 16),
                      &full[s]);
        if (P.p.op[4].active)
          tma_load_3d(st + 10240, &maps.tv1, 0, P.p.op[4].nb_node, int(e6_checked(P, gid + R.nb[4], nc) * 4),
                      &full[s]);
        if (P.p.op[5].active) {
          // the v2 face: the neighbour's slab, or its face in the ghost region
          // (a part's layer starts at a multiple of the layer size, so the
          // neighbour's in-layer slot is this cell's)
          const float* src5 =
              R.ghost5 ? P.p.ghost + e6_checked(P, gid % P.p.layer, P.p.layer) * 1024
                       : P.p.tin + e6_checked(P, gid + R.nb[5], nc) * 4096 + P.p.op[5].nb_node * 1024;
          bulk_load(st + 11264, src5, 4096u, &full[s]);
        }
        ++issued;
        if (++k == P.row_len) {
          k = 0;
          ++q;
        }
      }
      // on an abort, wait (bounded) for the copies still in flight before leaving
      if (!ok) {
        for (int it = issued - E6_STAGES < 0 ? 0 : issued - E6_STAGES; it < issued; ++it)
          mbar_wait(&full[it % E6_STAGES], (it / E6_STAGES) & 1, P.wait_limit);
      }
    }
    return;
  }

  // -------------------------------------------------------------------- consumers
  const LineOp<float>* L = P.p.op;
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
  // epilogue: each lane owns 4 float4 chunks of its warp's 512 phase-2 nodes,
  // nodes vnode + 1024 j + (0..3) with vnode = 4 (lane & 7) + 32 warp + 256 (lane >> 3)
  const int vnode = 4 * (lane & 7) + 32 * warp + 256 * (lane >> 3);
  const int vt = 32 * warp + 256 * (lane >> 3) + (((lane & 7) ^ warp) << 2);  // T / U tiles
  const int vo = 32 * warp + 256 * (lane >> 3) + (((lane & 7) ^ warp ^ (4 * ((lane >> 3) & 1))) << 2);

  float carry[4] = {0.f, 0.f, 0.f, 0.f};  // x0 face of the previous cell of the row
  float4 px1 = make_float4(0.f, 0.f, 0.f, 0.f);  // x1 face values of this thread's plane
  auto fetch_x1 = [&](long long g, int nb1) {
    if (L[1].active)
      px1 = __ldg(reinterpret_cast<const float4*>(P.p.tin + e6_checked(P, g + nb1, P.n_units) * NC + 16 * tid +
                                                  4 * L[1].nb_node));
  };

  // the first cell (or the producer's "no row" signal) decides whether there is work
  if (lane == 0 && !mbar_wait(&full[0], 0, P.wait_limit)) {
    *s_abort = 1;
    atomicExch(P.err, E6_ERR_TIMEOUT_FULL);
  }
  __syncwarp();
  if (tid == 0) s_cont[0] = (!*s_abort && s_rows[0] >= 0) ? 1 : 0;
  bar_compute();
  if (!s_cont[0]) return;
  int q = 0, k = 0;
  E6Row R = e6_row<DIM>(P, s_rows[0]);
  fetch_x1(e6_cell(P, R.first, 0), R.nb[1]);
  for (int it = 0;; ++it) {
    const int s = it % E6_STAGES;
    const long long gid = e6_cell(P, R.first, k);
    const float* st = s_stage + s * E6_STAGE_FLOATS;
    const bool new_row = k + 1 == P.row_len;

    // row start: x0 face of the upwind neighbour of the row's first cell (periodic wrap)
    if (DIM == 6 && k == 0 && L[0].active) {
      const long long g0 = R.first + (L[0].step < 0 ? P.row_len - 1 : 0);
      const float* src = P.p.tin + e6_checked(P, g0, P.n_units) * NC + 16 * tid + L[0].nb_node;
#pragma unroll
      for (int b = 0; b < 4; ++b) carry[b] = __ldg(src + 4 * b);
    }

    // one lane per warp waits for the slot (bounded); a time-out turns the rest
    // of the CTA's work into no-ops (no stores) without leaving any barrier
    if (lane == 0 && !*s_abort && !mbar_wait(&full[s], (it / E6_STAGES) & 1, P.wait_limit)) {
      *s_abort = 1;
      atomicExch(P.err, E6_ERR_TIMEOUT_FULL);
    }
    __syncwarp();
    // the CTA's next row was claimed before this row's first cell was issued
    // (s_rows is read after that cell's barrier); -1: no next row
    const int next_row = new_row ? s_rows[(q + 1) % 4] : -1;
    const bool has_next = !new_row || next_row >= 0;

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
        if constexpr (DIM == 4) {
          // the x0 upwind neighbour is a cell of this unit (a whole periodic
          // x0-row), staged with it: its face nb_node in this thread's plane
          const int nodeb = ((((tid >> 4) + L[0].step) & 15) << 8) + ((tid & 15) << 4) + L[0].nb_node;
#pragma unroll
          for (int b = 0; b < 4; ++b) carry[b] = st[swz_t(nodeb + 4 * b)];
        }
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
        if constexpr (DIM == 6) {
#pragma unroll
          for (int b = 0; b < 4; ++b) carry[b] = L[0].nb_node ? uu[3][b] : uu[0][b];
        }
      }
      if (L[1].active) {
        const float upv[4] = {px1.x, px1.y, px1.z, px1.w};
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
    // x1 face of the next cell of this CTA
    if (has_next) {
      if (new_row) {
        const E6Row Rn = e6_row<DIM>(P, next_row);
        fetch_x1(e6_cell(P, Rn.first, 0), Rn.nb[1]);
      } else {
        fetch_x1(e6_cell(P, R.first, k + 1), R.nb[1]);
      }
    }
    bar_compute();

    // ---------------- phase 1: directions x2 (a, stride 16) and v0 (b, stride 64)
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
      if (L[2].active) {
        const float* tr = st + 8192 + 64 * hi + lo;
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
        const float* tr = st + 9216 + 64 * hi + lo;
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
          const int Rr = (a >> 1) + 2 * b;
          const int e = (a & 1) ^ (Rr >> 2);
          so[ob1[Rr & 3][e] + 32 * Rr] = acc[a][b];
        }
    }
    bar_compute();

    // ---------------- phase 2: directions v1 (a, stride 256) and v2 (b, stride 1024), epilogue
    // (DIM = 4: the epilogue only; phase 1 left K in the accumulator tile)
    {
      float uu[4][4], acc[4][4];
      if constexpr (DIM == 6) {
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) {
          uu[a][b] = st[tb2 + 256 * a + 1024 * b];
          acc[a][b] = so[ob2[a & 1] + 256 * a + 1024 * b];
        }
      if (L[4].active) {
        const float* tr = st + 10240 + tid;
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
        const float* tr = st + 11264 + tid;
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
      }  // DIM == 6
      // U at the epilogue nodes (the T tile for the first stage), read before the slot is released
      float4 uv[4];
      if constexpr (MODE != kApply) {
        const float* ut = READ_U ? st + 4096 : st;
#pragma unroll
        for (int j = 0; j < 4; ++j) uv[j] = *reinterpret_cast<const float4*>(ut + vt + 1024 * j);
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(&empty[s]);
      // transpose K through this warp's private slice of the accumulator tile
      if constexpr (DIM == 6) {
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
          for (int b = 0; b < 4; ++b) so[ob2[a & 1] + 256 * a + 1024 * b] = acc[a][b];
      }
      __syncwarp();
#ifdef HD_CHECK
      const long long gcell = DIM == 4 ? gid * 16 : gid;
      const bool store_ok = gcell >= P.p.c_lo && gcell < P.p.c_hi;
      if (!store_ok) atomicExch(P.err, kCheckError);
#else
      constexpr bool store_ok = true;
#endif
      if (!*s_abort && store_ok) {
        float4* go = reinterpret_cast<float4*>(P.p.uout + gid * NC + vnode);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const float4 kv = *reinterpret_cast<const float4*>(so + vo + 1024 * j);
          // results are streamed out (read again only in the next stage): evict-first stores
          if constexpr (MODE == kApply) {
            __stcs(go + 256 * j, kv);
          } else {
            const float4 u = uv[j];
            __stcs(go + 256 * j, make_float4(fmaf(P.p.fb, kv.x, u.x), fmaf(P.p.fb, kv.y, u.y),
                                             fmaf(P.p.fb, kv.z, u.z), fmaf(P.p.fb, kv.w, u.w)));
            if constexpr (MODE != kStageLast) {
              float4* gt = reinterpret_cast<float4*>(P.p.tout + gid * NC + vnode);
              __stcs(gt + 256 * j, make_float4(fmaf(P.p.fa, kv.x, u.x), fmaf(P.p.fa, kv.y, u.y),
                                               fmaf(P.p.fa, kv.z, u.z), fmaf(P.p.fa, kv.w, u.w)));
            }
          }
        }
      }
    }
    // the accumulator tile is rewritten by the next cell's phase 0; whether
    // to continue is decided once (thread 0) for all compute warps
    if (tid == 0) s_cont[(it + 1) & 1] = (!*s_abort && has_next) ? 1 : 0;
    bar_compute();
    if (!s_cont[(it + 1) & 1]) break;
    if (new_row) {
      k = 0;
      ++q;
      R = e6_row<DIM>(P, next_row);
    } else {
      ++k;
    }
  }
}

}  // namespace hd
