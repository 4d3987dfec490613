// hd_batch.cu -- batched uneven instances: the C ABI hd_batch_* of
// include/hyperdeal_gb300.h.
//
// The reference runs independent problems one after the other, each with its
// own compile-time (dim, degree) instantiation (examples/advection/
// advection.cc:26-48, :253-259).  Here the instances are grouped by class
// (phase-space dimension, degree, storage type); a class with a batch kernel
// (hd_batch.cuh) advances all its instances in ONE persistent launch per RK
// stage, the others launch per instance.  A step can be recorded once as a
// CUDA graph (two steps, after which the three vectors of every instance are
// back in their roles) and replayed; the stage times of the replayed steps
// advance on the device.  Tiles (cells per CTA, CTAs per SM) are chosen per
// class by timing candidate tiles (hd_batch_autotune).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/hyperdeal_gb300.h"
#include "hd_batch.cuh"
#include "hd_internal.h"

namespace hd {

BatchLaunchers batch_launchers(int D, int N) {
  if (D == 4) return batch_launchers_d4(N);
  if (D == 5) return batch_launchers_d5(N);
  return BatchLaunchers{nullptr, nullptr, 0, 0, 0, 0, false};
}

namespace {

// slots[s * n + m].time += delta[m] for every slot s
template <typename T>
__global__ void advance_time_kernel(EclParams<T>* slots, int n_slots, int n, const double* __restrict__ delta) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n_slots * n) slots[i].time += delta[i % n];
}

}  // namespace

}  // namespace hd

namespace {

struct BatchClass {
  int D, N, dtype, gauss, arith;
  std::vector<int> members;  // instance indices
  bool batched;              // one launch per stage for the whole class
  hd::BatchLaunchers L;
  int cpb, per_sm;           // tile of the batch kernel
  long long* d_prefix;       // members + 1 block offsets
  void* d_slots;             // (2 * ns + 1) slots of members EclParams<T>
  double* d_delta;           // per member time advance of one graph replay
  size_t param_bytes;
};

}  // namespace

struct hd_batch {
  std::vector<hd_adv*> ops;
  hd_lsrk rk;
  std::vector<BatchClass> classes;
  cudaStream_t capture_stream;
  cudaGraph_t graph;
  cudaGraphExec_t exec;
  bool graph_ready;
};

namespace {

int bfail(int code, const char* msg) {
  hd::set_last_error(msg);
  return code;
}

int bcuda(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return HD_OK;
  char buf[256];
  std::snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(e));
  hd::set_last_error(buf);
  return HD_ERR_CUDA;
}

void batch_free(hd_batch* b) {
  if (!b) return;
  for (auto& c : b->classes) {
    cudaFree(c.d_prefix);
    cudaFree(c.d_slots);
    cudaFree(c.d_delta);
  }
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  if (b->capture_stream) cudaStreamDestroy(b->capture_stream);
  delete b;
}

// pointers, factors and time of one stage of one instance
struct StageArgs {
  int mode;
  const void* tin;
  const void* uin;
  void* uout;
  void* tout;
  double fb, fa, time;
};

// the stage sequence of one fused step (the rotation of hd_lsrk_step)
void step_stages(const hd_lsrk& rk, void* sol, void* Ki, void* Ti, double time, double dt, StageArgs* out,
                 void** new_sol, void** new_Ki, void** new_Ti) {
  void* X0 = sol;
  void* X1 = Ki;
  void* X2 = Ti;
  void* t_in = X0;
  void* t_free = X2;
  for (int st = 0; st < rk.ns; ++st) {
    const bool last = st == rk.ns - 1;
    int mode = st == 0 ? hd::kStageFirst : (last ? hd::kStageLast : hd::kStageMid);
    out[st] = StageArgs{mode, t_in, st == 0 ? t_in : X1, X1, last ? nullptr : t_free, rk.bi[st] * dt,
                        last ? 0.0 : rk.ai[st] * dt, time + rk.ci[st] * dt};
    if (!last) {
      void* next = t_free;
      t_free = (st == 0) ? X0 : t_in;
      t_in = next;
    }
  }
  *new_sol = X1;
  *new_Ki = X0;
  *new_Ti = X2;
}

template <typename T>
hd::EclParams<T> stage_params(const hd_adv* op, const StageArgs& a) {
  hd::EclParams<T> P;
  if constexpr (sizeof(T) == 8) P = op->p64;
  else P = op->p32;
  P.tin = (const T*)a.tin;
  P.uin = (const T*)a.uin;
  P.uout = (T*)a.uout;
  P.tout = (T*)a.tout;
  P.fb = T(a.fb);
  P.fa = T(a.fa);
  P.time = a.time;
  return P;
}

// copy the class's stage parameters into `slot` (stream-ordered)
int upload_slot(hd_batch* b, BatchClass& c, int slot, const std::vector<StageArgs>& args, cudaStream_t s) {
  const int n = int(c.members.size());
  cudaError_t e;
  if (c.dtype == HD_F64) {
    std::vector<hd::EclParams<double>> h(n);
    for (int k = 0; k < n; ++k) h[k] = stage_params<double>(b->ops[c.members[k]], args[k]);
    e = cudaMemcpyAsync((hd::EclParams<double>*)c.d_slots + size_t(slot) * n, h.data(), sizeof(h[0]) * n,
                        cudaMemcpyHostToDevice, s);
  } else {
    std::vector<hd::EclParams<float>> h(n);
    for (int k = 0; k < n; ++k) h[k] = stage_params<float>(b->ops[c.members[k]], args[k]);
    e = cudaMemcpyAsync((hd::EclParams<float>*)c.d_slots + size_t(slot) * n, h.data(), sizeof(h[0]) * n,
                        cudaMemcpyHostToDevice, s);
  }
  // pageable source: the call returns once the data is staged, so h may go
  return bcuda(e, "batch parameters");
}

// launch one stage of a class: the batch kernel on `slot`, or per instance
int launch_slot(hd_batch* b, BatchClass& c, int slot, const std::vector<StageArgs>& args, cudaStream_t s) {
  const int n = int(c.members.size());
  if (!c.batched) {
    for (int k = 0; k < n; ++k) {
      const StageArgs& a = args[k];
      const int rc = hd::adv_launch(b->ops[c.members[k]], a.mode, a.tin, a.uin, a.uout, a.tout, a.fb, a.fa, a.time, s);
      if (rc) return rc;
    }
    return HD_OK;
  }
  const int mode = args[0].mode;
  cudaError_t e;
  if (c.dtype == HD_F64)
    e = (c.arith == HD_ARITH_FP32X2 ? c.L.f64x : c.L.f64)(hd::BatchLaunch<double>{(hd::EclParams<double>*)c.d_slots + size_t(slot) * n, c.d_prefix, n, c.cpb,
                                        c.per_sm},
                mode, s);
  else
    e = c.L.f32(hd::BatchLaunch<float>{(hd::EclParams<float>*)c.d_slots + size_t(slot) * n, c.d_prefix, n, c.cpb,
                                       c.per_sm},
                mode, s);
  return bcuda(e, "batch kernel launch");
}

int run_class_stage(hd_batch* b, BatchClass& c, int slot, const std::vector<StageArgs>& args, cudaStream_t s) {
  if (c.batched) {
    const int rc = upload_slot(b, c, slot, args, s);
    if (rc) return rc;
  }
  return launch_slot(b, c, slot, args, s);
}

int check_vectors(const hd_batch* b, void* const* sol, void* const* Ki, void* const* Ti) {
  if (!sol || !Ki || !Ti) return bfail(HD_ERR_INVALID, "hd_batch: null vector array");
  for (size_t i = 0; i < b->ops.size(); ++i) {
    if (!sol[i] || !Ki[i] || !Ti[i]) return bfail(HD_ERR_INVALID, "hd_batch: null vector");
    if (sol[i] == Ki[i] || sol[i] == Ti[i] || Ki[i] == Ti[i]) return bfail(HD_ERR_INVALID, "hd_batch: vectors must differ");
    if ((reinterpret_cast<uintptr_t>(sol[i]) | reinterpret_cast<uintptr_t>(Ki[i]) |
         reinterpret_cast<uintptr_t>(Ti[i])) & 15u)
      return bfail(HD_ERR_INVALID, "hd_batch: vectors must be 16-byte aligned");
  }
  return HD_OK;
}

}  // namespace

extern "C" {

int hd_batch_create(hd_adv* const* ops, int n, const hd_lsrk* rk, hd_batch** out) {
  if (!ops || !rk || !out || n < 1) return bfail(HD_ERR_INVALID, "hd_batch_create: bad argument");
  *out = nullptr;
  if (rk->ns < 2) return bfail(HD_ERR_INVALID, "hd_batch_create: the scheme needs at least two stages");
  hd_batch* b = new (std::nothrow) hd_batch;
  if (!b) return bfail(HD_ERR_ALLOC, "out of host memory");
  b->rk = *rk;
  b->capture_stream = nullptr;
  b->graph = nullptr;
  b->exec = nullptr;
  b->graph_ready = false;
  for (int i = 0; i < n; ++i) {
    if (!ops[i]) { batch_free(b); return bfail(HD_ERR_INVALID, "hd_batch_create: null operator"); }
    if (ops[i]->n_parts > 1) {
      batch_free(b);
      return bfail(HD_ERR_UNSUPPORTED, "hd_batch_create: parts of a partitioned operator are not batched");
    }
    b->ops.push_back(ops[i]);
  }
  for (int i = 0; i < n; ++i) {
    const hd_adv* op = ops[i];
    auto it = std::find_if(b->classes.begin(), b->classes.end(), [&](const BatchClass& c) {
      return c.D == op->D && c.N == op->N && c.dtype == op->dtype && c.gauss == op->gauss && c.arith == op->arith;
    });
    if (it == b->classes.end()) {
      BatchClass c;
      c.D = op->D;
      c.N = op->N;
      c.dtype = op->dtype;
      c.gauss = op->gauss;
      c.arith = op->arith;
      c.L = hd::batch_launchers(op->D, op->N);
      c.batched = c.L.ok && !op->gauss;  // the batch kernel is the collocation operator
      c.cpb = 0;
      c.per_sm = 0;
      c.d_prefix = nullptr;
      c.d_slots = nullptr;
      c.d_delta = nullptr;
      c.param_bytes = op->dtype == HD_F64 ? sizeof(hd::EclParams<double>) : sizeof(hd::EclParams<float>);
      b->classes.push_back(c);
      it = b->classes.end() - 1;
    }
    it->members.push_back(i);
  }
  const int nslots = 2 * rk->ns + 1;
  for (auto& c : b->classes) {
    const int m = int(c.members.size());
    if (c.batched && m > hd::kBatchMaxInstances) c.batched = false;
    if (!c.batched) continue;
    cudaError_t e = cudaMalloc(&c.d_prefix, sizeof(long long) * (m + 1));
    if (e == cudaSuccess) e = cudaMalloc(&c.d_slots, c.param_bytes * size_t(nslots) * m);
    if (e == cudaSuccess) e = cudaMalloc(&c.d_delta, sizeof(double) * m);
    if (e == cudaSuccess) e = cudaMemset(c.d_slots, 0, c.param_bytes * size_t(nslots) * m);
    if (e != cudaSuccess) { batch_free(b); return bcuda(e, "hd_batch_create: cudaMalloc"); }
  }
  *out = b;
  return hd_batch_set_tile(b, -1, 0, 0);  // default tiles, block offsets
}

int hd_batch_destroy(hd_batch* b) {
  batch_free(b);
  return HD_OK;
}

int hd_batch_n_classes(const hd_batch* b) { return b ? int(b->classes.size()) : -1; }

int hd_batch_class_info(const hd_batch* b, int c, int* D, int* degree, int* dtype, int* n_members, int* batched,
                        int* cells_per_cta, int* ctas_per_sm) {
  if (!b || c < 0 || c >= int(b->classes.size())) return bfail(HD_ERR_INVALID, "hd_batch_class_info: bad class");
  const BatchClass& k = b->classes[c];
  const int maxc = k.dtype == HD_F64 ? k.L.max_cpb_f64 : k.L.max_cpb_f32;
  if (D) *D = k.D;
  if (degree) *degree = k.N - 1;
  if (dtype) *dtype = k.dtype;
  if (n_members) *n_members = int(k.members.size());
  if (batched) *batched = k.batched ? 1 : 0;
  if (cells_per_cta) *cells_per_cta = k.batched ? (k.cpb > 0 ? k.cpb : maxc) : 0;
  if (ctas_per_sm) *ctas_per_sm = k.per_sm;
  return HD_OK;
}

int hd_batch_class_arithmetic(const hd_batch* b, int c) {
  if (!b || c < 0 || c >= int(b->classes.size())) return -1;
  return b->classes[c].arith;
}

int hd_batch_set_tile(hd_batch* b, int c, int cells_per_cta, int ctas_per_sm) {
  if (!b) return bfail(HD_ERR_INVALID, "hd_batch_set_tile: null handle");
  if (cells_per_cta < 0 || ctas_per_sm < 0 || ctas_per_sm > 32)
    return bfail(HD_ERR_INVALID, "hd_batch_set_tile: cells_per_cta >= 0, 0 <= ctas_per_sm <= 32");
  for (int ci = 0; ci < int(b->classes.size()); ++ci) {
    if (c >= 0 && ci != c) continue;
    BatchClass& k = b->classes[ci];
    const int maxc = k.dtype == HD_F64 ? k.L.max_cpb_f64 : k.L.max_cpb_f32;
    const int defc = k.dtype == HD_F64 ? k.L.def_cpb_f64 : k.L.def_cpb_f32;
    k.cpb = (cells_per_cta < 1 || cells_per_cta > maxc) ? defc : cells_per_cta;
    k.per_sm = ctas_per_sm;
    if (!k.batched) {
      for (int m : k.members) hd_adv_set_tile(b->ops[m], cells_per_cta, ctas_per_sm);
      continue;
    }
    std::vector<long long> prefix(k.members.size() + 1, 0);
    for (size_t i = 0; i < k.members.size(); ++i)
      prefix[i + 1] = prefix[i] + (b->ops[k.members[i]]->n_cells + k.cpb - 1) / k.cpb;
    cudaError_t e = cudaMemcpy(k.d_prefix, prefix.data(), sizeof(long long) * prefix.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return bcuda(e, "hd_batch_set_tile: block offsets");
  }
  b->graph_ready = false;  // a recorded graph holds the old tiles
  return HD_OK;
}

int hd_batch_apply(hd_batch* b, void* const* dst, const void* const* src, const double* time, void* stream) {
  if (!b || !dst || !src) return bfail(HD_ERR_INVALID, "hd_batch_apply: null argument");
  cudaStream_t s = (cudaStream_t)stream;
  const int slot = 2 * b->rk.ns;
  for (auto& c : b->classes) {
    std::vector<StageArgs> args;
    for (int m : c.members) {
      if (!dst[m] || !src[m] || dst[m] == src[m]) return bfail(HD_ERR_INVALID, "hd_batch_apply: bad vectors");
      args.push_back(StageArgs{hd::kApply, src[m], src[m], dst[m], nullptr, 0.0, 0.0, time ? time[m] : 0.0});
    }
    const int rc = run_class_stage(b, c, slot, args, s);
    if (rc) return rc;
  }
  return HD_OK;
}

int hd_batch_lsrk_step(hd_batch* b, void** sol, void** Ki, void** Ti, const double* time, const double* dt,
                       void* stream) {
  if (!b || !dt) return bfail(HD_ERR_INVALID, "hd_batch_lsrk_step: null argument");
  int rc = check_vectors(b, sol, Ki, Ti);
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  const int n = int(b->ops.size()), ns = b->rk.ns;
  std::vector<StageArgs> st(size_t(n) * ns);
  std::vector<void*> ns_sol(n), ns_Ki(n), ns_Ti(n);
  for (int i = 0; i < n; ++i)
    step_stages(b->rk, sol[i], Ki[i], Ti[i], time ? time[i] : 0.0, dt[i], &st[size_t(i) * ns], &ns_sol[i], &ns_Ki[i],
                &ns_Ti[i]);
  b->graph_ready = false;  // the slots of a recorded graph are reused here
  for (int k = 0; k < ns; ++k)
    for (auto& c : b->classes) {
      std::vector<StageArgs> args;
      for (int m : c.members) args.push_back(st[size_t(m) * ns + k]);
      rc = run_class_stage(b, c, k, args, s);
      if (rc) return rc;
    }
  for (int i = 0; i < n; ++i) {
    sol[i] = ns_sol[i];
    Ki[i] = ns_Ki[i];
    Ti[i] = ns_Ti[i];
  }
  return HD_OK;
}

int hd_batch_graph_capture(hd_batch* b, void* const* sol, void* const* Ki, void* const* Ti, const double* time,
                           const double* dt) {
  if (!b || !dt) return bfail(HD_ERR_INVALID, "hd_batch_graph_capture: null argument");
  int rc = check_vectors(b, sol, Ki, Ti);
  if (rc) return rc;
  const int n = int(b->ops.size()), ns = b->rk.ns;
  for (auto& c : b->classes)
    if (!c.batched)
      for (int m : c.members)
        if (b->ops[m]->desc.bc_kind == HD_BC_FUNCTION)
          return bfail(HD_ERR_UNSUPPORTED,
                       "hd_batch_graph_capture: time-dependent boundary data needs a batch kernel for its class");
  if (b->exec) { cudaGraphExecDestroy(b->exec); b->exec = nullptr; }
  if (b->graph) { cudaGraphDestroy(b->graph); b->graph = nullptr; }
  b->graph_ready = false;
  if (!b->capture_stream) {
    cudaError_t e = cudaStreamCreateWithFlags(&b->capture_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) return bcuda(e, "hd_batch_graph_capture: stream");
  }
  // the stage arguments of two steps: after them every instance's vectors are back in their roles
  std::vector<StageArgs> st(size_t(n) * 2 * ns);
  for (int i = 0; i < n; ++i) {
    void *s1, *k1, *t1, *s2, *k2, *t2;
    const double t0 = time ? time[i] : 0.0;
    step_stages(b->rk, sol[i], Ki[i], Ti[i], t0, dt[i], &st[size_t(i) * 2 * ns], &s1, &k1, &t1);
    step_stages(b->rk, s1, k1, t1, t0 + dt[i], dt[i], &st[size_t(i) * 2 * ns + ns], &s2, &k2, &t2);
    if (s2 != sol[i] || k2 != Ki[i] || t2 != Ti[i])
      return bfail(HD_ERR_INVALID, "hd_batch_graph_capture: rotation of the scheme does not close after two steps");
  }
  // upload every slot before recording; the graph only launches kernels
  cudaStream_t cs = b->capture_stream;
  auto class_args = [&](const BatchClass& c, int k) {
    std::vector<StageArgs> args;
    for (int mm : c.members) args.push_back(st[size_t(mm) * 2 * ns + k]);
    return args;
  };
  for (auto& c : b->classes) {
    if (!c.batched) continue;
    const int m = int(c.members.size());
    std::vector<double> delta(m);
    for (int k = 0; k < m; ++k) delta[k] = 2.0 * dt[c.members[k]];
    cudaError_t e = cudaMemcpyAsync(c.d_delta, delta.data(), sizeof(double) * m, cudaMemcpyHostToDevice, cs);
    if (e != cudaSuccess) return bcuda(e, "hd_batch_graph_capture: deltas");
    for (int k = 0; k < 2 * ns; ++k) {
      rc = upload_slot(b, c, k, class_args(c, k), cs);
      if (rc) return rc;
    }
  }
  cudaError_t e = cudaStreamSynchronize(cs);
  if (e != cudaSuccess) return bcuda(e, "hd_batch_graph_capture: upload");
  e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeRelaxed);
  if (e != cudaSuccess) return bcuda(e, "hd_batch_graph_capture: begin");
  for (int k = 0; k < 2 * ns && !rc; ++k)
    for (auto& c : b->classes) {
      rc = launch_slot(b, c, k, class_args(c, k), cs);
      if (rc) break;
    }
  for (auto& c : b->classes) {
    if (rc || !c.batched) continue;
    const int m = int(c.members.size()), total = 2 * ns * m;
    if (c.dtype == HD_F64)
      hd::advance_time_kernel<double><<<(total + 127) / 128, 128, 0, cs>>>((hd::EclParams<double>*)c.d_slots, 2 * ns,
                                                                          m, c.d_delta);
    else
      hd::advance_time_kernel<float><<<(total + 127) / 128, 128, 0, cs>>>((hd::EclParams<float>*)c.d_slots, 2 * ns,
                                                                         m, c.d_delta);
  }
  cudaGraph_t g = nullptr;
  const cudaError_t e_end = cudaStreamEndCapture(cs, &g);
  if (rc) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (e_end != cudaSuccess) return bcuda(e_end, "hd_batch_graph_capture: end");
  b->graph = g;
  e = cudaGraphInstantiate(&b->exec, g, 0);
  if (e != cudaSuccess) return bcuda(e, "hd_batch_graph_capture: instantiate");
  b->graph_ready = true;
  return HD_OK;
}

int hd_batch_graph_launch(hd_batch* b, void* stream) {
  if (!b || !b->graph_ready) return bfail(HD_ERR_INVALID, "hd_batch_graph_launch: no graph recorded");
  return bcuda(cudaGraphLaunch(b->exec, (cudaStream_t)stream), "hd_batch_graph_launch");
}

int hd_batch_autotune(hd_batch* b, const void* const* src, void* const* dst, int reps, void* stream) {
  if (!b || !src || !dst) return bfail(HD_ERR_INVALID, "hd_batch_autotune: null argument");
  if (reps < 1) reps = 3;
  cudaStream_t s = (cudaStream_t)stream;
  const int slot = 2 * b->rk.ns;
  cudaEvent_t e0, e1;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)
    return bfail(HD_ERR_CUDA, "hd_batch_autotune: events");
  int rc = HD_OK;
  for (int ci = 0; ci < int(b->classes.size()) && !rc; ++ci) {
    BatchClass& c = b->classes[ci];
    std::vector<StageArgs> args;
    for (int m : c.members) {
      if (!dst[m] || !src[m] || dst[m] == src[m]) { rc = bfail(HD_ERR_INVALID, "hd_batch_autotune: bad vectors"); break; }
      args.push_back(StageArgs{hd::kApply, src[m], src[m], dst[m], nullptr, 0.0, 0.0, 0.0});
    }
    if (rc) break;
    if (c.batched) rc = upload_slot(b, c, slot, args, s);
    if (rc) break;
    // candidates: the largest tile and its halvings, each with the occupancy
    // limit or 2 CTAs per SM
    const int maxc = c.dtype == HD_F64 ? (c.batched ? c.L.max_cpb_f64 : 0) : (c.batched ? c.L.max_cpb_f32 : 0);
    int lim = maxc;
    if (!c.batched) {
      hd_adv_tile_limits(b->ops[c.members[0]], &lim, nullptr);
    }
    std::vector<int> cands;
    for (int v = lim; v >= 1 && cands.size() < 4; v /= 2) cands.push_back(v);
    float best = 1e30f;
    int best_c = 0, best_p = 0;
    for (int cand : cands)
      for (int per : {0, 2}) {
        rc = hd_batch_set_tile(b, ci, cand, per);
        if (!rc) rc = launch_slot(b, c, slot, args, s);  // warm-up
        if (rc) break;
        cudaEventRecord(e0, s);
        for (int r = 0; r < reps && !rc; ++r) rc = launch_slot(b, c, slot, args, s);
        cudaEventRecord(e1, s);
        if (rc) break;
        if (cudaEventSynchronize(e1) != cudaSuccess) { rc = bfail(HD_ERR_CUDA, "hd_batch_autotune: timing"); break; }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best) { best = ms; best_c = cand; best_p = per; }
      }
    if (!rc) rc = hd_batch_set_tile(b, ci, best_c, best_p);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return rc;
}

}  // extern "C"
