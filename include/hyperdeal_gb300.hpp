// hyperdeal_gb300.hpp -- header-only C++ interface over the C ABI with the
// class names and call signatures of hyper.deal's advection path:
//
//   AdvectionOperation::apply(dst, src, time)
//       include/hyper.deal/operators/advection/advection_operation.h:134-209
//   LowStorageRungeKuttaIntegrator(vec_Ki, vec_Ti, type, only_Ti_is_ghosted),
//   perform_time_step(solution, current_time, time_step, op), n_stages()
//       include/hyper.deal/base/time_integrators.h:47-115
//   TimeLoop::loop(solution, time_integrator, runnable, diagnostics)
//       source/base/time_loop.cc:33-67
//   VectorTools::interpolate / norm_and_error
//       include/hyper.deal/numerics/vector_tools.h:81-223
//   VlasovPoissonOperation (the right-hand side of the Vlasov-Poisson
//   application: moments, Poisson solve, field, advection)
//       examples/vlasov_poisson/include/application.h:516-602
//   PartitionedAdvectionOperation + GhostExchange (a rank's part of the
//   distributed operator and its ghost-face update)
//       include/hyper.deal/matrix_free/vector_partitioner.h:1385-1607
//
// Vectors are DeviceVector<Number> (device memory, the reference's DoF
// numbering).  Errors throw std::runtime_error with hd_last_error()'s message,
// as the reference throws dealii::ExceptionBase from AssertThrow.
#ifndef HYPERDEAL_GB300_HPP
#define HYPERDEAL_GB300_HPP

#include <cuda_runtime.h>

#include <cmath>
#include <functional>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "hyperdeal_gb300.h"

namespace hyperdeal_gb300 {

inline void check(int rc) {
  if (rc != HD_OK) {
    char buf[512];
    hd_last_error(buf, sizeof(buf));
    throw std::runtime_error(std::string("hyperdeal_gb300: ") + buf);
  }
}

inline void check_cuda(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

template <typename Number>
struct dtype_of;
template <>
struct dtype_of<double> {
  static constexpr int value = HD_F64;
};
template <>
struct dtype_of<float> {
  static constexpr int value = HD_F32;
};

// Device-resident DoF vector (owned; move-only; swap exchanges storages).
template <typename Number>
class DeviceVector {
 public:
  DeviceVector() = default;
  explicit DeviceVector(long long n) { reinit(n); }
  ~DeviceVector() { release(); }
  DeviceVector(const DeviceVector&) = delete;
  DeviceVector& operator=(const DeviceVector&) = delete;
  DeviceVector(DeviceVector&& o) noexcept { swap(o); }
  DeviceVector& operator=(DeviceVector&& o) noexcept {
    swap(o);
    return *this;
  }

  void reinit(long long n) {
    release();
    n_ = n;
    if (n > 0) {
      check_cuda(cudaMalloc(&data_, sizeof(Number) * size_t(n)), "cudaMalloc");
      check_cuda(cudaMemset(data_, 0, sizeof(Number) * size_t(n)), "cudaMemset");
    }
  }
  Number* data() { return data_; }
  const Number* data() const { return data_; }
  long long size() const { return n_; }
  void swap(DeviceVector& o) noexcept {
    std::swap(data_, o.data_);
    std::swap(n_, o.n_);
  }
  void copy_from_host(const Number* h) {
    check_cuda(cudaMemcpy(data_, h, sizeof(Number) * size_t(n_), cudaMemcpyHostToDevice), "copy to device");
  }
  void copy_to_host(Number* h) const {
    check_cuda(cudaMemcpy(h, data_, sizeof(Number) * size_t(n_), cudaMemcpyDeviceToHost), "copy to host");
  }
  std::vector<Number> to_host() const {
    std::vector<Number> v(static_cast<size_t>(n_));
    copy_to_host(v.data());
    return v;
  }

 private:
  void release() {
    if (data_) cudaFree(data_);
    data_ = nullptr;
    n_ = 0;
  }
  Number* data_ = nullptr;
  long long n_ = 0;
};

// Analytic function amp * prod_d trig_d(omega_d (x_d - speed_d t) + phase_d).
inline hd_function make_function(double amp, const std::vector<double>& omega, const std::vector<double>& speed,
                                 const std::vector<double>& phase, const std::vector<int>& cosine) {
  hd_function f{};
  f.kind = 2;
  f.amp = amp;
  for (size_t i = 0; i < omega.size() && i < HD_MAX_DIM; ++i) f.omega[i] = omega[i];
  for (size_t i = 0; i < speed.size() && i < HD_MAX_DIM; ++i) f.speed[i] = speed[i];
  for (size_t i = 0; i < phase.size() && i < HD_MAX_DIM; ++i) f.phase[i] = phase[i];
  for (size_t i = 0; i < cosine.size() && i < HD_MAX_DIM; ++i) f.cosine[i] = cosine[i];
  return f;
}

template <typename Number>
class AdvectionOperation {
 public:
  // AdvectionOperation(MatrixFree, table) + reinit(bc, velocity, param): the
  // descriptor carries mesh, degree, velocity, skew and boundary data.
  explicit AdvectionOperation(hd_adv_desc desc, cudaStream_t stream = nullptr) : stream_(stream) {
    desc.dtype = dtype_of<Number>::value;
    desc.n_points = desc.degree + 1;
    check(hd_adv_create(&desc, &h_));
  }
  ~AdvectionOperation() { hd_adv_destroy(h_); }
  AdvectionOperation(const AdvectionOperation&) = delete;
  AdvectionOperation& operator=(const AdvectionOperation&) = delete;

  // dst = M^{-1} A(src) at `time`; dst is overwritten.
  void apply(DeviceVector<Number>& dst, const DeviceVector<Number>& src, const Number time) const {
    check(hd_adv_apply(h_, dst.data(), src.data(), double(time), stream_));
  }
  // the operator signature of the reference's LSRK lambdas: op(src, dst, time)
  void operator()(const DeviceVector<Number>& src, DeviceVector<Number>& dst, const Number time) const {
    apply(dst, src, time);
  }

  long long n_dofs() const { return hd_adv_n_dofs(h_); }
  double critical_time_step() const { return hd_adv_critical_time_step(h_); }
  // pick the generic kernel's tile by timing (src read, dst overwritten)
  void autotune(const DeviceVector<Number>& src, DeviceVector<Number>& dst, int reps = 3) {
    int c = 0, p = 0;
    double ms = 0.0;
    check(hd_adv_autotune(h_, src.data(), dst.data(), reps, &c, &p, &ms, stream_));
  }
  // FP64 storage: contractions in FP64 (HD_ARITH_NATIVE) or double-word FP32 (HD_ARITH_FP32X2)
  void set_arithmetic(int arithmetic) { check(hd_adv_set_arithmetic(h_, arithmetic)); }
  hd_adv* handle() const { return h_; }
  cudaStream_t stream() const { return stream_; }
  DeviceVector<Number> create_vector() const { return DeviceVector<Number>(n_dofs()); }

 private:
  hd_adv* h_ = nullptr;
  cudaStream_t stream_;
};

// Ghost-face transport of a partitioned operator.  start() begins sending
// send_bytes of this part's packed faces to part send_to (if >= 0) and
// receiving recv_bytes into `ghost` (the ghost region of the vector being
// exchanged) from part recv_from (if >= 0), after the work already queued on
// `stream`; finish() makes `stream` wait for both.  An MPI implementation
// calls MPI_Isend / MPI_Irecv in start (CUDA-aware MPI, or through host
// buffers after a stream synchronisation) and MPI_Waitall in finish, the way
// the reference's Contiguous partitioner runs update_ghost_values_start /
// _finish (include/hyper.deal/matrix_free/vector_partitioner.h:1385-1607).
class GhostExchange {
 public:
  virtual ~GhostExchange() = default;
  virtual void start(const void* sendbuf, size_t send_bytes, int send_to, void* ghost, size_t recv_bytes,
                     int recv_from, cudaStream_t stream) = 0;
  virtual void finish(cudaStream_t stream) = 0;
};

// One v-slab part of the advection operator (hd_adv_create_part): its vectors
// hold the part's cells followed by the ghost region of the upwind part's
// faces.  apply() and LowStorageRungeKuttaIntegrator::perform_time_step
// exchange the operator input's faces before every evaluation and overlap the
// exchange with the cells that do not read the ghost region
// (matrix_free.templates.h:1178-1234, :1494-1581).
template <typename Number>
class PartitionedAdvectionOperation {
 public:
  PartitionedAdvectionOperation(hd_adv_desc desc, int n_parts, int part, cudaStream_t stream = nullptr)
      : stream_(stream) {
    desc.dtype = dtype_of<Number>::value;
    desc.n_points = desc.degree + 1;
    check(hd_adv_create_part(&desc, n_parts, part, &h_));
    check(hd_adv_part_layout(h_, &layout_));
    if (layout_.send_to >= 0) sendbuf_.reinit(layout_.layer_cells * layout_.face_values);
  }
  ~PartitionedAdvectionOperation() { hd_adv_destroy(h_); }
  PartitionedAdvectionOperation(const PartitionedAdvectionOperation&) = delete;
  PartitionedAdvectionOperation& operator=(const PartitionedAdvectionOperation&) = delete;

  long long n_dofs() const { return hd_adv_n_dofs(h_); }
  long long ghost_values() const { return layout_.ghost_values; }
  const hd_part_layout& layout() const { return layout_; }
  double critical_time_step() const { return hd_adv_critical_time_step(h_); }
  DeviceVector<Number> create_vector() const { return DeviceVector<Number>(n_dofs() + ghost_values()); }
  hd_adv* handle() const { return h_; }
  cudaStream_t stream() const { return stream_; }
  // this part's packed faces (valid after pack())
  const DeviceVector<Number>& send_buffer() const { return sendbuf_; }

  // the steps of an exchange, for drivers that interleave several parts
  void pack(const DeviceVector<Number>& v) {
    if (layout_.send_to >= 0) check(hd_adv_pack_faces(h_, v.data(), sendbuf_.data(), stream_));
  }
  void exchange_start(GhostExchange& ex, DeviceVector<Number>& v) {
    ex.start(sendbuf_.data(), sizeof(Number) * size_t(layout_.send_to >= 0 ? sendbuf_.size() : 0), layout_.send_to,
             v.data() + n_dofs(), sizeof(Number) * size_t(layout_.ghost_values), layout_.recv_from, stream_);
  }
  void apply_cells(DeviceVector<Number>& dst, const DeviceVector<Number>& src, const Number time, int cells) const {
    check(hd_adv_apply_cells(h_, dst.data(), src.data(), double(time), cells, stream_));
  }

  // dst = M^{-1} A(src): src's ghost region is filled through `ex` first
  void apply(DeviceVector<Number>& dst, DeviceVector<Number>& src, const Number time, GhostExchange& ex) {
    pack(src);
    exchange_start(ex, src);
    apply_cells(dst, src, time, HD_CELLS_INTERIOR);
    ex.finish(stream_);
    apply_cells(dst, src, time, HD_CELLS_BOUNDARY);
  }

 private:
  hd_adv* h_ = nullptr;
  cudaStream_t stream_;
  hd_part_layout layout_{};
  DeviceVector<Number> sendbuf_;
};

// The Vlasov-Poisson right-hand side f -> A(f) with the field of f
// (application.h:516-602); Gauss-Lobatto collocation, periodic meshes.
template <typename Number>
class VlasovPoissonOperation {
 public:
  explicit VlasovPoissonOperation(hd_vp_desc desc, cudaStream_t stream = nullptr)
      : stream_(stream), dim_x_(desc.dim_x) {
    desc.dtype = dtype_of<Number>::value;
    check(hd_vp_create(&desc, &h_));
  }
  ~VlasovPoissonOperation() { hd_vp_destroy(h_); }
  VlasovPoissonOperation(const VlasovPoissonOperation&) = delete;
  VlasovPoissonOperation& operator=(const VlasovPoissonOperation&) = delete;

  // dst = A(src) with the field of src (moments, Poisson solve, field, advection)
  void apply(DeviceVector<Number>& dst, const DeviceVector<Number>& src, const Number time) const {
    check(hd_vp_apply(h_, dst.data(), src.data(), double(time), stream_));
  }
  void operator()(const DeviceVector<Number>& src, DeviceVector<Number>& dst, const Number time) const {
    apply(dst, src, time);
  }
  void interpolate(const hd_function& f, DeviceVector<Number>& dst, double time = 0.0) const {
    check(hd_vp_interpolate(h_, &f, time, dst.data(), stream_));
  }
  // field energy per x-direction, mass, L2 norm, kinetic energy, momentum per
  // v-direction (diagnostics.h:28-141); the field is the last evaluation's
  std::vector<double> diagnostics(const DeviceVector<Number>& f) const {
    std::vector<double> out(size_t(2 * dim_x_ + 3), 0.0);
    check(hd_vp_diagnostics(h_, f.data(), out.data(), stream_));
    return out;
  }
  long long n_dofs() const { return hd_vp_n_dofs(h_); }
  // FP64 storage: advection contractions in FP64 (HD_ARITH_NATIVE) or double-word FP32 (HD_ARITH_FP32X2)
  void set_arithmetic(int arithmetic) { check(hd_vp_set_arithmetic(h_, arithmetic)); }
  hd_vp* handle() const { return h_; }
  cudaStream_t stream() const { return stream_; }
  DeviceVector<Number> create_vector() const { return DeviceVector<Number>(n_dofs()); }

 private:
  hd_vp* h_ = nullptr;
  cudaStream_t stream_;
  int dim_x_;
};

// perturbed Maxwellian (1 + amp prod_{d in pert} cos(k x_d)) prod_v exp(-v^2/2)/sqrt(2 pi)
// (examples/vlasov_poisson/cases/hyperrectangle.h:45-58)
inline hd_function perturbed_maxwellian(int dim_x, double amp, double k, const std::vector<int>& perturbed_dims) {
  hd_function f{};
  f.kind = 3;
  f.amp = amp;
  for (int d = 0; d < dim_x; ++d) f.omega[d] = k;
  for (int d : perturbed_dims) f.cosine[d] = 1;
  for (int d = 0; d < dim_x; ++d) f.cosine[dim_x + d] = 2;
  return f;
}

template <typename Number>
class LowStorageRungeKuttaIntegrator {
 public:
  using Operator = std::function<void(const DeviceVector<Number>&, DeviceVector<Number>&, Number)>;

  LowStorageRungeKuttaIntegrator(DeviceVector<Number>& vec_Ki, DeviceVector<Number>& vec_Ti, const std::string& type,
                                 const bool only_Ti_is_ghosted = true)
      : Ki_(vec_Ki), Ti_(vec_Ti), only_Ti_is_ghosted_(only_Ti_is_ghosted) {
    check(hd_lsrk_create(type.c_str(), &rk_));
    ns_ = hd_lsrk_n_stages(rk_);
    ai_.resize(ns_);
    bi_.resize(ns_);
    ci_.resize(ns_);
    check(hd_lsrk_coefficients(rk_, ai_.data(), bi_.data(), ci_.data()));
  }
  ~LowStorageRungeKuttaIntegrator() { hd_lsrk_destroy(rk_); }
  LowStorageRungeKuttaIntegrator(const LowStorageRungeKuttaIntegrator&) = delete;
  LowStorageRungeKuttaIntegrator& operator=(const LowStorageRungeKuttaIntegrator&) = delete;

  unsigned int n_stages() const { return unsigned(ns_); }

  // Fused: every stage is one kernel (operator + stage update).  The three
  // vectors rotate roles; storages are swapped back so that `solution` holds
  // the new state and vec_Ki / vec_Ti are scratch, as in the reference.
  void perform_time_step(DeviceVector<Number>& solution, const Number current_time, const Number time_step,
                         const AdvectionOperation<Number>& op) {
    void* s = solution.data();
    void* k = Ki_.data();
    void* t = Ti_.data();
    void* ki_storage = k;
    check(hd_lsrk_step(op.handle(), rk_, &s, &k, &t, double(current_time), double(time_step), op.stream()));
    if (s == ki_storage) solution.swap(Ki_);
  }

  // The Vlasov-Poisson operator: the stage update fused into its advection
  // kernel (hd_vp_lsrk_step_fused), vectors rotating as above.
  void perform_time_step(DeviceVector<Number>& solution, const Number current_time, const Number time_step,
                         const VlasovPoissonOperation<Number>& op) {
    void* s = solution.data();
    void* k = Ki_.data();
    void* t = Ti_.data();
    void* ki_storage = k;
    check(hd_vp_lsrk_step_fused(op.handle(), rk_, &s, &k, &t, double(current_time), double(time_step), op.stream()));
    if (s == ki_storage) solution.swap(Ki_);
  }

  // A part of a partitioned operator: the fused step stage by stage, the
  // stage input's faces exchanged through `ex` before every stage while the
  // interior cells run; the vectors rotate and are swapped back as above.
  void perform_time_step(DeviceVector<Number>& solution, const Number current_time, const Number time_step,
                         PartitionedAdvectionOperation<Number>& op, GhostExchange& ex) {
    DeviceVector<Number>* X[3] = {&solution, &Ki_, &Ti_};
    for (int s = 0; s < ns_; ++s) {
      DeviceVector<Number>& in = *X[hd_lsrk_stage_input(rk_, s)];
      op.pack(in);
      op.exchange_start(ex, in);
      stage(op, s, X, current_time, time_step, HD_CELLS_INTERIOR);
      ex.finish(op.stream());
      stage(op, s, X, current_time, time_step, HD_CELLS_BOUNDARY);
    }
    solution.swap(Ki_);  // the new solution was accumulated in X[1] = vec_Ki
  }

  // one stage of the fused step of a part on a cell subset (drivers that
  // interleave several parts call this between their exchanges)
  void stage(const PartitionedAdvectionOperation<Number>& op, int s, DeviceVector<Number>* const X[3],
             const Number current_time, const Number time_step, int cells) const {
    void* ptr[3] = {X[0]->data(), X[1]->data(), X[2]->data()};
    check(hd_lsrk_stage(op.handle(), rk_, s, ptr, double(current_time), double(time_step), cells, op.stream()));
  }
  int stage_input(int s) const { return hd_lsrk_stage_input(rk_, s); }

  // Any operator op(src, dst, t): the reference's stage sequence
  // (time_integrators.templates.h:91-184) with the CUDA vector update.
  void perform_time_step(DeviceVector<Number>& solution, const Number current_time, const Number time_step,
                         const Operator& op, cudaStream_t stream = nullptr) {
    const long long n = solution.size();
    const DeviceVector<Number>* cur = &solution;
    if (only_Ti_is_ghosted_) {
      check_cuda(cudaMemcpyAsync(Ti_.data(), solution.data(), sizeof(Number) * size_t(n), cudaMemcpyDeviceToDevice,
                                 stream),
                 "copy solution -> Ti");
      cur = &Ti_;
    }
    for (int s = 0; s < ns_; ++s) {
      op(*cur, Ki_, Number(current_time + ci_[s] * time_step));
      const double ai = s == ns_ - 1 ? 0.0 : ai_[s] * time_step;
      check(hd_lsrk_stage_update(dtype_of<Number>::value, n, bi_[s] * time_step, ai, Ki_.data(), solution.data(),
                                 Ti_.data(), stream));
      cur = &Ti_;
    }
  }

 private:
  DeviceVector<Number>& Ki_;
  DeviceVector<Number>& Ti_;
  bool only_Ti_is_ghosted_;
  hd_lsrk* rk_ = nullptr;
  int ns_ = 0;
  std::vector<double> ai_, bi_, ci_;
};

// Fixed-step time loop (source/base/time_loop.cc:33-67): diagnostics at the
// start time and after every step; final_time * (1 + 1e-13) guards round-off.
template <typename Number, typename Vector>
class TimeLoop {
 public:
  TimeLoop(Number time_step, Number start_time, Number final_time, unsigned max_steps = 100000000u)
      : dt_(time_step), t0_(start_time), t1_(final_time), max_steps_(max_steps) {}

  template <typename Integrator, typename Runnable, typename Diagnostics>
  int loop(Vector& solution, Integrator&& time_integrator, Runnable&& runnable, Diagnostics&& diagnostics) const {
    unsigned n = 1;
    diagnostics(t0_);
    for (Number t = t0_ + dt_; t <= t1_ * Number(1.0000000000001) && n <= max_steps_; t += dt_, ++n) {
      time_integrator(solution, t - dt_, dt_, runnable);
      diagnostics(t);
    }
    return int(n - 1);
  }

 private:
  Number dt_, t0_, t1_;
  unsigned max_steps_;
};

struct VectorTools {
  template <typename Number>
  static void interpolate(const AdvectionOperation<Number>& op, const hd_function& f, DeviceVector<Number>& dst,
                          const double time = 0.0) {
    check(hd_interpolate(op.handle(), &f, time, dst.data(), op.stream()));
  }
  // {L2 norm of src, L2 error against f(., time)} at the collocation points
  template <typename Number>
  static std::pair<double, double> norm_and_error(const AdvectionOperation<Number>& op, const hd_function& f,
                                                  const DeviceVector<Number>& src, const double time) {
    double r[2] = {0.0, 0.0};
    check(hd_norm_and_error(op.handle(), &f, time, src.data(), r, op.stream()));
    return {r[0], r[1]};
  }
};

// dt = min(TimeStep, CFL * dt_crit / k^1.5), then T / ceil(T / dt)
// (examples/advection/include/application.h:363-392)
inline double time_step_rule(double time_step, double cfl, double critical, int degree, double start, double final) {
  const double dt = std::fmin(time_step, cfl * critical / std::pow(double(degree), 1.5));
  return (final - start) / std::ceil((final - start) / dt);
}

}  // namespace hyperdeal_gb300

#endif  // HYPERDEAL_GB300_HPP
