// partitioned_advection.cc -- the partitioned operator through the C++
// interface include/hyperdeal_gb300.hpp: n_parts v-slab parts of one mesh in
// this process, their ghost faces moved by device copies (LocalExchange, a
// stand-in for the MPI transport of a multi-rank run), stepped in lockstep
// stage by stage with the exchange before every stage, and compared with the
// single operator.  Prints "max_diff <apply> <steps>"; both are 0 when the
// parts reproduce the single operator bit for bit.
//
// usage: partitioned_advection dim_x dim_v degree cells n_parts steps [f64|f32]
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <memory>
#include <string>
#include <vector>

#include "hyperdeal_gb300.hpp"

using namespace hyperdeal_gb300;

// device copies between parts of this process: the receiver copies its
// upwind part's packed faces (which the driver packs before any start)
template <typename Number>
class LocalExchange : public GhostExchange {
 public:
  explicit LocalExchange(const std::vector<std::unique_ptr<PartitionedAdvectionOperation<Number>>>& parts)
      : parts_(parts) {}
  void start(const void*, size_t, int, void* ghost, size_t recv_bytes, int recv_from, cudaStream_t stream) override {
    if (recv_from < 0) return;
    check_cuda(cudaMemcpyAsync(ghost, parts_[recv_from]->send_buffer().data(), recv_bytes, cudaMemcpyDeviceToDevice,
                               stream),
               "ghost copy");
  }
  void finish(cudaStream_t) override {}  // same stream: ordered

 private:
  const std::vector<std::unique_ptr<PartitionedAdvectionOperation<Number>>>& parts_;
};

template <typename Number>
double max_diff(const std::vector<Number>& a, const std::vector<Number>& b) {
  double m = 0.0;
  for (size_t i = 0; i < a.size(); ++i) m = std::fmax(m, std::fabs(double(a[i]) - double(b[i])));
  return m;
}

template <typename Number>
int run(int dim_x, int dim_v, int degree, int cells, int n_parts, int steps) {
  const int dim = dim_x + dim_v;
  hd_adv_desc desc{};
  desc.dim_x = dim_x;
  desc.dim_v = dim_v;
  desc.degree = degree;
  for (int d = 0; d < 3; ++d) {
    desc.cells_x[d] = desc.cells_v[d] = cells;
    desc.lo_x[d] = desc.lo_v[d] = 0.0;
    desc.hi_x[d] = desc.hi_v[d] = 1.0;
  }
  desc.periodic_x = desc.periodic_v = 1;
  const double vel[6] = {1.0, -0.8, 0.6, 0.4, -0.3, 0.2};
  for (int d = 0; d < dim; ++d) desc.velocity[d] = vel[d];
  std::vector<double> omega(dim, 2.0 * M_PI), speed(dim, 0.0), phase(dim, 0.3);
  std::vector<int> cosine(dim, 0);
  const hd_function f0 = make_function(1.0, omega, speed, phase, cosine);

  // the single operator
  AdvectionOperation<Number> op(desc);
  DeviceVector<Number> u = op.create_vector(), ref = op.create_vector(), Ki = op.create_vector(),
                       Ti = op.create_vector();
  VectorTools::interpolate(op, f0, u, 0.0);
  op.apply(ref, u, Number(0.1));
  const std::vector<Number> ref_apply = ref.to_host();
  const double dt = 0.2 * op.critical_time_step() / std::pow(double(degree), 1.5);
  LowStorageRungeKuttaIntegrator<Number> rk(Ki, Ti, "rk45");
  for (int s = 0; s < steps; ++s) rk.perform_time_step(u, Number(s * dt), Number(dt), op);
  const std::vector<Number> ref_steps = u.to_host();

  // the parts
  std::vector<std::unique_ptr<PartitionedAdvectionOperation<Number>>> parts;
  for (int p = 0; p < n_parts; ++p) parts.emplace_back(new PartitionedAdvectionOperation<Number>(desc, n_parts, p));
  LocalExchange<Number> ex(parts);
  std::vector<DeviceVector<Number>> src, dst, Kp, Tp;
  for (auto& p : parts) {
    src.push_back(p->create_vector());
    dst.push_back(p->create_vector());
    Kp.push_back(p->create_vector());
    Tp.push_back(p->create_vector());
  }
  std::vector<std::unique_ptr<LowStorageRungeKuttaIntegrator<Number>>> rks;
  for (int p = 0; p < n_parts; ++p)
    rks.emplace_back(new LowStorageRungeKuttaIntegrator<Number>(Kp[p], Tp[p], "rk45"));
  // each part's cells of the initial data: interpolate on the part itself (hd_interpolate)
  for (int p = 0; p < n_parts; ++p) check(hd_interpolate(parts[p]->handle(), &f0, 0.0, src[p].data(), nullptr));

  // apply, all parts: pack every part, then exchange, interior, boundary
  for (int p = 0; p < n_parts; ++p) parts[p]->pack(src[p]);
  for (int p = 0; p < n_parts; ++p) {
    parts[p]->exchange_start(ex, src[p]);
    parts[p]->apply_cells(dst[p], src[p], Number(0.1), HD_CELLS_INTERIOR);
    ex.finish(parts[p]->stream());
    parts[p]->apply_cells(dst[p], src[p], Number(0.1), HD_CELLS_BOUNDARY);
  }
  std::vector<Number> got_apply;
  for (int p = 0; p < n_parts; ++p) {
    std::vector<Number> h = dst[p].to_host();
    got_apply.insert(got_apply.end(), h.begin(), h.begin() + parts[p]->n_dofs());
  }
  // fused rk45 steps in lockstep, the stage input's faces exchanged before every stage
  for (int s = 0; s < steps; ++s) {
    for (int st = 0; st < int(rks[0]->n_stages()); ++st) {
      std::vector<DeviceVector<Number>*> in(n_parts);
      for (int p = 0; p < n_parts; ++p) {
        DeviceVector<Number>* X[3] = {&src[p], &Kp[p], &Tp[p]};
        in[p] = X[rks[p]->stage_input(st)];
        parts[p]->pack(*in[p]);
      }
      for (int p = 0; p < n_parts; ++p) {
        DeviceVector<Number>* X[3] = {&src[p], &Kp[p], &Tp[p]};
        parts[p]->exchange_start(ex, *in[p]);
        rks[p]->stage(*parts[p], st, X, Number(s * dt), Number(dt), HD_CELLS_INTERIOR);
        ex.finish(parts[p]->stream());
        rks[p]->stage(*parts[p], st, X, Number(s * dt), Number(dt), HD_CELLS_BOUNDARY);
      }
    }
    for (int p = 0; p < n_parts; ++p) src[p].swap(Kp[p]);
  }
  std::vector<Number> got_steps;
  for (int p = 0; p < n_parts; ++p) {
    std::vector<Number> h = src[p].to_host();
    got_steps.insert(got_steps.end(), h.begin(), h.begin() + parts[p]->n_dofs());
  }
  std::printf("max_diff %.17g %.17g\n", max_diff(got_apply, ref_apply), max_diff(got_steps, ref_steps));
  return 0;
}

int main(int argc, char** argv) {
  if (argc < 7) {
    std::fprintf(stderr, "usage: %s dim_x dim_v degree cells n_parts steps [f64|f32]\n", argv[0]);
    return 2;
  }
  const int dim_x = std::atoi(argv[1]), dim_v = std::atoi(argv[2]), degree = std::atoi(argv[3]);
  const int cells = std::atoi(argv[4]), n_parts = std::atoi(argv[5]), steps = std::atoi(argv[6]);
  const std::string dtype = argc > 7 ? argv[7] : "f64";
  try {
    return dtype == "f32" ? run<float>(dim_x, dim_v, degree, cells, n_parts, steps)
                          : run<double>(dim_x, dim_v, degree, cells, n_parts, steps);
  } catch (const std::exception& e) {
    std::fprintf(stderr, "error: %s\n", e.what());
    return 1;
  }
}
