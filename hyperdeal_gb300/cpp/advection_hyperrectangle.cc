// advection_hyperrectangle.cc -- the reference's advection application for
// its `hyperrectangle` case (examples/advection/advection.cc,
// examples/advection/include/application.h:96-567,
// examples/advection/cases/hyperrectangle.h:29-235) driven through the C++
// interface include/hyperdeal_gb300.hpp on one GPU.
//
// Prints the diagnostics lines of the reference ("Time, norm, error" at every
// DiagnosticsTick) so its output can be compared with the reference's .out
// files.  Gauss-Lobatto collocation (DoCollocation = true) or, with the
// `gauss` argument, Gauss quadrature.  Storage f64 (FP64 arithmetic), f64x
// (FP64 storage, double-word FP32 contractions) or f32.
//
// usage: advection_hyperrectangle dim_x dim_v degree subdivisions periodic(0|1)
//                                 final_time rk_type [f64|f64x|f32] [time_step cfl tick] [gauss]
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "hyperdeal_gb300.hpp"

using namespace hyperdeal_gb300;

template <typename Number>
int run(int dim_x, int dim_v, int degree, int subdivisions, bool periodic, double final_time, const std::string& rk,
        double time_step, double cfl, double tick, bool gauss, bool fp32x2) {
  const int dim = dim_x + dim_v;
  // ExactSolution: sin(2 pi (x0 - a0 t)) prod_{d>=1} cos(2 pi (x_d - a_d t)), a = (1, 0.15, -0.05, 0, ...),
  // domain [-1, 1]^dim, Dirichlet data = the exact solution (hyperrectangle.h:29-66, :220-235)
  const double adv[6] = {1.0, 0.15, -0.05, 0.0, 0.0, 0.0};
  std::vector<double> omega(dim, 2.0 * M_PI), speed(adv, adv + dim), phase(dim, 0.0);
  std::vector<int> cosine(dim, 1);
  cosine[0] = 0;
  const hd_function exact = make_function(1.0, omega, speed, phase, cosine);

  hd_adv_desc desc{};
  desc.dim_x = dim_x;
  desc.dim_v = dim_v;
  desc.degree = degree;
  for (int d = 0; d < 3; ++d) {
    desc.cells_x[d] = desc.cells_v[d] = subdivisions;
    desc.lo_x[d] = desc.lo_v[d] = -1.0;
    desc.hi_x[d] = desc.hi_v[d] = 1.0;
  }
  desc.periodic_x = desc.periodic_v = periodic ? 1 : 0;
  for (int d = 0; d < dim; ++d) desc.velocity[d] = adv[d];
  desc.bc_kind = periodic ? HD_BC_HOMOGENEOUS : HD_BC_FUNCTION;
  desc.bc = exact;
  desc.quadrature = gauss ? HD_QUAD_GAUSS : HD_QUAD_GAUSS_LOBATTO;

  AdvectionOperation<Number> op(desc);
  if (fp32x2) op.set_arithmetic(HD_ARITH_FP32X2);
  DeviceVector<Number> solution = op.create_vector(), Ki = op.create_vector(), Ti = op.create_vector();
  VectorTools::interpolate(op, exact, solution, 0.0);
  LowStorageRungeKuttaIntegrator<Number> integrator(Ki, Ti, rk);

  const double dt = time_step_rule(time_step, cfl, op.critical_time_step(), degree, 0.0, final_time);
  TimeLoop<double, DeviceVector<Number>> loop(dt, 0.0, final_time);
  loop.loop(
      solution,
      [&](DeviceVector<Number>& sol, double t, double h, const AdvectionOperation<Number>& o) {
        integrator.perform_time_step(sol, Number(t), Number(h), o);
      },
      op,
      [&](double t) {
        // application.h:464-471
        if (t != 0.0 && int((t + 0.00000000001) / tick) == int((t + 0.00000000001 - dt) / tick)) return;
        const auto ne = VectorTools::norm_and_error(op, exact, solution, t);
        std::printf("   Time:%10.3e, norm: %17.10e, error: %17.10e\n", t, ne.first, ne.second);
      });
  return 0;
}

int main(int argc, char** argv) {
  if (argc < 8) {
    std::fprintf(stderr,
                 "usage: %s dim_x dim_v degree subdivisions periodic final_time rk [f64|f64x|f32] "
                 "[time_step cfl tick] [gauss]\n",
                 argv[0]);
    return 2;
  }
  const int dim_x = std::atoi(argv[1]), dim_v = std::atoi(argv[2]), degree = std::atoi(argv[3]);
  const int sub = std::atoi(argv[4]);
  const bool periodic = std::atoi(argv[5]) != 0;
  const double final_time = std::atof(argv[6]);
  const std::string rk = argv[7];
  const std::string dtype = argc > 8 ? argv[8] : "f64";
  const double time_step = argc > 9 ? std::atof(argv[9]) : 0.1;
  const double cfl = argc > 10 ? std::atof(argv[10]) : 0.3;
  const double tick = argc > 11 ? std::atof(argv[11]) : 0.1;
  const bool gauss = argc > 12 && std::string(argv[12]) == "gauss";
  try {
    if (dtype == "f32")
      return run<float>(dim_x, dim_v, degree, sub, periodic, final_time, rk, time_step, cfl, tick, gauss, false);
    return run<double>(dim_x, dim_v, degree, sub, periodic, final_time, rk, time_step, cfl, tick, gauss,
                       dtype == "f64x");
  } catch (const std::exception& e) {
    std::fprintf(stderr, "error: %s\n", e.what());
    return 1;
  }
}
