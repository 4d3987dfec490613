// vlasov_poisson_hyperrectangle.cc -- the reference's Vlasov-Poisson
// application for its `hyperrectangle` case (examples/vlasov_poisson/
// include/application.h:345-602, cases/hyperrectangle.h:29-70) driven
// through the C++ interface include/hyperdeal_gb300.hpp on one GPU:
// x in [0, 4 pi]^dim_x, v in [-6, 6]^dim_x, periodic, f0 the perturbed
// Maxwellian with cos(0.5 x_0), the time-step rule with the transport
// velocity (1, .., 6, ..), rk45.  Prints "Time" and the diagnostics
// (field energy per x-direction, mass, L2 norm, kinetic energy, momentum)
// at every tick.  Gauss-Lobatto collocation, or Gauss quadrature with k + 1
// points (the reference's non-collocation runs, e.g. its VP golden).
//
// usage: vlasov_poisson_hyperrectangle dim_x degree cells_x cells_v final_time [f64|f32] [cfl tick] [gl|gauss]
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "hyperdeal_gb300.hpp"

using namespace hyperdeal_gb300;

template <typename Number>
int run(int dim_x, int degree, int cells_x, int cells_v, double final_time, double cfl, double tick, bool gauss) {
  hd_vp_desc desc{};
  desc.dim_x = desc.dim_v = dim_x;
  desc.degree = degree;
  for (int d = 0; d < dim_x; ++d) {
    desc.cells_x[d] = cells_x;
    desc.cells_v[d] = cells_v;
    desc.lo_x[d] = 0.0;
    desc.hi_x[d] = 4.0 * M_PI;
    desc.lo_v[d] = -6.0;
    desc.hi_v[d] = 6.0;
  }
  desc.cg_tol = 1e-12;
  desc.cg_max_iter = 100000;
  desc.guess = HD_VP_GUESS_PREVIOUS;
  desc.quadrature = gauss ? HD_QUAD_GAUSS : HD_QUAD_GAUSS_LOBATTO;
  VlasovPoissonOperation<Number> op(desc);
  DeviceVector<Number> f = op.create_vector(), Ki = op.create_vector(), Ti = op.create_vector();
  op.interpolate(perturbed_maxwellian(dim_x, 0.01, 0.5, {0}), f);
  LowStorageRungeKuttaIntegrator<Number> integrator(Ki, Ti, "rk45");
  // cfl.h:56-124 with the transport velocity (1, .., 6, ..)
  const double hx = 4.0 * M_PI / cells_x, hv = 12.0 / cells_v;
  const double critical = std::fmin(hx / 1.0, hv / 6.0);
  const double dt = time_step_rule(0.1, cfl, critical, degree, 0.0, final_time);
  TimeLoop<double, DeviceVector<Number>> loop(dt, 0.0, final_time);
  loop.loop(
      f,
      [&](DeviceVector<Number>& sol, double t, double h, const VlasovPoissonOperation<Number>& o) {
        integrator.perform_time_step(sol, Number(t), Number(h), o);
      },
      op,
      [&](double t) {
        if (t != 0.0 && int((t + 0.00000000001) / tick) == int((t + 0.00000000001 - dt) / tick)) return;
        const std::vector<double> d = op.diagnostics(f);
        std::printf("   Time:%17.10e", t);
        for (double x : d) std::printf(" %17.10e", x);
        std::printf("\n");
      });
  return 0;
}

int main(int argc, char** argv) {
  if (argc < 6) {
    std::fprintf(stderr, "usage: %s dim_x degree cells_x cells_v final_time [f64|f32] [cfl tick] [gl|gauss]\n",
                 argv[0]);
    return 2;
  }
  const int dim_x = std::atoi(argv[1]), degree = std::atoi(argv[2]);
  const int cx = std::atoi(argv[3]), cv = std::atoi(argv[4]);
  const double final_time = std::atof(argv[5]);
  const std::string dtype = argc > 6 ? argv[6] : "f64";
  const double cfl = argc > 7 ? std::atof(argv[7]) : 0.05;
  const double tick = argc > 8 ? std::atof(argv[8]) : 0.1;
  const bool gauss = argc > 9 && std::string(argv[9]) == "gauss";
  try {
    if (dtype == "f32") return run<float>(dim_x, degree, cx, cv, final_time, cfl, tick, gauss);
    return run<double>(dim_x, degree, cx, cv, final_time, cfl, tick, gauss);
  } catch (const std::exception& e) {
    std::fprintf(stderr, "error: %s\n", e.what());
    return 1;
  }
}
