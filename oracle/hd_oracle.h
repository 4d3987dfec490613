/*
 * hd_oracle.h -- CPU restatement of hyper.deal's phase-space upwind-DG
 * advection path (TEST INFRASTRUCTURE ONLY).
 *
 * This header and hd_oracle.c are the oracle against which the CUDA path of
 * hyperdeal_gb300 is checked.  Only the test suite, the smoke check and the
 * CPU-baseline leg of bench.py load it.  Nothing in the product library links
 * or calls it.
 *
 * What is restated (reference = hyper.deal, paths relative to its root):
 *   - ECL advection operator, collocation and Gauss (n_points = degree+1)
 *     branches, skew-symmetric form, periodic / Dirichlet faces:
 *       include/hyper.deal/operators/advection/advection_operation.h:218-566
 *   - metric terms of a Cartesian cell (JxW, inverse Jacobian, normals):
 *       include/hyper.deal/matrix_free/fe_evaluation_cell.h:219-348,
 *       include/hyper.deal/matrix_free/fe_evaluation_face.h:381-463,
 *       include/hyper.deal/matrix_free/fe_evaluation_cell_inverse.h:117-134
 *   - face node tables (which cell nodes a face reads):
 *       include/hyper.deal/matrix_free/shape_info.h:63-160
 *   - low-storage Runge-Kutta (rk33, rk45, rk47, rk59):
 *       include/hyper.deal/base/time_integrators.templates.h:22-184
 *   - nodal interpolation and L2 norm / error:
 *       include/hyper.deal/numerics/vector_tools.h:81-223
 *   - critical time step:  include/hyper.deal/operators/advection/cfl.h:56-124
 *   - DoF numbering: cell gid = gid_x + n_cells_x * gid_v with lexicographic
 *     cell order, node index = i_x + n^dim_x * i_v (lexicographic):
 *       include/hyper.deal/matrix_free/matrix_free.templates.h:535-563,
 *       include/hyper.deal/matrix_free/shape_info.h:141-160
 *
 * The Gauss-Lobatto / Gauss rules and Lagrange derivative matrices, which the
 * reference takes from deal.II (not part of the reference tree; CMake minimum
 * deal.II 9.1), are computed here from the Legendre recurrence with Newton
 * iterations (the published construction of these rules).
 */
#ifndef HD_ORACLE_H
#define HD_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

#define HDO_MAX_DIM 6
#define HDO_MAX_POINTS 8

/* Analytic scalar function used for initial data, exact solutions and
 * inhomogeneous Dirichlet data:
 *   kind 0: f = 0
 *   kind 1: f = amp
 *   kind 2: f = amp * prod_d trig_d(omega_d * (x_d - speed_d * t) + phase_d)
 *           with trig_d = cos if cosine[d] else sin.
 *   kind 3: f = (1 + amp * prod_{cosine[d]==1} cos(omega_d x_d + phase_d))
 *               * prod_{cosine[d]==2} exp(-x_d^2 / 2) / sqrt(2 pi)
 *           (perturbed Maxwellian of the Vlasov-Poisson cases).           */
typedef struct hdo_func {
  int kind;
  double amp;
  double omega[HDO_MAX_DIM];
  double speed[HDO_MAX_DIM];
  double phase[HDO_MAX_DIM];
  int cosine[HDO_MAX_DIM];
} hdo_func;

/* One phase-space advection problem on a Cartesian tensor-product mesh. */
typedef struct hdo_problem {
  int dim_x, dim_v;     /* 1..3 each                                     */
  int degree;           /* polynomial degree k                           */
  int n_points;         /* quadrature points per direction (= degree+1)  */
  int collocation;      /* 1: Gauss-Lobatto collocation, 0: Gauss        */
  int cells[HDO_MAX_DIM];
  double lo[HDO_MAX_DIM], hi[HDO_MAX_DIM];
  int periodic_x, periodic_v;
  double velocity[HDO_MAX_DIM];
  double skew;          /* skew-symmetric factor (0 = convective form)   */
  int bc_inhomogeneous; /* non-periodic faces: 0 -> u+ = -u-, 1 -> u+ = -u- + 2 g */
  hdo_func bc_func;     /* g(x, t) for bc_inhomogeneous                  */
  int n_threads;        /* 0: OpenMP default                             */
  /* Vlasov-Poisson phase-space velocity (dim_x == dim_v): when non-NULL the
     x-velocity is the point's v-coordinate and the v-velocity is
     efield[(gid_x * n^dim_x + qx) * dim_x + d] (the gradient of the
     potential at the x-quadrature points; velocity_field_view.h:103-209 of
     the vlasov_poisson example); `velocity` is then unused. */
  const double *efield;
} hdo_problem;

/* number of DoFs of the problem */
long long hdo_n_dofs(const hdo_problem *p);

/* 1D rules on [0,1]: Gauss-Lobatto (n >= 2) and Gauss (n >= 1) */
int hdo_gauss_lobatto(int n, double *x, double *w);
int hdo_gauss(int n, double *x, double *w);

/* dst = A(src) at time t (ECL operator incl. inverse mass); returns 0 on success */
int hdo_apply(const hdo_problem *p, const double *src, double *dst, double time);

/* the same operator evaluated only on the cells listed in `cells`; the
 * result of cells[i] is written to dst[i*(k+1)^D ...] (compact); neighbours
 * are read from the full src.  The _f32 form reads a float vector.         */
int hdo_apply_cells(const hdo_problem *p, const double *src, double *dst, double time,
                    const long long *cells, long long n_cells);
int hdo_apply_cells_f32(const hdo_problem *p, const float *src, double *dst, double time,
                        const long long *cells, long long n_cells);

/* one low-storage RK step (only_Ti_is_ghosted = true form); type = "rk33",
 * "rk45", "rk47", "rk59"; Ki and Ti are work vectors of n_dofs.           */
int hdo_lsrk_step(const hdo_problem *p, const char *type, double *sol,
                  double *Ki, double *Ti, double time, double dt);

/* number of stages of an LSRK scheme (0 if unknown) and its coefficients */
int hdo_lsrk_coefficients(const char *type, double *ai, double *bi);

/* same LSRK step with a user operator op(src, dst, t, ctx) */
typedef void (*hdo_operator)(const double *src, double *dst, double t, void *ctx);
int hdo_lsrk_step_op(long long n, const char *type, double *sol, double *Ki,
                     double *Ti, double time, double dt, hdo_operator op, void *ctx);

/* nodal interpolation of f(., t) at the Gauss-Lobatto support points */
int hdo_interpolate(const hdo_problem *p, const hdo_func *f, double time, double *dst);

/* L2 norm of src and L2 error against f(., t) with quadrature 0 of the
 * problem (Gauss-Lobatto under collocation, Gauss otherwise).            */
int hdo_norm_and_error(const hdo_problem *p, const hdo_func *f, double time,
                       const double *src, double *norm_error);

/* 1 / max_d |a_d / h_d| over x-space, the same over v-space, min of both */
double hdo_critical_time_step(const hdo_problem *p);

/* ---- Vlasov-Poisson (dim_x == dim_v, periodic x-mesh) ------------------- */

/* velocity-moment of f over v for every x-DoF (charge density without mean
 * removal): rho[x_dof] = sum over v-cells and v-nodes of f * JxW_v        */
int hdo_velocity_moment(const hdo_problem *p, const double *src, double *rho);

/* coordinate-moment of f over x for every v-DoF: out[v_dof] = sum over
 * x-cells and x-nodes of f * JxW_x at the Gauss-Lobatto points
 * (numerics/vector_tools.h:317-400, coordinate_space_integration) */
int hdo_coordinate_moment(const hdo_problem *p, const double *src, double *out);

/* SIPG Laplacian on the x-mesh (src mean removed first), its right-hand
 * side from rho, CG (phi: initial guess in, solution out), the potential
 * gradient at the x-quadrature points, one full Vlasov-Poisson operator
 * evaluation and the diagnostics (energy per x-direction, mass, L2 norm,
 * kinetic energy, momentum per v-direction).                             */
int hdo_poisson_apply(const hdo_problem *p, const double *src, double *dst);
int hdo_poisson_rhs(const hdo_problem *p, const double *rho, double *rhs);
int hdo_poisson_solve(const hdo_problem *p, const double *rhs, double *phi, double rel_tol, int max_it,
                      int *iterations);
int hdo_vp_field(const hdo_problem *p, const double *phi, double *E);
int hdo_vp_operator(const hdo_problem *p, const double *f, double *dst, double time, double *phi, double *E,
                    double cg_tol, int *iterations);
int hdo_vp_diagnostics(const hdo_problem *p, const double *f, const double *phi, double *out);

#ifdef __cplusplus
}
#endif
#endif
