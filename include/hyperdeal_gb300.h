/*
 * hyperdeal_gb300.h -- C ABI of the GB300 (sm_103a) phase-space advection
 * path: a drop-in for hyper.deal's element-centric (ECL) upwind-DG advection
 * operator at Gauss-Lobatto collocation and its low-storage Runge-Kutta
 * driver.
 *
 * Conventions
 *   - Every entry point returns an int status (HD_OK = 0).  No C++ exception
 *     crosses this boundary; hd_last_error() returns the message of the last
 *     failure on the calling thread.
 *   - Vectors are caller-owned DEVICE pointers holding n_dofs values of the
 *     handle's dtype (double for HD_F64, float for HD_F32), 16-byte aligned.
 *   - `stream` is a cudaStream_t passed as void* (NULL = legacy default
 *     stream).  All work of one call is enqueued on that stream; calls return
 *     without synchronising unless documented otherwise.
 *   - A handle is not thread-safe (as the reference operator, whose
 *     evaluators are members, is not re-entrant).  Calls on one handle from
 *     one thread may target different streams and overlap on the device (up
 *     to 64 launches of the pipelined kernel in flight at once: each launch
 *     takes its own row counter from a ring of 64).
 *
 * DoF numbering (identical to the reference's, 1 rank, NRefinements = 0):
 *   cell gid = gid_x + n_cells_x * gid_v, gid_x / gid_v lexicographic over
 *   the x- / v-cells (first direction fastest); each cell owns (k+1)^D
 *   contiguous values; inside a cell the node index is i_x + (k+1)^dim_x*i_v
 *   with lexicographic node order (first direction fastest).
 *   Reference: include/hyper.deal/matrix_free/matrix_free.templates.h:535-563
 *   (GlobaleCellIDTranslator::translate), :925-932 (sorted local cells),
 *   include/hyper.deal/matrix_free/vector_partitioner.h:723-724 (n^D values per
 *   cell), include/hyper.deal/matrix_free/shape_info.h:141-160 (x nodes
 *   fastest).
 */
#ifndef HYPERDEAL_GB300_H
#define HYPERDEAL_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HD_MAX_DIM 6

enum hd_status {
  HD_OK = 0,
  HD_ERR_INVALID = 1,     /* bad argument or descriptor                     */
  HD_ERR_UNSUPPORTED = 2, /* valid in the reference, not built here         */
  HD_ERR_CUDA = 3,        /* a CUDA runtime call failed                     */
  HD_ERR_ALLOC = 4,       /* host or device allocation failed               */
  HD_ERR_DEVICE = 5       /* a kernel reported an error through its flag    */
};

enum hd_dtype { HD_F64 = 0, HD_F32 = 1 };

enum hd_bc_kind {
  HD_BC_HOMOGENEOUS = 0, /* u+ = -u- on non-periodic faces                  */
  HD_BC_FUNCTION = 1     /* u+ = -u- + 2 g(x, t), g an hd_function          */
};

/* Analytic function family used for initial data, exact solutions and
 * Dirichlet data (the reference passes dealii::Function objects):
 *   kind 0: 0;  kind 1: amp;
 *   kind 2: amp * prod_d trig_d(omega_d * (x_d - speed_d * t) + phase_d),
 *           trig_d = cos if cosine[d] else sin;
 *   kind 3 (hd_vp_interpolate only): the perturbed Maxwellian
 *           (1 + amp prod_{cosine[d]==1} cos(omega_d x_d + phase_d))
 *             * prod_{cosine[d]==2} exp(-x_d^2 / 2) / sqrt(2 pi).          */
typedef struct hd_function {
  int kind;
  double amp;
  double omega[HD_MAX_DIM];
  double speed[HD_MAX_DIM];
  double phase[HD_MAX_DIM];
  int cosine[HD_MAX_DIM];
} hd_function;

/* Problem descriptor: what the reference sets up through MatrixFree::reinit,
 * AdvectionOperation::reinit, BoundaryDescriptor and ConstantVelocityFieldView
 * (include/hyper.deal/operators/advection/advection_operation.h:97-129,
 *  boundary_descriptor.h:77-104, velocity_field_view.h:64-166).           */
enum hd_quadrature {
  HD_QUAD_GAUSS_LOBATTO = 0, /* collocation: diagonal mass, no basis change   */
  HD_QUAD_GAUSS = 1          /* Gauss points: basis change and its inverse    */
};

typedef struct hd_adv_desc {
  int dim_x, dim_v;     /* 1..3 each                                       */
  int degree;           /* k; n_points must be k+1                         */
  int n_points;
  int dtype;            /* HD_F64 or HD_F32 (storage and arithmetic)       */
  int cells_x[3], cells_v[3];
  double lo_x[3], hi_x[3], lo_v[3], hi_v[3];
  int periodic_x, periodic_v;
  double velocity[HD_MAX_DIM]; /* constant a = (a_x, a_v)                  */
  double skew;          /* AdvectionOperationParamters::factor_skew        */
  int bc_kind;          /* enum hd_bc_kind, used on non-periodic faces     */
  hd_function bc;       /* g for HD_BC_FUNCTION                            */
  int quadrature;       /* enum hd_quadrature: Gauss-Lobatto collocation (0,
                           default) or Gauss (1); the reference's
                           quadrature 0 of MatrixFree (application.h:218-219) */
} hd_adv_desc;

typedef struct hd_adv hd_adv;
typedef struct hd_lsrk hd_lsrk;

/* Message of the last failure on this thread (empty if none); returns the
 * message length. */
int hd_last_error(char *buf, size_t len);

/* Library version string. */
const char *hd_version(void);

/* ---- operator ---------------------------------------------------------- */

/* Replaces AdvectionOperation(MatrixFree, table) + reinit(bc, velocity, param)
 * (advection_operation.h:85-129).  Selects the (dim, degree, dtype) kernel and
 * derives the per-direction line operators.  Uses the current CUDA device. */
int hd_adv_create(const hd_adv_desc *desc, hd_adv **out);
int hd_adv_destroy(hd_adv *op);

/* Number of DoFs = prod(cells) * (k+1)^(dim_x+dim_v). */
long long hd_adv_n_dofs(const hd_adv *op);

/* Tile of the generic kernel (the autotuner's knobs; no reference
 * counterpart -- the reference's cell batching is fixed by VectorizedArray):
 * cells per CTA (1..max, 0 = max) and CTAs per SM of the persistent grid
 * (0 = as many as fit).  Results do not depend on the tile. */
int hd_adv_set_tile(hd_adv *op, int cells_per_cta, int ctas_per_sm);
int hd_adv_tile_limits(const hd_adv *op, int *max_cells_per_cta, int *threads_per_cell);
/* time apply launches (src read, dst overwritten) for candidate tiles and
 * keep the fastest; returns it and its time per apply */
int hd_adv_autotune(hd_adv *op, const void *src, void *dst, int reps, int *cells_per_cta, int *ctas_per_sm,
                    double *ms, void *stream);

/* Kernel selection: AUTO picks the persistent TMA-pipelined kernel where it
 * applies (FP32, degree 3, fully periodic: 3x+3v meshes, and 2x+2v meshes
 * with 16 cells along x0 that are not parts) and the generic shared-memory
 * kernel otherwise; GENERIC forces the latter.  Both compute the same
 * operator.  hd_adv_kernel() returns the kernel that will run. */
enum hd_kernel { HD_KERNEL_AUTO = 0, HD_KERNEL_GENERIC = 1, HD_KERNEL_PIPELINED = 2 };
int hd_adv_set_kernel(hd_adv *op, int variant);
int hd_adv_kernel(const hd_adv *op);

/* Arithmetic of the FP64-storage form (no reference counterpart: the
 * reference computes in double).  NATIVE runs the contractions in FP64;
 * FP32X2 keeps FP64 storage, layout and stage update but runs the line
 * contractions in double-word FP32 arithmetic (hi + lo float pairs, about 48
 * significant bits) on the FP32 pipe, which GB300 issues at 64 times its FP64
 * rate.  FP32X2 needs dtype HD_F64 and Gauss-Lobatto collocation (generic
 * kernel); the default is NATIVE. */
enum hd_arithmetic { HD_ARITH_NATIVE = 0, HD_ARITH_FP32X2 = 1 };
int hd_adv_set_arithmetic(hd_adv *op, int arithmetic);
int hd_adv_arithmetic(const hd_adv *op);

/* Device-side error code since the last call (0 = none; 1/2 = a bounded wait
 * of the pipelined kernel on a copy / buffer slot timed out and the kernel
 * returned early; 4 = a bounds check failed and the access was skipped, in a
 * library built with -DHD_CHECK only).  Synchronises the device; clears the
 * flag. */
int hd_adv_device_status(hd_adv *op, int *status);

/* Test hook of the bounded waits (no reference counterpart): wait_limit sets
 * the try_wait rounds of every bounded wait of the pipelined kernel (0 = the
 * default, about seconds), and skip_issue >= 0 makes the producer warp that
 * claims the launch's first row of cells issue nothing for cell skip_issue of
 * that row (0 <= skip_issue < cells in x0), so that the compute warps' wait
 * for that slot runs out: the kernel records status 1 or 2, stops that CTA's
 * remaining work without stores, waits (bounded) for its own copies in flight
 * and returns.  skip_issue = -1 turns the hook off.  Nothing faults or hangs. */
int hd_adv_set_wait_test(hd_adv *op, unsigned wait_limit, int skip_issue);

/* dst = M^{-1} A(src) at `time` (boundary data time), i.e.
 * AdvectionOperation::apply<all>(dst, src, time) in its ECL branch
 * (advection_operation.h:134-209, :218-566).  dst is overwritten; dst and src
 * must not overlap. */
int hd_adv_apply(hd_adv *op, void *dst, const void *src, double time, void *stream);

/* dt_crit = min(1/max_x |a_d/h_d|, 1/max_v |a_d/h_d|)
 * (operators/advection/cfl.h:56-124, Cartesian mesh). */
double hd_adv_critical_time_step(const hd_adv *op);

/* ---- partitioned operator: v-slabs with one ghost-face exchange per stage --
 *
 * Replaces the reference's distributed MatrixFree with a v-only process grid
 * (size_x = 1) and its Contiguous ghost-face partitioner
 * (include/hyper.deal/matrix_free/vector_partitioner.h:670-1381 set-up,
 * :1385-1607 exchange) and the overlap of the exchange with the cells that do
 * not need it (matrix_free.templates.h:1178-1234, :1494-1581).
 *
 * The mesh is cut into n_parts slabs of whole layers of the last direction
 * (v_{dim_v-1}, the slowest in the cell numbering), so a part owns a
 * contiguous range of cell ids: part p owns layers [p L / P, (p+1) L / P)
 * (integer division; L = cells in that direction, P = n_parts <= L).  Only
 * faces across that direction cross parts, and only the upwind face is read
 * (the downwind neighbour's trace enters the reference's flux multiplied by
 * zero), so each part needs the faces of ONE layer of ONE neighbour part.
 *
 * A part's vectors hold its cells -- n_cells (k+1)^D values numbered as the
 * global vector restricted to the range -- followed by a ghost region of
 * ghost_values values: the upwind neighbour layer's face traces, (k+1)^(D-1)
 * values per cell (the nodes of the face slab in order), cells in their
 * in-layer order (the reference keeps ghost faces after the local cells as
 * well, vector_partitioner.h:916-993).  An exchange per stage: the sending
 * part packs the faces (hd_adv_pack_faces) and the host's transport (NCCL,
 * MPI, a peer copy) moves them into the receiving part's ghost region of the
 * same vector.  The layout is computed on the host alone: */
typedef struct hd_part_layout {
  long long first_cell;      /* global id of the part's first cell                 */
  long long n_cells;         /* cells of the part                                  */
  long long layer_cells;     /* cells per layer of the last direction              */
  long long face_values;     /* values per face, (k+1)^(D-1)                       */
  long long ghost_values;    /* values of the ghost region (0: no ghost faces)     */
  int recv_from;             /* part whose faces fill the ghost region (-1: none)  */
  int send_to;               /* part whose ghost region this part fills (-1: none) */
  long long send_first_cell; /* local id of the first cell of the sent layer       */
  int send_slab;             /* node index along the last direction of sent faces  */
  long long boundary_first;  /* local cells that read the ghost region: the       */
  long long boundary_cells;  /*   range [boundary_first, +boundary_cells)          */
} hd_part_layout;

/* Layout of part `part` of `n_parts` for the descriptor (no CUDA call). */
int hd_part_layout_get(const hd_adv_desc *desc, int n_parts, int part, hd_part_layout *out);

/* The operator of one part (Gauss-Lobatto collocation; any dimension split,
 * degree and dtype of hd_adv_create).  n_parts = 1 is hd_adv_create.  The
 * part's operator works on its vectors (hd_adv_n_dofs() values + ghost
 * region); hd_adv_apply reads the ghost region of src, which must hold the
 * neighbour's faces of src. */
int hd_adv_create_part(const hd_adv_desc *desc, int n_parts, int part, hd_adv **out);
int hd_adv_part_layout(const hd_adv *op, hd_part_layout *out);

/* Pack the faces of `vec` that part send_to reads into sendbuf
 * (ghost_values of the receiver = layer_cells * face_values values of the
 * handle's dtype, in the receiver's ghost-region order). */
int hd_adv_pack_faces(hd_adv *op, const void *vec, void *sendbuf, void *stream);

/* Cell subsets of a launch: the cells that read the ghost region (BOUNDARY,
 * one layer at one end of the part) and the others (INTERIOR), so that
 * INTERIOR runs while the ghost faces are in flight. */
enum hd_cells { HD_CELLS_ALL = 0, HD_CELLS_INTERIOR = 1, HD_CELLS_BOUNDARY = 2 };
int hd_adv_apply_cells(hd_adv *op, void *dst, const void *src, double time, int cells, void *stream);

/* ---- vector tools --------------------------------------------------------- */

/* dst = f(x_i, time) at the Gauss-Lobatto support points
 * (numerics/vector_tools.h:81-135, interpolate with quad_no = 2). */
int hd_interpolate(hd_adv *op, const hd_function *f, double time, void *dst, void *stream);

/* result[0] = ||src||_L2, result[1] = ||src - f(., time)||_L2 with the
 * operator's quadrature (Gauss-Lobatto under collocation)
 * (numerics/vector_tools.h:144-223).  Synchronises `stream`. */
int hd_norm_and_error(hd_adv *op, const hd_function *f, double time, const void *src,
                      double *result, void *stream);

/* The same result as hd_norm_and_error for callers that must not allocate
 * device memory (a host application that owns all device memory, a time loop
 * that forbids allocation after start-up).  No counterpart in the reference:
 * it takes the descriptor instead of a handle (hd_adv_create allocates) and
 * calls no cudaMalloc / cudaFree; its scratch is a fixed 256 KiB array in
 * device global memory inside the library, held by every GPU that loads the
 * library until exit.  Limits: at most 134,217,728 DoFs (larger meshes get
 * HD_ERR_INVALID; use hd_norm_and_error); Gauss-Lobatto collocation
 * descriptors only (HD_QUAD_GAUSS gets HD_ERR_UNSUPPORTED); function kinds
 * 0..2 (others get HD_ERR_INVALID).  All calls share the scratch, so
 * calls whose kernels overlap on the GPU race: serialise them.  The first call
 * on a device looks up the scratch address for that device (make it before
 * any stream capture).  Synchronises `stream`; result is host memory. */
int hd_norm_and_error_noalloc(const hd_adv_desc *desc, const hd_function *f, double time,
                              const void *src, double *result, void *stream);

/* ---- low-storage Runge-Kutta ------------------------------------------------ */

/* LowStorageRungeKuttaIntegrator(Ki, Ti, type, only_Ti_is_ghosted=true)
 * (base/time_integrators.h:57-77, time_integrators.templates.h:22-89);
 * type = "rk33", "rk45", "rk47" or "rk59". */
int hd_lsrk_create(const char *type, hd_lsrk **out);
int hd_lsrk_destroy(hd_lsrk *rk);
int hd_lsrk_n_stages(const hd_lsrk *rk);

/* One time step of perform_time_step(sol, t, dt, op) with op = the advection
 * operator (time_integrators.templates.h:91-184), fused: every stage is one
 * kernel that applies the operator and the stage update
 *   sol <- sol + b_s dt K,  T <- sol_old + a_s dt K
 * in a single pass.  Neighbours read the stage input while it is being
 * updated, so the three vectors rotate roles; on return the three pointers
 * are permuted so that *sol holds the new solution (the others are scratch).
 * The reference's own Ki/Ti vectors are scratch in the same way.  The values
 * equal the unfused step within round-off.  A part with a ghost region steps
 * with hd_lsrk_stage and an exchange between stages (HD_ERR_UNSUPPORTED). */
int hd_lsrk_step(hd_adv *op, const hd_lsrk *rk, void **sol, void **Ki, void **Ti,
                 double time, double dt, void *stream);

/* Stage `stage` of the same fused step on a subset of cells (enum hd_cells),
 * for drivers that exchange ghost faces between stages (partitioned
 * operators).  X[0..2] are the step's vectors sol, Ki, Ti in the roles they
 * had when the step began; stage s reads X[hd_lsrk_stage_input(rk, s)] (whose
 * ghost region must hold the neighbour's faces of that vector) and after the
 * last stage the new solution is X[1] (hd_lsrk_step's permutation: sol <- X1,
 * Ki <- X0, Ti <- X2).  hd_lsrk_step runs every stage on all cells. */
int hd_lsrk_stage(hd_adv *op, const hd_lsrk *rk, int stage, void *const *X, double time, double dt, int cells,
                  void *stream);
int hd_lsrk_stage_input(const hd_lsrk *rk, int stage);

/* The unfused reference form of the same step: op(Ti, Ki, t_s) followed by
 * the vector update, exactly in the reference's order
 * (time_integrators.templates.h:103-183).  sol, Ki, Ti keep their roles. */
int hd_lsrk_step_unfused(hd_adv *op, const hd_lsrk *rk, void *sol, void *Ki, void *Ti,
                         double time, double dt, void *stream);

/* The LSRK vector update of one stage for any operator (the loop of
 * time_integrators.templates.h:111-135): with factor_ai == 0 only
 * sol += factor_bi * K, else also next_T = sol_old + factor_ai * K. */
int hd_lsrk_stage_update(int dtype, long long n, double factor_bi, double factor_ai,
                         const void *K, void *sol, void *next_T, void *stream);

/* Stage count, coefficients (ai: n_stages-1 values, bi: n_stages) and the
 * stage times c_s (n_stages values, c_0 = 0). */
int hd_lsrk_coefficients(const hd_lsrk *rk, double *ai, double *bi, double *ci);

/* ---- batched uneven instances --------------------------------------------- */

/* Many independent advection problems (any dimension split, degree, velocity,
 * mesh, dtype) advanced together.  The reference runs such problems one
 * after the other (examples/advection/advection.cc:253-259), each with its
 * own compile-time (dim, degree) instantiation (:26-48).  Here instances are
 * grouped by class (dim_x + dim_v, degree, dtype); a class with a batch
 * kernel (dim_x + dim_v in {4, 5}, degree 2..5) runs as ONE persistent launch
 * per RK stage over all its instances, other classes launch per instance.
 * The scheme and the classes (dimension, degree, storage type and, for the
 * batched classes, the arithmetic set by hd_adv_set_arithmetic) are fixed at
 * creation; FP64 operators in FP32x2 arithmetic form their own classes.  The handle keeps pointers to the operators (they must outlive
 * it).  Results equal the per-instance hd_lsrk_step / hd_adv_apply. */
typedef struct hd_batch hd_batch;

int hd_batch_create(hd_adv *const *ops, int n_ops, const hd_lsrk *rk, hd_batch **out);
int hd_batch_destroy(hd_batch *b);
int hd_batch_n_classes(const hd_batch *b);
int hd_batch_class_info(const hd_batch *b, int cls, int *dim, int *degree, int *dtype, int *n_members, int *batched,
                        int *cells_per_cta, int *ctas_per_sm);
/* arithmetic of class cls (HD_ARITH_NATIVE / HD_ARITH_FP32X2), -1 on a bad class */
int hd_batch_class_arithmetic(const hd_batch *b, int cls);
/* tile of class cls (-1: all classes); 0 = default */
int hd_batch_set_tile(hd_batch *b, int cls, int cells_per_cta, int ctas_per_sm);
/* dst[i] = A_i src[i] at time[i] (time may be NULL: 0) */
int hd_batch_apply(hd_batch *b, void *const *dst, const void *const *src, const double *time, void *stream);
/* one fused LSRK step of every instance: arrays of n_ops vectors, permuted
 * per instance on return exactly like hd_lsrk_step's */
int hd_batch_lsrk_step(hd_batch *b, void **sol, void **Ki, void **Ti, const double *time, const double *dt,
                       void *stream);
/* record TWO steps of every instance (after which the three vectors of each
 * instance are back in their roles) as a CUDA graph; replays advance the
 * stage times on the device.  hd_batch_lsrk_step invalidates the graph. */
int hd_batch_graph_capture(hd_batch *b, void *const *sol, void *const *Ki, void *const *Ti, const double *time,
                           const double *dt);
int hd_batch_graph_launch(hd_batch *b, void *stream);
/* autotuner: per class, time apply launches (src read, dst overwritten) for
 * candidate tiles and keep the fastest */
int hd_batch_autotune(hd_batch *b, const void *const *src, void *const *dst, int reps, void *stream);

/* ---- Vlasov-Poisson ------------------------------------------------------- */

/* Electrostatic Vlasov-Poisson on periodic x- and v-meshes (dim_x == dim_v),
 * Gauss-Lobatto collocation or Gauss quadrature (hd_vp_desc::quadrature):
 * one right-hand-side evaluation computes the
 * charge density rho(x) = int f dv, solves the SIPG Poisson problem for the
 * potential by conjugate gradients in FP64, takes E = grad(phi) at the
 * x-nodes and applies the advection operator with the phase-space velocity
 * (v, grad phi) -- the reference's examples/vlasov_poisson/include/
 * application.h:516-602 (moments vector_tools.h:230-315, Poisson
 * poisson.h:52-610, field derivative_container.h:158-251, velocity
 * velocity_field_view.h:28-209).  f is stored in `dtype`; everything on the
 * x-mesh is FP64. */
enum hd_vp_guess {
  HD_VP_GUESS_ZERO = 0,     /* CG starts from 0                                 */
  HD_VP_GUESS_PREVIOUS = 1, /* from the previous potential (the reference's)    */
  HD_VP_GUESS_LEARNED = 2   /* from a network trained online on the solver's
                               own (right-hand side, potential) pairs; the fit
                               is chosen by hd_vp_desc::learn_fit            */
};

/* How the learned guess's network -- two linear layers, W1 (r x n) and
 * W2 (n x r), n = x-DoFs -- is fitted to the solver's pairs.
 * LEAST_SQUARES (default): FP64, the minimum-norm least-squares fit of the
 *   last pairs (rhs_j, phi_j), W2 W1 = [phi_j] [rhs_j]^+, computed by
 *   Gram-Schmidt orthogonalisation inside the Poisson launch: W1 = Q^T with Q
 *   an orthonormal basis of the rhs_j, W2 = Z the same combinations of the
 *   phi_j.  guess = W2 W1 rhs, used when its residual is below ||rhs||.
 *   learn_rank (0: 16, at most 16) basis columns; when they are used up the
 *   basis is rebuilt from the last learn_history pairs (0: 3/8 of the rank,
 *   less than the rank).
 * ADAM: FP32 weights trained by Adam on normalised differences between
 *   consecutive solves, guess = phi_prev + W2 W1 (rho - rho_prev), weighed
 *   against phi_prev (learn_rank 0: 32, learn_history 0: 64 pairs); its
 *   loss and gradients are exposed by hd_vp_learn_loss_grad. */
enum hd_vp_learn_fit { HD_VP_FIT_LEAST_SQUARES = 0, HD_VP_FIT_ADAM = 1 };

/* Preconditioner of the Poisson CG.  The reference preconditions its CG
 * with geometric multigrid and a Chebyshev smoother (examples/vlasov_poisson/
 * include/poisson.h:612-742); here the x-cells' diagonal blocks of the SIPG
 * matrix are inverted once (cell-block Jacobi), which damps the high-frequency
 * error that FP32 round-off in the density carries into the right-hand side. */
enum hd_vp_precond { HD_VP_PRECOND_NONE = 0, HD_VP_PRECOND_BLOCK_JACOBI = 1 };

/* Solver of the x-space Poisson problem.  CG (the reference's solver, with
 * the initial guess and preconditioner above) or, for x-spaces of up to 8192
 * DoFs, DIRECT: the fixed SIPG matrix's pseudo-inverse (on the mean-free
 * right-hand sides the problem has) is computed once at creation, on the
 * device by Gauss-Jordan elimination of A + beta 1 1^T, and kept in HBM
 * (8 n^2 bytes: 134 MB for 16^2 x-cells of degree 3); every solve is then one
 * dense matrix-vector product.  The guess and preconditioner fields are
 * ignored, and the CG statistics count solves with zero iterations. */
enum hd_vp_solver { HD_VP_SOLVER_CG = 0, HD_VP_SOLVER_DIRECT = 1 };

typedef struct hd_vp_desc {
  int dim_x, dim_v, degree, dtype;
  int cells_x[3], cells_v[3];
  double lo_x[3], hi_x[3], lo_v[3], hi_v[3];
  double cg_tol;        /* CG stops at ||r|| <= cg_tol ||r_0|| (deal.II
                           ReductionControl(reduce = cg_tol), poisson.h:596),
                           or at ||r|| <= cg_tol ||rhs|| with cg_rhs_relative */
  int cg_max_iter;
  int guess;            /* enum hd_vp_guess                                   */
  int learn_rank;       /* bottleneck r of the learned guess (0: the fit's default) */
  int learn_history;    /* pairs kept for the fit (0: the fit's default)      */
  int cg_rhs_relative;  /* 1: tolerance relative to ||rhs|| -- a fixed
                           accuracy, so a better initial guess saves
                           iterations                                         */
  int learn_every;      /* ADAM fit: the learned guess stores every solve's
                           pair and takes its Adam steps every learn_every-th
                           solve (0: 1, every solve)                          */
  int cg_precond;       /* enum hd_vp_precond (0: none)                       */
  int learn_fit;        /* enum hd_vp_learn_fit (0: least squares)            */
  int quadrature;       /* enum hd_quadrature: Gauss-Lobatto collocation (0)
                           or Gauss points (n_points = degree + 1; DoFs stay
                           Gauss-Lobatto nodal values; rho, E and every
                           integral at the Gauss points as the reference's
                           non-collocation runs; up to 3x+3v degree 3 in
                           FP64; FP32x2 arithmetic refused)                  */
  int poisson_solver;   /* enum hd_vp_solver (0: CG)                          */
} hd_vp_desc;

typedef struct hd_vp hd_vp;

int hd_vp_create(const hd_vp_desc *desc, hd_vp **out);
int hd_vp_destroy(hd_vp *vp);
long long hd_vp_n_dofs(const hd_vp *vp);
long long hd_vp_n_dofs_x(const hd_vp *vp);
/* f at the nodes of an analytic function (kind 3: perturbed Maxwellian) */
int hd_vp_interpolate(hd_vp *vp, const hd_function *f, double time, void *dst, void *stream);
/* steps 1-4 (rho, Poisson, field) for the distribution f; synchronises */
int hd_vp_solve_field(hd_vp *vp, const void *f, void *stream);
/* dst = the Vlasov-Poisson right-hand side of src (steps 1-5) */
int hd_vp_apply(hd_vp *vp, void *dst, const void *src, double time, void *stream);
/* one LSRK step with hd_vp_apply as the operator
 * (time_integrators.templates.h:91-184, unfused) */
int hd_vp_lsrk_step(hd_vp *vp, const hd_lsrk *rk, void *sol, void *Ki, void *Ti, double time, double dt,
                    void *stream);
/* the same step with the stage update fused into the advection kernel; the
 * three vectors rotate roles as in hd_lsrk_step (the new solution is in
 * *sol on return) */
int hd_vp_lsrk_step_fused(hd_vp *vp, const hd_lsrk *rk, void **sol, void **Ki, void **Ti, double time, double dt,
                          void *stream);
/* out: field energy int (d_d phi)^2 per x-direction, mass, L2 norm, kinetic
 * energy int |v|^2 f, momentum int v_d f per v-direction (diagnostics.h:28-141);
 * the field is the one of the last right-hand-side evaluation */
int hd_vp_diagnostics(hd_vp *vp, const void *f, double *out, void *stream);
/* copies of rho, phi (x-DoFs) and E (x-DoFs * dim_x) into device buffers (NULL: skip) */
int hd_vp_fields(hd_vp *vp, double *rho, double *phi, double *E, void *stream);
int hd_vp_cg_stats(const hd_vp *vp, int *last_iterations, long long *total_iterations, long long *solves,
                   double *last_residual, long long *learned_picked);
int hd_vp_set_guess(hd_vp *vp, int guess);
/* arithmetic of the FP64-storage phase-space advection (hd_adv_set_arithmetic):
 * HD_ARITH_NATIVE (default) or HD_ARITH_FP32X2 (dim_x = dim_v <= 2); the
 * moments, the Poisson solve, the field and the stage update stay FP64 */
int hd_vp_set_arithmetic(hd_vp *vp, int arithmetic);
/* FP32 advection kernel: AUTO (default) runs the TMA-pipelined kernel where it
 * applies -- FP32, 2x+2v, degree 3, collocation, 16 cells along x0: one x0-row
 * of 16 cells per unit, both neighbours' traces staged by TMA, every line's
 * upwind side from its velocity's sign -- and the generic kernel otherwise;
 * GENERIC forces the latter (enum hd_kernel; PIPELINED where it does not
 * apply is HD_ERR_UNSUPPORTED).  hd_vp_kernel returns the kernel that runs. */
int hd_vp_set_kernel(hd_vp *vp, int variant);
int hd_vp_kernel(const hd_vp *vp);
/* device status of the pipelined advection since the last call (0 = none;
 * 1/2 = a bounded wait timed out and the launch stopped early); synchronises
 * and resets it */
int hd_vp_device_status(hd_vp *vp, int *status);
/* test hook of the pipelined advection's bounded waits (as hd_adv_set_wait_test):
 * wait_limit try_wait rounds (0: the default); skip_issue 0 = the producer
 * holding unit 0 issues nothing for it, -1 = off */
int hd_vp_set_wait_test(hd_vp *vp, unsigned wait_limit, int skip_issue);
/* loss = 1/(2B) sum_b ||W2 W1 x_b - y_b||^2 and its gradients with the learned
 * guess's own training kernels (device pointers, row-major W1: r x n,
 * W2: n x r, X, Y: B x n) -- exposed to check them against a CPU reference */
int hd_vp_learn_loss_grad(long long n, int rank, int batch, const float *W1, const float *W2, const float *X,
                          const float *Y, float *dW1, float *dW2, float *loss, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* HYPERDEAL_GB300_H */
