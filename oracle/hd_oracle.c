/*
 * hd_oracle.c -- CPU restatement of hyper.deal's phase-space upwind-DG
 * advection path.  TEST INFRASTRUCTURE: the checker for the CUDA path and
 * the timed CPU baseline; never part of the product library.
 *
 * See hd_oracle.h for the list of reference functions restated here.  Each
 * function below names the reference lines it follows.  The code is a plain
 * restatement of the reference's arithmetic (JxW, inverse Jacobian, upwind
 * flux with alpha = 1, inverse mass), written for clarity first; OpenMP
 * threads over cells take the place of the reference's MPI ranks.
 */
#include "hd_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define MAXN HDO_MAX_POINTS

/* ------------------------------------------------------------------------ */
/* 1D rules (deal.II QGaussLobatto / QGauss, restated from the Legendre     */
/* recurrence; the reference uses them at                                    */
/* examples/advection/include/application.h:217-223)                          */
/* ------------------------------------------------------------------------ */

/* P_n(x) and P_n'(x) by the three-term recurrence */
static void legendre(int n, double x, double *p, double *dp) {
  double p0 = 1.0, p1 = x;
  if (n == 0) { *p = 1.0; *dp = 0.0; return; }
  for (int k = 2; k <= n; ++k) {
    double pk = ((2.0 * k - 1.0) * x * p1 - (k - 1.0) * p0) / k;
    p0 = p1;
    p1 = pk;
  }
  *p = p1;
  *dp = (fabs(x) < 1.0) ? n * (p0 - x * p1) / (1.0 - x * x)
                        : 0.5 * n * (n + 1.0) * (x > 0 ? 1.0 : (n % 2 ? 1.0 : -1.0));
}

int hdo_gauss(int n, double *x, double *w) {
  if (n < 1 || n > MAXN) return -1;
  for (int i = 0; i < n; ++i) {
    /* Chebyshev-like initial guess, then Newton on P_n */
    double z = cos(M_PI * (i + 0.75) / (n + 0.5));
    for (int it = 0; it < 100; ++it) {
      double p, dp;
      legendre(n, z, &p, &dp);
      double dz = p / dp;
      z -= dz;
      if (fabs(dz) < 1e-17) break;
    }
    double p, dp;
    legendre(n, z, &p, &dp);
    /* ascending order on [0,1] */
    x[n - 1 - i] = 0.5 * (1.0 + z);
    w[n - 1 - i] = 0.5 * 2.0 / ((1.0 - z * z) * dp * dp);
  }
  return 0;
}

int hdo_gauss_lobatto(int n, double *x, double *w) {
  if (n < 2 || n > MAXN) return -1;
  const int m = n - 1; /* interior nodes are the roots of P_m' */
  x[0] = 0.0;
  x[n - 1] = 1.0;
  for (int i = 1; i < m; ++i) {
    double z = -cos(M_PI * i / m); /* Chebyshev-Gauss-Lobatto guess */
    for (int it = 0; it < 100; ++it) {
      /* Newton on q(z) = P_m'(z); q'(z) = (2 z P_m' - m (m+1) P_m) / (1 - z^2) */
      double p, dp;
      legendre(m, z, &p, &dp);
      double ddp = (2.0 * z * dp - m * (m + 1.0) * p) / (1.0 - z * z);
      double dz = dp / ddp;
      z -= dz;
      if (fabs(dz) < 1e-17) break;
    }
    x[i] = 0.5 * (1.0 + z);
  }
  for (int i = 0; i < n; ++i) {
    double z = 2.0 * x[i] - 1.0, p, dp;
    legendre(m, z, &p, &dp);
    w[i] = 0.5 * 2.0 / (m * (m + 1.0) * p * p);
  }
  /* symmetrise to remove round-off asymmetry */
  for (int i = 0; i < n / 2; ++i) {
    double xs = 0.5 * (x[i] + (1.0 - x[n - 1 - i]));
    double ws = 0.5 * (w[i] + w[n - 1 - i]);
    x[i] = xs; x[n - 1 - i] = 1.0 - xs;
    w[i] = ws; w[n - 1 - i] = ws;
  }
  if (n % 2) x[n / 2] = 0.5;
  return 0;
}

/* Lagrange basis on nodes p[0..n-1] evaluated at y: out[j] = l_j(y) */
static void lagrange_values(int n, const double *p, double y, double *out) {
  for (int j = 0; j < n; ++j) {
    double v = 1.0;
    for (int m = 0; m < n; ++m)
      if (m != j) v *= (y - p[m]) / (p[j] - p[m]);
    out[j] = v;
  }
}

/* derivative of the Lagrange basis at y: out[j] = l_j'(y) */
static void lagrange_derivs(int n, const double *p, double y, double *out) {
  for (int j = 0; j < n; ++j) {
    double s = 0.0;
    for (int l = 0; l < n; ++l) {
      if (l == j) continue;
      double t = 1.0 / (p[j] - p[l]);
      for (int m = 0; m < n; ++m)
        if (m != j && m != l) t *= (y - p[m]) / (p[j] - p[m]);
      s += t;
    }
    out[j] = s;
  }
}

/* invert a small dense matrix (Gauss-Jordan with partial pivoting) */
static int invert(int n, const double *a, double *inv) {
  double m[MAXN][2 * MAXN];
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < 2 * n; ++j)
      m[i][j] = j < n ? a[i * n + j] : (j - n == i ? 1.0 : 0.0);
  for (int c = 0; c < n; ++c) {
    int piv = c;
    for (int r = c + 1; r < n; ++r)
      if (fabs(m[r][c]) > fabs(m[piv][c])) piv = r;
    if (m[piv][c] == 0.0) return -1;
    if (piv != c)
      for (int j = 0; j < 2 * n; ++j) { double t = m[c][j]; m[c][j] = m[piv][j]; m[piv][j] = t; }
    double d = m[c][c];
    for (int j = 0; j < 2 * n; ++j) m[c][j] /= d;
    for (int r = 0; r < n; ++r) {
      if (r == c) continue;
      double f = m[r][c];
      for (int j = 0; j < 2 * n; ++j) m[r][j] -= f * m[c][j];
    }
  }
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) inv[i * n + j] = m[i][n + j];
  return 0;
}

/* ------------------------------------------------------------------------ */
/* problem context                                                           */
/* ------------------------------------------------------------------------ */
typedef struct {
  int D, dx, dv, n, NC;
  long long ncx, ncv, ncells;
  int cells[HDO_MAX_DIM];
  long long cstride[HDO_MAX_DIM]; /* cell-index stride per direction  */
  int nstride[HDO_MAX_DIM];       /* node-index stride per direction  */
  double h[HDO_MAX_DIM];
  double gl[MAXN], glw[MAXN];     /* Gauss-Lobatto support points     */
  double pts[MAXN], w[MAXN];      /* quadrature 0 points / weights    */
  double Dq[MAXN * MAXN];         /* Dq[q*n+j] = psi_j'(pts_q)        */
  double S[MAXN * MAXN];          /* S[q*n+j] = l^GL_j(pts_q)         */
  double Sinv[MAXN * MAXN];
  double fval[2][MAXN];           /* psi_j(0), psi_j(1)               */
} ctx_t;

static int make_ctx(const hdo_problem *p, ctx_t *c) {
  memset(c, 0, sizeof(*c));
  if (p->dim_x < 1 || p->dim_x > 3 || p->dim_v < 1 || p->dim_v > 3) return -1;
  if (p->degree < 1 || p->degree + 1 > MAXN) return -1;
  if (p->n_points != p->degree + 1) return -1; /* only n_points = degree+1 */
  c->dx = p->dim_x; c->dv = p->dim_v; c->D = c->dx + c->dv; c->n = p->degree + 1;
  c->NC = 1;
  for (int d = 0; d < c->D; ++d) {
    if (p->cells[d] < 1) return -1;
    c->nstride[d] = c->NC;
    c->NC *= c->n;
    c->cells[d] = p->cells[d];
    c->h[d] = (p->hi[d] - p->lo[d]) / p->cells[d];
  }
  /* cell gid = gid_x + ncx * gid_v, each lexicographic
     (reference: matrix_free.templates.h:552-562) */
  c->ncx = 1; c->ncv = 1;
  for (int d = 0; d < c->dx; ++d) { c->cstride[d] = c->ncx; c->ncx *= c->cells[d]; }
  for (int d = c->dx; d < c->D; ++d) { c->cstride[d] = c->ncx * c->ncv; c->ncv *= c->cells[d]; }
  c->ncells = c->ncx * c->ncv;
  const int n = c->n;
  hdo_gauss_lobatto(n, c->gl, c->glw);
  if (p->collocation) {
    memcpy(c->pts, c->gl, sizeof(c->gl));
    memcpy(c->w, c->glw, sizeof(c->glw));
  } else {
    hdo_gauss(n, c->pts, c->w);
  }
  for (int q = 0; q < n; ++q) {
    double row[MAXN];
    lagrange_derivs(n, c->pts, c->pts[q], row);
    for (int j = 0; j < n; ++j) c->Dq[q * n + j] = row[j];
    lagrange_values(n, c->gl, c->pts[q], row);
    for (int j = 0; j < n; ++j) c->S[q * n + j] = p->collocation ? (q == j) : row[j];
  }
  if (invert(n, c->S, c->Sinv)) return -1;
  lagrange_values(n, c->pts, 0.0, c->fval[0]);
  lagrange_values(n, c->pts, 1.0, c->fval[1]);
  if (p->collocation)
    for (int j = 0; j < n; ++j) { c->fval[0][j] = (j == 0); c->fval[1][j] = (j == n - 1); }
  return 0;
}

long long hdo_n_dofs(const hdo_problem *p) {
  ctx_t c;
  if (make_ctx(p, &c)) return -1;
  return c.ncells * c.NC;
}

/* cell coordinates from gid */
static void cell_coords(const ctx_t *c, long long gid, int *cc) {
  long long gx = gid % c->ncx, gv = gid / c->ncx;
  for (int d = 0; d < c->dx; ++d) { cc[d] = (int)(gx % c->cells[d]); gx /= c->cells[d]; }
  for (int d = c->dx; d < c->D; ++d) { cc[d] = (int)(gv % c->cells[d]); gv /= c->cells[d]; }
}

static long long cell_gid(const ctx_t *c, const int *cc) {
  long long g = 0;
  for (int d = 0; d < c->D; ++d) g += cc[d] * c->cstride[d];
  return g;
}

/* out (+)= A along direction d (A[o*n+i], out_o = sum_i A[o][i] in_i);
   transpose: out_i = sum_o A[o][i] in_o */
static void apply_1d(const ctx_t *c, const double *A, int transpose, int d,
                     const double *in, double *out, int add) {
  const int n = c->n, s = c->nstride[d], NC = c->NC;
  for (int base = 0; base < NC; ++base) {
    if ((base / s) % n != 0) continue; /* first node of each line */
    double tin[MAXN], tout[MAXN];
    for (int i = 0; i < n; ++i) tin[i] = in[base + i * s];
    for (int o = 0; o < n; ++o) {
      double acc = 0.0;
      for (int i = 0; i < n; ++i)
        acc += (transpose ? A[i * n + o] : A[o * n + i]) * tin[i];
      tout[o] = acc;
    }
    for (int o = 0; o < n; ++o) out[base + o * s] = add ? out[base + o * s] + tout[o] : tout[o];
  }
}

static double func_value(const hdo_func *f, int D, const double *x, double t) {
  if (f->kind == 0) return 0.0;
  if (f->kind == 1) return f->amp;
  if (f->kind == 3) {
    /* (1 + amp prod_{cosine[d]==1} cos(omega_d x_d + phase_d)) prod_{cosine[d]==2} exp(-x_d^2/2)/sqrt(2 pi)
       (examples/vlasov_poisson/cases/hyperrectangle.h:45-58) */
    double pert = f->amp, r = 1.0;
    for (int d = 0; d < D; ++d)
      if (f->cosine[d] == 1) pert *= cos(f->omega[d] * x[d] + f->phase[d]);
    r += pert;
    for (int d = 0; d < D; ++d)
      if (f->cosine[d] == 2) r = r * exp(-0.5 * x[d] * x[d]) / sqrt(2.0 * M_PI);
    return r;
  }
  double r = f->amp;
  for (int d = 0; d < D; ++d) {
    double arg = f->omega[d] * (x[d] - f->speed[d] * t) + f->phase[d];
    r *= f->cosine[d] ? cos(arg) : sin(arg);
  }
  return r;
}

/* JxW of the cell at quadrature node q (multi-index via strides) */
static double cell_jxw(const ctx_t *c, int q) {
  double j = 1.0;
  for (int d = 0; d < c->D; ++d) j *= c->h[d] * c->w[(q / c->nstride[d]) % c->n];
  return j;
}

/* ------------------------------------------------------------------------ */
/* ECL cell operator                                                         */
/* reference: advection_operation.h:218-566                                  */
/* ------------------------------------------------------------------------ */
/* source vector: double, or float widened to double on read */
typedef struct {
  const double *d;
  const float *f;
} src_t;

static void read_cell(src_t src, long long gid, int NC, double *out) {
  if (src.d) {
    memcpy(out, src.d + gid * NC, sizeof(double) * NC);
  } else {
    const float *u = src.f + gid * NC;
    for (int i = 0; i < NC; ++i) out[i] = (double)u[i];
  }
}

/* velocity component d at the cell's quadrature point with multi-index
   (via node strides) q: constant (p->velocity) or the Vlasov-Poisson
   phase-space field, x-velocity = v-coordinate of the point, v-velocity =
   efield at the point's x-quadrature index (velocity_field_view.h:103-209 of
   the reference's vlasov_poisson example).  For face points the digit of
   the face-normal direction is ignored (the field does not depend on it). */
static double velocity_at(const hdo_problem *p, const ctx_t *c, const int *cc, int d, int q) {
  if (!p->efield) return p->velocity[d];
  const int dx = c->dx, n = c->n;
  if (d < dx) {
    const int dv = dx + d; /* the v-direction paired with x-direction d */
    return p->lo[dv] + (cc[dv] + c->pts[(q / c->nstride[dv]) % n]) * c->h[dv];
  }
  long long gx = 0;
  int qx = 0, sx = 1;
  for (int e = 0; e < dx; ++e) {
    gx += cc[e] * c->cstride[e];
    qx += ((q / c->nstride[e]) % n) * sx;
    sx *= n;
  }
  return p->efield[(gx * sx + qx) * dx + (d - dx)];
}

/* operator values of cell gid written to out[0 .. NC) */
static void apply_cell(const hdo_problem *p, const ctx_t *c, src_t src,
                       double *out, double time, long long gid, double *work) {
  const int D = c->D, n = c->n, NC = c->NC;
  double *v = work, *r = work + NC, *tmp = work + 2 * NC, *tmp2 = work + 3 * NC;
  double *nbuf = work + 4 * NC; /* neighbour cell (NC values) */
  const double s = p->skew;
  int cc[HDO_MAX_DIM];
  cell_coords(c, gid, cc);

  /* read_dof_values; values at quadrature points (basis change for Gauss,
     advection_operation.h:291-317) */
  read_cell(src, gid, NC, v);
  if (!p->collocation)
    for (int d = 0; d < D; ++d) { apply_1d(c, c->S, 0, d, v, tmp, 0); memcpy(v, tmp, sizeof(double) * NC); }

  /* volume terms: grad_in[d] = (1-s) u_q a_d, submit_gradient (J^{-T} JxW),
     integrate with the point-collocation gradient (advection_operation.h:325-404) */
  memset(r, 0, sizeof(double) * NC);
  for (int d = 0; d < D; ++d) {
    if (s != 1.0) {
      for (int q = 0; q < NC; ++q)
        tmp[q] = ((1.0 - s) * v[q] * velocity_at(p, c, cc, d, q)) * (1.0 / c->h[d]) * cell_jxw(c, q);
      apply_1d(c, c->Dq, 1, d, tmp, r, 1);
    }
    if (s != 0.0) {
      /* -s (a . grad u) JxW as a value term (submit_value) */
      apply_1d(c, c->Dq, 0, d, v, tmp2, 0);
      for (int q = 0; q < NC; ++q)
        r[q] += -s * (tmp2[q] * (1.0 / c->h[d]) * velocity_at(p, c, cc, d, q)) * cell_jxw(c, q);
    }
  }

  /* faces (advection_operation.h:406-526) */
  const int NF = NC / n;
  double *um = work + 5 * NC, *up = um + NF, *val = up + NF;
  int *fb = (int *)(val + NF);
  for (int f = 0; f < 2 * D; ++f) {
    const int d = f / 2, side = f % 2, sd = c->nstride[d];
    /* face point l <-> cell node base(l) with i_d = 0 (iterating the other dims) */
    {
      int l = 0;
      for (int i = 0; i < NC; ++i)
        if ((i / sd) % n == 0) fb[l++] = i;
    }
    /* u^- at face points: interpolate along d (quadrature_data_on_face) */
    for (int l = 0; l < NF; ++l) {
      double a = 0.0;
      for (int j = 0; j < n; ++j) a += c->fval[side][j] * v[fb[l] + j * sd];
      um[l] = a;
    }
    /* neighbour */
    int nc[HDO_MAX_DIM];
    memcpy(nc, cc, sizeof(nc));
    nc[d] += side ? 1 : -1;
    int interior = 1;
    if (nc[d] < 0 || nc[d] >= c->cells[d]) {
      const int periodic = d < c->dx ? p->periodic_x : p->periodic_v;
      if (periodic) nc[d] = (nc[d] + c->cells[d]) % c->cells[d];
      else interior = 0;
    }
    if (interior) {
      /* exterior trace: neighbour's nodes on the shared face
         (face_to_cell_index_nodal of the exterior face, shape_info.h:63-160) */
      read_cell(src, cell_gid(c, nc), NC, nbuf);
      const double *un = nbuf;
      const int inode = side ? 0 : n - 1;
      for (int l = 0; l < NF; ++l) up[l] = un[fb[l] + inode * sd];
      if (!p->collocation) {
        /* basis change on the face (eval_face.values, :436-446): apply S along
           every direction except d, on the face-restricted tensor */
        for (int l = 0; l < NF; ++l) tmp[fb[l]] = up[l];
        for (int e = 0; e < D; ++e) {
          if (e == d) continue;
          const int se = c->nstride[e];
          for (int l = 0; l < NF; ++l) {
            int b = fb[l];
            if ((b / se) % n != 0) continue;
            double tin[MAXN];
            for (int i = 0; i < n; ++i) tin[i] = tmp[b + i * se];
            for (int o = 0; o < n; ++o) {
              double acc = 0.0;
              for (int i = 0; i < n; ++i) acc += c->S[o * n + i] * tin[i];
              tmp[b + o * se] = acc;
            }
          }
        }
        for (int l = 0; l < NF; ++l) up[l] = tmp[fb[l]];
      }
    } else {
      for (int l = 0; l < NF; ++l) {
        if (!p->bc_inhomogeneous) {
          up[l] = -um[l];
        } else {
          double x[HDO_MAX_DIM];
          for (int e = 0; e < D; ++e) {
            if (e == d) x[e] = p->lo[e] + (cc[e] + side) * c->h[e];
            else x[e] = p->lo[e] + (cc[e] + c->pts[(fb[l] / c->nstride[e]) % n]) * c->h[e];
          }
          up[l] = -um[l] + 2.0 * func_value(&p->bc_func, D, x, time);
        }
      }
    }
    for (int l = 0; l < NF; ++l) {
      const double an = velocity_at(p, c, cc, d, fb[l]) * (side ? 1.0 : -1.0);
      double jxw = 1.0;
      for (int e = 0; e < D; ++e)
        if (e != d) jxw *= c->h[e] * c->w[(fb[l] / c->nstride[e]) % n];
      const double flux = 0.5 * ((um[l] + up[l]) * an + fabs(an) * (um[l] - up[l])) * 1.0;
      val[l] = -(flux - s * um[l] * an) * jxw;
    }
    /* distribute back along d */
    for (int l = 0; l < NF; ++l)
      for (int j = 0; j < n; ++j) r[fb[l] + j * sd] += c->fval[side][j] * val[l];
  }

  /* inverse mass (advection_operation.h:528-560; fe_evaluation_cell_inverse.h:131-133) */
  for (int q = 0; q < NC; ++q) r[q] /= cell_jxw(c, q);
  if (!p->collocation)
    for (int d = D - 1; d >= 0; --d) { apply_1d(c, c->Sinv, 0, d, r, tmp, 0); memcpy(r, tmp, sizeof(double) * NC); }

  memcpy(out, r, sizeof(double) * NC);
}

static int hdo_threads(const hdo_problem *p) {
#ifdef _OPENMP
  return p->n_threads > 0 ? p->n_threads : omp_get_max_threads();
#else
  (void)p;
  return 1;
#endif
}

int hdo_apply(const hdo_problem *p, const double *src, double *dst, double time) {
  ctx_t c;
  if (make_ctx(p, &c)) return -1;
  if (c.NC > MAXN * MAXN * MAXN * MAXN * MAXN * MAXN) return -1;
  int err = 0;
#pragma omp parallel num_threads(hdo_threads(p))
  {
    double *work = (double *)malloc(sizeof(double) * 8 * c.NC);
    if (!work) {
#pragma omp atomic write
      err = 1;
    } else {
#pragma omp for schedule(static)
      for (long long g = 0; g < c.ncells; ++g) {
        src_t sv = {src, NULL};
        apply_cell(p, &c, sv, dst + g * c.NC, time, g, work);
      }
      free(work);
    }
  }
  return err ? -1 : 0;
}

static int apply_cells_impl(const hdo_problem *p, src_t src, double *dst, double time,
                            const long long *cells, long long n_cells, int compact) {
  ctx_t c;
  if (make_ctx(p, &c)) return -1;
  int err = 0;
#pragma omp parallel num_threads(hdo_threads(p))
  {
    double *work = (double *)malloc(sizeof(double) * 8 * c.NC);
    if (!work) {
#pragma omp atomic write
      err = 1;
    } else {
#pragma omp for schedule(static)
      for (long long i = 0; i < n_cells; ++i) {
        if (cells[i] < 0 || cells[i] >= c.ncells) {
#pragma omp atomic write
          err = 1;
          continue;
        }
        /* compact: the result of cells[i] goes to dst[i*NC ...], else to its own place */
        apply_cell(p, &c, src, dst + (compact ? i : cells[i]) * c.NC, time, cells[i], work);
      }
      free(work);
    }
  }
  return err ? -1 : 0;
}

int hdo_apply_cells(const hdo_problem *p, const double *src, double *dst, double time,
                    const long long *cells, long long n_cells) {
  src_t sv = {src, NULL};
  return apply_cells_impl(p, sv, dst, time, cells, n_cells, 1);
}

int hdo_apply_cells_f32(const hdo_problem *p, const float *src, double *dst, double time,
                        const long long *cells, long long n_cells) {
  src_t sv = {NULL, src};
  return apply_cells_impl(p, sv, dst, time, cells, n_cells, 1);
}

/* ------------------------------------------------------------------------ */
/* low-storage Runge-Kutta (time_integrators.templates.h:22-184)             */
/* ------------------------------------------------------------------------ */
int hdo_lsrk_coefficients(const char *type, double *ai, double *bi) {
  /* Kennedy, Carpenter, Lewis (2000) 2N-storage coefficients as tabulated in
     time_integrators.templates.h:33-89 */
  if (!strcmp(type, "rk33")) {
    const double b[] = {0.245170287303492, 0.184896052186740, 0.569933660509768};
    const double a[] = {0.755726351946097, 0.386954477304099};
    memcpy(bi, b, sizeof(b)); memcpy(ai, a, sizeof(a));
    return 3;
  }
  if (!strcmp(type, "rk45")) {
    const double b[] = {1153189308089. / 22510343858157., 1772645290293. / 4653164025191.,
                        -1672844663538. / 4480602732383., 2114624349019. / 3568978502595.,
                        5198255086312. / 14908931495163.};
    const double a[] = {970286171893. / 4311952581923., 6584761158862. / 12103376702013.,
                        2251764453980. / 15575788980749., 26877169314380. / 34165994151039.};
    memcpy(bi, b, sizeof(b)); memcpy(ai, a, sizeof(a));
    return 5;
  }
  if (!strcmp(type, "rk47")) {
    const double b[] = {0.0941840925477795334, 0.149683694803496998, 0.285204742060440058,
                        -0.122201846148053668, 0.0605151571191401122, 0.345986987898399296,
                        0.186627171718797670};
    const double a0[] = {0.241566650129646868, 0.0423866513027719953, 0.215602732678803776,
                         0.232328007537583987, 0.256223412574146438, 0.0978694102142697230};
    memcpy(bi, b, sizeof(b));
    for (int i = 0; i < 6; ++i) ai[i] = a0[i] + b[i];
    return 7;
  }
  if (!strcmp(type, "rk59")) {
    const double b[] = {2274579626619. / 23610510767302., 693987741272. / 12394497460941.,
                        -347131529483. / 15096185902911., 1144057200723. / 32081666971178.,
                        1562491064753. / 11797114684756., 13113619727965. / 44346030145118.,
                        393957816125. / 7825732611452., 720647959663. / 6565743875477.,
                        3559252274877. / 14424734981077.};
    const double a[] = {1107026461565. / 5417078080134., 38141181049399. / 41724347789894.,
                        493273079041. / 11940823631197., 1851571280403. / 6147804934346.,
                        11782306865191. / 62590030070788., 9452544825720. / 13648368537481.,
                        4435885630781. / 26285702406235., 2357909744247. / 11371140753790.};
    memcpy(bi, b, sizeof(b)); memcpy(ai, a, sizeof(a));
    return 9;
  }
  return 0;
}

/* stage update, time_integrators.templates.h:111-135 */
static void stage_update(long long n, double bi, double ai, const double *K,
                         double *sol, double *next_T) {
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < n; ++i) {
    const double k = K[i], s0 = sol[i];
    sol[i] = s0 + bi * k;
    if (ai != 0.0) next_T[i] = s0 + ai * k;
  }
}

int hdo_lsrk_step_op(long long n, const char *type, double *sol, double *Ki,
                     double *Ti, double time, double dt, hdo_operator op, void *ctx) {
  double ai[16], bi[16];
  const int ns = hdo_lsrk_coefficients(type, ai, bi);
  if (ns == 0) return -1;
  /* first stage with only_Ti_is_ghosted = true: Ti = sol (:142-148) */
  memcpy(Ti, sol, sizeof(double) * n);
  op(Ti, Ki, time, ctx);
  stage_update(n, bi[0] * dt, ai[0] * dt, Ki, sol, Ti);
  double sum_previous_bi = 0.0;
  for (int st = 1; st < ns; ++st) {
    const double c_i = sum_previous_bi + ai[st - 1];
    op(Ti, Ki, time + c_i * dt, ctx);
    stage_update(n, bi[st] * dt, st == ns - 1 ? 0.0 : ai[st] * dt, Ki, sol, Ti);
    sum_previous_bi += bi[st - 1];
  }
  return 0;
}

static void problem_op(const double *src, double *dst, double t, void *ctx) {
  hdo_apply((const hdo_problem *)ctx, src, dst, t);
}

int hdo_lsrk_step(const hdo_problem *p, const char *type, double *sol, double *Ki,
                  double *Ti, double time, double dt) {
  const long long n = hdo_n_dofs(p);
  if (n < 0) return -1;
  return hdo_lsrk_step_op(n, type, sol, Ki, Ti, time, dt, problem_op, (void *)p);
}

/* ------------------------------------------------------------------------ */
/* interpolation and norms (vector_tools.h:81-223)                           */
/* ------------------------------------------------------------------------ */
int hdo_interpolate(const hdo_problem *p, const hdo_func *f, double time, double *dst) {
  ctx_t c;
  if (make_ctx(p, &c)) return -1;
#pragma omp parallel for schedule(static)
  for (long long g = 0; g < c.ncells; ++g) {
    int cc[HDO_MAX_DIM];
    cell_coords(&c, g, cc);
    for (int i = 0; i < c.NC; ++i) {
      double x[HDO_MAX_DIM];
      for (int d = 0; d < c.D; ++d)
        x[d] = p->lo[d] + (cc[d] + c.gl[(i / c.nstride[d]) % c.n]) * c.h[d];
      dst[g * c.NC + i] = func_value(f, c.D, x, time);
    }
  }
  return 0;
}

int hdo_norm_and_error(const hdo_problem *p, const hdo_func *f, double time,
                       const double *src, double *norm_error) {
  ctx_t c;
  if (make_ctx(p, &c)) return -1;
  double s0 = 0.0, s1 = 0.0;
#pragma omp parallel reduction(+ : s0, s1)
  {
    double *v = (double *)malloc(sizeof(double) * 2 * c.NC);
    double *tmp = v + c.NC;
#pragma omp for schedule(static)
    for (long long g = 0; g < c.ncells; ++g) {
      int cc[HDO_MAX_DIM];
      cell_coords(&c, g, cc);
      memcpy(v, src + g * c.NC, sizeof(double) * c.NC);
      if (!p->collocation)
        for (int d = 0; d < c.D; ++d) { apply_1d(&c, c.S, 0, d, v, tmp, 0); memcpy(v, tmp, sizeof(double) * c.NC); }
      double t0 = 0.0, t1 = 0.0;
      for (int q = 0; q < c.NC; ++q) {
        double x[HDO_MAX_DIM];
        for (int d = 0; d < c.D; ++d)
          x[d] = p->lo[d] + (cc[d] + c.pts[(q / c.nstride[d]) % c.n]) * c.h[d];
        const double e = v[q] - func_value(f, c.D, x, time);
        const double jxw = cell_jxw(&c, q);
        t0 += v[q] * v[q] * jxw;
        t1 += e * e * jxw;
      }
      s0 += t0;
      s1 += t1;
    }
    free(v);
  }
  norm_error[0] = sqrt(s0);
  norm_error[1] = sqrt(s1);
  return 0;
}

double hdo_critical_time_step(const hdo_problem *p) {
  /* cfl.h:56-124 on a Cartesian mesh: J^{-1} = diag(1/h) */
  ctx_t c;
  if (make_ctx(p, &c)) return -1.0;
  double vx = 0.0, vv = 0.0;
  for (int d = 0; d < c.dx; ++d) vx = fmax(vx, fabs(p->velocity[d] / c.h[d]));
  for (int d = c.dx; d < c.D; ++d) vv = fmax(vv, fabs(p->velocity[d] / c.h[d]));
  return fmin(1.0 / vx, 1.0 / vv);
}

/* ------------------------------------------------------------------------ */
/* Vlasov-Poisson pieces (examples/vlasov_poisson/include/application.h:516-602) */
/* ------------------------------------------------------------------------ */

/* v-space integral of f for every x-DoF: rho[gid_x * n^dim_x + i_x] =
   sum over v-cells and v-nodes of f * JxW_v with the Gauss-Lobatto support
   points (quad_no_v = 2) applied to the raw DoF values
   (numerics/vector_tools.h:230-315; the index i_x + n^dim_v i_v there equals
   i_x + n^dim_x i_v because dim_x == dim_v). */
int hdo_velocity_moment(const hdo_problem *p, const double *src, double *rho) {
  ctx_t c;
  if (make_ctx(p, &c)) return -1;
  int nx = 1, nv = 1;
  for (int d = 0; d < c.dx; ++d) nx *= c.n;
  for (int d = c.dx; d < c.D; ++d) nv *= c.n;
  double jv = 1.0;
  for (int d = c.dx; d < c.D; ++d) jv *= c.h[d];
#pragma omp parallel for schedule(static)
  for (long long gx = 0; gx < c.ncx; ++gx)
    for (int ix = 0; ix < nx; ++ix) {
      double acc = 0.0;
      for (long long gv = 0; gv < c.ncv; ++gv) {
        const double *u = src + (gx + c.ncx * gv) * c.NC;
        for (int iv = 0; iv < nv; ++iv) {
          double w = jv;
          int t = iv;
          for (int d = c.dx; d < c.D; ++d) { w *= c.glw[t % c.n]; t /= c.n; }
          acc += u[ix + nx * iv] * w;
        }
      }
      rho[gx * nx + ix] = acc;
    }
  return 0;
}

/* numerics/vector_tools.h:317-400 (coordinate_space_integration): the
 * x-space counterpart of the velocity moment, one v-DoF at a time: the raw
 * DoF values times the x-space JxW of the Gauss-Lobatto points (quad_no_x = 2
 * in the reference's tests), summed over every x-cell */
int hdo_coordinate_moment(const hdo_problem *p, const double *src, double *out) {
  ctx_t c;
  if (make_ctx(p, &c)) return -1;
  int nx = 1, nv = 1;
  for (int d = 0; d < c.dx; ++d) nx *= c.n;
  for (int d = c.dx; d < c.D; ++d) nv *= c.n;
  double jx = 1.0;
  for (int d = 0; d < c.dx; ++d) jx *= c.h[d];
#pragma omp parallel for schedule(static)
  for (long long gv = 0; gv < c.ncv; ++gv)
    for (int iv = 0; iv < nv; ++iv) {
      double acc = 0.0;
      for (long long gx = 0; gx < c.ncx; ++gx) {
        const double *u = src + (gx + c.ncx * gv) * c.NC;
        for (int ix = 0; ix < nx; ++ix) {
          double w = jx;
          int t = ix;
          for (int d = 0; d < c.dx; ++d) { w *= c.glw[t % c.n]; t /= c.n; }
          acc += u[ix + nx * iv] * w;
        }
      }
      out[gv * nv + iv] = acc;
    }
  return 0;
}

/* x-space view of a phase-space context */
typedef struct {
  int dx, n, NCx;
  long long ncx;
  int nstride[3];
  long long cstride[3];
  int cells[3];
  double h[3];
  const ctx_t *c;
  double dval[2][MAXN]; /* psi_j'(0), psi_j'(1) of the point basis */
} xctx_t;

static void make_xctx(const ctx_t *c, xctx_t *x) {
  x->dx = c->dx; x->n = c->n; x->c = c;
  x->NCx = 1;
  for (int d = 0; d < c->dx; ++d) {
    x->nstride[d] = x->NCx;
    x->NCx *= c->n;
    x->cstride[d] = c->cstride[d];
    x->cells[d] = c->cells[d];
    x->h[d] = c->h[d];
  }
  x->ncx = c->ncx;
  lagrange_derivs(c->n, c->pts, 0.0, x->dval[0]);
  lagrange_derivs(c->n, c->pts, 1.0, x->dval[1]);
}

/* out (+)= A along x-direction d of an x-space cell tensor */
static void xapply_1d(const xctx_t *x, const double *A, int transpose, int d, const double *in, double *out,
                      int add) {
  const int n = x->n, s = x->nstride[d];
  for (int base = 0; base < x->NCx; ++base) {
    if ((base / s) % n != 0) continue;
    double tout[MAXN];
    for (int o = 0; o < n; ++o) {
      double acc = 0.0;
      for (int i = 0; i < n; ++i) acc += (transpose ? A[i * n + o] : A[o * n + i]) * in[base + i * s];
      tout[o] = acc;
    }
    for (int o = 0; o < n; ++o) out[base + o * s] = add ? out[base + o * s] + tout[o] : tout[o];
  }
}

static double xjxw(const xctx_t *x, int q, int skip) {
  double j = 1.0;
  for (int d = 0; d < x->dx; ++d)
    if (d != skip) j *= x->h[d] * x->c->w[(q / x->nstride[d]) % x->n];
  return j;
}

/* point values of an x-space DG cell (basis change for Gauss) */
static void xvalues(const xctx_t *x, const double *u, double *v, double *tmp) {
  memcpy(v, u, sizeof(double) * x->NCx);
  for (int d = 0; d < x->dx; ++d) {
    xapply_1d(x, x->c->S, 0, d, v, tmp, 0);
    memcpy(v, tmp, sizeof(double) * x->NCx);
  }
}

/* point-basis test values -> DoF test values (S^T in every direction) */
static void xtest(const xctx_t *x, double *r, double *tmp) {
  for (int d = 0; d < x->dx; ++d) {
    xapply_1d(x, x->c->S, 1, d, r, tmp, 0);
    memcpy(r, tmp, sizeof(double) * x->NCx);
  }
}

static double vec_mean(const double *v, long long n) {
  double s = 0.0;
  for (long long i = 0; i < n; ++i) s += v[i];
  return s / (double)n;
}

/* SIPG Laplacian on the periodic x-mesh with the problem's quadrature, src
   mean removed first (examples/vlasov_poisson/include/poisson.h:100-255):
   cell  int grad u . grad v;
   faces int sigma [u][v] - {d_n u}[v] - [u]{d_n v},
         sigma = (1/h_- + 1/h_+) k (k+1) (the inverse cell extents normal to the face). */
int hdo_poisson_apply(const hdo_problem *p, const double *src, double *dst) {
  ctx_t c;
  if (make_ctx(p, &c)) return -1;
  xctx_t x;
  make_xctx(&c, &x);
  const int NCx = x.NCx, n = x.n;
  const long long N = x.ncx * NCx;
  double *u = (double *)malloc(sizeof(double) * N);
  double *vals = (double *)malloc(sizeof(double) * N);
  double *rp = (double *)calloc(N, sizeof(double));
  if (!u || !vals || !rp) { free(u); free(vals); free(rp); return -1; }
  const double mean = vec_mean(src, N);
  for (long long i = 0; i < N; ++i) u[i] = src[i] - mean;
  const int k = p->degree;
  const double pen = (double)(k > 1 ? k : 1) * (k + 1.0);
  /* point values of all cells */
  {
    double *tmp = (double *)malloc(sizeof(double) * NCx);
    for (long long g = 0; g < x.ncx; ++g) xvalues(&x, u + g * NCx, vals + g * NCx, tmp);
    free(tmp);
  }
  /* cells */
  for (long long g = 0; g < x.ncx; ++g) {
    double grad[MAXN * MAXN * MAXN], t[MAXN * MAXN * MAXN];
    for (int d = 0; d < x.dx; ++d) {
      xapply_1d(&x, c.Dq, 0, d, vals + g * NCx, grad, 0);
      for (int q = 0; q < NCx; ++q) t[q] = grad[q] / x.h[d] * xjxw(&x, q, -1) / x.h[d];
      xapply_1d(&x, c.Dq, 1, d, t, rp + g * NCx, 1);
    }
  }
  /* faces: the right face of every cell in every direction (periodic pairs) */
  for (long long g = 0; g < x.ncx; ++g) {
    int cc[3];
    long long rem = g;
    for (int d = 0; d < x.dx; ++d) { cc[d] = (int)(rem % x.cells[d]); rem /= x.cells[d]; }
    for (int d = 0; d < x.dx; ++d) {
      const long long gR = cc[d] + 1 < x.cells[d] ? g + x.cstride[d] : g - (long long)(x.cells[d] - 1) * x.cstride[d];
      const double *vL = vals + g * NCx, *vR = vals + gR * NCx;
      const int sd = x.nstride[d];
      const double sigma = (1.0 / x.h[d] + 1.0 / x.h[d]) * pen;
      for (int b = 0; b < NCx; ++b) {
        if ((b / sd) % n != 0) continue;
        double uL = 0.0, uR = 0.0, dL = 0.0, dR = 0.0;
        for (int j = 0; j < n; ++j) {
          uL += c.fval[1][j] * vL[b + j * sd];
          uR += c.fval[0][j] * vR[b + j * sd];
          dL += x.dval[1][j] * vL[b + j * sd];
          dR += x.dval[0][j] * vR[b + j * sd];
        }
        dL /= x.h[d];
        dR /= x.h[d];
        const double jxw = xjxw(&x, b, d);
        const double jump = uL - uR, avg = 0.5 * (dL + dR);
        const double vt = (sigma * jump - avg) * jxw, nt = -0.5 * jump * jxw;
        for (int j = 0; j < n; ++j) {
          rp[g * NCx + b + j * sd] += c.fval[1][j] * vt + x.dval[1][j] / x.h[d] * nt;
          rp[gR * NCx + b + j * sd] += -c.fval[0][j] * vt + x.dval[0][j] / x.h[d] * nt;
        }
      }
    }
  }
  {
    double *tmp = (double *)malloc(sizeof(double) * NCx);
    for (long long g = 0; g < x.ncx; ++g) xtest(&x, rp + g * NCx, tmp);
    free(tmp);
  }
  memcpy(dst, rp, sizeof(double) * N);
  free(u); free(vals); free(rp);
  return 0;
}

/* conjugate gradients on the singular SIPG system (no preconditioner; the
   converged solution does not depend on it).  phi holds the initial guess
   and receives the solution; stops at ||r|| <= rel_tol ||r_0||. */
int hdo_poisson_solve(const hdo_problem *p, const double *rhs, double *phi, double rel_tol, int max_it,
                      int *iterations) {
  ctx_t c;
  if (make_ctx(p, &c)) return -1;
  long long N = c.ncx;
  for (int d = 0; d < c.dx; ++d) N *= c.n;
  double *r = (double *)malloc(sizeof(double) * N), *pp = (double *)malloc(sizeof(double) * N);
  double *Ap = (double *)malloc(sizeof(double) * N);
  if (!r || !pp || !Ap) { free(r); free(pp); free(Ap); return -1; }
  hdo_poisson_apply(p, phi, Ap);
  double rr = 0.0;
  for (long long i = 0; i < N; ++i) { r[i] = rhs[i] - Ap[i]; pp[i] = r[i]; rr += r[i] * r[i]; }
  const double r0 = sqrt(rr);
  /* a floor at round-off level of the right-hand side keeps a warm start from
     iterating on noise */
  double bb = 0.0;
  for (long long i = 0; i < N; ++i) bb += rhs[i] * rhs[i];
  const double floor_tol = 1e-14 * sqrt(bb);
  int it = 0;
  while (sqrt(rr) > rel_tol * r0 && sqrt(rr) > floor_tol && it < max_it) {
    hdo_poisson_apply(p, pp, Ap);
    double pAp = 0.0;
    for (long long i = 0; i < N; ++i) pAp += pp[i] * Ap[i];
    if (!(pAp > 0.0)) break;
    const double alpha = rr / pAp;
    double rr_new = 0.0;
    for (long long i = 0; i < N; ++i) {
      phi[i] += alpha * pp[i];
      r[i] -= alpha * Ap[i];
      rr_new += r[i] * r[i];
    }
    const double beta = rr_new / rr;
    for (long long i = 0; i < N; ++i) pp[i] = r[i] + beta * pp[i];
    rr = rr_new;
    ++it;
  }
  if (iterations) *iterations = it;
  free(r); free(pp); free(Ap);
  return 0;
}

/* right-hand side of the Poisson problem from the charge density:
   rho~ = rho - mean(rho); rhs_i = -int psi_i rho~; rhs -= mean(rhs)
   (examples/vlasov_poisson/include/application.h:531-568) */
int hdo_poisson_rhs(const hdo_problem *p, const double *rho, double *rhs) {
  ctx_t c;
  if (make_ctx(p, &c)) return -1;
  xctx_t x;
  make_xctx(&c, &x);
  const long long N = x.ncx * x.NCx;
  const double mr = vec_mean(rho, N);
  double *v = (double *)malloc(sizeof(double) * x.NCx), *tmp = (double *)malloc(sizeof(double) * x.NCx);
  double *u = (double *)malloc(sizeof(double) * x.NCx);
  for (long long g = 0; g < x.ncx; ++g) {
    for (int i = 0; i < x.NCx; ++i) u[i] = rho[g * x.NCx + i] - mr;
    xvalues(&x, u, v, tmp);
    for (int q = 0; q < x.NCx; ++q) v[q] = -v[q] * xjxw(&x, q, -1);
    xtest(&x, v, tmp);
    memcpy(rhs + g * x.NCx, v, sizeof(double) * x.NCx);
  }
  const double m2 = vec_mean(rhs, N);
  for (long long i = 0; i < N; ++i) rhs[i] -= m2;
  free(v); free(tmp); free(u);
  return 0;
}

/* gradient of the potential at the x-quadrature points (the negative electric
   field, examples/vlasov_poisson/include/derivative_container.h:158-251):
   E[(gid_x * n^dim_x + q) * dim_x + d] */
int hdo_vp_field(const hdo_problem *p, const double *phi, double *E) {
  ctx_t c;
  if (make_ctx(p, &c)) return -1;
  xctx_t x;
  make_xctx(&c, &x);
  double v[MAXN * MAXN * MAXN], tmp[MAXN * MAXN * MAXN], g[MAXN * MAXN * MAXN];
  for (long long gx = 0; gx < x.ncx; ++gx) {
    xvalues(&x, phi + gx * x.NCx, v, tmp);
    for (int d = 0; d < x.dx; ++d) {
      xapply_1d(&x, c.Dq, 0, d, v, g, 0);
      for (int q = 0; q < x.NCx; ++q) E[(gx * x.NCx + q) * x.dx + d] = g[q] / x.h[d];
    }
  }
  return 0;
}

/* one evaluation of the Vlasov-Poisson right-hand side: rho, Poisson rhs,
   CG from the previous potential (phi, in/out), field E (out), then the
   advection operator with the phase-space velocity (v, E) */
int hdo_vp_operator(const hdo_problem *p, const double *f, double *dst, double time, double *phi, double *E,
                    double cg_tol, int *iterations) {
  ctx_t c;
  if (make_ctx(p, &c)) return -1;
  long long Nx = c.ncx;
  for (int d = 0; d < c.dx; ++d) Nx *= c.n;
  double *rho = (double *)malloc(sizeof(double) * Nx), *rhs = (double *)malloc(sizeof(double) * Nx);
  if (!rho || !rhs) { free(rho); free(rhs); return -1; }
  hdo_velocity_moment(p, f, rho);
  hdo_poisson_rhs(p, rho, rhs);
  hdo_poisson_solve(p, rhs, phi, cg_tol, 100000, iterations);
  hdo_vp_field(p, phi, E);
  hdo_problem q = *p;
  q.efield = E;
  const int rc = hdo_apply(&q, f, dst, time);
  free(rho); free(rhs);
  return rc;
}

/* diagnostics (examples/vlasov_poisson/include/diagnostics.h:28-141):
   out[0..dim_x) = int (d_d phi)^2 per direction; then mass, L2 norm,
   kinetic energy int |v|^2 f, and momentum int v_d f (dim_v values) */
int hdo_vp_diagnostics(const hdo_problem *p, const double *f, const double *phi, double *out) {
  ctx_t c;
  if (make_ctx(p, &c)) return -1;
  xctx_t x;
  make_xctx(&c, &x);
  const int dx = c.dx, dv = c.dv;
  for (int i = 0; i < dx + 3 + dv; ++i) out[i] = 0.0;
  {
    double v[MAXN * MAXN * MAXN], tmp[MAXN * MAXN * MAXN], g[MAXN * MAXN * MAXN];
    for (long long gx = 0; gx < x.ncx; ++gx) {
      xvalues(&x, phi + gx * x.NCx, v, tmp);
      for (int d = 0; d < dx; ++d) {
        xapply_1d(&x, c.Dq, 0, d, v, g, 0);
        for (int q = 0; q < x.NCx; ++q) {
          const double gd = g[q] / x.h[d];
          out[d] += gd * gd * xjxw(&x, q, -1);
        }
      }
    }
  }
  double mass = 0.0, l2 = 0.0, kin = 0.0, mom[3] = {0.0, 0.0, 0.0};
#pragma omp parallel reduction(+ : mass, l2, kin)
  {
    double *v = (double *)malloc(sizeof(double) * 2 * c.NC), *tmp = v + c.NC;
    double mloc[3] = {0.0, 0.0, 0.0};
#pragma omp for schedule(static)
    for (long long g = 0; g < c.ncells; ++g) {
      int cc[HDO_MAX_DIM];
      cell_coords(&c, g, cc);
      memcpy(v, f + g * c.NC, sizeof(double) * c.NC);
      if (!p->collocation)
        for (int d = 0; d < c.D; ++d) { apply_1d(&c, c.S, 0, d, v, tmp, 0); memcpy(v, tmp, sizeof(double) * c.NC); }
      for (int q = 0; q < c.NC; ++q) {
        const double jxw = cell_jxw(&c, q);
        double vv = 0.0, vel[3];
        for (int d = 0; d < dv; ++d) {
          const int e = dx + d;
          vel[d] = p->lo[e] + (cc[e] + c.pts[(q / c.nstride[e]) % c.n]) * c.h[e];
          vv += vel[d] * vel[d];
        }
        mass += v[q] * jxw;
        l2 += v[q] * v[q] * jxw;
        kin += vv * v[q] * jxw;
        for (int d = 0; d < dv; ++d) mloc[d] += vel[d] * v[q] * jxw;
      }
    }
#pragma omp critical
    for (int d = 0; d < dv; ++d) mom[d] += mloc[d];
    free(v);
  }
  out[dx] = mass;
  out[dx + 1] = sqrt(l2);
  out[dx + 2] = kin;
  for (int d = 0; d < dv; ++d) out[dx + 3 + d] = mom[d];
  return 0;
}
