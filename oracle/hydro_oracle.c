/*
 * hydro_oracle.c -- CPU oracle (plain C restatement) of hydro's time-step
 * hot path.  TEST INFRASTRUCTURE ONLY: used by tests/, the smoke check and the
 * cpu_baseline leg of bench.py as the checker; never linked into the product.
 *
 * Each function cites the reference code (divfree/hydro,
 * source/hydro2dmpi/...) whose arithmetic it restates.  Geometry is the
 * uniform Cartesian block of InitUniformMesh (mesh.hpp:722-736):
 * h_d = (B_d - A_d) / N_d, V = prod h, face area A_d = V / h_d.
 *
 * Linear rows are held as (2*dim+1) coefficients per cell in the order the
 * reference's Expression keeps its sorted terms (linear.hpp:110-115):
 *   3D: zm, ym, xm, c, xp, yp, zp     2D: ym, xm, c, xp, yp
 * plus one constant, so that sum_j a_j x_j + c = 0 (linear.hpp:547,705).
 */
#include "hydro_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#define MAXW 7

typedef struct {
  int dim;
  long n[3];
  long nc, nf;
  long fofs[3], fcnt[3];
  double h[3], V, A[3];
  double lo[3];
  int per[3]; /* periodic directions (mesh2d.hpp / mesh3d.hpp PERX, PERZ) */
  /* excluded cells (rigid box, mesh3d.hpp:183-215), NULL = none: a face
   * touching an excluded cell is not inner, and the excluded cell is not
   * its neighbour; a face with no valid neighbour is excluded */
  const unsigned char* ex;
} Mesh;

struct oracle_ctx {
  hydro_desc d;
  Mesh m;
  int nph;
  /* fluid layers: [layer][component] */
  double* u[4][3];
  double* p[4];
  double* F[4];
  /* mixture fields given to the fluid solver (hydro2d.hpp:449-463) */
  double *rho, *mu, *force[3], *stforce[3], *Sv, *Sm;
  double *rho_raw;
  /* phases */
  double* q[HYDRO_MAX_PHASES];
  double* alpha[HYDRO_MAX_PHASES];
  /* last pressure correction and momentum diagonal */
  double *pcorr, *Dc;
  /* boundary conditions per face (entries of boundary faces are used):
   * velocity of the value condition per component (walls and inlets fixed,
   * outlets refreshed every iteration), partial density of inlet faces */
  double* bcu[3];
  double* qin[HYDRO_MAX_PHASES];
  /* momentum rows of the iteration per component (kept for SIMPLER) */
  double* mrows[3];
  double* mrowc[3];
  /* heat (HeatSolver, heat.hpp:18-94), when attached */
  int heat_on;
  hydro_heat_desc hd;
  double* T[4];            /* temperature layers */
  double* kc;              /* mixture conductivity (hydro2d.hpp:1428) */
  double* tbval;           /* boundary temperature of box faces */
  unsigned char* tbder;    /* boundary faces with zero derivative */
  /* scratch */
  double* fw[10];   /* face arrays */
  double* cw[24];   /* cell arrays */
  double* rows;     /* (2*dim+1) * nc */
  double* rowc;     /* nc */
  double time, dt, adv_time, adv_dt;
  int iter_count, cd_iter_count;
  int vel_sweeps, p_iters;
  double p_res;
  int lin_status;
};

static int g_threads = 1;

int oracle_set_threads(int n) {
  g_threads = n > 0 ? n : 1;
  return HYDRO_OK;
}

/* ---------------------------------------------------------------- mesh -- */

static long cidx(const Mesh* m, long i, long j, long k) {
  return i + m->n[0] * (j + m->n[1] * k);
}
static long fidx(const Mesh* m, int d, long i, long j, long k) {
  long nx = m->n[0] + (d == 0), ny = m->n[1] + (d == 1);
  return m->fofs[d] + i + nx * (j + ny * k);
}
static void cmidx(const Mesh* m, long c, long* mi) {
  mi[0] = c % m->n[0];
  mi[1] = (c / m->n[0]) % m->n[1];
  mi[2] = c / (m->n[0] * m->n[1]);
}
/* Face q of cell c, q = 2*d + side, order xm,xp,ym,yp,zm,zp (mesh3d.hpp:297-303). */
static long cface(const Mesh* m, const long* mi, int q) {
  int d = q / 2, s = q % 2;
  long a[3] = {mi[0], mi[1], mi[2]};
  a[d] += s;
  return fidx(m, d, a[0], a[1], a[2]);
}
/* Neighbour cell across face q of cell mi, or -1; across a periodic
 * direction the last and first cells are neighbours (mesh3d.hpp:348-392). */
static long cnb(const Mesh* m, const long* mi, int q) {
  int d = q / 2, s = q % 2;
  long a[3] = {mi[0], mi[1], mi[2]};
  a[d] += s ? 1 : -1;
  if (a[d] < 0 || a[d] >= m->n[d]) {
    if (!m->per[d]) return -1;
    a[d] = a[d] < 0 ? m->n[d] - 1 : 0;
  }
  long nb = cidx(m, a[0], a[1], a[2]);
  if (m->ex && (m->ex[cidx(m, mi[0], mi[1], mi[2])] || m->ex[nb])) return -1;
  return nb;
}
static int cex(const Mesh* m, long c) { return m->ex && m->ex[c]; }
/* Decode face f: direction, multi-index, neighbour cells cm (id 0) and cp (id 1). */
static void fdecode(const Mesh* m, long f, int* dir, long* mi, long* cm, long* cp) {
  int d = 0;
  while (d < m->dim - 1 && f >= m->fofs[d + 1]) ++d;
  long r = f - m->fofs[d];
  long nx = m->n[0] + (d == 0), ny = m->n[1] + (d == 1);
  mi[0] = r % nx;
  mi[1] = (r / nx) % ny;
  mi[2] = r / (nx * ny);
  *dir = d;
  long a[3] = {mi[0], mi[1], mi[2]};
  *cp = (a[d] < m->n[d]) ? cidx(m, a[0], a[1], a[2]) : -1;
  a[d] -= 1;
  *cm = (a[d] >= 0) ? cidx(m, a[0], a[1], a[2]) : -1;
  if (m->per[d] && (*cm < 0 || *cp < 0)) {
    /* both end faces of a periodic direction join cells n-1 and 0 */
    long b[3] = {mi[0], mi[1], mi[2]};
    b[d] = m->n[d] - 1;
    *cm = cidx(m, b[0], b[1], b[2]);
    b[d] = 0;
    *cp = cidx(m, b[0], b[1], b[2]);
  }
  if (m->ex) {
    if (*cm >= 0 && m->ex[*cm]) *cm = -1;
    if (*cp >= 0 && m->ex[*cp]) *cp = -1;
  }
}
/* Side (enum hydro_side) of a boundary face, or -1 for an inner face. */
static int fside(const Mesh* m, int d, const long* mi) {
  if (mi[d] == 0) return 2 * d;
  if (mi[d] == m->n[d]) return 2 * d + 1;
  return -1;
}
/* Condition kind of a boundary face: its side's, or a wall for a face
 * between the rigid box and the fluid ("wall 0 0 0", hydro2d.hpp:386-396). */
static int fkind(const hydro_desc* d, const Mesh* m, int dir, const long* mi) {
  int side = fside(m, dir, mi);
  return side < 0 ? HYDRO_BC_WALL : d->bc_kind[side];
}
static double outward(int q) { return (q % 2) ? 1. : -1.; }

/* Row slot of the term for cell c itself / the neighbour across face q. */
static int slot_c(int dim) { return dim; }
static int slot_q(int dim, int q) {
  int d = q / 2, s = q % 2;
  return s ? dim + 1 + d : dim - 1 - d;
}

/* ------------------------------------------------------ interpolation -- */

enum { BC_VALUE = 0, BC_ZERODER = 1, BC_EXTRAP = 2, BC_NONE = 3, BC_FACE = 4 };

/* Interpolate (solver.hpp:392-470) of a scalar cell field to faces.
 * bc: BC_VALUE -> boundary face = bcval[side]; BC_ZERODER -> cell value
 * (ConditionFaceDerivativeFixed(0)); BC_EXTRAP -> ConditionFaceExtrapolation;
 * BC_NONE -> 0 (no conditions). */
static void interp(const Mesh* m, const double* fc, double* ff, int bc,
                   const double* bcval, int geometric) {
  long f;
#pragma omp parallel for num_threads(g_threads)
  for (f = 0; f < m->nf; ++f) {
    int d;
    long mi[3], cm, cp;
    fdecode(m, f, &d, mi, &cm, &cp);
    if (cm >= 0 && cp >= 0) {
      if (geometric) {
        ff[f] = sqrt(fc[cm] * fc[cp]);
      } else {
        ff[f] = fc[cm] * (1. - 0.5) + fc[cp] * 0.5;
      }
    } else {
      ff[f] = 0.;
    }
  }
  if (bc == BC_NONE) return;
  /* boundary faces in raw-index order (std::map iteration) */
  for (f = 0; f < m->nf; ++f) {
    int d;
    long mi[3], cm, cp;
    fdecode(m, f, &d, mi, &cm, &cp);
    if (cm >= 0 && cp >= 0) continue;
    if (cm < 0 && cp < 0) continue;  /* excluded face: no condition, 0 */
    int side = fside(m, d, mi);
    long cc = cm >= 0 ? cm : cp;
    double factor = cm >= 0 ? 1. : -1.;
    double dist = 0.5 * m->h[d];
    if (bc == BC_VALUE) {
      ff[f] = side >= 0 ? bcval[side] : 0.;
    } else if (bc == BC_FACE) {
      ff[f] = bcval[f];
    } else if (bc == BC_ZERODER) {
      ff[f] = fc[cc] + 0. * (dist * factor);
    } else {
      /* extrapolation: nom/den with the opposite face of the cell */
      long ci[3];
      cmidx(m, cc, ci);
      int qself = 2 * d + (cm >= 0 ? 1 : 0);
      int qopp = qself ^ 1;
      long fo = cface(m, ci, qopp);
      double nom = fc[cc] / dist;
      double den = 1. / dist;
      den -= m->A[d] / m->V;
      nom += ff[fo] * (-m->A[d]) / m->V;
      ff[f] = nom / den;
    }
  }
}

/* Interpolate of a vector cell field (components fc[0..dim-1]) with
 * zero-derivative boundaries.  With `geometric` the inner faces take the
 * Vect overload of GetGeometricAverage (solver.hpp:380-390): direction of
 * the arithmetic mean, magnitude sqrt(|a| |b|). */
static void interp_vec(const Mesh* m, double* const* fc, double* const* ff, int geometric) {
  int dim = m->dim;
  if (!geometric) {
    for (int k = 0; k < dim; ++k) interp(m, fc[k], ff[k], BC_ZERODER, NULL, 0);
    return;
  }
  long f;
#pragma omp parallel for num_threads(g_threads)
  for (f = 0; f < m->nf; ++f) {
    int d;
    long mi[3], cm, cp;
    fdecode(m, f, &d, mi, &cm, &cp);
    if (cm >= 0 && cp >= 0) {
      double av[3], n2 = 0., na = 0., nb = 0.;
      for (int k = 0; k < dim; ++k) {
        av[k] = (fc[k][cm] + fc[k][cp]) * 0.5;
        n2 += av[k] * av[k];
        na += fc[k][cm] * fc[k][cm];
        nb += fc[k][cp] * fc[k][cp];
      }
      double an = sqrt(n2);
      for (int k = 0; k < dim; ++k)
        ff[k][f] = an < 1e-8 ? av[k] : av[k] / an * sqrt(sqrt(na) * sqrt(nb));
    } else if (cm >= 0 || cp >= 0) {
      long cc = cm >= 0 ? cm : cp;
      for (int k = 0; k < dim; ++k) ff[k][f] = fc[k][cc];
    } else {
      for (int k = 0; k < dim; ++k) ff[k][f] = 0.;
    }
  }
}

/* Gradient (solver.hpp:658-677): Green-Gauss from face values. */
static void gradient(const Mesh* m, const double* ff, double* const* gc) {
  long c;
#pragma omp parallel for num_threads(g_threads)
  for (c = 0; c < m->nc; ++c) {
    long mi[3];
    cmidx(m, c, mi);
    for (int d = 0; d < m->dim; ++d) {
      if (cex(m, c)) {  /* excluded cells keep zero */
        gc[d][c] = 0.;
        continue;
      }
      long flo = cface(m, mi, 2 * d), fhi = cface(m, mi, 2 * d + 1);
      double sum = (-m->A[d]) * ff[flo];
      sum += m->A[d] * ff[fhi];
      gc[d][c] = sum / m->V;
    }
  }
}

/* GetSmoothField (solver.hpp:636-656): repeat { face average with
 * zero-derivative boundaries, then Average (solver.hpp:621-634) }. */
static void smooth(const Mesh* m, double* fc, int repeat, double* fface) {
  for (int r = 0; r < repeat; ++r) {
    interp(m, fc, fface, BC_ZERODER, NULL, 0);
    long c;
#pragma omp parallel for num_threads(g_threads)
    for (c = 0; c < m->nc; ++c) {
      long mi[3];
      cmidx(m, c, mi);
      double sum = 0.;
      for (int q = 0; q < 2 * m->dim; ++q) sum += fface[cface(m, mi, q)];
      fc[c] = sum / (double)(2 * m->dim);
    }
  }
}

/* ------------------------------------------------------ linear solvers -- */

/* rows: (2*dim+1) coefficients per cell, rowc: constants. */
static double row_offsum(const Mesh* m, const double* a, const long* mi,
                         const double* x, long c) {
  int dim = m->dim, w = 2 * dim + 1;
  double sum = 0.;
  /* sorted order: zm, ym, xm, xp, yp, zp */
  for (int s = 0; s < w; ++s) {
    if (s == dim) continue;
    int q = s < dim ? 2 * (dim - 1 - s) : 2 * (s - dim - 1) + 1;
    long nb = cnb(m, mi, q);
    if (nb < 0) continue;
    sum += a[c * w + s] * x[nb];
  }
  (void)mi;
  return sum;
}

/* GaussSeidel::Solve (linear.hpp:685-715). */
static int solve_gs(const Mesh* m, const double* a, const double* b, double* x,
                    double tol, int limit, double omega, int* iters) {
  int w = 2 * m->dim + 1;
  for (long c = 0; c < m->nc; ++c) x[c] = 0.;
  int iter = 0;
  double diff;
  do {
    diff = 0.;
    for (long c = 0; c < m->nc; ++c) {
      long mi[3];
      cmidx(m, c, mi);
      double sum = row_offsum(m, a, mi, x, c);
      double diag = a[c * w + m->dim];
      double value = -(b[c] + sum) / diag;
      double corr = value - x[c];
      if (fabs(corr) > diff) diff = fabs(corr);
      x[c] += corr * omega;
    }
  } while (diff > tol && iter++ < limit);
  *iters = iter;
  return (diff > tol) ? HYDRO_NOT_CONVERGED : HYDRO_OK;
}

/* Jacobi::Solve (linear.hpp:750-782). */
static int solve_jacobi(const Mesh* m, const double* a, const double* b,
                        double* x, double* next, double tol, int limit,
                        double omega, int* iters) {
  int w = 2 * m->dim + 1;
  for (long c = 0; c < m->nc; ++c) x[c] = 0.;
  int iter = 0;
  double diff;
  do {
    diff = 0.;
    long c;
    double dloc = 0.;
#pragma omp parallel for num_threads(g_threads) reduction(max : dloc)
    for (c = 0; c < m->nc; ++c) {
      long mi[3];
      cmidx(m, c, mi);
      double sum = row_offsum(m, a, mi, x, c);
      double diag = a[c * w + m->dim];
      double value = -(b[c] + sum) / diag;
      double corr = value - x[c];
      if (fabs(corr) > dloc) dloc = fabs(corr);
      next[c] = x[c] + corr * omega;
    }
    diff = dloc;
    memcpy(x, next, sizeof(double) * m->nc);
  } while (diff > tol && iter++ < limit);
  *iters = iter;
  return (diff > tol) ? HYDRO_NOT_CONVERGED : HYDRO_OK;
}

/* LuDecomposition::Solve (linear.hpp:533-566): forward sweep over terms of
 * lower raw index, then backward sweep over higher ones. */
static int solve_lu(const Mesh* m, const double* a, const double* b, double* x,
                    int* iters) {
  int dim = m->dim, w = 2 * dim + 1;
  for (long c = 0; c < m->nc; ++c) {
    long mi[3];
    cmidx(m, c, mi);
    double sum = 0.;
    for (int s = 0; s < dim; ++s) {
      int q = 2 * (dim - 1 - s);
      long nb = cnb(m, mi, q);
      if (nb < 0) continue;
      sum += a[c * w + s] * x[nb];
    }
    x[c] = (-b[c] - sum) / a[c * w + dim];
  }
  for (long c = m->nc; c > 0;) {
    --c;
    long mi[3];
    cmidx(m, c, mi);
    double sum = 0.;
    for (int s = w - 1; s > dim; --s) {
      int q = 2 * (s - dim - 1) + 1;
      long nb = cnb(m, mi, q);
      if (nb < 0) continue;
      sum += a[c * w + s] * x[nb];
    }
    x[c] -= sum / a[c * w + dim];
  }
  *iters = 1;
  return HYDRO_OK;
}

/* Jacobi-preconditioned CG for a symmetric positive (semi-)definite stencil
 * given as face couplings k_f >= 0 (coupling -k_f, diagonal sum k_f + shift).
 * New relative to the reference, which has no Krylov solver; the GPU path
 * runs the same algorithm. */
static double dotp(long n, const double* a, const double* b) {
  double s = 0.;
  long i;
#pragma omp parallel for num_threads(g_threads) reduction(+ : s)
  for (i = 0; i < n; ++i) s += a[i] * b[i];
  return s;
}

static void stencil_apply(const Mesh* m, const double* k, double shift,
                          long pin, const double* x, double* y) {
  long c;
#pragma omp parallel for num_threads(g_threads)
  for (c = 0; c < m->nc; ++c) {
    if (c == pin || cex(m, c)) {  /* identity rows */
      y[c] = x[c];
      continue;
    }
    long mi[3];
    cmidx(m, c, mi);
    double diag = shift, off = 0.;
    for (int q = 0; q < 2 * m->dim; ++q) {
      long nb = cnb(m, mi, q);
      if (nb < 0) continue;
      double kf = k[cface(m, mi, q)];
      diag += kf;
      if (nb != pin) off += kf * x[nb];
    }
    y[c] = diag * x[c] - off;
  }
}

static void stencil_diag(const Mesh* m, const double* k, double shift, long pin,
                         double* dg) {
  for (long c = 0; c < m->nc; ++c) {
    if (c == pin || cex(m, c)) {
      dg[c] = 1.;
      continue;
    }
    long mi[3];
    cmidx(m, c, mi);
    double diag = shift;
    for (int q = 0; q < 2 * m->dim; ++q) {
      if (cnb(m, mi, q) < 0) continue;
      diag += k[cface(m, mi, q)];
    }
    dg[c] = diag;
  }
}

/* Solves A x = f.  Work: 5 cell arrays. */
static int pcg(const Mesh* m, const double* k, double shift, long pin,
               const double* f_in, double* x, int use_guess, double tol,
               int limit, double** wk, int* iters, double* res) {
  long n = m->nc;
  double *r = wk[0], *z = wk[1], *pp = wk[2], *Ap = wk[3], *dg = wk[4];
  int singular = (shift == 0. && pin < 0);
  stencil_diag(m, k, shift, pin, dg);
  /* r = f (projected when singular) */
  /* mean over the cells that are not excluded (the singular block) */
  double mean = 0.;
  long nin = 0;
  for (long i = 0; i < n; ++i) nin += !cex(m, i);
  if (singular) {
    for (long i = 0; i < n; ++i)
      if (!cex(m, i)) mean += f_in[i];
    mean /= (double)nin;
  }
  for (long i = 0; i < n; ++i) r[i] = cex(m, i) ? f_in[i] : f_in[i] - mean;
  double fnorm = sqrt(dotp(n, r, r));
  /* a NaN in the system is reported, as the library does (the reference's
     Gauss-Seidel would carry it into p and throw, fluid.hpp:1164-1166) */
  if (isnan(fnorm)) return HYDRO_ERR_NAN;
  if (!use_guess) {
    for (long i = 0; i < n; ++i) x[i] = 0.;
  } else {
    stencil_apply(m, k, shift, pin, x, Ap);
    for (long i = 0; i < n; ++i) r[i] -= Ap[i];
  }
  *iters = 0;
  if (fnorm == 0.) {
    for (long i = 0; i < n; ++i) x[i] = 0.;
    *res = 0.;
    return HYDRO_OK;
  }
  double rnorm = sqrt(dotp(n, r, r));
  for (long i = 0; i < n; ++i) z[i] = r[i] / dg[i];
  for (long i = 0; i < n; ++i) pp[i] = z[i];
  double rz = dotp(n, r, z);
  int it = 0;
  while (rnorm > tol * fnorm && it < limit) {
    stencil_apply(m, k, shift, pin, pp, Ap);
    double pAp = dotp(n, pp, Ap);
    double al = rz / pAp;
    for (long i = 0; i < n; ++i) {
      x[i] += al * pp[i];
      r[i] -= al * Ap[i];
    }
    ++it;
    rnorm = sqrt(dotp(n, r, r));
    for (long i = 0; i < n; ++i) z[i] = r[i] / dg[i];
    double rz1 = dotp(n, r, z);
    double be = rz1 / rz;
    rz = rz1;
    for (long i = 0; i < n; ++i) pp[i] = z[i] + be * pp[i];
  }
  if (singular) {
    double xm = 0.;
    for (long i = 0; i < n; ++i)
      if (!cex(m, i)) xm += x[i];
    xm /= (double)nin;
    for (long i = 0; i < n; ++i)
      if (!cex(m, i)) x[i] -= xm;
  }
  *iters = it;
  *res = rnorm / fnorm;
  return rnorm > tol * fnorm ? HYDRO_NOT_CONVERGED : HYDRO_OK;
}

static int mesh_init(Mesh* m, int dim, const int* n, const double* lo,
                     const double* hi) {
  memset(m, 0, sizeof(*m));
  if (dim != 2 && dim != 3) return HYDRO_ERR_ARG;
  m->dim = dim;
  for (int d = 0; d < 3; ++d) {
    m->n[d] = d < dim ? n[d] : 1;
    if (m->n[d] < 1) return HYDRO_ERR_ARG;
    if (d < dim && m->n[d] < 2) return HYDRO_ERR_ARG;
    m->lo[d] = d < dim ? lo[d] : 0.;
    m->h[d] = d < dim ? (hi[d] - lo[d]) / (double)n[d] : 1.;
  }
  m->nc = m->n[0] * m->n[1] * m->n[2];
  long off = 0;
  for (int d = 0; d < dim; ++d) {
    long cnt = 1;
    for (int e = 0; e < 3; ++e) cnt *= m->n[e] + (e == d);
    m->fofs[d] = off;
    m->fcnt[d] = cnt;
    off += cnt;
  }
  for (int d = dim; d < 3; ++d) m->fofs[d] = off;
  m->nf = off;
  m->V = 1.;
  for (int d = 0; d < dim; ++d) m->V *= m->h[d];
  for (int d = 0; d < dim; ++d) m->A[d] = m->V / m->h[d];
  return HYDRO_OK;
}

int oracle_stencil_solve(int dim, int nx, int ny, int nz,
                         const double* face_coeff, double shift,
                         long pinned_cell, double pinned_value,
                         const double* rhs, double* x, int use_guess,
                         double tolerance, int iters_limit, int* iterations,
                         double* residual) {
  Mesh m;
  int n[3] = {nx, ny, nz};
  double lo[3] = {0, 0, 0}, hi[3] = {1, 1, 1};
  if (mesh_init(&m, dim, n, lo, hi)) return HYDRO_ERR_ARG;
  double* wk[6];
  for (int i = 0; i < 6; ++i) wk[i] = (double*)malloc(sizeof(double) * m.nc);
  double* f = wk[5];
  /* A x = -c with the pinned value substituted */
  for (long c = 0; c < m.nc; ++c) f[c] = -rhs[c];
  if (pinned_cell >= 0) {
    long mi[3];
    cmidx(&m, pinned_cell, mi);
    for (int q = 0; q < 2 * dim; ++q) {
      long nb = cnb(&m, mi, q);
      if (nb < 0) continue;
      f[nb] += face_coeff[cface(&m, mi, q)] * pinned_value;
    }
    f[pinned_cell] = pinned_value;
  }
  int it = 0;
  double res = 0.;
  int st = pcg(&m, face_coeff, shift, pinned_cell, f, x, use_guess, tolerance,
               iters_limit, wk, &it, &res);
  if (iterations) *iterations = it;
  if (residual) *residual = res;
  for (int i = 0; i < 6; ++i) free(wk[i]);
  return st;
}

/* ------------------------------------------------------------ context -- */

static double* alloc0(long n) { return (double*)calloc((size_t)(n > 0 ? n : 1), sizeof(double)); }

int oracle_create(const hydro_desc* desc, oracle_ctx** out) {
  if (!desc || !out) return HYDRO_ERR_ARG;
  if (desc->simpler && desc->rhie_chow_factor == 0.) return HYDRO_ERR_ARG;
  if (desc->num_phases < 1 || desc->num_phases > HYDRO_MAX_PHASES) return HYDRO_ERR_ARG;
  oracle_ctx* x = (oracle_ctx*)calloc(1, sizeof(oracle_ctx));
  x->d = *desc;
  if (mesh_init(&x->m, desc->dim, desc->n, desc->lo, desc->hi)) {
    free(x);
    return HYDRO_ERR_ARG;
  }
  for (int d = 0; d < desc->dim; ++d) x->m.per[d] = desc->periodic[d] != 0;
  if (desc->rigid_box) {
    /* cells whose centre lies in the box (Rect::IsInside, inclusive) */
    if (desc->simpler) {
      free(x);
      return HYDRO_ERR_UNSUPPORTED;
    }
    unsigned char* ex = (unsigned char*)calloc((size_t)x->m.nc, 1);
    long any = 0;
    for (long c = 0; c < x->m.nc; ++c) {
      long mi[3];
      cmidx(&x->m, c, mi);
      int in = 1;
      for (int k = 0; k < desc->dim; ++k) {
        double xc = x->m.lo[k] + (mi[k] + 0.5) * x->m.h[k];
        if (xc < desc->rigid_box_lo[k] || desc->rigid_box_hi[k] < xc) in = 0;
      }
      ex[c] = (unsigned char)in;
      any += in;
    }
    if (desc->pressure_fixed_cell >= 0 && desc->pressure_fixed_cell < x->m.nc &&
        ex[desc->pressure_fixed_cell]) {
      free(ex);
      free(x);
      return HYDRO_ERR_ARG;
    }
    if (any) x->m.ex = ex;
    else free(ex);
  }
  for (int s = 0; s < 2 * desc->dim; ++s)
    if (desc->bc_kind[s] < HYDRO_BC_WALL || desc->bc_kind[s] > HYDRO_BC_OUTLET) {
      free(x);
      return HYDRO_ERR_ARG;
    }
  const Mesh* m = &x->m;
  x->nph = desc->num_phases;
  for (int l = 0; l < 4; ++l) {
    for (int d = 0; d < 3; ++d) x->u[l][d] = alloc0(m->nc);
    x->p[l] = alloc0(m->nc);
    x->F[l] = alloc0(m->nf);
  }
  x->rho = alloc0(m->nc);
  x->mu = alloc0(m->nc);
  x->rho_raw = alloc0(m->nc);
  for (int d = 0; d < 3; ++d) {
    x->force[d] = alloc0(m->nc);
    x->stforce[d] = alloc0(m->nc);
  }
  x->Sv = alloc0(m->nc);
  x->Sm = alloc0(m->nc);
  for (int i = 0; i < HYDRO_MAX_PHASES; ++i) {
    x->q[i] = alloc0(m->nc);
    x->alpha[i] = alloc0(m->nc);
  }
  x->pcorr = alloc0(m->nc);
  x->Dc = alloc0(m->nc);
  for (int k = 0; k < 3; ++k) x->bcu[k] = alloc0(m->nf);
  for (int k = 0; k < 3; ++k) {
    x->mrows[k] = alloc0(m->nc * (2 * m->dim + 1));
    x->mrowc[k] = alloc0(m->nc);
  }
  for (int i = 0; i < HYDRO_MAX_PHASES; ++i) x->qin[i] = alloc0(m->nf);
  /* value conditions of the velocity: wall and inlet velocities as given,
   * outlets start at zero (OutletAuto, fluid.hpp:340-364) */
  for (long f = 0; f < m->nf; ++f) {
    int d;
    long mi[3], cm, cp;
    fdecode(m, f, &d, mi, &cm, &cp);
    if (cm >= 0 && cp >= 0) continue;
    if (cm < 0 && cp < 0) continue;  /* excluded face */
    int side = fside(m, d, mi);
    if (side < 0) continue;          /* rigid-box wall at rest */
    for (int k = 0; k < desc->dim; ++k)
      x->bcu[k][f] = desc->bc_kind[side] == HYDRO_BC_OUTLET ? 0. : desc->bc_velocity[side][k];
  }
  for (int i = 0; i < 10; ++i) x->fw[i] = alloc0(m->nf);
  for (int i = 0; i < 24; ++i) x->cw[i] = alloc0(m->nc);
  x->rows = alloc0(m->nc * (2 * m->dim + 1));
  x->rowc = alloc0(m->nc);
  x->dt = desc->dt;
  x->adv_dt = desc->dt * desc->advection_dt_factor;
  *out = x;
  return HYDRO_OK;
}

int oracle_destroy(oracle_ctx* x) {
  if (!x) return HYDRO_OK;
  for (int l = 0; l < 4; ++l) {
    for (int d = 0; d < 3; ++d) free(x->u[l][d]);
    free(x->p[l]);
    free(x->F[l]);
  }
  free(x->rho); free(x->mu); free(x->rho_raw);
  for (int d = 0; d < 3; ++d) { free(x->force[d]); free(x->stforce[d]); }
  free(x->Sv); free(x->Sm);
  for (int i = 0; i < HYDRO_MAX_PHASES; ++i) { free(x->q[i]); free(x->alpha[i]); }
  free(x->pcorr); free(x->Dc);
  for (int k = 0; k < 3; ++k) free(x->bcu[k]);
  for (int k = 0; k < 3; ++k) { free(x->mrows[k]); free(x->mrowc[k]); }
  for (int l = 0; l < 4; ++l) free(x->T[l]);
  free(x->kc); free(x->tbval); free(x->tbder);
  for (int i = 0; i < HYDRO_MAX_PHASES; ++i) free(x->qin[i]);
  for (int i = 0; i < 10; ++i) free(x->fw[i]);
  for (int i = 0; i < 24; ++i) free(x->cw[i]);
  free(x->rows); free(x->rowc);
  free((void*)x->m.ex);
  free(x);
  return HYDRO_OK;
}

static int field_arrays(oracle_ctx* x, int field, int layer, double** arr,
                        int* narr, long* len) {
  const Mesh* m = &x->m;
  int dim = m->dim;
  if (layer < 0 || layer > 3) return HYDRO_ERR_ARG;
  *len = m->nc;
  switch (field) {
    case HYDRO_FIELD_VELOCITY:
      for (int d = 0; d < dim; ++d) arr[d] = x->u[layer][d];
      *narr = dim;
      return HYDRO_OK;
    case HYDRO_FIELD_PRESSURE:
      arr[0] = x->p[layer]; *narr = 1; return HYDRO_OK;
    case HYDRO_FIELD_VOLUME_FLUX:
      arr[0] = x->F[layer]; *narr = 1; *len = m->nf; return HYDRO_OK;
    case HYDRO_FIELD_PARTIAL_DENSITY:
      for (int i = 0; i < x->nph; ++i) arr[i] = x->q[i];
      *narr = x->nph; return HYDRO_OK;
    case HYDRO_FIELD_VOLUME_FRACTION:
      for (int i = 0; i < x->nph; ++i) arr[i] = x->alpha[i];
      *narr = x->nph; return HYDRO_OK;
    case HYDRO_FIELD_DENSITY: arr[0] = x->rho; *narr = 1; return HYDRO_OK;
    case HYDRO_FIELD_VISCOSITY: arr[0] = x->mu; *narr = 1; return HYDRO_OK;
    case HYDRO_FIELD_FORCE:
      for (int d = 0; d < dim; ++d) arr[d] = x->force[d];
      *narr = dim; return HYDRO_OK;
    case HYDRO_FIELD_VOLUME_SOURCE: arr[0] = x->Sv; *narr = 1; return HYDRO_OK;
    case HYDRO_FIELD_MASS_SOURCE: arr[0] = x->Sm; *narr = 1; return HYDRO_OK;
    case HYDRO_FIELD_PRESSURE_CORRECTION: arr[0] = x->pcorr; *narr = 1; return HYDRO_OK;
    case HYDRO_FIELD_DIAG_COEFF: arr[0] = x->Dc; *narr = 1; return HYDRO_OK;
    case HYDRO_FIELD_SURFACE_FORCE:
      for (int d = 0; d < dim; ++d) arr[d] = x->stforce[d];
      *narr = dim; return HYDRO_OK;
  }
  return HYDRO_ERR_ARG;
}

int oracle_set_field(oracle_ctx* x, int field, int layer, const double* src, size_t n) {
  double* arr[HYDRO_MAX_PHASES > 3 ? HYDRO_MAX_PHASES : 3];
  int na;
  long len;
  int st = field_arrays(x, field, layer, arr, &na, &len);
  if (st) return st;
  if (n != (size_t)(na * len)) return HYDRO_ERR_ARG;
  for (int a = 0; a < na; ++a) memcpy(arr[a], src + a * len, sizeof(double) * len);
  return HYDRO_OK;
}

int oracle_get_field(oracle_ctx* x, int field, int layer, double* dst, size_t n) {
  double* arr[HYDRO_MAX_PHASES > 3 ? HYDRO_MAX_PHASES : 3];
  int na;
  long len;
  int st = field_arrays(x, field, layer, arr, &na, &len);
  if (st) return st;
  if (n != (size_t)(na * len)) return HYDRO_ERR_ARG;
  for (int a = 0; a < na; ++a) memcpy(dst + a * len, arr[a], sizeof(double) * len);
  return HYDRO_OK;
}

/* --------------------------------------------------------- properties -- */

/* hydro<Mesh>::UpdateFluidProperties (hydro2d.hpp:1404-1430) with
 * CalcPhasesVolumeFraction (980-997), GetVolumeAveraged (1221-1246),
 * GetSmoothField, CalcForce (1308-1376), CalcMixtureVolumeSource (1378-1400).
 * Mass sources are zero (chemistry intensity 0), no settling slip. */
int oracle_update_properties(oracle_ctx* x) {
  const Mesh* m = &x->m;
  int dim = m->dim, nph = x->nph;
  const hydro_desc* d = &x->d;
  for (long c = 0; c < m->nc; ++c) {
    double sum = 0.;
    for (int i = 0; i < nph; ++i) {
      x->alpha[i][c] = x->q[i][c] / d->density[i];
      sum += x->alpha[i][c];
    }
    for (int i = 0; i < nph; ++i) x->alpha[i][c] /= sum;
  }
  for (long c = 0; c < m->nc; ++c) {
    x->rho_raw[c] = 0.;
    x->mu[c] = 0.;
  }
  for (int i = 0; i < nph; ++i)
    for (long c = 0; c < m->nc; ++c) x->rho_raw[c] += d->density[i] * x->alpha[i][c];
  for (int i = 0; i < nph; ++i)
    for (long c = 0; c < m->nc; ++c) x->mu[c] += d->viscosity[i] * x->alpha[i][c];
  memcpy(x->rho, x->rho_raw, sizeof(double) * m->nc);
  smooth(m, x->rho, d->density_smooth_times, x->fw[0]);
  smooth(m, x->mu, d->viscosity_smooth_times, x->fw[0]);
  for (long c = 0; c < m->nc; ++c) {
    x->Sm[c] = 0.;
    x->Sv[c] = 0.;
  }
  /* force = gravity * rho + force (unsmoothed mixture density) */
  for (int k = 0; k < dim; ++k)
    for (long c = 0; c < m->nc; ++c)
      x->force[k][c] = d->gravity[k] * x->rho_raw[c] + d->force[k];
  /* surface tension (hydro2d.hpp:1318-1370) */
  for (int k = 0; k < dim; ++k)
    for (long c = 0; c < m->nc; ++c) x->stforce[k][c] = 0.;
  if (nph >= 2) {
    double* af = x->fw[1];
    double* gc[3] = {x->cw[0], x->cw[1], x->cw[2]};
    double* gf[3] = {x->fw[2], x->fw[3], x->fw[4]};
    interp(m, x->alpha[1], af, BC_ZERODER, NULL, 0);
    gradient(m, af, gc);
    for (int k = 0; k < dim; ++k) interp(m, gc[k], gf[k], BC_ZERODER, NULL, 0);
    for (long c = 0; c < m->nc; ++c) {
      long mi[3];
      cmidx(m, c, mi);
      double f[3] = {0, 0, 0};
      for (int q = 0; q < 2 * dim; ++q) {
        long fq = cface(m, mi, q);
        double g[3] = {0, 0, 0}, gn2 = 0.;
        for (int k = 0; k < dim; ++k) {
          g[k] = gf[k][fq];
          gn2 += g[k] * g[k];
        }
        double gn = sqrt(gn2);
        double nrm[3];
        for (int k = 0; k < dim; ++k) nrm[k] = g[k] / (gn + 1e-6);
        double s[3] = {0, 0, 0};
        s[q / 2] = m->A[q / 2] * outward(q);
        double sn = 0.;
        for (int k = 0; k < dim; ++k) sn += s[k] * nrm[k];
        for (int k = 0; k < dim; ++k) f[k] += g[k] * sn;
        for (int k = 0; k < dim; ++k) f[k] -= s[k] * gn;
      }
      for (int k = 0; k < dim; ++k) x->stforce[k][c] = f[k] / m->V * d->sigma;
    }
  }
  for (int k = 0; k < dim; ++k) smooth(m, x->force[k], d->force_smooth_times, x->fw[0]);
  if (x->heat_on) {
    /* fc_conductivity = sum_i alpha_i k_i (hydro2d.hpp:1428) */
    for (long c = 0; c < m->nc; ++c) {
      double s = 0.;
      for (int i = 0; i < nph; ++i) s += x->hd.conductivity[i] * x->alpha[i][c];
      x->kc[c] = s;
    }
  }
  return HYDRO_OK;
}

int oracle_smooth_field(oracle_ctx* x, double* field, int repeat) {
  smooth(&x->m, field, repeat, x->fw[0]);
  return HYDRO_OK;
}

/* Initial fluxes of the FluidSimple ctor (fluid.hpp:767-791) plus the
 * module's initial UpdateFluidProperties (hydro2d.hpp:962). */
int oracle_init_state(oracle_ctx* x) {
  const Mesh* m = &x->m;
  int dim = m->dim;
  for (int k = 0; k < dim; ++k)
    memcpy(x->u[HYDRO_TIME_PREV][k], x->u[HYDRO_TIME_CURR][k], sizeof(double) * m->nc);
  for (long c = 0; c < m->nc; ++c) {
    x->p[HYDRO_TIME_CURR][c] = 0.;
    x->p[HYDRO_TIME_PREV][c] = 0.;
  }
  double* uf = x->fw[1];
  double* F = x->F[HYDRO_TIME_CURR];
  for (long f = 0; f < m->nf; ++f) F[f] = 0.;
  /* inlet faces carry the initial partial density of their cell
   * (hydro2d.hpp:566-582) */
  for (long f = 0; f < m->nf; ++f) {
    int d;
    long mi[3], cm, cp;
    fdecode(m, f, &d, mi, &cm, &cp);
    if (cm >= 0 && cp >= 0) continue;
    if (cm < 0 && cp < 0) continue;
    if (fkind(&x->d, m, d, mi) != HYDRO_BC_INLET) continue;
    for (int i = 0; i < x->nph; ++i) x->qin[i][f] = x->q[i][cm >= 0 ? cm : cp];
  }
  for (int k = 0; k < dim; ++k) {
    interp(m, x->u[HYDRO_TIME_CURR][k], uf, BC_FACE, x->bcu[k], 0);
    long f0 = m->fofs[k], f1 = f0 + m->fcnt[k];
    for (long f = f0; f < f1; ++f) F[f] = uf[f] * m->A[k];
  }
  for (long f = 0; f < m->nf; ++f) {
    int d;
    long mi[3], cm, cp;
    fdecode(m, f, &d, mi, &cm, &cp);
    F[f] -= x->d.meshvel[d] * m->A[d];
  }
  memcpy(x->F[HYDRO_TIME_PREV], F, sizeof(double) * m->nf);
  x->time = 0.;
  x->adv_time = 0.;
  return oracle_update_properties(x);
}

/* -------------------------------------------------------------- fluid -- */

int oracle_start_step(oracle_ctx* x) {
  const Mesh* m = &x->m;
  double ge = x->d.guess_extrapolation;
  x->iter_count = 0;
  x->cd_iter_count = 0;
  x->vel_sweeps = 0;
  x->p_iters = 0;
  x->p_res = 0.;
  for (long c = 0; c < m->nc; ++c)
    if (isnan(x->p[HYDRO_TIME_CURR][c])) return HYDRO_ERR_NAN;
  for (int k = 0; k < m->dim; ++k)
    for (long c = 0; c < m->nc; ++c)
      x->u[HYDRO_ITER_CURR][k][c] =
          x->u[HYDRO_TIME_CURR][k][c] +
          (x->u[HYDRO_TIME_CURR][k][c] - x->u[HYDRO_TIME_PREV][k][c]) * ge;
  for (long c = 0; c < m->nc; ++c)
    x->p[HYDRO_ITER_CURR][c] = x->p[HYDRO_TIME_CURR][c] +
        (x->p[HYDRO_TIME_CURR][c] - x->p[HYDRO_TIME_PREV][c]) * ge;
  for (long f = 0; f < m->nf; ++f)
    x->F[HYDRO_ITER_CURR][f] = x->F[HYDRO_TIME_CURR][f] +
        (x->F[HYDRO_TIME_CURR][f] - x->F[HYDRO_TIME_PREV][f]) * ge;
  return HYDRO_OK;
}

/* GetDerivativeApproxCoeffs(0, {-2dt, -dt, 0}, skip) (solver.hpp:815-861). */
static void bdf_coeffs(double dt, int second, double* co) {
  double args[3] = {-2. * dt, -dt, 0.};
  int skip = second ? 0 : 1;
  int sz = 3 - skip;
  co[0] = co[1] = co[2] = 0.;
  for (int i = 0; i < sz; ++i) {
    double denom = 1., numer = 0.;
    for (int j = 0; j < sz; ++j) {
      if (j == i) continue;
      denom *= args[skip + i] - args[skip + j];
      double term = 1.;
      for (int k = 0; k < sz; ++k)
        if (k != i && k != j) term *= 0. - args[skip + k];
      numer += term;
    }
    co[skip + i] = numer / denom;
  }
}

/* One velocity component: ConvectionDiffusionScalarImplicit::MakeIteration
 * (conv_diff.hpp:130-251) assembly.  Writes rows/rowc (delta form, relaxed)
 * and returns nothing; u_prev is the iteration's starting field. */
/* Scalar form: scaling (NULL = 1) multiplies the unsteady and convective
 * terms, dfr is the face diffusion rate, bcval the per-face boundary
 * values; bcderiv (NULL = none) marks boundary faces with a zero-derivative
 * condition instead (InterpolationBoundaryFaceNearestCell /
 * DerivativeBoundaryFacePlain, solver.hpp:246-341). */
static void assemble_scalar(oracle_ctx* x, const double* u_prev, const double* u_tc,
                            const double* u_tp, const double* Fp, const double* dfr,
                            const double* src, const double* scaling, const double* bcval,
                            const unsigned char* bcderiv, double dt, int second_order,
                            double relax);

static void assemble_momentum(oracle_ctx* x, int n, const double* u_prev,
                              const double* u_tc, const double* u_tp,
                              const double* Fp, const double* muf,
                              const double* src) {
  assemble_scalar(x, u_prev, u_tc, u_tp, Fp, muf, src, x->rho, x->bcu[n], NULL, x->dt,
                  x->d.time_second_order, x->d.velocity_relaxation_factor);
}

static void assemble_scalar(oracle_ctx* x, const double* u_prev, const double* u_tc,
                            const double* u_tp, const double* Fp, const double* muf,
                            const double* src, const double* scaling, const double* bcval,
                            const unsigned char* bcderiv, double dt, int second_order,
                            double relax) {
  const Mesh* m = &x->m;
  int dim = m->dim, w = 2 * dim + 1;
  double* ff = x->fw[5];
  double* gc[3] = {x->cw[3], x->cw[4], x->cw[5]};
  interp(m, u_prev, ff, BC_FACE, bcval, 0);
  if (bcderiv)
    for (long f = 0; f < m->nf; ++f)
      if (bcderiv[f]) {
        int dd;
        long mi[3], cm, cp;
        fdecode(m, f, &dd, mi, &cm, &cp);
        if (cm >= 0 || cp >= 0) ff[f] = u_prev[cm >= 0 ? cm : cp];
      }
  gradient(m, ff, gc);
  double co[3];
  bdf_coeffs(dt, second_order, co);
  long c;
#pragma omp parallel for num_threads(g_threads)
  for (c = 0; c < m->nc; ++c) {
    long mi[3];
    cmidx(m, c, mi);
    if (cex(m, c)) {
      /* excluded cell: identity row, zero constant (conv_diff.hpp:222-226) */
      for (int t = 0; t < w; ++t) x->rows[c * w + t] = 0.;
      x->rows[c * w + slot_c(dim)] = 1.;
      x->rowc[c] = 0.;
      continue;
    }
    double cfl[MAXW] = {0}, dfl[MAXW] = {0};
    double cconst = 0., dconst = 0.;
    int sc = slot_c(dim);
    for (int q = 0; q < 2 * dim; ++q) {
      int d = q / 2, side = q % 2;
      double s = outward(q);
      long fq = cface(m, mi, q);
      long nb = cnb(m, mi, q);
      double Ff = Fp[fq];
      if (nb >= 0) {
        /* inner face: cm/cp and their slots */
        long cm = side ? c : nb, cp = side ? nb : c;
        int sm = side ? sc : slot_q(dim, q), sp = side ? slot_q(dim, q) : sc;
        double wm, wp, k;
        if (Ff > 1e-10) {
          wm = 1.; wp = 0.;
          k = -(gc[d][cm] * (-0.5 * m->h[d]));
        } else if (Ff < -1e-10) {
          wm = 0.; wp = 1.;
          k = -(gc[d][cp] * (0.5 * m->h[d]));
        } else {
          wm = 0.5; wp = 0.5; k = 0.;
        }
        cfl[sm] += (wm * Ff) * s;
        cfl[sp] += (wp * Ff) * s;
        cconst += (k * Ff) * s;
        /* diffusion: DerivativeInnerFacePlain (solver.hpp:284-303) */
        double al = 1. / m->h[d];
        double mA = -muf[fq];
        dfl[sm] += ((-al) * mA * m->A[d]) * s;
        dfl[sp] += ((al) * mA * m->A[d]) * s;
      } else if (bcderiv && bcderiv[fq]) {
        /* boundary with a zero-derivative condition: the face value is
           the cell's (coefficient 1), no diffusive flux */
        cfl[sc] += (1. * Ff) * s;
      } else {
        /* boundary: InterpolationBoundaryFaceNearestCell /
           DerivativeBoundaryFacePlain with a value condition */
        double val = bcval[fq];
        cconst += (val * Ff) * s;
        double factor = side ? 1. : -1.;  /* id 0 when cm is the valid cell */
        double al = 1. / (0.5 * m->h[d]) * factor;
        double mA = -muf[fq];
        dconst += ((al * val) * mA * m->A[d]) * s;
        dfl[sc] += ((-al) * mA * m->A[d]) * s;
      }
    }
    double rho = scaling ? scaling[c] : 1.;
    double a[MAXW];
    for (int t = 0; t < w; ++t) {
      double un = (t == sc) ? co[2] : 0.;
      a[t] = (cfl[t] / m->V + un) * rho + dfl[t] / m->V;
    }
    double cst = (cconst / m->V + (co[0] * u_tp[c] + co[1] * u_tc[c])) * rho +
                 dconst / m->V - src[c];
    /* delta form: constant = eqn evaluated at u_prev (sorted term order) */
    double ev = cst;
    for (int t = 0; t < w; ++t) {
      long idx;
      if (t == sc) idx = c;
      else {
        int q = t < dim ? 2 * (dim - 1 - t) : 2 * (t - dim - 1) + 1;
        idx = cnb(m, mi, q);
        if (idx < 0) { a[t] = 0.; continue; }
      }
      ev += u_prev[idx] * a[t];
    }
    a[sc] /= relax;
    for (int t = 0; t < w; ++t) x->rows[c * w + t] = a[t];
    x->rowc[c] = ev;
  }
}

static double coeff_sum(const Mesh* m, const double* rows, long c) {
  int w = 2 * m->dim + 1;
  double s = 0.;
  for (int t = 0; t < w; ++t) s += rows[c * w + t];
  return s;
}

static int linear_solve_k(oracle_ctx* x, int kind, double tol, int lim, double om, double* sol,
                          int* iters) {
  const Mesh* m = &x->m;
  switch (kind) {
    case HYDRO_LINEAR_GAUSS_SEIDEL:
      return solve_gs(m, x->rows, x->rowc, sol, tol, lim, om, iters);
    case HYDRO_LINEAR_JACOBI:
      return solve_jacobi(m, x->rows, x->rowc, sol, x->cw[23], tol, lim, om, iters);
    case HYDRO_LINEAR_LU:
      return solve_lu(m, x->rows, x->rowc, sol, iters);
  }
  return HYDRO_ERR_ARG;
}

static int linear_solve(oracle_ctx* x, int which, double* sol, int* iters) {
  const Mesh* m = &x->m;
  const hydro_desc* d = &x->d;
  int kind = which ? d->pressure_solver : d->velocity_solver;
  double tol = which ? d->pressure_tolerance : d->velocity_tolerance;
  int lim = which ? d->pressure_iters_limit : d->velocity_iters_limit;
  double om = which ? d->pressure_omega : d->velocity_omega;
  switch (kind) {
    case HYDRO_LINEAR_GAUSS_SEIDEL:
      return solve_gs(m, x->rows, x->rowc, sol, tol, lim, om, iters);
    case HYDRO_LINEAR_JACOBI:
      return solve_jacobi(m, x->rows, x->rowc, sol, x->cw[23], tol, lim, om, iters);
    case HYDRO_LINEAR_LU:
      return solve_lu(m, x->rows, x->rowc, sol, iters);
  }
  return HYDRO_ERR_ARG;
}

/* FluidSimple::MakeIteration (fluid.hpp:814-1158), SIMPLER off. */
/* UpdateOutletBaseConditions (fluid.hpp:542-600): outlet faces take the
 * velocity of their cell (the latest iterate), then a uniform normal
 * correction makes the outlet volume flux equal to the inlet flux plus the
 * volume sources; boundary faces in raw index order (std::map order). */
static void update_outlets(oracle_ctx* x) {
  const Mesh* m = &x->m;
  const hydro_desc* d = &x->d;
  int any = 0;
  for (int s = 0; s < 2 * m->dim; ++s)
    any |= d->bc_kind[s] == HYDRO_BC_OUTLET && !m->per[s / 2];
  if (!any) return;
  double** uic = x->u[HYDRO_ITER_CURR];
  double in = 0., out = 0., area = 0.;
  for (long f = 0; f < m->nf; ++f) {
    int dd;
    long mi[3], cm, cp;
    fdecode(m, f, &dd, mi, &cm, &cp);
    if (cm >= 0 && cp >= 0) continue;
    if (cm < 0 && cp < 0) continue;
    int kind = fkind(d, m, dd, mi);
    int id = cm >= 0 ? 0 : 1;
    long cc = id == 0 ? cm : cp;
    if (kind == HYDRO_BC_OUTLET) {
      double factor = id == 0 ? 1. : -1.;
      for (int k = 0; k < m->dim; ++k) x->bcu[k][f] = uic[k][cc];
      out += x->bcu[dd][f] * m->A[dd] * factor;
      area += m->A[dd];
    } else if (kind == HYDRO_BC_INLET) {
      double factor = id == 0 ? -1. : 1.;
      in += x->bcu[dd][f] * m->A[dd] * factor;
    }
  }
  for (long c = 0; c < m->nc; ++c) in += x->Sv[c] * m->V;
  double corr = (in - out) / area;
  for (long f = 0; f < m->nf; ++f) {
    int dd;
    long mi[3], cm, cp;
    fdecode(m, f, &dd, mi, &cm, &cp);
    if (cm >= 0 && cp >= 0) continue;
    if (cm < 0 && cp < 0) continue;
    if (fkind(d, m, dd, mi) != HYDRO_BC_OUTLET) continue;
    double factor = cm >= 0 ? 1. : -1.;
    x->bcu[dd][f] = x->bcu[dd][f] + corr * factor;
  }
}

int oracle_make_iteration(oracle_ctx* x) {
  const Mesh* m = &x->m;
  const hydro_desc* d = &x->d;
  int dim = m->dim, w = 2 * dim + 1;
  long nc = m->nc, nf = m->nf;
  double** uic = x->u[HYDRO_ITER_CURR];
  double** uip = x->u[HYDRO_ITER_PREV];
  double* pip = x->p[HYDRO_ITER_PREV];
  double* pic = x->p[HYDRO_ITER_CURR];
  /* layer shift (fluid.hpp:815-818) */
  memcpy(pip, pic, sizeof(double) * nc);
  memcpy(x->F[HYDRO_ITER_PREV], x->F[HYDRO_ITER_CURR], sizeof(double) * nf);
  const double* Fp = x->F[HYDRO_ITER_PREV];
  update_outlets(x);

  /* CalcExtForce (fluid.hpp:602-631) */
  double* ffext[3] = {x->fw[0], x->fw[1], x->fw[2]};
  double* fres[3] = {x->cw[6], x->cw[7], x->cw[8]};
  double* ffres[3] = {x->fw[3], x->fw[4], x->fw[6]};
  interp_vec(m, x->force, ffext, d->force_geometric_average);
  for (long c = 0; c < nc; ++c) {
    long mi[3];
    cmidx(m, c, mi);
    for (int k = 0; k < dim; ++k) {
      long flo = cface(m, mi, 2 * k), fhi = cface(m, mi, 2 * k + 1);
      double dist = 0.5 * m->h[k];
      double sum = (m->A[k] * ffext[k][flo]) * dist;
      sum += (m->A[k] * ffext[k][fhi]) * dist;
      fres[k][c] = sum / m->V;
    }
  }
  interp_vec(m, fres, ffres, d->force_geometric_average);

  /* CalcKinematicViscosity (fluid.hpp:632-641) */
  double* muf = x->fw[7];
  interp(m, x->mu, muf, BC_ZERODER, NULL, d->force_geometric_average);

  /* pressure gradient (fluid.hpp:827-832) */
  double* pf = x->fw[8];
  double* gp[3] = {x->cw[9], x->cw[10], x->cw[11]};
  interp(m, pip, pf, BC_EXTRAP, NULL, 0);
  gradient(m, pf, gp);
  /* face pressure gradient: component d only is needed on faces of dir d;
     computed on the fly below from gp (zero-derivative boundary) */

  /* explicit viscous term (fluid.hpp:835-854) */
  double* fo[3] = {x->cw[13], x->cw[14], x->cw[15]};
  for (int k = 0; k < dim; ++k)
    for (long c = 0; c < nc; ++c) fo[k][c] = 0.;
  {
    double* ff = x->fw[9];
    double* gc[3] = {x->cw[16], x->cw[17], x->cw[18]};
    for (int n = 0; n < dim; ++n) {
      interp(m, uic[n], ff, BC_FACE, x->bcu[n], 0);
      gradient(m, ff, gc);
      /* gf = Interpolate(gc, zero derivative): evaluate per face on the fly */
      for (long c = 0; c < nc; ++c) {
        long mi[3];
        cmidx(m, c, mi);
        double sum[3] = {0, 0, 0};
        for (int side = 0; side < 2; ++side) {
          int q = 2 * n + side;
          long fq = cface(m, mi, q);
          long nb = cnb(m, mi, q);
          double so = m->A[n] * outward(q);
          for (int k = 0; k < dim; ++k) {
            double g;
            if (nb >= 0) {
              long cm = side ? c : nb, cp = side ? nb : c;
              g = gc[k][cm] * (1. - 0.5) + gc[k][cp] * 0.5;
            } else {
              g = gc[k][c];
            }
            sum[k] += g * (muf[fq] * so);
          }
        }
        for (int k = 0; k < dim; ++k) fo[k][c] += sum[k] / m->V;
      }
    }
  }
  /* append to force (fluid.hpp:857-870) */
  for (long c = 0; c < nc; ++c)
    for (int k = 0; k < dim; ++k)
      fo[k][c] += ((gp[k][c] * (-1.) + fres[k][c]) + x->stforce[k][c]) +
                  uic[k][c] * (x->rho[c] * x->Sv[c] - x->Sm[c]);

  /* momentum: d scalar solves (fluid.hpp:157-165, conv_diff.hpp:130-251) */
  double* Dsum = x->cw[19];
  for (long c = 0; c < nc; ++c) Dsum[c] = 0.;
  x->cd_iter_count++;
  for (int n = 0; n < dim; ++n) {
    memcpy(uip[n], uic[n], sizeof(double) * nc);
    assemble_momentum(x, n, uip[n], x->u[HYDRO_TIME_CURR][n],
                      x->u[HYDRO_TIME_PREV][n], Fp, muf, fo[n]);
    for (long c = 0; c < nc; ++c) Dsum[c] += coeff_sum(m, x->rows, c);
    memcpy(x->mrows[n], x->rows, sizeof(double) * nc * w);
    memcpy(x->mrowc[n], x->rowc, sizeof(double) * nc);
    int it = 0;
    int st = linear_solve(x, 0, x->cw[20], &it);
    x->vel_sweeps += it;
    if (st != HYDRO_OK && st != HYDRO_NOT_CONVERGED) return st;
    for (long c = 0; c < nc; ++c) uic[n][c] = uip[n][c] + x->cw[20][c];
  }
  /* diag coefficient (fluid.hpp:876-887) */
  double* Dc = x->Dc;
  for (long c = 0; c < nc; ++c) Dc[c] = Dsum[c] / dim;
  double* Df = x->fw[9];
  interp(m, Dc, Df, BC_NONE, NULL, 0);

  /* Rhie-Chow (fluid.hpp:889-942) */
  double* Fs = x->fw[5];   /* F* */
  double* kf = x->fw[1];   /* -c_f = A/(h D_f) on inner faces, 0 elsewhere */
  {
    long f;
    for (f = 0; f < nf; ++f) {
      int dd;
      long mi[3], cm, cp;
      fdecode(m, f, &dd, mi, &cm, &cp);
      int side = fside(m, dd, mi);
      double uf;
      if (cm >= 0 && cp >= 0) uf = uic[dd][cm] * (1. - 0.5) + uic[dd][cp] * 0.5;
      else uf = x->bcu[dd][f];
      (void)side;
      double vfi = uf * m->A[dd];
      if (cm >= 0 && cp >= 0) {
        double gpf_ = gp[dd][cm] * (1. - 0.5) + gp[dd][cp] * 0.5;
        double wide = (gpf_ - ffres[dd][f]) * m->A[dd];
        double compact = (pip[cp] - pip[cm]) / m->h[dd] * m->A[dd] -
                         ffext[dd][f] * m->A[dd];
        Fs[f] = vfi + d->rhie_chow_factor * (wide - compact) / Df[f] + 0;
        kf[f] = m->A[dd] / (m->h[dd] * Df[f]);
      } else {
        Fs[f] = vfi;
        kf[f] = 0.;
      }
      Fs[f] -= d->meshvel[dd] * m->A[dd];
    }
  }

  /* pressure-correction system (fluid.hpp:972-1014); excluded cells:
   * identity rows with zero constant */
  for (long c = 0; c < nc; ++c) {
    long mi[3];
    cmidx(m, c, mi);
    if (cex(m, c)) {
      for (int t = 0; t < w; ++t) x->rows[c * w + t] = 0.;
      x->rows[c * w + slot_c(dim)] = 1.;
      x->rowc[c] = 0.;
      continue;
    }
    double a[MAXW] = {0};
    double cst = 0.;
    int sc = slot_c(dim);
    for (int q = 0; q < 2 * dim; ++q) {
      double s = outward(q);
      long fq = cface(m, mi, q);
      long nb = cnb(m, mi, q);
      if (nb >= 0) {
        double cf = -kf[fq];
        int side = q % 2;
        int sm = side ? sc : slot_q(dim, q), sp = side ? slot_q(dim, q) : sc;
        a[sm] += (-cf) * s;
        a[sp] += cf * s;
      }
      cst += Fs[fq] * s;
    }
    cst += -(x->Sv[c] * m->V);
    for (int t = 0; t < w; ++t) x->rows[c * w + t] = a[t];
    x->rowc[c] = cst;
  }
  long pin = d->pressure_fixed_cell;
  if (pin >= 0 && pin < nc) {
    double val = d->pressure_fixed_value;
    long mi[3];
    cmidx(m, pin, mi);
    for (int q = 0; q < 2 * dim; ++q) {
      long nb = cnb(m, mi, q);
      if (nb < 0) continue;
      long nmi[3];
      cmidx(m, nb, nmi);
      int t = slot_q(dim, q ^ 1);  /* term of pin in row nb */
      x->rowc[nb] += val * x->rows[nb * w + t];
      x->rows[nb * w + t] = 0.;
    }
    for (int t = 0; t < w; ++t) x->rows[pin * w + t] = 0.;
    x->rows[pin * w + slot_c(dim)] = 1.;
    x->rowc[pin] = -val;
  }

  /* pressure solve (fluid.hpp:1029-1031) */
  double* pc = x->pcorr;
  int it = 0;
  int st;
  /* the multigrid-preconditioned CG of the GPU converges to the same
     solution; the oracle uses plain CG for it */
  if (d->pressure_solver == HYDRO_LINEAR_CG || d->pressure_solver == HYDRO_LINEAR_MGCG) {
    double* f = x->cw[21];
    for (long c = 0; c < nc; ++c) f[c] = -x->rowc[c];
    if (pin >= 0) {
      /* rows already substituted; the CG path uses the face form */
      f[pin] = d->pressure_fixed_value;
    }
    double* wk[5] = {x->cw[0], x->cw[1], x->cw[2], x->cw[3], x->cw[4]};
    double res = 0.;
    st = pcg(m, kf, 0., pin, f, pc, 0, d->pressure_tolerance,
             d->pressure_iters_limit, wk, &it, &res);
    x->p_res = res;
  } else {
    st = linear_solve(x, 1, pc, &it);
  }
  x->p_iters += it;
  if (st != HYDRO_OK && st != HYDRO_NOT_CONVERGED) return st;

  /* correction (fluid.hpp:1033-1057) */
  for (long c = 0; c < nc; ++c) pic[c] = pip[c] + d->pressure_relaxation_factor * pc[c];
  interp(m, pc, pf, BC_EXTRAP, NULL, 0);
  gradient(m, pf, gp);
  for (int k = 0; k < dim; ++k)
    for (long c = 0; c < nc; ++c) uic[k][c] += gp[k][c] / (-Dc[c]);
  double* Fic = x->F[HYDRO_ITER_CURR];
  for (long f = 0; f < nf; ++f) {
    int dd;
    long mi[3], cm, cp;
    fdecode(m, f, &dd, mi, &cm, &cp);
    double v = Fs[f];
    if (cm >= 0 && cp >= 0) {
      double cf = -kf[f];
      v += pc[cm] * (-cf);
      v += pc[cp] * cf;
    }
    Fic[f] = v;
  }

  /* SIMPLER (fluid.hpp:1059-1155): the momentum equations evaluated at the
   * correction of this iteration, plus restored force and minus the
   * iteration's pressure gradient, give face terms whose divergence is the
   * constant of the pressure system (same matrix); solved in delta form
   * around the corrected pressure, which is then replaced. */
  if (d->simpler) {
    double* gp0[3] = {x->cw[16], x->cw[17], x->cw[18]};
    interp(m, pip, pf, BC_EXTRAP, NULL, 0);
    gradient(m, pf, gp0);
    double* ev[3] = {x->cw[13], x->cw[14], x->cw[15]};
    for (int n = 0; n < dim; ++n) {
      for (long c = 0; c < nc; ++c) {
        long mi[3];
        cmidx(m, c, mi);
        double r = x->mrowc[n][c];
        for (int t = 0; t < w; ++t) {
          long idx;
          if (t == slot_c(dim)) idx = c;
          else {
            int q = t < dim ? 2 * (dim - 1 - t) : 2 * (t - dim - 1) + 1;
            idx = cnb(m, mi, q);
            if (idx < 0) continue;
          }
          r += (uic[n][idx] - uip[n][idx]) * x->mrows[n][c * w + t];
        }
        ev[n][c] = r + (fres[n][c] - gp0[n][c]);
      }
    }
    /* face scratch: kf (fw[1]) and D_f (fw[9]) are still needed */
    double* ffx[3] = {x->fw[3], x->fw[4], x->fw[6]};
    double* fev[3] = {x->fw[0], x->fw[2], x->fw[5]};
    double* fvel = x->fw[7];
    double* rf = x->fw[8];
    interp_vec(m, x->force, ffx, d->force_geometric_average);
    for (int n = 0; n < dim; ++n) interp(m, ev[n], fev[n], BC_NONE, NULL, 0);
    for (long f = 0; f < nf; ++f) rf[f] = 0.;
    for (int n = 0; n < dim; ++n) {
      interp(m, uic[n], fvel, BC_FACE, x->bcu[n], 0);
      long f0 = m->fofs[n], f1 = f0 + m->fcnt[n];
      for (long f = f0; f < f1; ++f) {
        int dd;
        long mi[3], cm, cp;
        fdecode(m, f, &dd, mi, &cm, &cp);
        if (cm < 0 || cp < 0) continue;
        double e = fev[dd][f] - ffx[dd][f];
        rf[f] = e * m->A[dd] / Df[f] + (Fic[f] - fvel[f] * m->A[dd]) / d->rhie_chow_factor;
      }
    }
    for (long c = 0; c < nc; ++c) {
      long mi[3];
      cmidx(m, c, mi);
      double sum = 0.;
      for (int q = 0; q < 2 * dim; ++q) sum += rf[cface(m, mi, q)] * outward(q);
      x->rowc[c] = -sum;
    }
    if (pin >= 0 && pin < nc) x->rowc[pin] = -d->pressure_fixed_value;
    /* constant = equation evaluated at the corrected pressure */
    for (long c = 0; c < nc; ++c) {
      long mi[3];
      cmidx(m, c, mi);
      double r = x->rowc[c];
      for (int t = 0; t < w; ++t) {
        long idx;
        if (t == slot_c(dim)) idx = c;
        else {
          int q = t < dim ? 2 * (dim - 1 - t) : 2 * (t - dim - 1) + 1;
          idx = cnb(m, mi, q);
          if (idx < 0) continue;
        }
        r += pic[idx] * x->rows[c * w + t];
      }
      x->cw[12][c] = r;
    }
    memcpy(x->rowc, x->cw[12], sizeof(double) * nc);
    double* xs = x->cw[22];
    it = 0;
    if (d->pressure_solver == HYDRO_LINEAR_CG || d->pressure_solver == HYDRO_LINEAR_MGCG) {
      double* f = x->cw[21];
      for (long c = 0; c < nc; ++c) f[c] = -x->rowc[c];
      double* wk[5] = {x->cw[0], x->cw[1], x->cw[2], x->cw[3], x->cw[4]};
      double res = 0.;
      st = pcg(m, kf, 0., pin, f, xs, 0, d->pressure_tolerance, d->pressure_iters_limit, wk,
               &it, &res);
      x->p_res = res;
    } else {
      for (long c = 0; c < nc; ++c) xs[c] = 0.;
      st = linear_solve(x, 1, xs, &it);
    }
    x->p_iters += it;
    if (st != HYDRO_OK && st != HYDRO_NOT_CONVERGED) return st;
    for (long c = 0; c < nc; ++c) pic[c] += xs[c];
  }
  x->iter_count++;
  return HYDRO_OK;
}

int oracle_get_convergence_indicator(oracle_ctx* x, double* out) {
  if (x->cd_iter_count == 0) {
    *out = 1.;
    return HYDRO_OK;
  }
  const Mesh* m = &x->m;
  double res = 0.;
  for (long c = 0; c < m->nc; ++c) {
    double s = 0.;
    for (int k = 0; k < m->dim; ++k) {
      double dv = x->u[HYDRO_ITER_CURR][k][c] - x->u[HYDRO_ITER_PREV][k][c];
      s += dv * dv;
    }
    double dist = sqrt(s);
    if (dist > res) res = dist;
  }
  *out = res;
  return HYDRO_OK;
}

int oracle_get_iteration_count(oracle_ctx* x, int* out) {
  *out = x->iter_count;
  return HYDRO_OK;
}

int oracle_is_converged(oracle_ctx* x, int* out) {
  double ind;
  oracle_get_convergence_indicator(x, &ind);
  *out = (x->iter_count >= x->d.num_iterations_limit) ||
         (ind < x->d.convergence_tolerance);
  return HYDRO_OK;
}

int oracle_finish_step(oracle_ctx* x) {
  const Mesh* m = &x->m;
  memcpy(x->p[HYDRO_TIME_PREV], x->p[HYDRO_TIME_CURR], sizeof(double) * m->nc);
  memcpy(x->F[HYDRO_TIME_PREV], x->F[HYDRO_TIME_CURR], sizeof(double) * m->nf);
  memcpy(x->p[HYDRO_TIME_CURR], x->p[HYDRO_ITER_CURR], sizeof(double) * m->nc);
  memcpy(x->F[HYDRO_TIME_CURR], x->F[HYDRO_ITER_CURR], sizeof(double) * m->nf);
  for (long c = 0; c < m->nc; ++c)
    if (isnan(x->p[HYDRO_TIME_CURR][c])) return HYDRO_ERR_NAN;
  for (int k = 0; k < m->dim; ++k) {
    memcpy(x->u[HYDRO_TIME_PREV][k], x->u[HYDRO_TIME_CURR][k], sizeof(double) * m->nc);
    memcpy(x->u[HYDRO_TIME_CURR][k], x->u[HYDRO_ITER_CURR][k], sizeof(double) * m->nc);
  }
  x->time += x->dt;
  return HYDRO_OK;
}

/* FluidSimple::GetAutoTimeStep (fluid.hpp:1191-1206). */
int oracle_get_auto_time_step(oracle_ctx* x, double* out) {
  const Mesh* m = &x->m;
  double dt = 1e10;
  const double* F = x->F[HYDRO_TIME_CURR];
  for (long c = 0; c < m->nc; ++c) {
    if (cex(m, c)) continue;  /* fluid.hpp:1195 */
    long mi[3];
    cmidx(m, c, mi);
    for (int q = 0; q < 2 * m->dim; ++q) {
      double fl = F[cface(m, mi, q)];
      if (fl != 0.) {
        double v = fabs(m->V / fl);
        if (v < dt) dt = v;
      }
    }
  }
  *out = dt;
  return HYDRO_OK;
}

int oracle_set_time_step(oracle_ctx* x, double dt, double dta) {
  x->dt = dt;
  x->adv_dt = dta;
  return HYDRO_OK;
}

int oracle_get_time(oracle_ctx* x, double* ft, double* at) {
  if (ft) *ft = x->time;
  if (at) *at = x->adv_time;
  return HYDRO_OK;
}

/* ---------------------------------------------------------- advection -- */

static double superbee(double p, double q) {
  if (p > 0. && q > 0.) {
    double a = fmin(2 * p, q), b = fmin(p, 2 * q);
    return a > b ? a : b;
  } else if (p < 0. && q < 0.) {
    double a = fmin(-2 * p, -q), b = fmin(-p, -2 * q);
    return -(a > b ? a : b);
  }
  return 0.;
}

/* One AdvectionSolverMultiExplicit::MakeIteration (advection.hpp:440-539)
 * including StartStep/FinishStep, all phases.  Boundary condition of every
 * partial density: zero derivative on walls (hydro2d.hpp:576-590). */
static void advection_iteration(oracle_ctx* x) {
  const Mesh* m = &x->m;
  const hydro_desc* d = &x->d;
  int dim = m->dim;
  const double* F = x->F[HYDRO_ITER_CURR];
  double dt = x->adv_dt;
  double* qf = x->fw[6];
  double* ff = x->fw[7];
  double* gc[3] = {x->cw[0], x->cw[1], x->cw[2]};
  for (int i = 0; i < x->nph; ++i) {
    double* cur = x->q[i];
    int nst = d->tvd_split ? dim : 1;
    for (int stage = 0; stage < nst; ++stage) {
      /* advection conditions (hydro2d.hpp:566-582): inlet faces hold the
       * inlet value, the others zero derivative */
      interp(m, cur, ff, BC_ZERODER, NULL, 0);
      for (long f = 0; f < m->nf; ++f) {
        int dd;
        long mi[3], P, E;
        fdecode(m, f, &dd, mi, &P, &E);
        if (P >= 0 && E >= 0) continue;
        if (P < 0 && E < 0) continue;
        if (fkind(d, m, dd, mi) == HYDRO_BC_INLET) ff[f] = x->qin[i][f];
      }
      gradient(m, ff, gc);
      /* InterpolateSuperbee (solver.hpp:560-619) */
      for (long f = 0; f < m->nf; ++f) {
        int dd;
        long mi[3], P, E;
        fdecode(m, f, &dd, mi, &P, &E);
        if (P >= 0 && E >= 0) {
          double hv = 0.5 * m->h[dd];
          if (F[f] > 1e-8) {
            qf[f] = cur[P] + 0.5 * superbee(cur[E] - cur[P],
                                            -4. * (gc[dd][P] * (-hv)) - (cur[E] - cur[P]));
          } else if (F[f] < -1e-8) {
            qf[f] = cur[E] - 0.5 * superbee(cur[E] - cur[P],
                                            4. * (gc[dd][E] * hv) - (cur[E] - cur[P]));
          } else {
            qf[f] = 0.5 * (cur[P] + cur[E]);
          }
        } else if (P < 0 && E < 0) {
          qf[f] = 0.;  /* excluded face: no condition */
        } else if (fkind(d, m, dd, mi) == HYDRO_BC_INLET) {
          qf[f] = x->qin[i][f];
        } else {
          qf[f] = cur[P >= 0 ? P : E] + 0. * (0.5 * m->h[dd]);
        }
      }
      long c;
#pragma omp parallel for num_threads(g_threads)
      for (c = 0; c < m->nc; ++c) {
        long mi[3];
        cmidx(m, c, mi);
        double sum = 0.;
        for (int q = 0; q < 2 * dim; ++q) {
          if ((q / 2) % nst != stage) continue;
          long fq = cface(m, mi, q);
          sum += qf[fq] * F[fq] * outward(q);
        }
        cur[c] += -dt / m->V * sum;
      }
    }
    /* interface sharpening (advection.hpp:481-530) */
    double* shf = x->fw[8];
    for (long f = 0; f < m->nf; ++f) shf[f] = 0.;
    if (fabs(d->sharp) > 1e-10) {
      double* gf[3] = {x->fw[2], x->fw[3], x->fw[4]};
      interp(m, cur, ff, BC_ZERODER, NULL, 0);
      gradient(m, ff, gc);
      for (int k = 0; k < dim; ++k) interp(m, gc[k], gf[k], BC_ZERODER, NULL, 0);
      for (long f = 0; f < m->nf; ++f) {
        int dd;
        long mi[3], cm, cp;
        fdecode(m, f, &dd, mi, &cm, &cp);
        double nv[3] = {0, 0, 0}, n2 = 0.;
        for (int k = 0; k < dim; ++k) {
          nv[k] = gf[k][f];
          n2 += nv[k] * nv[k];
        }
        double nn = sqrt(n2);
        if (nn < 1.) continue;
        for (int k = 0; k < dim; ++k) nv[k] /= (nn + 1e-6);
        double nf_ = nv[dd];
        double uf = F[f];
        double am = d->density[i];
        double epsh = d->sharp * m->A[dd];
        shf[f] = fabs(uf * nf_) * nf_ * (epsh * nn - ff[f] * (1. - ff[f] / am));
      }
    }
    long c;
    for (c = 0; c < m->nc; ++c) {
      long mi[3];
      cmidx(m, c, mi);
      cur[c] += dt * 0.;  /* mass source of the phase: zero */
      double sh = 0.;
      for (int q = 0; q < 2 * dim; ++q) sh += outward(q) * shf[cface(m, mi, q)];
      cur[c] += dt * sh / m->V;
    }
  }
}

/* hydro2d.hpp:1596-1604: substeps until advection time reaches fluid time. */
int oracle_advection_substep(oracle_ctx* x) {
  advection_iteration(x);
  x->adv_time += x->adv_dt;
  return HYDRO_OK;
}

int oracle_advection_step(oracle_ctx* x, int* substeps) {
  int ns = 0;
  while (x->adv_time < x->time - 0.5 * x->adv_dt) {
    advection_iteration(x);
    x->adv_time += x->adv_dt;
    ++ns;
  }
  if (substeps) *substeps = ns;
  return HYDRO_OK;
}

/* hydro<Mesh>::step (hydro2d.hpp:1531-1621) without output. */
int oracle_step(oracle_ctx* x, hydro_step_stats* st) {
  const hydro_desc* d = &x->d;
  hydro_step_stats s;
  memset(&s, 0, sizeof(s));
  if (d->dt_auto) {
    double dtm;
    oracle_get_auto_time_step(x, &dtm);
    double dt = dtm * d->cfl, dta = dtm * d->cfl_advection;
    if (d->dt_max > 0. && dt > d->dt_max) {
      dta = dta * (d->dt_max / dt);
      dt = d->dt_max;
    }
    oracle_set_time_step(x, dt, dta);
  }
  int rc = oracle_start_step(x);
  if (rc) return rc;
  for (;;) {
    int conv;
    oracle_is_converged(x, &conv);
    if (conv) break;
    rc = oracle_make_iteration(x);
    if (rc) return rc;
  }
  oracle_get_convergence_indicator(x, &s.convergence_indicator);
  s.outer_iterations = x->iter_count;
  s.velocity_sweeps = x->vel_sweeps;
  s.pressure_iterations = x->p_iters;
  s.pressure_residual = x->p_res;
  rc = oracle_finish_step(x);
  if (rc) return rc;
  if (d->advection_enable) oracle_advection_step(x, &s.advection_substeps);
  /* heat after advection (hydro2d.hpp:1607-1613) */
  if (x->heat_on) {
    int hr = oracle_heat_step(x);
    if (hr) return hr;
  }
  oracle_update_properties(x);
  s.dt = x->dt;
  s.dt_advection = x->adv_dt;
  s.time = x->time;
  s.status = HYDRO_OK;
  if (st) *st = s;
  return HYDRO_OK;
}

/* hydro<Mesh>::CalcStat (hydro2d.hpp:1432-1493), plus sum q V. */
int oracle_calc_stat(oracle_ctx* x, hydro_stat* out) {
  const Mesh* m = &x->m;
  memset(out, 0, sizeof(*out));
  for (int i = 0; i < x->nph; ++i) {
    double vol = 0., pmin = 1e10, pmax = -1e10, pm = 0.;
    double cen[3] = {0, 0, 0}, vel[3] = {0, 0, 0};
    for (long c = 0; c < m->nc; ++c) {
      long mi[3];
      cmidx(m, c, mi);
      double a = x->alpha[i][c];
      vol += a * m->V;
      double pd = x->q[i][c];
      if (pd < pmin) pmin = pd;
      if (pd > pmax) pmax = pd;
      pm += pd * m->V;
      for (int k = 0; k < m->dim; ++k) {
        double xc = m->lo[k] + (mi[k] + 0.5) * m->h[k];
        cen[k] += xc * (a * m->V);
        vel[k] += x->u[HYDRO_TIME_CURR][k][c] * (a * m->V);
      }
    }
    out->volume[i] = vol;
    out->mass[i] = vol * x->d.density[i];
    out->pd_min[i] = pmin;
    out->pd_max[i] = pmax;
    out->partial_mass[i] = pm;
    for (int k = 0; k < m->dim; ++k) {
      out->center[i][k] = cen[k] / vol;
      out->velocity[i][k] = vel[k] / vol;
    }
    /* boundary volume fluxes of the phase (hydro2d.hpp:1474-1493): flux
     * towards the valid neighbour (+F on a low face, -F on a high face)
     * times its volume fraction, split by sign */
    double fin = 0., fout = 0.;
    for (int d = 0; d < m->dim; ++d) {
      long nn[3] = {m->n[0], m->n[1], m->n[2]};
      for (long k = 0; k < nn[2]; ++k)
        for (long j = 0; j < nn[1]; ++j)
          for (long ii = 0; ii < nn[0]; ++ii) {
            long mi[3] = {ii, j, k};
            long c = ii + nn[0] * (j + nn[1] * k);
            for (int side = 0; side < 2; ++side) {
              if (side ? mi[d] != nn[d] - 1 : mi[d] != 0) continue;
              long fm[3] = {ii, j, k};
              if (side) fm[d] += 1;
              double ftc = x->F[HYDRO_TIME_CURR][fidx(m, d, fm[0], fm[1], fm[2])];
              if (side) ftc = -ftc;
              if (ftc >= 0.) fin += ftc * x->alpha[i][c];
              else fout -= ftc * x->alpha[i][c];
            }
          }
    }
    out->volume_flux_in[i] = fin;
    out->volume_flux_out[i] = fout;
  }
  return HYDRO_OK;
}


/* ---------------------------------------------------------------- heat -- */

/* hydro<Mesh>::InitHeatSolver (hydro2d.hpp:650-687): temperature layers,
 * boundary faces in the box hold its temperature, the others zero
 * derivative (Rect::IsInside is inclusive, vect.hpp:239-246). */
int oracle_heat_create(oracle_ctx* x, const hydro_heat_desc* hd) {
  if (!x || !hd) return HYDRO_ERR_ARG;
  const Mesh* m = &x->m;
  x->hd = *hd;
  for (int l = 0; l < 4; ++l) {
    if (!x->T[l]) x->T[l] = alloc0(m->nc);
    for (long c = 0; c < m->nc; ++c) x->T[l][c] = hd->temperature_initial;
  }
  if (!x->kc) x->kc = alloc0(m->nc);
  if (!x->tbval) x->tbval = alloc0(m->nf);
  if (!x->tbder) x->tbder = (unsigned char*)calloc((size_t)m->nf, 1);
  for (long f = 0; f < m->nf; ++f) {
    int d;
    long mi[3], cm, cp;
    fdecode(m, f, &d, mi, &cm, &cp);
    x->tbder[f] = 0;
    if (cm >= 0 && cp >= 0) continue;
    double xc[3] = {0, 0, 0};
    for (int k = 0; k < m->dim; ++k)
      xc[k] = k == d ? m->lo[k] + mi[k] * m->h[k] : m->lo[k] + (mi[k] + 0.5) * m->h[k];
    int in = 1;
    for (int k = 0; k < m->dim; ++k)
      if (xc[k] < hd->box_lo[k] || hd->box_hi[k] < xc[k]) in = 0;
    if (in) x->tbval[f] = hd->box_temperature;
    else x->tbder[f] = 1;
  }
  x->heat_on = 1;
  /* mixture conductivity from the current volume fractions */
  for (long c = 0; c < m->nc; ++c) {
    double s = 0.;
    for (int i = 0; i < x->nph; ++i) s += hd->conductivity[i] * x->alpha[i][c];
    x->kc[c] = s;
  }
  return HYDRO_OK;
}

int oracle_heat_get_temperature(oracle_ctx* x, double* out, size_t n) {
  if (!x || !x->heat_on || !out || (long)n != x->m.nc) return HYDRO_ERR_ARG;
  memcpy(out, x->T[HYDRO_TIME_CURR], sizeof(double) * n);
  return HYDRO_OK;
}

/* HeatSolver StartStep, one MakeIteration (ConvectionDiffusionScalarImplicit,
 * conv_diff.hpp:130-251, unit scaling, conductivity as diffusion rate,
 * the fluid's iter_curr fluxes), FinishStep. */
int oracle_heat_step(oracle_ctx* x) {
  if (!x || !x->heat_on) return HYDRO_ERR_ARG;
  const Mesh* m = &x->m;
  long nc = m->nc;
  double** T = x->T;
  memcpy(T[HYDRO_ITER_CURR], T[HYDRO_TIME_CURR], sizeof(double) * nc);
  memcpy(T[HYDRO_ITER_PREV], T[HYDRO_ITER_CURR], sizeof(double) * nc);
  double* kf = x->fw[0];
  interp(m, x->kc, kf, BC_ZERODER, NULL, 0);
  double* src = x->cw[22];
  for (long c = 0; c < nc; ++c) src[c] = 0.;
  assemble_scalar(x, T[HYDRO_ITER_PREV], T[HYDRO_TIME_CURR], T[HYDRO_TIME_PREV],
                  x->F[HYDRO_ITER_CURR], kf, src, NULL, x->tbval, x->tbder, x->hd.dt,
                  x->hd.time_second_order, x->hd.relaxation_factor);
  double* corr = x->cw[20];
  for (long c = 0; c < nc; ++c) corr[c] = 0.;
  int it = 0;
  int st = linear_solve_k(x, x->hd.solver, x->hd.tolerance, x->hd.iters_limit, 1., corr, &it);
  if (st != HYDRO_OK && st != HYDRO_NOT_CONVERGED) return st;
  for (long c = 0; c < nc; ++c) T[HYDRO_ITER_CURR][c] = T[HYDRO_ITER_PREV][c] + corr[c];
  memcpy(T[HYDRO_TIME_PREV], T[HYDRO_TIME_CURR], sizeof(double) * nc);
  memcpy(T[HYDRO_TIME_CURR], T[HYDRO_ITER_CURR], sizeof(double) * nc);
  return HYDRO_OK;
}
