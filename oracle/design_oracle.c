/*
 * design_oracle.c -- CPU restatement of the design-update chain of the
 * reference's optimisation loop (test infrastructure only: the oracle the
 * GPU design update is compared with).
 *
 *   density filter   topOpt/densityFilter2d.cc:33-146, densityFilter3d.cc:60-139
 *   projection       topOpt/projectionFilter2d.cc:27-88 (tanh projection, beta, eta)
 *   double filter    topOpt/doubleProjectionFilter2d.cc (two filter+projection stages)
 *   volume           functionals/volumeConstraint.cc (ConstrainFluid / ConstrainMaterial)
 *   MMA              Svanberg (1987), method of moving asymptotes, with the
 *                    subproblem of the reference's topOpt/MMA.cc (GenSub: asymptote
 *                    rules, bounds and the p/q coefficients; y and z penalties of
 *                    XYZofLAMBDA) and a primal-dual Newton method on its dual.
 *
 * Parity of the MMA is pinned by running the reference's own MMA.cc (compiled
 * in oracle/_ref against the project's shim) on the same problems.  All
 * arithmetic is FP64.
 */
#include "design_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------ */
/* Filters                                                              */

static int in_box(const int* b, int x, int y, int z) {
  return x >= b[0] && x <= b[1] && y >= b[2] && y <= b[3] && z >= b[4] && z <= b[5];
}

/* Cone weight R - |d| for |d| <= R (zero at |d| = R). */
static double cone(int dx, int dy, int dz, int R, int* inside) {
  double d = sqrt((double)(dx * dx + dy * dy + dz * dz));
  *inside = d <= (double)R;
  return (double)R - d;
}

/* Row sums of the filter matrix: rows in the box carry the cone weights of
 * their neighbours inside the grid, other rows are identity rows. */
static void filter_denominator(const dsg_stage* st, int nx, int ny, int nz, double* den) {
  const int R = st->radius, R3 = nz > 1 ? R : 0;
  for (int z = 0; z < nz; ++z)
    for (int y = 0; y < ny; ++y)
      for (int x = 0; x < nx; ++x) {
        long long c = ((long long)z * ny + y) * nx + x;
        if (!in_box(st->box, x, y, z)) {
          den[c] = 1.;
          continue;
        }
        double s = 0.;
        for (int dz = -R3; dz <= R3; ++dz)
          for (int dy = -R; dy <= R; ++dy)
            for (int dx = -R; dx <= R; ++dx) {
              int xx = x + dx, yy = y + dy, zz = z + dz, ok;
              if (xx < 0 || yy < 0 || zz < 0 || xx >= nx || yy >= ny || zz >= nz) continue;
              double w = cone(dx, dy, dz, R, &ok);
              if (ok) s += w;
            }
        den[c] = s;
      }
}

static double proj_den(const dsg_stage* st) {
  return tanh(st->beta * st->eta) + tanh(st->beta * (1. - st->eta));
}

/* out = filter (then projection) of in, one stage; keep = the filtered field */
static void stage_forward(const dsg_stage* st, int nx, int ny, int nz, const double* in,
                          double* keep, double* out) {
  const int R = st->radius, R3 = nz > 1 ? R : 0;
  long long n = (long long)nx * ny * nz;
  double* den = (double*)malloc(sizeof(double) * n);
  filter_denominator(st, nx, ny, nz, den);
  for (int z = 0; z < nz; ++z)
    for (int y = 0; y < ny; ++y)
      for (int x = 0; x < nx; ++x) {
        long long c = ((long long)z * ny + y) * nx + x;
        double v;
        if (!in_box(st->box, x, y, z)) {
          v = in[c];
        } else {
          double s = 0.;
          for (int dz = -R3; dz <= R3; ++dz)
            for (int dy = -R; dy <= R; ++dy)
              for (int dx = -R; dx <= R; ++dx) {
                int xx = x + dx, yy = y + dy, zz = z + dz, ok;
                if (xx < 0 || yy < 0 || zz < 0 || xx >= nx || yy >= ny || zz >= nz) continue;
                double w = cone(dx, dy, dz, R, &ok);
                if (ok) s += w * in[((long long)zz * ny + yy) * nx + xx];
              }
          v = s / den[c];
        }
        keep[c] = v;
        if (st->project && in_box(st->box, x, y, z))
          v = (tanh(st->beta * st->eta) + tanh(st->beta * (v - st->eta))) / proj_den(st);
        out[c] = v;
      }
  free(den);
}

/* s <- chain rule of one stage at its filtered field `kept` (in place) */
static void stage_transpose(const dsg_stage* st, int nx, int ny, int nz, const double* kept,
                            double* s) {
  const int R = st->radius, R3 = nz > 1 ? R : 0;
  long long n = (long long)nx * ny * nz;
  double* den = (double*)malloc(sizeof(double) * n);
  double* t = (double*)malloc(sizeof(double) * n);
  filter_denominator(st, nx, ny, nz, den);
  for (int z = 0; z < nz; ++z)
    for (int y = 0; y < ny; ++y)
      for (int x = 0; x < nx; ++x) {
        long long c = ((long long)z * ny + y) * nx + x;
        double v = s[c];
        if (st->project && in_box(st->box, x, y, z)) {
          double th = tanh(st->beta * (kept[c] - st->eta));
          v *= (1. - th * th) * st->beta / proj_den(st);
        }
        t[c] = v / den[c];
      }
  /* s = H^T t: column c gathers the rows that hold it */
  for (int z = 0; z < nz; ++z)
    for (int y = 0; y < ny; ++y)
      for (int x = 0; x < nx; ++x) {
        long long c = ((long long)z * ny + y) * nx + x;
        double acc = in_box(st->box, x, y, z) ? 0. : t[c];
        for (int dz = -R3; dz <= R3; ++dz)
          for (int dy = -R; dy <= R; ++dy)
            for (int dx = -R; dx <= R; ++dx) {
              int xx = x + dx, yy = y + dy, zz = z + dz, ok;
              if (xx < 0 || yy < 0 || zz < 0 || xx >= nx || yy >= ny || zz >= nz) continue;
              if (!in_box(st->box, xx, yy, zz)) continue;
              double w = cone(dx, dy, dz, R, &ok);
              if (ok) acc += w * t[((long long)zz * ny + yy) * nx + xx];
            }
        s[c] = acc;
      }
  free(den);
  free(t);
}

int dsg_filter_forward(const dsg_chain* ch, const double* xfull, double* gamma) {
  long long n = (long long)ch->nx * ch->ny * ch->nz;
  double* a = (double*)malloc(sizeof(double) * n);
  double* keep = (double*)malloc(sizeof(double) * n);
  if (!a || !keep) return -4;
  memcpy(a, xfull, sizeof(double) * n);
  for (int k = 0; k < ch->nstages; ++k) {
    stage_forward(&ch->stage[k], ch->nx, ch->ny, ch->nz, a, keep, gamma);
    memcpy(a, gamma, sizeof(double) * n);
  }
  if (ch->nstages == 0) memcpy(gamma, xfull, sizeof(double) * n);
  free(a);
  free(keep);
  return 0;
}

int dsg_filter_transpose(const dsg_chain* ch, const double* xfull, double* s) {
  long long n = (long long)ch->nx * ch->ny * ch->nz;
  if (ch->nstages == 0) return 0;
  /* the filtered field of every stage, from the forward pass */
  double* kept = (double*)malloc(sizeof(double) * n * ch->nstages);
  double* a = (double*)malloc(sizeof(double) * n);
  double* b = (double*)malloc(sizeof(double) * n);
  if (!kept || !a || !b) return -4;
  memcpy(a, xfull, sizeof(double) * n);
  for (int k = 0; k < ch->nstages; ++k) {
    stage_forward(&ch->stage[k], ch->nx, ch->ny, ch->nz, a, kept + (size_t)k * n, b);
    memcpy(a, b, sizeof(double) * n);
  }
  for (int k = ch->nstages - 1; k >= 0; --k)
    stage_transpose(&ch->stage[k], ch->nx, ch->ny, ch->nz, kept + (size_t)k * n, s);
  free(kept);
  free(a);
  free(b);
  return 0;
}

/* ------------------------------------------------------------------ */
/* MMA                                                                  */

struct dsg_mma {
  int n, m, k;
  double asyminit, asymdec, asyminc;
  double *a, *c;                                /* m */
  double *x1, *x2, *L, *U, *al, *be, *p0, *q0;  /* n */
  double *P, *Q;                                /* m x n */
  double *b, *lam, *mu, *y;                     /* m */
  double z;
};

dsg_mma* dsg_mma_create(int n, int m, const double* x0, const double* a) {
  dsg_mma* s = (dsg_mma*)calloc(1, sizeof(dsg_mma));
  if (!s) return NULL;
  s->n = n;
  s->m = m;
  s->asyminit = 0.5;
  s->asymdec = 0.7;
  s->asyminc = 1.2;
  s->a = (double*)calloc(m, sizeof(double));
  s->c = (double*)calloc(m, sizeof(double));
  s->b = (double*)calloc(m, sizeof(double));
  s->lam = (double*)calloc(m, sizeof(double));
  s->mu = (double*)calloc(m, sizeof(double));
  s->y = (double*)calloc(m, sizeof(double));
  double** v[] = {&s->x1, &s->x2, &s->L, &s->U, &s->al, &s->be, &s->p0, &s->q0};
  for (int i = 0; i < 8; ++i) *v[i] = (double*)calloc(n, sizeof(double));
  s->P = (double*)calloc((size_t)m * n, sizeof(double));
  s->Q = (double*)calloc((size_t)m * n, sizeof(double));
  for (int j = 0; j < m; ++j) {
    s->a[j] = a ? a[j] : 0.;
    s->c[j] = 1000.;
  }
  memcpy(s->x1, x0, sizeof(double) * n);
  memcpy(s->x2, x0, sizeof(double) * n);
  return s;
}

void dsg_mma_destroy(dsg_mma* s) {
  if (!s) return;
  double* v[] = {s->a, s->c, s->b, s->lam, s->mu, s->y, s->x1, s->x2, s->L, s->U,
                 s->al, s->be, s->p0, s->q0, s->P, s->Q};
  for (size_t i = 0; i < sizeof(v) / sizeof(v[0]); ++i) free(v[i]);
  free(s);
}

static double dmax(double a, double b) { return a > b ? a : b; }
static double dmin(double a, double b) { return a < b ? a : b; }

/* x(lam), y(lam), z(lam): the minimisers of the Lagrangian */
static void mma_primal(dsg_mma* s, double* x) {
  double la = 0.;
  for (int j = 0; j < s->m; ++j) {
    if (s->lam[j] < 0.) s->lam[j] = 0.;
    s->y[j] = dmax(0., s->lam[j] - s->c[j]);
    la += s->lam[j] * s->a[j];
  }
  s->z = dmax(0., 10. * (la - 1.));
  for (int i = 0; i < s->n; ++i) {
    double p = s->p0[i], q = s->q0[i];
    for (int j = 0; j < s->m; ++j) {
      p += s->P[(size_t)j * s->n + i] * s->lam[j];
      q += s->Q[(size_t)j * s->n + i] * s->lam[j];
    }
    double sp = sqrt(p), sq = sqrt(q);
    double xi = (sp * s->L[i] + sq * s->U[i]) / (sp + sq);
    x[i] = dmin(dmax(xi, s->al[i]), s->be[i]);
  }
}

/* dual gradient g_j = sum_i (P/(U-x) + Q/(x-L)) - b - a z - y */
static void mma_grad(const dsg_mma* s, const double* x, double* g) {
  for (int j = 0; j < s->m; ++j) {
    double acc = 0.;
    for (int i = 0; i < s->n; ++i)
      acc += s->P[(size_t)j * s->n + i] / (s->U[i] - x[i]) +
             s->Q[(size_t)j * s->n + i] / (x[i] - s->L[i]);
    g[j] = acc - s->b[j] - s->a[j] * s->z - s->y[j];
  }
}

/* dual Hessian (negative semidefinite) at lam */
static void mma_hess(const dsg_mma* s, const double* x, double* H) {
  const int m = s->m;
  for (int k = 0; k < m * m; ++k) H[k] = 0.;
  double* pq = (double*)malloc(sizeof(double) * m);
  for (int i = 0; i < s->n; ++i) {
    double p = s->p0[i], q = s->q0[i];
    for (int j = 0; j < m; ++j) {
      p += s->P[(size_t)j * s->n + i] * s->lam[j];
      q += s->Q[(size_t)j * s->n + i] * s->lam[j];
    }
    double sp = sqrt(p), sq = sqrt(q);
    double xf = (sp * s->L[i] + sq * s->U[i]) / (sp + sq);
    if (xf < s->al[i] || xf > s->be[i]) continue; /* x at a bound: no curvature */
    double ux = s->U[i] - x[i], xl = x[i] - s->L[i];
    double d2 = -1. / (2. * p / (ux * ux * ux) + 2. * q / (xl * xl * xl));
    for (int j = 0; j < m; ++j)
      pq[j] = s->P[(size_t)j * s->n + i] / (ux * ux) - s->Q[(size_t)j * s->n + i] / (xl * xl);
    for (int j = 0; j < m; ++j)
      for (int k = 0; k < m; ++k) H[j * m + k] += pq[j] * d2 * pq[k];
  }
  free(pq);
  double la = 0.;
  for (int j = 0; j < m; ++j) {
    la += s->lam[j] * s->a[j];
    if (s->lam[j] > s->c[j]) H[j * m + j] -= 1.;
  }
  if (la > 1.)
    for (int j = 0; j < m; ++j)
      for (int k = 0; k < m; ++k) H[j * m + k] -= 10. * s->a[j] * s->a[k];
}

/* solve A x = r (m x m, Gaussian elimination with partial pivoting); A destroyed */
static void solve_small(double* A, double* r, int m) {
  for (int c = 0; c < m; ++c) {
    int piv = c;
    for (int k = c + 1; k < m; ++k)
      if (fabs(A[k * m + c]) > fabs(A[piv * m + c])) piv = k;
    if (piv != c) {
      for (int k = 0; k < m; ++k) {
        double t = A[c * m + k];
        A[c * m + k] = A[piv * m + k];
        A[piv * m + k] = t;
      }
      double t = r[c];
      r[c] = r[piv];
      r[piv] = t;
    }
    for (int k = c + 1; k < m; ++k) {
      double f = A[k * m + c] / A[c * m + c];
      for (int l = c; l < m; ++l) A[k * m + l] -= f * A[c * m + l];
      r[k] -= f * r[c];
    }
  }
  for (int c = m - 1; c >= 0; --c) {
    double acc = r[c];
    for (int l = c + 1; l < m; ++l) acc -= A[c * m + l] * r[l];
    r[c] = acc / A[c * m + c];
  }
}

int dsg_mma_update(dsg_mma* s, double* x, const double* df0, const double* g, const double* dg,
                   double movlim, int* dual_iterations, double* change) {
  const int n = s->n, m = s->m;
  s->k += 1;
  const double feps = 1.0e-6;
  for (int i = 0; i < n; ++i) {
    /* outer move limit inside [0, 1] */
    const double xmin = dmax(0., x[i] - movlim), xmax = dmin(1., x[i] + movlim);
    if (s->k < 3) {
      s->L[i] = x[i] - s->asyminit * (xmax - xmin);
      s->U[i] = x[i] + s->asyminit * (xmax - xmin);
    } else {
      const double sg = (x[i] - s->x1[i]) * (s->x1[i] - s->x2[i]);
      const double gm = sg < 0. ? s->asymdec : sg > 0. ? s->asyminc : 1.;
      s->L[i] = x[i] - gm * (s->x1[i] - s->L[i]);
      s->U[i] = x[i] + gm * (s->U[i] - s->x1[i]);
      const double w = dmax(1.0e-5, xmax - xmin);
      s->L[i] = dmin(dmax(s->L[i], x[i] - 10. * w), x[i] - 0.01 * w);
      s->U[i] = dmin(dmax(s->U[i], x[i] + 0.01 * w), x[i] + 10. * w);
    }
    s->al[i] = dmax(xmin, 0.9 * s->L[i] + 0.1 * x[i]);
    s->be[i] = dmin(xmax, 0.9 * s->U[i] + 0.1 * x[i]);
    const double ux = s->U[i] - x[i], xl = x[i] - s->L[i], reg = 0.5 * feps / (s->U[i] - s->L[i]);
    s->p0[i] = ux * ux * (dmax(0., df0[i]) + 0.001 * fabs(df0[i]) + reg);
    s->q0[i] = xl * xl * (dmax(0., -df0[i]) + 0.001 * fabs(df0[i]) + reg);
    for (int j = 0; j < m; ++j) {
      const double d = dg[(size_t)j * n + i];
      s->P[(size_t)j * n + i] = ux * ux * dmax(0., d);
      s->Q[(size_t)j * n + i] = xl * xl * dmax(0., -d);
    }
  }
  for (int j = 0; j < m; ++j) {
    double acc = 0.;
    for (int i = 0; i < n; ++i)
      acc += s->P[(size_t)j * n + i] / (s->U[i] - x[i]) + s->Q[(size_t)j * n + i] / (x[i] - s->L[i]);
    s->b[j] = acc - g[j];
  }
  memcpy(s->x2, s->x1, sizeof(double) * n);
  memcpy(s->x1, x, sizeof(double) * n);

  /* dual: maximise W(lam) over lam >= 0; barrier eps with multipliers mu
   * (mu lam = eps), Newton on (grad W + mu = 0, mu lam = eps), eps /= 10 */
  double* gr = (double*)malloc(sizeof(double) * m);
  double* H = (double*)malloc(sizeof(double) * m * m);
  double* ds = (double*)malloc(sizeof(double) * m);
  double* dm = (double*)malloc(sizeof(double) * m);
  for (int j = 0; j < m; ++j) {
    s->lam[j] = s->c[j] / 2.;
    s->mu[j] = 1.;
  }
  const double tol = 1.0e-9 * sqrt((double)(m + n));
  double eps = 1., err = 1.;
  int iters = 0;
  while (eps > tol) {
    int loop = 0;
    while (err > 0.9 * eps && loop < 100) {
      ++loop;
      ++iters;
      mma_primal(s, x);
      mma_grad(s, x, gr);
      mma_hess(s, x, H);
      double tr = 0.;
      for (int j = 0; j < m; ++j) {
        H[j * m + j] -= s->mu[j] / s->lam[j];
        tr += H[j * m + j];
      }
      /* keep the Newton matrix safely negative definite */
      const double shift = dmin(-1.0e-7, 1.0e-4 * tr / m);
      for (int j = 0; j < m; ++j) {
        H[j * m + j] += shift;
        ds[j] = -gr[j] - eps / s->lam[j];
      }
      solve_small(H, ds, m);
      for (int j = 0; j < m; ++j) dm[j] = -s->mu[j] + eps / s->lam[j] - ds[j] * s->mu[j] / s->lam[j];
      /* step to the boundary of lam, mu > 0, kept 1% inside */
      double th = 1.005;
      for (int j = 0; j < m; ++j) {
        th = dmax(th, -1.01 * ds[j] / s->lam[j]);
        th = dmax(th, -1.01 * dm[j] / s->mu[j]);
      }
      th = 1. / th;
      for (int j = 0; j < m; ++j) {
        s->lam[j] += th * ds[j];
        s->mu[j] += th * dm[j];
      }
      mma_primal(s, x);
      mma_grad(s, x, gr);
      err = 0.;
      for (int j = 0; j < m; ++j) {
        err = dmax(err, fabs(gr[j] + s->mu[j]));
        err = dmax(err, fabs(s->mu[j] * s->lam[j] - eps));
      }
    }
    eps *= 0.1;
  }
  free(gr);
  free(H);
  free(ds);
  free(dm);
  if (dual_iterations) *dual_iterations = iters;
  if (change) {
    double ch = 0.;
    for (int i = 0; i < n; ++i) ch = dmax(ch, fabs(x[i] - s->x1[i]));
    *change = ch;
  }
  return 0;
}

const double* dsg_mma_lambda(const dsg_mma* s) { return s->lam; }
