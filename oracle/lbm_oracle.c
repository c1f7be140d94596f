/*
 * lbm_oracle.c -- CPU restatement of the reference's forward/adjoint LBM hot
 * path, in plain C and FP64.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle: the pytest suite, the
 * package's smoke() and bench.py's CPU-baseline / reference arm call it to
 * produce the reference answer on the same inputs.  No product code path
 * links, loads or calls it.
 *
 * Every operator follows a file of northgaard/LBM-TopOpt (paths relative to
 * its src/ directory) and keeps the reference's order of floating-point
 * operations where the reference writes one out, so that the restatement
 * agrees with the reference code compiled from its own sources (the
 * oracle/_ref build) to the last bits in most cases.
 *
 * Layout: DMDA order, cell c = (z*ny + y)*nx + x, AoS f[c*Q + q], as the
 * reference's DMDAVecGetArrayDOF views (latticeBoltzmann/NewLBSolver2d.cc:12-16).
 */
#include "lbm_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------ */
/* Lattices: latticeBoltzmann/lattices2d.hh:16-62, lattices3d.hh:141-160 */

static const int D2Q9_EX[9] = {0, 1, 0, -1, -1, -1, 0, 1, 1};
static const int D2Q9_EY[9] = {0, -1, -1, -1, 0, 1, 1, 1, 0};
static const int D2Q9_EZ[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
static const int D2Q9_OPP[9] = {0, 5, 6, 7, 8, 1, 2, 3, 4};
static const double D2Q9_W[9] = {4. / 9., 1. / 36., 1. / 9., 1. / 36., 1. / 9.,
                                 1. / 36., 1. / 9., 1. / 36., 1. / 9.};

static const int D3Q19_EX[19] = {0, 0, 0, -1, 0, 0, -1, 1, -1, 1, 0, 0, 1, 0, 0, 1, -1, 1, -1};
static const int D3Q19_EY[19] = {0, 0, -1, 0, -1, 1, 0, 0, -1, -1, 0, 1, 0, 1, -1, 0, 0, 1, 1};
static const int D3Q19_EZ[19] = {0, -1, 0, 0, -1, -1, -1, -1, 0, 0, 1, 0, 0, 1, 1, 1, 1, 0, 0};
static const int D3Q19_OPP[19] = {0, 10, 11, 12, 13, 14, 15, 16, 17, 18,
                                  1, 2, 3, 4, 5, 6, 7, 8, 9};
static const double D3Q19_W[19] = {1. / 3., 1. / 18., 1. / 18., 1. / 18., 1. / 36., 1. / 36.,
                                   1. / 36., 1. / 36., 1. / 36., 1. / 36., 1. / 18., 1. / 18.,
                                   1. / 18., 1. / 36., 1. / 36., 1. / 36., 1. / 36., 1. / 36.,
                                   1. / 36.};

static const int D2Q5_EX[5] = {0, 0, -1, 0, 1};
static const int D2Q5_EY[5] = {0, -1, 0, 1, 0};
static const int D2Q5_EZ[5] = {0, 0, 0, 0, 0};
static const int D2Q5_OPP[5] = {0, 3, 4, 1, 2};
static const double D2Q5_W[5] = {1. / 3., 1. / 6., 1. / 6., 1. / 6., 1. / 6.};

typedef struct {
  int Q, half;
  const int *ex, *ey, *ez, *opp;
  const double* w;
} lattice_t;

static const lattice_t LAT_D2Q9 = {9, 4, D2Q9_EX, D2Q9_EY, D2Q9_EZ, D2Q9_OPP, D2Q9_W};
static const lattice_t LAT_D3Q19 = {19, 9, D3Q19_EX, D3Q19_EY, D3Q19_EZ, D3Q19_OPP, D3Q19_W};
static const lattice_t LAT_D2Q5 = {5, 2, D2Q5_EX, D2Q5_EY, D2Q5_EZ, D2Q5_OPP, D2Q5_W};

/* ------------------------------------------------------------------ */
/* MRT moment bases (rows of the non-conserved moments).
 * D2Q9: dynamics/incompressibleMRT2d.hh:50-60 (e, eps, qx, qy, pxx, pxy).
 * D3Q19: dynamics/MRT3d.hh:50-90 (e, eps, qx, qy, qz, 3pxx, 3pixx, pww,
 * piww, pxy, pyz, pxz, mx, my, mz).  The back-map coefficients of the
 * reference (MRT3d.hh:111-175, incompressibleMRT2d.hh:69-85) are
 * -M[k][i]/|M_k|^2, computed below from the rows. */

static const double MRT2D_M[6][9] = {
    {-4, 2, -1, 2, -1, 2, -1, 2, -1},
    {4, 1, -2, 1, -2, 1, -2, 1, -2},
    {0, 1, 0, -1, 2, -1, 0, 1, -2},
    {0, -1, 2, -1, 0, 1, -2, 1, 0},
    {0, 0, -1, 0, 1, 0, -1, 0, 1},
    {0, -1, 0, 1, 0, -1, 0, 1, 0}};

static const double MRT3D_M[15][19] = {
    {-30, -11, -11, -11, 8, 8, 8, 8, 8, 8, -11, -11, -11, 8, 8, 8, 8, 8, 8},
    {12, -4, -4, -4, 1, 1, 1, 1, 1, 1, -4, -4, -4, 1, 1, 1, 1, 1, 1},
    {0, 0, 0, 4, 0, 0, -1, 1, -1, 1, 0, 0, -4, 0, 0, 1, -1, 1, -1},
    {0, 0, 4, 0, -1, 1, 0, 0, -1, -1, 0, -4, 0, 1, -1, 0, 0, 1, 1},
    {0, 4, 0, 0, -1, -1, -1, -1, 0, 0, -4, 0, 0, 1, 1, 1, 1, 0, 0},
    {0, -1, -1, 2, -2, -2, 1, 1, 1, 1, -1, -1, 2, -2, -2, 1, 1, 1, 1},
    {0, 2, 2, -4, -2, -2, 1, 1, 1, 1, 2, 2, -4, -2, -2, 1, 1, 1, 1},
    {0, -1, 1, 0, 0, 0, -1, -1, 1, 1, -1, 1, 0, 0, 0, -1, -1, 1, 1},
    {0, 2, -2, 0, 0, 0, -1, -1, 1, 1, 2, -2, 0, 0, 0, -1, -1, 1, 1},
    {0, 0, 0, 0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 0, 0, 0, 1, -1},
    {0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0},
    {0, 0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 0, 0, 0, 1, -1, 0, 0},
    {0, 0, 0, 0, 0, 0, 1, -1, -1, 1, 0, 0, 0, 0, 0, -1, 1, 1, -1},
    {0, 0, 0, 0, -1, 1, 0, 0, 1, 1, 0, 0, 0, 1, -1, 0, 0, -1, -1},
    {0, 0, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 0, -1, -1, 1, 1, 0, 0}};

/* Back-map coefficient -M[k][i]/|M_k|^2 as the reference's reduced
 * fractions: the division of two exact integers is correctly rounded, so
 * e.g. 30./2394. is the same double as the reference's 5./399. */
static double backmap_coeff(const double* row, int Q, int i) {
  double n2 = 0.;
  for (int j = 0; j < Q; ++j) n2 += row[j] * row[j];
  return -row[i] / n2;
}

static double MRT2D_B[9][6];
static double MRT3D_B[19][15];

/* Sparse forms of the tables, same order as the dense loops: the nonzero
 * entries of each moment row (over i) and of each back-map row (over k). */
typedef struct {
  int n;
  int idx[19];
  double c[19];
} sparse_row;
static sparse_row MRT2D_MS[6], MRT3D_MS[15];   /* rows of M over i */
static sparse_row MRT2D_BS[9], MRT3D_BS[19];   /* rows of B over k */
static sparse_row MRT2D_MT[9], MRT3D_MT[19];   /* columns of M (over k) */
static int mrt_tables_ready = 0;

static void sparse_build(sparse_row* r, const double* v, int n, int stride) {
  r->n = 0;
  for (int j = 0; j < n; ++j) {
    double c = v[j * stride];
    if (c == 0.) continue;
    r->idx[r->n] = j;
    r->c[r->n] = c;
    r->n++;
  }
}

static void mrt_tables_init(void) {
  if (mrt_tables_ready) return;
  for (int i = 0; i < 9; ++i)
    for (int k = 0; k < 6; ++k) MRT2D_B[i][k] = backmap_coeff(MRT2D_M[k], 9, i);
  for (int i = 0; i < 19; ++i)
    for (int k = 0; k < 15; ++k) MRT3D_B[i][k] = backmap_coeff(MRT3D_M[k], 19, i);
  for (int k = 0; k < 6; ++k) sparse_build(&MRT2D_MS[k], MRT2D_M[k], 9, 1);
  for (int k = 0; k < 15; ++k) sparse_build(&MRT3D_MS[k], MRT3D_M[k], 19, 1);
  for (int i = 0; i < 9; ++i) sparse_build(&MRT2D_BS[i], MRT2D_B[i], 6, 1);
  for (int i = 0; i < 19; ++i) sparse_build(&MRT3D_BS[i], MRT3D_B[i], 15, 1);
  for (int i = 0; i < 9; ++i) sparse_build(&MRT2D_MT[i], &MRT2D_M[0][i], 6, 9);
  for (int i = 0; i < 19; ++i) sparse_build(&MRT3D_MT[i], &MRT3D_M[0][i], 15, 19);
  mrt_tables_ready = 1;
}

/* m_k = sum_i M[k][i] f_i, left to right over the nonzero entries. */
static double row_dot_sparse(const sparse_row* r, const double* f) {
  const int* ix = r->idx;
  const double* c = r->c;
  double s = (c[0] == 1.) ? f[ix[0]] : (c[0] == -1.) ? -f[ix[0]] : c[0] * f[ix[0]];
  for (int j = 1; j < r->n; ++j) {
    double cj = c[j], v = f[ix[j]];
    if (cj == -1.)
      s = s - v;
    else if (cj == 1.)
      s = s + v;
    else
      s = s + cj * v;
  }
  return s;
}

/* ------------------------------------------------------------------ */
/* Interpolations: core/interpolationFunctions.hh:17-54 */

static double bp(double s, double q) { return 1. - s * (1. + q) / (q + s); }
static double bp_diff(double s, double q) {
  return (-(1. + q) / (q + s) + s * (1. + q) / ((q + s) * (q + s)));
}
static double ramp(double s, double q, double ck) {
  return (s * (ck * (1. + q) - 1.) + 1.) / (ck * (1. + q * s));
}
static double ramp_diff(double s, double q, double ck) {
  return (ck * (1. + q) - 1.) / (ck * (1. + q * s)) -
         ((s * (ck * (1. + q) - 1.) + 1.) * q) / (ck * (1. + q * s) * (1. + q * s));
}

/* ------------------------------------------------------------------ */
/* Model context */

typedef struct {
  lbm_config cfg;
  const lattice_t* L;   /* flow lattice */
  int Qf;               /* flow populations per cell */
  int Qt;               /* temperature populations per cell (0 or 5) */
  int Q;                /* total per cell */
  int nmac;             /* macros per cell */
  int64_t ncell;
  int nx, ny, nz, dim;
  int t_phase;          /* step at which the last steady phase ended (LBM_TIME_RAMP) */
  int obj_from;         /* first step whose state's objective counts */
} model_t;

/* Phase of the runs that follow (orc_set_phase): INT_MAX / 1 = no steady phase. */
static int g_phase_start = 2147483647, g_obj_from = 1;

static int model_init(model_t* m, const lbm_config* cfg) {
  memset(m, 0, sizeof(*m));
  m->cfg = *cfg;
  mrt_tables_init();
  m->nx = cfg->nx;
  m->ny = cfg->ny;
  m->nz = cfg->nz > 0 ? cfg->nz : 1;
  if (cfg->lattice == LBM_D2Q9) {
    m->L = &LAT_D2Q9;
    m->Qf = 9;
    m->Qt = 0;
    m->nmac = 3;
    m->dim = 2;
  } else if (cfg->lattice == LBM_D3Q19) {
    m->L = &LAT_D3Q19;
    m->Qf = 19;
    m->Qt = 0;
    m->nmac = 4;
    m->dim = 3;
  } else if (cfg->lattice == LBM_D2Q9_D2Q5) {
    m->L = &LAT_D2Q9;
    m->Qf = 9;
    m->Qt = 5;
    m->nmac = 4;
    m->dim = 2;
  } else {
    return -1;
  }
  if (m->dim == 2) m->nz = 1;
  m->Q = m->Qf + m->Qt;
  m->ncell = (int64_t)m->nx * m->ny * m->nz;
  m->t_phase = g_phase_start;
  m->obj_from = g_obj_from;
  return 0;
}

int orc_set_phase(int t_phase, int obj_from) {
  g_phase_start = t_phase;
  g_obj_from = obj_from;
  return 0;
}

static double pbb_factor(const model_t* m, double g) {
  return 0.5 * (m->cfg.interp_scale * bp(g, m->cfg.interp_q));
}
static double pbb_factor_diff(const model_t* m, double g) {
  return 0.5 * (m->cfg.interp_scale * bp_diff(g, m->cfg.interp_q));
}

/* ------------------------------------------------------------------ */
/* Macros.  D2Q9: IncompressibleMacros2d<D2Q9> (dynamics/isothermalMacros2d.hh:199-208);
 * D3Q19: IncompressibleMacros3d (isothermalMacros3d.hh:6-24). */

static void macros_d2q9(const double* f, double* rho, double* ux, double* uy) {
  double jx = f[1] + f[7] + f[8];
  double jy = f[5] + f[6] + f[7];
  *rho = jx + jy - f[7] + f[0] + f[2] + f[3] + f[4];
  jx -= f[3] + f[4] + f[5];
  jy -= f[1] + f[2] + f[3];
  *ux = jx;
  *uy = jy;
}

static void macros_generic(const lattice_t* L, const double* f, double* mac) {
  double r = 0., jx = 0., jy = 0., jz = 0.;
  for (int i = 0; i < L->Q; ++i) {
    r += f[i];
    jx += L->ex[i] * f[i];
    jy += L->ey[i] * f[i];
    jz += L->ez[i] * f[i];
  }
  mac[0] = r;
  mac[1] = jx;
  mac[2] = jy;
  mac[3] = jz;
}

static void flow_macros(const model_t* m, const double* f, double* mac) {
  if (m->dim == 2) {
    macros_d2q9(f, &mac[0], &mac[1], &mac[2]);
  } else {
    macros_generic(m->L, f, mac);
  }
}

/* ------------------------------------------------------------------ */
/* Forward collision operators */

/* IncompressibleBGK2d<D2Q9>::operator() (dynamics/incompressibleBGK2d.hh:120-147) */
static void bgk_d2q9(const double* fin, double* fout, double* mac, double omega) {
  macros_d2q9(fin, &mac[0], &mac[1], &mac[2]);
  const double uSqr = mac[1] * mac[1] + mac[2] * mac[2];
  const double cFeq = mac[0] - 1.5 * uSqr;
  const double rel = 1. - omega;
  const double restW = 4. / 9., stW = 1. / 9., diagW = 1. / 36.;
  fout[0] = rel * fin[0] + omega * restW * cFeq;
  fout[2] = rel * fin[2] + omega * stW * (cFeq - 3. * mac[2] + 4.5 * mac[2] * mac[2]);
  fout[4] = rel * fin[4] + omega * stW * (cFeq - 3. * mac[1] + 4.5 * mac[1] * mac[1]);
  fout[6] = rel * fin[6] + omega * stW * (cFeq + 3. * mac[2] + 4.5 * mac[2] * mac[2]);
  fout[8] = rel * fin[8] + omega * stW * (cFeq + 3. * mac[1] + 4.5 * mac[1] * mac[1]);
  fout[1] = rel * fin[1] +
            omega * diagW * (cFeq + 3. * (mac[1] - mac[2]) + 4.5 * (uSqr - 2. * mac[1] * mac[2]));
  fout[3] = rel * fin[3] +
            omega * diagW * (cFeq - 3. * (mac[1] + mac[2]) + 4.5 * (uSqr + 2. * mac[1] * mac[2]));
  fout[5] = rel * fin[5] +
            omega * diagW * (cFeq + 3. * (mac[2] - mac[1]) + 4.5 * (uSqr - 2. * mac[1] * mac[2]));
  fout[7] = rel * fin[7] +
            omega * diagW * (cFeq + 3. * (mac[1] + mac[2]) + 4.5 * (uSqr + 2. * mac[1] * mac[2]));
}

/* Incompressible BGK on a generic lattice (incompressibleBGK2d.hh:38-47, BGK3d.hh). */
static void bgk_generic(const lattice_t* L, const double* fin, double* fout, double* mac,
                        double omega) {
  macros_generic(L, fin, mac);
  double uSqr = mac[1] * mac[1] + mac[2] * mac[2] + mac[3] * mac[3];
  for (int i = 0; i < L->Q; ++i) {
    double sc = L->ex[i] * mac[1] + L->ey[i] * mac[2] + L->ez[i] * mac[3];
    double eq = L->w[i] * (mac[0] + 3. * sc + 4.5 * sc * sc - 1.5 * uSqr);
    fout[i] = fin[i] * (1. - omega);
    fout[i] += omega * eq;
  }
}

/* Relaxation of the D2Q9 moments (incompressibleMRT2d.hh:62-67). */
static void mrt2d_relax(double* mo, const double* mac, const model_t* m) {
  const double s1 = m->cfg.mrt[0], s2 = m->cfg.mrt[1], s46 = m->cfg.mrt[2];
  const double om = m->cfg.omega;
  double uSqr = mac[1] * mac[1] + mac[2] * mac[2];
  mo[0] = s1 * (mo[0] + 2. * mac[0] - 3. * uSqr);
  mo[1] = s2 * (mo[1] - mac[0] + 3. * uSqr);
  mo[2] = s46 * (mo[2] + mac[1]);
  mo[3] = s46 * (mo[3] + mac[2]);
  mo[4] = om * (mo[4] - mac[1] * mac[1] + mac[2] * mac[2]);
  mo[5] = om * (mo[5] - mac[1] * mac[2]);
}

/* Relaxation of the D3Q19 moments (MRT3d.hh:92-109). */
static void mrt3d_relax(double* mo, const double* mac, const model_t* m) {
  const double* r = m->cfg.mrt;
  const double s1 = r[0], s2 = r[1], s4 = r[2], s10 = r[3], s16 = r[4];
  const double we = r[5], wej = r[6], wxx = r[7], om = m->cfg.omega;
  double jSqr = mac[1] * mac[1] + mac[2] * mac[2] + mac[3] * mac[3];
  mo[0] = s1 * (mo[0] + 11. * mac[0] - 19. * jSqr);
  mo[1] = s2 * (mo[1] - we * mac[0] - wej * jSqr);
  mo[2] = s4 * (mo[2] + (2. / 3.) * mac[1]);
  mo[3] = s4 * (mo[3] + (2. / 3.) * mac[2]);
  mo[4] = s4 * (mo[4] + (2. / 3.) * mac[3]);
  double tempEq = (2. * mac[1] * mac[1] - (mac[2] * mac[2] + mac[3] * mac[3]));
  mo[5] = om * (mo[5] - tempEq);
  mo[6] = s10 * (mo[6] - wxx * tempEq);
  tempEq = (mac[2] * mac[2] - mac[3] * mac[3]);
  mo[7] = om * (mo[7] - tempEq);
  mo[8] = s10 * (mo[8] - wxx * tempEq);
  mo[9] = om * (mo[9] - mac[1] * mac[2]);
  mo[10] = om * (mo[10] - mac[2] * mac[3]);
  mo[11] = om * (mo[11] - mac[1] * mac[3]);
  mo[12] *= s16;
  mo[13] *= s16;
  mo[14] *= s16;
}

static void mrt_collide(const model_t* m, const double* fin, double* fout, double* mac) {
  double mo[15];
  int Q = m->Qf, K = (m->dim == 2) ? 6 : 15;
  flow_macros(m, fin, mac);
  /* Dense left-to-right sums: the zero entries add exact zeros and products
   * with +-1 are exact, so the partial sums are those of the reference's
   * written-out expressions (MRT3d.hh:50-90, 111-175). */
  if (m->dim == 3) {
    for (int k = 0; k < 15; ++k) {
      double acc = 0.;
      for (int i = 0; i < 19; ++i) acc += MRT3D_M[k][i] * fin[i];
      mo[k] = acc;
    }
    mrt3d_relax(mo, mac, m);
    for (int i = 0; i < 19; ++i) {
      double v = fin[i];
      for (int k = 0; k < 15; ++k) v += MRT3D_B[i][k] * mo[k];
      fout[i] = v;
    }
    return;
  }
  const sparse_row* MS = MRT2D_MS;
  const sparse_row* BS = MRT2D_BS;
  for (int k = 0; k < K; ++k) mo[k] = row_dot_sparse(&MS[k], fin);
  mrt2d_relax(mo, mac, m);
  for (int i = 0; i < Q; ++i) {
    const sparse_row* b = &BS[i];
    double v = fin[i];
    for (int j = 0; j < b->n; ++j) v = v + b->c[j] * mo[b->idx[j]];
    fout[i] = v;
  }
}

static void base_collide(const model_t* m, const double* fin, double* fout, double* mac) {
  if (m->cfg.collision == LBM_MRT) {
    mrt_collide(m, fin, fout, mac);
  } else if (m->dim == 2) {
    bgk_d2q9(fin, fout, mac, m->cfg.omega);
  } else {
    bgk_generic(m->L, fin, fout, mac, m->cfg.omega);
  }
}

/* PartialBouncebackCollision::operator() (dynamics/partialBouncebackCollision.hh:53-65) */
static void pbb_collide(const model_t* m, const double* fin, double* fout, double* mac,
                        double g) {
  base_collide(m, fin, fout, mac);
  double imult = pbb_factor(m, g);
  int h = m->L->half;
  for (int d = 1; d <= h; ++d) {
    double ftemp = fout[d];
    fout[d] += imult * (fout[d + h] - fout[d]);
    fout[d + h] += imult * (ftemp - fout[d + h]);
  }
}

/* Temperature collision: ThermalBGK2d<D2Q5> with the obstacle rate of
 * ThermalObstacleCollision (dynamics/thermalBGK2d.hh:58-65,
 * thermalObstacleCollision.hh:47-53), composed after the flow collision as
 * in ThermalDualCollision (thermalDualCollision.hh:57-64), plus the solid
 * heating term g_i += (1-gamma) w_i heat_rate (heat_T - T). */
static double thermal_omega(const model_t* m, double g) {
  double imult = m->cfg.diffusivity * ramp(g, m->cfg.ramp_q, m->cfg.ramp_ck);
  return 1. / (3. * imult + 0.5);
}

static void thermal_collide(const model_t* m, const double* gin, double* gout, double* mac,
                            double g) {
  double om = thermal_omega(m, g);
  double T = gin[0] + gin[1] + gin[2] + gin[3] + gin[4];
  mac[3] = T;
  for (int i = 0; i < 5; ++i) {
    double sc = D2Q5_EX[i] * mac[1] + D2Q5_EY[i] * mac[2];
    double eq = D2Q5_W[i] * T * (1. + 3. * sc);
    gout[i] = gin[i] * (1. - om);
    gout[i] += om * eq;
  }
  double hs = (1. - g) * m->cfg.heat_rate * (m->cfg.heat_T - T);
  for (int i = 0; i < 5; ++i) gout[i] += D2Q5_W[i] * hs;
}

static void cell_collide(const model_t* m, const double* fin, double* fout, double* mac,
                         double g) {
  pbb_collide(m, fin, fout, mac, g);
  if (m->Qt) thermal_collide(m, fin + m->Qf, fout + m->Qf, mac, g);
}

/* ------------------------------------------------------------------ */
/* Reverse (adjoint) collision operators.  Each returns lam_in = (df_out/df_in)^T lam_out
 * and accumulates dgamma += (df_out/dgamma)^T lam_out. */

/* ReverseIncompressibleBGK2d<D2Q9>::operator() (adjointDynamics/reverseIncompressibleBGK2d.hh:112-169) */
static void rev_bgk_d2q9(const double* fin, const double* lo, double* li, double omega) {
  double mac[3], macRev[3] = {0., 0., 0.};
  macros_d2q9(fin, &mac[0], &mac[1], &mac[2]);
  const double rel = 1. - omega;
  const double restW = 4. / 9., stW = 1. / 9., diagW = 1. / 36.;
  double uSqrRev, cFeqRev, temp;
  for (int i = 0; i < 9; ++i) li[i] += rel * lo[i];
  temp = omega * diagW * lo[7];
  cFeqRev = temp;
  uSqrRev = temp;
  macRev[1] += temp * (9. * mac[2] + 3.);
  macRev[2] += 3. * temp * (3. * mac[1] + 1.);
  temp = omega * diagW * lo[5];
  cFeqRev += temp;
  uSqrRev += temp;
  macRev[1] -= temp * (9. * mac[2] + 3.);
  macRev[2] += temp * (3. - 9. * mac[1]);
  temp = omega * diagW * lo[3];
  cFeqRev += temp;
  uSqrRev += temp;
  macRev[1] += temp * (9. * mac[2] - 3.);
  macRev[2] += temp * (9. * mac[1] - 3.);
  temp = omega * diagW * lo[1];
  cFeqRev += temp;
  uSqrRev += temp;
  uSqrRev *= 4.5;
  macRev[1] += temp * (3 - 9. * mac[2]);
  macRev[2] -= temp * (9. * mac[1] + 3.);
  temp = omega * stW * lo[8];
  cFeqRev += temp;
  macRev[1] += (9. * mac[1] + 3.) * temp;
  temp = omega * stW * lo[6];
  cFeqRev += temp;
  macRev[2] = macRev[2] + (9. * mac[2] + 3.) * temp;
  temp = omega * stW * lo[4];
  cFeqRev += temp;
  macRev[1] = macRev[1] + (9. * mac[1] - 3.) * temp;
  temp = omega * stW * lo[2];
  cFeqRev += temp + omega * restW * lo[0];
  macRev[2] = macRev[2] + (9. * mac[2] - 3.) * temp;
  uSqrRev -= 1.5 * cFeqRev;
  macRev[0] = macRev[0] + cFeqRev;
  macRev[1] = macRev[1] + 2. * mac[1] * uSqrRev;
  macRev[2] = macRev[2] + 2. * mac[2] * uSqrRev;
  /* ReverseIncompressibleMacros2d<D2Q9>::compute (reverseIsothermalMacros2d.hh:198-214) */
  li[0] += macRev[0];
  li[1] += macRev[0] + macRev[1] - macRev[2];
  li[2] += macRev[0] - macRev[2];
  li[3] += macRev[0] - macRev[1] - macRev[2];
  li[4] += macRev[0] - macRev[1];
  li[5] += macRev[0] - macRev[1] + macRev[2];
  li[6] += macRev[0] + macRev[2];
  li[7] += macRev[0] + macRev[1] + macRev[2];
  li[8] += macRev[0] + macRev[1];
}

/* Transpose of bgk_generic: feq_i = w_i(rho + 3s + 4.5 s^2 - 1.5 u^2), s = e_i.j. */
static void rev_bgk_generic(const lattice_t* L, const double* fin, const double* lo, double* li,
                            double omega) {
  double mac[4];
  macros_generic(L, fin, mac);
  double rR = 0., jR[3] = {0., 0., 0.};
  for (int i = 0; i < L->Q; ++i) {
    double sc = L->ex[i] * mac[1] + L->ey[i] * mac[2] + L->ez[i] * mac[3];
    double a = omega * L->w[i] * lo[i];
    li[i] += (1. - omega) * lo[i];
    rR += a;
    double ds = a * (3. + 9. * sc);
    jR[0] += ds * L->ex[i] - 3. * a * mac[1];
    jR[1] += ds * L->ey[i] - 3. * a * mac[2];
    jR[2] += ds * L->ez[i] - 3. * a * mac[3];
  }
  for (int i = 0; i < L->Q; ++i)
    li[i] += rR + jR[0] * L->ex[i] + jR[1] * L->ey[i] + jR[2] * L->ez[i];
}

/* Transpose of the MRT collision f_out = f - sum_k B[i][k] r_k,
 * r_k = s_k (m_k - meq_k(rho, j)), derived from the forward operator
 * (reference transposes: reverseIncompressibleMRT2d.hh:29-83, reverseMRT3d.hh:29-365). */
static void rev_mrt(const model_t* m, const double* fin, const double* lo, double* li) {
  int Q = m->Qf, K = (m->dim == 2) ? 6 : 15;
  double mac[4] = {0., 0., 0., 0.};
  flow_macros(m, fin, mac);
  double a[15], rate[15];
  const double* r = m->cfg.mrt;
  const double om = m->cfg.omega;
  if (m->dim == 2) {
    double rr[6] = {r[0], r[1], r[2], r[2], om, om};
    for (int k = 0; k < 6; ++k) rate[k] = rr[k];
  } else {
    double rr[15] = {r[0], r[1], r[2], r[2], r[2], om, r[3], om, r[3], om, om, om,
                     r[4], r[4], r[4]};
    for (int k = 0; k < 15; ++k) rate[k] = rr[k];
  }
  if (m->dim == 3) {
    for (int k = 0; k < 15; ++k) {
      double acc = 0.;
      for (int i = 0; i < 19; ++i) acc += MRT3D_B[i][k] * lo[i];
      a[k] = rate[k] * acc;
    }
    for (int i = 0; i < 19; ++i) {
      double v = lo[i];
      for (int k = 0; k < 15; ++k) v += MRT3D_M[k][i] * a[k];
      li[i] += v;
    }
  }
  const sparse_row* MS = MRT2D_MS;
  const sparse_row* MT = MRT2D_MT;
  for (int k = 0; k < K && m->dim == 2; ++k) {
    /* sum_i B[i][k] lo_i = -(1/|M_k|^2) sum_i M[k][i] lo_i */
    const sparse_row* r = &MS[k];
    double s = 0., n2 = 0.;
    for (int j = 0; j < r->n; ++j) {
      s += (-r->c[j]) * lo[r->idx[j]];
      n2 += r->c[j] * r->c[j];
    }
    a[k] = rate[k] * (s / n2); /* adjoint of (m_k - meq_k) */
  }
  (void)Q;
  /* through m_k = M f */
  for (int i = 0; i < Q && m->dim == 2; ++i) {
    const sparse_row* c = &MT[i];
    double v = lo[i];
    for (int j = 0; j < c->n; ++j) v += c->c[j] * a[c->idx[j]];
    li[i] += v;
  }
  /* through -meq(rho, j) */
  double rR, jR[3];
  if (m->dim == 2) {
    double jx = mac[1], jy = mac[2];
    rR = -(a[0] * (-2.) + a[1] * 1.);
    jR[0] = -(a[0] * 6. * jx + a[1] * (-6.) * jx + a[2] * (-1.) + a[4] * 2. * jx + a[5] * jy);
    jR[1] = -(a[0] * 6. * jy + a[1] * (-6.) * jy + a[3] * (-1.) + a[4] * (-2.) * jy + a[5] * jx);
    jR[2] = 0.;
  } else {
    double jx = mac[1], jy = mac[2], jz = mac[3];
    double we = r[5], wej = r[6], wxx = r[7];
    rR = -(a[0] * (-11.) + a[1] * we);
    double c2 = -2. / 3.;
    jR[0] = -(a[0] * 38. * jx + a[1] * 2. * wej * jx + a[2] * c2 + (a[5] + wxx * a[6]) * 4. * jx +
              a[9] * jy + a[11] * jz);
    jR[1] = -(a[0] * 38. * jy + a[1] * 2. * wej * jy + a[3] * c2 - (a[5] + wxx * a[6]) * 2. * jy +
              (a[7] + wxx * a[8]) * 2. * jy + a[9] * jx + a[10] * jz);
    jR[2] = -(a[0] * 38. * jz + a[1] * 2. * wej * jz + a[4] * c2 - (a[5] + wxx * a[6]) * 2. * jz -
              (a[7] + wxx * a[8]) * 2. * jz + a[10] * jy + a[11] * jx);
  }
  const lattice_t* L = m->L;
  for (int i = 0; i < Q; ++i)
    li[i] += rR + jR[0] * L->ex[i] + jR[1] * L->ey[i] + jR[2] * L->ez[i];
}

static void rev_base(const model_t* m, const double* fin, const double* lo, double* li) {
  if (m->cfg.collision == LBM_MRT) {
    rev_mrt(m, fin, lo, li);
  } else if (m->dim == 2) {
    rev_bgk_d2q9(fin, lo, li, m->cfg.omega);
  } else {
    rev_bgk_generic(m->L, fin, lo, li, m->cfg.omega);
  }
}

/* ReversePartialBouncebackCollision::operator() (adjointDynamics/reversePartialBounceback.hh:18-41).
 * lo is modified in place (it is the reference's fdistOutRev). */
static void rev_pbb(const model_t* m, const double* fin, double* lo, double* li, double g,
                    double* dg) {
  double fout[19], mac[4];
  base_collide(m, fin, fout, mac);
  double imult = pbb_factor(m, g);
  double imultRev = 0.;
  int h = m->L->half;
  for (int d = 1; d <= h; ++d) {
    imultRev += (fout[d] - fout[d + h]) * lo[d + h];
    imultRev += (fout[d + h] - fout[d]) * lo[d];
    double ftempRev = lo[d + h];
    lo[d + h] += imult * (lo[d] - lo[d + h]);
    lo[d] += imult * (ftempRev - lo[d]);
  }
  *dg += pbb_factor_diff(m, g) * imultRev;
  rev_base(m, fin, lo, li);
}

/* Transpose of thermal_collide (the reference's ReverseThermalObstacleCollision /
 * ReverseThermalBGK2d, adjointDynamics/reverseThermalObstacleCollision.hh,
 * reverseThermalBGK2d.hh, derived here for the composed operator).  Needs the flow
 * velocity of the pre-collision state; adds its adjoint to ujR[0..1]. */
static void rev_thermal(const model_t* m, const double* fin, const double* lo, double* li,
                        double g, double* dg, double* ujR) {
  const double* gin = fin + 9;
  double mac[3];
  macros_d2q9(fin, &mac[0], &mac[1], &mac[2]);
  double T = gin[0] + gin[1] + gin[2] + gin[3] + gin[4];
  double om = thermal_omega(m, g);
  double TR = 0., uxR = 0., uyR = 0., omR = 0.;
  for (int i = 0; i < 5; ++i) {
    double sc = D2Q5_EX[i] * mac[1] + D2Q5_EY[i] * mac[2];
    double eq = D2Q5_W[i] * T * (1. + 3. * sc);
    li[9 + i] += (1. - om) * lo[9 + i];
    omR += (eq - gin[i]) * lo[9 + i];
    double a = om * lo[9 + i] * D2Q5_W[i];
    TR += a * (1. + 3. * sc);
    uxR += a * T * 3. * D2Q5_EX[i];
    uyR += a * T * 3. * D2Q5_EY[i];
  }
  /* heating hs = (1-g) h (Th - T), g_i += w_i hs */
  double hsR = 0.;
  for (int i = 0; i < 5; ++i) hsR += D2Q5_W[i] * lo[9 + i];
  TR += -(1. - g) * m->cfg.heat_rate * hsR;
  *dg += -m->cfg.heat_rate * (m->cfg.heat_T - T) * hsR;
  /* om = 1/(3 D ramp(g) + 0.5) */
  double den = 3. * m->cfg.diffusivity * ramp(g, m->cfg.ramp_q, m->cfg.ramp_ck) + 0.5;
  *dg += omR * (-1. / (den * den)) * 3. * m->cfg.diffusivity *
         ramp_diff(g, m->cfg.ramp_q, m->cfg.ramp_ck);
  for (int i = 0; i < 5; ++i) li[9 + i] += TR;
  ujR[0] += uxR;
  ujR[1] += uyR;
}

static void cell_reverse(const model_t* m, const double* fin, double* lo, double* li, double g,
                         double* dg) {
  for (int i = 0; i < m->Q; ++i) li[i] = 0.;
  if (m->Qt) {
    double ujR[2] = {0., 0.};
    rev_thermal(m, fin, lo, li, g, dg, ujR);
    /* u = j (incompressible): d j / d f_i = e_i */
    for (int i = 0; i < 9; ++i) li[i] += ujR[0] * D2Q9_EX[i] + ujR[1] * D2Q9_EY[i];
  }
  rev_pbb(m, fin, lo, li, g, dg);
}

/* ------------------------------------------------------------------ */
/* Streaming.  Pull with mid-way bounce-back (dynamics/isothermalLBLoops2d.hh:65-86),
 * generalised to 3D and to the temperature lattice. */

static void stream_lattice(const model_t* m, const lattice_t* L, int off, const double* src,
                           double* dst) {
  int nx = m->nx, ny = m->ny, nz = m->nz, Q = m->Q;
#pragma omp parallel for collapse(2) schedule(static)
  for (int z = 0; z < nz; ++z)
    for (int y = 0; y < ny; ++y)
      for (int x = 0; x < nx; ++x) {
        int64_t c = ((int64_t)z * ny + y) * nx + x;
        dst[c * Q + off] = src[c * Q + off];
        for (int d = 1; d < L->Q; ++d) {
          int sx = x - L->ex[d], sy = y - L->ey[d], sz = z - L->ez[d];
          if (sx >= 0 && sy >= 0 && sz >= 0 && sx < nx && sy < ny && sz < nz) {
            int64_t s = ((int64_t)sz * ny + sy) * nx + sx;
            dst[c * Q + off + d] = src[s * Q + off + d];
          } else {
            dst[c * Q + off + d] = src[c * Q + off + L->opp[d]];
          }
        }
      }
}

static void stream_all(const model_t* m, const double* src, double* dst) {
  stream_lattice(m, m->L, 0, src, dst);
  if (m->Qt) stream_lattice(m, &LAT_D2Q5, 9, src, dst);
}

/* Push transpose with the bounce-back transpose
 * (adjointDynamics/adjointIsothermalLBLoops2d.hh:139-163), generalised to 3D. */
static void adjoint_stream_lattice(const model_t* m, const lattice_t* L, int off,
                                   const double* src, double* dst) {
  int nx = m->nx, ny = m->ny, nz = m->nz, Q = m->Q;
#pragma omp parallel for collapse(2) schedule(static)
  for (int z = 0; z < nz; ++z)
    for (int y = 0; y < ny; ++y)
      for (int x = 0; x < nx; ++x) {
        int64_t c = ((int64_t)z * ny + y) * nx + x;
        dst[c * Q + off] = src[c * Q + off];
        for (int d = 1; d < L->Q; ++d) {
          int sx = x + L->ex[d], sy = y + L->ey[d], sz = z + L->ez[d];
          if (sx >= 0 && sy >= 0 && sz >= 0 && sx < nx && sy < ny && sz < nz) {
            int64_t s = ((int64_t)sz * ny + sy) * nx + sx;
            dst[c * Q + off + d] = src[s * Q + off + d];
          } else {
            dst[c * Q + off + d] = src[c * Q + off + L->opp[d]];
          }
        }
      }
}

static void adjoint_stream_all(const model_t* m, const double* src, double* dst) {
  adjoint_stream_lattice(m, m->L, 0, src, dst);
  if (m->Qt) adjoint_stream_lattice(m, &LAT_D2Q5, 9, src, dst);
}

/* ------------------------------------------------------------------ */
/* Boundary conditions */

static double time_factor(const model_t* m, const lbm_bc* b, int t) {
  if (b->time_law == LBM_TIME_SINE)
    return b->amp == 0. ? 0. : b->amp * sin(2. * M_PI * (double)t / b->period);
  if (b->time_law == LBM_TIME_RAMP) {
    /* StageTemp (applications/Regenerator2d/regenerator2d.cc:53-69) */
    if (m->t_phase == 2147483647 || t <= m->t_phase) return b->amp;
    double s = (double)t - (double)m->t_phase;
    return b->amp + (s < b->period ? sin(M_PI * s / (2. * b->period)) : 1.);
  }
  if (b->amp == 0.) return 1.;
  return 1. + b->amp * sin(2. * M_PI * (double)t / b->period);
}

/* Tabulated boundary inputs (the library's lbm_set_bc_profile), one per
 * boundary slot: nt rows of npos cells of ncomp values. */
static struct {
  double* v;
  int nt, ncomp;
  int64_t npos;
} g_tab[LBM_MAX_BC];

static int on_y_face(const lbm_bc* b) {
  return b->face == LBM_FACE_SOUTH || b->face == LBM_FACE_NORTH;
}

int orc_set_bc_profile(int k, int nt, int ncomp, int64_t npos, const double* table) {
  if (k < 0 || k >= LBM_MAX_BC) return -1;
  free(g_tab[k].v);
  g_tab[k].v = NULL;
  g_tab[k].nt = g_tab[k].ncomp = 0;
  g_tab[k].npos = 0;
  if (!table) return 0;
  size_t n = (size_t)nt * (size_t)npos * (size_t)ncomp;
  g_tab[k].v = (double*)malloc(sizeof(double) * n);
  if (!g_tab[k].v) return -4;
  memcpy(g_tab[k].v, table, sizeof(double) * n);
  g_tab[k].nt = nt;
  g_tab[k].ncomp = ncomp;
  g_tab[k].npos = npos;
  return 0;
}

/* Index of (x,y,z) among the box cells: along y, then z, on west/east faces;
 * along x on south/north faces. */
static int64_t bc_index(const lbm_bc* b, int x, int y, int z) {
  if (on_y_face(b)) return x - b->box[0];
  return (int64_t)(z - b->box[4]) * (b->box[3] - b->box[2] + 1) + (y - b->box[2]);
}

/* Velocity profile along the face: the reference applications' inflow
 * functors (applications/diffuser/diffuser.cc:22-31): vmax*(mid^2-(s-mid)^2)/mid^2
 * across the lattice (s = y on west/east faces, x on south/north faces). */
static double profile(const model_t* m, const lbm_bc* b, int x, int y, int z) {
  if (b->profile != LBM_PROFILE_PARABOLIC) return 1.;
  int n = on_y_face(b) ? m->nx : m->ny, s = on_y_face(b) ? x : y;
  double mid = (double)(n - 1) / 2.;
  double p = (mid * mid - (s - mid) * (s - mid)) / (mid * mid);
  if (m->dim == 3) {
    double mz = (double)(m->nz - 1) / 2.;
    p *= (mz * mz - (z - mz) * (z - mz)) / (mz * mz);
  }
  return p;
}

static const double* table_entry(const lbm_bc* b, int k, int t, int x, int y, int z) {
  if (b->profile != LBM_PROFILE_TABLE || !g_tab[k].v) return NULL;
  return g_tab[k].v + ((int64_t)(t % g_tab[k].nt) * g_tab[k].npos + bc_index(b, x, y, z)) *
                          g_tab[k].ncomp;
}

/* Scalar value (density, temperature) of boundary k at a cell. */
static double bc_scalar(const model_t* m, int k, int t, int x, int y, int z) {
  const lbm_bc* b = &m->cfg.bc[k];
  double v = b->value * time_factor(m, b, t);
  const double* e = table_entry(b, k, t, x, y, z);
  if (e) v *= e[0];
  return v;
}

/* Velocity of boundary k at a cell: value * T(t) * profile * dir, or the
 * tabulated vector. */
static void bc_velocity(const model_t* m, int k, int t, int x, int y, int z, double* u) {
  const lbm_bc* b = &m->cfg.bc[k];
  const double* e = table_entry(b, k, t, x, y, z);
  if (e && g_tab[k].ncomp >= 2) {
    u[0] = e[0];
    u[1] = e[1];
    u[2] = g_tab[k].ncomp == 3 ? e[2] : 0.;
    return;
  }
  double v = b->value * time_factor(m, b, t);
  v *= e ? e[0] : profile(m, b, x, y, z);
  int nodir = b->dir[0] == 0. && b->dir[1] == 0. && b->dir[2] == 0.;
  for (int a = 0; a < 3; ++a) u[a] = v * (nodir ? (a == 0 ? 1. : 0.) : b->dir[a]);
}

/* Zou-He boundaries of D2Q9 (boundaryConditions/ZouHe2d.hh):
 * IncompressibleZouHeVelocityWest/North/East2d (:29-44, 66-81, 103-118),
 * StandardZouHeVelocityWest2d (:146-163), IncompressibleZouHePressureEast/West2d
 * (:252-268, 292-308), StandardZouHePressureEast/West2d (:332-349, 366-383); the
 * south velocity is the north one mirrored in y, the north and south pressures
 * the east and west ones rotated by +90 degrees (no reference counterparts). */
static void zouhe2d(const model_t* m, int k, int t, double* F) {
  const lbm_bc* b = &m->cfg.bc[k];
  int Q = m->Q;
  for (int z = b->box[4]; z <= b->box[5]; ++z)
    for (int y = b->box[2]; y <= b->box[3]; ++y)
      for (int x = b->box[0]; x <= b->box[1]; ++x) {
        double* f = F + (((int64_t)z * m->ny + y) * m->nx + x) * Q;
        if (b->kind == LBM_BC_VELOCITY || b->kind == LBM_BC_VELOCITY_STANDARD) {
          double u[3];
          bc_velocity(m, k, t, x, y, z, u);
          double ux = u[0], uy = u[1];
          if (b->kind == LBM_BC_VELOCITY_STANDARD) {
            double rho = (f[0] + f[2] + f[6] + 2. * (f[3] + f[4] + f[5])) / (1. - ux);
            f[1] = f[5] + 0.5 * (f[6] - f[2]) + (1. / 6.) * rho * ux - 0.5 * rho * uy;
            f[7] = f[3] + 0.5 * (f[2] - f[6]) + (1. / 6.) * rho * ux + 0.5 * rho * uy;
            f[8] = f[4] + (2. / 3.) * rho * ux;
          } else if (b->face == LBM_FACE_WEST) {
            f[1] = 0.5 * (f[6] - f[2]) + f[5] + (1. / 6.) * ux - 0.5 * uy;
            f[7] = 0.5 * (f[2] - f[6]) + f[3] + (1. / 6.) * ux + 0.5 * uy;
            f[8] = f[4] + (2. / 3.) * ux;
          } else if (b->face == LBM_FACE_EAST) {
            f[3] = f[7] + 0.5 * (f[6] - f[2]) - (1. / 6.) * ux - 0.5 * uy;
            f[4] = f[8] - (2. / 3.) * ux;
            f[5] = f[1] + 0.5 * (f[2] - f[6]) - (1. / 6.) * ux + 0.5 * uy;
          } else if (b->face == LBM_FACE_NORTH) {
            f[1] = 0.5 * (f[4] - f[8]) + f[5] - (1. / 6.) * uy + 0.5 * ux;
            f[2] = f[6] - (2. / 3.) * uy;
            f[3] = 0.5 * (f[8] - f[4]) + f[7] - (1. / 6.) * uy - 0.5 * ux;
          } else {
            f[7] = 0.5 * (f[4] - f[8]) + f[3] + (1. / 6.) * uy + 0.5 * ux;
            f[6] = f[2] + (2. / 3.) * uy;
            f[5] = 0.5 * (f[8] - f[4]) + f[1] + (1. / 6.) * uy - 0.5 * ux;
          }
        } else if (b->kind == LBM_BC_PRESSURE || b->kind == LBM_BC_PRESSURE_STANDARD) {
          double rho0 = bc_scalar(m, k, t, x, y, z), ux0;
          if (b->kind == LBM_BC_PRESSURE_STANDARD && b->face == LBM_FACE_EAST) {
            ux0 = -1. + (f[0] + f[2] + f[6] + 2. * (f[1] + f[7] + f[8])) / rho0;
            f[4] = f[8] - (2. / 3.) * rho0 * ux0;
            f[3] = f[7] - (1. / 6.) * rho0 * ux0 + 0.5 * (f[6] - f[2]);
            f[5] = f[1] - (1. / 6.) * rho0 * ux0 + 0.5 * (f[2] - f[6]);
          } else if (b->kind == LBM_BC_PRESSURE_STANDARD) {
            ux0 = 1. - (f[0] + f[2] + f[6] + 2. * (f[3] + f[4] + f[5])) / rho0;
            f[1] = f[5] + (1. / 6.) * rho0 * ux0 + 0.5 * (f[6] - f[2]);
            f[7] = f[3] + (1. / 6.) * rho0 * ux0 + 0.5 * (f[2] - f[6]);
            f[8] = f[4] + (2. / 3.) * rho0 * ux0;
          } else if (b->face == LBM_FACE_EAST) {
            ux0 = -rho0 + (f[0] + f[2] + f[6] + 2. * (f[1] + f[7] + f[8]));
            f[4] = f[8] - (2. / 3.) * ux0;
            f[3] = f[7] - (1. / 6.) * ux0 + 0.5 * (f[6] - f[2]);
            f[5] = f[1] - (1. / 6.) * ux0 + 0.5 * (f[2] - f[6]);
          } else if (b->face == LBM_FACE_WEST) {
            ux0 = rho0 - (f[0] + f[2] + f[6] + 2. * (f[3] + f[4] + f[5]));
            f[8] = f[4] + (2. / 3.) * ux0;
            f[7] = f[3] + (1. / 6.) * ux0 + 0.5 * (f[2] - f[6]);
            f[1] = f[5] + (1. / 6.) * ux0 + 0.5 * (f[6] - f[2]);
          } else if (b->face == LBM_FACE_NORTH) {
            double uy0 = -rho0 + (f[0] + f[8] + f[4] + 2. * (f[7] + f[5] + f[6]));
            f[2] = f[6] - (2. / 3.) * uy0;
            f[1] = f[5] - (1. / 6.) * uy0 + 0.5 * (f[4] - f[8]);
            f[3] = f[7] - (1. / 6.) * uy0 + 0.5 * (f[8] - f[4]);
          } else {
            double uy0 = rho0 - (f[0] + f[8] + f[4] + 2. * (f[1] + f[2] + f[3]));
            f[6] = f[2] + (2. / 3.) * uy0;
            f[5] = f[1] + (1. / 6.) * uy0 + 0.5 * (f[8] - f[4]);
            f[7] = f[3] + (1. / 6.) * uy0 + 0.5 * (f[4] - f[8]);
          }
        } else if (b->kind == LBM_BC_TEMPERATURE) {
          /* ThermalZouHeWest2d<.,D2Q5,.> (boundaryConditions/thermalZouHe2d.hh:63-81) */
          double* g = f + 9;
          if (b->face == LBM_FACE_WEST) g[4] = bc_scalar(m, k, t, x, y, z) - g[0] - g[1] - g[2] - g[3];
        }
      }
}

/* IncompressibleHechtVelocityWest3d<D3Q19> (boundaryConditions/Hecht3d.hh:62-94) and
 * IncompressibleHechtPressureEast3d<D3Q19> (Hecht3d.hh:175-209). */
static void hecht3d(const model_t* m, int k, int t, double* F) {
  const lbm_bc* b = &m->cfg.bc[k];
  int Q = m->Q;
  for (int z = b->box[4]; z <= b->box[5]; ++z)
    for (int y = b->box[2]; y <= b->box[3]; ++y)
      for (int x = b->box[0]; x <= b->box[1]; ++x) {
        double* fd = F + (((int64_t)z * m->ny + y) * m->nx + x) * Q;
        if (b->kind == LBM_BC_VELOCITY && b->face == LBM_FACE_WEST) {
          double u[3];
          bc_velocity(m, k, t, x, y, z, u);
          double ux = u[0], uy = u[1], uz = u[2];
          double Nyx = 0.5 * (fd[5] + fd[11] + fd[13] - (fd[2] + fd[4] + fd[14])) - (1. / 3.) * uy;
          double Nzx = 0.5 * (fd[10] + fd[13] + fd[14] - (fd[1] + fd[4] + fd[5])) - (1. / 3.) * uz;
          fd[7] = fd[16] + (1. / 6.) * (ux - uz) + Nzx;
          fd[9] = fd[18] + (1. / 6.) * (ux - uy) + Nyx;
          fd[12] = fd[3] + (1. / 3.) * ux;
          fd[15] = fd[6] + (1. / 6.) * (ux + uz) - Nzx;
          fd[17] = fd[8] + (1. / 6.) * (ux + uy) - Nyx;
        } else if (b->kind == LBM_BC_PRESSURE && b->face == LBM_FACE_EAST) {
          double rho0 = bc_scalar(m, k, t, x, y, z);
          double ux = fd[0] + fd[1] + fd[2] + fd[4] + fd[5] + fd[10] + fd[11] + fd[13] + fd[14] +
                      2. * (fd[7] + fd[9] + fd[12] + fd[15] + fd[17]) - rho0;
          double Nyx = 0.5 * (fd[5] + fd[11] + fd[13] - (fd[2] + fd[4] + fd[14]));
          double Nzx = 0.5 * (fd[10] + fd[13] + fd[14] - (fd[1] + fd[4] + fd[5]));
          fd[3] = fd[12] - (1. / 3.) * ux;
          fd[6] = fd[15] - (1. / 6.) * ux + Nzx;
          fd[8] = fd[17] - (1. / 6.) * ux + Nyx;
          fd[16] = fd[7] - (1. / 6.) * ux - Nzx;
          fd[18] = fd[9] - (1. / 6.) * ux - Nyx;
        }
      }
}

static void apply_bcs(const model_t* m, int t, double* F) {
  for (int k = 0; k < m->cfg.nbc; ++k) {
    if (m->dim == 3)
      hecht3d(m, k, t, F);
    else
      zouhe2d(m, k, t, F);
  }
}

/* Adjoint boundary conditions, applied in reverse order of the forward ones.
 * adjointBoundaryConditions/adjointZouHe2d.cc:5-112, adjointHecht3d.cc:7-80,
 * adjointThermalZouHe2d.hh. */
static void adjoint_bcs(const model_t* m, int t, double* A) {
  (void)t;
  int Q = m->Q;
  for (int k = m->cfg.nbc - 1; k >= 0; --k) {
    const lbm_bc* b = &m->cfg.bc[k];
    for (int z = b->box[4]; z <= b->box[5]; ++z)
      for (int y = b->box[2]; y <= b->box[3]; ++y)
        for (int x = b->box[0]; x <= b->box[1]; ++x) {
          double* a = A + (((int64_t)z * m->ny + y) * m->nx + x) * Q;
          if (m->dim == 3) {
            if (b->kind == LBM_BC_VELOCITY && b->face == LBM_FACE_WEST) {
              a[1] += 0.5 * (a[15] - a[7]);
              a[2] += 0.5 * (a[17] - a[9]);
              a[3] += a[12];
              a[4] += 0.5 * (a[15] + a[17] - (a[7] + a[9]));
              a[5] += 0.5 * (a[9] + a[15] - (a[7] + a[17]));
              a[6] += a[15];
              a[8] += a[17];
              a[10] += 0.5 * (a[7] - a[15]);
              a[11] += 0.5 * (a[9] - a[17]);
              a[13] += 0.5 * (a[7] + a[9] - (a[15] + a[17]));
              a[14] += 0.5 * (a[7] + a[17] - (a[9] + a[15]));
              a[16] += a[7];
              a[18] += a[9];
              a[7] = 0.;
              a[9] = 0.;
              a[12] = 0.;
              a[15] = 0.;
              a[17] = 0.;
            } else if (b->kind == LBM_BC_PRESSURE && b->face == LBM_FACE_EAST) {
              double adjUx = -(1. / 3.) * a[3] - (1. / 6.) * (a[6] + a[8] + a[16] + a[18]);
              a[0] += adjUx;
              a[1] += adjUx + 0.5 * (a[16] - a[6]);
              a[2] += adjUx + 0.5 * (a[18] - a[8]);
              a[4] += adjUx + 0.5 * (a[16] + a[18] - (a[6] + a[8]));
              a[5] += adjUx + 0.5 * (a[8] + a[16] - (a[6] + a[18]));
              a[7] += 2. * adjUx + a[16];
              a[9] += 2. * adjUx + a[18];
              a[10] += adjUx + 0.5 * (a[6] - a[16]);
              a[11] += adjUx + 0.5 * (a[8] - a[18]);
              a[12] += 2. * adjUx + a[3];
              a[13] += adjUx + 0.5 * (a[6] + a[8] - (a[16] + a[18]));
              a[14] += adjUx + 0.5 * (a[6] + a[18] - (a[8] + a[16]));
              a[15] += 2. * adjUx + a[6];
              a[17] += 2. * adjUx + a[8];
              a[3] = 0.;
              a[6] = 0.;
              a[8] = 0.;
              a[16] = 0.;
              a[18] = 0.;
            }
            continue;
          }
          int pres = b->kind == LBM_BC_PRESSURE || b->kind == LBM_BC_PRESSURE_STANDARD;
          if (b->kind == LBM_BC_VELOCITY_STANDARD) {
            /* AdjointStandardZouHeVelocityWest2d (adjointZouHe2d.hh:62-80) */
            double u[3];
            bc_velocity(m, k, t, x, y, z, u);
            double ux = u[0], uy = u[1];
            double adjRho = ((1. / 6) * (ux / (1. - ux)) - 0.5 * (uy / (1. - ux))) * a[1] +
                            ((1. / 6) * (ux / (1. - ux)) + 0.5 * (uy / (1. - ux))) * a[7] +
                            (2. / 3.) * (ux / (1. - ux)) * a[8];
            a[0] += adjRho;
            a[2] += 0.5 * (a[7] - a[1]) + adjRho;
            a[3] += a[7] + 2. * adjRho;
            a[4] += a[8] + 2. * adjRho;
            a[5] += a[1] + 2. * adjRho;
            a[6] += 0.5 * (a[1] - a[7]) + adjRho;
            a[1] = 0.;
            a[7] = 0.;
            a[8] = 0.;
          } else if (b->kind == LBM_BC_VELOCITY && b->face == LBM_FACE_WEST) {
            a[2] += 0.5 * (a[7] - a[1]);
            a[3] += a[7];
            a[4] += a[8];
            a[5] += a[1];
            a[6] += 0.5 * (a[1] - a[7]);
            a[1] = 0.;
            a[7] = 0.;
            a[8] = 0.;
          } else if (b->kind == LBM_BC_VELOCITY && b->face == LBM_FACE_NORTH) {
            a[4] += 0.5 * (a[1] - a[3]);
            a[5] += a[1];
            a[6] += a[2];
            a[7] += a[3];
            a[8] += 0.5 * (a[3] - a[1]);
            a[1] = 0.;
            a[2] = 0.;
            a[3] = 0.;
          } else if (b->kind == LBM_BC_VELOCITY && b->face == LBM_FACE_SOUTH) {
            a[4] += 0.5 * (a[7] - a[5]);
            a[3] += a[7];
            a[2] += a[6];
            a[1] += a[5];
            a[8] += 0.5 * (a[5] - a[7]);
            a[5] = 0.;
            a[6] = 0.;
            a[7] = 0.;
          } else if (b->kind == LBM_BC_VELOCITY && b->face == LBM_FACE_EAST) {
            a[1] += a[5];
            a[2] += 0.5 * (a[5] - a[3]);
            a[6] += 0.5 * (a[3] - a[5]);
            a[7] += a[3];
            a[8] += a[4];
            a[3] = 0.;
            a[4] = 0.;
            a[5] = 0.;
          } else if (pres && b->face == LBM_FACE_EAST) {
            double adjU = -(1. / 6.) * a[3] - (2. / 3.) * a[4] - (1. / 6.) * a[5];
            a[0] += adjU;
            a[1] += 2. * adjU + a[5];
            a[2] += adjU + 0.5 * (a[5] - a[3]);
            a[6] += adjU + 0.5 * (a[3] - a[5]);
            a[7] += 2. * adjU + a[3];
            a[8] += 2. * adjU + a[4];
            a[3] = 0.;
            a[4] = 0.;
            a[5] = 0.;
          } else if (pres && b->face == LBM_FACE_WEST) {
            double adjU = (1. / 6.) * a[1] + (1. / 6.) * a[7] + (2. / 3.) * a[8];
            a[0] -= adjU;
            a[2] -= adjU - 0.5 * (a[7] - a[1]);
            a[3] -= 2. * adjU - a[7];
            a[4] -= 2. * adjU - a[8];
            a[5] -= 2. * adjU - a[1];
            a[6] -= adjU - 0.5 * (a[1] - a[7]);
            a[1] = 0.;
            a[7] = 0.;
            a[8] = 0.;
          } else if (pres && b->face == LBM_FACE_NORTH) {
            double adjU = -(1. / 6.) * a[1] - (2. / 3.) * a[2] - (1. / 6.) * a[3];
            a[0] += adjU;
            a[7] += 2. * adjU + a[3];
            a[8] += adjU + 0.5 * (a[3] - a[1]);
            a[4] += adjU + 0.5 * (a[1] - a[3]);
            a[5] += 2. * adjU + a[1];
            a[6] += 2. * adjU + a[2];
            a[1] = 0.;
            a[2] = 0.;
            a[3] = 0.;
          } else if (pres && b->face == LBM_FACE_SOUTH) {
            double adjU = (1. / 6.) * a[7] + (1. / 6.) * a[5] + (2. / 3.) * a[6];
            a[0] -= adjU;
            a[8] -= adjU - 0.5 * (a[5] - a[7]);
            a[1] -= 2. * adjU - a[5];
            a[2] -= 2. * adjU - a[6];
            a[3] -= 2. * adjU - a[7];
            a[4] -= adjU - 0.5 * (a[7] - a[5]);
            a[5] = 0.;
            a[6] = 0.;
            a[7] = 0.;
          } else if (b->kind == LBM_BC_TEMPERATURE && b->face == LBM_FACE_WEST) {
            double* g = a + 9;
            g[0] -= g[4];
            g[1] -= g[4];
            g[2] -= g[4];
            g[3] -= g[4];
            g[4] = 0.;
          }
        }
  }
}

/* ------------------------------------------------------------------ */
/* Objectives */

static int64_t box_count(const int* b) {
  return (int64_t)(b[1] - b[0] + 1) * (b[3] - b[2] + 1) * (b[5] - b[4] + 1);
}

/* Dissipated power of one cell (no reference counterpart):
 * D = 2*alpha(gamma)*|j|^2 + (9/2) nu omega^2 sum_ab Pneq_ab^2,
 * Pneq_ab = sum_i e_ia e_ib f_i - rho/3 delta_ab - j_a j_b,
 * alpha = 0.5*interp_scale*BP_q(gamma), nu = (1/omega - 1/2)/3. */
static double dissipation_cell(const model_t* m, const double* f, double g, double* dF,
                               double* dG) {
  const lattice_t* L = m->L;
  double mac[4] = {0., 0., 0., 0.};
  if (m->dim == 2)
    macros_d2q9(f, &mac[0], &mac[1], &mac[2]);
  else
    macros_generic(L, f, mac);
  double P[3][3] = {{0.}};
  for (int i = 0; i < L->Q; ++i) {
    int e[3] = {L->ex[i], L->ey[i], L->ez[i]};
    for (int a = 0; a < 3; ++a)
      for (int bb = 0; bb < 3; ++bb) P[a][bb] += e[a] * e[bb] * f[i];
  }
  int D = m->dim;
  for (int a = 0; a < D; ++a) {
    for (int bb = 0; bb < D; ++bb) P[a][bb] -= mac[1 + a] * mac[1 + bb];
    P[a][a] -= mac[0] / 3.;
  }
  double om = m->cfg.omega, nu = (1. / om - 0.5) / 3.;
  double cv = 4.5 * nu * om * om;
  double s2 = 0.;
  for (int a = 0; a < D; ++a)
    for (int bb = 0; bb < D; ++bb) s2 += P[a][bb] * P[a][bb];
  double j2 = mac[1] * mac[1] + mac[2] * mac[2] + mac[3] * mac[3];
  double alpha = pbb_factor(m, g);
  double val = 2. * alpha * j2 + cv * s2;
  if (dF) {
    double tr = 0.;
    for (int a = 0; a < D; ++a) tr += P[a][a];
    for (int i = 0; i < L->Q; ++i) {
      int e[3] = {L->ex[i], L->ey[i], L->ez[i]};
      double pe = 0., pej = 0.;
      for (int a = 0; a < D; ++a)
        for (int bb = 0; bb < D; ++bb) {
          pe += P[a][bb] * e[a] * e[bb];
          pej += P[a][bb] * e[a] * mac[1 + bb];
        }
      double ej = e[0] * mac[1] + e[1] * mac[2] + e[2] * mac[3];
      dF[i] = 4. * alpha * ej + cv * 2. * (pe - tr / 3. - 2. * pej);
    }
  }
  if (dG) *dG = 2. * pbb_factor_diff(m, g) * j2;
  return val;
}

/* F(f_t) times obj_weight.  PressureDrop2d::evaluate (functionals/pressureDrop2d.hh:30-48)
 * with the MPI_Allreduce replaced by the plain sum; ThermalOutflowEast2d::evaluate
 * (functionals/temperatureFlow2d.hh:106-119). */
static double objective(const model_t* m, const double* F, const double* gamma) {
  const lbm_config* c = &m->cfg;
  int Q = m->Q;
  double tc = c->obj_weight;
  if (c->objective == LBM_OBJ_PRESSURE_DROP) {
    double invIn = (double)(1. / box_count(c->obj_in));
    double invOut = (double)(1. / box_count(c->obj_out));
    double ps = 0.;
    const int* b = c->obj_in;
    for (int z = b[4]; z <= b[5]; ++z)
      for (int y = b[2]; y <= b[3]; ++y)
        for (int x = b[0]; x <= b[1]; ++x) {
          double mac[4];
          flow_macros(m, F + (((int64_t)z * m->ny + y) * m->nx + x) * Q, mac);
          ps += tc * invIn * mac[0];
        }
    b = c->obj_out;
    for (int z = b[4]; z <= b[5]; ++z)
      for (int y = b[2]; y <= b[3]; ++y)
        for (int x = b[0]; x <= b[1]; ++x) {
          double mac[4];
          flow_macros(m, F + (((int64_t)z * m->ny + y) * m->nx + x) * Q, mac);
          ps -= tc * invOut * mac[0];
        }
    return ps;
  } else if (c->objective == LBM_OBJ_OUTFLOW) {
    /* OutflowEast2d::evaluate (functionals/outflow2d.hh:15-27) */
    double invOut = (double)(1. / box_count(c->obj_out));
    double of = 0.;
    const int* b = c->obj_out;
    for (int z = b[4]; z <= b[5]; ++z)
      for (int y = b[2]; y <= b[3]; ++y)
        for (int x = b[0]; x <= b[1]; ++x) {
          double mac[4];
          flow_macros(m, F + (((int64_t)z * m->ny + y) * m->nx + x) * Q, mac);
          of -= tc * invOut * mac[1];
        }
    return of;
  } else if (c->objective == LBM_OBJ_THROUGH_FLOW) {
    /* ThroughFlow2d::evaluate (functionals/throughFlow2d.hh:17-40) */
    double invIn = (double)(1. / box_count(c->obj_in));
    double invOut = (double)(1. / box_count(c->obj_out));
    double iif = 0., of = 0.;
    const int* b = c->obj_in;
    for (int z = b[4]; z <= b[5]; ++z)
      for (int y = b[2]; y <= b[3]; ++y)
        for (int x = b[0]; x <= b[1]; ++x) {
          double mac[4];
          flow_macros(m, F + (((int64_t)z * m->ny + y) * m->nx + x) * Q, mac);
          iif -= tc * invIn * mac[1];
        }
    b = c->obj_out;
    for (int z = b[4]; z <= b[5]; ++z)
      for (int y = b[2]; y <= b[3]; ++y)
        for (int x = b[0]; x <= b[1]; ++x) {
          double mac[4];
          flow_macros(m, F + (((int64_t)z * m->ny + y) * m->nx + x) * Q, mac);
          of -= tc * invOut * mac[1];
        }
    return iif + of;
  } else if (c->objective == LBM_OBJ_DOMAIN_TEMPERATURE) {
    /* DomainTemperature2d::evaluate (functionals/domainTemperature2d.hh:13-27) */
    double inv = (double)(1. / box_count(c->obj_out)), pv = 0.;
    const int* b = c->obj_out;
    for (int z = b[4]; z <= b[5]; ++z)
      for (int y = b[2]; y <= b[3]; ++y)
        for (int x = b[0]; x <= b[1]; ++x) {
          const double* f = F + (((int64_t)z * m->ny + y) * m->nx + x) * Q;
          pv += tc * inv * (f[9] + f[10] + f[11] + f[12] + f[13]);
        }
    return pv;
  } else if (c->objective == LBM_OBJ_REGENERATOR_EFFICIENCY) {
    /* RegeneratorEfficiency2d::evaluate (functionals/regeneratorEfficiency2d.hh:16-35) */
    double Ti = c->obj_param[0], Tb = c->obj_param[1], pvn = 0., pvd = 0.;
    const int* b = c->obj_out;
    for (int z = b[4]; z <= b[5]; ++z)
      for (int y = b[2]; y <= b[3]; ++y)
        for (int x = b[0]; x <= b[1]; ++x) {
          int64_t k = ((int64_t)z * m->ny + y) * m->nx + x;
          const double* f = F + k * Q;
          double T = f[9] + f[10] + f[11] + f[12] + f[13];
          pvn += tc * (1. - gamma[k]) * (T - Ti);
          pvd += (1. - gamma[k]) * (Tb - Ti);
        }
    return pvn / pvd;
  } else if (c->objective == LBM_OBJ_HEAT_FLUX) {
    double pout = 0.;
    const int* b = c->obj_out;
    for (int z = b[4]; z <= b[5]; ++z)
      for (int y = b[2]; y <= b[3]; ++y)
        for (int x = b[0]; x <= b[1]; ++x) {
          const double* f = F + (((int64_t)z * m->ny + y) * m->nx + x) * Q;
          double mac[4];
          macros_d2q9(f, &mac[0], &mac[1], &mac[2]);
          double T = f[9] + f[10] + f[11] + f[12] + f[13];
          pout -= tc * mac[1] * T;
        }
    return pout;
  } else if (c->objective == LBM_OBJ_DISSIPATION) {
    double s = 0.;
    for (int64_t k = 0; k < m->ncell; ++k) s += dissipation_cell(m, F + k * Q, gamma[k], 0, 0);
    return tc * s;
  }
  return 0.;
}

/* adjointCollideSource (pressureDrop2d.hh:49-68, temperatureFlow2d.hh:120-142) and
 * adjointSensitivitySource for the dissipation objective. */
static void objective_source(const model_t* m, const double* F, const double* gamma, double* A,
                             double* sens) {
  const lbm_config* c = &m->cfg;
  int Q = m->Q;
  double tc = c->obj_weight;
  if (c->objective == LBM_OBJ_PRESSURE_DROP) {
    double invIn = (double)(1. / box_count(c->obj_in));
    double invOut = (double)(1. / box_count(c->obj_out));
    const int* b = c->obj_in;
    for (int z = b[4]; z <= b[5]; ++z)
      for (int y = b[2]; y <= b[3]; ++y)
        for (int x = b[0]; x <= b[1]; ++x) {
          double* a = A + (((int64_t)z * m->ny + y) * m->nx + x) * Q;
          for (int d = 0; d < m->Qf; ++d) a[d] += invIn * tc;
        }
    b = c->obj_out;
    for (int z = b[4]; z <= b[5]; ++z)
      for (int y = b[2]; y <= b[3]; ++y)
        for (int x = b[0]; x <= b[1]; ++x) {
          double* a = A + (((int64_t)z * m->ny + y) * m->nx + x) * Q;
          for (int d = 0; d < m->Qf; ++d) a[d] -= invOut * tc;
        }
  } else if (c->objective == LBM_OBJ_OUTFLOW) {
    /* OutflowEast2d::adjointCollideSource, incompressible macros (outflow2d.hh:28-40) */
    double invOut = (double)(1. / box_count(c->obj_out));
    const int* b = c->obj_out;
    for (int z = b[4]; z <= b[5]; ++z)
      for (int y = b[2]; y <= b[3]; ++y)
        for (int x = b[0]; x <= b[1]; ++x) {
          double* a = A + (((int64_t)z * m->ny + y) * m->nx + x) * Q;
          for (int d = 0; d < m->Qf; ++d) a[d] -= invOut * tc * m->L->ex[d];
        }
  } else if (c->objective == LBM_OBJ_THROUGH_FLOW) {
    /* ThroughFlow2d::adjointCollideSource, incompressible macros (throughFlow2d.hh:41-59) */
    double invIn = (double)(1. / box_count(c->obj_in));
    double invOut = (double)(1. / box_count(c->obj_out));
    const int* b = c->obj_in;
    for (int z = b[4]; z <= b[5]; ++z)
      for (int y = b[2]; y <= b[3]; ++y)
        for (int x = b[0]; x <= b[1]; ++x) {
          double* a = A + (((int64_t)z * m->ny + y) * m->nx + x) * Q;
          for (int d = 0; d < m->Qf; ++d) a[d] -= invIn * tc * m->L->ex[d];
        }
    b = c->obj_out;
    for (int z = b[4]; z <= b[5]; ++z)
      for (int y = b[2]; y <= b[3]; ++y)
        for (int x = b[0]; x <= b[1]; ++x) {
          double* a = A + (((int64_t)z * m->ny + y) * m->nx + x) * Q;
          for (int d = 0; d < m->Qf; ++d) a[d] -= invOut * tc * m->L->ex[d];
        }
  } else if (c->objective == LBM_OBJ_DOMAIN_TEMPERATURE) {
    /* DomainTemperature2d::adjointCollideSource (domainTemperature2d.hh:28-38) */
    double inv = (double)(1. / box_count(c->obj_out));
    const int* b = c->obj_out;
    for (int z = b[4]; z <= b[5]; ++z)
      for (int y = b[2]; y <= b[3]; ++y)
        for (int x = b[0]; x <= b[1]; ++x) {
          double* a = A + (((int64_t)z * m->ny + y) * m->nx + x) * Q;
          for (int d = 0; d < 5; ++d) a[9 + d] += tc * inv;
        }
  } else if (c->objective == LBM_OBJ_REGENERATOR_EFFICIENCY) {
    /* RegeneratorEfficiency2d::adjointCollideSource / adjointSensitivitySource
     * (regeneratorEfficiency2d.hh:36-88) with timeConst where the derivative of
     * the evaluate puts it: J_t = w N / D, N = sum (1-g)(T - Ti), D = sum (1-g)(Tb - Ti),
     * dJ_t/dT = w (1-g)/D, dJ_t/dg = w ((Tb - Ti) N - (T - Ti) D) / D^2 (the
     * reference divides by w D in the first and leaves w off the (T - Ti) D term in
     * the second, which agree for w = 1 only). */
    double Ti = c->obj_param[0], Tb = c->obj_param[1], vn = 0., vd = 0.;
    const int* b = c->obj_out;
    for (int z = b[4]; z <= b[5]; ++z)
      for (int y = b[2]; y <= b[3]; ++y)
        for (int x = b[0]; x <= b[1]; ++x) {
          int64_t k = ((int64_t)z * m->ny + y) * m->nx + x;
          const double* f = F + k * Q;
          double T = f[9] + f[10] + f[11] + f[12] + f[13];
          vn += (1. - gamma[k]) * (T - Ti);
          vd += (1. - gamma[k]) * (Tb - Ti);
        }
    for (int z = b[4]; z <= b[5]; ++z)
      for (int y = b[2]; y <= b[3]; ++y)
        for (int x = b[0]; x <= b[1]; ++x) {
          int64_t k = ((int64_t)z * m->ny + y) * m->nx + x;
          double* a = A + k * Q;
          const double* f = F + k * Q;
          double T = f[9] + f[10] + f[11] + f[12] + f[13];
          for (int d = 0; d < 5; ++d) a[9 + d] += tc * (1. - gamma[k]) / vd;
          sens[k] += tc * ((Tb - Ti) * vn - (T - Ti) * vd) / (vd * vd);
        }
  } else if (c->objective == LBM_OBJ_HEAT_FLUX) {
    const int* b = c->obj_out;
    for (int z = b[4]; z <= b[5]; ++z)
      for (int y = b[2]; y <= b[3]; ++y)
        for (int x = b[0]; x <= b[1]; ++x) {
          int64_t k = ((int64_t)z * m->ny + y) * m->nx + x;
          const double* f = F + k * Q;
          double* a = A + k * Q;
          double ux = f[1] + f[7] + f[8] - (f[3] + f[4] + f[5]);
          double T = f[9] + f[10] + f[11] + f[12] + f[13];
          for (int d = 0; d < 9; ++d) a[d] -= tc * D2Q9_EX[d] * T;
          for (int d = 0; d < 5; ++d) a[9 + d] -= tc * ux;
        }
  } else if (c->objective == LBM_OBJ_DISSIPATION) {
    double dF[19], dG;
    for (int64_t k = 0; k < m->ncell; ++k) {
      dissipation_cell(m, F + k * Q, gamma[k], dF, &dG);
      for (int d = 0; d < m->Qf; ++d) A[k * Q + d] += tc * dF[d];
      sens[k] += tc * dG;
    }
  }
}

/* ------------------------------------------------------------------ */
/* Driver pieces */

static void init_equilibrium(const model_t* m, const double* macros, double* F) {
  const lattice_t* L = m->L;
  int Q = m->Q, nm = m->nmac;
  for (int64_t k = 0; k < m->ncell; ++k) {
    double rho = 1., u[3] = {0., 0., 0.}, T = 0.;
    if (macros) {
      rho = macros[k * nm + 0];
      u[0] = macros[k * nm + 1];
      u[1] = macros[k * nm + 2];
      if (m->dim == 3) u[2] = macros[k * nm + 3];
      if (m->Qt) T = macros[k * nm + 3];
    }
    /* IncompressibleFeq2d/3d::setAllEquilibria (equilibriumDistributions2d.hh:336-342) */
    double uSqr = (m->dim == 3) ? u[0] * u[0] + u[1] * u[1] + u[2] * u[2] : u[0] * u[0] + u[1] * u[1];
    for (int i = 0; i < L->Q; ++i) {
      double sc = (m->dim == 3) ? L->ex[i] * u[0] + L->ey[i] * u[1] + L->ez[i] * u[2]
                                : L->ex[i] * u[0] + L->ey[i] * u[1];
      F[k * Q + i] = L->w[i] * (rho + 3. * sc + 4.5 * sc * sc - 1.5 * uSqr);
    }
    if (m->Qt) {
      /* ThermalFeq2d<D2Q5>::setAllEquilibria (thermalEquilibriumDistributions2d.hh:18-24) */
      for (int i = 0; i < 5; ++i) {
        double sc = D2Q5_EX[i] * u[0] + D2Q5_EY[i] * u[1];
        F[k * Q + 9 + i] = D2Q5_W[i] * T * (1. + 3. * sc);
      }
    }
  }
}

/* collide(f_t) in place (ObstIsoCollisionLoop2d::execute, isothermalLBLoops2d.hh:37-48) */
static void collide_all(const model_t* m, double* F, const double* gamma) {
  int Q = m->Q;
#pragma omp parallel for schedule(static)
  for (int64_t k = 0; k < m->ncell; ++k) {
    double fout[28], mac[4];
    cell_collide(m, F + k * Q, fout, mac, gamma[k]);
    memcpy(F + k * Q, fout, sizeof(double) * Q);
  }
}

static void copy_par(double* dst, const double* src, int64_t n) {
#pragma omp parallel for schedule(static)
  for (int64_t b = 0; b < (n + 4095) / 4096; ++b) {
    int64_t lo = b * 4096, len = (n - lo < 4096) ? n - lo : 4096;
    memcpy(dst + lo, src + lo, sizeof(double) * len);
  }
}

/* f_{t+1} = BC_{t+1}(stream(collide(f_t))) ; F holds f_t on entry, f_{t+1} on exit. */
static void step(const model_t* m, double* F, double* tmp, const double* gamma, int t) {
  collide_all(m, F, gamma);
  stream_all(m, F, tmp);
  apply_bcs(m, t + 1, tmp);
  copy_par(F, tmp, m->ncell * m->Q);
}

/* One reverse step at f_t (t >= 1): lam holds the adjoint of the post-collision
 * state of step t on entry (adjointGlobal), the one of step t-1 on exit. */
static void adjoint_step(const model_t* m, const double* F, double* lam, double* tmp,
                         const double* gamma, double* sens, int t) {
  int Q = m->Q;
  /* SourceAdjointObstIsoCollisionLoop2d::execute (adjointIsothermalLBLoops2d.hh:297-331) */
#pragma omp parallel for schedule(static)
  for (int64_t k = 0; k < m->ncell; ++k) {
    double li[28], dg = 0.;
    cell_reverse(m, F + k * Q, lam + k * Q, li, gamma[k], &dg);
    memcpy(lam + k * Q, li, sizeof(double) * Q);
    sens[k] += dg;
  }
  /* AdjointLBSolver::computeCollideSource (adjointLBSolver.cc:83-102); none for the
   * steps before the objective window (the regenerator's EmptyFunctional) */
  if (t >= m->obj_from) objective_source(m, F, gamma, lam, sens);
  /* AdjointLBSolver::adjointStream (adjointLBSolver.cc:50-81); f_0 has no boundary */
  if (t >= 1) adjoint_bcs(m, t, lam);
  adjoint_stream_all(m, lam, tmp);
  copy_par(lam, tmp, m->ncell * m->Q);
}

/* ------------------------------------------------------------------ */
/* Public entry points (see lbm_oracle.h) */

int orc_sizes(const lbm_config* cfg, int64_t* ncell, int* npop, int* nmac) {
  model_t m;
  if (model_init(&m, cfg)) return -1;
  if (ncell) *ncell = m.ncell;
  if (npop) *npop = m.Q;
  if (nmac) *nmac = m.nmac;
  return 0;
}

int orc_init(const lbm_config* cfg, const double* macros, double* f0) {
  model_t m;
  if (model_init(&m, cfg)) return -1;
  init_equilibrium(&m, macros, f0);
  return 0;
}

int orc_forward_from(const lbm_config* cfg, const double* gamma, double* f, int t0, int nsteps,
                     double* J_steps, double* J_sum) {
  model_t m;
  if (model_init(&m, cfg)) return -1;
  double* tmp = (double*)malloc(sizeof(double) * m.ncell * m.Q);
  if (!tmp) return -4;
  double acc = 0.;
  for (int s = 0; s < nsteps; ++s) {
    step(&m, f, tmp, gamma, t0 + s);
    double v = objective(&m, f, gamma);
    if (J_steps) J_steps[s] = v;
    acc += v;
  }
  if (J_sum) *J_sum = acc;
  free(tmp);
  return 0;
}

int orc_forward(const lbm_config* cfg, const double* gamma, const double* macros, int nsteps,
                double* f_out, double* J_steps, double* J_sum) {
  if (orc_init(cfg, macros, f_out)) return -1;
  return orc_forward_from(cfg, gamma, f_out, 0, nsteps, J_steps, J_sum);
}

int orc_adjoint_step(const lbm_config* cfg, const double* gamma, const double* f_t, int t,
                     double* lam, double* sens) {
  model_t m;
  if (model_init(&m, cfg)) return -1;
  double* tmp = (double*)malloc(sizeof(double) * m.ncell * m.Q);
  if (!tmp) return -4;
  adjoint_step(&m, f_t, lam, tmp, gamma, sens, t);
  free(tmp);
  return 0;
}

/* Forward + reverse with a two-level store: every k-th state kept, the states
 * of one segment recomputed during the reverse sweep. */
static int gradient_core(model_t* mp, const double* gamma, const double* macros, int nsteps,
                         double* J_sum, double* sens) {
  model_t m = *mp;
  int64_t S = m.ncell * m.Q;
  int k = (int)ceil(sqrt((double)nsteps + 1.));
  if (k < 1) k = 1;
  int nck = nsteps / k + 1;
  double* ck = (double*)malloc(sizeof(double) * S * nck);
  double* seg = (double*)malloc(sizeof(double) * S * (k + 1));
  double* f = (double*)malloc(sizeof(double) * S);
  double* tmp = (double*)malloc(sizeof(double) * S);
  double* lam = (double*)calloc(S, sizeof(double));
  if (!ck || !seg || !f || !tmp || !lam) {
    free(ck); free(seg); free(f); free(tmp); free(lam);
    return -4;
  }
  init_equilibrium(&m, macros, f);
  double acc = 0.;
  for (int t = 0; t < nsteps; ++t) {
    if (t % k == 0) memcpy(ck + (int64_t)(t / k) * S, f, sizeof(double) * S);
    step(&m, f, tmp, gamma, t);
    if (t + 1 >= m.obj_from) acc += objective(&m, f, gamma);
  }
  if (J_sum) *J_sum = acc;
  for (int64_t c = 0; c < m.ncell; ++c) sens[c] = 0.;
  int t = nsteps;
  while (t >= 1) {
    int base = ((t - 1) / k) * k; /* segment start, stored */
    memcpy(seg, ck + (int64_t)(base / k) * S, sizeof(double) * S);
    for (int s = base; s < t; ++s) {
      memcpy(seg + (int64_t)(s - base + 1) * S, seg + (int64_t)(s - base) * S, sizeof(double) * S);
      step(&m, seg + (int64_t)(s - base + 1) * S, tmp, gamma, s);
    }
    for (; t > base; --t) adjoint_step(&m, seg + (int64_t)(t - base) * S, lam, tmp, gamma, sens, t);
  }
  /* The collision of f_0 also depends on the design.  The reference's reverse loop
   * stops at step 1 (applications/RobustPump2d/robustPump2d.cc:268-276) and leaves
   * this term out; it is exactly zero for the isothermal operators when f_0 is a rest
   * state, and is added here so the gradient is the derivative of J. */
  memcpy(seg, ck, sizeof(double) * S);
#pragma omp parallel for schedule(static)
  for (int64_t c = 0; c < m.ncell; ++c) {
    double li[28], dg = 0.;
    cell_reverse(&m, seg + c * m.Q, lam + c * m.Q, li, gamma[c], &dg);
    sens[c] += dg;
  }
  free(ck); free(seg); free(f); free(tmp); free(lam);
  return 0;
}

int orc_gradient(const lbm_config* cfg, const double* gamma, const double* macros, int nsteps,
                 double* J_sum, double* sens) {
  model_t m;
  if (model_init(&m, cfg)) return -1;
  return gradient_core(&m, gamma, macros, nsteps, J_sum, sens);
}

/* The regenerator applications' gradient (applications/Regenerator2d/regenerator2d.cc:
 * 266-387): a steady phase (the largest one-step change of any population, every
 * check_every steps, below tol, or max_steady steps) without objective, then
 * n_unsteady steps with it; the reverse sweep through both.  The steady phase is
 * run once to find its length S and again inside the checkpointed sweep, with
 * LBM_TIME_RAMP ramps starting at S. */
int orc_gradient_steady(const lbm_config* cfg, const double* gamma, const double* macros,
                        int max_steady, int check_every, double tol, int n_unsteady,
                        double* J_sum, double* sens, int* steady_steps) {
  model_t m;
  if (model_init(&m, cfg)) return -1;
  m.t_phase = 2147483647;
  m.obj_from = 1;
  int64_t S = m.ncell * m.Q;
  double* f = (double*)malloc(sizeof(double) * S);
  double* prev = (double*)malloc(sizeof(double) * S);
  double* tmp = (double*)malloc(sizeof(double) * S);
  if (!f || !prev || !tmp) {
    free(f); free(prev); free(tmp);
    return -4;
  }
  init_equilibrium(&m, macros, f);
  int steps = 0;
  while (steps < max_steady) {
    memcpy(prev, f, sizeof(double) * S);
    step(&m, f, tmp, gamma, steps);
    ++steps;
    if (steps % check_every == 0 || steps == max_steady) {
      double mx = 0.;
      for (int64_t i = 0; i < S; ++i) {
        double d = fabs(f[i] - prev[i]);
        if (d > mx || d != d) mx = d;
      }
      if (mx < tol) break;
    }
  }
  free(f); free(prev); free(tmp);
  if (steady_steps) *steady_steps = steps;
  m.t_phase = steps;
  m.obj_from = steps + 1;
  return gradient_core(&m, gamma, macros, steps + n_unsteady, J_sum, sens);
}

int orc_macros(const lbm_config* cfg, const double* f, double* mac) {
  model_t m;
  if (model_init(&m, cfg)) return -1;
  for (int64_t k = 0; k < m.ncell; ++k) {
    double mc[4] = {0., 0., 0., 0.};
    flow_macros(&m, f + k * m.Q, mc);
    if (m.Qt) {
      const double* g = f + k * m.Q + 9;
      mc[3] = g[0] + g[1] + g[2] + g[3] + g[4];
    }
    for (int j = 0; j < m.nmac; ++j) mac[k * m.nmac + j] = mc[j];
  }
  return 0;
}

int orc_collide_cell(const lbm_config* cfg, const double* fin, double gamma, double* fout,
                     double* mac) {
  model_t m;
  if (model_init(&m, cfg)) return -1;
  double mc[4] = {0., 0., 0., 0.};
  cell_collide(&m, fin, fout, mc, gamma);
  if (mac)
    for (int j = 0; j < m.nmac; ++j) mac[j] = mc[j];
  return 0;
}

int orc_reverse_cell(const lbm_config* cfg, const double* fin, double gamma, const double* lam_out,
                     double* lam_in, double* dgamma) {
  model_t m;
  if (model_init(&m, cfg)) return -1;
  double lo[28];
  memcpy(lo, lam_out, sizeof(double) * m.Q);
  double dg = 0.;
  cell_reverse(&m, fin, lo, lam_in, gamma, &dg);
  if (dgamma) *dgamma = dg;
  return 0;
}

int orc_apply_bcs(const lbm_config* cfg, int t, double* f) {
  model_t m;
  if (model_init(&m, cfg)) return -1;
  if (t >= 1) apply_bcs(&m, t, f);
  return 0;
}

int orc_objective(const lbm_config* cfg, const double* f, const double* gamma, double* J) {
  model_t m;
  if (model_init(&m, cfg)) return -1;
  *J = objective(&m, f, gamma);
  return 0;
}

/* ------------------------------------------------------------------ */
/* Wang et al. checkpoint schedule, restated from topOpt/WangCheckpointing.cc:62-162 and
 * topOpt/dynamicCheckpointing.cc:9-54.  The checkpoint list is a doubly linked list of
 * nodes (front = newest).  An erased node keeps its fields and links, and freed nodes are
 * reused oldest-first, which matches what the reference's std::list iterators read. */

#define WANG_MAXLEVEL 2147483647

typedef struct {
  int step, level, slot, prev, next, live;
} wnode;

typedef struct {
  wnode* n;
  int cap, head, nused;
  int* freeq;     /* FIFO of freed node ids */
  int fq_head, fq_tail, fq_len;
  int* avail;     /* stack of free snapshot slots */
  int navail;
  int reader;     /* DynamicCheckpointing::reader */
  int64_t recomputed;
  int* slot_state; /* which state index each slot holds */
} wang_t;

static int wnode_alloc(wang_t* w) {
  if (w->fq_len > 0) {
    int id = w->freeq[w->fq_head];
    w->fq_head = (w->fq_head + 1) % w->cap;
    w->fq_len--;
    return id;
  }
  return w->nused++;
}

static void wnode_free(wang_t* w, int id) {
  w->freeq[w->fq_tail] = id;
  w->fq_tail = (w->fq_tail + 1) % w->cap;
  w->fq_len++;
}

static int wpush_front(wang_t* w, int step, int level, int slot) {
  int id = wnode_alloc(w);
  w->n[id].step = step;
  w->n[id].level = level;
  w->n[id].slot = slot;
  w->n[id].prev = -1;
  w->n[id].next = w->head;
  w->n[id].live = 1;
  if (w->head >= 0) w->n[w->head].prev = id;
  w->head = id;
  return id;
}

static void werase(wang_t* w, int id) {
  int p = w->n[id].prev, nx = w->n[id].next;
  if (p >= 0) w->n[p].next = nx; else w->head = nx;
  if (nx >= 0) w->n[nx].prev = p;
  w->n[id].live = 0;
  wnode_free(w, id);
}

static int wang_make_checkpoint(wang_t* w, int index) {
  if (w->head < 0) {
    int slot = w->avail[--w->navail];
    w->reader = wpush_front(w, index, WANG_MAXLEVEL, slot);
    return slot;
  }
  if (w->navail > 0) {
    int slot = w->avail[--w->navail];
    w->reader = wpush_front(w, index, 0, slot);
    return slot;
  }
  int movable = w->n[w->reader].next;
  if (w->n[movable].level < w->n[w->reader].level) {
    int slot = w->n[movable].slot;
    wpush_front(w, index, 0, slot);
    werase(w, movable);
    return slot;
  }
  int r = w->head;
  int newLevel = w->n[r].level + 1;
  int slot = w->n[r].slot;
  wpush_front(w, index, newLevel, slot);
  werase(w, r);
  w->reader = w->head;
  return slot;
}

static int wang_compute_new(wang_t* w, int index) {
  if (w->head < 0) {
    int slot = w->avail[--w->navail];
    wpush_front(w, 0, WANG_MAXLEVEL, slot);
  }
  int start = w->head, reader = w->head;
  int initStep = w->n[start].step, numSteps = index - initStep;
  for (int ii = initStep; ii < initStep + numSteps; ++ii) {
    if (w->navail > 0) {
      int slot = w->avail[--w->navail];
      wpush_front(w, ii + 1, 0, slot);
      reader = w->head;
      continue;
    }
    int movable = w->n[reader].next;
    if (w->n[movable].level < w->n[reader].level) {
      wpush_front(w, ii + 1, 0, w->n[movable].slot);
      werase(w, movable);
    } else {
      reader = w->head;
      int newLevel = w->n[reader].level + 1;
      wpush_front(w, ii + 1, newLevel, w->n[reader].slot);
      werase(w, reader);
      reader = w->head;
    }
  }
  return start;
}

/* getForwardSolution(index): state values are simulated by integers (the step a slot
 * holds); *ok is cleared if the returned state is not `index`. */
static void wang_get(wang_t* w, int index, int* ok) {
  int init = w->head;
  int value;
  if (w->n[init].step != index) {
    init = wang_compute_new(w, index);
    int cur = w->n[init].step;
    int state = w->slot_state[w->n[init].slot];
    if (state != cur) *ok = 0;
    init = w->n[init].prev;
    for (;;) {
      state += 1; /* advance() */
      cur += 1;
      w->recomputed += 1;
      if (w->n[init].step == cur) {
        if (w->n[init].step == index) break;
        w->slot_state[w->n[init].slot] = state;
        init = w->n[init].prev;
      }
    }
    value = state;
  } else {
    value = w->slot_state[w->n[init].slot];
  }
  if (value != index) *ok = 0;
  w->avail[w->navail++] = w->n[init].slot;
  werase(w, init);
}

int orc_wang_count(int nsteps, int nsnap, int64_t* recomputed, int* ok_out) {
  if (nsnap < 2 || nsteps < 1) return -1;
  wang_t w;
  memset(&w, 0, sizeof(w));
  w.cap = 4 * (nsteps + nsnap) + 16;
  w.n = (wnode*)calloc(w.cap, sizeof(wnode));
  w.freeq = (int*)calloc(w.cap, sizeof(int));
  w.avail = (int*)calloc(nsnap, sizeof(int));
  w.slot_state = (int*)calloc(nsnap, sizeof(int));
  if (!w.n || !w.freeq || !w.avail || !w.slot_state) return -4;
  w.head = -1;
  /* the reference pushes storage[0..K-1] on a stack: top is slot K-1 */
  for (int i = 0; i < nsnap; ++i) w.avail[w.navail++] = i;
  int ok = 1;
  for (int s = 0; s <= nsteps; ++s) {
    int slot = wang_make_checkpoint(&w, s);
    w.slot_state[slot] = s;
  }
  for (int s = nsteps; s >= 1; --s) wang_get(&w, s, &ok);
  *recomputed = w.recomputed;
  if (ok_out) *ok_out = ok;
  free(w.n); free(w.freeq); free(w.avail); free(w.slot_state);
  return 0;
}

/* StaticCheckpointing (topOpt/staticCheckpointing.cc:3-63): the placement the
 * online schedule computes for `nsteps` steps from an empty list
 * (computeNewCheckpoints(numTimestep - 1) with numTimestep = nsteps + 1),
 * recorded oldest first; the forward sweep then saves exactly those states and
 * the reverse sweep is the dynamic one.  *saved = states kept by the sweep. */
int orc_static_count(int nsteps, int nsnap, int64_t* recomputed, int* ok_out, int* saved) {
  if (nsnap < 2 || nsteps < 1) return -1;
  wang_t w;
  int cap = 4 * (nsteps + nsnap) + 16;
  int* plan_step = (int*)calloc(nsnap + 1, sizeof(int));
  int* plan_level = (int*)calloc(nsnap + 1, sizeof(int));
  memset(&w, 0, sizeof(w));
  w.cap = cap;
  w.n = (wnode*)calloc(cap, sizeof(wnode));
  w.freeq = (int*)calloc(cap, sizeof(int));
  w.avail = (int*)calloc(nsnap, sizeof(int));
  w.slot_state = (int*)calloc(nsnap, sizeof(int));
  if (!w.n || !w.freeq || !w.avail || !w.slot_state || !plan_step || !plan_level) return -4;
  w.head = -1;
  for (int i = 0; i < nsnap; ++i) w.avail[w.navail++] = i;
  wang_compute_new(&w, nsteps);
  /* the list from the back (oldest) to the front */
  int nplan = 0, tail = w.head;
  while (tail >= 0 && w.n[tail].next >= 0) tail = w.n[tail].next;
  for (int id = tail; id >= 0 && nplan <= nsnap; id = w.n[id].prev) {
    plan_step[nplan] = w.n[id].step;
    plan_level[nplan] = w.n[id].level;
    ++nplan;
  }
  /* reset: an empty list and all slots free again */
  memset(w.n, 0, cap * sizeof(wnode));
  w.head = -1;
  w.nused = 0;
  w.fq_head = w.fq_tail = w.fq_len = 0;
  w.navail = 0;
  for (int i = 0; i < nsnap; ++i) w.avail[w.navail++] = i;
  w.recomputed = 0;
  int pos = 0;
  for (int s = 0; s <= nsteps; ++s) {
    if (pos < nplan && plan_step[pos] == s) {
      int slot = w.avail[--w.navail];
      wpush_front(&w, s, plan_level[pos], slot);
      w.slot_state[slot] = s;
      ++pos;
    }
  }
  if (saved) *saved = pos;
  int ok = 1;
  for (int s = nsteps; s >= 1; --s) wang_get(&w, s, &ok);
  *recomputed = w.recomputed;
  if (ok_out) *ok_out = ok;
  free(w.n); free(w.freeq); free(w.avail); free(w.slot_state);
  free(plan_step); free(plan_level);
  return 0;
}

/* ------------------------------------------------------------------ */
/* CPU baseline timing: wall time of nsteps forward steps and of nsteps reverse
 * steps of this restatement on nthreads host threads (0 = all). */

static double now_s(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

int orc_time_steps(const lbm_config* cfg, const double* gamma, int nsteps, int nthreads,
                   double* sec_fwd, double* sec_adj) {
  model_t m;
  if (model_init(&m, cfg)) return -1;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
  int64_t S = m.ncell * m.Q;
  double* f = (double*)malloc(sizeof(double) * S);
  double* tmp = (double*)malloc(sizeof(double) * S);
  double* lam = (double*)calloc(S, sizeof(double));
  double* sens = (double*)calloc(m.ncell, sizeof(double));
  if (!f || !tmp || !lam || !sens) {
    free(f); free(tmp); free(lam); free(sens);
    return -4;
  }
  init_equilibrium(&m, NULL, f);
  /* first touch of every buffer outside the timed region, on the threads
   * that use them (fresh pages would otherwise fault inside it) */
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < S; ++i) {
    tmp[i] = 0.;
    lam[i] = 0.;
  }
  memset(sens, 0, sizeof(double) * m.ncell);
  double t0 = now_s();
  for (int t = 0; t < nsteps; ++t) {
    step(&m, f, tmp, gamma, t);
    (void)objective(&m, f, gamma);
  }
  double t1 = now_s();
  for (int t = nsteps; t >= 1; --t) adjoint_step(&m, f, lam, tmp, gamma, sens, t);
  double t2 = now_s();
  if (sec_fwd) *sec_fwd = t1 - t0;
  if (sec_adj) *sec_adj = t2 - t1;
  free(f); free(tmp); free(lam); free(sens);
  return 0;
}

int orc_max_threads(void) {
#ifdef _OPENMP
  return omp_get_num_procs();
#else
  return 1;
#endif
}
