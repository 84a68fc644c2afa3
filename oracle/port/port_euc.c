/*
 * ORACLE -- test infrastructure, never part of the product.
 *
 * C restatement of the Eucclhyd scheme with its remap (eucclhyd_remap/):
 * set-up of Eucclhyd::simulate (EucclhydRemap.cc:273-287), one iteration of
 * Eucclhyd::executeTimeLoopN (EucclhydRemap.cc:84-195), in the reference's
 * operation order.  Corner arrays are indexed (node, slot of the cell in
 * getCellsOfNode); per-cell corner arrays (cell, position of the node in
 * getNodesOfCell), as in the reference.  The two directional remap sweeps
 * are the shared ones of port_remap.c (remap/PhaseRemap1.cc, 2.cc).
 */
#include <float.h>
#include <stdlib.h>
#include <string.h>

#include "port_internal.h"

void port_face_geometry(port_run* R);

typedef struct {
  double *lpc, *nplus, *nminus; /* nn*4*2, constant (Euler mesh) */
  double *lplus, *lminus;       /* nn*4 */
  double *perim;                /* nc */
  double *F_n, *F_np1;          /* nn*4*2 sub-cell forces */
  double *Fe_n, *Fe_np1;        /* nn*4*3*2 per material */
  double *M;                    /* nn*4*4 corner dissipation matrices */
  double *Me;                   /* nn*4*3*4 */
  double *Mp;                   /* nn*4 node dissipation */
  double *G;                    /* nn*2 */
  double *node_f;               /* nn*3 */
  double *cdt;                  /* nc */
  double *p_ex, *pe_ex, *u_ex;  /* nc*4, nc*4*3, nc*4*2 */
  double *pgrad, *pgrad_e;      /* nc*2, nc*3*2 */
  double *vgrad;                /* nc*4 */
  double *lagvol;               /* nc*3 */
  double bcV[4][2];             /* left, right, top, bottom BC values */
} euc_work;

#define W(R) ((euc_work*)(R)->euc)
#define SWAPP(a, b)    \
  do {                 \
    double* t_ = (a);  \
    (a) = (b);         \
    (b) = t_;          \
  } while (0)

static double* zal(size_t n) {
  double* p = (double*)calloc(n ? n : 1, sizeof(double));
  if (!p) abort();
  return p;
}
/* includes/Freefunctions.h: dot accumulates from 0.0, norm = sqrt(dot) */
static inline double dot2(const double* a, const double* b) {
  double r = 0.0;
  r += a[0] * b[0];
  r += a[1] * b[1];
  return r;
}
static inline double nrm(const double* a) { return sqrt(dot2(a, a)); }
static inline double cross(const double* a, const double* b) {
  return a[0] * b[1] - a[1] * b[0];
}
/* MathFunctions::matVectProduct on a row-major 2x2 */
static inline void matvec(const double* m, const double* v, double* o) {
  o[0] = dot2(m, v);
  o[1] = dot2(m + 2, v);
}
/* slot of cell c in getCellsOfNode(p) */
static int node_slot(const port_run* R, long p, long c) {
  long cells[4];
  int loc[4];
  int k = port_node_cells(R, p, cells, loc);
  for (int t = 0; t < k; ++t)
    if (cells[t] == c) return t;
  return -1;
}

/* ----------------------------------------------------------------- set-up */
/* Eucclhyd::computeCornerNormal (PhaseLagrange.cc:27-66) */
static void corner_normal(port_run* R) {
  euc_work* w = W(R);
  for (long c = 0; c < R->nc; ++c) {
    long nd[4];
    port_cell_nodes(R, c, nd);
    for (int k = 0; k < 4; ++k) {
      long p = nd[k], pm = nd[(k + 3) % 4], pp = nd[(k + 1) % 4];
      int t = node_slot(R, p, c);
      const double *xp = R->X0 + 2 * p, *xpp = R->X0 + 2 * pp, *xpm = R->X0 + 2 * pm;
      double np[2] = {0.5 * (xpp[1] - xp[1]), 0.5 * (xp[0] - xpp[0])};
      double lp = nrm(np);
      np[0] = np[0] / lp;
      np[1] = np[1] / lp;
      double nm[2] = {0.5 * (xp[1] - xpm[1]), 0.5 * (xpm[0] - xp[0])};
      double lm = nrm(nm);
      nm[0] = nm[0] / lm;
      nm[1] = nm[1] / lm;
      long q = 4 * p + t;
      w->nplus[2 * q] = np[0];
      w->nplus[2 * q + 1] = np[1];
      w->lplus[q] = lp;
      w->nminus[2 * q] = nm[0];
      w->nminus[2 * q + 1] = nm[1];
      w->lminus[q] = lm;
      w->lpc[2 * q] = np[0] * lp + nm[0] * lm;
      w->lpc[2 * q + 1] = np[1] * lp + nm[1] * lm;
    }
  }
}

/* Eucclhyd::initMeshGeometryForCells (Init.cc:106-166) */
static void cell_geometry(port_run* R) {
  euc_work* w = W(R);
  for (long c = 0; c < R->nc; ++c) {
    long nd[4];
    port_cell_nodes(R, c, nd);
    double r11 = 0.0;
    for (int k = 0; k < 4; ++k)
      r11 = r11 + cross(R->X0 + 2 * nd[k], R->X0 + 2 * nd[(k + 1) % 4]);
    const double vol = 0.5 * r11;
    double r12[2] = {0.0, 0.0};
    for (int k = 0; k < 4; ++k) {
      const double *a = R->X0 + 2 * nd[k], *b = R->X0 + 2 * nd[(k + 1) % 4];
      const double cr = cross(a, b);
      r12[0] = r12[0] + (a[0] + b[0]) * cr;
      r12[1] = r12[1] + (a[1] + b[1]) * cr;
    }
    const double s = 1.0 / (6.0 * vol);
    R->Xc0[2 * c] = r12[0] * s;
    R->Xc0[2 * c + 1] = r12[1] * s;
    R->eulerV[c] = vol;
    double r13 = 0.0;
    for (int k = 0; k < 4; ++k) {
      const double *a = R->X0 + 2 * nd[k], *b = R->X0 + 2 * nd[(k + 1) % 4];
      double d[2] = {a[0] - b[0], a[1] - b[1]};
      r13 = r13 + nrm(d);
    }
    w->perim[c] = r13;
  }
}

/* Eucclhyd::initBoundaryConditions (Init.cc:15-98) */
static int init_bc(port_run* R) {
  const int t = R->s.test_case;
  euc_work* w = W(R);
  /* symmetry values: ey on the left / right, ex on top / bottom */
  const double ex[2] = {1.0, 0.0}, ey[2] = {0.0, 1.0};
  memcpy(w->bcV[0], ey, sizeof ey);
  memcpy(w->bcV[1], ey, sizeof ey);
  memcpy(w->bcV[2], ex, sizeof ex);
  memcpy(w->bcV[3], ex, sizeof ex);
  if (t == 4 || t == 5 || t == 15 || t == 16 || t == 2 || t == 13) {
    R->leftBC = R->rightBC = R->topBC = R->bottomBC = BC_SYM;
  } else if (t == 1 || t == 12 || t == 6 || t == 17) {
    R->leftBC = BC_SYM;
    R->bottomBC = BC_SYM;
    R->rightBC = BC_IMPOSED;
    R->topBC = BC_IMPOSED;
    w->bcV[1][0] = w->bcV[1][1] = 0.0;
    w->bcV[2][0] = w->bcV[2][1] = 0.0;
  } else if (t == 14) {
    /* BiShockBubble (Init.cc:30-46) */
    R->leftBC = BC_SYM;
    R->rightBC = BC_IMPOSED;
    w->bcV[1][0] = -124.824;
    w->bcV[1][1] = 0.0;
    R->rightFluxBC = 1;
    R->topBC = BC_SYM;
    R->bottomBC = BC_SYM;
  } else if (t == 0 || t == 11) {
    /* unit tests: no branch, the Cdl defaults (condition 0) */
    R->leftBC = R->rightBC = R->topBC = R->bottomBC = 0;
  } else {
    port_set_error("Eucclhyd: test case not supported by the restatement");
    return -1;
  }
  return 0;
}

/* Eucclhyd::initCellInternalEnergy, initCellVelocity, initDensity
 * (Init.cc:194-675).  init_variant 3 of BiTriplePoint scales the region
 * limits to a domain of size 7 x 3 (x <= 1, y <= 1.5) and gives material 3
 * density 0.125. */
static int init_state(port_run* R) {
  const int t = R->s.test_case;
  const double* g = R->s.gamma;
  const long nc = R->nc;
  const double xlim = (t == 13 && R->s.init_variant == 3) ? 1.0 : 0.01;
  const double ylim = (t == 13 && R->s.init_variant == 3) ? 1.5 : 0.015;
  const double rho3 = (t == 13 && R->s.init_variant == 3) ? 0.125 : 0.1;
  for (long c = 0; c < nc; ++c)
    for (int m = 0; m < NM; ++m) R->em_n0[NM * c + m] = 0.0;
  for (long c = 0; c < nc; ++c) {
    const double* xc = R->Xc0 + 2 * c;
    double* em = R->em_n0 + NM * c;
    if (t == 4 || t == 5) {
      const double r = (t == 4) ? xc[0] : xc[1];
      double p, rho;
      if (r <= 0.5) { p = 1.0; rho = 1.0; } else { p = 0.1; rho = 0.125; }
      const double e = p / ((g[0] - 1.0) * rho);
      R->e_n0[c] = e;
      em[0] = e;
    } else if (t == 15 || t == 16) {
      const double r = (t == 15) ? xc[0] : xc[1];
      if (r <= 0.5) {
        const double e = 1.0 / ((g[0] - 1.0) * 1.0);
        em[0] = e;
        em[1] = 0.;
        R->e_n0[c] = e;
      } else {
        const double e = 0.1 / ((g[1] - 1.0) * 0.125);
        em[0] = 0.;
        em[1] = e;
        R->e_n0[c] = e;
      }
    } else if (t == 2) {
      double p, rho;
      if (xc[0] <= 0.01) { p = 1.0; rho = 1.0; }
      else if (xc[1] <= 0.015) { p = 0.1; rho = 1.; }
      else { p = 0.1; rho = 0.1; }
      const double e = p / ((g[0] - 1.0) * rho);
      R->e_n0[c] = e;
      em[0] = e;
    } else if (t == 13) {
      if (xc[0] <= xlim) {
        const double e = 1.0 / ((g[0] - 1.0) * 1.0);
        R->e_n0[c] = e;
        em[0] = e;
      } else if (xc[1] <= ylim) {
        const double e = 0.1 / ((g[1] - 1.0) * 1.);
        R->e_n0[c] = e;
        em[1] = e;
      } else {
        const double e = 0.1 / ((g[2] - 1.0) * rho3);
        R->e_n0[c] = e;
        em[2] = e;
      }
    } else if (t == 1 || t == 12) {
      const double e1 = 1.e-6 / ((g[0] - 1.0) * 1.);
      long nd[4];
      port_cell_nodes(R, c, nd);
      int centre = 0;
      for (int k = 0; k < 4; ++k)
        if (nrm(R->X0 + 2 * nd[k]) < R->s.threshold) centre = 1;
      R->e_n0[c] = centre ? e1 + 0.244816 / (R->s.dx * R->s.dy) : e1;
      em[0] = R->e_n0[c];
    } else if (t == 14) {
      /* air everywhere, then the bubble (Init.cc:272-302) */
      double e = 1.e5 / ((g[0] - 1.0) * 1.0);
      em[0] = e;
      em[1] = 0.;
      R->e_n0[c] = e;
      const double r = sqrt((xc[0] - 0.320) * (xc[0] - 0.320) + (xc[1] - 0.04) * (xc[1] - 0.04));
      if (r <= 0.025) {
        e = 1.e5 / ((g[0] - 1.0) * 0.182);
        em[0] = 0.;
        em[1] = e;
        R->e_n0[c] = e;
      }
    } else if (t == 6 || t == 17 || t == 0 || t == 11) {
      /* Init.cc:202-214 */
      const double p0 = 1., rho0 = 1., gamma = 1.4;
      const double e0 = p0 / ((gamma - 1.0) * rho0);
      R->e_n0[c] = e0;
      for (int m = 0; m < NM; ++m) em[m] = e0;
    }
    /* initCellVelocity (Init.cc:391-421) */
    R->cell_u_n0[2 * c] = 0.0;
    R->cell_u_n0[2 * c + 1] = 0.0;
    if (t == 6 || t == 17) {
      const double u0 = 0.;
      const double n1 = xc[0], n2 = xc[1];
      const double nv = sqrt(n1 * n1 + n2 * n2);
      R->cell_u_n0[2 * c] = -u0 * n1 / nv;
      R->cell_u_n0[2 * c + 1] = -u0 * n2 / nv;
    } else if (t == 14) {
      if (xc[0] >= 0.60) R->cell_u_n0[2 * c] = -124.824;
    } else if (t == 0 || t == 11) {
      R->cell_u_n0[2 * c] = 1.0;
    }
  }
  /* initDensity */
  for (long c = 0; c < nc; ++c) {
    double *f = R->fm + NM * c, *mf = R->mfm + NM * c, *rm = R->rhom_n0 + NM * c;
    for (int m = 0; m < NM; ++m) f[m] = mf[m] = rm[m] = 0.0;
    const double* xc = R->Xc0 + 2 * c;
    if (t == 4 || t == 5) {
      f[0] = 1.; f[1] = 0.; mf[0] = 1.; mf[1] = 0.;
      const double r = (t == 4) ? xc[0] : xc[1];
      if (r <= 0.5) { R->rho_n0[c] = 1.0; rm[0] = 1.0; rm[1] = 1.0; }
      else { R->rho_n0[c] = 0.125; rm[0] = 0.125; rm[1] = 0.125; }
    } else if (t == 15 || t == 16) {
      const double r = (t == 15) ? xc[0] : xc[1];
      if (r <= 0.5) {
        f[0] = 1.; f[1] = 0.; mf[0] = 1.; mf[1] = 0.;
        R->rho_n0[c] = 1.0; rm[0] = 1.0; rm[1] = 0.;
      } else {
        f[0] = 0.; f[1] = 1.; mf[0] = 0.; mf[1] = 1.;
        R->rho_n0[c] = 0.125; rm[0] = 0.; rm[1] = 0.125;
      }
    } else if (t == 2) {
      f[0] = 1.; f[1] = 0.; mf[0] = 1.; mf[1] = 0.;
      if (xc[0] <= 0.01) R->rho_n0[c] = 1.0;
      else if (xc[1] <= 0.015) R->rho_n0[c] = 1.0;
      else R->rho_n0[c] = 0.1;
    } else if (t == 13) {
      if (xc[0] <= xlim) {
        R->rho_n0[c] = 1.0; f[0] = 1.; mf[0] = 1.; rm[0] = 1.0;
      } else if (xc[1] <= ylim) {
        R->rho_n0[c] = 1.0; f[1] = 1.; mf[1] = 1.; rm[1] = 1.0;
      } else {
        R->rho_n0[c] = rho3; f[2] = 1.; mf[2] = 1.; rm[2] = rho3;
      }
    } else if (t == 1) {
      R->rho_n0[c] = 1.0;
      rm[0] = 1.0;
    } else if (t == 14) {
      /* Init.cc:528-560 */
      rm[0] = 1.0;
      R->rho_n0[c] = 1.0;
      f[0] = 1.; f[1] = 0.; mf[0] = 1.; mf[1] = 0.;
      const double r = sqrt((xc[0] - 0.320) * (xc[0] - 0.320) + (xc[1] - 0.04) * (xc[1] - 0.04));
      if (r <= 0.025) {
        rm[0] = 0.0; rm[1] = 0.182; R->rho_n0[c] = 0.182;
        f[0] = 0.; f[1] = 1.; mf[0] = 0.; mf[1] = 1.;
      }
    } else if (t == 0 || t == 11) {
      /* Init.cc:438-480 */
      if (t == 0 || xc[0] <= 0.5) {
        f[0] = 1.; f[1] = 0.; mf[0] = 1.; mf[1] = 0.;
        R->rho_n0[c] = 1.0; rm[0] = 1.0; rm[1] = 0.;
      } else {
        f[0] = 0.; f[1] = 1.; mf[0] = 0.; mf[1] = 1.;
        R->rho_n0[c] = 1.; rm[0] = 0.; rm[1] = 1.0;
      }
    }
    if (R->nbmat == 1) {
      f[0] = 1.; f[1] = 0.; f[2] = 0.;
      mf[0] = 1.; mf[1] = 0.; mf[2] = 0.;
    }
    int matcell = 0, imatpure = -1;
    for (int m = 0; m < NM; ++m)
      if (f[m] > R->s.threshold) {
        matcell++;
        imatpure = m;
      }
    if (matcell > 1) {
      R->mixte[c] = 1;
      R->pure[c] = -1;
    } else {
      R->mixte[c] = 0;
      R->pure[c] = imatpure;
    }
  }
  return 0;
}

int port_euc_setup(port_run* R) {
  const long nc = R->nc, nn = R->nn;
  euc_work* w = (euc_work*)calloc(1, sizeof(euc_work));
  R->euc = w;
  w->lpc = zal(8 * nn); w->nplus = zal(8 * nn); w->nminus = zal(8 * nn);
  w->lplus = zal(4 * nn); w->lminus = zal(4 * nn); w->perim = zal(nc);
  w->F_n = zal(8 * nn); w->F_np1 = zal(8 * nn);
  w->Fe_n = zal(24 * nn); w->Fe_np1 = zal(24 * nn);
  w->M = zal(16 * nn); w->Me = zal(48 * nn); w->Mp = zal(4 * nn); w->G = zal(2 * nn);
  w->node_f = zal(3 * nn); w->cdt = zal(nc);
  w->p_ex = zal(4 * nc); w->pe_ex = zal(12 * nc); w->u_ex = zal(8 * nc);
  w->pgrad = zal(2 * nc); w->pgrad_e = zal(6 * nc); w->vgrad = zal(4 * nc);
  w->lagvol = zal(3 * nc);
  if (!R->cell_u_n) {
    R->cell_u_n = zal(2 * nc); R->cell_u_np1 = zal(2 * nc); R->cell_u_n0 = zal(2 * nc);
    R->pres = zal(nc); R->sound = zal(nc); R->pres_m = zal(NM * nc);
    R->sound_m = zal(NM * nc);
  }
  /* Eucclhyd::simulate set-up order (EucclhydRemap.cc:273-287) */
  corner_normal(R);
  cell_geometry(R);
  if (init_bc(R)) return -1;
  if (init_state(R)) return -1;
  port_face_geometry(R);  /* initMeshGeometryForFaces, on the centroids */
  /* setUpTimeLoopN (Init.cc:721-781) */
  memcpy(R->rho_n, R->rho_n0, nc * sizeof(double));
  memcpy(R->rhom_n, R->rhom_n0, NM * nc * sizeof(double));
  memcpy(R->cell_u_n, R->cell_u_n0, 2 * nc * sizeof(double));
  memcpy(R->e_n, R->e_n0, nc * sizeof(double));
  memcpy(R->em_n, R->em_n0, NM * nc * sizeof(double));
  const int t = R->s.test_case;
  if (t == 2 || t == 13)
    R->dt_init = 1.0e-5;
  else if (t == 14)
    R->dt_init = 1.0e-7;
  else if (t == 0 || t == 11)
    R->dt_init = 0.0; /* no branch: the value-initialised deltat_n */
  else
    R->dt_init = 1.0e-4;
  R->dt_n = R->dt_init;
  return 0;
}

void port_euc_free(port_run* R) {
  euc_work* w = W(R);
  if (!w) return;
  double* ptrs[] = {w->lpc, w->nplus, w->nminus, w->lplus, w->lminus, w->perim,
                    w->F_n, w->F_np1, w->Fe_n, w->Fe_np1, w->M, w->Me, w->Mp,
                    w->G, w->node_f, w->cdt, w->p_ex, w->pe_ex, w->u_ex,
                    w->pgrad, w->pgrad_e, w->vgrad, w->lagvol};
  for (size_t k = 0; k < sizeof ptrs / sizeof ptrs[0]; ++k) free(ptrs[k]);
  free(w);
  R->euc = NULL;
}

/* ------------------------------------------------------------ one cycle */
/* Eucclhyd::nodeVelocityBoundaryCondition (ConditionsLimites.cc:109-123) */
static void bc_velocity(int bc, const double* V, const double* Mp, const double* Gp,
                        double* out) {
  if (bc == BC_SYM) {
    double mv[2];
    matvec(Mp, V, mv);
    const double s = dot2(Gp, V) / dot2(mv, V);
    out[0] = V[0] * s;
    out[1] = V[1] * s;
  } else if (bc == BC_IMPOSED) {
    out[0] = V[0];
    out[1] = V[1];
  } else if (bc == BC_FREE) {
    const double alpha = 1.0 / (Mp[0] * Mp[3] - Mp[1] * Mp[2]);
    const double inv[4] = {Mp[3] * alpha, -Mp[1] * alpha, -Mp[2] * alpha, Mp[0] * alpha};
    matvec(inv, Gp, out);
  } else {
    out[0] = out[1] = 0.0;
  }
}
/* nodeVelocityBoundaryConditionCorner (ConditionsLimites.cc:125-145) */
static void bc_corner(int bc1, const double* V1, int bc2, const double* V2,
                      const double* Mp, const double* Gp, double* out) {
  out[0] = out[1] = 0.0;
  if (bc1 == BC_SYM && bc2 == BC_SYM) {
    if (fabs(fabs(dot2(V1, V2)) - nrm(V1) * nrm(V2)) < 1.0E-8)
      bc_velocity(BC_SYM, V1, Mp, Gp, out);
  } else if (bc1 == BC_IMPOSED && bc2 == BC_IMPOSED) {
    out[0] = 0.5 * (V1[0] + V2[0]);
    out[1] = 0.5 * (V1[1] + V2[1]);
  } else if (bc1 == BC_FREE && bc2 == BC_FREE) {
    bc_velocity(BC_FREE, V1, Mp, Gp, out);
  }
}

void port_euc_cycle(port_run* R) {
  euc_work* w = W(R);
  const int nb = R->nbmat;
  const long nc = R->nc, nn = R->nn;
  const double thr = R->s.threshold;
  R->n++;
  /* computeEOS (PhaseLagrange.cc:70-98) */
  for (int m = 0; m < nb; ++m) {
    const double gm = R->s.gamma[m];
    for (long c = 0; c < nc; ++c) {
      const long k = NM * c + m;
      if (R->s.eos[m] == HYDRO_EOS_PERFECT_GAS) {
        R->pres_m[k] = (gm - 1.0) * R->rhom_n[k] * R->em_n[k];
        if (R->rhom_n[k] > 0.)
          R->sound_m[k] = sqrt(gm * R->pres_m[k] / R->rhom_n[k]);
        else
          R->sound_m[k] = 1.e-20;
      } else if (R->s.eos[m] == HYDRO_EOS_VOID) {
        R->pres_m[k] = 0.;
        R->sound_m[k] = 1.e-20;
      }
    }
  }
  /* computePressionMoyenne (:139-155) */
  for (long c = 0; c < nc; ++c) {
    R->pres[c] = 0.;
    for (int m = 0; m < nb; ++m) {
      R->pres[c] += R->fm[NM * c + m] * R->pres_m[NM * c + m];
      R->sound[c] = smax(R->sound[c], R->sound_m[NM * c + m]);
    }
    if (R->rho_n[c] > 0.)
      R->sound[c] = sqrt(R->s.gamma[0] * R->pres[c] / R->rho_n[c]);
  }
  /* computeGradients (:160-246) */
  for (long p = 0; p < nn; ++p) {
    long cells[4];
    int loc[4];
    int kc = port_node_cells(R, p, cells, loc);
    for (int m = 0; m < nb; ++m) w->node_f[3 * p + m] = 0.;
    for (int t = 0; t < kc; ++t)
      for (int m = 0; m < nb; ++m)
        w->node_f[3 * p + m] += R->fm[NM * cells[t] + m] * 0.25;
  }
  if (R->s.space_order == 2) {
    for (long c = 0; c < nc; ++c) {
      long nd[4];
      port_cell_nodes(R, c, nd);
      double r14[4] = {0.0, 0.0, 0.0, 0.0};
      for (int k = 0; k < 4; ++k) {
        const long p = nd[k];
        const int t = node_slot(R, p, c);
        const double* u = R->u_n + 2 * p;
        const double* l = w->lpc + 2 * (4 * p + t);
        r14[0] = r14[0] + u[0] * l[0];
        r14[1] = r14[1] + u[0] * l[1];
        r14[2] = r14[2] + u[1] * l[0];
        r14[3] = r14[3] + u[1] * l[1];
      }
      const double V = R->eulerV[c];
      for (int q = 0; q < 4; ++q) w->vgrad[4 * c + q] = r14[q] / V;
      double r15[2] = {0.0, 0.0}, r15e[3][2] = {{0.0, 0.0}, {0.0, 0.0}, {0.0, 0.0}};
      for (int k = 0; k < 4; ++k) {
        const long p = nd[k];
        const int t = node_slot(R, p, c);
        const double* F = w->F_n + 2 * (4 * p + t);
        r15[0] = r15[0] + F[0];
        r15[1] = r15[1] + F[1];
        for (int m = 0; m < 3; ++m) {
          const double* Fe = w->Fe_n + 2 * (3 * (4 * p + t) + m);
          r15e[m][0] = r15e[m][0] + Fe[0];
          r15e[m][1] = r15e[m][1] + Fe[1];
        }
      }
      w->pgrad[2 * c] = r15[0] / V;
      w->pgrad[2 * c + 1] = r15[1] / V;
      for (int m = 0; m < 3; ++m) {
        w->pgrad_e[2 * (3 * c + m)] = r15e[m][0] / V;
        w->pgrad_e[2 * (3 * c + m) + 1] = r15e[m][1] / V;
      }
    }
  }
  /* computeMass (:251-261) */
  for (long c = 0; c < nc; ++c) {
    R->cell_mass[c] = R->rho_n[c] * R->eulerV[c];
    for (int m = 0; m < nb; ++m)
      R->cell_mass_m[NM * c + m] = R->mfm[NM * c + m] * R->cell_mass[c];
  }
  /* computeDissipationMatrix (:266-297) */
  for (long p = 0; p < nn; ++p) {
    long cells[4];
    int loc[4];
    int kc = port_node_cells(R, p, cells, loc);
    for (int t = 0; t < kc; ++t) {
      const long c = cells[t], q = 4 * p + t;
      const double *np = w->nplus + 2 * q, *nm = w->nminus + 2 * q;
      const double lp = w->lplus[q], lm = w->lminus[q];
      double cm[4];
      for (int i = 0; i < 2; ++i)
        for (int j = 0; j < 2; ++j)
          cm[2 * i + j] = (np[i] * np[j]) * lp + (nm[i] * nm[j]) * lm;
      const double s = R->rho_n[c] * R->sound[c];
      for (int e = 0; e < 4; ++e) w->M[4 * q + e] = cm[e] * s;
      for (int m = 0; m < 3; ++m) {
        const double se = R->rhom_n[NM * c + m] * R->sound[c];
        for (int e = 0; e < 4; ++e) w->Me[4 * (3 * q + m) + e] = cm[e] * se;
      }
    }
  }
  /* computem_cell_deltat (:302-316) */
  for (long c = 0; c < nc; ++c) {
    if (R->s.projection == 1)
      w->cdt[c] = R->eulerV[c] / (w->perim[c] * (nrm(R->cell_u_n + 2 * c) + R->sound[c]));
    else
      w->cdt[c] = R->eulerV[c] / (w->perim[c] * R->sound[c]);
  }
  /* extrapolateValue (:322-479) */
  if (R->s.space_order == 1) {
    for (long c = 0; c < nc; ++c)
      for (int k = 0; k < 4; ++k) {
        w->u_ex[2 * (4 * c + k)] = R->cell_u_n[2 * c];
        w->u_ex[2 * (4 * c + k) + 1] = R->cell_u_n[2 * c + 1];
        w->p_ex[4 * c + k] = R->pres[c];
        for (int m = 0; m < nb; ++m)
          w->pe_ex[3 * (4 * c + k) + m] = R->pres_m[NM * c + m];
      }
  } else {
    for (long p = 0; p < nn; ++p) {
      long cells[4];
      int loc[4];
      int kc = port_node_cells(R, p, cells, loc);
      double minP[4], maxP[4], minV[2], maxV[2];
      for (int q = 0; q < 4; ++q) {
        minP[q] = DBL_MAX;
        maxP[q] = DBL_MIN;
      }
      for (int t = 0; t < kc; ++t) {
        const long d = cells[t];
        minP[0] = smin(minP[0], R->pres[d]);
        for (int m = 0; m < 3; ++m) minP[1 + m] = smin(minP[1 + m], R->pres_m[NM * d + m]);
      }
      for (int t = 0; t < kc; ++t) {
        const long d = cells[t];
        maxP[0] = smax(maxP[0], R->pres[d]);
        for (int m = 0; m < 3; ++m) maxP[1 + m] = smax(maxP[1 + m], R->pres_m[NM * d + m]);
      }
      minV[0] = DBL_MAX;
      for (int t = 0; t < kc; ++t) minV[0] = smin(minV[0], R->cell_u_n[2 * cells[t]]);
      maxV[0] = DBL_MIN;
      for (int t = 0; t < kc; ++t) maxV[0] = smax(maxV[0], R->cell_u_n[2 * cells[t]]);
      minV[1] = DBL_MAX;
      for (int t = 0; t < kc; ++t) minV[1] = smin(minV[1], R->cell_u_n[2 * cells[t] + 1]);
      maxV[1] = DBL_MIN;
      for (int t = 0; t < kc; ++t) maxV[1] = smax(maxV[1], R->cell_u_n[2 * cells[t] + 1]);
      for (int t = 0; t < kc; ++t) {
        const long c = cells[t];
        const int k = loc[t];
        const double dxp[2] = {R->X0[2 * p] - R->Xc0[2 * c],
                               R->X0[2 * p + 1] - R->Xc0[2 * c + 1]};
        double* pe = w->pe_ex + 3 * (4 * c + k);
        for (int m = 0; m < 3; ++m) {
          const double pt = R->pres_m[NM * c + m] + dot2(w->pgrad_e + 2 * (3 * c + m), dxp);
          pe[m] = smax(smin(maxP[1 + m], pt), minP[1 + m]);
        }
        w->p_ex[4 * c + k] = 0.;
        for (int m = 0; m < nb; ++m) w->p_ex[4 * c + k] += R->fm[NM * c + m] * pe[m];
        double mv[2];
        matvec(w->vgrad + 4 * c, dxp, mv);
        const double Vt[2] = {R->cell_u_n[2 * c] + mv[0], R->cell_u_n[2 * c + 1] + mv[1]};
        w->u_ex[2 * (4 * c + k)] = smax(smin(maxV[0], Vt[0]), minV[0]);
        w->u_ex[2 * (4 * c + k) + 1] = smax(smin(maxV[1], Vt[1]), minV[1]);
      }
    }
  }
  /* computeG, computeNodeDissipationMatrixAndG (:484-527) */
  for (long p = 0; p < nn; ++p) {
    long cells[4];
    int loc[4];
    int kc = port_node_cells(R, p, cells, loc);
    double r1[2] = {0.0, 0.0};
    double r0[4] = {0.0, 0.0, 0.0, 0.0};
    for (int t = 0; t < kc; ++t) {
      const long c = cells[t], q = 4 * p + t;
      const int k = loc[t];
      double mv[2];
      matvec(w->M + 4 * q, w->u_ex + 2 * (4 * c + k), mv);
      const double pe = w->p_ex[4 * c + k];
      const double* l = w->lpc + 2 * q;
      r1[0] = r1[0] + (mv[0] + l[0] * pe);
      r1[1] = r1[1] + (mv[1] + l[1] * pe);
    }
    for (int t = 0; t < kc; ++t)
      for (int e = 0; e < 4; ++e) r0[e] = r0[e] + w->M[4 * (4 * p + t) + e];
    w->G[2 * p] = r1[0];
    w->G[2 * p + 1] = r1[1];
    for (int e = 0; e < 4; ++e) w->Mp[4 * p + e] = r0[e];
  }
  /* computedeltat (EucclhydRemap.cc:203-221) */
  {
    double red = DBL_MAX;
    for (long c = 0; c < nc; ++c)
      if (w->cdt[c] < red) red = w->cdt[c];
    R->dt_np1 = smin(R->s.cfl * red, R->dt_n * 1.05);
    if (R->dt_np1 < R->s.dt_min) {
      R->err |= HYDRO_ERR_DT_MIN;
      R->done = 1;
      return;
    }
  }
  /* computeBoundaryNodeVelocities (ConditionsLimites.cc:19-107) */
  const double *VL = w->bcV[0], *VR = w->bcV[1], *VT = w->bcV[2], *VB = w->bcV[3];
  for (long i = 0; i <= R->ny; ++i) {
    long p = port_nid(R, i, 0);
    bc_velocity(R->leftBC, VL, w->Mp + 4 * p, w->G + 2 * p, R->u_np1 + 2 * p);
  }
  for (long i = 0; i <= R->ny; ++i) {
    long p = port_nid(R, i, R->nx);
    bc_velocity(R->rightBC, VR, w->Mp + 4 * p, w->G + 2 * p, R->u_np1 + 2 * p);
  }
  for (long j = 0; j <= R->nx; ++j) {
    long p = port_nid(R, R->ny, j);
    bc_velocity(R->topBC, VT, w->Mp + 4 * p, w->G + 2 * p, R->u_np1 + 2 * p);
  }
  for (long j = 0; j <= R->nx; ++j) {
    long p = port_nid(R, 0, j);
    bc_velocity(R->bottomBC, VB, w->Mp + 4 * p, w->G + 2 * p, R->u_np1 + 2 * p);
  }
  {
    long p = port_nid(R, R->ny, 0);
    bc_corner(R->topBC, VT, R->leftBC, VL, w->Mp + 4 * p, w->G + 2 * p, R->u_np1 + 2 * p);
    p = port_nid(R, R->ny, R->nx);
    bc_corner(R->topBC, VT, R->rightBC, VR, w->Mp + 4 * p, w->G + 2 * p, R->u_np1 + 2 * p);
    p = port_nid(R, 0, 0);
    bc_corner(R->bottomBC, VB, R->leftBC, VL, w->Mp + 4 * p, w->G + 2 * p, R->u_np1 + 2 * p);
    p = port_nid(R, 0, R->nx);
    bc_corner(R->bottomBC, VB, R->rightBC, VR, w->Mp + 4 * p, w->G + 2 * p, R->u_np1 + 2 * p);
  }
  /* computeNodeVelocity (:532-543): inner nodes, inverse(Mp) . G */
  for (long i = 1; i < R->ny; ++i)
    for (long j = 1; j < R->nx; ++j) {
      const long p = port_nid(R, i, j);
      const double* a = w->Mp + 4 * p;
      const double alpha = 1.0 / (a[0] * a[3] - a[1] * a[2]);
      const double inv[4] = {a[3] * alpha, -a[1] * alpha, -a[2] * alpha, a[0] * alpha};
      matvec(inv, w->G + 2 * p, R->u_np1 + 2 * p);
    }
  /* updateTime */
  R->t_np1 = R->t_n + R->dt_np1;
  /* computeFaceVelocity (:548-568) */
  for (long f = 0; f < R->nf; ++f) {
    face_info F;
    port_face_decode(R, f, &F);
    const double *u1 = R->u_np1 + 2 * F.n1, *u2 = R->u_np1 + 2 * F.n2;
    double r5[2] = {(0.0 + u1[0]) + u2[0], (0.0 + u1[1]) + u2[1]};
    const double h[2] = {r5[0] * 0.5, r5[1] * 0.5};
    R->fnv[f] = dot2(h, R->fN + 2 * f);
  }
  /* computeLagrangePosition (:573-620) */
  for (long p = 0; p < nn; ++p) {
    R->XL[2 * p] = R->X0[2 * p] + R->u_np1[2 * p] * R->dt_n;
    R->XL[2 * p + 1] = R->X0[2 * p + 1] + R->u_np1[2 * p + 1] * R->dt_n;
  }
  for (long f = 0; f < R->nf; ++f) {
    face_info F;
    port_face_decode(R, f, &F);
    const double *a = R->XL + 2 * F.n1, *b = R->XL + 2 * F.n2;
    R->XfL[2 * f] = (a[0] + b[0]) * 0.5;
    R->XfL[2 * f + 1] = (a[1] + b[1]) * 0.5;
    const double v[2] = {b[0] - a[0], b[1] - a[1]};
    R->fLL[f] = nrm(v);
  }
  /* computeSubCellForce (:625-666) */
  for (long p = 0; p < nn; ++p) {
    long cells[4];
    int loc[4];
    int kc = port_node_cells(R, p, cells, loc);
    for (int t = 0; t < kc; ++t) {
      const long c = cells[t], q = 4 * p + t;
      const int k = loc[t];
      const double* l = w->lpc + 2 * q;
      const double* ue = w->u_ex + 2 * (4 * c + k);
      const double du[2] = {R->u_np1[2 * p] - ue[0], R->u_np1[2 * p + 1] - ue[1]};
      double mv[2];
      const double mp = -w->p_ex[4 * c + k];
      matvec(w->M + 4 * q, du, mv);
      w->F_np1[2 * q] = l[0] * mp + mv[0];
      w->F_np1[2 * q + 1] = l[1] * mp + mv[1];
      for (int m = 0; m < 3; ++m) {
        const double mpe = -w->pe_ex[3 * (4 * c + k) + m];
        matvec(w->Me + 4 * (3 * q + m), du, mv);
        w->Fe_np1[2 * (3 * q + m)] = l[0] * mpe + mv[0];
        w->Fe_np1[2 * (3 * q + m) + 1] = l[1] * mpe + mv[1];
      }
    }
  }
  /* computeLagrangeVolumeAndCenterOfGravity (:671-716) */
  for (long c = 0; c < nc; ++c) {
    long nd[4];
    port_cell_nodes(R, c, nd);
    double r6 = 0.0;
    for (int k = 0; k < 4; ++k)
      r6 = r6 + cross(R->XL + 2 * nd[k], R->XL + 2 * nd[(k + 1) % 4]);
    const double vol = 0.5 * r6;
    R->vL[c] = vol;
    for (int m = 0; m < nb; ++m) w->lagvol[3 * c + m] = R->fm[NM * c + m] * vol;
    double r7[2] = {0.0, 0.0};
    for (int k = 0; k < 4; ++k) {
      const double *a = R->XL + 2 * nd[k], *b = R->XL + 2 * nd[(k + 1) % 4];
      const double cr = cross(a, b);
      r7[0] = r7[0] + (a[0] + b[0]) * cr;
      r7[1] = r7[1] + (a[1] + b[1]) * cr;
    }
    const double s = 1.0 / (6.0 * vol);
    R->XcL[2 * c] = r7[0] * s;
    R->XcL[2 * c + 1] = r7[1] * s;
  }
  /* computeFacedeltaxLagrange (:721-741) */
  for (long f = 0; f < R->nf; ++f) {
    face_info F;
    port_face_decode(R, f, &F);
    if (F.front < 0) continue;
    const double d[2] = {R->XcL[2 * F.front] - R->XcL[2 * F.back],
                         R->XcL[2 * F.front + 1] - R->XcL[2 * F.back + 1]};
    R->dxL[f] = dot2(d, R->fN + 2 * f);
  }
  /* updateCellCenteredLagrangeVariables (:746-1010) */
  for (long c = 0; c < nc; ++c) {
    long nd[4];
    port_cell_nodes(R, c, nd);
    int slot[4];
    for (int k = 0; k < 4; ++k) slot[k] = node_slot(R, nd[k], c);
    double r2 = 0.0;
    for (int k = 0; k < 4; ++k)
      r2 = r2 + dot2(w->lpc + 2 * (4 * nd[k] + slot[k]), R->u_np1 + 2 * nd[k]);
    const double m = R->cell_mass[c];
    const double rhoL = 1 / (1 / R->rho_n[c] + R->dt_n / m * r2);
    double r3[2] = {0.0, 0.0};
    for (int k = 0; k < 4; ++k) {
      const double* F = w->F_np1 + 2 * (4 * nd[k] + slot[k]);
      r3[0] = r3[0] + F[0];
      r3[1] = r3[1] + F[1];
    }
    const double* uc = R->cell_u_n + 2 * c;
    const double uL[2] = {uc[0] + r3[0] * R->dt_n / m, uc[1] + r3[1] * R->dt_n / m};
    double r4 = 0.0, pr4[3] = {0.0, 0.0, 0.0};
    for (int k = 0; k < 4; ++k) {
      const long p = nd[k], q = 4 * p + slot[k];
      const double mid[2] = {(uc[0] + uL[0]) * 0.5, (uc[1] + uL[1]) * 0.5};
      const double du[2] = {R->u_np1[2 * p] - mid[0], R->u_np1[2 * p + 1] - mid[1]};
      r4 = r4 + dot2(w->F_np1 + 2 * q, du);
      for (int e = 0; e < 3; ++e) pr4[e] = pr4[e] + dot2(w->Fe_np1 + 2 * (3 * q + e), du);
    }
    (void)r4;
    double peL[3] = {0., 0., 0.};
    for (int e = 0; e < nb; ++e) {
      peL[e] = 0.;
      if (R->fm[NM * c + e] > thr && R->cell_mass_m[NM * c + e] != 0.)
        peL[e] = R->em_n[NM * c + e] +
                 R->fm[NM * c + e] * R->dt_n / R->cell_mass_m[NM * c + e] * pr4[e];
    }
    double* U = R->UL + NEQ * c;
    const double vl = R->vL[c];
    for (int e = 0; e < nb; ++e) {
      U[e] = w->lagvol[3 * c + e];
      U[nb + e] = R->mfm[NM * c + e] * vl * rhoL;
      U[2 * nb + e] = R->mfm[NM * c + e] * vl * rhoL * peL[e];
    }
    U[3 * nb] = vl * rhoL * uL[0];
    U[3 * nb + 1] = vl * rhoL * uL[1];
    if (R->s.projection_conservative == 1)
      U[3 * nb + 2] = 0.5 * vl * rhoL * (uL[0] * uL[0] + uL[1] * uL[1]);
    double* P = R->Phi + NEQ * c;
    if (R->s.pb == 1) {
      double sv = 0.;
      for (int e = 0; e < nb; ++e) sv += U[e];
      double sm = 0.;
      for (int e = 0; e < nb; ++e) {
        P[e] = U[e] / sv;
        if (U[e] != 0.)
          P[nb + e] = U[nb + e] / U[e];
        else
          P[nb + e] = 0.;
        sm += U[nb + e];
      }
      P[3 * nb] = U[3 * nb] / sm;
      P[3 * nb + 1] = U[3 * nb + 1] / sm;
      for (int e = 0; e < nb; ++e) {
        if (U[nb + e] != 0.)
          P[2 * nb + e] = U[2 * nb + e] / U[nb + e];
        else
          P[2 * nb + e] = 0.;
      }
      if (R->s.projection_conservative == 1) P[3 * nb + 2] = U[3 * nb + 2] / sm;
    } else {
      for (int e = 0; e < NEQ; ++e) P[e] = U[e] / vl;
    }
  }
  if (R->s.projection == 1) {
    port_remap_sweep(R, 1);
    port_remap_sweep(R, 2);
    /* remapCellcenteredVariable (PhaseRemapFinal.cc:17-232) */
    R->x_then_y_np1 = !R->x_then_y_n;
    unsigned err = 0;
    long errc = -1;
    for (long c = 0; c < nc; ++c) {
      const double* U = R->U2 + NEQ * c;
      const double vol = R->eulerV[c];
      double volt = 0., masset = 0., vn[NM];
      for (int e = 0; e < nb; ++e) {
        vn[e] = U[e];
        volt += vn[e];
        masset += U[nb + e];
      }
      double vnorm = 0.;
      for (int e = 0; e < nb; ++e) {
        vn[e] *= vol / volt;
        vnorm += vn[e];
      }
      double* f = R->fm + NM * c;
      double* mf = R->mfm + NM * c;
      double sf = 0.;
      for (int e = 0; e < nb; ++e) {
        f[e] = vn[e] / vnorm;
        if (f[e] < thr) f[e] = 0.;
        sf += f[e];
      }
      for (int e = 0; e < nb; ++e) f[e] = f[e] / sf;
      int matcell = 0, imatpure = -1;
      for (int e = 0; e < nb; ++e)
        if (f[e] > 0.) {
          matcell++;
          imatpure = e;
        }
      if (matcell > 1) {
        R->mixte[c] = 1;
        R->pure[c] = -1;
      } else {
        R->mixte[c] = 0;
        R->pure[c] = imatpure;
      }
      for (int e = 0; e < nb; ++e) mf[e] = U[nb + e] / masset;
      double fmt = 0.;
      for (int e = 0; e < nb; ++e) {
        if (f[e] < thr) mf[e] = 0.;
        fmt += mf[e];
      }
      for (int e = 0; e < nb; ++e) mf[e] /= fmt;
      double dm[NM] = {0., 0., 0.}, dens = 0.;
      for (int e = 0; e < nb; ++e) {
        if (f[e] > thr) dm[e] = U[nb + e] / vn[e];
        dens += f[e] * dm[e];
      }
      const double un[2] = {U[3 * nb] / (dens * vol), U[3 * nb + 1] / (dens * vol)};
      double pe[NM] = {0., 0., 0.};
      for (int e = 0; e < nb; ++e)
        if ((f[e] > thr) && (U[nb + e] != 0.)) pe[e] = U[2 * nb + e] / U[nb + e];
      R->rho_np1[c] = dens;
      R->cell_u_np1[2 * c] = un[0];
      R->cell_u_np1[2 * c + 1] = un[1];
      R->e_np1[c] = 0.;
      double dec = 0.;
      if (R->s.projection_conservative == 1)
        dec = U[3 * nb + 2] / masset - 0.5 * (un[0] * un[0] + un[1] * un[1]);
      for (int e = 0; e < nb; ++e) {
        R->rhom_np1[NM * c + e] = dm[e];
        R->em_np1[NM * c + e] = pe[e];
        R->em_np1[NM * c + e] += dec;
        R->e_np1[c] += mf[e] * R->em_np1[NM * c + e];
      }
      for (int e = 0; e < nb; ++e) {
        if (pe[e] < 0. || dm[e] < 0.) {
          R->rhom_np1[NM * c + e] = 0.;
          R->em_np1[NM * c + e] = 0.;
          mf[e] = 0.;
          f[e] = 0.;
          err |= HYDRO_ERR_NEGATIVE;
        }
      }
      if (R->e_np1[c] != R->e_np1[c] || R->rho_np1[c] != R->rho_np1[c]) {
        err |= HYDRO_ERR_NAN;
        if (errc < 0) errc = c;
      }
    }
    if (err) {
      R->err |= err;
      if (R->err_cell < 0 && errc >= 0) R->err_cell = errc;
    }
  }
  /* loop condition and swaps (EucclhydRemap.cc:140-169) */
  const int cont = (R->n + 1 < R->max_iter && R->t_np1 < R->s.final_time);
  if (cont && !(R->err & ~HYDRO_ERR_NEGATIVE)) {
    R->x_then_y_n = R->x_then_y_np1;
    R->t_n = R->t_np1;
    R->dt_n = R->dt_np1;
    SWAPP(R->u_n, R->u_np1);
    SWAPP(R->rho_n, R->rho_np1);
    SWAPP(R->rhom_n, R->rhom_np1);
    SWAPP(R->cell_u_n, R->cell_u_np1);
    SWAPP(R->e_n, R->e_np1);
    SWAPP(R->em_n, R->em_np1);
    SWAPP(w->F_n, w->F_np1);
    SWAPP(w->Fe_n, w->Fe_np1);
  } else {
    R->done = 1;
  }
}
