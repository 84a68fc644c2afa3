/*
 * ORACLE -- test infrastructure, never part of the product.
 *
 * C restatement of the VNR scheme of MaHyCo: mesh numbering, the reference
 * initial states, the Lagrange phase, the preparation of the remap, the
 * remap final and the time loop.  Each function cites the reference
 * function it restates (file:line inside the MaHyCo project).
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "port_internal.h"

static _Thread_local char g_err[512];
const char* port_last_error(void) { return g_err; }
void port_set_error(const char* msg) {
  snprintf(g_err, sizeof g_err, "%s", msg);
}
int port_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* ------------------------------------------------------------------ mesh */
/* Quad node order of CartesianMesh2DGenerator.cc:86-93 (n0 lower-left,
 * counter-clockwise). */
void port_cell_nodes(const port_run* R, long c, long nd[4]) {
  long i = c / R->nx, j = c - i * R->nx;
  long n0 = port_nid(R, i, j);
  nd[0] = n0;
  nd[1] = n0 + 1;
  nd[2] = n0 + R->nx + 2;
  nd[3] = n0 + R->nx + 1;
}

/* CartesianMesh2D::getCellsOfNode (CartesianMesh2D.cc:97-108); loc[] is the
 * node's position in each cell's node list (what utils::indexOf returns). */
int port_node_cells(const port_run* R, long p, long cells[4], int loc[4]) {
  long i = p / (R->nx + 1), j = p - i * (R->nx + 1);
  int k = 0;
  if (i < R->ny && j < R->nx) { cells[k] = port_cid(R, i, j); loc[k++] = 0; }
  if (i < R->ny && j > 0) { cells[k] = port_cid(R, i, j - 1); loc[k++] = 1; }
  if (i > 0 && j < R->nx) { cells[k] = port_cid(R, i - 1, j); loc[k++] = 3; }
  if (i > 0 && j > 0) { cells[k] = port_cid(R, i - 1, j - 1); loc[k++] = 2; }
  return k;
}

/* getFacesOfCell (CartesianMesh2D.cc:168-178): bottom, left, right, top. */
void port_cell_faces(const port_run* R, long c, long f[4]) {
  long i = c / R->nx, j = c - i * R->nx, W = 2 * R->nx + 1;
  long b = 2 * j + i * W;
  f[0] = b;
  f[1] = b + 1;
  f[2] = b + (j == R->nx - 1 ? 2 : 3);
  f[3] = b + (i < R->ny - 1 ? W : W - j);
}

int port_slot_of(const port_run* R, long c, long f) {
  long fs[4];
  port_cell_faces(R, c, fs);
  for (int k = 0; k < 4; ++k)
    if (fs[k] == f) return k;
  return -1;
}

/* Edge numbering of CartesianMesh2DGenerator.cc:72-82 and getCellsOfFace
 * (CartesianMesh2D.cc:110-136). */
void port_face_decode(const port_run* R, long f, face_info* F) {
  long nx = R->nx, ny = R->ny, W = 2 * nx + 1;
  long i = f / W, k = f - i * W;
  F->back = -1;
  F->front = -1;
  if (i < ny) {
    if (k == 2 * nx) {
      F->vertical = 1;
      F->n1 = port_nid(R, i, nx);
      F->n2 = port_nid(R, i + 1, nx);
      F->back = port_cid(R, i, nx - 1);
    } else if (k == 1) {
      F->vertical = 1;
      F->n1 = port_nid(R, i, 0);
      F->n2 = port_nid(R, i + 1, 0);
      F->back = port_cid(R, i, 0);
    } else if (k % 2 == 0) {
      long col = k / 2;
      F->vertical = 0;
      F->n1 = port_nid(R, i, col);
      F->n2 = port_nid(R, i, col + 1);
      F->back = port_cid(R, i, col);
      if (i > 0) F->front = port_cid(R, i - 1, col);
    } else {
      long col = (k - 1) / 2;
      F->vertical = 1;
      F->n1 = port_nid(R, i, col);
      F->n2 = port_nid(R, i + 1, col);
      F->back = port_cid(R, i, col - 1);
      F->front = port_cid(R, i, col);
    }
  } else {
    F->vertical = 0;
    F->n1 = port_nid(R, ny, k);
    F->n2 = port_nid(R, ny, k + 1);
    F->back = port_cid(R, ny - 1, k);
  }
}

/* CartesianMesh2D.cc:350-384 */
long port_left_node(const port_run* R, long p) {
  long i = p / (R->nx + 1), j = p - i * (R->nx + 1);
  return j != 0 ? port_nid(R, i, j - 1) : -1;
}
long port_right_node(const port_run* R, long p) {
  long i = p / (R->nx + 1), j = p - i * (R->nx + 1);
  return j != R->nx ? port_nid(R, i, j + 1) : -1;
}
long port_bottom_node(const port_run* R, long p) {
  long i = p / (R->nx + 1), j = p - i * (R->nx + 1);
  return i != 0 ? port_nid(R, i - 1, j) : -1;
}
long port_top_node(const port_run* R, long p) {
  long i = p / (R->nx + 1), j = p - i * (R->nx + 1);
  return i != R->ny ? port_nid(R, i + 1, j) : -1;
}

/* -------------------------------------------------------------- vectors */
static double* zalloc(size_t n) {
  double* p = (double*)calloc(n ? n : 1, sizeof(double));
  if (!p) {
    fprintf(stderr, "port: out of memory\n");
    abort();
  }
  return p;
}
#define SWAP(a, b)     \
  do {                 \
    double* t_ = (a);  \
    (a) = (b);         \
    (b) = t_;          \
  } while (0)

/* Freefunctions.h: norm = sqrt(dot(a,a)), dot accumulates from 0.0 */
static inline double norm2(double a, double b) {
  double r = 0.0;
  r = r + a * a;
  r = r + b * b;
  return sqrt(r);
}
static inline double cross2(const double* a, const double* b) {
  return a[0] * b[1] - a[1] * b[0];
}

/* ---------------------------------------------------- geometry set-up */
/* Vnr::initCellPos (vnr_remap/Init.cc:495-511) on given node coordinates. */
static void cell_centres(port_run* R, const double* X, double* Xc) {
#pragma omp parallel for
  for (long c = 0; c < R->nc; ++c) {
    long nd[4];
    port_cell_nodes(R, c, nd);
    double r0 = 0.0, r1 = 0.0;
    for (int k = 0; k < 4; ++k) {
      r0 = r0 + X[2 * nd[k]];
      r1 = r1 + X[2 * nd[k] + 1];
    }
    Xc[2 * c] = 0.25 * r0;
    Xc[2 * c + 1] = 0.25 * r1;
  }
}

/* Vnr::computeSubVol / initSubVol (vnr_remap/PhaseLagrange.cc:236-264,
 * Init.cc:400-429). */
static void sub_volumes(port_run* R, const double* X, const double* Xc,
                        double* Vpc) {
#pragma omp parallel for
  for (long c = 0; c < R->nc; ++c) {
    long nd[4];
    port_cell_nodes(R, c, nd);
    for (int k = 0; k < 4; ++k) {
      long pm = nd[(k + 3) % 4], pp = nd[(k + 1) % 4], p = nd[k];
      double x1[2] = {Xc[2 * c], Xc[2 * c + 1]};
      double x2[2] = {0.5 * (X[2 * pm] + X[2 * p]),
                      0.5 * (X[2 * pm + 1] + X[2 * p + 1])};
      double x3[2] = {X[2 * p], X[2 * p + 1]};
      double x4[2] = {0.5 * (X[2 * pp] + X[2 * p]),
                      0.5 * (X[2 * pp + 1] + X[2 * p + 1])};
      Vpc[4 * c + k] = 0.5 * (cross2(x1, x2) + cross2(x2, x3) +
                              cross2(x3, x4) + cross2(x4, x1));
    }
  }
}

/* Vnr::initMeshGeometryForFaces (vnr_remap/Init.cc:517-554); the same
 * computation as Eucclhyd::initMeshGeometryForFaces (eucclhyd_remap/Init.cc
 * :677-716) on that scheme's cell centres. */
void port_face_geometry(port_run* R) {
  for (long f = 0; f < R->nf; ++f) {
    face_info F;
    port_face_decode(R, f, &F);
    const double* a = R->X0 + 2 * F.n1;
    const double* b = R->X0 + 2 * F.n2;
    double Xface[2] = {0.5 * (a[0] + b[0]), 0.5 * (a[1] + b[1])};
    double v[2] = {b[0] - a[0], b[1] - a[1]};
    R->Xf[2 * f] = Xface[0];
    R->Xf[2 * f + 1] = Xface[1];
    R->fL[f] = norm2(v[0], v[1]);
    long cells[2] = {F.back, F.front};
    for (int t = 0; t < 2; ++t) {
      long c = cells[t];
      if (c < 0) continue;
      int s = port_slot_of(R, c, f);
      double d0 = Xface[0] - R->Xc0[2 * c], d1 = Xface[1] - R->Xc0[2 * c + 1];
      double nr = norm2(d0, d1);
      R->nOut[(4 * c + s) * 2] = d0 / nr;
      R->nOut[(4 * c + s) * 2 + 1] = d1 / nr;
    }
    double dotx = 0.0;
    dotx = dotx + v[0] * 1.0;
    dotx = dotx + v[1] * 0.0;
    if (fabs(dotx) < R->s.threshold) {
      R->fN[2 * f] = 1.0;
      R->fN[2 * f + 1] = 0.0;
    } else {
      R->fN[2 * f] = 0.0;
      R->fN[2 * f + 1] = 1.0;
    }
  }
}

/* Remap::FacesOfNode (remap/UtilesMesh.cc:53-108): inner faces visited in
 * id order, first hit in slot 0. */
static void faces_of_node(port_run* R) {
  for (long p = 0; p < R->nn; ++p) {
    R->VFoN[2 * p] = R->VFoN[2 * p + 1] = -1;
    R->HFoN[2 * p] = R->HFoN[2 * p + 1] = -1;
  }
  for (long f = 0; f < R->nf; ++f) {
    face_info F;
    port_face_decode(R, f, &F);
    if (F.front < 0) continue; /* outer face */
    long* T = F.vertical ? R->VFoN : R->HFoN;
    long nds[2] = {F.n1, F.n2};
    for (int t = 0; t < 2; ++t) {
      long p = nds[t];
      if (T[2 * p] == -1)
        T[2 * p] = f;
      else
        T[2 * p + 1] = f;
    }
  }
}

/* ------------------------------------------------------- VNR initial state */
/* Vnr::initBoundaryConditions (vnr_remap/Init.cc:9-95). */
static int vnr_init_bc(port_run* R) {
  int t = R->s.test_case;
  R->leftBC = R->rightBC = R->topBC = R->bottomBC = 0;
  R->leftV[0] = 0.0; R->leftV[1] = 1.0;
  R->rightV[0] = 0.0; R->rightV[1] = 1.0;
  R->topV[0] = 1.0; R->topV[1] = 0.0;
  R->bottomV[0] = 1.0; R->bottomV[1] = 0.0;
  R->leftCellBC = R->rightCellBC = R->topCellBC = R->bottomCellBC = 0;
  if (t == 4 || t == 15 || t == 5 || t == 16) {
    /* Sod X/Y, BiSod X/Y: symmetry walls */
    R->leftBC = R->rightBC = R->topBC = R->bottomBC = BC_SYM;
  } else if (t == 1) {
    /* Sedov (VNR extension): the Eucclhyd Sedov boundary conditions
     * (eucclhyd_remap/Init.cc:47-64) */
    R->leftBC = BC_SYM;
    R->bottomBC = BC_SYM;
    R->rightBC = BC_IMPOSED; R->rightV[0] = 0.0; R->rightV[1] = 0.0;
    R->topBC = BC_IMPOSED; R->topV[0] = 0.0; R->topV[1] = 0.0;
  } else if (t == 7 || t == 18 || t == 9 || t == 20) {
    R->rightBC = BC_IMPOSED; R->rightV[0] = 1.0; R->rightV[1] = 0.0;
    R->rightCellBC = BC_PERIODIC;
    R->leftBC = BC_IMPOSED; R->leftV[0] = 1.0; R->leftV[1] = 0.0;
    R->topBC = BC_SYM;
    R->bottomBC = BC_SYM;
  } else if (t == 0 || t == 11) {
    /* UnitTestCase / BiUnitTestCase (Init.cc:65-93): velocity (1, 0)
     * imposed on every side, a flux condition on the left */
    R->rightBC = BC_IMPOSED; R->rightV[0] = 1.0; R->rightV[1] = 0.0;
    R->leftBC = BC_IMPOSED; R->leftV[0] = 1.0; R->leftV[1] = 0.0;
    R->leftFluxBC = 1;
    R->bottomBC = BC_IMPOSED; R->bottomV[0] = 1.0; R->bottomV[1] = 0.0;
    R->topBC = BC_IMPOSED; R->topV[0] = 1.0; R->topV[1] = 0.0;
  } else if (t == 8 || t == 19) {
    R->bottomBC = BC_IMPOSED; R->bottomV[0] = 0.0; R->bottomV[1] = 1.0;
    R->bottomCellBC = BC_PERIODIC;
    R->topBC = BC_IMPOSED; R->topV[0] = 0.0; R->topV[1] = 1.0;
    R->topCellBC = BC_PERIODIC;
    R->leftBC = BC_SYM;
    R->rightBC = BC_SYM;
  } else {
    port_set_error("VNR: test case not supported by the VNR initialisation");
    return -1;
  }
  return 0;
}

/* Vnr::init (vnr_remap/Init.cc:103-394) for the VNR test cases, plus the
 * bi-material Sod mixed-row extension (init_variant 1). */
static int vnr_init_state(port_run* R) {
  const int t = R->s.test_case;
  const double g = R->s.gamma_scalar;
  for (long c = 0; c < R->nc; ++c)
    for (int m = 0; m < NM; ++m) {
      R->fm[NM * c + m] = 0.0;
      R->mfm[NM * c + m] = 0.0;
      R->rhom_n0[NM * c + m] = 0.0;
      R->pm_n0[NM * c + m] = 0.0;
    }
  if (t == 4 || t == 5) { /* SodCaseX / SodCaseY */
    for (long c = 0; c < R->nc; ++c) {
      double r = (t == 4) ? R->Xc0[2 * c] : R->Xc0[2 * c + 1];
      double* f = R->fm + NM * c;
      double* mf = R->mfm + NM * c;
      f[0] = 1.0;
      mf[0] = 1.0;
      if (r < 0.5) {
        R->rho_n0[c] = 1.0; R->p_n0[c] = 1.0;
        R->rhom_n0[NM * c] = 1.0; R->pm_n0[NM * c] = 1.0;
      } else {
        R->rho_n0[c] = 0.125; R->p_n0[c] = 0.1;
        R->rhom_n0[NM * c] = 0.125; R->pm_n0[NM * c] = 0.1;
      }
      R->cm_n0[NM * c] = sqrt(g * R->rhom_n0[NM * c] / R->pm_n0[NM * c]);
      R->c_n0[c] = R->cm_n0[NM * c];
    }
    for (long p = 0; p < R->nn; ++p) R->u_n0[2 * p] = R->u_n0[2 * p + 1] = 0.0;
  } else if (t == 15 || t == 16) { /* BiSodCaseX / BiSodCaseY */
    for (long c = 0; c < R->nc; ++c) {
      double r = (t == 15) ? R->Xc0[2 * c] : R->Xc0[2 * c + 1];
      double* f = R->fm + NM * c;
      double* mf = R->mfm + NM * c;
      if (r < 0.5) {
        f[0] = 1.0; f[1] = 0.0; mf[0] = 1.0; mf[1] = 0.0;
        R->rho_n0[c] = 1.0; R->p_n0[c] = 1.0;
        R->rhom_n0[NM * c] = 1.0; R->pm_n0[NM * c] = 1.0;
      } else {
        f[0] = 0.0; f[1] = 1.0; mf[0] = 0.0; mf[1] = 1.0;
        R->rho_n0[c] = 0.125; R->p_n0[c] = 0.1;
        R->rhom_n0[NM * c + 1] = 0.125; R->pm_n0[NM * c + 1] = 0.1;
      }
      R->cm_n0[NM * c] = sqrt(g * R->rhom_n0[NM * c] / R->pm_n0[NM * c]);
      R->cm_n0[NM * c + 1] =
          sqrt(g * R->rhom_n0[NM * c + 1] / R->pm_n0[NM * c + 1]);
      R->c_n0[c] = smin(R->cm_n0[NM * c], R->cm_n0[NM * c + 1]);
    }
    for (long p = 0; p < R->nn; ++p) R->u_n0[2 * p] = R->u_n0[2 * p + 1] = 0.0;
  } else if (t == 1) {
    /* Sedov (VNR extension after eucclhyd_remap/Init.cc:303-332): rho 1,
     * p 1e-6, energy 0.244816 deposited in the cell touching the origin,
     * written as its pressure; VNR Sod-style sound speed (Init.cc:139-142) */
    const double e1 = 1.e-6 / ((R->s.gamma[0] - 1.0) * 1.0);
    for (long c = 0; c < R->nc; ++c) {
      int centre = 0;
      const long i = c / R->nx, j = c - i * R->nx;
      const long n0 = i * (R->nx + 1) + j;
      const long nd[4] = {n0, n0 + 1, n0 + R->nx + 2, n0 + R->nx + 1};
      for (int k = 0; k < 4; ++k)
        if (norm2(R->X0[2 * nd[k]], R->X0[2 * nd[k] + 1]) < R->s.threshold) centre = 1;
      const double e = centre ? e1 + 0.244816 / (R->s.dx * R->s.dy) : e1;
      R->fm[NM * c] = 1.0;
      R->mfm[NM * c] = 1.0;
      R->rho_n0[c] = 1.0;
      R->rhom_n0[NM * c] = 1.0;
      R->p_n0[c] = (R->s.gamma[0] - 1.0) * 1.0 * e;
      R->pm_n0[NM * c] = R->p_n0[c];
      R->cm_n0[NM * c] = sqrt(g * R->rhom_n0[NM * c] / R->pm_n0[NM * c]);
      R->c_n0[c] = R->cm_n0[NM * c];
    }
    for (long p = 0; p < R->nn; ++p) R->u_n0[2 * p] = R->u_n0[2 * p + 1] = 0.0;
  } else if (t == 0 || t == 11) {
    /* unit tests (Init.cc:331-361): density 1 left of x = 0.4, 0.1 right
     * of it (the reference leaves a cell centred on 0.4 at 0), pressure 1,
     * sound speed sqrt(gamma), velocity (1, 0) */
    for (long c = 0; c < R->nc; ++c) {
      double* f = R->fm + NM * c;
      double* mf = R->mfm + NM * c;
      f[0] = 1.; f[1] = 0.;
      mf[0] = 1.; mf[1] = 0.;
      R->p_n0[c] = 1.0;
      R->pm_n0[NM * c] = 1.0;
      R->pm_n0[NM * c + 1] = 0.0;
      R->c_n0[c] = sqrt(g);
      R->cm_n0[NM * c] = sqrt(g);
      R->cm_n0[NM * c + 1] = sqrt(g);
      R->rhom_n0[NM * c + 1] = 0.;
      const double r = R->Xc0[2 * c];
      if (r < 0.4) {
        R->rho_n0[c] = 1.;
        R->rhom_n0[NM * c] = 1.;
      } else if (r > 0.4) {
        R->rho_n0[c] = 0.1;
        R->rhom_n0[NM * c] = 0.1;
      }
      if (r > 0.6) {
        R->rho_n0[c] = 0.1;
        R->rhom_n0[NM * c] = 0.1;
      }
    }
    for (long p = 0; p < R->nn; ++p) {
      R->u_n0[2 * p] = 1.0;
      R->u_n0[2 * p + 1] = 0.0;
    }
  } else if (t == 18 && R->s.init_variant == 2) {
    /* advection step (extension): material 1, rho 1, left of x = 0.5;
     * material 2, rho 0.1, right of it; uniform velocity (1, 0) */
    for (long c = 0; c < R->nc; ++c) {
      const double r = R->Xc0[2 * c];
      const int m = (r < 0.5) ? 0 : 1;
      const double d = (m == 0) ? 1.0 : 0.1;
      R->fm[NM * c + m] = 1.0;
      R->mfm[NM * c + m] = 1.0;
      R->rho_n0[c] = d;
      R->p_n0[c] = 0.0;
      R->rhom_n0[NM * c + m] = d;
      R->pm_n0[NM * c + m] = 0.0;
      R->cm_n0[NM * c] = 1.0;
      R->cm_n0[NM * c + 1] = 1.0;
      R->c_n0[c] = smin(R->cm_n0[NM * c], R->cm_n0[NM * c + 1]);
      R->em_n0[NM * c] = 1.0;
      R->em_n0[NM * c + 1] = 1.0;
      R->e_n0[c] = 1.0;
    }
    for (long p = 0; p < R->nn; ++p) {
      R->u_n0[2 * p] = 1.0;
      R->u_n0[2 * p + 1] = 0.0;
    }
  } else if (t == 7 || t == 8 || t == 18 || t == 19 || t == 20 || t == 21) {
    /* (Bi)AdvectionX/Y, BiAdvectionVitX/Y */
    const int isx = (t == 7 || t == 18 || t == 20);
    const int bi = (t >= 18);
    const int vit = (t == 20 || t == 21);
    for (long c = 0; c < R->nc; ++c) {
      double r = isx ? R->Xc0[2 * c] : R->Xc0[2 * c + 1];
      double* f = R->fm + NM * c;
      double* mf = R->mfm + NM * c;
      double dens_out = vit ? 4.0 : 1.0;
      if (r < 0.3) {
        f[0] = 1.0; mf[0] = 1.0;
        R->rho_n0[c] = dens_out; R->p_n0[c] = 0.0;
        R->rhom_n0[NM * c] = dens_out; R->pm_n0[NM * c] = 0.0;
      } else if ((r > 0.3) && (r < 0.5)) {
        if (!bi) {
          f[0] = 1.0; mf[0] = 1.0;
          R->rho_n0[c] = 10.0; R->p_n0[c] = 0.0;
          R->rhom_n0[NM * c] = 10.0; R->pm_n0[NM * c] = 0.0;
        } else {
          f[1] = 1.0; mf[1] = 1.0;
          R->rho_n0[c] = vit ? 4.0 : 1.0; R->p_n0[c] = 0.0;
          R->rhom_n0[NM * c + 1] = 1.0; R->pm_n0[NM * c + 1] = 0.0;
        }
      } else if (r > 0.5) {
        f[0] = 1.0; mf[0] = 1.0;
        R->rho_n0[c] = dens_out; R->p_n0[c] = 0.0;
        R->rhom_n0[NM * c] = dens_out; R->pm_n0[NM * c] = 0.0;
      }
      R->cm_n0[NM * c] = 1.0;
      R->cm_n0[NM * c + 1] = 1.0;
      R->c_n0[c] = smin(R->cm_n0[NM * c], R->cm_n0[NM * c + 1]);
      R->em_n0[NM * c] = 1.0;
      R->em_n0[NM * c + 1] = 1.0;
      R->e_n0[c] = 1.0;
    }
    for (long p = 0; p < R->nn; ++p) {
      double u0 = isx ? 1.0 : 0.0, u1 = isx ? 0.0 : 1.0;
      if (vit) {
        double r = isx ? R->X0[2 * p] : R->X0[2 * p + 1];
        double s;
        if (r <= 0.3) {
          R->u_n0[2 * p] = 0.2 * u0;
          R->u_n0[2 * p + 1] = 0.2 * u1;
        } else if ((r > 0.3) && (r <= 0.5)) {
          s = 4. * r - 1.;
          R->u_n0[2 * p] = s * u0;
          R->u_n0[2 * p + 1] = s * u1;
        } else if (r > 0.5) {
          R->u_n0[2 * p] = u0;
          R->u_n0[2 * p + 1] = u1;
        }
      } else {
        R->u_n0[2 * p] = u0;
        R->u_n0[2 * p + 1] = u1;
      }
    }
  } else {
    port_set_error("VNR: test case not supported by the VNR initialisation");
    return -1;
  }
  for (long p = 0; p < R->nn; ++p) {
    R->xvel[p] = R->u_n0[2 * p];
    R->yvel[p] = R->u_n0[2 * p + 1];
  }
  return 0;
}

/* Mixed interface row/column for bi-material Sod (extension, init_variant
 * 1): the first line of cells whose centre is not below 0.5 becomes a 50/50
 * mixed cell with both materials' states. */
static void vnr_init_mixed_row(port_run* R) {
  const int t = R->s.test_case;
  if (t != 15 && t != 16) return;
  const int ycase = (t == 16);
  const long nline = ycase ? R->ny : R->nx, other = ycase ? R->nx : R->ny;
  long first = -1;
  for (long k = 0; k < nline && first < 0; ++k) {
    long c = ycase ? k * R->nx : k;
    double r = ycase ? R->Xc0[2 * c + 1] : R->Xc0[2 * c];
    if (!(r < 0.5)) first = k;
  }
  if (first < 0) return;
  const double g = R->s.gamma_scalar;
  for (long tt = 0; tt < other; ++tt) {
    long c = ycase ? first * R->nx + tt : tt * R->nx + first;
    const double f0 = 0.5, f1 = 0.5, r0 = 1.0, r1 = 0.125, p0 = 1.0, p1 = 0.1;
    const double m0 = f0 * r0, m1 = f1 * r1;
    double* f = R->fm + NM * c;
    double* mf = R->mfm + NM * c;
    f[0] = f0; f[1] = f1;
    mf[0] = m0 / (m0 + m1);
    mf[1] = m1 / (m0 + m1);
    R->rhom_n0[NM * c] = r0; R->rhom_n0[NM * c + 1] = r1;
    R->pm_n0[NM * c] = p0; R->pm_n0[NM * c + 1] = p1;
    R->rho_n0[c] = f0 * r0 + f1 * r1;
    R->p_n0[c] = f0 * p0 + f1 * p1;
    R->cm_n0[NM * c] = sqrt(g * r0 / p0);
    R->cm_n0[NM * c + 1] = sqrt(g * r1 / p1);
    R->c_n0[c] = smin(R->cm_n0[NM * c], R->cm_n0[NM * c + 1]);
  }
}

/* Vnr::computeCellMass (vnr_remap/PhaseLagrange.cc:14-24). */
static void vnr_cell_mass(port_run* R) {
  for (long c = 0; c < R->nc; ++c) {
    R->cell_mass[c] = R->s.dx * R->s.dy * R->rho_n0[c];
    for (int m = 0; m < R->nbmat; ++m)
      R->cell_mass_m[NM * c + m] = R->mfm[NM * c + m] * R->cell_mass[c];
  }
}

/* Vnr::computeNodeMass (vnr_remap/PhaseLagrange.cc:31-48). */
static void vnr_node_mass(port_run* R) {
#pragma omp parallel for
  for (long p = 0; p < R->nn; ++p) {
    long cells[4];
    int loc[4];
    int k = port_node_cells(R, p, cells, loc);
    double r = 0.0;
    for (int t = 0; t < k; ++t) r = r + R->cell_mass[cells[t]];
    R->node_mass[p] = r / (double)k;
  }
}

static void update_mixte(port_run* R) {
  /* indicateur mailles mixtes at init (vnr_remap/Init.cc:373-393) */
  for (long c = 0; c < R->nc; ++c) {
    R->fracvol1[c] = R->fm[NM * c];
    R->fracvol2[c] = R->fm[NM * c + 1];
    R->fracvol3[c] = R->fm[NM * c + 2];
    int matcell = 0, imatpure = -1;
    for (int m = 0; m < NM; ++m)
      if (R->fm[NM * c + m] > R->s.threshold) {
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
}

/* ------------------------------------------------------------ allocation */
static void alloc_all(port_run* R) {
  long nc = R->nc, nn = R->nn, nf = R->nf;
#define A(ptr, n) R->ptr = zalloc((size_t)(n))
  A(X0, 2 * nn); A(Xc0, 2 * nc); A(Vpc0, 4 * nc); A(eulerV, nc);
  A(Xf, 2 * nf); A(fL, nf); A(fN, 2 * nf); A(nOut, 8 * nc);
  A(X_n, 2 * nn); A(X_np1, 2 * nn); A(Xc_n, 2 * nc); A(Xc_np1, 2 * nc);
  A(Vpc_n, 4 * nc); A(Vpc_np1, 4 * nc); A(cqs, 8 * nc);
  A(rho_n, nc); A(rho_np1, nc); A(rho_n0, nc);
  A(p_n, nc); A(p_np1, nc); A(p_n0, nc);
  A(q_n, nc); A(q_np1, nc); A(q_n0, nc);
  A(tau_n, nc); A(tau_np1, nc); A(tau_n0, nc);
  A(divu_n, nc); A(divu_np1, nc); A(divu_n0, nc);
  A(c_n, nc); A(c_np1, nc); A(c_n0, nc);
  A(e_n, nc); A(e_np1, nc); A(e_n0, nc);
  A(rhom_n, NM * nc); A(rhom_np1, NM * nc); A(rhom_n0, NM * nc);
  A(pm_n, NM * nc); A(pm_np1, NM * nc); A(pm_n0, NM * nc);
  A(qm_n, NM * nc); A(qm_np1, NM * nc); A(qm_n0, NM * nc);
  A(taum_n, NM * nc); A(taum_np1, NM * nc); A(taum_n0, NM * nc);
  A(cm_n, NM * nc); A(cm_np1, NM * nc); A(cm_n0, NM * nc);
  A(em_n, NM * nc); A(em_np1, NM * nc); A(em_n0, NM * nc);
  A(cell_mass, nc); A(cell_mass_m, NM * nc); A(fm, NM * nc); A(mfm, NM * nc);
  A(fracvol1, nc); A(fracvol2, nc); A(fracvol3, nc);
  A(u_n, 2 * nn); A(u_np1, 2 * nn); A(u_n0, 2 * nn);
  A(node_mass, nn); A(xvel, nn); A(yvel, nn);
  A(Phi, NEQ * nc); A(DualPhi, NEQ * nn); A(dxL, nf); A(XL, 2 * nn);
  A(XfL, 2 * nf); A(XcL, 2 * nc); A(fLL, nf); A(fnv, nf);
  A(UL, NEQ * nc); A(UDL, NEQ * nn); A(U2, NEQ * nc); A(UD2, NEQ * nn);
  A(vL, nc); A(rL, nc);
  A(Hv, nc); A(U1, NEQ * nc); A(UD1, NEQ * nn);
  A(gPF1, NEQ * nf); A(gPF2, NEQ * nf); A(gP1, NEQ * nc); A(gP2, NEQ * nc);
  A(gDP1, NEQ * nn); A(gDP2, NEQ * nn);
  A(phiF1, NEQ * nf); A(phiF2, NEQ * nf); A(DPF1, NEQ * nc); A(DPF2, NEQ * nc);
  A(Bid1, NEQ * nc); A(Bid2, NEQ * nc); A(dPAv, NEQ * nc); A(dPAr, NEQ * nc);
  A(FF1, 4 * NEQ * nc); A(FF2, 4 * NEQ * nc);
  A(RFM, nn); A(LFM, nn); A(TFM, nn); A(BFM, nn);
  A(Tuv, 2 * nn); A(Buv, 2 * nn); A(Ruv, 2 * nn); A(Luv, 2 * nn);
#undef A
  R->VFoN = (long*)calloc((size_t)(2 * nn), sizeof(long));
  R->HFoN = (long*)calloc((size_t)(2 * nn), sizeof(long));
  R->mixte = (int*)calloc((size_t)nc, sizeof(int));
  R->pure = (int*)calloc((size_t)nc, sizeof(int));
}

void port_destroy(port_run* R) {
  if (!R) return;
  double** ptrs[] = {
      &R->X0, &R->Xc0, &R->Vpc0, &R->eulerV, &R->Xf, &R->fL, &R->fN, &R->nOut,
      &R->X_n, &R->X_np1, &R->Xc_n, &R->Xc_np1, &R->Vpc_n, &R->Vpc_np1,
      &R->cqs, &R->rho_n, &R->rho_np1, &R->rho_n0, &R->p_n, &R->p_np1,
      &R->p_n0, &R->q_n, &R->q_np1, &R->q_n0, &R->tau_n, &R->tau_np1,
      &R->tau_n0, &R->divu_n, &R->divu_np1, &R->divu_n0, &R->c_n, &R->c_np1,
      &R->c_n0, &R->e_n, &R->e_np1, &R->e_n0, &R->rhom_n, &R->rhom_np1,
      &R->rhom_n0, &R->pm_n, &R->pm_np1, &R->pm_n0, &R->qm_n, &R->qm_np1,
      &R->qm_n0, &R->taum_n, &R->taum_np1, &R->taum_n0, &R->cm_n, &R->cm_np1,
      &R->cm_n0, &R->em_n, &R->em_np1, &R->em_n0, &R->cell_mass,
      &R->cell_mass_m, &R->fm, &R->mfm, &R->fracvol1, &R->fracvol2,
      &R->fracvol3, &R->u_n, &R->u_np1, &R->u_n0, &R->node_mass, &R->xvel,
      &R->yvel, &R->Phi, &R->DualPhi, &R->dxL, &R->XL, &R->XfL, &R->XcL,
      &R->fLL, &R->fnv, &R->UL, &R->UDL, &R->U2, &R->UD2, &R->vL, &R->rL,
      &R->Hv, &R->U1, &R->UD1, &R->gPF1, &R->gPF2, &R->gP1, &R->gP2,
      &R->gDP1, &R->gDP2, &R->phiF1, &R->phiF2, &R->DPF1, &R->DPF2,
      &R->Bid1, &R->Bid2, &R->dPAv, &R->dPAr, &R->FF1, &R->FF2, &R->RFM,
      &R->LFM, &R->TFM, &R->BFM, &R->Tuv, &R->Buv, &R->Ruv, &R->Luv,
      &R->cell_u_n, &R->cell_u_np1, &R->cell_u_n0, &R->pres, &R->sound,
      &R->pres_m, &R->sound_m};
  for (size_t i = 0; i < sizeof ptrs / sizeof ptrs[0]; ++i) free(*ptrs[i]);
  free(R->VFoN);
  free(R->HFoN);
  free(R->mixte);
  free(R->pure);
  port_euc_free(R);
  free(R);
}

/* --------------------------------------------------------- Lagrange (VNR) */
/* computeLpcPlus / computeNpcPlus / computeLpcNpc (includes/Freefunctions.h
 * :28-58) */
static void lpc_npc(const double* xp, const double* xpp, const double* xpm,
                    double out[2]) {
  double a0 = 0.5 * (xpp[1] - xp[1]), a1 = 0.5 * (xp[0] - xpp[0]);
  double la = norm2(a0, a1);
  double na0 = a0 / la, na1 = a1 / la;
  double b0 = 0.5 * (xp[1] - xpm[1]), b1 = 0.5 * (xpm[0] - xp[0]);
  double lb = norm2(b0, b1);
  double nb0 = b0 / lb, nb1 = b1 / lb;
  out[0] = na0 * la + nb0 * lb;
  out[1] = na1 * la + nb1 * lb;
}

/* Vnr::computeCornerNormal (vnr_remap/PhaseLagrange.cc:114-136) */
static void vnr_corner_normal(port_run* R) {
#pragma omp parallel for
  for (long c = 0; c < R->nc; ++c) {
    long nd[4];
    port_cell_nodes(R, c, nd);
    for (int k = 0; k < 4; ++k) {
      long p = nd[k], pp = nd[(k + 1) % 4], pm = nd[(k + 3) % 4];
      lpc_npc(R->X_n + 2 * p, R->X_n + 2 * pp, R->X_n + 2 * pm,
              R->cqs + (4 * c + k) * 2);
    }
  }
}

/* Vnr::computeDeltaT (vnr_remap/VnrRemap.cc:14-50) */
static void vnr_delta_t(port_run* R) {
  double Aveccfleuler = 0., cfl = 0.1;
  if (R->s.projection == 1) {
    Aveccfleuler = 1;
    cfl = 0.05;
  }
  double red = 1.7976931348623157e308;
#pragma omp parallel
  {
    double loc = 1.7976931348623157e308;
#pragma omp for
    for (long c = 0; c < R->nc; ++c) {
      long nd[4];
      port_cell_nodes(R, c, nd);
      double uc = 0.0, r1 = 0.0;
      for (int k = 0; k < 4; ++k) {
        long p = nd[k];
        r1 = r1 + R->Vpc_n[4 * c + k];
        uc += sqrt(R->u_n[2 * p] * R->u_n[2 * p] +
                   R->u_n[2 * p + 1] * R->u_n[2 * p + 1]) *
              0.25;
      }
      loc = smin(loc, cfl * sqrt(r1) / (Aveccfleuler * uc + R->c_n[c]));
    }
#pragma omp critical
    red = smin(red, loc);
  }
  R->dt_np1 = smin(red, 1.05 * R->dt_n);
}

/* Vnr::updateVelocity (vnr_remap/PhaseLagrange.cc:167-197) */
static void vnr_update_velocity(port_run* R) {
  const double dt = 0.5 * (R->dt_np1 + R->dt_n);
#pragma omp parallel for
  for (long i = 1; i < R->ny; ++i)
    for (long j = 1; j < R->nx; ++j) {
      long p = port_nid(R, i, j);
      long cells[4];
      int loc[4];
      int k = port_node_cells(R, p, cells, loc);
      double r0 = 0.0, r1 = 0.0;
      for (int t = 0; t < k; ++t) {
        long c = cells[t];
        double w = R->p_n[c] + R->q_n[c];
        r0 = r0 + w * R->cqs[(4 * c + loc[t]) * 2];
        r1 = r1 + w * R->cqs[(4 * c + loc[t]) * 2 + 1];
      }
      double s = dt / R->node_mass[p];
      R->u_np1[2 * p] = R->u_n[2 * p] + s * r0;
      R->u_np1[2 * p + 1] = R->u_n[2 * p + 1] + s * r1;
      R->xvel[p] = R->u_np1[2 * p];
      R->yvel[p] = R->u_np1[2 * p + 1];
    }
}

/* symmetric boundary node: sum of (p+q)(C + 2(C.s)s - C) over the node's
 * cells (vnr_remap/ConditionsLimites.cc:21-40, Freefunctions.h:60-65) */
static void sym_node(port_run* R, long p, double dt, const double sig[2]) {
  long cells[4];
  int loc[4];
  int k = port_node_cells(R, p, cells, loc);
  double r0 = 0.0, r1 = 0.0;
  for (int t = 0; t < k; ++t) {
    long c = cells[t];
    const double* C = R->cqs + (4 * c + loc[t]) * 2;
    double d = 0.0;
    d = d + C[0] * sig[0];
    d = d + C[1] * sig[1];
    double s2 = 2.0 * d;
    double sv0 = sig[0] * s2 - C[0], sv1 = sig[1] * s2 - C[1];
    double w = R->p_n[c] + R->q_n[c];
    r0 = r0 + w * (C[0] + sv0);
    r1 = r1 + w * (C[1] + sv1);
  }
  double s = dt / (R->node_mass[p]);
  R->u_np1[2 * p] = R->u_n[2 * p] + s * r0;
  R->u_np1[2 * p + 1] = R->u_n[2 * p + 1] + s * r1;
}

/* Vnr::updateVelocityBoundaryConditions (vnr_remap/ConditionsLimites.cc
 * :12-185): bottom, top, left, right sides then the four corners. */
static void vnr_velocity_bc(port_run* R) {
  const double dt = 0.5 * (R->dt_np1 + R->dt_n);
  const double sx[2] = {1.0, 0.0}, sy[2] = {0.0, 1.0};
  for (long j = 0; j <= R->nx; ++j) {
    long p = port_nid(R, 0, j);
    if (R->bottomBC == BC_SYM) sym_node(R, p, dt, sx);
    else if (R->bottomBC == BC_IMPOSED) { R->u_np1[2 * p] = R->bottomV[0]; R->u_np1[2 * p + 1] = R->bottomV[1]; }
  }
  for (long j = 0; j <= R->nx; ++j) {
    long p = port_nid(R, R->ny, j);
    if (R->topBC == BC_SYM) sym_node(R, p, dt, sx);
    else if (R->topBC == BC_IMPOSED) { R->u_np1[2 * p] = R->topV[0]; R->u_np1[2 * p + 1] = R->topV[1]; }
  }
  for (long i = 0; i <= R->ny; ++i) {
    long p = port_nid(R, i, 0);
    if (R->leftBC == BC_SYM) sym_node(R, p, dt, sy);
    else if (R->leftBC == BC_IMPOSED) { R->u_np1[2 * p] = R->leftV[0]; R->u_np1[2 * p + 1] = R->leftV[1]; }
  }
  for (long i = 0; i <= R->ny; ++i) {
    long p = port_nid(R, i, R->nx);
    if (R->rightBC == BC_SYM) sym_node(R, p, dt, sy);
    else if (R->rightBC == BC_IMPOSED) { R->u_np1[2 * p] = R->rightV[0]; R->u_np1[2 * p + 1] = R->rightV[1]; }
  }
  long tl = port_nid(R, R->ny, 0), tr = port_nid(R, R->ny, R->nx);
  long bl = port_nid(R, 0, 0), br = port_nid(R, 0, R->nx);
  if (R->topBC == BC_SYM && R->leftBC == BC_SYM) { R->u_np1[2 * tl] = 0.0; R->u_np1[2 * tl + 1] = 0.0; }
  else if (R->topBC == BC_IMPOSED && R->leftBC == BC_IMPOSED) { R->u_np1[2 * tl] = R->leftV[0]; R->u_np1[2 * tl + 1] = R->leftV[1]; }
  if (R->topBC == BC_SYM && R->rightBC == BC_SYM) { R->u_np1[2 * tr] = 0.0; R->u_np1[2 * tr + 1] = 0.0; }
  else if (R->topBC == BC_IMPOSED && R->rightBC == BC_IMPOSED) { R->u_np1[2 * tr] = R->rightV[0]; R->u_np1[2 * tr + 1] = R->rightV[1]; }
  if (R->bottomBC == BC_SYM && R->leftBC == BC_SYM) { R->u_np1[2 * bl] = 0.0; R->u_np1[2 * bl + 1] = 0.0; }
  else if (R->bottomBC == BC_IMPOSED && R->leftBC == BC_IMPOSED) { R->u_np1[2 * bl] = R->leftV[0]; R->u_np1[2 * bl + 1] = R->leftV[1]; }
  if (R->bottomBC == BC_SYM && R->rightBC == BC_SYM) { R->u_np1[2 * br] = 0.0; R->u_np1[2 * br + 1] = 0.0; }
  else if (R->bottomBC == BC_IMPOSED && R->rightBC == BC_IMPOSED) { R->u_np1[2 * br] = R->rightV[0]; R->u_np1[2 * br + 1] = R->rightV[1]; }
}

/* updatePosition, updateCellPos, computeSubVol, updateRho
 * (vnr_remap/PhaseLagrange.cc:203-296) */
static void vnr_move_and_density(port_run* R) {
#pragma omp parallel for
  for (long p = 0; p < R->nn; ++p) {
    R->X_np1[2 * p] = R->X_n[2 * p] + R->dt_np1 * R->u_np1[2 * p];
    R->X_np1[2 * p + 1] = R->X_n[2 * p + 1] + R->dt_np1 * R->u_np1[2 * p + 1];
  }
  cell_centres(R, R->X_np1, R->Xc_np1);
  sub_volumes(R, R->X_np1, R->Xc_np1, R->Vpc_np1);
#pragma omp parallel for
  for (long c = 0; c < R->nc; ++c) {
    double r = 0.0;
    for (int k = 0; k < 4; ++k) r = r + R->Vpc_np1[4 * c + k];
    R->vL[c] = r;
    R->rho_np1[c] = 0.;
    for (int m = 0; m < R->nbmat; ++m) {
      double f = R->fm[NM * c + m];
      if (f > R->s.threshold)
        R->rhom_np1[NM * c + m] = R->cell_mass_m[NM * c + m] / (f * r);
      R->rho_np1[c] += f * R->rhom_np1[NM * c + m];
    }
  }
}

/* Vnr::updatePeriodicBoundaryConditions (ConditionsLimites.cc:186-209) */
static void vnr_periodic(port_run* R) {
  if (R->rightCellBC != BC_PERIODIC) return;
  for (long i = 0; i < R->ny; ++i) {
    long c = port_cid(R, i, R->nx - 1), L = port_cid(R, i, 0);
    R->rho_np1[L] = R->rho_n0[L];
    R->e_np1[L] = R->e_n0[L];
    R->rho_np1[c] = R->rho_np1[L];
    R->e_np1[c] = R->e_np1[L];
    for (int m = 0; m < R->nbmat; ++m) {
      R->rhom_np1[NM * L + m] = R->rhom_n0[NM * L + m];
      R->em_np1[NM * L + m] = R->em_n0[NM * L + m];
      R->rhom_np1[NM * c + m] = R->rhom_np1[NM * L + m];
      R->em_np1[NM * c + m] = R->em_np1[NM * L + m];
    }
  }
}

/* computeTau, computeDivU, computeArtificialViscosity, updateEnergy
 * (vnr_remap/PhaseLagrange.cc:303-388, 54-107, 324-373) */
static void vnr_energy(port_run* R) {
  const int nb = R->nbmat;
  const double thr = R->s.threshold;
#pragma omp parallel for
  for (long c = 0; c < R->nc; ++c) {
    R->tau_np1[c] = 0.5 * (1.0 / R->rho_np1[c] + 1.0 / R->rho_n[c]);
    for (int m = 0; m < nb; ++m) {
      R->taum_np1[NM * c + m] = 0.;
      if ((R->rhom_np1[NM * c + m] > thr) && (R->rhom_n[NM * c + m] > thr))
        R->taum_np1[NM * c + m] =
            0.5 * (1.0 / R->rhom_np1[NM * c + m] + 1.0 / R->rhom_n[NM * c + m]);
    }
    R->divu_np1[c] = 1.0 / R->dt_np1 * (1.0 / R->rho_np1[c] - 1.0 / R->rho_n[c]) /
                     R->tau_np1[c];
  }
  /* Kokkos::Max reduction of p^n */
  double redP = -1.7976931348623157e308;
  for (long c = 0; c < R->nc; ++c)
    if (R->p_n[c] > redP) redP = R->p_n[c];
  const double g = R->s.gamma_scalar;
  unsigned err = 0;
  long errc = -1;
#pragma omp parallel for
  for (long c = 0; c < R->nc; ++c) {
    if (R->divu_n[c] < 0.0) {
      double r0 = 0.0, r1 = 0.0;
      for (int k = 0; k < 4; ++k) r0 = r0 + R->Vpc_n[4 * c + k];
      for (int k = 0; k < 4; ++k) r1 = r1 + R->Vpc_n[4 * c + k];
      R->q_np1[c] = 1.0 / R->tau_np1[c] *
                    (-0.5 * sqrt(r0) * R->c_n[c] * R->divu_np1[c] +
                     (g + 1) / 2.0 * r1 * R->divu_np1[c] * R->divu_np1[c]);
    } else
      R->q_np1[c] = 0.0;
    if (R->q_np1[c] > redP) R->q_np1[c] = redP;
    for (int m = 0; m < nb; ++m)
      R->qm_np1[NM * c + m] = R->fm[NM * c + m] * R->q_np1[c];
  }
#pragma omp parallel for
  for (long c = 0; c < R->nc; ++c) {
    R->e_np1[c] = 0.;
    for (int m = 0; m < nb; ++m) {
      long k = NM * c + m;
      R->em_np1[k] = 0.;
      if ((R->rhom_np1[k] > thr) && (R->rhom_n[k] > thr)) {
        double pseudo = 0.;
        if ((R->s.pseudo_centree == 1) &&
            ((R->qm_np1[k] + R->qm_n[k]) *
                 (1.0 / R->rhom_np1[k] - 1.0 / R->rhom_n[k]) >
             0.))
          pseudo = 0.5 * (R->qm_np1[k] + R->qm_n[k]);
        if (R->s.pseudo_centree == 0) pseudo = R->qm_np1[k];
        const double den = 1 + 0.5 * (R->s.gamma[m] - 1.0) * R->rhom_np1[k] *
                                    (1.0 / R->rhom_np1[k] - 1.0 / R->rhom_n[k]);
        const double num = R->em_n[k] - (0.5 * R->pm_n[k] + pseudo) *
                                            (1.0 / R->rhom_np1[k] - 1.0 / R->rhom_n[k]);
        R->em_np1[k] = num / den;
        R->e_np1[c] += R->mfm[k] * R->em_np1[k];
        if (R->s.energy_limit > 0 && fabs(R->em_np1[k]) > R->s.energy_limit) {
#pragma omp critical
          {
            err |= HYDRO_ERR_ENERGY;
            if (errc < 0 || c < errc) errc = c;
          }
        }
      }
    }
  }
  if (err) {
    R->err |= err;
    if (R->err_cell < 0) R->err_cell = errc;
  }
}

/* Vnr::computeEOS + computeEOSGP / computeEOSVoid (PhaseLagrange.cc:392-430)
 * then computePressionMoyenne (:464-485) */
static void vnr_eos_and_mean(port_run* R) {
  const int nb = R->nbmat;
  for (int m = 0; m < nb; ++m) {
    const double gm = R->s.gamma[m];
    if (R->s.eos[m] == HYDRO_EOS_PERFECT_GAS) {
#pragma omp parallel for
      for (long c = 0; c < R->nc; ++c) {
        long k = NM * c + m;
        R->pm_np1[k] = (gm - 1.0) * R->rhom_np1[k] * R->em_np1[k];
        R->cm_np1[k] = sqrt(gm * (gm - 1.0) * R->em_np1[k]);
      }
    } else if (R->s.eos[m] == HYDRO_EOS_VOID) {
      for (long c = 0; c < R->nc; ++c) {
        long k = NM * c + m;
        R->pm_np1[k] = R->pm_n[k];
        R->cm_np1[k] = R->cm_n[k];
        R->em_np1[k] = R->em_n[k];
        R->e_np1[c] = 0.;
      }
    }
  }
  const double g0 = R->s.gamma[0];
  for (long c = 0; c < R->nc; ++c) {
    R->p_np1[c] = 0.;
    for (int m = 0; m < nb; ++m) {
      R->p_np1[c] += R->fm[NM * c + m] * R->pm_np1[NM * c + m];
      R->c_np1[c] = smax(R->c_np1[c], R->cm_np1[NM * c + m]);
    }
    if (R->rho_np1[c] > 0.) R->c_np1[c] = sqrt(g0 * (g0 - 1.0) * R->e_np1[c]);
    for (int m = 0; m < nb; ++m)
      if (R->s.eos[m] == HYDRO_EOS_VOID)
        R->e_np1[c] += R->mfm[NM * c + m] * R->em_np1[NM * c + m];
  }
}

/* ----------------------------------------------------- PrepareRemap (VNR) */
/* computeVariablesForRemap, computeCellQuantitesForRemap,
 * computeFaceQuantitesForRemap (vnr_remap/PrepareRemap.cc:14-211) */
static void vnr_prepare_remap(port_run* R) {
  const int nb = R->nbmat;
#pragma omp parallel for
  for (long c = 0; c < R->nc; ++c) {
    double* U = R->UL + NEQ * c;
    double* P = R->Phi + NEQ * c;
    const double v = R->vL[c];
    for (int m = 0; m < nb; ++m) {
      U[m] = R->fm[NM * c + m] * v;
      U[nb + m] = R->mfm[NM * c + m] * v * R->rho_np1[c];
      U[2 * nb + m] = R->mfm[NM * c + m] * v * R->rho_np1[c] * R->e_np1[c];
    }
    U[3 * nb + 0] = 0.;
    U[3 * nb + 1] = 0.;
    U[3 * nb + 2] = 0.;
    U[3 * nb + 3] = R->q_np1[c] * v;
    if (R->s.pb == 1) {
      double sv = 0.;
      for (int m = 0; m < nb; ++m) sv += U[m];
      double sm = 0.;
      for (int m = 0; m < nb; ++m) {
        P[m] = U[m] / sv;
        if (U[m] != 0.)
          P[nb + m] = U[nb + m] / U[m];
        else
          P[nb + m] = 0.;
        sm += U[nb + m];
      }
      (void)sm;
      for (int m = 0; m < nb; ++m) {
        if (U[nb + m] != 0.)
          P[2 * nb + m] = U[2 * nb + m] / U[nb + m];
        else
          P[2 * nb + m] = 0.;
      }
      P[3 * nb + 0] = 0.;
      P[3 * nb + 1] = 0.;
      P[3 * nb + 2] = 0.;
      P[3 * nb + 3] = R->q_np1[c];
    } else {
      for (int k = 0; k < NEQ; ++k) P[k] = U[k] / v;
    }
    R->rL[c] = R->rho_np1[c];
  }
#pragma omp parallel for
  for (long p = 0; p < R->nn; ++p) {
    R->XL[2 * p] = R->X_np1[2 * p];
    R->XL[2 * p + 1] = R->X_np1[2 * p + 1];
    double* UD = R->UDL + NEQ * p;
    double* DP = R->DualPhi + NEQ * p;
    const double* u = R->u_np1 + 2 * p;
    UD[0] = R->node_mass[p] * u[0];
    UD[1] = R->node_mass[p] * u[1];
    UD[2] = R->node_mass[p];
    if (R->s.projection_conservative == 1)
      UD[3] = R->node_mass[p] * (u[0] * u[0] + u[1] * u[1]);
    DP[0] = u[0];
    DP[1] = u[1];
    DP[2] = R->node_mass[p];
    if (R->s.projection_conservative == 1) DP[3] = (u[0] * u[0] + u[1] * u[1]);
  }
  /* Lagrangian centroid (PrepareRemap.cc:65-90) */
#pragma omp parallel for
  for (long c = 0; c < R->nc; ++c) {
    long nd[4];
    port_cell_nodes(R, c, nd);
    double r0 = 0.0, r1 = 0.0;
    for (int k = 0; k < 4; ++k) {
      const double* a = R->XL + 2 * nd[k];
      const double* b = R->XL + 2 * nd[(k + 1) % 4];
      double cr = cross2(a, b);
      r0 = r0 + cr * (a[0] + b[0]);
      r1 = r1 + cr * (a[1] + b[1]);
    }
    double s = 1.0 / (6.0 * R->vL[c]);
    R->XcL[2 * c] = s * r0;
    R->XcL[2 * c + 1] = s * r1;
  }
  /* faces (PrepareRemap.cc:14-64) */
#pragma omp parallel for
  for (long f = 0; f < R->nf; ++f) {
    face_info F;
    port_face_decode(R, f, &F);
    if (F.front >= 0) {
      double d0 = R->XcL[2 * F.front] - R->XcL[2 * F.back];
      double d1 = R->XcL[2 * F.front + 1] - R->XcL[2 * F.back + 1];
      double d = 0.0;
      d = d + d0 * R->fN[2 * f];
      d = d + d1 * R->fN[2 * f + 1];
      R->dxL[f] = d;
    }
    const double* a = R->XL + 2 * F.n1;
    const double* b = R->XL + 2 * F.n2;
    R->XfL[2 * f] = 0.5 * (a[0] + b[0]);
    R->XfL[2 * f + 1] = 0.5 * (a[1] + b[1]);
    R->fLL[f] = norm2(b[0] - a[0], b[1] - a[1]);
    double r0 = 0.0, r1 = 0.0;
    r0 = r0 + R->u_np1[2 * F.n1];
    r1 = r1 + R->u_np1[2 * F.n1 + 1];
    r0 = r0 + R->u_np1[2 * F.n2];
    r1 = r1 + R->u_np1[2 * F.n2 + 1];
    double h0 = 0.5 * r0, h1 = 0.5 * r1;
    double d = 0.0;
    d = d + h0 * R->fN[2 * f];
    d = d + h1 * R->fN[2 * f + 1];
    R->fnv[f] = d;
  }
}

/* ------------------------------------------------------ remap final (VNR) */
/* Vnr::remapVariables (vnr_remap/PhaseRemapFinal.cc:18-234) */
static void vnr_remap_final(port_run* R) {
  const int nb = R->nbmat;
  const double thr = R->s.threshold;
  R->x_then_y_np1 = !R->x_then_y_n;
  unsigned err = 0;
  long errc = -1;
#pragma omp parallel for
  for (long c = 0; c < R->nc; ++c) {
    const double* U = R->U2 + NEQ * c;
    double* f = R->fm + NM * c;
    double* mf = R->mfm + NM * c;
    double vol = R->eulerV[c], volt = 0., masset = 0.;
    double vn[NM] = {0, 0, 0};
    for (int m = 0; m < nb; ++m) {
      vn[m] = U[m];
      volt += vn[m];
      masset += U[nb + m];
    }
    double vnorm = 0.;
    for (int m = 0; m < nb; ++m) {
      vn[m] *= vol / volt;
      vnorm += vn[m];
    }
    double sf = 0.;
    for (int m = 0; m < nb; ++m) {
      f[m] = vn[m] / vnorm;
      if (f[m] < thr) f[m] = 0.;
      sf += f[m];
    }
    for (int m = 0; m < nb; ++m) f[m] = f[m] / sf;
    int matcell = 0, imatpure = -1;
    for (int m = 0; m < nb; ++m)
      if (f[m] > 0.) {
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
    for (int m = 0; m < nb; ++m) mf[m] = U[nb + m] / masset;
    double fmt = 0.;
    for (int m = 0; m < nb; ++m) {
      if (f[m] < thr) mf[m] = 0.;
      fmt += mf[m];
    }
    for (int m = 0; m < nb; ++m) mf[m] /= fmt;
    double dm[NM] = {0., 0., 0.}, dens = 0.;
    for (int m = 0; m < nb; ++m) {
      if (f[m] > thr) dm[m] = U[nb + m] / vn[m];
      dens += f[m] * dm[m];
    }
    double em[NM] = {0., 0., 0.};
    for (int m = 0; m < nb; ++m)
      if ((f[m] > thr) && (U[nb + m] != 0.)) em[m] = U[2 * nb + m] / U[nb + m];
    R->rho_np1[c] = dens;
    R->e_np1[c] = 0.;
    R->cell_mass[c] = R->eulerV[c] * R->rho_np1[c];
    for (int m = 0; m < nb; ++m)
      R->cell_mass_m[NM * c + m] = mf[m] * R->cell_mass[c];
    R->q_np1[c] = U[3 * nb + 3] / vol;
    for (int m = 0; m < nb; ++m) {
      R->rhom_np1[NM * c + m] = dm[m];
      R->em_np1[NM * c + m] = em[m];
      R->e_np1[c] += mf[m] * R->em_np1[NM * c + m];
    }
    for (int m = 0; m < nb; ++m) {
      if (em[m] < 0. || dm[m] < 0.) {
        R->rhom_np1[NM * c + m] = 0.;
        R->em_np1[NM * c + m] = 0.;
        mf[m] = 0.;
        f[m] = 0.;
      }
    }
    if (R->e_np1[c] != R->e_np1[c] || R->rho_np1[c] != R->rho_np1[c]) {
#pragma omp critical
      {
        err |= HYDRO_ERR_NAN;
        if (errc < 0 || c < errc) errc = c;
      }
    }
    R->fracvol1[c] = f[0];
    R->fracvol2[c] = f[1];
    R->fracvol3[c] = f[2];
  }
  if (err) {
    R->err |= err;
    if (R->err_cell < 0) R->err_cell = errc;
  }
#pragma omp parallel for
  for (long p = 0; p < R->nn; ++p) {
    double mm = R->UD2[NEQ * p + 2];
    R->u_np1[2 * p] = R->UD2[NEQ * p] / mm;
    R->u_np1[2 * p + 1] = R->UD2[NEQ * p + 1] / mm;
    R->xvel[p] = R->u_np1[2 * p];
    R->yvel[p] = R->u_np1[2 * p + 1];
  }
}

/* ------------------------------------------------------------ time loop */
/* One iteration of Vnr::executeTimeLoopN (vnr_remap/VnrRemap.cc:127-222). */
static void vnr_cycle(port_run* R) {
  R->n++;
  if (R->s.sans_lagrange == 0) {
    vnr_corner_normal(R);
    vnr_delta_t(R);
  } else {
    R->dt_np1 = R->dt_n;
  }
  R->t_np1 = R->t_n + R->dt_np1;
  if (R->s.sans_lagrange == 0) {
    vnr_update_velocity(R);
    vnr_velocity_bc(R);
  } else {
    SWAP(R->u_n, R->u_np1);
  }
  vnr_move_and_density(R);
  vnr_periodic(R);
  if (R->s.sans_lagrange == 0) {
    vnr_energy(R);
    vnr_eos_and_mean(R);
  } else {
    SWAP(R->e_n, R->e_np1);
  }
  if (R->s.projection == 1) {
    vnr_prepare_remap(R);
    port_remap_sweep(R, 1);
    port_dual_sweep(R, 1);
    port_remap_sweep(R, 2);
    port_dual_sweep(R, 2);
    vnr_remap_final(R);
    vnr_node_mass(R);
    vnr_eos_and_mean(R);
  }
  int cont = (R->n + 1 < R->max_iter && R->t_np1 < R->s.final_time);
  R->swapped = cont;
  if (cont) {
    int tmp = R->x_then_y_np1;
    R->x_then_y_np1 = R->x_then_y_n;
    R->x_then_y_n = tmp;
    double t = R->t_np1;
    R->t_np1 = R->t_n;
    R->t_n = t;
    t = R->dt_np1;
    R->dt_np1 = R->dt_n;
    R->dt_n = t;
    SWAP(R->rho_np1, R->rho_n);
    SWAP(R->rhom_np1, R->rhom_n);
    SWAP(R->p_np1, R->p_n);
    SWAP(R->pm_np1, R->pm_n);
    SWAP(R->q_np1, R->q_n);
    SWAP(R->qm_np1, R->qm_n);
    SWAP(R->tau_np1, R->tau_n);
    SWAP(R->taum_np1, R->taum_n);
    SWAP(R->divu_np1, R->divu_n);
    SWAP(R->c_np1, R->c_n);
    SWAP(R->cm_np1, R->cm_n);
    SWAP(R->e_np1, R->e_n);
    SWAP(R->em_np1, R->em_n);
    SWAP(R->u_np1, R->u_n);
    if (R->s.projection == 0) {
      SWAP(R->Xc_np1, R->Xc_n);
      SWAP(R->Vpc_np1, R->Vpc_n);
      SWAP(R->X_np1, R->X_n);
    }
  } else {
    R->done = 1;
  }
}

/* Vnr::simulate set-up (vnr_remap/VnrRemap.cc:330-341). */
static int vnr_setup(port_run* R) {
  if (vnr_init_bc(R)) return -1;
  cell_centres(R, R->X0, R->Xc0);
  if (vnr_init_state(R)) return -1;
  if (R->s.init_variant == 1) vnr_init_mixed_row(R);
  update_mixte(R);
  sub_volumes(R, R->X0, R->Xc0, R->Vpc0);
  for (long c = 0; c < R->nc; ++c) R->eulerV[c] = R->s.dx * R->s.dy;
  port_face_geometry(R);
  faces_of_node(R);
  vnr_cell_mass(R);
  if (R->s.sans_lagrange == 0) {
    /* initDeltaT (Init.cc:435-457) */
    double red = 1.7976931348623157e308;
    for (long c = 0; c < R->nc; ++c) {
      double r1 = 0.0;
      for (int k = 0; k < 4; ++k) r1 = r1 + R->Vpc0[4 * c + k];
      red = smin(red, 0.1 * sqrt(r1) / R->c_n0[c]);
    }
    R->dt_init = red * 1.0E-6;
    /* initInternalEnergy (Init.cc:463-472) */
    for (long c = 0; c < R->nc; ++c) {
      for (int m = 0; m < NM; ++m)
        R->em_n0[NM * c + m] = R->pm_n0[NM * c + m] /
                               ((R->s.gamma[m] - 1.0) * R->rhom_n0[NM * c + m]);
      R->e_n0[c] = R->p_n0[c] / ((R->s.gamma_scalar - 1.0) * R->rho_n0[c]);
    }
    /* initPseudo (Init.cc:479-489) */
    for (long c = 0; c < R->nc; ++c) {
      R->tau_n0[c] = 1 / R->rho_n0[c];
      R->divu_n0[c] = 0.0;
      R->q_n0[c] = 0.0;
      for (int m = 0; m < NM; ++m) {
        R->taum_n0[NM * c + m] = 1 / R->rhom_n0[NM * c + m];
        R->qm_n0[NM * c + m] = 0.0;
      }
    }
  } else {
    R->dt_init = R->s.dt_init;
  }
  /* setUpTimeLoopN (VnrRemap.cc:68-87) */
  R->dt_n = R->dt_init;
  size_t nc = (size_t)R->nc, nn = (size_t)R->nn;
  memcpy(R->X_n, R->X0, 2 * nn * sizeof(double));
  memcpy(R->Vpc_n, R->Vpc0, 4 * nc * sizeof(double));
  memcpy(R->rho_n, R->rho_n0, nc * sizeof(double));
  memcpy(R->rhom_n, R->rhom_n0, NM * nc * sizeof(double));
  memcpy(R->p_n, R->p_n0, nc * sizeof(double));
  memcpy(R->pm_n, R->pm_n0, NM * nc * sizeof(double));
  memcpy(R->q_n, R->q_n0, nc * sizeof(double));
  memcpy(R->qm_n, R->qm_n0, NM * nc * sizeof(double));
  memcpy(R->tau_n, R->tau_n0, nc * sizeof(double));
  memcpy(R->taum_n, R->taum_n0, NM * nc * sizeof(double));
  memcpy(R->divu_n, R->divu_n0, nc * sizeof(double));
  memcpy(R->c_n, R->c_n0, nc * sizeof(double));
  memcpy(R->cm_n, R->cm_n0, NM * nc * sizeof(double));
  memcpy(R->e_n, R->e_n0, nc * sizeof(double));
  memcpy(R->em_n, R->em_n0, NM * nc * sizeof(double));
  memcpy(R->u_n, R->u_n0, 2 * nn * sizeof(double));
  memcpy(R->Xc_n, R->Xc0, 2 * nc * sizeof(double));
  vnr_node_mass(R);
  return 0;
}

/* ------------------------------------------------------------------ API */
port_run* port_create(const hydro_spec* spec) {
  if (spec->nx < 2 || spec->ny < 2) {
    port_set_error("nx and ny must be >= 2");
    return NULL;
  }
  if (spec->nbmat < 1 || spec->nbmat > 3) {
    port_set_error("nbmat must be 1..3");
    return NULL;
  }
  port_run* R = (port_run*)calloc(1, sizeof(port_run));
  R->s = *spec;
  R->nx = spec->nx;
  R->ny = spec->ny;
  R->nc = R->nx * R->ny;
  R->nn = (R->nx + 1) * (R->ny + 1);
  R->nf = 2 * R->nc + R->nx + R->ny;
  R->nbmat = spec->nbmat;
  R->max_iter = spec->max_cycles > 0 ? spec->max_cycles + 1 : 500000000L;
  R->x_then_y_n = R->x_then_y_np1 = 1;
  R->err_cell = -1;
  alloc_all(R);
  for (long i = 0; i <= R->ny; ++i)
    for (long j = 0; j <= R->nx; ++j) {
      long p = port_nid(R, i, j);
      R->X0[2 * p] = spec->dx * (double)j;
      R->X0[2 * p + 1] = spec->dy * (double)i;
    }
  int rc;
  if (spec->scheme == HYDRO_SCHEME_VNR)
    rc = vnr_setup(R);
  else if (spec->scheme == HYDRO_SCHEME_EUCCLHYD)
    rc = port_euc_setup(R);
  else {
    port_set_error("unknown scheme");
    rc = -1;
  }
  if (rc) {
    port_destroy(R);
    return NULL;
  }
  return R;
}

int port_step(port_run* R, int ncycles, int* done) {
  int k = 0;
  while (k < ncycles && !R->done && !(R->err & ~HYDRO_ERR_NEGATIVE)) {
    if (R->s.scheme == HYDRO_SCHEME_VNR)
      vnr_cycle(R);
    else
      port_euc_cycle(R);
    ++k;
  }
  if (R->err & ~HYDRO_ERR_NEGATIVE) R->done = 1;
  if (done) *done = R->done;
  return k;
}

int port_time(port_run* R, double* t, double* dt, long* cycle) {
  /* after the last cycle the reference does not swap: report t_{n+1}; a
   * VNR run stopped by an error after a cycle that swapped reports the
   * time it reached (the reference exits inside that cycle) */
  const int cur = !R->done || R->swapped;
  if (t) *t = cur ? R->t_n : R->t_np1;
  if (dt) *dt = cur ? R->dt_n : R->dt_np1;
  if (cycle) *cycle = R->n;
  return 0;
}

int port_error(port_run* R, unsigned* code, long* cell) {
  if (code) *code = R->err;
  if (cell) *cell = R->err_cell;
  return 0;
}

/* Fields are the state after the last completed cycle (the n+1 buffers of
 * the reference when the loop has ended, the swapped n buffers otherwise). */
static const double* field_ptr(port_run* R, const char* name, size_t* n) {
  const int fin = R->done;
  const size_t nc = (size_t)R->nc, nn = (size_t)R->nn;
#define F(nm, a, b, cnt)                   \
  if (!strcmp(name, nm)) {                 \
    *n = cnt;                              \
    return fin ? (b) : (a);                \
  }
  if (R->s.scheme == HYDRO_SCHEME_VNR) {
    F("density", R->rho_n, R->rho_np1, nc)
    F("pressure", R->p_n, R->p_np1, nc)
    F("energy", R->e_n, R->e_np1, nc)
    F("sound_speed", R->c_n, R->c_np1, nc)
    F("pseudo", R->q_n, R->q_np1, nc)
    F("divu", R->divu_n, R->divu_np1, nc)
    F("density_env", R->rhom_n, R->rhom_np1, NM * nc)
    F("energy_env", R->em_n, R->em_np1, NM * nc)
    F("pressure_env", R->pm_n, R->pm_np1, NM * nc)
    F("node_velocity", R->u_n, R->u_np1, 2 * nn)
    F("node_coord", R->X_n, R->X_np1, 2 * nn)
  } else {
    F("density", R->rho_n, R->rho_np1, nc)
    F("energy", R->e_n, R->e_np1, nc)
    F("density_env", R->rhom_n, R->rhom_np1, NM * nc)
    F("energy_env", R->em_n, R->em_np1, NM * nc)
    F("node_velocity", R->u_n, R->u_np1, 2 * nn)
    F("cell_velocity", R->cell_u_n, R->cell_u_np1, 2 * nc)
    F("pressure", R->pres, R->pres, nc)
    F("sound_speed", R->sound, R->sound, nc)
  }
  F("cell_mass", R->cell_mass, R->cell_mass, nc)
  F("fracvol_env", R->fm, R->fm, NM * nc)
  F("mass_fraction_env", R->mfm, R->mfm, NM * nc)
  F("node_mass", R->node_mass, R->node_mass, nn)
#undef F
  *n = 0;
  return NULL;
}

size_t port_field_size(port_run* R, const char* field) {
  size_t n = 0;
  field_ptr(R, field, &n);
  return n;
}

int port_fetch(port_run* R, const char* field, double* dst, size_t n) {
  size_t have = 0;
  const double* p = field_ptr(R, field, &have);
  if (!p) {
    port_set_error("unknown field");
    return -1;
  }
  if (n != have) {
    port_set_error("field size mismatch");
    return -2;
  }
  memcpy(dst, p, n * sizeof(double));
  return 0;
}
