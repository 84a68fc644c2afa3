/*
 * ORACLE -- test infrastructure.  Internal state of the C restatement.
 *
 * Layout follows the reference: 13-component vectors per cell
 * (RealArray1D<nbequamax>, includes/Constantes.h:9-13), per-material
 * triplets (RealArray1D<nbmatmax>), n / n+1 buffers swapped by pointer
 * exactly where the reference swaps Kokkos views (vnr_remap/VnrRemap.cc
 * :198-221), so stale-buffer semantics are reproduced too.
 */
#ifndef MAHYCO_PORT_INTERNAL_H
#define MAHYCO_PORT_INTERNAL_H
#include <math.h>
#include <stddef.h>

#include "mahyco_port.h"

#define NEQ 13 /* nbequamax */
#define NM 3   /* nbmatmax  */

/* includes/ConditionsLimites.h:14-17 */
#define BC_SYM 200
#define BC_IMPOSED 201
#define BC_FREE 202
#define BC_PERIODIC 203

/* std::min / std::max semantics (cppnabla/types/MathFunctions.h:22-23):
 * std::min(a,b) = (b < a) ? b : a ; std::max(a,b) = (a < b) ? b : a. */
static inline double smin(double a, double b) { return (b < a) ? b : a; }
static inline double smax(double a, double b) { return (a < b) ? b : a; }

typedef struct {
  long n1, n2;      /* first / second node (edge order of the generator) */
  long back, front; /* getBackCell / getFrontCell, -1 when absent         */
  int vertical;
} face_info;

struct port_run {
  hydro_spec s;
  long nx, ny, nc, nn, nf;
  int nbmat;
  long max_iter; /* GestTemps::max_time_iterations */

  /* boundary conditions (Cdl) */
  int leftBC, rightBC, topBC, bottomBC;
  double leftV[2], rightV[2], topV[2], bottomV[2];
  int leftCellBC, rightCellBC, topCellBC, bottomCellBC;
  int leftFluxBC, rightFluxBC, bottomFluxBC, topFluxBC; /* Cdl::*FluxBC */

  /* Euler geometry */
  double *X0, *Xc0, *Vpc0, *eulerV, *Xf, *fL, *fN, *nOut;
  long *VFoN, *HFoN; /* Vertical/HorizontalFaceOfNode, 2 slots per node */

  /* VNR node / cell geometry, n and n+1 */
  double *X_n, *X_np1, *Xc_n, *Xc_np1, *Vpc_n, *Vpc_np1, *cqs;

  /* cell state */
  double *rho_n, *rho_np1, *rho_n0;
  double *p_n, *p_np1, *p_n0;
  double *q_n, *q_np1, *q_n0;
  double *tau_n, *tau_np1, *tau_n0;
  double *divu_n, *divu_np1, *divu_n0;
  double *c_n, *c_np1, *c_n0;
  double *e_n, *e_np1, *e_n0;
  double *rhom_n, *rhom_np1, *rhom_n0; /* nc*NM */
  double *pm_n, *pm_np1, *pm_n0;
  double *qm_n, *qm_np1, *qm_n0;
  double *taum_n, *taum_np1, *taum_n0;
  double *cm_n, *cm_np1, *cm_n0;
  double *em_n, *em_np1, *em_n0;
  double *cell_mass, *cell_mass_m, *fm, *mfm;
  double *fracvol1, *fracvol2, *fracvol3;
  double *u_n, *u_np1, *u_n0; /* nn*2 */
  double *node_mass, *xvel, *yvel;

  /* Eucclhyd state (port_euc.c) */
  double *cell_u_n, *cell_u_np1, *cell_u_n0; /* nc*2 */
  double *pres, *sound, *pres_m, *sound_m;   /* single buffers */
  void* euc;                                 /* Eucclhyd work arrays */

  /* Lagrange <-> remap shared state (includes/VariablesLagRemap.h:23-84) */
  double *Phi, *DualPhi, *dxL, *XL, *XfL, *XcL, *fLL, *fnv;
  double *UL, *UDL, *U2, *UD2, *vL, *rL;
  int *mixte, *pure;
  int x_then_y_n, x_then_y_np1;

  /* Remap work arrays (remap/Remap.h:66-99) */
  double *Hv, *U1, *UD1, *gPF1, *gPF2, *gP1, *gP2, *gDP1, *gDP2;
  double *phiF1, *phiF2, *DPF1, *DPF2, *Bid1, *Bid2, *dPAv, *dPAr;
  double *FF1, *FF2; /* nc*4*NEQ */
  double *RFM, *LFM, *TFM, *BFM;           /* nodal mass fluxes */
  double *Tuv, *Buv, *Ruv, *Luv;           /* upwind velocities nn*2 */

  /* time */
  long n;
  double t_n, t_np1, dt_n, dt_np1, dt_init;
  int done;
  int swapped; /* the last VNR cycle swapped n and n+1 (it was not the last) */
  unsigned err;
  long err_cell;
};

/* mesh (cppnabla/mesh/CartesianMesh2D.cc, CartesianMesh2DGenerator.cc) */
static inline long port_nid(const port_run* R, long i, long j) {
  return i * (R->nx + 1) + j;
}
static inline long port_cid(const port_run* R, long i, long j) {
  return i * R->nx + j;
}
void port_cell_nodes(const port_run* R, long c, long nd[4]);
int port_node_cells(const port_run* R, long p, long cells[4], int loc[4]);
void port_cell_faces(const port_run* R, long c, long f[4]);
void port_face_decode(const port_run* R, long f, face_info* F);
int port_slot_of(const port_run* R, long c, long f);
/* neighbours (CartesianMesh2D.cc:350-384), -1 outside */
long port_left_node(const port_run* R, long p);
long port_right_node(const port_run* R, long p);
long port_bottom_node(const port_run* R, long p);
long port_top_node(const port_run* R, long p);

/* remap (port_remap.c) */
void port_remap_sweep(port_run* R, int sweep);
void port_dual_sweep(port_run* R, int sweep);

/* Eucclhyd (port_euc.c) */
int port_euc_setup(port_run* R);
void port_euc_cycle(port_run* R);
void port_euc_free(port_run* R);

void port_set_error(const char* msg);
#endif
