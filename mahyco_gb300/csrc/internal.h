// Internal declarations shared by the host runtime (.cc) and the CUDA
// kernels (.cu) of the GB300 hydro path.  Not part of the public ABI.
#ifndef MAHYCO_GB300_INTERNAL_H
#define MAHYCO_GB300_INTERNAL_H

#include <cstddef>
#include <cstdint>
#include <functional>
#include <string>

#include "hydro_gb300.h"

namespace hydro {

// Sets the thread's last-error message and returns rc.
int fail(int rc, const std::string& msg);

// includes/ConditionsLimites.h:14-17
constexpr int kBcSym = 200;
constexpr int kBcImposed = 201;
constexpr int kBcPeriodic = 203;
// sides with a boundary flux in the remap (Cdl::leftFluxBC ... topFluxBC)
constexpr int kFluxLeft = 1, kFluxRight = 2, kFluxBottom = 4, kFluxTop = 8;

// Number of conserved components carried through the remap.  The reference
// carries 13 (nbequamax, includes/Constantes.h:9-13); for nbmat materials
// only 3*nbmat+4 are ever non-zero, and the VNR scheme leaves the three
// velocity / kinetic-energy slots at zero too (vnr_remap/PrepareRemap.cc
// :121-123), so VNR remaps 3*nbmat+1 "live" slots: volumes, masses,
// energies, pseudo-viscosity.  Slot k of the device arrays maps to reference
// slot ref_slot(k).
constexpr int kMaxComp = 13;
// marker of the sound-speed argument plane: a NaN payload that arithmetic
// never produces (the hardware's NaNs are the default one), so no energy
// compares equal to it
constexpr unsigned long long kNoRoot = 0x7ff4000000000001ull;

// Device-side view of one run: sizes, options and raw device pointers.
// All cell arrays are SoA planes of `pitch` doubles (pitch >= nc, multiple
// of 32); per-material and per-component arrays are consecutive planes.
struct RunView {
  // ---- sizes
  int nx, ny;
  long long nc, nn;
  long long pitch;   // cell plane stride
  long long npitch;  // node plane stride
  long long fpitch;  // face-value plane stride
  int nbmat;
  int ncomp;         // live remap components
  int comp_ref[kMaxComp];

  // ---- options (reference option structs)
  int scheme;
  int order, pb, pb_mixte, pb_complet, limiter, limiter_pure, dual_method;
  int pseudo_centree, sans_lagrange, projection, conservative;
  int eos[3];
  double threshold, gamma[3], gamma_scalar, energy_limit;
  // per-run constants of the EOS expressions, formed once by the same IEEE
  // operations the per-cell expressions perform: gamma[m] - 1.0,
  // 0.5 * (gamma[m] - 1.0), gamma[0] * (gamma[0] - 1.0), 0.5 * (gamma_scalar + 1)
  double gm1[3], hgm1[3], g0gm1, hgs1;
  double dx, dy, euler_volume, dt_min, final_time, cfl;
  long long max_iter;

  // ---- boundary conditions (Cdl)
  int bc_left, bc_right, bc_bottom, bc_top;
  double v_left[2], v_right[2], v_bottom[2], v_top[2];
  int periodic_x;
  int flux_bc;        // kFlux* bits: sides whose remap takes a boundary flux

  // ---- constant Euler geometry
  const double* xs;      // nx+1 node abscissae (dx * j)
  const double* ys;      // ny+1 node ordinates (dy * i)
  const double* cqs;     // 8 planes: corner normals, [(k*2+d)]
  const double* cflsq;   // cfl * sqrt(sum of initial sub-volumes)
  const double* s0;      // sum of initial sub-volumes
  const double* sqs0;    // sqrt(s0)
  const double* nout;    // 4 planes: outer normal components (L.x,R.x,B.y,T.y)
  const double* flv;     // ny   Euler lengths of vertical faces per row
  const double* flh;     // nx   Euler lengths of horizontal faces per column

  // ---- persistent state
  double *rho, *p, *c, *e, *q, *divu, *cell_mass;
  double *rhom, *pm, *cm, *em, *qm, *fm, *mfm, *cmassm;  // nbmat planes
  int *mixte, *pure;
  double* u;          // 2 node planes
  double* node_mass;
  double* speed;      // |u| per node (dt reduction)
  const double* rho0_left;  // ny: initial density of column 0 (periodic)

  // ---- Lagrange -> remap
  double* XN;         // 2 node planes, runs without the remap only: the
                      // node positions at the cycle's start (the mesh
                      // moves; with the remap it is the Euler mesh)
  double* vout;       // 2 node planes, runs without the remap only: the
                      // dumped node velocity (m_x/y_velocity), which the
                      // reference then refreshes for interior nodes only
                      // (the boundary nodes keep their initial velocity)
  double* XL;         // 2 node planes
  double *vL, *rL, *XcL /*2 planes*/, *Hx, *Hy;
  double* UL;         // ncomp planes (also receives the second sweep)
  double* Phi;        // ncomp planes
  double* Phi2;       // fused sweeps: the first sweep's Phi of the cells it
                      // changed (aliases dPAv, which those runs do not
                      // use); null otherwise
  double* U1;         // ncomp planes
  unsigned char* u1s; // per cell (orders 1-2): the first sweep left every
                      // component unchanged and did not store U1
  double* gP;         // ncomp planes (limited gradients)
  double *dPAv, *dPAr;  // ncomp planes (plateau-slope swept integrals)
  unsigned char* pbz;   // per cell: bit 0 / bit 1 set where every dPAr /
                        // dPAv component is +0.0 and was not stored
  double* DPF;        // nbmat planes (plateau-slope dual mass flux)
  double* phiF;       // ncomp face planes
  double* phiG;       // ncomp face planes of face gradients (runs without
                      // PenteBorne: aliases dPAv / dPAr, unused by them)
  double* FFd;        // nbmat planes: each cell's share of the nodal mass
                      // fluxes of the sweep (A1 / A2 dual methods)
  const unsigned char* nsym;  // VNR: per node, 1 where the corner normals of
                      // its four cells cancel exactly in the force sum's
                      // order (both components), 0 otherwise
  double* sarg;       // VNR: 1 cell plane, the energy e from which the sound
                      // speed in c was formed as sqrt(gamma0 (gamma0 - 1) e),
                      // or kNoRoot where c came otherwise
  const double* geo0; // 5 cell planes, the Lagrangian geometry of the cell
                      // at rest (volume, centroid x / y, widths x / y)
  unsigned char* gL;  // VNR: per cell, 1 where vL, XcL, Hx, Hy hold the
                      // rest geometry (geo0) bit for bit; null otherwise
  double* o3g;        // order 3: ncomp cell planes, each cell's limited-free
                      // gradient along the sweep (eval_grad); null otherwise
                      // and in batched launches, which work per face
  const double* o3c;  // order 3: 16 cell planes, the width-only coefficients
                      // of the mesh at rest, per sweep axis (x: planes 0-7,
                      // y: 8-15): eval_grad's G0, A, B of each cell, then
                      // eval_ystar's T0..T4 of the face below / left of it
  double* o3y;        // order 3: ncomp face planes, the interpolated value
                      // at each inner face (eval_ystar)
  double* DPv;        // 2 node planes: nodal velocity after sweep 1
  double* gD;         // 2 node planes: limited nodal velocity gradient
  double* UD1;        // 3 node planes: m*u, m*v, m after sweep 1

  // ---- Eucclhyd (cell-centred velocity; all null for VNR runs)
  int space_order;
  double* uc;         // 2 cell planes: cell velocity
  double* uco;        // 2 cell planes: the dumped cell velocity
                      // (m_x/y_cell_velocity: clamped away from zero by the
                      // threshold, kept when the velocity is exactly zero)
  double* vg;         // 4 cell planes: velocity gradient (row-major)
  double* Fs;         // 2 + 2*nbmat cell planes: sums of the cell's corner
                      // forces (total, then per material) of the last cycle
  double* pex;        // 4 cell planes: extrapolated pressure per corner
  double* uex;        // 8 cell planes [2k + d]: extrapolated velocity
  double* peex;       // 4*nbmat cell planes [k*nbmat + m]: per material
  const double* lpc;  // 8 cell planes [2k + d]: corner l_pc n_pc
  const double* cmat; // 12 cell planes [3k + e]: corner matrix 00, 01, 11
  const double* xcc;  // 2 cell planes: cell centroids
  const double* perim;  // cell perimeter
  const double* evol;   // Euler cell volume
  double euc_cfl;

  // ---- control block (device)
  struct Ctrl* ctrl;
};

// The fused remap sweep (k_sweep_fused: slopes, plateau-slope integrals and
// update in one kernel per sweep) applies to VNR runs with the remap,
// PenteBorne without the mixed limiter or the "complet" variant, order 2,
// the A1 / A2 dual mass flux (not PenteBorne's) and no boundary flux.
inline bool fused_sweeps_ok(const RunView& v) {
  return v.scheme == HYDRO_SCHEME_VNR && v.projection == 1 && v.pb == 1 && v.pb_mixte == 0 &&
         v.pb_complet == 0 && v.order == 2 && v.dual_method != 2 && v.flux_bc == 0 &&
         v.ncomp <= 10;
}

// Per-run device control block.
struct Ctrl {
  double t_n, dt_n, t_np1, dt_np1;
  long long n;          // cycles done
  int done;             // reference loop condition failed
  int active;           // this cycle runs
  int x_then_y;         // direction of the first sweep of this cycle
  int nout_general;     // set up: some outer normal of the Euler mesh is not
                        // the Cartesian -1 / +1 (L.x, R.x, B.y, T.y), so the
                        // kernels load them (nout_at)
  unsigned long long dt_min_bits;  // ordered encoding of the dt partial min
  unsigned long long pmax_bits;    // ordered encoding of max pressure
  double pmax_prev;                // max pressure of the state at cycle start
  unsigned err;
  int pad2;
  long long err_cell;
  // output pause (hydro_run_step_to_output): while `pause` is set, a cycle
  // whose start time satisfies the dump condition does not run and `paused`
  // is set; `pause_skip` lets the first cycle after arming run regardless
  double t_out;
  int pause, pause_skip, paused, pad3;
  double rdt_np1;  // 1.0 / dt_np1, formed once per cycle (VNR divergence)
  double dt_vel;   // 0.5 * (dt_np1 + dt_n), formed once per cycle (VNR velocity)
};

#ifdef __CUDACC__
// The dump condition of Vnr::dumpVariables / Eucclhyd::dumpVariables
// (vnr_remap/VnrRemap.cc:257-258, eucclhyd_remap/EucclhydRemap.cc:36-37),
// t_n >= lastDump + output_time || t_n == 0, with t_out = lastDump +
// output_time computed by the host.  Called by the cycle-start kernels;
// true when this cycle must not run because the caller wants to write an
// output at its start first.
__device__ __forceinline__ bool output_pause_here(Ctrl& C) {
  if (!C.pause) return false;
  if (C.pause_skip) {
    C.pause_skip = 0;
    return false;
  }
  if (C.t_n >= C.t_out || C.t_n == 0.) {
    C.paused = 1;
    return true;
  }
  return false;
}
#endif

// Per-kernel timing hook for launch_cycle.
using LaunchHook = std::function<void(int)>;
constexpr int kNumKernelKinds = 20;
extern const char* const kKernelNames[kNumKernelKinds];

// ---- batched execution: many independent runs advance in one launch per
// phase.  The items of every run (cells, or nodes / faces) are cut into
// tiles of kBatchThreads items; a launch walks a device-resident tile table
// with a persistent grid, so the table can change without re-capturing the
// CUDA graph that holds the launch.
constexpr int kBatchThreads = 128;
struct Tile {
  int inst;    // index into the batch's RunView array
  int i0, j0;  // first row / column of the tile
  int pad;
};
struct BatchArgs {
  const RunView* views;
  const Tile* tiles;
  const int* ntiles;  // device-resident tile count
  int tw_log2;        // tile width 2^tw_log2
  int rows;           // item rows per thread row
  int sweep;
};
// Item phases of a cycle, in launch order; the two domains are cells
// (nx x ny) and nodes ((nx+1) x (ny+1), which also index the faces).
// The Eucclhyd phases (kPhEuc*) run on the batch's Eucclhyd runs, the VNR
// Lagrange, dual and final phases on its VNR runs, the sweep phases on all.
enum BatchPhase {
  kPhLagNodes, kPhLagCells, kPhFaceGrad, kPhSweepGrad, kPhSweepFace,
  kPhSweepUpdate, kPhDualGrad, kPhDualUpdate, kPhFinal,
  kPhEucCellPre, kPhEucNodes, kPhEucCells, kPhEucFinal, kNumPhases
};
constexpr bool phase_on_nodes(int ph) {
  return ph == kPhLagNodes || ph == kPhFaceGrad || ph == kPhSweepFace ||
         ph == kPhDualGrad || ph == kPhDualUpdate || ph == kPhEucNodes;
}
// Tile shapes: 2^tw_log2 items wide; each of the block's
// kBatchThreads >> tw_log2 thread rows covers `rows` item rows, so one tile
// (one staging of the run's view) serves kBatchThreads * rows items.
struct TileShape {
  int tw_log2;
  int rows;
};
constexpr int kNumTileShapes = 5;
constexpr TileShape kTileShapes[kNumTileShapes] = {
    {5, 1}, {5, 4}, {5, 8}, {6, 4}, {7, 2}};
struct BatchLaunch {
  const RunView* views;
  const int* ninst;      // device-resident number of runs
  int max_inst;          // capacity of views / done
  int* done;             // per run: Ctrl.done after the cycle
  const Tile* tiles[2][kNumTileShapes];   // [on_nodes][shape]
  const int* ntiles[2][kNumTileShapes];
  int shape[kNumPhases];  // tile shape index per phase
  int grid[kNumPhases];   // persistent grid size per phase
  int any_order2;         // launch the slope phases
  int any_face;           // launch the face phase (order 3, or order 1
                          // without PenteBorne)
  int any_face_grad;      // launch the face-gradient phase (order 2
                          // without PenteBorne)
  int variant;            // kBatch* bits: lighter kernels when no run needs
                          // the order-3 faces / the PenteBorne slopes
  int any_vnr, any_euc;   // the batch holds runs of that scheme
};
constexpr int kBatchNoOrder3 = 1;
constexpr int kBatchNoPB = 2;

}  // namespace hydro

#endif
