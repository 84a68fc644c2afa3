// FP64 CUDA kernels of one VNR Lagrange + remap cycle on GB300 (sm_103a).
//
// Cycle structure (reference: Vnr::executeTimeLoopN, vnr_remap/VnrRemap.cc
// :127-222):
//   k_begin        dt_{n+1}, t_{n+1} from the previous cycle's reductions
//   k_lag_nodes    node mass, node velocity + boundary conditions, Lagrange
//                  node positions                       (PhaseLagrange.cc,
//                                                        ConditionsLimites.cc)
//   k_lag_cells    sub-volumes, densities, div u, pseudo-viscosity, energy,
//                  EOS, mean pressure, then the cell part of PrepareRemap
//   sweep x2:  without PenteBorne k_face_grad (face gradients) and
//              k_sweep_grad (limited slopes, the order-2 face values of
//              upwind cells); with PenteBorne k_sweep_grad_pb (its face
//              gradients, slopes and plateau-slope integrals); k_sweep_update
//              (conservative update; k_sweep_update_f forms the PenteBorne
//              face values itself; order 3: k_o3_grad, k_o3_ystar,
//              k_sweep_face3 first; order 1: k_sweep_face first),
//              k_dual_grad + k_dual_update (nodal momentum remap)
//   k_final        remapVariables + EOS + mean pressure + next dt / pmax
//   k_end          loop condition and time swap
//
// Every state array is updated in place: each kernel only writes the items
// it owns and reads neighbours written by an earlier kernel, which is what
// the reference's n / n+1 buffers guarantee.  All arithmetic keeps the
// reference's operation order (compiled with --fmad=false).
#include <cuda_runtime.h>

#include "../internal.h"
#include "items.cuh"
#include "scheme_math.cuh"

namespace hydro {

namespace {

constexpr int kBX = 32, kBY = 4;  // 2D cell / node tiles

#define DV __device__ __forceinline__

DV double ld(const double* p, long long i) { return __ldg(p + i); }

// Outer normal q (L.x, R.x, B.y, T.y) of cell c: the Cartesian -1 / +1 the
// set-up found in every cell, or the stored plane where it did not
DV double nout_at(const RunView& v, int q, long long c) {
  if (v.ctrl->nout_general) return __ldg(v.nout + q * v.pitch + c);
  return (q & 1) ? 1.0 : -1.0;
}
DV unsigned ld_u8(const unsigned char* p, long long i) { return __ldg(p + i); }

// Store of a value this thread read from the same address earlier in the
// kernel: left out when the bits are the ones already there, so the location
// ends up holding the same bits either way.  At rest most Lagrange outputs
// that are also inputs (velocity, divergence, sound speed, the root's
// argument, the pseudo-viscosity) come back unchanged, and a sector none of
// whose stores happen is not written back to HBM.
DV void st_if_new(double* a, double old_v, double new_v) {
  if (ubits(new_v) != ubits(old_v)) *a = new_v;
}

// Per-material options read by select rather than by a dynamic index, so a
// RunView copied into registers (batched launches) is never spilled whole to
// local memory.
DV double gamma_of(const RunView& v, int m) {
  return m == 0 ? v.gamma[0] : (m == 1 ? v.gamma[1] : v.gamma[2]);
}
DV double gm1_of(const RunView& v, int m) {
  return m == 0 ? v.gm1[0] : (m == 1 ? v.gm1[1] : v.gm1[2]);
}
DV double hgm1_of(const RunView& v, int m) {
  return m == 0 ? v.hgm1[0] : (m == 1 ? v.hgm1[1] : v.hgm1[2]);
}
DV int eos_of(const RunView& v, int m) {
  return m == 0 ? v.eos[0] : (m == 1 ? v.eos[1] : v.eos[2]);
}

// ----------------------------------------------------------------- control
// Cycle start: dt_{n+1} and t_{n+1} from the previous cycle's reductions
// (VnrRemap.cc:190-200), then the reduction slots are reset before this
// cycle's final kernel accumulates into them.
__device__ __forceinline__ void begin_at(const RunView& v) {
  Ctrl& C = *v.ctrl;
  if (C.done || (C.err & ~HYDRO_ERR_NEGATIVE)) {
    C.active = 0;
    C.done = 1;
    return;
  }
  if (output_pause_here(C)) {
    C.active = 0;
    return;
  }
  C.active = 1;
  C.n += 1;
  if (v.sans_lagrange == 0) {
    double red = from_ord(C.dt_min_bits);
    C.dt_np1 = smin(red, 1.05 * C.dt_n);
  } else {
    C.dt_np1 = C.dt_n;
  }
  C.t_np1 = C.t_n + C.dt_np1;
  C.rdt_np1 = 1.0 / C.dt_np1;
  // updateVelocity's time step (PhaseLagrange.cc:167-197)
  C.dt_vel = half(C.dt_np1 + C.dt_n);
}

__device__ __forceinline__ void reset_at(const RunView& v) {
  Ctrl& C = *v.ctrl;
  if (!C.active) return;
  C.pmax_prev = from_ord(C.pmax_bits);
  C.dt_min_bits = ord_bits(1.7976931348623157e308);
  C.pmax_bits = ord_bits(-1.7976931348623157e308);
}

// Loop condition and time swap (VnrRemap.cc:194-221).
__device__ __forceinline__ void end_at(const RunView& v) {
  Ctrl& C = *v.ctrl;
  if (!C.active) return;
  bool cont = (C.n + 1 < v.max_iter && C.t_np1 < v.final_time);
  C.t_n = C.t_np1;
  C.dt_n = C.dt_np1;
  if (cont)
    C.x_then_y = !C.x_then_y;
  else
    C.done = 1;
  if (C.err & ~HYDRO_ERR_NEGATIVE) C.done = 1;
}

__global__ void k_begin(RunView v) { begin_at(v); }
__global__ void k_reset_reductions(RunView v) { reset_at(v); }
__global__ void k_end(RunView v) { end_at(v); }

// block-wide min / max of ordered encodings, one atomic per block
__device__ void block_reduce_minmax(unsigned long long dtv,
                                    unsigned long long pv, Ctrl* C) {
  __shared__ unsigned long long smin_s[32], smax_s[32];
  const int lane = (threadIdx.y * blockDim.x + threadIdx.x) & 31;
  const int warp = (threadIdx.y * blockDim.x + threadIdx.x) >> 5;
  const int nw = (blockDim.x * blockDim.y + 31) >> 5;
  for (int o = 16; o > 0; o >>= 1) {
    unsigned long long a = __shfl_xor_sync(0xffffffffu, dtv, o);
    unsigned long long b = __shfl_xor_sync(0xffffffffu, pv, o);
    dtv = a < dtv ? a : dtv;
    pv = b > pv ? b : pv;
  }
  if (lane == 0) {
    smin_s[warp] = dtv;
    smax_s[warp] = pv;
  }
  __syncthreads();
  if (warp == 0) {
    dtv = lane < nw ? smin_s[lane] : ~0ull;
    pv = lane < nw ? smax_s[lane] : 0ull;
    for (int o = 16; o > 0; o >>= 1) {
      unsigned long long a = __shfl_xor_sync(0xffffffffu, dtv, o);
      unsigned long long b = __shfl_xor_sync(0xffffffffu, pv, o);
      dtv = a < dtv ? a : dtv;
      pv = b > pv ? b : pv;
    }
    if (lane == 0) {
      atomicMin(&C->dt_min_bits, dtv);
      atomicMax(&C->pmax_bits, pv);
    }
  }
  // the shared slots are reused by the next tile of a batched block
  __syncthreads();
}

// dt candidate of one cell (Vnr::computeDeltaT, VnrRemap.cc:26-46):
// cfl*sqrt(sum V_pc) / (A*uc + c), uc = sum_p 0.25*|u_p|, with A = 1 and cfl
// 0.05 with the remap, A = 0 and cfl 0.1 without it (the reference then
// multiplies the nodal speed by zero).
DV double cell_dt(const RunView& v, long long c, int i, int j) {
  const long long n0 = (long long)i * (v.nx + 1) + j;
  const long long nd[4] = {n0, n0 + 1, n0 + v.nx + 2, n0 + v.nx + 1};
  // 0.0 + x = x for the first term (a speed is >= +0)
  double uc = quarter(ld(v.speed, nd[0]));
#pragma unroll
  for (int k = 1; k < 4; ++k) uc = addz(uc, quarter(ld(v.speed, nd[k])));
  if (v.projection == 0) return div_ip(ld(v.cflsq, c), 0. * uc + v.c[c]);
  return div_ip(ld(v.cflsq, c), addz(uc, v.c[c]));
}

// ------------------------------------------------------- Lagrange: nodes
// Vnr::computeNodeMass (PhaseLagrange.cc:31-48), updateVelocity (:167-197),
// updateVelocityBoundaryConditions (ConditionsLimites.cc:12-185),
// updatePosition (:203-208).
struct LagNodes {
  __device__ __forceinline__ void operator()(const RunView& v, int i, int j) const {
    const Ctrl& C = *v.ctrl;
    if (i > v.ny || j > v.nx) return;
    const long long p = (long long)i * (v.nx + 1) + j;
    // cells of node, getCellsOfNode order (CartesianMesh2D.cc:97-108); loc is
    // the node's position in each cell's node list
    long long cells[4];
    int loc[4], k = 0;
    if (i < v.ny && j < v.nx) { cells[k] = (long long)i * v.nx + j; loc[k++] = 0; }
    if (i < v.ny && j > 0) { cells[k] = (long long)i * v.nx + j - 1; loc[k++] = 1; }
    if (i > 0 && j < v.nx) { cells[k] = (long long)(i - 1) * v.nx + j; loc[k++] = 3; }
    if (i > 0 && j > 0) { cells[k] = (long long)(i - 1) * v.nx + j - 1; loc[k++] = 2; }
    // sums from 0.0: first addition as plus_zero (k >= 1 cells)
    double msum = plus_zero(v.cell_mass[cells[0]]);
    for (int t = 1; t < k; ++t) msum = msum + v.cell_mass[cells[t]];
    const double m = div_pow2(msum, k);  // msum / k, k in {1, 2, 4}

    double ux = v.u[p], uy = v.u[v.npitch + p];
    // updatePosition (PhaseLagrange.cc:203-208) starts from the cycle's start
    // positions (the Euler mesh with the remap); read with the other inputs,
    // before any store (a store would order the later loads behind it)
    const double X0 = v.XN ? v.XN[p] : ld(v.xs, j);
    const double X1 = v.XN ? v.XN[v.npitch + p] : ld(v.ys, i);
    double xl0, xl1;
    if (v.sans_lagrange == 0) {
      const double dt = C.dt_vel;  // 0.5 * (dt^{n+1} + dt^n), formed once per cycle
      // s = dt / m, formed only when a force is not exactly zero: with dt and
      // m positive and of moderate size, s * (+-0) is +-0 itself (the force
      // sums cancel exactly on a mesh at rest)
      const bool s_easy = pos(dt) && pos(m) && div_safe_exp(dt) && div_safe_exp(m);
      double s_val = 0.0;
      bool s_have = false;
      auto step = [&](double r) {
        if (s_easy && iszero(r)) return r;
        if (!s_have) {
          s_val = div_ip(dt, m);
          s_have = true;
        }
        return s_val * r;
      };
      // Corner normal of this node in cell t.  With the remap the mesh is
      // the Euler one at every cycle's start and the set-up stored them;
      // without it (Vnr::computeCornerNormal, PhaseLagrange.cc:114-136, at
      // each cycle's start) they come from the current positions of the
      // node and of its successor / predecessor in the cell's node order.
      const long long NP = v.npitch, W = v.nx + 1;
      auto corner = [&](int t, double& C0, double& C1) {
        if (!v.XN) {
          C0 = ld(v.cqs, (2 * loc[t]) * v.pitch + cells[t]);
          C1 = ld(v.cqs, (2 * loc[t] + 1) * v.pitch + cells[t]);
          return;
        }
        // successor, predecessor: (right, up), (up, left), (left, down),
        // (down, right) for the cell's bottom-left, bottom-right, top-right
        // and top-left node
        const long long nxt[4] = {p + 1, p + W, p - 1, p - W};
        const long long prv[4] = {p + W, p - 1, p - W, p + 1};
        const long long a = nxt[loc[t]], b = prv[loc[t]];
        const double xp[2] = {v.XN[p], v.XN[NP + p]};
        const double xa[2] = {v.XN[a], v.XN[NP + a]};
        const double xb[2] = {v.XN[b], v.XN[NP + b]};
        double o[2];
        lpc_npc(xp, xa, xb, o);
        C0 = o[0];
        C1 = o[1];
      };
      auto force = [&](bool sym, double sx, double sy, double& r0, double& r1) {
        r0 = 0.0;
        r1 = 0.0;
        for (int t = 0; t < k; ++t) {
          const long long c = cells[t];
          double C0, C1;
          corner(t, C0, C1);
          const double w = addz(v.p[c], v.q[c]);
          double t0, t1;
          if (!sym) {
            t0 = w * C0;
            t1 = w * C1;
          } else {
            double d = plus_zero(C0 * sx);
            d = d + C1 * sy;
            const double s2 = dbl(d);
            const double sv0 = sx * s2 - C0, sv1 = sy * s2 - C1;
            t0 = w * (C0 + sv0);
            t1 = w * (C1 + sv1);
          }
          r0 = (t == 0) ? plus_zero(t0) : r0 + t0;
          r1 = (t == 0) ? plus_zero(t1) : r1 + t1;
        }
      };
      const double u0x = ux, u0y = uy;
      const bool inner = i > 0 && i < v.ny && j > 0 && j < v.nx;
      // one pressure in the four cells around an inner node whose corner
      // normals cancel exactly (nsym, set up with the derivation): the force
      // sum is +0 without the products.  The four p + q are compared where
      // the sums are exact on the integer pipe (p or q a zero); elsewhere the
      // products run, and give the same +0.
      bool zero = false;
      if (inner && !v.XN && ld_u8(v.nsym, p)) {  // a flag of the Euler mesh
        constexpr unsigned long long kMod = 1523ull << 52;  // 2^500
        unsigned long long w0 = 0ull, w = 0ull;
        zero = addz_bits(v.p[cells[0]], v.q[cells[0]], w0) && (w0 & kMag) < kMod;
  #pragma unroll
        for (int t = 1; t < 4; ++t)
          zero = zero && addz_bits(v.p[cells[t]], v.q[cells[t]], w) && w == w0;
      }
      // An inner node at rest: a zero force sum, so s = dt / m is not formed
      // (s * (+0) = +0); a zero velocity, (+-0) + (+0) = +0; dt^{n+1}
      // positive and finite, so X + dt^{n+1} * (+0) = X + (+0) is X (+0 for a
      // zero X, X not NaN).  One branch for the whole node: the general
      // path's FP64 operations, if-converted, would be issued for it too.
      const bool rest = zero && s_easy && ((ubits(u0x) | ubits(u0y)) & kMag) == 0 &&
                        pos(C.dt_np1) && is_finite(C.dt_np1) && !is_nan(X0) && !is_nan(X1);
      if (rest) {
        ux = 0.0;
        uy = 0.0;
        xl0 = iszero(X0) ? 0.0 : X0;
        xl1 = iszero(X1) ? 0.0 : X1;
        if (v.vout) {  // m_x/y_velocity, inner nodes only (PhaseLagrange.cc:193)
          v.vout[p] = ux;
          v.vout[v.npitch + p] = uy;
        }
      } else {
        double r0, r1;
        if (inner) {
          if (zero) {
            r0 = 0.0;
            r1 = 0.0;
          } else {
            force(false, 0., 0., r0, r1);
          }
          ux = addz(u0x, step(r0));
          uy = addz(u0y, step(r1));
          if (v.vout) {
            v.vout[p] = ux;
            v.vout[v.npitch + p] = uy;
          }
        }
        // sides in the reference's order: bottom, top, left, right
        if (i == 0) {
          if (v.bc_bottom == kBcSym) {
            force(true, 1.0, 0.0, r0, r1);
            ux = addz(u0x, step(r0));
            uy = addz(u0y, step(r1));
          } else if (v.bc_bottom == kBcImposed) {
            ux = v.v_bottom[0];
            uy = v.v_bottom[1];
          }
        }
        if (i == v.ny) {
          if (v.bc_top == kBcSym) {
            force(true, 1.0, 0.0, r0, r1);
            ux = addz(u0x, step(r0));
            uy = addz(u0y, step(r1));
          } else if (v.bc_top == kBcImposed) {
            ux = v.v_top[0];
            uy = v.v_top[1];
          }
        }
        if (j == 0) {
          if (v.bc_left == kBcSym) {
            force(true, 0.0, 1.0, r0, r1);
            ux = addz(u0x, step(r0));
            uy = addz(u0y, step(r1));
          } else if (v.bc_left == kBcImposed) {
            ux = v.v_left[0];
            uy = v.v_left[1];
          }
        }
        if (j == v.nx) {
          if (v.bc_right == kBcSym) {
            force(true, 0.0, 1.0, r0, r1);
            ux = addz(u0x, step(r0));
            uy = addz(u0y, step(r1));
          } else if (v.bc_right == kBcImposed) {
            ux = v.v_right[0];
            uy = v.v_right[1];
          }
        }
        // corners (ConditionsLimites.cc:133-184)
        const bool top = (i == v.ny), bot = (i == 0), lft = (j == 0), rgt = (j == v.nx);
        if ((top || bot) && (lft || rgt)) {
          const int bv = top ? v.bc_top : v.bc_bottom;
          const int bh = lft ? v.bc_left : v.bc_right;
          const double vh0 = lft ? v.v_left[0] : v.v_right[0];
          const double vh1 = lft ? v.v_left[1] : v.v_right[1];
          if (bv == kBcSym && bh == kBcSym) {
            ux = 0.0;
            uy = 0.0;
          } else if (bv == kBcImposed && bh == kBcImposed) {
            ux = vh0;
            uy = vh1;
          }
        }
        xl0 = addz(X0, mulz(C.dt_np1, ux));
        xl1 = addz(X1, mulz(C.dt_np1, uy));
      }
      st_if_new(v.u + p, u0x, ux);
      st_if_new(v.u + v.npitch + p, u0y, uy);
    } else {
      xl0 = addz(X0, mulz(C.dt_np1, ux));
      xl1 = addz(X1, mulz(C.dt_np1, uy));
    }
    v.node_mass[p] = m;
    v.XL[p] = xl0;
    v.XL[v.npitch + p] = xl1;
  }
};

// ------------------------------------------------------- Lagrange: cells
// updateCellPos, computeSubVol, updateRho (PhaseLagrange.cc:214-296),
// updatePeriodicBoundaryConditions (ConditionsLimites.cc:186-209),
// computeTau, computeDivU, computeArtificialViscosity, updateEnergy,
// computeEOS, computePressionMoyenne (PhaseLagrange.cc:54-107, 303-485),
// then computeVariablesForRemap / computeCellQuantitesForRemap
// (vnr_remap/PrepareRemap.cc:65-176) and the Lagrangian face lengths that
// give HvLagrange (remap/PhaseRemap1.cc:57-71, 104-119).
// e + sum over the Void materials of mf * em (computePressionMoyenne's
// last loop, vnr_remap/PhaseLagrange.cc:480-483), behind a call:
// the runs without a Void material skip it whole (inline, the products and
// sums of the unrolled material loop would be if-converted into FP64
// instructions that run for every cell)
static __device__ __noinline__ double void_energy(unsigned mask, double e, double mf0,
                                                  double mf1, double mf2, double em0,
                                                  double em1, double em2) {
  if (mask & 1u) e += mf0 * em0;
  if (mask & 2u) e += mf1 * em1;
  if (mask & 4u) e += mf2 * em2;
  return e;
}

struct LagCells {
  __device__ __forceinline__ void operator()(const RunView& v, int i, int j) const {
    Ctrl& C = *v.ctrl;
    if (i >= v.ny || j >= v.nx) return;
    const long long c = (long long)i * v.nx + j;
    const long long P = v.pitch, NP = v.npitch;
    const long long n0 = (long long)i * (v.nx + 1) + j;
    const long long nd[4] = {n0, n0 + 1, n0 + v.nx + 2, n0 + v.nx + 1};
    double X[4][2];
  #pragma unroll
    for (int k = 0; k < 4; ++k) {
      X[k][0] = v.XL[nd[k]];
      X[k][1] = v.XL[NP + nd[k]];
    }
    // Lagrangian geometry; a cell whose four nodes did not move (positions
    // equal to the Euler coordinates, bit for bit) has the geometry the
    // set-up stored for it, formed by the same function from the same
    // numbers
    // the stored geometry is loaded with the positions (its use waits on the
    // comparison below, its latency does not)
    double g0v[5] = {0., 0., 0., 0., 0.};
    bool rest = v.geo0 != nullptr;
    // gL: this cell's Lagrange geometry planes (vL, XcL, Hx, Hy) already
    // hold the rest geometry, stored when the cell was last found at rest;
    // a cell at rest again then needs only the volume from it, and stores
    // none of them
    const bool held = v.gL && v.projection == 1 && v.gL[c] != 0;
    if (rest) {
      g0v[0] = ld(v.geo0, c);
      if (!held) {
  #pragma unroll
        for (int q = 1; q < 5; ++q) g0v[q] = ld(v.geo0, q * P + c);
      }
    }
    if (rest) {
      const unsigned long long x0 = ubits(ld(v.xs, j)), x1 = ubits(ld(v.xs, j + 1));
      const unsigned long long y0 = ubits(ld(v.ys, i)), y1 = ubits(ld(v.ys, i + 1));
      rest = ubits(X[0][0]) == x0 && ubits(X[0][1]) == y0 && ubits(X[1][0]) == x1 &&
             ubits(X[1][1]) == y0 && ubits(X[2][0]) == x1 && ubits(X[2][1]) == y1 &&
             ubits(X[3][0]) == x0 && ubits(X[3][1]) == y1;
    }
    CellGeom G;
    if (rest) {
      G.vol = g0v[0];
      G.xc0 = g0v[1];
      G.xc1 = g0v[2];
      G.hx = g0v[3];
      G.hy = g0v[4];
    } else {
      G = vnr_cell_geometry(X, v.order > 1);
    }
    const double vol = G.vol;
    const int nb = v.nbmat;
    const double thr = v.threshold;
    double f[3], mf[3] = {0., 0., 0.}, rhom_new[3], rho_o[3], em_o[3], pm_o[3], qm_o[3];
    double rho_new = 0.;
    // every value read before the first store (the stores would otherwise
    // order the later loads behind them)
    const double rho_old = v.rho[c], divu_old = v.divu[c], c_old = v.c[c];
    const double sarg_old = v.sarg[c];
    // sum of the sub-volumes at the cycle's start (the pseudo-viscosity's
    // volume): the Euler cell's with the remap, the Lagrangian volume of the
    // previous cycle (vL) without it
    const double vol_start = (v.projection == 0) ? v.vL[c] : 0.0;
    // A cell holding one material p (f = mf = 1 for it, +0 for the others,
    // whose densities are finite and at most the threshold), with the
    // remap, perfect gases only, a threshold in [0, 1), a positive finite
    // volume and a sound speed not negative: the material loops below run
    // over p alone (slot 0, plane mat(0) = p), every sum over the materials
    // keeping its value (the others add zeros: x + -0 = x, 0.0 + x as
    // plus_zero), and the others' stores are the signed zeros the loops
    // would form (below).  One branch for the whole cell; decided per value,
    // the loops' shortcuts are if-converted into FP64 instructions that run
    // for every material.
    int p = -1;
    bool single = v.projection == 1 && v.sans_lagrange == 0 && nonneg(thr) && dlt(thr, 1.0) &&
                  pos(vol) && is_finite(vol) && !neg(c_old);
    double fa[3] = {0., 0., 0.}, mfa[3] = {0., 0., 0.}, rma[3] = {0., 0., 0.};
  #pragma unroll
    for (int m = 0; m < 3; ++m) {
      if (m >= nb) break;
      fa[m] = v.fm[m * P + c];
      mfa[m] = v.mfm[m * P + c];
      rma[m] = v.rhom[m * P + c];
      constexpr unsigned long long kOne = 0x3ff0000000000000ull;
      single = single && eos_of(v, m) == HYDRO_EOS_PERFECT_GAS;
      if (ubits(fa[m]) == kOne && ubits(mfa[m]) == kOne) {
        single = single && p < 0;
        p = m;
      } else {
        single = single && (ubits(fa[m]) | ubits(mfa[m])) == 0ull && is_finite(rma[m]) &&
                 !dgt(rma[m], thr);
      }
    }
    single = single && p >= 0;
    const int nbl = single ? 1 : nb;              // material slots of the loops
    auto mat = [&](int m) { return single ? p : m; };  // a slot's planes
    auto pick = [&](const double* a, int m) {     // a slot's value, by select
      const int q = mat(m);
      return q == 0 ? a[0] : (q == 1 ? a[1] : a[2]);
    };
  #pragma unroll
    for (int m = 0; m < 3; ++m) {
      if (m >= nbl) break;
      em_o[m] = v.em[mat(m) * P + c];
      pm_o[m] = v.pm[mat(m) * P + c];
      qm_o[m] = v.qm[mat(m) * P + c];
    }
  #pragma unroll
    for (int m = 0; m < 3; ++m) {
      if (m >= nbl) break;
      f[m] = pick(fa, m);
      mf[m] = pick(mfa, m);
      const double rm = pick(rma, m);
      rho_o[m] = rm;
      rhom_new[m] = rm;
      if (dgt(f[m], thr)) rhom_new[m] = qdiv(v.cmassm[mat(m) * P + c], mul_frac(f[m], vol));
      const double fr = mul_frac(f[m], rhom_new[m]);
      rho_new = (m == 0) ? plus_zero(fr) : addz(rho_new, fr);
    }
    double e_new, q_new;
    if (v.sans_lagrange == 0) {
      const double rdt = C.rdt_np1;
      // A density that came through the Lagrange phase bit for bit unchanged,
      // positive and within [2^-1000, 2^1001) (so 1/rho is a positive finite
      // normal number), with the previous divergence >= 0: the new
      // divergence is rdt * (1/rho - 1/rho) / tau = rdt * (+0) / tau = +0
      // (rdt and tau = 1/rho positive and finite), q is 0, and a material
      // whose old and new densities are the cell's has equal reciprocals.
      // 1/rho itself is then formed only if something else needs it.
      const unsigned long long eo = ubits(rho_old) >> 52;  // sign and exponent
      const bool rest = ubits(rho_new) == ubits(rho_old) && eo >= 23 && eo <= 2023 &&
                        !neg(divu_old) && pos(rdt) && is_finite(rdt);
      double irho_old = 0., irho_new = 0.;
      bool have_irho = false;
      double divu_new;
      if (rest) {
        divu_new = 0.0;
        q_new = 0.0;
      } else {
        irho_old = div_ip(1.0, rho_old);
        // a density unchanged has the old reciprocal, and the difference of
        // the two is then +0 (x - x, x finite)
        const bool same_rho = ubits(rho_new) == ubits(rho_old) && is_finite(irho_old);
        irho_new = same_rho ? irho_old : div_ip(1.0, rho_new);
        have_irho = true;
        const double tau = half(irho_new + irho_old);
        // qdiv: the density, hence the divergence, is unchanged where the
        // flow has not arrived (0 / tau)
        divu_new = qdiv(rdt * (same_rho ? 0.0 : irho_new - irho_old), tau);
        if (neg(divu_old)) {
          const double s0 = (v.projection == 0) ? vol_start : ld(v.s0, c);
          const double sq0 = (v.projection == 0) ? sqrt_ip(vol_start) : ld(v.sqs0, c);
          q_new = div_ip(1.0, tau) *
                  (-half(sq0) * c_old * divu_new +
                   v.hgs1 * s0 * divu_new * divu_new);
        } else {
          q_new = 0.0;
        }
      }
      if (dgt(q_new, C.pmax_prev)) q_new = C.pmax_prev;
      st_if_new(v.divu + c, divu_old, divu_new);
      // energies (updateEnergy) and EOS
      e_new = 0.;
      bool e_first = true;  // 0.0 + x is plus_zero(x)
      double cm_new[3], em_new[3] = {0., 0., 0.};
      bool bad = false;
  #pragma unroll
      for (int m = 0; m < 3; ++m) {
        if (m >= nbl) break;
        const double qm_old = qm_o[m];
        const double qm_new = mul_frac(f[m], q_new);
        st_if_new(v.qm + mat(m) * P + c, qm_old, qm_new);
        const double rn = rhom_new[m], ro = rho_o[m];
        em_new[m] = 0.;
        if (dgt(rn, thr) && dgt(ro, thr)) {
          // 1/rho_m: in a pure cell the material density is the cell's,
          // bit for bit, and so is its reciprocal (at rest both are 1/rho_old)
          const bool rn_cell = ubits(rn) == ubits(rho_new), ro_cell = ubits(ro) == ubits(rho_old);
          double irn = 0., iro = 0.;
          bool eq_inv;
          if (rest && rn_cell && ro_cell) {
            eq_inv = true;  // both 1 / rho_old, finite; not formed
          } else {
            if (!have_irho && (rn_cell || ro_cell)) {
              irho_old = div_ip(1.0, rho_old);
              irho_new = irho_old;  // rest: rho_new == rho_old
              have_irho = true;
            }
            irn = rn_cell ? irho_new : div_ip(1.0, rn);
            iro = ro_cell ? irho_old : div_ip(1.0, ro);
            eq_inv = ubits(irn) == ubits(iro) && is_finite(irn);
          }
          const double em_old = em_o[m], pm_old = pm_o[m];
          constexpr unsigned long long kBig = 0x7fd0000000000000ull;   // 2^1022
          constexpr unsigned long long kSafe = 0x5fe0000000000000ull;  // 2^511
          const double hg = hgm1_of(v, mat(m));
          if (eq_inv && nz(em_old) && !is_nan(em_old) &&
              (ubits(pm_old) & kMag) < kBig &&
              (v.pseudo_centree != 0 || (ubits(qm_new) & kMag) < kBig) &&
              (ubits(hg) & kMag) < kSafe && (ubits(rn) & kMag) < kSafe) {
            // specific volume unchanged: dvi = irn - iro = +0, so the
            // work term (0.5 pm + pseudo) * dvi is a zero (its factor is
            // finite; the centred pseudo is 0 then), num = em - (a zero) =
            // em, den = 1 + (a zero) = 1 and em / 1 = em
            em_new[m] = em_old;
          } else {
            const double dvi = eq_inv ? 0.0 : irn - iro;  // x - x = +0 (finite x)
            double pseudo = 0.;
            if ((v.pseudo_centree == 1) && pos((qm_new + qm_old) * dvi))
              pseudo = half(qm_new + qm_old);
            if (v.pseudo_centree == 0) pseudo = qm_new;
            const double den = 1 + hg * rn * dvi;
            const double num = em_old - (half(pm_old) + pseudo) * dvi;
            em_new[m] = qdiv(num, den);  // den is exactly 1 at rest
          }
          const double te = mul_frac(mf[m], em_new[m]);
          e_new = e_first ? plus_zero(te) : addz(e_new, te);
          e_first = false;
          if (pos(v.energy_limit) && abs_gt(em_new[m], v.energy_limit)) bad = true;
        }
      }
      if (bad) {
        atomicOr(&C.err, HYDRO_ERR_ENERGY);
        atomicMin((unsigned long long*)&C.err_cell, (unsigned long long)c);
      }
      // computeEOS: only the materials' sound speeds and the Void state
      // matter here (the pressures are recomputed after the remap)
  #pragma unroll
      for (int m = 0; m < 3; ++m) {
        if (m >= nbl) break;
        if (eos_of(v, mat(m)) != HYDRO_EOS_PERFECT_GAS) {  // Void: state kept
          cm_new[m] = v.cm[mat(m) * P + c];
          em_new[m] = v.em[mat(m) * P + c];
        }
      }
      unsigned void_mask = 0;  // the run's Void materials
  #pragma unroll
      for (int m = 0; m < 3; ++m)
        if (m < nb && eos_of(v, m) == HYDRO_EOS_VOID) void_mask |= 1u << m;
      if (void_mask) e_new = 0.;
      // computePressionMoyenne: max of the in-place c and the materials'
      // sound speeds, replaced by the mixture's when rho > 0 (then the
      // materials' values are not needed)
      double cc = c_old;
      double sarg_new = from_bits(kNoRoot);
      if (pos(rho_new)) {
        // c_old is sqrt(g0 (g0 - 1) e) of the energy in sarg: the same energy
        // (bit for bit) gives the same root
        cc = (ubits(e_new) == ubits(sarg_old) && !is_nan(e_new)) ? c_old
                                                                 : sqrt_ip(v.g0gm1 * e_new);
        sarg_new = e_new;
      } else {
  #pragma unroll
        for (int m = 0; m < 3; ++m) {
          if (m >= nbl) break;
          if (eos_of(v, mat(m)) == HYDRO_EOS_PERFECT_GAS) {
            const double g = gamma_of(v, mat(m));
            cm_new[m] = sqrt_ip(g * (g - 1.0) * em_new[m]);
          }
          cc = smax(cc, cm_new[m]);
        }
      }
      if (void_mask) e_new = void_energy(void_mask, e_new, mf[0], mf[1], mf[2], em_new[0],
                                         em_new[1], em_new[2]);
      st_if_new(v.c + c, c_old, cc);
      st_if_new(v.sarg + c, sarg_old, sarg_new);
      if (v.projection == 0) {
        // Without the remap no later kernel forms the state after this
        // phase: its densities, energies, pseudo-viscosity, and the
        // pressures of computeEOSGP ((gamma - 1) rho e; a Void material
        // keeps its pressure) and computePressionMoyenne (the sum from 0.0
        // of f p) are stored here (PhaseLagrange.cc:392-485)
        double pmean = 0.;
  #pragma unroll
        for (int m = 0; m < 3; ++m) {
          if (m >= nbl) break;
          const double pmm = (eos_of(v, mat(m)) == HYDRO_EOS_PERFECT_GAS)
                                 ? gm1_of(v, mat(m)) * rhom_new[m] * em_new[m]
                                 : pm_o[m];
          pmean += f[m] * pmm;
          v.pm[mat(m) * P + c] = pmm;
          v.rhom[mat(m) * P + c] = rhom_new[m];
          v.em[mat(m) * P + c] = em_new[m];
          if (!pos(rho_new) && eos_of(v, mat(m)) == HYDRO_EOS_PERFECT_GAS)
            v.cm[mat(m) * P + c] = cm_new[m];
        }
        v.p[c] = pmean;
        v.rho[c] = rho_new;
        v.e[c] = e_new;
        v.q[c] = q_new;
      }
    } else {
      // no Lagrange phase (advection cases): energy and q are carried over
      e_new = v.e[c];
      q_new = v.q[c];
      // updatePeriodicBoundaryConditions: first and last column take the
      // initial density of the row's first cell
      if (v.periodic_x && (j == v.nx - 1 || j == 0)) rho_new = ld(v.rho0_left, i);
    }
    // ---- PrepareRemap (cell part): the conserved values per material
    // (volume, mass, energy; indexes known at compile time, so they stay in
    // registers) and the pseudo-viscosity slot 3 nbmat
    double uv[3], um[3], ue[3];
  #pragma unroll
    for (int m = 0; m < 3; ++m) {
      if (m >= nbl) break;
      uv[m] = mul_frac(f[m], vol);
      const double mv = mul_frac(mf[m], vol);  // (mf * vol) * rho_new ...
      um[m] = mulz(mv, rho_new);
      ue[m] = mulz(mulz(mv, rho_new), e_new);
    }
    const double uq = mulz(q_new, vol);  // reference slot 3*nbmat+3
  #pragma unroll
    for (int m = 0; m < 3; ++m) {
      if (m >= nbl) break;
      v.UL[mat(m) * P + c] = uv[m];
      v.UL[(nb + mat(m)) * P + c] = um[m];
      v.UL[(2 * nb + mat(m)) * P + c] = ue[m];
    }
    v.UL[3 * nb * P + c] = uq;
    if (v.pb == 1) {
      double sv = plus_zero(uv[0]);
  #pragma unroll
      for (int m = 1; m < 3; ++m)
        if (m < nbl) sv = addz(sv, uv[m]);
  #pragma unroll
      for (int m = 0; m < 3; ++m) {
        if (m >= nbl) break;
        v.Phi[mat(m) * P + c] = qdiv(uv[m], sv);
        v.Phi[(nb + mat(m)) * P + c] = nz(uv[m]) ? qdiv(um[m], uv[m]) : 0.;
        v.Phi[(2 * nb + mat(m)) * P + c] = nz(um[m]) ? qdiv(ue[m], um[m]) : 0.;
      }
      v.Phi[3 * nb * P + c] = q_new;
    } else {
      const SharedDiv Sv = shared_div(vol);  // one denominator, 3 nbmat + 1 quotients
  #pragma unroll
      for (int m = 0; m < 3; ++m) {
        if (m >= nbl) break;
        v.Phi[mat(m) * P + c] = qdiv_shared(Sv, uv[m]);
        v.Phi[(nb + mat(m)) * P + c] = qdiv_shared(Sv, um[m]);
        v.Phi[(2 * nb + mat(m)) * P + c] = qdiv_shared(Sv, ue[m]);
      }
      v.Phi[3 * nb * P + c] = qdiv_shared(Sv, uq);
    }
    if (single && nb > 1) {
      // the other materials, as the loops form them for f = mf = +0 and a
      // density at most the threshold: q_m = +0 * q; U = (+0 * vol, (+0 *
      // vol) * rho, ((+0 * vol) * rho) * e); Phi = +0 / V or 0 (with
      // PenteBorne), +0 / vol and the two zeros over vol (without): zeros
      // whose signs follow from q, rho, e (vol > 0).  Non-finite q, rho or e
      // take the products themselves.
      constexpr unsigned long long kS = 0x8000000000000000ull;
      if (is_finite(q_new) && is_finite(rho_new) && is_finite(e_new)) {
        const double zq = from_bits(ubits(q_new) & kS);
        const double zm = from_bits(ubits(rho_new) & kS);
        const double ze = from_bits((ubits(rho_new) ^ ubits(e_new)) & kS);
  #pragma unroll
        for (int m = 0; m < 3; ++m) {
          if (m >= nb) break;
          if (m == p) continue;
          v.qm[m * P + c] = zq;
          v.UL[m * P + c] = 0.0;
          v.UL[(nb + m) * P + c] = zm;
          v.UL[(2 * nb + m) * P + c] = ze;
          v.Phi[m * P + c] = 0.0;
          v.Phi[(nb + m) * P + c] = (v.pb == 1) ? 0.0 : zm;
          v.Phi[(2 * nb + m) * P + c] = (v.pb == 1) ? 0.0 : ze;
        }
      } else {
        const double zm = mulz(0.0, rho_new), ze = mulz(mulz(0.0, rho_new), e_new);
  #pragma unroll
        for (int m = 0; m < 3; ++m) {
          if (m >= nb) break;
          if (m == p) continue;
          v.qm[m * P + c] = mul_frac(0.0, q_new);
          v.UL[m * P + c] = 0.0;
          v.UL[(nb + m) * P + c] = zm;
          v.UL[(2 * nb + m) * P + c] = ze;
          v.Phi[m * P + c] = 0.0;
          v.Phi[(nb + m) * P + c] = (v.pb == 1) ? 0.0 : qdiv(zm, vol);
          v.Phi[(2 * nb + m) * P + c] =
              (v.pb == 1) ? (nz(zm) ? qdiv(ze, zm) : 0.0) : qdiv(ze, vol);
        }
      }
    }
    v.rL[c] = rho_new;
    if (!(rest && held)) {
      v.vL[c] = vol;
      // Lagrangian centroid (PrepareRemap.cc:65-90) and the widths behind
      // HvLagrange for both sweep directions
      v.XcL[c] = G.xc0;
      v.XcL[P + c] = G.xc1;
      if (v.order > 1) {
        v.Hx[c] = G.hx;
        v.Hy[c] = G.hy;
      }
    }
    if (v.gL && v.projection == 1 && rest != held) v.gL[c] = rest ? 1 : 0;
  }
};

// Face normal velocity (PrepareRemap.cc:42-63): mean of the two nodes'
// Lagrange velocities along the face normal; "+ 0.0" is the dot product's
// zero start for the other axis.
// (addz: the sum of two zero velocities, the case at rest, on the integer
// pipe)
DV double fnv_vertical(const RunView& v, long long na, long long nb) {
  return plus_zero(half(addz(v.u[na], v.u[nb])));
}
DV double fnv_horizontal(const RunView& v, long long na, long long nb) {
  return plus_zero(half(addz(v.u[v.npitch + na], v.u[v.npitch + nb])));
}
// either of the two, by the sweep direction: the component along the sweep
DV double face_mean(const RunView& v, bool dirx, long long na, long long nb) {
  const double* u = v.u + (dirx ? 0 : v.npitch);
  return plus_zero(half(addz(u[na], u[nb])));
}

// ----------------------------------------------------------- remap sweep
// Face gradients of one sweep for runs without PenteBorne
// (Remap::computeGradPhiFace{1,2}, remap/PhaseRemap1.cc:22-55,
// PhaseRemap2.cc:21-55): one thread per inner face perpendicular to the
// sweep, (Phi(front) - Phi(back)) / deltaxLagrange, into the face-gradient
// planes.  Every component has a slope there, and each face's gradients
// are formed once (the PenteBorne slope kernel forms its few itself).
struct FaceGrad {
  int sweep;
  __device__ __forceinline__ void operator()(const RunView& v, int i, int j) const {
    if (v.order != 2 || v.pb != 0) return;
    const Ctrl& C = *v.ctrl;
    const bool dirx = (sweep == 1) ? C.x_then_y : !C.x_then_y;
    const long long P = v.pitch, FP = v.fpitch;
    long long back, front, fidx;
    int ax;
    if (dirx) {
      if (i >= v.ny || j < 1 || j >= v.nx) return;
      front = (long long)i * v.nx + j;
      back = front - 1;
      fidx = (long long)i * (v.nx + 1) + j;
      ax = 0;
    } else {
      if (j >= v.nx || i < 1 || i >= v.ny) return;
      back = (long long)i * v.nx + j;
      front = back - v.nx;
      fidx = (long long)i * v.nx + j;
      ax = 1;
    }
    const double dx = plus_zero(v.XcL[ax * P + front] - v.XcL[ax * P + back]);
    for (int k = 0; k < v.ncomp; ++k)
      v.phiG[k * FP + fidx] = qdiv(v.Phi[k * P + front] - v.Phi[k * P + back], dx);
  }
};

// Limited slopes and plateau-slope integrals of one sweep
// (Remap::computeGradPhiFace{1,2} + computeGradPhi{1,2},
// remap/PhaseRemap1.cc:22-323, remap/PhaseRemap2.cc:21-323).
// The plateau-slope reconstruction of one component and its integrals over
// the back / front swept lengths and the dual length (computeFluxPP,
// remap/UtilesRemap-Impl.h:182-257).  Only cells where the component is not
// at an extremum need it (the others take "formule 16"): kept out of line so
// that the slope kernel carries neither its registers nor its code.
struct PPFluxes {
  double a, b, d;
};
__device__ __noinline__ PPFluxes pp_fluxes_call(int plim, double thr, double y0, double yp,
                                                double ym, double hh, double hp, double hm,
                                                double grad, double ppa, double ppb, double ppd,
                                                bool do_ab, bool dual_k) {
  const PPShape sh = pp_shape(plim, thr, y0, yp, ym, hh, hp, hm, grad);
  PPFluxes r;
  r.a = do_ab ? pp_integral(sh, half(-hh), half(-hh) + ppa, hh, y0, yp, ym, ppa) : 0.;
  r.b = do_ab ? pp_integral(sh, half(hh) - ppb, half(hh), hh, y0, yp, ym, ppb) : 0.;
  r.d = dual_k ? pp_integral(sh, 0., ppd, hh, y0, yp, ym, ppd) : 0.;
  return r;
}

// PB: 2 = the run's option decides (batched launches), 0 / 1 = compiled
// for runs without / with PenteBorne only (plain launches).
template <int PB>
struct SweepGradT {
  int sweep;
  // Fused sweeps (PenteBorne): the cell's flag and integrals go to a tile in
  // shared memory (tz[ti]; tr / tv[k * ts + ti]) instead of pbz / dPAr /
  // dPAv, and (phi2) the second sweep reads the Phi of a cell the first
  // sweep changed from Phi2, where that sweep wrote it.
  unsigned char* tz = nullptr;
  double *tr = nullptr, *tv = nullptr;
  int ti = 0, ts = 0;
  bool phi2 = false;
  DV const double* phi_of(const RunView& v, long long x) const {
    return (phi2 && v.u1s[x] == 0) ? v.Phi2 + x : v.Phi + x;
  }
  DV void put_z(const RunView& v, long long c, unsigned char z) const {
    if (tz) tz[ti] = z;
    else v.pbz[c] = z;
  }
  __device__ __forceinline__ void operator()(const RunView& v, int i, int j) const {
    const int pb = (PB == 2) ? v.pb : PB;
    // no slopes at order 1, nor at order 3 without PenteBorne (batched
    // launches; the plain cycle does not launch these then)
    if (v.order <= 1 || (v.order == 3 && pb == 0)) return;
    const Ctrl& C = *v.ctrl;
    if (i >= v.ny || j >= v.nx) return;
    const bool dirx = (sweep == 1) ? C.x_then_y : !C.x_then_y;
    const long long P = v.pitch;
    const long long c = (long long)i * v.nx + j;
    const double* H = dirx ? v.Hx : v.Hy;
    // reference naming: cf = "front" (right / below), cb = "back" (left / above)
    long long cf, cb;
    bool has_gp, has_gm;       // gradient faces exist (inner)
    if (dirx) {
      cf = (j < v.nx - 1) ? c + 1 : c;
      cb = (j > 0) ? c - 1 : c;
      has_gp = (j < v.nx - 1);  // right face
      has_gm = (j > 0);         // left face
    } else {
      cf = (i > 0) ? c - v.nx : c;
      cb = (i < v.ny - 1) ? c + v.nx : c;
      has_gp = (i > 0);          // bottom face
      has_gm = (i < v.ny - 1);   // top face
    }
    // With PenteBorne the two face gradients are formed here
    // (Remap::computeGradPhiFace{1,2}, remap/PhaseRemap1.cc:22-55):
    // (Phi(front) - Phi(back)) / (XcL(front) - XcL(back)) with the
    // reference's back / front cells, the "plus" face between c (back) and
    // cf (front), the "minus" face between cb (back) and c (front).  Each
    // inner face's gradient is formed by both of its cells with the same
    // operations, so no face plane is written and read back, and a cell that
    // takes the no-flux exit below forms neither (the few integrated
    // components only).  Without PenteBorne FaceGrad formed them once per
    // face for every component.
    // Eucclhyd carries momentum (and kinetic energy) after the material
    // components instead of the VNR pseudo-viscosity, and has no dual remap
    const bool euc = (v.scheme == HYDRO_SCHEME_EUCCLHYD);
    const bool cfd = !euc && (v.dual_method == 2);
    const int ncomp = v.ncomp, nb = v.nbmat;
    // PenteBorne: Flux_sortant of the two faces, dual normal velocity, face
    // lengths, and the swept lengths they give
    double ppa = 0., ppb = 0., ppd = 0., flen = 0.;
    if (pb == 1) {
      const long long n0 = (long long)i * (v.nx + 1) + j;
      // the four node velocities along the sweep all zeros (and dt finite):
      // each face velocity is plus_zero(half(+-0 + +-0)) = +0, so every
      // swept length below is a zero and the cell takes the no-flux exit
      // without forming them
      {
        const long long NP = v.npitch, o = dirx ? 0 : NP;
        const unsigned long long z = ubits(v.u[o + n0]) | ubits(v.u[o + n0 + 1]) |
                                     ubits(v.u[o + n0 + v.nx + 1]) | ubits(v.u[o + n0 + v.nx + 2]);
        if ((z & kMag) == 0 && is_finite(C.dt_n)) {
          put_z(v, c, 3);  // both integral planes all +0.0, not stored
          if (cfd) {
            const double l = dirx ? ld(v.flv, i) : ld(v.flh, j);
            const double zf = 0.0 * half(l + l);
            for (int m = 0; m < nb; ++m) v.DPF[m * P + c] = zf;
          }
          return;
        }
      }
      // the faces' nodes and normals selected by direction, then one set of
      // operations (two branches, if-converted, would issue both sets): the
      // left and right faces of an x sweep (fnv_vertical), the bottom and
      // top faces of a y sweep (fnv_horizontal)
      const long long W = v.nx + 1;
      const long long a1 = dirx ? n0 + W : n0 + 1, b0 = dirx ? n0 + 1 : n0 + W;
      const double fa_v = face_mean(v, dirx, n0, a1);
      const double fb_v = face_mean(v, dirx, b0, n0 + W + 1);
      const int qa = dirx ? 0 : 2;
      const double Fa = mul_pm1(fa_v, nout_at(v, qa, c));
      const double Fb = mul_pm1(fb_v, nout_at(v, qa + 1, c));
      const double l = dirx ? ld(v.flv, i) : ld(v.flh, j);
      flen = half(l + l);
      const double fdual = half(fa_v + fb_v);
      const double dt = C.dt_n;
      ppa = half(Fa + fabs(Fa)) * dt;
      ppb = half(Fb + fabs(Fb)) * dt;
      ppd = half(fdual + fabs(fdual)) * dt;
      // nothing leaves the cell through either face, nor through its dual
      // half-faces: every flux stored below is then exactly 0 (0 * flen for
      // the dual one) whatever the slopes, so they are not formed
      if (iszero(ppa) && iszero(ppb) && (!cfd || iszero(ppd))) {
        put_z(v, c, 3);
        if (cfd) {
          const double z = 0.0 * flen;
          for (int m = 0; m < nb; ++m) v.DPF[m * P + c] = z;
        }
        return;
      }
    }
    const bool vp = (v.pb_mixte == 1) &&
                    (v.mixte[c] == 0 && v.mixte[cf] == 0 && v.mixte[cb] == 0 &&
                     v.pure[c] == v.pure[cf] && v.pure[c] == v.pure[cb]);
    int lim = v.limiter;
    if ((pb == 1) && vp) lim = v.limiter_pure;
    // "plus" / "minus" neighbours in computeAndLimitGradPhi's argument order
    const long long cp = dirx ? cf : cb, cm = dirx ? cb : cf;
    const double h0 = H[c], hp = H[cp], hm = H[cm];
    // which components are integrated with PenteBorne: volumes always;
    // masses for the pure variant; masses + energies (+ momentum for
    // Eucclhyd) for the "complet" variant; the dual flux needs the mass
    // components (computeFluxPP, UtilesRemap-Impl.h:259-313).  Only their
    // limited slopes are read; without PenteBorne every slope is stored.
    const int nint = (v.pb_complet == 1) ? (euc ? ncomp : 3 * nb) : (vp ? 2 * nb : nb);
    const int nuse = (cfd && nint < 2 * nb) ? 2 * nb : nint;
    const int ngrad = (pb == 1) ? nuse : ncomp;
    const int ax = dirx ? 0 : 1;
    const double xc = v.XcL[ax * P + c];
    // one denominator per face, shared by its components (the IEEE quotient
    // bit for bit, see shared_div)
    const double dxp = has_gp ? plus_zero(v.XcL[ax * P + cf] - xc) : 1.0;
    const double dxm = has_gm ? plus_zero(xc - v.XcL[ax * P + cb]) : 1.0;
    const SharedDiv Sp = shared_div(pb == 1 ? dxp : 1.0);
    const SharedDiv Sm = shared_div(pb == 1 ? dxm : 1.0);
    // Without PenteBorne the order-2 face values (SweepFace) are formed here:
    // a face's value is Phi(cu) + (x_f - XcL(cu)) * slope(cu) of its upwind
    // cell cu = pos(fnv * dxl) ? back : front, with dxl = XcL(front) -
    // XcL(back), the plus face's denominator above (c its back cell) or the
    // minus face's (c its front cell).  Each inner face has one upwind cell,
    // which writes its value; the slopes themselves are not stored.  (The
    // update cannot form these values: in the first sweep it rewrites Phi,
    // which a neighbour's face value reads.)
    bool up_p = false, up_m = false;
    double sp = 0., sm = 0.;
    long long fp = 0, fm = 0;
    const long long FP = v.fpitch;
    if (dirx) {
      fm = (long long)i * (v.nx + 1) + j;  // left face
      fp = fm + 1;                         // right face
    } else {
      fp = (long long)i * v.nx + j;        // bottom face
      fm = fp + v.nx;                      // top face
    }
    if (pb == 0) {
      const long long n0 = (long long)i * (v.nx + 1) + j;
      // x sweep: minus = left face (n0, n0 + W), plus = right face;
      // y sweep: plus = bottom face (n0, n0 + 1), minus = top face
      const long long W = v.nx + 1;
      const long long lo1 = dirx ? n0 + W : n0 + 1, hi0 = dirx ? n0 + 1 : n0 + W;
      const double f_lo = face_mean(v, dirx, n0, lo1), f_hi = face_mean(v, dirx, hi0, n0 + W + 1);
      const double fnv_m = dirx ? f_lo : f_hi, fnv_p = dirx ? f_hi : f_lo;
      const double xf_m = dirx ? ld(v.xs, j) : ld(v.ys, i + 1);
      const double xf_p = dirx ? ld(v.xs, j + 1) : ld(v.ys, i);
      up_p = has_gp && pos(fnv_p * dxp);   // c is the plus face's back cell
      up_m = has_gm && !pos(fnv_m * dxm);  // c is the minus face's front cell
      sp = plus_zero(xf_p - xc);
      sm = plus_zero(xf_m - xc);
    }
    // Phi of the cell and of its front / back neighbours
    const double* Pc = phi_of(v, c);
    const double* Pf = phi_of(v, cf);
    const double* Pb = phi_of(v, cb);
    const double* Pp = dirx ? Pf : Pb;  // plus / minus neighbours
    const double* Pm = dirx ? Pb : Pf;
    double grad[kMaxComp];
    for (int k = 0; k < ngrad; ++k) {
      const double y0 = Pc[k * P];
      const double yp = Pp[k * P], ym = Pm[k * P];
      double gp = 0., gm = 0.;
      if (pb == 1) {
        if (has_gp) gp = qdiv_shared(Sp, Pf[k * P] - y0);
        if (has_gm) gm = qdiv_shared(Sm, y0 - Pb[k * P]);
      } else {
        if (has_gp) gp = v.phiG[k * FP + fp];
        if (has_gm) gm = v.phiG[k * FP + fm];
      }
      grad[k] = limit_grad1(lim, gp, gm, yp, ym, h0, hp, hm);
      if (pb == 0) {
        // y0 + s * slope exactly (a zero slope on the integer pipe)
        if (up_p) v.phiF[k * FP + fp] = addz(y0, mulz(sp, grad[k]));
        if (up_m) v.phiF[k * FP + fm] = addz(y0, mulz(sm, grad[k]));
      }
    }
    if (pb == 1) {
      const int plim = vp ? v.limiter_pure : v.limiter;
      double Fr[kMaxComp], Fv[kMaxComp];
      const double hh = h0;
      for (int k = 0; k < nuse; ++k) {
        const double y0 = Pc[k * P];
        const double yp = Pp[k * P], ym = Pm[k * P];
        const bool dual_k = cfd && k >= nb && k < 2 * nb;
        double fa_, fb_, fd_;
        if (nonneg((yp - y0) * (ym - y0))) {
          // "formule 16" (UtilesRemap-Impl.h:201-203): the reference replaces
          // every integral of this component by y0 * swept length, so the
          // reconstruction is not built (y0, a volume fraction here, is
          // mostly exactly 1 or 0: mul_frac)
          fa_ = mul_frac(y0, ppa);
          fb_ = mul_frac(y0, ppb);
          fd_ = dual_k ? mul_frac(y0, ppd) : 0.;
        } else {
          const PPFluxes r = pp_fluxes_call(plim, v.threshold, y0, yp, ym, hh, hp, hm, grad[k],
                                            ppa, ppb, ppd, k < nint, dual_k);
          fa_ = r.a;
          fb_ = r.b;
          fd_ = r.d;
        }
        if (k < nint) {
          Fr[k] = fa_;
          Fv[k] = fb_;
        }
        if (dual_k) {
          double d = fd_;
          if (iszero(ppd)) d = 0.;
          v.DPF[(k - nb) * P + c] = d * flen;
        }
      }
      // derived fluxes
      auto finish = [&](double* F, double* out, long long stride) {
        if (v.pb_complet == 1) {
          double sfm = 0., sfv = plus_zero(F[0]);
          for (int m = 1; m < nb; m++) sfv += F[m];
          if (dgt(fabs(sfv), v.threshold)) {
            for (int m = 0; m < nb; m++) {
              if (!vp) F[nb + m] = div_ip(F[nb + m], sfv) * F[m];
              F[2 * nb + m] = div_ip(F[2 * nb + m], sfv) * F[nb + m];
              sfm = (m == 0) ? plus_zero(F[nb + m]) : sfm + F[nb + m];
            }
            if (euc)
              for (int k = 3 * nb; k < ncomp; ++k) F[k] = div_ip(F[k], sfv) * sfm;
            else
              F[3 * nb] = Pc[3 * nb * P] * sfv;
          } else {
            for (int k = 0; k < ncomp; ++k) F[k] = 0.0;
          }
        } else {
          double sfv = 0., sfm = 0.;
          for (int m = 0; m < nb; m++) {
            // an absent material's volume flux is exactly 0 (mul_frac)
            if (!vp) F[nb + m] = mul_frac(F[m], Pc[(nb + m) * P]);
            F[2 * nb + m] = mul_frac(F[nb + m], Pc[(2 * nb + m) * P]);
            sfm = (m == 0) ? plus_zero(F[nb + m]) : sfm + F[nb + m];
            sfv = (m == 0) ? plus_zero(F[m]) : sfv + F[m];
          }
          if (euc)
            for (int k = 3 * nb; k < ncomp; ++k) F[k] = Pc[k * P] * sfm;
          else
            F[3 * nb] = Pc[3 * nb * P] * sfv;
        }
        for (int k = 0; k < ncomp; ++k) out[k * stride] = F[k];
      };
      // a zero swept length makes every integral of that side exactly +0.0:
      // recorded in pbz instead of stored (bit 0: dPAr, bit 1: dPAv)
      put_z(v, c, (iszero(ppa) ? 1 : 0) | (iszero(ppb) ? 2 : 0));
      if (!iszero(ppa)) {
        if (tz) finish(Fr, tr + ti, ts);
        else finish(Fr, v.dPAr + c, P);
      }
      if (!iszero(ppb)) {
        if (tz) finish(Fv, tv + ti, ts);
        else finish(Fv, v.dPAv + c, P);
      }
    }
  }
};

// Order-3 face values (ComputeFluxOrdre3) share most of their work between
// neighbouring faces: each cell's gradient (eval_grad) enters four faces,
// each face's interpolated value (eval_ystar) three.  They are computed once
// per sweep by O3Grad (one thread per cell) and O3Ystar (one thread per
// inner face) and read by SweepFace for faces whose six-cell stencil is not
// clamped at the ends of the row / column (the two faces next to each end
// compute everything themselves).  Same arithmetic, same values.
// The parabola and its interval (o3_tail) and the face's time-step
// coefficients behind calls: inline, the compiler issues them under a
// predicate for every component, also where the face does not move.
struct O3Dt {
  double Q1, Q2, R1, R2;
  bool fwd;
};
__device__ __noinline__ O3Dt o3_dt_call(double h2, double h3, double vdt) {
  const double h[4] = {0., 0., h2, h3};
  O3Face F;
  o3_face_dt(F, h, vdt);
  return O3Dt{F.Q1, F.Q2, F.R1, F.R2, F.fwd};
}
__device__ __noinline__ double o3_tail_call(O3Dt d, double ys0, double ys1, double ys2,
                                            double y1, double ym, double yp, double y4) {
  O3Face F;
  F.Q1 = d.Q1;
  F.Q2 = d.Q2;
  F.R1 = d.R1;
  F.R2 = d.R2;
  F.fwd = d.fwd;
  const double ys[3] = {ys0, ys1, ys2};
  return o3_tail(F, ys, y1, ym, yp, y4);
}
DV double o3_value(const RunView& v, int sweep, int k, long long c) {
  // the component value the order-3 reconstruction works on: U / vLagrange,
  // which is what Phi holds without PenteBorne (same division)
  if (v.pb == 0) return v.Phi[k * v.pitch + c];
  const double* Uin = (sweep == 1) ? v.UL : v.U1;
  return qdiv(Uin[k * v.pitch + c], v.vL[c]);
}
struct O3Grad {
  int sweep;
  __device__ __forceinline__ void operator()(const RunView& v, int i, int j) const {
    if (i >= v.ny || j >= v.nx || !v.o3g) return;
    const Ctrl& C = *v.ctrl;
    const bool dirx = (sweep == 1) ? C.x_then_y : !C.x_then_y;
    const long long P = v.pitch;
    const long long c = (long long)i * v.nx + j;
    const double* H = dirx ? v.Hx : v.Hy;
    const int q = dirx ? j : i, n = dirx ? v.nx : v.ny;
    const long long st = dirx ? 1 : v.nx;  // cell stride along the axis
    // neighbours clamped at the ends, as the face stencil clamps them
    const long long cm = q > 0 ? c - st : c, cp = q < n - 1 ? c + st : c;
    double G0, A, B;
    // widths equal (bit for bit) to the rest widths: the coefficients formed
    // from those at set-up
    const double* Hr = v.geo0 + (dirx ? 3 : 4) * P;
    const double* oc = v.o3c ? v.o3c + (dirx ? 0 : 8) * P : nullptr;
    if (oc && ubits(H[cm]) == ubits(ld(Hr, cm)) && ubits(H[c]) == ubits(ld(Hr, c)) &&
        ubits(H[cp]) == ubits(ld(Hr, cp))) {
      G0 = ld(oc, c);
      A = ld(oc, P + c);
      B = ld(oc, 2 * P + c);
    } else {
      o3_grad_coef(H[cm], H[c], H[cp], G0, A, B);
    }
    for (int k = 0; k < v.ncomp; ++k)
      v.o3g[k * P + c] = o3_grad(G0, A, B, o3_value(v, sweep, k, cm),
                                 o3_value(v, sweep, k, c), o3_value(v, sweep, k, cp));
  }
};
// the inner face between positions q-1 and q of cell c's row / column
struct O3Ystar {
  int sweep;
  __device__ __forceinline__ void operator()(const RunView& v, int i, int j) const {
    if (i >= v.ny || j >= v.nx || !v.o3g) return;
    const Ctrl& C = *v.ctrl;
    const bool dirx = (sweep == 1) ? C.x_then_y : !C.x_then_y;
    const long long P = v.pitch, FP = v.fpitch;
    const long long c = (long long)i * v.nx + j;
    const int q = dirx ? j : i, n = dirx ? v.nx : v.ny;
    if (q < 1) return;
    const double* H = dirx ? v.Hx : v.Hy;
    const long long st = dirx ? 1 : v.nx;
    const long long cm = c - st;                           // q-1
    const long long cmm = q > 1 ? cm - st : cm;            // left(q-1)
    const long long cpp = q < n - 1 ? c + st : c;          // right(q)
    double T[5];
    // widths equal (bit for bit) to the rest widths: the coefficients formed
    // from those at set-up
    const double* Hr = v.geo0 + (dirx ? 3 : 4) * P;
    const double* oc = v.o3c ? v.o3c + (dirx ? 3 : 11) * P : nullptr;
    if (oc && ubits(H[cmm]) == ubits(ld(Hr, cmm)) && ubits(H[cm]) == ubits(ld(Hr, cm)) &&
        ubits(H[c]) == ubits(ld(Hr, c)) && ubits(H[cpp]) == ubits(ld(Hr, cpp))) {
  #pragma unroll
      for (int t = 0; t < 5; ++t) T[t] = ld(oc, t * P + c);
    } else {
      o3_ystar_coef(H[cmm], H[cm], H[c], H[cpp], T);
    }
    const long long f = dirx ? (long long)i * (v.nx + 1) + j : c;
    for (int k = 0; k < v.ncomp; ++k)
      v.o3y[k * FP + f] = o3_ystar(T, o3_value(v, sweep, k, cm), o3_value(v, sweep, k, c),
                                   v.o3g[k * P + cm], v.o3g[k * P + c]);
  }
};

// Face values of one sweep (Remap::computeUpwindFaceQuantitiesForProjection
// {1,2}, remap/PhaseRemap1.cc:331-452, PhaseRemap2.cc:331-447).  One thread
// per inner face perpendicular to the sweep; face (i, j) is the left face of
// cell (i, j) (x sweep) or the bottom face of cell (i, j) (y sweep).
// ORDERS: 3 = the run's order decides (batched launches), 2 = orders 1-2
// only, 1 = order 3 only (the plain launches compile the two apart so that
// neither carries the other's registers).
template <int ORDERS>
struct SweepFaceT {
  int sweep;
  __device__ __forceinline__ void operator()(const RunView& v, int i, int j) const {
    // batched launches: an order-2 run without PenteBorne has its face
    // values from the slope kernel, a PenteBorne run of orders 1-2 forms them
    // in the update
    if (ORDERS == 3 && (v.order == 2 || (v.order == 1 && v.pb == 1))) return;
    const Ctrl& C = *v.ctrl;
    const bool dirx = (sweep == 1) ? C.x_then_y : !C.x_then_y;
    const long long P = v.pitch, FP = v.fpitch;
    const int ncomp = v.ncomp;
    long long cb, cf, fidx;
    if (dirx) {
      if (i >= v.ny || j < 1 || j >= v.nx) return;
      cb = (long long)i * v.nx + j - 1;  // back = left
      cf = cb + 1;                        // front = right
      fidx = (long long)i * (v.nx + 1) + j;
    } else {
      if (j >= v.nx || i < 1 || i >= v.ny) return;
      cb = (long long)i * v.nx + j;       // back = above
      cf = cb - v.nx;                     // front = below
      fidx = (long long)i * v.nx + j;
    }
    // the face's two nodes: (n0, n0 + W) for an x sweep (fnv_vertical),
    // (n0, n0 + 1) for a y sweep (fnv_horizontal); one set of operations
    const long long n0 = (long long)i * (v.nx + 1) + j;
    const double fnv = face_mean(v, dirx, n0, dirx ? n0 + v.nx + 1 : n0 + 1);
    double* out = v.phiF + fidx;
    const int ax = dirx ? 0 : 1;
    const bool low = (ORDERS == 2) || (ORDERS == 3 && v.order <= 2);
    if (low) {
      if (v.pb == 0) {
        const double dxl = plus_zero(v.XcL[ax * P + cf] - v.XcL[ax * P + cb]);
        const double xf = dirx ? ld(v.xs, j) : ld(v.ys, i);
        const long long cu = pos(fnv * dxl) ? cb : cf;
        const double s = plus_zero(xf - v.XcL[ax * P + cu]);
        // four components at a time, loads ahead of the stores
        for (int k0 = 0; k0 < ncomp; k0 += 4) {
          double a[4], g[4];
  #pragma unroll
          for (int t = 0; t < 4; ++t) {
            const int k = k0 + t;
            a[t] = (k < ncomp) ? v.Phi[k * P + cu] : 0.;
            g[t] = (k < ncomp) ? v.gP[k * P + cu] : 0.;
          }
  #pragma unroll
          for (int t = 0; t < 4; ++t)
            if (k0 + t < ncomp) out[(k0 + t) * FP] = a[t] + s * g[t];
        }
      }
      // (with PenteBorne the update forms the face values of orders 1-2 from
      // the integral planes and their zero flags: nothing to store here)
    } else {
      // order 3: six cells along the sweep, "minus" side first, clamped
      long long cs[6];
      if (dirx) {
        const int jb = j - 1, jf = j;
        const int jbb = jb > 0 ? jb - 1 : jb, jbbb = jbb > 0 ? jbb - 1 : jbb;
        const int jff = jf < v.nx - 1 ? jf + 1 : jf;
        const int jfff = jff < v.nx - 1 ? jff + 1 : jff;
        const long long r = (long long)i * v.nx;
        cs[0] = r + jbbb; cs[1] = r + jbb; cs[2] = cb; cs[3] = cf;
        cs[4] = r + jff; cs[5] = r + jfff;
      } else {
        const int i_f = i - 1, i_b = i;
        const int iff = i_f > 0 ? i_f - 1 : i_f, ifff = iff > 0 ? iff - 1 : iff;
        const int ibb = i_b < v.ny - 1 ? i_b + 1 : i_b;
        const int ibbb = ibb < v.ny - 1 ? ibb + 1 : ibb;
        cs[0] = (long long)ifff * v.nx + j; cs[1] = (long long)iff * v.nx + j;
        cs[2] = cf; cs[3] = cb;
        cs[4] = (long long)ibb * v.nx + j; cs[5] = (long long)ibbb * v.nx + j;
      }
      const double* H = dirx ? v.Hx : v.Hy;
      const double vdt = fnv * C.dt_n;
      double h[6];
      for (int t = 0; t < 6; ++t) h[t] = H[cs[t]];
      // every division of the order-3 value depends on the face only; the
      // coefficients shared with the neighbouring faces come from O3Coef
      // unless the stencil is clamped (faces next to the ends)
      const int q = dirx ? j : i, n = dirx ? v.nx : v.ny;
      if (v.o3g && q >= 2 && q <= n - 2) {
        // interior face: gradients and interpolated values from O3Grad /
        // O3Ystar, only the parabola and its interval here
        O3Dt F;
        bool have_F = false;
        const long long fst = dirx ? 1 : v.nx;  // face stride along the axis
        // A face that does not move: its normal velocity is exactly zero, so
        // (without PenteBorne) the sweep update multiplies its value by a
        // zero coefficient, and the flux is a zero whatever the value, as
        // long as it is finite.  It is: with vdt = +-0, dt finite and a
        // positive finite upwind width, Q1 = Q2 = +-0 and the value is the
        // interpolated one clamped into a finite interval, once the seven
        // inputs below are finite and under 2^1000 (no sum or the factor 6
        // overflows).  The value itself is then not formed: 0 is stored
        // (the product's zero may differ in sign, which no later sum sees).
        constexpr unsigned long long kMod = 2023ull << 52;  // 2^1000
        const bool still = v.pb == 0 && iszero(fnv) && is_finite(C.dt_n) && pos(h[2]) &&
                           is_finite(h[2]);
        for (int k = 0; k < ncomp; ++k) {
          const double ys[3] = {v.o3y[k * FP + fidx - fst], v.o3y[k * FP + fidx],
                                v.o3y[k * FP + fidx + fst]};
          const double y1 = o3_value(v, sweep, k, cs[1]), ym = o3_value(v, sweep, k, cs[2]);
          const double yp = o3_value(v, sweep, k, cs[3]), y4 = o3_value(v, sweep, k, cs[4]);
          if (still && ((ubits(ys[0]) & kMag) < kMod) && ((ubits(ys[1]) & kMag) < kMod) &&
              ((ubits(ys[2]) & kMag) < kMod) && ((ubits(y1) & kMag) < kMod) &&
              ((ubits(ym) & kMag) < kMod) && ((ubits(yp) & kMag) < kMod) &&
              ((ubits(y4) & kMag) < kMod)) {
            out[k * FP] = 0.0;
            continue;
          }
          if (!have_F) {
            F = o3_dt_call(h[2], h[3], vdt);
            have_F = true;
          }
          out[k * FP] = o3_tail_call(F, ys[0], ys[1], ys[2], y1, ym, yp, y4);
        }
      } else {
        const O3Face F = o3_face(h, vdt);
        for (int k = 0; k < ncomp; ++k) {
          double y[6];
          for (int t = 0; t < 6; ++t) y[t] = o3_value(v, sweep, k, cs[t]);
          out[k * FP] = flux_ordre3_c(F, y);
        }
      }
    }
  }
};

// PenteBorne face values of orders 1-2 (Remap::computeUpwindFaceQuantities
// ForProjection{1,2}, remap/PhaseRemap1.cc:331-452) formed where they are
// used: the update of each cell forms the values of its two faces,
// dPAv(av) - dPAr(ar) as SweepFace forms them (each inner face's value is
// formed by both of its cells, bit for bit the same), instead of reading
// them from a face plane.  The update writes neither plane, so this is safe
// while it rewrites Phi.
struct LowFace {
  long long av, ar;
  bool zv, zr;  // dPAv(av) / dPAr(ar) all +0.0 (pbz)
};
DV LowFace low_face(const RunView& v, bool dirx, long long cb, long long cf) {
  LowFace F;
  F.av = dirx ? cb : cf;
  F.ar = dirx ? cf : cb;
  F.zv = (v.pbz[F.av] & 2) != 0;
  F.zr = (v.pbz[F.ar] & 1) != 0;
  return F;
}
// the same from a fused sweep's tile: tz[] flags, tv / tr[k * ts + x]
// integrals, x the tile index of the face's back / front cell
DV LowFace low_face_tile(const unsigned char* tz, bool dirx, int cb, int cf) {
  LowFace F;
  F.av = dirx ? cb : cf;
  F.ar = dirx ? cf : cb;
  F.zv = (tz[F.av] & 2) != 0;
  F.zr = (tz[F.ar] & 1) != 0;
  return F;
}
DV double low_face_value_tile(const double* tv, const double* tr, int ts, const LowFace& F,
                              int k) {
  const double a = F.zv ? 0.0 : tv[k * ts + F.av];
  const double b = F.zr ? 0.0 : tr[k * ts + F.ar];
  return subz(a, b);
}
DV double low_face_value(const RunView& v, const LowFace& F, int k) {
  const long long P = v.pitch;
  // an integral plane flagged in pbz holds +0.0 for every component (the
  // slope kernel did not store it); subz: a - b exactly, on the integer pipe
  // when b (or both) is a zero -- the usual case, as only the face's upwind
  // cell integrates an outflow, and everywhere at rest (each face value is
  // formed twice here, so its subtraction should not cost two FP64
  // instructions)
  const double a = F.zv ? 0.0 : v.dPAv[k * P + F.av];
  const double b = F.zr ? 0.0 : v.dPAr[k * P + F.ar];
  return subz(a, b);
}

// Conservative update of one sweep (Remap::computeUremap{1,2},
// remap/PhaseRemap1.cc:459-568, PhaseRemap2.cc:454-497).
// FACES: 0 = the face values come from the face plane (written by the slope
// kernel at order 2 without PenteBorne, by SweepFace otherwise), 1 = they
// are formed here (PenteBorne at orders 1-2), 2 = the run's options decide
// (batched launches).
template <int FACES>
struct SweepUpdateT {
  int sweep;
  // Fused sweeps (PenteBorne, orders 1-2): the faces' flags and integrals
  // come from the tile (lc: the cell's tile index, lm / lp: its neighbours'
  // at -1 / +1 along the sweep axis), and (phi2) the first sweep writes the
  // Phi of the cells it changes to Phi2 instead of Phi.
  const unsigned char* tz = nullptr;
  const double *tr = nullptr, *tv = nullptr;
  int lc = 0, lm = 0, lp = 0, ts = 0;
  bool phi2 = false;
  __device__ __forceinline__ void operator()(const RunView& v, int i, int j) const {
    const Ctrl& C = *v.ctrl;
    if (i >= v.ny || j >= v.nx) return;
    const bool dirx = (sweep == 1) ? C.x_then_y : !C.x_then_y;
    const long long P = v.pitch, FP = v.fpitch;
    const long long c = (long long)i * v.nx + j;
    const int ncomp = v.ncomp, nb = v.nbmat;
    // Orders 1-2: a cell whose components all come through the first sweep
    // bit for bit unchanged is flagged in u1s instead of having them copied
    // into U1; the second sweep then takes its input from UL (which holds
    // them) and, if it leaves them unchanged too, stores nothing (UL already
    // holds the result).  The order-3 reconstruction reads neighbours' U1,
    // so order-3 runs store U1 always.
    const bool lowo = v.order <= 2;
    const bool from_ul = (sweep == 2) && lowo && v.u1s[c] != 0;
    const double* Uin = (sweep == 1 || from_ul) ? v.UL : v.U1;
    const double dt = C.dt_n;
    // PenteBorne, known at compile time for the kernel that forms its faces
    const int pbv = (FACES == 1) ? 1 : v.pb;
    // the two faces perpendicular to the sweep, in getNeighbourCells order
    // (below before above, left before right); faces parallel to the sweep
    // contribute 0 * phiFace and are skipped.
    bool has[2];
    long long fidx[2];
    double coef[2];
    double nrm[2];  // outer normal component of face 0 / face 1 along the sweep
    const long long n0 = (long long)i * (v.nx + 1) + j;
    if (dirx) {
      has[0] = (j >= 1);
      has[1] = (j < v.nx - 1);
      fidx[0] = (long long)i * (v.nx + 1) + j;
      fidx[1] = fidx[0] + 1;
      const double fl = ld(v.flv, i);
      const double va = fnv_vertical(v, n0, n0 + v.nx + 1);
      const double vb = fnv_vertical(v, n0 + 1, n0 + v.nx + 2);
      const double na = nout_at(v, 0, c), nb_ = nout_at(v, 1, c);
      nrm[0] = na;
      nrm[1] = nb_;
      if (pbv == 0) {
        // ((n * u_f) * L) * dt exactly; a face at rest gives a zero on the
        // integer pipe
        coef[0] = mulz(mulz(mulz(na, va), fl), dt);
        coef[1] = mulz(mulz(mulz(nb_, vb), fl), dt);
      } else {
        coef[0] = mul_pm1(fl, na);
        coef[1] = mul_pm1(fl, nb_);
      }
    } else {
      has[0] = (i >= 1);
      has[1] = (i < v.ny - 1);
      fidx[0] = (long long)i * v.nx + j;
      fidx[1] = fidx[0] + v.nx;
      const double fl = ld(v.flh, j);
      const double va = fnv_horizontal(v, n0, n0 + 1);
      const double vb = fnv_horizontal(v, n0 + v.nx + 1, n0 + v.nx + 2);
      const double na = nout_at(v, 2, c), nb_ = nout_at(v, 3, c);
      nrm[0] = na;
      nrm[1] = nb_;
      if (pbv == 0) {
        // ((n * u_f) * L) * dt exactly; a face at rest gives a zero on the
        // integer pipe
        coef[0] = mulz(mulz(mulz(na, va), fl), dt);
        coef[1] = mulz(mulz(mulz(nb_, vb), fl), dt);
      } else {
        coef[0] = mul_pm1(fl, na);
        coef[1] = mul_pm1(fl, nb_);
      }
    }
    // PenteBorne at orders 1-2: the two faces' back / front cells as
    // SweepFace names them
    const bool form = (FACES == 1) || (FACES == 2 && v.order <= 2 && v.pb == 1);
    LowFace lf[2];
    if (form && tz) {
      if (dirx) {
        if (has[0]) lf[0] = low_face_tile(tz, true, lm, lc);
        if (has[1]) lf[1] = low_face_tile(tz, true, lc, lp);
      } else {
        if (has[0]) lf[0] = low_face_tile(tz, false, lc, lm);
        if (has[1]) lf[1] = low_face_tile(tz, false, lp, lc);
      }
    } else if (form) {
      if (dirx) {
        if (has[0]) lf[0] = low_face(v, true, c - 1, c);
        if (has[1]) lf[1] = low_face(v, true, c, c + 1);
      } else {
        if (has[0]) lf[0] = low_face(v, false, c, c - v.nx);
        if (has[1]) lf[1] = low_face(v, false, c + v.nx, c);
      }
    }
    // Boundary flux (Remap::computeBoundaryFluxes, remap/BoundaryFluxes.cc
    // :14-120, added after the neighbour faces' fluxes): on a side with a
    // flux condition, the flux through the cell's boundary face carries the
    // value of its opposite face.  bcf 1: face 0 (left / bottom) with face
    // 1's value; 2: face 1 (right / top) with face 0's value.  The branches
    // and their order are the reference's, including its test for the top
    // side, which every cell up to the first one of the top row passes.
    int bcf = 0;
    if (v.flux_bc) {
      if (dirx) {
        if ((v.flux_bc & kFluxLeft) && j == 0) bcf = 1;
        else if ((v.flux_bc & kFluxRight) && j == v.nx - 1) bcf = 2;
      } else {
        if ((v.flux_bc & kFluxBottom) && i == 0) bcf = 1;
        else if ((v.flux_bc & kFluxTop) && c <= (long long)v.nx * (v.ny - 1)) bcf = 2;
      }
    }
    // A face whose coefficient is a zero (without PenteBorne: its normal
    // velocity is, the face does not move) carries coef * q = the zero of
    // sign(coef) xor sign(q) for every finite q, as a zero value q does:
    // such faces take the still paths below.  Not with a boundary flux,
    // whose term pairs one face's coefficient with the other's value.
    const bool zc0 = bcf == 0 && iszero(coef[0]), zc1 = bcf == 0 && iszero(coef[1]);
    // dual-method components: masses (A1) or volumes (A2)
    const int doff = (v.dual_method == 1) ? 0 : nb;
    double U[kMaxComp];
    bool same = true;  // every component unchanged, bit for bit
    const bool cfin = is_finite(coef[0]) && is_finite(coef[1]);
    const bool dual_share = v.scheme != HYDRO_SCHEME_EUCCLHYD && v.dual_method != 2;
    const double rl = (dual_share && v.dual_method == 1) ? v.rL[c] : 0.;
    const double vl = (sweep == 1 && pbv != 1) ? v.vL[c] : 0.;
    // Both faces with integral planes flagged all +0.0 (PenteBorne face
    // values formed here, each +0 - +0 = +0), finite coefficients, normals
    // and rL, no boundary flux, no NaN input: every flux is the zero of
    // sign(coef), each component keeps its value and each mass-flux share
    // is a signed zero.  The whole cell takes one branch without FP64
    // instructions (the cell at rest); decided per value, the branches are
    // if-converted into FP64 instructions that run anyway.
    // (the still paths form the mass-flux shares' signed zeros from the sign
    // bits: they need finite coefficients, normals and rL)
    const bool still_ok = cfin && is_finite(rl) && is_finite(nrm[0]) && is_finite(nrm[1]);
    bool zface = form && still_ok && bcf == 0 && (!has[0] || (lf[0].zv && lf[0].zr)) &&
                 (!has[1] || (lf[1].zv && lf[1].zr));
    // Such a VNR cell in the first sweep at orders 1-2, or in the second one
    // where its components come from UL (the first left them unchanged),
    // stores none of them (only the flag saying they are unchanged), and
    // keeps its Phi: its components are not even read.  (A NaN component
    // then keeps its bits, where the per-component path would give the
    // subtraction's NaN; the final's NaN check stops the run either way.)
    const bool zskip =
        zface && v.scheme == HYDRO_SCHEME_VNR && ((sweep == 1 && lowo) || from_ul);
    if (zface && !zskip) {
  #pragma unroll
      for (int k = 0; k < kMaxComp; ++k) {
        if (k >= ncomp) break;
        U[k] = Uin[k * P + c];
        zface = zface && !is_nan(U[k]);
      }
    }
    if (zface && dual_share) {
      // F = coef * (+0): the zero of sign(coef) (+0 for a missing face);
      // times the normal: its sign xor the normal's; the two summed: -0
      // only when both are -0
      constexpr unsigned long long kS = 0x8000000000000000ull;
      const unsigned long long s0 = ((has[0] ? ubits(coef[0]) : 0ull) ^ ubits(nrm[0])) & kS;
      const unsigned long long s1 = ((has[1] ? ubits(coef[1]) : 0ull) ^ ubits(nrm[1])) & kS;
      unsigned long long w = s0 & s1;
      if (v.dual_method == 1) w ^= ubits(rl) & kS;
      for (int m = 0; m < nb; ++m) v.FFd[m * P + c] = from_bits(w);
    }
    // components four at a time: the loads of a group are issued together,
    // ahead of the group's stores (which would otherwise order each
    // component's loads behind the previous component's stores)
    for (int k0 = 0; k0 < (zface ? 0 : ncomp); k0 += 4) {
      double qa[4], qb[4], ui[4];
  #pragma unroll
      for (int t = 0; t < 4; ++t) {
        const int k = k0 + t;
        if (form && tz) {
          qa[t] = (k < ncomp && has[0]) ? low_face_value_tile(tv, tr, ts, lf[0], k) : 0.;
          qb[t] = (k < ncomp && has[1]) ? low_face_value_tile(tv, tr, ts, lf[1], k) : 0.;
        } else if (form) {
          qa[t] = (k < ncomp && has[0]) ? low_face_value(v, lf[0], k) : 0.;
          qb[t] = (k < ncomp && has[1]) ? low_face_value(v, lf[1], k) : 0.;
        } else {
          qa[t] = (k < ncomp && has[0]) ? v.phiF[k * FP + fidx[0]] : 0.;
          qb[t] = (k < ncomp && has[1]) ? v.phiF[k * FP + fidx[1]] : 0.;
        }
        ui[t] = (k < ncomp) ? Uin[k * P + c] : 0.;
      }
      // a group whose faces all carry zero fluxes (zero values, or faces
      // with a zero coefficient): each component keeps its value (see
      // below), decided once so that the arithmetic is branched over rather
      // than issued under a predicate
      bool group_still = still_ok;
  #pragma unroll
      for (int t = 0; t < 4; ++t)
        if (k0 + t < ncomp)
          group_still = group_still && (iszero(qa[t]) || (zc0 && is_finite(qa[t]))) &&
                        (iszero(qb[t]) || (zc1 && is_finite(qb[t]))) && !is_nan(ui[t]);
      if (group_still) {
  #pragma unroll
        for (int t = 0; t < 4; ++t) {
          const int k = k0 + t;
          if (k >= ncomp) break;
          U[k] = ui[t];
          if (dual_share && k >= doff && k < doff + nb) {
            // the signed-zero fluxes (+0 for a missing face) times the
            // finite normals: sign xor sign; summed: -0 only when both terms
            // are -0; times the finite rL: sign xor sign again
            constexpr unsigned long long kS = 0x8000000000000000ull;
            const unsigned long long s0 =
                ((has[0] ? ubits(coef[0]) ^ ubits(qa[t]) : 0ull) ^ ubits(nrm[0])) & kS;
            const unsigned long long s1 =
                ((has[1] ? ubits(coef[1]) ^ ubits(qb[t]) : 0ull) ^ ubits(nrm[1])) & kS;
            unsigned long long w = s0 & s1;
            if (v.dual_method == 1) w ^= ubits(rl) & kS;
            v.FFd[(k - doff) * P + c] = from_bits(w);
          }
        }
        continue;
      }
  #pragma unroll
      for (int t = 0; t < 4; ++t) {
        const int k = k0 + t;
        if (k >= ncomp) break;
        const double q0 = qa[t], q1 = qb[t], uin = ui[t];
        double F0 = 0., F1 = 0.;
        if (cfin && (iszero(q0) || (zc0 && is_finite(q0))) &&
            (iszero(q1) || (zc1 && is_finite(q1))) && !is_nan(uin)) {
          // nothing crosses either face: each flux coef * q is the zero of
          // sign(coef) xor sign(q), their sum from 0.0 is +0, and uin - +0 is
          // uin
          if (has[0]) F0 = from_bits((ubits(coef[0]) ^ ubits(q0)) & ~kMag);
          if (has[1]) F1 = from_bits((ubits(coef[1]) ^ ubits(q1)) & ~kMag);
          U[k] = uin;
        } else {
          double red = 0.0;
          if (has[0]) {
            F0 = coef[0] * q0;
            red = plus_zero(F0);  // 0.0 + F0
          }
          if (has[1]) {
            F1 = coef[1] * q1;
            red = has[0] ? red + F1 : plus_zero(F1);
          }
          if (bcf == 1) red = red + coef[0] * q1;
          else if (bcf == 2) red = red + coef[1] * q0;
          U[k] = uin - red;
        }
        same = same && ubits(U[k]) == ubits(uin);
        if (dual_share && k >= doff && k < doff + nb) {
          // the cell's share of the nodal mass flux (UtilesDualRemap.cc A1
          // :10-233, A2 :401-644): the two face fluxes times their outer
          // normals, summed; every node this cell feeds uses the same value
          // (its two sums differ only in the order of the terms, and IEEE
          // addition commutes)
          double w = mul_pm1(F0, nrm[0]) + mul_pm1(F1, nrm[1]);
          if (v.dual_method == 1) w = rl * w;
          v.FFd[(k - doff) * P + c] = w;
        }
      }
    }
    // the stores, after every load
    if (sweep == 1) {
      if (lowo) v.u1s[c] = same ? 1 : 0;
      if (!(lowo && same))
        for (int k = 0; k < ncomp; ++k) v.U1[k * P + c] = U[k];
    } else if (!(from_ul && same)) {
      for (int k = 0; k < ncomp; ++k) v.UL[k * P + c] = U[k];
    }
    if (sweep == 1) {
      // (fused sweeps: to Phi2, which the second sweep reads for the cells
      // changed here; Phi itself stays as the Lagrange kernel left it, since
      // neighbouring tiles still read it)
      double* Phi = phi2 ? v.Phi2 : v.Phi;
      // a VNR cell whose conserved values came through the sweep unchanged
      // keeps the Phi the Lagrange kernel formed from exactly these values
      // with the same formulas (the pseudo-viscosity slot is not updated
      // here in either case)
      const bool keep = same && v.scheme == HYDRO_SCHEME_VNR;
      if (keep) {
      } else if (v.pb == 1) {
        double sv = 0.;
        for (int m = 0; m < nb; m++) sv += U[m];
        double sm = 0.;
        for (int m = 0; m < nb; m++) {
          Phi[m * P + c] = qdiv(U[m], sv);
          Phi[(nb + m) * P + c] = nz(U[m]) ? qdiv(U[nb + m], U[m]) : 0.;
          sm += U[nb + m];
        }
        for (int m = 0; m < nb; m++)
          Phi[(2 * nb + m) * P + c] = nz(U[nb + m]) ? qdiv(U[2 * nb + m], U[nb + m]) : 0.;
        // Eucclhyd momentum / kinetic energy per unit mass (the VNR
        // pseudo-viscosity slot is not updated here in the reference: in
        // Phi2 it is the Lagrange kernel's value, copied)
        if (v.scheme == HYDRO_SCHEME_EUCCLHYD)
          for (int k = 3 * nb; k < ncomp; ++k) Phi[k * P + c] = qdiv(U[k], sm);
        else if (phi2)
          Phi[3 * nb * P + c] = v.Phi[3 * nb * P + c];
      } else {
        // vl: the Lagrangian volume, read with the inputs
        const SharedDiv Sv = shared_div(vl);  // one denominator, ncomp quotients
        for (int k = 0; k < ncomp; ++k) Phi[k * P + c] = qdiv_shared(Sv, U[k]);
      }
      const double* Pr = keep ? v.Phi : Phi;  // the cell's Phi after the sweep
      int matcell = 0, imatpure = -1;
      for (int m = 0; m < nb; m++)
        if (pos(Pr[m * P + c])) {
          matcell++;
          imatpure = m;
        }
      if (matcell > 1) {
        v.mixte[c] = 1;
        v.pure[c] = -1;
      } else {
        v.mixte[c] = 0;
        v.pure[c] = imatpure;
      }
    }
  }
};

// ------------------------------------------------------------- dual remap
// Limited nodal velocity gradient along the sweep
// (Remap::computeDualHorizontalGradPhi / computeDualVerticalGradPhi,
// remap/UtilesRemap-Impl.h:8-97).  Only the two velocity components are
// consumed downstream.
struct DualGrad {
  int sweep;
  __device__ __forceinline__ void operator()(const RunView& v, int i, int j) const {
    const Ctrl& C = *v.ctrl;
    if (i > v.ny || j > v.nx) return;
    const bool dirx = (sweep == 1) ? C.x_then_y : !C.x_then_y;
    const long long NP = v.npitch;
    const long long p = (long long)i * (v.nx + 1) + j;
    const double* D = (sweep == 1) ? v.u : v.DPv;  // DualPhi velocity
    double g0 = 0.0, g1 = 0.0;
    if (v.order > 1) {
      const int ax = dirx ? 0 : 1;
      const int at = dirx ? j : i, lastpos = dirx ? v.nx : v.ny;
      const long long stride = dirx ? 1 : (v.nx + 1);
      if (at != 0 && at != lastpos) {
        const long long L = p - stride, R = p + stride;
        const double xp = v.XL[ax * NP + p], xr = v.XL[ax * NP + R],
                     xl = v.XL[ax * NP + L];
        // Velocities +0 at the node and both neighbours, positions strictly
        // increasing well inside the double range: both face gradients are
        // +0 / (a positive length) = +0, and the one-ratio limiters
        // (minmod, superBee, vanLeer) give 0.5 * (phi * (+0) + phi' * (+0))
        // = +0 for their finite phi; the lengths and the limiter are not needed.
        constexpr unsigned long long kHuge = 0x7fd0000000000000ull;  // 2^1022
        if (v.limiter < HYDRO_LIM_MINMODG &&
            (ubits(D[p]) | ubits(D[NP + p]) | ubits(D[L]) | ubits(D[NP + L]) | ubits(D[R]) |
             ubits(D[NP + R])) == 0 &&
            (ubits(xl) & kMag) < kHuge && (ubits(xr) & kMag) < kHuge && dlt(xl, xp) &&
            dlt(xp, xr)) {
          v.gD[p] = 0.0;
          v.gD[NP + p] = 0.0;
          return;
        }
        double hm, hp;
        const double h0 = half(xr - xl);
        const bool hasLL = (at - 1 != 0), hasRR = (at + 1 != lastpos);
        if (!hasLL) {
          hm = 0.;
          const double xrr = hasRR ? v.XL[ax * NP + R + stride] : 0.0;
          hp = half(xrr - xp);
        } else if (!hasRR) {
          hp = 0.;
          hm = half(xp - v.XL[ax * NP + L - stride]);
        } else {
          hm = half(xp - v.XL[ax * NP + L - stride]);
          hp = half(v.XL[ax * NP + R + stride] - xp);
        }
        double g[2];
  #pragma unroll
        for (int k = 0; k < 2; ++k) {
          const double dp = D[k * NP + p], dr = D[k * NP + R], dl = D[k * NP + L];
          const double gr = qdiv(dr - dp, xr - xp);
          const double gl = qdiv(dp - dl, xp - xl);
          g[k] = limit_grad1(v.limiter, gr, gl, dr, dl, h0, hp, hm);
        }
        g0 = g[0];
        g1 = g[1];
      }
    }
    v.gD[p] = g0;
    v.gD[NP + p] = g1;
  }
};

// Nodal mass fluxes, upwind velocities and nodal momentum update
// (Remap::computeDualUremap{1,2}, remap/DualPhaseRemap1.cc:33-135,
// DualPhaseRemap2.cc:36-125; mass fluxes remap/UtilesDualRemap.cc A1
// :10-233, A2 :401-644, PB :648-818; upwind velocities :234-397).
struct DualUpdate {
  int sweep;
  __device__ __forceinline__ void operator()(const RunView& v, int i, int j) const {
    Ctrl& C = *v.ctrl;
    if (i > v.ny || j > v.nx) return;
    const bool dirx = (sweep == 1) ? C.x_then_y : !C.x_then_y;
    const long long P = v.pitch, NP = v.npitch;
    const long long p = (long long)i * (v.nx + 1) + j;
    const int nb = v.nbmat;
    const int ax = dirx ? 0 : 1;
    // inner faces of the sweep through this node (Vertical/HorizontalFaceOfNode,
    // remap/UtilesMesh.cc:53-108): for an x sweep the vertical faces below and
    // above the node, for a y sweep the horizontal faces left and right of it.
    // cplus[s] / cminus[s]: the cells right/above and left/below of face s.
    long long cplus[2], cminus[2];
    int nface = 0;
    if (dirx) {
      if (j >= 1 && j <= v.nx - 1) {
        if (i >= 1) {
          cminus[nface] = (long long)(i - 1) * v.nx + j - 1;
          cplus[nface++] = (long long)(i - 1) * v.nx + j;
        }
        if (i <= v.ny - 1) {
          cminus[nface] = (long long)i * v.nx + j - 1;
          cplus[nface++] = (long long)i * v.nx + j;
        }
      }
    } else {
      if (i >= 1 && i <= v.ny - 1) {
        if (j >= 1) {
          cminus[nface] = (long long)(i - 1) * v.nx + j - 1;
          cplus[nface++] = (long long)i * v.nx + j - 1;
        }
        if (j <= v.nx - 1) {
          cminus[nface] = (long long)(i - 1) * v.nx + j;
          cplus[nface++] = (long long)i * v.nx + j;
        }
      }
    }
    // mass fluxes through the node's dual faces; when every share is a
    // zero, each sum below is +0 (sums from 0.0 of zeros)
    const double* W = (v.dual_method == 2) ? v.DPF : v.FFd;  // FFd: each cell's share
    unsigned long long wor = 0;
    for (int m = 0; m < nb; ++m)
      for (int s = 0; s < nface; ++s)
        wor |= ubits(W[m * P + cplus[s]]) | ubits(W[m * P + cminus[s]]);
    const bool fzero = (wor & kMag) == 0;
    double Fp = 0., Fm = 0.;
    for (int m = 0; m < nb && !fzero; ++m) {
      // sums from 0.0: the first addition is plus_zero (integer pipe)
      double pp = 0., pm = 0.;
      for (int s = 0; s < nface; ++s) {
        const long long a = cplus[s], b = cminus[s];
        const double wa = W[m * P + a], wb = W[m * P + b];
        pp = (s == 0) ? plus_zero(wa) : pp + wa;
        pm = (s == 0) ? plus_zero(wb) : pm + wb;
      }
      if (v.dual_method == 2) {
        if (nface != 0) {
          pp = div_pow2(pp, nface);
          pm = div_pow2(pm, nface);
        }
      } else if (nface != 0) {
        pp = div_pow2(pp, 2 * nface);
        pm = div_pow2(pm, 2 * nface);
      }
      Fp = (m == 0) ? plus_zero(pp) : Fp + pp;
      Fm = (m == 0) ? plus_zero(pm) : Fm + pm;
    }
    // previous nodal conserved values and DualPhi
    const double* D = (sweep == 1) ? v.u : v.DPv;
    const int at = dirx ? j : i, lastpos = dirx ? v.nx : v.ny;
    const long long stride = dirx ? 1 : (v.nx + 1);
    const bool hasL = at != 0, hasR = at != lastpos;
    const long long L = p - stride, R = p + stride;
    const double dt = C.dt_n;
    const double dp0 = D[p], dp1 = D[NP + p], xp = v.XL[ax * NP + p];
    const double gp0 = v.gD[p], gp1 = v.gD[NP + p];
    const double dl0 = hasL ? D[L] : 0.0, dl1 = hasL ? D[NP + L] : 0.0;
    const double dr0 = hasR ? D[R] : 0.0, dr1 = hasR ? D[NP + R] : 0.0;
    const double xl = hasL ? v.XL[ax * NP + L] : 0.0, xr = hasR ? v.XL[ax * NP + R] : 0.0;
    double Ui0, Ui1, Ui2;
    const double nmass = (sweep == 1) ? v.node_mass[p] : 0.0;
    if (sweep == 1) {
      Ui2 = nmass;
    } else {
      Ui0 = v.UD1[p];
      Ui1 = v.UD1[NP + p];
      Ui2 = v.UD1[2 * NP + p];
    }
    // A node that nothing reaches: no mass flux (Fm = Fp = +0), velocities
    // +0 at the node and at its neighbours along the sweep, zero slopes at
    // the node, finite positions well inside the double range.  Then both
    // upwind velocities are +0 + (a zero), i.e. +0, every flux term is +0,
    // and each new conserved value is the old one plus +0 minus +0: the old
    // value with a zero made +0.  (In the first sweep the momenta are
    // mass * (+0), zeros for a finite mass.)
    constexpr unsigned long long kHuge = 0x7fd0000000000000ull;  // 2^1022
    const bool quiet =
        fzero && ((ubits(dp0) | ubits(dp1) | ubits(dl0) | ubits(dl1) | ubits(dr0) |
                   ubits(dr1)) == 0) &&
        (((ubits(gp0) | ubits(gp1)) & kMag) == 0) && (ubits(xp) & kMag) < kHuge &&
        (ubits(xl) & kMag) < kHuge && (ubits(xr) & kMag) < kHuge && is_finite(dt) &&
        (sweep == 1 ? is_finite(nmass)
                    : (!is_nan(Ui0) && !is_nan(Ui1) && !is_nan(Ui2)));
    double Un0, Un1, Un2;
    if (quiet) {
      Un0 = (sweep == 1 || iszero(Ui0)) ? 0.0 : Ui0;
      Un1 = (sweep == 1 || iszero(Ui1)) ? 0.0 : Ui1;
      Un2 = iszero(Ui2) ? 0.0 : Ui2;
    } else {
      if (sweep == 1) {
        Ui0 = nmass * dp0;
        Ui1 = nmass * dp1;
      }
      Un2 = Ui2 + Fm - Fp;
      const int order2 = v.order - 1;
      // minus side (left / bottom)
      double um[2], up[2];
      {
        const double dn0 = dl0, dn1 = dl1;
        const double xn = xl;
        const double u = half((ax == 0 ? dn0 : dn1) + (ax == 0 ? dp0 : dp1));
        const double dx = xp - xn;
        const double sdx = pos(u) ? dx : -dx;  // sign(u) * dx
        // the upwind node's value and slope, selected before the one
        // expression both cases share (as two branches, if-converted, both
        // sets of FP64 operations would be issued)
        const bool nbr = pos(Fm);
        const double gn0 = hasL ? v.gD[L] : 0.0, gn1 = hasL ? v.gD[NP + L] : 0.0;
        const double b0 = nbr ? dn0 : dp0, b1 = nbr ? dn1 : dp1;
        const double g0 = nbr ? gn0 : gp0, g1 = nbr ? gn1 : gp1;
        const double w = sdx - dt * u;
        um[0] = b0 + mul_012(order2, half(g0) * w);
        um[1] = b1 + mul_012(order2, half(g1) * w);
      }
      // plus side (right / top)
      {
        const double dn0 = dr0, dn1 = dr1;
        const double xn = xr;
        const double u = half((ax == 0 ? dp0 : dp1) + (ax == 0 ? dn0 : dn1));
        const double dx = xn - xp;
        const double sdx = pos(u) ? dx : -dx;  // sign(u) * dx
        const bool nbr = neg(Fp);
        const double gn0 = hasR ? v.gD[R] : 0.0, gn1 = hasR ? v.gD[NP + R] : 0.0;
        const double b0 = nbr ? dn0 : dp0, b1 = nbr ? dn1 : dp1;
        const double g0 = nbr ? gn0 : gp0, g1 = nbr ? gn1 : gp1;
        const double w = sdx - dt * u;
        up[0] = b0 + mul_012(order2, half(g0) * w);
        up[1] = b1 + mul_012(order2, half(g1) * w);
      }
      Un0 = Ui0 + Fm * um[0] - Fp * up[0];
      Un1 = Ui1 + Fm * um[1] - Fp * up[1];
    }
    if (sweep == 1) {
      v.UD1[p] = Un0;
      v.UD1[NP + p] = Un1;
      v.UD1[2 * NP + p] = Un2;
      // qdiv: momentum is exactly 0 wherever the flow has not arrived
      v.DPv[p] = qdiv(Un0, Un2);
      v.DPv[NP + p] = qdiv(Un1, Un2);
    } else {
      // remapVariables node part (vnr_remap/PhaseRemapFinal.cc:207-234)
      const double ux = qdiv(Un0, Un2), uy = qdiv(Un1, Un2);
      v.u[p] = ux;
      v.u[NP + p] = uy;
      v.speed[p] = face_len(ux, uy);  // sqrt(ux*ux + uy*uy), |ux| when uy is 0
    }
  }
};

// ----------------------------------------------------------- remap final
// Vnr::remapVariables cell part (vnr_remap/PhaseRemapFinal.cc:18-205), then
// computeEOS + computePressionMoyenne (PhaseLagrange.cc:392-485), and the
// next cycle's dt candidate (VnrRemap.cc:14-50) and max pressure
// (PhaseLagrange.cc:55-61).
// material loops unrolled to the three possible materials (the arrays they
// index stay in registers instead of local memory); iterations m >= nbmat do
// nothing
#define MAT_LOOP(m, first) _Pragma("unroll") for (int m = (first); m < 3; ++m) if (m < nb)

// final_cell for a cell that holds one material p: the other materials'
// volume, mass and energy are +0.0 (bits), p's volume and mass are positive,
// every material is a perfect gas, the threshold lies in [0, 1), and (for
// the time step) the four node speeds are +0.0.  The general path then
// reduces exactly to: volt = vn_p, masset = Um_p (x + +0 = x), rv = vol /
// vn_p, vn_p' = vn_p * rv and the others +0 * rv = +0 (rv > 0), f = 1 and +0
// (x / x = 1, +0 / x = +0, neither moved by the threshold), mf likewise,
// rho = 0.0 + Um_p / vn_p', e = 0.0 + Ue_p / Um_p, p = 0.0 + pm_p with pm_p
// = (g_p - 1) rho_p e_p, the others' pm = ((g_m - 1) * +0) * +0 (the zero
// of sign(g_m - 1)), cmassm = cmass and the zero of sign(cmass), and the
// time-step denominator 0.0 + c.  The few products and quotients that
// remain are the reference's; a value that leaves these ranges (a negative
// density or energy, a NaN, a non-finite product) returns false before any
// store, and the general path runs.  One branch for the whole cell: decided
// per value inside the general path, the shortcuts are if-converted into
// FP64 instructions that run anyway.
__device__ __forceinline__ bool final_single(const RunView& v, Ctrl& C, long long c, int nb,
                                             double thr, double vol, const double* vn,
                                             const double* Um, const double* Ue, double Uq,
                                             double c_in, double sarg_in, const double* spd,
                                             double cflsq, unsigned long long& dtb,
                                             unsigned long long& pb) {
  constexpr unsigned long long kS = 0x8000000000000000ull;
  int p = -1, nonzero = 0;
  bool ok = nonneg(thr) && dlt(thr, 1.0);
  MAT_LOOP(m, 0) {
    const bool z = (ubits(vn[m]) | ubits(Um[m]) | ubits(Ue[m])) == 0ull;
    if (!z) {
      p = m;
      ++nonzero;
    }
    ok = ok && eos_of(v, m) == HYDRO_EOS_PERFECT_GAS && is_finite(gm1_of(v, m));
  }
  if (v.sans_lagrange == 0)
    ok = ok && (ubits(spd[0]) | ubits(spd[1]) | ubits(spd[2]) | ubits(spd[3])) == 0ull;
  if (!ok || nonzero != 1) return false;
  // p's values by select over the unrolled materials (an index held in a
  // register would put the arrays in local memory)
  double vnp0 = 0., ump = 0., uep = 0.;
  MAT_LOOP(m, 0) {
    if (m == p) {
      vnp0 = vn[m];
      ump = Um[m];
      uep = Ue[m];
    }
  }
  if (!(pos(vnp0) && is_finite(vnp0) && pos(ump) && is_finite(ump))) return false;
  const double rv = qdiv(vol, vnp0);
  if (!(pos(rv) && is_finite(rv))) return false;
  const double vnp = mul1z(vnp0, rv);
  if (!(pos(vnp) && is_finite(vnp))) return false;
  const double dmp = qdiv(ump, vnp), emp = qdiv(uep, ump);
  if (neg(dmp) || neg(emp) || is_nan(dmp) || is_nan(emp)) return false;
  const double rho = plus_zero(dmp), e = plus_zero(emp);
  if (!pos(rho)) return false;
  const double cmass = v.euler_volume * rho;
  if (!is_finite(cmass)) return false;
  const double pmp = (gm1_of(v, p) * dmp) * emp;
  const double pres = plus_zero(pmp);
  // the state, as the general path stores it
  const long long P = v.pitch;
  v.mixte[c] = 0;
  v.pure[c] = p;
  v.cell_mass[c] = cmass;
  v.q[c] = qdiv(Uq, vol);
  const double cc = (ubits(e) == ubits(sarg_in)) ? c_in : sqrt_ip(v.g0gm1 * e);
  v.rho[c] = rho;
  v.e[c] = e;
  v.p[c] = pres;
  st_if_new(v.c + c, c_in, cc);
  st_if_new(v.sarg + c, sarg_in, e);
  MAT_LOOP(m, 0) {
    const bool here = m == p;
    v.cmassm[m * P + c] = here ? cmass : from_bits(ubits(cmass) & kS);
    v.fm[m * P + c] = here ? 1.0 : 0.0;
    v.mfm[m * P + c] = here ? 1.0 : 0.0;
    v.rhom[m * P + c] = here ? dmp : 0.0;
    v.em[m * P + c] = here ? emp : 0.0;
    v.pm[m * P + c] = here ? pmp : from_bits(ubits(gm1_of(v, m)) & kS);
  }
  if (v.sans_lagrange == 0) {
    const double d = div_ip(cflsq, plus_zero(cc));
    if (!is_nan(d)) dtb = ord_bits(d) < dtb ? ord_bits(d) : dtb;
  }
  if (!is_nan(pres)) pb = ord_bits(pres) > pb ? ord_bits(pres) : pb;
  return true;
}
__device__ __forceinline__ void final_cell(const RunView& v, Ctrl& C, int i,
                                           int j, unsigned long long& dtb,
                                           unsigned long long& pb) {
  const long long P = v.pitch;
  const long long c = (long long)i * v.nx + j;
  const int nb = v.nbmat;
  const double thr = v.threshold;
  const double* U = v.UL + c;  // second sweep output
  const double vol = v.euler_volume;
  // every value read up front, before the first store (stores would order
  // the later loads behind them): the remapped volumes, masses and energies,
  // the pseudo-viscosity, the sound speed kept for rho <= 0, and the dt
  // candidate's inputs
  double vn[3], Um[3], Ue[3];
#pragma unroll
  for (int m = 0; m < 3; ++m) {
    if (m >= nb) break;
    vn[m] = U[m * P];
    Um[m] = U[(nb + m) * P];
    Ue[m] = U[(2 * nb + m) * P];
  }
  const double Uq = U[3 * nb * P];
  const double c_in = v.c[c], sarg_in = v.sarg[c];
  double spd[4] = {0., 0., 0., 0.}, cflsq = 0.;
  if (v.sans_lagrange == 0) {
    const long long n0 = (long long)i * (v.nx + 1) + j;
    spd[0] = ld(v.speed, n0);
    spd[1] = ld(v.speed, n0 + 1);
    spd[2] = ld(v.speed, n0 + v.nx + 2);
    spd[3] = ld(v.speed, n0 + v.nx + 1);
    cflsq = ld(v.cflsq, c);
  }
  if (final_single(v, C, c, nb, thr, vol, vn, Um, Ue, Uq, c_in, sarg_in, spd, cflsq, dtb, pb))
    return;
  // every sum below starts from 0.0 in the reference: its first addition
  // 0.0 + x is plus_zero(x), on the integer pipe (materials 0 .. nb-1, nb >= 1)
  double volt = plus_zero(vn[0]), masset = plus_zero(Um[0]);
  MAT_LOOP(m, 1) {
    volt = addz(volt, vn[m]);
    masset = addz(masset, Um[m]);
  }
  const double rv = qdiv(vol, volt);
  vn[0] = mul1z(vn[0], rv);
  double vnorm = plus_zero(vn[0]);
  MAT_LOOP(m, 1) {
    vn[m] = mul1z(vn[m], rv);
    vnorm = addz(vnorm, vn[m]);
  }
  double f[3], mf[3], sf = 0.;
  MAT_LOOP(m, 0) {
    f[m] = qdiv(vn[m], vnorm);
    if (dlt(f[m], thr)) f[m] = 0.;
    sf = (m == 0) ? plus_zero(f[m]) : addz(sf, f[m]);
  }
  MAT_LOOP(m, 0) f[m] = qdiv(f[m], sf);
  int matcell = 0, imatpure = -1;
  MAT_LOOP(m, 0)
    if (pos(f[m])) {
      matcell++;
      imatpure = m;
    }
  v.mixte[c] = (matcell > 1) ? 1 : 0;
  v.pure[c] = (matcell > 1) ? -1 : imatpure;
  MAT_LOOP(m, 0) mf[m] = qdiv(Um[m], masset);
  double fmt = 0.;
  MAT_LOOP(m, 0) {
    if (dlt(f[m], thr)) mf[m] = 0.;
    fmt = (m == 0) ? plus_zero(mf[m]) : addz(fmt, mf[m]);
  }
  MAT_LOOP(m, 0) mf[m] = qdiv(mf[m], fmt);
  double dm[3] = {0., 0., 0.}, dens = 0.;
  MAT_LOOP(m, 0) {
    if (dgt(f[m], thr)) dm[m] = qdiv(Um[m], vn[m]);
    const double fd = mul_frac(f[m], dm[m]);
    dens = (m == 0) ? plus_zero(fd) : addz(dens, fd);
  }
  double em[3] = {0., 0., 0.};
  MAT_LOOP(m, 0)
    if (dgt(f[m], thr) && nz(Um[m]))
      em[m] = qdiv(Ue[m], Um[m]);
  const double rho = dens;
  double e = 0.;
  const double cmass = v.euler_volume * rho;
  v.cell_mass[c] = cmass;
  MAT_LOOP(m, 0) v.cmassm[m * P + c] = mul_frac(mf[m], cmass);
  v.q[c] = qdiv(Uq, vol);
  MAT_LOOP(m, 0) {
    const double t = mul_frac(mf[m], em[m]);
    e = (m == 0) ? plus_zero(t) : addz(e, t);
  }
  double rhom[3], emo[3];
  MAT_LOOP(m, 0) {
    rhom[m] = dm[m];
    emo[m] = em[m];
  }
  MAT_LOOP(m, 0) {
    if (neg(em[m]) || neg(dm[m])) {
      rhom[m] = 0.;
      emo[m] = 0.;
      mf[m] = 0.;
      f[m] = 0.;
      atomicOr(&C.err, HYDRO_ERR_NEGATIVE);
    }
  }
  if (is_nan(e) || is_nan(rho)) {
    atomicOr(&C.err, HYDRO_ERR_NAN);
    atomicMin((unsigned long long*)&C.err_cell, (unsigned long long)c);
  }
  // EOS after the remap.  A perfect gas's sound speed only matters to the
  // mean-pressure step when rho <= 0 (otherwise the mixture's replaces the
  // maximum), and nothing else reads it: it is formed only then.
  double pm[3], cm[3];
  MAT_LOOP(m, 0) {
    if (eos_of(v, m) == HYDRO_EOS_PERFECT_GAS) {
      pm[m] = mulz(mulz(gm1_of(v, m), rhom[m]), emo[m]);
    } else {
      pm[m] = v.pm[m * P + c];
      cm[m] = v.cm[m * P + c];
      emo[m] = v.em[m * P + c];
      e = 0.;
    }
  }
  double p = 0., cc = c_in;
  MAT_LOOP(m, 0) {
    const double t = mul_frac(f[m], pm[m]);
    p = (m == 0) ? plus_zero(t) : addz(p, t);
  }
  double sarg_out = from_bits(kNoRoot);
  if (pos(rho)) {
    // c_in is sqrt(g0 (g0 - 1) e') of the energy e' in sarg: the same
    // energy (bit for bit) gives the same root
    cc = (ubits(e) == ubits(sarg_in) && !is_nan(e)) ? c_in : sqrt_ip(v.g0gm1 * e);
    sarg_out = e;
  } else {
    MAT_LOOP(m, 0) {
      if (eos_of(v, m) == HYDRO_EOS_PERFECT_GAS) {
        const double g = gamma_of(v, m);
        cm[m] = sqrt_ip(g * (g - 1.0) * emo[m]);
        v.cm[m * P + c] = cm[m];
      }
      cc = smax(cc, cm[m]);
    }
  }
  MAT_LOOP(m, 0)
    if (eos_of(v, m) == HYDRO_EOS_VOID) e += mf[m] * emo[m];
  v.rho[c] = rho;
  v.e[c] = e;
  v.p[c] = p;
  st_if_new(v.c + c, c_in, cc);
  st_if_new(v.sarg + c, sarg_in, sarg_out);
  MAT_LOOP(m, 0) {
    v.fm[m * P + c] = f[m];
    v.mfm[m * P + c] = mf[m];
    v.rhom[m * P + c] = rhom[m];
    v.em[m * P + c] = emo[m];
    v.pm[m * P + c] = pm[m];
  }
  // reductions feeding the next cycle
  if (v.sans_lagrange == 0) {
    // dt candidate (Vnr::computeDeltaT, VnrRemap.cc:26-46) with this
    // cell's new sound speed
    double uc = quarter(spd[0]);
  #pragma unroll
    for (int k = 1; k < 4; ++k) uc = addz(uc, quarter(spd[k]));
    const double d = div_ip(cflsq, addz(uc, cc));
    if (!is_nan(d)) dtb = ord_bits(d) < dtb ? ord_bits(d) : dtb;
  }
  if (!is_nan(p)) pb = ord_bits(p) > pb ? ord_bits(p) : pb;
}

struct Final {
  __device__ __forceinline__ void operator()(const RunView& v, int i, int j) const {
    Ctrl& C = *v.ctrl;
    unsigned long long dtb = ~0ull, pb = 0ull;
    if (i < v.ny && j < v.nx) final_cell(v, C, i, j, dtb, pb);
    block_reduce_minmax(dtb, pb, &C);
  }
};

// Initial reductions (dt candidate and max pressure of the initial state).
__global__ void __launch_bounds__(kBX* kBY) k_init_reductions(RunView v) {
  Ctrl& C = *v.ctrl;
  const int j = blockIdx.x * kBX + threadIdx.x;
  const int i = blockIdx.y * kBY + threadIdx.y;
  unsigned long long dtb = ~0ull, pb = 0ull;
  if (i < v.ny && j < v.nx) {
    const long long c = (long long)i * v.nx + j;
    if (v.sans_lagrange == 0) {
      const double d = cell_dt(v, c, i, j);
      if (!is_nan(d)) dtb = ord_bits(d);
    }
    const double p = v.p[c];
    if (!is_nan(p)) pb = ord_bits(p);
  }
  block_reduce_minmax(dtb, pb, &C);
}

// Vnr::computeNodeMass (PhaseLagrange.cc:31-48) from the current cell
// masses; the cycle recomputes it at its start, this refreshes it for a fetch.
__global__ void k_node_mass(RunView v) {
  const int j = blockIdx.x * kBX + threadIdx.x;
  const int i = blockIdx.y * kBY + threadIdx.y;
  if (i > v.ny || j > v.nx) return;
  double r = 0.0;
  int k = 0;
  if (i < v.ny && j < v.nx) { r = r + v.cell_mass[(long long)i * v.nx + j]; ++k; }
  if (i < v.ny && j > 0) { r = r + v.cell_mass[(long long)i * v.nx + j - 1]; ++k; }
  if (i > 0 && j < v.nx) { r = r + v.cell_mass[(long long)(i - 1) * v.nx + j]; ++k; }
  if (i > 0 && j > 0) { r = r + v.cell_mass[(long long)(i - 1) * v.nx + j - 1]; ++k; }
  v.node_mass[(long long)i * (v.nx + 1) + j] = r / (double)k;
}

__global__ void k_node_speed(RunView v) {
  const int j = blockIdx.x * kBX + threadIdx.x;
  const int i = blockIdx.y * kBY + threadIdx.y;
  if (i > v.ny || j > v.nx) return;
  const long long p = (long long)i * (v.nx + 1) + j;
  const double ux = v.u[p], uy = v.u[v.npitch + p];
  v.speed[p] = face_len(ux, uy);  // sqrt(ux*ux + uy*uy)
}


// ------------------------------------------------- Lagrange phase only
// A run without the remap (AvecProjection = non): the Lagrange cell update,
// then the next cycle's dt candidate (Vnr::computeDeltaT, VnrRemap.cc
// :14-50: cfl 0.1, the sub-volumes just formed, the new node velocities and
// sound speed, A = 0) and pressure maximum, which the remap's final kernel
// reduces otherwise.
struct LagCellsLagrangeOnly {
  __device__ __forceinline__ void operator()(const RunView& v, int i, int j) const {
    Ctrl& C = *v.ctrl;
    unsigned long long dtb = ~0ull, pb = 0ull;
    if (i < v.ny && j < v.nx) {
      LagCells{}(v, i, j);
      const long long c = (long long)i * v.nx + j, NP = v.npitch;
      const long long n0 = (long long)i * (v.nx + 1) + j;
      const long long nd[4] = {n0, n0 + 1, n0 + v.nx + 2, n0 + v.nx + 1};
      double uc = 0.0;
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const double a = v.u[nd[k]], b = v.u[NP + nd[k]];
        uc += sqrt_ip(a * a + b * b) * 0.25;
      }
      const double d = div_ip(0.1 * sqrt_ip(v.vL[c]), 0. * uc + v.c[c]);
      if (v.sans_lagrange == 0 && !is_nan(d)) dtb = ord_bits(d);
      const double p = v.p[c];
      if (!is_nan(p)) pb = ord_bits(p);
    }
    block_reduce_minmax(dtb, pb, &C);
  }
};

// The new positions become the next cycle's (the reference swaps its node
// coordinate views, VnrRemap.cc:217-221) unless the run has just ended:
// after its last cycle the reference does not swap, and its final output
// shows the last cycle's start positions.
struct NextPositions {
  __device__ __forceinline__ void operator()(const RunView& v, int i, int j) const {
    if (i > v.ny || j > v.nx || v.ctrl->done) return;
    const long long p = (long long)i * (v.nx + 1) + j;
    v.XN[p] = v.XL[p];
    v.XN[v.npitch + p] = v.XL[v.npitch + p];
  }
};

// ---------------------------------------------------------------- wrappers
// Plain launches: one run, a 2D grid of kBX x kBY thread tiles.
template <class F>
__device__ __forceinline__ void plain_items(const RunView& v, const F& f) {
  if (!v.ctrl->active) return;
  f(v, blockIdx.y * kBY + threadIdx.y, blockIdx.x * kBX + threadIdx.x);
}

__global__ void __launch_bounds__(kBX* kBY, 10) k_lag_nodes(RunView v) { plain_items(v, LagNodes{}); }
__global__ void __launch_bounds__(kBX* kBY, 8) k_lag_cells(RunView v) { plain_items(v, LagCells{}); }
__global__ void __launch_bounds__(kBX* kBY) k_lag_cells_lo(RunView v) { plain_items(v, LagCellsLagrangeOnly{}); }
__global__ void __launch_bounds__(kBX* kBY) k_next_positions(RunView v) { plain_items(v, NextPositions{}); }
__global__ void __launch_bounds__(kBX* kBY) k_face_grad(RunView v, int sweep) { plain_items(v, FaceGrad{sweep}); }
__global__ void __launch_bounds__(kBX* kBY) k_o3_grad(RunView v, int sweep) { plain_items(v, O3Grad{sweep}); }
__global__ void __launch_bounds__(kBX* kBY) k_o3_ystar(RunView v, int sweep) { plain_items(v, O3Ystar{sweep}); }
__global__ void __launch_bounds__(kBX* kBY) k_sweep_grad(RunView v, int sweep) { plain_items(v, SweepGradT<0>{sweep}); }
// eight resident blocks: the kernel waits on memory more than it computes
// at rest; measured faster than the register-limited four to six
__global__ void __launch_bounds__(kBX* kBY, 8) k_sweep_grad_pb(RunView v, int sweep) { plain_items(v, SweepGradT<1>{sweep}); }
__global__ void __launch_bounds__(kBX* kBY) k_sweep_face(RunView v, int sweep) { plain_items(v, SweepFaceT<2>{sweep}); }
__global__ void __launch_bounds__(kBX* kBY, 4) k_sweep_face3(RunView v, int sweep) { plain_items(v, SweepFaceT<1>{sweep}); }
__global__ void __launch_bounds__(kBX* kBY) k_sweep_update(RunView v, int sweep) { plain_items(v, SweepUpdateT<0>{sweep}); }
__global__ void __launch_bounds__(kBX* kBY, 9) k_sweep_update_f(RunView v, int sweep) { plain_items(v, SweepUpdateT<1>{sweep}); }

// ------------------------------------------------------- fused remap sweep
// One launch per sweep for VNR runs with PenteBorne pure at order 2 (the
// benchmark's options; fused_sweeps_ok): the slopes and plateau-slope
// integrals of SweepGradT and the update of SweepUpdateT, with the
// integrals and their zero flags kept in shared memory instead of the
// dPAr / dPAv / pbz planes.  A cell's face values need the integrals of
// its neighbours along the sweep, so a tile computes them for one cell more
// on each side (the same arithmetic as the neighbouring tile, the same
// bits).  The first sweep writes the new Phi of the cells it changes to
// Phi2 (a neighbouring tile may still read their Phi for its halo); the
// second reads Phi2 for those cells.  The blocks take the sweep direction
// from the control block:
//  - along x: 8 rows of 126 cells, each row's 128 slope cells computed,
//    then its 126 cells updated;
//  - along y: a strip of 32 columns by 60 rows, walked down 4 rows at a time
//    with the slope rows in a ring of 8 (the rows above and below the strip,
//    and two beyond, are its only extra slope work).
constexpr int kFxCells = 128, kFxRows = 8;   // x: slope cells per row, rows per block
constexpr int kFyW = 32, kFyH = 60, kFyRing = 8;  // y: strip width, height, ring rows
constexpr int kFusedCells = kFyRing * kFyW;       // tile cells held (>= kFxCells)

// shared memory of a tile of `cells` slope cells: their flags, then the
// dPAr-side and dPAv-side integrals (ncomp planes of `cells` each)
size_t fused_smem_bytes(int ncomp, int cells) {
  return (size_t)cells + (size_t)2 * ncomp * cells * sizeof(double);
}
dim3 fused_grid_x(const RunView& v) {
  return dim3((unsigned)((long long)((v.nx + kFxCells - 3) / (kFxCells - 2)) *
                         ((v.ny + kFxRows - 1) / kFxRows)));
}
dim3 fused_grid_y(const RunView& v) {
  return dim3((unsigned)((long long)((v.nx + kFyW - 1) / kFyW) * ((v.ny + kFyH - 1) / kFyH)));
}

// DIRX: the kernel of the sweeps along x (the other returns at once)
template <bool DIRX>
__device__ __forceinline__ void sweep_fused(const RunView& v, int sweep) {
  const Ctrl& C = *v.ctrl;
  if (!C.active) return;
  const bool dirx = (sweep == 1) ? C.x_then_y : !C.x_then_y;
  if (dirx != DIRX) return;
  constexpr int cells = DIRX ? kFxCells : kFusedCells;  // tile slope cells
  extern __shared__ double fused_smem[];
  unsigned char* sz = reinterpret_cast<unsigned char*>(fused_smem);
  double* sr = fused_smem + cells / 8;
  double* sv = sr + (size_t)v.ncomp * cells;
  const int tid = threadIdx.x;
  if (DIRX) {
    const int ntx = (v.nx + kFxCells - 3) / (kFxCells - 2);
    const int bx = blockIdx.x % ntx, by = blockIdx.x / ntx;
    if (by * kFxRows >= v.ny) return;
    const int j = bx * (kFxCells - 2) - 1 + tid;
    for (int r = 0; r < kFxRows; ++r) {
      const int i = by * kFxRows + r;
      if (i >= v.ny) break;  // uniform over the block
      if (j >= 0 && j < v.nx)
        SweepGradT<1>{sweep, sz, sr, sv, tid, cells, sweep == 2}(v, i, j);
      __syncthreads();
      if (tid >= 1 && tid <= kFxCells - 2 && j < v.nx)
        SweepUpdateT<1>{sweep, sz, sr, sv, tid, tid - 1, tid + 1, cells, sweep == 1}(v, i, j);
      __syncthreads();
    }
  } else {
    const int nty = (v.nx + kFyW - 1) / kFyW;
    const int bx = blockIdx.x % nty, by = blockIdx.x / nty;
    const int i0 = by * kFyH;
    if (i0 >= v.ny) return;
    const int tx = tid & (kFyW - 1), ty = tid / kFyW;  // 4 rows of 32
    const int j = bx * kFyW + tx;
    const int i1 = (i0 + kFyH < v.ny) ? i0 + kFyH : v.ny;  // rows i0 .. i1 - 1
    auto slot = [&](int row) { return (row & (kFyRing - 1)) * kFyW + tx; };
    // step s: the slope rows i0 - 1 + 4s .. + 3 (one per warp), then the rows
    // i0 + 4(s - 1) .. + 3, whose slope rows (one above, one below) are all
    // in the ring of 8 now; the next step's slope rows overwrite those of
    // rows 4 older, which no update reads any more
    for (int s = 0;; ++s) {
      const int g = i0 - 1 + 4 * s + ty;
      if (g >= 0 && g <= i1 && g < v.ny && j < v.nx)
        SweepGradT<1>{sweep, sz, sr, sv, slot(g), cells, sweep == 2}(v, g, j);
      __syncthreads();
      const int r = i0 + 4 * (s - 1);
      const int row = r + ty;
      if (s >= 1 && row < i1 && j < v.nx)
        SweepUpdateT<1>{sweep, sz, sr, sv, slot(row), slot(row - 1), slot(row + 1), cells,
                        sweep == 1}(v, row, j);
      if (s >= 1 && r + 4 >= i1) break;  // uniform over the block
      __syncthreads();
    }
  }
}
__global__ void __launch_bounds__(128, 7) k_sweep_fused_x(RunView v, int sweep) {
  sweep_fused<true>(v, sweep);
}
__global__ void __launch_bounds__(128, 7) k_sweep_fused_y(RunView v, int sweep) {
  sweep_fused<false>(v, sweep);
}
__global__ void __launch_bounds__(kBX* kBY, 10) k_dual_grad(RunView v, int sweep) { plain_items(v, DualGrad{sweep}); }
// ten resident blocks: where nodes are quiet the kernel waits on memory
__global__ void __launch_bounds__(kBX* kBY, 12) k_dual_update(RunView v, int sweep) { plain_items(v, DualUpdate{sweep}); }
__global__ void __launch_bounds__(kBX* kBY, 8) k_final(RunView v) { plain_items(v, Final{}); }

__global__ void __launch_bounds__(kBatchThreads, 10) kb_lag_nodes(BatchArgs b) { batch_items(b, LagNodes{}, HYDRO_SCHEME_VNR); }
__global__ void __launch_bounds__(kBatchThreads, 8) kb_lag_cells(BatchArgs b) { batch_items(b, LagCells{}, HYDRO_SCHEME_VNR); }
__global__ void __launch_bounds__(kBatchThreads) kb_face_grad(BatchArgs b) { batch_items(b, FaceGrad{b.sweep}); }
__global__ void __launch_bounds__(kBatchThreads, 8) kb_sweep_grad(BatchArgs b) { batch_items(b, SweepGradT<2>{b.sweep}); }
__global__ void __launch_bounds__(kBatchThreads, 8) kb_sweep_grad_nopb(BatchArgs b) { batch_items(b, SweepGradT<0>{b.sweep}); }
__global__ void __launch_bounds__(kBatchThreads) kb_sweep_face(BatchArgs b) { batch_items(b, SweepFaceT<3>{b.sweep}); }
__global__ void __launch_bounds__(kBatchThreads, 8) kb_sweep_update(BatchArgs b) { batch_items(b, SweepUpdateT<2>{b.sweep}); }
__global__ void __launch_bounds__(kBatchThreads, 10) kb_dual_grad(BatchArgs b) { batch_items(b, DualGrad{b.sweep}, HYDRO_SCHEME_VNR); }
__global__ void __launch_bounds__(kBatchThreads, 12) kb_dual_update(BatchArgs b) { batch_items(b, DualUpdate{b.sweep}, HYDRO_SCHEME_VNR); }
__global__ void __launch_bounds__(kBatchThreads, 7) kb_final(BatchArgs b) { batch_items(b, Final{}, HYDRO_SCHEME_VNR); }

// One thread per VNR run: cycle start (begin + reduction reset) and cycle
// end (Eucclhyd runs of the batch: kbe_begin / kbe_end).
__global__ void kb_begin(const RunView* views, const int* ninst) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= *ninst) return;
  const RunView v = views[r];
  if (v.scheme != HYDRO_SCHEME_VNR) return;
  begin_at(v);
  reset_at(v);
}

__global__ void kb_end(const RunView* views, const int* ninst, int* done) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= *ninst) return;
  const RunView v = views[r];
  if (v.scheme != HYDRO_SCHEME_VNR) return;
  end_at(v);
  done[r] = v.ctrl->done;
}

}  // namespace

// ----------------------------------------------------------------- launch
static dim3 cell_grid(const RunView& v) {
  return dim3((v.nx + kBX - 1) / kBX, (v.ny + kBY - 1) / kBY);
}
static dim3 node_grid(const RunView& v) {
  return dim3((v.nx + 1 + kBX - 1) / kBX, (v.ny + 1 + kBY - 1) / kBY);
}

// Computes the node speeds and the initial dt / pressure reductions.
void launch_prologue(const RunView& v, cudaStream_t s) {
  k_node_speed<<<node_grid(v), dim3(kBX, kBY), 0, s>>>(v);
  k_init_reductions<<<cell_grid(v), dim3(kBX, kBY), 0, s>>>(v);
}

void launch_node_mass(const RunView& v, cudaStream_t s) {
  k_node_mass<<<node_grid(v), dim3(kBX, kBY), 0, s>>>(v);
}

// Kernel kinds of one cycle (for per-kernel timing).
const char* const kKernelNames[kNumKernelKinds] = {
    "k_begin",      "k_reset_reductions", "k_lag_nodes", "k_lag_cells",
    "k_sweep_grad", "k_sweep_face",       "k_sweep_update", "k_dual_grad",
    "k_dual_update", "k_final",           "k_end",         "k_face_grad",
    "ke_cell_pre",  "ke_nodes",           "ke_cells",      "ke_final",
    "k_o3_grad",    "k_o3_ystar",        "k_next_positions", "k_sweep_fused"};

// Enqueues one full cycle on stream s; hook(kind) is called before each
// launch (and with kind = -1 after the last) when given.  Returns the number
// of kernels.
// One directional remap sweep (Remap::computeGradPhiFace, computeGradPhi,
// computeUpwindFaceQuantitiesForProjection, computeUremap) on stream s,
// shared by both Lagrange schemes.  Returns the number of kernels.
int launch_sweep(const RunView& v, int sweep, cudaStream_t s, const LaunchHook* hook) {
  const dim3 blk(kBX, kBY);
  const dim3 cg = cell_grid(v), fg = node_grid(v);
  int nk = 0;
  auto H = [&](int kind) {
    if (hook) (*hook)(kind);
  };
  if (v.Phi2) {
    // one kernel per direction; the one whose direction this sweep is not
    // returns at once (the direction is decided on the device)
    H(19);
    k_sweep_fused_x<<<fused_grid_x(v), kFxCells, fused_smem_bytes(v.ncomp, kFxCells), s>>>(v, sweep);
    k_sweep_fused_y<<<fused_grid_y(v), kFxCells, fused_smem_bytes(v.ncomp, kFusedCells), s>>>(v,
                                                                                       sweep);
    return 2;
  }
  // limited slopes (with their face gradients) feed the order-2 face values
  // and PenteBorne only
  if (v.order == 2 || (v.order == 3 && v.pb == 1)) {
    if (v.pb == 0) {
      H(11); k_face_grad<<<fg, blk, 0, s>>>(v, sweep); ++nk;
    }
    H(4);
    if (v.pb == 1) k_sweep_grad_pb<<<cg, blk, 0, s>>>(v, sweep);
    else k_sweep_grad<<<cg, blk, 0, s>>>(v, sweep);
    ++nk;
  }
  if (v.order == 3) {
    H(16); k_o3_grad<<<cg, blk, 0, s>>>(v, sweep); ++nk;
    H(17); k_o3_ystar<<<cg, blk, 0, s>>>(v, sweep); ++nk;
    H(5); k_sweep_face3<<<fg, blk, 0, s>>>(v, sweep); ++nk;
    H(6); k_sweep_update<<<cg, blk, 0, s>>>(v, sweep); ++nk;
  } else if (v.pb == 1) {
    // PenteBorne, orders 1-2: the update forms its face values
    H(6); k_sweep_update_f<<<cg, blk, 0, s>>>(v, sweep); ++nk;
  } else {
    // without PenteBorne the slope kernel wrote the order-2 face values; at
    // order 1 (no slopes) the face kernel forms them
    if (v.order == 1) {
      H(5); k_sweep_face<<<fg, blk, 0, s>>>(v, sweep); ++nk;
    }
    H(6); k_sweep_update<<<cg, blk, 0, s>>>(v, sweep); ++nk;
  }
  return nk;
}

int launch_cycle_euc(const RunView& v, cudaStream_t s, const LaunchHook* hook);

int launch_cycle(const RunView& v, cudaStream_t s, const LaunchHook* hook) {
  if (v.scheme == HYDRO_SCHEME_EUCCLHYD) return launch_cycle_euc(v, s, hook);
  const dim3 blk(kBX, kBY);
  const dim3 cg = cell_grid(v), ng = node_grid(v);
  int nk = 0;
  auto H = [&](int kind) {
    if (hook) (*hook)(kind);
  };
  H(0); k_begin<<<1, 1, 0, s>>>(v); ++nk;
  H(1); k_reset_reductions<<<1, 1, 0, s>>>(v); ++nk;
  H(2); k_lag_nodes<<<ng, blk, 0, s>>>(v); ++nk;
  if (v.projection == 0) {
    // the Lagrange phase only: its cell kernel reduces the next dt, and the
    // new positions are carried to the next cycle after the loop test
    H(3); k_lag_cells_lo<<<cg, blk, 0, s>>>(v); ++nk;
    H(10); k_end<<<1, 1, 0, s>>>(v); ++nk;
    H(18); k_next_positions<<<ng, blk, 0, s>>>(v); ++nk;
    H(-1);
    return nk;
  }
  H(3); k_lag_cells<<<cg, blk, 0, s>>>(v); ++nk;
  for (int sweep = 1; sweep <= 2; ++sweep) {
    nk += launch_sweep(v, sweep, s, hook);
    H(7); k_dual_grad<<<ng, blk, 0, s>>>(v, sweep); ++nk;
    H(8); k_dual_update<<<ng, blk, 0, s>>>(v, sweep); ++nk;
  }
  H(9); k_final<<<cg, blk, 0, s>>>(v); ++nk;
  H(10); k_end<<<1, 1, 0, s>>>(v); ++nk;
  H(-1);
  return nk;
}


// Kernels of the batched cycle in launch order (same kind ids as above; the
// batched cycle start covers kinds 0 and 1).
void launch_batch_euc(int ph, const BatchLaunch& L, const BatchArgs& a, int grid,
                      cudaStream_t s);
int batch_occupancy_euc(int* blocks_per_sm);

// One cycle of every run of a batch: each scheme's Lagrange and final phases
// over its own runs (their phase kernels skip the other scheme's tiles,
// and are launched only when the batch holds runs of that scheme), the
// remap sweeps over all.
int launch_batch_cycle(const BatchLaunch& L, cudaStream_t s,
                       const LaunchHook* hook) {
  int nk = 0;
  auto H = [&](int kind) {
    if (hook) (*hook)(kind);
  };
  auto args = [&](int ph, int sweep) {
    const int on = phase_on_nodes(ph) ? 1 : 0, w = L.shape[ph];
    return BatchArgs{L.views, L.tiles[on][w], L.ntiles[on][w],
                     kTileShapes[w].tw_log2, kTileShapes[w].rows, sweep};
  };
  auto euc = [&](int kind, int ph) {
    H(kind);
    launch_batch_euc(ph, L, ph >= 0 ? args(ph, 0) : BatchArgs{}, ph >= 0 ? L.grid[ph] : 0, s);
    ++nk;
  };
  const int T = kBatchThreads;
  const int rg = (L.max_inst + T - 1) / T;
  if (L.any_vnr) {
    H(0); kb_begin<<<rg, T, 0, s>>>(L.views, L.ninst); ++nk;
  }
  if (L.any_euc) {
    euc(0, -1);
    euc(12, kPhEucCellPre);
  }
  if (L.any_vnr) {
    H(2); kb_lag_nodes<<<L.grid[kPhLagNodes], T, 0, s>>>(args(kPhLagNodes, 0)); ++nk;
  }
  if (L.any_euc) euc(13, kPhEucNodes);
  if (L.any_vnr) {
    H(3); kb_lag_cells<<<L.grid[kPhLagCells], T, 0, s>>>(args(kPhLagCells, 0)); ++nk;
  }
  if (L.any_euc) euc(14, kPhEucCells);
  for (int sweep = 1; sweep <= 2; ++sweep) {
    if (L.any_order2) {
      if (L.any_face_grad) {
        H(11); kb_face_grad<<<L.grid[kPhFaceGrad], T, 0, s>>>(args(kPhFaceGrad, sweep)); ++nk;
      }
      H(4);
      if (L.variant & kBatchNoPB)
        kb_sweep_grad_nopb<<<L.grid[kPhSweepGrad], T, 0, s>>>(args(kPhSweepGrad, sweep));
      else
        kb_sweep_grad<<<L.grid[kPhSweepGrad], T, 0, s>>>(args(kPhSweepGrad, sweep));
      ++nk;
    }
    // face values of order-3 runs and of order-1 runs without PenteBorne
    // (the slope phase writes those of order-2 runs without PenteBorne, the
    // update forms the PenteBorne ones)
    if (L.any_face) {
      H(5); kb_sweep_face<<<L.grid[kPhSweepFace], T, 0, s>>>(args(kPhSweepFace, sweep)); ++nk;
    }
    H(6); kb_sweep_update<<<L.grid[kPhSweepUpdate], T, 0, s>>>(args(kPhSweepUpdate, sweep)); ++nk;
    if (L.any_vnr) {
      H(7); kb_dual_grad<<<L.grid[kPhDualGrad], T, 0, s>>>(args(kPhDualGrad, sweep)); ++nk;
      H(8); kb_dual_update<<<L.grid[kPhDualUpdate], T, 0, s>>>(args(kPhDualUpdate, sweep)); ++nk;
    }
  }
  if (L.any_vnr) {
    H(9); kb_final<<<L.grid[kPhFinal], T, 0, s>>>(args(kPhFinal, 0)); ++nk;
  }
  if (L.any_euc) euc(15, kPhEucFinal);
  if (L.any_vnr) {
    H(10); kb_end<<<rg, T, 0, s>>>(L.views, L.ninst, L.done); ++nk;
  }
  if (L.any_euc) euc(10, -2);
  H(-1);
  return nk;
}

// Resident blocks per SM of each batched phase kernel at kBatchThreads
// threads (for the persistent grid sizes).
int batch_occupancy(int* blocks_per_sm, int variant) {
  const void* fns[kPhFinal + 1] = {
      (const void*)kb_lag_nodes,   (const void*)kb_lag_cells,
      (const void*)kb_face_grad,
      (variant & kBatchNoPB) ? (const void*)kb_sweep_grad_nopb : (const void*)kb_sweep_grad,
      (const void*)kb_sweep_face,
      (const void*)kb_sweep_update,
      (const void*)kb_dual_grad,   (const void*)kb_dual_update,
      (const void*)kb_final};
  for (int ph = 0; ph <= kPhFinal; ++ph) {
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fns[ph], kBatchThreads, 0) !=
        cudaSuccess)
      return -1;
    blocks_per_sm[ph] = n;
  }
  return batch_occupancy_euc(blocks_per_sm);
}

}  // namespace hydro
