// FP64 CUDA kernels of one Eucclhyd Lagrange + remap cycle on GB300.
//
// Cycle structure (reference: Eucclhyd::executeTimeLoopN,
// eucclhyd_remap/EucclhydRemap.cc:84-195):
//   ke_begin     cycle start, reset of the dt reduction
//   ke_cell_pre  computeEOS, computePressionMoyenne, computeGradients,
//                computeMass, computem_cell_deltat (+ block min of dt)
//   ke_nodes     extrapolateValue, computeG, computeNodeDissipationMatrixAndG,
//                computeBoundaryNodeVelocities, computeNodeVelocity, the
//                Lagrange node positions
//   ke_cells     computeLagrangeVolumeAndCenterOfGravity, computeSubCellForce
//                (recomputed per cell from the corner extrapolations),
//                updateCellCenteredLagrangeVariables, the Lagrangian face
//                lengths of the remap
//   sweep x2     the shared directional remap (vnr.cu launch_sweep)
//   ke_final     remapCellcenteredVariable (PhaseRemapFinal.cc:17-232)
//   ke_end       computedeltat, updateTime, loop condition and time swap
//
// Corner quantities live per (cell, corner k); the reference keeps them per
// (node, slot of the cell).  The sub-cell forces are not stored: the cell
// kernel recomputes them from the corner extrapolations and the new node
// velocities, and keeps only their per-material sums for the next cycle's
// pressure gradients (computeGradients, PhaseLagrange.cc:225-244).  All
// arithmetic keeps the reference's operation order (--fmad=false).
#include <cuda_runtime.h>

#include "../internal.h"
#include "items.cuh"
#include "scheme_math.cuh"

namespace hydro {

int launch_sweep(const RunView& v, int sweep, cudaStream_t s, const LaunchHook* hook);

namespace {

constexpr int kBX = 32, kBY = 4;

#define DV __device__ __forceinline__

DV double ldg(const double* p, long long i) { return __ldg(p + i); }
DV double gam(const RunView& v, int m) {
  return m == 0 ? v.gamma[0] : (m == 1 ? v.gamma[1] : v.gamma[2]);
}
DV int eosm(const RunView& v, int m) {
  return m == 0 ? v.eos[0] : (m == 1 ? v.eos[1] : v.eos[2]);
}
// dot product accumulated from 0.0 (includes/Freefunctions.h:15-20); the
// first addition 0.0 + a0 b0 is plus_zero (integer pipe)
DV double dot2(double a0, double a1, double b0, double b1) {
  double r = plus_zero(a0 * b0);
  r += a1 * b1;
  return r;
}
// dot2 is exactly +0 when one vector is two zeros and the other finite
// (plus_zero of a signed zero, plus a signed zero)
DV bool dot2_zero(double a0, double a1, double b0, double b1) {
  return (iszero(a0) && iszero(a1) && is_finite(b0) && is_finite(b1)) ||
         (iszero(b0) && iszero(b1) && is_finite(a0) && is_finite(a1));
}
// x + dot2(a, b), with x + (+0) = plus_zero(x) where the product is +0
DV double add_dot2(double x, double a0, double a1, double b0, double b1) {
  return dot2_zero(a0, a1, b0, b1) ? plus_zero(x) : x + dot2(a0, a1, b0, b1);
}

// block-wide min of ordered encodings, one atomic per block
DV void block_min(unsigned long long dtv, Ctrl* C) {
  __shared__ unsigned long long smin_s[32];
  const int tid = threadIdx.y * blockDim.x + threadIdx.x;
  const int lane = tid & 31, warp = tid >> 5;
  const int nw = (blockDim.x * blockDim.y + 31) >> 5;
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long a = __shfl_xor_sync(0xffffffffu, dtv, o);
    dtv = a < dtv ? a : dtv;
  }
  if (lane == 0) smin_s[warp] = dtv;
  __syncthreads();
  if (warp == 0) {
    dtv = lane < nw ? smin_s[lane] : ~0ull;
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long a = __shfl_xor_sync(0xffffffffu, dtv, o);
      dtv = a < dtv ? a : dtv;
    }
    if (lane == 0 && dtv != ~0ull) atomicMin(&C->dt_min_bits, dtv);
  }
  __syncthreads();
}

// ------------------------------------------------------------- control
DV void euc_begin_at(const RunView& v) {
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
  C.dt_min_bits = ord_bits(1.7976931348623157e308);
}
__global__ void ke_begin(RunView v) { euc_begin_at(v); }

// computedeltat (EucclhydRemap.cc:203-221): the cycle's cell dt minimum
// gives dt_{n+1}; updateTime; the loop condition and the swap of t, dt.
// The Lagrange positions and the remap of this cycle used dt_n.
DV void euc_end_at(const RunView& v) {
  Ctrl& C = *v.ctrl;
  if (!C.active) return;
  const double red = from_ord(C.dt_min_bits);
  C.dt_np1 = smin(v.euc_cfl * red, C.dt_n * 1.05);
  if (dlt(C.dt_np1, v.dt_min)) C.err |= HYDRO_ERR_DT_MIN;
  C.t_np1 = C.t_n + C.dt_np1;
  const bool cont = (C.n + 1 < v.max_iter) && dlt(C.t_np1, v.final_time);
  C.t_n = C.t_np1;
  C.dt_n = C.dt_np1;
  if (cont)
    C.x_then_y = !C.x_then_y;
  else
    C.done = 1;
  if (C.err & ~HYDRO_ERR_NEGATIVE) C.done = 1;
}
__global__ void ke_end(RunView v) { euc_end_at(v); }

// computeEOSGP / computeEOSVoid for material m of cell c (PhaseLagrange.cc
// :70-109); the other EOS ids keep the stored values (their reference
// routines only print).
DV void cell_eos(const RunView& v, int m, long long c, double& pm, double& cm) {
  const long long P = v.pitch;
  const double rm = v.rhom[m * P + c], em = v.em[m * P + c];
  const double g = gam(v, m);
  const int eos = eosm(v, m);
  if (eos == HYDRO_EOS_PERFECT_GAS) {
    pm = (g - 1.0) * rm * em;
    if (pos(rm)) {
      // the volatile barrier keeps the division and the root inside this
      // branch (a select would form them for absent materials too)
      asm volatile("");
      cm = sqrt_ip(div_ip(g * pm, rm));
    } else {
      cm = 1.e-20;
    }
  } else if (eos == HYDRO_EOS_VOID) {
    pm = 0.;
    cm = 1.e-20;
  } else {
    pm = v.pm[m * P + c];
    cm = v.cm[m * P + c];
  }
}

// ------------------------------------------------- cell state of step n
// computeEOS + computeEOSGP / computeEOSVoid (PhaseLagrange.cc:70-109),
// computePressionMoyenne (:139-155), computeGradients (:160-246; the
// fracvol-gradient part only feeds the particle scheme), computeMass
// (:251-261), computem_cell_deltat (:302-316).
struct EucCellPre {
  __device__ __forceinline__ void operator()(const RunView& v, int i, int j) const {
    unsigned long long dtb = ~0ull;
    if (i < v.ny && j < v.nx) {
      const long long P = v.pitch, NP = v.npitch;
      const long long c = (long long)i * v.nx + j;
      const int nb = v.nbmat;
      double pm[3], cm[3];
#pragma unroll
      for (int m = 0; m < 3; ++m) {
        if (m >= nb) break;
        cell_eos(v, m, c, pm[m], cm[m]);
        v.pm[m * P + c] = pm[m];
        v.cm[m * P + c] = cm[m];
      }
      double p = 0., snd = v.c[c];
#pragma unroll
      for (int m = 0; m < 3; ++m) {
        if (m >= nb) break;
        const double t = mul_frac(v.fm[m * P + c], pm[m]);
        p = (m == 0) ? plus_zero(t) : p + t;  // 0.0 + t first
        snd = smax(snd, cm[m]);
      }
      const double rho = v.rho[c];
      if (pos(rho)) snd = sqrt_ip(div_ip(v.gamma[0] * p, rho));
      v.p[c] = p;
      v.c[c] = snd;
      const double V = ldg(v.evol, c);
      if (v.space_order == 2) {
        const long long n0 = (long long)i * (v.nx + 1) + j;
        const long long nd[4] = {n0, n0 + 1, n0 + v.nx + 2, n0 + v.nx + 1};
        double r14[4] = {0.0, 0.0, 0.0, 0.0};
        double cu[4][2], cl[4][2];
        bool still = true;  // every corner velocity a zero, every l finite
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          cu[k][0] = v.u[nd[k]];
          cu[k][1] = v.u[NP + nd[k]];
          cl[k][0] = ldg(v.lpc, (2 * k) * P + c);
          cl[k][1] = ldg(v.lpc, (2 * k + 1) * P + c);
          still = still && iszero(cu[k][0]) && iszero(cu[k][1]) && is_finite(cl[k][0]) &&
                  is_finite(cl[k][1]);
        }
        // then every product is a signed zero and each sum from 0.0 is +0
        if (!still) {
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            const double u0 = cu[k][0], u1 = cu[k][1], l0 = cl[k][0], l1 = cl[k][1];
            const double t[4] = {u0 * l0, u0 * l1, u1 * l0, u1 * l1};
#pragma unroll
            for (int q = 0; q < 4; ++q) r14[q] = (k == 0) ? plus_zero(t[q]) : r14[q] + t[q];
          }
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) v.vg[q * P + c] = qdiv(r14[q], V);
        // per-material pressure gradients from last cycle's corner-force
        // sums, in place
        for (int q = 0; q < 2 * nb; ++q) v.Fs[q * P + c] = qdiv(v.Fs[q * P + c], V);
      }
      const double cmass = rho * V;
      v.cell_mass[c] = cmass;
#pragma unroll
      for (int m = 0; m < 3; ++m) {
        if (m >= nb) break;
        v.cmassm[m * P + c] = mul_frac(v.mfm[m * P + c], cmass);
      }
      const double u0 = v.uc[c], u1 = v.uc[P + c];
      const double un = face_len(u0, u1);  // sqrt(dot(u, u))
      const double cdt = (v.projection == 1) ? div_ip(V, ldg(v.perim, c) * (un + snd))
                                             : div_ip(V, ldg(v.perim, c) * snd);
      if (!is_nan(cdt)) dtb = ord_bits(cdt);
    }
    block_min(dtb, v.ctrl);
  }
};

// Eucclhyd::nodeVelocityBoundaryCondition (ConditionsLimites.cc:109-123)
DV void bc_velocity(int bc, double V0, double V1, const double* Mp, const double* G,
                    double& o0, double& o1) {
  if (bc == kBcSym) {
    const double mv0 = dot2(Mp[0], Mp[1], V0, V1), mv1 = dot2(Mp[2], Mp[3], V0, V1);
    const double s = div_ip(dot2(G[0], G[1], V0, V1), dot2(mv0, mv1, V0, V1));
    o0 = V0 * s;
    o1 = V1 * s;
  } else if (bc == kBcImposed) {
    o0 = V0;
    o1 = V1;
  } else if (bc == 202) {  // free: inverse(Mp) . G
    const double alpha = div_ip(1.0, Mp[0] * Mp[3] - Mp[1] * Mp[2]);
    const double i0 = Mp[3] * alpha, i1 = -Mp[1] * alpha, i2 = -Mp[2] * alpha,
                 i3 = Mp[0] * alpha;
    o0 = dot2(i0, i1, G[0], G[1]);
    o1 = dot2(i2, i3, G[0], G[1]);
  } else {
    o0 = 0.0;
    o1 = 0.0;
  }
}

// ----------------------------------------------------------- node solve
// extrapolateValue (:322-479), computeG (:484-505),
// computeNodeDissipationMatrixAndG (:511-527), computeBoundaryNodeVelocities
// (ConditionsLimites.cc:19-107), computeNodeVelocity (:532-543),
// computeLagrangePosition nodes (:573-580).
struct EucNodes {
  __device__ __forceinline__ void operator()(const RunView& v, int i, int j) const {
    if (i > v.ny || j > v.nx) return;
    const Ctrl& C = *v.ctrl;
    const long long P = v.pitch, NP = v.npitch;
    const long long p = (long long)i * (v.nx + 1) + j;
    const int nb = v.nbmat;
    // cells of the node in getCellsOfNode order (CartesianMesh2D.cc:97-108)
    // and the node's position in each
    long long cells[4];
    int loc[4], kc = 0;
    if (i < v.ny && j < v.nx) { cells[kc] = (long long)i * v.nx + j; loc[kc++] = 0; }
    if (i < v.ny && j > 0) { cells[kc] = (long long)i * v.nx + j - 1; loc[kc++] = 1; }
    if (i > 0 && j < v.nx) { cells[kc] = (long long)(i - 1) * v.nx + j; loc[kc++] = 3; }
    if (i > 0 && j > 0) { cells[kc] = (long long)(i - 1) * v.nx + j - 1; loc[kc++] = 2; }
    const double X0 = ldg(v.xs, j), X1 = ldg(v.ys, i);
    double pe_tot[4], ue0[4], ue1[4];
    if (v.space_order == 2) {
      double minP[3], maxP[3];
#pragma unroll
      for (int m = 0; m < 3; ++m) {
        if (m >= nb) break;
        minP[m] = 1.7976931348623157e308;
        for (int t = 0; t < kc; ++t) minP[m] = smin(minP[m], v.pm[m * P + cells[t]]);
        maxP[m] = 2.2250738585072014e-308;  // numeric_limits<double>::min()
        for (int t = 0; t < kc; ++t) maxP[m] = smax(maxP[m], v.pm[m * P + cells[t]]);
      }
      double minVx = 1.7976931348623157e308, maxVx = 2.2250738585072014e-308;
      double minVy = 1.7976931348623157e308, maxVy = 2.2250738585072014e-308;
      for (int t = 0; t < kc; ++t) minVx = smin(minVx, v.uc[cells[t]]);
      for (int t = 0; t < kc; ++t) maxVx = smax(maxVx, v.uc[cells[t]]);
      for (int t = 0; t < kc; ++t) minVy = smin(minVy, v.uc[P + cells[t]]);
      for (int t = 0; t < kc; ++t) maxVy = smax(maxVy, v.uc[P + cells[t]]);
      for (int t = 0; t < kc; ++t) {
        const long long c = cells[t];
        const int k = loc[t];
        const double d0 = X0 - ldg(v.xcc, c), d1 = X1 - ldg(v.xcc, P + c);
        double pt = 0.;
#pragma unroll
        for (int m = 0; m < 3; ++m) {
          if (m >= nb) break;
          const double pr = add_dot2(v.pm[m * P + c], v.Fs[(2 * m) * P + c],
                                     v.Fs[(2 * m + 1) * P + c], d0, d1);
          const double pe = smax(smin(maxP[m], pr), minP[m]);
          v.peex[(k * nb + m) * P + c] = pe;
          const double tp = mul_frac(v.fm[m * P + c], pe);
          pt = (m == 0) ? plus_zero(tp) : pt + tp;
        }
        pe_tot[t] = pt;
        v.pex[k * P + c] = pt;
        const double vt0 = add_dot2(v.uc[c], v.vg[c], v.vg[P + c], d0, d1);
        const double vt1 = add_dot2(v.uc[P + c], v.vg[2 * P + c], v.vg[3 * P + c], d0, d1);
        ue0[t] = smax(smin(maxVx, vt0), minVx);
        ue1[t] = smax(smin(maxVy, vt1), minVy);
        v.uex[(2 * k) * P + c] = ue0[t];
        v.uex[(2 * k + 1) * P + c] = ue1[t];
      }
    } else {
      for (int t = 0; t < kc; ++t) {
        const long long c = cells[t];
        const int k = loc[t];
        pe_tot[t] = v.p[c];
        ue0[t] = v.uc[c];
        ue1[t] = v.uc[P + c];
        v.pex[k * P + c] = pe_tot[t];
        v.uex[(2 * k) * P + c] = ue0[t];
        v.uex[(2 * k + 1) * P + c] = ue1[t];
#pragma unroll
        for (int m = 0; m < 3; ++m) {
          if (m >= nb) break;
          v.peex[(k * nb + m) * P + c] = v.pm[m * P + c];
        }
      }
    }
    // G and the node dissipation matrix
    double G[2] = {0.0, 0.0};
    double Mp[4] = {0.0, 0.0, 0.0, 0.0};
    for (int t = 0; t < kc; ++t) {
      const long long c = cells[t];
      const int k = loc[t];
      const double s = v.rho[c] * v.c[c];
      const double m00 = ldg(v.cmat, (3 * k) * P + c) * s;
      const double m01 = ldg(v.cmat, (3 * k + 1) * P + c) * s;
      const double m11 = ldg(v.cmat, (3 * k + 2) * P + c) * s;
      const double l0 = ldg(v.lpc, (2 * k) * P + c), l1 = ldg(v.lpc, (2 * k + 1) * P + c);
      // mv + l * pe, with (+0) + y = plus_zero(y) where mv = dot2(m, ue) is +0
      const double g0 = dot2_zero(m00, m01, ue0[t], ue1[t])
                            ? plus_zero(l0 * pe_tot[t])
                            : dot2(m00, m01, ue0[t], ue1[t]) + l0 * pe_tot[t];
      const double g1 = dot2_zero(m01, m11, ue0[t], ue1[t])
                            ? plus_zero(l1 * pe_tot[t])
                            : dot2(m01, m11, ue0[t], ue1[t]) + l1 * pe_tot[t];
      if (t == 0) {  // sums from 0.0: 0.0 + x as plus_zero
        G[0] = plus_zero(g0);
        G[1] = plus_zero(g1);
        Mp[0] = plus_zero(m00);
        Mp[1] = plus_zero(m01);
        Mp[2] = Mp[1];
        Mp[3] = plus_zero(m11);
      } else {
        G[0] = G[0] + g0;
        G[1] = G[1] + g1;
        Mp[0] = Mp[0] + m00;
        Mp[1] = Mp[1] + m01;
        Mp[2] = Mp[2] + m01;
        Mp[3] = Mp[3] + m11;
      }
    }
    // node velocity: the boundary rule of the last list holding the node
    // (sides, then corners), inverse(Mp) . G inside
    double u0, u1;
    const bool top = (i == v.ny), bot = (i == 0), lft = (j == 0), rgt = (j == v.nx);
    if ((top || bot) && (lft || rgt)) {
      const int b1 = top ? v.bc_top : v.bc_bottom;
      const double* V1 = top ? v.v_top : v.v_bottom;
      const int b2 = lft ? v.bc_left : v.bc_right;
      const double* V2 = lft ? v.v_left : v.v_right;
      const double A0 = V1[0], A1 = V1[1], B0 = V2[0], B1 = V2[1];
      u0 = 0.0;
      u1 = 0.0;
      if (b1 == kBcSym && b2 == kBcSym) {
        const double na = sqrt_ip(dot2(A0, A1, A0, A1)), nbb = sqrt_ip(dot2(B0, B1, B0, B1));
        if (fabs(fabs(dot2(A0, A1, B0, B1)) - na * nbb) < 1.0E-8)
          bc_velocity(kBcSym, A0, A1, Mp, G, u0, u1);
      } else if (b1 == kBcImposed && b2 == kBcImposed) {
        u0 = half(A0 + B0);
        u1 = half(A1 + B1);
      } else if (b1 == 202 && b2 == 202) {
        bc_velocity(202, A0, A1, Mp, G, u0, u1);
      }
    } else if (lft) {
      bc_velocity(v.bc_left, v.v_left[0], v.v_left[1], Mp, G, u0, u1);
    } else if (rgt) {
      bc_velocity(v.bc_right, v.v_right[0], v.v_right[1], Mp, G, u0, u1);
    } else if (top) {
      bc_velocity(v.bc_top, v.v_top[0], v.v_top[1], Mp, G, u0, u1);
    } else if (bot) {
      bc_velocity(v.bc_bottom, v.v_bottom[0], v.v_bottom[1], Mp, G, u0, u1);
    } else {
      // inverse(Mp) . G: with G two zeros the result is dot2(i, G) = +0 as
      // long as the inverse is finite: |Mp| < 2^500 and |det| >= 2^-500
      // bound it by 2^1000, so the reciprocal and the products are not
      // formed
      constexpr unsigned long long kLo = 523ull << 52, kHi = 1523ull << 52;
      bool gz = iszero(G[0]) && iszero(G[1]) && (ubits(Mp[0]) & kMag) < kHi &&
                (ubits(Mp[1]) & kMag) < kHi && (ubits(Mp[2]) & kMag) < kHi &&
                (ubits(Mp[3]) & kMag) < kHi;
      if (gz) {
        const double det = Mp[0] * Mp[3] - Mp[1] * Mp[2];
        gz = (ubits(det) & kMag) >= kLo;  // finite: |Mp| < 2^500
      }
      if (gz) {
        u0 = 0.0;
        u1 = 0.0;
      } else {
        bc_velocity(202, 0.0, 0.0, Mp, G, u0, u1);
      }
    }
    v.u[p] = u0;
    v.u[NP + p] = u1;
    v.XL[p] = addz(X0, mulz(u0, C.dt_n));
    v.XL[NP + p] = addz(X1, mulz(u1, C.dt_n));
  }
};

// ----------------------------------------------------- cell Lagrange step
// computeLagrangeVolumeAndCenterOfGravity (:671-716), computeSubCellForce
// (:625-666), updateCellCenteredLagrangeVariables (:746-1010), and the
// Lagrangian face lengths that give HvLagrange (remap/PhaseRemap1.cc:57-71).
struct EucCells {
  __device__ __forceinline__ void operator()(const RunView& v, int i, int j) const {
    if (i >= v.ny || j >= v.nx) return;
    const Ctrl& C = *v.ctrl;
    const long long P = v.pitch, NP = v.npitch;
    const long long c = (long long)i * v.nx + j;
    const int nb = v.nbmat;
    const long long n0 = (long long)i * (v.nx + 1) + j;
    const long long nd[4] = {n0, n0 + 1, n0 + v.nx + 2, n0 + v.nx + 1};
    double X[4][2];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      X[k][0] = v.XL[nd[k]];
      X[k][1] = v.XL[NP + nd[k]];
    }
    // Lagrangian geometry; a cell whose four nodes kept their Euler
    // positions (bit for bit) has the geometry the set-up formed with the
    // same function from the same numbers (loaded with the positions).
    // The geometry is stored at the end: a store here would order every
    // later load behind it.
    double g0v[5];
#pragma unroll
    for (int q = 0; q < 5; ++q) g0v[q] = ldg(v.geo0, q * P + c);
    const unsigned long long x0 = ubits(ldg(v.xs, j)), x1 = ubits(ldg(v.xs, j + 1));
    const unsigned long long y0 = ubits(ldg(v.ys, i)), y1 = ubits(ldg(v.ys, i + 1));
    const bool rest = ubits(X[0][0]) == x0 && ubits(X[0][1]) == y0 && ubits(X[1][0]) == x1 &&
                      ubits(X[1][1]) == y0 && ubits(X[2][0]) == x1 && ubits(X[2][1]) == y1 &&
                      ubits(X[3][0]) == x0 && ubits(X[3][1]) == y1;
    CellGeom G;
    if (rest) {
      G.vol = g0v[0];
      G.xc0 = g0v[1];
      G.xc1 = g0v[2];
      G.hx = g0v[3];
      G.hy = g0v[4];
    } else {
      G = euc_cell_geometry(X, v.order > 1);
    }
    const double vol = G.vol;
    // sub-cell forces of the cell's corners with the new node velocities.
    // Zero shortcuts (where the mesh is at rest the node velocities and
    // their differences are zeros): dot2(a, b) with b0, b1 zeros and a0, a1
    // finite is +0 (plus_zero of a signed zero, plus a signed zero), so
    // x + dot2 is plus_zero(x) (x + 0.0), and a product c * s with |c| and
    // |s| under 2^511 is finite without being formed.
    constexpr unsigned long long kSafe = 0x5fe0000000000000ull;  // 2^511
    auto small = [](double x) { return (ubits(x) & kMag) < kSafe; };
    const double rho = v.rho[c], snd = v.c[c];
    const double s = rho * snd;
    double se[3];
#pragma unroll
    for (int m = 0; m < 3; ++m) se[m] = (m < nb) ? v.rhom[m * P + c] * snd : 0.0;
    double r2 = 0.0, r3a = 0.0, r3b = 0.0;
    double un0[4], un1[4], Fe0[4][3], Fe1[4][3];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const double u0 = v.u[nd[k]], u1 = v.u[NP + nd[k]];
      un0[k] = u0;
      un1[k] = u1;
      const double l0 = ldg(v.lpc, (2 * k) * P + c), l1 = ldg(v.lpc, (2 * k + 1) * P + c);
      const bool uz = iszero(u0) && iszero(u1);
      const bool t2z = uz && is_finite(l0) && is_finite(l1);  // dot2(l, u) = +0
      const double t2 = t2z ? 0.0 : dot2(l0, l1, u0, u1);
      r2 = (k == 0) ? plus_zero(t2) : (t2z ? plus_zero(r2) : r2 + t2);
      const double ux0 = v.uex[(2 * k) * P + c], ux1 = v.uex[(2 * k + 1) * P + c];
      // velocity differences; any zero difference gives the same dot2, so
      // two zeros minus two zeros need not be formed
      double du0 = 0.0, du1 = 0.0;
      bool duz = uz && iszero(ux0) && iszero(ux1);
      if (!duz) {
        du0 = u0 - ux0;
        du1 = u1 - ux1;
        duz = iszero(du0) && iszero(du1);
      }
      const double c00 = ldg(v.cmat, (3 * k) * P + c), c01 = ldg(v.cmat, (3 * k + 1) * P + c),
                   c11 = ldg(v.cmat, (3 * k + 2) * P + c);
      const bool cz = duz && small(c00) && small(c01) && small(c11);
      {
        const double mp = -v.pex[k * P + c];
        double f0, f1;
        if (cz && small(s)) {
          f0 = plus_zero(l0 * mp);
          f1 = plus_zero(l1 * mp);
        } else {
          const double m00 = c00 * s, m01 = c01 * s, m11 = c11 * s;
          f0 = l0 * mp + dot2(m00, m01, du0, du1);
          f1 = l1 * mp + dot2(m01, m11, du0, du1);
        }
        r3a = (k == 0) ? plus_zero(f0) : r3a + f0;
        r3b = (k == 0) ? plus_zero(f1) : r3b + f1;
      }
#pragma unroll
      for (int m = 0; m < 3; ++m) {
        if (m >= nb) break;
        const double mp = -v.peex[(k * nb + m) * P + c];
        if (cz && small(se[m])) {
          Fe0[k][m] = plus_zero(l0 * mp);
          Fe1[k][m] = plus_zero(l1 * mp);
        } else {
          const double m00 = c00 * se[m], m01 = c01 * se[m], m11 = c11 * se[m];
          Fe0[k][m] = l0 * mp + dot2(m00, m01, du0, du1);
          Fe1[k][m] = l1 * mp + dot2(m01, m11, du0, du1);
        }
      }
    }
    const double dt = C.dt_n;
    const double cmass = v.cell_mass[c];
    // (dt / cmass) * r2: a zero r2 times a finite quotient (|dt| < 2^500,
    // |cmass| >= 2^-500) is the zero of the xor of the three signs
    constexpr unsigned long long kLo = 523ull << 52, kHi = 1523ull << 52;  // 2^-500, 2^500
    const bool qfin = (ubits(dt) & kMag) < kHi && (ubits(cmass) & kMag) >= kLo &&
                      is_finite(cmass);
    const double dr2 = (iszero(r2) && qfin) ? from_bits((ubits(dt) ^ ubits(cmass) ^ ubits(r2)) & ~kMag)
                                            : div_ip(dt, cmass) * r2;
    const double rhoL = div_ip(1.0, addz(div_ip(1.0, rho), dr2));
    const double uc0 = v.uc[c], uc1 = v.uc[P + c];
    const double uL0 = addz(uc0, qdiv(mulz(r3a, dt), cmass));
    const double uL1 = addz(uc1, qdiv(mulz(r3b, dt), cmass));
    const double mid0 = half(addz(uc0, uL0)), mid1 = half(addz(uc1, uL1));
    double pr4[3] = {0.0, 0.0, 0.0}, fsa[3] = {0.0, 0.0, 0.0}, fsb[3] = {0.0, 0.0, 0.0};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const double d0 = subz(un0[k], mid0), d1 = subz(un1[k], mid1);
      const bool dz = iszero(d0) && iszero(d1);
#pragma unroll
      for (int m = 0; m < 3; ++m) {
        if (m >= nb) break;
        const bool t4z = dz && is_finite(Fe0[k][m]) && is_finite(Fe1[k][m]);  // dot2 = +0
        const double t4 = t4z ? 0.0 : dot2(Fe0[k][m], Fe1[k][m], d0, d1);
        pr4[m] = (k == 0) ? plus_zero(t4) : (t4z ? plus_zero(pr4[m]) : pr4[m] + t4);
        fsa[m] = (k == 0) ? plus_zero(Fe0[k][m]) : fsa[m] + Fe0[k][m];
        fsb[m] = (k == 0) ? plus_zero(Fe1[k][m]) : fsb[m] + Fe1[k][m];
      }
    }
    double peL[3];
    const double thr = v.threshold;
#pragma unroll
    for (int m = 0; m < 3; ++m) {
      if (m >= nb) break;
      peL[m] = 0.;
      const double f = v.fm[m * P + c], cmm = v.cmassm[m * P + c];
      if (dgt(f, thr) && nz(cmm)) {
        // ((f * dt) / cmm) * pr4: a zero pr4 times a finite quotient (|f| and
        // |dt| below 2^250, |cmm| >= 2^-500: under 2^1000) is a signed zero
        constexpr unsigned long long kMid = 1273ull << 52;  // 2^250
        const double em = v.em[m * P + c];
        const bool pz = iszero(pr4[m]) && (ubits(f) & kMag) < kMid && (ubits(dt) & kMag) < kMid &&
                        (ubits(cmm) & kMag) >= kLo && is_finite(cmm);
        const double w = pz ? from_bits((ubits(f) ^ ubits(dt) ^ ubits(cmm) ^ ubits(pr4[m])) & ~kMag)
                            : div_ip(f * dt, cmm) * pr4[m];
        peL[m] = addz(em, w);
      }
    }
    // ULagrange and Phi
    const int ncomp = v.ncomp;
    double U[kMaxComp];
#pragma unroll
    for (int m = 0; m < 3; ++m) {
      if (m >= nb) break;
      const double mf = v.mfm[m * P + c];
      U[m] = mul_frac(v.fm[m * P + c], vol);
      U[nb + m] = mulz(mulz(mf, vol), rhoL);
      U[2 * nb + m] = mulz(mulz(mulz(mf, vol), rhoL), peL[m]);
    }
    U[3 * nb] = mulz(vol * rhoL, uL0);
    U[3 * nb + 1] = mulz(vol * rhoL, uL1);
    if (v.conservative == 1) U[3 * nb + 2] = 0.5 * vol * rhoL * (uL0 * uL0 + uL1 * uL1);
    for (int k = 0; k < ncomp; ++k) v.UL[k * P + c] = U[k];
    if (v.pb == 1) {
      double sv = 0.;
      for (int m = 0; m < nb; ++m) sv += U[m];
      double sm = 0.;
      for (int m = 0; m < nb; ++m) {
        v.Phi[m * P + c] = qdiv(U[m], sv);
        v.Phi[(nb + m) * P + c] = nz(U[m]) ? qdiv(U[nb + m], U[m]) : 0.;
        sm += U[nb + m];
      }
      v.Phi[3 * nb * P + c] = qdiv(U[3 * nb], sm);
      v.Phi[(3 * nb + 1) * P + c] = qdiv(U[3 * nb + 1], sm);
      for (int m = 0; m < nb; ++m)
        v.Phi[(2 * nb + m) * P + c] = nz(U[nb + m]) ? qdiv(U[2 * nb + m], U[nb + m]) : 0.;
      if (v.conservative == 1) v.Phi[(3 * nb + 2) * P + c] = qdiv(U[3 * nb + 2], sm);
    } else {
      const SharedDiv Sv = shared_div(vol);  // one denominator, ncomp quotients
      for (int k = 0; k < ncomp; ++k) v.Phi[k * P + c] = qdiv_shared(Sv, U[k]);
    }
    // per-material corner-force sums for the next cycle's gradients, and
    // the Lagrangian geometry (volume, centroid, HvLagrange widths)
#pragma unroll
    for (int m = 0; m < 3; ++m) {
      if (m >= nb) break;
      v.Fs[(2 * m) * P + c] = fsa[m];
      v.Fs[(2 * m + 1) * P + c] = fsb[m];
    }
    v.vL[c] = vol;
    v.XcL[c] = G.xc0;
    v.XcL[P + c] = G.xc1;
    if (v.order > 1) {
      v.Hx[c] = G.hx;
      v.Hy[c] = G.hy;
    }
  }
};

// --------------------------------------------------------- remap final
// Eucclhyd::remapCellcenteredVariable (PhaseRemapFinal.cc:17-200)
struct EucFinal {
  __device__ __forceinline__ void operator()(const RunView& v, int i, int j) const {
    if (i >= v.ny || j >= v.nx) return;
    Ctrl& C = *v.ctrl;
    const long long P = v.pitch;
    const long long c = (long long)i * v.nx + j;
    const int nb = v.nbmat;
    const double thr = v.threshold;
    const double* U = v.UL + c;  // second sweep output
    const double vol = ldg(v.evol, c);
    double volt = 0., masset = 0., vn[3];
#pragma unroll
    for (int m = 0; m < 3; ++m) {
      if (m >= nb) break;
      vn[m] = U[m * P];
      volt = (m == 0) ? plus_zero(vn[m]) : volt + vn[m];  // 0.0 + x first
      masset = (m == 0) ? plus_zero(U[(nb + m) * P]) : masset + U[(nb + m) * P];
    }
    double vnorm = 0.;
    const double r = qdiv(vol, volt);
#pragma unroll
    for (int m = 0; m < 3; ++m) {
      if (m >= nb) break;
      vn[m] *= r;
      vnorm = (m == 0) ? plus_zero(vn[m]) : vnorm + vn[m];
    }
    double f[3], mf[3], sf = 0.;
#pragma unroll
    for (int m = 0; m < 3; ++m) {
      if (m >= nb) break;
      f[m] = qdiv(vn[m], vnorm);
      if (dlt(f[m], thr)) f[m] = 0.;
      sf = (m == 0) ? plus_zero(f[m]) : sf + f[m];
    }
#pragma unroll
    for (int m = 0; m < 3; ++m) {
      if (m >= nb) break;
      f[m] = qdiv(f[m], sf);
    }
    int matcell = 0, imatpure = -1;
    for (int m = 0; m < nb; ++m)
      if (pos(f[m])) {
        matcell++;
        imatpure = m;
      }
    v.mixte[c] = (matcell > 1) ? 1 : 0;
    v.pure[c] = (matcell > 1) ? -1 : imatpure;
#pragma unroll
    for (int m = 0; m < 3; ++m) {
      if (m >= nb) break;
      mf[m] = qdiv(U[(nb + m) * P], masset);
    }
    double fmt = 0.;
#pragma unroll
    for (int m = 0; m < 3; ++m) {
      if (m >= nb) break;
      if (dlt(f[m], thr)) mf[m] = 0.;
      fmt = (m == 0) ? plus_zero(mf[m]) : fmt + mf[m];
    }
#pragma unroll
    for (int m = 0; m < 3; ++m) {
      if (m >= nb) break;
      mf[m] = qdiv(mf[m], fmt);
    }
    double dm[3] = {0., 0., 0.}, dens = 0.;
#pragma unroll
    for (int m = 0; m < 3; ++m) {
      if (m >= nb) break;
      if (dgt(f[m], thr)) dm[m] = qdiv(U[(nb + m) * P], vn[m]);
      const double fd = mul_frac(f[m], dm[m]);
      dens = (m == 0) ? plus_zero(fd) : dens + fd;
    }
    const double mv = dens * vol;
    const double un0 = qdiv(U[3 * nb * P], mv), un1 = qdiv(U[(3 * nb + 1) * P], mv);
    double pe[3] = {0., 0., 0.};
#pragma unroll
    for (int m = 0; m < 3; ++m) {
      if (m >= nb) break;
      if (dgt(f[m], thr) && nz(U[(nb + m) * P]))
        pe[m] = qdiv(U[(2 * nb + m) * P], U[(nb + m) * P]);
    }
    double dec = 0.;
    if (v.conservative == 1)
      dec = qdiv(U[(3 * nb + 2) * P], masset) - 0.5 * (un0 * un0 + un1 * un1);
    double e = 0.;
    double rhom[3], em[3];
#pragma unroll
    for (int m = 0; m < 3; ++m) {
      if (m >= nb) break;
      rhom[m] = dm[m];
      em[m] = pe[m];
      em[m] += dec;
      const double te = mul_frac(mf[m], em[m]);
      e = (m == 0) ? plus_zero(te) : e + te;
    }
#pragma unroll
    for (int m = 0; m < 3; ++m) {
      if (m >= nb) break;
      if (neg(pe[m]) || neg(dm[m])) {
        rhom[m] = 0.;
        em[m] = 0.;
        mf[m] = 0.;
        f[m] = 0.;
        atomicOr(&C.err, HYDRO_ERR_NEGATIVE);
      }
    }
    if (is_nan(e) || is_nan(dens)) {
      atomicOr(&C.err, HYDRO_ERR_NAN);
      atomicMin((unsigned long long*)&C.err_cell, (unsigned long long)c);
    }
    v.rho[c] = dens;
    v.uc[c] = un0;
    v.uc[P + c] = un1;
    v.e[c] = e;
    // velocities for the outputs (PhaseRemapFinal.cc:200-213): kept where
    // the velocity is zero, else pushed away from zero to the threshold
    if (pos(un0)) v.uco[c] = smax(un0, thr);
    else if (neg(un0)) v.uco[c] = smin(un0, -thr);
    if (pos(un1)) v.uco[P + c] = smax(un1, thr);
    else if (neg(un1)) v.uco[P + c] = smin(un1, -thr);
#pragma unroll
    for (int m = 0; m < 3; ++m) {
      if (m >= nb) break;
      v.fm[m * P + c] = f[m];
      v.mfm[m * P + c] = mf[m];
      v.rhom[m * P + c] = rhom[m];
      v.em[m * P + c] = em[m];
    }
  }
};

// The mean pressure that Eucclhyd::dumpVariables writes: computeEOS +
// computePressionMoyenne (PhaseLagrange.cc:70-155) on the current state,
// i.e. what the next cycle's first kernel computes, into out[c].
__global__ void __launch_bounds__(kBX* kBY) ke_out_pressure(RunView v, double* out) {
  const int i = blockIdx.y * kBY + threadIdx.y, j = blockIdx.x * kBX + threadIdx.x;
  if (i >= v.ny || j >= v.nx) return;
  const long long c = (long long)i * v.nx + j;
  double p = 0.;
  for (int m = 0; m < v.nbmat; ++m) {
    double pm, cm;
    cell_eos(v, m, c, pm, cm);
    p += v.fm[m * v.pitch + c] * pm;
  }
  out[c] = p;
}

template <class F>
__device__ __forceinline__ void plain_items(const RunView& v, const F& f) {
  if (!v.ctrl->active) return;
  f(v, blockIdx.y * kBY + threadIdx.y, blockIdx.x * kBX + threadIdx.x);
}

__global__ void __launch_bounds__(kBX* kBY, 12) ke_cell_pre(RunView v) { plain_items(v, EucCellPre{}); }
__global__ void __launch_bounds__(kBX* kBY, 8) ke_nodes(RunView v) { plain_items(v, EucNodes{}); }
__global__ void __launch_bounds__(kBX* kBY, 8) ke_cells(RunView v) { plain_items(v, EucCells{}); }
__global__ void __launch_bounds__(kBX* kBY, 10) ke_final(RunView v) { plain_items(v, EucFinal{}); }

// Batched launches of the Eucclhyd phases (the batch's VNR runs are skipped;
// the remap sweeps are the shared batched kernels of vnr.cu).
constexpr int kE = HYDRO_SCHEME_EUCCLHYD;
__global__ void __launch_bounds__(kBatchThreads, 12) kbe_cell_pre(BatchArgs b) { batch_items(b, EucCellPre{}, kE); }
__global__ void __launch_bounds__(kBatchThreads, 8) kbe_nodes(BatchArgs b) { batch_items(b, EucNodes{}, kE); }
__global__ void __launch_bounds__(kBatchThreads, 8) kbe_cells(BatchArgs b) { batch_items(b, EucCells{}, kE); }
__global__ void __launch_bounds__(kBatchThreads, 10) kbe_final(BatchArgs b) { batch_items(b, EucFinal{}, kE); }
// one thread per Eucclhyd run: cycle start and end
__global__ void kbe_begin(const RunView* views, const int* ninst) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= *ninst) return;
  const RunView v = views[r];
  if (v.scheme == kE) euc_begin_at(v);
}
__global__ void kbe_end(const RunView* views, const int* ninst, int* done) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= *ninst) return;
  const RunView v = views[r];
  if (v.scheme != kE) return;
  euc_end_at(v);
  done[r] = v.ctrl->done;
}

}  // namespace

int launch_euc_out_pressure(const RunView& v, double* out, cudaStream_t s) {
  const dim3 cg((v.nx + kBX - 1) / kBX, (v.ny + kBY - 1) / kBY);
  ke_out_pressure<<<cg, dim3(kBX, kBY), 0, s>>>(v, out);
  return 1;
}

// One Eucclhyd phase of a batched cycle: kPhEucCellPre, kPhEucNodes,
// kPhEucCells, kPhEucFinal on the tile arguments a, or (ph < 0) the
// per-run cycle start (-1) / end (-2).
void launch_batch_euc(int ph, const BatchLaunch& L, const BatchArgs& a, int grid,
                      cudaStream_t s) {
  const int T = kBatchThreads, rg = (L.max_inst + T - 1) / T;
  switch (ph) {
    case -1: kbe_begin<<<rg, T, 0, s>>>(L.views, L.ninst); break;
    case -2: kbe_end<<<rg, T, 0, s>>>(L.views, L.ninst, L.done); break;
    case kPhEucCellPre: kbe_cell_pre<<<grid, T, 0, s>>>(a); break;
    case kPhEucNodes: kbe_nodes<<<grid, T, 0, s>>>(a); break;
    case kPhEucCells: kbe_cells<<<grid, T, 0, s>>>(a); break;
    case kPhEucFinal: kbe_final<<<grid, T, 0, s>>>(a); break;
    default: break;
  }
}
// resident blocks per SM of the Eucclhyd phase kernels
int batch_occupancy_euc(int* blocks_per_sm) {
  const int ph[4] = {kPhEucCellPre, kPhEucNodes, kPhEucCells, kPhEucFinal};
  const void* fns[4] = {(const void*)kbe_cell_pre, (const void*)kbe_nodes,
                        (const void*)kbe_cells, (const void*)kbe_final};
  for (int k = 0; k < 4; ++k) {
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fns[k], kBatchThreads, 0) !=
        cudaSuccess)
      return -1;
    blocks_per_sm[ph[k]] = n;
  }
  return 0;
}

// One Eucclhyd cycle on stream s (kind ids: 0 begin, 12 cell_pre, 13 nodes,
// 14 cells, sweeps, 15 final, 10 end).  Returns the number of kernels.
int launch_cycle_euc(const RunView& v, cudaStream_t s, const LaunchHook* hook) {
  const dim3 blk(kBX, kBY);
  const dim3 cg((v.nx + kBX - 1) / kBX, (v.ny + kBY - 1) / kBY);
  const dim3 ng((v.nx + 1 + kBX - 1) / kBX, (v.ny + 1 + kBY - 1) / kBY);
  int nk = 0;
  auto H = [&](int kind) {
    if (hook) (*hook)(kind);
  };
  H(0); ke_begin<<<1, 1, 0, s>>>(v); ++nk;
  H(12); ke_cell_pre<<<cg, blk, 0, s>>>(v); ++nk;
  H(13); ke_nodes<<<ng, blk, 0, s>>>(v); ++nk;
  H(14); ke_cells<<<cg, blk, 0, s>>>(v); ++nk;
  for (int sweep = 1; sweep <= 2; ++sweep) nk += launch_sweep(v, sweep, s, hook);
  H(15); ke_final<<<cg, blk, 0, s>>>(v); ++nk;
  H(10); ke_end<<<1, 1, 0, s>>>(v); ++nk;
  H(-1);
  return nk;
}

}  // namespace hydro
