// Initial state and constant Euler geometry of a run, built on the device.
//
// The set-up sequences restated here, operation by operation (the kernels
// are compiled with --fmad=false and IEEE division / square root, so every
// value equals the reference's):
//   VNR      Vnr::simulate (vnr_remap/VnrRemap.cc:330-341): initCellPos,
//            init, initSubVol, initMeshGeometryForFaces, computeCellMass,
//            initDeltaT, initInternalEnergy, computeNodeMass
//            (vnr_remap/Init.cc:103-554, PhaseLagrange.cc:14-48)
//   Eucclhyd Eucclhyd::simulate (eucclhyd_remap/EucclhydRemap.cc:273-287):
//            computeCornerNormal (PhaseLagrange.cc:27-66), initMeshGeometry-
//            ForCells, initCellInternalEnergy, initCellVelocity, initDensity,
//            initMeshGeometryForFaces (eucclhyd_remap/Init.cc:106-716)
// plus the extensions selected by init_variant (mixed interface row of the
// bi-material Sod, advection step, scaled triple point) and the VNR Sedov
// case.  One thread per cell writes the cell's state and geometry, then one
// thread per node its velocity, mass and the per-row / per-column arrays.
// Only the arena (zeroed beforehand) is written; the host uploads nothing
// but the control block.
#include <cuda_runtime.h>

#include "../internal.h"
#include "scheme_math.cuh"

namespace hydro {

namespace {

constexpr int kBX = 32, kBY = 4;
#define DV __device__ __forceinline__

// node coordinates of the Cartesian mesh (CartesianMesh2DGenerator.cc:52-54)
DV double xs(const RunView& v, long long j) { return v.dx * (double)j; }
DV double ys(const RunView& v, long long i) { return v.dy * (double)i; }

DV double cross2(const double* a, const double* b) { return a[0] * b[1] - a[1] * b[0]; }


// block-wide min of ordered encodings into *dst, one atomic per block
DV void block_min_into(unsigned long long x, unsigned long long* dst) {
  __shared__ unsigned long long s[32];
  const int tid = threadIdx.y * blockDim.x + threadIdx.x;
  const int lane = tid & 31, warp = tid >> 5;
  const int nw = (blockDim.x * blockDim.y + 31) >> 5;
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long a = __shfl_xor_sync(0xffffffffu, x, o);
    x = a < x ? a : x;
  }
  if (lane == 0) s[warp] = x;
  __syncthreads();
  if (warp == 0) {
    x = lane < nw ? s[lane] : ~0ull;
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long a = __shfl_xor_sync(0xffffffffu, x, o);
      x = a < x ? a : x;
    }
    if (lane == 0 && x != ~0ull) atomicMin(dst, x);
  }
}

// the cell's four nodes in the reference's order (bottom-left, bottom-right,
// top-right, top-left), as coordinates
DV void cell_nodes(const RunView& v, long long i, long long j, double X[4][2]) {
  X[0][0] = xs(v, j);     X[0][1] = ys(v, i);
  X[1][0] = xs(v, j + 1); X[1][1] = ys(v, i);
  X[2][0] = xs(v, j + 1); X[2][1] = ys(v, i + 1);
  X[3][0] = xs(v, j);     X[3][1] = ys(v, i + 1);
}

// centre coordinate (initCellPos, vnr_remap/Init.cc:495-511) of row i
// (along y) or column j (along x): 0.25 * (((0 + a) + a) + b) + b) in node
// order
DV double centre_y(const RunView& v, long long i) {
  double r = 0.0;
  r = r + ys(v, i);
  r = r + ys(v, i);
  r = r + ys(v, i + 1);
  r = r + ys(v, i + 1);
  return 0.25 * r;
}
DV double centre_x(const RunView& v, long long j) {
  double r = 0.0;
  r = r + xs(v, j);
  r = r + xs(v, j + 1);
  r = r + xs(v, j + 1);
  r = r + xs(v, j);
  return 0.25 * r;
}

// ------------------------------------------------------------------- VNR
__global__ void __launch_bounds__(kBX* kBY) kd_init_cells_vnr(RunView v, int t, int variant) {
  const long long j = blockIdx.x * kBX + threadIdx.x;
  const long long i = blockIdx.y * kBY + threadIdx.y;
  unsigned long long dtb = ~0ull;
  if (i < v.ny && j < v.nx) {
    const long long c = i * v.nx + j, P = v.pitch;
    const int nb = v.nbmat;
    double X[4][2];
    cell_nodes(v, i, j, X);
    const double Xc[2] = {centre_x(v, j), centre_y(v, i)};
    const double g = v.gamma_scalar;
    double rho = 0., p = 0., snd = 0., e = 0.;
    double fm[3] = {0., 0., 0.}, mfm[3] = {0., 0., 0.}, rhom[3] = {0., 0., 0.},
           pm[3] = {0., 0., 0.}, cm[3] = {0., 0., 0.}, em[3] = {0., 0., 0.};
    if (t == 4 || t == 5) {  // Sod (Init.cc:103-143)
      const double r = (t == 4) ? Xc[0] : Xc[1];
      fm[0] = 1.;
      mfm[0] = 1.;
      if (r < 0.5) {
        rho = 1.0; p = 1.0; rhom[0] = 1.0; pm[0] = 1.0;
      } else {
        rho = 0.125; p = 0.1; rhom[0] = 0.125; pm[0] = 0.1;
      }
      cm[0] = sqrt(g * rhom[0] / pm[0]);
      snd = cm[0];
    } else if (t == 15 || t == 16) {  // bi-material Sod (Init.cc:144-183)
      const double r = (t == 15) ? Xc[0] : Xc[1];
      if (r < 0.5) {
        fm[0] = 1.; mfm[0] = 1.;
        rho = 1.0; p = 1.0; rhom[0] = 1.0; pm[0] = 1.0;
      } else {
        fm[1] = 1.; mfm[1] = 1.;
        rho = 0.125; p = 0.1; rhom[1] = 0.125; pm[1] = 0.1;
      }
      cm[0] = sqrt(g * rhom[0] / pm[0]);
      cm[1] = sqrt(g * rhom[1] / pm[1]);
      snd = smin(cm[0], cm[1]);
      if (variant == 1) {
        // extension: the first cell line whose centre is not below 0.5 is a
        // 50/50 mix (centres grow with the line index, so that line is the
        // one whose predecessor is below 0.5)
        const bool ycase = (t == 16);
        const long long k = ycase ? i : j;
        const double rk = ycase ? centre_y(v, k) : centre_x(v, k);
        const bool first = !(rk < 0.5) &&
                           (k == 0 || (ycase ? centre_y(v, k - 1) : centre_x(v, k - 1)) < 0.5);
        if (first) {
          const double f0 = 0.5, f1 = 0.5, r0 = 1.0, r1 = 0.125, p0 = 1.0, p1 = 0.1;
          const double m0 = f0 * r0, m1 = f1 * r1;
          fm[0] = f0; fm[1] = f1;
          mfm[0] = m0 / (m0 + m1);
          mfm[1] = m1 / (m0 + m1);
          rhom[0] = r0; rhom[1] = r1;
          pm[0] = p0; pm[1] = p1;
          rho = f0 * r0 + f1 * r1;
          p = f0 * p0 + f1 * p1;
          cm[0] = sqrt(g * r0 / p0);
          cm[1] = sqrt(g * r1 / p1);
          snd = smin(cm[0], cm[1]);
        }
      }
    } else if (t == 1) {
      // Sedov (extension, after eucclhyd_remap/Init.cc:303-332): the energy
      // deposited in the cell touching the origin, written as its pressure
      const double e1 = 1.e-6 / ((v.gamma[0] - 1.0) * 1.0);
      bool centre = false;
      for (int k = 0; k < 4; ++k)
        if (norm2(X[k][0], X[k][1]) < v.threshold) centre = true;
      const double ee = centre ? e1 + 0.244816 / (v.dx * v.dy) : e1;
      fm[0] = 1.; mfm[0] = 1.;
      rho = 1.0; rhom[0] = 1.0;
      p = (v.gamma[0] - 1.0) * 1.0 * ee;
      pm[0] = p;
      cm[0] = sqrt(g * rhom[0] / pm[0]);
      snd = cm[0];
    } else if (t == 0 || t == 11) {
      // unit tests (Init.cc:331-361): density 1 left of x = 0.4, 0.1 right
      // of it (a cell centred on 0.4 keeps 0), pressure 1, sound speed
      // sqrt(gamma), material 1 in every cell
      fm[0] = 1.; mfm[0] = 1.;
      p = 1.0; pm[0] = 1.0; pm[1] = 0.0;
      snd = sqrt(g); cm[0] = sqrt(g); cm[1] = sqrt(g);
      const double r = Xc[0];
      if (r < 0.4) {
        rho = 1.; rhom[0] = 1.;
      } else if (r > 0.4) {
        rho = 0.1; rhom[0] = 0.1;
      }
      if (r > 0.6) {
        rho = 0.1; rhom[0] = 0.1;
      }
    } else if (t == 18 && variant == 2) {
      // advection step (extension): rho 1 | 0.1 at x = 0.5, two materials
      const int m = (Xc[0] < 0.5) ? 0 : 1;
      const double d = (m == 0) ? 1.0 : 0.1;
      fm[m] = 1.; mfm[m] = 1.;
      rho = d; p = 0.0; rhom[m] = d; pm[m] = 0.0;
      cm[0] = 1.; cm[1] = 1.;
      snd = smin(cm[0], cm[1]);
      em[0] = 1.; em[1] = 1.;
      e = 1.;
    } else {  // advection cases 7, 8, 18-21 (Init.cc:185-372)
      const bool isx = (t == 7 || t == 18 || t == 20);
      const bool bi = (t >= 18);
      const bool vit = (t == 20 || t == 21);
      const double r = isx ? Xc[0] : Xc[1];
      const double dens_out = vit ? 4.0 : 1.0;
      if (r < 0.3) {
        fm[0] = 1.; mfm[0] = 1.;
        rho = dens_out; p = 0.0; rhom[0] = dens_out; pm[0] = 0.0;
      } else if ((r > 0.3) && (r < 0.5)) {
        if (!bi) {
          fm[0] = 1.; mfm[0] = 1.;
          rho = 10.; p = 0.0; rhom[0] = 10.0; pm[0] = 0.0;
        } else {
          fm[1] = 1.; mfm[1] = 1.;
          rho = vit ? 4. : 1.; p = 0.0; rhom[1] = 1.0; pm[1] = 0.0;
        }
      } else if (r > 0.5) {
        fm[0] = 1.; mfm[0] = 1.;
        rho = dens_out; p = 0.0; rhom[0] = dens_out; pm[0] = 0.0;
      }
      cm[0] = 1.; cm[1] = 1.;
      snd = smin(cm[0], cm[1]);
      em[0] = 1.; em[1] = 1.;
      e = 1.;
    }
    // mixed-cell indicator (Init.cc:373-393)
    int matcell = 0, imatpure = -1;
    for (int m = 0; m < 3; ++m)
      if (fm[m] > v.threshold) {
        matcell++;
        imatpure = m;
      }
    v.mixte[c] = matcell > 1 ? 1 : 0;
    v.pure[c] = matcell > 1 ? -1 : imatpure;

    // sub-volumes (initSubVol, Init.cc:400-429) and their sums
    double s0 = 0.0;
    for (int k = 0; k < 4; ++k) {
      const double* xm = X[(k + 3) % 4];
      const double* xk = X[k];
      const double* xp = X[(k + 1) % 4];
      const double x2[2] = {0.5 * (xm[0] + xk[0]), 0.5 * (xm[1] + xk[1])};
      const double x4[2] = {0.5 * (xp[0] + xk[0]), 0.5 * (xp[1] + xk[1])};
      const double vpc =
          0.5 * (cross2(Xc, x2) + cross2(x2, xk) + cross2(xk, x4) + cross2(x4, Xc));
      s0 = s0 + vpc;
    }
    const double sq = sqrt(s0);
    const double cfl = (v.projection == 1) ? 0.05 : 0.1;
    // without the remap the Lagrange kernel takes the cell's volume of the
    // cycle's start from vL (the sum of its current sub-volumes)
    if (v.projection == 0) v.vL[c] = s0;
    const_cast<double*>(v.s0)[c] = s0;
    const_cast<double*>(v.sqs0)[c] = sq;
    const_cast<double*>(v.cflsq)[c] = cfl * sq;
    // corner normals of the Euler mesh (PhaseLagrange.cc:114-136)
    for (int k = 0; k < 4; ++k) {
      double o[2];
      lpc_npc(X[k], X[(k + 1) % 4], X[(k + 3) % 4], o);
      const_cast<double*>(v.cqs)[(2 * k) * P + c] = o[0];
      const_cast<double*>(v.cqs)[(2 * k + 1) * P + c] = o[1];
    }
    // outer face normals along each face's sweep axis (Init.cc:517-554):
    // planes L.x (nodes 0-3), R.x (1-2), B.y (0-1), T.y (3-2)
    const int ends[4][2] = {{0, 3}, {1, 2}, {0, 1}, {3, 2}};
    for (int q = 0; q < 4; ++q) {
      const double* a = X[ends[q][0]];
      const double* b = X[ends[q][1]];
      const double d0 = 0.5 * (a[0] + b[0]) - Xc[0], d1 = 0.5 * (a[1] + b[1]) - Xc[1];
      const double nr = norm2(d0, d1);
      const double n = (q < 2 ? d0 : d1) / nr;
      const_cast<double*>(v.nout)[q * P + c] = n;
      if (ubits(n) != ubits((q & 1) ? 1.0 : -1.0)) atomicOr(&v.ctrl->nout_general, 1);
    }
    // the Lagrangian geometry of the cell at rest, by the Lagrange kernel's
    // own function from the Euler coordinates its nodes keep then
    {
      const CellGeom Gr = vnr_cell_geometry(X, v.order > 1);
      double* g0 = const_cast<double*>(v.geo0);
      g0[c] = Gr.vol;
      g0[P + c] = Gr.xc0;
      g0[2 * P + c] = Gr.xc1;
      g0[3 * P + c] = Gr.hx;
      g0[4 * P + c] = Gr.hy;
    }
    v.sarg[c] = from_bits(kNoRoot);  // the initial sound speed is not a root of e
    // cell masses (computeCellMass, PhaseLagrange.cc:14-24)
    const double cmass = v.dx * v.dy * rho;
    if (v.sans_lagrange == 0) {
      // initDeltaT's minimum (Init.cc:435-457) and initInternalEnergy
      // (Init.cc:463-472)
      const double d = 0.1 * sq / snd;
      if (!is_nan(d)) dtb = ord_bits(d);
      for (int m = 0; m < 3; ++m) em[m] = pm[m] / ((v.gamma[m] - 1.0) * rhom[m]);
      e = p / ((v.gamma_scalar - 1.0) * rho);
    }
    v.rho[c] = rho;
    v.p[c] = p;
    v.c[c] = snd;
    v.e[c] = e;
    v.cell_mass[c] = cmass;
    for (int m = 0; m < nb; ++m) {
      v.fm[m * P + c] = fm[m];
      v.mfm[m * P + c] = mfm[m];
      v.rhom[m * P + c] = rhom[m];
      v.pm[m * P + c] = pm[m];
      v.cm[m * P + c] = cm[m];
      v.em[m * P + c] = em[m];
      v.cmassm[m * P + c] = mfm[m] * cmass;
    }
  }
  block_min_into(dtb, &v.ctrl->dt_min_bits);
}

__global__ void __launch_bounds__(kBX* kBY) kd_init_nodes_vnr(RunView v, int t, int variant) {
  const long long j = blockIdx.x * kBX + threadIdx.x;
  const long long i = blockIdx.y * kBY + threadIdx.y;
  if (i > v.ny || j > v.nx) return;
  const long long pn = i * (v.nx + 1) + j;
  const double x0 = xs(v, j), x1 = ys(v, i);
  if (v.XN) {  // a run without the remap starts from the generated mesh
    v.XN[pn] = x0;
    v.XN[v.npitch + pn] = x1;
  }
  double u = 0.0, w = 0.0;
  if ((t == 18 && variant == 2) || t == 0 || t == 11) {
    u = 1.0;  // the advection step extension; the unit tests (Init.cc:362-370)
  } else if (t == 7 || t == 8 || t == 18 || t == 19 || t == 20 || t == 21) {
    const bool isx = (t == 7 || t == 18 || t == 20);
    const bool vit = (t == 20 || t == 21);
    const double u0 = isx ? 1.0 : 0.0, u1 = isx ? 0.0 : 1.0;
    if (vit) {
      const double r = isx ? x0 : x1;
      if (r <= 0.3) {
        u = 0.2 * u0; w = 0.2 * u1;
      } else if ((r > 0.3) && (r <= 0.5)) {
        const double sc = 4. * r - 1.;
        u = sc * u0; w = sc * u1;
      } else if (r > 0.5) {
        u = u0; w = u1;
      }
    } else {
      u = u0;
      w = u1;
    }
  }
  v.u[pn] = u;
  v.u[v.npitch + pn] = w;
  if (v.vout) {
    v.vout[pn] = u;
    v.vout[v.npitch + pn] = w;
  }
  // exact cancellation of the interior force sum (updateVelocity,
  // PhaseLagrange.cc:167-197): with one pressure w in the four cells the sum
  // is ((w C_0 + w C_1) + w C_2) + w C_3 per component, the first addition
  // from 0.0.  It is +0 for any |w| < 2^500 when C_1 = -C_0 and C_3 = -C_2,
  // or when C_1 = C_0 and C_2 = C_3 = -C_0 (bit for bit, |C| < 2^500):
  // w(-c) = -(wc), x + (-x) = +0, 2x - x = x, all exact.
  {
    unsigned char sym = 0;
    if (i > 0 && i < v.ny && j > 0 && j < v.nx) {
      const long long P = v.pitch;
      const long long cl[4] = {i * v.nx + j, i * v.nx + j - 1, (i - 1) * v.nx + j,
                               (i - 1) * v.nx + j - 1};
      const int loc[4] = {0, 1, 3, 2};
      constexpr unsigned long long kS = 0x8000000000000000ull, kMod = 1523ull << 52;
      bool ok = true;
      for (int comp = 0; comp < 2; ++comp) {
        unsigned long long b[4];
        for (int t = 0; t < 4; ++t) {
          b[t] = ubits(v.cqs[(2 * loc[t] + comp) * P + cl[t]]);
          ok = ok && (b[t] & kMag) < kMod;
        }
        const bool pa = b[1] == (b[0] ^ kS) && b[3] == (b[2] ^ kS);
        const bool pb = b[1] == b[0] && b[2] == (b[0] ^ kS) && b[3] == b[2];
        ok = ok && (pa || pb);
      }
      sym = ok ? 1 : 0;
    }
    const_cast<unsigned char*>(v.nsym)[pn] = sym;
  }
  // node masses (computeNodeMass, PhaseLagrange.cc:31-48)
  double r = 0.0;
  int k = 0;
  const long long nx = v.nx;
  if (i < v.ny && j < nx) { r = r + v.cell_mass[i * nx + j]; ++k; }
  if (i < v.ny && j > 0) { r = r + v.cell_mass[i * nx + j - 1]; ++k; }
  if (i > 0 && j < nx) { r = r + v.cell_mass[(i - 1) * nx + j]; ++k; }
  if (i > 0 && j > 0) { r = r + v.cell_mass[(i - 1) * nx + j - 1]; ++k; }
  v.node_mass[pn] = r / (double)k;
  // per-row / per-column arrays: node coordinates, Euler face lengths and
  // the periodic rebuild source (ConditionsLimites.cc:186-209)
  if (i == 0) {
    const_cast<double*>(v.xs)[j] = x0;
    if (j < nx) const_cast<double*>(v.flh)[j] = norm2(xs(v, j + 1) - x0, 0.0);
  }
  if (j == 0) {
    const_cast<double*>(v.ys)[i] = x1;
    if (i < v.ny) {
      const_cast<double*>(v.flv)[i] = norm2(0.0, ys(v, i + 1) - x1);
      const_cast<double*>(v.rho0_left)[i] = v.rho[i * nx];
    }
  }
}

// dt_n = initDeltaT's minimum * 1e-6 (Init.cc:455), then the dt reduction
// slot is made ready for the first cycle's prologue
__global__ void kd_init_finish_vnr(RunView v) {
  Ctrl& C = *v.ctrl;
  if (v.sans_lagrange == 0) C.dt_n = from_ord(C.dt_min_bits) * 1.0E-6;
  C.dt_min_bits = ord_bits(1.7976931348623157e308);
}

// -------------------------------------------------------------- Eucclhyd
DV double dot2(const double* a, const double* b) {
  double r = 0.0;
  r += a[0] * b[0];
  r += a[1] * b[1];
  return r;
}
DV double nrm(const double* a) { return sqrt(dot2(a, a)); }

__global__ void __launch_bounds__(kBX* kBY) kd_init_cells_euc(RunView v, int t, int variant) {
  const long long j = blockIdx.x * kBX + threadIdx.x;
  const long long i = blockIdx.y * kBY + threadIdx.y;
  if (i >= v.ny || j >= v.nx) return;
  const long long c = i * v.nx + j, P = v.pitch;
  const int nb = v.nbmat;
  double X[4][2];
  cell_nodes(v, i, j, X);
  // computeCornerNormal (PhaseLagrange.cc:27-66): l_pc n_pc and the corner
  // matrix l+ n+ (x) n+ + l- n- (x) n- (PhaseLagrange.cc:281-287)
  double* lpc = const_cast<double*>(v.lpc);
  double* cmat = const_cast<double*>(v.cmat);
  for (int k = 0; k < 4; ++k) {
    const double* xp = X[k];
    const double* xpp = X[(k + 1) % 4];
    const double* xpm = X[(k + 3) % 4];
    double np[2] = {0.5 * (xpp[1] - xp[1]), 0.5 * (xp[0] - xpp[0])};
    const double lp = nrm(np);
    np[0] = np[0] / lp;
    np[1] = np[1] / lp;
    double nm[2] = {0.5 * (xp[1] - xpm[1]), 0.5 * (xpm[0] - xp[0])};
    const double lm = nrm(nm);
    nm[0] = nm[0] / lm;
    nm[1] = nm[1] / lm;
    lpc[(2 * k) * P + c] = np[0] * lp + nm[0] * lm;
    lpc[(2 * k + 1) * P + c] = np[1] * lp + nm[1] * lm;
    cmat[(3 * k) * P + c] = (np[0] * np[0]) * lp + (nm[0] * nm[0]) * lm;
    cmat[(3 * k + 1) * P + c] = (np[0] * np[1]) * lp + (nm[0] * nm[1]) * lm;
    cmat[(3 * k + 2) * P + c] = (np[1] * np[1]) * lp + (nm[1] * nm[1]) * lm;
  }
  // initMeshGeometryForCells (Init.cc:106-166): volume, centroid, perimeter
  double r11 = 0.0;
  for (int k = 0; k < 4; ++k) r11 = r11 + cross2(X[k], X[(k + 1) % 4]);
  const double vol = 0.5 * r11;
  double r12[2] = {0.0, 0.0};
  for (int k = 0; k < 4; ++k) {
    const double* a = X[k];
    const double* b = X[(k + 1) % 4];
    const double cr = cross2(a, b);
    r12[0] = r12[0] + (a[0] + b[0]) * cr;
    r12[1] = r12[1] + (a[1] + b[1]) * cr;
  }
  const double sc = 1.0 / (6.0 * vol);
  const double x0 = r12[0] * sc, x1 = r12[1] * sc;
  const_cast<double*>(v.xcc)[c] = x0;
  const_cast<double*>(v.xcc)[P + c] = x1;
  const_cast<double*>(v.evol)[c] = vol;
  double r13 = 0.0;
  for (int k = 0; k < 4; ++k) {
    const double d[2] = {X[k][0] - X[(k + 1) % 4][0], X[k][1] - X[(k + 1) % 4][1]};
    r13 = r13 + nrm(d);
  }
  const_cast<double*>(v.perim)[c] = r13;
  // the Lagrangian geometry of the cell at rest, by the Lagrange kernel's
  // own function from the Euler coordinates its nodes keep then
  {
    const CellGeom Gr = euc_cell_geometry(X, v.order > 1);
    double* g0 = const_cast<double*>(v.geo0);
    g0[c] = Gr.vol;
    g0[P + c] = Gr.xc0;
    g0[2 * P + c] = Gr.xc1;
    g0[3 * P + c] = Gr.hx;
    g0[4 * P + c] = Gr.hy;
  }
  // initCellInternalEnergy, initCellVelocity, initDensity (Init.cc
  // :194-675); init_variant 3 of BiTriplePoint scales the regions to a 7 x 3
  // domain and gives material 3 density 0.125
  const bool scaled = (t == 13 && variant == 3);
  const double xlim = scaled ? 1.0 : 0.01, ylim = scaled ? 1.5 : 0.015;
  const double rho3 = scaled ? 0.125 : 0.1;
  const double* g = v.gamma;
  double rho = 0., e = 0.;
  double fm[3] = {0., 0., 0.}, mfm[3] = {0., 0., 0.}, rhom[3] = {0., 0., 0.},
         em[3] = {0., 0., 0.};
  if (t == 4 || t == 5) {
    const double r = (t == 4) ? x0 : x1;
    double p, d;
    if (r <= 0.5) { p = 1.0; d = 1.0; } else { p = 0.1; d = 0.125; }
    e = p / ((g[0] - 1.0) * d);
    em[0] = e;
    fm[0] = 1.; mfm[0] = 1.;
    rho = d;
    rhom[0] = d;
    rhom[1] = d;
  } else if (t == 15 || t == 16) {
    const double r = (t == 15) ? x0 : x1;
    if (r <= 0.5) {
      e = 1.0 / ((g[0] - 1.0) * 1.0);
      em[0] = e;
      fm[0] = 1.; mfm[0] = 1.;
      rho = 1.0;
      rhom[0] = 1.0;
    } else {
      e = 0.1 / ((g[1] - 1.0) * 0.125);
      em[1] = e;
      fm[1] = 1.; mfm[1] = 1.;
      rho = 0.125;
      rhom[1] = 0.125;
    }
  } else if (t == 2) {
    double p, d;
    if (x0 <= 0.01) { p = 1.0; d = 1.0; }
    else if (x1 <= 0.015) { p = 0.1; d = 1.; }
    else { p = 0.1; d = 0.1; }
    e = p / ((g[0] - 1.0) * d);
    em[0] = e;
    fm[0] = 1.; mfm[0] = 1.;
    rho = (x0 <= 0.01) ? 1.0 : ((x1 <= 0.015) ? 1.0 : 0.1);
  } else if (t == 13) {
    int m;
    double d, p;
    if (x0 <= xlim) { m = 0; d = 1.0; p = 1.0; }
    else if (x1 <= ylim) { m = 1; d = 1.0; p = 0.1; }
    else { m = 2; d = rho3; p = 0.1; }
    e = p / ((g[m] - 1.0) * d);
    em[m] = e;
    rho = d;
    fm[m] = 1.; mfm[m] = 1.;
    rhom[m] = d;
  } else if (t == 14) {
    // BiShockBubble (Init.cc:272-302, 411-415, 528-560): air everywhere,
    // the bubble (centre (0.320, 0.04), radius 0.025) overrides it; both
    // energies with the first material's exponent, as the reference writes
    e = 1.e5 / ((g[0] - 1.0) * 1.0);
    em[0] = e;
    rho = 1.0;
    rhom[0] = 1.0;
    fm[0] = 1.; mfm[0] = 1.;
    const double r = sqrt((x0 - 0.320) * (x0 - 0.320) + (x1 - 0.04) * (x1 - 0.04));
    if (r <= 0.025) {
      e = 1.e5 / ((g[0] - 1.0) * 0.182);
      em[0] = 0.;
      em[1] = e;
      rhom[0] = 0.0;
      rhom[1] = 0.182;
      rho = 0.182;
      fm[0] = 0.; fm[1] = 1.;
      mfm[0] = 0.; mfm[1] = 1.;
    }
    if (x0 >= 0.60) {
      v.uc[c] = -124.824;
      v.uco[c] = -124.824;
    }
  } else if (t == 6 || t == 17 || t == 0 || t == 11) {
    // Noh, unit tests (Init.cc:202-214): e0 = p0 / ((1.4 - 1) rho0) with
    // p0 = rho0 = 1, for the cell and every material
    const double e0 = 1. / ((1.4 - 1.0) * 1.);
    e = e0;
    em[0] = em[1] = em[2] = e0;
    if (t == 6 || t == 17) {
      // initCellVelocity (Init.cc:394-401): -u0 * n / |n| with u0 = 0 (a
      // signed zero); no density initialisation (zero density)
      const double u0 = 0.;
      const double nv = sqrt(x0 * x0 + x1 * x1);
      v.uc[c] = -u0 * x0 / nv;
      v.uc[P + c] = -u0 * x1 / nv;
      v.uco[c] = v.uc[c];
      v.uco[P + c] = v.uc[P + c];
    } else {
      // velocity (1, 0) (Init.cc:416-419); density 1, material 1 left of
      // x = 0.5 and (bi-material) material 2 right of it (Init.cc:438-480)
      v.uc[c] = 1.0;
      v.uc[P + c] = 0.0;
      v.uco[c] = 1.0;
      v.uco[P + c] = 0.0;
      rho = 1.0;
      const int m = (t == 11 && !(x0 <= 0.5)) ? 1 : 0;
      fm[m] = 1.; mfm[m] = 1.;
      rhom[m] = 1.0;
    }
  } else {  // Sedov (test case 1; 12 has no density initialisation)
    const double e1 = 1.e-6 / ((g[0] - 1.0) * 1.);
    bool centre = false;
    for (int k = 0; k < 4; ++k)
      if (nrm(X[k]) < v.threshold) centre = true;
    e = centre ? e1 + 0.244816 / (v.dx * v.dy) : e1;
    em[0] = e;
    if (t == 1) {
      rho = 1.0;
      rhom[0] = 1.0;
    }
  }
  if (nb == 1) {
    fm[0] = 1.; fm[1] = 0.; fm[2] = 0.;
    mfm[0] = 1.; mfm[1] = 0.; mfm[2] = 0.;
  }
  int matcell = 0, imatpure = -1;
  for (int m = 0; m < 3; ++m)
    if (fm[m] > v.threshold) {
      matcell++;
      imatpure = m;
    }
  v.mixte[c] = matcell > 1 ? 1 : 0;
  v.pure[c] = matcell > 1 ? -1 : imatpure;
  // initMeshGeometryForFaces (Init.cc:677-716): outer normals along each
  // face's sweep axis from the centroid; planes L.x, R.x, B.y, T.y
  const int ends[4][2] = {{0, 3}, {1, 2}, {0, 1}, {3, 2}};
  for (int q = 0; q < 4; ++q) {
    const double* a = X[ends[q][0]];
    const double* b = X[ends[q][1]];
    const double d[2] = {0.5 * (a[0] + b[0]) - x0, 0.5 * (a[1] + b[1]) - x1};
    const double n = (q < 2 ? d[0] : d[1]) / nrm(d);
    const_cast<double*>(v.nout)[q * P + c] = n;
    if (ubits(n) != ubits((q & 1) ? 1.0 : -1.0)) atomicOr(&v.ctrl->nout_general, 1);
  }
  v.rho[c] = rho;
  v.e[c] = e;
  for (int m = 0; m < nb; ++m) {
    v.fm[m * P + c] = fm[m];
    v.mfm[m * P + c] = mfm[m];
    v.rhom[m * P + c] = rhom[m];
    v.em[m * P + c] = em[m];
  }
}

__global__ void kd_init_rows_euc(RunView v) {
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k <= v.nx) {
    const_cast<double*>(v.xs)[k] = xs(v, k);
    if (k < v.nx) {
      const double d[2] = {xs(v, k + 1) - xs(v, k), 0.0};
      const_cast<double*>(v.flh)[k] = nrm(d);
    }
  }
  if (k <= v.ny) {
    const_cast<double*>(v.ys)[k] = ys(v, k);
    if (k < v.ny) {
      const double d[2] = {0.0, ys(v, k + 1) - ys(v, k)};
      const_cast<double*>(v.flv)[k] = nrm(d);
    }
  }
}

}  // namespace

// Order-3 coefficients of the mesh at rest: eval_grad's and eval_ystar's
// coefficients depend on the cell widths along the sweep only; with the
// widths of the cells at rest (the stored rest geometry) they are formed here
// once, by the functions the order-3 kernels use, for both sweep axes.
__global__ void __launch_bounds__(kBX* kBY) kd_init_o3c(RunView v) {
  const long long j = blockIdx.x * kBX + threadIdx.x;
  const long long i = blockIdx.y * kBY + threadIdx.y;
  if (i >= v.ny || j >= v.nx) return;
  const long long c = i * v.nx + j, P = v.pitch;
  double* o = const_cast<double*>(v.o3c);
  for (int ax = 0; ax < 2; ++ax) {
    const double* Hr = v.geo0 + (3 + ax) * P;
    const int q = ax == 0 ? (int)j : (int)i, n = ax == 0 ? v.nx : v.ny;
    const long long st = ax == 0 ? 1 : v.nx;
    double* oa = o + 8 * ax * P;
    {
      const long long cm = q > 0 ? c - st : c, cp = q < n - 1 ? c + st : c;
      double G0, A, B;
      o3_grad_coef(Hr[cm], Hr[c], Hr[cp], G0, A, B);
      oa[c] = G0;
      oa[P + c] = A;
      oa[2 * P + c] = B;
    }
    if (q >= 1) {
      const long long cm = c - st, cmm = q > 1 ? cm - st : cm, cpp = q < n - 1 ? c + st : c;
      double T[5];
      o3_ystar_coef(Hr[cmm], Hr[cm], Hr[c], Hr[cpp], T);
      for (int t = 0; t < 5; ++t) oa[(3 + t) * P + c] = T[t];
    }
  }
}

// Queues the device initialisation of a run whose arena is zeroed and whose
// control block holds the ordered encoding of +DBL_MAX in dt_min_bits.
// Returns the number of kernels.
int launch_device_init(const RunView& v, int test_case, int init_variant, cudaStream_t s) {
  const dim3 blk(kBX, kBY);
  const dim3 cg((v.nx + kBX - 1) / kBX, (v.ny + kBY - 1) / kBY);
  const dim3 ng((v.nx + 1 + kBX - 1) / kBX, (v.ny + 1 + kBY - 1) / kBY);
  if (v.scheme == HYDRO_SCHEME_EUCCLHYD) {
    kd_init_cells_euc<<<cg, blk, 0, s>>>(v, test_case, init_variant);
    const int n = (v.nx > v.ny ? v.nx : v.ny) + 1;
    kd_init_rows_euc<<<(n + 127) / 128, 128, 0, s>>>(v);
    if (v.o3c) kd_init_o3c<<<cg, blk, 0, s>>>(v);
    return v.o3c ? 3 : 2;
  }
  kd_init_cells_vnr<<<cg, blk, 0, s>>>(v, test_case, init_variant);
  kd_init_nodes_vnr<<<ng, blk, 0, s>>>(v, test_case, init_variant);
  kd_init_finish_vnr<<<1, 1, 0, s>>>(v);
  if (v.o3c) kd_init_o3c<<<cg, blk, 0, s>>>(v);
  return v.o3c ? 4 : 3;
}

}  // namespace hydro
