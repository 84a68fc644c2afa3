// Host-side initial state of a VNR run and its constant Euler geometry.
//
// Restates the set-up sequence of Vnr::simulate (vnr_remap/VnrRemap.cc
// :330-341): initBoundaryConditions, initCellPos, init, initSubVol,
// initMeshGeometryForFaces, computeCellMass, initDeltaT, initInternalEnergy,
// initPseudo, computeNodeMass (vnr_remap/Init.cc, PhaseLagrange.cc:14-48).
// Arithmetic follows the reference operation by operation; this file must be
// compiled without floating-point contraction (-ffp-contract=off) so that
// aarch64 hosts do not fuse multiply-adds.
//
// Only quantities the GPU path consumes are produced: the Euler-constant
// geometry the kernels would otherwise recompute every cycle (corner
// normals, sub-volume sums, outer face normals, face lengths) is computed
// once here.
#include "init.h"

#include <cmath>
#include <cstring>

#include "../internal.h"

namespace hydro {
namespace {

inline double smin(double a, double b) { return (b < a) ? b : a; }  // std::min
inline double smax(double a, double b) { return (a < b) ? b : a; }  // std::max

// sqrt(dot(v, v)) with dot accumulated from 0.0 (includes/Freefunctions.h)
inline double norm2(double a, double b) {
  double r = 0.0;
  r = r + a * a;
  r = r + b * b;
  return std::sqrt(r);
}
inline double cross2(const double* a, const double* b) {
  return a[0] * b[1] - a[1] * b[0];
}

struct Mesh {
  long long nx, ny;
  long long nid(long long i, long long j) const { return i * (nx + 1) + j; }
  void nodes(long long c, long long nd[4]) const {
    long long i = c / nx, j = c - i * nx;
    long long n0 = nid(i, j);
    nd[0] = n0;
    nd[1] = n0 + 1;
    nd[2] = n0 + nx + 2;
    nd[3] = n0 + nx + 1;
  }
};

// includes/Freefunctions.h:28-58 (computeLpcNpc)
void lpc_npc(const double* xp, const double* xpp, const double* xpm,
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

int init_bc(const hydro_spec& s, HostInit& h) {
  const int t = s.test_case;
  if (t == 4 || t == 15 || t == 5 || t == 16) {
    // Sod / BiSod (vnr_remap/Init.cc:10-37): walls
    h.bc_left = h.bc_right = h.bc_top = h.bc_bottom = kBcSym;
  } else if (t == 1) {
    // Sedov (extension for VNR): the boundary conditions of the Eucclhyd
    // Sedov case (eucclhyd_remap/Init.cc:47-64): symmetry on the left and
    // bottom, zero imposed velocity on the right and top
    h.bc_left = kBcSym;
    h.bc_bottom = kBcSym;
    h.bc_right = kBcImposed;
    h.v_right[0] = 0.0;
    h.v_right[1] = 0.0;
    h.bc_top = kBcImposed;
    h.v_top[0] = 0.0;
    h.v_top[1] = 0.0;
  } else if (t == 7 || t == 18 || t == 9 || t == 20) {
    // Advection X (Init.cc:38-50)
    h.bc_right = kBcImposed;
    h.v_right[0] = 1.0;
    h.v_right[1] = 0.0;
    h.periodic_x = 1;
    h.bc_left = kBcImposed;
    h.v_left[0] = 1.0;
    h.v_left[1] = 0.0;
    h.bc_top = kBcSym;
    h.bc_bottom = kBcSym;
  } else if (t == 8 || t == 19) {
    // Advection Y (Init.cc:51-64)
    h.bc_bottom = kBcImposed;
    h.v_bottom[0] = 0.0;
    h.v_bottom[1] = 1.0;
    h.bc_top = kBcImposed;
    h.v_top[0] = 0.0;
    h.v_top[1] = 1.0;
    h.bc_left = kBcSym;
    h.bc_right = kBcSym;
  } else {
    return fail(-10, "VNR initialisation: test case " + std::to_string(t) +
                         " is not a VNR test case");
  }
  return 0;
}

}  // namespace

int build_initial_state(const hydro_spec& s, HostInit& h) {
  if (s.scheme != HYDRO_SCHEME_VNR)
    return fail(-11, "only the VNR scheme is built on the GPU path so far");
  if (s.nx < 2 || s.ny < 2) return fail(-12, "nx and ny must be >= 2");
  const long long nx = s.nx, ny = s.ny, nc = nx * ny, nn = (nx + 1) * (ny + 1);
  h.nx = nx;
  h.ny = ny;
  h.nc = nc;
  h.nn = nn;
  Mesh M{nx, ny};
  if (int rc = init_bc(s, h)) return rc;

  // node coordinates (CartesianMesh2DGenerator.cc:52-54)
  h.xs.resize(nx + 1);
  h.ys.resize(ny + 1);
  for (long long j = 0; j <= nx; ++j) h.xs[j] = s.dx * (double)j;
  for (long long i = 0; i <= ny; ++i) h.ys[i] = s.dy * (double)i;
  std::vector<double> X(2 * nn);
  for (long long i = 0; i <= ny; ++i)
    for (long long j = 0; j <= nx; ++j) {
      X[2 * M.nid(i, j)] = h.xs[j];
      X[2 * M.nid(i, j) + 1] = h.ys[i];
    }
  // cell centres (initCellPos, Init.cc:495-511)
  std::vector<double> Xc(2 * nc);
  for (long long c = 0; c < nc; ++c) {
    long long nd[4];
    M.nodes(c, nd);
    double r0 = 0.0, r1 = 0.0;
    for (int k = 0; k < 4; ++k) {
      r0 = r0 + X[2 * nd[k]];
      r1 = r1 + X[2 * nd[k] + 1];
    }
    Xc[2 * c] = 0.25 * r0;
    Xc[2 * c + 1] = 0.25 * r1;
  }

  // ---- state (Vnr::init, Init.cc:103-394)
  auto Z = [&](std::vector<double>& v, long long n) { v.assign(n, 0.0); };
  Z(h.rho, nc); Z(h.p, nc); Z(h.c, nc); Z(h.e, nc); Z(h.q, nc); Z(h.divu, nc);
  Z(h.cell_mass, nc);
  Z(h.rhom, 3 * nc); Z(h.pm, 3 * nc); Z(h.cm, 3 * nc); Z(h.em, 3 * nc);
  Z(h.qm, 3 * nc); Z(h.fm, 3 * nc); Z(h.mfm, 3 * nc); Z(h.cmassm, 3 * nc);
  Z(h.u, 2 * nn);
  h.mixte.assign(nc, 0);
  h.pure.assign(nc, -1);
  const int t = s.test_case;
  const double g = s.gamma_scalar;
  auto F = [&](std::vector<double>& v, int m, long long c) -> double& {
    return v[m * nc + c];
  };
  if (t == 4 || t == 5) {
    for (long long c = 0; c < nc; ++c) {
      double r = (t == 4) ? Xc[2 * c] : Xc[2 * c + 1];
      F(h.fm, 0, c) = 1.;
      F(h.mfm, 0, c) = 1.;
      if (r < 0.5) {
        h.rho[c] = 1.0; h.p[c] = 1.0;
        F(h.rhom, 0, c) = 1.0; F(h.pm, 0, c) = 1.0;
      } else {
        h.rho[c] = 0.125; h.p[c] = 0.1;
        F(h.rhom, 0, c) = 0.125; F(h.pm, 0, c) = 0.1;
      }
      F(h.cm, 0, c) = std::sqrt(g * F(h.rhom, 0, c) / F(h.pm, 0, c));
      h.c[c] = F(h.cm, 0, c);
    }
  } else if (t == 15 || t == 16) {
    for (long long c = 0; c < nc; ++c) {
      double r = (t == 15) ? Xc[2 * c] : Xc[2 * c + 1];
      if (r < 0.5) {
        F(h.fm, 0, c) = 1.; F(h.fm, 1, c) = 0.;
        F(h.mfm, 0, c) = 1.; F(h.mfm, 1, c) = 0.;
        h.rho[c] = 1.0; h.p[c] = 1.0;
        F(h.rhom, 0, c) = 1.0; F(h.pm, 0, c) = 1.0;
      } else {
        F(h.fm, 0, c) = 0.; F(h.fm, 1, c) = 1.;
        F(h.mfm, 0, c) = 0.; F(h.mfm, 1, c) = 1.;
        h.rho[c] = 0.125; h.p[c] = 0.1;
        F(h.rhom, 1, c) = 0.125; F(h.pm, 1, c) = 0.1;
      }
      F(h.cm, 0, c) = std::sqrt(g * F(h.rhom, 0, c) / F(h.pm, 0, c));
      F(h.cm, 1, c) = std::sqrt(g * F(h.rhom, 1, c) / F(h.pm, 1, c));
      h.c[c] = smin(F(h.cm, 0, c), F(h.cm, 1, c));
    }
    if (s.init_variant == 1) {
      // extension: the first line of cells not below 0.5 is a 50/50 mix
      const bool ycase = (t == 16);
      const long long nline = ycase ? ny : nx, other = ycase ? nx : ny;
      long long first = -1;
      for (long long k = 0; k < nline && first < 0; ++k) {
        long long c = ycase ? k * nx : k;
        double r = ycase ? Xc[2 * c + 1] : Xc[2 * c];
        if (!(r < 0.5)) first = k;
      }
      for (long long tt = 0; first >= 0 && tt < other; ++tt) {
        long long c = ycase ? first * nx + tt : tt * nx + first;
        const double f0 = 0.5, f1 = 0.5, r0 = 1.0, r1 = 0.125, p0 = 1.0,
                     p1 = 0.1;
        const double m0 = f0 * r0, m1 = f1 * r1;
        F(h.fm, 0, c) = f0; F(h.fm, 1, c) = f1;
        F(h.mfm, 0, c) = m0 / (m0 + m1);
        F(h.mfm, 1, c) = m1 / (m0 + m1);
        F(h.rhom, 0, c) = r0; F(h.rhom, 1, c) = r1;
        F(h.pm, 0, c) = p0; F(h.pm, 1, c) = p1;
        h.rho[c] = f0 * r0 + f1 * r1;
        h.p[c] = f0 * p0 + f1 * p1;
        F(h.cm, 0, c) = std::sqrt(g * r0 / p0);
        F(h.cm, 1, c) = std::sqrt(g * r1 / p1);
        h.c[c] = smin(F(h.cm, 0, c), F(h.cm, 1, c));
      }
    }
  } else if (t == 1) {
    // Sedov (extension for VNR, after eucclhyd_remap/Init.cc:303-332): rho 1,
    // p 1e-6, the energy 0.244816 deposited in the cell that touches the
    // origin, expressed as that cell's pressure; sound speed as the VNR Sod
    // initialisation writes it (Init.cc:139-142)
    const double e1 = 1.e-6 / ((s.gamma[0] - 1.0) * 1.0);
    for (long long c = 0; c < nc; ++c) {
      long long nd[4];
      M.nodes(c, nd);
      bool centre = false;
      for (int k = 0; k < 4; ++k)
        if (norm2(X[2 * nd[k]], X[2 * nd[k] + 1]) < s.threshold) centre = true;
      const double e = centre ? e1 + 0.244816 / (s.dx * s.dy) : e1;
      F(h.fm, 0, c) = 1.;
      F(h.mfm, 0, c) = 1.;
      h.rho[c] = 1.0;
      F(h.rhom, 0, c) = 1.0;
      h.p[c] = (s.gamma[0] - 1.0) * 1.0 * e;
      F(h.pm, 0, c) = h.p[c];
      F(h.cm, 0, c) = std::sqrt(g * F(h.rhom, 0, c) / F(h.pm, 0, c));
      h.c[c] = F(h.cm, 0, c);
    }
  } else if (t == 18 && s.init_variant == 2) {
    // advection step (extension): material 1 with rho 1 left of x = 0.5,
    // material 2 with rho 0.1 right of it, uniform velocity (1, 0); pressure,
    // energy and sound speed as the reference advection cases (Init.cc
    // :185-260)
    for (long long c = 0; c < nc; ++c) {
      const double r = Xc[2 * c];
      const int m = (r < 0.5) ? 0 : 1;
      const double d = (m == 0) ? 1.0 : 0.1;
      F(h.fm, m, c) = 1.;
      F(h.mfm, m, c) = 1.;
      h.rho[c] = d;
      h.p[c] = 0.0;
      F(h.rhom, m, c) = d;
      F(h.pm, m, c) = 0.0;
      F(h.cm, 0, c) = 1.;
      F(h.cm, 1, c) = 1.;
      h.c[c] = smin(F(h.cm, 0, c), F(h.cm, 1, c));
      F(h.em, 0, c) = 1.;
      F(h.em, 1, c) = 1.;
      h.e[c] = 1.;
    }
    for (long long pn = 0; pn < nn; ++pn) {
      h.u[pn] = 1.0;
      h.u[nn + pn] = 0.0;
    }
  } else if (t == 7 || t == 8 || t == 18 || t == 19 || t == 20 || t == 21) {
    const bool isx = (t == 7 || t == 18 || t == 20);
    const bool bi = (t >= 18);
    const bool vit = (t == 20 || t == 21);
    for (long long c = 0; c < nc; ++c) {
      double r = isx ? Xc[2 * c] : Xc[2 * c + 1];
      const double dens_out = vit ? 4.0 : 1.0;
      if (r < 0.3) {
        F(h.fm, 0, c) = 1.; F(h.mfm, 0, c) = 1.;
        h.rho[c] = dens_out; h.p[c] = 0.0;
        F(h.rhom, 0, c) = dens_out; F(h.pm, 0, c) = 0.0;
      } else if ((r > 0.3) && (r < 0.5)) {
        if (!bi) {
          F(h.fm, 0, c) = 1.; F(h.mfm, 0, c) = 1.;
          h.rho[c] = 10.; h.p[c] = 0.0;
          F(h.rhom, 0, c) = 10.0; F(h.pm, 0, c) = 0.0;
        } else {
          F(h.fm, 1, c) = 1.; F(h.mfm, 1, c) = 1.;
          h.rho[c] = vit ? 4. : 1.; h.p[c] = 0.0;
          F(h.rhom, 1, c) = 1.0; F(h.pm, 1, c) = 0.0;
        }
      } else if (r > 0.5) {
        F(h.fm, 0, c) = 1.; F(h.mfm, 0, c) = 1.;
        h.rho[c] = dens_out; h.p[c] = 0.0;
        F(h.rhom, 0, c) = dens_out; F(h.pm, 0, c) = 0.0;
      }
      F(h.cm, 0, c) = 1.;
      F(h.cm, 1, c) = 1.;
      h.c[c] = smin(F(h.cm, 0, c), F(h.cm, 1, c));
      F(h.em, 0, c) = 1.;
      F(h.em, 1, c) = 1.;
      h.e[c] = 1.;
    }
    for (long long i = 0; i <= ny; ++i)
      for (long long j = 0; j <= nx; ++j) {
        long long pn = M.nid(i, j);
        double u0 = isx ? 1.0 : 0.0, u1 = isx ? 0.0 : 1.0;
        double* up = &h.u[pn];
        double* vp = &h.u[nn + pn];
        if (vit) {
          double r = isx ? X[2 * pn] : X[2 * pn + 1];
          if (r <= 0.3) {
            *up = 0.2 * u0; *vp = 0.2 * u1;
          } else if ((r > 0.3) && (r <= 0.5)) {
            double sc = 4. * r - 1.;
            *up = sc * u0; *vp = sc * u1;
          } else if (r > 0.5) {
            *up = u0; *vp = u1;
          }
        } else {
          *up = u0;
          *vp = u1;
        }
      }
  } else {
    return fail(-10, "VNR initialisation: unsupported test case");
  }
  // mixed-cell indicator (Init.cc:373-393)
  for (long long c = 0; c < nc; ++c) {
    int matcell = 0, imatpure = -1;
    for (int m = 0; m < 3; ++m)
      if (F(h.fm, m, c) > s.threshold) {
        matcell++;
        imatpure = m;
      }
    if (matcell > 1) {
      h.mixte[c] = 1;
      h.pure[c] = -1;
    } else {
      h.mixte[c] = 0;
      h.pure[c] = imatpure;
    }
  }
  // periodic rebuild source (ConditionsLimites.cc:186-209)
  h.rho0_left.resize(ny);
  for (long long i = 0; i < ny; ++i) h.rho0_left[i] = h.rho[i * nx];

  // ---- initial sub-volumes (initSubVol, Init.cc:400-429)
  std::vector<double> Vpc(4 * nc);
  for (long long c = 0; c < nc; ++c) {
    long long nd[4];
    M.nodes(c, nd);
    for (int k = 0; k < 4; ++k) {
      long long pm = nd[(k + 3) % 4], pp = nd[(k + 1) % 4], pk = nd[k];
      double x1[2] = {Xc[2 * c], Xc[2 * c + 1]};
      double x2[2] = {0.5 * (X[2 * pm] + X[2 * pk]),
                      0.5 * (X[2 * pm + 1] + X[2 * pk + 1])};
      double x3[2] = {X[2 * pk], X[2 * pk + 1]};
      double x4[2] = {0.5 * (X[2 * pp] + X[2 * pk]),
                      0.5 * (X[2 * pp + 1] + X[2 * pk + 1])};
      Vpc[4 * c + k] = 0.5 * (cross2(x1, x2) + cross2(x2, x3) + cross2(x3, x4) +
                              cross2(x4, x1));
    }
  }
  // sums used by computeDeltaT (VnrRemap.cc:29-37) and the pseudo-viscosity
  // (PhaseLagrange.cc:65-84); with projection the Lagrangian mesh is reset
  // each cycle so these sub-volumes stay the initial ones.
  const double cfl = (s.projection == 1) ? 0.05 : 0.1;
  h.s0.resize(nc);
  h.sqs0.resize(nc);
  h.cflsq.resize(nc);
  for (long long c = 0; c < nc; ++c) {
    double r = 0.0;
    for (int k = 0; k < 4; ++k) r = r + Vpc[4 * c + k];
    h.s0[c] = r;
    h.sqs0[c] = std::sqrt(r);
    h.cflsq[c] = cfl * h.sqs0[c];
  }
  // corner normals of the (constant) Euler mesh (PhaseLagrange.cc:114-136)
  h.cqs.resize(8 * nc);
  for (long long c = 0; c < nc; ++c) {
    long long nd[4];
    M.nodes(c, nd);
    for (int k = 0; k < 4; ++k) {
      double o[2];
      lpc_npc(&X[2 * nd[k]], &X[2 * nd[(k + 1) % 4]], &X[2 * nd[(k + 3) % 4]],
              o);
      h.cqs[(2 * k) * nc + c] = o[0];
      h.cqs[(2 * k + 1) * nc + c] = o[1];
    }
  }
  // outer face normals (initMeshGeometryForFaces, Init.cc:517-554): only the
  // component along each face's sweep axis is ever read.
  h.nout.resize(4 * nc);
  for (long long c = 0; c < nc; ++c) {
    long long nd[4];
    M.nodes(c, nd);
    // faces: bottom (nd0-nd1), left (nd0-nd3), right (nd1-nd2), top (nd3-nd2)
    const long long fa[4][2] = {{nd[1], nd[2]}, {nd[0], nd[3]}, {nd[0], nd[1]},
                                {nd[3], nd[2]}};
    // order of planes: L.x, R.x, B.y, T.y
    const int comp[4] = {0, 0, 1, 1};
    const int which[4] = {1, 0, 2, 3};  // left, right, bottom, top in fa
    for (int q = 0; q < 4; ++q) {
      const long long* e = fa[which[q]];
      double Xf0 = 0.5 * (X[2 * e[0]] + X[2 * e[1]]);
      double Xf1 = 0.5 * (X[2 * e[0] + 1] + X[2 * e[1] + 1]);
      double d0 = Xf0 - Xc[2 * c], d1 = Xf1 - Xc[2 * c + 1];
      double nr = norm2(d0, d1);
      h.nout[q * nc + c] = (comp[q] == 0 ? d0 : d1) / nr;
    }
  }
  // Euler face lengths: vertical faces per row, horizontal per column
  h.flv.resize(ny);
  h.flh.resize(nx);
  for (long long i = 0; i < ny; ++i) h.flv[i] = norm2(0.0, h.ys[i + 1] - h.ys[i]);
  for (long long j = 0; j < nx; ++j) h.flh[j] = norm2(h.xs[j + 1] - h.xs[j], 0.0);

  // cell masses (computeCellMass, PhaseLagrange.cc:14-24)
  for (long long c = 0; c < nc; ++c) {
    h.cell_mass[c] = s.dx * s.dy * h.rho[c];
    for (int m = 0; m < s.nbmat; ++m)
      F(h.cmassm, m, c) = F(h.mfm, m, c) * h.cell_mass[c];
  }
  if (s.sans_lagrange == 0) {
    // initDeltaT (Init.cc:435-457)
    double red = 1.7976931348623157e308;
    for (long long c = 0; c < nc; ++c)
      red = smin(red, 0.1 * h.sqs0[c] / h.c[c]);
    h.dt_init = red * 1.0E-6;
    // initInternalEnergy (Init.cc:463-472)
    for (long long c = 0; c < nc; ++c) {
      for (int m = 0; m < 3; ++m)
        F(h.em, m, c) = F(h.pm, m, c) / ((s.gamma[m] - 1.0) * F(h.rhom, m, c));
      h.e[c] = h.p[c] / ((s.gamma_scalar - 1.0) * h.rho[c]);
    }
  } else {
    h.dt_init = s.dt_init;
  }
  // node masses (computeNodeMass, PhaseLagrange.cc:31-48)
  h.node_mass.resize(nn);
  for (long long i = 0; i <= ny; ++i)
    for (long long j = 0; j <= nx; ++j) {
      double r = 0.0;
      int k = 0;
      if (i < ny && j < nx) { r = r + h.cell_mass[i * nx + j]; ++k; }
      if (i < ny && j > 0) { r = r + h.cell_mass[i * nx + j - 1]; ++k; }
      if (i > 0 && j < nx) { r = r + h.cell_mass[(i - 1) * nx + j]; ++k; }
      if (i > 0 && j > 0) { r = r + h.cell_mass[(i - 1) * nx + j - 1]; ++k; }
      h.node_mass[M.nid(i, j)] = r / (double)k;
    }
  (void)smax;
  return 0;
}

}  // namespace hydro
