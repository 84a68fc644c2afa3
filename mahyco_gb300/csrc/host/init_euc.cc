// Host-side initial state of a Eucclhyd run and its constant Euler geometry.
//
// Restates the set-up sequence of Eucclhyd::simulate (eucclhyd_remap/
// EucclhydRemap.cc:273-287): computeCornerNormal (PhaseLagrange.cc:27-66),
// initMeshGeometryForCells, initBoundaryConditions, initCellInternalEnergy,
// initCellVelocity, initDensity, initMeshGeometryForFaces, setUpTimeLoopN
// (Init.cc), operation by operation; compiled with -ffp-contract=off.
//
// Corner quantities are stored per (cell, corner k), k being the node's
// position in the cell's node list; the reference stores the same numbers
// per (node, slot of the cell in the node's cell list).
#include <cmath>
#include <cstring>

#include "../internal.h"
#include "init.h"

namespace hydro {
namespace {

inline double dot2(const double* a, const double* b) {
  double r = 0.0;
  r += a[0] * b[0];
  r += a[1] * b[1];
  return r;
}
inline double nrm(const double* a) { return std::sqrt(dot2(a, a)); }
inline double cross(const double* a, const double* b) {
  return a[0] * b[1] - a[1] * b[0];
}

}  // namespace

int build_initial_state_euc(const hydro_spec& s, HostInit& h) {
  if (s.nx < 2 || s.ny < 2) return fail(-12, "nx and ny must be >= 2");
  const long long nx = s.nx, ny = s.ny, nc = nx * ny, nn = (nx + 1) * (ny + 1);
  h.nx = nx;
  h.ny = ny;
  h.nc = nc;
  h.nn = nn;
  const int t = s.test_case;
  // ---- initBoundaryConditions (Init.cc:15-98)
  if (t == 4 || t == 5 || t == 15 || t == 16 || t == 2 || t == 13) {
    h.bc_left = h.bc_right = h.bc_top = h.bc_bottom = kBcSym;
  } else if (t == 1 || t == 12) {
    h.bc_left = kBcSym;
    h.bc_bottom = kBcSym;
    h.bc_right = kBcImposed;
    h.bc_top = kBcImposed;
    h.v_right[0] = h.v_right[1] = 0.0;
    h.v_top[0] = h.v_top[1] = 0.0;
  } else {
    return fail(-10, "Eucclhyd initialisation: test case " + std::to_string(t) +
                         " is not supported");
  }
  // symmetry values: ey on the left / right sides, ex on top / bottom
  if (h.bc_left == kBcSym) { h.v_left[0] = 0.0; h.v_left[1] = 1.0; }
  if (h.bc_right == kBcSym) { h.v_right[0] = 0.0; h.v_right[1] = 1.0; }
  if (h.bc_top == kBcSym) { h.v_top[0] = 1.0; h.v_top[1] = 0.0; }
  if (h.bc_bottom == kBcSym) { h.v_bottom[0] = 1.0; h.v_bottom[1] = 0.0; }

  // node coordinates (CartesianMesh2DGenerator.cc:52-54)
  h.xs.resize(nx + 1);
  h.ys.resize(ny + 1);
  for (long long j = 0; j <= nx; ++j) h.xs[j] = s.dx * (double)j;
  for (long long i = 0; i <= ny; ++i) h.ys[i] = s.dy * (double)i;
  auto X = [&](long long p, double out[2]) {
    const long long i = p / (nx + 1), j = p - i * (nx + 1);
    out[0] = h.xs[j];
    out[1] = h.ys[i];
  };
  auto nodes = [&](long long c, long long nd[4]) {
    const long long i = c / nx, j = c - i * nx, n0 = i * (nx + 1) + j;
    nd[0] = n0;
    nd[1] = n0 + 1;
    nd[2] = n0 + nx + 2;
    nd[3] = n0 + nx + 1;
  };
  // ---- computeCornerNormal (PhaseLagrange.cc:27-66): lpc and the corner
  // matrix l+ n+ (x) n+ + l- n- (x) n- (PhaseLagrange.cc:281-287)
  h.lpc.assign(8 * nc, 0.0);
  h.cmat.assign(12 * nc, 0.0);
  for (long long c = 0; c < nc; ++c) {
    long long nd[4];
    nodes(c, nd);
    for (int k = 0; k < 4; ++k) {
      double xp[2], xpp[2], xpm[2];
      X(nd[k], xp);
      X(nd[(k + 1) % 4], xpp);
      X(nd[(k + 3) % 4], xpm);
      double np[2] = {0.5 * (xpp[1] - xp[1]), 0.5 * (xp[0] - xpp[0])};
      const double lp = nrm(np);
      np[0] = np[0] / lp;
      np[1] = np[1] / lp;
      double nm[2] = {0.5 * (xp[1] - xpm[1]), 0.5 * (xpm[0] - xp[0])};
      const double lm = nrm(nm);
      nm[0] = nm[0] / lm;
      nm[1] = nm[1] / lm;
      h.lpc[(2 * k) * nc + c] = np[0] * lp + nm[0] * lm;
      h.lpc[(2 * k + 1) * nc + c] = np[1] * lp + nm[1] * lm;
      h.cmat[(3 * k) * nc + c] = (np[0] * np[0]) * lp + (nm[0] * nm[0]) * lm;
      h.cmat[(3 * k + 1) * nc + c] = (np[0] * np[1]) * lp + (nm[0] * nm[1]) * lm;
      h.cmat[(3 * k + 2) * nc + c] = (np[1] * np[1]) * lp + (nm[1] * nm[1]) * lm;
    }
  }
  // ---- initMeshGeometryForCells (Init.cc:106-166)
  h.xc.assign(2 * nc, 0.0);
  h.evol.assign(nc, 0.0);
  h.perim.assign(nc, 0.0);
  for (long long c = 0; c < nc; ++c) {
    long long nd[4];
    nodes(c, nd);
    double P[4][2];
    for (int k = 0; k < 4; ++k) X(nd[k], P[k]);
    double r11 = 0.0;
    for (int k = 0; k < 4; ++k) r11 = r11 + cross(P[k], P[(k + 1) % 4]);
    const double vol = 0.5 * r11;
    double r12[2] = {0.0, 0.0};
    for (int k = 0; k < 4; ++k) {
      const double* a = P[k];
      const double* b = P[(k + 1) % 4];
      const double cr = cross(a, b);
      r12[0] = r12[0] + (a[0] + b[0]) * cr;
      r12[1] = r12[1] + (a[1] + b[1]) * cr;
    }
    const double sc = 1.0 / (6.0 * vol);
    h.xc[c] = r12[0] * sc;
    h.xc[nc + c] = r12[1] * sc;
    h.evol[c] = vol;
    double r13 = 0.0;
    for (int k = 0; k < 4; ++k) {
      const double d[2] = {P[k][0] - P[(k + 1) % 4][0], P[k][1] - P[(k + 1) % 4][1]};
      r13 = r13 + nrm(d);
    }
    h.perim[c] = r13;
  }
  // ---- initCellInternalEnergy, initCellVelocity, initDensity (Init.cc
  // :194-675).  init_variant 3 of BiTriplePoint scales the regions to a
  // 7 x 3 domain (x <= 1, y <= 1.5) and gives material 3 density 0.125.
  const bool scaled = (t == 13 && s.init_variant == 3);
  const double xlim = scaled ? 1.0 : 0.01, ylim = scaled ? 1.5 : 0.015;
  const double rho3 = scaled ? 0.125 : 0.1;
  const double* g = s.gamma;
  auto Z = [&](std::vector<double>& v, long long n) { v.assign(n, 0.0); };
  Z(h.rho, nc); Z(h.p, nc); Z(h.c, nc); Z(h.e, nc); Z(h.q, nc); Z(h.divu, nc);
  Z(h.cell_mass, nc);
  Z(h.rhom, 3 * nc); Z(h.pm, 3 * nc); Z(h.cm, 3 * nc); Z(h.em, 3 * nc);
  Z(h.qm, 3 * nc); Z(h.fm, 3 * nc); Z(h.mfm, 3 * nc); Z(h.cmassm, 3 * nc);
  Z(h.u, 2 * nn);
  Z(h.uc, 2 * nc);
  Z(h.node_mass, nn);
  h.mixte.assign(nc, 0);
  h.pure.assign(nc, -1);
  auto F = [&](std::vector<double>& v, int m, long long c) -> double& {
    return v[m * nc + c];
  };
  for (long long c = 0; c < nc; ++c) {
    const double x0 = h.xc[c], x1 = h.xc[nc + c];
    if (t == 4 || t == 5) {
      const double r = (t == 4) ? x0 : x1;
      double p, rho;
      if (r <= 0.5) { p = 1.0; rho = 1.0; } else { p = 0.1; rho = 0.125; }
      const double e = p / ((g[0] - 1.0) * rho);
      h.e[c] = e;
      F(h.em, 0, c) = e;
      F(h.fm, 0, c) = 1.; F(h.mfm, 0, c) = 1.;
      h.rho[c] = rho;
      F(h.rhom, 0, c) = rho;
      F(h.rhom, 1, c) = rho;
    } else if (t == 15 || t == 16) {
      const double r = (t == 15) ? x0 : x1;
      if (r <= 0.5) {
        const double e = 1.0 / ((g[0] - 1.0) * 1.0);
        F(h.em, 0, c) = e;
        h.e[c] = e;
        F(h.fm, 0, c) = 1.; F(h.mfm, 0, c) = 1.;
        h.rho[c] = 1.0;
        F(h.rhom, 0, c) = 1.0;
      } else {
        const double e = 0.1 / ((g[1] - 1.0) * 0.125);
        F(h.em, 1, c) = e;
        h.e[c] = e;
        F(h.fm, 1, c) = 1.; F(h.mfm, 1, c) = 1.;
        h.rho[c] = 0.125;
        F(h.rhom, 1, c) = 0.125;
      }
    } else if (t == 2) {
      double p, rho;
      if (x0 <= 0.01) { p = 1.0; rho = 1.0; }
      else if (x1 <= 0.015) { p = 0.1; rho = 1.; }
      else { p = 0.1; rho = 0.1; }
      const double e = p / ((g[0] - 1.0) * rho);
      h.e[c] = e;
      F(h.em, 0, c) = e;
      F(h.fm, 0, c) = 1.; F(h.mfm, 0, c) = 1.;
      h.rho[c] = (x0 <= 0.01) ? 1.0 : ((x1 <= 0.015) ? 1.0 : 0.1);
    } else if (t == 13) {
      int m;
      double rho, p;
      if (x0 <= xlim) { m = 0; rho = 1.0; p = 1.0; }
      else if (x1 <= ylim) { m = 1; rho = 1.0; p = 0.1; }
      else { m = 2; rho = rho3; p = 0.1; }
      const double e = p / ((g[m] - 1.0) * rho);
      h.e[c] = e;
      F(h.em, m, c) = e;
      h.rho[c] = rho;
      F(h.fm, m, c) = 1.; F(h.mfm, m, c) = 1.;
      F(h.rhom, m, c) = rho;
    } else {  // Sedov (test case 1; 12 has no density initialisation)
      const double e1 = 1.e-6 / ((g[0] - 1.0) * 1.);
      long long nd[4];
      nodes(c, nd);
      bool centre = false;
      for (int k = 0; k < 4; ++k) {
        double xp[2];
        X(nd[k], xp);
        if (nrm(xp) < s.threshold) centre = true;
      }
      h.e[c] = centre ? e1 + 0.244816 / (s.dx * s.dy) : e1;
      F(h.em, 0, c) = h.e[c];
      if (t == 1) {
        h.rho[c] = 1.0;
        F(h.rhom, 0, c) = 1.0;
      }
    }
    if (s.nbmat == 1) {
      F(h.fm, 0, c) = 1.; F(h.fm, 1, c) = 0.; F(h.fm, 2, c) = 0.;
      F(h.mfm, 0, c) = 1.; F(h.mfm, 1, c) = 0.; F(h.mfm, 2, c) = 0.;
    }
    int matcell = 0, imatpure = -1;
    for (int m = 0; m < 3; ++m)
      if (F(h.fm, m, c) > s.threshold) {
        matcell++;
        imatpure = m;
      }
    h.mixte[c] = matcell > 1 ? 1 : 0;
    h.pure[c] = matcell > 1 ? -1 : imatpure;
  }
  // ---- initMeshGeometryForFaces (Init.cc:677-716): outer normals along
  // each face's sweep axis from the centroids; Euler face lengths
  h.nout.resize(4 * nc);
  for (long long c = 0; c < nc; ++c) {
    long long nd[4];
    nodes(c, nd);
    double P[4][2];
    for (int k = 0; k < 4; ++k) X(nd[k], P[k]);
    // planes L.x, R.x, B.y, T.y: left (nd0-nd3), right (nd1-nd2),
    // bottom (nd0-nd1), top (nd3-nd2)
    const int ends[4][2] = {{0, 3}, {1, 2}, {0, 1}, {3, 2}};
    const int comp[4] = {0, 0, 1, 1};
    for (int q = 0; q < 4; ++q) {
      const double* a = P[ends[q][0]];
      const double* b = P[ends[q][1]];
      const double Xf0 = 0.5 * (a[0] + b[0]), Xf1 = 0.5 * (a[1] + b[1]);
      const double d[2] = {Xf0 - h.xc[c], Xf1 - h.xc[nc + c]};
      const double nr = nrm(d);
      h.nout[q * nc + c] = (comp[q] == 0 ? d[0] : d[1]) / nr;
    }
  }
  h.flv.resize(ny);
  h.flh.resize(nx);
  for (long long i = 0; i < ny; ++i) {
    const double d[2] = {0.0, h.ys[i + 1] - h.ys[i]};
    h.flv[i] = nrm(d);
  }
  for (long long j = 0; j < nx; ++j) {
    const double d[2] = {h.xs[j + 1] - h.xs[j], 0.0};
    h.flh[j] = nrm(d);
  }
  h.rho0_left.assign(ny, 0.0);
  // ---- setUpTimeLoopN (Init.cc:721-760)
  h.dt_init = (t == 2 || t == 13) ? 1.0e-5 : 1.0e-4;
  return 0;
}

}  // namespace hydro
