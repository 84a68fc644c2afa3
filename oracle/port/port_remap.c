/*
 * ORACLE -- test infrastructure, never part of the product.
 *
 * C restatement of MaHyCo's directionally split remap (remap/PhaseRemap1.cc,
 * remap/PhaseRemap2.cc), its limiters and plateau-slope ("PenteBorne") flux
 * integrals (remap/UtilesRemap.cc, remap/UtilesRemap-Impl.h) and the VNR
 * nodal (dual) remap (remap/DualPhaseRemap1.cc, DualPhaseRemap2.cc,
 * remap/UtilesDualRemap.cc).  Operation order follows the reference.
 */
#include <stdlib.h>
#include <string.h>

#include "port_internal.h"

/* ----------------------------------------------------------- limiters */
/* Remap::fluxLimiter (remap/UtilesRemap.cc:9-23) */
static double flux_limiter(int id, double r) {
  if (id == HYDRO_LIM_MINMOD) return smax(0.0, smin(1.0, r));
  if (id == HYDRO_LIM_SUPERBEE)
    return smax(0.0, smax(smin(2.0 * r, 1.0), smin(r, 2.0)));
  if (id == HYDRO_LIM_VANLEER) {
    if (r <= 0.0) return 0.0;
    return 2.0 * r / (1.0 + r);
  }
  return 0.0;
}

/* divideNoExcept (includes/Freefunctions.h:86-92) */
static double divide_no_except(double a, double b) {
  if (fabs(b) < 1.0E-12) return 0.0;
  return a / b;
}

/* Remap::fluxLimiterPP (remap/UtilesRemap.cc:25-72) */
static double flux_limiter_pp(int id, double gp, double gm, double y0,
                              double yp, double ym, double h0, double hp,
                              double hm) {
  double grady = 0.0, gradM, gradMplus, gradMmoins;
  (void)y0;
  if (gp * gm < 0.0) return 0.;
  if (id == HYDRO_LIM_MINMODG) {
    if ((yp - ym) > 0.)
      grady = smin(fabs(gp), fabs(gm));
    else
      grady = -smin(fabs(gp), fabs(gm));
  } else if (id == HYDRO_LIM_SUPERBEEG) {
    if ((yp - ym) > 0.)
      grady = smax(fabs(gp), fabs(gm));
    else
      grady = -smax(fabs(gp), fabs(gm));
  } else if (id == HYDRO_LIM_VANLEERG) {
    double lp = (h0 / 2. + hp) / (h0 + hp + hm);
    double lm = (h0 / 2. + hm) / (h0 + hp + hm);
    if ((lp * gp + lm * gm) != 0.)
      grady = gp * gm / (lp * gp + lm * gm);
    else
      grady = 0.;
  } else if (id == HYDRO_LIM_ULTRABEEG) {
    grady = (yp - ym) / h0;
  } else if (id == HYDRO_LIM_ARITHMETICG) {
    double lp = (h0 / 2. + hp) / (h0 + hp + hm);
    double lm = (h0 / 2. + hm) / (h0 + hp + hm);
    grady = lm * gp + lp * gm;
  }
  gradMplus = gp * (h0 + hp) / h0;
  gradMmoins = gm * (h0 + hm) / h0;
  gradM = smin(fabs(gradMplus), fabs(gradMmoins));
  if ((yp - ym) > 0.)
    grady = smin(fabs(gradM), fabs(grady));
  else
    grady = -smin(fabs(gradM), fabs(grady));
  return grady;
}

/* Remap::computeAndLimitGradPhi (remap/UtilesRemap-Impl.h:99-126), d comps */
static void limit_grad(int id, const double* gp, const double* gm,
                       const double* phi, const double* phip,
                       const double* phim, double h0, double hp, double hm,
                       double* res, int d) {
  if (id < HYDRO_LIM_MINMODG) {
    for (int i = 0; i < d; i++)
      res[i] = (flux_limiter(id, divide_no_except(gp[i], gm[i])) * gm[i] +
                flux_limiter(id, divide_no_except(gm[i], gp[i])) * gp[i]) /
               2.0;
  } else {
    for (int i = 0; i < d; i++)
      res[i] = flux_limiter_pp(id, gp[i], gm[i], phi[i], phip[i], phim[i], h0,
                               hp, hm);
  }
}

/* Remap::computeY0 (remap/UtilesRemap.cc:74-125) */
static double compute_y0(int id, double y0, double yp, double ym, double h0,
                         double hp, double hm, int type) {
  double y0p = 0., y0m = 0.;
  (void)y0;
  if (id == HYDRO_LIM_MINMODG || id == HYDRO_LIM_MINMOD) {
    y0p = yp;
    y0m = ym;
  } else if (id == HYDRO_LIM_SUPERBEEG || id == HYDRO_LIM_SUPERBEE) {
    y0p = ((h0 + hm) * yp + h0 * ym) / (2 * h0 + hm);
    y0m = ((h0 + hp) * ym + h0 * yp) / (2 * h0 + hp);
  } else if (id == HYDRO_LIM_VANLEERG || id == HYDRO_LIM_VANLEER) {
    double a = smin(yp, ym);
    double b = smax(yp, ym);
    double xp = (h0 * h0 + 3 * h0 * hm + 2 * hm * hm) * yp;
    double xm = (h0 * h0 + 3 * h0 * hp + 2 * hp * hp) * ym;
    xp += (h0 * h0 - h0 * hp - 2 * hp * hp + 2 * h0 * hm) * ym;
    xm += (h0 * h0 - h0 * hm - 2 * hm * hm + 2 * h0 * hp) * yp;
    xp /= (2 * h0 * h0 + 5 * h0 * hm + 2 * hm * hm - h0 * hp - 2 * hp * hp);
    xm /= (2 * h0 * h0 + 5 * h0 * hp + 2 * hp * hp - h0 * hm - 2 * hm * hm);
    y0p = smin(smax(xp, a), b);
    y0m = smin(smax(xm, a), b);
  } else if (id == HYDRO_LIM_ULTRABEEG) {
    y0p = (yp + ym) / 2.;
    y0m = (yp + ym) / 2.;
  } else if (id == HYDRO_LIM_ARITHMETICG) {
    y0p = ((h0 + hm + hp) * yp + h0 * ym) / (2 * h0 + hm + hp);
    y0m = ((h0 + hm + hp) * ym + h0 * yp) / (2 * h0 + hm + hp);
  } else if (id == 3000) {
    y0p = yp;
    y0m = ym;
  }
  if (type == 0) return y0p;
  if (type == 1) return y0m;
  return 0.0;
}

/* Remap::computexgxd (remap/UtilesRemap.cc:127-145) */
static double compute_xgxd(double thr, double y0, double yp, double ym,
                           double h0, double y0p, double y0m, int type) {
  double xd, xg, xp = 1., xm = 1.;
  if (fabs(y0p - yp) > thr) xp = (y0 - yp) / (y0p - yp) - 1. / 2.;
  if (fabs(y0m - ym) > thr) xm = (y0 - ym) / (y0m - ym) - 1. / 2.;
  xd = +h0 * smin(smax(xp, -1. / 2.), 1. / 2.);
  xg = -h0 * smin(smax(xm, -1. / 2.), 1. / 2.);
  if (type == 0) return xg;
  if (type == 1) return xd;
  return 0.0;
}

/* Remap::computeygyd (remap/UtilesRemap.cc:147-166) */
static double compute_ygyd(double y0, double yp, double ym, double h0,
                           double y0p, double y0m, double grady, int type) {
  double xtd = y0 + h0 / 2 * grady;
  double xtg = y0 - h0 / 2 * grady;
  double ad = smin(yp, 2. * y0m - ym);
  double bd = smax(yp, 2. * y0m - ym);
  double ag = smin(ym, 2. * y0p - yp);
  double bg = smax(ym, 2. * y0p - yp);
  double yd = smin(smax(xtd, ad), bd);
  double yg = smin(smax(xtg, ag), bg);
  if (type == 0) return yg;
  if (type == 1) return yd;
  return 0.0;
}

/* Remap::INT2Y (remap/UtilesRemap.cc:177-188) */
static double int2y(double X, double x0, double y0, double x1, double y1) {
  double flux = 0.;
  if (fabs(x1 - x0) > 1.e-14) {
    double eta = smin(smax(0., (X - x0) / (x1 - x0)), 1.);
    flux = (y0 + 0.5 * eta * (y1 - y0)) * (x1 - x0) * eta;
  }
  return flux;
}

/* Remap::computeFluxPP / computeFluxPPPure (remap/UtilesRemap-Impl.h
 * :142-489).  pure selects the pure-cell variant. */
static void flux_pp(const port_run* R, int pure, const double* gradphi,
                    const double* phi, const double* phip, const double* phim,
                    double h0, double hp, double hm, double v, double dt,
                    int type, double dualv, int cfd, double* pFlux,
                    double* pFluxDual) {
  const int nb = R->nbmat;
  const double thr = R->s.threshold;
  const int lim = pure ? R->s.limiter_pure : R->s.limiter;
  double Flux[NEQ], Fd[NEQ];
  for (int i = 0; i < NEQ; ++i) Flux[i] = Fd[i] = 0.0;
  double ppv = 0.5 * (v + fabs(v)) * dt;
  double ppdv = 0.5 * (dualv + fabs(dualv)) * dt;
  for (int i = 0; i < NEQ; i++) {
    double y0p = compute_y0(lim, phi[i], phip[i], phim[i], h0, hp, hm, 0);
    double y0m = compute_y0(lim, phi[i], phip[i], phim[i], h0, hp, hm, 1);
    double xg = compute_xgxd(thr, phi[i], phip[i], phim[i], h0, y0p, y0m, 0);
    double xd = compute_xgxd(thr, phi[i], phip[i], phim[i], h0, y0p, y0m, 1);
    double yg =
        compute_ygyd(phi[i], phip[i], phim[i], h0, y0p, y0m, gradphi[i], 0);
    double yd =
        compute_ygyd(phi[i], phip[i], phim[i], h0, y0p, y0m, gradphi[i], 1);
    double f1, f2, f3, f1m, f2m, f3m;
    if (type == 0) {
      f1m = int2y(-h0 / 2. + ppv, -h0 / 2., phim[i], xg, yg);
      f1 = int2y(-h0 / 2., -h0 / 2., phim[i], xg, yg);
      f2m = int2y(-h0 / 2. + ppv, xg, yg, xd, yd);
      f2 = int2y(-h0 / 2., xg, yg, xd, yd);
      f3m = int2y(-h0 / 2. + ppv, xd, yd, h0 / 2., phip[i]);
      f3 = int2y(-h0 / 2., xd, yd, h0 / 2., phip[i]);
      Flux[i] = smax(((f1m - f1) + (f2m - f2) + (f3m - f3)), 0.);
      if (((phip[i] - phi[i]) * (phim[i] - phi[i])) >= 0.)
        Flux[i] = phi[i] * ppv;
      if (cfd == 1) {
        f1m = int2y(ppdv, -h0 / 2., phim[i], xg, yg);
        f1 = int2y(0., -h0 / 2., phim[i], xg, yg);
        f2m = int2y(ppdv, xg, yg, xd, yd);
        f2 = int2y(0., xg, yg, xd, yd);
        f3m = int2y(ppdv, xd, yd, h0 / 2., phip[i]);
        f3 = int2y(0., xd, yd, h0 / 2., phip[i]);
        Fd[i] = smax(((f1m - f1) + (f2m - f2) + (f3m - f3)), 0.);
        if (((phip[i] - phi[i]) * (phim[i] - phi[i])) >= 0.)
          Fd[i] = phi[i] * ppdv;
      }
    } else if (type == 1) {
      f1 = int2y(h0 / 2. - ppv, -h0 / 2., phim[i], xg, yg);
      f1m = int2y(h0 / 2., -h0 / 2., phim[i], xg, yg);
      f2 = int2y(h0 / 2. - ppv, xg, yg, xd, yd);
      f2m = int2y(h0 / 2., xg, yg, xd, yd);
      f3 = int2y(h0 / 2. - ppv, xd, yd, h0 / 2., phip[i]);
      f3m = int2y(h0 / 2., xd, yd, h0 / 2., phip[i]);
      Flux[i] = smax(((f1m - f1) + (f2m - f2) + (f3m - f3)), 0.);
      if (((phip[i] - phi[i]) * (phim[i] - phi[i])) >= 0.)
        Flux[i] = phi[i] * ppv;
      if (cfd == 1) Fd[i] = 0.;
    }
  }
  if (R->s.pb_complet == 1) {
    double sfm = 0., sfv = 0.;
    for (int m = 0; m < nb; m++) sfv += Flux[m];
    if (fabs(sfv) > thr) {
      for (int m = 0; m < nb; m++) {
        if (!pure) Flux[nb + m] = (Flux[nb + m] / sfv) * Flux[m];
        Flux[2 * nb + m] = (Flux[2 * nb + m] / sfv) * Flux[nb + m];
        sfm += Flux[nb + m];
      }
      Flux[3 * nb] = (Flux[3 * nb] / sfv) * sfm;
      Flux[3 * nb + 1] = (Flux[3 * nb + 1] / sfv) * sfm;
      Flux[3 * nb + 2] = (Flux[3 * nb + 2] / sfv) * sfm;
      Flux[3 * nb + 3] = phi[3 * nb + 3] * sfv;
    } else {
      for (int i = 0; i < NEQ; ++i) Flux[i] = 0.0;
    }
  } else {
    double sfm = 0., sfv = 0.;
    for (int m = 0; m < nb; m++) {
      if (!pure) Flux[nb + m] = phi[nb + m] * Flux[m];
      Flux[2 * nb + m] = phi[2 * nb + m] * Flux[nb + m];
      sfm += Flux[nb + m];
      sfv += Flux[m];
    }
    Flux[3 * nb] = phi[3 * nb] * sfm;
    Flux[3 * nb + 1] = phi[3 * nb + 1] * sfm;
    Flux[3 * nb + 2] = phi[3 * nb + 2] * sfm;
    Flux[3 * nb + 3] = phi[3 * nb + 3] * sfv;
  }
  for (int i = 0; i < NEQ; ++i) {
    pFlux[i] = (ppv == 0.) ? 0.0 : Flux[i];
    pFluxDual[i] = (ppdv == 0.) ? 0.0 : Fd[i];
  }
}

/* order-3 helpers (remap/UtilesRemap.cc:200-320) */
static double eval_grad(double hm, double h0, double hp, double ym, double y0,
                        double yp) {
  return h0 / (hm + h0 + hp) *
         ((2. * hm + h0) / (h0 + hp) * (yp - y0) +
          (h0 + 2. * hp) / (hm + h0) * (y0 - ym));
}
static double eval_ystar(double hmm, double hm, double hp, double hpp,
                         double ymm, double ym, double yp, double ypp,
                         double gradm, double gradp) {
  double tmp1 = (2. * hp * hm) / (hm + hp) *
                ((hmm + hm) / (2. * hm + hp) - (hpp + hp) / (2. * hp + hm)) *
                (yp - ym);
  double tmp2 = -hm * (hmm + hm) / (2. * hm + hp) * gradp +
                hp * (hp + hpp) / (hm + 2. * hp) * gradm;
  return ym + hm / (hm + hp) * (yp - ym) +
         1. / (hmm + hm + hp + hpp) * (tmp1 + tmp2);
}
static double eval_fm(double x, double dx, double up, double du, double u6) {
  return up - 0.5 * x / dx * (du - (1. - 2. / 3. * x / dx) * u6);
}
static double eval_fp(double x, double dx, double um, double du, double u6) {
  return um + 0.5 * x / dx * (du - (1. - 2. / 3. * x / dx) * u6);
}
static double flux_ordre3(double ymmm, double ymm, double ym, double yp,
                          double ypp, double yppp, double hmmm, double hmm,
                          double hm, double hp, double hpp, double hppp,
                          double vdt) {
  double gradmm = eval_grad(hmmm, hmm, hm, ymmm, ymm, ym);
  double gradm = eval_grad(hmm, hm, hp, ymm, ym, yp);
  double gradp = eval_grad(hm, hp, hpp, ym, yp, ypp);
  double gradpp = eval_grad(hp, hpp, hppp, yp, ypp, yppp);
  double ystarm = eval_ystar(hmmm, hmm, hm, hp, ymmm, ymm, ym, yp, gradmm, gradm);
  double ystar = eval_ystar(hmm, hm, hp, hpp, ymm, ym, yp, ypp, gradm, gradp);
  double ystarp = eval_ystar(hm, hp, hpp, hppp, ym, yp, ypp, yppp, gradp, gradpp);
  double ym_m = ystarm, ym_p = ystar, yp_m = ystar, yp_p = ystarp;
  double grad_m = ym_p - ym_m, grad_p = yp_p - yp_m;
  double ym6 = 6. * (ym - 0.5 * (ym_m + ym_p));
  double yp6 = 6. * (yp - 0.5 * (yp_m + yp_p));
  double flux;
  if (vdt >= 0.)
    flux = eval_fm(vdt, hm, ym_p, grad_m, ym6);
  else
    flux = eval_fp(-vdt, hp, yp_m, grad_p, yp6);
  double num = vdt / hm, nup = vdt / hp;
  double ym_ym = ym + (1. - num) / num * (ym - ymm);
  double yp_ym = yp - (1. + nup) / nup * (yp - ypp);
  double i1inf, i1sup, i2inf, i2sup;
  i1inf = smin(ym, yp);
  i1sup = smax(ym, yp);
  if (vdt >= 0.) {
    i2inf = smin(ym, ym_ym);
    i2sup = smax(ym, ym_ym);
  } else {
    i2inf = smin(yp, yp_ym);
    i2sup = smax(yp, yp_ym);
  }
  double linf, lsup;
  if ((i1sup < i2inf) || (i2sup < i1inf)) {
    linf = 0.;
    lsup = 0.;
  } else {
    linf = smax(i1inf, i2inf);
    lsup = smin(i1sup, i2sup);
  }
  if (flux < linf) flux = linf;
  if (flux > lsup) flux = lsup;
  return flux;
}

/* ------------------------------------------------------------- sweeps */
static double dot2(const double* a, const double* b) {
  double r = 0.0;
  r = r + a[0] * b[0];
  r = r + a[1] * b[1];
  return r;
}

/* One directional sweep: computeGradPhiFace{1,2}, computeGradPhi{1,2},
 * computeUpwindFaceQuantitiesForProjection{1,2}, computeUremap{1,2}
 * (remap/PhaseRemap1.cc:22-568, remap/PhaseRemap2.cc:21-497). */
void port_remap_sweep(port_run* R, int sweep) {
  const int dirx = (sweep == 1) ? R->x_then_y_n : !R->x_then_y_n;
  const double exy[2] = {dirx ? 1.0 : 0.0, dirx ? 0.0 : 1.0};
  double* gPF = sweep == 1 ? R->gPF1 : R->gPF2;
  double* gP = sweep == 1 ? R->gP1 : R->gP2;
  double* phiF = sweep == 1 ? R->phiF1 : R->phiF2;
  double* DPF = sweep == 1 ? R->DPF1 : R->DPF2;
  double* Bid = sweep == 1 ? R->Bid1 : R->Bid2;
  double* FF = sweep == 1 ? R->FF1 : R->FF2;
  const double* Uin = sweep == 1 ? R->UL : R->U1;
  double* Uout = sweep == 1 ? R->U1 : R->U2;
  const int nb = R->nbmat;
  const int order = R->s.projection_order;
  const int pb = R->s.pb;
  const double dt = R->dt_n;

  if (order > 1) {
#pragma omp parallel for
    for (long f = 0; f < R->nf; ++f) {
      face_info F;
      port_face_decode(R, f, &F);
      if (F.front < 0 || F.vertical != dirx) continue;
      for (int k = 0; k < NEQ; ++k)
        gPF[NEQ * f + k] =
            (R->Phi[NEQ * F.front + k] - R->Phi[NEQ * F.back + k]) / R->dxL[f];
    }
#pragma omp parallel for
    for (long c = 0; c < R->nc; ++c) {
      long fs[4];
      port_cell_faces(R, c, fs);
      double h = 0.;
      if (dirx) {
        h += 0.5 * R->fLL[fs[0]];
        h += 0.5 * R->fLL[fs[3]];
      } else {
        h += 0.5 * R->fLL[fs[2]];
        h += 0.5 * R->fLL[fs[1]];
      }
      R->Hv[c] = h;
    }
#pragma omp parallel for
    for (long c = 0; c < R->nc; ++c) {
      long fs[4];
      port_cell_faces(R, c, fs);
      long i = c / R->nx, j = c - i * R->nx;
      long cplus, cminus; /* reference's cf / cb */
      long fa, fb;        /* face of the type-0 (arriere) / type-1 flux */
      if (dirx) {
        cplus = (j < R->nx - 1) ? c + 1 : c;  /* front of right face */
        cminus = (j > 0) ? c - 1 : c;         /* back of left face  */
        fa = fs[1];
        fb = fs[2];
      } else {
        cplus = (i > 0) ? c - R->nx : c;          /* cf: cell below */
        cminus = (i < R->ny - 1) ? c + R->nx : c; /* cb: cell above */
        fa = fs[0];
        fb = fs[3];
      }
      long cf = cplus, cb = cminus;
      int vp = (R->s.pb_mixte == 1) &&
               (R->mixte[c] == 0 && R->mixte[cf] == 0 && R->mixte[cb] == 0 &&
                R->pure[c] == R->pure[cf] && R->pure[c] == R->pure[cb]);
      int lim = R->s.limiter;
      if ((pb == 1) && vp) lim = R->s.limiter_pure;
      const double *phi = R->Phi + NEQ * c;
      if (dirx) {
        limit_grad(lim, gPF + NEQ * fs[2], gPF + NEQ * fs[1], phi,
                   R->Phi + NEQ * cf, R->Phi + NEQ * cb, R->Hv[c], R->Hv[cf],
                   R->Hv[cb], gP + NEQ * c, NEQ);
      } else {
        limit_grad(lim, gPF + NEQ * fs[0], gPF + NEQ * fs[3], phi,
                   R->Phi + NEQ * cb, R->Phi + NEQ * cf, R->Hv[c], R->Hv[cb],
                   R->Hv[cf], gP + NEQ * c, NEQ);
      }
      if (pb == 1) {
        int sa = dirx ? 1 : 0, sb = dirx ? 2 : 3;
        double Fa = dot2(R->nOut + (4 * c + sa) * 2, exy) * R->fnv[fa];
        double Fb = dot2(R->nOut + (4 * c + sb) * 2, exy) * R->fnv[fb];
        double fdual = 0.5 * (R->fnv[fa] + R->fnv[fb]);
        int cfd = (R->s.dual_mass_flux == 2) ? 1 : 0;
        const double *pp, *pm;
        double hp, hm;
        if (dirx) {
          pp = R->Phi + NEQ * cf; pm = R->Phi + NEQ * cb;
          hp = R->Hv[cf]; hm = R->Hv[cb];
        } else {
          pp = R->Phi + NEQ * cb; pm = R->Phi + NEQ * cf;
          hp = R->Hv[cb]; hm = R->Hv[cf];
        }
        flux_pp(R, vp, gP + NEQ * c, phi, pp, pm, R->Hv[c], hp, hm, Fa, dt, 0,
                fdual, cfd, R->dPAr + NEQ * c, DPF + NEQ * c);
        double s = (R->fL[fa] + R->fL[fb]) * 0.5;
        for (int k = 0; k < NEQ; ++k) DPF[NEQ * c + k] *= s;
        flux_pp(R, vp, gP + NEQ * c, phi, pp, pm, R->Hv[c], hp, hm, Fb, dt, 1,
                fdual, cfd, R->dPAv + NEQ * c, Bid + NEQ * c);
      }
    }
  }

  /* face values (computeUpwindFaceQuantitiesForProjection) */
#pragma omp parallel for
  for (long f = 0; f < R->nf; ++f) {
    face_info F;
    port_face_decode(R, f, &F);
    if (F.front < 0 || F.vertical != dirx) continue;
    long cb = F.back, cf = F.front;
    double* out = phiF + NEQ * f;
    if (order <= 2) {
      if (pb == 0) {
        const double* n = R->fN + 2 * f;
        if (R->fnv[f] * R->dxL[f] > 0.0) {
          double d[2] = {R->Xf[2 * f] - R->XcL[2 * cb],
                         R->Xf[2 * f + 1] - R->XcL[2 * cb + 1]};
          double s = dot2(d, n);
          for (int k = 0; k < NEQ; ++k)
            out[k] = Uin[NEQ * cb + k] / R->vL[cb] + s * gP[NEQ * cb + k];
        } else {
          double d[2] = {R->Xf[2 * f] - R->XcL[2 * cf],
                         R->Xf[2 * f + 1] - R->XcL[2 * cf + 1]};
          double s = dot2(d, n);
          for (int k = 0; k < NEQ; ++k)
            out[k] = Uin[NEQ * cf + k] / R->vL[cf] + s * gP[NEQ * cf + k];
        }
      } else {
        long av = dirx ? cb : cf, ar = dirx ? cf : cb;
        for (int k = 0; k < NEQ; ++k)
          out[k] = R->dPAv[NEQ * av + k] - R->dPAr[NEQ * ar + k];
      }
    } else if (order == 3) {
      /* six cells ordered along the sweep, "m" side first */
      long cs[6];
      if (dirx) {
        long i = cb / R->nx, jb = cb - i * R->nx, jf = cf - i * R->nx;
        long jbb = jb > 0 ? jb - 1 : jb, jbbb = jbb > 0 ? jbb - 1 : jbb;
        long jff = jf < R->nx - 1 ? jf + 1 : jf;
        long jfff = jff < R->nx - 1 ? jff + 1 : jff;
        cs[0] = port_cid(R, i, jbbb); cs[1] = port_cid(R, i, jbb);
        cs[2] = cb; cs[3] = cf;
        cs[4] = port_cid(R, i, jff); cs[5] = port_cid(R, i, jfff);
      } else {
        long j = cf % R->nx, i_f = cf / R->nx, i_b = cb / R->nx;
        long iff = i_f > 0 ? i_f - 1 : i_f, ifff = iff > 0 ? iff - 1 : iff;
        long ibb = i_b < R->ny - 1 ? i_b + 1 : i_b;
        long ibbb = ibb < R->ny - 1 ? ibb + 1 : ibb;
        cs[0] = port_cid(R, ifff, j); cs[1] = port_cid(R, iff, j);
        cs[2] = cf; cs[3] = cb;
        cs[4] = port_cid(R, ibb, j); cs[5] = port_cid(R, ibbb, j);
      }
      double vdt = R->fnv[f] * dt;
      for (int k = 0; k < NEQ; ++k) {
        double y[6];
        for (int t = 0; t < 6; ++t) y[t] = Uin[NEQ * cs[t] + k] / R->vL[cs[t]];
        out[k] = flux_ordre3(y[0], y[1], y[2], y[3], y[4], y[5], R->Hv[cs[0]],
                             R->Hv[cs[1]], R->Hv[cs[2]], R->Hv[cs[3]],
                             R->Hv[cs[4]], R->Hv[cs[5]], vdt);
      }
    }
  }

  /* conservative update (computeUremap{1,2}) */
  int nerr = 0;
#pragma omp parallel for reduction(+ : nerr)
  for (long c = 0; c < R->nc; ++c) {
    long i = c / R->nx, j = c - i * R->nx;
    long fs[4];
    port_cell_faces(R, c, fs);
    double red[NEQ];
    for (int k = 0; k < NEQ; ++k) red[k] = 0.0;
    /* getNeighbourCells order: below, above, left, right */
    int slots[4], ns = 0;
    if (i >= 1) slots[ns++] = 0;
    if (i < R->ny - 1) slots[ns++] = 3;
    if (j >= 1) slots[ns++] = 1;
    if (j < R->nx - 1) slots[ns++] = 2;
    for (int t = 0; t < ns; ++t) {
      int sl = slots[t];
      long f = fs[sl];
      double* ffc = FF + (4 * c + sl) * NEQ;
      const double* n = R->fN + 2 * f;
      const double* no = R->nOut + (4 * c + sl) * 2;
      if (fabs(dot2(n, exy)) < 1.0E-10) {
        for (int k = 0; k < NEQ; ++k) ffc[k] = 0.0 * phiF[NEQ * f + k];
      } else {
        double s;
        if (pb == 0)
          s = dot2(no, exy) * R->fnv[f] * R->fL[f] * dt;
        else
          s = dot2(no, exy) * R->fL[f];
        for (int k = 0; k < NEQ; ++k) ffc[k] = s * phiF[NEQ * f + k];
      }
      for (int k = 0; k < NEQ; ++k) red[k] = red[k] + ffc[k];
    }
    /* Remap::computeBoundaryFluxes (remap/BoundaryFluxes.cc:14-120): the
     * flux through a boundary face with a flux condition, carrying the
     * value of the cell's opposite face; branches in the reference's order
     * (slots: 0 bottom, 1 left, 2 right, 3 top) */
    if (R->leftFluxBC + R->rightFluxBC + R->bottomFluxBC + R->topFluxBC > 0) {
      int fb = -1, fo = -1;
      if (R->bottomFluxBC == 1 && c < R->nx && exy[1] == 1) {
        fb = 0; fo = 3;
      } else if (R->topFluxBC == 1 && c <= R->nx * (R->ny - 1) && c < R->nc && exy[1] == 1) {
        fb = 3; fo = 0;
      } else if (R->leftFluxBC == 1 && exy[0] == 1 && j == 0) {
        fb = 1; fo = 2;
      } else if (R->rightFluxBC == 1 && exy[0] == 1 && j == R->nx - 1) {
        fb = 2; fo = 1;
      }
      if (fb >= 0) {
        const long f = fs[fb], fo_ = fs[fo];
        const double* n = R->fN + 2 * f;
        const double* no = R->nOut + (4 * c + fb) * 2;
        double bf[NEQ];
        if (fabs(dot2(n, exy)) < 1.0E-10) {
          for (int k = 0; k < NEQ; ++k) bf[k] = 0.0 * phiF[NEQ * fo_ + k];
        } else {
          double s;
          if (pb == 0)
            s = dot2(no, exy) * R->fnv[f] * R->fL[f] * dt;
          else
            s = dot2(no, exy) * R->fL[f];
          for (int k = 0; k < NEQ; ++k) bf[k] = s * phiF[NEQ * fo_ + k];
        }
        for (int k = 0; k < NEQ; ++k) red[k] = red[k] + bf[k];
      }
    }
    double* U = Uout + NEQ * c;
    for (int k = 0; k < NEQ; ++k) U[k] = Uin[NEQ * c + k] - red[k];
    if (sweep == 1) {
      double* P = R->Phi + NEQ * c;
      if (pb == 1) {
        double sv = 0.;
        for (int m = 0; m < nb; m++) sv += U[m];
        double sm = 0.;
        for (int m = 0; m < nb; m++) {
          P[m] = U[m] / sv;
          if (U[m] != 0.)
            P[nb + m] = U[nb + m] / (U[m]);
          else
            P[nb + m] = 0.;
          sm += U[nb + m];
        }
        P[3 * nb] = U[3 * nb] / sm;
        P[3 * nb + 1] = U[3 * nb + 1] / sm;
        for (int m = 0; m < nb; m++) {
          if (U[nb + m] != 0.)
            P[2 * nb + m] = U[2 * nb + m] / U[nb + m];
          else
            P[2 * nb + m] = 0.;
        }
        if (R->s.projection_conservative == 1) P[3 * nb + 2] = U[3 * nb + 2] / sm;
      } else {
        for (int k = 0; k < NEQ; ++k) P[k] = U[k] / R->vL[c];
      }
      int matcell = 0, imatpure = -1;
      for (int m = 0; m < nb; m++)
        if (P[m] > 0.) {
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
  (void)nerr;
}

/* ---------------------------------------------------------- dual remap */
static inline const double* dphi(const port_run* R, long p, const double* z) {
  return p >= 0 ? R->DualPhi + NEQ * p : z;
}
static inline const double* xlag(const port_run* R, long p, const double* z) {
  return p >= 0 ? R->XL + 2 * p : z;
}

/* Remap::computeDualHorizontalGradPhi / computeDualVerticalGradPhi
 * (remap/UtilesRemap-Impl.h:8-97); only the two velocity components are
 * consumed downstream, so only those are limited. */
static void dual_grad(const port_run* R, long p, int dirx, double* g) {
  static const double z[NEQ] = {0};
  g[0] = g[1] = 0.0;
  long L, Rn, LL, RR;
  int ax = dirx ? 0 : 1;
  if (dirx) {
    L = port_left_node(R, p);
    Rn = port_right_node(R, p);
  } else {
    L = port_bottom_node(R, p);
    Rn = port_top_node(R, p);
  }
  if (L == -1 || Rn == -1) return;
  const double *DP = R->DualPhi + NEQ * p, *DR = R->DualPhi + NEQ * Rn,
               *DL = R->DualPhi + NEQ * L;
  const double *Xp = R->XL + 2 * p, *XR = R->XL + 2 * Rn, *XLn = R->XL + 2 * L;
  double gr[2], gl[2];
  for (int k = 0; k < 2; ++k) {
    gr[k] = (DR[k] - DP[k]) / (XR[ax] - Xp[ax]);
    gl[k] = (DP[k] - DL[k]) / (Xp[ax] - XLn[ax]);
  }
  if (dirx) {
    LL = port_left_node(R, L);
    RR = port_right_node(R, Rn);
  } else {
    LL = port_bottom_node(R, L);
    RR = port_top_node(R, Rn);
  }
  double hm, h0, hp;
  h0 = 0.5 * (XR[ax] - XLn[ax]);
  if (LL == -1) {
    hm = 0.;
    hp = 0.5 * (xlag(R, RR, z)[ax] - Xp[ax]);
  } else if (RR == -1) {
    hp = 0.;
    hm = 0.5 * (Xp[ax] - xlag(R, LL, z)[ax]);
  } else {
    hm = 0.5 * (Xp[ax] - R->XL[2 * LL + ax]);
    hp = 0.5 * (R->XL[2 * RR + ax] - Xp[ax]);
  }
  limit_grad(R->s.limiter, gr, gl, DP, DR, DL, h0, hp, hm, g, 2);
}

/* nodal mass fluxes of one sweep through the two cells each side of the
 * node (remap/UtilesDualRemap.cc A1 :10-233, A2 :401-644, PB :648-818;
 * cell/face pattern of remap/FacesLeftAndRight.h, FacesTopAndBottom.h).
 * Returns the "minus" side (left / bottom) and "plus" side (right / top). */
static void dual_mass_flux(const port_run* R, long p, int dirx, int sweep,
                           double* fminus, double* fplus) {
  const int nb = R->nbmat;
  const int meth = R->s.dual_mass_flux;
  const double* FF = sweep == 1 ? R->FF1 : R->FF2;
  const double* DPF = sweep == 1 ? R->DPF1 : R->DPF2;
  const long* T = dirx ? R->VFoN : R->HFoN;
  long cm[2] = {-1, -1}, cp[2] = {-1, -1};
  int nfaces = 0, ncell = 0, has[2] = {0, 0};
  for (int s = 0; s < 2; ++s) {
    long f = T[2 * p + s];
    if (f == -1) continue;
    face_info F;
    port_face_decode(R, f, &F);
    has[s] = 1;
    if (dirx) {
      cp[s] = F.front; /* right cell */
      cm[s] = F.back;  /* left cell  */
    } else {
      cp[s] = F.back;  /* above cell */
      cm[s] = F.front; /* below cell */
    }
    nfaces += 2;
    ncell++;
  }
  /* slot of the crossing face and of the far face in the plus / minus cells */
  const int ax = dirx ? 0 : 1;
  const int sp_near = dirx ? 1 : 0, sp_far = dirx ? 2 : 3; /* plus cell  */
  const int sm_near = dirx ? 2 : 3, sm_far = dirx ? 1 : 0; /* minus cell */
  double Fp = 0., Fm = 0.;
  for (int m = 0; m < nb; m++) {
    double pp = 0, pm = 0;
    for (int s = 0; s < 2; ++s) {
      if (!has[s]) continue;
      long a = cp[s], b = cm[s];
      if (meth == 0 || meth == 1) {
        int comp = (meth == 0) ? nb + m : m;
        double va = FF[(4 * a + sp_near) * NEQ + comp] *
                        R->nOut[(4 * a + sp_near) * 2 + ax] +
                    FF[(4 * a + sp_far) * NEQ + comp] *
                        R->nOut[(4 * a + sp_far) * 2 + ax];
        double vb = FF[(4 * b + sm_near) * NEQ + comp] *
                        R->nOut[(4 * b + sm_near) * 2 + ax] +
                    FF[(4 * b + sm_far) * NEQ + comp] *
                        R->nOut[(4 * b + sm_far) * 2 + ax];
        if (meth == 1) {
          va = R->rL[a] * va;
          vb = R->rL[b] * vb;
        }
        pp += va;
        pm += vb;
      } else {
        pp += DPF[NEQ * a + nb + m];
        pm += DPF[NEQ * b + nb + m];
      }
    }
    if (meth == 2) {
      if (ncell != 0) {
        pp /= ncell;
        pm /= ncell;
      }
    } else if (nfaces != 0) {
      pp /= nfaces;
      pm /= nfaces;
    }
    Fp += pp;
    Fm += pm;
  }
  *fplus = Fp;
  *fminus = Fm;
}

/* Remap::getLeft/Right/Bottom/TopUpwindVelocity (UtilesDualRemap.cc
 * :234-397).  side: 0 minus (left / bottom), 1 plus (right / top). */
static void upwind_velocity(const port_run* R, long nb_node, long p, int dirx,
                            int side, double flux, const double* gnb,
                            const double* g0, double* out) {
  static const double z[NEQ] = {0};
  const int order2 = R->s.projection_order - 1;
  const int ax = dirx ? 0 : 1;
  const double* Dn = dphi(R, nb_node, z);
  const double* Dp = R->DualPhi + NEQ * p;
  const double* Xn = xlag(R, nb_node, z);
  const double* Xp = R->XL + 2 * p;
  double u, dx;
  int sg;
  int from_nb;
  if (side == 0) {
    u = 0.5 * (Dn[ax] + Dp[ax]);
    dx = Xp[ax] - Xn[ax];
    from_nb = (flux > 0);
  } else {
    u = 0.5 * (Dp[ax] + Dn[ax]);
    dx = Xn[ax] - Xp[ax];
    from_nb = (flux < 0);
  }
  sg = (u > 0) ? 1 : -1;
  const double* base = from_nb ? Dn : Dp;
  const double* gr = from_nb ? gnb : g0;
  for (int k = 0; k < 2; ++k)
    out[k] = base[k] +
             order2 * (0.5 * gr[k] * (sg * dx - R->dt_n * u));
}

/* Remap::computeDualUremap1 / computeDualUremap2 (remap/DualPhaseRemap1.cc
 * :18-136, remap/DualPhaseRemap2.cc:18-127) */
void port_dual_sweep(port_run* R, int sweep) {
  const int dirx = (sweep == 1) ? R->x_then_y_n : !R->x_then_y_n;
  double* gDP = sweep == 1 ? R->gDP1 : R->gDP2;
  const double* UDin = sweep == 1 ? R->UDL : R->UD1;
  double* UDout = sweep == 1 ? R->UD1 : R->UD2;
  /* gradDualPhi stored with 2 live components per node (stride NEQ) */
#pragma omp parallel for
  for (long p = 0; p < R->nn; ++p) {
    double* g = gDP + NEQ * p;
    if (R->s.projection_order > 1)
      dual_grad(R, p, dirx, g);
    else
      g[0] = g[1] = 0.0;
  }
  static const double z[NEQ] = {0};
#pragma omp parallel for
  for (long p = 0; p < R->nn; ++p) {
    double fm, fp;
    dual_mass_flux(R, p, dirx, sweep, &fm, &fp);
    double* U = UDout + NEQ * p;
    const double* Ui = UDin + NEQ * p;
    U[2] = Ui[2] + fm - fp;
    long Lm = dirx ? port_left_node(R, p) : port_bottom_node(R, p);
    long Lp = dirx ? port_right_node(R, p) : port_top_node(R, p);
    const double* gm = Lm >= 0 ? gDP + NEQ * Lm : z;
    const double* gp = Lp >= 0 ? gDP + NEQ * Lp : z;
    double um[2], up[2];
    upwind_velocity(R, Lm, p, dirx, 0, fm, gm, gDP + NEQ * p, um);
    upwind_velocity(R, Lp, p, dirx, 1, fp, gp, gDP + NEQ * p, up);
    double* sm = dirx ? R->Luv : R->Buv;
    double* sp = dirx ? R->Ruv : R->Tuv;
    sm[2 * p] = um[0]; sm[2 * p + 1] = um[1];
    sp[2 * p] = up[0]; sp[2 * p + 1] = up[1];
    U[0] = Ui[0] + fm * um[0] - fp * up[0];
    U[1] = Ui[1] + fm * um[1] - fp * up[1];
  }
  if (sweep == 1) {
#pragma omp parallel for
    for (long p = 0; p < R->nn; ++p) {
      double* D = R->DualPhi + NEQ * p;
      const double* U = R->UD1 + NEQ * p;
      D[0] = U[0] / U[2];
      D[1] = U[1] / U[2];
      D[2] = U[2];
      D[3] = U[3] / U[2];
    }
  }
}
