// Scalar FP64 building blocks of the remap, as __device__ functions.
//
// Restated from the reference's limiter and plateau-slope routines
// (remap/UtilesRemap.cc:9-320, remap/UtilesRemap-Impl.h:99-316) in the same
// operation order.  The kernels are compiled with --fmad=false and IEEE
// division / square root, so every value is bit-identical to the reference
// on the same inputs.  std::min / std::max semantics (including the NaN
// behaviour) are kept: smin(a,b) = (b<a)?b:a, smax(a,b) = (a<b)?b:a.
#ifndef MAHYCO_GB300_SCHEME_MATH_CUH
#define MAHYCO_GB300_SCHEME_MATH_CUH

#include "hydro_gb300.h"

namespace hydro {

#define HD __device__ __forceinline__

HD double smin(double a, double b) { return (b < a) ? b : a; }
HD double smax(double a, double b) { return (a < b) ? b : a; }

// Order-preserving 64-bit encoding of doubles (for atomicMin/atomicMax).
HD unsigned long long ord_bits(double x) {
  unsigned long long b = (unsigned long long)__double_as_longlong(x);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
HD double from_ord(unsigned long long o) {
  unsigned long long b = (o >> 63) ? (o & 0x7fffffffffffffffull) : ~o;
  return __longlong_as_double((long long)b);
}

// IEEE division behind a call: the optimizer cannot if-convert a branch
// around it into an unconditional division, so divisions on paths that are
// rarely taken cost nothing when they are not taken.
static __device__ __noinline__ double ddiv_call(double n, double d) { return n / d; }

// n / d with the exact shortcuts decided on the integer pipe:
//   n = +-0, d finite non-zero   -> zero with sign(n) xor sign(d)
//   d = 1                        -> n
//   n = d, finite non-zero       -> 1
// (uniform and single-material cells produce many of these); otherwise the
// IEEE division.  Bit-identical to n / d (NaN results stay NaN).
HD double qdiv(double n, double d) {
  const unsigned long long nb = (unsigned long long)__double_as_longlong(n);
  const unsigned long long db = (unsigned long long)__double_as_longlong(d);
  const bool dfin = ((db >> 52) & 0x7ffull) != 0x7ffull;
  const bool dnz = (db << 1) != 0ull;
  if ((nb << 1) == 0ull && dnz && dfin)
    return __longlong_as_double((long long)((nb ^ db) & 0x8000000000000000ull));
  if (db == 0x3ff0000000000000ull) return n;
  if (nb == db && dnz && dfin) return 1.0;
  return ddiv_call(n, d);
}

// x / k for k = 1, 2 or 4, as the exact multiplication by 1/k (division by
// a power of two and multiplication by its reciprocal round identically).
HD double div_pow2(double x, int k) {
  return x * (k == 4 ? 0.25 : (k == 2 ? 0.5 : 1.0));
}

// Remap::fluxLimiter (remap/UtilesRemap.cc:9-23)
HD double flux_limiter(int id, double r) {
  if (id == HYDRO_LIM_MINMOD) return smax(0.0, smin(1.0, r));
  if (id == HYDRO_LIM_SUPERBEE)
    return smax(0.0, smax(smin(2.0 * r, 1.0), smin(r, 2.0)));
  if (id == HYDRO_LIM_VANLEER) {
    if (r <= 0.0) return 0.0;
    return 2.0 * r / (1.0 + r);
  }
  return 0.0;
}

// divideNoExcept (includes/Freefunctions.h:86-92)
HD double divide_no_except(double a, double b) {
  if (fabs(b) < 1.0E-12) return 0.0;
  return qdiv(a, b);
}

// Remap::fluxLimiterPP (remap/UtilesRemap.cc:25-72)
HD double flux_limiter_pp(int id, double gp, double gm, double yp, double ym,
                          double h0, double hp, double hm) {
  double grady = 0.0;
  if (gp * gm < 0.0) return 0.;
  if (id == HYDRO_LIM_MINMODG) {
    grady = ((yp - ym) > 0.) ? smin(fabs(gp), fabs(gm)) : -smin(fabs(gp), fabs(gm));
  } else if (id == HYDRO_LIM_SUPERBEEG) {
    grady = ((yp - ym) > 0.) ? smax(fabs(gp), fabs(gm)) : -smax(fabs(gp), fabs(gm));
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
  double gMp = gp * (h0 + hp) / h0;
  double gMm = gm * (h0 + hm) / h0;
  double gM = smin(fabs(gMp), fabs(gMm));
  if ((yp - ym) > 0.)
    grady = smin(fabs(gM), fabs(grady));
  else
    grady = -smin(fabs(gM), fabs(grady));
  return grady;
}

// one component of Remap::computeAndLimitGradPhi (UtilesRemap-Impl.h:99-126)
//
// Classic limiters: res = (phi(r1)*gm + phi(r2)*gp) / 2 with
// r1 = divideNoExcept(gp, gm), r2 = divideNoExcept(gm, gp).  For minmod and
// superBee, phi(r) only depends on the exact value of r in some ranges, and
// r1, r2 are reciprocal, so for finite gradients of the same sign one
// division decides both: the other phi is a constant fixed by comparing
// |gp| and |gm| (phi is continuous at its breakpoints, so ratios that round
// onto a breakpoint give the same constant).  Opposite signs give phi = 0
// for both.  Anything else (NaN, infinities, other limiters) takes the
// reference's two divisions.  The result is bit-identical in every case.
HD double limit_grad1(int id, double gp, double gm, double yp, double ym,
                      double h0, double hp, double hm) {
  if (id >= HYDRO_LIM_MINMODG) return flux_limiter_pp(id, gp, gm, yp, ym, h0, hp, hm);
  const double a = fabs(gp), b = fabs(gm);
  if ((id == HYDRO_LIM_MINMOD || id == HYDRO_LIM_SUPERBEE) && isfinite(gp) &&
      isfinite(gm)) {
    double f1, f2;  // phi(r1), phi(r2)
    if (b < 1.0E-12) {
      f1 = 0.0;
      f2 = flux_limiter(id, divide_no_except(gm, gp));
    } else if (a < 1.0E-12) {
      f2 = 0.0;
      f1 = flux_limiter(id, qdiv(gp, gm));
    } else if ((gp < 0.0) != (gm < 0.0)) {
      f1 = 0.0;  // r1, r2 < 0 (or -0 after underflow)
      f2 = 0.0;
    } else if (id == HYDRO_LIM_MINMOD) {
      if (a <= b) {
        f1 = flux_limiter(id, qdiv(gp, gm));
        f2 = 1.0;  // r2 >= 1
      } else {
        f1 = 1.0;  // r1 >= 1
        f2 = flux_limiter(id, qdiv(gm, gp));
      }
    } else {  // superBee: 2r on [0,1/2], 1 on [1/2,1], r on [1,2], 2 above
      if (a <= 0.5 * b) {
        f1 = flux_limiter(id, qdiv(gp, gm));
        f2 = 2.0;  // r2 >= 2
      } else if (a <= b) {
        f1 = 1.0;  // r1 in [1/2, 1]
        f2 = flux_limiter(id, qdiv(gm, gp));
      } else if (a <= 2.0 * b) {
        f1 = flux_limiter(id, qdiv(gp, gm));
        f2 = 1.0;  // r2 in [1/2, 1]
      } else {
        f1 = 2.0;  // r1 >= 2
        f2 = flux_limiter(id, qdiv(gm, gp));
      }
    }
    return (f1 * gm + f2 * gp) / 2.0;
  }
  return (flux_limiter(id, divide_no_except(gp, gm)) * gm +
          flux_limiter(id, divide_no_except(gm, gp)) * gp) /
         2.0;
}

// Remap::computeY0 (remap/UtilesRemap.cc:74-125): both thresholds at once.
HD void compute_y0(int id, double yp, double ym, double h0, double hp,
                   double hm, double& y0p, double& y0m) {
  y0p = 0.;
  y0m = 0.;
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
}

// Remap::INT2Y (remap/UtilesRemap.cc:177-188).  eta = min(max(0, n/d), 1)
// is decided by comparison when the quotient is certainly <= 0 (eta = +0)
// or >= 1 (eta = 1) for finite operands; the division is only performed for
// points strictly inside the interval (or non-finite operands).  Same
// result bit for bit.
HD double int2y(double X, double x0, double y0, double x1, double y1) {
  double flux = 0.;
  const double d = x1 - x0;
  if (fabs(d) > 1.e-14) {
    const double n = X - x0;
    double eta;
    const bool fin = isfinite(n) && isfinite(d);
    if (fin && (d > 0. ? n <= 0. : n >= 0.))
      eta = 0.;
    else if (fin && (d > 0. ? n >= d : n <= d))
      eta = 1.;
    else
      eta = smin(smax(0., ddiv_call(n, d)), 1.);
    flux = (y0 + 0.5 * eta * (y1 - y0)) * d * eta;
  }
  return flux;
}

// The reconstruction of one component for a plateau-slope integral:
// computeY0 + computexgxd + computeygyd (remap/UtilesRemap.cc:74-166).
struct PPShape {
  double xg, xd, yg, yd;
};
HD PPShape pp_shape(int lim, double thr, double y0, double yp, double ym,
                    double h0, double hp, double hm, double grad) {
  double y0p, y0m;
  compute_y0(lim, yp, ym, h0, hp, hm, y0p, y0m);
  double xp = 1., xm = 1.;
  if (fabs(y0p - yp) > thr) xp = qdiv(y0 - yp, y0p - yp) - 1. / 2.;
  if (fabs(y0m - ym) > thr) xm = qdiv(y0 - ym, y0m - ym) - 1. / 2.;
  PPShape s;
  s.xd = +h0 * smin(smax(xp, -1. / 2.), 1. / 2.);
  s.xg = -h0 * smin(smax(xm, -1. / 2.), 1. / 2.);
  double xtd = y0 + h0 / 2 * grad;
  double xtg = y0 - h0 / 2 * grad;
  double ad = smin(yp, 2. * y0m - ym);
  double bd = smax(yp, 2. * y0m - ym);
  double ag = smin(ym, 2. * y0p - yp);
  double bg = smax(ym, 2. * y0p - yp);
  s.yd = smin(smax(xtd, ad), bd);
  s.yg = smin(smax(xtg, ag), bg);
  return s;
}

// Integral of the reconstruction between a and b (the three pieces of
// computeFluxPP, remap/UtilesRemap-Impl.h:182-257), clipped at 0, with the
// "formule 16" replacement at extrema.
HD double pp_integral(const PPShape& s, double a, double b, double h0,
                      double y0, double yp, double ym, double ppv) {
  double f1b = int2y(b, -h0 / 2., ym, s.xg, s.yg);
  double f1a = int2y(a, -h0 / 2., ym, s.xg, s.yg);
  double f2b = int2y(b, s.xg, s.yg, s.xd, s.yd);
  double f2a = int2y(a, s.xg, s.yg, s.xd, s.yd);
  double f3b = int2y(b, s.xd, s.yd, h0 / 2., yp);
  double f3a = int2y(a, s.xd, s.yd, h0 / 2., yp);
  double F = smax(((f1b - f1a) + (f2b - f2a) + (f3b - f3a)), 0.);
  if (((yp - y0) * (ym - y0)) >= 0.) F = y0 * ppv;
  return F;
}

// order-3 face value (remap/UtilesRemap.cc:200-320)
HD double eval_grad(double hm, double h0, double hp, double ym, double y0,
                    double yp) {
  return h0 / (hm + h0 + hp) *
         ((2. * hm + h0) / (h0 + hp) * (yp - y0) +
          (h0 + 2. * hp) / (hm + h0) * (y0 - ym));
}
HD double eval_ystar(double hmm, double hm, double hp, double hpp, double ymm,
                     double ym, double yp, double ypp, double gradm,
                     double gradp) {
  double tmp1 = (2. * hp * hm) / (hm + hp) *
                ((hmm + hm) / (2. * hm + hp) - (hpp + hp) / (2. * hp + hm)) *
                (yp - ym);
  double tmp2 = -hm * (hmm + hm) / (2. * hm + hp) * gradp +
                hp * (hp + hpp) / (hm + 2. * hp) * gradm;
  return ym + hm / (hm + hp) * (yp - ym) +
         1. / (hmm + hm + hp + hpp) * (tmp1 + tmp2);
}
HD double flux_ordre3(double ymmm, double ymm, double ym, double yp,
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
  double grad_m = ystar - ystarm, grad_p = ystarp - ystar;
  double ym6 = 6. * (ym - 0.5 * (ystarm + ystar));
  double yp6 = 6. * (yp - 0.5 * (ystar + ystarp));
  double flux;
  if (vdt >= 0.) {
    double x = vdt, dx = hm;
    flux = ystar - 0.5 * x / dx * (grad_m - (1. - 2. / 3. * x / dx) * ym6);
  } else {
    double x = -vdt, dx = hp;
    flux = ystar + 0.5 * x / dx * (grad_p - (1. - 2. / 3. * x / dx) * yp6);
  }
  double num = vdt / hm, nup = vdt / hp;
  double ym_ym = ym + (1. - num) / num * (ym - ymm);
  double yp_ym = yp - (1. + nup) / nup * (yp - ypp);
  double i1inf = smin(ym, yp), i1sup = smax(ym, yp), i2inf, i2sup;
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

}  // namespace hydro
#endif
