// Host-side check of the integer-pipe comparison helpers and the one-division
// limiter of scheme_math.cuh against the plain IEEE expressions they replace
// (compiled by nvcc for the host, run on the CPU).  Exit status 0 = all equal.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include <vector>

#include "kernels/scheme_math.cuh"

using namespace hydro;

static double ref_smin(double a, double b) { return (b < a) ? b : a; }
static double ref_smax(double a, double b) { return (a < b) ? b : a; }
static double ref_flux_limiter(int id, double r) {
  if (id == HYDRO_LIM_MINMOD) return ref_smax(0.0, ref_smin(1.0, r));
  return ref_smax(0.0, ref_smax(ref_smin(2.0 * r, 1.0), ref_smin(r, 2.0)));
}
static double ref_dne(double a, double b) {
  if (std::fabs(b) < 1.0E-12) return 0.0;
  return a / b;
}
static double ref_limit(int id, double gp, double gm) {
  return (ref_flux_limiter(id, ref_dne(gp, gm)) * gm +
          ref_flux_limiter(id, ref_dne(gm, gp)) * gp) / 2.0;
}
static bool same(double a, double b) {
  unsigned long long x, y;
  memcpy(&x, &a, 8);
  memcpy(&y, &b, 8);
  if (std::isnan(a) && std::isnan(b)) return true;
  return x == y;
}

int main() {
  std::vector<double> v = {0.0, -0.0, 1.0, -1.0, 0.5, -0.5, 2.0, -2.0, 1e-12, -1e-12,
                           std::nextafter(1e-12, 0.0), std::nextafter(1e-12, 1.0),
                           4.9e-324, -4.9e-324, 2.2250738585072014e-308,
                           -2.2250738585072014e-308, 1.7976931348623157e308,
                           -1.7976931348623157e308, 8.98846567431158e307,
                           INFINITY, -INFINITY, NAN, -NAN, 3.0, 1e-300, -7.5,
                           std::nextafter(1.0, 0.0), std::nextafter(1.0, 2.0),
                           std::nextafter(2.0, 0.0), std::nextafter(0.5, 1.0)};
  std::mt19937_64 g(12345);
  for (int i = 0; i < 2000; ++i) {
    unsigned long long b = g();
    double d;
    memcpy(&d, &b, 8);
    v.push_back(d);
    v.push_back(std::ldexp((double)(g() % 1000) - 500.0, (int)(g() % 80) - 40));
  }
  long bad = 0, n = 0;
  for (double a : v)
    for (double b : v) {
      ++n;
      bad += dlt(a, b) != (a < b);
      bad += dle(a, b) != (a <= b);
      bad += dgt(a, b) != (a > b);
      bad += dge(a, b) != (a >= b);
      bad += !same(smin(a, b), ref_smin(a, b));
      bad += !same(smax(a, b), ref_smax(a, b));
      bad += !same(addz(a, b), a + b);
      bad += !same(subz(a, b), a - b);
      bad += !same(mulz(a, b), a * b);
      bad += !same(qdiv(a, b), a / b);
      bad += !same(mul1z(a, b), a * b);
    }
  for (double a : v) {
    bad += pos(a) != (a > 0.0);
    bad += neg(a) != (a < 0.0);
    bad += nonneg(a) != (a >= 0.0);
    bad += nonpos(a) != (a <= 0.0);
    bad += is_nan(a) != (bool)std::isnan(a);
    bad += is_finite(a) != (bool)std::isfinite(a);
    bad += abs_lt(a, 1e-12) != (std::fabs(a) < 1e-12);
    bad += abs_gt(a, 1e-14) != (std::fabs(a) > 1e-14);
    bad += !same(half(a), a * 0.5);
    bad += !same(quarter(a), a * 0.25);
    bad += !same(dbl(a), 2.0 * a);
    bad += !same(plus_zero(a), a + 0.0);
    bad += !same(addz(a, -a), a + (-a)) + !same(subz(a, a), a - a);
    bad += !same(addz(-a, a), (-a) + a) + !same(subz(-a, -a), (-a) - (-a));
    for (int k = 0; k < 3; ++k) bad += !same(mul_012(k, a), (double)k * a);
    for (double f : {1.0, 0.0, -0.0, 0.5, 0.25, 1e-300})
      bad += !same(mul_frac(f, a), f * a);
    for (double n : {1.0, -1.0, 0.5, -2.0, 3.0, 0.0, -0.0})
      bad += !same(mul_pm1(a, n), a * n) + !same(mul_pm1(n, a), n * a);
    if (!std::isnan(a)) {
      bad += !same(twice(a), 2.0 * a);
      for (int id : {HYDRO_LIM_MINMOD, HYDRO_LIM_SUPERBEE})
        bad += !same(flux_limiter_q(id, a), ref_flux_limiter(id, a));
    }
  }
  // qdiv by powers of two: every exponent, numerators from the value list and
  // random patterns (quotients across the subnormal and overflow edges)
  for (int e = -1074; e <= 1023; ++e) {
    const double d = std::ldexp(1.0, e);
    for (double a : v) {
      bad += !same(qdiv(a, d), a / d) + !same(qdiv(a, -d), a / -d);
    }
  }
  // order-3 gradient / interpolated value on uniform rows (the coarse
  // shortcut) and near-uniform ones, against the plain expressions
  for (double y : v)
    for (double a : {0.0, -0.0, 1.5, -2.25, 1e-300, 3e200}) {
      const double G0 = a, A = -a * 0.5 + 0.25, B = a * 3.0 - 1.0;
      bad += !same(o3_grad(G0, A, B, y, y, y), G0 * (A * (y - y) + B * (y - y)));
      bad += !same(o3_grad(G0, -A, -B, y, y, y), G0 * (-A * (y - y) + -B * (y - y)));
      const double T[5] = {a, -a, A, B, G0};
      const double T2[5] = {-a, a, -A, -B, -G0};
      for (double g : {0.0, -0.0})
        for (double g2 : {0.0, -0.0}) {
          const double t1 = T2[0] * (y - y), t2 = T2[1] * g2 + T2[2] * g;
          bad += !same(o3_ystar(T2, y, y, g, g2), y + T2[3] * (y - y) + T2[4] * (t1 + t2));
        }
      for (double g : {0.0, -0.0, 1.0})
        for (double g2 : {0.0, -0.0}) {
          const double t1 = T[0] * (y - y), t2 = T[1] * g2 + T[2] * g;
          bad += !same(o3_ystar(T, y, y, g, g2), y + T[3] * (y - y) + T[4] * (t1 + t2));
        }
    }
  // the node force cancellation the node kernel relies on: with one pressure
  // w in the four cells, ((w c0 + w c1) + w c2) + w c3 (first addition from
  // 0.0) is +0 when c1 = -c0, c3 = -c2, or c1 = c0, c2 = c3 = -c0, for
  // |w|, |c| < 2^500
  {
    long fbad = 0;
    auto rnd = [&](int emax) {
      unsigned long long b = g();
      const unsigned long long e = 1023 - emax + g() % (2 * emax);
      b = (b & 0x800fffffffffffffull) | (e << 52);
      double x;
      memcpy(&x, &b, 8);
      return x;
    };
    auto fsum = [](double w, double c0, double c1, double c2, double c3) {
      double r = plus_zero(w * c0);
      r = r + w * c1;
      r = r + w * c2;
      return r + w * c3;
    };
    for (int i = 0; i < 2000000; ++i) {
      const double w = (i % 97 == 0) ? 0.0 : rnd(499), a = rnd(499), b = rnd(499);
      const double z = (i % 89 == 0) ? -0.0 : a;
      fbad += !same(fsum(w, z, -z, b, -b), 0.0) || (std::signbit(fsum(w, z, -z, b, -b)));
      fbad += !same(fsum(w, z, z, -z, -z), 0.0) || (std::signbit(fsum(w, z, z, -z, -z)));
    }
    if (fbad) printf("force cancellation: %ld mismatches\n", fbad);
    bad += fbad;
  }
  // the order-3 face value of a face that does not move (vdt = +-0, finite
  // positive upwind width, inputs finite below 2^1000) is finite, so its
  // product with the zero sweep coefficient is a zero
  {
    long obad = 0;
    auto rnd = [&](int emax) {
      unsigned long long b = g();
      const unsigned long long e = 1023 - emax + g() % (2 * emax);
      b = (b & 0x800fffffffffffffull) | (e << 52);
      double x;
      memcpy(&x, &b, 8);
      return (g() % 13 == 0) ? 0.0 : x;
    };
    for (int i = 0; i < 1000000; ++i) {
      const double h[4] = {0., 0., std::fabs(rnd(900)) + 1e-300, (i % 5 == 0) ? 0.0 : std::fabs(rnd(900))};
      const double vdt = (i & 1) ? 0.0 : -0.0;
      if (!(h[2] > 0.0)) continue;
      O3Face F;
      o3_face_dt(F, h, vdt);
      const double ys[3] = {rnd(999), rnd(999), rnd(999)};
      const double y = o3_tail(F, ys, rnd(999), rnd(999), rnd(999), rnd(999));
      obad += !std::isfinite(y);
    }
    if (obad) printf("still order-3 faces: %ld non-finite values\n", obad);
    bad += obad;
  }
  // the dual update of a quiet node (no mass flux, velocities +0 at the node
  // and its neighbours, zero slopes at the node, positions below 2^1022, dt
  // finite): the new conserved value is the old one with a zero made +0
  {
    long qbad = 0;
    auto rnd = [&](int emax) {
      unsigned long long b = g();
      const unsigned long long e = 1023 - emax + g() % (2 * emax);
      b = (b & 0x800fffffffffffffull) | (e << 52);
      double x;
      memcpy(&x, &b, 8);
      return x;
    };
    for (int i = 0; i < 1000000; ++i) {
      const double Fm = 0.0, Fp = 0.0, dp = 0.0, dn = 0.0;
      const double gp = (i & 1) ? 0.0 : -0.0, dt = rnd(300);
      const double xp = rnd(1020), xn = (i % 7 == 0) ? 0.0 : rnd(1020);
      const int order2 = i % 3;
      double Ui = (i % 5 == 0) ? ((i & 2) ? -0.0 : 0.0) : rnd(1000);
      if (i % 11 == 0) Ui = INFINITY;
      // the kernel's expressions (minus side and plus side, one component)
      const double u = half(dn + dp);
      const double dxm = xp - xn, sdm = pos(u) ? dxm : -dxm;
      const double um = dp + mul_012(order2, half(gp) * (sdm - dt * u));
      const double dxp = xn - xp, sdp = pos(u) ? dxp : -dxp;
      const double up = dp + mul_012(order2, half(gp) * (sdp - dt * u));
      const double Un = Ui + Fm * um - Fp * up;
      const double want = iszero(Ui) ? 0.0 : Ui;
      qbad += !same(Un, want) || (iszero(Un) && std::signbit(Un));
    }
    if (qbad) printf("quiet dual update: %ld mismatches\n", qbad);
    bad += qbad;
  }
  // exponent helpers: every significand pattern class near and below the
  // smallest normal exponents, both signs
  long pbad = 0, pn = 0;
  for (int i = 0; i < 4000000; ++i) {
    unsigned long long b = g();
    const unsigned long long e = g() % 6;  // exponents 0..5
    b = (b & 0x800fffffffffffffull) | (e << 52);
    if (i % 7 == 0) b = (b & ~0xfull) | (g() & 0xf);  // low bits that round
    double a;
    memcpy(&a, &b, 8);
    ++pn;
    pbad += !same(half(a), a * 0.5);
    pbad += !same(quarter(a), a * 0.25);
    pbad += !same(dbl(a), 2.0 * a);
  }
  if (pbad) printf("exponent helpers: %ld mismatches of %ld\n", pbad, pn);
  bad += pbad;
  // shared-denominator division against the IEEE quotient: random bit
  // patterns (all exponents, so the fallback is exercised), operands of
  // similar scale, and quotients next to rounding ties (a = b * m rounded,
  // m the midpoint of two neighbouring doubles)
  long dbad = 0, dn = 0;
  auto check_div = [&](double a, double b) {
    ++dn;
    const SharedDiv S = shared_div(b);
    if (!same(div_shared(S, a), a / b) || !same(qdiv_shared(S, a), qdiv(a, b))) {
      if (dbad < 5) printf("div_shared(%a, %a) = %a, want %a\n", a, b, div_shared(S, a), a / b);
      ++dbad;
    }
  };
  for (double a : v)
    for (double b : v) check_div(a, b);
  // power-of-two denominators (exact reciprocal, exponent-shift quotients)
  for (int e = -1074; e <= 1023; e += 3)
    for (double a : v) {
      check_div(a, std::ldexp(1.0, e));
      check_div(a, -std::ldexp(1.0, e));
    }
  for (int i = 0; i < 3000000; ++i) {
    unsigned long long ba = g(), bb = g();
    double a, b;
    memcpy(&a, &ba, 8);
    memcpy(&b, &bb, 8);
    check_div(a, b);
    a = std::ldexp(1.0 + (double)(g() >> 11) * 0x1p-53, (int)(g() % 1200) - 600);
    b = std::ldexp(1.0 + (double)(g() >> 11) * 0x1p-53, (int)(g() % 1200) - 600);
    if (g() & 1) a = -a;
    if (g() & 1) b = -b;
    check_div(a, b);
    // near ties: q and its successor, a = RN(b * midpoint) nudged by an ulp
    const double q = std::ldexp(1.0 + (double)(g() >> 11) * 0x1p-53, (int)(g() % 200) - 100);
    const double mid = q + (std::nextafter(q, 1e300) - q) * 0.5;  // rounds to q or next
    double a2 = b * mid;
    unsigned long long x;
    memcpy(&x, &a2, 8);
    x += (long long)(g() % 3) - 1;
    memcpy(&a2, &x, 8);
    check_div(a2, b);
    check_div(b * q, b);
  }
  if (dbad) printf("shared division: %ld mismatches of %ld\n", dbad, dn);
  // face lengths: axis-aligned (one exact zero) and general, all exponents
  long lbad2 = 0;
  for (int i = 0; i < 2000000; ++i) {
    unsigned long long ba = g(), bb = g();
    double a, b;
    memcpy(&a, &ba, 8);
    memcpy(&b, &bb, 8);
    if (i % 3 == 0) b = (g() & 1) ? 0.0 : -0.0;
    if (i % 3 == 1) a = (g() & 1) ? 0.0 : -0.0;
    if (i % 5 == 0) a = std::ldexp(1.0 + (double)(g() >> 11) * 0x1p-53, (int)(g() % 1200) - 600);
    double r = 0.0;
    r = r + a * a;
    r = r + b * b;
    if (!same(face_len(a, b), std::sqrt(r))) {
      if (lbad2 < 5) printf("face_len(%a, %a) = %a, want %a\n", a, b, face_len(a, b), std::sqrt(r));
      ++lbad2;
    }
  }
  bad += lbad2;
  bad += dbad;
  // limiter on gradient pairs: specials, random, and ratios near breakpoints
  std::vector<std::pair<double, double>> pairs;
  for (double a : v)
    for (double b : v) pairs.push_back({a, b});
  for (int i = 0; i < 400000; ++i) {
    double b = std::ldexp((double)(g() % 100000) + 1.0, (int)(g() % 60) - 50);
    if (g() & 1) b = -b;
    const double k[] = {0.5, 1.0, 2.0, 0.25, 4.0};
    double r = k[g() % 5];
    double a = b * r;
    unsigned long long ab;
    memcpy(&ab, &a, 8);
    ab += (long long)(g() % 5) - 2;  // a few ulps around the breakpoint
    memcpy(&a, &ab, 8);
    if (g() & 1) a = -a;
    pairs.push_back({a, b});
  }
  long lbad = 0;
  for (auto& pr : pairs)
    for (int id : {HYDRO_LIM_MINMOD, HYDRO_LIM_SUPERBEE}) {
      const double got = limit_grad1(id, pr.first, pr.second, 0, 0, 1, 1, 1);
      const double want = ref_limit(id, pr.first, pr.second);
      if (!same(got, want)) {
        if (lbad < 5)
          printf("limit_grad1(%d, %.17g, %.17g) = %.17g, want %.17g\n", id, pr.first,
                 pr.second, got, want);
        ++lbad;
      }
    }
  // order-3 face value with hoisted face constants vs the direct form
  long obad = 0, on = 0;
  for (int it = 0; it < 200000; ++it) {
    double h[6], y[6];
    for (int t = 0; t < 6; ++t) {
      h[t] = std::ldexp(1.0 + (double)(g() % 1000000) * 1e-6, -(int)(g() % 12));
      y[t] = (g() % 7 == 0) ? 0.0 : ((double)(g() % 2000000) - 1e6) * 1e-6;
    }
    if (g() % 5 == 0) y[2] = y[3];
    const double vdt = ((double)(g() % 2000001) - 1e6) * 1e-9 * (it % 3 ? 1.0 : 1e3);
    const double want = flux_ordre3(y[0], y[1], y[2], y[3], y[4], y[5], h[0], h[1],
                                    h[2], h[3], h[4], h[5], vdt);
    const O3Face F = o3_face(h, vdt);
    const double got = flux_ordre3_c(F, y);
    ++on;
    if (!same(got, want)) {
      if (obad < 5) printf("order3 mismatch: got %.17g want %.17g\n", got, want);
      ++obad;
    }
  }
  printf("compares: %ld value pairs, %ld mismatches; limiter: %zu pairs, %ld mismatches; "
         "order3: %ld faces, %ld mismatches\n",
         n, bad, pairs.size(), lbad, on, obad);
  return (bad || lbad || obad) ? 1 : 0;
}
