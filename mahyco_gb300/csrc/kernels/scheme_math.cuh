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
#include "softfp.cuh"

namespace hydro {

#define HD __host__ __device__ __forceinline__

// ---------------------------------------------------------------------------
// Comparisons on the integer pipe.  On GB300 a double comparison or min/max
// occupies the FP64 pipe like an addition (1/16 warp instruction per cycle
// and SM), and the hot kernels are bound by that pipe; the integer pipe is
// 32x wider.  Every helper below has exactly the IEEE semantics of the
// comparison it names: false when an operand is NaN, -0 == +0.
constexpr unsigned long long kMag = 0x7fffffffffffffffull;
constexpr unsigned long long kInfBits = 0x7ff0000000000000ull;

// The device reinterpretation is an opaque move: a plain bit cast lets the
// optimizer recognise the tests below (x == 0, isnan, isfinite, ...) and turn
// them back into FP64 comparisons, which run on the FP64 pipe.
HD unsigned long long ubits(double x) {
#ifdef __CUDA_ARCH__
  unsigned long long b;
  asm("mov.b64 %0, %1;" : "=l"(b) : "d"(x));
  return b;
#else
  unsigned long long b;
  __builtin_memcpy(&b, &x, sizeof b);
  return b;
#endif
}
HD double from_bits(unsigned long long b) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)b);
#else
  double x;
  __builtin_memcpy(&x, &b, sizeof x);
  return x;
#endif
}
HD bool is_nan(double x) { return (ubits(x) & kMag) > kInfBits; }
HD bool is_finite(double x) { return (ubits(x) & kInfBits) != kInfBits; }
// monotone signed key of a non-NaN double; both zeros map to 0
HD long long dkey(double x) {
  const unsigned long long b = ubits(x);
  const long long m = (long long)(b & kMag);
  return (b >> 63) ? -m : m;
}
HD bool dlt(double a, double b) { return !is_nan(a) && !is_nan(b) && dkey(a) < dkey(b); }
HD bool dle(double a, double b) { return !is_nan(a) && !is_nan(b) && dkey(a) <= dkey(b); }
HD bool dgt(double a, double b) { return dlt(b, a); }
HD bool dge(double a, double b) { return dle(b, a); }
// x > 0, x < 0, x >= 0, x <= 0
HD bool pos(double x) { return (unsigned long long)((long long)ubits(x) - 1) < kInfBits; }
HD bool neg(double x) {
  const unsigned long long m = ubits(x) & kMag;
  return (ubits(x) >> 63) && m != 0 && m <= kInfBits;
}
HD bool nonneg(double x) { return !is_nan(x) && !neg(x); }
HD bool nonpos(double x) { return !is_nan(x) && !pos(x); }
// x != 0 (true for NaN), x == 0
HD bool nz(double x) { return (ubits(x) & kMag) != 0; }
HD bool iszero(double x) { return (ubits(x) & kMag) == 0; }
// |x| < c, |x| > c for a constant c >= 0 (c not NaN)
HD bool abs_lt(double x, double c) { return (ubits(x) & kMag) < ubits(c); }
HD bool abs_gt(double x, double c) {
  const unsigned long long m = ubits(x) & kMag;
  return m > ubits(c) && m <= kInfBits;
}

// std::min / std::max: min(a,b) = (b<a)?b:a, max(a,b) = (a<b)?b:a
HD double smin(double a, double b) { return dlt(b, a) ? b : a; }
HD double smax(double a, double b) { return dlt(a, b) ? b : a; }

// Order-preserving 64-bit encoding of doubles (for atomicMin/atomicMax).
HD unsigned long long ord_bits(double x) {
  unsigned long long b = ubits(x);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
HD double from_ord(unsigned long long o) {
  unsigned long long b = (o >> 63) ? (o & 0x7fffffffffffffffull) : ~o;
  return from_bits(b);
}

// IEEE division behind a call: the optimizer cannot if-convert a branch
// around it into an unconditional division, so divisions on paths that are
// rarely taken cost nothing when they are not taken.
#ifdef __CUDA_ARCH__
static __device__ __noinline__ double ddiv_native(double n, double d) { return n / d; }
#else
static inline double ddiv_native(double n, double d) { return n / d; }
#endif
// n / d, the common case on the integer pipe (softfp.cuh), else the FP64
// division behind its call.  Bit-identical to n / d for all inputs.
HD double div_ip(double n, double d) {
  unsigned long long r;
  return sfp::div_fast(ubits(n), ubits(d), r) ? from_bits(r) : ddiv_native(n, d);
}

// n / d with the exact shortcuts decided on the integer pipe:
//   n = +-0, d finite non-zero   -> zero with sign(n) xor sign(d)
//   d = 1                        -> n
//   n = d, finite non-zero       -> 1
// (uniform and single-material cells produce many of these); otherwise the
// IEEE division.  Bit-identical to n / d (NaN results stay NaN).
//   d = +-2^k (normal), n normal, quotient normal -> n with its exponent
//                                   lowered by k and the sign xor-ed
// (a power-of-two denominator only shifts the exponent; the cell volume of a
// mesh with 2^-j spacing is one)
HD double qdiv(double n, double d) {
  const unsigned long long nb = ubits(n);
  const unsigned long long db = ubits(d);
  const bool dfin = ((db >> 52) & 0x7ffull) != 0x7ffull;
  const bool dnz = (db << 1) != 0ull;
  if ((nb << 1) == 0ull && dnz && dfin)
    return from_bits((nb ^ db) & 0x8000000000000000ull);
  if (db == 0x3ff0000000000000ull) return n;
  if (nb == db && dnz && dfin) return 1.0;
  const long long en = (long long)((nb >> 52) & 0x7ffull), ed = (long long)((db >> 52) & 0x7ffull);
  const long long er = en - ed + 1023;
  if ((db & 0xfffffffffffffull) == 0 && ed != 0 && ed != 0x7ff && en != 0 && en != 0x7ff &&
      er >= 1 && er <= 0x7fe)
    return from_bits(((nb ^ db) & 0x8000000000000000ull) | ((unsigned long long)er << 52) |
                     (nb & 0xfffffffffffffull));
  unsigned long long r;
  return sfp::div_fast(nb, db, r) ? from_bits(r) : ddiv_native(n, d);
}


// IEEE operations with their common case on the integer pipe (softfp.cuh):
// the fast path when it applies, else the FP64 instruction behind a call
// (so that the optimizer does not issue it under a predicate for every
// thread).  Bit-identical to the plain operators for all inputs.
#ifdef __CUDA_ARCH__
static __device__ __noinline__ double dmul_call(double a, double b) { return a * b; }
static __device__ __noinline__ double dadd_call(double a, double b) { return a + b; }
static __device__ __noinline__ double dsub_call(double a, double b) { return a - b; }
static __device__ __noinline__ double dsqrt_call(double a) { return sqrt(a); }
#else
static inline double dmul_call(double a, double b) { return a * b; }
static inline double dadd_call(double a, double b) { return a + b; }
static inline double dsub_call(double a, double b) { return a - b; }
static inline double dsqrt_call(double a) { return __builtin_sqrt(a); }
#endif
HD double mul_ip(double a, double b) {
  unsigned long long r;
  return sfp::mul_fast(ubits(a), ubits(b), r) ? from_bits(r) : dmul_call(a, b);
}
HD double add_ip(double a, double b) {
  unsigned long long r;
  return sfp::add_fast(ubits(a), ubits(b), r) ? from_bits(r) : dadd_call(a, b);
}
// a - b: the sum with b's sign flipped on the fast path (which takes no
// NaN); the fallback is the FP64 subtraction itself
HD double sub_ip(double a, double b) {
  unsigned long long r;
  return sfp::add_fast(ubits(a), ubits(b) ^ 0x8000000000000000ull, r) ? from_bits(r)
                                                                     : dsub_call(a, b);
}
HD double sqrt_ip(double a) {
  unsigned long long r;
  return sfp::sqrt_fast(ubits(a), r) ? from_bits(r) : dsqrt_call(a);
}

// Remap::fluxLimiter (remap/UtilesRemap.cc:9-23)
HD double flux_limiter(int id, double r) {
  if (id == HYDRO_LIM_MINMOD) return smax(0.0, smin(1.0, r));
  if (id == HYDRO_LIM_SUPERBEE)
    return smax(0.0, smax(smin(2.0 * r, 1.0), smin(r, 2.0)));
  if (id == HYDRO_LIM_VANLEER) {
    if (nonpos(r)) return 0.0;
    return 2.0 * r / (1.0 + r);
  }
  return 0.0;
}

// 2 * x, exactly as the IEEE product, for a non-NaN x, on the integer pipe.
HD double twice(double x) {
  const unsigned long long b = ubits(x), m = b & kMag, e = m >> 52;
  unsigned long long m2;
  if (e == 0)
    m2 = m << 1;                      // zero / subnormal: exact doubling
  else if (e >= 0x7fe)
    m2 = kInfBits;                    // overflow (or infinity)
  else
    m2 = m + (1ull << 52);            // exponent + 1
  return from_bits((b & ~kMag) | m2);
}

// x * 2^-K (K = 1: x * 0.5, K = 2: x * 0.25), exactly as the IEEE product,
// on the integer pipe: when the result is normal only the exponent field
// changes.  The rest (results in the subnormal range: the significand shifts
// with round-to-nearest-even; infinities and NaNs: the FP64 multiply) is the
// out-of-line slow path.
template <int K>
HD double mul_pow2m_slow(double x) {
  const unsigned long long b = ubits(x), m = b & kMag, e = m >> 52;
  if (e == 0x7ffull) return x * (K == 1 ? 0.5 : 0.25);
  // value = sig * 2^-1074 * 2^(e ? e - 1 : 0); result = value * 2^-K
  const unsigned long long sig = e ? ((m & 0xfffffffffffffull) | (1ull << 52)) : m;
  const int sh = e ? (K + 1 - (int)e) : K;  // 1 .. K
  const unsigned long long q = sig >> sh, r = sig & ((1ull << sh) - 1);
  const unsigned long long hw = 1ull << (sh - 1);
  const unsigned long long qq = q + ((r > hw || (r == hw && (q & 1ull))) ? 1ull : 0ull);
  return from_bits((b & ~kMag) | qq);
}
#ifdef __CUDA_ARCH__
template <int K>
static __device__ __noinline__ double mul_pow2m_call(double x) { return mul_pow2m_slow<K>(x); }
#else
template <int K>
static inline double mul_pow2m_call(double x) { return mul_pow2m_slow<K>(x); }
#endif
template <int K>
HD double mul_pow2m(double x) {
  const unsigned long long b = ubits(x);
  const unsigned e = (unsigned)(b >> 52) & 0x7ffu;
  if (e - (unsigned)(K + 1) < 0x7feu - (unsigned)K)  // K < e < 0x7ff
    return from_bits(b - ((unsigned long long)K << 52));
  if ((b << 1) == 0ull) return x;  // +-0 * 2^-K = +-0
  return mul_pow2m_call<K>(x);
}
// Several numerators over one denominator, each result the IEEE quotient
// a / b bit for bit: the divisor's integer reciprocal is formed once
// (softfp.cuh), each quotient then costs one high product and an exact
// remainder correction on the integer pipe.  Operands or quotients outside
// the normal range take the IEEE division.
struct SharedDiv {
  double b;
  sfp::Divisor d;
};
HD bool div_safe_exp(double x) {
  const unsigned e = (unsigned)(ubits(x) >> 52) & 0x7ffu;
  return e - (1023u - 500u) <= 1000u;  // 523 <= e <= 1523
}
HD SharedDiv shared_div(double b) {
  SharedDiv S;
  S.b = b;
  S.d = sfp::make_divisor(ubits(b));
  return S;
}
HD double fma_rn(double a, double b, double c) {
#ifdef __CUDA_ARCH__
  return __fma_rn(a, b, c);
#else
  return __builtin_fma(a, b, c);
#endif
}
HD double div_shared(const SharedDiv& S, double a) {
  unsigned long long r;
  return sfp::div_fast_by(ubits(a), S.d, r) ? from_bits(r) : ddiv_native(a, S.b);
}
// A face length as the reference forms it, sqrt(0.0 + a*a + b*b).  For an
// axis-aligned face (one component exactly zero) it is |a| (or |b|): the
// sum is the single square, and sqrt(RN(x*x)) = |x| for binary floating
// point with correct rounding whenever x*x neither overflows nor
// underflows (exponents within [-500, 500] here; checked on 2e8 values).
HD double face_len(double a, double b) {
  if (iszero(a) && iszero(b)) return 0.0;  // sqrt(+0)
  if (iszero(b) && div_safe_exp(a)) return fabs(a);
  if (iszero(a) && div_safe_exp(b)) return fabs(b);
  double r = mul_ip(a, a);  // 0.0 + a square (never -0) is the square
  r = add_ip(r, mul_ip(b, b));
  return sqrt_ip(r);
}

// qdiv's exact shortcuts (0 / d, x / 1, x / x), then div_shared
HD double qdiv_shared(const SharedDiv& S, double n) {
  const unsigned long long nb = ubits(n);
  const unsigned long long db = ubits(S.b);
  const bool dfin = ((db >> 52) & 0x7ffull) != 0x7ffull;
  const bool dnz = (db << 1) != 0ull;
  if ((nb << 1) == 0ull && dnz && dfin)
    return from_bits((nb ^ db) & 0x8000000000000000ull);
  if (db == 0x3ff0000000000000ull) return n;
  if (nb == db && dnz && dfin) return 1.0;
  // a power-of-two denominator only shifts the exponent (normal operands
  // and quotient)
  const long long en = (long long)((nb >> 52) & 0x7ffull), ed = (long long)((db >> 52) & 0x7ffull);
  const long long er = en - ed + 1023;
  if ((db & 0xfffffffffffffull) == 0 && ed != 0 && ed != 0x7ff && en != 0 && en != 0x7ff &&
      er >= 1 && er <= 0x7fe)
    return from_bits(((nb ^ db) & 0x8000000000000000ull) | ((unsigned long long)er << 52) |
                     (nb & 0xfffffffffffffull));
  return div_shared(S, n);
}

// x / k for k = 1, 2 or 4, as the exact multiplication by 1/k (division by
// a power of two and multiplication by its reciprocal round identically).
HD double div_pow2(double x, int k) {
  return k == 4 ? mul_pow2m<2>(x) : (k == 2 ? mul_pow2m<1>(x) : x);
}
HD double half(double x) { return mul_pow2m<1>(x); }
HD double quarter(double x) { return mul_pow2m<2>(x); }
// 2 * x for any x: exponent + 1 while the result stays finite and normal;
// zeros, subnormals, overflow, infinities and NaNs through twice / the FP64
// multiply
#ifdef __CUDA_ARCH__
static __device__ __noinline__ double dbl_slow(double x) { return is_nan(x) ? 2.0 * x : twice(x); }
#else
static inline double dbl_slow(double x) { return is_nan(x) ? 2.0 * x : twice(x); }
#endif
HD double dbl(double x) {
  const unsigned long long b = ubits(x);
  const unsigned e = (unsigned)(b >> 52) & 0x7ffu;
  if (e - 1u < 0x7fdu) return from_bits(b + (1ull << 52));  // 1 <= e <= 0x7fd
  if ((b << 1) == 0ull) return x;  // 2 * +-0 = +-0
  return dbl_slow(x);
}
// x + 0.0 (turns -0 into +0; NaN through the FP64 addition, behind a call:
// inline, the select would issue the addition for every value)
HD double plus_zero(double x) {
  const unsigned long long b = ubits(x);
  if (b == 0x8000000000000000ull) return 0.0;
  return is_nan(x) ? dadd_call(x, 0.0) : x;
}
// f * x for a volume or mass fraction f: in single-material cells the
// fractions are exactly 1 or +0, and the product is x or the IEEE product's
// signed zero (NaN for a non-finite x), decided on the integer pipe
HD double mul_frac(double f, double x) {
  const unsigned long long b = ubits(f);
  if (b == 0x3ff0000000000000ull) return x;
  if (b == 0ull && is_finite(x)) return from_bits(ubits(x) & ~kMag);
  // a mixed cell (inline: behind a call, the callers' register allocation
  // around it costs the Lagrange cell kernel more than the product saves)
  return f * x;
}

// a + b, a - b and a * b with the exact shortcuts of zero operands decided on
// the integer pipe (fields at rest are mostly zeros: velocities, fluxes,
// slopes).  IEEE, round to nearest: x + (+-0) = x for every non-NaN x != 0;
// two zeros sum to -0 only when both are -0; x - x = +0 for finite x; a zero
// times a finite number is the zero of the xor of the signs.  Otherwise (and
// whenever a NaN or an infinity could decide the result) the FP64
// instruction runs.  Bit-identical to the plain operators.
HD double addz(double a, double b) {
  const unsigned long long ua = ubits(a), ub = ubits(b);
  const unsigned long long ma = ua & kMag, mb = ub & kMag;
  if (mb == 0 && ma <= kInfBits) return from_bits(ma == 0 ? (ua & ub) : ua);
  if (ma == 0 && mb <= kInfBits) return b;
  if ((ua ^ ub) == ~kMag && ma < kInfBits) return 0.0;  // a + (-a)
  return a + b;
}
// The bits of a + b when one of addz's shortcuts gives them; false when the
// sum needs the FP64 addition (which this form never issues).
HD bool addz_bits(double a, double b, unsigned long long& r) {
  const unsigned long long ua = ubits(a), ub = ubits(b);
  const unsigned long long ma = ua & kMag, mb = ub & kMag;
  if (mb == 0 && ma <= kInfBits) {
    r = (ma == 0) ? (ua & ub) : ua;
    return true;
  }
  if (ma == 0 && mb <= kInfBits) {
    r = ub;
    return true;
  }
  if ((ua ^ ub) == ~kMag && ma < kInfBits) {
    r = 0ull;
    return true;
  }
  return false;
}
// a - b = a + (-b) exactly; the sign of b is flipped on the integer pipe
// (a negated double operand may otherwise cost an FP64 instruction)
HD double subz(double a, double b) {
  return addz(a, from_bits(ubits(b) ^ 0x8000000000000000ull));
}
HD double mulz(double a, double b) {
  const unsigned long long ua = ubits(a), ub = ubits(b);
  const unsigned long long ma = ua & kMag, mb = ub & kMag;
  if ((ma == 0 && mb < kInfBits) || (mb == 0 && ma < kInfBits))
    return from_bits((ua ^ ub) & ~kMag);
  return a * b;
}
// a * b with the shortcuts of mulz and of a factor exactly 1 (1 * x = x for
// every non-NaN x)
HD double mul1z(double a, double b) {
  constexpr unsigned long long kOne = 0x3ff0000000000000ull;
  const unsigned long long ua = ubits(a), ub = ubits(b);
  if (ub == kOne && (ua & kMag) <= kInfBits) return a;
  if (ua == kOne && (ub & kMag) <= kInfBits) return b;
  return mulz(a, b);
}

// Lagrangian geometry of a VNR cell from its four node positions
// (updateCellPos, computeSubVol, vnr_remap/PhaseLagrange.cc:210-296; the
// Lagrangian centroid, vnr_remap/PrepareRemap.cc:65-90; the face lengths
// behind HvLagrange, remap/PhaseRemap1.cc:57-71): volume (sum of the four
// sub-volumes around the node-averaged centre), centroid, and the widths
// along x / y (order > 1).  Sums from 0.0 start with plus_zero.
struct CellGeom {
  double vol, xc0, xc1, hx, hy;
};
// sqrt(dot(a, a)) with the dot product accumulated from 0.0
// (includes/Freefunctions.h:15-20)
HD double norm2(double a, double b) {
  double r = 0.0;
  r = r + a * a;
  r = r + b * b;
  return sqrt_ip(r);
}
// Corner normal l+ n+ + l- n- of a node xp between its successor xpp and
// predecessor xpm in the cell's node order (includes/Freefunctions.h:28-58,
// computeLpcNpc)
HD void lpc_npc(const double* xp, const double* xpp, const double* xpm, double out[2]) {
  const double a0 = 0.5 * (xpp[1] - xp[1]), a1 = 0.5 * (xp[0] - xpp[0]);
  const double la = norm2(a0, a1);
  const double na0 = div_ip(a0, la), na1 = div_ip(a1, la);
  const double b0 = 0.5 * (xp[1] - xpm[1]), b1 = 0.5 * (xpm[0] - xp[0]);
  const double lb = norm2(b0, b1);
  const double nb0 = div_ip(b0, lb), nb1 = div_ip(b1, lb);
  out[0] = na0 * la + nb0 * lb;
  out[1] = na1 * la + nb1 * lb;
}

HD CellGeom vnr_cell_geometry(const double X[4][2], bool widths) {
  CellGeom G;
  double xc0 = plus_zero(X[0][0]), xc1 = plus_zero(X[0][1]);
#pragma unroll
  for (int k = 1; k < 4; ++k) {
    xc0 = xc0 + X[k][0];
    xc1 = xc1 + X[k][1];
  }
  xc0 = quarter(xc0);
  xc1 = quarter(xc1);
  double vol = 0.0;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int km = (k + 3) & 3, kp = (k + 1) & 3;
    const double x2a = half(X[km][0] + X[k][0]), x2b = half(X[km][1] + X[k][1]);
    const double x4a = half(X[kp][0] + X[k][0]), x4b = half(X[kp][1] + X[k][1]);
    const double c12 = xc0 * x2b - xc1 * x2a;
    const double c23 = x2a * X[k][1] - x2b * X[k][0];
    const double c34 = X[k][0] * x4b - X[k][1] * x4a;
    const double c41 = x4a * xc1 - x4b * xc0;
    const double t = half(c12 + c23 + c34 + c41);
    vol = (k == 0) ? plus_zero(t) : vol + t;
  }
  G.vol = vol;
  double r0 = 0.0, r1 = 0.0;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int kp = (k + 1) & 3;
    const double cr = X[k][0] * X[kp][1] - X[k][1] * X[kp][0];
    const double t0 = cr * (X[k][0] + X[kp][0]), t1 = cr * (X[k][1] + X[kp][1]);
    r0 = (k == 0) ? plus_zero(t0) : r0 + t0;
    r1 = (k == 0) ? plus_zero(t1) : r1 + t1;
  }
  const double sc = div_ip(1.0, 6.0 * vol);
  G.xc0 = sc * r0;
  G.xc1 = sc * r1;
  G.hx = G.hy = 0.0;
  if (widths) {
    auto len = [&](int a, int b) { return face_len(X[b][0] - X[a][0], X[b][1] - X[a][1]); };
    // lengths are >= +0: 0.0 + the first half-length is that half-length
    G.hx = half(len(0, 1));  // bottom face
    G.hx += half(len(3, 2)); // top face
    G.hy = half(len(1, 2));  // right face
    G.hy += half(len(0, 3)); // left face
  }
  return G;
}

// Lagrangian geometry of an Eucclhyd cell from its four node positions
// (computeLagrangeVolumeAndCenterOfGravity, eucclhyd_remap/PhaseLagrange.cc
// :671-716; the face lengths behind HvLagrange, remap/PhaseRemap1.cc:57-71):
// volume (half the shoelace sum), centroid, widths along x / y (order > 1).
HD CellGeom euc_cell_geometry(const double X[4][2], bool widths) {
  CellGeom G;
  double r6 = 0.0;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int kp = (k + 1) & 3;
    const double t = X[k][0] * X[kp][1] - X[k][1] * X[kp][0];
    r6 = (k == 0) ? plus_zero(t) : r6 + t;
  }
  G.vol = half(r6);
  double r7a = 0.0, r7b = 0.0;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int kp = (k + 1) & 3;
    const double cr = X[k][0] * X[kp][1] - X[k][1] * X[kp][0];
    const double ta = (X[k][0] + X[kp][0]) * cr, tb = (X[k][1] + X[kp][1]) * cr;
    r7a = (k == 0) ? plus_zero(ta) : r7a + ta;
    r7b = (k == 0) ? plus_zero(tb) : r7b + tb;
  }
  const double sc = div_ip(1.0, 6.0 * G.vol);
  G.xc0 = r7a * sc;
  G.xc1 = r7b * sc;
  G.hx = G.hy = 0.0;
  if (widths) {
    auto len = [&](int a, int b) { return face_len(X[b][0] - X[a][0], X[b][1] - X[a][1]); };
    // lengths are >= +0: 0.0 + the first half-length is that half-length
    G.hx = half(len(0, 1));
    G.hx += half(len(3, 2));
    G.hy = half(len(1, 2));
    G.hy += half(len(0, 3));
  }
  return G;
}

// x * n, with n = +1 or -1 (the outer normals of the Cartesian Euler mesh)
// decided on the integer pipe: x or -x, exactly the IEEE products
HD double mul_pm1(double x, double n) {
  const unsigned long long b = ubits(n);
  if (b == 0x3ff0000000000000ull) return x;
  if (b == 0xbff0000000000000ull) return from_bits(ubits(x) ^ 0x8000000000000000ull);
  return dmul_call(x, n);
}

// k * x for a small integer k in {0, 1, 2} (k = 0: the IEEE product's signed
// zero, or NaN for a non-finite x)
HD double mul_012(int k, double x) {
  if (k == 1) return x;
  if (k == 2) return dbl(x);
  return is_finite(x) ? from_bits(ubits(x) & ~kMag) : dmul_call(0.0, x);
}

// minmod / superBee limiter of a quotient that is not NaN, with the
// comparisons on the integer pipe (same values as flux_limiter).
HD double flux_limiter_q(int id, double r) {
  const long long one = 0x3ff0000000000000ll, two = 0x4000000000000000ll;
  // for non-NaN x: x < c  <=>  signed bits(x) < bits(c) when c > 0
  const long long br = (long long)ubits(r);
  if (id == HYDRO_LIM_MINMOD) {
    const double t = (br < one) ? r : 1.0;          // smin(1.0, r)
    return ((long long)ubits(t) > 0) ? t : 0.0;     // smax(0.0, t)
  }
  const double u = twice(r);
  const double s1 = ((long long)ubits(u) > one) ? 1.0 : u;  // smin(2r, 1.0)
  const double s2 = (br > two) ? 2.0 : r;                   // smin(r, 2.0)
  const double w = (dkey(s1) < dkey(s2)) ? s2 : s1;        // smax(s1, s2)
  return ((long long)ubits(w) > 0) ? w : 0.0;              // smax(0.0, w)
}

// divideNoExcept (includes/Freefunctions.h:86-92)
HD double divide_no_except(double a, double b) {
  if (abs_lt(b, 1.0E-12)) return 0.0;
  return qdiv(a, b);
}

// Remap::fluxLimiterPP (remap/UtilesRemap.cc:25-72)
HD double flux_limiter_pp(int id, double gp, double gm, double yp, double ym,
                          double h0, double hp, double hm) {
  double grady = 0.0;
  if (neg(gp * gm)) return 0.;
  if (id == HYDRO_LIM_MINMODG) {
    grady = pos(yp - ym) ? smin(fabs(gp), fabs(gm)) : -smin(fabs(gp), fabs(gm));
  } else if (id == HYDRO_LIM_SUPERBEEG) {
    grady = pos(yp - ym) ? smax(fabs(gp), fabs(gm)) : -smax(fabs(gp), fabs(gm));
  } else if (id == HYDRO_LIM_VANLEERG) {
    double lp = div_ip(half(h0) + hp, h0 + hp + hm);
    double lm = div_ip(half(h0) + hm, h0 + hp + hm);
    if (nz(lp * gp + lm * gm))
      grady = div_ip(gp * gm, lp * gp + lm * gm);
    else
      grady = 0.;
  } else if (id == HYDRO_LIM_ULTRABEEG) {
    grady = div_ip(yp - ym, h0);
  } else if (id == HYDRO_LIM_ARITHMETICG) {
    double lp = div_ip(half(h0) + hp, h0 + hp + hm);
    double lm = div_ip(half(h0) + hm, h0 + hp + hm);
    grady = lm * gp + lp * gm;
  }
  double gMp = div_ip(gp * (h0 + hp), h0);
  double gMm = div_ip(gm * (h0 + hm), h0);
  double gM = smin(fabs(gMp), fabs(gMm));
  if (pos(yp - ym))
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
// the generalised limiters out of line: runs use one limiter, and the
// minmod / superBee kernels need not carry these registers
#ifdef __CUDA_ARCH__
static __device__ __noinline__ double flux_limiter_pp_call(int id, double gp, double gm,
                                                           double yp, double ym, double h0,
                                                           double hp, double hm) {
  return flux_limiter_pp(id, gp, gm, yp, ym, h0, hp, hm);
}
#else
static inline double flux_limiter_pp_call(int id, double gp, double gm, double yp, double ym,
                                          double h0, double hp, double hm) {
  return flux_limiter_pp(id, gp, gm, yp, ym, h0, hp, hm);
}
#endif
HD double limit_grad1(int id, double gp, double gm, double yp, double ym,
                      double h0, double hp, double hm) {
  if (id >= HYDRO_LIM_MINMODG) return flux_limiter_pp_call(id, gp, gm, yp, ym, h0, hp, hm);
  if ((id == HYDRO_LIM_MINMOD || id == HYDRO_LIM_SUPERBEE) && is_finite(gp) &&
      is_finite(gm)) {
    // every case needs at most one quotient: q = gp / gm gives phi(r1)
    // (which = 1), q = gm / gp gives phi(r2) (which = 2); the other phi is
    // a constant.  One division call site for the whole warp.
    const unsigned long long ma = ubits(gp) & kMag, mb = ubits(gm) & kMag;
    const unsigned long long eps = 0x3d719799812dea11ull;  // bits of 1.0E-12
    int which;
    double c1, c2;  // the constant phi(r1) / phi(r2) of the case
    bool zero_q = false;
    if (mb < eps) {  // b < 1e-12: phi(r1) = 0, r2 = divideNoExcept(gm, gp)
      which = 2;
      c1 = 0.0;
      c2 = 0.0;
      zero_q = ma < eps;
    } else if (ma < eps) {  // a < 1e-12: phi(r2) = 0
      which = 1;
      c1 = 0.0;
      c2 = 0.0;
    } else if ((ubits(gp) ^ ubits(gm)) >> 63) {  // opposite signs (non-zero)
      which = 0;
      c1 = 0.0;
      c2 = 0.0;
    } else if (id == HYDRO_LIM_MINMOD) {
      which = (ma <= mb) ? 1 : 2;  // the other ratio is >= 1: phi = 1
      c1 = 1.0;
      c2 = 1.0;
    } else {  // superBee: 2r on [0,1/2], 1 on [1/2,1], r on [1,2], 2 above
      // 0.5 * b and 2 * b exactly (b >= 1e-12 is normal)
      const unsigned long long hb = mb - (1ull << 52);
      const unsigned long long db = (mb >= 0x7fe0000000000000ull) ? kInfBits : mb + (1ull << 52);
      if (ma <= hb) {
        which = 1;
        c2 = 2.0;  // r2 >= 2
        c1 = 0.0;
      } else if (ma <= mb) {
        which = 2;
        c1 = 1.0;  // r1 in [1/2, 1]
        c2 = 0.0;
      } else if (ma <= db) {
        which = 1;
        c2 = 1.0;  // r2 in [1/2, 1]
        c1 = 0.0;
      } else {
        which = 2;
        c1 = 2.0;  // r1 >= 2
        c2 = 0.0;
      }
    }
    const bool dodiv = which != 0 && !zero_q;
    const double num = dodiv ? (which == 1 ? gp : gm) : 0.0;
    const double den = dodiv ? (which == 1 ? gm : gp) : 1.0;
    const double phi = flux_limiter_q(id, qdiv(num, den));
    const double f1 = (which == 1) ? phi : c1;
    const double f2 = (which == 2) ? phi : c2;
    return half(f1 * gm + f2 * gp);
  }
  return (flux_limiter(id, divide_no_except(gp, gm)) * gm +
          flux_limiter(id, divide_no_except(gm, gp)) * gp) *
         0.5;
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
    y0p = div_ip((h0 + hm) * yp + h0 * ym, dbl(h0) + hm);
    y0m = div_ip((h0 + hp) * ym + h0 * yp, dbl(h0) + hp);
  } else if (id == HYDRO_LIM_VANLEERG || id == HYDRO_LIM_VANLEER) {
    double a = smin(yp, ym);
    double b = smax(yp, ym);
    double xp = (h0 * h0 + 3 * h0 * hm + 2 * hm * hm) * yp;
    double xm = (h0 * h0 + 3 * h0 * hp + 2 * hp * hp) * ym;
    xp += (h0 * h0 - h0 * hp - 2 * hp * hp + 2 * h0 * hm) * ym;
    xm += (h0 * h0 - h0 * hm - 2 * hm * hm + 2 * h0 * hp) * yp;
    xp = div_ip(xp, 2 * h0 * h0 + 5 * h0 * hm + 2 * hm * hm - h0 * hp - 2 * hp * hp);
    xm = div_ip(xm, 2 * h0 * h0 + 5 * h0 * hp + 2 * hp * hp - h0 * hm - 2 * hm * hm);
    y0p = smin(smax(xp, a), b);
    y0m = smin(smax(xm, a), b);
  } else if (id == HYDRO_LIM_ULTRABEEG) {
    y0p = half(yp + ym);
    y0m = half(yp + ym);
  } else if (id == HYDRO_LIM_ARITHMETICG) {
    y0p = div_ip((h0 + hm + hp) * yp + h0 * ym, dbl(h0) + hm + hp);
    y0m = div_ip((h0 + hm + hp) * ym + h0 * yp, dbl(h0) + hm + hp);
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
  if (abs_gt(d, 1.e-14)) {
    const double n = X - x0;
    double eta;
    const bool fin = is_finite(n) && is_finite(d);
    if (fin && (pos(d) ? nonpos(n) : nonneg(n)))
      eta = 0.;
    else if (fin && (pos(d) ? dge(n, d) : dle(n, d)))
      eta = 1.;
    else
      eta = smin(smax(0., div_ip(n, d)), 1.);
    flux = (y0 + half(eta) * (y1 - y0)) * d * eta;
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
  if (dgt(fabs(y0p - yp), thr)) xp = qdiv(y0 - yp, y0p - yp) - 0.5;
  if (dgt(fabs(y0m - ym), thr)) xm = qdiv(y0 - ym, y0m - ym) - 0.5;
  PPShape s;
  s.xd = +h0 * smin(smax(xp, -0.5), 0.5);
  s.xg = -h0 * smin(smax(xm, -0.5), 0.5);
  double xtd = y0 + half(h0) * grad;
  double xtg = y0 - half(h0) * grad;
  double ad = smin(yp, dbl(y0m) - ym);
  double bd = smax(yp, dbl(y0m) - ym);
  double ag = smin(ym, dbl(y0p) - yp);
  double bg = smax(ym, dbl(y0p) - yp);
  s.yd = smin(smax(xtd, ad), bd);
  s.yg = smin(smax(xtg, ag), bg);
  return s;
}

// Integral of the reconstruction between a and b (the three pieces of
// computeFluxPP, remap/UtilesRemap-Impl.h:182-257), clipped at 0, with the
// "formule 16" replacement at extrema.
HD double pp_integral(const PPShape& s, double a, double b, double h0,
                      double y0, double yp, double ym, double ppv) {
  double f1b = int2y(b, half(-h0), ym, s.xg, s.yg);
  double f1a = int2y(a, half(-h0), ym, s.xg, s.yg);
  double f2b = int2y(b, s.xg, s.yg, s.xd, s.yd);
  double f2a = int2y(a, s.xg, s.yg, s.xd, s.yd);
  double f3b = int2y(b, s.xd, s.yd, half(h0), yp);
  double f3a = int2y(a, s.xd, s.yd, half(h0), yp);
  double F = smax(((f1b - f1a) + (f2b - f2a) + (f3b - f3a)), 0.);
  if (nonneg((yp - y0) * (ym - y0))) F = y0 * ppv;
  return F;
}

// order-3 face value (remap/UtilesRemap.cc:200-320)
HD double eval_grad(double hm, double h0, double hp, double ym, double y0,
                    double yp) {
  return div_ip(h0, hm + h0 + hp) *
         (div_ip(2. * hm + h0, h0 + hp) * (yp - y0) +
          div_ip(h0 + 2. * hp, hm + h0) * (y0 - ym));
}
HD double eval_ystar(double hmm, double hm, double hp, double hpp, double ymm,
                     double ym, double yp, double ypp, double gradm,
                     double gradp) {
  double tmp1 = div_ip(2. * hp * hm, hm + hp) *
                (div_ip(hmm + hm, 2. * hm + hp) - div_ip(hpp + hp, 2. * hp + hm)) *
                (yp - ym);
  double tmp2 = div_ip(-hm * (hmm + hm), 2. * hm + hp) * gradp +
                div_ip(hp * (hp + hpp), hm + 2. * hp) * gradm;
  return ym + div_ip(hm, hm + hp) * (yp - ym) +
         div_ip(1., hmm + hm + hp + hpp) * (tmp1 + tmp2);
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
  if (nonneg(vdt)) {
    double x = vdt, dx = hm;
    flux = ystar - div_ip(0.5 * x, dx) * (grad_m - (1. - div_ip(2. / 3. * x, dx)) * ym6);
  } else {
    double x = -vdt, dx = hp;
    flux = ystar + div_ip(0.5 * x, dx) * (grad_p - (1. - div_ip(2. / 3. * x, dx)) * yp6);
  }
  double num = div_ip(vdt, hm), nup = div_ip(vdt, hp);
  double ym_ym = ym + div_ip(1. - num, num) * (ym - ymm);
  double yp_ym = yp - div_ip(1. + nup, nup) * (yp - ypp);
  double i1inf = smin(ym, yp), i1sup = smax(ym, yp), i2inf, i2sup;
  if (nonneg(vdt)) {
    i2inf = smin(ym, ym_ym);
    i2sup = smax(ym, ym_ym);
  } else {
    i2inf = smin(yp, yp_ym);
    i2sup = smax(yp, yp_ym);
  }
  double linf, lsup;
  if (dlt(i1sup, i2inf) || dlt(i2sup, i1inf)) {
    linf = 0.;
    lsup = 0.;
  } else {
    linf = smax(i1inf, i2inf);
    lsup = smin(i1sup, i2sup);
  }
  if (dlt(flux, linf)) flux = linf;
  if (dgt(flux, lsup)) flux = lsup;
  return flux;
}

// The order-3 face value with its face constants hoisted: every division
// of flux_ordre3 depends only on the six cell widths and on vdt, so they are
// evaluated once per face (o3_face) and reused for every component
// (flux_ordre3_c).  Each expression keeps the operation order of
// eval_grad / eval_ystar / flux_ordre3 above, so the value is bit-identical.
struct O3Face {
  double G0[4], A[4], B[4];                  // eval_grad coefficients
  double T1[3], T2[3], T3[3], T4[3], T5[3];  // eval_ystar coefficients
  double Q1, Q2;                             // 0.5 x / dx, 2/3 x / dx
  double R1, R2;                             // (1 - nu-) / nu-, (1 + nu+) / nu+
  bool fwd;                                  // vdt >= 0
};
// eval_grad's coefficients for a cell of width h0 between widths hm, hp
HD void o3_grad_coef(double hm, double h0, double hp, double& G0, double& A, double& B) {
  G0 = div_ip(h0, hm + h0 + hp);
  A = div_ip(2. * hm + h0, h0 + hp);
  B = div_ip(h0 + 2. * hp, hm + h0);
}
// eval_ystar's coefficients for a face between widths hm | hp, with the
// next widths hmm, hpp outside
HD void o3_ystar_coef(double hmm, double hm, double hp, double hpp, double* T) {
  T[0] = div_ip(2. * hp * hm, hm + hp) *
         (div_ip(hmm + hm, 2. * hm + hp) - div_ip(hpp + hp, 2. * hp + hm));
  T[1] = div_ip(-hm * (hmm + hm), 2. * hm + hp);
  T[2] = div_ip(hp * (hp + hpp), hm + 2. * hp);
  T[3] = div_ip(hm, hm + hp);
  T[4] = div_ip(1., hmm + hm + hp + hpp);
}
// the face's coefficients that depend on vdt
HD void o3_face_dt(O3Face& F, const double* h, double vdt) {
  F.fwd = nonneg(vdt);
  const double x = F.fwd ? vdt : -vdt, dx = F.fwd ? h[2] : h[3];
  F.Q1 = div_ip(0.5 * x, dx);
  F.Q2 = div_ip(2. / 3. * x, dx);
  const double num = div_ip(vdt, h[2]), nup = div_ip(vdt, h[3]);
  F.R1 = div_ip(1. - num, num);
  F.R2 = div_ip(1. + nup, nup);
}
HD O3Face o3_face(const double* h, double vdt) {
  O3Face F;
#pragma unroll
  for (int g = 0; g < 4; ++g)  // eval_grad(h[g], h[g+1], h[g+2], ...)
    o3_grad_coef(h[g], h[g + 1], h[g + 2], F.G0[g], F.A[g], F.B[g]);
#pragma unroll
  for (int g = 0; g < 3; ++g) {  // eval_ystar(h[g], .., h[g+3], ...)
    double T[5];
    o3_ystar_coef(h[g], h[g + 1], h[g + 2], h[g + 3], T);
    F.T1[g] = T[0];
    F.T2[g] = T[1];
    F.T3[g] = T[2];
    F.T4[g] = T[3];
    F.T5[g] = T[4];
  }
  o3_face_dt(F, h, vdt);
  return F;
}
// eval_grad with its coefficients
// A uniform row (the three values equal bit for bit, finite) has zero
// differences: A * (+0) + B * (+0) is the zero -0 only when A and B are both
// negative, times G0 (finite coefficients) the zero of the xor with G0's
// sign.  One coarse test, so that the arithmetic is branched over rather
// than issued under a predicate.
HD double o3_grad(double G0, double A, double B, double ym, double y0, double yp) {
  const unsigned long long b0 = ubits(y0);
  if (ubits(ym) == b0 && ubits(yp) == b0 && is_finite(y0) && is_finite(G0) && is_finite(A) &&
      is_finite(B))
    return from_bits(((ubits(A) & ubits(B)) ^ ubits(G0)) & ~kMag);
  return G0 * (A * (yp - y0) + B * (y0 - ym));
}
// eval_ystar with its coefficients T (o3_ystar_coef) at the face between
// ym | yp, from the gradients of the cells on its minus / plus side
// Equal values (bit for bit, finite) and zero gradients with finite
// coefficients: every term after ym is a signed zero, so the value is ym
// when ym is not zero; for a zero ym it is the zero the sign rules give
// (x + y of two zeros is -0 only when both are -0, a zero product has the
// xor of the signs).  One coarse test, as in o3_grad.
HD double o3_ystar(const double* T, double ym, double yp, double grm, double grp) {
  if (ubits(yp) == ubits(ym) && is_finite(ym) && iszero(grm) && iszero(grp) &&
      is_finite(T[0]) && is_finite(T[1]) && is_finite(T[2]) && is_finite(T[3]) &&
      is_finite(T[4])) {
    if (nz(ym)) return ym;
    // yp - ym = +0; T3 (+0) has T3's sign; T0 (+0) + (T1 grp + T2 grm)
    const unsigned long long t2 = (ubits(T[1]) ^ ubits(grp)) & (ubits(T[2]) ^ ubits(grm));
    const unsigned long long z2 = ubits(T[4]) ^ (ubits(T[0]) & t2);
    return from_bits(ubits(ym) & ubits(T[3]) & z2 & ~kMag);
  }
  const double tmp1 = T[0] * (yp - ym);
  const double tmp2 = T[1] * grp + T[2] * grm;
  return ym + T[3] * (yp - ym) + T[4] * (tmp1 + tmp2);
}
// the face value from the interpolated values ys of the faces at -1, 0, +1
// and the cell values y1 | ym | yp | y4 (ComputeFluxOrdre3's parabola and
// its TVD interval)
HD double o3_tail(const O3Face& F, const double* ys, double y1, double ym, double yp,
                  double y4) {
  const double grad_m = ys[1] - ys[0], grad_p = ys[2] - ys[1];
  const double ym6 = 6. * (ym - 0.5 * (ys[0] + ys[1]));
  const double yp6 = 6. * (yp - 0.5 * (ys[1] + ys[2]));
  double flux;
  if (F.fwd)
    flux = ys[1] - F.Q1 * (grad_m - (1. - F.Q2) * ym6);
  else
    flux = ys[1] + F.Q1 * (grad_p - (1. - F.Q2) * yp6);
  const double ym_ym = ym + F.R1 * (ym - y1);
  const double yp_ym = yp - F.R2 * (yp - y4);
  const double i1inf = smin(ym, yp), i1sup = smax(ym, yp);
  double i2inf, i2sup;
  if (F.fwd) {
    i2inf = smin(ym, ym_ym);
    i2sup = smax(ym, ym_ym);
  } else {
    i2inf = smin(yp, yp_ym);
    i2sup = smax(yp, yp_ym);
  }
  double linf, lsup;
  if (dlt(i1sup, i2inf) || dlt(i2sup, i1inf)) {
    linf = 0.;
    lsup = 0.;
  } else {
    linf = smax(i1inf, i2inf);
    lsup = smin(i1sup, i2sup);
  }
  if (dlt(flux, linf)) flux = linf;
  if (dgt(flux, lsup)) flux = lsup;
  return flux;
}
HD double flux_ordre3_c(const O3Face& F, const double* y) {
  double gr[4];
#pragma unroll
  for (int g = 0; g < 4; ++g) gr[g] = o3_grad(F.G0[g], F.A[g], F.B[g], y[g], y[g + 1], y[g + 2]);
  double ys[3];
#pragma unroll
  for (int g = 0; g < 3; ++g) {
    const double T[5] = {F.T1[g], F.T2[g], F.T3[g], F.T4[g], F.T5[g]};
    ys[g] = o3_ystar(T, y[g + 1], y[g + 2], gr[g], gr[g + 1]);
  }
  return o3_tail(F, ys, y[1], y[2], y[3], y[4]);
}

}  // namespace hydro
#endif
