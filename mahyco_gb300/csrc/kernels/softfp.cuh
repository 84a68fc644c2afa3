// Binary64 arithmetic on the integer pipe, correctly rounded (IEEE 754
// round-to-nearest-even), for the FP64-bound kernels.
//
// On GB300 the FP64 pipe of an SM sub-partition completes one warp
// instruction every 64 cycles (1.25 TFLOP/s for the whole GPU), while its
// integer and FP32 pipes each take one every 2 cycles.  An IEEE division or
// square root on the FP64 pipe is a sequence of about seven FP64
// instructions (~450 cycles per warp); the same correctly rounded result
// formed from integer products takes a few tens of integer instructions.
// Products and sums can move too, to balance the two pipes.
//
// Each operation has a fast path for the common case -- normal operands, a
// normal result, and zeros where their rules are simple -- and returns
// false for everything else (subnormals, infinities, NaNs, results that
// would overflow or underflow); the callers then use the FP64 instruction,
// so special cases keep the hardware's exact behaviour, including its NaN
// encodings.  Correct rounding makes the result unique: a fast path gives
// exactly the bits of the FP64 instruction.
//
// Methods (restated from the mathematics, not from any library):
//  - product: the exact 106-bit product of the 53-bit significands, the
//    53 bits above the rounding position, a round bit and a sticky bit;
//  - sum: alignment with a "jamming" right shift (lost bits ORed into the
//    last of 10 guard bits), one normalisation step, or a count of leading
//    zeros after cancellation, as in the classic guard / round / sticky
//    adder (e.g. Goldberg, "What every computer scientist should know about
//    floating-point arithmetic", 1991);
//  - quotient: a 24-bit FP32 reciprocal estimate (rcp.approx), one
//    Newton-Raphson step z <- z + z (1 - d z) on 32-bit halves and one in
//    64-bit fixed point, arranged so that the reciprocal never exceeds
//    1/d (a Newton step on 1/d ends below it from either side); the
//    quotient estimate from it is the floor or one below, and the exact
//    remainder n - q d (integer arithmetic modulo 2^64) corrects it and
//    decides the rounding (no midpoint can occur for a quotient of two
//    53-bit significands);
//  - square root: the same with a reciprocal square root estimate
//    (rsqrt.approx) and steps y <- y + y (1 - x y^2) / 2, s = x y, and the
//    exact remainder x - s^2 (no midpoint: (s + 1/2)^2 is never an
//    integer).
#ifndef MAHYCO_GB300_SOFTFP_CUH
#define MAHYCO_GB300_SOFTFP_CUH

namespace hydro {
namespace sfp {

#ifndef HD
#define HD __host__ __device__ __forceinline__
#endif

typedef unsigned long long u64;
typedef long long i64;
typedef unsigned int u32;

constexpr u64 kSignBit = 0x8000000000000000ull;
constexpr u64 kFracMask = 0x000fffffffffffffull;
constexpr u64 kHidden = 1ull << 52;

HD u64 mulhi(u64 a, u64 b) {
#ifdef __CUDA_ARCH__
  return __umul64hi(a, b);
#else
  return (u64)(((unsigned __int128)a * b) >> 64);
#endif
}
HD int clz64(u64 x) {  // x != 0
#ifdef __CUDA_ARCH__
  return __clzll((long long)x);
#else
  return __builtin_clzll(x);
#endif
}
HD u32 exp_of(u64 b) { return (u32)(b >> 52) & 0x7ffu; }

// Assembles sign | (E - 1) << 52 + m for a significand m in [2^52, 2^53]:
// m = 2^53 (a rounding carry) raises the exponent by one, and E - 1 = 2046
// with that carry gives the infinity round-to-nearest asks for.
HD u64 pack(u64 sign, u32 E, u64 m) { return sign | ((((u64)E - 1) << 52) + m); }

// ---------------------------------------------------------------- product
HD bool mul_fast(u64 ab, u64 bb, u64& out) {
  const u64 sign = (ab ^ bb) & kSignBit;
  const u32 ea = exp_of(ab), eb = exp_of(bb), es = ea + eb;
  // both normal and the biased result exponent es - 1023 (+1) in [1, 2046]
  if (ea - 1u < 2046u && eb - 1u < 2046u && es - 1024u < 2045u) {
    const u64 ma = (ab & kFracMask) | kHidden, mb = (bb & kFracMask) | kHidden;
    const u64 hi = mulhi(ma, mb), lo = ma * mb;  // P in [2^104, 2^106)
    const u32 top = (u32)(hi >> 41);             // P >= 2^105
    const u32 sh = 12 - top;                     // 64 - (52 + top)
    u64 m = (hi << sh) | (lo >> (52 + top));     // P >> (52 + top)
    const u64 rest = lo << sh;                   // bits below m, round bit first
    m += (rest > kSignBit) | ((rest == kSignBit) & (u32)m);
    out = pack(sign, es - 1023 + top, m);
    return true;
  }
  // a zero times a finite value (zero, subnormal or normal)
  if (((ab << 1) == 0 && eb != 0x7ffu) || ((bb << 1) == 0 && ea != 0x7ffu)) {
    out = sign;
    return true;
  }
  return false;
}

// ------------------------------------------------------------------- sum
HD bool add_fast(u64 ab, u64 bb, u64& out) {
  const u64 aa = ab & ~kSignBit, ba = bb & ~kSignBit;
  const bool sw = ba > aa;
  const u64 x = sw ? bb : ab;  // |x| >= |y|
  const u64 xm = sw ? ba : aa, ym = sw ? aa : ba;
  const u32 ex = (u32)(xm >> 52), ey = (u32)(ym >> 52);
  // x normal and below the top binade (a carry out of it is handled by
  // pack only as far as the infinity of round-to-nearest)
  if (ex - 1u >= 2045u) return false;
  if (ym == 0) {  // x + (+-0) = x for x != 0
    out = x;
    return true;
  }
  if (ey == 0) return false;  // subnormal y
  const u32 d = ex - ey, dd = d < 63u ? d : 63u;
  const u64 X = ((xm & kFracMask) | kHidden) << 10;  // [2^62, 2^63)
  u64 Y = ((ym & kFracMask) | kHidden) << 10;
  Y = (Y >> dd) | (u64)((Y & ((1ull << dd) - 1)) != 0);  // jamming shift
  u64 S;
  u32 E = ex;
  if (((ab ^ bb) >> 63) == 0) {
    S = X + Y;  // < 2^64
    const u32 c = (u32)(S >> 63);
    S = (S >> c) | (S & c);
    E += c;
  } else {
    S = X - Y;  // >= 0
    if (S == 0) {  // exact cancellation: +0
      out = 0;
      return true;
    }
    const u32 n = (u32)clz64(S) - 1u;  // S < 2^63
    if (n >= E) return false;          // subnormal result
    S <<= n;
    E -= n;
  }
  // S in [2^62, 2^63): the significand above 10 guard bits
  u64 m = S >> 10;
  const u32 r = (u32)S & 0x3ffu;
  m += (u32)(r > 0x200u) | ((u32)(r == 0x200u) & (u32)m);
  out = pack(x & kSignBit, E, m);
  return true;
}

// --------------------------------------------------------------- quotient
HD u32 hi32(u64 x) { return (u32)(x >> 32); }
HD u64 wide(u32 a, u32 b) { return (u64)a * b; }  // one 32 x 32 -> 64 product

// One Newton-Raphson correction in 64-bit fixed point: x + sign(e) *
// floor(hi32(x) (|e| >> sh) / 2^k) for a signed residual e.
HD u64 newton_step(u64 x, i64 e, int sh, int k) {
  const u64 mag = e < 0 ? (u64)(-e) : (u64)e;
  const u64 corr = wide(hi32(x), (u32)(mag >> sh)) >> k;
  return e < 0 ? x - corr : x + corr;
}

// Z ~ 2^127 / D for D in (2^63, 2^64) (the divisor's significand shifted
// left by 11), never above it and at most ~2^-57 below.
//  - FP32 estimate of 1 / (t + 1) (t: D's top 24 bits) scaled by
//    2^87 (1 - 2^-17): below, relative error < 2^-16.8;
//  - step 1 on the top halves, with the divisor's top word rounded up:
//    e = 2^63 - (D32 + 1) Z32 > 0, z e / 2^63 ~ Z32 (e >> 16) / 2^15; its
//    truncations leave |relative error| < 2^-29.8, on either side;
//  - step 2: e / 2^64 = 2^63 - floor(D Z1 / 2^64) - 1 (signed,
//    |e| < 2^34), correction z e / 2^63 ~ Z1hi (|e| >> 3) / 2^28.  A step
//    z <- z (2 - d z) ends below 1/d from either side (1/d - z' =
//    d (1/d - z)^2); a margin of 32 units covers its truncations.
HD u64 recip127(u64 D) {
  const u32 t = (u32)(D >> 40);
#ifdef __CUDA_ARCH__
  const float y = __uint_as_float(0x4b000000u | (t & 0x7fffffu)) + 1.0f;  // t + 1, exact
  float rf;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(rf) : "f"(y));
  const u64 Z0 = __float2ull_rz(rf * 0x1.ffffp86f);
#else
  const float rf = 1.0f / ((float)t + 1.0f);
  const u64 Z0 = (u64)(rf * 0x1.ffffp86f);
#endif
  const u32 D32 = hi32(D), Z32 = hi32(Z0);
  const u64 e1 = (1ull << 63) - (wide(D32, Z32) + Z32);
  const u64 Z1 = Z0 + (wide(Z32, (u32)(e1 >> 16)) >> 15);
  const i64 e2 = (i64)((1ull << 63) - mulhi(D, Z1) - 1);
  return newton_step(Z1, e2, 3, 28) - 32;
}

// The quotient's significand from N in [mb, 2 mb) (the dividend's
// significand, doubled when it is below the divisor's), the divisor's
// significand mb in (2^52, 2^53) and Z = recip127(mb << 11):
// Q = floor(N 2^52 / mb) in [2^52, 2^53), rounded to nearest.
HD u64 div_significand(u64 N, u64 mb, u64 Z) {
  // N 2^52 / mb = N 2^63 / D ~ N Z / 2^64, never above: Q is the floor or
  // one below it (N Z / 2^64 is within 2^54 2^-58 of N 2^63 / D)
  u64 Q = mulhi(N, Z);
  // exact remainder N 2^52 - Q mb in [0, 2 mb) (arithmetic modulo 2^64)
  u64 R = (N << 52) - Q * mb;
  if (R >= mb) {
    ++Q;
    R -= mb;
  }
  // round to nearest: 2R > mb (2R = mb cannot occur)
  return Q + (u64)((R << 1) > mb);
}

// A divisor prepared once for several quotients: its bits, significand and
// reciprocal (ok: the divisor is normal).
struct Divisor {
  u64 bits, mb, Z;
  bool ok;
};
HD Divisor make_divisor(u64 bb) {
  Divisor d;
  d.bits = bb;
  const u32 eb = exp_of(bb);
  d.ok = eb - 1u < 2046u;
  d.mb = (bb & kFracMask) | kHidden;
  d.Z = (d.ok && d.mb != kHidden) ? recip127(d.mb << 11) : 0;
  return d;
}

// a / d for a prepared divisor
HD bool div_fast_by(u64 ab, const Divisor& d, u64& out) {
  if (!d.ok) return false;  // divisor zero, subnormal, inf or NaN
  const u64 sign = (ab ^ d.bits) & kSignBit;
  if ((ab << 1) == 0) {  // +-0 / normal
    out = sign;
    return true;
  }
  const u32 ea = exp_of(ab), eb = exp_of(d.bits);
  if (ea - 1u >= 2046u) return false;
  u64 N = (ab & kFracMask) | kHidden;
  const u32 lt = N < d.mb;
  const i64 E = (i64)ea - (i64)eb + 1023 - (i64)lt;
  if ((u64)(E - 1) >= 2046ull) return false;  // subnormal or overflowing result
  N <<= lt;                                   // N in [mb, 2 mb)
  out = pack(sign, (u32)E, d.mb == kHidden ? N : div_significand(N, d.mb, d.Z));
  return true;
}

HD bool div_fast(u64 ab, u64 bb, u64& out) {
  const u64 sign = (ab ^ bb) & kSignBit;
  const u32 ea = exp_of(ab), eb = exp_of(bb);
  if (eb - 1u >= 2046u) return false;  // divisor zero, subnormal, inf or NaN
  if ((ab << 1) == 0) {                // +-0 / normal
    out = sign;
    return true;
  }
  if (ea - 1u >= 2046u) return false;
  u64 N = (ab & kFracMask) | kHidden;
  const u64 mb = (bb & kFracMask) | kHidden;
  const u32 lt = N < mb;
  const i64 E = (i64)ea - (i64)eb + 1023 - (i64)lt;
  if ((u64)(E - 1) >= 2046ull) return false;  // subnormal or overflowing result
  N <<= lt;                                   // N in [mb, 2 mb)
  // a power-of-two divisor: the significand is the dividend's, exactly
  out = pack(sign, (u32)E, mb == kHidden ? N : div_significand(N, mb, recip127(mb << 11)));
  return true;
}

// ------------------------------------------------------------ square root
// Y ~ 2^94 / sqrt(W) for W in [2^62, 2^64): in (2^62, 2^63], never above
// and at most ~2^-56 below.
HD u64 rsqrt94(u64 W) {
  // Y ~ 2^94 / sqrt(W) in (2^62, 2^63], never above and at most ~2^-56
  // below, as recip127 forms 1 / D, with y <- y + y (1 - W y^2) / 2 (which
  // also ends below 1 / sqrt(W) from either side: with y = (1 + d) /
  // sqrt(W), y' = (1 - 3d^2/2 - d^3/2) / sqrt(W)):
  //  - FP32 estimate from the top 24 bits of W rounded up, scaled by
  //    2^74 (1 - 2^-17);
  //  - step 1 on the top halves: Y32^2 / 2^30 ~ 2^94 / W, e = 2^62 -
  //    (W32 + 1) y2 > 0, y e / 2^63 ~ Y32 (e >> 16) / 2^15 (|relative
  //    error| < 2^-29 after it);
  //  - step 2: e / 2^64 = 2^60 - floor(W floor(Y1^2 / 2^64) / 2^64) - 1
  //    (signed, |e| < 2^32), correction y e / 2^61 ~ Y1hi (|e| >> 2) / 2^27,
  //    then a margin of 16 units.
  const u32 t = (u32)(W >> 40);      // [2^22, 2^24)
  const float wf = (float)(t + 1u);  // exact
#ifdef __CUDA_ARCH__
  float rf;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(rf) : "f"(wf));
  const u64 Y0 = __float2ull_rz(rf * 0x1.ffffp73f);
#else
  const float rf = 1.0f / __builtin_sqrtf(wf);
  const u64 Y0 = (u64)(rf * 0x1.ffffp73f);
#endif
  const u32 W32 = hi32(W), Y32 = hi32(Y0);
  const u32 y2 = (u32)(wide(Y32, Y32) >> 30);
  const u64 e1 = (1ull << 62) - (wide(W32, y2) + y2);
  const u64 Y1 = Y0 + (wide(Y32, (u32)(e1 >> 16)) >> 15);
  const i64 e2 = (i64)((1ull << 60) - mulhi(W, mulhi(Y1, Y1)) - 1);
  return newton_step(Y1, e2, 2, 27) - 16;
}

HD bool sqrt_fast(u64 ab, u64& out) {
  if ((ab << 1) == 0) {  // sqrt(+-0) = +-0
    out = ab;
    return true;
  }
  const u32 ea = exp_of(ab);
  if ((ab >> 63) != 0 || ea - 1u >= 2046u) return false;  // negative, subnormal, inf, NaN
  // a = ma 2^(ea - 1075); with an even exponent: a = M 2^k, M in [2^52, 2^54)
  // (odd: ea - 1075 odd, i.e. ea even), so that
  // sqrt(a) = sqrt(M 2^52) 2^((k - 52) / 2) and S = floor(sqrt(M 2^52)) is a
  // 53-bit significand with the biased exponent (ea + 1023 - odd) / 2
  const u32 odd = (ea & 1u) ^ 1u;
  const u64 M = ((ab & kFracMask) | kHidden) << odd;
  const u32 E = (ea + 1023u - odd) >> 1;
  // W = M 2^10 in [2^62, 2^64): M 2^52 = W 2^42, sqrt(M 2^52) = sqrt(W) 2^21
  const u64 W = M << 10;
  const u64 Y = rsqrt94(W);
  // S = floor(W Y / 2^73) ~ sqrt(W) 2^21 = sqrt(M 2^52), never above and
  // at most one below; the exact remainder M 2^52 - S^2 (modulo 2^64)
  // corrects it
  u64 S = mulhi(W, Y) >> 9;
  u64 R = (M << 52) - S * S;
  if (R > 2 * S) {  // (S + 1)^2 = S^2 + 2S + 1
    R -= 2 * S + 1;
    ++S;
  }
  // round to nearest: sqrt > S + 1/2  <=>  R > S (R = S + 1/4 is impossible)
  S += (u64)(R > S);
  out = pack(0, E, S);
  return true;
}

}  // namespace sfp
}  // namespace hydro

#endif  // MAHYCO_GB300_SOFTFP_CUH
