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
//  - quotient: a 24-bit FP32 reciprocal estimate, two Newton-Raphson steps
//    z <- z + z (1 - d z) in 64-bit fixed point, the quotient estimate from
//    the reciprocal, then the exact remainder n - q d (integer, exact modulo
//    2^64) corrects the estimate and decides the rounding (no midpoint can
//    occur for a quotient of two 53-bit significands);
//  - square root: a 24-bit FP32 reciprocal square root estimate, Newton
//    steps y <- y (3 - x y^2) / 2 in fixed point, s = x y, and the exact
//    remainder x - s^2 corrects s and decides the rounding (no midpoint:
//    (s + 1/2)^2 is never an integer).
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
// 2^127 / D for D in (2^63, 2^64) (the significand of the divisor shifted
// left by 11), to within a few units: Z in [2^63, 2^64).
HD u64 recip127(u64 D) {
  // FP32 estimate of 2^87 / (t + 1) with t = D >> 40 (24 bits), an
  // underestimate of 2^127 / D by at most about 2^-22 relative
  const u32 t = (u32)(D >> 40);
#ifdef __CUDA_ARCH__
  const float y = __uint_as_float(0x4b000000u | (t & 0x7fffffu)) + 1.0f;  // t + 1, exact
  float rf;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(rf) : "f"(y));
  u64 Z = __float2ull_rz(rf * 0x1p87f);  // saturates at 2^64 - 1
#else
  const float y = (float)t + 1.0f;
  const float rf = 1.0f / y;
  const double zs = (double)rf * 0x1p87;
  u64 Z = zs >= 0x1p64 ? ~0ull : (u64)zs;
#endif
  if (Z < (1ull << 63)) Z = 1ull << 63;
  // Newton-Raphson: z <- z + z e / 2^127 with e = 2^127 - D z (signed)
#pragma unroll
  for (int it = 0; it < 2; ++it) {
    const u64 ph = mulhi(D, Z), pl = D * Z;  // D Z = ph 2^64 + pl, near 2^127
    // e / 2^63, truncated toward minus infinity: (2^127 - D Z) >> 63
    // = 2^64 - (ph << 1 | pl >> 63) - (low bits != 0 ? 1 : 0), as a signed
    // 64-bit value (|e| < 2^106 after the FP32 estimate)
    const u64 p63 = (ph << 1) | (pl >> 63);
    const u64 lowz = (pl << 1) != 0;
    const i64 e63 = (i64)(0ull - p63 - lowz);
    const u64 mag = e63 < 0 ? (u64)(-e63) : (u64)e63;
    const u64 corr = mulhi(Z, mag);  // Z |e| / 2^127 = Z |e63| / 2^64
    Z = e63 < 0 ? Z - corr : Z + corr;
  }
  return Z;
}

// The quotient's significand from N in [mb, 2 mb) (the dividend's
// significand, doubled when it is below the divisor's), the divisor's
// significand mb in (2^52, 2^53) and Z = recip127(mb << 11):
// Q = floor(N 2^52 / mb) in [2^52, 2^53), rounded to nearest.
HD u64 div_significand(u64 N, u64 mb, u64 Z) {
  // N 2^52 / mb = N 2^63 / D ~ N Z / 2^64
  u64 Q = mulhi(N, Z);
  // exact remainder N 2^52 - Q mb (|R| < 2^63: the arithmetic modulo 2^64
  // gives it exactly), then at most two correction steps each way
  i64 R = (i64)((N << 52) - Q * mb);
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    if (R < 0) {
      --Q;
      R += (i64)mb;
    }
  }
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    if (R >= (i64)mb) {
      ++Q;
      R -= (i64)mb;
    }
  }
  // round to nearest: 2R > mb (2R = mb cannot occur)
  return Q + (u64)((u64)R << 1 > mb);
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
  // Y ~ 2^94 / sqrt(W) in (2^62, 2^63]: FP32 estimate from the top 24 bits
  // of W (rounded up, an underestimate by about 2^-22 at most)
  const u32 t = (u32)(W >> 40);  // [2^22, 2^24)
  const float wf = (float)(t + 1u);  // exact
#ifdef __CUDA_ARCH__
  float rf;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(rf) : "f"(wf));
  u64 Y = __float2ull_rz(rf * 0x1p74f);
#else
  const float rf = 1.0f / __builtin_sqrtf(wf);
  u64 Y = (u64)((double)rf * 0x1p74);
#endif
  if (Y < (1ull << 62)) Y = 1ull << 62;
  // Newton-Raphson on 1 / sqrt: y <- y + y e / 2 with e = 1 - W y^2 / 2^188
#pragma unroll
  for (int it = 0; it < 2; ++it) {
    const u64 y2 = mulhi(Y, Y);                // ~ 2^124 / W
    const u64 ph = mulhi(W, y2), pl = W * y2;  // W y2 ~ 2^124
    // (2^124 - W y2) >> 60, signed (|.| < 2^45 after the FP32 estimate)
    const u64 p60 = (ph << 4) | (pl >> 60);
    const u64 lowz = (pl << 4) != 0;
    const i64 e60 = (i64)(0ull - p60 - lowz);
    const u64 mag = e60 < 0 ? (u64)(-e60) : (u64)e60;
    const u64 corr = mulhi(Y, mag) >> 1;  // Y |e| / 2 = Y |e60| / 2^65
    Y = e60 < 0 ? Y - corr : Y + corr;
  }
  // S ~ sqrt(W) 2^21 = W Y / 2^73, then the exact remainder M 2^52 - S^2
  // (|.| < 2^63: exact modulo 2^64) corrects S to floor(sqrt(M 2^52))
  u64 S = mulhi(W, Y) >> 9;
  i64 R = (i64)((M << 52) - S * S);
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    if (R < 0) {  // (S - 1)^2 = S^2 - 2S + 1
      R += (i64)(2 * S - 1);
      --S;
    }
  }
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    if (R > (i64)(2 * S)) {  // (S + 1)^2 = S^2 + 2S + 1
      R -= (i64)(2 * S + 1);
      ++S;
    }
  }
  // round to nearest: sqrt > S + 1/2  <=>  R > S (R = S + 1/4 is impossible)
  S += (u64)(R > (i64)S);
  out = pack(0, E, S);
  return true;
}

}  // namespace sfp
}  // namespace hydro

#endif  // MAHYCO_GB300_SOFTFP_CUH
