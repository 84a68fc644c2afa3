// Host check of the integer-pipe binary64 operations (softfp.cuh): for
// seeded random operands over the whole exponent range, operands with few
// or many significand bits (exact products, ties), near-cancelling sums and
// structured edge values, every fast-path result must equal the host's IEEE
// operation bit for bit.  Prints one line per operation and exits non-zero
// on a mismatch.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include <vector>

#include "kernels/softfp.cuh"

using namespace hydro::sfp;

static u64 B(double x) {
  u64 b;
  std::memcpy(&b, &x, 8);
  return b;
}
static double D(u64 b) {
  double x;
  std::memcpy(&x, &b, 8);
  return x;
}

static std::mt19937_64 rng(20241204);

static u64 operand(int mode) {
  const u64 s = rng() & kSignBit;
  u64 f = rng() & kFracMask;
  u32 e;
  switch (mode) {
    case 0: e = 1 + rng() % 2046; break;                 // any normal
    case 1: e = 1023 - 40 + rng() % 80; break;           // moderate
    case 2: e = rng() % 2048; if (rng() % 16 == 0) f = 0; break;  // incl. special
    case 3: {                                            // few bits or many ones
      e = 1020 + rng() % 7;
      const u64 k = (1ull << (rng() % 52)) - 1;
      f = (rng() & 1) ? (f & ~k) : (f | k);
      break;
    }
    default: e = (rng() & 1) ? 1 + rng() % 4 : 2046 - rng() % 4; break;  // extremes
  }
  return s | ((u64)e << 52) | f;
}

static long bad_total = 0;

static void check(const char* name, int op, u64 a, u64 b, long& fast, long& bad) {
  u64 r = 0;
  bool f = false;
  double w = 0;
  switch (op) {
    case 0: f = mul_fast(a, b, r); w = D(a) * D(b); break;
    case 1: f = add_fast(a, b, r); w = D(a) + D(b); break;
    case 2: f = div_fast(a, b, r); w = D(a) / D(b); break;
    case 3: f = sqrt_fast(a, r); w = std::sqrt(D(a)); break;
    case 4: f = div_fast_by(a, make_divisor(b), r); w = D(a) / D(b); break;
  }
  if (!f) return;
  ++fast;
  if (r != B(w)) {
    if (bad++ < 5)
      std::printf("%s mismatch: %a %a -> %a, IEEE %a\n", name, D(a), D(b), D(r), w);
  }
}

// floor(sqrt(x)) of a 128-bit integer, exactly
static unsigned __int128 isqrt128(unsigned __int128 x) {
  unsigned __int128 r = (unsigned __int128)std::sqrt((long double)x);
  while (r * r > x) --r;
  while ((r + 1) * (r + 1) <= x) ++r;
  return r;
}

// The estimates behind the quotient and the square root: for a divisor
// significand mb, Q = mulhi(N, recip127(mb << 11)) must be floor(N 2^52 /
// mb) or one below (never above); for M in [2^52, 2^54),
// S = mulhi(W, rsqrt94(W)) >> 9 with W = M 2^10 must be floor(sqrt(M 2^52))
// or one below.  Divisors and radicands at the ends of their ranges and of
// the 24-bit estimate's steps, then random ones.
static long check_estimates() {
  long bad = 0, n = 0;
  auto qcheck = [&](u64 mb, u64 N) {
    const u64 Q = mulhi(N, recip127(mb << 11));
    const u64 Qt = (u64)(((unsigned __int128)N << 52) / mb);
    ++n;
    if (Q > Qt || Qt - Q > 1) {
      if (bad++ < 5) std::printf("quotient estimate: mb %llx N %llx Q %llx floor %llx\n", mb, N, Q, Qt);
    }
  };
  auto scheck = [&](u64 M) {
    const u64 W = M << 10;
    const u64 S = mulhi(W, rsqrt94(W)) >> 9;
    const u64 St = (u64)isqrt128((unsigned __int128)M << 52);
    ++n;
    if (S > St || St - S > 1) {
      if (bad++ < 5) std::printf("root estimate: M %llx S %llx floor %llx\n", M, S, St);
    }
  };
  std::vector<u64> mbs;
  for (u64 k = 1; k < 3000; ++k) {
    mbs.push_back(kHidden + k);
    mbs.push_back((kHidden << 1) - k);
  }
  for (int k = 0; k < 20000; ++k) {  // the 24-bit steps of the FP32 estimate
    const u64 top = (rng() & ((1ull << 23) - 1)) | (1ull << 23);
    const u64 low = (rng() & 1) ? 0 : ((1ull << 29) - 1);
    mbs.push_back((top << 29) | (low ^ (rng() & 7)));
  }
  for (int k = 0; k < 300000; ++k) mbs.push_back(kHidden | (rng() & kFracMask));
  for (u64 mb : mbs) {
    if (mb <= kHidden) continue;
    qcheck(mb, mb);
    qcheck(mb, 2 * mb - 1);
    qcheck(mb, kHidden | (rng() & kFracMask) | ((u64)(rng() & 1) << 52));
    const u64 Nr = mb + rng() % mb;
    qcheck(mb, Nr);
  }
  std::vector<u64> ms;
  for (u64 k = 0; k < 3000; ++k) {
    ms.push_back(kHidden + k);
    ms.push_back((kHidden << 2) - 1 - k);
    ms.push_back((kHidden << 1) + k);
    ms.push_back((kHidden << 1) - 1 - k);
  }
  for (int k = 0; k < 400000; ++k)
    ms.push_back(kHidden + rng() % (3 * kHidden));
  for (int k = 0; k < 20000; ++k) {  // perfect squares and their neighbours
    const u64 r = (1ull << 52) + rng() % (1ull << 52);
    const unsigned __int128 sq = (unsigned __int128)r * r;
    if ((sq & ((1ull << 52) - 1)) == 0) ms.push_back((u64)(sq >> 52));
    ms.push_back((u64)(sq >> 52));
    ms.push_back((u64)(sq >> 52) + 1);
  }
  for (u64 M : ms)
    if (M >= kHidden && M < (kHidden << 2)) scheck(M);
  std::printf("estimates: %ld checked, %ld outside [floor - 1, floor]\n", n, bad);
  return bad;
}

int main() {
  const char* names[5] = {"mul", "add", "div", "sqrt", "div_by"};
  // structured edge values
  std::vector<u64> edge;
  const double base[] = {1.0, 1.5, 2.0, 3.0, 0.1, 1.0 / 3.0, 1e-300, 1e300, 0x1p-1022,
                         0x1.fffffffffffffp1023, 0x1.0000000000001p0, 0x1.fffffffffffffp0,
                         0x1.0000002p0, 0x1.8000001p0, 0x1p-1000, 0x1p1000, 0x1.1p511,
                         0x1.1p-511, 0.0, 4.9e-324, 1e-310, INFINITY, NAN};
  for (double v : base) {
    edge.push_back(B(v));
    edge.push_back(B(-v));
    edge.push_back(B(v) + 1);
    edge.push_back(B(v) - 1);
  }
  for (int op = 0; op < 5; ++op) {
    long fast = 0, bad = 0, tot = 0;
    for (u64 a : edge)
      for (u64 b : edge) {
        check(names[op], op, a, b, fast, bad);
        ++tot;
      }
    for (long i = 0; i < 3000000; ++i) {
      u64 a = operand(i % 5), b = operand((i / 5 + i) % 5);
      if (i % 7 == 0) {  // correlated: near cancellation, close quotients
        b = ((a & ~kFracMask) ^ ((rng() & 1) ? kSignBit : 0)) |
            ((a & kFracMask) ^ (rng() & ((1ull << (rng() % 53)) - 1)));
        if (i % 21 == 0) b += (u64)((long long)(rng() % 5) - 2) << 52;
      }
      check(names[op], op, a, b, fast, bad);
      ++tot;
    }
    std::printf("%s: %ld of %ld on the fast path, %ld mismatches\n", names[op], fast, tot, bad);
    bad_total += bad;
  }
  bad_total += check_estimates();
  std::printf("softfp: %ld mismatches\n", bad_total);
  return bad_total ? 1 : 0;
}
