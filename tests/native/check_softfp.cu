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
  std::printf("softfp: %ld mismatches\n", bad_total);
  return bad_total ? 1 : 0;
}
