// Host check of npbench_gb300/csrc/f64emu.cuh against the CPU's IEEE binary64.
//
// Built by tests/test_fx64.py with -ffp-contract=off.  For operands inside the
// emulation's range (dadd_ok) it checks, bit for bit, that dadd_int(a, b) is
// the CPU's a + b, over random operands of independent magnitudes and over
// adversarial ones: equal and neighbouring exponents (carries and deep
// cancellation), exponent gaps around the guard and sticky bits, trailing
// zero/one patterns that make ties, and exact negations.  It also checks that
// dadd_ok refuses zeros, subnormals, infinities, NaNs and out-of-range
// exponents.  Prints "OK <count>" and exits 0, or the first mismatch and exits 1.
#include <cinttypes>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <random>

#include "../npbench_gb300/csrc/f64emu.cuh"

using npbgb::f64emu::dadd_int;
using npbgb::f64emu::dadd_ok;
using npbgb::f64emu::dadd_z;
using npbgb::f64emu::dadd_z_ok;
using npbgb::f64emu::dsub_z;

static std::mt19937_64 rng(2024);

static uint64_t bits(double x) { uint64_t b; std::memcpy(&b, &x, 8); return b; }
static double dbl(uint64_t b) { double x; std::memcpy(&x, &b, 8); return x; }

static uint64_t mant() {
  uint64_t m = rng() & ((1ull << 52) - 1);
  switch (rng() % 6) {
    case 0: m &= ~((1ull << (rng() % 53)) - 1); break;        // trailing zeros
    case 1: m |= (1ull << (rng() % 53)) - 1; break;           // trailing ones
    case 2: m = (rng() % 2) ? 0 : ((1ull << 52) - 1); break;  // extremes
    default: break;
  }
  return m & ((1ull << 52) - 1);
}

static double make(uint32_t e) {
  return dbl((static_cast<uint64_t>(rng() & 1) << 63) | (static_cast<uint64_t>(e) << 52) | mant());
}

static int check(double a, double b, long long& n) {
  if (!dadd_ok(bits(a), bits(b))) return 0;
  const uint64_t got = dadd_int(bits(a), bits(b));
  const uint64_t want = bits(a + b);
  ++n;
  if (got != want) {
    std::printf("MISMATCH a=%a b=%a got=%a want=%a\n", a, b, dbl(got), dbl(want));
    return 1;
  }
  return 0;
}

int main(int argc, char** argv) {
  const long long iters = argc > 1 ? std::atoll(argv[1]) : 1000000;
  long long n = 0;
  for (long long it = 0; it < iters; ++it) {
    const uint32_t ea = 64 + rng() % 1920;
    uint32_t eb;
    switch (rng() % 5) {
      case 0: eb = ea; break;                                        // same exponent
      case 1: eb = ea > 64 ? ea - 1 : ea + 1; break;                 // neighbours
      case 2: eb = ea > 64 + 70 ? ea - static_cast<uint32_t>(rng() % 70) : ea; break;  // gaps 0..69
      case 3: eb = 64 + rng() % 1920; break;                         // anything
      default: eb = ea > 64 + 12 ? ea - 9 - static_cast<uint32_t>(rng() % 4) : ea; break;
    }
    double a = make(ea), b = make(eb);
    if (rng() % 7 == 0) b = -a;                              // exact zero
    if (rng() % 5 == 0) b = dbl(bits(a) ^ (1ull << 63) ^ (rng() % 3));  // deep cancellation
    if (check(a, b, n) || check(b, a, n)) return 1;
  }
  // Zeros and subtraction (dadd_z / dsub_z).
  const double zs[] = {0.0, -0.0};
  for (long long it = 0; it < iters / 4; ++it) {
    double a = make(64 + rng() % 1920), b = make(64 + rng() % 1920);
    if (rng() % 3 == 0) a = zs[rng() & 1];
    if (rng() % 3 == 0) b = zs[rng() & 1];
    if (rng() % 5 == 0) b = a;
    if (!dadd_z_ok(bits(a), bits(b))) { std::printf("REFUSED %a %a\n", a, b); return 1; }
    const uint64_t s1 = dadd_z(bits(a), bits(b)), s2 = dsub_z(bits(a), bits(b));
    if (s1 != bits(a + b) || s2 != bits(a - b)) {
      std::printf("ZERO/SUB MISMATCH a=%a b=%a add=%a (%a) sub=%a (%a)\n", a, b, dbl(s1), a + b,
                  dbl(s2), a - b);
      return 1;
    }
    n += 2;
  }
  // hdiff's Laplacian fl(fl(4c) - s): for c with biased exponent 64..1981, 4c is
  // an exponent increment by two and stays in range, so the difference is one
  // emulated subtraction of (c with exponent + 2) and s.
  for (long long it = 0; it < iters / 4; ++it) {
    const uint32_t ec = 64 + rng() % 1918;
    const double c = make(ec);
    double s;
    switch (rng() % 4) {
      case 0: s = make(ec + 2); break;                             // same scale as 4c
      case 1: s = dbl(bits(c) + (2ull << 52)); break;               // s == 4c: exact zero
      case 2: s = make(64 + rng() % 1920); break;                   // anything
      default: s = rng() & 1 ? 0.0 : -0.0; break;                   // signed zeros
    }
    const double four_c = dbl(bits(c) + (2ull << 52));
    volatile double prod = 4.0 * c;
    if (bits(four_c) != bits(prod)) { std::printf("4C MISMATCH c=%a\n", c); return 1; }
    if (!dadd_z_ok(bits(four_c), bits(s))) { std::printf("4C REFUSED c=%a s=%a\n", c, s); return 1; }
    const uint64_t got = dsub_z(bits(four_c), bits(s));
    const double want = prod - s;
    if (got != bits(want)) {
      std::printf("LAPLACIAN MISMATCH c=%a s=%a got=%a want=%a\n", c, s, dbl(got), want);
      return 1;
    }
    ++n;
  }
  // Refusals.
  const double bad[] = {0.0, -0.0, 1e-310, -1e-310, std::numeric_limits<double>::infinity(),
                        std::nan(""), 1e300, std::ldexp(1.0, -970), std::ldexp(1.0, 961)};
  for (double x : bad)
    if (dadd_ok(bits(x), bits(1.0)) || dadd_ok(bits(1.0), bits(x))) {
      std::printf("ACCEPTED %a\n", x);
      return 1;
    }
  if (!dadd_ok(bits(std::ldexp(1.0, -959)), bits(std::ldexp(1.999, 960)))) {
    std::printf("REFUSED range ends\n");
    return 1;
  }
  std::printf("OK %lld\n", n);
  return 0;
}
