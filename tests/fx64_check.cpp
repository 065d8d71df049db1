// Host check of npbench_gb300/csrc/fx64.cuh against the CPU's IEEE binary64.
//
// Built by tests/test_fx64.py with -ffp-contract=off.  For random and
// adversarial operands it checks, bit for bit, that the fixed-point
// emulation reproduces:
//   * single additions and subtractions, including ties to even;
//   * the Heat-3D update ((t0 + t1) + t2) + c, tx = 0.125 * ((nx - 2c) + px);
//   * the Jacobi-2D sum (((c + w) + e) + s) + n.
// Prints "OK <count>" and exits 0, or prints the first mismatch and exits 1.
#include <cinttypes>
#include <cstdio>
#include <cstdlib>
#include <random>

#include "../npbench_gb300/csrc/fx64.cuh"

using namespace npbgb::fx;

static std::mt19937_64 rng(12345);

static uint64_t bits(double x) { return bits_of(x); }

// Doubles in [2^-7, 1) or +0, with a bias towards patterns that make ties.
static double draw() {
  const int kind = static_cast<int>(rng() % 8);
  if (kind == 0) return 0.0;
  const uint64_t e = 1016 + rng() % 7;  // exponent field for [2^-7, 1)
  uint64_t m = rng() & ((1ull << 52) - 1);
  if (kind == 1) m &= ~((1ull << (rng() % 52)) - 1);  // trailing zeros
  if (kind == 2) m |= (1ull << (rng() % 52)) - 1;     // trailing ones
  if (kind == 3) m = 0;                                // powers of two
  if (kind == 4) m = (1ull << 52) - 1;
  return double_of((e << 52) | m);
}

static int fail(const char* what, double a, double b, double want, double got) {
  std::printf("MISMATCH %s: a=%a b=%a want=%a (%016" PRIx64 ") got=%a (%016" PRIx64 ")\n", what,
              a, b, want, bits(want), got, bits(got));
  return 1;
}

int main(int argc, char** argv) {
  const long n = argc > 1 ? std::atol(argv[1]) : 2000000;
  long checks = 0;
  for (long it = 0; it < n; ++it) {
    const double a = draw(), b = draw();
    bool oka, okb;
    const int64_t A = from_f64_f59(a, oka), B = from_f64_f59(b, okb);
    if (!oka || !okb) return fail("conversion rejected an in-range value", a, b, 0, 0);
    if (to_f64<59>(A) != a || bits(to_f64<59>(A)) != bits(a)) return fail("roundtrip", a, b, a, to_f64<59>(A));
    if (from_f64_f59_cvt(a) != A) return fail("cvt conversion", a, b, a, 0);
    if (to_f64_cvt<59>(A) != a || bits(to_f64_cvt<59>(A)) != bits(a)) return fail("cvt roundtrip", a, b, a, to_f64_cvt<59>(A));
    if (round53m(A - 2 * B, 1u) != round53(A - 2 * B)) return fail("round53m", a, b, 0, 0);
    if (add64(A, -2 * B, 1u) != A - 2 * B) return fail("add64", a, b, 0, 0);
    volatile double s = a + b, d = a - b, d2 = a - 2.0 * b;
    if (bits(to_f64<59>(round53(A + B))) != bits(s)) return fail("add", a, b, s, to_f64<59>(round53(A + B)));
    if (bits(to_f64<59>(round53(A - B))) != bits(d)) return fail("sub", a, b, d, to_f64<59>(round53(A - B)));
    if (bits(to_f64<59>(round53(A - 2 * B))) != bits(d2))
      return fail("sub2", a, b, d2, to_f64<59>(round53(A - 2 * B)));
    // frame change: 0.125 * x is the same integer in frame 62
    volatile double e = 0.125 * d2;
    if (bits(to_f64<62>(round53(A - 2 * B))) != bits(e)) return fail("scale", a, b, e, to_f64<62>(round53(A - 2 * B)));
    checks += 5;
  }
  // Heat-3D update.
  for (long it = 0; it < n / 2; ++it) {
    double v[7];
    int64_t X[7];
    for (int q = 0; q < 7; ++q) {
      bool ok;
      v[q] = draw();
      X[q] = from_f64_f59(v[q], ok);
    }
    const double c = v[0];
    volatile double t0 = 0.125 * ((v[1] - 2.0 * c) + v[2]);
    volatile double t1 = 0.125 * ((v[3] - 2.0 * c) + v[4]);
    volatile double t2 = 0.125 * ((v[5] - 2.0 * c) + v[6]);
    volatile double want = ((t0 + t1) + t2) + c;
    const int64_t C2 = X[0] * 2;
    const int64_t S0 = round53(round53(X[1] - C2) + X[2]);
    const int64_t S1 = round53(round53(X[3] - C2) + X[4]);
    const int64_t S2 = round53(round53(X[5] - C2) + X[6]);
    const int64_t W = round53(round53(round53(S0 + S1) + S2) + X[0] * 8);
    const double got = to_f64<62>(W);
    if (bits(got) != bits(want)) return fail("heat", v[0], v[1], want, got);
    if (bits(to_f64_cvt<62>(W)) != bits(want)) return fail("heat cvt", v[0], v[1], want, to_f64_cvt<62>(W));
    const double fused = round_to_f64<62>(round53(round53(S0 + S1) + S2) + X[0] * 8);
    if (bits(fused) != bits(want)) return fail("heat fused rounding", v[0], v[1], want, fused);
    ++checks;
  }
  // Jacobi-2D update: the fixed-point sum and its product by 0.2 on integers.
  for (long it = 0; it < n / 2; ++it) {
    double v[5];
    int64_t X[5];
    for (int q = 0; q < 5; ++q) {
      bool ok;
      v[q] = draw();
      X[q] = from_f64_f59(v[q], ok);
    }
    volatile double want = (((v[0] + v[1]) + v[2]) + v[3]) + v[4];
    const int64_t S = round53(round53(round53(round53(X[0] + X[1]) + X[2]) + X[3]) + X[4]);
    const double got = to_f64<59>(S);
    if (bits(got) != bits(want)) return fail("jacobi", v[0], v[1], want, got);
    const int64_t Sp = round53p(round53p(round53p(round53p(X[0] + X[1]) + X[2]) + X[3]) + X[4]);
    if (Sp != S) return fail("jacobi round53p", v[0], v[1], want, to_f64<59>(Sp));
    volatile double want02 = 0.2 * want;
    if (bits(mul02<59>(S)) != bits(want02)) return fail("jacobi 0.2", v[0], v[1], want02, mul02<59>(S));
    checks += 2;
  }
  // The product by 0.2 on frame-59 integers m * 2^k (m odd, 1 to 53 bits) over the
  // whole range a sum of five inputs in [2^-7, 1) can take, [2^52, 5 * 2^59):
  // small m give the exact ties (m * 0x1999999999999A with 54 significant bits).
  for (long it = 0; it < n; ++it) {
    const int bitsm = 1 + static_cast<int>(rng() % 53);
    uint64_t m = (rng() >> (64 - bitsm)) | 1u | (uint64_t(1) << (bitsm - 1));
    const int lo_k = 52 - (bitsm - 1) > 0 ? 52 - (bitsm - 1) : 0;
    const int hi_k = 61 - (bitsm - 1);
    if (hi_k < lo_k) continue;
    const int k = lo_k + static_cast<int>(rng() % static_cast<uint64_t>(hi_k - lo_k + 1));
    const int64_t W = static_cast<int64_t>(m << k);
    if (W < (int64_t(1) << 52) || W >= 5 * (int64_t(1) << 59)) continue;
    volatile double x = to_f64<59>(W);
    volatile double want02 = 0.2 * x;
    if (bits(mul02<59>(W)) != bits(want02)) return fail("0.2 product", x, 0.2, want02, mul02<59>(W));
    ++checks;
  }
  // The product by 0.2 over the whole domain of mul02, [2^12, 2^62) with at
  // most 53 significant bits: its 32-bit path (the top 64 product bits at
  // least 2^32) and its general path against each other and against the CPU.
  for (long it = 0; it < n; ++it) {
    const int bitsm = 1 + static_cast<int>(rng() % 53);
    const uint64_t m = (rng() >> (64 - bitsm)) | (uint64_t(1) << (bitsm - 1));
    const int lead = 12 + static_cast<int>(rng() % 50);  // leading bit 12 .. 61
    if (lead < bitsm - 1) continue;
    const int64_t W = static_cast<int64_t>(m << (lead - (bitsm - 1)));
    if (mul02<59>(W) != mul02_wide<59>(W) || bits(mul02<59>(W)) != bits(mul02_wide<59>(W)))
      return fail("0.2 product paths", to_f64<59>(W), 0.2, mul02_wide<59>(W), mul02<59>(W));
    volatile double x = to_f64<59>(W);
    volatile double want02 = 0.2 * x;
    if (bits(mul02<59>(W)) != bits(want02)) return fail("0.2 product, any length", x, 0.2, want02, mul02<59>(W));
    ++checks;
  }
  // round53p against round53 on non-negative integers of every length.
  for (long it = 0; it < n; ++it) {
    const int len = static_cast<int>(rng() % 63);
    const int64_t x = static_cast<int64_t>(rng() >> (63 - len)) & ((int64_t(1) << 62) | ((int64_t(1) << 62) - 1));
    if (x < 0) continue;
    if (round53p(x) != round53(x)) return fail("round53p", 0, 0, 0, 0);
    if (round53q(x, 1u) != round53(x)) return fail("round53q", 0, 0, 0, 0);
    ++checks;
  }
  // round53 (leading non-sign bit, clamped shifts) against the sign-fold form
  // on integers of every length and both signs, and at the edges of its range
  // and of the 53-bit window.
  for (long it = 0; it < n; ++it) {
    const int len = 1 + static_cast<int>(rng() % 63);
    int64_t x = static_cast<int64_t>(rng() >> (64 - len));  // 0 .. 2^63 - 1
    if (rng() & 1) x = -x;
    const int64_t lim = (int64_t(1) << 62) + ((int64_t(1) << 62) - 2048);  // 2^63 - 2^11
    if (x >= lim || x <= -lim) continue;
    if (round53(x) != round53_fold(x)) return fail("round53 signed", 0, 0, 0, 0);
    if (bits(round_to_f64<62>(x)) != bits(to_f64<62>(round53_fold(x))))
      return fail("round_to_f64", 0, 0, to_f64<62>(round53_fold(x)), round_to_f64<62>(x));
    if (bits(round_to_f64<59>(x)) != bits(to_f64<59>(round53_fold(x))))
      return fail("round_to_f64<59>", 0, 0, to_f64<59>(round53_fold(x)), round_to_f64<59>(x));
    ++checks;
  }
  for (int e = 0; e < 63; ++e)
    for (int64_t d = -3; d <= 3; ++d)
      for (int s : {1, -1}) {
        const int64_t x = s * ((int64_t(1) << e) + d);
        if (x > (int64_t(1) << 62) || x < -(int64_t(1) << 62)) continue;
        if (round53(x) != round53_fold(x)) return fail("round53 edge", 0, 0, 0, 0);
        if (bits(round_to_f64<62>(x)) != bits(to_f64<62>(round53_fold(x))))
          return fail("round_to_f64 edge", 0, 0, to_f64<62>(round53_fold(x)), round_to_f64<62>(x));
        // ties: 53 significant bits followed by exactly one half
        if (e >= 54 && e <= 61) {
          const int64_t t = s * ((int64_t(1) << e) + (int64_t(1) << (e - 53)) * (d & 3) + (int64_t(1) << (e - 54)));
          if (round53(t) != round53_fold(t)) return fail("round53 tie", 0, 0, 0, 0);
          if (bits(round_to_f64<62>(t)) != bits(to_f64<62>(round53_fold(t))))
            return fail("round_to_f64 tie", 0, 0, to_f64<62>(round53_fold(t)), round_to_f64<62>(t));
        }
        ++checks;
      }
  // mul02_any against the CPU's 0.2 * x over every exponent, both signs, and
  // the special values.
  for (long it = 0; it < n; ++it) {
    const uint64_t b = rng();
    volatile double x = double_of(b);
    volatile double want = 0.2 * x;
    const double got = mul02_any(x);
    if (!(want != want && got != got) && bits(got) != bits(want)) return fail("mul02_any", x, 0.2, want, got);
    ++checks;
  }
  for (long it = 0; it < n; ++it) {  // significands with few bits: the ties
    const int bitsm = 1 + static_cast<int>(rng() % 8);
    const uint64_t m = (rng() >> (64 - bitsm)) | 1u | (uint64_t(1) << (bitsm - 1));
    const uint64_t e = 1 + rng() % 2046;
    const uint64_t frac = (m << (53 - bitsm)) & 0xfffffffffffffull;
    volatile double x = double_of((e << 52) | frac | ((rng() & 1) << 63));
    volatile double want = 0.2 * x;
    if (bits(mul02_any(x)) != bits(want)) return fail("mul02_any tie", x, 0.2, want, mul02_any(x));
    ++checks;
  }
  for (double x : {0.0, -0.0, 0x1p-1074, -0x1p-1074, 0x1p-1022, 0x1.fffffffffffffp+1023,
                   __builtin_inf(), -__builtin_inf(), 1.0, 0.375, 5.0, 4.999999999999999}) {
    volatile double want = 0.2 * x;
    if (bits(mul02_any(x)) != bits(want)) return fail("mul02_any special", x, 0.2, want, mul02_any(x));
    ++checks;
  }
  if (bits(mul02<59>(0)) != bits(0.0)) return fail("0.2 product of +0", 0.0, 0.2, 0.0, mul02<59>(0));
  for (int e = 52; e < 62; ++e)  // ties: 3 * 2^k
    for (uint64_t m : {1ull, 3ull, 5ull, 7ull, 9ull, 15ull, 17ull, 255ull, 257ull}) {
      if ((m << e) >= 5 * (uint64_t(1) << 59) || (m << e) < (uint64_t(1) << 52)) continue;
      const int64_t W = static_cast<int64_t>(m << e);
      volatile double x = to_f64<59>(W);
      volatile double want02 = 0.2 * x;
      if (bits(mul02<59>(W)) != bits(want02)) return fail("0.2 tie", x, 0.2, want02, mul02<59>(W));
      ++checks;
    }
  // The poison-marking conversion against from_f64_f59 on every kind of bit
  // pattern: equal where accepted, poisoned where refused.
  for (long it = 0; it < 4 * n; ++it) {
    uint64_t b = rng();
    const int kind = static_cast<int>(rng() % 4);
    if (kind == 0) b = (b & 0x800fffffffffffffull) | ((1016ull + rng() % 7) << 52);  // in range, either sign
    if (kind == 1) b = (b & 0x800fffffffffffffull) | ((1008ull + rng() % 24) << 52);  // around the range
    if (kind == 2 && (rng() & 1)) b = (rng() & 3) == 0 ? 0 : (rng() & 1 ? 0x8000000000000000ull : b & 0xfffffffffffffull);
    bool ok;
    const int64_t want = from_f64_f59(double_of(b), ok);
    const int64_t got = from_f64_f59_or_poison(double_of(b));
    if (ok && got != want) return fail("poison conversion value", double_of(b), 0, 0, 0);
    if (!ok && !(hi32(got) & kPoisonHi)) return fail("poison conversion mark", double_of(b), 0, 0, 0);
    ++checks;
  }
  // Values the fast path must refuse.
  const double refuse[] = {-0.0, -0.5, 1.0, 1.5, 0x1p-8, 0x1p-1030, 1e300, __builtin_inf(),
                           __builtin_nan("")};
  for (double r : refuse) {
    bool ok;
    from_f64_f59(r, ok);
    if (ok) return fail("refuse", r, 0, 0, 0);
    if (!(hi32(from_f64_f59_cvt(r)) & kPoisonHi)) return fail("refuse cvt", r, 0, 0, 0);
    if (!(hi32(from_f64_f59_or_poison(r)) & kPoisonHi)) return fail("refuse poison", r, 0, 0, 0);
  }
  std::printf("OK %ld\n", checks);
  return 0;
}
