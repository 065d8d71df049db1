// Exact binary64 addition on the integer pipe, in fixed point.
//
// GB300's binary64 pipe retires about 1.6 operations per SM per clock (about
// 0.5 Tflop/s for the whole GPU), against 128 binary32 lanes, so a stencil
// written with hardware binary64 adds is bound by that pipe, not by HBM.
// These helpers reproduce IEEE round-to-nearest-even binary64 addition
// exactly with 32-bit integer instructions for operands held in a fixed-point
// frame:
//
//   a frame F represents the value v by the int64 X with v = X * 2^-F.
//
// A double x is representable in frame F when its unit in the last place is at
// least 2^-F.  If x and y are representable in F and |X + Y| < 2^62, then
//   fl(x + y) = round53(X + Y) * 2^-F
// where round53 rounds the exact integer sum to 53 significant bits with ties
// to even.  If |X + Y| < 2^53 the exact sum has at most 53 significant bits
// and is a normal double (F is far below 1022), so IEEE returns it unchanged;
// otherwise IEEE rounds at integer bit p - 52 (p the leading-bit position of
// |X + Y|), which is exactly what round53 does.  Zero results are +0, as IEEE
// gives for x + (-x) under round-to-nearest, so -0.0 inputs must be excluded
// by the caller.
//
// Multiplying by a power of two is a change of frame (exact, no instruction):
// 0.125 * v in frame F is the same integer read in frame F + 3.
//
// The header compiles for the device (nvcc) and for the host (any C++17
// compiler), so the host build can be checked against the CPU's IEEE doubles.
#pragma once

#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define NPBGB_FX_FN __host__ __device__ __forceinline__
#else
#define NPBGB_FX_FN inline
#endif

namespace npbgb {
namespace fx {

NPBGB_FX_FN int clz32(uint32_t v) {
#if defined(__CUDA_ARCH__)
  return __clz(static_cast<int>(v));
#else
  return v ? __builtin_clz(v) : 32;
#endif
}

NPBGB_FX_FN int clz64(uint64_t v) {
#if defined(__CUDA_ARCH__)
  return __clzll(static_cast<long long>(v));
#else
  return v ? __builtin_clzll(v) : 64;
#endif
}

NPBGB_FX_FN uint64_t bits_of(double x) {
#if defined(__CUDA_ARCH__)
  return static_cast<uint64_t>(__double_as_longlong(x));
#else
  uint64_t b;
  std::memcpy(&b, &x, 8);
  return b;
#endif
}

NPBGB_FX_FN double double_of(uint64_t b) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double(static_cast<long long>(b));
#else
  double x;
  std::memcpy(&x, &b, 8);
  return x;
#endif
}

// Position of the most significant bit of v that differs from its sign bit
// (the leading 1 of v >= 0, the leading 0 of v < 0); -1 for v == 0 and v == -1.
// One instruction on the GPU (PTX bfind.s32).
NPBGB_FX_FN int msb_nonsign32(uint32_t v) {
#if defined(__CUDA_ARCH__)
  int p;
  asm("bfind.s32 %0, %1;" : "=r"(p) : "r"(v));
  return p;
#else
  const uint32_t h = v ^ static_cast<uint32_t>(static_cast<int32_t>(v) >> 31);
  return 31 - clz32(h);
#endif
}

// v >> s for a shift amount s read as unsigned, with amounts of 32 and more
// giving 0 (PTX shr.b32 clamps the amount to the register width).
NPBGB_FX_FN uint32_t shr_clamp32(uint32_t v, uint32_t s) {
#if defined(__CUDA_ARCH__)
  uint32_t r;
  asm("shr.b32 %0, %1, %2;" : "=r"(r) : "r"(v), "r"(s));
  return r;
#else
  return s >= 32u ? 0u : v >> s;
#endif
}

// Rounds the exact integer x (|x| < 2^63 - 2^11) to 53 significant bits,
// ties to even.  Works on two's complement directly: for negative x the
// leading bit of ~x = |x| - 1 is that of |x| unless |x| is a power of two, and
// then x has no bits below the rounding point anyway.
//
// With p the leading non-sign bit of the high word, sh = p - 20 bits (0..11)
// lie below the 53-bit window.  mask = 2^sh - 1 comes from one clamped shift
// (0 whenever p <= 20, i.e. |x| < 2^53, which is exact already), and
// floor((x + mask/2 + lsb) / 2^sh) * 2^sh, lsb = bit sh of x, is
// round-half-even on two's complement.  The lsb is taken as
// (lo >> sh) & mask & 1, so that it is 0 when nothing is rounded (mask = 0).
NPBGB_FX_FN int64_t round53(int64_t x) {
  const uint32_t hi = static_cast<uint32_t>(static_cast<uint64_t>(x) >> 32);
  const uint32_t lo = static_cast<uint32_t>(x);
  const int p = msb_nonsign32(hi);
  const uint32_t mask = shr_clamp32(0xffffffffu, static_cast<uint32_t>(52 - p));
  const uint32_t lsb = shr_clamp32(lo, static_cast<uint32_t>(p - 20)) & mask & 1u;
  const uint64_t r = static_cast<uint64_t>(x) + ((mask >> 1) + lsb);
  return static_cast<int64_t>(r & ~static_cast<uint64_t>(mask));
}

// The former form of round53: sign fold, count of leading zeros, shift
// clamped at zero, increment masked.  Kept as a second statement of the same
// rounding for the host check.
NPBGB_FX_FN int64_t round53_fold(int64_t x) {
  const int32_t hi = static_cast<int32_t>(x >> 32);
  const uint32_t h = static_cast<uint32_t>(hi ^ (hi >> 31));
  int sh = (31 - clz32(h)) - 20;  // bits below the 53-bit window
  sh = sh < 0 ? 0 : sh;           // 0..11, all within the low word
  const uint32_t mask = (1u << sh) - 1u;
  const uint32_t lo = static_cast<uint32_t>(x);
  const uint32_t add = ((mask >> 1) + ((lo >> sh) & 1u)) & mask;
  return static_cast<int64_t>((static_cast<uint64_t>(x) + add) & ~static_cast<uint64_t>(mask));
}

// round53 for 0 <= x < 2^63: the leading bit comes from hi | 2^20 directly
// (a non-negative value needs no sign fold, and the OR keeps the shift >= 0
// for x < 2^53, which is exact already).
NPBGB_FX_FN int64_t round53p(int64_t x) {
  const uint32_t hi = static_cast<uint32_t>(static_cast<uint64_t>(x) >> 32);
  const int sh = 11 - clz32(hi | 0x100000u);  // (31 - clz) - 20, 0..11
  const uint32_t mask = (1u << sh) - 1u;
  const uint32_t lo = static_cast<uint32_t>(x);
  const uint32_t add = ((mask >> 1) + ((lo >> sh) & 1u)) & mask;
  return static_cast<int64_t>((static_cast<uint64_t>(x) + add) & ~static_cast<uint64_t>(mask));
}

// x -> frame-59 integer for x == +0.0 or x in [2^-7, 1).  Sets ok = false for
// anything else (negative, -0.0, >= 1, < 2^-7, subnormal, inf, nan); the
// returned value is then meaningless.
NPBGB_FX_FN int64_t from_f64_f59(double x, bool& ok) {
  const uint64_t b = bits_of(x);
  const uint32_t hi = static_cast<uint32_t>(b >> 32);
  const uint32_t lo = static_cast<uint32_t>(b);
  const uint32_t sh = (hi >> 20) - 1016u;  // sign bit set -> huge -> rejected
  const bool zero = b == 0;
  ok = (sh <= 6u) || zero;
  const uint32_t s = sh & 7u;
  const uint32_t mh = (hi & 0xfffffu) | 0x100000u;
  const uint32_t xh = s ? ((mh << s) | (lo >> (32u - s))) : mh;
  const uint32_t xl = lo << s;
  const int64_t X = static_cast<int64_t>((static_cast<uint64_t>(xh) << 32) | xl);
  return zero ? 0 : X;
}

// Poison mark for values the fixed-point path refuses.  Accepted frame-59
// values lie in [0, 2^59), so bit 30 of their high word is never set; OR-ing
// the high words of a point's inputs and testing this bit finds any refused
// input in one step.
constexpr uint32_t kPoisonHi = 0x40000000u;

// v << s for a shift amount s read as unsigned, with amounts of 32 and more
// giving 0 (PTX shl.b32 clamps the amount to the register width).
NPBGB_FX_FN uint32_t shl_clamp32(uint32_t v, uint32_t s) {
#if defined(__CUDA_ARCH__)
  uint32_t r;
  asm("shl.b32 %0, %1, %2;" : "=r"(r) : "r"(v), "r"(s));
  return r;
#else
  return s >= 32u ? 0u : v << s;
#endif
}

// from_f64_f59 with refused values marked by the poison bit in the high word
// (the low word of a poisoned value is unspecified).
//
// For x in [2^-7, 1) the exponent field e is 1016 .. 1022, so sh = e - 1016 =
// 0 .. 6 and X = significand << sh: a funnel shift for the high word and a
// shift for the low word.  The implicit leading bit is the exponent field's
// bit 9 (set for every e in 1016 .. 1022, clear for +0.0) moved to bit 20, so
// +0.0 gives X = 0 with no select.  Every other x has sh > 6 as an unsigned
// number (a sign bit or a smaller exponent wraps it around) and is poisoned,
// except +0.0.
NPBGB_FX_FN int64_t from_f64_f59_or_poison(double x) {
  const uint64_t b = bits_of(x);
  const uint32_t hi = static_cast<uint32_t>(b >> 32);
  const uint32_t lo = static_cast<uint32_t>(b);
  const uint32_t sh = (hi >> 20) - 1016u;
  const uint32_t mh = (hi & 0xfffffu) | ((hi >> 9) & 0x100000u);
  const bool ok = sh <= 6u || b == 0;
#if defined(__CUDA_ARCH__)
  const uint32_t xh = __funnelshift_l(lo, mh, sh);  // the amount is taken mod 32
#else
  const uint32_t xh = static_cast<uint32_t>(((static_cast<uint64_t>(mh) << 32 | lo) << (sh & 31u)) >> 32);
#endif
  const uint32_t xl = shl_clamp32(lo, sh);
  return static_cast<int64_t>((static_cast<uint64_t>(ok ? xh : kPoisonHi) << 32) | xl);
}

NPBGB_FX_FN uint32_t hi32(int64_t x) { return static_cast<uint32_t>(static_cast<uint64_t>(x) >> 32); }

// x + y for 64-bit integers, issued as two 32-bit multiply-adds with the
// multiplier `one` (== 1, passed at run time so the compiler cannot fold it
// away).  On the GPU this moves the add from the integer ALU pipe, which the
// rounding steps saturate, to the multiply-add pipe.
NPBGB_FX_FN int64_t add64(int64_t x, int64_t y, uint32_t one) {
#if defined(__CUDA_ARCH__)
  uint64_t r;
  const uint32_t ylo = static_cast<uint32_t>(y), yhi = static_cast<uint32_t>(static_cast<uint64_t>(y) >> 32);
  asm("mad.wide.u32 %0, %1, %2, %3;" : "=l"(r) : "r"(ylo), "r"(one), "l"(x));
  uint32_t rlo = static_cast<uint32_t>(r), rhi = static_cast<uint32_t>(r >> 32);
  asm("mad.lo.u32 %0, %1, %2, %3;" : "=r"(rhi) : "r"(yhi), "r"(one), "r"(rhi));
  return static_cast<int64_t>((static_cast<uint64_t>(rhi) << 32) | rlo);
#else
  (void)one;
  return static_cast<int64_t>(static_cast<uint64_t>(x) + static_cast<uint64_t>(y));
#endif
}

// round53 with its final 64-bit add on the multiply-add pipe (see add64).
NPBGB_FX_FN int64_t round53m(int64_t x, uint32_t one) {
  const int32_t hi = static_cast<int32_t>(x >> 32);
  const uint32_t h = static_cast<uint32_t>(hi ^ (hi >> 31));
  int sh = (31 - clz32(h)) - 20;
  sh = sh < 0 ? 0 : sh;
  const uint32_t mask = (1u << sh) - 1u;
  const uint32_t lo = static_cast<uint32_t>(x);
  const uint32_t add = ((mask >> 1) + ((lo >> sh) & 1u)) & mask;
#if defined(__CUDA_ARCH__)
  uint64_t r;
  asm("mad.wide.u32 %0, %1, %2, %3;" : "=l"(r) : "r"(add), "r"(one), "l"(x));
#else
  (void)one;
  const uint64_t r = static_cast<uint64_t>(x) + add;
#endif
  return static_cast<int64_t>(r & ~static_cast<uint64_t>(mask));
}

// round53p with its additions issued as multiply-adds (the multiplier `one`
// == 1 at run time), so that four of its twelve instructions run on the
// multiply-add pipe instead of the integer ALU: 11 - clz, pow - 1, the sum of
// the rounding increment, and the 64-bit add of it (one wide multiply-add).
// For 0 <= x < 2^63.
NPBGB_FX_FN int64_t round53q(int64_t x, uint32_t one) {
  const uint32_t hi = static_cast<uint32_t>(static_cast<uint64_t>(x) >> 32);
  const uint32_t lo = static_cast<uint32_t>(x);
  const uint32_t c = static_cast<uint32_t>(clz32(hi | 0x100000u));  // 9..11 -> sh 0..11
#if defined(__CUDA_ARCH__)
  uint32_t sh, mask, add;
  uint64_t r;
  asm("mad.lo.u32 %0, %1, %2, %3;" : "=r"(sh) : "r"(c), "r"(0u - one), "r"(11u));
  const uint32_t pow = 1u << sh;
  asm("mad.lo.u32 %0, %1, %2, %3;" : "=r"(mask) : "r"(pow), "r"(one), "r"(0xffffffffu));
  asm("mad.lo.u32 %0, %1, %2, %3;" : "=r"(add) : "r"((lo >> sh) & 1u), "r"(one), "r"(mask >> 1));
  add &= mask;
  asm("mad.wide.u32 %0, %1, %2, %3;" : "=l"(r) : "r"(add), "r"(one), "l"(x));
#else
  (void)one;
  const uint32_t sh = 11u - c;
  const uint32_t mask = (1u << sh) - 1u;
  const uint32_t add = ((mask >> 1) + ((lo >> sh) & 1u)) & mask;
  const uint64_t r = static_cast<uint64_t>(x) + add;
#endif
  return static_cast<int64_t>(r & ~static_cast<uint64_t>(mask));
}

// x -> frame-59 integer using the binary64 conversion path instead of integer
// bit manipulation: x * 2^59 (an exponent change, exact for accepted x) is
// converted with round-toward-zero, which is exact because the scaled value is
// an integer.  +0.0 maps to a tiny positive double and then to 0.  Refused
// values get the poison mark.
NPBGB_FX_FN int64_t from_f64_f59_cvt(double x) {
  const uint64_t b = bits_of(x);
  const uint32_t hi = static_cast<uint32_t>(b >> 32);
  const bool ok = ((hi >> 20) - 1016u <= 6u) || b == 0;
#if defined(__CUDA_ARCH__)
  const int64_t v = __double2ll_rz(double_of(b + (static_cast<uint64_t>(59) << 52)));
#else
  const int64_t v = static_cast<int64_t>(double_of(b + (static_cast<uint64_t>(59) << 52)));
#endif
  return ok ? v : static_cast<int64_t>(static_cast<uint64_t>(kPoisonHi) << 32);
}

// Frame-F integer (53 significant bits) -> double via the binary64 conversion
// path: the integer converts exactly, then the exponent drops by F.
template <int F>
NPBGB_FX_FN double to_f64_cvt(int64_t w) {
#if defined(__CUDA_ARCH__)
  const double d = __ll2double_rn(w);
#else
  const double d = static_cast<double>(w);
#endif
  const uint64_t b = bits_of(d) - (static_cast<uint64_t>(F) << 52);
  return w == 0 ? 0.0 : double_of(b);
}

// Frame-F integer (already rounded to 53 significant bits, |w| < 2^63) -> double.
template <int F>
NPBGB_FX_FN double to_f64(int64_t w) {
  const uint64_t sign = static_cast<uint64_t>(w) & 0x8000000000000000ull;
  const uint64_t m = w < 0 ? static_cast<uint64_t>(0) - static_cast<uint64_t>(w)
                           : static_cast<uint64_t>(w);
  const int lz = clz64(m);
  const uint64_t norm = m << (lz & 63);
  // exponent field = 1086 - F - lz; the implicit bit of norm >> 11 adds one.
  const uint64_t bits = (norm >> 11) + (static_cast<uint64_t>(1085 - F - lz) << 52);
  return m == 0 ? 0.0 : double_of(bits | sign);
}

// to_f64<F>(round53(x)) in one step, for an exact integer x with
// |x| < 2^63 - 2^11: the IEEE double nearest x * 2^-F (ties to even).
//
// For 2^52 <= x < 2^63 (the common case of a non-negative sum) the rounding
// and the conversion share their work: with p the leading bit of the high word
// (20..30), sh = p - 20 bits lie below the 53-bit window, and
// sig = (x + 2^(sh-1) - 1 + lsb) >> sh is the rounded significand, 2^52 <= sig
// <= 2^53.  value = sig * 2^(sh - F), so its bits are sig plus the biased
// exponent minus one, (sh + 1074 - F), shifted to bit 52; a carry out of the
// rounding (sig == 2^53) moves into the exponent field by itself.  Other x
// (smaller, negative) take round53 and to_f64.
template <int F>
NPBGB_FX_FN double round_to_f64(int64_t x) {
  const uint32_t hi = static_cast<uint32_t>(static_cast<uint64_t>(x) >> 32);
  if (hi - 0x100000u >= 0x7ff00000u) return to_f64<F>(round53(x));  // x < 2^52 or x < 0
  const uint32_t lo = static_cast<uint32_t>(x);
  const int p = msb_nonsign32(hi);                    // 20 .. 30
  const uint32_t sh = static_cast<uint32_t>(p - 20);  // 0 .. 10
  const uint32_t mask = shr_clamp32(0xffffffffu, static_cast<uint32_t>(52 - p));
  const uint32_t lsb = (lo >> sh) & mask & 1u;
  const uint64_t sig = (static_cast<uint64_t>(x) + ((mask >> 1) + lsb)) >> sh;
  return double_of(sig + (static_cast<uint64_t>(sh + 1074u - F) << 52));
}

template <int F>
NPBGB_FX_FN double mul02_wide(int64_t w);

// The high word of (hi:lo) << k, for k < 32 (one funnel shift on the GPU).
NPBGB_FX_FN uint32_t funnel_left_hi(uint32_t lo, uint32_t hi, uint32_t k) {
#if defined(__CUDA_ARCH__)
  return __funnelshift_l(lo, hi, k);
#else
  return static_cast<uint32_t>(((static_cast<uint64_t>(hi) << 32 | lo) << k) >> 32);
#endif
}

// RN(0.2 * w * 2^-F), the IEEE binary64 product of 0.2 and the frame-F value
// w, on the integer pipes.  Precondition: w == 0, or 2^12 <= w < 2^62 with at
// most 53 significant bits (a round53 result) and a normal double result.
//
// The double nearest 0.2 is M * 2^-55 with M = 0x1999999999999A (53 bits), so
// the exact product is the integer P = w * M (65 to 115 bits) times
// 2^-(F + 55).  Its top 53 bits, rounded to nearest with ties to even on the
// bits below them, are the significand of the IEEE product; a carry out of the
// rounding lands in the exponent field by itself.  This is the textbook
// multiplication of two binary floating-point numbers (exact integer product
// of the significands, then one rounding), specialised to one constant factor.
//
// The product's top 64 bits hi decide the shift.  When 2^32 <= hi < 2^51
// (every sum of five inputs of [2^-7, 1) that is not 0 is at least 2^52, and
// then hi >= 2^40) the top 53 bits start in hi's high word, at bit p <= 18 of it, and the
// work is 32-bit: with k = 20 - p, the significand is hi:lo_hi shifted left by
// k (two funnel shifts), the discarded bits of lo_hi shifted left by k are the
// top of the remainder, and the low word of lo only decides whether the
// remainder is exactly a half.  Rounding up happens exactly when
// remainder + 2^63 - 1 + lsb carries out of 64 bits; the low word's
// contribution to that is its being non-zero, folded into the remainder's
// bit 0, which the shift by k >= 2 leaves free.  mul02_wide is the general
// form, for small w.
template <int F>
NPBGB_FX_FN double mul02(int64_t w) {
  constexpr uint64_t M = 0x1999999999999Aull;
  const uint64_t a = static_cast<uint64_t>(w);
#if defined(__CUDA_ARCH__)
  const uint64_t lo = a * M;
  const uint64_t hi = __umul64hi(a, M);
#else
  const unsigned __int128 pr = static_cast<unsigned __int128>(a) * M;
  const uint64_t lo = static_cast<uint64_t>(pr);
  const uint64_t hi = static_cast<uint64_t>(pr >> 64);
#endif
  const uint32_t hh = static_cast<uint32_t>(hi >> 32), hl = static_cast<uint32_t>(hi);
  const uint32_t lh = static_cast<uint32_t>(lo >> 32), ll = static_cast<uint32_t>(lo);
  if (hh - 1u >= (1u << 19) - 1u) return mul02_wide<F>(w);   // hi < 2^32, or w too large
  const int p = msb_nonsign32(hh);                    // 0 .. 18
  const uint32_t k = static_cast<uint32_t>(20 - p);   // 2 .. 20: sh = 64 - k bits dropped
  const uint32_t sig_hi = funnel_left_hi(hl, hh, k);
  const uint32_t sig_lo = funnel_left_hi(lh, hl, k);
  const uint32_t rem = (lh << k) | (ll != 0u ? 1u : 0u);
  const uint32_t inc = static_cast<uint32_t>((static_cast<uint64_t>(rem) + 0x7fffffffu + (sig_lo & 1u)) >> 32);
  // value = sig * 2^(sh - F - 55), sh = p + 44: biased exponent minus one is p + 1063 - F
  const uint64_t sig = (static_cast<uint64_t>(sig_hi) << 32 | sig_lo) + inc;
  return double_of(sig + (static_cast<uint64_t>(p + 1063 - F) << 52));
}

template <int F>
NPBGB_FX_FN double mul02_wide(int64_t w) {
  constexpr uint64_t M = 0x1999999999999Aull;
  const uint64_t a = static_cast<uint64_t>(w);
#if defined(__CUDA_ARCH__)
  const uint64_t lo = a * M;
  const uint64_t hi = __umul64hi(a, M);
#else
  const unsigned __int128 p = static_cast<unsigned __int128>(a) * M;
  const uint64_t lo = static_cast<uint64_t>(p);
  const uint64_t hi = static_cast<uint64_t>(p >> 64);
#endif
  const int sh = (128 - clz64(hi)) - 53;          // bits below the top 53: 12 .. 62
  uint64_t sig = (hi << ((64 - sh) & 63)) | (lo >> sh);
  const uint64_t below = lo & ((uint64_t(1) << (sh - 1)) - 1);
  const uint64_t half = (lo >> (sh - 1)) & 1;     // the first discarded bit
  sig += half & static_cast<uint64_t>((below != 0) | (sig & 1));
  // value = sig * 2^(sh - F - 55) = (sig / 2^52) * 2^(sh - F - 3)
  const uint64_t bits = (static_cast<uint64_t>(sh - F - 3 + 1023) << 52) + (sig - (uint64_t(1) << 52));
  return w == 0 ? 0.0 : double_of(bits);
}

// RN(0.2 * x) for a binary64 x, on the integer pipes when x is normal with a
// biased exponent in [24, 2000] (then the product is normal too): the 53-bit
// significand times M (106 bits) rounded once to nearest even, as mul02 does;
// any other x (zeros, subnormals, huge, infinite, NaN) takes the hardware
// multiply.
NPBGB_FX_FN double mul02_any(double x) {
  constexpr uint64_t M = 0x1999999999999Aull;
  const uint64_t b = bits_of(x);
  const uint32_t e = static_cast<uint32_t>(b >> 52) & 0x7ffu;
  if (e - 24u > 2000u - 24u) return 0.2 * x;
  const uint64_t sig = (b & 0xfffffffffffffull) | 0x10000000000000ull;
#if defined(__CUDA_ARCH__)
  const uint64_t lo = sig * M;
  const uint64_t hi = __umul64hi(sig, M);
#else
  const unsigned __int128 p = static_cast<unsigned __int128>(sig) * M;
  const uint64_t lo = static_cast<uint64_t>(p);
  const uint64_t hi = static_cast<uint64_t>(p >> 64);
#endif
  const int sh = (128 - clz64(hi)) - 53;          // 52 or 53
  uint64_t s = (hi << (64 - sh)) | (lo >> sh);
  const uint64_t below = lo & ((uint64_t(1) << (sh - 1)) - 1);
  const uint64_t half = (lo >> (sh - 1)) & 1;
  s += half & static_cast<uint64_t>((below != 0) | (s & 1));
  // x = sig * 2^(e - 1075), 0.2 = M * 2^-55: the product is s * 2^(sh + e - 1130)
  const uint64_t mag = (static_cast<uint64_t>(sh + static_cast<int>(e) - 55) << 52) +
                       (s - (uint64_t(1) << 52));
  return double_of(mag | (b & 0x8000000000000000ull));
}

}  // namespace fx
}  // namespace npbgb
