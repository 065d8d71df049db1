// Exact IEEE binary64 addition (round to nearest, ties to even) on the
// integer pipes, for operands in a safe range.
//
// GB300's binary64 pipe retires about 1.6 operations per SM per clock while
// its integer pipes retire tens of 32-bit operations, so an addition built
// from integer instructions can run next to the hardware one and add to the
// binary64 throughput of a kernel.  Unlike the fixed-point helpers (fx64.cuh)
// this works for operands of any magnitude within the range below:
//
//   dadd_ok(a, b): both a and b finite, normal and with biased exponent in
//                  [64, 1983] (|x| between about 2^-959 and 2^960);
//   dadd_int(a, b) then returns exactly fl(a + b): +0 for an exact zero sum,
//                  otherwise a normal double (the exponent range keeps the
//                  result away from subnormals and overflow).
//
// Method (the textbook one): order the operands by magnitude, give both
// significands 9 guard bits (leading bit at bit 61), shift the smaller right
// by the exponent difference keeping a sticky bit, add or subtract, move the
// leading bit to 62 (no shift after a carry, left after no carry or after
// cancellation, which is exact), and round the 10 low bits to nearest even as
// (n + 2^9 - 1 + lsb) >> 10.  With 9 guard bits and a sticky bit the rounding
// is exact in every case (at most one bit of cancellation can follow a lossy
// alignment).
//
// Host and device: the header compiles for both, so the host build is
// checked against the CPU's IEEE addition.
#pragma once

#include <cstdint>

#include "fx64.cuh"

namespace npbgb {
namespace f64emu {

NPBGB_FX_FN bool dadd_ok(uint64_t a, uint64_t b) {
  const uint32_t ea = static_cast<uint32_t>(a >> 52) & 0x7ffu;
  const uint32_t eb = static_cast<uint32_t>(b >> 52) & 0x7ffu;
  return (ea - 64u) < 1920u && (eb - 64u) < 1920u;
}

// dadd_ok, or either operand a signed zero with the other in range or zero too
// (dadd_z handles those).
NPBGB_FX_FN bool dadd_z_ok(uint64_t a, uint64_t b) {
  constexpr uint64_t kAbs = 0x7fffffffffffffffull;
  const uint32_t ea = static_cast<uint32_t>(a >> 52) & 0x7ffu;
  const uint32_t eb = static_cast<uint32_t>(b >> 52) & 0x7ffu;
  const bool za = (a & kAbs) == 0, zb = (b & kAbs) == 0;
  return (za || (ea - 64u) < 1920u) && (zb || (eb - 64u) < 1920u);
}

NPBGB_FX_FN uint64_t dadd_int(uint64_t a, uint64_t b) {
  constexpr uint64_t kAbs = 0x7fffffffffffffffull, kMant = (1ull << 52) - 1;
  const bool swap = (b & kAbs) > (a & kAbs);
  const uint64_t x = swap ? b : a, y = swap ? a : b;  // |x| >= |y|
  const uint32_t ex = static_cast<uint32_t>(x >> 52) & 0x7ffu;
  const uint32_t ey = static_cast<uint32_t>(y >> 52) & 0x7ffu;
  const uint64_t mx = ((x & kMant) | (1ull << 52)) << 9;  // leading bit at 61
  const uint64_t my = ((y & kMant) | (1ull << 52)) << 9;
  uint32_t d = ex - ey;
  d = d < 63u ? d : 63u;
  const uint64_t yt = my >> d;
  const uint64_t ya = yt | ((yt << d) != my ? 1ull : 0ull);  // sticky: a bit was shifted out
  const bool sub = ((x ^ y) >> 63) != 0;
  const uint64_t s = sub ? mx - ya : mx + ya;
  if (s == 0) return 0;  // x + (-x) = +0 in round to nearest
  const int lz = fx::clz64(s);  // 1 (carry), 2 (aligned) or more (cancellation)
  // n: leading bit 62, mantissa bits 62..10, round bit 9, sticky bits 8..0.
  const uint64_t n = s << (lz - 1);
  const uint64_t m = (n + 0x1ffull + ((n >> 10) & 1ull)) >> 10;  // [2^52, 2^53]; 2^53 carries on
  // exponent of the sum: ex + 2 - lz; the field is that minus one plus m's leading bit
  return (x & 0x8000000000000000ull) + ((static_cast<uint64_t>(int(ex) + 1 - lz) << 52) + m);
}

}  // namespace f64emu
}  // namespace npbgb

namespace npbgb {
namespace f64emu {

// fl(a + b) for dadd_z_ok operands: zeros follow IEEE round-to-nearest
// (x + 0 = x for x != 0; +0 + -0 = +0; -0 + -0 = -0).
NPBGB_FX_FN uint64_t dadd_z(uint64_t a, uint64_t b) {
  constexpr uint64_t kAbs = 0x7fffffffffffffffull;
  const bool za = (a & kAbs) == 0, zb = (b & kAbs) == 0;
  if (za || zb) return za ? (zb ? (a & b) : b) : a;
  return dadd_int(a, b);
}

// fl(a - b) = fl(a + (-b)) (IEEE defines subtraction so), same operand rules.
NPBGB_FX_FN uint64_t dsub_z(uint64_t a, uint64_t b) {
  return dadd_z(a, b ^ 0x8000000000000000ull);
}

}  // namespace f64emu
}  // namespace npbgb

#if defined(__CUDACC__)
// Device forms on raw bit patterns, for kernels that keep emulated values in
// integer registers.  Operands outside the emulation's range take the hardware
// instruction, out of line (so it is not predicated into the common path);
// every form returns the IEEE round-to-nearest result.
namespace npbgb {
namespace f64emu {

constexpr uint64_t kSignBit = 0x8000000000000000ull;

__device__ __forceinline__ uint64_t u64(double v) { return static_cast<uint64_t>(__double_as_longlong(v)); }
__device__ __forceinline__ double f64(uint64_t b) { return __longlong_as_double(static_cast<long long>(b)); }

static __device__ __noinline__ uint64_t add_bits_hw(uint64_t a, uint64_t b) {
  return u64(__dadd_rn(f64(a), f64(b)));
}
// fl(a + b)
__device__ __forceinline__ uint64_t add_bits(uint64_t a, uint64_t b) {
  return dadd_z_ok(a, b) ? dadd_z(a, b) : add_bits_hw(a, b);
}
// fl(a - b)
__device__ __forceinline__ uint64_t sub_bits(uint64_t a, uint64_t b) { return add_bits(a, b ^ kSignBit); }

static __device__ __noinline__ uint64_t half_bits_hw(uint64_t d) { return u64(__dmul_rn(0.5, f64(d))); }
// fl(0.5 * d): an exponent decrement for normal d whose half is normal, d itself
// for signed zeros, the hardware product otherwise.
__device__ __forceinline__ uint64_t half_bits(uint64_t d) {
  const uint32_t e = static_cast<uint32_t>(d >> 52) & 0x7ffu;
  if (e - 2u < 2045u) return d - (1ull << 52);
  if ((d << 1) == 0) return d;
  return half_bits_hw(d);
}

}  // namespace f64emu
}  // namespace npbgb
#endif
