// Heat-3D point arithmetic and the plain-load tile streamer, shared by the
// single-grid kernels (heat3d.cu) and the batched persistent kernel (batch.cu).
//
// Per interior point, in the reference's order (heat_3d_numpy.py:7-13):
//   tx  = 0.125 * ((next_x - 2*c) + prev_x)      x = axis 0, 1, 2
//   dst = ((t0 + t1) + t2) + c
#pragma once

#include <type_traits>

#include "fx64.cuh"
#include "npbgb_common.cuh"

namespace npbgb {
namespace hcore {

constexpr int kTK = 32;   // tile extent along axis 2 (one warp)
constexpr int kTJ = 8;    // tile extent along axis 1 (warps per CTA)
constexpr int kThreads = kTK * kTJ;
using fx::hi32;
using fx::kPoisonHi;

__device__ __forceinline__ int64_t to_fx(double v) { return fx::from_f64_f59_or_poison(v); }

template <bool CG, typename T>
__device__ __forceinline__ T ld(const T* p) {
  if constexpr (CG) return __ldcg(p); else return *p;
}

// The exact binary64 products 2*x and 0.125*x on the integer pipe: an
// exponent change for normal x whose result stays normal, x itself for
// signed zeros.  Subnormals, infinities, NaN and overflow take the literal
// product, out of line so that it is not predicated into the common path
// (GB300's binary64 pipe is the bound of the hardware rows).
static __device__ __noinline__ double twice_literal(double x) { return mul_rn(2.0, x); }
static __device__ __noinline__ double eighth_literal(double x) { return mul_rn(0.125, x); }
__device__ __forceinline__ double twice(double x) {
  const uint64_t b = static_cast<uint64_t>(__double_as_longlong(x));
  const uint32_t e = static_cast<uint32_t>(b >> 52) & 0x7ffu;
  if (e - 1u < 2045u) return __longlong_as_double(static_cast<long long>(b + (1ull << 52)));
  if ((b << 1) == 0) return x;
  return twice_literal(x);
}
__device__ __forceinline__ double eighth(double x) {
  const uint64_t b = static_cast<uint64_t>(__double_as_longlong(x));
  const uint32_t e = static_cast<uint32_t>(b >> 52) & 0x7ffu;
  if (e - 4u < 2043u) return __longlong_as_double(static_cast<long long>(b - (3ull << 52)));
  if ((b << 1) == 0) return x;
  return eighth_literal(x);
}
__device__ __forceinline__ float twice(float x) { return mul_rn(2.0f, x); }
__device__ __forceinline__ float eighth(float x) { return mul_rn(0.125f, x); }

template <typename T>
__device__ __forceinline__ T heat_point(T c, T ip, T im, T jp, T jm, T kp, T km) {
  const T c2 = twice(c);
  const T t0 = eighth(add_rn(sub_rn(ip, c2), im));
  const T t1 = eighth(add_rn(sub_rn(jp, c2), jm));
  const T t2 = eighth(add_rn(sub_rn(kp, c2), km));
  return add_rn(add_rn(add_rn(t0, t1), t2), c);
}

// Two binary32 points at once (packed f32x2, npbgb_common.cuh); each result is
// bit-identical to heat_point<float>.  Element x is the first point, y the second.
__device__ __forceinline__ F2 heat_point2(F2 c, F2 ip, F2 im, F2 jp, F2 jm, F2 kp, F2 km) {
  const F2 two = f2(2.0f, 2.0f), eighth = f2(0.125f, 0.125f);
  const F2 c2 = mul2(two, c);
  const F2 t0 = mul2(eighth, add2(sub2(ip, c2), im));
  const F2 t1 = mul2(eighth, add2(sub2(jp, c2), jm));
  const F2 t2 = mul2(eighth, add2(sub2(kp, c2), km));
  return add2(add2(add2(t0, t1), t2), c);
}

// Fixed-point form of heat_point; inputs in frame 59, result as a double.
__device__ __forceinline__ double heat_point_fx(int64_t c, int64_t ip, int64_t im, int64_t jp,
                                                int64_t jm, int64_t kp, int64_t km) {
  using fx::round53;
  const int64_t c2 = c * 2;
  const int64_t s0 = round53(round53(ip - c2) + im);  // 8 * t0 in frame 59 == t0 in frame 62
  const int64_t s1 = round53(round53(jp - c2) + jm);
  const int64_t s2 = round53(round53(kp - c2) + km);
  return fx::round_to_f64<62>(round53(round53(s0 + s1) + s2) + c * 8);
}

// Evaluates one point from staged values (T for the plain path, frame-59
// integers with poison marks for binary64), falling back to hardware binary64
// from global memory `q` (pointer to the centre) when an input is poisoned.
template <typename T, bool FX, bool CG = false, typename S>
__device__ __forceinline__ T eval_point(S c, S ip, S im, S jp, S jm, S kp, S km, const T* q,
                                        int64_t s0, int64_t s1) {
  if constexpr (FX) {
    const uint32_t tag = hi32(c) | hi32(ip) | hi32(im) | hi32(jp) | hi32(jm) | hi32(kp) | hi32(km);
    if (!(tag & kPoisonHi)) return heat_point_fx(c, ip, im, jp, jm, kp, km);
    return heat_point<T>(ld<CG>(q), ld<CG>(q + s0), ld<CG>(q - s0), ld<CG>(q + s1),
                         ld<CG>(q - s1), ld<CG>(q + 1), ld<CG>(q - 1));
  } else {
    return heat_point<T>(c, ip, im, jp, jm, kp, km);
  }
}

template <typename T, bool FX>
using PlaneBuf = typename std::conditional<FX, int64_t, T>::type[3][kTJ + 2][kTK + 2];

// Streams the kTJ x kTK tile at (j0, k0) along axis 0 over planes [ib, ie):
// each plane tile plus its one-element halo is staged by plain loads into
// three rotating shared buffers (one CTA barrier per plane); the axis-0
// neighbours of a thread's own column stay in registers.  CTA-collective.
// CG: loads and stores through L2 (data shared with other CTAs of a
// persistent kernel).
template <typename T, bool FX, bool CG>
__device__ __forceinline__ void tile_stream(const T* src, T* dst, int64_t n1, int64_t n2, int64_t j0,
                                            int64_t k0, int64_t ib, int64_t ie,
                                            PlaneBuf<T, FX>& plane) {
  using S = typename std::conditional<FX, int64_t, T>::type;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const int64_t k = k0 + tx, j = j0 + ty;
  const bool active = k < n2 - 1 && j < n1 - 1;
  const bool own_inb = k < n2 && j < n1;
  const int64_t s0 = n1 * n2, s1 = n2;

  // Halo roles: warp 0 the row before the tile, warp 1 the row after, warps
  // 2 and 3 (first kTJ lanes) the columns before and after.  No corners: the
  // stencil has no diagonal neighbours.
  int er = -1, ec = -1;
  int64_t ej = 0, ek = 0;
  if (ty == 0) { ej = j0 - 1; ek = k; er = 0; ec = tx + 1; }
  else if (ty == 1) { ej = j0 + kTJ; ek = k; er = kTJ + 1; ec = tx + 1; }
  else if (ty == 2 && tx < kTJ) { ej = j0 + tx; ek = k0 - 1; er = tx + 1; ec = 0; }
  else if (ty == 3 && tx < kTJ) { ej = j0 + tx; ek = k0 + kTK; er = tx + 1; ec = kTK + 1; }
  const bool has_extra = er >= 0 && ej < n1 && ek < n2;
  const T* own_p = src + j * s1 + k;
  const T* extra_p = src + ej * s1 + ek;

  auto stage = [&](int64_t i, int b, S& own) {
    if (own_inb) {
      const T v = ld<CG>(own_p + i * s0);
      if constexpr (FX) own = to_fx(v); else own = v;
      plane[b][ty + 1][tx + 1] = own;
    }
    if (has_extra) {
      const T v = ld<CG>(extra_p + i * s0);
      if constexpr (FX) plane[b][er][ec] = to_fx(v); else plane[b][er][ec] = v;
    }
  };

  S xp = S(0), xc = S(0), xn = S(0);
  int bc = 1, bn = 2;
  stage(ib - 1, 0, xp);
  stage(ib, bc, xc);
  for (int64_t i = ib; i < ie; ++i) {
    stage(i + 1, bn, xn);
    __syncthreads();
    if (active) {
      const S* P = &plane[bc][ty + 1][tx + 1];
      const T out = eval_point<T, FX, CG>(xc, xn, xp, P[kTK + 2], P[-(kTK + 2)], P[1], P[-1],
                                          own_p + i * s0, s0, s1);
      if constexpr (CG) __stcg(dst + i * s0 + j * s1 + k, out); else dst[i * s0 + j * s1 + k] = out;
    }
    const int t = (bn + 1) % 3;  // buffer of plane i-1, free after this barrier round
    bc = bn;
    bn = t;
    xp = xc;
    xc = xn;
  }
  __syncthreads();  // the buffers may be restaged by the caller's next tile
}

}  // namespace hcore
}  // namespace npbgb
