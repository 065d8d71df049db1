// Warp-strip Jacobi-2D half-sweep shared by the single-grid and batched kernels.
//
// A warp owns 32 consecutive columns (one per lane, the contiguous axis) and
// walks down rows [r0, r1).  Rows i-1, i, i+1 of the lane's column stay in
// registers; the w/e neighbours come from the adjacent lanes by shuffle, and
// lanes 0 and 31 also read the strip's halo columns.  Rows are loaded U at a
// time ahead of use so that U independent loads per lane are in flight.
//
// Per point, in the reference's order (jacobi_2d_numpy.py:7-8):
//   dst = 0.2 * ((((c + w) + e) + s) + n)
// binary64 uses the exact fixed-point path (fx64.cuh) for points whose inputs
// lie in [2^-7, 1) or are +0, hardware binary64 otherwise.
#pragma once

#include <type_traits>

#include "fx64.cuh"
#include "npbgb_common.cuh"
#include "tma.cuh"

namespace npbgb {

extern int64_t g_cfg_jacobi_hw_warps;

// Warps of 8 per CTA that take the hardware binary64 path next to the
// fixed-point warps (binary64 Jacobi-2D).  Measured on GB300 at 500^2 to
// 4096^2, 4 of 8 keeps both the integer and the binary64 pipe busiest
// (1.2-2.4x faster than 1 of 8); NPBGB_CFG_JACOBI_HW_WARPS overrides.
inline int jacobi_hw_warps() {
  return int(g_cfg_jacobi_hw_warps >= 0 ? g_cfg_jacobi_hw_warps : 4);
}

namespace jcore {

template <bool CG, typename T>
__device__ __forceinline__ T ld(const T* p) {
  if constexpr (CG) return __ldcg(p); else return *p;
}
template <bool CG, typename T>
__device__ __forceinline__ void st(T* p, T v) {
  if constexpr (CG) __stcg(p, v); else *p = v;
}

// MAD: 1, the fixed-point additions are issued as multiply-adds (fx::add64,
// fx::round53m) on the FMA pipe; 2, the same with more of the rounding on it
// (fx::round53q); 0, plain integer additions, which measured fastest on GB300
// at every size once the product by 0.2 left the binary64 pipe (1000^2: 1.83
// ms against 1.94 and 2.10 for 198 half-sweeps; 4096^2 4.33 against 4.66).
// IMUL: the fixed-point points' product by 0.2 on the integer pipes
// (fx::mul02, exact product and one rounding), else a hardware binary64
// multiply; the binary64 pipe is the scarcer one on GB300.  HWIMUL: the same
// for the hardware binary64 path (fx::mul02_any), used by the hardware warps
// that work next to fixed-point warps.
template <typename T, bool FX, bool CG, int MAD = 0, bool IMUL = true, bool HWIMUL = false>
struct Strip {
  using S = typename std::conditional<FX, int64_t, T>::type;
  const T* src;
  T* dst;
  int64_t nx, j, hj;
  bool active, own_inb, has_halo;
  uint32_t one;

  __device__ __forceinline__ Strip(const T* s, T* d, int64_t nx_, int64_t k0, uint32_t one_)
      : src(s), dst(d), nx(nx_), one(one_) {
    const int lane = threadIdx.x & 31;
    j = k0 + lane;
    active = j < nx - 1;
    own_inb = j < nx;
    hj = lane == 0 ? k0 - 1 : k0 + 32;
    has_halo = (lane == 0) || (lane == 31 && hj < nx);
  }

  __device__ __forceinline__ void load(int64_t i, S& own, S& halo) const {
    const T* row = src + i * nx;
    if (own_inb) {
      const T v = ld<CG>(row + j);
      if constexpr (FX) own = fx::from_f64_f59_or_poison(v); else own = v;
    }
    if (has_halo) {
      const T v = ld<CG>(row + hj);
      if constexpr (FX) halo = fx::from_f64_f59_or_poison(v); else halo = v;
    }
  }

  // Output row i from rows i-1 (xp), i (xc, halo hc) and i+1 (xn).
  __device__ __forceinline__ void point(int64_t i, S xp, S xc, S xn, S hc) const {
    const int lane = threadIdx.x & 31;
    S w = __shfl_up_sync(0xffffffffu, xc, 1), e = __shfl_down_sync(0xffffffffu, xc, 1);
    if (lane == 0) w = hc;
    if (lane == 31) e = hc;
    const T k02 = T(0.2);
    T out;
    if constexpr (FX) {
      using fx::hi32;
      const uint32_t tag = hi32(xc) | hi32(w) | hi32(e) | hi32(xn) | hi32(xp);
      if (!(tag & fx::kPoisonHi)) {
        auto radd = [this](int64_t x, int64_t y) -> int64_t {
          if constexpr (MAD == 2) return fx::round53q(fx::add64(x, y, one), one);
          else if constexpr (MAD == 1) return fx::round53m(fx::add64(x, y, one), one);
          else return fx::round53(int64_t(uint64_t(x) + uint64_t(y)));
        };
        int64_t acc = radd(xc, w);
        acc = radd(acc, e);
        acc = radd(acc, xn);
        acc = radd(acc, xp);
        if constexpr (IMUL) out = fx::mul02<59>(acc);
        else out = mul_rn(k02, fx::to_f64<59>(acc));
      } else {
        out = T(0);
        if (active) {
          const T* r = src + i * nx + j;
          T acc = add_rn(ld<CG>(r), ld<CG>(r - 1));
          acc = add_rn(acc, ld<CG>(r + 1));
          acc = add_rn(acc, ld<CG>(r + nx));
          acc = add_rn(acc, ld<CG>(r - nx));
          out = mul_rn(k02, acc);
        }
      }
    } else {
      T acc = add_rn(xc, w);
      acc = add_rn(acc, e);
      acc = add_rn(acc, xn);
      acc = add_rn(acc, xp);
      if constexpr (HWIMUL && std::is_same<T, double>::value) out = fx::mul02_any(acc);
      else out = mul_rn(k02, acc);
    }
    if (active) st<CG>(dst + i * nx + j, out);
  }
};

// binary32, two consecutive output rows i and i+1 at once: rows i-1 .. i+2 of
// the column (x0..x3) and the halo values of rows i and i+1 (h1, h2).  The
// five operators run as packed f32x2 instructions (two IEEE round-to-nearest
// operations each), so both results are bit-identical to Strip::point.
template <bool CG, int MAD, bool IMUL, bool HWIMUL>
__device__ __forceinline__ void points2_f32(const Strip<float, false, CG, MAD, IMUL, HWIMUL>& sp, int64_t i, float x0,
                                            float x1, float x2, float x3, float h1, float h2) {
  const int lane = threadIdx.x & 31;
  float w1 = __shfl_up_sync(0xffffffffu, x1, 1), e1 = __shfl_down_sync(0xffffffffu, x1, 1);
  float w2 = __shfl_up_sync(0xffffffffu, x2, 1), e2 = __shfl_down_sync(0xffffffffu, x2, 1);
  if (lane == 0) { w1 = h1; w2 = h2; }
  if (lane == 31) { e1 = h1; e2 = h2; }
  F2 acc = add2(f2(x1, x2), f2(w1, w2));
  acc = add2(acc, f2(e1, e2));
  acc = add2(acc, f2(x2, x3));
  acc = add2(acc, f2(x0, x1));
  const F2 out = mul2(f2(0.2f, 0.2f), acc);
  if (sp.active) {
    st<CG>(sp.dst + i * sp.nx + sp.j, f2x(out));
    st<CG>(sp.dst + (i + 1) * sp.nx + sp.j, f2y(out));
  }
}

// ---------------------------------------------------------------------------
// TMA form: each warp streams its strip's rows through its own ring
// ---------------------------------------------------------------------------
// The plain-load strip keeps one row per warp in flight (binary64), so at
// 4096^2 the kernel waits on load latency with DRAM at a quarter of its
// bandwidth.  Here every warp owns a ring of kTmaRing boxes of kTmaRows rows
// of its strip and the two halo columns (34 columns of binary64, 36 of
// binary32: a 16-byte multiple), each box one cp.async.bulk.tensor copy that
// completes on the box's own mbarrier.  Lane 0 issues; every lane reads its
// column (and lanes 0 and 31 the halo columns) from shared memory into the
// same register queue as the plain-load strip, and a box's slot is refilled
// as soon as its last row has been read.  The warps of a CTA never wait on
// each other.  Rows beyond the array read as zero (the tensor map's
// out-of-bounds fill) and are never written.
constexpr int kTmaRows = 4;  // rows per box
constexpr int kTmaRing = 4;  // boxes per warp: 16 rows in flight

template <typename T, int kWarps>
struct TmaStrip {
  static constexpr int BX = sizeof(T) == 8 ? 34 : 36;  // box columns k0-1 .. k0+BX-2
  static constexpr int kBoxBytes = BX * kTmaRows * int(sizeof(T));
  static constexpr int kSlot = (kBoxBytes + 127) / 128 * 128;  // 128-byte aligned slots
  static constexpr int kWarpBytes = kTmaRing * kSlot;
  static constexpr size_t smem() { return size_t(kWarps) * (kWarpBytes + kTmaRing * sizeof(uint64_t)); }
};

// Output rows [ib, ie) of the strip at columns k0 .. k0+31 (warp-collective),
// from the tensor map `map` of the source array (read through the tensormap
// proxy; a map in global memory must be fenced before its first use).  FXW:
// this warp evaluates in fixed point.  Returns false when a wait gave up
// (after waiting, bounded, for the copies it still had in flight).
template <typename T, bool FXW, int MAD, bool IMUL>
__device__ __forceinline__ bool tma_strip_rows(const CUtensorMap* map, const T* src, T* dst, int64_t nx,
                                               int64_t k0, int64_t ib, int64_t ie, unsigned char* ring,
                                               uint64_t* bars, uint32_t one) {
  using G = TmaStrip<T, 8>;
  using St = Strip<T, FXW, false, MAD, IMUL, false>;
  using S = typename St::S;
  const St s(src, dst, nx, k0, one);
  const int lane = threadIdx.x & 31;
  const int nrows = int(ie - ib) + 2;  // staged rows ib-1 .. ie
  const int nbox = (nrows + kTmaRows - 1) / kTmaRows;
  const int x0 = int(k0 - 1), y0 = int(ib - 1);  // x0 = 32 * strip: a 16-byte multiple
  auto issue = [&](int b) {
    uint64_t* bar = &bars[b % kTmaRing];
    tma::mbar_arrive_expect_tx(bar, G::kBoxBytes);
    tma::load_3d(ring + (b % kTmaRing) * G::kSlot, map, x0, y0 + b * kTmaRows, 0, bar);
  };
  auto read = [&](int q, S& own, S& halo) {
    const T* row = reinterpret_cast<const T*>(ring + ((q / kTmaRows) % kTmaRing) * G::kSlot) +
                   (q % kTmaRows) * G::BX;
    const T v = row[lane + 1];
    if constexpr (FXW) own = fx::from_f64_f59_or_poison(v); else own = v;
    if (lane == 0 || lane == 31) {
      const T h = row[lane == 0 ? 0 : 33];
      if constexpr (FXW) halo = fx::from_f64_f59_or_poison(h); else halo = h;
    }
  };
  const int first = nbox < kTmaRing ? nbox : kTmaRing;
  if (lane == 0)
    for (int b = 0; b < first; ++b) issue(b);
  int issued = first, waited = 0;  // boxes issued; boxes whose wait completed
  bool ok = tma::mbar_wait(&bars[0], 0);
  if (ok) waited = 1;
  S xp = S(0), xc = S(0), xn = S(0), hp = S(0), hc = S(0), hn = S(0);
  if (ok) {
    read(0, xp, hp);
    read(1, xc, hc);
  }
  for (int q = 1; ok && q + 1 < nrows; ++q) {  // output row ib - 1 + q
    const int qn = q + 1;
    if (qn % kTmaRows == 0) {
      const int b = qn / kTmaRows;
      ok = tma::mbar_wait(&bars[b % kTmaRing], uint32_t((b / kTmaRing) & 1));
      if (!ok) break;
      waited = b + 1;
    }
    read(qn, xn, hn);
    if (qn % kTmaRows == kTmaRows - 1) {  // box fully read: refill its slot
      tma::fence_proxy_async();
      __syncwarp();
      const int b = qn / kTmaRows + kTmaRing;
      if (b < nbox) {
        if (lane == 0) issue(b);
        issued = b + 1;
      }
    }
    s.point(ib - 1 + q, xp, xc, xn, hc);
    xp = xc;
    xc = xn;
    hc = hn;
  }
  if (!ok)  // let the copies still in flight (the late one included) land, bounded, before exit
    for (int b = waited; b < issued; ++b)
      tma::mbar_wait_for(&bars[b % kTmaRing], uint32_t((b / kTmaRing) & 1), tma::kWaitLimitNs / 16);
  return ok;
}

// One strip (columns k0 .. k0+31) over rows [r0, r1).  Warp-collective.
template <typename T, bool FX, bool CG, int U, int MAD = 0, bool IMUL = true, bool HWIMUL = false>
__device__ __forceinline__ void strip_rows(const T* src, T* dst, int64_t nx, int64_t k0, int64_t r0,
                                           int64_t r1, uint32_t one) {
  using St = Strip<T, FX, CG, MAD, IMUL, HWIMUL>;
  using S = typename St::S;
  const St s(src, dst, nx, k0, one);
  S x[U + 2], h[U + 2];
#pragma unroll
  for (int u = 0; u < U + 2; ++u) { x[u] = S(0); h[u] = S(0); }
  s.load(r0 - 1, x[0], h[0]);
  s.load(r0, x[1], h[1]);
  int64_t i = r0;
  for (; i + U <= r1; i += U) {
#pragma unroll
    for (int u = 0; u < U; ++u) s.load(i + 1 + u, x[2 + u], h[2 + u]);
    if constexpr (!FX && std::is_same<T, float>::value && U % 2 == 0) {
#pragma unroll
      for (int u = 0; u < U; u += 2)
        points2_f32<CG, MAD, IMUL, HWIMUL>(s, i + u, x[u], x[u + 1], x[u + 2], x[u + 3], h[u + 1], h[u + 2]);
    } else {
#pragma unroll
      for (int u = 0; u < U; ++u) s.point(i + u, x[u], x[u + 1], x[u + 2], h[u + 1]);
    }
    x[0] = x[U];
    x[1] = x[U + 1];
    h[1] = h[U + 1];
  }
  for (; i < r1; ++i) {
    s.load(i + 1, x[2], h[2]);
    s.point(i, x[0], x[1], x[2], h[1]);
    x[0] = x[1];
    x[1] = x[2];
    h[1] = h[2];
  }
}

}  // namespace jcore
}  // namespace npbgb
