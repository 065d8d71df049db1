// 3D 7-point heat time loop (polybench/heat_3d/heat_3d_numpy.py:4-20).
//
// Per interior point, in the reference's order:
//   tx  = 0.125 * ((next_x - 2*c) + prev_x)      x = axis 0, 1, 2
//   dst = ((t0 + t1) + t2) + c
//
// One launch per half-sweep.  A CTA owns a TJ x 32 tile of the
// (axis 1, axis 2) plane -- axis 2 contiguous, one element per lane -- and
// streams along axis 0 over a chunk of planes.
//
// heat3d_tma (used when the arrays meet the TMA alignment rules): each
//   halo'd plane tile arrives by one cp.async.bulk.tensor copy into an
//   NSTAGE-deep ring of shared-memory buffers, completion tracked by one
//   mbarrier per buffer, so several planes per CTA are in flight while the
//   current one is computed.  Planes i-1, i, i+1 are read from shared memory.
// heat3d_ldg (any layout): each plane tile is staged by plain loads into
//   three rotating shared buffers; axis-0 neighbours stay in registers.
//
// binary32 uses IEEE float operations.  binary64 runs in fixed point on the
// integer pipe (fx64.cuh): staged values are converted once to frame-59
// integers, values outside [2^-7, 1) (other than +0) are marked with a poison
// bit, and a point whose seven inputs are all clean is evaluated with exact
// integer adds and round53; any other point is evaluated with hardware
// binary64 from global memory.  Both give the IEEE result bit for bit.
#include <algorithm>
#include <type_traits>

#include "fx64.cuh"
#include "heat_core.cuh"
#include "npbgb_common.cuh"
#include "tma.cuh"

namespace npbgb {

extern int64_t g_cfg_f64_emulation;
extern int64_t g_cfg_heat_chunk;
extern int64_t g_cfg_heat_tma;
extern int64_t g_cfg_heat_rows;
extern int64_t g_cfg_heat_hw_rows;
extern int64_t g_cfg_f64_cvt;
extern int64_t g_cfg_heat_tb;
extern int64_t g_cfg_heat_stages;
extern int64_t g_cfg_heat_mad_rows;

int32_t heat3d_tb2_run(float* a, float* b, int64_t n0, int64_t n1, int64_t n2, int32_t tsteps,
                       cudaStream_t st, int32_t (*single_pairs)(float*, float*, int64_t, int64_t,
                                                                int64_t, int32_t, cudaStream_t));

namespace {

__device__ unsigned int g_heat_error;  // bit 0: an mbarrier wait timed out

using hcore::kThreads;
using hcore::kTJ;
using hcore::kTK;
using hcore::heat_point;
using hcore::to_fx;
using fx::hi32;
using fx::kPoisonHi;

// ---------------------------------------------------------------------------
// TMA pipeline
// ---------------------------------------------------------------------------
// Fixed-point point update.  MAD: the 64-bit adds are issued as multiply-adds
// (fx::add64 / fx::round53m) to shift work from the integer ALU pipe to the
// multiply-add pipe; otherwise plain integer adds.
template <bool CVT, bool MAD>
__device__ __forceinline__ double heat_point_fxm(int64_t c, int64_t ip, int64_t im, int64_t jp,
                                                 int64_t jm, int64_t kp, int64_t km, uint32_t one) {
  auto add = [one](int64_t x, int64_t y) {
    if constexpr (MAD) return fx::add64(x, y, one); else return int64_t(uint64_t(x) + uint64_t(y));
  };
  auto rnd = [one](int64_t x) {
    if constexpr (MAD) return fx::round53m(x, one); else return fx::round53(x);
  };
  const int64_t nc2 = -2 * c;
  const int64_t s0 = rnd(add(rnd(add(ip, nc2)), im));
  const int64_t s1 = rnd(add(rnd(add(jp, nc2)), jm));
  const int64_t s2 = rnd(add(rnd(add(kp, nc2)), km));
  const int64_t u = rnd(add(s0, s1));
  const int64_t v = rnd(add(u, s2));
  if constexpr (!CVT && !MAD) return fx::round_to_f64<62>(add(v, c * 8));
  const int64_t w = rnd(add(v, c * 8));
  if constexpr (CVT) return fx::to_f64_cvt<62>(w);
  return fx::to_f64<62>(w);
}

template <typename T, int R>
struct TmaGeom {
  static constexpr int BX = sizeof(T) == 8 ? 34 : 36;  // rows of a 16-byte multiple
  static constexpr int TJ = kTJ * R;                   // tile rows (axis 1)
  static constexpr int BY = TJ + 2;
  static constexpr int kElems = BX * BY;
  static constexpr int kBytes = kElems * int(sizeof(T));
  static constexpr int kStride = (kBytes + 127) / 128 * 128;  // stage pitch, 128-byte aligned
};

constexpr int kStages = 8;  // ring depth of the binary64 kernels (binary32: NPBGB_CFG_HEAT_STAGES)
// Output planes per CTA barrier: fixed point (the barrier also publishes the
// conversion of the staged planes; 3 measured 3% faster than 1 at 256^3) and
// plain binary32/binary64.  The prologue stages kStages - kSync planes and
// the first step converts planes 2 .. kSync + 1, and the planes a step
// converts must not share buffers with the kSync + 2 planes that slower warps
// may still read for the previous step: both need kStages >= 2 * kSync + 2.
constexpr int kSyncFx = 3, kSyncPlain = 1;
static_assert(kSyncFx >= 1 && 2 * kSyncFx + 2 <= kStages && kSyncPlain >= 1 &&
                  2 * kSyncPlain + 2 <= kStages,
              "staging ring too short for the planes per barrier");

// R: tile rows per thread.  FX: binary64 in fixed point.  CVT: fixed-point
// conversions through the binary64 conversion path.  hw_rows: the last
// hw_rows tile rows are evaluated with hardware binary64 (from global memory)
// so that the binary64 pipe works alongside the integer pipe.  one == 1.
template <typename T, bool FX, int R, bool CVT, int NS>
__global__ void __launch_bounds__(kThreads)
heat3d_tma(const __grid_constant__ CUtensorMap src_map, const T* __restrict__ src,
           T* __restrict__ dst, int64_t n0, int64_t n1, int64_t n2, int chunk, int hw_rows,
           int mad_rows, uint32_t one) {
  pdl_begin();
  using G = TmaGeom<T, R>;
  using S = typename std::conditional<FX, int64_t, T>::type;
  constexpr int kSync = FX ? kSyncFx : kSyncPlain;
  constexpr int kStages = NS;
  static_assert(2 * kSync + 2 <= kStages, "staging ring too short for the planes per barrier");
  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + kStages * G::kStride);

  const int tid = threadIdx.x;
  const int tx = tid & 31, ty = tid >> 5;
  const int64_t k0 = 1 + int64_t(blockIdx.x) * kTK, j0 = 1 + int64_t(blockIdx.y) * G::TJ;
  const int64_t k = k0 + tx;
  const bool k_ok = k < n2 - 1;
  const int64_t s0 = n1 * n2, s1 = n2;
  const int64_t ib = 1 + int64_t(blockIdx.z) * chunk;
  const int64_t ie = (ib + chunk < n0 - 1) ? ib + chunk : n0 - 1;
  const int M = int(ie - ib);     // output planes
  const int Q = M + 2;            // staged planes ib-1 .. ie
  // Tile origin: x = k0 - 1 = 32 * blockIdx.x, a multiple of 4 elements (16 bytes).
  const int x0 = int(k0 - 1), y0 = int(j0 - 1);

  auto stage_ptr = [&](int q) -> S* {
    return reinterpret_cast<S*>(smem + (q % kStages) * G::kStride);
  };
  int issued = 0;     // planes issued so far (thread 0 issues them, in order)
  int next_wait = 0;  // planes this thread has seen land
  auto issue = [&](int q) {
    uint64_t* bar = &bars[q % kStages];
    tma::mbar_arrive_expect_tx(bar, G::kBytes);
    tma::load_3d(smem + (q % kStages) * G::kStride, &src_map, x0, y0, int(ib - 1 + q), bar);
    issued = q + 1;
  };
  auto wait = [&](int q) -> bool {
    const bool landed = tma::mbar_wait(&bars[q % kStages], uint32_t((q / kStages) & 1));
    if (landed) next_wait = q + 1;
    return landed;
  };
  auto convert = [&](int q) {
    if constexpr (FX) {
      unsigned char* base = smem + (q % kStages) * G::kStride;
      for (int e = tid; e < G::kElems; e += kThreads) {
        const double v = reinterpret_cast<const double*>(base)[e];
        reinterpret_cast<int64_t*>(base)[e] =
            CVT ? fx::from_f64_f59_cvt(v) : fx::from_f64_f59_or_poison(v);
      }
    }
  };

  if (tid == 0) {
    for (int s = 0; s < kStages; ++s) tma::mbar_init(&bars[s], 1);
    tma::fence_mbar_init();
  }
  __syncthreads();
  if (tid == 0) {
    const int n_first = Q < kStages - kSync ? Q : kStages - kSync;
    for (int q = 0; q < n_first; ++q) issue(q);
  }
  bool ok = wait(0);
  if (ok) convert(0);
  ok = ok && wait(1);
  if (ok) convert(1);

  // kSync output planes per CTA barrier: the barrier publishes the conversion
  // of staged planes m2+2 .. m2+kSync+1 and frees the buffers of planes
  // m2-kSync .. m2-1, which are refilled with planes kStages further on.
  for (int m2 = 0; m2 < M; m2 += kSync) {
#pragma unroll
    for (int d = 0; d < kSync; ++d) {
      const int q = m2 + 2 + d;
      if (q < Q) {
        ok = ok && wait(q);
        if (ok) convert(q);
      }
    }
    tma::fence_proxy_async();  // order this thread's generic smem accesses before later bulk writes
    if (__syncthreads_or(!ok)) {
      if (tid == 0) {
        atomicOr(&g_heat_error, 1u);
        // let the copies still in flight land (bounded) before the CTA exits
        for (int q = next_wait; q < issued; ++q)
          tma::mbar_wait_for(&bars[q % kStages], uint32_t((q / kStages) & 1), tma::kWaitLimitNs / 16);
      }
      return;
    }
    if (tid == 0) {
#pragma unroll
      for (int d = 0; d < kSync; ++d) {
        const int q = m2 - kSync + d + kStages;
        if (q < Q) issue(q);
      }
    }
#pragma unroll 1
    for (int m = m2; m < m2 + kSync && m < M; ++m) {
    const int64_t i = ib + m;
    // This warp's rows row0 .. row0+R-1; the column of plane i for rows
    // row0-1 .. row0+R is read once and reused as the rows' j-neighbours.
    const int row0 = ty * R;
    const S* pm = stage_ptr(m);
    const S* pc = stage_ptr(m + 1);
    const S* pp = stage_ptr(m + 2);
    S col[R + 2];
#pragma unroll
    for (int r = 0; r < R + 2; ++r) col[r] = pc[(row0 + r) * G::BX + tx + 1];
    const int64_t gbase = i * s0 + (j0 + row0) * s1 + k;
    if constexpr (!FX && sizeof(T) == 4 && R % 2 == 0) {
      // binary32: rows r and r+1 in one packed f32x2 evaluation.
      if (k_ok) {
#pragma unroll
        for (int r = 0; r < R; r += 2) {
          const int row = row0 + r;
          if (j0 + row >= n1 - 1) break;
          const int off = (row + 1) * G::BX + (tx + 1);
          const int64_t g = gbase + r * s1;
          const F2 o = hcore::heat_point2(
              f2(col[r + 1], col[r + 2]), f2(pp[off], pp[off + G::BX]), f2(pm[off], pm[off + G::BX]),
              f2(col[r + 2], col[r + 3]), f2(col[r], col[r + 1]),
              f2(pc[off + 1], pc[off + 1 + G::BX]), f2(pc[off - 1], pc[off - 1 + G::BX]));
          dst[g] = f2x(o);
          if (j0 + row + 1 < n1 - 1) dst[g + s1] = f2y(o);
        }
      }
    } else {
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const int row = row0 + r;
        if (!k_ok || j0 + row >= n1 - 1) continue;
        const int off = (row + 1) * G::BX + (tx + 1);
        const int64_t g = gbase + r * s1;
        const T* q = src + g;
        T out;
        if constexpr (FX) {
          const bool hw = row >= G::TJ - hw_rows;  // warp-uniform
          if (hw) {
            out = heat_point<T>(q[0], q[s0], q[-s0], q[s1], q[-s1], q[1], q[-1]);
          } else {
            const int64_t c = col[r + 1], ip = pp[off], im = pm[off], jp = col[r + 2], jm = col[r],
                          kp = pc[off + 1], km = pc[off - 1];
            const uint32_t tag =
                hi32(c) | hi32(ip) | hi32(im) | hi32(jp) | hi32(jm) | hi32(kp) | hi32(km);
            if (!(tag & kPoisonHi))
              out = row < mad_rows ? heat_point_fxm<CVT, true>(c, ip, im, jp, jm, kp, km, one)
                                   : heat_point_fxm<CVT, false>(c, ip, im, jp, jm, kp, km, one);
            else
              out = heat_point<T>(q[0], q[s0], q[-s0], q[s1], q[-s1], q[1], q[-1]);
          }
        } else {
          out = heat_point<T>(col[r + 1], pp[off], pm[off], col[r + 2], col[r], pc[off + 1],
                              pc[off - 1]);
        }
        dst[g] = out;
      }
    }
    }
  }
}

// ---------------------------------------------------------------------------
// Plain-load pipeline (any alignment)
// ---------------------------------------------------------------------------
template <typename T, bool FX>
__global__ void __launch_bounds__(kThreads)
heat3d_ldg(const T* __restrict__ src, T* __restrict__ dst, int64_t n0, int64_t n1, int64_t n2,
           int chunk) {
  pdl_begin();
  __shared__ hcore::PlaneBuf<T, FX> plane;
  const int64_t k0 = 1 + int64_t(blockIdx.x) * kTK, j0 = 1 + int64_t(blockIdx.y) * kTJ;
  const int64_t ib = 1 + int64_t(blockIdx.z) * chunk;
  const int64_t ie = (ib + chunk < n0 - 1) ? ib + chunk : n0 - 1;
  hcore::tile_stream<T, FX, false>(src, dst, n1, n2, j0, k0, ib, ie, plane);
}

int auto_chunk(int64_t n0, int64_t tiles, int ctas_per_sm, int waves) {
  // Smallest number of axis-0 chunks that fills about `waves` waves of CTAs:
  // 2 for binary32 (memory-bound; long chunks amortise the halo planes), 16
  // for binary64 (pipe-bound; many short CTAs balance the last wave: 8-plane
  // chunks measured 6% faster than 64 at 256^3).
  const int64_t slots = int64_t(sm_count()) * (ctas_per_sm > 0 ? ctas_per_sm : 1);
  int64_t chunks = cdiv(int64_t(waves) * slots, tiles > 0 ? tiles : 1);
  if (chunks < 1) chunks = 1;
  int64_t c = cdiv(n0 - 2, chunks);
  if (c < 4) c = 4;
  if (c > n0 - 2) c = n0 - 2;
  return int(c);
}

// Binary32 planes per CTA.  A CTA whose chunk's planes (chunk + 2) all fit in
// the ring's first copies (kStages - 1) issues every copy at once, so short
// chunks keep many CTAs' copies in flight.  Measured on GB300 (TSTEPS=21, 4
// tile rows per warp, 8-deep ring, fraction of the measured copy bandwidth at
// 8 bytes per update): 5 planes give 0.77, 0.80, 0.83 and 0.86 at 384^3,
// 416^3, 512^3 and 640^3 (4 planes: 0.76-0.83; 6: 0.75-0.79), against 0.62,
// 0.60, 0.55 and 0.50 for the 2-wave chunks; at 256^3, whose pair L2 largely
// holds, 8 planes give 0.71 (5: 0.69, 2-wave: 0.70).
int f32_chunk_cap(int64_t array_bytes) {
  return array_bytes >= (int64_t(128) << 20) ? 5 : 8;
}

template <typename T, bool FX, int R, bool CVT, int NS = kStages>
int32_t launch_tma(T* a, T* b, int64_t n0, int64_t n1, int64_t n2, int32_t tsteps, cudaStream_t st) {
  using G = TmaGeom<T, R>;
  constexpr int kStages = NS;
  const size_t smem = size_t(kStages) * G::kStride + kStages * sizeof(uint64_t);
  CUtensorMap map_a, map_b;
  const uint64_t dims[3] = {uint64_t(n2), uint64_t(n1), uint64_t(n0)};
  const uint32_t box[3] = {uint32_t(G::BX), uint32_t(G::BY), 1u};
  if (tma::encode_3d(&map_a, sizeof(T), a, dims, box) != cudaSuccess ||
      tma::encode_3d(&map_b, sizeof(T), b, dims, box) != cudaSuccess)
    return NPBGB_ERR_STATE;  // caller falls back to plain staging
  static bool attr_done = false;
  if (!attr_done) {
    cudaError_t e = cudaFuncSetAttribute(heat3d_tma<T, FX, R, CVT, NS>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess) return cuda_status(e, "heat3d: smem attribute");
    attr_done = true;
  }
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, heat3d_tma<T, FX, R, CVT, NS>, kThreads, smem);
  const int64_t gx = cdiv(n2 - 2, kTK), gy = cdiv(n1 - 2, G::TJ);
  int chunk = g_cfg_heat_chunk > 0 ? int(g_cfg_heat_chunk)
                                   : auto_chunk(n0, gx * gy, per_sm, FX ? 16 : 2);
  if (g_cfg_heat_chunk <= 0 && sizeof(T) == 4)
    chunk = std::min(chunk, f32_chunk_cap(n0 * n1 * n2 * int64_t(sizeof(T))));
  const int64_t gz = cdiv(n0 - 2, chunk);
  if (gy > 65535 || gz > 65535 || gx > 0x7fffffff)
    return set_error(NPBGB_ERR_ARG, "heat3d: extent too large");
  const dim3 grid{unsigned(gx), unsigned(gy), unsigned(gz)};
  // Tile rows on the hardware binary64 pipe, measured best at 256^3 (40
  // half-sweeps): 5 of 16 with 2 rows per warp (5.18 ms; 4 rows 5.22, 6 rows
  // 5.30, 7 rows 5.76) since the fixed-point rounding takes one leading-bit
  // instruction and clamped shifts; 3 of 8 with 1 row per warp (5.24 ms), 6 of
  // 32 with 4 (6.15 ms).
  const int hw_default = R == 2 ? 5 : (R == 1 ? 3 : 6);
  int hw = g_cfg_heat_hw_rows >= 0 ? int(g_cfg_heat_hw_rows) : (FX ? hw_default : 0);
  if (hw > G::TJ) hw = G::TJ;
  // Fixed-point tile rows (the first mad rows) whose 64-bit adds go to the
  // multiply-add pipe instead of the integer ALU.
  const int mad = FX ? int(std::min<int64_t>(g_cfg_heat_mad_rows, G::TJ)) : 0;
  const dim3 block{unsigned(kThreads)};
  cudaError_t e = cudaSuccess;
  for (int32_t t = 1; t < tsteps && e == cudaSuccess; ++t) {
    e = launch_chained(heat3d_tma<T, FX, R, CVT, NS>, grid, block, smem, st, map_a, a, b, n0, n1, n2,
                       chunk, hw, mad, 1u);
    if (e == cudaSuccess)
      e = launch_chained(heat3d_tma<T, FX, R, CVT, NS>, grid, block, smem, st, map_b, b, a, n0, n1,
                         n2, chunk, hw, mad, 1u);
  }
  return cuda_status(e, "heat3d_tma");
}

template <typename T, bool FX>
int32_t launch_ldg(T* a, T* b, int64_t n0, int64_t n1, int64_t n2, int32_t tsteps, cudaStream_t st) {
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, heat3d_ldg<T, FX>, kThreads, 0);
  const int64_t gx = cdiv(n2 - 2, kTK), gy = cdiv(n1 - 2, kTJ);
  const int chunk = g_cfg_heat_chunk > 0 ? int(g_cfg_heat_chunk)
                                         : auto_chunk(n0, gx * gy, per_sm, FX ? 16 : 2);
  const int64_t gz = cdiv(n0 - 2, chunk);
  if (gy > 65535 || gz > 65535 || gx > 0x7fffffff)
    return set_error(NPBGB_ERR_ARG, "heat3d: extent too large");
  const dim3 grid{unsigned(gx), unsigned(gy), unsigned(gz)};
  const dim3 block{unsigned(kThreads)};
  cudaError_t e = cudaSuccess;
  for (int32_t t = 1; t < tsteps && e == cudaSuccess; ++t) {
    e = launch_chained(heat3d_ldg<T, FX>, grid, block, 0, st, a, b, n0, n1, n2, chunk);
    if (e == cudaSuccess)
      e = launch_chained(heat3d_ldg<T, FX>, grid, block, 0, st, b, a, n0, n1, n2, chunk);
  }
  return cuda_status(e, "heat3d_ldg");
}

template <typename T, bool FX>
int32_t run_single(T* a, T* b, int64_t n0, int64_t n1, int64_t n2, int32_t tsteps, cudaStream_t st) {
  if (tsteps <= 1 || n0 < 3 || n1 < 3 || n2 < 3) return NPBGB_OK;
  if (g_cfg_heat_tma) {
    // Tuned on GB300 (256^3): binary32 is memory-latency bound and wants more
    // rows per thread; binary64 (integer-pipe bound) wants one.
    const int rows = g_cfg_heat_rows > 0 ? int(g_cfg_heat_rows) : (sizeof(T) == 4 ? 4 : 2);
    const bool cvt = g_cfg_f64_cvt != 0;
    int32_t r;
    if constexpr (sizeof(T) == 4 && !FX) {
      // binary32: the depth of the plane ring is a knob (no conversion step)
      const int64_t ns = g_cfg_heat_stages;
      if (rows >= 4)
        r = ns == 4   ? launch_tma<T, FX, 4, false, 4>(a, b, n0, n1, n2, tsteps, st)
            : ns == 6 ? launch_tma<T, FX, 4, false, 6>(a, b, n0, n1, n2, tsteps, st)
                      : launch_tma<T, FX, 4, false, 8>(a, b, n0, n1, n2, tsteps, st);
      else if (rows == 2)
        r = launch_tma<T, FX, 2, false>(a, b, n0, n1, n2, tsteps, st);
      else
        r = launch_tma<T, FX, 1, false>(a, b, n0, n1, n2, tsteps, st);
    } else if (rows >= 4)
      r = cvt ? launch_tma<T, FX, 4, true>(a, b, n0, n1, n2, tsteps, st)
              : launch_tma<T, FX, 4, false>(a, b, n0, n1, n2, tsteps, st);
    else if (rows == 2)
      r = cvt ? launch_tma<T, FX, 2, true>(a, b, n0, n1, n2, tsteps, st)
              : launch_tma<T, FX, 2, false>(a, b, n0, n1, n2, tsteps, st);
    else
      r = cvt ? launch_tma<T, FX, 1, true>(a, b, n0, n1, n2, tsteps, st)
              : launch_tma<T, FX, 1, false>(a, b, n0, n1, n2, tsteps, st);
    if (r != NPBGB_ERR_STATE) return r;
  }
  return launch_ldg<T, FX>(a, b, n0, n1, n2, tsteps, st);
}

int32_t run_single_f32(float* a, float* b, int64_t n0, int64_t n1, int64_t n2, int32_t tsteps,
                       cudaStream_t st) {
  return run_single<float, false>(a, b, n0, n1, n2, tsteps, st);
}

// Binary32 takes two half-sweeps per launch (heat_tb.cu) only when asked
// (NPBGB_CFG_HEAT_TB = 2).  Measured on GB300 at TSTEPS=21, the single-step
// kernel with 5-plane chunks reaches 0.77-0.86 of the measured copy bandwidth
// at 384^3 to 640^3, and the two-step kernel at most 0.62-0.69 over its chunk
// sizes: the two-step kernel halves the HBM bytes but is bound by its
// instruction issue.  Binary64 (bound by its arithmetic pipes) takes one.
template <typename T, bool FX>
int32_t run(T* a, T* b, int64_t n0, int64_t n1, int64_t n2, int32_t tsteps, cudaStream_t st) {
  if constexpr (sizeof(T) == 4) {
    if (g_cfg_heat_tb == 2 && g_cfg_heat_tma && tsteps >= 4) {
      const int32_t r = heat3d_tb2_run(a, b, n0, n1, n2, tsteps, st, run_single_f32);
      if (r != NPBGB_ERR_STATE) return r;
    }
  }
  return run_single<T, FX>(a, b, n0, n1, n2, tsteps, st);
}

// One CTA waits, with a short limit, on an mbarrier that nothing completes;
// the timeout path records the error word exactly as a lost copy would.
__global__ void wait_timeout_selftest(uint64_t limit_ns) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) {
    tma::mbar_init(&bar, 1);
    tma::fence_mbar_init();
  }
  __syncthreads();
  const bool ok = tma::mbar_wait_for(&bar, 0, limit_ns);
  if (__syncthreads_or(!ok) && threadIdx.x == 0) atomicOr(&g_heat_error, 1u);
}

}  // namespace

int32_t launch_wait_timeout_selftest(uint64_t limit_ns, cudaStream_t st) {
  wait_timeout_selftest<<<1, 64, 0, st>>>(limit_ns);
  NPBGB_CHECK_LAUNCH("wait_timeout_selftest");
  return NPBGB_OK;
}

// Reads and clears this file's device error word (host; synchronises with the device).
uint32_t take_heat_device_error() {
  unsigned int v = 0, zero = 0;
  if (cudaMemcpyFromSymbol(&v, g_heat_error, sizeof(v)) != cudaSuccess) return 0xffffffffu;
  if (v) cudaMemcpyToSymbol(g_heat_error, &zero, sizeof(zero));
  return v;
}

}  // namespace npbgb

extern "C" int32_t npbgb_heat3d(void* A, void* B, int64_t n0, int64_t n1, int64_t n2,
                                int32_t tsteps, int32_t dtype, void* stream) {
  using namespace npbgb;
  if (n0 < 0 || n1 < 0 || n2 < 0) return set_error(NPBGB_ERR_ARG, "heat3d: negative extent");
  if (tsteps > 1 && n0 >= 3 && n1 >= 3 && n2 >= 3) {
    if (!A || !B) return set_error(NPBGB_ERR_ARG, "heat3d: null array");
    if (A == B) return set_error(NPBGB_ERR_ARG, "heat3d: A and B alias");
  }
  cudaStream_t st = as_stream(stream);
  if (dtype == NPBGB_F64) {
    double* a = static_cast<double*>(A);
    double* b = static_cast<double*>(B);
    return g_cfg_f64_emulation ? run<double, true>(a, b, n0, n1, n2, tsteps, st)
                               : run<double, false>(a, b, n0, n1, n2, tsteps, st);
  }
  if (dtype == NPBGB_F32)
    return run<float, false>(static_cast<float*>(A), static_cast<float*>(B), n0, n1, n2, tsteps, st);
  return set_error(NPBGB_ERR_DTYPE, "heat3d: dtype %d", dtype);
}
