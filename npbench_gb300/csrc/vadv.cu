// Vertical advection, vadv(utens_stage, u_stage, wcon, u_pos, utens, dtr_stage)
// (weather_stencils/vadv/vadv_numpy.py:9-78), binary64.
//
// Arrays are (I, J, K) with K contiguous; wcon is (I+1, J, K).  Every (i, j)
// column is an independent tridiagonal (Thomas) solve along K, so one thread
// owns one column and walks it: forward elimination k = 0..K-1, then back
// substitution k = K-1..0.  With w_k = wcon[i+1,j,k] + wcon[i,j,k] and
// q_k = (0.25 * w_k) * 0.5, the reference's coefficients are
//   gcv*BET_M = gcv*BET_P = q_{k+1}         (cs and the unscaled ccol_k)
//   gav*BET_M = gav*BET_P = -q_k            (as and acol)
// (0.25*w)*0.5 and (-0.25*w)*0.5 differ only in sign, bit for bit), and per
// level, in the reference's order:
//   bcol    = (dtr - acol) - q_{k+1}
//   corr    = q_k*(u[k-1] - u[k]) - q_{k+1}*(u[k+1] - u[k])     ((-as) = q_k)
//   d       = ((dtr*u_pos[k] + utens[k]) + utens_stage[k]) + corr
//   divided = 1.0 / (bcol - ccol_{k-1}*acol)
//   ccol_k  = q_{k+1}*divided;  dcol_k = (d - dcol_{k-1}*acol)*divided
// with the one-sided forms at k = 0 and k = K-1; then
//   data = dcol_k - ccol_k*data;  utens_stage[k] = dtr*(data - u_pos[k]).
// Every operator is one correctly rounded IEEE operation (no contraction), and
// 1.0/x is the correctly rounded reciprocal, so results are bit-identical to
// NumPy's.  The exact scalings (q_k from w_k, negation) are done on the
// integer pipe; GB300's binary64 pipe is the bound of this kernel.
//
// Storage: ccol_k goes to a workspace laid out [K-1][I*J] (a warp's 32
// columns write one contiguous 256-byte run per level); dcol_k is kept in
// utens_stage[.., k] itself, which the forward sweep has already read and the
// back substitution overwrites with the result.
#include "npbgb_common.cuh"

namespace npbgb {
namespace {

constexpr int kThreads = 64;

// (0.25 * w) * 0.5 as the reference rounds it.  For a normal w whose
// exponent field is at least 4 both products are exact and together subtract
// 3 from the exponent; everything else (zero, subnormal results, inf, NaN)
// takes the literal products, out of line so the common path stays unpredicated.
__device__ __noinline__ double eighth_literal(double w) { return mul_rn(mul_rn(0.25, w), 0.5); }
__device__ __forceinline__ double eighth_of(double w) {
  const uint64_t b = static_cast<uint64_t>(__double_as_longlong(w));
  const uint32_t e = static_cast<uint32_t>(b >> 52) & 0x7ffu;
  if (e >= 4u && e <= 2046u) return __longlong_as_double(static_cast<long long>(b - (3ull << 52)));
  return eighth_literal(w);
}
__device__ __forceinline__ double neg(double x) {
  return __longlong_as_double(__double_as_longlong(x) ^ static_cast<long long>(0x8000000000000000ull));
}
__device__ __forceinline__ double ld(const double* p) { return __ldg(p); }

// The values one forward level reads (wh/wl/u ahead of it, u_pos/utens/
// utens_stage at it), and those one back-substitution level reads.
struct FwdLevel { double wh, wl, u, up, ut, s; };
struct BwdLevel { double s, c, up; };

// Each thread's loads hit its own column, K doubles apart from its
// neighbours', and the recurrence consumes them at once; loaded in place, every
// level would wait out a memory latency.  So both sweeps keep a ring of kRing
// levels in registers: level m lives in slot m % kRing, and the slot of the
// level just consumed is refilled with the level kRing further on (indices
// clamped into [0, K), so loads past either end are in bounds and unused).  The
// loops are unrolled by kRing so every slot index is a compile-time constant
// and no register holding an in-flight load is ever copied (a copy would wait
// for the load); the latency overlaps the binary64 work of kRing-1 levels.
constexpr int kRing = 6;

__global__ void __launch_bounds__(kThreads)
vadv_columns(double* __restrict__ us, const double* __restrict__ u, const double* __restrict__ wcon,
             const double* __restrict__ up, const double* __restrict__ ut, double dtr,
             int64_t ncol, int64_t J, int64_t K, double* __restrict__ ccol) {
  const int64_t c = int64_t(blockIdx.x) * kThreads + threadIdx.x;
  if (c >= ncol) return;
  const int64_t base = c * K;
  const double* wl = wcon + base;      // wcon[i, j, :]
  const double* wh = wl + J * K;       // wcon[i+1, j, :]
  const double* uc = u + base;
  const double* upc = up + base;
  const double* utc = ut + base;
  double* s = us + base;
  auto fwd = [&](int64_t m) {
    m = m < K ? m : K - 1;
    return FwdLevel{ld(wh + m), ld(wl + m), ld(uc + m), ld(upc + m), ld(utc + m), s[m]};
  };

  FwdLevel r[kRing];
#pragma unroll
  for (int i = 0; i < kRing; ++i) r[i] = fwd(i);

  // k = 0 (slots 0 and 1)
  double qn = eighth_of(add_rn(r[1].wh, r[1].wl));  // q_1
  double ucur = r[0].u, unext = r[1].u;
  double d = add_rn(add_rn(add_rn(mul_rn(dtr, r[0].up), r[0].ut), r[0].s),
                    mul_rn(neg(qn), sub_rn(unext, ucur)));
  double dv = __drcp_rn(sub_rn(dtr, qn));
  double cprev = mul_rn(qn, dv);
  double dprev = mul_rn(d, dv);
  ccol[c] = cprev;
  s[0] = dprev;
  r[0] = fwd(kRing);

  // k = 1 .. K-2: level k in slot k % kRing, level k+1 in the next slot.
  for (int64_t kb = 0; kb < K - 1; kb += kRing) {
#pragma unroll
    for (int j = 0; j < kRing; ++j) {
      const int64_t k = kb + j;
      if (k < 1 || k > K - 2) continue;
      FwdLevel& cur = r[j];
      const FwdLevel& nxt = r[(j + 1) % kRing];
      const double q = qn;                                 // -acol = -as
      qn = eighth_of(add_rn(nxt.wh, nxt.wl));              // cs = unscaled ccol_k
      const double uprev = ucur;
      ucur = unext;
      unext = nxt.u;
      const double acol = neg(q);
      const double corr = sub_rn(mul_rn(q, sub_rn(uprev, ucur)), mul_rn(qn, sub_rn(unext, ucur)));
      d = add_rn(add_rn(add_rn(mul_rn(dtr, cur.up), cur.ut), cur.s), corr);
      const double bcol = sub_rn(sub_rn(dtr, acol), qn);
      dv = __drcp_rn(sub_rn(bcol, mul_rn(cprev, acol)));
      cprev = mul_rn(qn, dv);
      dprev = mul_rn(sub_rn(d, mul_rn(dprev, acol)), dv);
      ccol[k * ncol + c] = cprev;
      s[k] = dprev;
      cur = fwd(k + kRing);
    }
  }

  // k = K-1, read again (it may have been overwritten in its ring slot by a
  // clamped refill, which loads the same level).
  const FwdLevel last = fwd(K - 1);
  {
    const double q = qn;
    const double acol = neg(q);
    const double corr = mul_rn(q, sub_rn(ucur, unext));    // (-as)*(u[K-2] - u[K-1])
    d = add_rn(add_rn(add_rn(mul_rn(dtr, last.up), last.ut), last.s), corr);
    const double bcol = sub_rn(dtr, acol);
    dv = __drcp_rn(sub_rn(bcol, mul_rn(cprev, acol)));
    dprev = mul_rn(sub_rn(d, mul_rn(dprev, acol)), dv);
  }

  // Back substitution, levels K-2 .. 0: level K-2-t in slot t % kRing.
  auto bwd = [&](int64_t m) {
    m = m > 0 ? m : 0;
    return BwdLevel{s[m], ccol[m * ncol + c], ld(upc + m)};
  };
  double data = dprev;
  s[K - 1] = mul_rn(dtr, sub_rn(data, last.up));
  BwdLevel b[kRing];
#pragma unroll
  for (int i = 0; i < kRing; ++i) b[i] = bwd(K - 2 - i);
  for (int64_t tb = 0; tb < K - 1; tb += kRing) {
#pragma unroll
    for (int j = 0; j < kRing; ++j) {
      const int64_t k = K - 2 - (tb + j);
      if (k < 0) continue;
      const BwdLevel cur = b[j];
      b[j] = bwd(k - kRing);
      data = sub_rn(cur.s, mul_rn(cur.c, data));
      s[k] = mul_rn(dtr, sub_rn(data, cur.up));
    }
  }
}

// ---------------------------------------------------------------------------
// Sector-wide form, for K a multiple of 4 and 32-byte aligned arrays (every
// NPBench preset: K = 40, 80, 160).  Each lane moves 4 levels of its column
// with one 256-bit load or store (ld/st .v4.f64), i.e. one whole 32-byte
// sector, so no sector is fetched twice and the L1 miss slots carry 4x the
// useful bytes of the one-level form above.  The forward sweep double-buffers
// 4-level chunks (chunk g+1 is in flight while chunk g is processed; the two
// buffers swap roles by unrolling, never by copying); the back substitution
// keeps three chunks in flight, since its per-level work is short.
struct Chunk { double wh[4], wl[4], u[4], up[4], ut[4], s[4]; };

struct BChunk { double s[4], up[4], c[4]; };

// All of these are volatile so that the compiler keeps each prefetch where it
// is written (early), instead of sinking it towards its first use.
__device__ __forceinline__ void ld4_ro(const double* p, double (&v)[4]) {
  asm volatile("ld.global.nc.v4.f64 {%0,%1,%2,%3}, [%4];"
      : "=d"(v[0]), "=d"(v[1]), "=d"(v[2]), "=d"(v[3]) : "l"(p));
}
// utens_stage is read and written by the same thread: keep these in program
// order with the stores (volatile + memory clobber).
__device__ __forceinline__ void ld4_rw(const double* p, double (&v)[4]) {
  asm volatile("ld.global.v4.f64 {%0,%1,%2,%3}, [%4];"
               : "=d"(v[0]), "=d"(v[1]), "=d"(v[2]), "=d"(v[3]) : "l"(p) : "memory");
}
__device__ __forceinline__ void st4(double* p, const double (&v)[4]) {
  asm volatile("st.global.v4.f64 [%0], {%1,%2,%3,%4};"
               :: "l"(p), "d"(v[0]), "d"(v[1]), "d"(v[2]), "d"(v[3]) : "memory");
}

// 7 CTAs of 64 threads per SM (at most 144 registers a thread) keep the
// 256x256-column paper problem (6.7 CTAs per SM) in a single wave.
__global__ void __launch_bounds__(kThreads, 7)
vadv_columns_v4(double* __restrict__ us, const double* __restrict__ u,
                const double* __restrict__ wcon, const double* __restrict__ up,
                const double* __restrict__ ut, double dtr, int64_t ncol, int64_t J, int64_t K,
                double* __restrict__ ccol) {
  const int64_t c = int64_t(blockIdx.x) * kThreads + threadIdx.x;
  if (c >= ncol) return;
  const int64_t base = c * K;
  const int64_t G = K / 4;
  const double* wl = wcon + base;
  const double* wh = wl + J * K;
  const double* uc = u + base;
  const double* upc = up + base;
  const double* utc = ut + base;
  double* s = us + base;
  auto load = [&](Chunk& x, int64_t g) {
    g = g < G ? g : G - 1;
    const int64_t o = 4 * g;
    ld4_ro(wh + o, x.wh); ld4_ro(wl + o, x.wl); ld4_ro(uc + o, x.u);
    ld4_ro(upc + o, x.up); ld4_ro(utc + o, x.ut); ld4_rw(s + o, x.s);
  };

  double qn = 0.0, ucur = 0.0, unext = 0.0, cprev = 0.0, dprev = 0.0;
  // Levels 4g .. 4g+3 of chunk `cur`; the level after the chunk is nxt's first.
  auto forward = [&](const Chunk& cur, const Chunk& nxt, int64_t g) {
    double dc[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int64_t k = 4 * g + j;
      const double wh1 = j < 3 ? cur.wh[(j + 1) & 3] : nxt.wh[0];
      const double wl1 = j < 3 ? cur.wl[(j + 1) & 3] : nxt.wl[0];
      const double u1 = j < 3 ? cur.u[(j + 1) & 3] : nxt.u[0];
      if (k == 0) {
        qn = eighth_of(add_rn(wh1, wl1));
        ucur = cur.u[0];
        unext = u1;
        const double d = add_rn(add_rn(add_rn(mul_rn(dtr, cur.up[0]), cur.ut[0]), cur.s[0]),
                                mul_rn(neg(qn), sub_rn(unext, ucur)));
        const double dv = __drcp_rn(sub_rn(dtr, qn));
        cprev = mul_rn(qn, dv);
        dprev = mul_rn(d, dv);
        ccol[c] = cprev;
      } else if (k < K - 1) {
        const double q = qn;
        qn = eighth_of(add_rn(wh1, wl1));
        const double uprev = ucur;
        ucur = unext;
        unext = u1;
        const double acol = neg(q);
        const double corr =
            sub_rn(mul_rn(q, sub_rn(uprev, ucur)), mul_rn(qn, sub_rn(unext, ucur)));
        const double d =
            add_rn(add_rn(add_rn(mul_rn(dtr, cur.up[j]), cur.ut[j]), cur.s[j]), corr);
        const double bcol = sub_rn(sub_rn(dtr, acol), qn);
        const double dv = __drcp_rn(sub_rn(bcol, mul_rn(cprev, acol)));
        cprev = mul_rn(qn, dv);
        dprev = mul_rn(sub_rn(d, mul_rn(dprev, acol)), dv);
        ccol[k * ncol + c] = cprev;
      } else {
        const double q = qn;
        const double acol = neg(q);
        const double corr = mul_rn(q, sub_rn(ucur, unext));  // (-as)*(u[K-2] - u[K-1])
        const double d =
            add_rn(add_rn(add_rn(mul_rn(dtr, cur.up[j]), cur.ut[j]), cur.s[j]), corr);
        const double bcol = sub_rn(dtr, acol);
        const double dv = __drcp_rn(sub_rn(bcol, mul_rn(cprev, acol)));
        dprev = mul_rn(sub_rn(d, mul_rn(dprev, acol)), dv);
      }
      dc[j] = dprev;
    }
    st4(s + 4 * g, dc);
  };

  {
    Chunk A, B;
    load(A, 0);
    load(B, 1);
    for (int64_t g = 0; g < G; g += 2) {
      forward(A, B, g);
      load(A, g + 2);
      if (g + 1 < G) {
        forward(B, A, g + 1);
        load(B, g + 3);
      }
    }
  }

  // Back substitution: chunk g holds levels 4g..4g+3, walked from the top.
  auto bload = [&](BChunk& x, int64_t g) {
    g = g > 0 ? g : 0;
    const int64_t o = 4 * g;
    ld4_rw(s + o, x.s);
    ld4_ro(upc + o, x.up);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int64_t k = o + j < K - 1 ? o + j : K - 2;  // level K-1 has no ccol
      x.c[j] = ccol[k * ncol + c];
    }
  };
  double data = dprev;
  auto backward = [&](const BChunk& cur, int64_t g) {
    double out[4];
#pragma unroll
    for (int j = 3; j >= 0; --j) {
      const int64_t k = 4 * g + j;
      if (k < K - 1) data = sub_rn(cur.s[j], mul_rn(cur.c[j], data));
      out[j] = mul_rn(dtr, sub_rn(data, cur.up[j]));
    }
    st4(s + 4 * g, out);
  };
  BChunk X, Y, Z;
  bload(X, G - 1);
  bload(Y, G - 2);
  bload(Z, G - 3);
  for (int64_t g = G - 1; g >= 0; g -= 3) {
    backward(X, g);
    bload(X, g - 3);
    if (g - 1 >= 0) {
      backward(Y, g - 1);
      bload(Y, g - 4);
    }
    if (g - 2 >= 0) {
      backward(Z, g - 2);
      bload(Z, g - 5);
    }
  }
}

}  // namespace
}  // namespace npbgb

extern "C" int64_t npbgb_vadv_workspace_bytes(int64_t I, int64_t J, int64_t K) {
  if (I <= 0 || J <= 0 || K < 2) return 0;
  return int64_t(sizeof(double)) * (K - 1) * I * J;
}

extern "C" int32_t npbgb_vadv(void* utens_stage, const void* u_stage, const void* wcon,
                              const void* u_pos, const void* utens, double dtr_stage, int64_t I,
                              int64_t J, int64_t K, int32_t dtype, void* workspace,
                              int64_t workspace_bytes, void* stream) {
  using namespace npbgb;
  if (dtype != NPBGB_F64) return set_error(NPBGB_ERR_DTYPE, "vadv: binary64 only");
  if (I < 0 || J < 0 || K < 0) return set_error(NPBGB_ERR_ARG, "vadv: negative extent");
  if (K < 2) return set_error(NPBGB_ERR_ARG, "vadv: K = %lld < 2 (level 1 is read)", (long long)K);
  if (I == 0 || J == 0) return NPBGB_OK;
  if (!utens_stage || !u_stage || !wcon || !u_pos || !utens)
    return set_error(NPBGB_ERR_ARG, "vadv: null array");
  if (utens_stage == u_stage || utens_stage == wcon || utens_stage == u_pos || utens_stage == utens)
    return set_error(NPBGB_ERR_ARG, "vadv: utens_stage aliases an input");
  const int64_t ncol = I * J;
  const int64_t blocks = cdiv(ncol, kThreads);
  if (blocks > 0x7fffffff) return set_error(NPBGB_ERR_ARG, "vadv: extent too large");
  const int64_t need = npbgb_vadv_workspace_bytes(I, J, K);
  cudaStream_t st = as_stream(stream);
  void* ws = workspace;
  if (ws != nullptr && workspace_bytes < need)
    return set_error(NPBGB_ERR_ARG, "vadv: workspace of %lld bytes, %lld needed",
                     (long long)workspace_bytes, (long long)need);
  if (ws == nullptr) {
    cudaError_t e = cudaMallocAsync(&ws, size_t(need), st);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return set_error(NPBGB_ERR_NOMEM, "vadv: workspace of %lld bytes: %s", (long long)need,
                       cudaGetErrorString(e));
    }
  }
  auto a32 = [](const void* p) { return (reinterpret_cast<uintptr_t>(p) & 31u) == 0; };
  const bool sector = K % 4 == 0 && a32(utens_stage) && a32(u_stage) && a32(wcon) &&
                      a32(u_pos) && a32(utens);
  if (sector)
    vadv_columns_v4<<<unsigned(blocks), kThreads, 0, st>>>(
        static_cast<double*>(utens_stage), static_cast<const double*>(u_stage),
        static_cast<const double*>(wcon), static_cast<const double*>(u_pos),
        static_cast<const double*>(utens), dtr_stage, ncol, J, K, static_cast<double*>(ws));
  else
    vadv_columns<<<unsigned(blocks), kThreads, 0, st>>>(
        static_cast<double*>(utens_stage), static_cast<const double*>(u_stage),
        static_cast<const double*>(wcon), static_cast<const double*>(u_pos),
        static_cast<const double*>(utens), dtr_stage, ncol, J, K, static_cast<double*>(ws));
  cudaError_t le = counted(cudaGetLastError());
  if (workspace == nullptr) cudaFreeAsync(ws, st);
  return cuda_status(le, "vadv_columns");
}
