// Horizontal diffusion with flux limiter (weather_stencils/hdiff/hdiff_numpy.py:5-29).
//
// In in_field coordinates (x, y) = (i + 2, j + 2), the reference computes
//   L(x, y)   = 4*in(x,y) - (((in(x+1,y) + in(x-1,y)) + in(x,y+1)) + in(x,y-1))      (:7-9)
//   F(x, y)   = L(x+1,y) - L(x,y), set to +0 where F * (in(x+1,y) - in(x,y)) > 0  (:11-17)
//   G(x, y)   = L(x,y+1) - L(x,y), set to +0 where G * (in(x,y+1) - in(x,y)) > 0  (:19-25)
//   out(x, y) = in(x,y) - coeff * (((F(x,y) - F(x-1,y)) + G(x,y)) - G(x,y-1))     (:27-29)
// with every operator one correctly rounded binary64 operation.
//
// Layout: a CTA owns a kTI x kTJ tile of output columns (x, y) and 32
// consecutive k (the contiguous axis, one per lane).  It evaluates into
// shared memory the Laplacian on the (kTI+2) x (kTJ+2) ring around the tile,
// then F on (kTI+1) x kTJ and G on kTI x (kTJ+1), each once per tile, and
// writes out.  All points of a stage are independent, which keeps the
// binary64 pipe fed; two CTA barriers per tile.  (A variant streaming along x
// with one Laplacian plane per step does fewer redundant Laplacians but
// serialises three barriers and the binary64 latency per plane; measured
// slower on GB300.)
//
// binary64 work per output point is about 13.5 operations (the binary64 pipe
// bounds this kernel on GB300):
// * 4*c - s is one fused multiply-add: 4*c is exact, so fma(4, c, -s) rounds
//   exactly as the reference's two operations (unless 4*c would overflow,
//   which takes the two-operation path);
// * the limiter's test `res * grad > 0` is decided from signs, with no
//   multiply and no subtraction, whenever the product cannot underflow to
//   zero (|res| >= 2^-500 or res == 0, and both in values >= 2^-448 in
//   magnitude or equal); otherwise it is evaluated literally.  Signs give the
//   same answer for infinities and NaNs (all comparisons with NaN are false);
//   those comparisons are integer operations on the bit patterns.
#include "f64emu.cuh"
#include "npbgb_common.cuh"

namespace npbgb {
namespace {

constexpr int kTI = 8, kTJ = 8, kLanes = 32, kRows = 8;
constexpr int kThreads = kLanes * kRows;
constexpr int kLapN = (kTI + 2) * (kTJ + 2);
constexpr int kFlxN = (kTI + 1) * kTJ;
constexpr size_t kSmemBytes = size_t(kLapN + kFlxN) * kLanes * sizeof(double);
static_assert(kRows == kTI, "one warp per output row");

__device__ __forceinline__ int64_t bits(double v) { return __double_as_longlong(v); }
__device__ __forceinline__ uint32_t exp_field(int64_t b) {
  return static_cast<uint32_t>(static_cast<uint64_t>(b) >> 52) & 0x7ffu;
}

// The two-operation forms, kept out of line so that the compiler does not
// predicate them into the common path (binary64 instructions, predicated or
// not, occupy GB300's small binary64 pipe).
__device__ __noinline__ double lap_literal(double c, double s) { return sub_rn(mul_rn(4.0, c), s); }
__device__ __noinline__ bool product_positive(double res, double hi, double lo) {
  return mul_rn(res, sub_rn(hi, lo)) > 0.0;
}

// 4*c - s, rounded as the reference's fl(fl(4*c) - s).
__device__ __forceinline__ double lap_of(double c, double s) {
  if (exp_field(bits(c)) < 2044u) return __fma_rn(4.0, c, -s);  // |c| < 2^1021: 4*c exact
  return lap_literal(c, s);
}

// res, or +0 where res * (hi - lo) > 0 (the reference's limiter).  When the
// product can neither underflow to zero nor involve a non-finite value, its
// sign decides: res != 0 and hi != lo with matching signs.  The comparisons
// run on the integer pipe: for finite non-zero doubles the key b ^ (b >> 63
// masked to the magnitude bits) orders as the values do.
__device__ __forceinline__ double limit(double res, double hi, double lo) {
  const int64_t br = bits(res), bh = bits(hi), bl = bits(lo);
  const uint32_t er = exp_field(br), eh = exp_field(bh), el = exp_field(bl);
  const bool r_zero = (static_cast<uint64_t>(br) << 1) == 0;
  const bool res_ok = r_zero || (er >= 523u && er <= 2046u);  // 0 or finite, |res| >= 2^-500
  const bool in_ok = bh == bl || (eh >= 575u && eh <= 2046u && el >= 575u && el <= 2046u);
  bool positive;
  if (res_ok && in_ok) {
    const int64_t kh = bh ^ ((bh >> 63) & 0x7fffffffffffffffll);
    const int64_t kl = bl ^ ((bl >> 63) & 0x7fffffffffffffffll);
    positive = !r_zero && ((br > 0 && kh > kl) || (br < 0 && kh < kl));
  } else {
    positive = product_positive(res, hi, lo);
  }
  return positive ? 0.0 : res;
}

// ---------------------------------------------------------------------------
// Integer-pipe forms.  Items of the Laplacian, flux and output stages can be
// evaluated with the exact integer emulation of binary64 addition
// (f64emu.cuh) on the raw bit patterns, so that the integer pipes take part of
// the additions while the binary64 pipe does the rest; NPBGB_CFG_HDIFF_EMU
// picks the items (default: every flux item, measured best on GB300).  Each
// emulated operation checks its operands and takes the hardware operation (out
// of line) for anything outside the emulation's range (subnormals, infinities,
// NaN, magnitudes beyond about 2^+-960); results are the IEEE ones either way.
constexpr uint32_t kDefaultEmu = 0xff00;  // every flux item
using f64emu::add_bits;
using f64emu::f64;
using f64emu::sub_bits;
using f64emu::u64;

// fl(fl(4*c) - s) from bits: 4*c is an exponent increment when c is normal and
// the result stays in the emulation's range; other c take the literal form.
__device__ __noinline__ uint64_t lap_bits_hw(uint64_t c, uint64_t s) {
  return u64(sub_rn(mul_rn(4.0, f64(c)), f64(s)));
}
__device__ __forceinline__ uint64_t lap_bits(uint64_t c, uint64_t s) {
  const uint32_t ec = static_cast<uint32_t>(c >> 52) & 0x7ffu;
  if (ec - 64u < 1918u) return sub_bits(c + (2ull << 52), s);
  return lap_bits_hw(c, s);
}

// limit() on bit patterns (same decisions, same results).
__device__ __noinline__ bool product_positive_bits(uint64_t res, uint64_t hi, uint64_t lo) {
  return product_positive(f64(res), f64(hi), f64(lo));
}
__device__ __forceinline__ uint64_t limit_bits(uint64_t res, uint64_t hi, uint64_t lo) {
  const int64_t br = static_cast<int64_t>(res), bh = static_cast<int64_t>(hi),
                bl = static_cast<int64_t>(lo);
  const uint32_t er = exp_field(br), eh = exp_field(bh), el = exp_field(bl);
  const bool r_zero = (res << 1) == 0;
  const bool res_ok = r_zero || (er >= 523u && er <= 2046u);
  const bool in_ok = bh == bl || (eh >= 575u && eh <= 2046u && el >= 575u && el <= 2046u);
  bool positive;
  if (res_ok && in_ok) {
    const int64_t kh = bh ^ ((bh >> 63) & 0x7fffffffffffffffll);
    const int64_t kl = bl ^ ((bl >> 63) & 0x7fffffffffffffffll);
    positive = !r_zero && ((br > 0 && kh > kl) || (br < 0 && kh < kl));
  } else {
    positive = product_positive_bits(res, hi, lo);
  }
  return positive ? 0ull : res;
}

__global__ void __launch_bounds__(kThreads)
hdiff_tile(const double* __restrict__ in, double* __restrict__ out,
           const double* __restrict__ coeff, int64_t I, int64_t J, int64_t K, int64_t tiles_i,
           int64_t tiles_j, uint32_t emu) {
  extern __shared__ double smem[];
  double* lap = smem;                      // [kLapN][kLanes]
  double* flx = lap + kLapN * kLanes;      // [kFlxN][kLanes]

  const int lane = threadIdx.x & 31, row = threadIdx.x >> 5;
  int64_t bid = blockIdx.x;
  const int64_t tj = bid % tiles_j;  bid /= tiles_j;
  const int64_t ti = bid % tiles_i;  bid /= tiles_i;
  const int64_t k = bid * kLanes + lane;
  const int64_t i0 = ti * kTI, j0 = tj * kTJ;
  const bool k_ok = k < K;
  const int64_t s0 = (J + 4) * K, s1 = K;
  auto in_at = [&](int64_t x, int64_t y) -> double { return in[x * s0 + y * s1 + k]; };
  const uint64_t* inb = reinterpret_cast<const uint64_t*>(in);
  auto inb_at = [&](int64_t x, int64_t y) -> uint64_t { return inb[x * s0 + y * s1 + k]; };
  uint64_t* lapb = reinterpret_cast<uint64_t*>(lap);
  uint64_t* flxb = reinterpret_cast<uint64_t*>(flx);

  // L at lap_field[i0 + a, j0 + b] = in-field centre (i0+a+1, j0+b+1).  Item
  // t of a warp runs on the integer pipes when bit t % 8 of emu is set (a
  // warp-uniform choice).
  for (int t = 0, idx = row; idx < kLapN; ++t, idx += kRows) {
    const int a = idx / (kTJ + 2), b = idx % (kTJ + 2);
    const int64_t x = i0 + a + 1, y = j0 + b + 1;
    const bool live = k_ok && x < I + 3 && y < J + 3;
    uint64_t v = 0;
    if (live) {
      if ((emu >> (t & 7)) & 1u) {
        uint64_t nb = add_bits(inb_at(x + 1, y), inb_at(x - 1, y));
        nb = add_bits(nb, inb_at(x, y + 1));
        nb = add_bits(nb, inb_at(x, y - 1));
        v = lap_bits(inb_at(x, y), nb);
      } else {
        double nb = add_rn(in_at(x + 1, y), in_at(x - 1, y));
        nb = add_rn(nb, in_at(x, y + 1));
        nb = add_rn(nb, in_at(x, y - 1));
        v = u64(lap_of(in_at(x, y), nb));
      }
    }
    lapb[idx * kLanes + lane] = v;
  }
  __syncthreads();

  // F at flx_field[i0 + a, j0 + b]: lap[a+1][b+1] - lap[a][b+1], limited by
  // in(i0+a+2, j0+b+2) - in(i0+a+1, j0+b+2).
  for (int t = 0, idx = row; idx < kFlxN; ++t, idx += kRows) {
    const int a = idx / kTJ, b = idx % kTJ;
    const int64_t x = i0 + a + 1, y = j0 + b + 2;
    const bool live = k_ok && i0 + a < I + 1 && j0 + b < J;
    const int hi_i = ((a + 1) * (kTJ + 2) + b + 1) * kLanes + lane;
    const int lo_i = (a * (kTJ + 2) + b + 1) * kLanes + lane;
    if ((emu >> (8 + (t & 7))) & 1u) {
      flxb[idx * kLanes + lane] =
          live ? limit_bits(sub_bits(lapb[hi_i], lapb[lo_i]), inb_at(x + 1, y), inb_at(x, y)) : 0ull;
    } else {
      flx[idx * kLanes + lane] =
          live ? limit(sub_rn(lap[hi_i], lap[lo_i]), in_at(x + 1, y), in_at(x, y)) : 0.0;
    }
  }
  __syncthreads();

  // Warp `row` writes output row a = row.  G at fly_field[i0 + a, j0 + b] is
  // lap[a+1][b+1] - lap[a+1][b], limited by in(i0+a+2, j0+b+2) -
  // in(i0+a+2, j0+b+1); the warp walks b upwards and keeps the last G and in
  // value in registers, so each G is evaluated once.  The output point (a, b)
  // is in - coeff * (((F[a+1][b] - F[a][b]) + G[a][b+1]) - G[a][b]) with
  // in = in(i0+a+2, j0+b+2), the hi operand of G[a][b].
  {
    const int a = row;
    const int64_t i = i0 + a, x = i + 2;
    if (k_ok && i < I) {
      const uint64_t* lrow = lapb + (a + 1) * (kTJ + 2) * kLanes + lane;
      uint64_t l_lo = lrow[0];
      uint64_t in_lo = inb_at(x, j0 + 1);
      uint64_t g_lo = 0;
      {
        const uint64_t l_hi = lrow[kLanes], in_hi = inb_at(x, j0 + 2);
        g_lo = ((emu >> 8) & 1u) ? limit_bits(sub_bits(l_hi, l_lo), in_hi, in_lo)
                                 : u64(limit(sub_rn(f64(l_hi), f64(l_lo)), f64(in_hi), f64(in_lo)));
        l_lo = l_hi;
        in_lo = in_hi;
      }
#pragma unroll
      for (int bb = 0; bb < kTJ; ++bb) {
        const int64_t j = j0 + bb;
        if (j >= J) break;
        // G[a][bb+1]; in_lo holds in(x, j + 2), the centre of this point.
        const uint64_t centre = in_lo;
        const uint64_t l_hi = lrow[(bb + 2) * kLanes];
        const uint64_t in_hi = inb_at(x, j + 3);  // j < J: G[a][bb+1] is inside fly_field
        const uint64_t g_hi = ((emu >> (8 + ((bb + 1) & 7))) & 1u)
                                  ? limit_bits(sub_bits(l_hi, l_lo), in_hi, centre)
                                  : u64(limit(sub_rn(f64(l_hi), f64(l_lo)), f64(in_hi), f64(centre)));
        const int64_t o = (i * J + j) * K + k;
        const int f1 = ((a + 1) * kTJ + bb) * kLanes + lane, f0 = (a * kTJ + bb) * kLanes + lane;
        if ((emu >> (16 + (bb & 7))) & 1u) {
          uint64_t div = sub_bits(flxb[f1], flxb[f0]);
          div = add_bits(div, g_hi);
          div = sub_bits(div, g_lo);
          const uint64_t prod = u64(mul_rn(coeff[o], f64(div)));
          reinterpret_cast<uint64_t*>(out)[o] = sub_bits(centre, prod);
        } else {
          double div = sub_rn(flx[f1], flx[f0]);
          div = add_rn(div, f64(g_hi));
          div = sub_rn(div, f64(g_lo));
          out[o] = sub_rn(f64(centre), mul_rn(coeff[o], div));
        }
        g_lo = g_hi;
        l_lo = l_hi;
        in_lo = in_hi;
      }
    }
  }
}

}  // namespace
}  // namespace npbgb

extern "C" int32_t npbgb_hdiff(const void* in_field, void* out_field, const void* coeff,
                               int64_t I, int64_t J, int64_t K, int32_t dtype, void* stream) {
  using namespace npbgb;
  if (dtype != NPBGB_F64) return set_error(NPBGB_ERR_DTYPE, "hdiff: binary64 only");
  if (I < 0 || J < 0 || K < 0) return set_error(NPBGB_ERR_ARG, "hdiff: negative extent");
  if (I == 0 || J == 0 || K == 0) return NPBGB_OK;
  if (!in_field || !out_field || !coeff) return set_error(NPBGB_ERR_ARG, "hdiff: null array");
  if (out_field == in_field || out_field == coeff)
    return set_error(NPBGB_ERR_ARG, "hdiff: out_field aliases an input");
  const int64_t tiles_i = cdiv(I, kTI), tiles_j = cdiv(J, kTJ), tiles_k = cdiv(K, kLanes);
  const int64_t blocks = tiles_i * tiles_j * tiles_k;
  if (blocks > 0x7fffffff) return set_error(NPBGB_ERR_ARG, "hdiff: extent too large");
  static bool attr_set = false;
  if (!attr_set) {
    cudaError_t e = cudaFuncSetAttribute(hdiff_tile, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         int(kSmemBytes));
    if (e != cudaSuccess) return cuda_status(e, "hdiff: smem attribute");
    attr_set = true;
  }
  hdiff_tile<<<unsigned(blocks), kThreads, kSmemBytes, as_stream(stream)>>>(
      static_cast<const double*>(in_field), static_cast<double*>(out_field),
      static_cast<const double*>(coeff), I, J, K, tiles_i, tiles_j,
      uint32_t(g_cfg_hdiff_emu >= 0 ? g_cfg_hdiff_emu : kDefaultEmu));
  NPBGB_CHECK_LAUNCH("hdiff_tile");
  return NPBGB_OK;
}
