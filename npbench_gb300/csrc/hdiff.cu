// Horizontal diffusion with flux limiter (weather_stencils/hdiff/hdiff_numpy.py:5-29).
//
// One CTA owns a TI x TJ tile of output columns and 32 consecutive k (the
// contiguous axis, one k per lane).  It stages, in shared memory,
//   lap on the (TI+2) x (TJ+2) ring around the tile   (hdiff_numpy.py:7-9)
//   flx on (TI+1) x TJ,  fly on TI x (TJ+1)            (hdiff_numpy.py:11-25)
// so each Laplacian and each flux is evaluated once per tile, then writes
//   out = c - coeff * (((flx[i+1] - flx[i]) + fly[j+1]) - fly[j])   (:27-29)
// Every operator is one correctly rounded binary64 operation in the
// reference's order; the limiter keeps the reference's product test
// `res * grad > 0`, including its underflow and NaN behaviour.
#include "npbgb_common.cuh"

namespace npbgb {
namespace {

constexpr int kTI = 8, kTJ = 8, kLanes = 32, kRows = 8;
constexpr int kLapN = (kTI + 2) * (kTJ + 2);
constexpr int kFlxN = (kTI + 1) * kTJ;
constexpr int kFlyN = kTI * (kTJ + 1);
constexpr size_t kSmemBytes = size_t(kLapN + kFlxN + kFlyN) * kLanes * sizeof(double);

__device__ __forceinline__ double limit(double res, double grad) {
  return (mul_rn(res, grad) > 0.0) ? 0.0 : res;
}

__global__ void __launch_bounds__(kLanes * kRows)
hdiff_tile(const double* __restrict__ in, double* __restrict__ out,
           const double* __restrict__ coeff, int64_t I, int64_t J, int64_t K,
           int64_t tiles_i, int64_t tiles_j) {
  extern __shared__ double smem[];
  double* lap = smem;                      // [kLapN][kLanes]
  double* flx = lap + kLapN * kLanes;      // [kFlxN][kLanes]
  double* fly = flx + kFlxN * kLanes;      // [kFlyN][kLanes]

  int64_t bid = blockIdx.x;
  const int64_t tj = bid % tiles_j;  bid /= tiles_j;
  const int64_t ti = bid % tiles_i;  bid /= tiles_i;
  const int64_t k = bid * kLanes + threadIdx.x;
  const int64_t i0 = ti * kTI, j0 = tj * kTJ;
  const bool k_ok = k < K;
  const int64_t s0 = (J + 4) * K, s1 = K;
  // in-field point (x, y) at this lane's k
  auto in_at = [&](int64_t x, int64_t y) -> double { return in[x * s0 + y * s1 + k]; };

  // Laplacian at lap_field[i0 + a, j0 + b] = in-field centre (i0+a+1, j0+b+1).
  for (int idx = threadIdx.y; idx < kLapN; idx += kRows) {
    const int a = idx / (kTJ + 2), b = idx % (kTJ + 2);
    const int64_t x = i0 + a + 1, y = j0 + b + 1;
    double v = 0.0;
    if (k_ok && x < I + 3 && y < J + 3) {
      double nb = add_rn(in_at(x + 1, y), in_at(x - 1, y));
      nb = add_rn(nb, in_at(x, y + 1));
      nb = add_rn(nb, in_at(x, y - 1));
      v = sub_rn(mul_rn(4.0, in_at(x, y)), nb);
    }
    lap[idx * kLanes + threadIdx.x] = v;
  }
  __syncthreads();

  // flx_field[i0 + a, j0 + b] = lap[a+1][b+1] - lap[a][b+1], limited by
  // in(i0+a+2, j0+b+2) - in(i0+a+1, j0+b+2).
  for (int idx = threadIdx.y; idx < kFlxN; idx += kRows) {
    const int a = idx / kTJ, b = idx % kTJ;
    const int64_t x = i0 + a + 1, y = j0 + b + 2;
    double v = 0.0;
    if (k_ok && i0 + a < I + 1 && j0 + b < J) {
      const double res = sub_rn(lap[((a + 1) * (kTJ + 2) + b + 1) * kLanes + threadIdx.x],
                                lap[(a * (kTJ + 2) + b + 1) * kLanes + threadIdx.x]);
      v = limit(res, sub_rn(in_at(x + 1, y), in_at(x, y)));
    }
    flx[idx * kLanes + threadIdx.x] = v;
  }
  // fly_field[i0 + a, j0 + b] = lap[a+1][b+1] - lap[a+1][b], limited by
  // in(i0+a+2, j0+b+2) - in(i0+a+2, j0+b+1).
  for (int idx = threadIdx.y; idx < kFlyN; idx += kRows) {
    const int a = idx / (kTJ + 1), b = idx % (kTJ + 1);
    const int64_t x = i0 + a + 2, y = j0 + b + 1;
    double v = 0.0;
    if (k_ok && i0 + a < I && j0 + b < J + 1) {
      const double res = sub_rn(lap[((a + 1) * (kTJ + 2) + b + 1) * kLanes + threadIdx.x],
                                lap[((a + 1) * (kTJ + 2) + b) * kLanes + threadIdx.x]);
      v = limit(res, sub_rn(in_at(x, y + 1), in_at(x, y)));
    }
    fly[idx * kLanes + threadIdx.x] = v;
  }
  __syncthreads();

  for (int idx = threadIdx.y; idx < kTI * kTJ; idx += kRows) {
    const int a = idx / kTJ, b = idx % kTJ;
    const int64_t i = i0 + a, j = j0 + b;
    if (!k_ok || i >= I || j >= J) continue;
    double div = sub_rn(flx[((a + 1) * kTJ + b) * kLanes + threadIdx.x],
                        flx[(a * kTJ + b) * kLanes + threadIdx.x]);
    div = add_rn(div, fly[(a * (kTJ + 1) + b + 1) * kLanes + threadIdx.x]);
    div = sub_rn(div, fly[(a * (kTJ + 1) + b) * kLanes + threadIdx.x]);
    const int64_t o = (i * J + j) * K + k;
    out[o] = sub_rn(in_at(i + 2, j + 2), mul_rn(coeff[o], div));
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
  hdiff_tile<<<unsigned(blocks), dim3(kLanes, kRows), kSmemBytes, as_stream(stream)>>>(
      static_cast<const double*>(in_field), static_cast<double*>(out_field),
      static_cast<const double*>(coeff), I, J, K, tiles_i, tiles_j);
  NPBGB_CHECK_LAUNCH("hdiff_tile");
  return NPBGB_OK;
}
