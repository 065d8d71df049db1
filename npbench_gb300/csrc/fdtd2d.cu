// 2D FDTD time loop (polybench/fdtd_2d/fdtd_2d_numpy.py:4-11).
//
// Per time step t, in the reference's order (arrays (nx, ny), C order):
//   ey[0, :]  = fict[t]
//   ey[i, j] -= 0.5 * (hz[i, j] - hz[i-1, j])                         i >= 1
//   ex[i, j] -= 0.5 * (hz[i, j] - hz[i, j-1])                         j >= 1
//   hz[i, j] -= 0.7 * (((ex[i, j+1] - ex[i, j]) + ey[i+1, j]) - ey[i, j])   i < nx-1, j < ny-1
// The ey and ex updates read only hz, so one launch does both (and the row-0
// source); the hz update reads the new ex and ey and is a second launch.
// Every operator is one correctly rounded IEEE operation; the binary64
// products by 0.5, which are exact, are done as exponent decrements on the
// integer pipe (GB300's binary64 pipe is the bound).
#include "npbgb_common.cuh"

namespace npbgb {
namespace {

constexpr int kBX = 32, kBY = 8;

// 0.5 * x without the binary64 pipe: halving is exact (an exponent decrement)
// for normal x whose halving stays normal; zero, subnormal, inf and NaN take
// the literal multiply, kept out of line so it is not predicated into the
// common path.
__device__ __noinline__ double half_literal(double x) { return mul_rn(0.5, x); }
__device__ __forceinline__ double half_of(double x) {
  const uint64_t b = static_cast<uint64_t>(__double_as_longlong(x));
  const uint32_t e = static_cast<uint32_t>(b >> 52) & 0x7ffu;
  if (e >= 2u && e <= 2046u) return __longlong_as_double(static_cast<long long>(b - (1ull << 52)));
  return half_literal(x);
}
__device__ __forceinline__ float half_of(float x) { return mul_rn(0.5f, x); }

template <typename T>
__global__ void __launch_bounds__(kBX * kBY)
fdtd_e(T* __restrict__ ex, T* __restrict__ ey, const T* __restrict__ hz, const T* __restrict__ fict,
       int64_t nx, int64_t ny, int t) {
  pdl_begin();
  const int64_t j = int64_t(blockIdx.x) * kBX + threadIdx.x;
  if (j >= ny) return;
  for (int64_t i = int64_t(blockIdx.y) * kBY + threadIdx.y; i < nx; i += int64_t(gridDim.y) * kBY) {
    const int64_t o = i * ny + j;
    const T h = hz[o];
    if (i == 0)
      ey[o] = fict[t];
    else
      ey[o] = sub_rn(ey[o], half_of(sub_rn(h, hz[o - ny])));
    if (j >= 1) ex[o] = sub_rn(ex[o], half_of(sub_rn(h, hz[o - 1])));
  }
}

template <typename T>
__global__ void __launch_bounds__(kBX * kBY)
fdtd_h(const T* __restrict__ ex, const T* __restrict__ ey, T* __restrict__ hz, int64_t nx, int64_t ny) {
  pdl_begin();
  const T c07 = T(0.7);
  const int64_t j = int64_t(blockIdx.x) * kBX + threadIdx.x;
  if (j >= ny - 1) return;
  for (int64_t i = int64_t(blockIdx.y) * kBY + threadIdx.y; i < nx - 1; i += int64_t(gridDim.y) * kBY) {
    const int64_t o = i * ny + j;
    T d = sub_rn(ex[o + 1], ex[o]);
    d = add_rn(d, ey[o + ny]);
    d = sub_rn(d, ey[o]);
    hz[o] = sub_rn(hz[o], mul_rn(c07, d));
  }
}

template <typename T>
int32_t run(T* ex, T* ey, T* hz, const T* fict, int64_t nx, int64_t ny, int32_t tmax,
            cudaStream_t st) {
  if (tmax <= 0 || nx <= 0 || ny <= 0) return NPBGB_OK;
  const int64_t gx = cdiv(ny, kBX), gy0 = cdiv(nx, kBY);
  if (gx > 0x7fffffff) return set_error(NPBGB_ERR_ARG, "fdtd2d: extent too large");
  const dim3 grid{unsigned(gx), unsigned(gy0 > 65535 ? 65535 : gy0)};
  const dim3 block{unsigned(kBX), unsigned(kBY)};
  cudaError_t e = cudaSuccess;
  for (int32_t t = 0; t < tmax && e == cudaSuccess; ++t) {
    e = launch_chained(fdtd_e<T>, grid, block, 0, st, ex, ey, hz, fict, nx, ny, t);
    if (e == cudaSuccess && nx > 1 && ny > 1)
      e = launch_chained(fdtd_h<T>, grid, block, 0, st, ex, ey, hz, nx, ny);
  }
  return cuda_status(e, "fdtd2d");
}

}  // namespace
}  // namespace npbgb

extern "C" int32_t npbgb_fdtd2d(void* ex, void* ey, void* hz, const void* fict, int64_t fict_len,
                                int64_t nx, int64_t ny, int32_t tmax, int32_t dtype, void* stream) {
  using namespace npbgb;
  if (nx < 0 || ny < 0) return set_error(NPBGB_ERR_ARG, "fdtd2d: negative extent");
  if (tmax > 0 && fict_len < tmax)
    return set_error(NPBGB_ERR_ARG, "fdtd2d: _fict_ has %lld entries, TMAX is %d (index out of range)",
                     (long long)fict_len, tmax);
  if (tmax > 0 && nx > 0 && ny > 0) {
    if (!ex || !ey || !hz || !fict) return set_error(NPBGB_ERR_ARG, "fdtd2d: null array");
    if (ex == ey || ex == hz || ey == hz) return set_error(NPBGB_ERR_ARG, "fdtd2d: arrays alias");
  }
  cudaStream_t st = as_stream(stream);
  if (dtype == NPBGB_F64)
    return run<double>(static_cast<double*>(ex), static_cast<double*>(ey), static_cast<double*>(hz),
                       static_cast<const double*>(fict), nx, ny, tmax, st);
  if (dtype == NPBGB_F32)
    return run<float>(static_cast<float*>(ex), static_cast<float*>(ey), static_cast<float*>(hz),
                      static_cast<const float*>(fict), nx, ny, tmax, st);
  return set_error(NPBGB_ERR_DTYPE, "fdtd2d: dtype %d", dtype);
}
