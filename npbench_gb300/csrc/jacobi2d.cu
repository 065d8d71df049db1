// 2D 5-point Jacobi time loop (polybench/jacobi_2d/jacobi_2d_numpy.py:4-10).
//
// One launch per half-sweep.  Each thread owns one interior point and
// evaluates dst = 0.2 * ((((c + w) + e) + s) + n) with separately rounded IEEE
// operations, the reference's operator order.
#include "npbgb_common.cuh"

namespace npbgb {
namespace {

constexpr int kBX = 32, kBY = 8;

template <typename T>
__global__ void __launch_bounds__(kBX * kBY)
jacobi2d_half(const T* __restrict__ src, T* __restrict__ dst, int64_t ny, int64_t nx) {
  const T k02 = T(0.2);
  const int64_t j = 1 + int64_t(blockIdx.x) * kBX + threadIdx.x;
  if (j >= nx - 1) return;
  for (int64_t i = 1 + int64_t(blockIdx.y) * kBY + threadIdx.y; i < ny - 1;
       i += int64_t(gridDim.y) * kBY) {
    const T* r = src + i * nx + j;
    T acc = add_rn(r[0], r[-1]);
    acc = add_rn(acc, r[1]);
    acc = add_rn(acc, r[nx]);
    acc = add_rn(acc, r[-nx]);
    dst[i * nx + j] = mul_rn(k02, acc);
  }
}

template <typename T>
int32_t run(T* a, T* b, int64_t ny, int64_t nx, int32_t tsteps, cudaStream_t st) {
  if (tsteps <= 1 || ny < 3 || nx < 3) return NPBGB_OK;
  dim3 block(kBX, kBY);
  int64_t gy = cdiv(ny - 2, kBY);
  dim3 grid(unsigned(cdiv(nx - 2, kBX)), unsigned(gy > 65535 ? 65535 : gy));
  for (int32_t t = 1; t < tsteps; ++t) {
    jacobi2d_half<T><<<grid, block, 0, st>>>(a, b, ny, nx);
    jacobi2d_half<T><<<grid, block, 0, st>>>(b, a, ny, nx);
  }
  NPBGB_CHECK_LAUNCH("jacobi2d_half");
  return NPBGB_OK;
}

}  // namespace
}  // namespace npbgb

extern "C" int32_t npbgb_jacobi2d(void* A, void* B, int64_t ny, int64_t nx, int32_t tsteps,
                                  int32_t dtype, void* stream) {
  using namespace npbgb;
  if (ny < 0 || nx < 0) return set_error(NPBGB_ERR_ARG, "jacobi2d: negative extent");
  if (nx > (int64_t(1) << 31) * kBX) return set_error(NPBGB_ERR_ARG, "jacobi2d: nx too large");
  if (tsteps > 1 && ny >= 3 && nx >= 3) {
    if (!A || !B) return set_error(NPBGB_ERR_ARG, "jacobi2d: null array");
    if (A == B) return set_error(NPBGB_ERR_ARG, "jacobi2d: A and B alias");
  }
  if (dtype == NPBGB_F64)
    return run<double>(static_cast<double*>(A), static_cast<double*>(B), ny, nx, tsteps,
                       as_stream(stream));
  if (dtype == NPBGB_F32)
    return run<float>(static_cast<float*>(A), static_cast<float*>(B), ny, nx, tsteps,
                      as_stream(stream));
  return set_error(NPBGB_ERR_DTYPE, "jacobi2d: dtype %d", dtype);
}
