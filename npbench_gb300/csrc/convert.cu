// Binary32 <-> binary64 conversion of a dense array, for grids that run in
// binary64 on behalf of binary32 callers (the float64 guard): widening is
// exact, rounding back is IEEE round-to-nearest-even (NumPy's astype).
#include "npbgb_common.cuh"

namespace npbgb {
namespace {

__global__ void __launch_bounds__(256) widen_f32(double* __restrict__ dst,
                                                 const float* __restrict__ src, int64_t n) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * blockDim.x)
    dst[i] = double(src[i]);
}

__global__ void __launch_bounds__(256) round_f64(float* __restrict__ dst,
                                                 const double* __restrict__ src, int64_t n) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * blockDim.x)
    dst[i] = __double2float_rn(src[i]);
}

}  // namespace
}  // namespace npbgb

extern "C" int32_t npbgb_convert(void* dst, int32_t dst_dtype, const void* src, int32_t src_dtype,
                                 int64_t n, void* stream) {
  using namespace npbgb;
  if (n < 0) return set_error(NPBGB_ERR_ARG, "convert: negative count");
  if (n == 0) return NPBGB_OK;
  if (!dst || !src || dst == src) return set_error(NPBGB_ERR_ARG, "convert: null or aliased arrays");
  const int64_t blocks64 = std::min<int64_t>(cdiv(n, 256), int64_t(sm_count()) * 16);
  const dim3 grid{unsigned(blocks64)}, block{256u};
  cudaStream_t st = as_stream(stream);
  if (dst_dtype == NPBGB_F64 && src_dtype == NPBGB_F32)
    widen_f32<<<grid, block, 0, st>>>(static_cast<double*>(dst), static_cast<const float*>(src), n);
  else if (dst_dtype == NPBGB_F32 && src_dtype == NPBGB_F64)
    round_f64<<<grid, block, 0, st>>>(static_cast<float*>(dst), static_cast<const double*>(src), n);
  else
    return set_error(NPBGB_ERR_DTYPE, "convert: %d -> %d", src_dtype, dst_dtype);
  NPBGB_CHECK_LAUNCH("convert");
  return NPBGB_OK;
}
