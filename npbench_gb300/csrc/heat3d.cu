// 3D 7-point heat time loop (polybench/heat_3d/heat_3d_numpy.py:4-20).
//
// One launch per half-sweep.  Threads cover the (axis-1, axis-2) interior
// plane, axis 2 contiguous across the warp, and stream along axis 0 with a
// register queue (prev, centre, next).  Per point:
//   tx  = 0.125 * ((next_x - 2*c) + prev_x)      for x = 0, 1, 2
//   dst = ((t0 + t1) + t2) + c
// 2*c is exact and identical for the three axes, so it is formed once.
#include "npbgb_common.cuh"

namespace npbgb {
namespace {

constexpr int kBX = 32, kBY = 8, kChunk0 = 32;

template <typename T>
__global__ void __launch_bounds__(kBX * kBY)
heat3d_half(const T* __restrict__ src, T* __restrict__ dst, int64_t n0, int64_t n1, int64_t n2) {
  const T two = T(2.0), eighth = T(0.125);
  const int64_t k = 1 + int64_t(blockIdx.x) * kBX + threadIdx.x;
  const int64_t j = 1 + int64_t(blockIdx.y) * kBY + threadIdx.y;
  if (k >= n2 - 1 || j >= n1 - 1) return;
  const int64_t s0 = n1 * n2, s1 = n2;
  const int64_t i_begin = 1 + int64_t(blockIdx.z) * kChunk0;
  const int64_t i_end = (i_begin + kChunk0 < n0 - 1) ? i_begin + kChunk0 : n0 - 1;
  const T* p = src + j * s1 + k;
  T prev = p[(i_begin - 1) * s0];
  T cur = p[i_begin * s0];
  for (int64_t i = i_begin; i < i_end; ++i) {
    const T* q = p + i * s0;
    const T next = q[s0];
    const T c2 = mul_rn(two, cur);
    const T t0 = mul_rn(eighth, add_rn(sub_rn(next, c2), prev));
    const T t1 = mul_rn(eighth, add_rn(sub_rn(q[s1], c2), q[-s1]));
    const T t2 = mul_rn(eighth, add_rn(sub_rn(q[1], c2), q[-1]));
    dst[i * s0 + j * s1 + k] = add_rn(add_rn(add_rn(t0, t1), t2), cur);
    prev = cur;
    cur = next;
  }
}

template <typename T>
int32_t run(T* a, T* b, int64_t n0, int64_t n1, int64_t n2, int32_t tsteps, cudaStream_t st) {
  if (tsteps <= 1 || n0 < 3 || n1 < 3 || n2 < 3) return NPBGB_OK;
  dim3 block(kBX, kBY);
  dim3 grid(unsigned(cdiv(n2 - 2, kBX)), unsigned(cdiv(n1 - 2, kBY)),
            unsigned(cdiv(n0 - 2, kChunk0)));
  for (int32_t t = 1; t < tsteps; ++t) {
    heat3d_half<T><<<grid, block, 0, st>>>(a, b, n0, n1, n2);
    heat3d_half<T><<<grid, block, 0, st>>>(b, a, n0, n1, n2);
  }
  NPBGB_CHECK_LAUNCH("heat3d_half");
  return NPBGB_OK;
}

}  // namespace
}  // namespace npbgb

extern "C" int32_t npbgb_heat3d(void* A, void* B, int64_t n0, int64_t n1, int64_t n2,
                                int32_t tsteps, int32_t dtype, void* stream) {
  using namespace npbgb;
  if (n0 < 0 || n1 < 0 || n2 < 0) return set_error(NPBGB_ERR_ARG, "heat3d: negative extent");
  if (cdiv(n2, kBX) > 0x7fffffff || cdiv(n1, kBY) > 65535 || cdiv(n0, kChunk0) > 65535)
    return set_error(NPBGB_ERR_ARG, "heat3d: extent too large");
  if (tsteps > 1 && n0 >= 3 && n1 >= 3 && n2 >= 3) {
    if (!A || !B) return set_error(NPBGB_ERR_ARG, "heat3d: null array");
    if (A == B) return set_error(NPBGB_ERR_ARG, "heat3d: A and B alias");
  }
  if (dtype == NPBGB_F64)
    return run<double>(static_cast<double*>(A), static_cast<double*>(B), n0, n1, n2, tsteps,
                       as_stream(stream));
  if (dtype == NPBGB_F32)
    return run<float>(static_cast<float*>(A), static_cast<float*>(B), n0, n1, n2, tsteps,
                      as_stream(stream));
  return set_error(NPBGB_ERR_DTYPE, "heat3d: dtype %d", dtype);
}
