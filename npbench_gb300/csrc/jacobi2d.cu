// 2D 5-point Jacobi time loop (polybench/jacobi_2d/jacobi_2d_numpy.py:4-10).
//
// Per interior point, in the reference's order:
//   dst = 0.2 * ((((c + w) + e) + s) + n)
// with w/e the column neighbours j-1/j+1 and s/n the row neighbours i+1/i-1.
//
// Kernel layout (one launch per half-sweep): every warp owns a strip of 32
// columns and streams down a chunk of rows (jacobi_core.cuh: rows i-1, i,
// i+1 in registers, w/e neighbours by shuffle, kUnroll rows loaded ahead).
// Warps never wait on each other.
//
// binary32 uses IEEE float operations.  binary64 runs its four additions
// exactly in fixed point on the integer pipe (fx64.cuh) for every point whose
// five inputs lie in [2^-7, 1) or are +0 (refused values carry a poison bit),
// and uses hardware binary64 for any other point.  The fixed-point points also
// take the final product by 0.2 on the integer pipes (fx::mul02: the exact
// integer product of the significands, rounded once to nearest even), so they
// leave the binary64 pipe to the hardware warps.  Both paths give the IEEE
// result bit for bit.
#include "jacobi_core.cuh"
#include "tma.cuh"

namespace npbgb {

extern int64_t g_cfg_f64_emulation;
extern int64_t g_cfg_jacobi_chunk;
extern int64_t g_cfg_jacobi_hw_warps;
extern int64_t g_cfg_jacobi_fx_mul;
extern int64_t g_cfg_jacobi_fx_adds;
extern int64_t g_cfg_jacobi_tma;

template <typename T>
int32_t jacobi2d_bands_run(T* a, T* b, int64_t ny, int64_t nx, int32_t tsteps, cudaStream_t st);

namespace {

constexpr int kWarps = 8;
constexpr int kUnroll = 4;

// Grid: x over groups of kWarps column strips, y over chunks of rows.  With
// FX, warps below hw_warps take the hardware binary64 path so that the
// binary64 pipe works next to the integer pipe (same results either way).
template <typename T, bool FX, int MAD, bool IMUL, bool HWIMUL>
__global__ void __launch_bounds__(32 * kWarps)
jacobi2d_strip(const T* __restrict__ src, T* __restrict__ dst, int64_t ny, int64_t nx, int chunk,
               int hw_warps, uint32_t one) {
  pdl_begin();
  const int warp = threadIdx.x >> 5;
  const int64_t k0 = 1 + (int64_t(blockIdx.x) * kWarps + warp) * 32;
  if (k0 >= nx - 1) return;  // whole strip outside the interior (warp-uniform)
  const int64_t ib = 1 + int64_t(blockIdx.y) * chunk;
  const int64_t ie = (ib + chunk < ny - 1) ? ib + chunk : ny - 1;
  // Rows loaded ahead: 4 for binary32; 1 for binary64, whose chunks are short
  // (2 ahead measured 5-10% slower at 500^2 to 4096^2 with 4 hardware warps).
  if (FX && warp < hw_warps)
    jcore::strip_rows<T, false, false, 1, 0, true, HWIMUL>(src, dst, nx, k0, ib, ie, one);
  else
    jcore::strip_rows<T, FX, false, FX ? 1 : kUnroll, MAD, IMUL>(src, dst, nx, k0, ib, ie, one);
}

__device__ unsigned int g_jacobi_tma_error;  // bit 0: an mbarrier wait timed out

using jcore::kTmaRing;
using jcore::kTmaRows;
using jcore::tma_strip_rows;
template <typename T>
using TmaStrip = jcore::TmaStrip<T, kWarps>;

template <typename T, bool FX, int MAD, bool IMUL>
__global__ void __launch_bounds__(32 * kWarps)
jacobi2d_tma(const __grid_constant__ CUtensorMap map, const T* __restrict__ src, T* __restrict__ dst,
             int64_t ny, int64_t nx, int chunk, int hw_warps, uint32_t one) {
  pdl_begin();
  using G = TmaStrip<T>;
  extern __shared__ __align__(128) unsigned char smem[];
  const int warp = threadIdx.x >> 5;
  unsigned char* ring = smem + warp * G::kWarpBytes;
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + kWarps * G::kWarpBytes) + warp * kTmaRing;
  const int64_t k0 = 1 + (int64_t(blockIdx.x) * kWarps + warp) * 32;
  if (k0 >= nx - 1) return;  // whole strip outside the interior (warp-uniform)
  const int64_t ib = 1 + int64_t(blockIdx.y) * chunk;
  const int64_t ie = (ib + chunk < ny - 1) ? ib + chunk : ny - 1;
  if ((threadIdx.x & 31) == 0) {
    for (int b = 0; b < kTmaRing; ++b) tma::mbar_init(&bars[b], 1);
    tma::fence_mbar_init();
  }
  __syncwarp();
  const bool ok = (FX && warp < hw_warps)
                      ? tma_strip_rows<T, false, MAD, IMUL>(&map, src, dst, nx, k0, ib, ie, ring, bars, one)
                      : tma_strip_rows<T, FX, MAD, IMUL>(&map, src, dst, nx, k0, ib, ie, ring, bars, one);
  if (!ok && (threadIdx.x & 31) == 0) atomicOr(&g_jacobi_tma_error, 1u);
}

int pick_chunk(int64_t ny, int64_t col_blocks) {
  if (g_cfg_jacobi_chunk > 0) return int(g_cfg_jacobi_chunk);
  // About 16 warps per SM over 152 SMs, rows per warp at least 3 (small
  // grids want short chunks for enough CTAs: 3-4 rows measured best at 500^2
  // and 1000^2, the computed chunk at 2000^2 and 4096^2).
  const int64_t target_blocks = int64_t(sm_count()) * 16 / kWarps * 4;
  int64_t chunks = cdiv(target_blocks, col_blocks > 0 ? col_blocks : 1);
  int64_t c = cdiv(ny - 2, chunks > 0 ? chunks : 1);
  if (c < 3) c = 3;
  if (c > ny - 2) c = ny - 2;
  return int(c);
}

// The chained half-sweeps with the TMA kernel; NPBGB_ERR_STATE (nothing
// launched) when the arrays do not meet TMA's rules (16-byte aligned base and
// rows) or a form other than plain integer additions is asked for.
template <typename T, bool FX>
int32_t run_tma(T* a, T* b, int64_t ny, int64_t nx, int32_t tsteps, dim3 grid, int chunk, int hw,
                int mad, int64_t im, cudaStream_t st) {
  using G = TmaStrip<T>;
  if (mad != 0 || im == 2) return NPBGB_ERR_STATE;
  if ((nx * int64_t(sizeof(T))) % 16 != 0 || ny > 0x7fffffff || nx > 0x7fffffff) return NPBGB_ERR_STATE;
  CUtensorMap map_a, map_b;
  const uint64_t dims[3] = {uint64_t(nx), uint64_t(ny), 1u};
  const uint32_t box[3] = {uint32_t(G::BX), uint32_t(kTmaRows), 1u};
  if (tma::encode_3d(&map_a, sizeof(T), a, dims, box) != cudaSuccess ||
      tma::encode_3d(&map_b, sizeof(T), b, dims, box) != cudaSuccess)
    return NPBGB_ERR_STATE;
  auto kern = im == 0 ? jacobi2d_tma<T, FX, 0, false> : jacobi2d_tma<T, FX, 0, true>;
  const dim3 block{32u * kWarps};
  cudaError_t e = cudaSuccess;
  for (int32_t t = 1; t < tsteps && e == cudaSuccess; ++t) {
    e = launch_chained(kern, grid, block, G::smem(), st, map_a, a, b, ny, nx, chunk, hw, 1u);
    if (e == cudaSuccess)
      e = launch_chained(kern, grid, block, G::smem(), st, map_b, b, a, ny, nx, chunk, hw, 1u);
  }
  return cuda_status(e, "jacobi2d_tma");
}

template <typename T, bool FX>
int32_t run(T* a, T* b, int64_t ny, int64_t nx, int32_t tsteps, cudaStream_t st) {
  if (tsteps <= 1 || ny < 3 || nx < 3) return NPBGB_OK;
  {
    const int32_t r = jacobi2d_bands_run<T>(a, b, ny, nx, tsteps, st);
    if (r != NPBGB_ERR_STATE) return r;
  }
  const int64_t gx = cdiv(nx - 2, 32 * kWarps);
  const int chunk = pick_chunk(ny, gx);
  const int64_t gy = cdiv(ny - 2, chunk);
  if (gx > 0x7fffffff || gy > 65535) return set_error(NPBGB_ERR_ARG, "jacobi2d: extent too large");
  const dim3 grid{unsigned(gx), unsigned(gy)};
  const int hw = jacobi_hw_warps();
  const dim3 block{32u * kWarps};
  // Fixed-point additions as plain integer adds (with the integer product by
  // 0.2 they measured fastest at every size: 1000^2 TSTEPS=100 1.83 ms against
  // 1.94 with multiply-add adds and 2.10 with the rounding on the multiply-add
  // pipe) unless NPBGB_CFG_JACOBI_FX_ADDS says otherwise; the product by 0.2 on
  // the integer pipes unless NPBGB_CFG_JACOBI_FX_MUL = 0.
  const int mad = (FX && g_cfg_jacobi_fx_adds > 0) ? int(g_cfg_jacobi_fx_adds) - 1 : 0;
  const int64_t im = g_cfg_jacobi_fx_mul;
  // The TMA ring where it pays: binary64 arrays of 48 MiB and more (the pair
  // beyond most of the L2), automatically; any aligned grid when forced
  // (NPBGB_CFG_JACOBI_TMA = 2).  Measured on GB300 (TSTEPS=21 at 4096^2 and
  // 2800^2, 41 at 2048^2, 100 at 1000^2 and 500^2; best settings of each
  // form, ms): 4096^2 binary64 3.44 against 4.04 with plain loads, 2800^2
  // 1.88 / 1.99; grids the L2 holds lose (2048^2, 32 MiB arrays: 2.11 / 1.92,
  // 1000^2 1.91 / 1.64, 500^2 1.45 / 0.89), and binary32 loses at every size
  // (4096^2 1.68 / 1.16): its plain strips already load four rows ahead.
  const bool big = nx * ny * int64_t(sizeof(T)) >= (int64_t(48) << 20);
  if (g_cfg_jacobi_tma == 2 || (g_cfg_jacobi_tma == 1 && FX && big)) {
    // 16-row chunks and 3 of 8 warps on hardware binary64 measured best with the
    // ring at 4096^2 (3.44 ms; the plain form's 54-row chunks 3.63, 4 warps 3.61).
    const int tchunk = g_cfg_jacobi_chunk > 0 ? int(g_cfg_jacobi_chunk) : (ny - 2 < 16 ? int(ny - 2) : 16);
    const int thw = g_cfg_jacobi_hw_warps >= 0 ? int(g_cfg_jacobi_hw_warps) : 3;
    const int64_t tgy = cdiv(ny - 2, tchunk);
    if (tgy <= 65535) {
      const int32_t r = run_tma<T, FX>(a, b, ny, nx, tsteps, dim3{unsigned(gx), unsigned(tgy)}, tchunk,
                                       thw, mad, im, st);
      if (r != NPBGB_ERR_STATE) return r;
    }
  }
  using Kern = void (*)(const T*, T*, int64_t, int64_t, int, int, uint32_t);
  Kern kern;
  if (mad == 2)
    kern = im == 0 ? jacobi2d_strip<T, FX, 2, false, false>
         : im == 1 ? jacobi2d_strip<T, FX, 2, true, false> : jacobi2d_strip<T, FX, 2, true, true>;
  else if (mad == 1)
    kern = im == 0 ? jacobi2d_strip<T, FX, 1, false, false>
         : im == 1 ? jacobi2d_strip<T, FX, 1, true, false> : jacobi2d_strip<T, FX, 1, true, true>;
  else
    kern = im == 0 ? jacobi2d_strip<T, FX, 0, false, false>
         : im == 1 ? jacobi2d_strip<T, FX, 0, true, false> : jacobi2d_strip<T, FX, 0, true, true>;
  cudaError_t e = cudaSuccess;
  for (int32_t t = 1; t < tsteps && e == cudaSuccess; ++t) {
    e = launch_chained(kern, grid, block, 0, st, a, b, ny, nx, chunk, hw, 1u);
    if (e == cudaSuccess) e = launch_chained(kern, grid, block, 0, st, b, a, ny, nx, chunk, hw, 1u);
  }
  return cuda_status(e, "jacobi2d_strip");
}

}  // namespace

// Reads and clears the TMA kernel's device error word (host; synchronises).
uint32_t take_jacobi_tma_device_error() {
  unsigned int v = 0, zero = 0;
  if (cudaMemcpyFromSymbol(&v, g_jacobi_tma_error, sizeof(v)) != cudaSuccess) return 0xffffffffu;
  if (v) cudaMemcpyToSymbol(g_jacobi_tma_error, &zero, sizeof(zero));
  return v;
}

}  // namespace npbgb

extern "C" int32_t npbgb_jacobi2d(void* A, void* B, int64_t ny, int64_t nx, int32_t tsteps,
                                  int32_t dtype, void* stream) {
  using namespace npbgb;
  if (ny < 0 || nx < 0) return set_error(NPBGB_ERR_ARG, "jacobi2d: negative extent");
  if (tsteps > 1 && ny >= 3 && nx >= 3) {
    if (!A || !B) return set_error(NPBGB_ERR_ARG, "jacobi2d: null array");
    if (A == B) return set_error(NPBGB_ERR_ARG, "jacobi2d: A and B alias");
  }
  cudaStream_t st = as_stream(stream);
  if (dtype == NPBGB_F64) {
    double* a = static_cast<double*>(A);
    double* b = static_cast<double*>(B);
    return g_cfg_f64_emulation ? run<double, true>(a, b, ny, nx, tsteps, st)
                               : run<double, false>(a, b, ny, nx, tsteps, st);
  }
  if (dtype == NPBGB_F32)
    return run<float, false>(static_cast<float*>(A), static_cast<float*>(B), ny, nx, tsteps, st);
  return set_error(NPBGB_ERR_DTYPE, "jacobi2d: dtype %d", dtype);
}
