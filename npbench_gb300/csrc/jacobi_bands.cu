// Jacobi-2D with the whole time loop in one launch: bands resident in shared memory.
//
// For grids that L2 holds (about 1000^2 binary64), the chained launches of
// jacobi2d.cu spend much of each half-sweep on launch ramp-up, short row
// chunks and L2 latency rather than arithmetic.  Here one cooperative launch
// runs all 2*(TSTEPS-1) half-sweeps of
// polybench/jacobi_2d/jacobi_2d_numpy.py:6-10:
//
//   * CTA b owns the band of interior rows [r0, r1) and keeps both fields of
//     the ping-pong in shared memory, each with the band's rows, one halo row
//     on either side, and every column; the even field's faces are A's and
//     the odd field's faces are B's, as in the reference's arrays;
//   * each half-sweep evaluates the band's first and last rows first, writes
//     them to an exchange buffer in global memory and publishes a step counter
//     with a release reduction; then the interior rows, which hide the hand-off;
//     then it waits (acquire, bounded) for both neighbours' counters and copies
//     their edge rows in as its halo rows;
//   * at the end the newest field goes to A and the previous one to B.
//
// The exchange buffer has two slots per band (by step parity).  A band
// overwrites a slot two steps later, after its neighbours have published the
// step in between, so they have finished reading it.  Per point the arithmetic
// is jacobi_core.cuh's warp strips (fixed-point binary64 next to hardware
// binary64 warps), so the results are bit-identical to the chained kernel and
// to the reference.  Every wait is bounded: a neighbour that publishes nothing
// for two seconds sets an error word and the kernel ends.
#include <algorithm>
#include <mutex>

#include "jacobi_core.cuh"
#include "npbgb_common.cuh"
#include "tma.cuh"

namespace npbgb {

extern int64_t g_cfg_f64_emulation;
extern int64_t g_cfg_jacobi_bands;
extern int64_t g_cfg_jacobi_bands_warps;

namespace {

constexpr uint64_t kJLimitNs = 2000000000ull;

__device__ unsigned int g_jbands_error;  // bit 0: a neighbour wait gave up

__device__ __forceinline__ uint32_t ld_acquire_u32(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void red_release_add_u32(uint32_t* p, uint32_t v) {
  asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Half-sweep of buffer rows [ra, rb) of one band: every warp takes strips of
// 32 columns in turn; with FX the first hw_warps warps use hardware binary64.
template <typename T, bool FX, int W>
__device__ __forceinline__ void band_rows(const T* src, T* dst, int64_t nx, int ra, int rb,
                                          int hw_warps, uint32_t one) {
  if (ra >= rb) return;
  const int warp = threadIdx.x >> 5;
  for (int64_t k0 = 1 + int64_t(warp) * 32; k0 < nx - 1; k0 += 32 * W) {
    if (FX && (warp % 8) < hw_warps)
      jcore::strip_rows<T, false, false, 1>(src, dst, nx, k0, ra, rb, one);
    else
      jcore::strip_rows<T, FX, false, FX ? 1 : 4>(src, dst, nx, k0, ra, rb, one);
  }
}

// W warps per CTA; with FX, warps w with w % 8 < hw_warps use hardware binary64.
template <typename T, bool FX, int W>
__global__ void __launch_bounds__(32 * W, 1)
jacobi2d_bands(T* __restrict__ A, T* __restrict__ B, int64_t ny, int64_t nx, int32_t halfsweeps,
               int rpb, T* __restrict__ exch, uint32_t* __restrict__ counters, int hw_warps,
               uint32_t one) {
  constexpr int kJThreads = 32 * W;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_ok;
  const int tid = threadIdx.x;
  const int nb = gridDim.x, b = blockIdx.x;
  const int64_t r0 = 1 + int64_t(b) * rpb;
  const int64_t r1 = std::min<int64_t>(r0 + rpb, ny - 1);
  const int rows = int(r1 - r0);               // >= 1 (the host sizes the bands)
  const int64_t plane = int64_t(rows + 2) * nx;  // buffer row k <-> grid row r0 - 1 + k
  T* buf[2] = {reinterpret_cast<T*>(smem_raw), reinterpret_cast<T*>(smem_raw) + plane};

  // Field 0 (A, with A's faces) and the odd fields' faces (B).
  for (int64_t e = tid; e < plane; e += kJThreads) {
    buf[0][e] = __ldcg(A + (r0 - 1) * nx + e);
    buf[1][e] = __ldcg(B + (r0 - 1) * nx + e);
  }
  __syncthreads();

  auto slot = [&](int parity, int band, int side) -> T* {
    return exch + ((int64_t(parity) * nb + band) * 2 + side) * nx;
  };
  bool ok = true;
  for (int32_t s = 0; s < halfsweeps && ok; ++s) {
    const T* src = buf[s & 1];
    T* dst = buf[(s + 1) & 1];
    // Edge rows first, then publish them.
    band_rows<T, FX, W>(src, dst, nx, 1, 2, hw_warps, one);
    if (rows > 1) band_rows<T, FX, W>(src, dst, nx, rows, rows + 1, hw_warps, one);
    __syncthreads();
    T* top = slot(s & 1, b, 0);
    T* bot = slot(s & 1, b, 1);
    for (int64_t j = tid; j < nx; j += kJThreads) {
      __stcg(top + j, dst[nx + j]);
      __stcg(bot + j, dst[int64_t(rows) * nx + j]);
    }
    __syncthreads();  // the CTA's stores before thread 0's release, which is cumulative
    if (tid == 0) red_release_add_u32(counters + b, 1u);
    // The interior hides the neighbours' hand-off.
    band_rows<T, FX, W>(src, dst, nx, 2, rows, hw_warps, one);
    if (tid == 0) {
      const uint32_t want = uint32_t(s + 1);
      const uint64_t t0 = tma::globaltimer();
      bool good = true;
      for (int n = b - 1; n <= b + 1 && good; n += 2) {
        if (n < 0 || n >= nb) continue;
        while (ld_acquire_u32(counters + n) < want) {
          if (tma::globaltimer() - t0 > kJLimitNs) {
            good = false;
            break;
          }
          __nanosleep(32);
        }
      }
      s_ok = good ? 1 : 0;
    }
    __syncthreads();
    ok = s_ok != 0;
    if (!ok) {
      if (tid == 0) atomicOr(&g_jbands_error, 1u);
      break;
    }
    // Halo rows of the new field from the neighbours' edge rows.
    if (b > 0) {
      const T* up = slot(s & 1, b - 1, 1);
      for (int64_t j = tid; j < nx; j += kJThreads) dst[j] = __ldcg(up + j);
    }
    if (b + 1 < nb) {
      const T* dn = slot(s & 1, b + 1, 0);
      for (int64_t j = tid; j < nx; j += kJThreads) dst[int64_t(rows + 1) * nx + j] = __ldcg(dn + j);
    }
    __syncthreads();
  }
  if (!ok) return;
  // The newest field (even: buffer 0) to A, the previous one to B: band rows,
  // interior columns only (faces are never written).
  const T* newest = buf[halfsweeps & 1];
  const T* previous = buf[(halfsweeps + 1) & 1];
  for (int64_t e = tid; e < int64_t(rows) * nx; e += kJThreads) {
    const int64_t j = e % nx;
    if (j == 0 || j == nx - 1) continue;
    A[r0 * nx + e] = newest[nx + e];
    B[r0 * nx + e] = previous[nx + e];
  }
}

cudaError_t scratch_pool(cudaMemPool_t* out) {
  static std::mutex mu;
  static cudaMemPool_t pools[64] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(mu);
  if (!pools[dev]) {
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    cudaMemPool_t p;
    if ((e = cudaMemPoolCreate(&p, &props)) != cudaSuccess) return e;
    uint64_t keep = ~0ull;
    cudaMemPoolSetAttribute(p, cudaMemPoolAttrReleaseThreshold, &keep);
    pools[dev] = p;
  }
  *out = pools[dev];
  return cudaSuccess;
}

// Warps per CTA: by default one 32-column strip per warp and row, at least 8
// and at most 32 warps.  Measured on GB300 (binary64, TSTEPS=100): 1000^2
// takes 2.02 ms with 32 warps against 3.68 with 8, 500^2 1.01 ms with 16
// against 1.06 with 32, and 150^2 (TSTEPS=50) 0.315 ms with 8.
int bands_warps(int64_t nx) {
  const int64_t w = g_cfg_jacobi_bands_warps;
  if (w == 8 || w == 16 || w == 32) return int(w);
  const int64_t strips = cdiv(nx - 2, int64_t(32));
  return strips <= 8 ? 8 : strips <= 16 ? 16 : 32;
}

}  // namespace

// Runs the whole time loop of Jacobi-2D in one cooperative launch when asked
// (NPBGB_CFG_JACOBI_BANDS = 2) and the bands fit in shared memory (about 1.4 M
// binary64 cells or 2.8 M binary32 cells on 152 SMs); NPBGB_ERR_STATE
// otherwise (the caller then uses the chained kernels).  It is not the
// automatic choice.  Measured on GB300 against the chained launches: binary64
// 1000^2 TSTEPS=100 2.01 against 2.08 ms and 150^2 TSTEPS=50 0.32 against 0.39
// ms, but over 120 grids of the batched configuration (64 to 2048 per side,
// binary64) 337 against 330 ms in all: one CTA per SM leaves tall, narrow
// grids latency-bound, and grids wider than 1026 columns give some warps two
// strips.  On the served stream it also cost 3-5% of throughput, because the
// cooperative launch holds every SM while other streams' kernels wait.
// Binary32 measured slower at every size (1000^2: 1.02 against 0.71 ms).  The
// autotuner takes it per shape class where it measures faster.
template <typename T>
int32_t jacobi2d_bands_run(T* a, T* b, int64_t ny, int64_t nx, int32_t tsteps, cudaStream_t st) {
  if (g_cfg_jacobi_bands != 2) return NPBGB_ERR_STATE;
  if (tsteps <= 1 || ny < 3 || nx < 3) return NPBGB_ERR_STATE;
  const int32_t hs = 2 * (tsteps - 1);
  int dev = 0, sms = 0, smem_max = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  const int64_t interior = ny - 2;
  const int nb = int(std::min<int64_t>(sms, interior));
  const int rpb = int(cdiv(interior, nb));
  const int nbands = int(cdiv(interior, rpb));  // every band holds >= 1 row
  const size_t smem = 2 * size_t(rpb + 2) * size_t(nx) * sizeof(T);
  if (smem + 1024 > size_t(smem_max)) return NPBGB_ERR_STATE;
  const bool fx = sizeof(T) == 8 && g_cfg_f64_emulation;
  const int warps = bands_warps(nx);
  using Kern = void (*)(T*, T*, int64_t, int64_t, int32_t, int, T*, uint32_t*, int, uint32_t);
  Kern kern = warps == 8 ? (fx ? jacobi2d_bands<T, true, 8> : jacobi2d_bands<T, false, 8>)
            : warps == 16 ? (fx ? jacobi2d_bands<T, true, 16> : jacobi2d_bands<T, false, 16>)
                          : (fx ? jacobi2d_bands<T, true, 32> : jacobi2d_bands<T, false, 32>);
  const int kJThreads = 32 * warps;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
  if (e != cudaSuccess) return cuda_status(e, "jacobi2d_bands: smem attribute");
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kJThreads, smem);
  if (per_sm < 1 || int64_t(per_sm) * sms < nbands) return NPBGB_ERR_STATE;
  // exchange rows (2 parities x 2 sides per band) and the step counters
  const size_t ex_bytes = size_t(4) * nbands * size_t(nx) * sizeof(T);
  const size_t bytes = ex_bytes + size_t(nbands) * sizeof(uint32_t) + 256;
  cudaMemPool_t pool;
  void* scratch = nullptr;
  if ((e = scratch_pool(&pool)) != cudaSuccess ||
      (e = cudaMallocFromPoolAsync(&scratch, bytes, pool, st)) != cudaSuccess)
    return cuda_status(e, "jacobi2d_bands: scratch");
  T* ex = static_cast<T*>(scratch);
  uint32_t* counters = reinterpret_cast<uint32_t*>(static_cast<unsigned char*>(scratch) + ex_bytes);
  e = cudaMemsetAsync(counters, 0, size_t(nbands) * sizeof(uint32_t), st);
  if (e == cudaSuccess) {
    int hw = jacobi_hw_warps();
    uint32_t one = 1;
    int64_t ny_ = ny, nx_ = nx;
    int32_t hs_ = hs;
    int rpb_ = rpb;
    void* args[] = {&a, &b, &ny_, &nx_, &hs_, &rpb_, &ex, &counters, &hw, &one};
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(unsigned(nbands));
    cfg.blockDim = dim3(kJThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    e = counted(cudaLaunchKernelExC(&cfg, reinterpret_cast<const void*>(kern), args));
  }
  cudaFreeAsync(scratch, st);
  return cuda_status(e, "jacobi2d_bands");
}

template int32_t jacobi2d_bands_run<double>(double*, double*, int64_t, int64_t, int32_t, cudaStream_t);
template int32_t jacobi2d_bands_run<float>(float*, float*, int64_t, int64_t, int32_t, cudaStream_t);

uint32_t take_jacobi_bands_device_error() {
  unsigned int v = 0, zero = 0;
  if (cudaMemcpyFromSymbol(&v, g_jbands_error, sizeof(v)) != cudaSuccess) return 0xffffffffu;
  if (v) cudaMemcpyToSymbol(g_jbands_error, &zero, sizeof(zero));
  return v;
}

}  // namespace npbgb
