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

// ---------------------------------------------------------------------------
// TMA form: each warp streams its strip's rows through its own ring
// ---------------------------------------------------------------------------
// The plain-load strip keeps one row per warp in flight (binary64), so at
// 4096^2 the kernel waits on load latency with DRAM at a quarter of its
// bandwidth.  Here every warp owns a ring of kTmaRing boxes of kTmaRows rows
// of its strip and the two halo columns (34 columns of binary64, 36 of
// binary32: a 16-byte multiple), each box one cp.async.bulk.tensor copy that
// completes on the box's own mbarrier.  Lane 0 issues; every lane reads its
// column (and lanes 0 and 31 the halo columns) from shared memory into the
// same register queue as the plain-load strip, and a box's slot is refilled
// as soon as its last row has been read.  The warps of a CTA never wait on
// each other.  Rows beyond the array read as zero (the tensor map's
// out-of-bounds fill) and are never written.
constexpr int kTmaRows = 4;  // rows per box
constexpr int kTmaRing = 4;  // boxes per warp: 16 rows in flight

template <typename T>
struct TmaStrip {
  static constexpr int BX = sizeof(T) == 8 ? 34 : 36;  // box columns k0-1 .. k0+BX-2
  static constexpr int kBoxBytes = BX * kTmaRows * int(sizeof(T));
  static constexpr int kSlot = (kBoxBytes + 127) / 128 * 128;  // 128-byte aligned slots
  static constexpr int kWarpBytes = kTmaRing * kSlot;
  static constexpr size_t smem() { return size_t(kWarps) * (kWarpBytes + kTmaRing * sizeof(uint64_t)); }
};

__device__ unsigned int g_jacobi_tma_error;  // bit 0: an mbarrier wait timed out

// Output rows [ib, ie) of the strip at columns k0 .. k0+31 (warp-collective).
// FXW: this warp evaluates in fixed point.  Returns false when a wait gave up
// (after waiting, bounded, for the copies it still had in flight).
template <typename T, bool FXW, int MAD, bool IMUL>
__device__ __forceinline__ bool tma_strip_rows(const CUtensorMap* map, const T* src, T* dst, int64_t nx,
                                               int64_t k0, int64_t ib, int64_t ie, unsigned char* ring,
                                               uint64_t* bars, uint32_t one) {
  using G = TmaStrip<T>;
  using St = jcore::Strip<T, FXW, false, MAD, IMUL, false>;
  using S = typename St::S;
  const St s(src, dst, nx, k0, one);
  const int lane = threadIdx.x & 31;
  const int nrows = int(ie - ib) + 2;  // staged rows ib-1 .. ie
  const int nbox = (nrows + kTmaRows - 1) / kTmaRows;
  const int x0 = int(k0 - 1), y0 = int(ib - 1);  // x0 = 32 * strip: a 16-byte multiple
  auto issue = [&](int b) {
    uint64_t* bar = &bars[b % kTmaRing];
    tma::mbar_arrive_expect_tx(bar, G::kBoxBytes);
    tma::load_3d(ring + (b % kTmaRing) * G::kSlot, map, x0, y0 + b * kTmaRows, 0, bar);
  };
  auto read = [&](int q, S& own, S& halo) {
    const T* row = reinterpret_cast<const T*>(ring + ((q / kTmaRows) % kTmaRing) * G::kSlot) +
                   (q % kTmaRows) * G::BX;
    const T v = row[lane + 1];
    if constexpr (FXW) own = fx::from_f64_f59_or_poison(v); else own = v;
    if (lane == 0 || lane == 31) {
      const T h = row[lane == 0 ? 0 : 33];
      if constexpr (FXW) halo = fx::from_f64_f59_or_poison(h); else halo = h;
    }
  };
  const int first = nbox < kTmaRing ? nbox : kTmaRing;
  if (lane == 0)
    for (int b = 0; b < first; ++b) issue(b);
  int issued = first, waited = 1;
  bool ok = tma::mbar_wait(&bars[0], 0);
  S xp = S(0), xc = S(0), xn = S(0), hp = S(0), hc = S(0), hn = S(0);
  if (ok) {
    read(0, xp, hp);
    read(1, xc, hc);
  }
  for (int q = 1; ok && q + 1 < nrows; ++q) {  // output row ib - 1 + q
    const int qn = q + 1;
    if (qn % kTmaRows == 0) {
      const int b = qn / kTmaRows;
      ok = tma::mbar_wait(&bars[b % kTmaRing], uint32_t((b / kTmaRing) & 1));
      waited = b + 1;
      if (!ok) break;
    }
    read(qn, xn, hn);
    if (qn % kTmaRows == kTmaRows - 1) {  // box fully read: refill its slot
      tma::fence_proxy_async();
      __syncwarp();
      const int b = qn / kTmaRows + kTmaRing;
      if (b < nbox) {
        if (lane == 0) issue(b);
        issued = b + 1;
      }
    }
    s.point(ib - 1 + q, xp, xc, xn, hc);
    xp = xc;
    xc = xn;
    hc = hn;
  }
  if (!ok)  // let the copies still in flight land (bounded) before the CTA may exit
    for (int b = waited; b < issued; ++b)
      tma::mbar_wait_for(&bars[b % kTmaRing], uint32_t((b / kTmaRing) & 1), tma::kWaitLimitNs / 16);
  return ok;
}

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
  // The TMA ring where it pays: binary64 arrays of 64 MiB and more (beyond
  // the L2), automatically; any aligned grid when forced (NPBGB_CFG_JACOBI_TMA
  // = 2).  Measured on GB300 (TSTEPS=21 at 4096^2, 41 at 2048^2, 100 at 1000^2
  // and 500^2; best settings of each form, ms): 4096^2 binary64 3.44 against
  // 4.04 with plain loads; L2-resident grids lose (2048^2 2.11 / 1.92, 1000^2
  // 1.91 / 1.64, 500^2 1.45 / 0.89), and binary32 loses at every size (4096^2
  // 1.68 / 1.16): its plain strips already load four rows ahead.
  const bool big = nx * ny * int64_t(sizeof(T)) >= (int64_t(64) << 20);
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
