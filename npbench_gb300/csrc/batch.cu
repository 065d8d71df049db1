// Batched time stepping of many independent Jacobi-2D grids in one persistent launch.
//
// Every grid of the batch (any shape, binary32 or binary64, its own TSTEPS) is
// cut into bands of rows.  A band is owned by exactly one CTA of a
// cooperative (all-resident) persistent kernel; the host assigns bands to
// CTAs so that the CTAs carry equal work (longest-processing-time greedy).
// Each band keeps in global memory the number of half-sweeps it has
// completed.  A CTA advances one of its bands by one half-sweep when both
// neighbouring bands of the same grid have completed at least as many
// half-sweeps: that gives the band the rows it reads (read-after-write) and
// guarantees that no neighbour still reads the rows it overwrites
// (write-after-read).  Counters are published with release semantics after
// the CTA's stores, read with acquire semantics, and grid data is read
// through L2 (ld.global.cg) so no SM sees stale L1 lines.  The band whose
// count is the global minimum is always ready, so the batch cannot deadlock;
// every wait is still bounded (no progress for kBatchLimitNs -> error word,
// kernel exits).
//
// Per point the arithmetic is that of jacobi2d.cu (bit-identical to
// polybench/jacobi_2d/jacobi_2d_numpy.py:6-10), including the fixed-point
// binary64 path.
//
// Large batches take a second form ("stepped"): one launch per half-sweep
// index s covers every tile of every grid that still has a half-sweep s to do,
// and consecutive launches are chained (programmatic dependent launch), so the
// kernel boundary is the only dependency and no CTA ever waits on another.
// Grids are sorted by their half-sweep count, so the grids active at s are a
// prefix and launch s simply covers the first N_s tiles; a tile table maps each
// CTA to its grid.  Small batches keep the persistent form, whose launch count
// does not grow with the step count.
#include <algorithm>
#include <cstring>
#include <mutex>
#include <new>
#include <queue>
#include <utility>
#include <vector>

#include "heat_core.cuh"
#include "jacobi_core.cuh"
#include "npbgb_common.cuh"
#include "queue.cuh"
#include "tma.cuh"

namespace npbgb {

extern int64_t g_cfg_f64_emulation;
extern int64_t g_cfg_jacobi_hw_warps;
extern int64_t g_cfg_batch_ctas_per_sm;
extern int64_t g_cfg_batch_mode;
extern int64_t g_cfg_batch_tma;

namespace {

constexpr int kBWarps = 8;
constexpr int kBThreads = 32 * kBWarps;
constexpr uint64_t kBatchLimitNs = 2000000000ull;  // two seconds without progress

struct BandDesc {
  void* a;          // array holding the field after an even number of half-sweeps
  void* b;          // the other array
  int32_t n0, n1, n2;  // grid extents (Jacobi-2D: n0 rows, n1 columns, n2 = 1)
  int32_t r0, r1;   // interior range [r0, r1) of this band along axis 0
  int32_t steps;    // half-sweeps to perform in this launch
  int32_t step0;    // half-sweeps the grid has already had (parity of the first source)
  int16_t dtype;    // NPBGB_F64 / NPBGB_F32
  int16_t kind;     // NPBGB_KIND_JACOBI2D / NPBGB_KIND_HEAT3D
  int32_t left;     // band before (axis-0 indices < r0) of the same grid, or -1
  int32_t right;    // band after (indices >= r1), or -1
};

// One grid of a stepped batch.
struct StepGrid {
  void* a;
  void* b;
  int64_t first_tile;  // index of the grid's first tile in the tile table
  int32_t n0, n1, n2;
  int32_t step0;       // half-sweeps already done (parity of the first source)
  int32_t count;       // half-sweeps to do in this launch chain
  int32_t chunk;       // rows (Jacobi-2D) or planes (Heat-3D) per tile
  int32_t tx, ty;      // tiles along the contiguous axis and the next one
  int16_t dtype, kind;
  int32_t map;         // binary64 Jacobi-2D: index of the grid's tensor-map pair, or -1
};

// A share of one grid's arrays for the binary32 <-> binary64 conversions of a
// stepped batch (grids run in binary64 for binary32 callers).
struct ConvChunk {
  double* a;
  double* b;
  float* a32;
  float* b32;
  int64_t off, count;
};
constexpr int64_t kConvChunk = 1 << 16;  // elements per conversion CTA

__device__ unsigned int g_batch_error;  // bit 0: a CTA made no progress for the limit; bit 1: a TMA wait gave up

__device__ __forceinline__ uint32_t ld_acquire(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void red_release_add(uint32_t* p, uint32_t v) {
  asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// One half-sweep of band rows [r0, r1) from src to dst over all interior
// columns: the CTA's warps take the band's 32-column strips in turn.  Loads
// and stores go through L2 (other CTAs wrote, or will read, these rows).
template <typename T, bool FX>
__device__ __noinline__ void band_half_sweep(const T* src, T* dst, int64_t nx, int r0, int r1,
                                             int hw_warps, uint32_t one) {
  const int warp = threadIdx.x >> 5;
  for (int64_t k0 = 1 + int64_t(warp) * 32; k0 < nx - 1; k0 += 32 * kBWarps) {
    if (FX && warp < hw_warps)
      jcore::strip_rows<T, false, true, 1>(src, dst, nx, k0, r0, r1, one);
    else
      jcore::strip_rows<T, FX, true, 4>(src, dst, nx, k0, r0, r1, one);
  }
}

// One half-sweep of Heat-3D planes [r0, r1): the CTA walks the plane's
// 8 x 32 tiles and streams each along axis 0 (heat_core.cuh), through L2.
template <typename T, bool FX>
__device__ __noinline__ void heat_band_half_sweep(const T* src, T* dst, int64_t n1, int64_t n2,
                                                  int r0, int r1) {
  static_assert(hcore::kThreads == kBThreads, "tile streamer uses the whole CTA");
  __shared__ hcore::PlaneBuf<T, FX> plane;
  const int64_t tiles_j = (n1 - 2 + hcore::kTJ - 1) / hcore::kTJ;
  const int64_t tiles_k = (n2 - 2 + hcore::kTK - 1) / hcore::kTK;
  for (int64_t t = 0; t < tiles_j * tiles_k; ++t) {
    const int64_t j0 = 1 + (t / tiles_k) * hcore::kTJ, k0 = 1 + (t % tiles_k) * hcore::kTK;
    hcore::tile_stream<T, FX, true>(src, dst, n1, n2, j0, k0, r0, r1, plane);
  }
}

// MINB: CTAs per SM the register allocation aims for (more CTAs hide more
// memory latency; fewer registers spill more).
template <int MINB>
__global__ void __launch_bounds__(kBThreads, MINB)
batch_persistent(const BandDesc* __restrict__ bands, uint32_t* done, const int32_t* __restrict__ cta_off,
                 const int32_t* __restrict__ cta_bands, int f64_emulation, int hw_warps,
                 uint32_t one) {
  __shared__ int s_flag;
  const int tid = threadIdx.x;
  const int b_begin = cta_off[blockIdx.x], b_end = cta_off[blockIdx.x + 1];
  uint64_t last_progress = tma::globaltimer();
  int cursor = b_begin;
  for (;;) {
    bool all_done = true, progressed = false;
    for (int n = 0; n < b_end - b_begin; ++n) {
      const int idx = cta_bands[cursor];
      cursor = cursor + 1 < b_end ? cursor + 1 : b_begin;
      const BandDesc d = bands[idx];
      // Advance this band as far as its neighbours allow.
      for (;;) {
        if (tid == 0) {
          const uint32_t s = done[idx];  // only this CTA writes it
          int state = 0;                 // 0 finished, 1 ready, 2 blocked
          if (int(s) < d.steps) {
            const bool ok_l = d.left < 0 || ld_acquire(done + d.left) >= s;
            const bool ok_r = d.right < 0 || ld_acquire(done + d.right) >= s;
            state = (ok_l && ok_r) ? 1 : 2;
          }
          s_flag = state == 1 ? int(s) : (state == 0 ? -1 : -2);
        }
        __syncthreads();
        const int s = s_flag;
        __syncthreads();
        if (s == -1) break;           // finished
        all_done = false;
        if (s == -2) break;           // blocked for now
        const bool odd = ((d.step0 + s) & 1) != 0;
        const void* src = odd ? d.b : d.a;
        void* dst = odd ? d.a : d.b;
        if (d.kind == NPBGB_KIND_HEAT3D) {
          if (d.dtype == NPBGB_F64) {
            if (f64_emulation)
              heat_band_half_sweep<double, true>(static_cast<const double*>(src),
                                                 static_cast<double*>(dst), d.n1, d.n2, d.r0, d.r1);
            else
              heat_band_half_sweep<double, false>(static_cast<const double*>(src),
                                                  static_cast<double*>(dst), d.n1, d.n2, d.r0, d.r1);
          } else {
            heat_band_half_sweep<float, false>(static_cast<const float*>(src),
                                               static_cast<float*>(dst), d.n1, d.n2, d.r0, d.r1);
          }
        } else if (d.dtype == NPBGB_F64) {
          if (f64_emulation)
            band_half_sweep<double, true>(static_cast<const double*>(src), static_cast<double*>(dst),
                                          d.n1, d.r0, d.r1, hw_warps, one);
          else
            band_half_sweep<double, false>(static_cast<const double*>(src), static_cast<double*>(dst),
                                           d.n1, d.r0, d.r1, hw_warps, one);
        } else {
          band_half_sweep<float, false>(static_cast<const float*>(src), static_cast<float*>(dst),
                                        d.n1, d.r0, d.r1, hw_warps, one);
        }
        // bar.sync orders the CTA's stores before thread 0's release, which is
        // cumulative; the counter is written by this CTA only and goes s -> s+1,
        // so a release reduction publishes it (measured faster per hand-off on
        // GB300 than a fence plus release store).
        __syncthreads();
        if (tid == 0) red_release_add(done + idx, 1u);
        progressed = true;
      }
    }
    if (all_done) return;
    if (progressed) {
      last_progress = tma::globaltimer();
    } else {
      if (tma::globaltimer() - last_progress > kBatchLimitNs) {
        if (tid == 0) atomicOr(&g_batch_error, 1u);
        return;
      }
      __nanosleep(200);
    }
  }
}

// Half-sweep s of every tile in [0, gridDim.x): CTA t finds its grid in the
// tile table and processes one tile (Jacobi-2D: 8 warps x 32 columns x chunk
// rows; Heat-3D: a 32 x 8 column tile streamed over chunk planes).  Five CTAs
// per SM (48 registers, a few spilled): on the 4096-grid batch 3.13 s per pass
// against 3.36 s with four (64 registers) and 3.47 s with six (40 registers,
// more spills).
__global__ void __launch_bounds__(kBThreads, 5)
batch_step(const StepGrid* __restrict__ grids, const int32_t* __restrict__ tile_grid, int32_t s,
           int f64_emulation, int hw_warps, uint32_t one, const CUtensorMap* __restrict__ maps) {
  pdl_begin();
  extern __shared__ __align__(128) unsigned char ring_smem[];  // the TMA rings (binary64 Jacobi-2D)
  const int64_t t = blockIdx.x;
  const StepGrid G = grids[tile_grid[t]];
  const int64_t r = t - G.first_tile;
  const bool odd = ((G.step0 + s) & 1) != 0;
  const void* src = odd ? G.b : G.a;
  void* dst = odd ? G.a : G.b;
  const int64_t bx = r % G.tx, rest = r / G.tx;
  if (G.kind == NPBGB_KIND_HEAT3D) {
    __shared__ hcore::PlaneBuf<double, true> plane;  // the largest element type
    const int64_t by = rest % G.ty, bz = rest / G.ty;
    const int64_t k0 = 1 + bx * hcore::kTK, j0 = 1 + by * hcore::kTJ;
    const int64_t ib = 1 + bz * G.chunk, ie = min(ib + G.chunk, int64_t(G.n0) - 1);
    if (G.dtype == NPBGB_F64) {
      if (f64_emulation)
        hcore::tile_stream<double, true, false>(static_cast<const double*>(src),
                                                static_cast<double*>(dst), G.n1, G.n2, j0, k0, ib,
                                                ie, plane);
      else
        hcore::tile_stream<double, false, false>(static_cast<const double*>(src),
                                                 static_cast<double*>(dst), G.n1, G.n2, j0, k0, ib,
                                                 ie, reinterpret_cast<hcore::PlaneBuf<double, false>&>(plane));
    } else {
      hcore::tile_stream<float, false, false>(static_cast<const float*>(src),
                                              static_cast<float*>(dst), G.n1, G.n2, j0, k0, ib,
                                              ie, reinterpret_cast<hcore::PlaneBuf<float, false>&>(plane));
    }
    return;
  }
  const int warp = threadIdx.x >> 5;
  const int64_t k0 = 1 + (bx * kBWarps + warp) * 32;
  if (k0 >= G.n1 - 1) return;  // warp-uniform; the strip path has no CTA barrier
  const int64_t ib = 1 + rest * G.chunk, ie = min(ib + G.chunk, int64_t(G.n0) - 1);
  if (G.dtype == NPBGB_F64 && G.map >= 0) {
    // Each warp's ring of TMA copies (jcore::tma_strip_rows), from the source's map.
    using TS = jcore::TmaStrip<double, kBWarps>;
    const double* sp = static_cast<const double*>(src);
    double* dp = static_cast<double*>(dst);
    const CUtensorMap* map = &maps[2 * G.map + (odd ? 1 : 0)];
    // The rings start at the first 128-byte boundary of the dynamic shared
    // memory (TMA destinations are 128-byte aligned; the launch adds 128 bytes).
    unsigned char* rings = ring_smem + ((128u - (tma::smem_u32(ring_smem) & 127u)) & 127u);
    unsigned char* ring = rings + warp * TS::kWarpBytes;
    uint64_t* bars = reinterpret_cast<uint64_t*>(rings + kBWarps * TS::kWarpBytes) + warp * jcore::kTmaRing;
    if ((threadIdx.x & 31) == 0) {
      tma::fence_tensormap_acquire(map);
      for (int q = 0; q < jcore::kTmaRing; ++q) tma::mbar_init(&bars[q], 1);
      tma::fence_mbar_init();
    }
    __syncwarp();
    const bool ok = (!f64_emulation || warp < hw_warps)
                        ? jcore::tma_strip_rows<double, false, 0, true>(map, sp, dp, G.n1, k0, ib, ie, ring, bars, one)
                        : jcore::tma_strip_rows<double, true, 0, true>(map, sp, dp, G.n1, k0, ib, ie, ring, bars, one);
    if (!ok && (threadIdx.x & 31) == 0) atomicOr(&g_batch_error, 2u);
  } else if (G.dtype == NPBGB_F64) {
    const double* sp = static_cast<const double*>(src);
    double* dp = static_cast<double*>(dst);
    // Two rows loaded ahead (measured 12% faster than one with 128-row tiles; with
    // 64-row tiles and 5 CTAs per SM three and four rows ahead spill and measured
    // 3.77 and 3.88 s per pass of the 4096 grids against 3.13 s).
    if (!f64_emulation || warp < hw_warps)
      jcore::strip_rows<double, false, false, 2>(sp, dp, G.n1, k0, ib, ie, one);
    else
      jcore::strip_rows<double, true, false, 2>(sp, dp, G.n1, k0, ib, ie, one);
  } else {
    jcore::strip_rows<float, false, false, 4>(static_cast<const float*>(src),
                                              static_cast<float*>(dst), G.n1, k0, ib, ie, one);
  }
}

// Widens (before the first half-sweep) or rounds back (after the last) the
// binary32 arrays of the batch's binary64-promoted grids, one chunk per CTA.
__global__ void __launch_bounds__(256) batch_convert(const ConvChunk* __restrict__ chunks, int widen) {
  pdl_begin();
  const ConvChunk c = chunks[blockIdx.x];
  for (int64_t i = c.off + threadIdx.x; i < c.off + c.count; i += blockDim.x) {
    if (widen) {
      c.a[i] = double(c.a32[i]);
      c.b[i] = double(c.b32[i]);
    } else {
      c.a32[i] = __double2float_rn(c.a[i]);
      c.b32[i] = __double2float_rn(c.b[i]);
    }
  }
}

using PersistentFn = void (*)(const BandDesc*, uint32_t*, const int32_t*, const int32_t*, int, int,
                              uint32_t);

PersistentFn persistent_kernel(int ctas_per_sm) {
  return ctas_per_sm >= 3 ? batch_persistent<3> : batch_persistent<2>;
}

}  // namespace

uint32_t take_batch_device_error() {
  unsigned int v = 0, zero = 0;
  if (cudaMemcpyFromSymbol(&v, g_batch_error, sizeof(v)) != cudaSuccess) return 0xffffffffu;
  if (v) cudaMemcpyToSymbol(g_batch_error, &zero, sizeof(zero));
  return v;
}

}  // namespace npbgb

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
struct npbgb_batch {
  int device = 0;
  int64_t nbands = 0;
  int nctas = 0;
  npbgb::BandDesc* d_bands = nullptr;
  uint32_t* d_done = nullptr;
  int32_t* d_cta_off = nullptr;
  int32_t* d_cta_bands = nullptr;
  int64_t updates = 0;
  int64_t cap_bands = 0;  // allocated capacity of d_bands / d_done / d_cta_bands
  int64_t cap_ctas = 0;   // allocated capacity of d_cta_off
  int ctas_per_sm = 2;  // persistent kernel variant chosen when planned
  cudaGraphExec_t graph = nullptr;
  int64_t graph_kernels = 0;  // kernel launches in the graph, counted at each replay
  cudaStream_t graph_stream = nullptr;
  // Stepped form (mode NPBGB_BATCH_STEPPED).
  int32_t mode = NPBGB_BATCH_PERSISTENT;
  npbgb::StepGrid* d_step = nullptr;
  int32_t* d_tiles = nullptr;
  int64_t cap_step = 0, cap_tiles = 0, ntiles = 0;
  std::vector<int32_t> launch_tiles;  // CTAs of launch s = tiles of the grids active at s
  npbgb::ConvChunk* d_conv = nullptr;  // stepped form: conversion chunks of promoted grids
  int64_t cap_conv = 0, nconv = 0;
  CUtensorMap* d_maps = nullptr;  // stepped form: tensor maps (a, b) of the TMA grids
  int64_t cap_maps = 0;
  size_t step_smem = 0;           // dynamic shared memory of each stepped launch
  // Queue form (mode NPBGB_BATCH_QUEUE).
  npbgb::qhost::StaticQueue* sq = nullptr;
};

namespace {

// Validates grid g and describes its bands through emit(BandDesc) (left/right
// are filled in relative to `first`, the index the grid's first band gets).
// Returns NPBGB_OK with *nbands_out = 0 for grids with nothing to do.
template <typename Emit>
int32_t plan_grid(const npbgb_grid& G, int64_t g, int32_t band_rows, int first, int64_t* nbands_out,
                  int64_t* updates_out, Emit emit, bool heat_allowed, bool conv_allowed = false) {
  using namespace npbgb;
  *nbands_out = 0;
  *updates_out = 0;
  if (G.kind != NPBGB_KIND_JACOBI2D && !(heat_allowed && G.kind == NPBGB_KIND_HEAT3D))
    return set_error(NPBGB_ERR_ARG, "batch: grid %lld: kind %d not supported here", (long long)g, G.kind);
  if (G.dtype != NPBGB_F64 && G.dtype != NPBGB_F32)
    return set_error(NPBGB_ERR_DTYPE, "batch: grid %lld: dtype %d", (long long)g, G.dtype);
  const bool heat = G.kind == NPBGB_KIND_HEAT3D;
  const int64_t n2 = heat ? G.n2 : 1;
  if (G.n0 < 0 || G.n1 < 0 || n2 < 0 || G.n0 > 0x7fffffff || G.n1 > 0x7fffffff || n2 > 0x7fffffff)
    return set_error(NPBGB_ERR_ARG, "batch: grid %lld: bad extents", (long long)g);
  if (G.step0 < 0 || G.nsteps < 0)
    return set_error(NPBGB_ERR_ARG, "batch: grid %lld: negative step0 or nsteps", (long long)g);
  if ((G.a32 || G.b32) && !conv_allowed)
    return set_error(NPBGB_ERR_ARG,
                     "batch: grid %lld: binary32 arrays for a binary64 run need the stepped or "
                     "queue form",
                     (long long)g);
  if ((G.a32 || G.b32) &&
      (!G.a32 || !G.b32 || G.a32 == G.b32 || G.dtype != NPBGB_F64 || G.a32 == G.a || G.a32 == G.b ||
       G.b32 == G.a || G.b32 == G.b))
    return set_error(NPBGB_ERR_ARG,
                     "batch: grid %lld: binary32 arrays need a binary64 grid and two distinct arrays",
                     (long long)g);
  const int64_t total = G.tsteps > 1 ? 2 * int64_t(G.tsteps - 1) : 0;
  int64_t todo = total - G.step0;
  if (G.nsteps > 0 && G.nsteps < todo) todo = G.nsteps;
  if (todo <= 0 || G.n0 < 3 || G.n1 < 3 || (heat && n2 < 3)) return NPBGB_OK;
  if (!G.a || !G.b || G.a == G.b)
    return set_error(NPBGB_ERR_ARG, "batch: grid %lld: null or aliased arrays", (long long)g);
  const int n0 = int(G.n0), n1 = int(G.n1);
  const int h = G.band_rows > 0 ? G.band_rows : (band_rows > 0 ? band_rows : (heat ? 8 : 32));
  const int64_t nb = cdiv(n0 - 2, h);
  for (int q = 0; q < int(nb); ++q) {
    BandDesc d;
    d.a = G.a;
    d.b = G.b;
    d.n0 = n0;
    d.n1 = n1;
    d.n2 = int32_t(n2);
    d.r0 = 1 + q * h;
    d.r1 = std::min(1 + (q + 1) * h, n0 - 1);
    d.steps = int32_t(todo);
    d.step0 = G.step0;
    d.dtype = int16_t(G.dtype);
    d.kind = int16_t(G.kind);
    d.left = q > 0 ? first + q - 1 : -1;
    d.right = q + 1 < int(nb) ? first + q + 1 : -1;
    emit(d);
  }
  *nbands_out = nb;
  *updates_out = todo * int64_t(n0 - 2) * (n1 - 2) * (heat ? (n2 - 2) : 1);
  return NPBGB_OK;
}

double band_work(const npbgb::BandDesc& d) {
  const double plane = d.kind == NPBGB_KIND_HEAT3D ? double(d.n1 - 2) * double(d.n2 - 2) * 2.0
                                                    : double(d.n1 - 2);
  return double(d.r1 - d.r0) * plane * d.steps * (d.dtype == NPBGB_F64 ? 2.0 : 1.0);
}

void free_batch(npbgb_batch* b) {
  if (!b) return;
  if (b->graph) cudaGraphExecDestroy(b->graph);
  npbgb::qhost::free_static(b->sq);
  cudaFree(b->d_conv);
  cudaFree(b->d_maps);
  cudaFree(b->d_step);
  cudaFree(b->d_tiles);
  cudaFree(b->d_bands);
  cudaFree(b->d_done);
  cudaFree(b->d_cta_off);
  cudaFree(b->d_cta_bands);
  delete b;
}

int32_t launch_stepped(npbgb_batch* b, cudaStream_t st) {
  using namespace npbgb;
  const int f64_emul = int(g_cfg_f64_emulation);
  const int hw_warps = jacobi_hw_warps();
  cudaError_t e = cudaSuccess;
  if (b->nconv > 0)
    e = launch_chained(batch_convert, dim3{unsigned(b->nconv)}, dim3{256u}, 0, st,
                       static_cast<const ConvChunk*>(b->d_conv), 1);
  for (size_t s = 0; s < b->launch_tiles.size() && e == cudaSuccess; ++s)
    e = launch_chained(batch_step, dim3{unsigned(b->launch_tiles[s])}, dim3{unsigned(kBThreads)},
                       b->step_smem, st, b->d_step, b->d_tiles, int32_t(s), f64_emul, hw_warps, 1u,
                       static_cast<const CUtensorMap*>(b->d_maps));
  if (b->nconv > 0 && e == cudaSuccess)
    e = launch_chained(batch_convert, dim3{unsigned(b->nconv)}, dim3{256u}, 0, st,
                       static_cast<const ConvChunk*>(b->d_conv), 0);
  return cuda_status(e, "batch: stepped launch");
}

int32_t launch_batch(npbgb_batch* b, cudaStream_t st) {
  using namespace npbgb;
  if (b->mode == NPBGB_BATCH_STEPPED) return launch_stepped(b, st);
  if (b->mode == NPBGB_BATCH_QUEUE) return qhost::launch_static(b->sq, st);
  cudaError_t e = cudaMemsetAsync(b->d_done, 0, sizeof(uint32_t) * size_t(b->nbands), st);
  if (e != cudaSuccess) return cuda_status(e, "batch: reset counters");
  int f64_emul = int(g_cfg_f64_emulation);
  int hw_warps = jacobi_hw_warps();
  uint32_t one = 1;
  void* args[] = {&b->d_bands, &b->d_done, &b->d_cta_off, &b->d_cta_bands, &f64_emul, &hw_warps, &one};
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(unsigned(b->nctas));
  cfg.blockDim = dim3(kBThreads);
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  e = counted(cudaLaunchKernelExC(&cfg, reinterpret_cast<const void*>(persistent_kernel(b->ctas_per_sm)), args));
  if (e != cudaSuccess) return cuda_status(e, "batch: cooperative launch");
  return NPBGB_OK;
}

}  // namespace

namespace {

// Batches of at least this many cells take the stepped form by default: each
// half-sweep launch then has enough tiles to fill the GPU many times over.
constexpr int64_t kSteppedCells = int64_t(1) << 24;

// The stepped form of `grids` (already validated by plan_grid).
int32_t plan_stepped(npbgb_batch* b, const npbgb_grid* grids, int64_t count, int32_t band_rows,
                     int64_t updates) {
  using namespace npbgb;
  std::vector<StepGrid> sg;
  std::vector<CUtensorMap> maps;
  for (int64_t g = 0; g < count; ++g) {
    const npbgb_grid& G = grids[g];
    const bool heat = G.kind == NPBGB_KIND_HEAT3D;
    const int64_t total = G.tsteps > 1 ? 2 * int64_t(G.tsteps - 1) : 0;
    int64_t todo = total - G.step0;
    if (G.nsteps > 0 && G.nsteps < todo) todo = G.nsteps;
    if (todo <= 0 || G.n0 < 3 || G.n1 < 3 || (heat && G.n2 < 3)) continue;
    StepGrid d{};
    d.a = G.a;
    d.b = G.b;
    d.n0 = int32_t(G.n0);
    d.n1 = int32_t(G.n1);
    d.n2 = heat ? int32_t(G.n2) : 1;
    d.step0 = G.step0;
    d.count = int32_t(todo);
    d.dtype = int16_t(G.dtype);
    d.kind = int16_t(G.kind);
    d.map = -1;
    // On request (NPBGB_CFG_BATCH_TMA), binary64 Jacobi-2D grids whose rows are
    // 16-byte multiples stream through each warp's ring of TMA copies (box: 34
    // columns x kTmaRows rows).  Off by default: on the 4096-grid batch the
    // rings measured 1.5-2.6% slower than two rows loaded ahead (3.21 against
    // 3.13 s per pass with 64-row tiles and 5 CTAs per SM; 3.73 against 3.68
    // with 32-row tiles and 4).
    if (!heat && G.dtype == NPBGB_F64 && g_cfg_batch_tma && (G.n1 * 8) % 16 == 0) {
      CUtensorMap ma, mb;
      const uint64_t dims[3] = {uint64_t(G.n1), uint64_t(G.n0), 1u};
      const uint32_t box[3] = {uint32_t(jcore::TmaStrip<double, kBWarps>::BX), uint32_t(jcore::kTmaRows), 1u};
      if (tma::encode_3d(&ma, 8, G.a, dims, box) == cudaSuccess &&
          tma::encode_3d(&mb, 8, G.b, dims, box) == cudaSuccess) {
        d.map = int32_t(maps.size() / 2);
        maps.push_back(ma);
        maps.push_back(mb);
      }
    }
    const int32_t rows = G.band_rows > 0 ? G.band_rows : (band_rows > 0 ? band_rows : (heat ? 16 : 32));
    d.chunk = rows;
    if (heat) {
      d.tx = int32_t(cdiv(G.n2 - 2, hcore::kTK));
      d.ty = int32_t(cdiv(G.n1 - 2, hcore::kTJ));
    } else {
      d.tx = int32_t(cdiv(G.n1 - 2, 32 * kBWarps));
      d.ty = 1;
    }
    sg.push_back(d);
  }
  std::vector<ConvChunk> conv;
  for (int64_t g = 0; g < count; ++g) {
    const npbgb_grid& G = grids[g];
    if (!G.a32) continue;
    const bool heat = G.kind == NPBGB_KIND_HEAT3D;
    const int64_t total = G.tsteps > 1 ? 2 * int64_t(G.tsteps - 1) : 0;
    int64_t todo = total - G.step0;
    if (G.nsteps > 0 && G.nsteps < todo) todo = G.nsteps;
    if (todo <= 0 || G.n0 < 3 || G.n1 < 3 || (heat && G.n2 < 3)) continue;  // nothing to do
    const int64_t cells = G.n0 * G.n1 * (heat ? G.n2 : 1);
    for (int64_t off = 0; off < cells; off += kConvChunk)
      conv.push_back(ConvChunk{static_cast<double*>(G.a), static_cast<double*>(G.b),
                               static_cast<float*>(G.a32), static_cast<float*>(G.b32), off,
                               std::min(kConvChunk, cells - off)});
  }
  if (int64_t(conv.size()) > 0x7fffffff) return set_error(NPBGB_ERR_NOMEM, "batch: too many chunks");
  std::stable_sort(sg.begin(), sg.end(),
                   [](const StepGrid& x, const StepGrid& y) { return x.count > y.count; });
  std::vector<int32_t> tiles;
  for (size_t q = 0; q < sg.size(); ++q) {
    StepGrid& d = sg[q];
    const int64_t n = int64_t(d.tx) * d.ty * cdiv(int64_t(d.n0) - 2, d.chunk);
    d.first_tile = int64_t(tiles.size());
    if (int64_t(tiles.size()) + n > 0x7fffffff) return set_error(NPBGB_ERR_NOMEM, "batch: too many tiles");
    tiles.insert(tiles.end(), size_t(n), int32_t(q));
  }
  // Launch s covers the grids with count > s: a prefix of the sorted list.
  std::vector<int32_t> launch_tiles;
  {
    size_t active = sg.size();
    const int32_t smax = sg.empty() ? 0 : sg.front().count;
    for (int32_t st = 0; st < smax; ++st) {
      while (active > 0 && sg[active - 1].count <= st) --active;
      launch_tiles.push_back(int32_t(active == sg.size() ? int64_t(tiles.size())
                                                         : sg[active].first_tile));
    }
  }
  cudaError_t e;
  const int64_t need_step = std::max<int64_t>(1, int64_t(sg.size()));
  if (need_step > b->cap_step) {
    cudaFree(b->d_step);
    b->d_step = nullptr;
    b->cap_step = 0;
    if ((e = cudaMalloc(&b->d_step, sizeof(StepGrid) * size_t(need_step))) != cudaSuccess)
      return cuda_status(e, "batch: alloc");
    b->cap_step = need_step;
  }
  const int64_t need_tiles = std::max<int64_t>(1, int64_t(tiles.size()));
  if (need_tiles > b->cap_tiles) {
    cudaFree(b->d_tiles);
    b->d_tiles = nullptr;
    b->cap_tiles = 0;
    if ((e = cudaMalloc(&b->d_tiles, sizeof(int32_t) * size_t(need_tiles))) != cudaSuccess)
      return cuda_status(e, "batch: alloc");
    b->cap_tiles = need_tiles;
  }
  if (!sg.empty() &&
      ((e = cudaMemcpy(b->d_step, sg.data(), sizeof(StepGrid) * sg.size(), cudaMemcpyHostToDevice)) != cudaSuccess ||
       (e = cudaMemcpy(b->d_tiles, tiles.data(), sizeof(int32_t) * tiles.size(), cudaMemcpyHostToDevice)) != cudaSuccess))
    return cuda_status(e, "batch: upload");
  if (int64_t(conv.size()) > b->cap_conv) {
    cudaFree(b->d_conv);
    b->d_conv = nullptr;
    b->cap_conv = 0;
    if ((e = cudaMalloc(&b->d_conv, sizeof(ConvChunk) * conv.size())) != cudaSuccess)
      return cuda_status(e, "batch: alloc");
    b->cap_conv = int64_t(conv.size());
  }
  if (!conv.empty() &&
      (e = cudaMemcpy(b->d_conv, conv.data(), sizeof(ConvChunk) * conv.size(), cudaMemcpyHostToDevice)) != cudaSuccess)
    return cuda_status(e, "batch: upload");
  b->nconv = int64_t(conv.size());
  if (int64_t(maps.size()) > b->cap_maps) {
    cudaFree(b->d_maps);
    b->d_maps = nullptr;
    b->cap_maps = 0;
    if ((e = cudaMalloc(&b->d_maps, sizeof(CUtensorMap) * maps.size())) != cudaSuccess)
      return cuda_status(e, "batch: alloc");
    b->cap_maps = int64_t(maps.size());
  }
  if (!maps.empty() &&
      (e = cudaMemcpy(b->d_maps, maps.data(), sizeof(CUtensorMap) * maps.size(), cudaMemcpyHostToDevice)) != cudaSuccess)
    return cuda_status(e, "batch: upload");
  b->step_smem = maps.empty() ? 0 : jcore::TmaStrip<double, kBWarps>::smem() + 128;
  b->mode = NPBGB_BATCH_STEPPED;
  b->ntiles = int64_t(tiles.size());
  b->launch_tiles = std::move(launch_tiles);
  b->nbands = b->ntiles;  // "nothing to do" checks use nbands
  b->nctas = int(b->launch_tiles.size());
  b->updates = updates;
  return NPBGB_OK;
}

// Plans `grids` into batch b, reusing its device buffers when they are large
// enough (they grow otherwise).  Invalidates a captured graph.
int32_t plan_into(npbgb_batch* b, const npbgb_grid* grids, int64_t count, int32_t band_rows) {
  using namespace npbgb;
  if (count < 0 || (count > 0 && !grids)) return set_error(NPBGB_ERR_ARG, "batch: bad grid list");
  if (band_rows < 0) return set_error(NPBGB_ERR_ARG, "batch: band_rows < 0");
  int64_t cells = 0;
  for (int64_t g = 0; g < count; ++g) {
    const npbgb_grid& G = grids[g];
    cells += int64_t(G.n0) * G.n1 * (G.kind == NPBGB_KIND_HEAT3D ? G.n2 : 1);
  }
  bool conv = false;
  for (int64_t g = 0; g < count && !conv; ++g) conv = grids[g].a32 || grids[g].b32;
  // Grids promoted to binary64 for binary32 callers need conversion launches,
  // which the stepped and queue forms have; by default they take the stepped one.
  const int32_t mode = g_cfg_batch_mode != 0
                           ? int32_t(g_cfg_batch_mode)
                           : ((conv || cells >= kSteppedCells) ? NPBGB_BATCH_STEPPED
                                                               : NPBGB_BATCH_PERSISTENT);
  if (mode == NPBGB_BATCH_QUEUE) {
    // The queue planner validates the grids itself (it also takes binary32
    // arrays of grids run in binary64).
    qhost::StaticQueue* sq = nullptr;
    int64_t qup = 0, qtiles = 0;
    const int32_t r = qhost::plan_static(grids, count, band_rows, int(g_cfg_batch_ctas_per_sm),
                                         &sq, &qup, &qtiles);
    if (r != NPBGB_OK) return r;
    if (b->graph) {
      cudaGraphExecDestroy(b->graph);
      b->graph = nullptr;
    }
    qhost::free_static(b->sq);
    b->sq = sq;
    b->mode = NPBGB_BATCH_QUEUE;
    b->launch_tiles.clear();
    b->ntiles = qtiles;
    b->nbands = qtiles;  // "nothing to do" checks use nbands
    b->nctas = qhost::static_ctas(b->sq);
    b->updates = qup;
    return NPBGB_OK;
  }
  std::vector<BandDesc> bands;
  int64_t updates = 0;
  for (int64_t g = 0; g < count; ++g) {
    int64_t nb = 0, up = 0;
    const int32_t r = plan_grid(grids[g], g, band_rows, int(bands.size()), &nb, &up,
                                [&](const BandDesc& d) { bands.push_back(d); }, true,
                                mode == NPBGB_BATCH_STEPPED);
    if (r != NPBGB_OK) return r;
    if (int64_t(bands.size()) > 0x7fffffff) return set_error(NPBGB_ERR_NOMEM, "batch: too many bands");
    updates += up;
  }
  if (b->graph) {
    cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
  }
  qhost::free_static(b->sq);
  b->sq = nullptr;
  b->nconv = 0;
  if (mode == NPBGB_BATCH_STEPPED) return plan_stepped(b, grids, count, band_rows, updates);
  b->mode = NPBGB_BATCH_PERSISTENT;
  b->launch_tiles.clear();
  int per_sm = 0;
  const int ctas_per_sm = int(g_cfg_batch_ctas_per_sm);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, persistent_kernel(ctas_per_sm), kBThreads, 0);
  if (per_sm <= 0) per_sm = 1;
  const int64_t slots = int64_t(sm_count()) * per_sm;
  const int nctas = int(std::max<int64_t>(1, std::min<int64_t>(slots, int64_t(bands.size()))));
  // Longest-processing-time greedy assignment of bands to CTAs by work.
  std::vector<std::vector<int32_t>> lists(static_cast<size_t>(nctas));
  {
    std::vector<int32_t> order(bands.size());
    for (size_t i = 0; i < order.size(); ++i) order[i] = int32_t(i);
    auto work = [&](int32_t i) { return band_work(bands[size_t(i)]); };
    std::stable_sort(order.begin(), order.end(), [&](int32_t x, int32_t y) { return work(x) > work(y); });
    using Item = std::pair<double, int>;
    std::priority_queue<Item, std::vector<Item>, std::greater<Item>> heap;
    for (int c = 0; c < nctas; ++c) heap.push({0.0, c});
    for (int32_t i : order) {
      Item it = heap.top();
      heap.pop();
      lists[size_t(it.second)].push_back(i);
      heap.push({it.first + work(i), it.second});
    }
  }
  std::vector<int32_t> off(static_cast<size_t>(nctas) + 1, 0), flat;
  flat.reserve(bands.size());
  for (int c = 0; c < nctas; ++c) {
    off[size_t(c)] = int32_t(flat.size());
    flat.insert(flat.end(), lists[size_t(c)].begin(), lists[size_t(c)].end());
  }
  off[size_t(nctas)] = int32_t(flat.size());

  cudaError_t e;
  const int64_t need_bands = std::max<int64_t>(1, int64_t(bands.size()));
  if (need_bands > b->cap_bands) {
    cudaFree(b->d_bands);
    cudaFree(b->d_done);
    cudaFree(b->d_cta_bands);
    b->d_bands = nullptr;
    b->d_done = nullptr;
    b->d_cta_bands = nullptr;
    b->cap_bands = 0;
    if ((e = cudaMalloc(&b->d_bands, sizeof(BandDesc) * size_t(need_bands))) != cudaSuccess ||
        (e = cudaMalloc(&b->d_done, sizeof(uint32_t) * size_t(need_bands))) != cudaSuccess ||
        (e = cudaMalloc(&b->d_cta_bands, sizeof(int32_t) * size_t(need_bands))) != cudaSuccess)
      return cuda_status(e, "batch: alloc");
    b->cap_bands = need_bands;
  }
  if (int64_t(off.size()) > b->cap_ctas) {
    cudaFree(b->d_cta_off);
    b->d_cta_off = nullptr;
    b->cap_ctas = 0;
    if ((e = cudaMalloc(&b->d_cta_off, sizeof(int32_t) * off.size())) != cudaSuccess)
      return cuda_status(e, "batch: alloc");
    b->cap_ctas = int64_t(off.size());
  }
  if (!bands.empty()) {
    if ((e = cudaMemcpy(b->d_bands, bands.data(), sizeof(BandDesc) * bands.size(), cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemcpy(b->d_cta_bands, flat.data(), sizeof(int32_t) * flat.size(), cudaMemcpyHostToDevice)) != cudaSuccess)
      return cuda_status(e, "batch: upload");
  }
  if ((e = cudaMemcpy(b->d_cta_off, off.data(), sizeof(int32_t) * off.size(), cudaMemcpyHostToDevice)) != cudaSuccess)
    return cuda_status(e, "batch: upload");
  b->nbands = int64_t(bands.size());
  b->updates = updates;
  b->nctas = nctas;
  b->ctas_per_sm = ctas_per_sm;
  return NPBGB_OK;
}

}  // namespace

extern "C" {

int32_t npbgb_batch_create(const npbgb_grid* grids, int64_t count, int32_t band_rows,
                           npbgb_batch** out) {
  using namespace npbgb;
  if (!out) return set_error(NPBGB_ERR_ARG, "batch: null output");
  *out = nullptr;
  auto* b = new (std::nothrow) npbgb_batch();
  if (!b) return set_error(NPBGB_ERR_NOMEM, "batch: host allocation");
  cudaGetDevice(&b->device);
  const int32_t r = plan_into(b, grids, count, band_rows);
  if (r != NPBGB_OK) {
    free_batch(b);
    return r;
  }
  *out = b;
  return NPBGB_OK;
}

int32_t npbgb_batch_replan(npbgb_batch* b, const npbgb_grid* grids, int64_t count, int32_t band_rows) {
  using namespace npbgb;
  if (!b) return set_error(NPBGB_ERR_ARG, "batch: null handle");
  return plan_into(b, grids, count, band_rows);
}

int32_t npbgb_batch_launch(npbgb_batch* b, int32_t use_graph, void* stream) {
  using namespace npbgb;
  if (!b) return set_error(NPBGB_ERR_ARG, "batch: null handle");
  if (b->nbands == 0) return NPBGB_OK;
  cudaStream_t st = as_stream(stream);
  if (!use_graph) return launch_batch(b, st);
  if (!b->graph) {
    cudaStream_t cap;
    cudaError_t e = cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking);
    if (e != cudaSuccess) return cuda_status(e, "batch: capture stream");
    e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) {
      cudaStreamDestroy(cap);
      return cuda_status(e, "batch: begin capture");
    }
    const int64_t before = add_launches(0);
    const int32_t r = launch_batch(b, cap);
    const int64_t recorded = add_launches(0) - before;
    add_launches(-recorded);  // counted at each replay instead
    b->graph_kernels = recorded;
    cudaGraph_t graph = nullptr;
    e = cudaStreamEndCapture(cap, &graph);
    cudaStreamDestroy(cap);
    if (r != NPBGB_OK) {
      if (graph) cudaGraphDestroy(graph);
      return r;
    }
    if (e != cudaSuccess) return cuda_status(e, "batch: end capture");
    e = cudaGraphInstantiate(&b->graph, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
      b->graph = nullptr;
      return cuda_status(e, "batch: instantiate graph");
    }
  }
  cudaError_t e = cudaGraphLaunch(b->graph, st);
  if (e != cudaSuccess) return cuda_status(e, "batch: graph launch");
  add_launches(b->graph_kernels);
  return NPBGB_OK;
}

int32_t npbgb_batch_info(const npbgb_batch* b, int64_t* nbands, int64_t* nctas, int64_t* updates) {
  using namespace npbgb;
  if (!b) return set_error(NPBGB_ERR_ARG, "batch: null handle");
  if (nbands) *nbands = b->nbands;
  if (nctas) *nctas = b->nctas;
  if (updates) *updates = b->updates;
  return NPBGB_OK;
}

int32_t npbgb_batch_mode(const npbgb_batch* b, int32_t* mode) {
  using namespace npbgb;
  if (!b || !mode) return set_error(NPBGB_ERR_ARG, "batch: null handle or output");
  *mode = b->mode;
  return NPBGB_OK;
}

int32_t npbgb_batch_destroy(npbgb_batch* b) {
  free_batch(b);
  return NPBGB_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Batches without allocation
// ---------------------------------------------------------------------------
// npbgb_batch_run_noalloc serves callers that must not allocate device
// memory: for example a host that owns every byte of the GPU through its own
// pool or an HBM admission budget, where a cudaMalloc behind its back would
// break the accounting or fail against a full pool, or a loop that cannot
// afford the implicit device synchronisation of cudaMalloc/cudaFree.  It runs
// the same persistent batch kernel, but its band table, CTA lists and step
// counters live in one file-scope __device__ array of fixed size instead of
// memory from cudaMalloc.  Nothing on its path allocates: host-side planning
// uses fixed static buffers, and the plan reaches the device by copies into
// that array.
namespace {

constexpr int kNoAllocMaxBands = 32768;  // bands per call (about 2.1 MB of scratch)
constexpr int kNoAllocMaxCtas = 2048;

struct NoAllocLayout {
  npbgb::BandDesc bands[kNoAllocMaxBands];
  uint32_t done[kNoAllocMaxBands];
  int32_t cta_off[kNoAllocMaxCtas + 1];
  int32_t cta_bands[kNoAllocMaxBands];
};

// Device scratch shared by every call on a device; it keeps the last call's
// contents.  In host code this name is only a stand-in for the symbol, not a
// device address: npbgb_batch_run_noalloc looks the address up with
// cudaGetSymbolAddress once per device and passes that pointer to the kernel.
static __device__ __align__(256) unsigned char g_noalloc_scratch[sizeof(NoAllocLayout)];

struct NoAllocDevice {
  NoAllocLayout* scratch = nullptr;  // device address of g_noalloc_scratch
  int slots = 0;                     // co-resident CTAs of batch_persistent
};
constexpr int kNoAllocMaxDevices = 64;
NoAllocDevice g_noalloc_devices[kNoAllocMaxDevices];
std::mutex g_noalloc_mutex;

// Host staging for the plan (static: the call allocates nothing).
npbgb::BandDesc g_na_bands[kNoAllocMaxBands];
double g_na_work[kNoAllocMaxBands];
int32_t g_na_order[kNoAllocMaxBands];
int32_t g_na_cta_of[kNoAllocMaxBands];
int32_t g_na_cta_bands[kNoAllocMaxBands];
int32_t g_na_cta_off[kNoAllocMaxCtas + 1];
int32_t g_na_fill[kNoAllocMaxCtas];
std::pair<double, int32_t> g_na_heap[kNoAllocMaxCtas];

}  // namespace

extern "C" int32_t npbgb_batch_run_noalloc(const npbgb_grid* grids, int64_t count, int32_t band_rows,
                                           void* stream) {
  using namespace npbgb;
  if (count < 0 || (count > 0 && !grids)) return set_error(NPBGB_ERR_ARG, "batch(no-alloc): bad grid list");
  if (band_rows < 0) return set_error(NPBGB_ERR_ARG, "batch(no-alloc): band_rows < 0");
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);

  // Plan the bands exactly as npbgb_batch_create does, into static buffers.
  int nb = 0;
  for (int64_t g = 0; g < count; ++g) {
    int64_t nbg = 0, up = 0;
    bool overflow = false;
    const int32_t r = plan_grid(grids[g], g, band_rows, nb, &nbg, &up,
                                [&](const BandDesc& d) {
                                  if (nb >= kNoAllocMaxBands) { overflow = true; return; }
                                  g_na_bands[nb] = d;
                                  g_na_work[nb] = band_work(d);
                                  g_na_order[nb] = nb;
                                  ++nb;
                                },
                                false);
    if (r != NPBGB_OK) return r;
    if (overflow)
      return set_error(NPBGB_ERR_NOMEM,
                       "batch(no-alloc): more than %d bands (its fixed scratch capacity); use "
                       "larger band_rows, fewer grids, or npbgb_batch_create",
                       kNoAllocMaxBands);
  }
  if (nb == 0) return NPBGB_OK;

  // The plan is staged from the shared static host buffers above, so a
  // captured copy would replay whatever a later call left there: refuse.
  cudaStream_t st = as_stream(stream);
  cudaStreamCaptureStatus capturing = cudaStreamCaptureStatusNone;
  cudaError_t e = cudaStreamIsCapturing(st, &capturing);
  if (e != cudaSuccess) return cuda_status(e, "batch(no-alloc): stream state");
  if (capturing != cudaStreamCaptureStatusNone)
    return set_error(NPBGB_ERR_ARG,
                     "batch(no-alloc): the stream is capturing a graph; this entry point stages "
                     "its plan from shared host buffers and cannot be captured");

  // Once per device, with that device current: the scratch symbol's address
  // and the co-resident CTA count of that device.
  int dev = 0;
  e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_status(e, "batch(no-alloc): current device");
  if (dev < 0 || dev >= kNoAllocMaxDevices) return set_error(NPBGB_ERR_ARG, "batch(no-alloc): device %d", dev);
  NoAllocDevice& D = g_noalloc_devices[dev];
  if (!D.scratch) {
    void* ptr = nullptr;
    e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_status(e, "batch(no-alloc): cudaGetSymbolAddress");
    int per_sm = 0, sms = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batch_persistent<2>, kBThreads, 0);
    if (e != cudaSuccess) return cuda_status(e, "batch(no-alloc): occupancy");
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return cuda_status(e, "batch(no-alloc): SM count");
    D.slots = std::max(1, per_sm) * std::max(1, sms);
    D.scratch = static_cast<NoAllocLayout*>(ptr);
  }

  // Longest-processing-time greedy assignment, as npbgb_batch_create.
  const int nctas = std::max(1, std::min({D.slots, nb, kNoAllocMaxCtas}));
  std::sort(g_na_order, g_na_order + nb, [](int32_t x, int32_t y) {
    return g_na_work[x] > g_na_work[y] || (g_na_work[x] == g_na_work[y] && x < y);
  });
  auto later = [](const std::pair<double, int32_t>& x, const std::pair<double, int32_t>& y) { return x > y; };
  for (int c = 0; c < nctas; ++c) g_na_heap[c] = {0.0, c};
  std::make_heap(g_na_heap, g_na_heap + nctas, later);
  for (int c = 0; c < nctas; ++c) g_na_fill[c] = 0;
  for (int n = 0; n < nb; ++n) {
    const int32_t band = g_na_order[n];
    std::pop_heap(g_na_heap, g_na_heap + nctas, later);
    std::pair<double, int32_t>& top = g_na_heap[nctas - 1];
    g_na_cta_of[band] = top.second;
    ++g_na_fill[top.second];
    top.first += g_na_work[band];
    std::push_heap(g_na_heap, g_na_heap + nctas, later);
  }
  g_na_cta_off[0] = 0;
  for (int c = 0; c < nctas; ++c) {
    g_na_cta_off[c + 1] = g_na_cta_off[c] + g_na_fill[c];
    g_na_fill[c] = g_na_cta_off[c];
  }
  for (int n = 0; n < nb; ++n) {
    const int32_t band = g_na_order[n];
    g_na_cta_bands[g_na_fill[g_na_cta_of[band]]++] = band;
  }

  // Upload the plan, clear the counters (they must start at zero), launch.
  NoAllocLayout* S = D.scratch;
  if ((e = cudaMemcpyAsync(S->bands, g_na_bands, sizeof(BandDesc) * size_t(nb), cudaMemcpyHostToDevice, st)) != cudaSuccess ||
      (e = cudaMemcpyAsync(S->cta_off, g_na_cta_off, sizeof(int32_t) * size_t(nctas + 1), cudaMemcpyHostToDevice, st)) != cudaSuccess ||
      (e = cudaMemcpyAsync(S->cta_bands, g_na_cta_bands, sizeof(int32_t) * size_t(nb), cudaMemcpyHostToDevice, st)) != cudaSuccess ||
      (e = cudaMemsetAsync(S->done, 0, sizeof(uint32_t) * size_t(nb), st)) != cudaSuccess)
    return cuda_status(e, "batch(no-alloc): upload plan");
  const BandDesc* d_bands = S->bands;
  uint32_t* d_done = S->done;
  const int32_t* d_cta_off = S->cta_off;
  const int32_t* d_cta_bands = S->cta_bands;
  int f64_emul = int(g_cfg_f64_emulation);
  int hw_warps = jacobi_hw_warps();
  uint32_t one = 1;
  void* args[] = {&d_bands, &d_done, &d_cta_off, &d_cta_bands, &f64_emul, &hw_warps, &one};
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(unsigned(nctas));
  cfg.blockDim = dim3(kBThreads);
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  e = counted(cudaLaunchKernelExC(&cfg, reinterpret_cast<const void*>(batch_persistent<2>), args));
  if (e != cudaSuccess) return cuda_status(e, "batch(no-alloc): cooperative launch");
  return NPBGB_OK;
}
