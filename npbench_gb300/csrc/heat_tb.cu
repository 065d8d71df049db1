// Heat-3D binary32 with temporal blocking: two half-sweeps per launch.
//
// The reference's loop (polybench/heat_3d/heat_3d_numpy.py:6-20) alternates
// A -> B and B -> A.  Binary32 Heat-3D is bound by HBM traffic, not by
// arithmetic, so this kernel reads the field at step t once and writes the
// field at step t+2, keeping step t+1 in shared memory:
//
//   * a CTA owns a 32 x 32 tile of the (axis 1, axis 2) plane and streams
//     along axis 0 over a chunk of planes;
//   * each input plane tile arrives with a halo of two by one TMA copy
//     (cp.async.bulk.tensor, 40 x 36 box whose x origin is rounded down to a
//     16-byte boundary) into a ring of shared buffers tracked by mbarriers;
//   * step t+1 is evaluated on the tile plus a halo of one (34 x 34) into a
//     four-plane ring in shared memory, step t+2 on the tile from three of
//     those planes, and only step t+2 goes to global memory.
//
// Every point is evaluated with the reference's operators in its order
// (heat_core.cuh), so each step's values are those of the single-step kernel
// bit for bit; the halo points of step t+1 are merely evaluated twice, by
// neighbouring CTAs.
//
// Step t+2 cannot be written over step t in place (neighbouring CTAs still
// read step t around their tiles), so the even steps alternate between A and
// a scratch array W, initialised as a copy of A (its faces are A's faces,
// which the even steps keep).  Faces are never written; the faces of the odd
// step t+1 are B's, read from B.  The call arranges the launches so that the
// last two half-sweeps are ordinary single-step ones, A -> B -> A: A ends with
// the newest field and B with the previous one, as in the reference.
#include <cuda.h>

#include <mutex>

#include "heat_core.cuh"
#include "npbgb_common.cuh"
#include "tma.cuh"

namespace npbgb {

extern int64_t g_cfg_heat_tb_chunk;

namespace {

constexpr int kTile = 32;             // output tile, both axes
constexpr int kBoxX = 40;             // TMA box width (axis 2): 16-byte aligned origin
constexpr int kBoxY = kTile + 4;      // TMA box height (axis 1): halo of two
constexpr int kXOff = 5;              // tile column kk lives at box column kk + kXOff
constexpr int kYOff = 2;              // tile row jj lives at box row jj + kYOff
constexpr int kPlaneBytes = kBoxX * kBoxY * 4;                 // 5760
constexpr int kStageStride = (kPlaneBytes + 127) / 128 * 128;  // 5760
constexpr int kStages = 6;
constexpr int kS1 = kTile + 2;        // step t+1 region (34)
constexpr int kS1Pitch = 36;          // row pitch of a step t+1 plane
constexpr int kS1Planes = 4;
constexpr int kThreads = 256;
constexpr size_t kSmemBytes = size_t(kStages) * kStageStride +
                              size_t(kS1Planes) * kS1 * kS1Pitch * 4 + kStages * 8;

__device__ unsigned int g_heat_tb_error;  // bit 0: an mbarrier wait timed out

__global__ void __launch_bounds__(kThreads)
heat3d_tb2(const __grid_constant__ CUtensorMap src_map, const float* __restrict__ odd_faces,
           float* __restrict__ dst, int64_t n0, int64_t n1, int64_t n2, int chunk) {
  pdl_begin();
  extern __shared__ __align__(128) unsigned char smem[];
  float* s1 = reinterpret_cast<float*>(smem + kStages * kStageStride);
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + kStages * kStageStride +
                                               kS1Planes * kS1 * kS1Pitch * 4);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t k0 = 1 + int64_t(blockIdx.x) * kTile, j0 = 1 + int64_t(blockIdx.y) * kTile;
  const int64_t ib = 1 + int64_t(blockIdx.z) * chunk;
  const int64_t ie = (ib + chunk < n0 - 1) ? ib + chunk : n0 - 1;  // output planes [ib, ie)
  const int64_t qlo = ib - 2 > 0 ? ib - 2 : 0;                      // input planes [qlo, qhi]
  const int64_t qhi = ie + 1 < n0 - 1 ? ie + 1 : n0 - 1;
  const int nq = int(qhi - qlo + 1);
  const int64_t s0 = n1 * n2;
  // Box origin: x = k0 - kXOff = 32 * blockIdx.x - 4, a multiple of 4 floats
  // (16 bytes); y = j0 - kYOff (no alignment rule).  Coordinates below zero
  // or past the end read as zeros and are never used.
  const int x0 = int(k0) - kXOff, y0 = int(j0) - kYOff;

  auto stage = [&](int64_t q) -> const float* {
    return reinterpret_cast<const float*>(smem + int((q - qlo) % kStages) * kStageStride);
  };
  int64_t issued = qlo;  // next plane to issue (thread 0 issues them, in order)
  auto issue = [&](int64_t q) {
    const int st = int((q - qlo) % kStages);
    uint64_t* bar = &bars[st];
    tma::mbar_arrive_expect_tx(bar, kPlaneBytes);
    tma::load_3d(smem + st * kStageStride, &src_map, x0, y0, int(q), bar);
    issued = q + 1;
  };
  auto wait = [&](int64_t q) -> bool {
    const int r = int(q - qlo);
    return tma::mbar_wait(&bars[r % kStages], uint32_t((r / kStages) & 1));
  };
  auto s1p = [&](int64_t p) -> float* { return s1 + int(p & 3) * kS1 * kS1Pitch; };

  if (tid == 0) {
    for (int s = 0; s < kStages; ++s) tma::mbar_init(&bars[s], 1);
    tma::fence_mbar_init();
  }
  __syncthreads();
  if (tid == 0)
    for (int r = 0; r < nq && r < kStages; ++r) issue(qlo + r);

  // Faces of the odd step along axes 1 and 2 (only CTAs at the domain's edge).
  const bool edge = j0 - 1 == 0 || k0 - 1 == 0 || j0 + kTile + 1 > n1 - 1 || k0 + kTile + 1 > n2 - 1;
  int64_t waited = qlo - 1;  // input planes up to here have been waited for
  bool ok = true;

  // Step t+1 planes p = ib-1 .. ie; after each, step t+2 plane p-1.
  for (int64_t p = ib - 1; p <= ie; ++p) {
    float* out1 = s1p(p);
    if (p == 0 || p == n0 - 1) {
      // a face plane of the odd step: B's values, never written
      const float* fp = odd_faces + p * s0;
      for (int e = tid; e < kS1 * kS1; e += kThreads) {
        const int jj = e / kS1 - 1, kk = e % kS1 - 1;
        const int64_t j = j0 + jj, k = k0 + kk;
        out1[(jj + 1) * kS1Pitch + kk + 1] = (j < n1 && k < n2) ? __ldg(fp + j * n2 + k) : 0.0f;
      }
    } else {
      while (waited < p + 1 && ok) {
        ++waited;
        ok = wait(waited);
      }
      if (ok) {
        const float* pm = stage(p - 1);
        const float* pc = stage(p);
        const float* pn = stage(p + 1);
        // main 32 x 32: warp rows 4w .. 4w+3, lane = column; rows in packed pairs
#pragma unroll
        for (int r = 0; r < 4; r += 2) {
          const int jj = warp * 4 + r, kk = lane;
          const int o = (jj + kYOff) * kBoxX + kk + kXOff;
          const F2 v = hcore::heat_point2(f2(pc[o], pc[o + kBoxX]), f2(pn[o], pn[o + kBoxX]),
                                          f2(pm[o], pm[o + kBoxX]),
                                          f2(pc[o + kBoxX], pc[o + 2 * kBoxX]),
                                          f2(pc[o - kBoxX], pc[o]), f2(pc[o + 1], pc[o + 1 + kBoxX]),
                                          f2(pc[o - 1], pc[o - 1 + kBoxX]));
          out1[(jj + 1) * kS1Pitch + kk + 1] = f2x(v);
          out1[(jj + 2) * kS1Pitch + kk + 1] = f2y(v);
        }
        // the ring around it: rows -1 and 32 (34 each), columns -1 and 32 (32 each)
        if (tid < 132) {
          int jj, kk;
          if (tid < 68) {
            jj = tid < 34 ? -1 : kTile;
            kk = (tid % 34) - 1;
          } else {
            const int t = tid - 68;
            kk = t < 32 ? -1 : kTile;
            jj = t % 32;
          }
          const int o = (jj + kYOff) * kBoxX + kk + kXOff;
          out1[(jj + 1) * kS1Pitch + kk + 1] =
              hcore::heat_point<float>(pc[o], pn[o], pm[o], pc[o + kBoxX], pc[o - kBoxX], pc[o + 1],
                                pc[o - 1]);
        }
        if (edge) {
          // Cells of the odd step on a face along axis 1 or 2 keep B's value;
          // this CTA's own evaluations there must not be used.  Each thread
          // fixes the cells it wrote above.
          const float* fp = odd_faces + p * s0;
          auto fix = [&](int jj, int kk) {
            const int64_t j = j0 + jj, k = k0 + kk;
            if (j < n1 && k < n2 && (j == 0 || k == 0 || j == n1 - 1 || k == n2 - 1))
              out1[(jj + 1) * kS1Pitch + kk + 1] = __ldg(fp + j * n2 + k);
          };
          for (int r = 0; r < 4; ++r) fix(warp * 4 + r, lane);
          if (tid < 132) {
            int jj, kk;
            if (tid < 68) {
              jj = tid < 34 ? -1 : kTile;
              kk = (tid % 34) - 1;
            } else {
              const int t = tid - 68;
              kk = t < 32 ? -1 : kTile;
              jj = t % 32;
            }
            fix(jj, kk);
          }
        }
      }
    }
    tma::fence_proxy_async();  // this thread's reads of the stage before it is refilled
    if (__syncthreads_or(!ok)) {
      if (tid == 0) {
        atomicOr(&g_heat_tb_error, 1u);
        // let the copies still in flight (the late one included) land, bounded, before exit
        for (int64_t q = ok ? waited + 1 : waited; q < issued; ++q) {
          const int r = int(q - qlo);
          tma::mbar_wait_for(&bars[r % kStages], uint32_t((r / kStages) & 1), tma::kWaitLimitNs / 16);
        }
      }
      return;
    }
    // Input plane p-1 is no longer needed: refill its buffer kStages planes on.
    if (tid == 0 && p - 1 >= qlo && p - 1 + kStages <= qhi) issue(p - 1 + kStages);
    // Step t+2, plane p-1, from step t+1 planes p-2, p-1, p.
    const int64_t o = p - 1;
    if (o >= ib) {
      const float* qm = s1p(o - 1);
      const float* qc = s1p(o);
      const float* qn = s1p(o + 1);
      const int kk = lane;
      const int64_t k = k0 + kk;
#pragma unroll
      for (int r = 0; r < 4; r += 2) {
        const int jj = warp * 4 + r;
        const int c = (jj + 1) * kS1Pitch + kk + 1;
        const F2 v = hcore::heat_point2(f2(qc[c], qc[c + kS1Pitch]), f2(qn[c], qn[c + kS1Pitch]),
                                        f2(qm[c], qm[c + kS1Pitch]),
                                        f2(qc[c + kS1Pitch], qc[c + 2 * kS1Pitch]),
                                        f2(qc[c - kS1Pitch], qc[c]), f2(qc[c + 1], qc[c + 1 + kS1Pitch]),
                                        f2(qc[c - 1], qc[c - 1 + kS1Pitch]));
        const int64_t j = j0 + jj;
        if (k < n2 - 1) {
          if (j < n1 - 1) dst[o * s0 + j * n2 + k] = f2x(v);
          if (j + 1 < n1 - 1) dst[o * s0 + (j + 1) * n2 + k] = f2y(v);
        }
      }
    }
  }
}

// A stream-ordered pool per device for the scratch array, keeping its memory
// between calls (release threshold at the maximum).
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

}  // namespace

// Runs 2*(tsteps-1) half-sweeps of binary32 Heat-3D with two per launch
// where it can.  Returns NPBGB_ERR_STATE when the arrays do not meet the TMA
// rules (the caller then uses the single-step kernels), or a status.
// single_pair(a, b) must queue one single-step half-sweep pair A -> B -> A.
int32_t heat3d_tb2_run(float* a, float* b, int64_t n0, int64_t n1, int64_t n2, int32_t tsteps,
                       cudaStream_t st, int32_t (*single_pairs)(float*, float*, int64_t, int64_t,
                                                                int64_t, int32_t, cudaStream_t)) {
  if (tsteps < 4 || n0 < 3 || n1 < 3 || n2 < 3) return NPBGB_ERR_STATE;
  const uint64_t bytes = uint64_t(n0) * n1 * n2 * 4;
  if (reinterpret_cast<uintptr_t>(a) % 16 || (n2 * 4) % 16) return NPBGB_ERR_STATE;
  // Pairs done by the single-step kernels: the last one, and one at the start
  // when the number of two-step launches would otherwise be odd.
  const int32_t m2 = tsteps - 2;                 // two-step launches, if even
  const bool lead = (m2 % 2) != 0;
  const int32_t launches = lead ? m2 - 1 : m2;   // even
  float* w = nullptr;
  cudaMemPool_t pool;
  cudaError_t e = scratch_pool(&pool);
  if (e == cudaSuccess) e = cudaMallocFromPoolAsync(reinterpret_cast<void**>(&w), bytes, pool, st);
  if (e != cudaSuccess) return cuda_status(e, "heat3d_tb2: scratch");
  CUtensorMap map_a, map_w;
  const uint64_t dims[3] = {uint64_t(n2), uint64_t(n1), uint64_t(n0)};
  const uint32_t box[3] = {uint32_t(kBoxX), uint32_t(kBoxY), 1u};
  if (tma::encode_3d(&map_a, 4, a, dims, box) != cudaSuccess ||
      tma::encode_3d(&map_w, 4, w, dims, box) != cudaSuccess) {
    cudaFreeAsync(w, st);
    return NPBGB_ERR_STATE;
  }
  static bool attr_done = false;
  if (!attr_done) {
    e = cudaFuncSetAttribute(heat3d_tb2, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kSmemBytes));
    if (e != cudaSuccess) {
      cudaFreeAsync(w, st);
      return cuda_status(e, "heat3d_tb2: smem attribute");
    }
    attr_done = true;
  }
  int32_t r = NPBGB_OK;
  if (lead) r = single_pairs(a, b, n0, n1, n2, 2, st);  // A -> B -> A
  if (r == NPBGB_OK) {
    e = cudaMemcpyAsync(w, a, bytes, cudaMemcpyDeviceToDevice, st);  // W's faces = A's faces
    if (e != cudaSuccess) r = cuda_status(e, "heat3d_tb2: scratch copy");
  }
  if (r == NPBGB_OK) {
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, heat3d_tb2, kThreads, kSmemBytes);
    const int64_t gx = cdiv(n2 - 2, kTile), gy = cdiv(n1 - 2, kTile);
    int chunk = int(g_cfg_heat_tb_chunk);
    if (chunk <= 0) {
      // about 4 waves of CTAs; at least 16 planes (the pipeline reloads 4 halo planes)
      const int64_t slots = int64_t(sm_count()) * (per_sm > 0 ? per_sm : 1);
      int64_t chunks = cdiv(4 * slots, gx * gy);
      int64_t c = cdiv(n0 - 2, chunks > 0 ? chunks : 1);
      if (c < 16) c = 16;
      if (c > n0 - 2) c = n0 - 2;
      chunk = int(c);
    }
    const int64_t gz = cdiv(n0 - 2, chunk);
    if (gy > 65535 || gz > 65535 || gx > 0x7fffffff) {
      r = set_error(NPBGB_ERR_ARG, "heat3d: extent too large");
    } else {
      const dim3 grid{unsigned(gx), unsigned(gy), unsigned(gz)};
      for (int32_t s = 0; s < launches && e == cudaSuccess; s += 2) {
        e = launch_chained(heat3d_tb2, grid, dim3{kThreads}, kSmemBytes, st, map_a,
                           static_cast<const float*>(b), w, n0, n1, n2, chunk);
        if (e == cudaSuccess)
          e = launch_chained(heat3d_tb2, grid, dim3{kThreads}, kSmemBytes, st, map_w,
                             static_cast<const float*>(b), a, n0, n1, n2, chunk);
      }
      if (e != cudaSuccess) r = cuda_status(e, "heat3d_tb2");
    }
  }
  cudaFreeAsync(w, st);
  if (r == NPBGB_OK) r = single_pairs(a, b, n0, n1, n2, 2, st);  // the last pair: A -> B -> A
  return r;
}

uint32_t take_heat_tb_device_error() {
  unsigned int v = 0, zero = 0;
  if (cudaMemcpyFromSymbol(&v, g_heat_tb_error, sizeof(v)) != cudaSuccess) return 0xffffffffu;
  if (v) cudaMemcpyToSymbol(g_heat_tb_error, &zero, sizeof(zero));
  return v;
}

}  // namespace npbgb
