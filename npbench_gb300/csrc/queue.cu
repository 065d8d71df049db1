// Device-side tile work queue: one persistent kernel that advances many
// independent Jacobi-2D and Heat-3D grids, fed while it runs.
//
// Work is cut into half-sweeps of grids ("segments") and each segment into
// tiles (Jacobi-2D: 8 warps x 32 columns x `chunk` rows; Heat-3D: a 32 x 8
// column tile streamed over `chunk` planes).  Segments sit in a ring in
// device memory.  Every CTA of the worker kernel loops:
//
//   claim  the next tiles of the segment at the ring's head: one 64-bit
//          fetch-and-add on the entry's claim word, whose high half is the
//          ring position (a claimer whose add lands on a recycled entry owns
//          the tiles it counted there, so every add is a valid claim);
//   sweep  that tile (the same per-point arithmetic as the single-grid
//          kernels, loads and stores through L2);
//   count  the tile into its grid's completion counter (acquire-release); the
//          CTA that completes the last tile of half-sweep s appends segment
//          s + 1 of that grid to the ring, or, after the grid's last
//          half-sweep, writes the grid's completion word.
//
// A segment is appended only once every tile of the grid's previous
// half-sweep is complete, which orders both read-after-write and
// write-after-read between the ping-pong buffers; tiles are claimed in ring
// order, so a claimed tile never waits on anything and the kernel needs no
// co-residency (plain launch, not cooperative).  A claim takes several tiles
// of a large segment at once (ntiles / (4 * CTAs), at least one).  Grids of
// different sizes, kinds and precisions interleave tile by tile, and a grid's
// next half-sweep starts as soon as its own previous one is done.
//
// Small grids (NPBGB_CFG_QUEUE_WHOLE_CELLS) run whole: their segments are one
// claimable unit, the claiming CTA sweeps every tile of the half-sweep and
// then runs on to the grid's next half-sweeps itself (a CTA barrier between
// them), up to kLocalRun, before it returns the grid to the ring.  A stream of
// many small grids then costs one claim per kLocalRun half-sweeps instead of
// one per tile, and its parallelism comes from the grids, one per CTA.
//
// New grids arrive through an inbox that the host may append to while the
// kernel runs: a descriptor table, a ring of slot indices and a published
// count, in host-mapped pinned memory, written by the host with release
// stores and read here with system-scope acquires.  An idle CTA takes the
// inbox lock, copies new descriptors into the device slot table and appends
// their first segments.  Completion words (the grid's residency number) are
// written to host-mapped memory with system-scope release stores; the host
// polls them, so no host synchronisation stands between arrivals and the
// running kernel.
//
// The kernel ends when nothing is outstanding and the inbox is closed, or
// has stayed empty for `idle_ns`; the host launches it again when new grids
// arrive.  Every wait is bounded: with work outstanding, a ring whose head and
// tail stay unchanged for kQueueLimitNs sets an error word and the kernel ends.
//
// Per point the arithmetic is that of jacobi2d.cu / heat3d.cu (bit-identical
// to polybench/jacobi_2d/jacobi_2d_numpy.py:6-10 and
// polybench/heat_3d/heat_3d_numpy.py:6-20), binary64 fixed-point paths
// included.
#include <algorithm>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

#include "heat_core.cuh"
#include "jacobi_core.cuh"
#include "npbgb_common.cuh"
#include "queue.cuh"
#include "tma.cuh"

namespace npbgb {

extern int64_t g_cfg_queue_whole_cells;

extern int64_t g_cfg_f64_emulation;

namespace {

using namespace qdev;

constexpr int kQWarps = 8;
constexpr int kQThreads = 32 * kQWarps;
constexpr uint64_t kQueueLimitNs = 2000000000ull;  // two seconds without the ring moving

__device__ unsigned int g_queue_error;  // any launch's error bits, for npbgb_device_status

__device__ __forceinline__ uint32_t ld_acq_gpu(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ uint32_t ld_acq_sys(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.acquire.sys.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ uint32_t ld_rlx_gpu(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ int32_t ld_rlx_gpu(const int32_t* p) {
  return int32_t(ld_rlx_gpu(reinterpret_cast<const uint32_t*>(p)));
}
__device__ __forceinline__ uint32_t ld_rlx_sys(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.relaxed.sys.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ uint64_t ld_rlx_gpu64(const unsigned long long* p) {
  uint64_t v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ uint64_t ld_rlx_sys64(const uint64_t* p) {
  uint64_t v;
  asm volatile("ld.relaxed.sys.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_rlx_gpu64(unsigned long long* p, uint64_t v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ void st_rel_gpu(uint32_t* p, uint32_t v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void st_rel_sys(uint32_t* p, uint32_t v) {
  asm volatile("st.release.sys.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ uint32_t atom_add_acq_rel(uint32_t* p, uint32_t v) {
  uint32_t old;
  asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
  return old;
}
__device__ __forceinline__ uint32_t atom_cas_acq(uint32_t* p, uint32_t cmp, uint32_t v) {
  uint32_t old;
  asm volatile("atom.acquire.gpu.global.cas.b32 %0, [%1], %2, %3;"
               : "=r"(old) : "l"(p), "r"(cmp), "r"(v) : "memory");
  return old;
}

// Appends segment (slot, s) of `ntiles` tiles.  The claim word is written
// before the entry's sequence number is published with a release store.
__device__ void produce(const QArgs& q, int32_t slot, int32_t s, int32_t ntiles) {
  const uint32_t p = atomicAdd(&q.st->tail, 1u);
  QSeg* e = &q.ring[p % q.ring_size];
  volatile QSeg* ve = e;
  ve->slot = slot;
  ve->s = s;
  ve->ntiles = ntiles;
  st_rlx_gpu64(&q.claim[p % q.ring_size], uint64_t(p) << 32);
  st_rel_gpu(&e->seq, p);
}

// Under the inbox lock: moves new inbox entries into the slot table and
// appends their first segments.  Returns true if it activated any.
__device__ bool activate(const QArgs& q) {
  const uint32_t published = ld_acq_sys(&q.inbox_ctl[0]);
  if (ld_rlx_gpu(&q.st->inbox_head) == published) return false;
  if (atom_cas_acq(&q.st->lock, 0u, 1u) != 0u) return false;
  bool did = false;
  if (!ld_rlx_gpu(&q.st->shutdown)) {
    uint32_t ih = ld_rlx_gpu(&q.st->inbox_head);
    const uint32_t tail = ld_acq_sys(&q.inbox_ctl[0]);
    for (int n = 0; ih != tail && n < 64; ++n, ++ih) {
      const int32_t slot = int32_t(ld_rlx_sys(reinterpret_cast<const uint32_t*>(
          &q.inbox[ih % q.inbox_cap])));
      if (slot < 0 || slot >= q.max_slots) {
        atomicOr(&q.st->error, 2u);
        atomicOr(&g_queue_error, 2u);
        if (q.status_out) st_rel_sys(q.status_out, 2u);
        continue;
      }
      const uint64_t* src = reinterpret_cast<const uint64_t*>(q.host_slots + slot);
      uint64_t* dst = reinterpret_cast<uint64_t*>(q.slots + slot);
#pragma unroll
      for (int w = 0; w < int(sizeof(QSlot) / 8); ++w) {
        volatile uint64_t* vd = dst + w;
        *vd = ld_rlx_sys64(src + w);
      }
      volatile uint32_t* vdone = q.done + slot;
      *vdone = 0u;
      atomicAdd(&q.st->active, 1u);
      const int32_t units = ld_rlx_gpu(&q.slots[slot].whole) ? 1 : ld_rlx_gpu(&q.slots[slot].ntiles);
      produce(q, slot, 0, units);
      did = true;
    }
    st_rel_gpu(&q.st->inbox_head, ih);
    if (q.consumed_out) st_rel_sys(q.consumed_out, ih);
  }
  st_rel_gpu(&q.st->lock, 0u);
  return did;
}

// Under the inbox lock: ends the launch when no grid is active and the inbox
// holds nothing new.
__device__ bool try_shutdown(const QArgs& q) {
  if (atom_cas_acq(&q.st->lock, 0u, 1u) != 0u) return false;
  const bool quiet = ld_rlx_gpu(&q.st->inbox_head) == ld_acq_sys(&q.inbox_ctl[0]) &&
                     ld_acq_gpu(&q.st->active) == 0u;
  if (quiet) st_rel_gpu(&q.st->shutdown, 1u);
  st_rel_gpu(&q.st->lock, 0u);
  return quiet;
}

__device__ void record_error(const QArgs& q, uint32_t bits) {
  atomicOr(&q.st->error, bits);
  atomicOr(&g_queue_error, bits);
  st_rel_gpu(&q.st->shutdown, 1u);
  if (q.status_out) st_rel_sys(q.status_out, ld_rlx_gpu(&q.st->error));
}

struct Waiting {
  uint64_t idle_since = 0;   // 0: not idle
  uint64_t seen_t = 0;       // when (seen_h, seen_t) was last seen to change
  uint32_t seen_h = 0xffffffffu, seen_tail = 0xffffffffu;
};

struct Claim {
  int32_t slot = -1, s = 0, t0 = 0, t1 = 0;  // tiles [t0, t1) of half-sweep segment s
};

// Thread 0: the next tiles (slot >= 0), or slot = -1 when the launch ends.
__device__ void next_tiles(const QArgs& q, Claim* out, Waiting& w) {
  const uint32_t div = 4u * gridDim.x;
  for (;;) {
    const uint32_t h = ld_acq_gpu(&q.st->head);
    const uint32_t t = ld_acq_gpu(&q.st->tail);
    if (h != t) {
      QSeg* e = &q.ring[h % q.ring_size];
      const uint32_t seq = ld_acq_gpu(&e->seq);
      if (seq == h) {
        const int32_t nt = ld_rlx_gpu(&e->ntiles);
        const uint32_t per = max(1u, uint32_t(nt) / div);
        const uint64_t old = atomicAdd(&q.claim[h % q.ring_size], (unsigned long long)per);
        const uint32_t tag = uint32_t(old >> 32), n = uint32_t(old);
        if (tag == h) {
          if (n < uint32_t(nt)) {
            out->slot = ld_rlx_gpu(&e->slot);
            out->s = ld_rlx_gpu(&e->s);
            out->t0 = int32_t(n);
            out->t1 = int32_t(min(n + per, uint32_t(nt)));
            w.idle_since = 0;
            return;
          }
          atomicCAS(&q.st->head, h, h + 1u);  // exhausted: help the head along
          continue;
        }
        // The add landed on the entry recycled for position `tag` (> h): the
        // tiles [n, n + per) of that segment are this claimer's.  Its producer
        // wrote the claim word before publishing the entry; wait for that.
        QSeg* r = &q.ring[tag % q.ring_size];
        const uint64_t t_start = tma::globaltimer();
        for (;;) {
          const uint32_t rs = ld_acq_gpu(&r->seq);
          if (rs == tag) break;
          if ((rs != kSeqEmpty && int32_t(rs - tag) > 0) ||
              tma::globaltimer() - t_start > kQueueLimitNs) {
            // recycled again before this claim could be read, or never
            // published: both mean lost tiles; end with an error
            record_error(q, 1u);
            out->slot = -1;
            return;
          }
          __nanosleep(32);
        }
        const int32_t rn = ld_rlx_gpu(&r->ntiles);
        if (n < uint32_t(rn)) {
          out->slot = ld_rlx_gpu(&r->slot);
          out->s = ld_rlx_gpu(&r->s);
          out->t0 = int32_t(n);
          out->t1 = int32_t(min(n + per, uint32_t(rn)));
          w.idle_since = 0;
          return;
        }
        continue;
      }
      if (seq != kSeqEmpty && int32_t(seq - h) > 0) {  // stale head over a recycled entry
        atomicCAS(&q.st->head, h, h + 1u);
        continue;
      }
      // otherwise the producer of position h is still writing it
    }
    if (activate(q)) continue;
    const uint64_t now = tma::globaltimer();
    if (ld_acq_gpu(&q.st->shutdown)) {
      out->slot = -1;
      return;
    }
    const uint32_t active = ld_acq_gpu(&q.st->active);
    if (h != w.seen_h || t != w.seen_tail) {
      w.seen_h = h;
      w.seen_tail = t;
      w.seen_t = now;
    }
    if (active == 0u && h == t) {
      if (w.idle_since == 0) w.idle_since = now;
      const bool closed = ld_acq_sys(&q.inbox_ctl[1]) != 0u;
      if ((closed || now - w.idle_since > q.idle_ns) && try_shutdown(q)) {
        out->slot = -1;
        return;
      }
    } else {
      w.idle_since = 0;
      if (now - w.seen_t > kQueueLimitNs) {  // work outstanding, ring not moving
        record_error(q, 1u);
        out->slot = -1;
        return;
      }
    }
    __nanosleep(active ? 100 : 400);
  }
}

// Thread 0, after the CTA's barrier: counts the units (tiles, or whole
// segments) up to segment s and hands on the grid.
__device__ void complete_tiles(const QArgs& q, int32_t slot, int32_t s, int32_t count,
                               const QSlot& G) {
  // bar.sync ordered the CTA's stores before this release, which is cumulative.
  const uint32_t units = uint32_t(seg_units(G));
  const uint32_t old = atom_add_acq_rel(&q.done[slot], uint32_t(count));
  if (old + uint32_t(count) == uint32_t(s + 1) * units) {
    if (s + 1 < G.steps) {
      produce(q, slot, s + 1, int32_t(units));
    } else {
      if (q.finished) st_rel_sys(&q.finished[slot], G.gen);
      atomicSub(&q.st->active, 1u);
    }
  }
}

template <typename T, bool FX>
__device__ __forceinline__ void heat_tile(const QSlot& G, const void* src, void* dst, int64_t bx,
                                          int64_t rest, hcore::PlaneBuf<double, true>& plane) {
  const int64_t by = rest % G.ty, bz = rest / G.ty;
  const int64_t k0 = 1 + bx * hcore::kTK, j0 = 1 + by * hcore::kTJ;
  const int64_t ib = 1 + bz * G.chunk;
  const int64_t ie = min(ib + int64_t(G.chunk), int64_t(G.n0) - 1);
  hcore::tile_stream<T, FX, true>(static_cast<const T*>(src), static_cast<T*>(dst), G.n1, G.n2, j0,
                                  k0, ib, ie,
                                  reinterpret_cast<hcore::PlaneBuf<T, FX>&>(plane));
}

// Tile `tile` of a conversion segment: a contiguous share of both arrays,
// binary32 -> binary64 (exact) or binary64 -> binary32 (round to nearest even).
__device__ __forceinline__ void convert_tile(const QSlot& G, int32_t tile, bool widen) {
  const int64_t per = (G.cells + G.ntiles - 1) / G.ntiles;
  const int64_t i0 = int64_t(tile) * per;
  const int64_t i1 = min(i0 + per, G.cells);
  double* a = static_cast<double*>(G.a);
  double* b = static_cast<double*>(G.b);
  float* a32 = static_cast<float*>(G.a32);
  float* b32 = static_cast<float*>(G.b32);
  for (int64_t i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
    if (widen) {
      __stcg(a + i, double(__ldcg(a32 + i)));
      __stcg(b + i, double(__ldcg(b32 + i)));
    } else {
      __stcg(a32 + i, __double2float_rn(__ldcg(a + i)));
      __stcg(b32 + i, __double2float_rn(__ldcg(b + i)));
    }
  }
}

__device__ __forceinline__ void sweep_tile(const QArgs& q, const QSlot& G, int32_t seg, int32_t tile,
                                           hcore::PlaneBuf<double, true>& plane) {
  int32_t s = seg;  // half-sweep index
  if (G.conv) {
    if (seg == 0 || seg == G.steps - 1) {
      convert_tile(G, tile, seg == 0);
      return;
    }
    s = seg - 1;
  }
  const bool odd = ((G.step0 + s) & 1) != 0;
  const void* src = odd ? G.b : G.a;
  void* dst = odd ? G.a : G.b;
  const int64_t bx = tile % G.tx, rest = tile / G.tx;
  if (G.kind == NPBGB_KIND_HEAT3D) {
    if (G.dtype == NPBGB_F64) {
      if (q.f64_emulation)
        heat_tile<double, true>(G, src, dst, bx, rest, plane);
      else
        heat_tile<double, false>(G, src, dst, bx, rest, plane);
    } else {
      heat_tile<float, false>(G, src, dst, bx, rest, plane);
    }
    return;
  }
  const int warp = threadIdx.x >> 5;
  const int64_t k0 = 1 + (bx * kQWarps + warp) * 32;
  if (k0 >= int64_t(G.n1) - 1) return;  // warp-uniform; strips have no CTA barrier
  const int64_t ib = 1 + rest * G.chunk;
  const int64_t ie = min(ib + int64_t(G.chunk), int64_t(G.n0) - 1);
  if (G.dtype == NPBGB_F64) {
    const double* sp = static_cast<const double*>(src);
    double* dp = static_cast<double*>(dst);
    if (!q.f64_emulation || warp < q.hw_warps)
      jcore::strip_rows<double, false, true, 2>(sp, dp, G.n1, k0, ib, ie, q.one);
    else
      jcore::strip_rows<double, true, true, 2>(sp, dp, G.n1, k0, ib, ie, q.one);
  } else {
    jcore::strip_rows<float, false, true, 4>(static_cast<const float*>(src), static_cast<float*>(dst),
                                             G.n1, k0, ib, ie, q.one);
  }
}

template <int MINB>
__global__ void __launch_bounds__(kQThreads, MINB) queue_worker(const QArgs q) {
  __shared__ int32_t s_cmd[4];
  __shared__ __align__(16) QSlot s_slot;
  __shared__ hcore::PlaneBuf<double, true> plane;  // Heat-3D staging (largest element type)
  const int tid = threadIdx.x;
  Waiting w;
  for (;;) {
    if (tid == 0) {
      Claim c;
      next_tiles(q, &c, w);
      const int32_t slot = c.slot;
      s_cmd[0] = slot;
      s_cmd[1] = c.s;
      s_cmd[2] = c.t0;
      s_cmd[3] = c.t1;
      if (slot >= 0) {
        // The slot was written by the activating CTA before it published the
        // segment this thread acquired; read it through L2.
        const unsigned long long* src = reinterpret_cast<const unsigned long long*>(q.slots + slot);
        uint64_t* d = reinterpret_cast<uint64_t*>(&s_slot);
#pragma unroll
        for (int k = 0; k < int(sizeof(QSlot) / 8); ++k) d[k] = ld_rlx_gpu64(src + k);
      }
    }
    __syncthreads();
    const int32_t slot = s_cmd[0];
    if (slot < 0) return;
    const int32_t s = s_cmd[1], t0 = s_cmd[2], t1 = s_cmd[3];
    const QSlot G = s_slot;
    if (!G.whole) {
      for (int32_t tile = t0; tile < t1; ++tile) sweep_tile(q, G, s, tile, plane);
      __syncthreads();
      if (tid == 0) complete_tiles(q, slot, s, t1 - t0, G);
      continue;
    }
    // Whole-grid slot: this CTA owns the segment (its one unit), so it runs
    // the grid's next segments itself, a CTA barrier between consecutive
    // half-sweeps ordering them, and returns the grid to the ring after
    // kLocalRun segments or at its end.
    const int32_t end = min(G.steps, s + kLocalRun);
    for (int32_t s2 = s; s2 < end; ++s2) {
      if (s2 > s) __syncthreads();  // the previous half-sweep's stores before these loads
      for (int32_t tile = 0; tile < G.ntiles; ++tile) sweep_tile(q, G, s2, tile, plane);
    }
    __syncthreads();
    if (tid == 0) complete_tiles(q, slot, end - 1, end - s, G);
  }
}

using WorkerFn = void (*)(const QArgs);

WorkerFn worker_fn(int ctas_per_sm) {
  return ctas_per_sm >= 5   ? queue_worker<5>
         : ctas_per_sm == 4 ? queue_worker<4>
                            : (ctas_per_sm == 3 ? queue_worker<3> : queue_worker<2>);
}

}  // namespace

// Reads and clears the queue kernels' device error word (host; synchronises).
uint32_t take_queue_device_error() {
  unsigned int v = 0, zero = 0;
  if (cudaMemcpyFromSymbol(&v, g_queue_error, sizeof(v)) != cudaSuccess) return 0xffffffffu;
  if (v) cudaMemcpyToSymbol(g_queue_error, &zero, sizeof(zero));
  return v;
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
namespace qhost {

// target_tiles: tiles per half-sweep the automatic tile extent aims at (about
// the worker's CTA count, so that one grid alone still spreads over the GPU).
int32_t describe(const npbgb_grid& G, int64_t g, int32_t tile_rows, int32_t tile_planes,
                 QSlot* out, int64_t* updates, int64_t target_tiles) {
  *updates = 0;
  if (G.kind != NPBGB_KIND_JACOBI2D && G.kind != NPBGB_KIND_HEAT3D)
    return set_error(NPBGB_ERR_ARG, "queue: grid %lld: kind %d", (long long)g, G.kind);
  if (G.dtype != NPBGB_F64 && G.dtype != NPBGB_F32)
    return set_error(NPBGB_ERR_DTYPE, "queue: grid %lld: dtype %d", (long long)g, G.dtype);
  const bool heat = G.kind == NPBGB_KIND_HEAT3D;
  const int64_t n2 = heat ? G.n2 : 1;
  if (G.n0 < 0 || G.n1 < 0 || n2 < 0 || G.n0 > 0x7fffffff || G.n1 > 0x7fffffff || n2 > 0x7fffffff)
    return set_error(NPBGB_ERR_ARG, "queue: grid %lld: bad extents", (long long)g);
  if (G.step0 < 0 || G.nsteps < 0)
    return set_error(NPBGB_ERR_ARG, "queue: grid %lld: negative step0 or nsteps", (long long)g);
  const int64_t total = G.tsteps > 1 ? 2 * int64_t(G.tsteps - 1) : 0;
  int64_t todo = total - G.step0;
  if (G.nsteps > 0 && G.nsteps < todo) todo = G.nsteps;
  std::memset(out, 0, sizeof(QSlot));
  if (todo <= 0 || G.n0 < 3 || G.n1 < 3 || (heat && n2 < 3)) return NPBGB_OK;  // total = 0
  if (!G.a || !G.b || G.a == G.b)
    return set_error(NPBGB_ERR_ARG, "queue: grid %lld: null or aliased arrays", (long long)g);
  const bool conv = G.a32 || G.b32;
  if (conv && (!G.a32 || !G.b32 || G.a32 == G.b32 || G.dtype != NPBGB_F64 || G.a32 == G.a ||
               G.a32 == G.b || G.b32 == G.a || G.b32 == G.b))
    return set_error(NPBGB_ERR_ARG,
                     "queue: grid %lld: binary32 arrays need a binary64 grid and two distinct arrays",
                     (long long)g);
  out->a = G.a;
  out->b = G.b;
  out->n0 = int32_t(G.n0);
  out->n1 = int32_t(G.n1);
  out->n2 = int32_t(n2);
  out->kind = int16_t(G.kind);
  out->dtype = int16_t(G.dtype);
  out->a32 = G.a32;
  out->b32 = G.b32;
  out->step0 = G.step0;
  out->total = int32_t(todo);
  out->conv = conv ? 1 : 0;
  out->steps = int32_t(todo) + (conv ? 2 : 0);
  out->cells = G.n0 * G.n1 * n2;
  int64_t ntiles;
  const int64_t target = std::max<int64_t>(1, target_tiles);
  if (heat) {
    out->tx = int32_t(cdiv(n2 - 2, hcore::kTK));
    out->ty = int32_t(cdiv(G.n1 - 2, hcore::kTJ));
    // automatic: planes for about `target` tiles, 4 .. 64 (a tile streams them)
    const int64_t autoc = std::min<int64_t>(64, std::max<int64_t>(
        4, cdiv((G.n0 - 2) * out->tx * out->ty, target)));
    const int32_t c = G.band_rows > 0 ? G.band_rows : (tile_planes > 0 ? tile_planes : int32_t(autoc));
    out->chunk = c;
    ntiles = int64_t(out->tx) * out->ty * cdiv(G.n0 - 2, c);
  } else {
    out->tx = int32_t(cdiv(G.n1 - 2, 32 * kQWarps));
    out->ty = 1;
    // automatic: rows for about `target` tiles, 8 .. 256
    const int64_t autoc = std::min<int64_t>(256, std::max<int64_t>(
        8, cdiv((G.n0 - 2) * out->tx, target)));
    const int32_t c = G.band_rows > 0 ? G.band_rows : (tile_rows > 0 ? tile_rows : int32_t(autoc));
    out->chunk = c;
    ntiles = int64_t(out->tx) * cdiv(G.n0 - 2, c);
  }
  if (ntiles * (todo + 2) >= (int64_t(1) << 32))
    return set_error(NPBGB_ERR_ARG, "queue: grid %lld: more than 2^32 tiles in one run", (long long)g);
  out->ntiles = int32_t(ntiles);
  // Small grids run whole: one CTA per half-sweep, several half-sweeps in a
  // row, with no ring traffic in between (their tiles would each carry a
  // claim and a hand-off for very little arithmetic).
  out->whole = (g_cfg_queue_whole_cells > 0 && out->cells <= g_cfg_queue_whole_cells) ? 1 : 0;
  *updates = todo * (G.n0 - 2) * (G.n1 - 2) * (heat ? (n2 - 2) : 1);
  return NPBGB_OK;
}

// CTAs per SM a worker launch uses: the requested count, at most what fits.
int slots_per_sm(int ctas_per_sm, int* per_sm_out) {
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, worker_fn(ctas_per_sm), kQThreads, 0);
  if (per_sm <= 0) per_sm = 1;
  per_sm = std::min(per_sm, std::max(1, ctas_per_sm));
  if (per_sm_out) *per_sm_out = per_sm;
  return per_sm;
}

cudaError_t launch_worker(const QArgs& args, int nctas, int ctas_per_sm, cudaStream_t st) {
  worker_fn(ctas_per_sm)<<<dim3(unsigned(nctas)), dim3(kQThreads), 0, st>>>(args);
  return counted(cudaGetLastError());
}

}  // namespace qhost
}  // namespace npbgb

// ---------------------------------------------------------------------------
// Streaming queue (npbgb_queue_*)
// ---------------------------------------------------------------------------
struct npbgb_queue {
  int device = 0;
  int32_t max_slots = 0;
  uint32_t ring_size = 0, inbox_cap = 0;
  int32_t tile_rows = 0, tile_planes = 0, ctas_per_sm = 3;
  int64_t target_tiles = 1;
  uint64_t idle_ns = 0;
  // device memory
  npbgb::qdev::QSlot* d_slots = nullptr;
  npbgb::qdev::QSeg* d_ring = nullptr;
  unsigned long long* d_claim = nullptr;
  uint32_t* d_done = nullptr;
  npbgb::qdev::QState* d_state = nullptr;
  // host-mapped pinned memory (host pointers; the device uses the same addresses)
  npbgb::qdev::QSlot* h_slots = nullptr;
  int32_t* h_inbox = nullptr;
  uint32_t* h_ctl = nullptr;  // [0] published, [1] closed, [2] consumed, [3] status
  uint32_t* h_finished = nullptr;
  std::vector<uint32_t> gen;
  std::vector<uint8_t> busy;
  std::vector<int32_t> free_slots;
  uint32_t published = 0;
  cudaEvent_t done_ev = nullptr;
  bool launched = false;
  int64_t launches = 0;
  std::mutex mu;
};

namespace {

void free_queue(npbgb_queue* q) {
  if (!q) return;
  if (q->done_ev) cudaEventDestroy(q->done_ev);
  cudaFree(q->d_slots);
  cudaFree(q->d_ring);
  cudaFree(q->d_claim);
  cudaFree(q->d_done);
  cudaFree(q->d_state);
  cudaFreeHost(q->h_slots);
  cudaFreeHost(q->h_inbox);
  cudaFreeHost(q->h_ctl);
  cudaFreeHost(q->h_finished);
  delete q;
}

inline uint32_t load_acquire(const uint32_t* p) { return __atomic_load_n(p, __ATOMIC_ACQUIRE); }
inline void store_release(uint32_t* p, uint32_t v) { __atomic_store_n(p, v, __ATOMIC_RELEASE); }

// True while the worker launched last is still running.
bool running(npbgb_queue* q) {
  if (!q->launched) return false;
  if (cudaEventQuery(q->done_ev) == cudaErrorNotReady) return true;
  q->launched = false;
  return false;
}

npbgb::qdev::QArgs queue_args(npbgb_queue* q) {
  npbgb::qdev::QArgs a{};
  a.slots = q->d_slots;
  a.ring = q->d_ring;
  a.claim = q->d_claim;
  a.done = q->d_done;
  a.st = q->d_state;
  a.host_slots = q->h_slots;
  a.inbox = q->h_inbox;
  a.inbox_ctl = q->h_ctl;
  a.consumed_out = q->h_ctl + 2;
  a.status_out = q->h_ctl + 3;
  a.finished = q->h_finished;
  a.ring_size = q->ring_size;
  a.inbox_cap = q->inbox_cap;
  a.max_slots = q->max_slots;
  a.idle_ns = q->idle_ns;
  a.f64_emulation = int(npbgb::g_cfg_f64_emulation);
  a.hw_warps = npbgb::jacobi_hw_warps();
  a.one = 1u;
  return a;
}

}  // namespace

extern "C" {

int32_t npbgb_queue_create(int32_t max_slots, int32_t tile_rows, int32_t tile_planes,
                           int32_t ctas_per_sm, int64_t idle_us, npbgb_queue** out) {
  using namespace npbgb;
  if (!out) return set_error(NPBGB_ERR_ARG, "queue: null output");
  *out = nullptr;
  if (max_slots < 1 || max_slots > (1 << 20)) return set_error(NPBGB_ERR_ARG, "queue: max_slots");
  if (tile_rows < 0 || tile_planes < 0) return set_error(NPBGB_ERR_ARG, "queue: tile extents");
  if (ctas_per_sm < 0 || ctas_per_sm > 5) return set_error(NPBGB_ERR_ARG, "queue: ctas_per_sm");
  if (idle_us < 0 || idle_us > 10000000) return set_error(NPBGB_ERR_ARG, "queue: idle_us");
  auto* q = new (std::nothrow) npbgb_queue();
  if (!q) return set_error(NPBGB_ERR_NOMEM, "queue: host allocation");
  cudaGetDevice(&q->device);
  q->max_slots = max_slots;
  // Each active grid has at most one segment not yet exhausted, so twice the
  // slot count keeps a recycled entry exhausted before it is overwritten.
  q->ring_size = uint32_t(2 * max_slots + 2);
  q->inbox_cap = uint32_t(max_slots);
  q->tile_rows = tile_rows;
  q->tile_planes = tile_planes;
  q->ctas_per_sm = ctas_per_sm > 0 ? ctas_per_sm : 3;
  q->idle_ns = uint64_t(idle_us) * 1000ull;
  {
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, q->device);
    q->target_tiles = int64_t(std::max(1, sms)) * qhost::slots_per_sm(q->ctas_per_sm, nullptr);
  }
  cudaError_t e;
  const unsigned mapped = cudaHostAllocMapped | cudaHostAllocPortable;
  if ((e = cudaMalloc(&q->d_slots, sizeof(qdev::QSlot) * size_t(max_slots))) != cudaSuccess ||
      (e = cudaMalloc(&q->d_ring, sizeof(qdev::QSeg) * q->ring_size)) != cudaSuccess ||
      (e = cudaMalloc(&q->d_claim, sizeof(unsigned long long) * q->ring_size)) != cudaSuccess ||
      (e = cudaMalloc(&q->d_done, sizeof(uint32_t) * size_t(max_slots))) != cudaSuccess ||
      (e = cudaMalloc(&q->d_state, sizeof(qdev::QState))) != cudaSuccess ||
      (e = cudaHostAlloc(&q->h_slots, sizeof(qdev::QSlot) * size_t(max_slots), mapped)) != cudaSuccess ||
      (e = cudaHostAlloc(&q->h_inbox, sizeof(int32_t) * q->inbox_cap, mapped)) != cudaSuccess ||
      (e = cudaHostAlloc(&q->h_ctl, sizeof(uint32_t) * 4, mapped)) != cudaSuccess ||
      (e = cudaHostAlloc(&q->h_finished, sizeof(uint32_t) * size_t(max_slots), mapped)) != cudaSuccess ||
      (e = cudaEventCreateWithFlags(&q->done_ev, cudaEventDisableTiming)) != cudaSuccess) {
    free_queue(q);
    return cuda_status(e, "queue: create");
  }
  std::memset(q->h_slots, 0, sizeof(qdev::QSlot) * size_t(max_slots));
  std::memset(q->h_inbox, 0, sizeof(int32_t) * q->inbox_cap);
  std::memset(q->h_ctl, 0, sizeof(uint32_t) * 4);
  std::memset(q->h_finished, 0, sizeof(uint32_t) * size_t(max_slots));
  q->gen.assign(size_t(max_slots), 0u);
  q->busy.assign(size_t(max_slots), 0);
  for (int32_t s = max_slots - 1; s >= 0; --s) q->free_slots.push_back(s);
  *out = q;
  return NPBGB_OK;
}

int32_t npbgb_queue_submit(npbgb_queue* q, const npbgb_grid* grid, int32_t* slot_out) {
  using namespace npbgb;
  if (!q || !grid || !slot_out) return set_error(NPBGB_ERR_ARG, "queue: null argument");
  *slot_out = -1;
  qdev::QSlot d;
  int64_t updates = 0;
  std::lock_guard<std::mutex> lock(q->mu);
  const int32_t r = qhost::describe(*grid, 0, q->tile_rows, q->tile_planes, &d, &updates,
                                    q->target_tiles);
  if (r != NPBGB_OK) return r;
  if (d.total == 0) return NPBGB_OK;  // nothing to do: finished at once
  if (load_acquire(q->h_ctl + 3) != 0u)
    return set_error(NPBGB_ERR_STATE, "queue: the worker recorded an error (status %u)",
                     load_acquire(q->h_ctl + 3));
  if (load_acquire(q->h_ctl + 1) != 0u) return set_error(NPBGB_ERR_STATE, "queue: closed");
  if (q->free_slots.empty())
    return set_error(NPBGB_ERR_NOMEM, "queue: all %d slots busy", q->max_slots);
  const int32_t slot = q->free_slots.back();
  q->free_slots.pop_back();
  d.gen = ++q->gen[size_t(slot)];
  if (d.gen == 0) d.gen = q->gen[size_t(slot)] = 1;  // 0 means "never finished"
  q->h_slots[slot] = d;
  q->busy[size_t(slot)] = 1;
  q->h_inbox[q->published % q->inbox_cap] = slot;
  store_release(q->h_ctl + 0, ++q->published);
  *slot_out = slot;
  return NPBGB_OK;
}

int32_t npbgb_queue_kick(npbgb_queue* q, void* stream) {
  using namespace npbgb;
  if (!q) return set_error(NPBGB_ERR_ARG, "queue: null handle");
  std::lock_guard<std::mutex> lock(q->mu);
  if (running(q)) return NPBGB_OK;
  const uint32_t status = load_acquire(q->h_ctl + 3);
  if (status != 0u) return set_error(NPBGB_ERR_TIMEOUT, "queue: the worker recorded an error (status %u)", status);
  const uint32_t consumed = load_acquire(q->h_ctl + 2);
  bool outstanding = consumed != q->published;
  for (int32_t s = 0; s < q->max_slots && !outstanding; ++s)
    outstanding = q->busy[size_t(s)] && load_acquire(q->h_finished + s) != q->gen[size_t(s)];
  if (!outstanding) return NPBGB_OK;
  if (consumed == q->published) {
    // A grid was taken from the inbox but has not finished, and no worker runs.
    return set_error(NPBGB_ERR_STATE, "queue: a grid is outstanding but the worker ended");
  }
  // A fresh launch: every earlier grid finished, so the ring holds nothing
  // live; reset it and keep the inbox position.
  cudaStream_t st = as_stream(stream);
  qdev::QState init{};
  init.inbox_head = consumed;
  cudaError_t e;
  if ((e = cudaMemsetAsync(q->d_ring, 0xff, sizeof(qdev::QSeg) * q->ring_size, st)) != cudaSuccess ||
      (e = cudaMemsetAsync(q->d_claim, 0, sizeof(unsigned long long) * q->ring_size, st)) != cudaSuccess ||
      (e = cudaMemcpyAsync(q->d_state, &init, sizeof(init), cudaMemcpyHostToDevice, st)) != cudaSuccess)
    return cuda_status(e, "queue: reset");
  const int per_sm = qhost::slots_per_sm(q->ctas_per_sm, nullptr);
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, q->device);
  const qdev::QArgs args = queue_args(q);
  if ((e = qhost::launch_worker(args, per_sm * std::max(1, sms), q->ctas_per_sm, st)) != cudaSuccess)
    return cuda_status(e, "queue: worker launch");
  if ((e = cudaEventRecord(q->done_ev, st)) != cudaSuccess) return cuda_status(e, "queue: event");
  q->launched = true;
  ++q->launches;
  return NPBGB_OK;
}

int32_t npbgb_queue_poll(npbgb_queue* q, int32_t* slots, int32_t cap, int32_t* count) {
  using namespace npbgb;
  if (!q || !count || (cap > 0 && !slots)) return set_error(NPBGB_ERR_ARG, "queue: null argument");
  *count = 0;
  std::lock_guard<std::mutex> lock(q->mu);
  int32_t n = 0;
  for (int32_t s = 0; s < q->max_slots && n < cap; ++s) {
    if (!q->busy[size_t(s)] || load_acquire(q->h_finished + s) != q->gen[size_t(s)]) continue;
    q->busy[size_t(s)] = 0;
    q->free_slots.push_back(s);
    slots[n++] = s;
  }
  *count = n;
  return NPBGB_OK;
}

int32_t npbgb_queue_state(npbgb_queue* q, int32_t* running_out, int32_t* busy_out,
                          int64_t* launches_out) {
  using namespace npbgb;
  if (!q) return set_error(NPBGB_ERR_ARG, "queue: null handle");
  std::lock_guard<std::mutex> lock(q->mu);
  if (running_out) *running_out = running(q) ? 1 : 0;
  if (busy_out) {
    int32_t b = 0;
    for (uint8_t x : q->busy) b += x;
    *busy_out = b;
  }
  if (launches_out) *launches_out = q->launches;
  const uint32_t status = load_acquire(q->h_ctl + 3);
  if (status != 0u)
    return set_error(NPBGB_ERR_TIMEOUT, "queue: the worker recorded an error (status %u)", status);
  return NPBGB_OK;
}

int32_t npbgb_queue_close(npbgb_queue* q) {
  using namespace npbgb;
  if (!q) return set_error(NPBGB_ERR_ARG, "queue: null handle");
  std::lock_guard<std::mutex> lock(q->mu);
  store_release(q->h_ctl + 1, 1u);
  return NPBGB_OK;
}

int32_t npbgb_queue_destroy(npbgb_queue* q) {
  using namespace npbgb;
  if (!q) return NPBGB_OK;
  {
    std::lock_guard<std::mutex> lock(q->mu);
    store_release(q->h_ctl + 1, 1u);
    if (q->launched) cudaEventSynchronize(q->done_ev);  // ends: closed, and bounded waits
  }
  free_queue(q);
  return NPBGB_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Static batches in queue form (npbgb_batch, NPBGB_BATCH_QUEUE)
// ---------------------------------------------------------------------------
namespace npbgb {
namespace qhost {

struct StaticQueue {
  int32_t nslots = 0;
  uint32_t ring_size = 0;
  int ctas_per_sm = 3;
  int nctas = 0;
  qdev::QSlot* d_slots = nullptr;
  qdev::QSeg* d_ring = nullptr;         // live ring
  qdev::QSeg* d_ring0 = nullptr;        // initial ring (first segment of every grid)
  unsigned long long* d_claim = nullptr;
  unsigned long long* d_claim0 = nullptr;
  uint32_t* d_done = nullptr;
  qdev::QState* d_state = nullptr;
  qdev::QState* d_state0 = nullptr;
  uint32_t* d_ctl = nullptr;             // inbox control in device memory: empty and closed
};

void free_static(StaticQueue* s) {
  if (!s) return;
  cudaFree(s->d_slots);
  cudaFree(s->d_ring);
  cudaFree(s->d_ring0);
  cudaFree(s->d_claim);
  cudaFree(s->d_claim0);
  cudaFree(s->d_done);
  cudaFree(s->d_state);
  cudaFree(s->d_state0);
  cudaFree(s->d_ctl);
  delete s;
}

int32_t plan_static(const npbgb_grid* grids, int64_t count, int32_t tile_rows, int32_t ctas_per_sm,
                    StaticQueue** out, int64_t* updates, int64_t* tiles) {
  *out = nullptr;
  *updates = 0;
  *tiles = 0;
  int sms0 = 0, dev0 = 0;
  cudaGetDevice(&dev0);
  cudaDeviceGetAttribute(&sms0, cudaDevAttrMultiProcessorCount, dev0);
  const int64_t target = int64_t(std::max(1, sms0)) *
                         slots_per_sm(ctas_per_sm > 0 ? ctas_per_sm : 3, nullptr);
  std::vector<qdev::QSlot> slots;
  for (int64_t g = 0; g < count; ++g) {
    qdev::QSlot d;
    int64_t up = 0;
    const int32_t r = describe(grids[g], g, tile_rows, tile_rows, &d, &up, target);
    if (r != NPBGB_OK) return r;
    if (d.total == 0) continue;
    d.gen = 1;
    slots.push_back(d);
    *updates += up;
    *tiles += int64_t(d.ntiles) * d.steps;
  }
  if (slots.size() > (1u << 24)) return set_error(NPBGB_ERR_NOMEM, "queue: too many grids");
  // Longest runs first: their half-sweeps chain the longest.
  std::stable_sort(slots.begin(), slots.end(), [](const qdev::QSlot& x, const qdev::QSlot& y) {
    return int64_t(x.steps) * x.ntiles > int64_t(y.steps) * y.ntiles;
  });
  auto* s = new (std::nothrow) StaticQueue();
  if (!s) return set_error(NPBGB_ERR_NOMEM, "queue: host allocation");
  s->nslots = int32_t(slots.size());
  s->ring_size = uint32_t(2 * std::max<size_t>(1, slots.size()) + 2);
  s->ctas_per_sm = ctas_per_sm > 0 ? ctas_per_sm : 3;
  const size_t ns = std::max<size_t>(1, slots.size());
  std::vector<qdev::QSeg> ring(s->ring_size);
  std::vector<unsigned long long> claim(s->ring_size, 0ull);
  for (size_t i = 0; i < ring.size(); ++i) ring[i] = qdev::QSeg{-1, -1, -1, qdev::kSeqEmpty};
  for (size_t i = 0; i < slots.size(); ++i) {
    ring[i] = qdev::QSeg{int32_t(i), 0, qdev::seg_units(slots[i]), uint32_t(i)};
    claim[i] = uint64_t(i) << 32;
  }
  qdev::QState st0{};
  st0.tail = uint32_t(slots.size());
  st0.active = uint32_t(slots.size());
  const uint32_t ctl[4] = {0u, 1u, 0u, 0u};
  cudaError_t e;
  if ((e = cudaMalloc(&s->d_slots, sizeof(qdev::QSlot) * ns)) != cudaSuccess ||
      (e = cudaMalloc(&s->d_ring, sizeof(qdev::QSeg) * s->ring_size)) != cudaSuccess ||
      (e = cudaMalloc(&s->d_ring0, sizeof(qdev::QSeg) * s->ring_size)) != cudaSuccess ||
      (e = cudaMalloc(&s->d_claim, sizeof(unsigned long long) * s->ring_size)) != cudaSuccess ||
      (e = cudaMalloc(&s->d_claim0, sizeof(unsigned long long) * s->ring_size)) != cudaSuccess ||
      (e = cudaMalloc(&s->d_done, sizeof(uint32_t) * ns)) != cudaSuccess ||
      (e = cudaMalloc(&s->d_state, sizeof(qdev::QState))) != cudaSuccess ||
      (e = cudaMalloc(&s->d_state0, sizeof(qdev::QState))) != cudaSuccess ||
      (e = cudaMalloc(&s->d_ctl, sizeof(ctl))) != cudaSuccess ||
      (!slots.empty() &&
       (e = cudaMemcpy(s->d_slots, slots.data(), sizeof(qdev::QSlot) * slots.size(),
                       cudaMemcpyHostToDevice)) != cudaSuccess) ||
      (e = cudaMemcpy(s->d_ring0, ring.data(), sizeof(qdev::QSeg) * ring.size(),
                      cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaMemcpy(s->d_claim0, claim.data(), sizeof(unsigned long long) * claim.size(),
                      cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaMemcpy(s->d_state0, &st0, sizeof(st0), cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaMemcpy(s->d_ctl, ctl, sizeof(ctl), cudaMemcpyHostToDevice)) != cudaSuccess) {
    free_static(s);
    return cuda_status(e, "queue: static plan");
  }
  int sms = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int per_sm = slots_per_sm(s->ctas_per_sm, nullptr);
  s->nctas = int(std::max<int64_t>(1, std::min<int64_t>(int64_t(per_sm) * std::max(1, sms),
                                                        std::max<int64_t>(1, *tiles))));
  *out = s;
  return NPBGB_OK;
}

// Restores the initial ring and counters, then runs the worker until every
// grid is done (the inbox is empty and closed).  Capturable into a graph.
int32_t launch_static(StaticQueue* s, cudaStream_t st) {
  if (s->nslots == 0) return NPBGB_OK;
  cudaError_t e;
  if ((e = cudaMemcpyAsync(s->d_ring, s->d_ring0, sizeof(qdev::QSeg) * s->ring_size,
                           cudaMemcpyDeviceToDevice, st)) != cudaSuccess ||
      (e = cudaMemcpyAsync(s->d_claim, s->d_claim0, sizeof(unsigned long long) * s->ring_size,
                           cudaMemcpyDeviceToDevice, st)) != cudaSuccess ||
      (e = cudaMemcpyAsync(s->d_state, s->d_state0, sizeof(qdev::QState), cudaMemcpyDeviceToDevice,
                           st)) != cudaSuccess ||
      (e = cudaMemsetAsync(s->d_done, 0, sizeof(uint32_t) * size_t(s->nslots), st)) != cudaSuccess)
    return cuda_status(e, "queue: reset");
  qdev::QArgs a{};
  a.slots = s->d_slots;
  a.ring = s->d_ring;
  a.claim = s->d_claim;
  a.done = s->d_done;
  a.st = s->d_state;
  a.host_slots = s->d_slots;
  a.inbox = nullptr;
  a.inbox_ctl = s->d_ctl;
  a.consumed_out = nullptr;
  a.status_out = nullptr;
  a.finished = nullptr;
  a.ring_size = s->ring_size;
  a.inbox_cap = 1;
  a.max_slots = s->nslots;
  a.idle_ns = 0;
  a.f64_emulation = int(g_cfg_f64_emulation);
  a.hw_warps = jacobi_hw_warps();
  a.one = 1u;
  if ((e = launch_worker(a, s->nctas, s->ctas_per_sm, st)) != cudaSuccess)
    return cuda_status(e, "queue: worker launch");
  return NPBGB_OK;
}

int static_ctas(const StaticQueue* s) { return s->nctas; }

}  // namespace qhost
}  // namespace npbgb
