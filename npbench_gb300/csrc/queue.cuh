// Shapes shared by the device-side tile work queue (queue.cu) and the batch
// planner (batch.cu).
#pragma once

#include <cstdint>

#include "npbgb_common.cuh"

namespace npbgb {
namespace qdev {

constexpr uint32_t kSeqEmpty = 0xffffffffu;

// One grid's residency in the queue (128 bytes, copied word by word).  Its
// segments are numbered 0 .. steps-1: with `conv`, segment 0 widens a32/b32
// into a/b, segments 1 .. total are the half-sweeps and the last one rounds
// a/b back into a32/b32; without it, segment s is half-sweep s.
struct QSlot {
  void* a;            // first source for even step0
  void* b;
  void* a32;          // binary32 arrays of a grid run in binary64 (conv), else null
  void* b32;
  int32_t n0, n1, n2;
  int16_t kind, dtype;
  int32_t step0;      // half-sweeps already applied (parity of the first source)
  int32_t total;      // half-sweeps to perform in this residency (>= 1)
  int32_t ntiles;     // tiles per segment
  int32_t chunk;      // rows (Jacobi-2D) or planes (Heat-3D) per tile
  int32_t tx, ty;     // tiles along the contiguous axis; along axis 1 (Heat-3D)
  uint32_t gen;       // residency number, written to the completion word
  int32_t steps;      // segments: total, plus 2 with conv
  int32_t conv;
  int32_t whole;      // 1: one CTA sweeps all tiles of a segment and runs on
                      // to the next ones (the ring holds one unit per segment)
  int64_t cells;      // elements per array
  int64_t pad1[4];
};
static_assert(sizeof(QSlot) == 128, "QSlot is copied as sixteen 64-bit words");

// One half-sweep of one grid.  seq == ring position once the entry is written.
struct QSeg {
  int32_t slot;
  int32_t s;
  int32_t ntiles;
  uint32_t seq;
};

// Claimable units per segment: every tile, or one for a whole-grid slot.
__host__ __device__ inline int32_t seg_units(const QSlot& G) { return G.whole ? 1 : G.ntiles; }

// Segments a CTA runs in a row on a whole-grid slot before it hands the grid
// back to the ring (bounds how long one grid holds a CTA).
constexpr int32_t kLocalRun = 256;

struct QState {
  uint32_t head;        // ring position tiles are claimed from
  uint32_t tail;        // next ring position to write
  uint32_t active;      // grids taken in and not finished
  uint32_t inbox_head;  // inbox entries taken in
  uint32_t lock;        // inbox lock (activation and shutdown)
  uint32_t shutdown;    // 1: every CTA leaves at its next idle moment
  uint32_t error;       // bit 0: the ring did not move within the limit; bit 1: bad inbox entry
  uint32_t pad;
};

struct QArgs {
  QSlot* slots;                  // device slot table
  QSeg* ring;
  unsigned long long* claim;     // per ring entry: (position << 32) | tiles claimed
  uint32_t* done;                // per slot: tiles completed in the residency
  QState* st;
  const QSlot* host_slots;       // descriptors of inbox entries
  const int32_t* inbox;          // ring of slot indices
  const uint32_t* inbox_ctl;     // [0] entries published, [1] closed
  uint32_t* consumed_out;        // mirror of inbox_head for the host, or null
  uint32_t* status_out;          // mirror of the error word for the host, or null
  uint32_t* finished;            // per slot: gen of the last finished residency, or null
  uint32_t ring_size, inbox_cap;
  int32_t max_slots;
  uint64_t idle_ns;              // end the launch after this long with nothing to do
  int f64_emulation, hw_warps;
  uint32_t one;                  // == 1 (keeps constant folding out of the fixed-point adds)
};

}  // namespace qdev

namespace qhost {

// A batch run as one queue launch: every grid's first half-sweep is in the
// ring from the start and the inbox is empty and closed.
struct StaticQueue;

int32_t plan_static(const npbgb_grid* grids, int64_t count, int32_t tile_rows, int32_t ctas_per_sm,
                    StaticQueue** out, int64_t* updates, int64_t* tiles);
int32_t launch_static(StaticQueue* s, cudaStream_t st);
void free_static(StaticQueue* s);
int static_ctas(const StaticQueue* s);

}  // namespace qhost
}  // namespace npbgb
