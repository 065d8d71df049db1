/* npbgb.h -- C ABI of libnpbgb, the GB300 (sm_103a) structured-grid stencil library.
 *
 * Every entry point takes plain device pointers, element counts and a CUDA
 * stream (cudaStream_t passed as void*; NULL = the legacy default stream),
 * launches its kernels asynchronously on that stream and returns an int32
 * status (NPBGB_OK = 0).  No C++ exception crosses this boundary.  On a
 * non-zero status npbgb_last_error() holds a message for the calling thread.
 *
 * Arrays are C-ordered (last axis contiguous), densely packed, and must not
 * alias unless stated.  Element type is selected by `dtype`
 * (NPBGB_F64 = IEEE binary64, NPBGB_F32 = binary32).
 *
 * Arithmetic is bit-identical to NPBench's NumPy kernels: every binary
 * operator of the reference is one correctly rounded IEEE operation, in the
 * reference's order, with no fused multiply-add.
 */
#ifndef NPBGB_H
#define NPBGB_H

#include <stdint.h>

#if defined(__GNUC__)
#define NPBGB_API __attribute__((visibility("default")))
#else
#define NPBGB_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. */
#define NPBGB_OK 0
#define NPBGB_ERR_ARG 1        /* bad size, null pointer, aliasing */
#define NPBGB_ERR_DTYPE 2      /* dtype not supported by this entry point */
#define NPBGB_ERR_CUDA 3       /* a CUDA runtime call failed (see npbgb_last_error) */
#define NPBGB_ERR_TIMEOUT 4    /* a bounded device-side wait gave up */
#define NPBGB_ERR_NOMEM 5      /* a budget or capacity limit would be exceeded */
#define NPBGB_ERR_STATE 6      /* call not valid in the object's current state */

/* Element types. */
#define NPBGB_F64 0
#define NPBGB_F32 1

/* Configuration keys for npbgb_set_config / npbgb_get_config.  Settings are
 * process-wide and read when an entry point launches its kernels. */
#define NPBGB_CFG_F64_EMULATION 1 /* 1 (default): binary64 additions run exactly in
                                     fixed point on the integer pipe where every
                                     operand allows it, else hardware binary64;
                                     0: hardware binary64 only.  Results are
                                     identical either way. */
#define NPBGB_CFG_HEAT_CHUNK 2    /* axis-0 planes per CTA in heat3d; 0 = automatic */
#define NPBGB_CFG_HEAT_TMA 3      /* 1 (default): heat3d stages planes with TMA when the
                                     arrays allow it; 0: plain loads only */
#define NPBGB_CFG_JACOBI_CHUNK 4  /* rows per warp in jacobi2d; 0 = automatic */
#define NPBGB_CFG_HEAT_ROWS 5     /* axis-1 tile rows per thread in heat3d (TMA): 1, 2, 4;
                                     0 (default) = 4 for binary32, 2 for binary64 */
#define NPBGB_CFG_HEAT_HW_ROWS 6  /* heat3d binary64: tile rows per CTA evaluated with
                                     hardware binary64 next to the fixed-point rows;
                                     -1 (default) = 7 of 16 with 2 rows per thread,
                                     3 of 8 with 1, 8 of 32 with 4 */
#define NPBGB_CFG_F64_CVT 7       /* 1: fixed-point conversions use the binary64
                                     convert instructions; 0: integer bit operations */
#define NPBGB_CFG_JACOBI_HW_WARPS 8 /* jacobi2d / batch binary64: warps per CTA (of 8)
                                       that use hardware binary64 next to the
                                       fixed-point warps; -1 (default) = 4 */
#define NPBGB_CFG_BATCH_CTAS_PER_SM 9 /* persistent and queue batch kernels: 2 to 5
                                         (default 5) CTAs per SM (the persistent form
                                         uses 3 for 3 and more); read when a batch is
                                         planned.  The queue form of the 4096-grid
                                         batch: 0.91e11 / 1.14e11 / 1.32e11 updates/s
                                         with 3 / 4 / 5. */
#define NPBGB_CFG_PDL 10              /* 1 (default): the per-half-sweep launches of the
                                         time loops use programmatic dependent launch;
                                         0: plain stream order */
#define NPBGB_CFG_BATCH_MODE 11       /* form of a batch, read when it is planned:
                                         0 (default) automatic by size, 1 persistent,
                                         2 stepped, 3 queue (NPBGB_BATCH_*) */
#define NPBGB_CFG_HDIFF_EMU 12        /* hdiff: which Laplacian and flux items run on the
                                         integer pipes (exact binary64 addition in
                                         integer arithmetic) next to the hardware
                                         binary64 ones.  Bit t of the low byte: the
                                         Laplacian items i of a warp with i % 8 == t;
                                         bits 8..15 the same for the flux items,
                                         bits 16..23 for the output points.
                                         -1 (default) = the library's choice; 0 =
                                         hardware binary64 only.  Results are
                                         identical for every mask. */
#define NPBGB_CFG_JACOBI1D_CTAS 14    /* jacobi1d: segments (CTAs) per SM; 0 (default)
                                         = the library's choice.  Reading returns
                                         the value in effect. */
#define NPBGB_CFG_JACOBI1D_DEPTH 15   /* jacobi1d: half-sweeps per launch, which is
                                         also the halo width; an even number up to
                                         64, 0 (default) = the library's choice.
                                         Reading returns the value in effect. */
#define NPBGB_CFG_HEAT_TB 16          /* heat3d binary32: half-sweeps per launch.
                                         2: two (temporal blocking) wherever the
                                         arrays meet the TMA rules and TSTEPS >= 4;
                                         0 (default) or 1: one (the single-step
                                         kernel with short plane chunks measured
                                         faster at every size).  Results are
                                         identical either way. */
#define NPBGB_CFG_HEAT_TB_CHUNK 17    /* heat3d binary32 two-step kernel: axis-0
                                         planes per CTA; 0 (default) = automatic */
#define NPBGB_CFG_JACOBI_BANDS 18     /* jacobi2d: the whole time loop in one launch with
                                         bands of rows resident in shared memory.
                                         2: whenever the bands fit; 0 (default) or 1:
                                         chained launches (measured faster over mixed
                                         shapes and under concurrent streams; the
                                         autotuner picks 2 per shape class where it
                                         wins).  Results are identical either way. */
#define NPBGB_CFG_JACOBI_BANDS_WARPS 19 /* warps per CTA of that kernel: 8, 16 or 32;
                                           0 (default): one 32-column strip per warp,
                                           8 to 32 warps */
#define NPBGB_CFG_HEAT_STAGES 20      /* heat3d binary32 TMA kernel: depth of the
                                         shared-memory plane ring, 4, 6 or 8;
                                         0 (default) = automatic */
#define NPBGB_CFG_LAUNCHES 21         /* read: kernels the library has put on a
                                         stream, each batch graph replay counting the
                                         kernels it holds (a launch recorded into a
                                         caller's graph counts once, when recorded);
                                         set 0 to reset */
#define NPBGB_CFG_HEAT_MAD_ROWS 22    /* heat3d binary64 TMA kernel: fixed-point tile
                                         rows (the first ones) whose 64-bit adds run as
                                         multiply-adds on the FMA pipe; 0 (default) */
#define NPBGB_CFG_QUEUE_WHOLE_CELLS 23 /* tile queue: grids of at most this many cells
                                          per array run whole (one CTA sweeps every
                                          tile of a half-sweep and runs on to the next
                                          ones, up to 256, before returning the grid
                                          to the ring); 0 = never; default 65536 */
#define NPBGB_CFG_JACOBI_FX_MUL 24    /* jacobi2d single-grid kernel, binary64: the
                                         product by 0.2 on the integer pipes for the
                                         fixed-point points (1, default), for those and
                                         the hardware warps' points (2), or a hardware
                                         binary64 multiply everywhere (0).  Results are
                                         identical. */
#define NPBGB_CFG_JACOBI_FX_ADDS 25   /* jacobi2d single-grid kernel, binary64 fixed-
                                         point additions: 0 (default) or 1 integer
                                         adds, 2 multiply-add 64-bit adds, 3 most of
                                         the rounding on the multiply-add pipe.
                                         Results are identical. */
#define NPBGB_CFG_BATCH_TMA 27        /* stepped batches, read when planned: binary64
                                         Jacobi-2D grids whose rows are 16-byte
                                         multiples stream each warp's rows through a
                                         ring of TMA copies (1) or use plain loads
                                         (0, default: the rings measured 1.5-2.6%
                                         slower on the 4096-grid batch, whose
                                         32-64-row tiles are short).  Results are
                                         identical. */
#define NPBGB_CFG_JACOBI_TMA 26       /* jacobi2d single-grid kernel: each warp
                                         streams its rows through its own ring of
                                         TMA copies (rows a multiple of 16 bytes)
                                         for binary64 arrays of 48 MiB and more (1,
                                         default), for every aligned grid (2), or
                                         never (0).  Results are identical. */

/* Batch forms. */
#define NPBGB_BATCH_PERSISTENT 1
#define NPBGB_BATCH_STEPPED 2
#define NPBGB_BATCH_QUEUE 3

/* Grid kinds for batches. */
#define NPBGB_KIND_JACOBI2D 0
#define NPBGB_KIND_HEAT3D 1

/* One grid of a batch: a ping-pong pair of device arrays and its own step
 * count.  For NPBGB_KIND_JACOBI2D the arrays are (n0, n1) and n2 is ignored;
 * for NPBGB_KIND_HEAT3D they are (n0, n1, n2).  A run may be split over
 * several launches: step0 half-sweeps are taken as already applied (the
 * first source is a for even step0, b for odd), and at most nsteps are
 * performed (0 = all remaining), so consecutive launches with step0 advanced
 * by what the previous one did reproduce the uninterrupted run bit for bit. */
typedef struct npbgb_grid {
  void* a;           /* holds the field at step 0 and the newest field at the end */
  void* b;           /* second buffer (holds the previous field at the end) */
  int64_t n0, n1, n2;
  int32_t kind;      /* NPBGB_KIND_* */
  int32_t dtype;     /* NPBGB_F64 or NPBGB_F32 */
  int32_t tsteps;    /* the reference's TSTEPS: 2*(tsteps-1) half-sweeps */
  int32_t band_rows; /* axis-0 extent of a scheduling band; 0 = the batch default
                        (32 rows for Jacobi-2D, 8 planes for Heat-3D) */
  int32_t step0;     /* half-sweeps already applied (0 = start of the run) */
  int32_t nsteps;    /* half-sweeps to perform now; 0 = all remaining */
  void* a32;         /* queue forms only, else NULL: binary32 arrays of a grid run in
                        binary64 (dtype NPBGB_F64, a and b the binary64 pair).  Before
                        the first half-sweep a32/b32 are widened exactly into a/b; after
                        the last, a/b are rounded to nearest back into a32/b32. */
  void* b32;
} npbgb_grid;

typedef struct npbgb_batch npbgb_batch;

/* Library identification: "npbgb <version> sm_103a". */
NPBGB_API const char* npbgb_version(void);

/* Message describing the last non-OK status returned to this thread. */
NPBGB_API const char* npbgb_last_error(void);

/* Text for a status code. */
NPBGB_API const char* npbgb_status_string(int32_t status);

/* Sets / reads a configuration value (NPBGB_CFG_*).  NPBGB_ERR_ARG for an
 * unknown key or an out-of-range value.  No counterpart in the reference,
 * whose NumPy kernels have no tuning knobs. */
NPBGB_API int32_t npbgb_set_config(int32_t key, int64_t value);
NPBGB_API int32_t npbgb_get_config(int32_t key, int64_t* value);

/* Synchronises `stream` (NULL: the whole device), then reads and clears the
 * library's device error words.  NPBGB_ERR_TIMEOUT if a kernel gave up a
 * bounded wait (for example on a TMA copy that never completed) since the
 * last call.  Counterpart of the harness's per-run timeout,
 * npbench/infrastructure/timeout_decorator.py:46-72, on the device side. */
NPBGB_API int32_t npbgb_device_status(void* stream);

/* Launches one CTA that waits on an mbarrier nothing completes, with a limit
 * of limit_ns (1 .. 2e9).  The wait gives up and records the error that
 * npbgb_device_status then reports: a check of the timeout path that needs
 * no fault.  No counterpart in the reference. */
NPBGB_API int32_t npbgb_selftest_wait_timeout(int64_t limit_ns, void* stream);

/* Converts n elements: NPBGB_F32 -> NPBGB_F64 (exact) or NPBGB_F64 -> NPBGB_F32
 * (round to nearest even, as NumPy's astype).  For binary32 requests that run
 * in binary64 because their binary32 error would exceed NPBench's acceptance
 * bound (npbench/infrastructure/utilities.py:154-180); the reference has no such
 * step (it runs in the dtype it is given). */
NPBGB_API int32_t npbgb_convert(void* dst, int32_t dst_dtype, const void* src, int32_t src_dtype,
                                int64_t n, void* stream);

/* Arithmetic pipe probe: launches `ctas` CTAs of 256 threads in which every
 * thread runs 8 independent chains of `iters` operations of one kind
 * (op: 0 binary64 add, 1 binary64 multiply, 2 binary64 fused multiply-add,
 * 3 binary32 fused multiply-add, 4 32-bit three-input logic, 5 32-bit add,
 * 6 32-bit multiply-add); the caller times it on `stream`, and
 * ctas * 256 * 8 * iters / time is that pipe's throughput.  `sink` holds
 * ctas * 256 doubles.  These are the compute roofs that the binary64 kernels,
 * which GB300's binary64 pipe bounds rather than HBM, are measured against.
 * No counterpart in the reference. */
NPBGB_API int32_t npbgb_probe_pipe(int32_t op, int64_t iters, int32_t ctas, void* sink,
                                   void* stream);

/* 2D 5-point Jacobi, the whole time loop of
 *   kernel(TSTEPS, A, B)   polybench/jacobi_2d/jacobi_2d_numpy.py:4-10
 * A and B are (ny, nx).  For t in 1..tsteps-1 it performs the half-sweep
 * A -> B and then B -> A over the interior [1, ny-1) x [1, nx-1):
 *   dst = 0.2 * ((((c + w) + e) + s) + n)
 * Boundary rows and columns are never written.  On return A holds the newest
 * field and B the previous one, as in the reference.  tsteps <= 1 is a no-op.
 * One chained launch per half-sweep; with NPBGB_CFG_JACOBI_BANDS = 2, grids
 * whose bands of rows fit in shared memory run the whole loop in one
 * cooperative launch (its exchange rows come from a stream-ordered pool). */
NPBGB_API int32_t npbgb_jacobi2d(void* A, void* B, int64_t ny, int64_t nx, int32_t tsteps,
                       int32_t dtype, void* stream);

/* 3D 7-point heat, the whole time loop of
 *   kernel(TSTEPS, A, B)   polybench/heat_3d/heat_3d_numpy.py:4-20
 * A and B are (n0, n1, n2); half-sweeps A -> B then B -> A, tsteps-1 times:
 *   dst = ((t0 + t1) + t2) + c,   tx = 0.125 * ((next_x - 2.0 * c) + prev_x)
 * Faces are never written. */
NPBGB_API int32_t npbgb_heat3d(void* A, void* B, int64_t n0, int64_t n1, int64_t n2,
                     int32_t tsteps, int32_t dtype, void* stream);

/* 4th-order horizontal diffusion with flux limiter,
 *   hdiff(in_field, out_field, coeff)   weather_stencils/hdiff/hdiff_numpy.py:5-29
 * in_field is (I+4, J+4, K) with a halo of two in I and J; out_field and coeff
 * are (I, J, K); K is contiguous.  Writes all of out_field.  dtype must be
 * NPBGB_F64 (the limiter's sign tests are kept in binary64). */
NPBGB_API int32_t npbgb_hdiff(const void* in_field, void* out_field, const void* coeff, int64_t I,
                    int64_t J, int64_t K, int32_t dtype, void* stream);

/* 1D 3-point Jacobi, the whole time loop of
 *   kernel(TSTEPS, A, B)   polybench/jacobi_1d/jacobi_1d_numpy.py:4-8
 * A and B have n points; tsteps-1 times: dst[i] = 0.33333 * ((src[i-1] + src[i]) + src[i+1])
 * over [1, n-1), A -> B then B -> A.  Temporal blocking in shared memory: one
 * launch per NPBGB_CFG_JACOBI1D_DEPTH half-sweeps (48 by default). */
NPBGB_API int32_t npbgb_jacobi1d(void* A, void* B, int64_t n, int32_t tsteps, int32_t dtype,
                                 void* stream);

/* 2D FDTD, the whole time loop of
 *   kernel(TMAX, ex, ey, hz, _fict_)   polybench/fdtd_2d/fdtd_2d_numpy.py:4-11
 * ex, ey, hz are (nx, ny); fict has fict_len >= tmax entries (NPBGB_ERR_ARG
 * otherwise, where the reference raises IndexError).  Updates ex, ey, hz in
 * place. */
NPBGB_API int32_t npbgb_fdtd2d(void* ex, void* ey, void* hz, const void* fict, int64_t fict_len,
                               int64_t nx, int64_t ny, int32_t tmax, int32_t dtype, void* stream);

/* Vertical advection, a tridiagonal (Thomas) solve along K per (i, j) column,
 *   vadv(utens_stage, u_stage, wcon, u_pos, utens, dtr_stage)
 *                               weather_stencils/vadv/vadv_numpy.py:9-78
 * utens_stage, u_stage, u_pos, utens are (I, J, K) and wcon is (I+1, J, K);
 * K is contiguous.  Writes all of utens_stage (the only output; its values are
 * also read).  dtype must be NPBGB_F64.  K < 2 is NPBGB_ERR_ARG (the reference
 * raises IndexError: it reads level 1 unconditionally).  The solve keeps one
 * coefficient per point in a device workspace of npbgb_vadv_workspace_bytes()
 * bytes (8*(K-1)*I*J); pass it, or NULL to have the call allocate and free it
 * stream-ordered (cudaMallocAsync / cudaFreeAsync on `stream`).  A caller that
 * passes a workspace must not use it concurrently for another call. */
NPBGB_API int64_t npbgb_vadv_workspace_bytes(int64_t I, int64_t J, int64_t K);
NPBGB_API int32_t npbgb_vadv(void* utens_stage, const void* u_stage, const void* wcon,
                             const void* u_pos, const void* utens, double dtr_stage, int64_t I,
                             int64_t J, int64_t K, int32_t dtype, void* workspace,
                             int64_t workspace_bytes, void* stream);

/* Lid-driven cavity flow, the whole time loop of
 *   cavity_flow(nx, ny, nt, nit, u, v, dt, dx, dy, p, rho, nu)
 *                               cavity_flow/cavity_flow_numpy.py:41-82
 * u, v, p are (ny, nx) and updated in place.  Per time step: build_up_b, nit
 * pressure iterations with the reference's boundary statements, the momentum
 * updates and the walls, every operation rounded as NumPy rounds it (the
 * scalars dx**2 etc. are formed with the C library's pow, as Python's float
 * power is).  One cooperative persistent launch runs all nt steps.
 * dtype must be NPBGB_F64.  With nt >= 1, ny or nx below 1, or below 2 when
 * nit >= 1, is NPBGB_ERR_ARG (the reference raises IndexError).  Grids of 3 x 3
 * and more need a workspace of npbgb_cavity_flow_workspace_bytes(ny, nx)
 * (four fields and the band counters); pass it, or NULL to have the call
 * allocate and free it stream-ordered.  Bounded waits: a band that sees no
 * progress from its neighbours for two seconds records an error reported by
 * npbgb_device_status. */
NPBGB_API int64_t npbgb_cavity_flow_workspace_bytes(int64_t ny, int64_t nx);
NPBGB_API int32_t npbgb_cavity_flow(void* u, void* v, void* p, int64_t ny, int64_t nx, int32_t nt,
                                    int32_t nit, double dt, double dx, double dy, double rho,
                                    double nu, int32_t dtype, void* workspace,
                                    int64_t workspace_bytes, void* stream);

/* Channel flow, the whole convergence loop of
 *   channel_flow(nit, u, v, dt, dx, dy, p, rho, nu, F)
 *                               channel_flow/channel_flow_numpy.py:69-152
 * u, v, p are (ny, nx), periodic in x, updated in place; the loop runs while
 * (sum(u) - sum(un)) / sum(u) > .001, the sums being np.sum's (+0.0 plus
 * NumPy's pairwise summation) bit for bit, so the step count matches the
 * reference's.  *steps (if not NULL; the call then synchronizes `stream`)
 * receives it, negated if max_steps steps ran without converging.  dtype must
 * be NPBGB_F64.  nx < 2, ny < 1, or ny < 2 with nit >= 1 is NPBGB_ERR_ARG (the
 * reference raises IndexError).  Workspace: npbgb_channel_flow_workspace_bytes
 * (ny, nx) bytes, or NULL for a stream-ordered allocation inside the call. */
NPBGB_API int64_t npbgb_channel_flow_workspace_bytes(int64_t ny, int64_t nx);
NPBGB_API int32_t npbgb_channel_flow(void* u, void* v, void* p, int64_t ny, int64_t nx,
                                     int32_t nit, double dt, double dx, double dy, double rho,
                                     double nu, double F, int64_t max_steps, int32_t dtype,
                                     void* workspace, int64_t workspace_bytes, int64_t* steps,
                                     void* stream);

/* Batches: many independent grids advanced by one persistent launch.
 *
 * npbgb_batch_create plans a batch of Jacobi-2D and Heat-3D grids: each grid
 * is cut along axis 0 into bands (the grid's band_rows, else band_rows, else
 * the kind's default), bands are assigned
 * to the CTAs of one cooperative launch with equal work per CTA, and the
 * plan (band table, per-band step counters) is stored in device memory
 * allocated here.  Each grid ends exactly as npbgb_jacobi2d / npbgb_heat3d
 * would leave it (bit-identical), i.e. as the reference's kernel(TSTEPS, A, B)
 * per grid, polybench/jacobi_2d/jacobi_2d_numpy.py:4-10 and
 * polybench/heat_3d/heat_3d_numpy.py:4-20.
 * npbgb_batch_launch runs the whole batch: a counter reset and one
 * persistent kernel on `stream`; with use_graph != 0 the two are captured
 * once into a CUDA graph and replayed.  Bounded waits: a CTA that makes no
 * progress for two seconds records an error reported by npbgb_device_status.
 * The grids' arrays must stay allocated while the batch is in use. */
NPBGB_API int32_t npbgb_batch_create(const npbgb_grid* grids, int64_t count, int32_t band_rows,
                                     npbgb_batch** out);
NPBGB_API int32_t npbgb_batch_launch(npbgb_batch* batch, int32_t use_graph, void* stream);
/* Re-plans an existing batch for a new grid list (for example the next round
 * of a server), reusing its device buffers when they are large enough.
 * A captured graph is dropped and recaptured by the next graph launch. */
NPBGB_API int32_t npbgb_batch_replan(npbgb_batch* batch, const npbgb_grid* grids, int64_t count,
                                     int32_t band_rows);
NPBGB_API int32_t npbgb_batch_info(const npbgb_batch* batch, int64_t* nbands, int64_t* nctas,
                                   int64_t* updates);
/* The form the batch was planned in (NPBGB_BATCH_PERSISTENT, NPBGB_BATCH_STEPPED
 * or NPBGB_BATCH_QUEUE).
 * Persistent: one cooperative launch whose CTAs advance bands of rows as their
 * neighbours allow (best when the batch is small).  Stepped: one launch per
 * half-sweep index over all tiles of the grids still active, chained by
 * programmatic dependent launch (best when the batch fills the GPU; batches of
 * 2^24 cells or more by default).  Queue: one launch of the device-side tile
 * work queue (npbgb_queue_create below) with every grid's first half-sweep in
 * its ring; a grid's next half-sweep is appended by the CTA that completes its
 * previous one, and tiles are claimed in ring order (band_rows = rows or planes
 * per tile).  In the stepped and queue forms npbgb_batch_info reports the tiles
 * as nbands (queue: over all half-sweeps) and the launches (stepped) or CTAs
 * (queue) as nctas.  All forms leave the same bits. */
NPBGB_API int32_t npbgb_batch_mode(const npbgb_batch* batch, int32_t* mode);
NPBGB_API int32_t npbgb_batch_destroy(npbgb_batch* batch);

/* Device-side tile work queue: a persistent worker kernel that advances
 * Jacobi-2D and Heat-3D grids of any sizes, precisions and step counts while
 * the host keeps adding grids.  Its CTAs claim tiles of grid half-sweeps from a
 * ring in device memory; the CTA that completes a grid's half-sweep appends the
 * next one, so grids interleave tile by tile and none waits for a launch
 * boundary.  The host adds grids through an inbox in pinned host memory that
 * the running kernel reads (no synchronisation, no launch per grid) and learns
 * of finished grids by polling completion words the kernel writes to host
 * memory.  Each grid ends bit-identical to npbgb_jacobi2d / npbgb_heat3d on it,
 * i.e. to the reference's kernel(TSTEPS, A, B),
 * polybench/jacobi_2d/jacobi_2d_numpy.py:4-10 and
 * polybench/heat_3d/heat_3d_numpy.py:4-20; the reference has no queue (it
 * runs one grid per call), so this is the serving counterpart of those calls.
 *
 * npbgb_queue_create: up to max_slots grids in flight; tile_rows / tile_planes
 *   are the Jacobi-2D rows and Heat-3D planes per tile (0 = sized per grid for
 *   about one tile per worker CTA, 8-256 rows or 4-64 planes; a grid's band_rows
 *   overrides); ctas_per_sm (1-5, 0 = 3) sizes the worker launch;
 *   the worker ends after idle_us microseconds with nothing to do.  Device
 *   buffers and pinned host memory are allocated here, never later.
 * npbgb_queue_submit: takes a grid (npbgb_grid, step0/nsteps honoured) and
 *   returns its slot, or -1 for a grid with nothing to do.  NPBGB_ERR_NOMEM
 *   when every slot is busy.  The arrays must stay allocated until the slot is
 *   reported finished.
 * npbgb_queue_kick: launches the worker on `stream` unless one is running;
 *   call it after submitting.  A running worker takes new grids in by itself.
 * npbgb_queue_poll: up to cap slots finished since the last poll; their grids
 *   are complete in device memory and the slots are free again.
 * npbgb_queue_state: whether a worker is running, busy slots, launches so far;
 *   NPBGB_ERR_TIMEOUT once a worker gave up a bounded wait (no tile completed
 *   for two seconds while work was outstanding).
 * npbgb_queue_close: no more grids; a running worker ends once all are done.
 * npbgb_queue_destroy: closes, waits for a running worker to end, frees. */
typedef struct npbgb_queue npbgb_queue;
NPBGB_API int32_t npbgb_queue_create(int32_t max_slots, int32_t tile_rows, int32_t tile_planes,
                                     int32_t ctas_per_sm, int64_t idle_us, npbgb_queue** out);
NPBGB_API int32_t npbgb_queue_submit(npbgb_queue* queue, const npbgb_grid* grid, int32_t* slot);
NPBGB_API int32_t npbgb_queue_kick(npbgb_queue* queue, void* stream);
NPBGB_API int32_t npbgb_queue_poll(npbgb_queue* queue, int32_t* slots, int32_t cap,
                                   int32_t* count);
NPBGB_API int32_t npbgb_queue_state(npbgb_queue* queue, int32_t* running, int32_t* busy,
                                    int64_t* launches);
NPBGB_API int32_t npbgb_queue_close(npbgb_queue* queue);
NPBGB_API int32_t npbgb_queue_destroy(npbgb_queue* queue);

/* Runs a batch of Jacobi-2D grids like npbgb_batch_create + npbgb_batch_launch, for callers that
 * must not allocate device memory: a host whose pool or HBM budget owns every
 * byte of the GPU (an allocation behind its back breaks its accounting or
 * fails against a full pool), or a loop that cannot take the implicit device
 * synchronisation of cudaMalloc/cudaFree.  No counterpart in the reference.
 *
 * Nothing on this path allocates.  The band table, CTA lists and step counters
 * live in one fixed file-scope __device__ array of about 2.1 MB, which every
 * GPU that loads the library holds until exit.  A call may plan at most 32768
 * bands (NPBGB_ERR_NOMEM beyond, before any GPU work).  The first call on a
 * device looks up that array's address (cudaGetSymbolAddress) with the device
 * current; make that first call before any stream capture.  Every call shares
 * the array and the counters are cleared each call, so calls whose work
 * overlaps on the GPU (for example on two streams) race; calls on one stream
 * are ordered.  The plan is copied from shared static host buffers with
 * cudaMemcpyAsync from pageable memory: each call first waits for the work
 * already queued on `stream`, and returns once the plan is staged.  A stream
 * that is capturing a graph is refused with NPBGB_ERR_ARG (a replay would read
 * whatever plan a later call left in those buffers).  Results are
 * bit-identical to npbgb_batch_create + npbgb_batch_launch. */
NPBGB_API int32_t npbgb_batch_run_noalloc(const npbgb_grid* grids, int64_t count,
                                          int32_t band_rows, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* NPBGB_H */
