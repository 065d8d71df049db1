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

/* 2D 5-point Jacobi, the whole time loop of
 *   kernel(TSTEPS, A, B)   polybench/jacobi_2d/jacobi_2d_numpy.py:4-10
 * A and B are (ny, nx).  For t in 1..tsteps-1 it performs the half-sweep
 * A -> B and then B -> A over the interior [1, ny-1) x [1, nx-1):
 *   dst = 0.2 * ((((c + w) + e) + s) + n)
 * Boundary rows and columns are never written.  On return A holds the newest
 * field and B the previous one, as in the reference.  tsteps <= 1 is a no-op. */
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

#ifdef __cplusplus
}
#endif

#endif /* NPBGB_H */
